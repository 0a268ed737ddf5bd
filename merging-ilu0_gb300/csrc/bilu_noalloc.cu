// bilu_solve_noalloc: the batched solve without any device allocation.
//
// Who needs it.  bilu_solve keeps the intermediate factors (the ILU(0) /
// ParILU(0) values and the ISAI values of every system in the batch) in a
// per-plan workspace that it grows with cudaMalloc on first use.  Some
// callers cannot let a solve allocate: a simulation that calls the batched
// solver inside its time-step loop (the reference's matrices come from
// reacting-flow chemistry, one batch per step) fixes its device-memory
// footprint at start-up and must not grow it later, and cudaMalloc/cudaFree
// synchronise the device, stalling the caller's other streams in the middle
// of a step.  This entry point runs the same kernels with the same results,
// but its scratch lives in one fixed file-scope device array that the
// library reserves when its module is loaded.
//
// Limits and rules.
//  * Scratch is kNoAllocScratchBytes (32 MiB) per device, held by every GPU
//    that loads the library until the process exits.  A call whose
//    intermediates do not fit is rejected with BILU_ERR_CAPACITY (split the
//    batch).
//  * Every call on a device shares that one array, and the last call's
//    contents stay in it.  The kernels write every scratch element before
//    reading it, so nothing has to be cleared between calls; but two calls
//    whose kernels overlap on the GPU (different streams, or different host
//    threads, without ordering between them) race on the array.
//  * The first call on a device does the set-up: with that device current it
//    resolves the array's device address (cudaGetSymbolAddress), which loads
//    the library's device module there if that has not happened yet.  Make
//    that first call before any stream capture.  Later calls resolve the
//    address again (a table look-up, no allocation), so it stays right after
//    a cudaDeviceReset has unloaded and reloaded the module.
//  * The scratch layout and the launches are bilu_solve's own
//    (solve_scratch_layout, solve_launch): the same kernels, SELL-32 copies
//    and results bit for bit; only where the scratch lives differs.
//  * The plan itself (bilu_plan_create) allocates its pattern data once;
//    create plans at start-up.  The solve calls no cudaMalloc, cudaFree or
//    allocating library routine.
#include <cuda_runtime.h>

#include <string>

#include "bilu.h"
#include "bilu_internal.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;

// The fixed scratch.  In host code `g_noalloc_scratch` names a host-side
// stand-in, not device memory: only the address from cudaGetSymbolAddress
// may be handed to kernels.
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the scratch on the current device.
bilu_status scratch_address(void** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return bilu::set_error(BILU_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
  *out = p;
  return BILU_OK;
}

}  // namespace

extern "C" bilu_status bilu_solve_noalloc(bilu_plan* P, int nsys, const double* d_values, const double* d_b,
                                          double* d_x, const bilu_results* R, void* stream) {
  using namespace bilu;
  if (!P) return set_error(BILU_ERR_INVALID, "bilu_solve_noalloc: NULL plan");
  if (nsys < 0 || (nsys > 0 && (!d_values || !d_b || !d_x)))
    return set_error(BILU_ERR_INVALID, "bilu_solve_noalloc: bad arguments");
  if (P->opts.isai_lower_diag)
    return set_error(BILU_ERR_INVALID, "bilu_solve_noalloc: plans with isai_lower_diag = 1 only serve bilu_isai");
  if (nsys == 0) return BILU_OK;
  const SolveScratch sc = solve_scratch_layout(P, nsys);
  if (sc.total > kNoAllocScratchBytes)
    return set_error(BILU_ERR_CAPACITY, "bilu_solve_noalloc: " + std::to_string(nsys) + " systems need " +
                                            std::to_string(sc.total) + " bytes of scratch, more than the fixed " +
                                            std::to_string(kNoAllocScratchBytes) + "; split the batch");
  void* base = nullptr;
  if (sc.total > 0) {
    bilu_status st = scratch_address(&base);
    if (st) return st;
  }
  return solve_launch(P, nsys, d_values, nullptr, d_b, d_x, R, static_cast<char*>(base), sc,
                      static_cast<cudaStream_t>(stream));
}
