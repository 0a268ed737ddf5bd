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
//  * The first call on a device resolves the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture.
//  * The plan itself (bilu_plan_create) allocates its pattern data once;
//    create plans at start-up.  The solve calls no cudaMalloc, cudaFree or
//    allocating library routine.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "bilu.h"
#include "bilu_internal.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;

// The fixed scratch.  In host code `g_noalloc_scratch` names a host-side
// stand-in, not device memory: only the address from cudaGetSymbolAddress
// may be handed to kernels.
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {nullptr};

// Device address of the scratch on the current device (set-up once per device).
bilu_status scratch_address(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return bilu::set_error(BILU_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return bilu::set_error(BILU_ERR_CAPACITY, "device ordinal beyond 64");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return bilu::set_error(BILU_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return BILU_OK;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

bilu_status cuda_fail(cudaError_t e, const char* what) {
  return bilu::set_error(BILU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
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
  const bilu_options& o = P->opts;
  const int prec = o.precond;
  const bool fp32 = o.factor_precision == BILU_FP32;
  const bool isai =
      prec == BILU_PRECOND_ILU0_ISAI || prec == BILU_PRECOND_PARILU0_ISAI || prec == BILU_PRECOND_GENERAL_ISAI;
  const bool needs_factors = !(prec == BILU_PRECOND_ILU0 || prec == BILU_PRECOND_NONE);
  // scratch layout: [expanded values][LU][LU as float | aiL][aiU]
  const size_t nz = (size_t)P->nnz * nsys;
  size_t need = 0;
  const size_t off_exp = need;
  if (needs_factors && P->missing) need += align256(nz * 8);
  const size_t off_lu = need;
  if (needs_factors) need += align256(nz * 8);
  const size_t off_f = need;
  if (needs_factors && fp32 && !isai) need += align256(nz * 4);
  const size_t off_ail = need;
  if (isai) need += align256((size_t)P->dp.ail_nnz * nsys * (fp32 ? 4 : 8));
  const size_t off_aiu = need;
  if (isai) need += align256((size_t)P->dp.aiu_nnz * nsys * (fp32 ? 4 : 8));
  if (need > kNoAllocScratchBytes)
    return set_error(BILU_ERR_CAPACITY, "bilu_solve_noalloc: " + std::to_string(nsys) + " systems need " +
                                            std::to_string(need) + " bytes of scratch, more than the fixed " +
                                            std::to_string(kNoAllocScratchBytes) + "; split the batch");
  char* ws = nullptr;
  if (needs_factors) {
    void* base = nullptr;
    bilu_status st = scratch_address(&base);
    if (st) return st;
    ws = static_cast<char*>(base);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  SolveArgs a;
  a.pat = P->dp;
  a.lay = P->lay;
  a.nsys = nsys;
  a.A = d_values;
  a.b = d_b;
  a.x = d_x;
  if (R) {
    a.iters = R->iter_counts;
    a.conv = R->conv_flags;
    a.res = R->iter_res_norms;
    a.status = R->status;
    a.true_res = o.compute_true_residual ? R->true_res_norms : nullptr;
  }
  a.tol = o.tol;
  a.tol_mode = o.tol_mode;
  a.max_iter = o.max_iter;
  a.approach = o.ilu_approach;
  a.dot_serial = isai ? 1 : 0;
  cudaError_t e = cudaSuccess;
  const int ft = P->n > 512 ? 512 : ((P->n < 64 ? 64 : P->n) + 31) / 32 * 32;
  if (prec == BILU_PRECOND_ILU0) {
    a.prec = PK_ILU_INKERNEL;
  } else if (prec == BILU_PRECOND_NONE) {
    a.prec = PK_NONE;
  } else {
    const double* fv = d_values;
    if (P->missing) {
      e = launch_expand(P->dp, nsys, d_values, reinterpret_cast<double*>(ws + off_exp), s);
      if (e != cudaSuccess) return cuda_fail(e, "expand");
      fv = reinterpret_cast<const double*>(ws + off_exp);
    }
    double* lu = reinterpret_cast<double*>(ws + off_lu);
    if (prec == BILU_PRECOND_GENERAL_ISAI) {
      e = launch_isai_general(P->dp, nsys, fv, ws + off_ail, fp32 ? 1 : 0, ft, s);
      if (e != cudaSuccess) return cuda_fail(e, "general isai");
    } else if (prec == BILU_PRECOND_ILU0_SPLIT || prec == BILU_PRECOND_ILU0_ISAI)
      e = launch_ilu0(P->dp, nsys, fv, lu, o.ilu_approach, ft, s);
    else
      e = launch_parilu0(P->dp, nsys, fv, nullptr, lu, o.parilu_sweeps, ft, s, o.parilu_res_tol,
                         R ? R->parilu_sweeps : nullptr, R ? R->ilu_residual : nullptr,
                         o.reduction == BILU_REDUCE_FAST ? 1 : 0);
    if (e != cudaSuccess) return cuda_fail(e, "factorisation");
    if (isai) {
      if (prec != BILU_PRECOND_GENERAL_ISAI) {
        e = launch_isai(P->dp, nsys, lu, ws + off_ail, ws + off_aiu, fp32 ? 1 : 0, ft, s,
                        o.reduction == BILU_REDUCE_FAST ? 1 : 0);
        if (e != cudaSuccess) return cuda_fail(e, "isai");
      }
      a.prec = PK_ISAI;
      a.ail = ws + off_ail;
      a.aiu = prec == BILU_PRECOND_GENERAL_ISAI ? nullptr : ws + off_aiu;
    } else {
      a.prec = PK_LU_GLOBAL;
      if (fp32) {
        float* f = reinterpret_cast<float*>(ws + off_f);
        e = launch_to_float(lu, f, nz, s);
        if (e != cudaSuccess) return cuda_fail(e, "convert");
        a.F = f;
      } else {
        a.F = lu;
      }
    }
  }
  int maxl = P->a_maxl;
  if (P->has_isai)
    for (int i = 0; i < P->n; ++i) {
      maxl = maxl > P->ail_rp[i + 1] - P->ail_rp[i] ? maxl : P->ail_rp[i + 1] - P->ail_rp[i];
      maxl = maxl > P->aiu_rp[i + 1] - P->aiu_rp[i] ? maxl : P->aiu_rp[i + 1] - P->aiu_rp[i];
    }
  e = P->rr ? launch_solve_rr(a, P->rr_lay, P->rr_threads, P->rr_pv, fp32 ? 1 : 0,
                              o.reduction == BILU_REDUCE_FAST ? 0 : 1, P->rr_occ4 ? 1 : 0, s)
            : launch_solve(a, P->threads, fp32 ? 1 : 0, o.reduction == BILU_REDUCE_FAST ? 1 : 0, maxl, s);
  if (e != cudaSuccess) return cuda_fail(e, "solver launch");
  return BILU_OK;
}
