// Occupancy variants of the register-resident solver (k_solve_rr.cuh), in a
// translation unit of their own so that they compile in parallel with the rest.
#include "k_solve_rr.cuh"

namespace bilu {
namespace {

// Occupancy variants of the same solver (staging bit 4): launch bounds that
// fit more threads per SM at fewer registers per thread, at the cost of a few
// spilled values (tens of bytes per thread, through L1) and a smaller L1
// beside the extra CTAs' shared memory.  Same arithmetic as k_bicgstab_rr at
// the same threads per system:
//   R = 8   128 threads, 4 CTAs per SM (128 registers instead of 168)
//   R = 4   256 threads, 4 CTAs per SM (64 registers), 3 with ILU factors (85)
//   R = 2   512 threads, 2 CTAs per SM (64 registers)
// FP64 issue bounds the solver, and its stalls are load and FP64 latency, so
// more warps per SM keep the FP64 pipe busier.  Measured on GB300 with the
// headline batch (4096 3D 10x10x10 systems, FP32 ISAI): 8 rows per thread on
// 4 CTAs of 128 threads 4.23 ms per solve, 4 rows on 4 CTAs of 256 threads
// 3.49 ms.  ILU factors at 8 rows per thread keep k_bicgstab_rr, whose
// shared-memory layout admits 3 CTAs per SM anyway.  The plan's autotuner
// chooses.
template <int R, int PV>
struct OccBounds {
  static constexpr int threads = R == 8 ? 128 : (R == 4 ? 256 : 512);
  static constexpr int ctas = R == 8 ? 4 : (R == 4 ? (PV == 3 ? 3 : 4) : 2);
};

template <int R, int PV, typename FT>
__global__ void __launch_bounds__(OccBounds<R, PV>::threads, OccBounds<R, PV>::ctas)
    k_bicgstab_rr_occ(const SolveArgs a, const RRLayout L) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int sys = blockIdx.x;
  if (sys >= a.nsys) return;
  const DevPattern& P = a.pat;
  rr_solve<R, PV, FT, true, false>(a, P, L, smem, sys, a.A + (size_t)sys * P.a_nnz, a.b + (size_t)sys * P.n,
                                   a.x + (size_t)sys * P.n);
}

template <int PV, typename FT>
const void* rr_occ_kernel_pv(int R) {
  switch (R) {
    case 2: return (const void*)k_bicgstab_rr_occ<2, PV, FT>;
    case 4: return (const void*)k_bicgstab_rr_occ<4, PV, FT>;
    default: return PV == 3 ? nullptr : (const void*)k_bicgstab_rr_occ<(PV == 3 ? 4 : 8), PV, FT>;
  }
}

}  // namespace

const void* rr_occ_kernel(int pv, int fp32, int R) {
  if (pv == 0) return rr_occ_kernel_pv<0, double>(R);
  if (pv == 1) return fp32 ? rr_occ_kernel_pv<1, float>(R) : rr_occ_kernel_pv<1, double>(R);
  if (pv == 2) return fp32 ? rr_occ_kernel_pv<2, float>(R) : rr_occ_kernel_pv<2, double>(R);
  return fp32 ? rr_occ_kernel_pv<3, float>(R) : rr_occ_kernel_pv<3, double>(R);
}

}  // namespace bilu
