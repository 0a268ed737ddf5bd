// Register-resident batched BiCGSTAB: the main kernel (one CTA per system of
// a batch sharing one pattern) and the launch code; the device code is in
// k_solve_rr.cuh, the occupancy variants in k_solve_rr_occ.cu and the
// uneven-batch kernel in k_solve_rr_uneven.cu.
#include "k_solve_rr.cuh"

namespace bilu {
namespace {

// one CTA per system of a batch sharing one pattern
// REF: the reference's operation order.  Warp w's lane l owns rows
// l + 32 (w R + k), a block of the reference's lane-strided inner-product
// terms; the inner products chain through the warps in order (ref_chain_sum),
// so every scalar is the reference's bit for bit.
template <int R, int PV, typename FT, bool REF = false>
__global__ void BILU_RR_BOUNDS k_bicgstab_rr(const SolveArgs a, const RRLayout L) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int sys = blockIdx.x;
  if (sys >= a.nsys) return;
  const DevPattern& P = a.pat;
  rr_solve<R, PV, FT, true, REF>(a, P, L, smem, sys, a.A + (size_t)sys * P.a_nnz, a.b + (size_t)sys * P.n,
                                 a.x + (size_t)sys * P.n);
}

template <int PV, typename FT, bool REF>
const void* rr_kernel_pv(int R) {
  switch (R) {
    case 1: return (const void*)k_bicgstab_rr<1, PV, FT, REF>;
    case 2: return (const void*)k_bicgstab_rr<2, PV, FT, REF>;
    case 4: return (const void*)k_bicgstab_rr<4, PV, FT, REF>;
    default: return (const void*)k_bicgstab_rr<8, PV, FT, REF>;
  }
}

}  // namespace

int rr_rows_per_thread(int n, int nt) {
  for (int R : {1, 2, 4, 8})
    if ((long long)R * nt >= n) return R;
  return 0;
}

int rr_max_threads(int R) { return R <= 1 ? 1024 : (R == 2 ? 512 : (R == 4 ? 256 : 128)); }

const void* rr_kernel(int pv, int fp32, int R, int ref, int occ) {
  if (occ) {  // FAST order, the occupancy variants (R = 2, 4, 8; ILU factors at R = 2, 4)
    if (ref || (R != 2 && R != 4 && R != 8) || (R == 8 && pv == 3)) return nullptr;
    return rr_occ_kernel(pv, fp32, R);
  }
  if (ref) {  // reference order: no preconditioner or ILU factors (one warp per system)
    if (pv == 0) return rr_kernel_pv<0, double, true>(R);
    if (pv == 3) return fp32 ? rr_kernel_pv<3, float, true>(R) : rr_kernel_pv<3, double, true>(R);
    return nullptr;
  }
  if (pv == 0) return rr_kernel_pv<0, double, false>(R);
  if (pv == 1) return fp32 ? rr_kernel_pv<1, float, false>(R) : rr_kernel_pv<1, double, false>(R);
  if (pv == 3) return fp32 ? rr_kernel_pv<3, float, false>(R) : rr_kernel_pv<3, double, false>(R);
  return fp32 ? rr_kernel_pv<2, float, false>(R) : rr_kernel_pv<2, double, false>(R);
}

cudaError_t launch_solve_rr(const SolveArgs& a, const RRLayout& L, int nt, int pv, int fp32, int ref, int occ,
                            cudaStream_t st) {
  if (a.nsys == 0) return cudaSuccess;
  const int R = rr_rows_per_thread(a.pat.n, nt);
  if (R == 0 || nt % 32 || nt > rr_max_threads(R)) return cudaErrorInvalidConfiguration;
  const void* k = rr_kernel(pv, fp32, R, ref, occ);
  if (!k) return cudaErrorInvalidConfiguration;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, L.total);
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<SolveArgs*>(&a), const_cast<RRLayout*>(&L)};
  return cudaLaunchKernel(k, dim3(a.nsys), dim3(nt), args, (size_t)L.total, st);
}

}  // namespace bilu
