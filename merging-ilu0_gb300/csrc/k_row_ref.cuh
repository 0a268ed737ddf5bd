// The reference-order row sum of the solver kernels (k_solve.cu,
// k_solve_rr.cu).  Device code only; include inside the anonymous namespace
// of namespace bilu.
#pragma once

// REF: value of the reference's warp-per-row SpMV (Bicgstab_common.hpp:254-290)
// for a row of L entries: lane l holds sum_k fma over entries l, l+32, ...,
// then shfl_down offsets 16..1.  Lanes without entries hold +0, and the
// partial sums are never -0 (fma(a, x, +0) is +0 when the product is zero),
// so an addition of such a lane is an exact no-op and is skipped.  S = the
// smallest power of two >= min(max row length, 32).
template <int S, typename VT, typename IT>
__device__ __forceinline__ double row_ref(const VT* __restrict__ a, const IT* __restrict__ ci, int beg, int L,
                                          const double* __restrict__ x) {
  double v[S];
#pragma unroll
  for (int l = 0; l < S; ++l) {
    double acc = 0.0;
    if (l < L) {
      acc = fma((double)a[beg + l], x[__ldg(ci + beg + l)], 0.0);
      if (S == 32)
        for (int k = l + 32; k < L; k += 32) acc = fma((double)a[beg + k], x[__ldg(ci + beg + k)], acc);
    }
    v[l] = acc;
  }
  int lc = L < S ? L : S;
#pragma unroll
  for (int off = S / 2; off >= 1; off >>= 1) {
#pragma unroll
    for (int i = 0; i < off; ++i)
      if (i + off < lc) v[i] += v[i + off];
    lc = lc < off ? lc : off;
  }
  return v[0];
}
