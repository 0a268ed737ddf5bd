// In-kernel ILU(0) of one system, shared by the solver kernels (k_solve.cu,
// k_solve_rr.cu).  Device code only; include inside the anonymous namespace
// of namespace bilu, after bilu_internal.h.
#pragma once

// --------------------------------------------------------------------------
// ILU(0) of one system in shared memory, rows in level order
// --------------------------------------------------------------------------
// Per entry (i,j) in column order within row i, with the dependency pairs
// (l_ik, u_kj), k ascending, k < min(i,j):
//   approach 1/4 (ILU_0_gpu.cu:26-171, 947-1229): a = fma(-l, u, a) per pair
//   approach 3   (ILU_0_gpu.cu:760-869):          s = fma(l, u, s) ascending, a - s
//   approach 2   (ILU_0_gpu.cu:525-630):          s = fma(u, l, s) descending, a - s
// then a / u_jj below the diagonal.  Rows of one level are independent.
// Block-wide: every thread must call it.
__device__ void ilu_rows(const DevPattern& P, double* LU, int approach) {
  const int* __restrict__ rp = P.rp;
  const int* __restrict__ ci = P.ci;
  const int* __restrict__ dg = P.diag;
  for (int lev = 0; lev < P.nlev_lo; ++lev) {
    const int b = __ldg(P.lev_lo_ptr + lev), e = __ldg(P.lev_lo_ptr + lev + 1);
    for (int q = b + threadIdx.x; q < e; q += blockDim.x) {
      const int i = __ldg(P.lev_lo_rows + q);
      const int rb = __ldg(rp + i), re = __ldg(rp + i + 1);
      for (int k = rb; k < re; ++k) {
        const int j = __ldg(ci + k);
        const int pb = __ldg(P.dep_ptr + k), pe = __ldg(P.dep_ptr + k + 1);
        double v;
        if (approach == 1 || approach == 4) {
          v = LU[k];
          for (int q2 = pb; q2 < pe; ++q2) {
            const int2 d = __ldg(P.dep + q2);
            v = fma(-LU[d.x], LU[d.y], v);
          }
        } else {
          double s = 0.0;
          if (approach == 3) {
            for (int q2 = pb; q2 < pe; ++q2) {
              const int2 d = __ldg(P.dep + q2);
              s = fma(LU[d.x], LU[d.y], s);
            }
          } else {
            for (int q2 = pe - 1; q2 >= pb; --q2) {
              const int2 d = __ldg(P.dep + q2);
              s = fma(LU[d.y], LU[d.x], s);
            }
          }
          v = LU[k] - s;
        }
        if (j < i) v = v / LU[__ldg(dg + j)];
        LU[k] = v;
      }
    }
    __syncthreads();
  }
}
