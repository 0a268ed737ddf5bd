// Batched FP64 dense LU with partial pivoting: the forward-error reference of
// the iterative solves (no counterpart in the reference, which reports only
// iteration counts).  One CTA per sampled system; the dense matrix lives in a
// global workspace (n*n doubles per system, L2-resident while the CTA works).
//
// Operation order (identical to the oracle's orc_dense_solve, so the two agree
// bit for bit): pivot = first row with the largest |a_ik|, k <= i; rows swapped
// with the right-hand side; multipliers f_i = a_ik / a_kk stored in place;
// a_ij = fma(-f_i, a_kj, a_ij) and y_i = fma(-f_i, y_k, y_i); back substitution
// by columns: x_j = y_j / u_jj, then y_i = fma(-u_ij, x_j, y_i) for i < j.
#include <cuda_runtime.h>

#include "bilu_internal.h"

namespace bilu {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__global__ void __launch_bounds__(512) k_dense_solve(const int n, const int nnz, const int* __restrict__ rp,
                                                     const int* __restrict__ ci, const int* __restrict__ sys_ids,
                                                     const int nsample, const double* __restrict__ A,
                                                     const double* __restrict__ b, double* __restrict__ work,
                                                     double* __restrict__ x_out) {
  __shared__ double s_val[32];
  __shared__ int s_idx[32];
  __shared__ int s_piv;
  const int q = blockIdx.x;
  if (q >= nsample) return;
  const int s = sys_ids[q];
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  double* M = work + (size_t)q * ((size_t)n * n + n);
  double* y = M + (size_t)n * n;
  const double* As = A + (size_t)s * nnz;
  for (size_t e = tid; e < (size_t)n * n; e += nt) M[e] = 0.0;
  __syncthreads();
  for (int i = tid; i < n; i += nt) {
    for (int k = rp[i]; k < rp[i + 1]; ++k) M[(size_t)i * n + ci[k]] = As[k];
    y[i] = b[(size_t)s * n + i];
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    // pivot: largest |a_ik|, first on ties
    double best = -1.0;
    int bi = n;
    for (int i = k + tid; i < n; i += nt) {
      const double v = fabs(M[(size_t)i * n + k]);
      if (v > best) {  // rows visited in ascending order: keeps the first maximum
        best = v;
        bi = i;
      }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const double ov = __shfl_down_sync(kFull, best, off);
      const int oi = __shfl_down_sync(kFull, bi, off);
      if (ov > best || (ov == best && oi < bi)) {
        best = ov;
        bi = oi;
      }
    }
    if (lane == 0) {
      s_val[warp] = best;
      s_idx[warp] = bi;
    }
    __syncthreads();
    if (tid == 0) {
      double bv = s_val[0];
      int bx = s_idx[0];
      for (int w = 1; w < nw; ++w)
        if (s_val[w] > bv || (s_val[w] == bv && s_idx[w] < bx)) {
          bv = s_val[w];
          bx = s_idx[w];
        }
      s_piv = bx < n ? bx : k;
    }
    __syncthreads();
    const int p = s_piv;
    if (p != k) {
      for (int j = tid; j < n; j += nt) {
        const double t = M[(size_t)k * n + j];
        M[(size_t)k * n + j] = M[(size_t)p * n + j];
        M[(size_t)p * n + j] = t;
      }
      if (tid == 0) {
        const double t = y[k];
        y[k] = y[p];
        y[p] = t;
      }
    }
    __syncthreads();
    const double d = M[(size_t)k * n + k];
    for (int i = k + 1 + tid; i < n; i += nt) M[(size_t)i * n + k] = M[(size_t)i * n + k] / d;
    __syncthreads();
    // rows with f == 0 are skipped, as the oracle does (the update would be exact anyway)
    const int w = n - k - 1;
    for (long long e = tid; e < (long long)w * (w + 1); e += nt) {
      const int i = k + 1 + (int)(e / (w + 1));
      const int jj = (int)(e % (w + 1));
      const double f = M[(size_t)i * n + k];
      if (f == 0.0) continue;
      if (jj < w) {
        const int j = k + 1 + jj;
        M[(size_t)i * n + j] = fma(-f, M[(size_t)k * n + j], M[(size_t)i * n + j]);
      } else {
        y[i] = fma(-f, y[k], y[i]);
      }
    }
    __syncthreads();
  }
  double* xs = x_out + (size_t)q * n;
  __shared__ double s_x;
  for (int j = n - 1; j >= 0; --j) {
    if (tid == 0) {
      s_x = y[j] / M[(size_t)j * n + j];
      xs[j] = s_x;
    }
    __syncthreads();
    const double xj = s_x;
    for (int i = tid; i < j; i += nt) y[i] = fma(-M[(size_t)i * n + j], xj, y[i]);
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_dense_solve(const DevPattern& p, int nsample, const int* sys_ids, const double* A, const double* b,
                               double* work, double* x_out, cudaStream_t st) {
  if (nsample == 0) return cudaSuccess;
  k_dense_solve<<<nsample, 512, 0, st>>>(p.n, p.a_nnz, p.a_rp, p.a_ci, sys_ids, nsample, A, b, work, x_out);
  return cudaGetLastError();
}

}  // namespace bilu
