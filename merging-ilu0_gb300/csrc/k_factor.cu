// Preconditioner-generation kernels: ILU(0) (all four reference approaches'
// arithmetic), ParILU(0) Jacobi sweeps, ISAI of L and U, the reference's L/U
// split, missing-diagonal value scatter and the true-residual kernel.  One
// CTA per system, the system's values staged in shared memory.
//
// Reference (paths inside Batched-ILU0-merged/ILU0_ISAI_bicgstab/):
//   ILU(0)      ILU_0_gpu.cu:26-186 (approach 1), :376-685 (2), :693-935 (3), :947-1229 (4)
//   ParILU(0)   parILU_0_gpu.cu:18-113, dependency list :118-220
//   ISAI        isai_gpu.cu:209-287 (extraction), :325-389 (triangular solves), :559-626
//   L/U split   factorization.cu:216-344
//   diag add    factorization.cu:169-188
//   true res.   Bicgstab_common.hpp:294-342
#include <cuda_runtime.h>

#include <type_traits>

#include "bilu_internal.h"
#include "k_intfp.cuh"

namespace bilu {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------- value scatter
__global__ void k_expand(const int* __restrict__ src, int nnz, int nnz_in, int nsys, const double* __restrict__ vin,
                         double* __restrict__ vout) {
  const size_t total = (size_t)nnz * nsys;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < total; g += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(g % nnz);
    const size_t s = g / nnz;
    const int sidx = __ldg(src + k);
    vout[g] = sidx < 0 ? 0.0 : __ldg(vin + s * nnz_in + sidx);
  }
}

// ---------------------------------------------------------------- ILU(0)
// Same per-entry arithmetic as the solver kernel's in-kernel factorisation.
// (The ILU program of the register-resident solver measured 5-15 % slower
// here: this kernel's small CTAs hide the metadata latency by occupancy, and
// the prefetched program words cost it registers.)
__global__ void __launch_bounds__(512) k_ilu0(const DevPattern P, int nsys, const double* __restrict__ A,
                                              double* __restrict__ LUout, int approach) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int sys = blockIdx.x;
  if (sys >= nsys) return;
  const int nnz = P.nnz;
  double* LU = reinterpret_cast<double*>(smem);
  for (int k = threadIdx.x; k < nnz; k += blockDim.x) LU[k] = __ldg(A + (size_t)sys * nnz + k);
  __syncthreads();
  for (int lev = 0; lev < P.nlev_lo; ++lev) {
    const int b = __ldg(P.lev_lo_ptr + lev), e = __ldg(P.lev_lo_ptr + lev + 1);
    for (int q = b + threadIdx.x; q < e; q += blockDim.x) {
      const int i = __ldg(P.lev_lo_rows + q);
      const int rb = __ldg(P.rp + i), re = __ldg(P.rp + i + 1);
      for (int k = rb; k < re; ++k) {
        const int j = __ldg(P.ci + k);
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
        if (j < i) v = v / LU[__ldg(P.diag + j)];
        LU[k] = v;
      }
    }
    __syncthreads();
  }
  for (int k = threadIdx.x; k < nnz; k += blockDim.x) LUout[(size_t)sys * nnz + k] = LU[k];
}

// ---------------------------------------------------------------- ParILU(0)
// Jacobi sweeps: every entry of sweep t+1 is computed from the values of
// sweep t (parilu0_sweep_for_batch_entry_approach2's formula,
// parILU_0_gpu.cu:18-57: sum of l_ik*u_kj by fma from 0 in ascending k, then
// (a_ij - sum)/u_jj below the diagonal, (a_ij - sum)/1 elsewhere).
// With res_tol > 0 the ILU residual of the current iterate,
// ||(A - LU)|_S||_F / ||A||_F, is formed in the same pass (one more fma per
// entry) and the sweeps stop once it is <= res_tol (at most `sweeps`).
__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(kFull, v, off);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  return s;
}

// fast = true (BILU_REDUCE_FAST): the entries below the diagonal are
// multiplied by reciprocals of the current diagonal, formed once per sweep,
// instead of divided (n divisions per sweep instead of one per lower entry).
// TRACK: the ILU residual is formed (res_tol > 0 or res_out); a kernel of its
// own, because FP64 instructions skipped under a runtime condition are
// if-converted into predicated instructions that still take their FP64-unit
// slots on GB300 (measured: about half of the FP64 warp instructions of the
// non-tracking sweeps, before this split).
// SMALL: CTAs of at most 384 threads (n <= 384), bounded for four CTAs per SM
// instead of two (the per-entry register caches below do not fit it).
template <bool FAST, bool TRACK, bool SMALL>
__global__ void __launch_bounds__(SMALL ? 384 : 512, SMALL ? 4 : 2)
    k_parilu0(const DevPattern P, int nsys, const double* __restrict__ A, const double* __restrict__ init,
              double* __restrict__ LUout, int sweeps, double res_tol, int* __restrict__ sweeps_out,
              double* __restrict__ res_out) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red[32];
  const int sys = blockIdx.x;
  if (sys >= nsys) return;
  const int nnz = P.nnz, bd = blockDim.x, tid = threadIdx.x;
  // A is read through L1 rather than staged: two iterates in shared memory
  // (instead of three arrays) fit two CTAs per SM at n = 1000
  double* cur = reinterpret_cast<double*>(smem);
  double* nxt = cur + nnz;
  double* rinv = nxt + nnz;  // FAST only: n reciprocals
  const double* __restrict__ Ag = A + (size_t)sys * nnz;
  const double* Ig = init ? init + (size_t)sys * nnz : Ag;
  double anorm2 = 0.0;
  if constexpr (TRACK) {
    for (int k = tid; k < nnz; k += bd) {
      const double a = __ldg(Ag + k);
      cur[k] = __ldg(Ig + k);
      anorm2 = fma(a, a, anorm2);
    }
    anorm2 = block_sum(anorm2, red);
  } else {
    for (int k = tid; k < nnz; k += bd) cur[k] = __ldg(Ig + k);
  }
  const int lend = P.pl_ndep + P.pl_nlow;
  const int nhi = P.pl_ndep - P.pl_ndep_low;  // entries with pairs on or above the diagonal: [0, nhi)
  // What every sweep reads about this thread's entries is the same in every
  // sweep, so the first CD entries with dependency pairs (program offset, k,
  // j, pair count, a_k), the first CL lower entries without pairs (k, j, a_k)
  // and the first CR diagonal positions are loaded once into registers (the
  // sweeps' loads were dependent chains through L2: the two iterates leave
  // little L1); entries past them are read every sweep as before.  Same
  // arithmetic per entry, so the same bits.  The sizes are the fastest of
  // those that fit 64 registers (two CTAs of 512 threads per SM) without
  // spilling, on the 3D 7-point 10x10x10 headline setup: 1.142 -> 1.065 ms
  // per 4096 systems (CD, CL, CR = 1, 4, 2; 2, 2, 2: 1.125 ms; 0, 6, 0:
  // 1.081 ms).
  // SMALL (CTAs of at most 384 threads, n <= 384): four CTAs per SM at 40
  // registers, which leaves no room for the caches.
  constexpr int CD = SMALL ? 0 : 1, CL = SMALL ? 0 : 4, CR = SMALL ? 0 : 2;
  int dk[CD > 0 ? CD : 1], dj[CD > 0 ? CD : 1], dcnt[CD > 0 ? CD : 1], doff[CD > 0 ? CD : 1];
  double da[CD > 0 ? CD : 1];
#pragma unroll
  for (int c = 0; c < CD; ++c) {
    const int q = tid + c * bd;
    dk[c] = dj[c] = dcnt[c] = doff[c] = 0;
    da[c] = 0.0;
    if (q < P.pl_ndep) {
      const int o = __ldg(P.pl_prog_ptr + (q >> 5)) + (q & 31);
      dk[c] = __ldg(P.pl_prog + o);
      dj[c] = __ldg(P.pl_prog + o + 32) >> 1;
      dcnt[c] = __ldg(P.pl_prog + o + 64);
      doff[c] = o + 96;
      da[c] = __ldg(Ag + dk[c]);
    }
  }
  int lk[CL > 0 ? CL : 1], lj[CL > 0 ? CL : 1];
  double la[CL > 0 ? CL : 1];
#pragma unroll
  for (int c = 0; c < CL; ++c) {
    const int q = P.pl_ndep + tid + c * bd;
    lk[c] = lj[c] = 0;
    la[c] = 0.0;
    if (q < lend) {
      lk[c] = __ldg(P.pl_ent + q);
      lj[c] = __ldg(P.ci + lk[c]);
      la[c] = __ldg(Ag + lk[c]);
    }
  }
  int rd[CR > 0 ? CR : 1];
#pragma unroll
  for (int c = 0; c < CR; ++c) rd[c] = tid + c * bd < P.n ? __ldg(P.diag + tid + c * bd) : 0;
  __syncthreads();
  int done = 0;
  double res = -1.0;
  for (int it = 0; it <= sweeps; ++it) {
    double r2 = 0.0;
    const bool last = (it == sweeps);
    if (!TRACK && last) break;
    if (FAST && !last) {
      // the correctly rounded reciprocal, the same value as 1.0 / u, by integer arithmetic (ifp::rcp): off
      // the FP64 unit, which the sweeps' FMAs and products keep busy
#pragma unroll
      for (int c = 0; c < CR; ++c)
        if (tid + c * bd < P.n) rinv[tid + c * bd] = ifp::rcp(cur[rd[c]]);
      for (int r = tid + CR * bd; r < P.n; r += bd) rinv[r] = ifp::rcp(cur[__ldg(P.diag + r)]);
      __syncthreads();
    }
    // entries with dependency pairs (most pairs first, so a warp's lanes run
    // alike), read from the warp-blocked program: the words of a slot do not
    // depend on one another, so their loads overlap.  LOW (j < i) is a
    // compile-time class: the two classes are separate ranges of entries.
    auto dep_entry = [&](auto low_tag, int k, int j, int cnt, int off, double a) {
      constexpr bool LOW = decltype(low_tag)::value;
      const int* w = P.pl_prog + off;
      double s = 0.0;
#pragma unroll 4
      for (int u = 0; u < cnt; ++u) {
        s = fma(cur[__ldg(w)], cur[__ldg(w + 32)], s);
        w += 64;
      }
      const double as = a - s;
      if constexpr (TRACK) {  // (A - LU)_ij = (a - s) - l_ij u_jj below the diagonal, (a - s) - u_ij on or above it
        const double r = LOW ? fma(-cur[k], cur[__ldg(P.diag + j)], as) : as - cur[k];
        r2 = fma(r, r, r2);
        if (last) return;
      }
      if constexpr (LOW)
        nxt[k] = FAST ? as * rinv[j] : as / cur[__ldg(P.diag + j)];
      else
        nxt[k] = as;
    };
    using HiTag = std::integral_constant<bool, false>;
    using LoTag = std::integral_constant<bool, true>;
#pragma unroll
    for (int c = 0; c < CD; ++c) {
      const int q = tid + c * bd;
      if (q < nhi)
        dep_entry(HiTag{}, dk[c], dj[c], dcnt[c], doff[c], da[c]);
      else if (q < P.pl_ndep)
        dep_entry(LoTag{}, dk[c], dj[c], dcnt[c], doff[c], da[c]);
    }
    auto dep_loaded = [&](auto tag, int q) {
      const int o = __ldg(P.pl_prog_ptr + (q >> 5)) + (q & 31);
      const int k = __ldg(P.pl_prog + o);
      dep_entry(tag, k, __ldg(P.pl_prog + o + 32) >> 1, __ldg(P.pl_prog + o + 64), o + 96, __ldg(Ag + k));
    };
    int q = tid + CD * bd;
    for (; q < nhi; q += bd) dep_loaded(HiTag{}, q);
    for (; q < P.pl_ndep; q += bd) dep_loaded(LoTag{}, q);
    // lower entries without pairs: the sum is 0, so l = a / u_jj (a - 0 == a exactly)
    auto low_entry = [&](int k, int j, double a) {
      if constexpr (TRACK) {
        const double r = fma(-cur[k], cur[__ldg(P.diag + j)], a);
        r2 = fma(r, r, r2);
        if (last) return;
      }
      nxt[k] = FAST ? a * rinv[j] : a / cur[__ldg(P.diag + j)];
    };
#pragma unroll
    for (int c = 0; c < CL; ++c)
      if (P.pl_ndep + tid + c * bd < lend) low_entry(lk[c], lj[c], la[c]);
    for (int q2 = P.pl_ndep + tid + CL * bd; q2 < lend; q2 += bd) {
      const int k = __ldg(P.pl_ent + q2);
      low_entry(k, __ldg(P.ci + k), __ldg(Ag + k));
    }
    // upper entries without pairs: u = a, no arithmetic; their residual a - u
    // is exactly 0 once one sweep has run, so only the initial guess is checked.
    // Each of the two buffers receives the copies once (sweeps 0 and 1) and
    // keeps them: later sweeps would write the same values again.
    if (TRACK && it == 0) {
      for (int q2 = lend + tid; q2 < nnz; q2 += bd) {
        const int k = __ldg(P.pl_ent + q2);
        const double r = __ldg(Ag + k) - cur[k];
        r2 = fma(r, r, r2);
        if (!last) nxt[k] = __ldg(Ag + k);
      }
    } else if (it < 2 && !last) {
      for (int q2 = lend + tid; q2 < nnz; q2 += bd) {
        const int k = __ldg(P.pl_ent + q2);
        nxt[k] = __ldg(Ag + k);
      }
    }
    if constexpr (TRACK) {
      const double tot = block_sum(r2, red);
      res = anorm2 > 0.0 ? sqrt(tot / anorm2) : sqrt(tot);
      if (res_tol > 0.0 && res <= res_tol) break;  // uniform: every thread holds the same sum
    }
    if (last) break;
    __syncthreads();
    double* tswap = cur;
    cur = nxt;
    nxt = tswap;
    ++done;
  }
  __syncthreads();
  if (tid == 0) {
    if (sweeps_out) sweeps_out[sys] = done;
    if (res_out) res_out[sys] = res;
  }
  for (int k = tid; k < nnz; k += bd) LUout[(size_t)sys * nnz + k] = cur[k];
}

// ---------------------------------------------------------------- ISAI
// One thread per ISAI row.  For row i with pattern J (|J| = sz <= 32) the
// reference solves T(J,J)^T m = e_pos with one warp lane per unknown
// (isai_gpu.cu:325-389); the same operations in the same order per unknown:
//   L (lower, unit diagonal): m_{sz-1} = 1; for t = sz-2..0:
//        acc = 0; for c = sz-1..t+1: acc = fma(-m_c, L(J_c,J_t), acc); m_t = acc / 1
//   U (upper): m_0 = 1 / u_ii; for t = 1..sz-1:
//        acc = 0; for c = 0..t-1: acc = fma(-m_c, U(J_c,J_t), acc); m_t = acc / U(J_t,J_t)
// The per-row program lists the structurally nonzero (c, position) pairs in
// exactly that order (zeros of T(J,J) give exact no-op updates).  Thread slot
// s takes row ail_perm[s] / aiu_perm[s]: rows ordered by program length, so a
// warp's lanes run programs of about the same length (one thread computes a
// whole row into its own output range, so which thread does it changes no
// bit).  m is
// accumulated in FP64 in shared memory and rounded to FT on the way out.
// FAST (BILU_REDUCE_FAST): the aiU entries are multiplied by the correctly
// rounded reciprocal of the diagonal (ifp::rcp, one per row, the same value
// as 1.0 / u) instead of divided -- one FP64 reciprocal per row instead of a
// division per aiU entry.  The unit-diagonal aiL is unchanged.
template <typename FT, bool FAST>
__global__ void __launch_bounds__(512) k_isai(const DevPattern P, int nsys, const double* __restrict__ LUg,
                                              FT* __restrict__ ail, FT* __restrict__ aiu) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int sys = blockIdx.x;
  if (sys >= nsys) return;
  const int n = P.n, nnz = P.nnz;
  // the factors are read through L1: only the ISAI values being solved for
  // occupy shared memory (two CTAs per SM at n = 1000 instead of one)
  const double* __restrict__ LU = LUg + (size_t)sys * nnz;
  double* M = reinterpret_cast<double*>(smem);  // max(ail_nnz, aiu_nnz)
  // ---- aiL
  for (int sl = threadIdx.x; sl < n; sl += blockDim.x) {
    const int i = __ldg(P.ail_perm + sl);
    const int beg = __ldg(P.ail_rp + i), sz = __ldg(P.ail_rp + i + 1) - beg;
    double* m = M + beg;
    m[sz - 1] = P.l_diag ? 1.0 / LU[__ldg(P.diag + i)] : 1.0;
    int q = __ldg(P.ail_prog_ptr + (sl >> 5)) + (sl & 31);
    for (int blk = 0; blk < sz - 1; ++blk) {
      const int h = __ldg(P.ail_prog + q);  // t | count << 5; a row's words are 32 apart
      const int ht = h & 31, hc = h >> 5;
      q += 32;
      double acc = 0.0;
      for (int u = 0; u < hc; ++u) {
        const int e = __ldg(P.ail_prog + q);  // c | position in LU << 5
        q += 32;
        acc = fma(-m[e & 31], LU[e >> 5], acc);
      }
      m[ht] = P.l_diag ? acc / LU[__ldg(P.diag + __ldg(P.ail_ci + beg + ht))] : acc;
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < P.ail_nnz; k += blockDim.x) ail[(size_t)sys * P.ail_nnz + k] = (FT)M[k];
  __syncthreads();
  // ---- aiU
  double* rinv = M + (P.ail_nnz > P.aiu_nnz ? P.ail_nnz : P.aiu_nnz);  // FAST: n reciprocals
  if (FAST) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) rinv[i] = ifp::rcp(LU[__ldg(P.diag + i)]);
    __syncthreads();
  }
  for (int sl = threadIdx.x; sl < n; sl += blockDim.x) {
    const int i = __ldg(P.aiu_perm + sl);
    const int beg = __ldg(P.aiu_rp + i), sz = __ldg(P.aiu_rp + i + 1) - beg;
    double* m = M + beg;
    m[0] = FAST ? rinv[i] : 1.0 / LU[__ldg(P.diag + i)];
    int q = __ldg(P.aiu_prog_ptr + (sl >> 5)) + (sl & 31);
    for (int blk = 1; blk < sz; ++blk) {
      const int h = __ldg(P.aiu_prog + q);  // t | count << 5; a row's words are 32 apart
      const int ht = h & 31, hc = h >> 5;
      q += 32;
      double acc = 0.0;
      for (int u = 0; u < hc; ++u) {
        const int e = __ldg(P.aiu_prog + q);  // c | position in LU << 5
        q += 32;
        acc = fma(-m[e & 31], LU[e >> 5], acc);
      }
      const int jt = __ldg(P.aiu_ci + beg + ht);
      m[ht] = FAST ? acc * rinv[jt] : acc / LU[__ldg(P.diag + jt)];
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < P.aiu_nnz; k += blockDim.x) aiu[(size_t)sys * P.aiu_nnz + k] = (FT)M[k];
}

// The products of one block of a row's FP32 ISAI program (fmaf from 0 in
// program order), advancing q past it.  The entries are loaded four at a time
// so that their latencies overlap.
__device__ __forceinline__ float isai_block_f32(const int* __restrict__ prog, int& q, int hc, const float* m,
                                                const float* LU) {
  float acc = 0.0f;
  int u = 0;
  for (; u + 4 <= hc; u += 4) {
    int e[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) e[j] = __ldg(prog + q + 32 * j);  // c | position in LU << 5
    q += 128;
#pragma unroll
    for (int j = 0; j < 4; ++j) acc = fmaf(-m[e[j] & 31], LU[e[j] >> 5], acc);
  }
  for (; u < hc; ++u) {
    const int e = __ldg(prog + q);
    q += 32;
    acc = fmaf(-m[e & 31], LU[e >> 5], acc);
  }
  return acc;
}

// FAST ISAI stored in FP32 (BILU_REDUCE_FAST with BILU_FP32), computed in
// FP32: the factors are rounded to float once into shared memory, every
// product is an fmaf in the order of k_isai's program, and the aiU entries are
// multiplied by the float reciprocal of the rounded diagonal (__frcp_rn, the
// value of 1.0f / u).  The result is what the solver applies (FP32 values,
// FP32 arithmetic); the FP64 pipe only rounds the factors.  No reference
// counterpart (the library's definition; orc_isai_values_ex mode 2).
__global__ void __launch_bounds__(512) k_isai_f32(const DevPattern P, int nsys, const double* __restrict__ LUg,
                                                  float* __restrict__ ail, float* __restrict__ aiu) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int sys = blockIdx.x;
  if (sys >= nsys) return;
  const int n = P.n, nnz = P.nnz;
  float* LU = reinterpret_cast<float*>(smem);
  float* M = LU + nnz;                                                  // max(ail_nnz, aiu_nnz)
  float* rinv = M + (P.ail_nnz > P.aiu_nnz ? P.ail_nnz : P.aiu_nnz);  // n
  for (int k = threadIdx.x; k < nnz; k += blockDim.x) LU[k] = ifp::f32(__ldg(LUg + (size_t)sys * nnz + k));
  __syncthreads();
  // ---- aiL (unit diagonal)
  for (int sl = threadIdx.x; sl < n; sl += blockDim.x) {
    const int i = __ldg(P.ail_perm + sl);
    const int beg = __ldg(P.ail_rp + i), sz = __ldg(P.ail_rp + i + 1) - beg;
    float* m = M + beg;
    m[sz - 1] = 1.0f;
    int q = __ldg(P.ail_prog_ptr + (sl >> 5)) + (sl & 31);
    // blocks 0 .. sz-2; each block's header (t | count << 5) is loaded while the block before it runs
    int h = sz > 1 ? __ldg(P.ail_prog + q) : 0;
    for (int blk = 0; blk < sz - 1; ++blk) {
      const int ht = h & 31, hc = h >> 5;
      q += 32;
      h = blk + 1 < sz - 1 ? __ldg(P.ail_prog + q + 32 * hc) : 0;
      m[ht] = isai_block_f32(P.ail_prog, q, hc, m, LU);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < P.ail_nnz; k += blockDim.x) ail[(size_t)sys * P.ail_nnz + k] = M[k];
  __syncthreads();
  // ---- aiU
  for (int i = threadIdx.x; i < n; i += blockDim.x) rinv[i] = __frcp_rn(LU[__ldg(P.diag + i)]);
  __syncthreads();
  for (int sl = threadIdx.x; sl < n; sl += blockDim.x) {
    const int i = __ldg(P.aiu_perm + sl);
    const int beg = __ldg(P.aiu_rp + i), sz = __ldg(P.aiu_rp + i + 1) - beg;
    float* m = M + beg;
    m[0] = rinv[i];
    int q = __ldg(P.aiu_prog_ptr + (sl >> 5)) + (sl & 31);
    // blocks 1 .. sz-1, headers loaded one block ahead as for aiL
    int h = sz > 1 ? __ldg(P.aiu_prog + q) : 0;
    for (int blk = 1; blk < sz; ++blk) {
      const int ht = h & 31, hc = h >> 5;
      q += 32;
      h = blk + 1 < sz ? __ldg(P.aiu_prog + q + 32 * hc) : 0;
      const float acc = isai_block_f32(P.aiu_prog, q, hc, m, LU);
      m[ht] = acc * rinv[__ldg(P.aiu_ci + beg + ht)];
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < P.aiu_nnz; k += blockDim.x) aiu[(size_t)sys * P.aiu_nnz + k] = M[k];
}

// ---------------------------------------------------------------- general ISAI
// ISAI of A itself (solve_general_dense, isai_gpu.cu:392-554), one thread per
// ISAI row and system.  Lane t of the reference holds row t of A(J,J)^T; here
// T[t][k] = A(J_k, J_t) and the thread runs every lane's operations in the
// same order: for each pivot column dp, the pivot is the first row with the
// largest |T[r][dp]| (the reference's shfl_down tree keeps the lower lane on
// ties), rows are swapped with the right-hand side, every other row r does
// T[r][c] = fma(-m_r, T[dp][c], T[r][c]) with m_r = T[r][dp] / T[dp][dp], and
// finally sol_t / T[t][t].
template <typename FT, int MAXS>
__global__ void __launch_bounds__(256) k_isai_general(const DevPattern P, int nsys, const double* __restrict__ A,
                                                      FT* __restrict__ ai) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int sys = blockIdx.x;
  if (sys >= nsys) return;
  double* As = reinterpret_cast<double*>(smem);
  for (int k = threadIdx.x; k < P.nnz; k += blockDim.x) As[k] = __ldg(A + (size_t)sys * P.nnz + k);
  __syncthreads();
  for (int i = threadIdx.x; i < P.n; i += blockDim.x) {
    const int beg = __ldg(P.ail_rp + i), sz = __ldg(P.ail_rp + i + 1) - beg;
    const int* map = P.gen_map + __ldg(P.gen_map_ptr + i);
    double T[MAXS][MAXS], sol[MAXS];
    for (int k = 0; k < sz; ++k)
      for (int t = 0; t < sz; ++t) {
        const int pos = __ldg(map + k * sz + t);
        T[t][k] = pos >= 0 ? As[pos] : 0.0;
      }
    const int pi = __ldg(P.gen_pos + i);
    for (int t = 0; t < sz; ++t) sol[t] = (t == pi) ? 1.0 : 0.0;
    for (int dp = 0; dp < sz; ++dp) {
      int piv = dp;
      double best = fabs(T[dp][dp]);
      for (int r = dp + 1; r < sz; ++r)
        if (fabs(T[r][dp]) > best) {
          best = fabs(T[r][dp]);
          piv = r;
        }
      if (piv != dp) {
        for (int c = 0; c < sz; ++c) {
          const double tmp = T[dp][c];
          T[dp][c] = T[piv][c];
          T[piv][c] = tmp;
        }
        const double tmp = sol[dp];
        sol[dp] = sol[piv];
        sol[piv] = tmp;
      }
      const double d = T[dp][dp];
      for (int r = 0; r < sz; ++r) {
        if (r == dp) continue;
        const double mult = T[r][dp] / d;
        for (int c = 0; c < sz; ++c) T[r][c] = fma(-mult, T[dp][c], T[r][c]);
        sol[r] = fma(-mult, sol[dp], sol[r]);
      }
    }
    for (int t = 0; t < sz; ++t) ai[(size_t)sys * P.ail_nnz + beg + t] = (FT)(sol[t] / T[t][t]);
  }
}

// ---------------------------------------------------------------- L / U split
__global__ void k_split(const DevPattern P, int nsys, const double* __restrict__ LU, double* __restrict__ L,
                        double* __restrict__ U) {
  const size_t totL = (size_t)P.nnz_L * nsys, totU = (size_t)P.nnz_U * nsys;
  const size_t tot = totL > totU ? totL : totU;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < tot; g += (size_t)gridDim.x * blockDim.x) {
    if (g < totL) {
      const int k = (int)(g % P.nnz_L);
      const size_t s = g / P.nnz_L;
      const int src = __ldg(P.l_src + k);
      L[g] = src < 0 ? 1.0 : __ldg(LU + s * P.nnz + src);
    }
    if (g < totU) {
      const int k = (int)(g % P.nnz_U);
      const size_t s = g / P.nnz_U;
      U[g] = __ldg(LU + s * P.nnz + __ldg(P.u_src + k));
    }
  }
}

// ---------------------------------------------------------------- true residual
// One warp per system: rows in the SpMV tree order of the reference
// (ComputeResidualVec, warp per row), norm = sqrt of the serial inner product
// (L2Norm(n, v), Bicgstab_common.hpp:132) accumulated by lane 0.
__global__ void k_true_residual(const DevPattern P, int nsys, const double* __restrict__ A,
                                const double* __restrict__ b, const double* __restrict__ x, double* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int sys = blockIdx.x;
  if (sys >= nsys) return;
  const int n = P.n;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  double* rs = reinterpret_cast<double*>(smem);
  const double* As = A + (size_t)sys * P.nnz;
  const double* xs = x + (size_t)sys * n;
  const double* bs = b + (size_t)sys * n;
  for (int i = warp; i < n; i += nw) {
    const int beg = __ldg(P.rp + i), end = __ldg(P.rp + i + 1);
    double t = 0.0;
    for (int k = beg + lane; k < end; k += 32) t = fma(__ldg(As + k), __ldg(xs + __ldg(P.ci + k)), t);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(kFull, t, off);
    if (lane == 0) rs[i] = __ldg(bs + i) - t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double acc = 0.0;
    for (int i = 0; i < n; ++i) acc = fma(rs[i], rs[i], acc);
    out[sys] = sqrt(acc);
  }
}

__global__ void k_to_float(const double* __restrict__ a, float* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

template <typename T>
__global__ void k_to_sell(const int* __restrict__ src, int sell_nnz, int csr_nnz, size_t total,
                          const T* __restrict__ in, T* __restrict__ out) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
    const size_t s = q / sell_nnz;
    const int p = (int)(q - s * sell_nnz);
    const int c = __ldg(src + p);
    out[q] = c >= 0 ? in[s * csr_nnz + c] : T(0);
  }
}

int grid_for(size_t total, int threads) {
  size_t g = (total + threads - 1) / threads;
  if (g > 65536) g = 65536;
  if (g < 1) g = 1;
  return (int)g;
}

}  // namespace

cudaError_t launch_expand(const DevPattern& p, int nsys, const double* vin, double* vout, cudaStream_t st) {
  if (nsys == 0) return cudaSuccess;
  k_expand<<<grid_for((size_t)p.nnz * nsys, 256), 256, 0, st>>>(p.src_map, p.nnz, p.nnz_in, nsys, vin, vout);
  return cudaGetLastError();
}

cudaError_t launch_ilu0(const DevPattern& p, int nsys, const double* A, double* lu, int approach, int threads,
                        cudaStream_t st) {
  if (nsys == 0) return cudaSuccess;
  const int smem = p.nnz * 8;
  cudaError_t e = cudaFuncSetAttribute(k_ilu0, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k_ilu0<<<nsys, threads, smem, st>>>(p, nsys, A, lu, approach);
  return cudaGetLastError();
}

cudaError_t launch_parilu0(const DevPattern& p, int nsys, const double* A, const double* init, double* lu,
                           int sweeps, int threads, cudaStream_t st, double res_tol, int* sweeps_out,
                           double* res_out, int fast) {
  if (nsys == 0) return cudaSuccess;
  const int smem = p.nnz * 8 * 2 + (fast ? p.n * 8 : 0);
  const bool track = res_tol > 0.0 || res_out != nullptr;
  const bool small = threads <= 384;
  auto k = small ? (fast ? (track ? k_parilu0<true, true, true> : k_parilu0<true, false, true>)
                         : (track ? k_parilu0<false, true, true> : k_parilu0<false, false, true>))
                 : (fast ? (track ? k_parilu0<true, true, false> : k_parilu0<true, false, false>)
                         : (track ? k_parilu0<false, true, false> : k_parilu0<false, false, false>));
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k<<<nsys, threads, smem, st>>>(p, nsys, A, init, lu, sweeps, res_tol, sweeps_out, res_out);
  return cudaGetLastError();
}

cudaError_t launch_isai(const DevPattern& p, int nsys, const double* lu, void* ail, void* aiu, int fp32, int threads,
                        cudaStream_t st, int fast) {
  if (nsys == 0) return cudaSuccess;
  const bool f32 = fp32 && fast && !p.l_diag;  // FAST FP32 ISAI: computed in FP32 (k_isai_f32)
  // k_isai_f32 stages the factors rounded to float; k_isai reads the FP64 factors through L1
  const int smem = ((f32 ? p.nnz : 0) + (p.ail_nnz > p.aiu_nnz ? p.ail_nnz : p.aiu_nnz) + (fast ? p.n : 0)) *
                   (f32 ? 4 : 8);
  void* k = f32 ? (void*)k_isai_f32
                : fp32 ? (fast ? (void*)k_isai<float, true> : (void*)k_isai<float, false>)
                       : (fast ? (void*)k_isai<double, true> : (void*)k_isai<double, false>);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<DevPattern*>(&p), &nsys, &lu, &ail, &aiu};
  return cudaLaunchKernel(k, dim3(nsys), dim3(threads), args, (size_t)smem, st);
}

cudaError_t launch_to_sell(const int* src, int sell_nnz, int csr_nnz, int nsys, const void* in, void* out,
                           int elem_bytes, cudaStream_t st) {
  const size_t total = (size_t)sell_nnz * nsys;
  if (total == 0) return cudaSuccess;
  if (elem_bytes == 8)
    k_to_sell<double><<<grid_for(total, 256), 256, 0, st>>>(src, sell_nnz, csr_nnz, total,
                                                           static_cast<const double*>(in), static_cast<double*>(out));
  else
    k_to_sell<float><<<grid_for(total, 256), 256, 0, st>>>(src, sell_nnz, csr_nnz, total,
                                                          static_cast<const float*>(in), static_cast<float*>(out));
  return cudaGetLastError();
}

cudaError_t launch_to_float(const double* a, float* b, size_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_to_float<<<grid_for(n, 256), 256, 0, st>>>(a, b, n);
  return cudaGetLastError();
}

cudaError_t launch_isai_general(const DevPattern& p, int nsys, const double* A, void* ai, int fp32, int threads,
                                cudaStream_t st) {
  if (nsys == 0) return cudaSuccess;
  const int smem = p.nnz * 8;
  threads = threads > 256 ? 256 : threads;
  void* k;
  if (p.gen_maxs <= 8)
    k = fp32 ? (void*)k_isai_general<float, 8> : (void*)k_isai_general<double, 8>;
  else if (p.gen_maxs <= 16)
    k = fp32 ? (void*)k_isai_general<float, 16> : (void*)k_isai_general<double, 16>;
  else
    k = fp32 ? (void*)k_isai_general<float, 32> : (void*)k_isai_general<double, 32>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  void* args[] = {const_cast<DevPattern*>(&p), &nsys, &A, &ai};
  return cudaLaunchKernel(k, dim3(nsys), dim3(threads), args, (size_t)smem, st);
}

cudaError_t launch_split(const DevPattern& p, int nsys, const double* lu, double* L, double* U, cudaStream_t st) {
  if (nsys == 0) return cudaSuccess;
  const size_t tot = (size_t)(p.nnz_L > p.nnz_U ? p.nnz_L : p.nnz_U) * nsys;
  k_split<<<grid_for(tot, 256), 256, 0, st>>>(p, nsys, lu, L, U);
  return cudaGetLastError();
}

cudaError_t launch_true_residual(const DevPattern& p, int nsys, const double* A, const double* b, const double* x,
                                 double* out, int threads, cudaStream_t st) {
  if (nsys == 0) return cudaSuccess;
  const int smem = p.n * 8;
  cudaError_t e = cudaFuncSetAttribute(k_true_residual, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k_true_residual<<<nsys, threads, smem, st>>>(p, nsys, A, b, x, out);
  return cudaGetLastError();
}

}  // namespace bilu
