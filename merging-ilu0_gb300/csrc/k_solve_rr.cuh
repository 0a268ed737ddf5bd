// Device code of the register-resident batched BiCGSTAB solver, shared by
// the translation units that instantiate its kernels (k_solve_rr.cu: the
// main kernel and the launch code; k_solve_rr_occ.cu: the occupancy
// variants; k_solve_rr_uneven.cu: the uneven-batch kernel), which compile
// in parallel.  Everything here is in an anonymous namespace: each unit
// gets its own copy of what it instantiates.
//
// Register-resident batched BiCGSTAB for BILU_REDUCE_FAST with an ISAI
// preconditioner (two triangles or the general ISAI of A), in-place ILU
// factors (factorised in the kernel, the merged form, or given) or none; and
// ILU factors or none in the reference's operation order (REF: rows of at
// most 16 entries; ref_chain_sum says why the order is the reference's).
//
// Same method, exits and iteration counting as the shared-memory kernel
// (k_solve.cu, after PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu:249-538,
// PrecondBiCGSTAB_ilu_isai_gpu.cu:89-257 and Bicgstab_common.hpp:195-250);
// only the reduction order differs, and it is fixed by (threads per system,
// rows per thread), so the oracle restates it bit for bit
// (orc_bicgstab_fast).
//
// GB300 mapping.  FP64 issue is the bound (about two FP64 lane-operations per
// clock per SM, one warp instruction costs the same whatever its active
// mask), and the shared-memory kernel loses most of it to serialisation: one
// 200 KB CTA per SM, warp-0 inner products (32 dependent FMAs at n = 1000) and
// ~15 block barriers per iteration during which the SM's FP64 pipes idle.
// Here:
//   * thread t of an NT-thread CTA owns rows t + k*NT, k < R (R <= 8); the
//     vectors x, r/s, p, v and t live in its registers (r_hat = b is re-read
//     through L1, p_hat / s_hat are read back from shared memory);
//   * shared memory holds only what other rows read: the SpMV input p_hat /
//     s_hat (FP64), the preconditioner input and intermediate (FT), and, when
//     they fit without costing occupancy, A and the ISAI values;
//   * the six inner products of an iteration run as four block reductions
//     in one shared slot (orders below); warp 0 alone forms the scalar
//     recurrence (divisions, square roots, the next beta) and broadcasts it
//     through shared memory, so those FP64 instructions run once per CTA, not
//     once per warp; 13 barriers per iteration besides the preconditioner's;
//   * the CTA is small (one warp for n <= 256), so several systems share an SM
//     and one system's barrier or reduction latency overlaps another's FMAs;
//   * with FP32 ISAI values (BILU_FP32) both preconditioner SpMVs run on the
//     FP32 pipe; FP64 stays in A*x, the inner products and the recurrences;
//   * ILU factors live in shared memory (the merged form factorises there
//     from the plan's ILU program); the triangular solves run level by level
//     over the whole CTA from the plan's per-level solve programs, in place on
//     the preconditioner vector, one barrier per level;
//   * SpMV column indices are read as 16-bit copies, and A and aiU optionally
//     from SELL-32 copies (coalesced per warp) made before the launch.
//
// Reduction order (what orc_bicgstab_fast restates):
//   thread partial   d = fma(a_i, b_i, d) over its rows in k order, from 0.0
//   no ILU factors   lane l: s_l = d_l; s_l = s_l + d_(l+32j) for warps j = 1 .. NT/32-1,
//                    then for off = 16, 8, 4, 2, 1: s_l = s_l + s_(l^off); lane 0's value
//   ILU factors      per warp: for off = 16 .. 1: d_l = d_l + d_(l^off), lane 0's value
//                    w_j; then s = w_0 + w_1 + ... over the warps in order
//   SpMV row         acc = fma(a_k, x_ci(k), acc), k ascending, from 0.0 (FP64)
//   ISAI row (FT)    the same in FT; input rounded to FT, output widened to FP64
//   LU solve (FT)    input rounded to FT; lower row i: a = y_i, a = fma(-l_ik, y_k, a)
//                    over k ascending, y_i = a; upper row i: a = y_i, a = fma(-u_ik,
//                    z_k, a) over k descending, z_i = a * rinv_i with rinv_i =
//                    1.0 / u_ii in FP64 (rounded to float for FP32 factors); z
//                    widened to FP64
#pragma once

#include <cuda_runtime.h>

#include "bilu_internal.h"
#include "k_intfp.cuh"

namespace bilu {
namespace {

constexpr unsigned kFull = 0xffffffffu;

#include "k_ilu_rows.cuh"
#include "k_row_ref.cuh"

// K values summed over the CTA into the threads of warp 0 (the other warps'
// v is left as it was); returns true on warp 0, which then forms the scalar
// recurrence alone and broadcasts it, so the divisions and square roots of an
// iteration run once per CTA.  Two orders (red: K * nt doubles):
//   LANES_FIRST  every thread stores its partial; lane l of warp 0 sums
//                partials l, l+32, l+64, ... in order, then an xor butterfly
//                (v_l = v_l + v_(l^off), off = 16 .. 1).  Only warp 0 adds.
//   otherwise    an xor butterfly in every warp, lane 0 stores the warp's sum,
//                and warp 0 sums the warps' sums in order.  Fewer dependent
//                adds after the barrier: better where barriers are on the
//                critical path (ILU factors, level-scheduled solves).
template <int K, bool LANES_FIRST>
__device__ __forceinline__ bool block_sum_w0(double (&v)[K], double* red, int nw) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nt = nw * 32;
  if (LANES_FIRST) {
#pragma unroll
    for (int k = 0; k < K; ++k) red[k * nt + threadIdx.x] = v[k];
  } else {
#pragma unroll
    for (int k = 0; k < K; ++k) {
#pragma unroll
      for (int off = 16; off >= 1; off >>= 1) v[k] = v[k] + __shfl_xor_sync(kFull, v[k], off);
      if (lane == 0) red[k * nt + warp] = v[k];
    }
  }
  __syncthreads();
  if (warp != 0) return false;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    if (LANES_FIRST) {
      double s = red[k * nt + lane];
      for (int w = 1; w < nw; ++w) s = s + red[k * nt + w * 32 + lane];
#pragma unroll
      for (int off = 16; off >= 1; off >>= 1) s = s + __shfl_xor_sync(kFull, s, off);
      v[k] = s;
    } else {
      double s = red[k * nt];
      for (int w = 1; w < nw; ++w) s = s + red[k * nt + w];
      v[k] = s;
    }
  }
  return true;
}

// Reference order with W = nw warps.  The reference sums an inner product on
// one warp: lane l runs fma over rows l, l+32, l+64, ... in order from 0.0,
// then a shfl_down tree (Bicgstab_common.hpp:195-250).  Warp w owns lane l's
// rows l + 32 (w R + k), k < R, the w-th block of that sequence, so the chain
// passes from warp to warp through red (one barrier per warp).  The last warp
// then runs the xor butterfly: its lane 0 adds the same pairs as the shfl_down
// tree (IEEE addition commutes).  term(k, acc) adds row k's terms to the K
// accumulators (nothing for rows >= n).  Returns true on the last warp, which
// forms the scalar recurrence and broadcasts it.  One warp: no barrier.
template <int K, int R, typename Term>
__device__ __forceinline__ bool ref_chain_sum(double (&v)[K], Term term, double* red, int nw) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int w = 0; w < nw; ++w) {
    if (warp == w) {
#pragma unroll
      for (int j = 0; j < K; ++j) v[j] = w == 0 ? 0.0 : red[j * 32 + lane];
#pragma unroll
      for (int k = 0; k < R; ++k) term(k, v);
      if (w + 1 < nw) {
#pragma unroll
        for (int j = 0; j < K; ++j) red[j * 32 + lane] = v[j];
      }
    }
    if (w + 1 < nw) __syncthreads();
  }
  if (warp != nw - 1) return false;
#pragma unroll
  for (int j = 0; j < K; ++j) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v[j] = v[j] + __shfl_xor_sync(kFull, v[j], off);
  }
  return true;
}

__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }
// FP64 -> FT and FT -> FP64 with the integer conversions for float (k_intfp.cuh).
// Used where the conversions share the SMs with FP64 work (the ISAI paths:
// preconditioner input and output around the FP32 SpMVs).  The level-scheduled
// triangular solves keep the hardware conversions: those phases issue no FP64
// arithmetic, and the integer form only adds latency there (measured 1-2 %
// slower on the FP32-factor paths).
template <typename FT>
__device__ __forceinline__ FT round_t(double x) {
  if constexpr (sizeof(FT) == 4)
    return ifp::f32(x);
  else
    return x;
}
template <typename FT>
__device__ __forceinline__ double widen_t(FT y) {
  if constexpr (sizeof(FT) == 4)
    return ifp::f64(y);
  else
    return y;
}

// out[k] = row (tid + k*nt) of M times xv, for the R rows of this thread
// (rows >= n give 0).  The R rows advance together, entry j of every row per
// step, so the thread has R independent FMA chains in flight (64-cycle FP64
// latency) instead of one; each row still sums its entries in ascending order
// from 0.
template <int R, typename VT, typename XT, typename IT>
__device__ __forceinline__ void rows_acc(const VT* __restrict__ val, const IT* __restrict__ ci,
                                         const int* __restrict__ rp, int tid, int nt, int n,
                                         const XT* __restrict__ xv, XT (&out)[R]) {
  int beg[R], len[R];
  int jmax = 0;
#pragma unroll
  for (int k = 0; k < R; ++k) {
    const int i = tid + k * nt;
    beg[k] = i < n ? __ldg(rp + i) : 0;
    len[k] = i < n ? __ldg(rp + i + 1) - beg[k] : 0;
    jmax = max(jmax, len[k]);
    out[k] = XT(0);
  }
  for (int j = 0; j < jmax; ++j) {
#pragma unroll
    for (int k = 0; k < R; ++k)
      if (j < len[k]) out[k] = fma_t((XT)val[beg[k] + j], xv[__ldg(ci + beg[k] + j)], out[k]);
  }
}

// rows_acc on a matrix in the SELL-32 layout (DevPattern::sa_* / su_*): the
// same FMAs in the same order; entry j of the warp's 32 rows (tid + k*nt for
// one k: 32 consecutive rows, one slice) is one contiguous line of values and
// of column indices.
template <int R, typename VT, typename XT, typename IT>
__device__ __forceinline__ void rows_acc_sell(const VT* __restrict__ val, const IT* __restrict__ sci,
                                              const int* __restrict__ soff, const int* __restrict__ rp, int tid,
                                              int nt, int n, const XT* __restrict__ xv, XT (&out)[R]) {
  int pos[R], len[R];
  int jmax = 0;
#pragma unroll
  for (int k = 0; k < R; ++k) {
    const int i = tid + k * nt;
    pos[k] = i < n ? __ldg(soff + (i >> 5)) + (i & 31) : 0;
    len[k] = i < n ? __ldg(rp + i + 1) - __ldg(rp + i) : 0;
    jmax = max(jmax, len[k]);
    out[k] = XT(0);
  }
  for (int j = 0; j < jmax; ++j) {
#pragma unroll
    for (int k = 0; k < R; ++k)
      if (j < len[k]) out[k] = fma_t((XT)val[pos[k] + 32 * j], xv[__ldg(sci + pos[k] + 32 * j)], out[k]);
  }
}

// One triangle of z = U^{-1} L^{-1} y over the CTA, level by level, in place
// on y, from the triangle's solve program (DevPattern::tp_*).  Thread t takes
// slot t of every level (and t + nt, ... of wider ones); the record and the
// first kTrsvPrefetch entries of its next slot are loaded one level ahead and
// the level headers two levels ahead, so the global-memory latency of the
// program overlaps the current level's arithmetic and barrier.
// Row i starts from y_i and subtracts its products in program order (one FMA
// each, no separate subtraction); UPPER then scales by rinv_i and also widens
// z_i into zd for FP32 factors.  Ends with a barrier.
// REF: the reference's order instead (PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu:22-108):
// s = sum of fma(F, y, s) from 0 in program order, then y_i - s, and for UPPER
// (y_i - s) / u_ii with FP64 factors (rinv then holds u_ii itself) or
// (y_i - s) * rinv_i with FP32 factors (the library's FP32 definition).
template <bool UPPER, typename FT, bool REF>
__device__ __forceinline__ void tri_solve(const int2* __restrict__ hdr, const int* __restrict__ prog, int nlev,
                                          const FT* __restrict__ F, const FT* __restrict__ rinv, FT* y, double* zd,
                                          int tid, int nt, int maxcnt) {
  constexpr int PF = kTrsvPrefetch;
  // maxcnt: the most entries of any row of this triangle (the plan's
  // DevPattern::tp_maxcnt_*).  With FP64 factors, triangles whose rows have at
  // most two entries (5-point stencils) run a copy of the row code with two
  // product slots instead of kTrsvPrefetch: a guarded FMA can be if-converted
  // into a predicated one, which still takes its FP64-unit slot on GB300.
  // Measured (CUDA events): 2D 16x16 reference order 1.01 -> 1.12M systems/s,
  // FAST with the reference's stopping rule 84.2 -> 68.7 ms, 24x24 414k ->
  // 423k; 3D 10x10x10 (three entries per row) unchanged.  The choice is one
  // uniform branch between two fully unrolled copies (a per-slot runtime bound
  // cost the 3D solves 5-8 %); FP32 factors keep the single copy (their FMAs
  // use the FP32 pipe, and the second copy cost the FP32 3D solve 4 %).
  const bool two = sizeof(FT) == 8 && maxcnt <= 2;
  auto row = [&](int rec, const int (&e)[PF], int off, int w, int s) {
    const int i = rec & 1023, cnt = rec >> 10;
    if (REF) {
      FT acc = FT(0);
      if (two) {
#pragma unroll
        for (int j = 0; j < 2; ++j)
          if (j < cnt) acc = fma_t(F[e[j] >> 10], y[e[j] & 1023], acc);
      } else {
#pragma unroll
        for (int j = 0; j < PF; ++j)
          if (j < cnt) acc = fma_t(F[e[j] >> 10], y[e[j] & 1023], acc);
      }
      for (int j = PF; j < cnt; ++j) {
        const int en = __ldg(prog + off + w + j * w + s);
        acc = fma_t(F[en >> 10], y[en & 1023], acc);
      }
      const FT d = y[i] - acc;
      if (UPPER) {
        const FT z = sizeof(FT) == 8 ? d / rinv[i] : d * rinv[i];
        y[i] = z;
        if (sizeof(FT) == 4) zd[i] = (double)z;
      } else {
        y[i] = d;
      }
      return;
    }
    FT acc = y[i];
    if (two) {
#pragma unroll
      for (int j = 0; j < 2; ++j)
        if (j < cnt) acc = fma_t(-F[e[j] >> 10], y[e[j] & 1023], acc);
    } else {
#pragma unroll
      for (int j = 0; j < PF; ++j)
        if (j < cnt) acc = fma_t(-F[e[j] >> 10], y[e[j] & 1023], acc);
    }
    for (int j = PF; j < cnt; ++j) {
      const int en = __ldg(prog + off + w + j * w + s);
      acc = fma_t(-F[en >> 10], y[en & 1023], acc);
    }
    if (UPPER) {
      const FT z = acc * rinv[i];
      y[i] = z;
      if (sizeof(FT) == 4) zd[i] = (double)z;
    } else {
      y[i] = acc;
    }
  };
  auto fetch = [&](int2 h, int& rec, int (&e)[PF]) {
    rec = 0;
    if (tid < h.y) {
      rec = __ldg(prog + h.x + tid);
#pragma unroll
      for (int j = 0; j < PF; ++j) e[j] = __ldg(prog + h.x + h.y + j * h.y + tid);
    }
  };
  const int2 zero = make_int2(0, 0);
  int2 h = nlev > 0 ? __ldg(hdr) : zero;
  int2 hn = nlev > 1 ? __ldg(hdr + 1) : zero;
  int rec, e[PF];
  fetch(h, rec, e);
  for (int lev = 0; lev < nlev; ++lev) {
    const int2 hnn = lev + 2 < nlev ? __ldg(hdr + lev + 2) : zero;
    int recn, en[PF];
    fetch(hn, recn, en);
    if (tid < h.y) row(rec, e, h.x, h.y, tid);
    for (int s = tid + nt; s < h.y; s += nt) {
      int r2, e2[PF];
      r2 = __ldg(prog + h.x + s);
#pragma unroll
      for (int j = 0; j < PF; ++j) e2[j] = __ldg(prog + h.x + h.y + j * h.y + s);
      row(r2, e2, h.x, h.y, s);
    }
    __syncthreads();
    h = hn;
    hn = hnn;
    rec = recn;
#pragma unroll
    for (int j = 0; j < PF; ++j) e[j] = en[j];
  }
}

// z = U^{-1} L^{-1} y over the CTA (y: the preconditioner input, already
// rounded to FT; for FP64 factors y is the FP64 SpMV input itself, for FP32
// factors the upper solve widens z into zd).  Ends with a barrier: z is
// visible to every thread.
template <typename FT, bool REF>
__device__ __forceinline__ void lu_apply(const DevPattern& P, const FT* __restrict__ F, const FT* __restrict__ rinv,
                                         FT* y, double* zd, int tid, int nt) {
  tri_solve<false, FT, REF>(P.tp_lo_hdr, P.tp_lo, P.nlev_lo, F, rinv, y, zd, tid, nt, P.tp_maxcnt_lo);
  tri_solve<true, FT, REF>(P.tp_up_hdr, P.tp_up, P.nlev_up, F, rinv, y, zd, tid, nt, P.tp_maxcnt_up);
}

// The reference-order SpMV rows (row_ref, the reference's warp-per-row tree
// for rows of at most 16 entries) for this thread's rows, one row at a time.
template <int R, typename VT, typename IT>
__device__ __forceinline__ void rows_acc_ref(const VT* __restrict__ val, const IT* __restrict__ ci,
                                             const int* __restrict__ rp, int tid, int nt, int n,
                                             const double* __restrict__ xv, double (&out)[R]) {
#pragma unroll
  for (int k = 0; k < R; ++k) {
    const int i = tid + k * nt;
    out[k] = 0.0;
    if (i < n) {
      const int beg = __ldg(rp + i);
      out[k] = row_ref<16>(val, ci, beg, __ldg(rp + i + 1) - beg, xv);
    }
  }
}

// PV: 0 none, 1 ISAI of L and U (z = aiU (aiL v)), 2 general ISAI (z = aiA v),
// 3 in-place ILU factors (a.prec: PK_ILU_INKERNEL factorises A here,
// PK_LU_GLOBAL reads a.F).
// FT: type of the ISAI values / factors and of the preconditioner arithmetic.
// column indices for the SpMVs: the plan's 16-bit copies (C16) or the int32 arrays
template <bool C16>
__device__ __forceinline__ auto pick_ci(const unsigned short* c16, const int* c32) {
  if constexpr (C16)
    return c16;
  else
    return c32;
}

// Solves system `sys` (result slot) with the CTA: P its pattern, L its
// shared-memory carve-up, Ag / bg / xg its values, right-hand side and
// solution.  Block-wide.
template <int R, int PV, typename FT, bool C16, bool REF>
__device__ __forceinline__ void rr_solve(const SolveArgs& a, const DevPattern& P, const RRLayout& L,
                                         unsigned char* smem, const int sys, const double* Ag, const double* bg,
                                         double* xg) {
  const int n = P.n, nt = blockDim.x, tid = threadIdx.x, nw = nt >> 5;
  // this thread's rows: rb + k * rs, k < R.  FAST: tid + k * nt.  REF: lane +
  // 32 (warp R + k), so that a warp's rows are a block of the reference's
  // lane-strided inner-product terms (ref_chain_sum)
  const int rb = REF ? (tid & 31) + 32 * R * (tid >> 5) : tid;
  const int rs = REF ? 32 : nt;
  const int* __restrict__ arp = P.a_rp;
  const auto* __restrict__ aci = pick_ci<C16>(P.a_ci16, P.a_ci);
  const auto* __restrict__ lci = pick_ci<C16>(P.ail_ci16, P.ail_ci);
  const auto* __restrict__ uci = pick_ci<C16>(P.aiu_ci16, P.aiu_ci);
  const auto* __restrict__ saci = pick_ci<C16>(P.sa_ci16, P.sa_ci);
  const auto* __restrict__ suci = pick_ci<C16>(P.su_ci16, P.su_ci);

  double* red = reinterpret_cast<double*>(smem + L.red);  // 2 partials per thread, then 16 broadcast scalars
  double* sph = reinterpret_cast<double*>(smem + L.ph);
  FT* sin = reinterpret_cast<FT*>(smem + L.in);
  FT* smid = reinterpret_cast<FT*>(smem + L.mid);

  const double* Am = Ag;
  if (L.A >= 0) {
    double* s = reinterpret_cast<double*>(smem + L.A);
    for (int k = tid; k < P.a_nnz; k += nt) s[k] = __ldg(Ag + k);
    Am = s;
  }
  // A in the SELL-32 layout when the caller converted it and it is not staged
  const double* Asell = (L.A < 0 && a.A_sell) ? a.A_sell + (size_t)sys * P.sa_nnz : nullptr;
  const FT* AIL = nullptr;
  const FT* AIU = nullptr;
  if (PV != 0) {
    const FT* g = reinterpret_cast<const FT*>(a.ail) + (size_t)sys * P.ail_nnz;
    if (L.ail >= 0) {
      FT* s = reinterpret_cast<FT*>(smem + L.ail);
      for (int k = tid; k < P.ail_nnz; k += nt) s[k] = g[k];
      AIL = s;
    } else {
      AIL = g;
    }
  }
  if (PV == 1) {
    const FT* g = reinterpret_cast<const FT*>(a.aiu) + (size_t)sys * P.aiu_nnz;
    if (L.aiu >= 0) {
      FT* s = reinterpret_cast<FT*>(smem + L.aiu);
      for (int k = tid; k < P.aiu_nnz; k += nt) s[k] = g[k];
      AIU = s;
    } else {
      AIU = g;
    }
  }
  const FT* AIUsell =
      (PV == 1 && L.aiu < 0 && a.aiu_sell) ? reinterpret_cast<const FT*>(a.aiu_sell) + (size_t)sys * P.su_nnz : nullptr;

  FT* Fs = nullptr;
  FT* rinv = nullptr;
  if (PV == 3) {
    Fs = reinterpret_cast<FT*>(smem + L.F);
    rinv = reinterpret_cast<FT*>(smem + L.rinv);
    const int nnz = P.nnz;
    if (a.prec == PK_ILU_INKERNEL) {
      // merged form: ILU(0) of A in FP64 in the factor slot (the factor
      // pattern is the operator pattern: no inserted diagonals)
      double* LUd = reinterpret_cast<double*>(smem + L.F);
      for (int k = tid; k < nnz; k += nt) LUd[k] = __ldg(Ag + k);
      __syncthreads();
      if (P.ilu_prog && P.ilu_prog_approach == a.approach)
        ilu_program_rows(P, LUd, a.approach, tid, nt);
      else
        ilu_rows(P, LUd, a.approach);
      if (sizeof(FT) == 4) {
        // round to float in place, in chunks of 8 values per thread: chunk c's
        // float writes end at byte 4 * (its last index + 1), before the first
        // double of any later chunk, and its own reads finish at the barrier
        constexpr int C = 8;
        for (int base = 0; base < nnz; base += C * nt) {
          double tv[C];
#pragma unroll
          for (int c = 0; c < C; ++c) {
            const int k = base + c * nt + tid;
            tv[c] = k < nnz ? LUd[k] : 0.0;
          }
          __syncthreads();
#pragma unroll
          for (int c = 0; c < C; ++c) {
            const int k = base + c * nt + tid;
            if (k < nnz) Fs[k] = (FT)tv[c];
          }
        }
      }
    } else {
      const FT* g = reinterpret_cast<const FT*>(a.F) + (size_t)sys * nnz;
      for (int k = tid; k < nnz; k += nt) Fs[k] = g[k];
    }
    __syncthreads();
    for (int i = tid; i < n; i += nt) {
      const double dgi = (double)Fs[__ldg(P.diag + i)];
      rinv[i] = (REF && sizeof(FT) == 8) ? (FT)dgi : (FT)(1.0 / dgi);  // REF FP64 divides by u_ii
    }
    // visible to the solves after the first reduction's barrier
  }

  // registers: x, r (s in the middle of an iteration), p, v, t; r_hat = b is
  // re-read from global memory (L1) and p_hat / s_hat from shared memory
  double x[R], r[R], p[R], v[R], t[R];
  double q[1] = {0.0};
#pragma unroll
  for (int k = 0; k < R; ++k) {
    const int i = rb + k * rs;
    const double bi = i < n ? __ldg(bg + i) : 0.0;
    x[k] = 0.0;
    p[k] = 0.0;
    v[k] = 0.0;
    t[k] = 0.0;
    r[k] = bi;
    if (i < n) q[0] = fma(bi, bi, q[0]);
  }
  // ||b||^2 = (r, r_hat) at the start: one reduction serves both (its barrier
  // also completes the staging above).  bc: the scalars warp 0 broadcasts.
  double* bc = red + 2 * nt;
  const bool lane0 = (tid & 31) == 0;
  // the CTA's sum of q (and of its second slot for K = 2): FAST, the block
  // reduction of the thread partials; REF, the reference's chain over the
  // rows, term(k, acc) per row
#define BILU_RR_SUM(K, qv, TERM) \
  (REF ? ref_chain_sum<K, R>(qv, TERM, red, nw) : block_sum_w0<K, PV != 3>(qv, red, nw))
  auto t_bb = [&](int k, double(&acc)[1]) {
    if (rb + k * rs < n) acc[0] = fma(r[k], r[k], acc[0]);
  };
  if (BILU_RR_SUM(1, q, t_bb) && lane0) {
    bc[0] = sqrt(q[0]);
    bc[1] = q[0];
  }
  __syncthreads();
  const double bnorm = bc[0];
  const double thr = (a.tol_mode == BILU_TOL_ABS) ? a.tol : a.tol * bnorm;
  double rho = bc[1], rho_old = 1.0, alpha = 1.0, omega_old = 1.0, res = bnorm;
  double beta = (rho / rho_old) * (alpha / omega_old);  // the first iteration's; warp 0 forms the later ones
  float iter = 0.0f;
  int status = BILU_SYS_MAX_ITER;
  bool stop = false;
  if (bnorm == 0.0) {
    res = 0.0;
    status = BILU_SYS_ZERO_RHS;
    stop = true;
  } else if (bnorm < thr) {
    status = BILU_SYS_INITIAL_OK;
    stop = true;
  }

// z = M in for this thread's rows.  The input is in `sin` (sph for PV 0 and
// for FP64 factors), made visible by a barrier; z lands in sph, followed by a
// barrier.
#define BILU_RR_APPLY()                                                                                          \
  do {                                                                                                           \
    if (PV == 1) {                                                                                               \
      FT z_[R];                                                                                                  \
      rows_acc<R>(AIL, lci, P.ail_rp, rb, rs, n, sin, z_);                                                 \
      _Pragma("unroll") for (int k = 0; k < R; ++k) {                                                            \
        const int i = rb + k * rs;                                                                              \
        if (i < n) smid[i] = z_[k];                                                                              \
      }                                                                                                          \
      __syncthreads();                                                                                           \
      if (AIUsell)                                                                                               \
        rows_acc_sell<R>(AIUsell, suci, P.su_off, P.aiu_rp, rb, rs, n, smid, z_);                            \
      else                                                                                                       \
        rows_acc<R>(AIU, uci, P.aiu_rp, rb, rs, n, smid, z_);                                              \
      _Pragma("unroll") for (int k = 0; k < R; ++k) {                                                            \
        const int i = rb + k * rs;                                                                              \
        if (i < n) sph[i] = widen_t(z_[k]);                                                                      \
      }                                                                                                          \
      __syncthreads();                                                                                           \
    } else if (PV == 2) {                                                                                        \
      FT z_[R];                                                                                                  \
      rows_acc<R>(AIL, lci, P.ail_rp, rb, rs, n, sin, z_);                                                 \
      _Pragma("unroll") for (int k = 0; k < R; ++k) {                                                            \
        const int i = rb + k * rs;                                                                              \
        if (i < n) sph[i] = widen_t(z_[k]);                                                                      \
      }                                                                                                          \
      __syncthreads();                                                                                           \
    } else if (PV == 3) {                                                                                        \
      lu_apply<FT, REF>(P, Fs, rinv, sizeof(FT) == 8 ? reinterpret_cast<FT*>(sph) : sin, sph, tid, nt);         \
    }                                                                                                            \
  } while (0)
// writes this thread's rows of `vec` as the preconditioner input
#define BILU_RR_INPUT(vec)                       \
  do {                                           \
    _Pragma("unroll") for (int k = 0; k < R; ++k) { \
      const int i = rb + k * rs;                \
      if (i < n) {                               \
        if (PV == 0 || (PV == 3 && sizeof(FT) == 8)) \
          sph[i] = vec[k];                       \
        else                                     \
          sin[i] = PV == 3 ? (FT)vec[k] : round_t<FT>(vec[k]); \
      }                                          \
    }                                            \
  } while (0)

  const float max_iter = (float)a.max_iter;
  while (!stop && iter < max_iter) {
    if (rho == 0.0) {
      status = BILU_SYS_BREAKDOWN_RHO;
      break;
    }
#pragma unroll
    for (int k = 0; k < R; ++k) p[k] = fma(beta, fma(-omega_old, v[k], p[k]), r[k]);
    BILU_RR_INPUT(p);
    __syncthreads();
    BILU_RR_APPLY();  // p_hat in sph
    // v = A p_hat, (r_hat, v)
    if (REF)
      rows_acc_ref<R>(Am, aci, arp, rb, rs, n, sph, v);
    else if (Asell)
      rows_acc_sell<R>(Asell, saci, P.sa_off, arp, rb, rs, n, sph, v);
    else
      rows_acc<R>(Am, aci, arp, rb, rs, n, sph, v);
    q[0] = 0.0;
    auto t_bv = [&](int k, double(&acc)[1]) {
      const int i = rb + k * rs;
      if (i < n) acc[0] = fma(__ldg(bg + i), v[k], acc[0]);
    };
    if (!REF) {
#pragma unroll
      for (int k = 0; k < R; ++k) t_bv(k, q);
    }
    if (BILU_RR_SUM(1, q, t_bv) && lane0) bc[2] = rho / q[0];
    __syncthreads();
    alpha = bc[2];
    // x += alpha p_hat, s = r - alpha v, ||s||.  p_hat is read before anyone
    // rewrites sph (PV 0 rewrites it with s right here, after the reduction's
    // barrier has ended every SpMV read).
    q[0] = 0.0;
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const int i = rb + k * rs;
      if (i < n) {
        x[k] = fma(alpha, sph[i], x[k]);
        r[k] = fma(-alpha, v[k], r[k]);
        if (!REF) q[0] = fma(r[k], r[k], q[0]);
      }
    }
    BILU_RR_INPUT(r);
    if (BILU_RR_SUM(1, q, t_bb) && lane0) bc[3] = sqrt(q[0]);
    __syncthreads();
    res = bc[3];
    iter = iter + 0.5f;
    if (res < thr) {
      status = BILU_SYS_CONVERGED;
      break;
    }
    BILU_RR_APPLY();  // s_hat in sph
    // t = A s_hat, (t, s), (t, t)
    if (REF)
      rows_acc_ref<R>(Am, aci, arp, rb, rs, n, sph, t);
    else if (Asell)
      rows_acc_sell<R>(Asell, saci, P.sa_off, arp, rb, rs, n, sph, t);
    else
      rows_acc<R>(Am, aci, arp, rb, rs, n, sph, t);
    double q2[2] = {0.0, 0.0};
    auto t_ts = [&](int k, double(&acc)[2]) {
      if (rb + k * rs < n) {
        acc[0] = fma(t[k], r[k], acc[0]);
        acc[1] = fma(t[k], t[k], acc[1]);
      }
    };
    if (!REF) {
#pragma unroll
      for (int k = 0; k < R; ++k) t_ts(k, q2);
    }
    if (BILU_RR_SUM(2, q2, t_ts) && lane0) bc[4] = q2[0] / q2[1];
    __syncthreads();
    const double omega = bc[4];
    // x += omega s_hat, r = s - omega t, ||r||, next rho = (r, r_hat)
    q2[0] = 0.0;
    q2[1] = 0.0;
    auto t_rr = [&](int k, double(&acc)[2]) {
      const int i = rb + k * rs;
      if (i < n) {
        acc[0] = fma(r[k], r[k], acc[0]);
        acc[1] = fma(__ldg(bg + i), r[k], acc[1]);
      }
    };
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const int i = rb + k * rs;
      if (i < n) {
        x[k] = fma(omega, sph[i], x[k]);
        r[k] = fma(-omega, t[k], r[k]);
      }
      if (!REF) t_rr(k, q2);
    }
    if (BILU_RR_SUM(2, q2, t_rr) && lane0) {
      bc[5] = sqrt(q2[0]);
      bc[6] = q2[1];
      bc[7] = (q2[1] / rho) * (alpha / omega);  // the next iteration's beta: (rho_new / rho_old) * (alpha / omega_old)
    }
    __syncthreads();
    res = bc[5];
    iter = iter + 0.5f;
    omega_old = omega;
    rho = bc[6];
    beta = bc[7];
    if (res < thr) {
      status = BILU_SYS_CONVERGED;
      break;
    }
  }
#undef BILU_RR_APPLY
#undef BILU_RR_SUM
#undef BILU_RR_INPUT

  // ---- write back
#pragma unroll
  for (int k = 0; k < R; ++k) {
    const int i = rb + k * rs;
    if (i < n) xg[i] = x[k];
  }
  if (tid == 0) {
    int st = status;
    if (st == BILU_SYS_MAX_ITER && !isfinite(res)) st = BILU_SYS_NONFINITE;
    const bool ok = (st == BILU_SYS_CONVERGED || st == BILU_SYS_ZERO_RHS || st == BILU_SYS_INITIAL_OK);
    if (a.iters) a.iters[sys] = iter;
    if (a.conv) a.conv[sys] = ok ? 1 : -1;
    if (a.res) a.res[sys] = res;
    if (a.status) a.status[sys] = st;
  }
  // ---- true residual ||b - A x||: x through shared memory, same reduction order
  if (a.true_res) {
    __syncthreads();  // every reader of sph is done
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const int i = rb + k * rs;
      if (i < n) sph[i] = x[k];
    }
    __syncthreads();
    double ax[R];
    if (REF) {
      // KernelFillTrueResNorms (Bicgstab_common.hpp:294-342): row_ref sums, then one serial
      // inner product over i = 0 .. n-1.  Warp w holds rows 32 (w R + k) + l: it passes each
      // row's residual to every lane in row order, every lane runs the same FMA chain, and the
      // chain moves on to the next warp through red
      rows_acc_ref<R>(Am, aci, arp, rb, rs, n, sph, ax);
      const int lane = tid & 31, warp = tid >> 5;
      double acc = 0.0;
      for (int w = 0; w < nw; ++w) {
        if (warp == w) {
          if (w > 0) acc = red[0];
#pragma unroll
          for (int k = 0; k < R; ++k) {
            const int i0 = rb + k * rs;
            const double ri = i0 < n ? __ldg(bg + i0) - ax[k] : 0.0;
            for (int l = 0; l < 32; ++l) {
              const double rl = __shfl_sync(kFull, ri, l);
              if (32 * (w * R + k) + l < n) acc = fma(rl, rl, acc);
            }
          }
          if (w + 1 < nw && lane == 0) red[0] = acc;
        }
        if (w + 1 < nw) __syncthreads();
      }
      if (warp == nw - 1 && lane == 0) a.true_res[sys] = sqrt(acc);
      return;
    }
    if (Asell)
      rows_acc_sell<R>(Asell, saci, P.sa_off, arp, rb, rs, n, sph, ax);
    else
      rows_acc<R>(Am, aci, arp, rb, rs, n, sph, ax);
    q[0] = 0.0;
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const int i = rb + k * rs;
      if (i < n) {
        const double ri = __ldg(bg + i) - ax[k];
        q[0] = fma(ri, ri, q[0]);
      }
    }
    if (block_sum_w0<1, PV != 3>(q, red, nw) && tid == 0) a.true_res[sys] = sqrt(q[0]);
  }
}

#define BILU_RR_BOUNDS __launch_bounds__(R <= 1 ? 1024 : (R == 2 ? 512 : (R == 4 ? 256 : 128)), R == 8 ? 3 : 1)

}  // namespace
}  // namespace bilu
