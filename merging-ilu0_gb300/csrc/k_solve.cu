// Fused batched BiCGSTAB: one CTA per system, every operand staged in shared
// memory where the plan's layout puts it; preconditioner generation (ILU(0)
// in-kernel for the merged form), SpMV, preconditioner application, inner
// products, convergence test and the true-residual epilogue in one launch.
//
// Reference behaviour followed (paths inside Batched-ILU0-merged/ILU0_ISAI_bicgstab/):
//   loop, exits, half iterations   PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu:324-533
//                                  PrecondBiCGSTAB_ilu_gpu.cu:218-433
//                                  PrecondBiCGSTAB_ilu_isai_gpu.cu:89-257
//   building blocks                Bicgstab_common.hpp:5-290
//   in-kernel ILU(0) (merged)      PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu:145-246
//   true residual                  Bicgstab_common.hpp:294-342
//
// GB300 mapping.  FP64 issue is the scarce resource on this part (about two
// FP64 lane-operations per clock per SM, and a warp instruction costs the same
// whatever its active mask), so the kernel is written to issue as few FP64
// warp instructions as possible: one thread per row everywhere (the
// reference's warp-per-row SpMV leaves 25-27 of 32 lanes idle), its
// shuffle-tree row sums reproduced per thread with the additions of known
// zeros skipped (exact), level-scheduled triangular solves instead of
// spin-waits, and the scalar recurrences on one lane.
//
// Reduction orders.  REF = true reproduces the reference's floating-point
// operation order exactly (bit-identical iterates); REF = false
// (BILU_REDUCE_FAST) sums rows sequentially and multiplies by the reciprocal
// of the diagonal instead of dividing.
#include <cuda_runtime.h>

#include "bilu_internal.h"

namespace bilu {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// --------------------------------------------------------------------------
// one row of A*x
// --------------------------------------------------------------------------
#include "k_row_ref.cuh"

template <typename VT>
__device__ __forceinline__ double row_seq(const VT* __restrict__ a, const int* __restrict__ ci, int beg, int end,
                                          const double* __restrict__ x) {
  double acc = 0.0;
  for (int k = beg; k < end; ++k) acc = fma((double)a[k], x[__ldg(ci + k)], acc);
  return acc;
}

template <bool REF, int S, typename VT>
__device__ __forceinline__ double row_dot(const VT* a, const int* ci, int beg, int end, const double* x) {
  if (REF) return row_ref<S>(a, ci, beg, end - beg, x);
  return row_seq(a, ci, beg, end, x);
}

// y = M x over the rows of one system, one thread per row
template <bool REF, int S, typename VT>
__device__ __forceinline__ void spmv(int n, const int* __restrict__ rp, const int* __restrict__ ci, const VT* a,
                                     const double* x, double* y) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) y[i] = row_dot<REF, S>(a, ci, __ldg(rp + i), __ldg(rp + i + 1), x);
}

// FP32 ISAI application: tmp = aiL * v, z = aiU * tmp, float fmas in CSR
// order (library definition for BILU_FP32; no reference counterpart).
__device__ __forceinline__ float row_f32(const float* __restrict__ a, const int* __restrict__ ci, int beg, int end,
                                         const float* __restrict__ x) {
  float acc = 0.0f;
  for (int k = beg; k < end; ++k) acc = fmaf(a[k], x[__ldg(ci + k)], acc);
  return acc;
}

// --------------------------------------------------------------------------
// inner products
// --------------------------------------------------------------------------
// inner_product(n, v1, v2, result) (Bicgstab_common.hpp:97-128): lane-strided
// fma partial sums in one warp, shfl_down tree; result valid on lane 0.
__device__ __forceinline__ double warp_dot(const double* a, const double* b, int n, int lane) {
  double acc = 0.0;
  for (int i = lane; i < n; i += 32) acc = fma(a[i], b[i], acc);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(kFull, acc, off);
  return acc;
}

// inner_product(n, v1, v2) (Bicgstab_common.hpp:82-95): one serial sum.
__device__ __forceinline__ double serial_dot(const double* a, const double* b, int n) {
  double acc = 0.0;
  for (int i = 0; i < n; ++i) acc = fma(a[i], b[i], acc);
  return acc;
}

// Returns the inner product on lane 0 of `owner_warp` (other threads: 0).
__device__ __forceinline__ double dot_on(int owner_warp, bool serial, const double* a, const double* b, int n) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double r = 0.0;
  if (warp == owner_warp) {
    if (serial) {
      if (lane == 0) r = serial_dot(a, b, n);
    } else {
      r = warp_dot(a, b, n, lane);
    }
  }
  return r;
}

// --------------------------------------------------------------------------
// triangular solves with in-place factors, level scheduled
// --------------------------------------------------------------------------
__device__ __forceinline__ void team_sync(int team_threads) {
  if (team_threads <= 32)
    __syncwarp();
  else
    asm volatile("bar.sync 1, %0;" ::"r"(team_threads) : "memory");
}

// out = U^{-1} L^{-1} in (FP64 factors), reference arithmetic
// (PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu:22-108): lower sums ascending,
// upper sums descending, then (y - sum) / u_ii.  `out` holds y and is
// overwritten in place by z.  Executed by the first `team` threads; the
// caller synchronises the block afterwards.
template <bool REF>
__device__ __forceinline__ void trsv_f64(const DevPattern& P, const double* F, const double* rinv, const double* in,
                                         double* out, int team) {
  const int tid = threadIdx.x;
  if (tid >= team) return;
  const int* __restrict__ rp = P.rp;
  const int* __restrict__ ci = P.ci;
  const int* __restrict__ dg = P.diag;
  for (int lev = 0; lev < P.nlev_lo; ++lev) {
    const int b = __ldg(P.lev_lo_ptr + lev), e = __ldg(P.lev_lo_ptr + lev + 1);
    for (int q = b + tid; q < e; q += team) {
      const int i = __ldg(P.lev_lo_rows + q);
      const int beg = __ldg(rp + i), d = __ldg(dg + i);
      double s = 0.0;
      for (int k = beg; k < d; ++k) s = fma(F[k], out[__ldg(ci + k)], s);
      out[i] = in[i] - s;
    }
    team_sync(team);
  }
  for (int lev = 0; lev < P.nlev_up; ++lev) {
    const int b = __ldg(P.lev_up_ptr + lev), e = __ldg(P.lev_up_ptr + lev + 1);
    for (int q = b + tid; q < e; q += team) {
      const int i = __ldg(P.lev_up_rows + q);
      const int end = __ldg(rp + i + 1), d = __ldg(dg + i);
      double s = 0.0;
      for (int k = end - 1; k > d; --k) s = fma(F[k], out[__ldg(ci + k)], s);
      const double y = out[i] - s;
      out[i] = REF ? y / F[d] : y * rinv[i];
    }
    team_sync(team);
  }
}

// FP32 factors applied in FP32 (library definition, mirrored by the oracle's
// trsv_lu_f32): fy = float scratch; result widened into out.  Caller syncs.
__device__ __forceinline__ void trsv_f32(const DevPattern& P, const float* F, const float* rinv, const double* in,
                                         float* fy, int team) {
  const int tid = threadIdx.x;
  if (tid >= team) return;
  const int* __restrict__ rp = P.rp;
  const int* __restrict__ ci = P.ci;
  const int* __restrict__ dg = P.diag;
  for (int lev = 0; lev < P.nlev_lo; ++lev) {
    const int b = __ldg(P.lev_lo_ptr + lev), e = __ldg(P.lev_lo_ptr + lev + 1);
    for (int q = b + tid; q < e; q += team) {
      const int i = __ldg(P.lev_lo_rows + q);
      const int beg = __ldg(rp + i), d = __ldg(dg + i);
      float s = 0.0f;
      for (int k = beg; k < d; ++k) s = fmaf(F[k], fy[__ldg(ci + k)], s);
      fy[i] = (float)in[i] - s;
    }
    team_sync(team);
  }
  for (int lev = 0; lev < P.nlev_up; ++lev) {
    const int b = __ldg(P.lev_up_ptr + lev), e = __ldg(P.lev_up_ptr + lev + 1);
    for (int q = b + tid; q < e; q += team) {
      const int i = __ldg(P.lev_up_rows + q);
      const int end = __ldg(rp + i + 1), d = __ldg(dg + i);
      float s = 0.0f;
      for (int k = end - 1; k > d; --k) s = fmaf(F[k], fy[__ldg(ci + k)], s);
      fy[i] = (fy[i] - s) * rinv[i];
    }
    team_sync(team);
  }
}

#include "k_ilu_rows.cuh"

// --------------------------------------------------------------------------
// the solver kernel
// --------------------------------------------------------------------------
struct Scal {
  double rho_new, rho_old, omega_old, omega, alpha, beta, res, thr, tt, bnorm;
  float iter;
  int stop;    // 1: leave the loop
  int status;  // BILU_SYS_*
};

// Solves system `sys` with the CTA: P = its pattern, lay = its shared-memory
// carve-up, Ag / bg / xg = its values, right-hand side and solution, Fg / Lg /
// Ug = its factors or ISAI values in global memory (when precomputed).
// Block-wide: every thread of the CTA must call it.
template <typename FT, bool REF, int S>
__device__ __forceinline__ void solve_one(const SolveArgs& a, const DevPattern& P, const SmemLayout& lay,
                                          unsigned char* smem, const int sys, const double* Ag, const double* bg,
                                          double* xg, const FT* Fg, const FT* Lg, const FT* Ug) {
  const int n = P.n, nnz = P.nnz, annz = P.a_nnz;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int* __restrict__ rp = P.a_rp;  // operator pattern
  const int* __restrict__ ci = P.a_ci;
  const bool serial = a.dot_serial != 0 && REF;
  constexpr bool kFP32 = sizeof(FT) == 4;

  // ---- shared-memory carve-up
  Scal* sc = reinterpret_cast<Scal*>(smem + lay.red);
  double* vec = reinterpret_cast<double*>(smem + lay.vec);
  double* x = vec;
  double* r = vec + n;  // r, overwritten by s each half step
  double* rh = vec + 2 * n;
  double* p = vec + 3 * n;
  double* v = vec + 4 * n;
  double* t = vec + 5 * n;
  double* ph = vec + 6 * n;  // p_hat, then s_hat
  double* tmpv = lay.tmpv >= 0 ? reinterpret_cast<double*>(smem + lay.tmpv) : nullptr;
  float* fy = lay.fvec >= 0 ? reinterpret_cast<float*>(smem + lay.fvec) : nullptr;

  const double* Am = Ag;
  if (lay.A >= 0) {
    double* As = reinterpret_cast<double*>(smem + lay.A);
    for (int k = tid; k < annz; k += nt) As[k] = __ldg(Ag + k);
    Am = As;
  }

  // ---- preconditioner generation / staging
  const FT* F = nullptr;
  const FT* AIL = nullptr;
  const FT* AIU = nullptr;
  void* rinv_raw = lay.rinv >= 0 ? (void*)(smem + lay.rinv) : nullptr;
  if (a.prec == PK_ILU_INKERNEL) {
    FT* Fs = reinterpret_cast<FT*>(smem + lay.F);
    double* LUd = kFP32 ? vec : reinterpret_cast<double*>(Fs);
    __syncthreads();  // A staged
    for (int k = tid; k < nnz; k += nt) LUd[k] = Am[k];
    __syncthreads();
    ilu_rows(P, LUd, a.approach);
    if (kFP32) {
      for (int k = tid; k < nnz; k += nt) Fs[k] = (FT)LUd[k];
      __syncthreads();
    }
    F = Fs;
  } else if (a.prec == PK_LU_GLOBAL) {
    if (lay.F >= 0) {
      FT* Fs = reinterpret_cast<FT*>(smem + lay.F);
      for (int k = tid; k < nnz; k += nt) Fs[k] = Fg[k];
      F = Fs;
    } else {
      F = Fg;
    }
  } else if (a.prec == PK_ISAI) {
    if (lay.ail >= 0) {
      FT* s = reinterpret_cast<FT*>(smem + lay.ail);
      for (int k = tid; k < P.ail_nnz; k += nt) s[k] = Lg[k];
      AIL = s;
    } else {
      AIL = Lg;
    }
    if (lay.aiu >= 0) {
      FT* s = reinterpret_cast<FT*>(smem + lay.aiu);
      for (int k = tid; k < P.aiu_nnz; k += nt) s[k] = Ug[k];
      AIU = s;
    } else {
      AIU = Ug;
    }
  }
  __syncthreads();
  const bool lu_prec = (a.prec == PK_ILU_INKERNEL || a.prec == PK_LU_GLOBAL);
  if (lu_prec && rinv_raw) {
    for (int i = tid; i < n; i += nt) {
      const double d = (double)F[__ldg(P.diag + i)];
      if (kFP32)
        reinterpret_cast<float*>(rinv_raw)[i] = (float)(1.0 / d);
      else
        reinterpret_cast<double*>(rinv_raw)[i] = 1.0 / d;
    }
  }
  // ---- initialization (Bicgstab_common.hpp:151-192): x = 0, r = b - A*0 = b, r_hat = r
  for (int i = tid; i < n; i += nt) {
    const double bi = __ldg(bg + i);
    x[i] = 0.0;
    p[i] = 0.0;
    v[i] = 0.0;
    r[i] = bi;
    rh[i] = bi;
  }
  __syncthreads();

  // Triangular-solve team: the first warps, enough for the widest level, never more than the CTA
  // (nt is a multiple of 32, so `team` is too and the named barrier count is valid).
  const int team = min(nt, (max(max(P.maxw_lo, P.maxw_up), 1) + 31) & ~31);
  // preconditioner application: out = M^{-1} in
  auto apply = [&](const double* in, double* out) {
    if (lu_prec) {
      if (kFP32) {
        trsv_f32(P, reinterpret_cast<const float*>(F), reinterpret_cast<const float*>(rinv_raw), in, fy, team);
        __syncthreads();
        for (int i = tid; i < n; i += nt) out[i] = (double)fy[i];
      } else {
        trsv_f64<REF>(P, reinterpret_cast<const double*>(F), reinterpret_cast<const double*>(rinv_raw), in, out,
                      team);
      }
    } else if (a.prec == PK_ISAI && P.aiu_nnz == 0) {  // general ISAI: z = aiA * v
      if (kFP32) {
        float* fin = fy;
        for (int i = tid; i < n; i += nt) fin[i] = (float)in[i];
        __syncthreads();
        const float* L = reinterpret_cast<const float*>(AIL);
        for (int i = tid; i < n; i += nt)
          out[i] = (double)row_f32(L, P.ail_ci, __ldg(P.ail_rp + i), __ldg(P.ail_rp + i + 1), fin);
      } else {
        spmv<REF, S>(n, P.ail_rp, P.ail_ci, reinterpret_cast<const double*>(AIL), in, out);
      }
    } else if (a.prec == PK_ISAI) {
      if (kFP32) {
        float* fin = fy;
        float* fmid = fy + n;
        for (int i = tid; i < n; i += nt) fin[i] = (float)in[i];
        __syncthreads();
        const float* L = reinterpret_cast<const float*>(AIL);
        for (int i = tid; i < n; i += nt) fmid[i] = row_f32(L, P.ail_ci, __ldg(P.ail_rp + i), __ldg(P.ail_rp + i + 1), fin);
        __syncthreads();
        const float* U = reinterpret_cast<const float*>(AIU);
        for (int i = tid; i < n; i += nt)
          out[i] = (double)row_f32(U, P.aiu_ci, __ldg(P.aiu_rp + i), __ldg(P.aiu_rp + i + 1), fmid);
      } else {
        spmv<REF, S>(n, P.ail_rp, P.ail_ci, reinterpret_cast<const double*>(AIL), in, tmpv);
        __syncthreads();
        spmv<REF, S>(n, P.aiu_rp, P.aiu_ci, reinterpret_cast<const double*>(AIU), tmpv, out);
      }
    } else {
      for (int i = tid; i < n; i += nt) out[i] = in[i];
    }
    __syncthreads();
  };

  // ---- norms: res_initial = ||r|| = ||b|| (r = b exactly)
  {
    const double d = dot_on(0, serial, r, r, n);
    if (tid == 0) {
      const double nb = sqrt(d);
      sc->bnorm = nb;
      sc->res = nb;
      sc->thr = (a.tol_mode == BILU_TOL_ABS) ? a.tol : a.tol * nb;
      sc->rho_old = sc->rho_new = sc->omega_old = sc->omega = sc->alpha = sc->beta = 1.0;
      sc->iter = 0.0f;
      sc->stop = 0;
      sc->status = BILU_SYS_MAX_ITER;
      if (nb == 0.0) {
        sc->res = 0.0;
        sc->status = BILU_SYS_ZERO_RHS;
        sc->stop = 1;
      } else if (nb < sc->thr) {
        sc->status = BILU_SYS_INITIAL_OK;
        sc->stop = 1;
      }
    }
    __syncthreads();
  }

  const float max_iter = (float)a.max_iter;
  while (!sc->stop && sc->iter < max_iter) {
    // rho = (r, r_hat); beta
    {
      const double d = dot_on(0, serial, r, rh, n);
      if (tid == 0) {
        sc->rho_new = d;
        if (d == 0.0) {
          sc->status = BILU_SYS_BREAKDOWN_RHO;
          sc->stop = 1;
        } else {
          sc->beta = (d / sc->rho_old) * (sc->alpha / sc->omega_old);
        }
      }
      __syncthreads();
      if (sc->stop) break;
    }
    {
      const double beta = sc->beta, om = sc->omega_old;
      for (int i = tid; i < n; i += nt) p[i] = fma(beta, fma(-om, v[i], p[i]), r[i]);
    }
    __syncthreads();
    apply(p, ph);
    spmv<REF, S>(n, rp, ci, Am, ph, v);
    __syncthreads();
    {
      const double d = dot_on(0, serial, rh, v, n);
      if (tid == 0) sc->alpha = sc->rho_new / d;
      __syncthreads();
    }
    {
      const double al = sc->alpha;
      for (int i = tid; i < n; i += nt) {
        x[i] = fma(al, ph[i], x[i]);  // = Update_x_middle, and the first half of Update_x
        r[i] = fma(-al, v[i], r[i]);  // s
      }
    }
    __syncthreads();
    {
      const double d = dot_on(0, serial, r, r, n);
      if (tid == 0) {
        const double res = sqrt(d);
        sc->res = res;
        sc->iter = sc->iter + 0.5f;
        if (res < sc->thr) {
          sc->status = BILU_SYS_CONVERGED;
          sc->stop = 1;
        }
      }
      __syncthreads();
      if (sc->stop) break;
    }
    apply(r, ph);  // s_hat
    spmv<REF, S>(n, rp, ci, Am, ph, t);
    __syncthreads();
    {
      const double ts = dot_on(0, serial, t, r, n);
      const double tt = dot_on(1 % ((nt + 31) >> 5), serial, t, t, n);
      if (tid == 32 || (nt <= 32 && tid == 0)) sc->tt = tt;
      __syncthreads();
      if (tid == 0) sc->omega = ts / sc->tt;
      __syncthreads();
    }
    {
      const double om = sc->omega;
      for (int i = tid; i < n; i += nt) {
        x[i] = fma(om, ph[i], x[i]);
        r[i] = fma(-om, t[i], r[i]);
      }
    }
    __syncthreads();
    {
      const double d = dot_on(0, serial, r, r, n);
      if (tid == 0) {
        const double res = sqrt(d);
        sc->res = res;
        sc->iter = sc->iter + 0.5f;
        sc->rho_old = sc->rho_new;
        sc->omega_old = sc->omega;
        if (res < sc->thr) {
          sc->status = BILU_SYS_CONVERGED;
          sc->stop = 1;
        }
      }
      __syncthreads();
    }
  }
  __syncthreads();

  // ---- write back
  for (int i = tid; i < n; i += nt) xg[i] = x[i];
  if (tid == 0) {
    int st = sc->status;
    if (st == BILU_SYS_MAX_ITER && !isfinite(sc->res)) st = BILU_SYS_NONFINITE;
    const bool ok = (st == BILU_SYS_CONVERGED || st == BILU_SYS_ZERO_RHS || st == BILU_SYS_INITIAL_OK);
    if (a.iters) a.iters[sys] = sc->iter;
    if (a.conv) a.conv[sys] = ok ? 1 : -1;
    if (a.res) a.res[sys] = sc->res;
    if (a.status) a.status[sys] = st;
  }
  // ---- true residual epilogue (KernelFillTrueResNorms, Bicgstab_common.hpp:294-342):
  // r = b - A x (row tree order), norm = sqrt(serial inner product).  r_hat still holds b.
  if (a.true_res) {
    for (int i = tid; i < n; i += nt) t[i] = rh[i] - row_dot<true, S>(Am, ci, __ldg(rp + i), __ldg(rp + i + 1), x);
    __syncthreads();
    const double d = dot_on(0, REF, t, t, n);
    if (tid == 0) a.true_res[sys] = sqrt(d);
  }
}

// One CTA per system of a batch sharing one pattern.
template <typename FT, bool REF, int S>
__global__ void __launch_bounds__(1024) k_bicgstab(const SolveArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int sys = blockIdx.x;
  if (sys >= a.nsys) return;
  const DevPattern& P = a.pat;
  solve_one<FT, REF, S>(a, P, a.lay, smem, sys, a.A + (size_t)sys * P.a_nnz, a.b + (size_t)sys * P.n,
                        a.x + (size_t)sys * P.n,
                        a.F ? reinterpret_cast<const FT*>(a.F) + (size_t)sys * P.nnz : nullptr,
                        a.ail ? reinterpret_cast<const FT*>(a.ail) + (size_t)sys * P.ail_nnz : nullptr,
                        a.aiu ? reinterpret_cast<const FT*>(a.aiu) + (size_t)sys * P.aiu_nnz : nullptr);
}

// Persistent CTAs over a work queue of systems with their own sizes and
// patterns (one size bucket, longest systems first).  A CTA takes the next
// queue position with one atomicAdd, solves that system with the merged
// in-kernel ILU(0) and takes the next, until the queue is empty; there is no
// waiting on other CTAs.
template <typename FT, bool REF, int S>
__global__ void __launch_bounds__(1024) k_bicgstab_uneven(const UnevenArgs u) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_job;
  constexpr bool kFP32 = sizeof(FT) == 4;
  for (;;) {
    if (threadIdx.x == 0) s_job = atomicAdd(u.counter, 1);
    __syncthreads();
    const int job = s_job;
    __syncthreads();
    if (job >= u.count) break;
    const int sys = __ldg(u.order + job);
    const SysDesc d = u.desc[sys];
    DevPattern P;
    P.n = d.n;
    P.nnz = P.a_nnz = d.nnz;
    P.a_maxl = d.maxl;
    P.rp = P.a_rp = u.meta + d.o_rp;
    P.ci = P.a_ci = u.meta + d.o_ci;
    P.diag = u.meta + d.o_diag;
    P.nlev_lo = d.nlev_lo;
    P.nlev_up = d.nlev_up;
    P.maxw_lo = P.maxw_up = d.maxw;
    P.lev_lo_ptr = u.meta + d.o_llp;
    P.lev_lo_rows = u.meta + d.o_llr;
    P.lev_up_ptr = u.meta + d.o_lup;
    P.lev_up_rows = u.meta + d.o_lur;
    P.dep_ptr = u.meta + d.o_dp;
    P.dep = reinterpret_cast<const int2*>(u.meta + d.o_dep);
    const SmemLayout lay = layout_for(d.n, d.nnz, d.nnz, u.base.prec, kFP32, !REF, 0, 0, u.smem_budget);
    solve_one<FT, REF, S>(u.base, P, lay, smem, sys, u.base.A + d.val_off, u.base.b + d.vec_off,
                          u.base.x + d.vec_off, nullptr, nullptr, nullptr);
    __syncthreads();
  }
}

template <typename FT, bool REF>
cudaError_t launch_t(const SolveArgs& a, int threads, int maxl, cudaStream_t st) {
  void (*kern)(const SolveArgs);
  if (maxl <= 8)
    kern = k_bicgstab<FT, REF, 8>;
  else if (maxl <= 16)
    kern = k_bicgstab<FT, REF, 16>;
  else
    kern = k_bicgstab<FT, REF, 32>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, a.lay.total);
  if (e != cudaSuccess) return e;
  kern<<<a.nsys, threads, a.lay.total, st>>>(a);
  return cudaGetLastError();
}

}  // namespace

template <typename FT, bool REF>
void* uneven_kernel_t(int maxl) {
  if (maxl <= 8) return (void*)k_bicgstab_uneven<FT, REF, 8>;
  if (maxl <= 16) return (void*)k_bicgstab_uneven<FT, REF, 16>;
  return (void*)k_bicgstab_uneven<FT, REF, 32>;
}

void* uneven_kernel(int fp32, int reduce_fast, int maxl) {
  if (fp32) return reduce_fast ? uneven_kernel_t<float, false>(maxl) : uneven_kernel_t<float, true>(maxl);
  return reduce_fast ? uneven_kernel_t<double, false>(maxl) : uneven_kernel_t<double, true>(maxl);
}

cudaError_t launch_uneven(const UnevenArgs& u, int threads, int grid, int fp32, int reduce_fast, int maxl,
                          cudaStream_t st) {
  if (u.count == 0 || grid == 0) return cudaSuccess;
  void* k = uneven_kernel(fp32, reduce_fast, maxl);
  void* args[] = {const_cast<UnevenArgs*>(&u)};
  return cudaLaunchKernel(k, dim3(grid), dim3(threads), args, (size_t)u.smem_budget, st);
}

cudaError_t launch_solve(const SolveArgs& a, int threads, int fp32, int reduce_fast, int maxl, cudaStream_t st) {
  if (a.nsys == 0) return cudaSuccess;
  if (fp32) return reduce_fast ? launch_t<float, false>(a, threads, maxl, st) : launch_t<float, true>(a, threads, maxl, st);
  return reduce_fast ? launch_t<double, false>(a, threads, maxl, st) : launch_t<double, true>(a, threads, maxl, st);
}

}  // namespace bilu

namespace bilu {
// Largest dynamic shared memory a CTA may opt into on the current device.
size_t solve_max_smem() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || v <= 0) {
    cudaGetLastError();
    return 232448;  // 227 KiB, the sm_100/sm_103 limit
  }
  return (size_t)v;
}
}  // namespace bilu
