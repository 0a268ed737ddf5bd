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

// In-kernel ILU(0) from the plan's ILU program (DevPattern::ilu_*): the same
// operations in the same order as ilu_rows, with the row metadata of the next
// level loaded while the current level computes (ilu_rows chases level,
// row, row-pointer, dependency-pointer and pair loads one after another, each
// an L2 round trip once the solver's shared memory has squeezed L1).  Ops are
// decoded from registers by a small state machine; ops beyond the prefetched
// kIluPrefetch words are loaded when reached.  Block-wide; ends with a barrier.
struct IluOp {
  int st = 0, k = 0, np = 0, lower = 0, dpos = 0, px = 0;
  double v = 0.0, s = 0.0;
};

__device__ __forceinline__ void ilu_step(IluOp& o, int wd, double* LU, int approach) {
  if (o.st == 0) {  // entry header
    o.k = wd & 0xFFFFF;
    o.np = (wd >> 20) & 0x3FF;
    o.lower = (wd >> 30) & 1;
    o.v = LU[o.k];
    o.s = 0.0;
    o.st = o.lower ? 1 : 2;
    return;
  }
  if (o.st == 1) {  // diagonal position of a lower entry's column
    o.dpos = wd;
    o.st = 2;
  } else if (o.st == 2) {  // l position of a pair
    o.px = wd;
    o.st = 3;
    return;
  } else {  // u position of a pair
    if (approach == 1 || approach == 4)
      o.v = fma(-LU[o.px], LU[wd], o.v);
    else
      o.s = fma(LU[o.px], LU[wd], o.s);
    --o.np;
    o.st = 2;
  }
  if (o.np == 0) {  // entry complete
    double r = (approach == 1 || approach == 4) ? o.v : o.v - o.s;
    if (o.lower) r = r / LU[o.dpos];
    LU[o.k] = r;
    o.st = 0;
  }
}

__device__ __forceinline__ void ilu_slot(const int (&w)[kIluPrefetch + 1], const int* __restrict__ prog, int4 h, int s,
                                         double* LU, int approach) {
  IluOp o;
  const int cnt = w[0];
#pragma unroll
  for (int j = 1; j <= kIluPrefetch; ++j)
    if (j <= cnt) ilu_step(o, w[j], LU, approach);
  for (int j = kIluPrefetch + 1; j <= cnt; ++j) ilu_step(o, __ldg(prog + h.x + j * h.y + s), LU, approach);
}

__device__ __forceinline__ void ilu_fetch(const int* __restrict__ prog, int4 h, int s, int (&w)[kIluPrefetch + 1]) {
  if (s < h.y) {
#pragma unroll
    for (int j = 0; j <= kIluPrefetch; ++j) w[j] = __ldg(prog + h.x + j * h.y + s);
  } else {
    w[0] = 0;
  }
}

__device__ void ilu_program_rows(const DevPattern& P, double* LU, int approach, int tid, int nt) {
  const int4* __restrict__ hdr = P.ilu_hdr;
  const int* __restrict__ prog = P.ilu_prog;
  const int nlev = P.nlev_lo;
  const int4 zero = make_int4(0, 0, 0, 0);
  int4 h = nlev > 0 ? __ldg(hdr) : zero;
  int w[kIluPrefetch + 1];
  ilu_fetch(prog, h, tid, w);
  for (int lev = 0; lev < nlev; ++lev) {
    const int4 hn = lev + 1 < nlev ? __ldg(hdr + lev + 1) : zero;
    int wn[kIluPrefetch + 1];
    ilu_fetch(prog, hn, tid, wn);
    if (tid < h.y) ilu_slot(w, prog, h, tid, LU, approach);
    for (int s2 = tid + nt; s2 < h.y; s2 += nt) {
      int w2[kIluPrefetch + 1];
      ilu_fetch(prog, h, s2, w2);
      ilu_slot(w2, prog, h, s2, LU, approach);
    }
    __syncthreads();
    h = hn;
#pragma unroll
    for (int j = 0; j <= kIluPrefetch; ++j) w[j] = wn[j];
  }
}
