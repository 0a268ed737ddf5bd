// Host side of the C ABI: pattern analysis (missing diagonals, diagonal
// pointers, L/U split, level schedules, factorisation dependency lists, ISAI
// patterns and per-row solve programs), the shared-memory layout of the
// solver kernel, and the entry points declared in include/bilu.h.
//
// Reference host code this replaces (paths inside Batched-ILU0-merged/ILU0_ISAI_bicgstab/):
//   factorization.cu:399-575   missing diagonals, diagonal pointers, L/U row pointers and fill
//   parILU_0_gpu.cu:118-220    create_dependency_graph_parilu (built once per plan here,
//                              not once per call after six device-to-host copies)
//   ILU_0_gpu.cu:693-756, 947-1053  dependency lists of approaches 3 and 4
//   isai_gpu.cu:40-179         pattern of |A|^power (sparse here, not a dense n^3 product)
//   *_gpu.cu helpers           Batched_*_Gpu_helper launch sequences
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "bilu.h"
#include "bilu_internal.h"

namespace bilu {

namespace {
thread_local std::string g_last_error;
}

bilu_status set_error(bilu_status code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

// Level schedules: a row of the unit-lower solve depends on its strictly-lower
// columns, a row of the upper solve on its strictly-upper columns; rows of one
// level are independent.  Rows within a level ascend.
void pattern_levels(int n, const int* rp, const int* ci, const int* diag, std::vector<int>& lo_ptr,
                    std::vector<int>& lo_rows, int& maxw_lo, std::vector<int>& up_ptr, std::vector<int>& up_rows,
                    int& maxw_up) {
  auto bucket = [&](const std::vector<int>& lv, int nlev, std::vector<int>& ptr, std::vector<int>& rows, int& maxw) {
    ptr.assign(nlev + 1, 0);
    for (int i = 0; i < n; ++i) ptr[lv[i] + 1]++;
    for (int l = 0; l < nlev; ++l) ptr[l + 1] += ptr[l];
    rows.assign(n, 0);
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (int i = 0; i < n; ++i) rows[fill[lv[i]]++] = i;
    maxw = 0;
    for (int l = 0; l < nlev; ++l) maxw = std::max(maxw, ptr[l + 1] - ptr[l]);
  };
  std::vector<int> lev(n, 0);
  int nl = 0;
  for (int i = 0; i < n; ++i) {
    int l = 0;
    for (int k = rp[i]; k < diag[i]; ++k) l = std::max(l, lev[ci[k]] + 1);
    lev[i] = l;
    nl = std::max(nl, l + 1);
  }
  bucket(lev, nl, lo_ptr, lo_rows, maxw_lo);
  std::vector<int> levu(n, 0);
  int nu = 0;
  for (int i = n - 1; i >= 0; --i) {
    int l = 0;
    for (int k = diag[i] + 1; k < rp[i + 1]; ++k) l = std::max(l, levu[ci[k]] + 1);
    levu[i] = l;
    nu = std::max(nu, l + 1);
  }
  bucket(levu, nu, up_ptr, up_rows, maxw_up);
}

// (l_ik, u_kj) position pairs per entry (i,j), k ascending, k < min(i, j)
// (the dependency lists of create_dependency_graph_parilu, parILU_0_gpu.cu:118-220,
// and of ILU approach 3, ILU_0_gpu.cu:693-756, without the written position).
void pattern_deps(int n, const int* rp, const int* ci, const int* diag, std::vector<int>& dep_ptr,
                  std::vector<int>& dep) {
  (void)diag;
  dep_ptr.assign(rp[n] + 1, 0);
  dep.clear();
  for (int i = 0; i < n; ++i)
    for (int e = rp[i]; e < rp[i + 1]; ++e) {
      const int j = ci[e];
      const int kmax = std::min(i, j);
      for (int lk = rp[i]; lk < rp[i + 1] && ci[lk] < kmax; ++lk) {
        const int k = ci[lk];
        const int* b = ci + rp[k];
        const int* en = ci + rp[k + 1];
        const int* it = std::lower_bound(b, en, j);
        if (it != en && *it == j) {
          dep.push_back(lk);
          dep.push_back((int)(it - ci));
        }
      }
      dep_ptr[e + 1] = (int)(dep.size() / 2);
    }
}

void build_trsv_program(const int* rp, const int* ci, const int* diag, const std::vector<int>& lptr,
                        const std::vector<int>& lrows, bool upper, std::vector<int>& hdr, std::vector<int>& prog) {
  hdr.clear();
  prog.clear();
  for (int l = 0; l + 1 < (int)lptr.size(); ++l) {
    const int w = lptr[l + 1] - lptr[l];
    int maxc = 0;
    for (int q = lptr[l]; q < lptr[l + 1]; ++q) {
      const int i = lrows[q];
      maxc = std::max(maxc, upper ? rp[i + 1] - 1 - diag[i] : diag[i] - rp[i]);
    }
    const int rows_e = std::max(maxc, kTrsvPrefetch);
    const int off = (int)prog.size();
    hdr.push_back(off);
    hdr.push_back(w);
    prog.resize(off + (size_t)w * (1 + rows_e), 0);
    for (int s = 0; s < w; ++s) {
      const int i = lrows[lptr[l] + s];
      int j = 0;
      if (upper) {
        for (int k = rp[i + 1] - 1; k > diag[i]; --k, ++j) prog[off + w + (size_t)j * w + s] = k << 10 | ci[k];
      } else {
        for (int k = rp[i]; k < diag[i]; ++k, ++j) prog[off + w + (size_t)j * w + s] = k << 10 | ci[k];
      }
      prog[off + s] = i | j << 10;
    }
  }
}

void build_ilu_program(const int* rp, const int* ci, const int* diag, const std::vector<int>& lptr,
                       const std::vector<int>& lrows, const std::vector<int>& dep_ptr, const std::vector<int>& dep,
                       int approach, std::vector<int>& hdr, std::vector<int>& prog) {
  hdr.clear();
  prog.clear();
  std::vector<std::vector<int>> slot;
  for (int l = 0; l + 1 < (int)lptr.size(); ++l) {
    const int w = lptr[l + 1] - lptr[l];
    slot.assign(w, {});
    int len = kIluPrefetch + 1;
    for (int s = 0; s < w; ++s) {
      const int i = lrows[lptr[l] + s];
      std::vector<int>& ops = slot[s];
      ops.push_back(0);
      for (int k = rp[i]; k < rp[i + 1]; ++k) {
        const int j = ci[k], pb = dep_ptr[k], pe = dep_ptr[k + 1], np = pe - pb;
        const bool lower = j < i;
        if (!lower && np == 0) continue;  // a = a: an exact no-op in every approach
        ops.push_back(k | np << 20 | (lower ? 1 : 0) << 30);
        if (lower) ops.push_back(diag[j]);
        for (int q = 0; q < np; ++q) {
          const int qq = approach == 2 ? pe - 1 - q : pb + q;  // approach 2 sums the pairs descending
          ops.push_back(dep[2 * qq]);
          ops.push_back(dep[2 * qq + 1]);
        }
      }
      ops[0] = (int)ops.size() - 1;
      len = std::max(len, (int)ops.size());
    }
    const int off = (int)prog.size();
    hdr.insert(hdr.end(), {off, w, len, 0});
    prog.resize(off + (size_t)w * len, 0);
    for (int s = 0; s < w; ++s)
      for (int j = 0; j < (int)slot[s].size(); ++j) prog[off + (size_t)j * w + s] = slot[s][j];
  }
}

}  // namespace bilu

using namespace bilu;

// struct bilu_plan is defined in bilu_internal.h

namespace plan_detail {

bool is_fp32(const bilu_options& o) { return o.factor_precision == BILU_FP32; }
bool is_isai(int p) {
  return p == BILU_PRECOND_ILU0_ISAI || p == BILU_PRECOND_PARILU0_ISAI || p == BILU_PRECOND_GENERAL_ISAI;
}

int round_up(int v, int m) { return (v + m - 1) / m * m; }

bilu_status cuda_err(cudaError_t e, const char* what) {
  return set_error(BILU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// position of column c in row r of (rp, ci), or -1
int find_pos(const std::vector<int>& rp, const std::vector<int>& ci, int r, int c) {
  auto b = ci.begin() + rp[r], e = ci.begin() + rp[r + 1];
  auto it = std::lower_bound(b, e, c);
  if (it != e && *it == c) return (int)(it - ci.begin());
  return -1;
}

void build_levels(bilu_plan& P) {
  bilu::pattern_levels(P.n, P.rp.data(), P.ci.data(), P.diag.data(), P.lev_lo_ptr, P.lev_lo_rows, P.maxw_lo,
                       P.lev_up_ptr, P.lev_up_rows, P.maxw_up);
}

// Triangular-solve programs (DevPattern::tp_*) from the level schedules; only
// for n <= 1024 (10-bit rows and columns), the register-resident solver's range.
void build_trsv_programs(bilu_plan& P) {
  P.tp_lo_hdr.clear();
  P.tp_lo.clear();
  P.tp_up_hdr.clear();
  P.tp_up.clear();
  if (P.n > 1024) return;
  bilu::build_trsv_program(P.rp.data(), P.ci.data(), P.diag.data(), P.lev_lo_ptr, P.lev_lo_rows, false, P.tp_lo_hdr,
                           P.tp_lo);
  bilu::build_trsv_program(P.rp.data(), P.ci.data(), P.diag.data(), P.lev_up_ptr, P.lev_up_rows, true, P.tp_up_hdr,
                           P.tp_up);
}

// SELL-32 layout of a pattern with n <= 1024 rows (DevPattern::sa_* / su_*).
void build_sell(int n, const std::vector<int>& rp, const std::vector<int>& ci, std::vector<int>& off,
                std::vector<int>& sci, std::vector<int>& src) {
  off.clear();
  sci.clear();
  src.clear();
  if (n > 1024 || rp.empty()) return;
  const int ns = (n + 31) / 32;
  off.assign(ns + 1, 0);
  for (int s = 0; s < ns; ++s) {
    int w = 0;
    for (int i = 32 * s; i < std::min(n, 32 * s + 32); ++i) w = std::max(w, rp[i + 1] - rp[i]);
    off[s + 1] = off[s] + 32 * w;
  }
  sci.assign(off[ns], 0);
  src.assign(off[ns], -1);
  for (int i = 0; i < n; ++i) {
    const int base = off[i / 32] + (i % 32);
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      sci[base + 32 * (k - rp[i])] = ci[k];
      src[base + 32 * (k - rp[i])] = k;
    }
  }
}

void build_deps(bilu_plan& P) {
  bilu::pattern_deps(P.n, P.rp.data(), P.ci.data(), P.diag.data(), P.dep_ptr, P.dep);
  P.ilu_hdr.clear();
  P.ilu_prog.clear();
  // the merged form's in-kernel ILU(0) in the register-resident solver (n <= 1024, 20-bit positions)
  if (P.n <= 1024 && P.nnz < (1 << 20) && P.opts.precond == BILU_PRECOND_ILU0)
    bilu::build_ilu_program(P.rp.data(), P.ci.data(), P.diag.data(), P.lev_lo_ptr, P.lev_lo_rows, P.dep_ptr, P.dep,
                            P.opts.ilu_approach, P.ilu_hdr, P.ilu_prog);
}

// structural pattern of T^power, T given by (trp, tci)
void pattern_power(int n, const std::vector<int>& trp, const std::vector<int>& tci, int power, std::vector<int>& orp,
                   std::vector<int>& oci) {
  std::vector<int> crp = trp, cci = tci;
  std::vector<char> mark(n, 0);
  std::vector<int> row;
  for (int p = 2; p <= power; ++p) {
    std::vector<int> nrp(n + 1, 0), nci;
    // (T * C)(r, :) = union over k in T(r, :) of C(k, :)
    for (int r = 0; r < n; ++r) {
      row.clear();
      for (int a = trp[r]; a < trp[r + 1]; ++a) {
        const int k = tci[a];
        for (int b = crp[k]; b < crp[k + 1]; ++b) {
          const int c = cci[b];
          if (!mark[c]) {
            mark[c] = 1;
            row.push_back(c);
          }
        }
      }
      std::sort(row.begin(), row.end());
      for (int c : row) mark[c] = 0;
      nci.insert(nci.end(), row.begin(), row.end());
      nrp[r + 1] = (int)nci.size();
    }
    crp.swap(nrp);
    cci.swap(nci);
  }
  orp.swap(crp);
  oci.swap(cci);
}

// general ISAI of A: pattern of |A|^power, per-row position maps of A(J,J)
bilu_status build_isai_general(bilu_plan& P) {
  const int n = P.n;
  const int power = std::max(1, P.opts.isai_power);
  pattern_power(n, P.rp, P.ci, power, P.ail_rp, P.ail_ci);
  P.aiu_rp.assign(n + 1, 0);
  P.aiu_ci.clear();
  P.ail_prog_ptr.assign(n + 1, 0);
  P.aiu_prog_ptr.assign(n + 1, 0);
  P.gen_map_ptr.assign(n + 1, 0);
  P.gen_map.clear();
  P.gen_pos.assign(n, 0);
  for (int i = 0; i < n; ++i) {
    const int beg = P.ail_rp[i], sz = P.ail_rp[i + 1] - beg;
    if (sz > 32)
      return set_error(BILU_ERR_CAPACITY, "general ISAI row " + std::to_string(i) + " has " + std::to_string(sz) +
                                              " entries (limit 32, isai_gpu.cu:223)");
    const int* J = P.ail_ci.data() + beg;
    for (int t = 0; t < sz; ++t)
      if (J[t] == i) P.gen_pos[i] = t;
    for (int k = 0; k < sz; ++k)
      for (int t = 0; t < sz; ++t) P.gen_map.push_back(find_pos(P.rp, P.ci, J[k], J[t]));
    P.gen_map_ptr[i + 1] = (int)P.gen_map.size();
  }
  return BILU_OK;
}

// Per-row ISAI programs, one 32-bit word per step: a header t | count << 5
// (the unknown solved next and how many products it takes), then per product
// c | pos << 5 (the unknown it reads and the factor entry's position).  Rows
// have at most 32 entries, so t, count and c take 5 bits; pos needs nnz < 2^26.
bilu_status build_isai(bilu_plan& P) {
  if (P.general_isai) return build_isai_general(P);
  const int n = P.n;
  if (P.nnz >= (1 << 26))
    return set_error(BILU_ERR_CAPACITY, "ISAI: factor patterns of 2^26 or more entries are not supported");
  const int power = std::max(1, P.opts.isai_power);
  pattern_power(n, P.l_rp, P.l_ci, power, P.ail_rp, P.ail_ci);
  pattern_power(n, P.u_rp, P.u_ci, power, P.aiu_rp, P.aiu_ci);
  // lower programs
  P.ail_prog_ptr.assign(n + 1, 0);
  P.ail_prog.clear();
  for (int i = 0; i < n; ++i) {
    const int beg = P.ail_rp[i], sz = P.ail_rp[i + 1] - beg;
    if (sz > 32)
      return set_error(BILU_ERR_CAPACITY, "ISAI row " + std::to_string(i) + " of aiL has " + std::to_string(sz) +
                                              " entries (limit 32, isai_gpu.cu:223)");
    if (sz < 1 || P.ail_ci[beg + sz - 1] != i) return set_error(BILU_ERR_PATTERN, "ISAI(L) row without its diagonal");
    for (int t = sz - 2; t >= 0; --t) {
      const size_t hdr = P.ail_prog.size();
      P.ail_prog.push_back(t);
      int cnt = 0;
      for (int c = sz - 1; c > t; --c) {
        const int pos = find_pos(P.rp, P.ci, P.ail_ci[beg + c], P.ail_ci[beg + t]);
        if (pos >= 0) {
          P.ail_prog.push_back(c | pos << 5);
          ++cnt;
        }
      }
      P.ail_prog[hdr] = t | cnt << 5;
    }
    P.ail_prog_ptr[i + 1] = (int)P.ail_prog.size();
  }
  P.aiu_prog_ptr.assign(n + 1, 0);
  P.aiu_prog.clear();
  for (int i = 0; i < n; ++i) {
    const int beg = P.aiu_rp[i], sz = P.aiu_rp[i + 1] - beg;
    if (sz > 32)
      return set_error(BILU_ERR_CAPACITY, "ISAI row " + std::to_string(i) + " of aiU has " + std::to_string(sz) +
                                              " entries (limit 32, isai_gpu.cu:223)");
    if (sz < 1 || P.aiu_ci[beg] != i) return set_error(BILU_ERR_PATTERN, "ISAI(U) row without its diagonal");
    for (int t = 1; t < sz; ++t) {
      const size_t hdr = P.aiu_prog.size();
      P.aiu_prog.push_back(t);
      int cnt = 0;
      for (int c = 0; c < t; ++c) {
        const int pos = find_pos(P.rp, P.ci, P.aiu_ci[beg + c], P.aiu_ci[beg + t]);
        if (pos >= 0) {
          P.aiu_prog.push_back(c | pos << 5);
          ++cnt;
        }
      }
      P.aiu_prog[hdr] = t | cnt << 5;
    }
    P.aiu_prog_ptr[i + 1] = (int)P.aiu_prog.size();
  }
  return BILU_OK;
}

// Shared-memory layout of the solver kernel and its CTA size.
int prec_kind(int precond) {
  switch (precond) {
    case BILU_PRECOND_ILU0: return PK_ILU_INKERNEL;
    case BILU_PRECOND_ILU0_SPLIT:
    case BILU_PRECOND_PARILU0: return PK_LU_GLOBAL;
    case BILU_PRECOND_ILU0_ISAI:
    case BILU_PRECOND_PARILU0_ISAI:
    case BILU_PRECOND_GENERAL_ISAI: return PK_ISAI;
    default: return PK_NONE;
  }
}

void choose_layout(bilu_plan& P) {
  const bilu_options& o = P.opts;
  const int n = P.n;
  P.lay = layout_for(n, P.nnz_in, P.nnz, prec_kind(o.precond), is_fp32(o), o.reduction == BILU_REDUCE_FAST,
                     P.has_isai ? P.ail_rp[n] : 0, P.has_isai ? P.aiu_rp[n] : 0, (int)solve_max_smem());
  int th = o.threads_per_system > 0 ? o.threads_per_system : round_up(std::max(n, 64), 32);
  th = std::min(round_up(std::max(th, 32), 32), 1024);
  P.threads = th;
}

// Register-resident FAST solver: FAST order, any preconditioner kind, at most
// 8 rows per thread.  rr_configure sets the plan up for `nt` threads per system
// and the shared-memory staging `mask` (bit 0 A, bit 1 aiL / aiA, bit 2 aiU;
// operands that would cost occupancy are left in global memory, read through
// L1; ILU factors are always staged; bit 3: the SpMVs read SELL-32 copies of
// the operands left in global memory; bit 4: the occupancy variant of the
// kernel (k_bicgstab_rr_occ: 8 rows per thread on 4 CTAs of 128 threads, 4 rows
// on 4 CTAs of 256 (3 with ILU factors), 2 rows on 2 CTAs of 512; ignored for
// ILU factors at 8 rows per thread); false when the kernel does not apply or
// that configuration is invalid.
bool rr_configure(bilu_plan& P, int nt, int mask) {
  const bilu_options& o = P.opts;
  const int pk = prec_kind(o.precond);
  const bool ref = o.reduction != BILU_REDUCE_FAST;
  const int n = P.n;
  nt = std::max(round_up(nt, 32), 32);
  const int R = rr_rows_per_thread(n, nt);
  if (R == 0 || nt > rr_max_threads(R)) return false;
  const bool lu = (pk == PK_ILU_INKERNEL || pk == PK_LU_GLOBAL);
  const int pv = pk == PK_NONE ? 0 : (lu ? 3 : (P.general_isai ? 2 : 1));
  // Reference order: the inner products chain through the warps as the
  // reference's warp-0 sums; ILU factors or none (the ISAI solvers' serial
  // inner products stay on the shared-memory kernel), rows of at most 16
  // entries (row_ref<16>), no SELL-32 copies, no 4-CTA variant.
  if (ref) {
    if ((pv != 0 && pv != 3) || P.a_maxl > 16) return false;
    mask &= 7;
  }
  // bit 4: the occupancy variant, for 2, 4 or 8 rows per thread (ILU factors: 2 or 4) and at most its
  // launch bound of threads
  const int occ_nt = R == 8 ? 128 : (R == 4 ? 256 : 512);
  const bool occ_variant = (mask & 16) != 0 && (R == 2 || R == 4 || (R == 8 && pv != 3)) && nt <= occ_nt;
  const bool fp32 = is_fp32(o);
  const int fts = fp32 ? 4 : 8;
  if (pv == 3 && P.tp_lo.empty()) return false;
  // the merged form factorises in FP64 in the factor slot before rounding to FT
  RRLayout L = rr_layout_base(n, P.nnz, pv, fp32, pk == PK_ILU_INKERNEL, nt);
  int off = L.total;
  auto take = [&](int& dst, long long bytes) {
    dst = off;
    off = (int)((off + bytes + 15) & ~15LL);
  };
  int dev = 0, per_sm = 0, reserved = 0, optin = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const void* k = rr_kernel(pv, fp32 ? 1 : 0, R, ref ? 1 : 0, occ_variant ? 1 : 0);
  if (!k) return false;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, std::max(optin, off)) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, nt, off) != cudaSuccess || occ < 1) {
    cudaGetLastError();
    return false;
  }
  const int budget = std::min(optin, per_sm / occ - reserved);
  if (off > budget) return false;
  auto stage = [&](int& dst, long long bytes, int bit) {
    if ((mask & bit) && bytes > 0 && off + bytes <= budget) take(dst, bytes);
  };
  stage(L.A, (long long)P.nnz_in * 8, 1);
  if (pv == 1 || pv == 2) stage(L.ail, (long long)P.ail_rp[n] * fts, 2);
  if (pv == 1) stage(L.aiu, (long long)P.aiu_rp[n] * fts, 4);
  L.total = off;
  P.rr = true;
  P.rr_threads = nt;
  P.rr_pv = pv;
  P.rr_lay = L;
  P.rr_sell = (mask & 8) != 0 && !P.sa_off.empty();
  P.rr_occ = occ_variant;
  return true;
}

// Default: the caller's threads per system, else the fewest warps that give
// every thread at most 8 rows (one warp for n <= 256); the caller's staging
// mask, else the ISAI values but not A; SELL-32 copies for ILU factors at
// n > 512.  Measured on GB300 (3D 7-point 10x10x10, 7x7x7, 2D 16x16): A read
// through L1 beats A in shared memory, whose carve-out shrinks the L1 left for
// the column indices and ISAI values; the FP32 aiL in shared memory helps when
// it fits; the SELL-32 copy of A gains 5 % with ILU factors at 10x10x10
// (128 threads) and loses up to 6 % on the smaller systems and with ISAI.
void choose_rr(bilu_plan& P) {
  const bilu_options& o = P.opts;
  P.rr = false;
  int nt = o.threads_per_system > 0 ? o.threads_per_system : round_up((P.n + 7) / 8, 32);
  const bool lu = prec_kind(o.precond) == PK_ILU_INKERNEL || prec_kind(o.precond) == PK_LU_GLOBAL;
  rr_configure(P, nt, o.smem_staging >= 0 ? o.smem_staging : (6 | (lu && P.n > 512 ? 8 : 0)));
}

bilu_status upload(bilu_plan& P) {
  std::vector<int> buf;
  auto put = [&](const std::vector<int>& v) {
    while (buf.size() % 4) buf.push_back(0);  // 16-byte alignment
    const size_t o = buf.size();
    buf.insert(buf.end(), v.begin(), v.end());
    if (v.empty()) buf.push_back(0);
    return o;
  };
  const size_t o_in_rp = put(P.in_rp), o_in_ci = put(P.in_ci);
  const size_t o_rp = put(P.rp), o_ci = put(P.ci), o_diag = put(P.diag), o_row = put(P.row_of), o_src = put(P.src);
  const size_t o_llp = put(P.lev_lo_ptr), o_llr = put(P.lev_lo_rows), o_lup = put(P.lev_up_ptr),
               o_lur = put(P.lev_up_rows);
  const size_t o_dp = put(P.dep_ptr), o_dep = put(P.dep);
  const size_t o_lsrc = put(P.l_src), o_usrc = put(P.u_src);
  const size_t o_rlev = put(P.row_lev), o_tpos = put(P.tpos), o_ment = put(P.mlp_ent);
  const size_t o_plent = put(P.pl_ent);
  const size_t o_plpp = put(P.pl_prog_ptr), o_plp = put(P.pl_prog);
  const size_t o_tlh = put(P.tp_lo_hdr), o_tl = put(P.tp_lo), o_tuh = put(P.tp_up_hdr), o_tu = put(P.tp_up);
  const size_t o_sao = put(P.sa_off), o_sac = put(P.sa_ci), o_sas = put(P.sa_src);
  const size_t o_ih = put(P.ilu_hdr), o_ip = put(P.ilu_prog);
  // 16-bit column indices, two per int
  auto put16 = [&](const std::vector<int>& v) {
    std::vector<int> packed((v.size() + 1) / 2, 0);
    for (size_t q = 0; q < v.size(); ++q) {
      const unsigned int u = (unsigned int)v[q] & 0xFFFFu;
      packed[q / 2] |= (int)(u << (16 * (q % 2)));
    }
    return put(packed);
  };
  const bool ci16 = P.n <= 65535;
  const size_t o_a16 = ci16 ? put16(P.in_ci) : 0, o_sa16 = ci16 ? put16(P.sa_ci) : 0;
  size_t o_l16 = 0, o_u16 = 0, o_su16 = 0;
  if (ci16 && P.has_isai) {
    o_l16 = put16(P.ail_ci);
    o_u16 = put16(P.aiu_ci);
    o_su16 = put16(P.su_ci);
  }
  const size_t o_suo = put(P.su_off), o_suc = put(P.su_ci), o_sus = put(P.su_src);
  size_t o_alrp = 0, o_alci = 0, o_aurp = 0, o_auci = 0, o_alpp = 0, o_alp = 0, o_aupp = 0, o_aup = 0;
  size_t o_alperm = 0, o_auperm = 0;
  size_t o_gmp = 0, o_gm = 0, o_gp = 0;
  if (P.general_isai) {
    o_gmp = put(P.gen_map_ptr);
    o_gm = put(P.gen_map);
    o_gp = put(P.gen_pos);
  }
  if (P.has_isai) {
    o_alrp = put(P.ail_rp);
    o_alci = put(P.ail_ci);
    o_aurp = put(P.aiu_rp);
    o_auci = put(P.aiu_ci);
    // device layout of the per-row ISAI programs: rows in blocks of 32 (a warp's rows), word j of
    // row 32b+l at off[b] + 32j + l, so a warp's program loads are contiguous lines
    // rows are taken in slot order perm (longest program first), so slot s = 32b+l runs row perm[s]
    auto blocked = [&](const std::vector<int>& ptr, const std::vector<int>& prog, std::vector<int>& perm,
                       std::vector<int>& off, std::vector<int>& words) {
      perm.resize(P.n);
      for (int i = 0; i < P.n; ++i) perm[i] = i;
      std::stable_sort(perm.begin(), perm.end(),
                       [&](int a, int b) { return ptr[a + 1] - ptr[a] > ptr[b + 1] - ptr[b]; });
      const int nb = (P.n + 31) / 32;
      off.assign(nb + 1, 0);
      for (int bk = 0; bk < nb; ++bk) {
        int len = 0;
        for (int sl = 32 * bk; sl < std::min(P.n, 32 * bk + 32); ++sl)
          len = std::max(len, ptr[perm[sl] + 1] - ptr[perm[sl]]);
        off[bk + 1] = off[bk] + 32 * len;
      }
      words.assign((size_t)off[nb], 0);
      for (int sl = 0; sl < P.n; ++sl) {
        const int i = perm[sl];
        for (int j = 0; j < ptr[i + 1] - ptr[i]; ++j) words[(size_t)off[sl / 32] + 32 * j + sl % 32] = prog[ptr[i] + j];
      }
    };
    std::vector<int> off, words;
    blocked(P.ail_prog_ptr, P.ail_prog, P.ail_perm, off, words);
    o_alpp = put(off);
    o_alp = put(words);
    o_alperm = put(P.ail_perm);
    blocked(P.aiu_prog_ptr, P.aiu_prog, P.aiu_perm, off, words);
    o_aupp = put(off);
    o_aup = put(words);
    o_auperm = put(P.aiu_perm);
  }
  cudaError_t e = cudaMalloc((void**)&P.dbuf, buf.size() * sizeof(int));
  if (e != cudaSuccess) return set_error(BILU_ERR_ALLOC, std::string("plan upload: ") + cudaGetErrorString(e));
  e = cudaMemcpy(P.dbuf, buf.data(), buf.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_err(e, "plan upload");
  DevPattern& d = P.dp;
  const int* b = P.dbuf;
  d.n = P.n;
  d.nnz = P.nnz;
  d.a_nnz = P.nnz_in;
  d.a_rp = b + o_in_rp;
  d.a_ci = b + o_in_ci;
  d.a_maxl = P.a_maxl;
  d.rp = b + o_rp;
  d.ci = b + o_ci;
  d.diag = b + o_diag;
  d.row_of = b + o_row;
  d.nlev_lo = (int)P.lev_lo_ptr.size() - 1;
  d.nlev_up = (int)P.lev_up_ptr.size() - 1;
  d.maxw_lo = P.maxw_lo;
  d.maxw_up = P.maxw_up;
  d.lev_lo_ptr = b + o_llp;
  d.lev_lo_rows = b + o_llr;
  d.lev_up_ptr = b + o_lup;
  d.lev_up_rows = b + o_lur;
  d.dep_ptr = b + o_dp;
  d.dep = reinterpret_cast<const int2*>(b + o_dep);
  d.nnz_in = P.nnz_in;
  d.src_map = b + o_src;
  d.nnz_L = (int)P.l_src.size();
  d.nnz_U = (int)P.u_src.size();
  d.l_src = b + o_lsrc;
  d.u_src = b + o_usrc;
  d.row_lev = b + o_rlev;
  d.tpos = b + o_tpos;
  d.n_mlp = (int)P.mlp_ent.size();
  d.mlp_ent = b + o_ment;
  d.pl_ent = b + o_plent;
  d.pl_prog_ptr = b + o_plpp;
  d.pl_prog = b + o_plp;
  if (ci16) {
    d.a_ci16 = reinterpret_cast<const unsigned short*>(b + o_a16);
    if (!P.sa_ci.empty()) d.sa_ci16 = reinterpret_cast<const unsigned short*>(b + o_sa16);
    if (P.has_isai) {
      d.ail_ci16 = reinterpret_cast<const unsigned short*>(b + o_l16);
      d.aiu_ci16 = reinterpret_cast<const unsigned short*>(b + o_u16);
      if (!P.su_ci.empty()) d.su_ci16 = reinterpret_cast<const unsigned short*>(b + o_su16);
    }
  }
  if (!P.ilu_prog.empty()) {
    d.ilu_hdr = reinterpret_cast<const int4*>(b + o_ih);
    d.ilu_prog = b + o_ip;
    d.ilu_prog_approach = P.opts.ilu_approach;
  }
  if (!P.sa_off.empty()) {
    d.sa_nnz = P.sa_off.back();
    d.sa_off = b + o_sao;
    d.sa_ci = b + o_sac;
    d.sa_src = b + o_sas;
  }
  if (!P.su_off.empty()) {
    d.su_nnz = P.su_off.back();
    d.su_off = b + o_suo;
    d.su_ci = b + o_suc;
    d.su_src = b + o_sus;
  }
  if (!P.tp_lo.empty()) {
    d.tp_lo_hdr = reinterpret_cast<const int2*>(b + o_tlh);
    d.tp_lo = b + o_tl;
    d.tp_up_hdr = reinterpret_cast<const int2*>(b + o_tuh);
    d.tp_up = b + o_tu;
    int ml = 0, mu = 0;
    for (int i = 0; i < P.n; ++i) {
      ml = std::max(ml, P.diag[i] - P.rp[i]);
      mu = std::max(mu, P.rp[i + 1] - P.diag[i] - 1);
    }
    d.tp_maxcnt_lo = ml;
    d.tp_maxcnt_up = mu;
  }
  d.pl_ndep = P.pl_ndep;
  d.pl_nlow = P.pl_nlow;
  d.pl_ndep_low = P.pl_ndep_low;
  if (P.has_isai) {
    d.ail_nnz = P.ail_rp[P.n];
    d.l_diag = P.opts.isai_lower_diag ? 1 : 0;
    d.aiu_nnz = P.aiu_rp[P.n];
    d.ail_rp = b + o_alrp;
    d.ail_ci = b + o_alci;
    d.aiu_rp = b + o_aurp;
    d.aiu_ci = b + o_auci;
    d.ail_prog_ptr = b + o_alpp;
    d.ail_prog = b + o_alp;
    d.aiu_prog_ptr = b + o_aupp;
    d.aiu_prog = b + o_aup;
    d.ail_perm = b + o_alperm;
    d.aiu_perm = b + o_auperm;
  }
  if (P.general_isai) {
    d.gen_map_ptr = b + o_gmp;
    d.gen_map = b + o_gm;
    d.gen_pos = b + o_gp;
    for (int i = 0; i < P.n; ++i) d.gen_maxs = std::max(d.gen_maxs, P.ail_rp[i + 1] - P.ail_rp[i]);
  }
  return BILU_OK;
}

bilu_status ensure_ws(bilu_plan* P, size_t bytes) {
  if (bytes <= P->ws_bytes) return BILU_OK;
  if (P->ws) cudaFree(P->ws);
  P->ws = nullptr;
  P->ws_bytes = 0;
  cudaError_t e = cudaMalloc(&P->ws, bytes);
  if (e != cudaSuccess) return set_error(BILU_ERR_ALLOC, std::string("workspace: ") + cudaGetErrorString(e));
  P->ws_bytes = bytes;
  return BILU_OK;
}

size_t align_up(size_t v) { return (v + 255) & ~(size_t)255; }

bilu_status check_opts(const bilu_options* o) {
  if (!o) return BILU_OK;
  if (o->precond < 0 || o->precond > BILU_PRECOND_GENERAL_ISAI) return set_error(BILU_ERR_INVALID, "options: bad precond");
  if (o->ilu_approach < 1 || o->ilu_approach > 4) return set_error(BILU_ERR_INVALID, "options: ilu_approach must be 1..4");
  if (o->parilu_sweeps < 0) return set_error(BILU_ERR_INVALID, "options: parilu_sweeps < 0");
  if (o->isai_power < 1) return set_error(BILU_ERR_INVALID, "options: isai_power < 1");
  if (o->tol_mode != BILU_TOL_ABS && o->tol_mode != BILU_TOL_REL) return set_error(BILU_ERR_INVALID, "options: tol_mode");
  if (!(o->tol >= 0.0)) return set_error(BILU_ERR_INVALID, "options: tol must be >= 0");
  if (o->max_iter < 0) return set_error(BILU_ERR_INVALID, "options: max_iter < 0");
  if (o->factor_precision != BILU_FP64 && o->factor_precision != BILU_FP32)
    return set_error(BILU_ERR_INVALID, "options: factor_precision");
  if (o->reduction != BILU_REDUCE_REF && o->reduction != BILU_REDUCE_FAST)
    return set_error(BILU_ERR_INVALID, "options: reduction");
  if (o->threads_per_system < 0 || o->threads_per_system > 1024)
    return set_error(BILU_ERR_INVALID, "options: threads_per_system must be 0..1024");
  if (!(o->parilu_res_tol >= 0.0)) return set_error(BILU_ERR_INVALID, "options: parilu_res_tol must be >= 0");
  if (o->isai_lower_diag != 0 && o->isai_lower_diag != 1) return set_error(BILU_ERR_INVALID, "options: isai_lower_diag");
  if (o->smem_staging < -1 || o->smem_staging > 31) return set_error(BILU_ERR_INVALID, "options: smem_staging must be -1..31");
  return BILU_OK;
}

bilu_status solve_impl(bilu_plan* P, int nsys, const double* vals, const double* lu_init, const double* b, double* x,
                       const bilu_results* R, cudaStream_t st);

}  // namespace plan_detail

using namespace plan_detail;

// ===========================================================================
// entry points
// ===========================================================================
extern "C" {

void bilu_default_options(bilu_options* o) {
  if (!o) return;
  o->precond = BILU_PRECOND_ILU0;
  o->ilu_approach = 1;
  o->parilu_sweeps = 5;
  o->isai_power = 2;
  o->tol_mode = BILU_TOL_ABS;
  o->tol = 1e-11;
  o->max_iter = 500;
  o->factor_precision = BILU_FP64;
  o->reduction = BILU_REDUCE_REF;
  o->compute_true_residual = 1;
  o->threads_per_system = 0;
  o->parilu_res_tol = 0.0;
  o->isai_lower_diag = 0;
  o->smem_staging = -1;
}

const char* bilu_last_error(void) { return g_last_error.c_str(); }
const char* bilu_version(void) { return "bilu 0.1 (sm_103a)"; }

int bilu_device_count(void) {
  int c = 0;
  if (cudaGetDeviceCount(&c) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return c;
}

bilu_status bilu_plan_create(bilu_plan** out, int n, int nnz, const int* h_rp, const int* h_ci,
                             const bilu_options* opts) {
  if (!out) return set_error(BILU_ERR_INVALID, "bilu_plan_create: out is NULL");
  *out = nullptr;
  if (n <= 0 || nnz < 0 || !h_rp || (nnz > 0 && !h_ci)) return set_error(BILU_ERR_INVALID, "bilu_plan_create: bad sizes");
  bilu_status st = check_opts(opts);
  if (st) return st;
  // validate CSR
  if (h_rp[0] != 0 || h_rp[n] != nnz) return set_error(BILU_ERR_PATTERN, "row pointers must start at 0 and end at nnz");
  for (int i = 0; i < n; ++i) {
    if (h_rp[i + 1] < h_rp[i]) return set_error(BILU_ERR_PATTERN, "row pointers decrease at row " + std::to_string(i));
    for (int k = h_rp[i]; k < h_rp[i + 1]; ++k) {
      if (h_ci[k] < 0 || h_ci[k] >= n)
        return set_error(BILU_ERR_PATTERN, "column index out of range in row " + std::to_string(i));
      if (k > h_rp[i] && h_ci[k] <= h_ci[k - 1])
        return set_error(BILU_ERR_PATTERN, "columns not strictly ascending in row " + std::to_string(i));
    }
  }
  if (bilu_device_count() == 0) return set_error(BILU_ERR_NO_DEVICE, "no CUDA device");
  bilu_plan* P = new bilu_plan();
  if (opts)
    P->opts = *opts;
  else
    bilu_default_options(&P->opts);
  cudaGetDevice(&P->device);
  P->n = n;
  P->nnz_in = nnz;
  P->in_rp.assign(h_rp, h_rp + n + 1);
  P->in_ci.assign(h_ci, h_ci + nnz);
  // missing diagonals (Count/Add_Missing_Diagonal_Elements, factorization.cu:399-467)
  P->rp.assign(n + 1, 0);
  P->ci.clear();
  P->src.clear();
  for (int i = 0; i < n; ++i) {
    bool has = false;
    for (int k = h_rp[i]; k < h_rp[i + 1]; ++k) has |= (h_ci[k] == i);
    bool placed = has;
    if (!has) P->missing++;
    for (int k = h_rp[i]; k < h_rp[i + 1]; ++k) {
      if (!placed && h_ci[k] > i) {
        P->ci.push_back(i);
        P->src.push_back(-1);
        placed = true;
      }
      P->ci.push_back(h_ci[k]);
      P->src.push_back(k);
    }
    if (!placed) {
      P->ci.push_back(i);
      P->src.push_back(-1);
    }
    P->rp[i + 1] = (int)P->ci.size();
  }
  P->nnz = (int)P->ci.size();
  if (P->missing > 0 && P->opts.precond == BILU_PRECOND_ILU0) {
    delete P;
    return set_error(BILU_ERR_PATTERN,
                     "the merged ILU(0) solver requires every diagonal entry in the pattern (as the reference's "
                     "merged solver, which asserts); use BILU_PRECOND_ILU0_SPLIT");
  }
  P->diag.assign(n, -1);
  P->row_of.assign(P->nnz, 0);
  for (int i = 0; i < n; ++i)
    for (int k = P->rp[i]; k < P->rp[i + 1]; ++k) {
      P->row_of[k] = i;
      if (P->ci[k] == i) P->diag[i] = k;
      P->maxl = std::max(P->maxl, P->rp[i + 1] - P->rp[i]);
    }
  for (int i = 0; i < n; ++i) P->a_maxl = std::max(P->a_maxl, h_rp[i + 1] - h_rp[i]);
  // L / U split (factorization.cu:216-344)
  P->l_rp.assign(n + 1, 0);
  P->u_rp.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    for (int k = P->rp[i]; k < P->diag[i]; ++k) {
      P->l_ci.push_back(P->ci[k]);
      P->l_src.push_back(k);
    }
    P->l_ci.push_back(i);
    P->l_src.push_back(-1);
    for (int k = P->diag[i]; k < P->rp[i + 1]; ++k) {
      P->u_ci.push_back(P->ci[k]);
      P->u_src.push_back(k);
    }
    P->l_rp[i + 1] = (int)P->l_ci.size();
    P->u_rp[i + 1] = (int)P->u_ci.size();
  }
  build_levels(*P);
  build_trsv_programs(*P);
  build_deps(*P);
  P->row_lev.assign(n, 0);
  for (int l = 0; l + 1 < (int)P->lev_lo_ptr.size(); ++l)
    for (int q = P->lev_lo_ptr[l]; q < P->lev_lo_ptr[l + 1]; ++q) P->row_lev[P->lev_lo_rows[q]] = l;
  P->tpos.assign(P->nnz, -1);
  for (int i = 0; i < n; ++i)
    for (int k = P->rp[i]; k < P->rp[i + 1]; ++k) {
      P->tpos[k] = find_pos(P->rp, P->ci, P->ci[k], i);
      if (P->ci[k] < i || P->dep_ptr[k + 1] > P->dep_ptr[k]) P->mlp_ent.push_back(k);
    }
  {
    std::vector<int> dep_up, dep_low, lower, upper;
    for (int i = 0; i < n; ++i)
      for (int k = P->rp[i]; k < P->rp[i + 1]; ++k) {
        if (P->dep_ptr[k + 1] > P->dep_ptr[k])
          (P->ci[k] < i ? dep_low : dep_up).push_back(k);
        else
          (P->ci[k] < i ? lower : upper).push_back(k);
      }
    auto most_pairs_first = [&](int a, int b) {
      return P->dep_ptr[a + 1] - P->dep_ptr[a] > P->dep_ptr[b + 1] - P->dep_ptr[b];
    };
    std::stable_sort(dep_up.begin(), dep_up.end(), most_pairs_first);
    std::stable_sort(dep_low.begin(), dep_low.end(), most_pairs_first);
    std::vector<int> with_deps = dep_up;
    with_deps.insert(with_deps.end(), dep_low.begin(), dep_low.end());
    P->pl_ndep = (int)with_deps.size();
    P->pl_ndep_low = (int)dep_low.size();
    P->pl_nlow = (int)lower.size();
    P->pl_ent = with_deps;
    P->pl_ent.insert(P->pl_ent.end(), lower.begin(), lower.end());
    P->pl_ent.insert(P->pl_ent.end(), upper.begin(), upper.end());
    // the entries with pairs as a warp-blocked program (DevPattern::pl_prog)
    const int nb = (P->pl_ndep + 31) / 32;
    P->pl_prog_ptr.assign(nb + 1, 0);
    for (int bk = 0; bk < nb; ++bk) {
      int len = 0;
      for (int q = 32 * bk; q < std::min(P->pl_ndep, 32 * bk + 32); ++q) {
        const int k = P->pl_ent[q];
        len = std::max(len, 3 + 2 * (P->dep_ptr[k + 1] - P->dep_ptr[k]));
      }
      P->pl_prog_ptr[bk + 1] = P->pl_prog_ptr[bk] + 32 * len;
    }
    P->pl_prog.assign(P->pl_prog_ptr[nb], 0);
    for (int q = 0; q < P->pl_ndep; ++q) {
      const int k = P->pl_ent[q], i = P->row_of[k], j = P->ci[k];
      int* w = P->pl_prog.data() + P->pl_prog_ptr[q / 32] + q % 32;
      w[0] = k;
      w[32] = j << 1 | (j < i ? 1 : 0);
      w[64] = P->dep_ptr[k + 1] - P->dep_ptr[k];
      for (int u = 0; u < w[64]; ++u) {
        w[96 + 64 * u] = P->dep[2 * (P->dep_ptr[k] + u)];
        w[128 + 64 * u] = P->dep[2 * (P->dep_ptr[k] + u) + 1];
      }
    }
  }
  P->has_isai = is_isai(P->opts.precond);
  P->general_isai = P->opts.precond == BILU_PRECOND_GENERAL_ISAI;
  if (P->has_isai) {
    st = build_isai(*P);
    if (st) {
      delete P;
      return st;
    }
  }
  build_sell(n, P->in_rp, P->in_ci, P->sa_off, P->sa_ci, P->sa_src);
  if (P->has_isai && !P->general_isai) build_sell(n, P->aiu_rp, P->aiu_ci, P->su_off, P->su_ci, P->su_src);
  choose_layout(*P);
  choose_rr(*P);
  if (!P->rr && P->lay.total > (int)solve_max_smem()) {
    const int need = P->lay.total;
    delete P;
    return set_error(BILU_ERR_CAPACITY, "solver needs " + std::to_string(need) + " bytes of shared memory per system");
  }
  st = upload(*P);
  if (st) {
    if (P->dbuf) cudaFree(P->dbuf);
    delete P;
    return st;
  }
  *out = P;
  return BILU_OK;
}

bilu_status bilu_plan_enable_timing(bilu_plan* P, int enable) {
  if (!P) return set_error(BILU_ERR_INVALID, "bilu_plan_enable_timing: NULL plan");
  if (enable && !P->ev[0]) {
    for (auto& e : P->ev) {
      cudaError_t r = cudaEventCreate(&e);
      if (r != cudaSuccess) return cuda_err(r, "cudaEventCreate");
    }
  }
  P->timing = enable != 0;
  return BILU_OK;
}

bilu_status bilu_plan_last_timing(bilu_plan* P, bilu_timing* t) {
  if (!P || !t) return set_error(BILU_ERR_INVALID, "bilu_plan_last_timing: NULL argument");
  if (!P->timing) return set_error(BILU_ERR_INVALID, "bilu_plan_last_timing: timing not enabled");
  cudaError_t r = cudaEventSynchronize(P->ev[2]);
  if (r != cudaSuccess) return cuda_err(r, "cudaEventSynchronize");
  cudaEventElapsedTime(&t->setup_ms, P->ev[0], P->ev[1]);
  cudaEventElapsedTime(&t->solve_ms, P->ev[1], P->ev[2]);
  cudaEventElapsedTime(&t->total_ms, P->ev[0], P->ev[2]);
  return BILU_OK;
}

bilu_status bilu_plan_autotune(bilu_plan* P, int nsys, const double* d_values, const double* d_b, double* d_x,
                               void* stream) {
  if (!P) return set_error(BILU_ERR_INVALID, "bilu_plan_autotune: NULL plan");
  if (nsys <= 0 || !d_values || !d_b || !d_x) return set_error(BILU_ERR_INVALID, "bilu_plan_autotune: bad arguments");
  if (!P->rr) return BILU_OK;  // only the register-resident solver has choices
  const bool had_timing = P->timing;
  bilu_status st = bilu_plan_enable_timing(P, 1);
  if (st) return st;
  const int base = round_up((P->n + 7) / 8, 32);
  const int keep_nt = P->rr_threads;
  const RRLayout keep_lay = P->rr_lay;
  const bool keep_sell = P->rr_sell, keep_occ = P->rr_occ;
  float best = -1.0f;
  int best_nt = keep_nt, best_mask = -1;
  for (int f : {1, 2, 4}) {
    for (int mask : {0, 2, 6, 1, 8, 10, 14, 16, 18, 22, 24, 26}) {
      const int rf = rr_rows_per_thread(P->n, base * f);
      if ((mask & 16) && (rf < 2 || (rf == 8 && P->rr_pv == 3))) continue;  // bit 4 ignored
      if ((mask & 24) && P->opts.reduction != BILU_REDUCE_FAST) continue;                         // bits 3, 4 ignored
      if (!rr_configure(*P, base * f, mask)) continue;
      float ms = 0.0f;
      for (int rep = 0; rep < 2; ++rep) {  // the first run warms caches; the second is timed
        st = solve_impl(P, nsys, d_values, nullptr, d_b, d_x, nullptr, (cudaStream_t)stream);
        if (st) break;
        bilu_timing t;
        st = bilu_plan_last_timing(P, &t);
        if (st) break;
        ms = t.solve_ms;
      }
      if (st) break;
      if (best < 0.0f || ms < best) {
        best = ms;
        best_nt = base * f;
        best_mask = mask;
      }
    }
    if (st) break;
  }
  if (best_mask >= 0) {
    rr_configure(*P, best_nt, best_mask);
  } else {
    P->rr_threads = keep_nt;
    P->rr_lay = keep_lay;
    P->rr_sell = keep_sell;
    P->rr_occ = keep_occ;
  }
  P->timing = had_timing;
  return st;
}

bilu_status bilu_plan_destroy(bilu_plan* P) {
  if (!P) return BILU_OK;
  for (auto& e : P->ev)
    if (e) cudaEventDestroy(e);
  if (P->dbuf) cudaFree(P->dbuf);
  if (P->ws) cudaFree(P->ws);
  delete P;
  return BILU_OK;
}

bilu_status bilu_plan_get_info(const bilu_plan* P, bilu_plan_info* info) {
  if (!P || !info) return set_error(BILU_ERR_INVALID, "bilu_plan_get_info: NULL argument");
  info->n = P->n;
  info->nnz = P->nnz;
  info->nnz_in = P->nnz_in;
  info->missing_diag = P->missing;
  info->nnz_L = (int)P->l_src.size();
  info->nnz_U = (int)P->u_src.size();
  info->nnz_isai_L = P->has_isai ? P->ail_rp[P->n] : 0;
  info->nnz_isai_U = P->has_isai ? P->aiu_rp[P->n] : 0;
  info->levels_lower = (int)P->lev_lo_ptr.size() - 1;
  info->levels_upper = (int)P->lev_up_ptr.size() - 1;
  info->max_row_len = P->maxl;
  info->threads = P->threads;
  info->smem_bytes = P->lay.total;
  info->operands_in_smem = (P->lay.A >= 0 ? 1 : 0) | ((P->lay.F >= 0 || P->lay.ail >= 0) ? 2 : 0) |
                           (P->lay.aiu >= 0 ? 4 : 0);
  info->solver_kernel = P->rr ? 1 : 0;
  if (P->rr) {
    info->threads = P->rr_threads;
    info->smem_bytes = P->rr_lay.total;
    info->operands_in_smem = (P->rr_lay.A >= 0 ? 1 : 0) | (P->rr_lay.ail >= 0 ? 2 : 0) | (P->rr_lay.aiu >= 0 ? 4 : 0) |
                             (P->rr_sell ? 8 : 0) | (P->rr_occ ? 16 : 0);
  }
  return BILU_OK;
}

bilu_status bilu_plan_get_pattern(const bilu_plan* P, int which, int* n, int* nnz, int* h_rp, int* h_ci) {
  if (!P) return set_error(BILU_ERR_INVALID, "bilu_plan_get_pattern: NULL plan");
  const std::vector<int>* rp = nullptr;
  const std::vector<int>* ci = nullptr;
  switch (which) {
    case 0: rp = &P->rp; ci = &P->ci; break;
    case 1: rp = &P->ail_rp; ci = &P->ail_ci; break;
    case 2: rp = &P->aiu_rp; ci = &P->aiu_ci; break;
    case 3: rp = &P->l_rp; ci = &P->l_ci; break;
    case 4: rp = &P->u_rp; ci = &P->u_ci; break;
    default: return set_error(BILU_ERR_INVALID, "bilu_plan_get_pattern: which must be 0..4");
  }
  if ((which == 1 || which == 2) && !P->has_isai)
    return set_error(BILU_ERR_INVALID, "bilu_plan_get_pattern: the plan has no ISAI pattern");
  if (n) *n = P->n;
  if (nnz) *nnz = rp->empty() ? 0 : rp->back();
  if (h_rp) std::memcpy(h_rp, rp->data(), sizeof(int) * rp->size());
  if (h_ci && !ci->empty()) std::memcpy(h_ci, ci->data(), sizeof(int) * ci->size());
  return BILU_OK;
}

bilu_status bilu_expand_values(const bilu_plan* P, int nsys, const double* vin, double* vout, void* stream) {
  if (!P || nsys < 0 || (nsys > 0 && (!vin || !vout))) return set_error(BILU_ERR_INVALID, "bilu_expand_values: bad args");
  cudaError_t e = launch_expand(P->dp, nsys, vin, vout, (cudaStream_t)stream);
  return e == cudaSuccess ? BILU_OK : cuda_err(e, "expand");
}

}  // extern "C"

namespace plan_detail {
const double* factor_values(bilu_plan* P, int nsys, const double* vin, double* scratch, cudaStream_t st,
                            cudaError_t* err);
}  // namespace plan_detail

namespace bilu {

int fact_threads(const bilu_plan* P) { return std::min(512, round_up(std::max(P->n, 64), 32)); }

// Tight scratch of one solve, every region 256-byte aligned: the expanded
// values (inserted diagonals only), the FP64 factors (ILU / ParILU
// preconditioners), their FP32 copy (triangular-solve preconditioners with
// FP32 factors), the ISAI values in the preconditioner's type, and the
// SELL-32 copies of A and aiU that the register-resident solver reads when its
// configuration asks for them.
SolveScratch solve_scratch_layout(const bilu_plan* P, int nsys) {
  SolveScratch s;
  const bilu_options& o = P->opts;
  const int prec = o.precond;
  const bool fp32 = is_fp32(o);
  const size_t nz = (size_t)P->nnz * nsys;
  const bool factors = prec == BILU_PRECOND_ILU0_SPLIT || prec == BILU_PRECOND_PARILU0 ||
                       prec == BILU_PRECOND_ILU0_ISAI || prec == BILU_PRECOND_PARILU0_ISAI;
  const bool pre = factors || prec == BILU_PRECOND_GENERAL_ISAI;  // preconditioner generated before the solve
  const size_t fts = fp32 ? 4 : 8;
  size_t need = 0;
  auto take = [&](size_t& off, size_t bytes) {
    off = need;
    need += align_up(bytes);
  };
  if (pre && P->missing) take(s.exp, nz * 8);
  if (factors) take(s.lu, nz * 8);
  if (fp32 && (prec == BILU_PRECOND_ILU0_SPLIT || prec == BILU_PRECOND_PARILU0)) take(s.f, nz * 4);
  if (P->has_isai) take(s.ail, (size_t)P->dp.ail_nnz * nsys * fts);
  if (P->has_isai && !P->general_isai) take(s.aiu, (size_t)P->dp.aiu_nnz * nsys * fts);
  s.sell_a = P->rr && P->rr_sell && P->rr_lay.A < 0 && P->dp.sa_nnz > 0;
  s.sell_u = P->rr && P->rr_sell && P->rr_pv == 1 && P->rr_lay.aiu < 0 && P->dp.su_nnz > 0;
  if (s.sell_a) take(s.asell, (size_t)P->dp.sa_nnz * nsys * 8);
  if (s.sell_u) take(s.usell, (size_t)P->dp.su_nnz * nsys * fts);
  s.total = need;
  return s;
}

bilu_status solve_launch(bilu_plan* P, int nsys, const double* vals, const double* lu_init, const double* b,
                         double* x, const bilu_results* R, char* ws, const SolveScratch& sc, cudaStream_t st) {
  const bilu_options& o = P->opts;
  const bool fp32 = is_fp32(o);
  const size_t nz = (size_t)P->nnz * nsys;
  const int prec = o.precond;
  if (P->timing) cudaEventRecord(P->ev[0], st);
  SolveArgs a;
  a.pat = P->dp;
  a.lay = P->lay;
  a.nsys = nsys;
  a.A = vals;
  a.b = b;
  a.x = x;
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
  a.dot_serial = is_isai(prec) ? 1 : 0;
  cudaError_t e = cudaSuccess;
  const int ft = fact_threads(P);
  if (prec == BILU_PRECOND_ILU0) {
    a.prec = PK_ILU_INKERNEL;
  } else if (prec == BILU_PRECOND_NONE) {
    a.prec = PK_NONE;
  } else {
    const double* fv = factor_values(P, nsys, vals, (double*)(ws + sc.exp), st, &e);
    if (e != cudaSuccess) return cuda_err(e, "expand");
    if (prec == BILU_PRECOND_GENERAL_ISAI) {
      e = launch_isai_general(P->dp, nsys, fv, ws + sc.ail, fp32 ? 1 : 0, ft, st);
      if (e != cudaSuccess) return cuda_err(e, "general isai");
      a.prec = PK_ISAI;
      a.ail = ws + sc.ail;
      a.aiu = nullptr;
    } else {
      double* lu = (double*)(ws + sc.lu);
      if (prec == BILU_PRECOND_ILU0_SPLIT || prec == BILU_PRECOND_ILU0_ISAI)
        e = launch_ilu0(P->dp, nsys, fv, lu, o.ilu_approach, ft, st);
      else
        e = launch_parilu0(P->dp, nsys, fv, lu_init, lu, o.parilu_sweeps, ft, st, o.parilu_res_tol,
                           R ? R->parilu_sweeps : nullptr, R ? R->ilu_residual : nullptr,
                           o.reduction == BILU_REDUCE_FAST ? 1 : 0);
      if (e != cudaSuccess) return cuda_err(e, "factorisation");
      if (is_isai(prec)) {
        void* ail = ws + sc.ail;
        void* aiu = ws + sc.aiu;
        e = launch_isai(P->dp, nsys, lu, ail, aiu, fp32 ? 1 : 0, ft, st, o.reduction == BILU_REDUCE_FAST ? 1 : 0);
        if (e != cudaSuccess) return cuda_err(e, "isai");
        a.prec = PK_ISAI;
        a.ail = ail;
        a.aiu = aiu;
      } else {
        a.prec = PK_LU_GLOBAL;
        if (fp32) {
          float* f = (float*)(ws + sc.f);
          e = launch_to_float(lu, f, nz, st);
          if (e != cudaSuccess) return cuda_err(e, "convert");
          a.F = f;
        } else {
          a.F = lu;
        }
      }
    }
  }
  int maxl = P->a_maxl;
  if (P->has_isai) {
    for (int i = 0; i < P->n; ++i) {
      maxl = std::max(maxl, P->ail_rp[i + 1] - P->ail_rp[i]);
      maxl = std::max(maxl, P->aiu_rp[i + 1] - P->aiu_rp[i]);
    }
  }
  if (P->timing) cudaEventRecord(P->ev[1], st);
  if (sc.sell_u) {
    e = launch_to_sell(P->dp.su_src, P->dp.su_nnz, P->dp.aiu_nnz, nsys, a.aiu, ws + sc.usell, fp32 ? 4 : 8, st);
    if (e != cudaSuccess) return cuda_err(e, "SELL copy of aiU");
    a.aiu_sell = ws + sc.usell;
  }
  if (sc.sell_a) {
    e = launch_to_sell(P->dp.sa_src, P->dp.sa_nnz, P->dp.a_nnz, nsys, vals, ws + sc.asell, 8, st);
    if (e != cudaSuccess) return cuda_err(e, "SELL copy of A");
    a.A_sell = (const double*)(ws + sc.asell);
  }
  e = P->rr ? launch_solve_rr(a, P->rr_lay, P->rr_threads, P->rr_pv, fp32 ? 1 : 0,
                              o.reduction == BILU_REDUCE_FAST ? 0 : 1, P->rr_occ ? 1 : 0, st)
            : launch_solve(a, P->threads, fp32 ? 1 : 0, o.reduction == BILU_REDUCE_FAST ? 1 : 0, maxl, st);
  if (e != cudaSuccess) return cuda_err(e, "solver launch");
  if (P->timing) cudaEventRecord(P->ev[2], st);
  return BILU_OK;
}

}  // namespace bilu

namespace plan_detail {

// factor-pattern values for the factorisation kernels: the caller's array
// when no diagonal was inserted, else an expanded copy in `scratch`
const double* factor_values(bilu_plan* P, int nsys, const double* vin, double* scratch, cudaStream_t st,
                            cudaError_t* err) {
  *err = cudaSuccess;
  if (P->missing == 0) return vin;
  *err = launch_expand(P->dp, nsys, vin, scratch, st);
  return scratch;
}

bilu_status solve_impl(bilu_plan* P, int nsys, const double* vals, const double* lu_init, const double* b, double* x,
                       const bilu_results* R, cudaStream_t st) {
  if (nsys < 0 || (nsys > 0 && (!vals || !b || !x))) return set_error(BILU_ERR_INVALID, "bilu_solve: bad arguments");
  if (P->opts.isai_lower_diag)
    return set_error(BILU_ERR_INVALID, "bilu_solve: plans with isai_lower_diag = 1 only serve bilu_isai");
  if (nsys == 0) return BILU_OK;
  const SolveScratch sc = solve_scratch_layout(P, nsys);
  if (sc.total > 0) {
    bilu_status s = ensure_ws(P, sc.total);
    if (s) return s;
  }
  return solve_launch(P, nsys, vals, lu_init, b, x, R, static_cast<char*>(P->ws), sc, st);
}

}  // namespace plan_detail

extern "C" {

bilu_status bilu_solve(bilu_plan* P, int nsys, const double* d_values, const double* d_b, double* d_x,
                       const bilu_results* R, void* stream) {
  if (!P) return set_error(BILU_ERR_INVALID, "bilu_solve: NULL plan");
  return solve_impl(P, nsys, d_values, nullptr, d_b, d_x, R, (cudaStream_t)stream);
}

bilu_status bilu_solve_warm(bilu_plan* P, int nsys, const double* d_values, const double* d_lu_init,
                            const double* d_b, double* d_x, const bilu_results* R, void* stream) {
  if (!P) return set_error(BILU_ERR_INVALID, "bilu_solve_warm: NULL plan");
  if (P->opts.precond != BILU_PRECOND_PARILU0 && P->opts.precond != BILU_PRECOND_PARILU0_ISAI)
    return set_error(BILU_ERR_INVALID, "bilu_solve_warm: only for ParILU preconditioners");
  return solve_impl(P, nsys, d_values, d_lu_init, d_b, d_x, R, (cudaStream_t)stream);
}

bilu_status bilu_ilu0(const bilu_plan* Pc, int nsys, const double* d_values, double* d_lu, int approach,
                      void* stream) {
  bilu_plan* P = const_cast<bilu_plan*>(Pc);
  if (!P || nsys < 0 || (nsys > 0 && (!d_values || !d_lu)) || approach < 1 || approach > 4)
    return set_error(BILU_ERR_INVALID, "bilu_ilu0: bad arguments");
  if (nsys == 0) return BILU_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const double* fv = d_values;
  cudaError_t e;
  if (P->missing) {  // expand straight into the output, factorise in place
    e = launch_expand(P->dp, nsys, d_values, d_lu, st);
    if (e != cudaSuccess) return cuda_err(e, "expand");
    fv = d_lu;
  }
  e = launch_ilu0(P->dp, nsys, fv, d_lu, approach, fact_threads(P), st);
  return e == cudaSuccess ? BILU_OK : cuda_err(e, "ilu0");
}

bilu_status bilu_parilu0(const bilu_plan* Pc, int nsys, const double* d_values, const double* d_lu_init, double* d_lu,
                         int sweeps, void* stream) {
  bilu_plan* P = const_cast<bilu_plan*>(Pc);
  if (!P || nsys < 0 || sweeps < 0 || (nsys > 0 && (!d_values || !d_lu)))
    return set_error(BILU_ERR_INVALID, "bilu_parilu0: bad arguments");
  if (nsys == 0) return BILU_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const double* fv = d_values;
  if (P->missing) {
    bilu_status s = ensure_ws(P, align_up((size_t)P->nnz * nsys * 8));
    if (s) return s;
    cudaError_t e = launch_expand(P->dp, nsys, d_values, (double*)P->ws, st);
    if (e != cudaSuccess) return cuda_err(e, "expand");
    fv = (const double*)P->ws;
  }
  cudaError_t e = launch_parilu0(P->dp, nsys, fv, d_lu_init, d_lu, sweeps, fact_threads(P), st);
  return e == cudaSuccess ? BILU_OK : cuda_err(e, "parilu0");
}

bilu_status bilu_split_lu(const bilu_plan* P, int nsys, const double* d_lu, double* d_L, double* d_U, void* stream) {
  if (!P || nsys < 0 || (nsys > 0 && (!d_lu || !d_L || !d_U))) return set_error(BILU_ERR_INVALID, "bilu_split_lu: bad args");
  cudaError_t e = launch_split(P->dp, nsys, d_lu, d_L, d_U, (cudaStream_t)stream);
  return e == cudaSuccess ? BILU_OK : cuda_err(e, "split");
}

bilu_status bilu_isai(const bilu_plan* P, int nsys, const double* d_lu, double* d_ail, double* d_aiu, void* stream) {
  if (!P || nsys < 0 || (nsys > 0 && (!d_lu || !d_ail || (!d_aiu && !P->general_isai))))
    return set_error(BILU_ERR_INVALID, "bilu_isai: bad args");
  if (!P->has_isai) return set_error(BILU_ERR_INVALID, "bilu_isai: plan was not created with an ISAI preconditioner");
  cudaError_t e = P->general_isai
                      ? launch_isai_general(P->dp, nsys, d_lu, d_ail, 0, fact_threads(P), (cudaStream_t)stream)
                      : launch_isai(P->dp, nsys, d_lu, d_ail, d_aiu, 0, fact_threads(P), (cudaStream_t)stream,
                                    P->opts.reduction == BILU_REDUCE_FAST ? 1 : 0);
  return e == cudaSuccess ? BILU_OK : cuda_err(e, "isai");
}

bilu_status bilu_true_residual(const bilu_plan* P, int nsys, const double* d_values, const double* d_b,
                               const double* d_x, double* d_norms, void* stream) {
  if (!P || nsys < 0 || (nsys > 0 && (!d_values || !d_b || !d_x || !d_norms)))
    return set_error(BILU_ERR_INVALID, "bilu_true_residual: bad args");
  // the operator pattern is the caller's pattern
  DevPattern d = P->dp;
  d.rp = d.a_rp;
  d.ci = d.a_ci;
  d.nnz = d.a_nnz;
  cudaError_t e = launch_true_residual(d, nsys, d_values, d_b, d_x, d_norms, 256, (cudaStream_t)stream);
  return e == cudaSuccess ? BILU_OK : cuda_err(e, "true residual");
}

}  // extern "C"

extern "C" bilu_status bilu_forward_error(const bilu_plan* P, int nsample, const int* h_sys_ids, const double* d_values,
                                          const double* d_b, const double* d_x, double* h_fwd_err, double* d_x_dense,
                                          void* stream) {
  if (!P || nsample < 0 || (nsample > 0 && (!h_sys_ids || !d_values || !d_b || !h_fwd_err)))
    return set_error(BILU_ERR_INVALID, "bilu_forward_error: bad arguments");
  if (nsample == 0) return BILU_OK;
  const int n = P->n;
  cudaStream_t st = (cudaStream_t)stream;
  int* ids = nullptr;
  double* work = nullptr;
  double* xd = nullptr;
  const size_t per = (size_t)n * n + n;
  cudaError_t e = cudaMalloc((void**)&ids, sizeof(int) * nsample);
  if (e == cudaSuccess) e = cudaMalloc((void**)&work, sizeof(double) * per * nsample);
  if (e == cudaSuccess && !d_x_dense) e = cudaMalloc((void**)&xd, sizeof(double) * (size_t)n * nsample);
  double* xout = d_x_dense ? d_x_dense : xd;
  std::vector<double> hx((size_t)n * nsample), hs((size_t)n * nsample);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ids, h_sys_ids, sizeof(int) * nsample, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = launch_dense_solve(P->dp, nsample, ids, d_values, d_b, work, xout, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hx.data(), xout, sizeof(double) * hx.size(), cudaMemcpyDeviceToHost, st);
  for (int q = 0; q < nsample && e == cudaSuccess && d_x; ++q)
    e = cudaMemcpyAsync(hs.data() + (size_t)q * n, d_x + (size_t)h_sys_ids[q] * n, sizeof(double) * n,
                        cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(ids);
  cudaFree(work);
  cudaFree(xd);
  if (e != cudaSuccess) return cuda_err(e, "forward error");
  for (int q = 0; q < nsample; ++q) {
    double num = 0.0, den = 0.0;
    for (int i = 0; i < n; ++i) {
      const double xe = hx[(size_t)q * n + i];
      const double dx = (d_x ? hs[(size_t)q * n + i] : 0.0) - xe;
      num += dx * dx;
      den += xe * xe;
    }
    h_fwd_err[q] = den > 0.0 ? std::sqrt(num / den) : std::sqrt(num);
  }
  return BILU_OK;
}
