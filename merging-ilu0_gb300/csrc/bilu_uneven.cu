// Uneven batches: systems of different sizes and sparsity patterns solved
// together (merged ILU(0) + BiCGSTAB per system, the reference's merged
// solver arithmetic, PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu:249-538).
//
// The reference needs one shared pattern per batch (ReadWriteData.cpp:398-433);
// here every system carries its own pattern.  The host analyses each pattern
// once (diagonal pointers, level schedules, dependency pairs, triangular-solve
// programs; OpenMP over systems) and sorts the systems into size buckets,
// longest first.  In the reference operation order each bucket runs as one
// persistent kernel whose CTAs take systems from an atomic work queue; in FAST
// order, buckets of systems with n <= 1024 run the register-resident solver,
// either one CTA per system or as a persistent grid over the bucket's work
// queue.  The per-bucket CTA size and grid come from an autotuner that times
// the candidates on the caller's batch.  All bucket
// launches (and the zeroing of the queue heads) are captured once into a CUDA
// graph whose branches run concurrently; a solve is one graph launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "bilu.h"
#include "bilu_internal.h"

using namespace bilu;

namespace {

struct Bucket {
  int lo = 0, hi = 0;        // n range (lo, hi]
  std::vector<int> sys;      // systems, longest first
  int order_off = 0;         // offset into the device order array
  int maxl = 0;              // longest row
  int smem = 0;              // dynamic shared memory per CTA
  int threads = 0;           // CTA size (autotuned)
  int grid = 0;              // persistent CTAs
  float tuned_ms = -1.0f;
  int maxn = 0;
  bool rr = false;           // register-resident solver (FAST order, n <= 1024)
  int R = 0;                 // its rows per thread
  int rr_occ = 0;            // its resident CTAs per SM (the persistent grid is rr_occ x SMs)
  int rr_rest = 0;           // its largest layout without the reduction slot (which depends on the CTA size)
};

}  // namespace

struct bilu_uneven_plan {
  bilu_options opts;
  int nsys = 0;
  long long total_rows = 0, total_nnz = 0;
  std::vector<SysDesc> desc;
  std::vector<Bucket> buckets;
  int* d_meta = nullptr;
  SysDesc* d_desc = nullptr;
  int* d_order = nullptr;
  int* d_counters = nullptr;
  int nsm = 0;
  // captured graph and the pointers baked into it
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const void* key[8] = {};
  cudaStream_t cap = nullptr;
  std::vector<cudaStream_t> side;
  std::vector<cudaEvent_t> ev;
};

namespace {

bilu_status cuda_fail(cudaError_t e, const char* what) {
  return set_error(BILU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int round32(int v) { return (v + 31) / 32 * 32; }

int prec_kind_uneven(const bilu_options& o) { return o.precond == BILU_PRECOND_NONE ? PK_NONE : PK_ILU_INKERNEL; }

UnevenArgs make_args(const bilu_uneven_plan* U, const Bucket& b, int bi, const double* vals, const double* rhs,
                     double* x, const bilu_results* R) {
  const bilu_options& o = U->opts;
  UnevenArgs u;
  u.base.A = vals;
  u.base.b = rhs;
  u.base.x = x;
  if (R) {
    u.base.iters = R->iter_counts;
    u.base.conv = R->conv_flags;
    u.base.res = R->iter_res_norms;
    u.base.status = R->status;
    u.base.true_res = o.compute_true_residual ? R->true_res_norms : nullptr;
  }
  u.base.tol = o.tol;
  u.base.tol_mode = o.tol_mode;
  u.base.max_iter = o.max_iter;
  u.base.prec = prec_kind_uneven(o);
  u.base.approach = o.ilu_approach;
  u.base.dot_serial = 0;
  u.desc = U->d_desc;
  u.meta = U->d_meta;
  u.order = U->d_order + b.order_off;
  u.count = (int)b.sys.size();
  u.counter = U->d_counters + bi;
  u.smem_budget = b.smem;
  return u;
}

int rr_pv(const bilu_options& o) { return o.precond == BILU_PRECOND_NONE ? 0 : 3; }

// Sets the register-resident configuration of bucket b for nt threads per
// system; false when it does not fit (rows per thread, registers, shared memory).
bool rr_setup(const bilu_uneven_plan* U, Bucket& b, int nt) {
  const int R = rr_rows_per_thread(b.maxn, nt);
  if (R == 0 || nt % 32 || nt > rr_max_threads(R)) return false;
  b.smem = rr_red_bytes(nt) + b.rr_rest;
  if (b.smem > (int)solve_max_smem()) return false;
  const void* k = rr_uneven_kernel(rr_pv(U->opts), U->opts.factor_precision == BILU_FP32, R);
  int occ = 0;
  // buckets can share a kernel with different layouts: allow the device maximum, launch with b.smem
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)solve_max_smem()) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, nt, b.smem) != cudaSuccess || occ < 1) {
    cudaGetLastError();
    return false;
  }
  b.rr = true;
  b.R = R;
  b.threads = nt;
  b.rr_occ = occ;
  b.grid = (int)b.sys.size();
  return true;
}

// The persistent grid of a register-resident bucket: every resident CTA slot, at most one per system.
int rr_persistent_grid(const bilu_uneven_plan* U, const Bucket& b) {
  return std::min((int)b.sys.size(), b.rr_occ * U->nsm);
}

int occupancy_grid(const bilu_uneven_plan* U, const Bucket& b, int threads) {
  const bool fp32 = U->opts.factor_precision == BILU_FP32;
  const bool fast = U->opts.reduction == BILU_REDUCE_FAST;
  void* k = uneven_kernel(fp32, fast, b.maxl);
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, b.smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, b.smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return std::min(per_sm * U->nsm, (int)b.sys.size());
}

bilu_status launch_bucket(bilu_uneven_plan* U, int bi, const double* vals, const double* rhs, double* x,
                          const bilu_results* R, cudaStream_t st) {
  const Bucket& b = U->buckets[bi];
  if (b.sys.empty()) return BILU_OK;
  const UnevenArgs u = make_args(U, b, bi, vals, rhs, x, R);
  cudaError_t e = b.rr ? launch_uneven_rr(u, b.threads, b.R, rr_pv(U->opts), U->opts.factor_precision == BILU_FP32,
                                          b.grid, st)
                       : launch_uneven(u, b.threads, b.grid, U->opts.factor_precision == BILU_FP32,
                                       U->opts.reduction == BILU_REDUCE_FAST, b.maxl, st);
  return e == cudaSuccess ? BILU_OK : cuda_fail(e, "uneven launch");
}

void drop_graph(bilu_uneven_plan* U) {
  if (U->exec) cudaGraphExecDestroy(U->exec);
  if (U->graph) cudaGraphDestroy(U->graph);
  U->exec = nullptr;
  U->graph = nullptr;
  std::memset(U->key, 0, sizeof(U->key));
}

bilu_status capture(bilu_uneven_plan* U, const double* vals, const double* rhs, double* x, const bilu_results* R) {
  drop_graph(U);
  const int nb = (int)U->buckets.size();
  // kernel attributes are set outside the capture
  for (int bi = 0; bi < nb; ++bi) {
    const Bucket& b = U->buckets[bi];
    if (b.sys.empty()) continue;
    const void* k = b.rr ? rr_uneven_kernel(rr_pv(U->opts), U->opts.factor_precision == BILU_FP32, b.R)
                         : uneven_kernel(U->opts.factor_precision == BILU_FP32, U->opts.reduction == BILU_REDUCE_FAST,
                                         b.maxl);
    // register-resident buckets can share a kernel with different layouts: allow the device maximum
    // (the kernel has no static shared memory) and launch with b.smem; the persistent kernel keeps b.smem
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         b.rr ? (int)solve_max_smem() : b.smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
  }
  cudaError_t e = cudaStreamBeginCapture(U->cap, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
  bilu_status st = BILU_OK;
  e = cudaMemsetAsync(U->d_counters, 0, sizeof(int) * nb, U->cap);
  if (e == cudaSuccess) e = cudaEventRecord(U->ev[0], U->cap);
  // the biggest systems' bucket first; every bucket on its own branch
  for (int bi = nb - 1; bi >= 0 && e == cudaSuccess && st == BILU_OK; --bi) {
    e = cudaStreamWaitEvent(U->side[bi], U->ev[0], 0);
    if (e != cudaSuccess) break;
    st = launch_bucket(U, bi, vals, rhs, x, R, U->side[bi]);
    if (st) break;
    e = cudaEventRecord(U->ev[1 + bi], U->side[bi]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(U->cap, U->ev[1 + bi], 0);
  }
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(U->cap, &g);
  if (st) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return cuda_fail(e, "graph capture");
  }
  if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
  U->graph = g;
  e = cudaGraphInstantiate(&U->exec, g, 0);
  if (e != cudaSuccess) {
    drop_graph(U);
    return cuda_fail(e, "cudaGraphInstantiate");
  }
  const void* k[8] = {vals, rhs, x, R ? R->iter_counts : nullptr, R ? R->conv_flags : nullptr,
                      R ? R->iter_res_norms : nullptr, R ? R->true_res_norms : nullptr, R ? R->status : nullptr};
  std::memcpy(U->key, k, sizeof(k));
  return BILU_OK;
}

}  // namespace

extern "C" {

bilu_status bilu_uneven_plan_create(bilu_uneven_plan** out, int nsys, const int* h_sys_n, const int* h_sys_nnz,
                                    const int* h_row_ptrs, const int* h_col_idxs, const bilu_options* opts) {
  if (!out) return set_error(BILU_ERR_INVALID, "bilu_uneven_plan_create: out is NULL");
  *out = nullptr;
  if (nsys < 0 || (nsys > 0 && (!h_sys_n || !h_sys_nnz || !h_row_ptrs || !h_col_idxs)))
    return set_error(BILU_ERR_INVALID, "bilu_uneven_plan_create: bad arguments");
  bilu_options o;
  if (opts)
    o = *opts;
  else
    bilu_default_options(&o);
  if (o.precond != BILU_PRECOND_ILU0 && o.precond != BILU_PRECOND_NONE)
    return set_error(BILU_ERR_INVALID, "uneven batches support BILU_PRECOND_ILU0 (merged) and BILU_PRECOND_NONE");
  if (o.ilu_approach < 1 || o.ilu_approach > 4) return set_error(BILU_ERR_INVALID, "ilu_approach must be 1..4");
  std::vector<long long> roff(nsys + 1, 0), zoff(nsys + 1, 0);
  for (int s = 0; s < nsys; ++s) {
    if (h_sys_n[s] <= 0 || h_sys_nnz[s] < 0) return set_error(BILU_ERR_INVALID, "bad system size");
    roff[s + 1] = roff[s] + h_sys_n[s];
    zoff[s + 1] = zoff[s] + h_sys_nnz[s];
  }
  // per-system analysis
  struct Meta {
    std::vector<int> rp, ci, diag, llp, llr, lup, lur, dp, dep, tlh, tl, tuh, tu, ih, ip;
    int maxw = 0, maxl = 0;
    int err = 0;
  };
  std::vector<Meta> M(nsys);
#pragma omp parallel for schedule(dynamic, 8)
  for (int s = 0; s < nsys; ++s) {
    Meta& m = M[s];
    const int n = h_sys_n[s];
    const int* rp = h_row_ptrs + roff[s] + s;
    const int* ci = h_col_idxs + zoff[s];
    if (rp[0] != 0 || rp[n] != h_sys_nnz[s]) {
      m.err = 1;
      continue;
    }
    m.rp.assign(rp, rp + n + 1);
    m.ci.assign(ci, ci + h_sys_nnz[s]);
    m.diag.assign(n, -1);
    for (int i = 0; i < n && !m.err; ++i) {
      if (rp[i + 1] < rp[i]) m.err = 1;
      for (int k = rp[i]; k < rp[i + 1] && !m.err; ++k) {
        if (ci[k] < 0 || ci[k] >= n || (k > rp[i] && ci[k] <= ci[k - 1])) m.err = 1;
        if (ci[k] == i) m.diag[i] = k;
      }
      if (m.diag[i] < 0 && o.precond == BILU_PRECOND_ILU0) m.err = 2;
      m.maxl = std::max(m.maxl, rp[i + 1] - rp[i]);
    }
    if (m.err) continue;
    if (o.precond == BILU_PRECOND_ILU0) {
      int wl = 0, wu = 0;
      pattern_levels(n, rp, ci, m.diag.data(), m.llp, m.llr, wl, m.lup, m.lur, wu);
      m.maxw = std::max(wl, wu);
      pattern_deps(n, rp, ci, m.diag.data(), m.dp, m.dep);
      if (n <= 1024 && o.reduction == BILU_REDUCE_FAST) {
        build_trsv_program(rp, ci, m.diag.data(), m.llp, m.llr, false, m.tlh, m.tl);
        build_trsv_program(rp, ci, m.diag.data(), m.lup, m.lur, true, m.tuh, m.tu);
        // no ILU(0) program: on these random patterns the rows carry many dependency pairs, most ops
        // fall outside the prefetched words, and the program form measured 10 % slower than ilu_rows
      }
    }
  }
  for (int s = 0; s < nsys; ++s) {
    if (M[s].err == 1) return set_error(BILU_ERR_PATTERN, "system " + std::to_string(s) + ": invalid CSR pattern");
    if (M[s].err == 2)
      return set_error(BILU_ERR_PATTERN, "system " + std::to_string(s) +
                                             ": missing diagonal entry (the merged ILU(0) solver requires it)");
  }
  if (bilu_device_count() == 0) return set_error(BILU_ERR_NO_DEVICE, "no CUDA device");
  bilu_uneven_plan* U = new bilu_uneven_plan();
  U->opts = o;
  U->nsys = nsys;
  U->total_rows = roff[nsys];
  U->total_nnz = zoff[nsys];
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&U->nsm, cudaDevAttrMultiProcessorCount, dev);
  // concatenate metadata
  std::vector<int> meta;
  auto put = [&](const std::vector<int>& v) {
    while (meta.size() % 4) meta.push_back(0);
    const int off = (int)meta.size();
    meta.insert(meta.end(), v.begin(), v.end());
    if (v.empty()) meta.push_back(0);
    return off;
  };
  U->desc.resize(nsys);
  for (int s = 0; s < nsys; ++s) {
    Meta& m = M[s];
    SysDesc& d = U->desc[s];
    d.n = h_sys_n[s];
    d.nnz = h_sys_nnz[s];
    d.maxw = std::max(m.maxw, 1);
    d.maxl = m.maxl;
    d.nlev_lo = m.llp.empty() ? 0 : (int)m.llp.size() - 1;
    d.nlev_up = m.lup.empty() ? 0 : (int)m.lup.size() - 1;
    d.val_off = zoff[s];
    d.vec_off = roff[s];
    d.o_rp = put(m.rp);
    d.o_ci = put(m.ci);
    d.o_diag = put(m.diag);
    d.o_llp = put(m.llp);
    d.o_llr = put(m.llr);
    d.o_lup = put(m.lup);
    d.o_lur = put(m.lur);
    d.o_dp = put(m.dp);
    d.o_dep = put(m.dep);
    d.o_tlh = put(m.tlh);
    d.o_tl = put(m.tl);
    d.o_tuh = put(m.tuh);
    d.o_tu = put(m.tu);
    d.o_ih = m.ip.empty() ? -1 : put(m.ih);
    d.o_ip = m.ip.empty() ? -1 : put(m.ip);
    m = Meta();  // release the per-system copies
  }
  if (meta.size() > (size_t)0x7fffffff) {
    delete U;
    return set_error(BILU_ERR_CAPACITY, "uneven batch metadata exceeds 2^31 entries");
  }
  // size buckets (n in (lo, hi]).  FAST order: edges a factor of about sqrt(2)
  // apart, because a register-resident bucket launches every system with the
  // threads and shared memory of its largest one
  const bool fp32 = o.factor_precision == BILU_FP32;
  const bool fast = o.reduction == BILU_REDUCE_FAST;
  const std::vector<int> edges = fast ? std::vector<int>{0, 64, 96, 128, 192, 256, 384, 512, 768, 1024, 1 << 30}
                                      : std::vector<int>{0, 128, 256, 512, 1024, 1 << 30};
  const int budget = (int)solve_max_smem();
  for (size_t e = 0; e + 1 < edges.size(); ++e) {
    Bucket b;
    b.lo = edges[e];
    b.hi = edges[e + 1];
    U->buckets.push_back(b);
  }
  for (int s = 0; s < nsys; ++s)
    for (auto& b : U->buckets)
      if (h_sys_n[s] > b.lo && h_sys_n[s] <= b.hi) b.sys.push_back(s);
  std::vector<int> order;
  for (auto& b : U->buckets) {
    std::sort(b.sys.begin(), b.sys.end(), [&](int a, int c) {
      return (long long)h_sys_nnz[a] * h_sys_n[a] > (long long)h_sys_nnz[c] * h_sys_n[c];
    });
    b.order_off = (int)order.size();
    order.insert(order.end(), b.sys.begin(), b.sys.end());
    for (int s : b.sys) {
      const SmemLayout L = layout_for(h_sys_n[s], h_sys_nnz[s], h_sys_nnz[s], prec_kind_uneven(o), fp32, fast, 0, 0,
                                      budget);
      b.smem = std::max(b.smem, L.total);
      b.maxl = std::max(b.maxl, U->desc[s].maxl);
      b.maxn = std::max(b.maxn, h_sys_n[s]);
    }
    // FAST order: the register-resident solver's layout for every system of the bucket
    if (fast && !b.sys.empty() && b.maxn <= 1024) {
      int rest = 0;
      for (int s : b.sys)
        rest = std::max(rest, rr_layout_base(h_sys_n[s], h_sys_nnz[s], rr_pv(o), fp32, true, 0).total - rr_red_bytes(0));
      b.rr = true;
      b.rr_rest = rest;  // rr_setup checks the total for its CTA size
    }
    if (b.smem > budget) {
      const int need = b.smem;
      delete U;
      return set_error(BILU_ERR_CAPACITY, "an uneven-batch system needs " + std::to_string(need) +
                                              " bytes of shared memory");
    }
    // default CTA size before autotuning: one thread per row of the largest system
    b.threads = std::min(1024, round32(std::max(b.maxn, 64)));
  }
  cudaError_t e = cudaMalloc((void**)&U->d_meta, meta.size() * sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(U->d_meta, meta.data(), meta.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc((void**)&U->d_desc, std::max<size_t>(1, U->desc.size()) * sizeof(SysDesc));
  if (e == cudaSuccess && nsys)
    e = cudaMemcpy(U->d_desc, U->desc.data(), U->desc.size() * sizeof(SysDesc), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc((void**)&U->d_order, std::max<size_t>(1, order.size()) * sizeof(int));
  if (e == cudaSuccess && !order.empty())
    e = cudaMemcpy(U->d_order, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc((void**)&U->d_counters, U->buckets.size() * sizeof(int));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&U->cap, cudaStreamNonBlocking);
  for (size_t i = 0; i < U->buckets.size() && e == cudaSuccess; ++i) {
    cudaStream_t s2;
    e = cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking);
    if (e == cudaSuccess) U->side.push_back(s2);
  }
  for (size_t i = 0; i < U->buckets.size() + 1 && e == cudaSuccess; ++i) {
    cudaEvent_t ev;
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) U->ev.push_back(ev);
  }
  if (e != cudaSuccess) {
    bilu_status st = cuda_fail(e, "uneven plan upload");
    bilu_uneven_plan_destroy(U);
    return st;
  }
  for (auto& b : U->buckets) {
    if (b.sys.empty()) continue;
    if (b.rr) {
      // default: the fewest warps that give the largest system 8 rows per thread
      if (!rr_setup(U, b, round32((b.maxn + 7) / 8))) {
        b.rr = false;  // back to the shared-memory kernel and its layout
        b.smem = 0;
        for (int s : b.sys)
          b.smem = std::max(b.smem, layout_for(h_sys_n[s], h_sys_nnz[s], h_sys_nnz[s], prec_kind_uneven(o), fp32,
                                               fast, 0, 0, budget).total);
        b.threads = std::min(1024, round32(std::max(b.maxn, 64)));
      }
    }
    if (!b.rr) b.grid = occupancy_grid(U, b, b.threads);
  }
  *out = U;
  return BILU_OK;
}

bilu_status bilu_uneven_plan_destroy(bilu_uneven_plan* U) {
  if (!U) return BILU_OK;
  drop_graph(U);
  for (auto s : U->side) cudaStreamDestroy(s);
  for (auto ev : U->ev) cudaEventDestroy(ev);
  if (U->cap) cudaStreamDestroy(U->cap);
  cudaFree(U->d_meta);
  cudaFree(U->d_desc);
  cudaFree(U->d_order);
  cudaFree(U->d_counters);
  delete U;
  return BILU_OK;
}

bilu_status bilu_uneven_autotune(bilu_uneven_plan* U, const double* d_values, const double* d_b, double* d_x,
                                 void* stream) {
  if (!U || (U->nsys > 0 && (!d_values || !d_b || !d_x)))
    return set_error(BILU_ERR_INVALID, "bilu_uneven_autotune: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int cands[] = {64, 128, 256, 512, 1024};
  bilu_status res = BILU_OK;
  // Persistent shared-memory buckets (reference order): each CTA size timed on the bucket alone.
  for (int bi = 0; bi < (int)U->buckets.size() && !res; ++bi) {
    Bucket& b = U->buckets[bi];
    if (b.sys.empty() || b.rr) continue;
    int best_t = b.threads, best_g = b.grid;
    float best = 1e30f;
    for (int t : cands) {
      const int g = occupancy_grid(U, b, t);
      if (g <= 0) continue;
      Bucket trial = b;
      trial.threads = t;
      trial.grid = g;
      std::swap(U->buckets[bi], trial);
      float ms_min = 1e30f;
      for (int rep = 0; rep < 2 && !res; ++rep) {
        cudaMemsetAsync(U->d_counters + bi, 0, sizeof(int), st);
        cudaEventRecord(e0, st);
        res = launch_bucket(U, bi, d_values, d_b, d_x, nullptr, st);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ms_min = std::min(ms_min, ms);
      }
      std::swap(U->buckets[bi], trial);
      if (res) break;
      if (ms_min < best) {
        best = ms_min;
        best_t = t;
        best_g = g;
      }
    }
    b.threads = best_t;
    b.grid = best_g;
    b.tuned_ms = best;
  }
  // Register-resident buckets (FAST order): the bucket launches run concurrently in the solve's graph, so a
  // bucket's configuration is judged by the whole graph-launched batch, not by the bucket alone.  Measured
  // on GB300 with the 8192-system benchmark batch: timed alone, the persistent grid won for four of nine
  // buckets and larger CTAs for several, and together those choices made the batch slower than the
  // untuned plan.  One greedy pass over the buckets, largest systems first: each tries 1x, 2x and 4x the
  // fewest threads, each with one CTA per system and with the persistent grid over its work queue, and
  // keeps whatever makes the whole batch fastest (best of three graph launches per candidate).
  auto whole = [&](float* out) -> bilu_status {
    bilu_status r = capture(U, d_values, d_b, d_x, nullptr);
    float best_ms = 1e30f;
    for (int rep = 0; rep < 3 && !r; ++rep) {
      cudaEventRecord(e0, st);
      cudaError_t ce = cudaGraphLaunch(U->exec, st);
      cudaEventRecord(e1, st);
      if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
      if (ce != cudaSuccess) r = cuda_fail(ce, "autotune graph launch");
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      best_ms = std::min(best_ms, ms);
    }
    *out = best_ms;
    return r;
  };
  bool any_rr = false;
  for (const Bucket& b : U->buckets) any_rr = any_rr || (b.rr && !b.sys.empty());
  float base = 0.0f;
  if (any_rr && !res) res = whole(&base);
  for (int bi = (int)U->buckets.size() - 1; bi >= 0 && any_rr && !res; --bi) {
    Bucket& b = U->buckets[bi];
    if (!b.rr || b.sys.empty()) continue;
    const Bucket keep = b;
    Bucket best_cfg = b;
    const int rr_base = round32((b.maxn + 7) / 8);
    for (int f : {1, 2, 4}) {
      Bucket trial = keep;
      if (!rr_setup(U, trial, f * rr_base)) continue;
      const int pgrid = rr_persistent_grid(U, trial);
      for (int g : {trial.grid, pgrid}) {
        if (g == pgrid && pgrid >= trial.grid) continue;  // the persistent grid is one CTA per system anyway
        if (f * rr_base == keep.threads && g == keep.grid) continue;  // the configuration already timed
        Bucket cfg = trial;
        cfg.grid = g;
        b = cfg;
        float ms = 0.0f;
        res = whole(&ms);
        if (res) break;
        if (ms < base) {
          base = ms;
          best_cfg = cfg;
        }
      }
      if (res) break;
    }
    b = best_cfg;
    b.tuned_ms = base;  // the whole batch with this bucket's choice
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  drop_graph(U);  // the captured graph used the previous configuration
  cudaError_t e = cudaGetLastError();
  if (!res && e != cudaSuccess) return cuda_fail(e, "autotune");
  return res;
}

bilu_status bilu_uneven_solve(bilu_uneven_plan* U, const double* d_values, const double* d_b, double* d_x,
                              const bilu_results* R, void* stream) {
  if (!U || (U->nsys > 0 && (!d_values || !d_b || !d_x))) return set_error(BILU_ERR_INVALID, "bilu_uneven_solve: bad arguments");
  if (U->nsys == 0) return BILU_OK;
  const void* k[8] = {d_values, d_b, d_x, R ? R->iter_counts : nullptr, R ? R->conv_flags : nullptr,
                      R ? R->iter_res_norms : nullptr, R ? R->true_res_norms : nullptr, R ? R->status : nullptr};
  if (!U->exec || std::memcmp(k, U->key, sizeof(k)) != 0) {
    bilu_status st = capture(U, d_values, d_b, d_x, R);
    if (st) return st;
  }
  cudaError_t e = cudaGraphLaunch(U->exec, (cudaStream_t)stream);
  return e == cudaSuccess ? BILU_OK : cuda_fail(e, "cudaGraphLaunch");
}

bilu_status bilu_uneven_set_config(bilu_uneven_plan* U, int bucket, int threads, int grid) {
  if (!U) return set_error(BILU_ERR_INVALID, "bilu_uneven_set_config: NULL plan");
  if (bucket < 0 || bucket >= (int)U->buckets.size()) return set_error(BILU_ERR_INVALID, "bucket out of range");
  if (threads < 0 || grid < 0) return set_error(BILU_ERR_INVALID, "bilu_uneven_set_config: negative size");
  Bucket& b = U->buckets[bucket];
  if (b.sys.empty()) return BILU_OK;
  const int count = (int)b.sys.size();
  if (b.rr) {
    Bucket trial = b;
    if (!rr_setup(U, trial, threads > 0 ? threads : b.threads))
      return set_error(BILU_ERR_INVALID, "bilu_uneven_set_config: " + std::to_string(threads) +
                                             " threads do not fit this bucket's register-resident solver");
    trial.grid = grid > 0 ? std::min(grid, count) : count;
    b = trial;
  } else {
    const int t = threads > 0 ? threads : b.threads;
    const int g = occupancy_grid(U, b, t);
    if (t % 32 || t > 1024 || g <= 0)
      return set_error(BILU_ERR_INVALID, "bilu_uneven_set_config: " + std::to_string(t) + " threads do not fit");
    b.threads = t;
    b.grid = grid > 0 ? std::min(grid, g) : g;
  }
  b.tuned_ms = -1.0f;
  drop_graph(U);  // the captured graph used the previous configuration
  return BILU_OK;
}

bilu_status bilu_uneven_get_info(const bilu_uneven_plan* U, int bucket, int* n_lo, int* n_hi, int* systems,
                                 int* threads, int* grid, int* smem_bytes, float* tuned_ms) {
  if (!U) return set_error(BILU_ERR_INVALID, "bilu_uneven_get_info: NULL plan");
  if (bucket < 0 || bucket >= (int)U->buckets.size()) return set_error(BILU_ERR_INVALID, "bucket out of range");
  const Bucket& b = U->buckets[bucket];
  if (n_lo) *n_lo = b.lo;
  if (n_hi) *n_hi = b.hi;
  if (systems) *systems = (int)b.sys.size();
  if (threads) *threads = b.threads;
  if (grid) *grid = b.grid;
  if (smem_bytes) *smem_bytes = b.smem;
  if (tuned_ms) *tuned_ms = b.tuned_ms;
  return BILU_OK;
}

}  // extern "C"
