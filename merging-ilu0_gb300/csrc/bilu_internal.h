// Internal declarations shared by the host plan code (bilu_plan.cpp) and the
// CUDA kernels (k_*.cu).  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "bilu.h"

namespace bilu {

// entries per row of a triangular-solve program that the register-resident
// solver loads one level ahead (the rest it loads when it needs them)
constexpr int kTrsvPrefetch = 4;
// op words per row of an ILU(0) program loaded one level ahead
constexpr int kIluPrefetch = 16;

// learned warm start: 9 features -> 64 -> 64 -> 1
constexpr int kMlpFeatures = 9;
constexpr int kMlpHidden = 64;
constexpr int kMlpParams = kMlpHidden * kMlpFeatures + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden + kMlpHidden + 1;

// Records the message for bilu_last_error() and returns the code.
bilu_status set_error(bilu_status code, const std::string& msg);

// pattern analysis shared by the plans (bilu_plan.cu)
void pattern_levels(int n, const int* rp, const int* ci, const int* diag, std::vector<int>& lo_ptr,
                    std::vector<int>& lo_rows, int& maxw_lo, std::vector<int>& up_ptr, std::vector<int>& up_rows,
                    int& maxw_up);
void pattern_deps(int n, const int* rp, const int* ci, const int* diag, std::vector<int>& dep_ptr,
                  std::vector<int>& dep);
size_t solve_max_smem();

// Device views of one pattern plan (all pointers into one device allocation).
struct DevPattern {
  int n = 0, nnz = 0;
  // operator pattern = the caller's pattern (SpMV with A, true residual)
  int a_nnz = 0;
  const int* a_rp = nullptr;
  const int* a_ci = nullptr;
  int a_maxl = 0;               // longest row of the operator pattern
  const int* rp = nullptr;      // n+1   factor pattern (A with diagonals)
  const int* ci = nullptr;      // nnz
  const int* diag = nullptr;    // n     position of (i,i)
  const int* row_of = nullptr;  // nnz   row of each entry
  // level schedules of the unit-lower and upper triangular solves
  int nlev_lo = 0, nlev_up = 0, maxw_lo = 0, maxw_up = 0;
  const int* lev_lo_ptr = nullptr;   // nlev_lo+1
  const int* lev_lo_rows = nullptr;  // n (rows in level order)
  const int* lev_up_ptr = nullptr;
  const int* lev_up_rows = nullptr;
  // factorisation dependencies per entry: pairs (pos l_ik, pos u_kj) with k
  // ascending, k < min(i, j)
  const int* dep_ptr = nullptr;  // nnz+1
  const int2* dep = nullptr;     // ndep
  // ISAI patterns and per-row solve programs
  int ail_nnz = 0, aiu_nnz = 0;
  const int* ail_rp = nullptr;
  const int* ail_ci = nullptr;
  const int* aiu_rp = nullptr;
  const int* aiu_ci = nullptr;
  // program per ISAI row: blocks {t, k} followed by k entries {c, pos}; rows
  // in blocks of 32, word j of row 32b+l at prog[prog_ptr[b] + 32j + l]
  // ISAI thread slot -> row: rows by program length, longest first, so a
  // warp's 32 slots run programs of about the same length; the programs are
  // warp-blocked in slot order
  const int* ail_perm = nullptr;
  const int* aiu_perm = nullptr;
  const int* ail_prog_ptr = nullptr;  // (n+31)/32 + 1 block offsets (words)
  const int* ail_prog = nullptr;      // words t | count << 5 and c | pos << 5 (build_isai)
  const int* aiu_prog_ptr = nullptr;
  const int* aiu_prog = nullptr;
  int l_diag = 0;  // 1: aiL divides by the stored diagonal of a lower triangular matrix
  // general ISAI: per row the sz*sz positions of A(J_k, J_t) in the factor
  // pattern (row-major over k, -1 = structural zero), and the position of i in J
  int gen_maxs = 0;
  const int* gen_map_ptr = nullptr;  // n+1
  const int* gen_map = nullptr;
  const int* gen_pos = nullptr;      // n
  // input -> factor pattern value map (src index or -1 for inserted diagonals)
  int nnz_in = 0;
  const int* src_map = nullptr;  // nnz
  // reference L / U split maps: factor position of each L / U entry (-1 = unit diagonal)
  int nnz_L = 0, nnz_U = 0;
  const int* l_src = nullptr;
  const int* u_src = nullptr;
  // triangular-solve programs of the register-resident solver (n <= 1024),
  // one per triangle.  Level l: header {off, w}; at prog[off + s] the record
  // of slot s < w, row | count << 10; at prog[off + w + j*w + s] its entry j,
  // k << 10 | column, in summation order (lower ascending, upper descending k);
  // every level has at least kTrsvPrefetch entry rows (padding reads as 0).
  const int2* tp_lo_hdr = nullptr;
  const int* tp_lo = nullptr;
  const int2* tp_up_hdr = nullptr;
  const int* tp_up = nullptr;
  // the most entries of any row of the lower / upper solve program (the
  // solves run no product slot past it); kTrsvPrefetch when not known
  int tp_maxcnt_lo = kTrsvPrefetch, tp_maxcnt_up = kTrsvPrefetch;
  // ILU(0) program of the register-resident solver's merged form (n <= 1024),
  // per lower level: header {off, w, len, 0}; slot s word j at prog[off + j*w + s]:
  // word 0 = number of op words that follow; ops per entry k of the row in
  // column order (upper entries without pairs, exact no-ops, left out):
  // k | pairs << 20 | lower << 30, then for a lower entry the diagonal position
  // of its column, then the pairs (l position, u position) in summation order.
  // Every level has at least kIluPrefetch + 1 words per slot.
  const int4* ilu_hdr = nullptr;
  const int* ilu_prog = nullptr;
  int ilu_prog_approach = 0;  // the approach (1..4) whose pair order the program holds
  // 16-bit copies of the column indices read by the register-resident solver's
  // SpMVs (n <= 65535): half the L1 footprint of the int32 arrays
  const unsigned short* a_ci16 = nullptr;
  const unsigned short* ail_ci16 = nullptr;
  const unsigned short* aiu_ci16 = nullptr;
  const unsigned short* sa_ci16 = nullptr;
  const unsigned short* su_ci16 = nullptr;
  // SELL-32 copies for the register-resident solver's SpMVs, of A (sa_*) and of
  // aiU (su_*): slice s holds rows 32s .. 32s+31, entry j of row 32s+l at
  // off[s] + 32j + l, so a warp's 32 rows read one contiguous line per entry;
  // src = the CSR position each SELL position copies (-1: padding, never read)
  int sa_nnz = 0, su_nnz = 0;
  const int* sa_off = nullptr;
  const int* sa_ci = nullptr;
  const int* sa_src = nullptr;
  const int* su_off = nullptr;
  const int* su_ci = nullptr;
  const int* su_src = nullptr;
  // per row: lower-solve level; per entry: position of the transposed entry or -1
  const int* row_lev = nullptr;
  const int* tpos = nullptr;
  // entries whose converged ParILU value is not simply a_ij (all but the upper
  // entries without dependency pairs): the ones the learned warm start predicts
  int n_mlp = 0;
  const int* mlp_ent = nullptr;
  // ParILU sweep order: entries with dependency pairs on or above the diagonal,
  // then those below it (each most pairs first), then lower entries without
  // pairs (l = a / u_jj), then upper entries without pairs (u = a); warps of
  // one class do the same operations, so no FP64 instruction of another class
  // is issued predicated off (which still costs its FP64-unit slot on GB300)
  const int* pl_ent = nullptr;  // nnz
  int pl_ndep = 0, pl_nlow = 0;
  int pl_ndep_low = 0;  // the last pl_ndep_low of the pl_ndep entries with pairs are below the diagonal
  // the entries with dependency pairs as a warp-blocked program: slot q
  // (= pl_ent position q < pl_ndep) holds the words k, j << 1 | (j < i), the
  // pair count, then x, y per pair (sum order); word w of slot 32b + l at
  // pl_prog[pl_prog_ptr[b] + 32 w + l], so a warp's loads are contiguous and
  // none waits on another
  const int* pl_prog_ptr = nullptr;
  const int* pl_prog = nullptr;
};

// Shared-memory carve-up of the solver kernel for one system (byte offsets;
// -1 = operand read from global memory instead).
struct SmemLayout {
  int A = -1;      // double[nnz]
  int F = -1;      // factors: FT[nnz]
  int ail = -1;    // FT[ail_nnz]
  int aiu = -1;    // FT[aiu_nnz]
  int rinv = -1;   // double[n] (FP64) / float[n] (FP32)
  int vec = -1;    // 7 double vectors of n (x, r/s, r_hat, p, v, t, p_hat/s_hat)
  int fvec = -1;   // 2 float vectors of n (FP32 preconditioner scratch)
  int tmpv = -1;   // 1 double vector of n (ISAI intermediate / ILU scratch)
  int red = -1;    // 64 doubles of scalars
  int total = 0;
};

enum PrecKind : int {
  PK_ILU_INKERNEL = 0,  // factorise inside the solver kernel (merged)
  PK_LU_GLOBAL = 1,     // in-place factors given in global memory
  PK_ISAI = 2,          // aiL / aiU given in global memory
  PK_NONE = 3,
};

struct SolveArgs {
  DevPattern pat;
  SmemLayout lay;
  int nsys = 0;
  const double* A = nullptr;   // nsys*a_nnz, operator (caller's) pattern
  const double* b = nullptr;
  double* x = nullptr;
  const double* A_sell = nullptr;  // A in the SELL-32 layout (register-resident solver; null: CSR)
  const void* aiu_sell = nullptr;  // aiU in the SELL-32 layout (register-resident solver; null: CSR)
  const void* F = nullptr;     // PK_LU_GLOBAL factors (double or float)
  const void* ail = nullptr;   // PK_ISAI
  const void* aiu = nullptr;
  float* iters = nullptr;
  int* conv = nullptr;
  double* res = nullptr;
  int* status = nullptr;
  double* true_res = nullptr;  // fused true-residual epilogue when non-null
  double tol = 1e-11;
  int tol_mode = BILU_TOL_ABS;
  int max_iter = 500;
  int prec = PK_ILU_INKERNEL;
  int approach = 1;
  int dot_serial = 0;  // 1: serial inner products (ISAI solver family, reference order)
};

// Shared-memory carve-up for one system; the same on host (plan creation)
// and device (persistent kernel, per system).  Mandatory: scalars, 7 FP64
// vectors (x, r/s, r_hat, p, v, t, p_hat/s_hat), FP32 preconditioner
// scratch, ISAI intermediate, diagonal reciprocals; then, most re-used
// first, factors or ISAI values and A while they fit in `budget`.
__host__ __device__ inline SmemLayout layout_for(int n, int annz, int fnnz, int pk, bool fp32, bool fast,
                                                 int ail_nnz, int aiu_nnz, int budget) {
  SmemLayout L;
  int off = 0;
  const int fts = fp32 ? 4 : 8;
  const bool lu = (pk == PK_ILU_INKERNEL || pk == PK_LU_GLOBAL);
#define BILU_TAKE(dst, bytes) \
  do {                        \
    (dst) = off;              \
    off = (off + (bytes) + 15) & ~15; \
  } while (0)
  BILU_TAKE(L.red, 128);
  int vecd = 7 * n;
  if (pk == PK_ILU_INKERNEL && fp32 && fnnz > vecd) vecd = fnnz;  // FP64 factorisation scratch
  BILU_TAKE(L.vec, vecd * 8);
  if (fp32) BILU_TAKE(L.fvec, 2 * n * 4);
  if (pk == PK_ISAI && !fp32) BILU_TAKE(L.tmpv, n * 8);
  if (lu && (fp32 || fast)) BILU_TAKE(L.rinv, n * fts);
  if (lu) {
    if (pk == PK_ILU_INKERNEL || off + fnnz * fts <= budget) BILU_TAKE(L.F, fnnz * fts);
  } else if (pk == PK_ISAI) {
    if (off + ail_nnz * fts <= budget) BILU_TAKE(L.ail, ail_nnz * fts);
    if (off + aiu_nnz * fts <= budget) BILU_TAKE(L.aiu, aiu_nnz * fts);
  }
  if (off + annz * 8 <= budget) BILU_TAKE(L.A, annz * 8);
#undef BILU_TAKE
  L.total = off;
  return L;
}

// Triangular-solve program of one triangle (DevPattern::tp_*) from its level
// schedule (n <= 1024): header pairs {off, w} per level and the slot words.
void build_trsv_program(const int* rp, const int* ci, const int* diag, const std::vector<int>& lptr,
                        const std::vector<int>& lrows, bool upper, std::vector<int>& hdr, std::vector<int>& prog);
// ILU(0) program (DevPattern::ilu_*) of the factor pattern for one approach (1..4).
void build_ilu_program(const int* rp, const int* ci, const int* diag, const std::vector<int>& lptr,
                       const std::vector<int>& lrows, const std::vector<int>& dep_ptr, const std::vector<int>& dep,
                       int approach, std::vector<int>& hdr, std::vector<int>& prog);

// Shared-memory carve-up of the register-resident FAST solver (k_solve_rr.cu):
// reduction slots, the SpMV input (FP64), the preconditioner input and
// intermediate (FT), for LU preconditioners the in-place factors (FP64 while
// the kernel factorises, FT after) and the diagonal reciprocals, then
// optionally A and the ISAI values.  -1 = not used / read from global memory.
struct RRLayout {
  int red = -1, ph = -1, in = -1, mid = -1, F = -1, rinv = -1, A = -1, ail = -1, aiu = -1, total = 0;
};

// Bytes of the reduction slot of an nt-thread CTA: two partial sums per
// thread and 16 broadcast scalars.
__host__ __device__ inline int rr_red_bytes(int nt) { return (2 * nt + 16) * 8; }

// The mandatory part of an RRLayout (no optional staging) for nt threads, the
// same on host and device: pv 0 none, 1 two-triangle ISAI, 2 general ISAI, 3
// ILU factors (inkernel: the FP64 factorisation slot of the merged form).  The
// reduction slot comes first, so the rest of the layout does not depend on nt.
__host__ __device__ inline RRLayout rr_layout_base(int n, int nnz, int pv, bool fp32, bool inkernel, int nt) {
  RRLayout L;
  int off = 0;
  const int fts = fp32 ? 4 : 8;
  auto take = [&](int& dst, long long bytes) {
    dst = off;
    off = (int)((off + bytes + 15) & ~15LL);
  };
  take(L.red, rr_red_bytes(nt));
  take(L.ph, (long long)n * 8);
  if (pv == 1 || pv == 2 || (pv == 3 && fp32)) take(L.in, (long long)n * fts);
  if (pv == 1) take(L.mid, (long long)n * fts);
  if (pv == 3) {
    take(L.F, (long long)nnz * (inkernel ? 8 : fts));
    take(L.rinv, (long long)n * fts);
  }
  L.total = off;
  return L;
}

// One system of an uneven batch (own size and pattern); offsets in ints into
// the plan's metadata buffer, value / vector offsets into the concatenated
// batch arrays.
struct SysDesc {
  int n, nnz, maxw, maxl;
  int nlev_lo, nlev_up;
  long long val_off, vec_off;
  int o_rp, o_ci, o_diag, o_llp, o_llr, o_lup, o_lur, o_dp, o_dep;
  int o_tlh, o_tl, o_tuh, o_tu;  // triangular-solve programs (n <= 1024; else 0)
  int o_ih, o_ip;                // ILU(0) program (n <= 1024; else 0)
};

struct UnevenArgs {
  SolveArgs base;            // tolerance, options, concatenated A / b / x, result arrays
  const SysDesc* desc = nullptr;
  const int* meta = nullptr;
  const int* order = nullptr;  // systems of this bucket, longest first
  int count = 0;
  int* counter = nullptr;      // work-queue head (zeroed before each launch)
  int smem_budget = 0;         // dynamic shared memory of the launch
};

// kernel launch wrappers (k_solve.cu / k_factor.cu)
// register-resident solver over one uneven-batch bucket with nt threads, R rows
// per thread (pv 0 none, 3 merged ILU(0)): CTA b solves system order[b]
// (grid = the bucket's systems), or a persistent grid of fewer CTAs takes the
// systems from the bucket's work queue (u.counter, zeroed before the launch)
const void* rr_uneven_kernel(int pv, int fp32, int R);
cudaError_t launch_uneven_rr(const UnevenArgs& u, int nt, int R, int pv, int fp32, int grid, cudaStream_t st);
void* uneven_kernel(int fp32, int reduce_fast, int maxl);
cudaError_t launch_uneven(const UnevenArgs& u, int threads, int grid, int fp32, int reduce_fast, int maxl,
                          cudaStream_t st);
cudaError_t launch_solve(const SolveArgs& a, int threads, int fp32, int reduce_fast, int maxl, cudaStream_t st);
// register-resident solver: pv 0 none, 1 ISAI of L and U, 2 general ISAI, 3 ILU factors;
// ref: the reference's operation order; occ: the occupancy variant (k_bicgstab_rr_occ: R = 2, 4, 8;
// ILU factors at R = 2, 4)
int rr_rows_per_thread(int n, int nt);  // smallest R in {1, 2, 4, 8} with R * nt >= n, else 0
int rr_max_threads(int R);
const void* rr_kernel(int pv, int fp32, int R, int ref, int occ);  // null: no such variant
// the occupancy variant (k_bicgstab_rr_occ, k_solve_rr_occ.cu) for R rows per thread; null: none
const void* rr_occ_kernel(int pv, int fp32, int R);
cudaError_t launch_solve_rr(const SolveArgs& a, const RRLayout& L, int nt, int pv, int fp32, int ref, int occ,
                            cudaStream_t st);
size_t solve_max_smem();
cudaError_t launch_expand(const DevPattern& p, int nsys, const double* vin, double* vout, cudaStream_t st);
cudaError_t launch_ilu0(const DevPattern& p, int nsys, const double* A, double* lu, int approach, int threads,
                        cudaStream_t st);
cudaError_t launch_parilu0(const DevPattern& p, int nsys, const double* A, const double* init, double* lu,
                           int sweeps, int threads, cudaStream_t st, double res_tol = 0.0, int* sweeps_out = nullptr,
                           double* res_out = nullptr, int fast = 0);
cudaError_t launch_isai(const DevPattern& p, int nsys, const double* lu, void* ail, void* aiu, int fp32,
                        int threads, cudaStream_t st, int fast = 0);
cudaError_t launch_dense_solve(const DevPattern& p, int nsample, const int* sys_ids, const double* A, const double* b,
                               double* work, double* x_out, cudaStream_t st);
cudaError_t launch_mlp_rowstats(const DevPattern& p, int nsys, const double* A, float* rown, float* coln, float* corr,
                                cudaStream_t st);
size_t mlp_train_smem();
cudaError_t launch_mlp_train(const DevPattern& p, int nsys, const double* A, const double* LUt, const float* rown,
                             const float* coln, const float* corr, const void* pbf, int nsample, const int* idx,
                             uint64_t seed, float* grad, float* loss, cudaStream_t st);
cudaError_t launch_mlp_adam(float* p, float* m, float* v, const float* g, void* pbf, int count, float lr, int step,
                            cudaStream_t st);
cudaError_t launch_mlp_to_bf16(const float* p, void* pbf, int count, cudaStream_t st);
cudaError_t launch_mlp_eval(const DevPattern& p, int nsys, const double* A, const float* rown, const float* coln,
                            const float* corr, const void* pbf, int nsample, const int* idx, float* feat, float* out,
                            double* base, cudaStream_t st);
cudaError_t launch_mlp_warm(const DevPattern& p, int nsys, const double* A, const float* rown, const float* coln,
                            const float* corr, const void* pbf, double threshold, double* lu0, double* res, int* used,
                            cudaStream_t st);
cudaError_t launch_to_float(const double* a, float* b, size_t n, cudaStream_t st);
// out[s][p] = in[s][src[p]] (0 where src[p] < 0) for nsys systems of csr_nnz
// values into sell_nnz positions; elem_bytes 8 (double) or 4 (float)
cudaError_t launch_to_sell(const int* src, int sell_nnz, int csr_nnz, int nsys, const void* in, void* out,
                           int elem_bytes, cudaStream_t st);
cudaError_t launch_isai_general(const DevPattern& p, int nsys, const double* A, void* ai, int fp32, int threads,
                                cudaStream_t st);
cudaError_t launch_split(const DevPattern& p, int nsys, const double* lu, double* L, double* U, cudaStream_t st);
cudaError_t launch_true_residual(const DevPattern& p, int nsys, const double* A, const double* b, const double* x,
                                 double* out, int threads, cudaStream_t st);

// Scratch of one solve (intermediate factors, ISAI values, SELL-32 copies of
// the solver's operands): 256-byte aligned byte offsets into one workspace,
// the plan's own (bilu_solve) or the library's fixed array (bilu_solve_noalloc).
struct SolveScratch {
  size_t exp = 0, lu = 0, f = 0, ail = 0, aiu = 0, asell = 0, usell = 0, total = 0;
  bool sell_a = false, sell_u = false;  // the solver reads SELL-32 copies of A / aiU made before its launch
};
SolveScratch solve_scratch_layout(const bilu_plan* P, int nsys);
// The launches of one solve (factorisation, ISAI, SELL-32 copies, solver) with
// the scratch at ws (solve_scratch_layout(P, nsys).total bytes); allocates nothing.
bilu_status solve_launch(bilu_plan* P, int nsys, const double* vals, const double* lu_init, const double* b,
                         double* x, const bilu_results* R, char* ws, const SolveScratch& sc, cudaStream_t st);
// CTA size of the factorisation and ISAI kernels for a plan
int fact_threads(const bilu_plan* P);

}  // namespace bilu

// Plan object behind the opaque bilu_plan handle of the C ABI.
struct bilu_plan {
  bilu_options opts;
  int device = 0;
  int n = 0, nnz_in = 0, nnz = 0, missing = 0;
  std::vector<int> in_rp, in_ci;      // caller's pattern
  std::vector<int> rp, ci, diag, row_of, src;
  std::vector<int> lev_lo_ptr, lev_lo_rows, lev_up_ptr, lev_up_rows;
  int maxw_lo = 0, maxw_up = 0, maxl = 0, a_maxl = 0;
  std::vector<int> dep_ptr;
  std::vector<int> dep;  // pairs
  std::vector<int> l_rp, l_ci, l_src, u_rp, u_ci, u_src;
  std::vector<int> row_lev, tpos, mlp_ent;
  std::vector<int> tp_lo_hdr, tp_lo, tp_up_hdr, tp_up;  // triangular-solve programs (DevPattern::tp_*)
  std::vector<int> ilu_hdr, ilu_prog;                    // ILU(0) program (DevPattern::ilu_*)
  std::vector<int> sa_off, sa_ci, sa_src, su_off, su_ci, su_src;  // SELL-32 layouts (DevPattern::sa_*, su_*)
  std::vector<int> pl_ent;  // ParILU entry classes (see DevPattern::pl_ent)
  int pl_ndep = 0, pl_nlow = 0, pl_ndep_low = 0;
  std::vector<int> pl_prog_ptr, pl_prog;  // ParILU program (DevPattern::pl_prog)
  bool has_isai = false;
  std::vector<int> ail_rp, ail_ci, aiu_rp, aiu_ci;
  std::vector<int> ail_prog_ptr, ail_prog, aiu_prog_ptr, aiu_prog;  // per-row programs, one word per step
  std::vector<int> ail_perm, aiu_perm;                              // ISAI slot -> row (DevPattern::ail_perm)
  bool general_isai = false;
  std::vector<int> gen_map_ptr, gen_map, gen_pos;
  int* dbuf = nullptr;
  bilu::DevPattern dp;
  // solver kernel configuration
  int threads = 0;
  bilu::SmemLayout lay;
  // register-resident FAST solver (k_solve_rr.cu), when it applies
  bool rr = false;
  int rr_threads = 0, rr_pv = 0;
  bool rr_sell = false;  // SpMVs read SELL-32 copies of A (and of aiU) made before the solver launch
  bool rr_occ = false;  // the 4-CTAs-per-SM kernel variant (staging bit 4)
  bilu::RRLayout rr_lay;
  // workspace
  void* ws = nullptr;
  size_t ws_bytes = 0;
  // stage timing events (PST / IST / OET)
  bool timing = false;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
};
