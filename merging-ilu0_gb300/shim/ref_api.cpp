// Drop-in solver interface: the five batched BiCGSTAB entry points of
// PrecondBiCGSTAB.h:15-30 and the factorisation / ISAI functions of ILU_0.h,
// parILU_0.h and isai.h (Batched-ILU0-merged/ILU0_ISAI_bicgstab), implemented
// on the bilu C ABI (include/bilu.h).  Code written against the original
// headers links against libbilu_ref.so unchanged.
//
// Entry point -> bilu preconditioner (all: x0 = 0, |r| < ATOL absolute,
// MAX_ITER iterations, reference arithmetic order):
//   Batched_ILU_Preconditioned_BiCGSTAB_Gpu           PARILU0 (sweeps) or ILU0_SPLIT (approach 1..4)
//   Batched_ILU_ISAI_Preconditioned_BiCGSTAB_Gpu      PARILU0_ISAI (sweeps) or ILU0_ISAI (approach 3), power 2
//   Batched_General_ISAI_Preconditioned_BiCGSTAB_Gpu  GENERAL_ISAI, power 1
//   Batched_conv_ILU_app1_..._merged_Gpu              ILU0 (factorised inside the solver kernel)
//   Batched_conv_ILU_app1_..._segregated_Gpu          ILU0_SPLIT approach 1 (separate factorisation)
// These are the preconditioners and powers the original helpers hard-code
// (PrecondBiCGSTAB_ilu_gpu.cu:455-469, PrecondBiCGSTAB_ilu_isai_gpu.cu:281-299,
// PrecondBiCGSTAB_general_isai_gpu.cu:261).
//
// Side effects kept: the solution is copied to the host and written as
// x_*.mtx into every subdirectory under the original file names; the
// SolverResults device arrays receive iteration counts, flags, iteration and
// true residual norms; time taken / PST / IST / OET are reported in ms.
// Timing: OET is the host wall time of the call up to the end of the solve
// (pattern read-back, plan look-up, preconditioner generation and solve, as
// the original's chrono interval), IST the solver kernel's CUDA-event time and
// PST = OET - IST.  The true residual is computed after the timed interval, as
// in the original.
//
// Plans (pattern analysis + device upload) are cached per device, pattern and
// options (8 entries, least recently used evicted), so repeated calls on one
// pattern analyse it once.  Calls are serialised by one mutex.  Failures print
// a message on stderr and throw std::runtime_error, where the original asserts.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <iostream>
#include <list>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "ILU_0.h"
#include "PrecondBiCGSTAB.h"
#include "ReadWriteData.h"
#include "SolverResults.h"
#include "bilu.h"
#include "isai.h"
#include "matrix.h"
#include "parILU_0.h"

namespace {

[[noreturn]] void fail(const std::string& where, const std::string& what) {
  const std::string msg = where + ": " + what;
  std::cerr << msg << std::endl;
  throw std::runtime_error(msg);
}

void ck(bilu_status s, const char* where) {
  if (s != BILU_OK) fail(where, bilu_last_error());
}

void ck(cudaError_t e, const char* where) {
  if (e != cudaSuccess) fail(where, cudaGetErrorString(e));
}

struct Pattern {
  int n = 0, nnz = 0;
  std::vector<int> rp, ci;
};

// the pattern as the device holds it (the host copy of a container may be stale)
Pattern device_pattern(const PagedCSRMatrices& A, const char* where) {
  if (!A.ExistsGPU()) fail(where, "matrix pages are not on the GPU");
  if (A.GetNumRows() != A.GetNumCols()) fail(where, "matrices must be square");
  Pattern p;
  p.n = A.GetNumRows();
  p.nnz = A.GetNumNz();
  p.rp.resize(p.n + 1);
  p.ci.resize(p.nnz);
  ck(cudaMemcpy(p.rp.data(), A.GetPtrToGpuRowPtrs(), sizeof(int) * (p.n + 1), cudaMemcpyDeviceToHost), where);
  if (p.nnz)
    ck(cudaMemcpy(p.ci.data(), A.GetPtrToGpuColInd(), sizeof(int) * p.nnz, cudaMemcpyDeviceToHost), where);
  return p;
}

bool same_options(const bilu_options& a, const bilu_options& b) {
  return a.precond == b.precond && a.ilu_approach == b.ilu_approach && a.parilu_sweeps == b.parilu_sweeps &&
         a.isai_power == b.isai_power && a.tol_mode == b.tol_mode && a.tol == b.tol && a.max_iter == b.max_iter &&
         a.factor_precision == b.factor_precision && a.reduction == b.reduction &&
         a.compute_true_residual == b.compute_true_residual && a.threads_per_system == b.threads_per_system &&
         a.parilu_res_tol == b.parilu_res_tol && a.isai_lower_diag == b.isai_lower_diag &&
         a.smem_staging == b.smem_staging;
}

class PlanCache {
 public:
  std::mutex mu;

  // caller holds mu
  bilu_plan* get(const Pattern& p, const bilu_options& o, const char* where) {
    int dev = 0;
    ck(cudaGetDevice(&dev), where);
    for (auto it = lru_.begin(); it != lru_.end(); ++it)
      if (it->dev == dev && it->rp == p.rp && it->ci == p.ci && same_options(it->opts, o)) {
        lru_.splice(lru_.begin(), lru_, it);
        return lru_.front().plan;
      }
    bilu_plan* plan = nullptr;
    ck(bilu_plan_create(&plan, p.n, p.nnz, p.rp.data(), p.ci.data(), &o), where);
    lru_.push_front(Entry{dev, p.rp, p.ci, o, plan});
    while (lru_.size() > kCapacity) {
      bilu_plan_destroy(lru_.back().plan);
      lru_.pop_back();
    }
    return plan;
  }

 private:
  struct Entry {
    int dev;
    std::vector<int> rp, ci;
    bilu_options opts;
    bilu_plan* plan;
  };
  static constexpr size_t kCapacity = 8;
  std::list<Entry> lru_;  // plans are released at process exit with the context
};

PlanCache& cache() {
  static PlanCache* c = new PlanCache();  // never destroyed: no CUDA calls during static teardown
  return *c;
}

bilu_options base_options(int precond) {
  bilu_options o;
  bilu_default_options(&o);
  o.precond = precond;
  o.tol_mode = BILU_TOL_ABS;
  o.tol = ATOL;
  o.max_iter = MAX_ITER;
  o.factor_precision = BILU_FP64;
  o.reduction = BILU_REDUCE_REF;
  o.compute_true_residual = 0;
  return o;
}

template <typename T>
struct DevBuf {
  T* p = nullptr;
  DevBuf(size_t count, const char* where) {
    if (count) ck(cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T)), where);
  }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};

bilu_plan_info info_of(bilu_plan* plan, const char* where) {
  bilu_plan_info info;
  ck(bilu_plan_get_info(plan, &info), where);
  return info;
}

// sets up `T` as npages pages on plan pattern `which` and uploads that pattern
void shape_pages(PagedCSRMatrices& T, bilu_plan* plan, int which, int npages, const char* where) {
  int n = 0, nnz = 0;
  ck(bilu_plan_get_pattern(plan, which, &n, &nnz, nullptr, nullptr), where);
  std::vector<int> rp(n + 1), ci(std::max(nnz, 1));
  ck(bilu_plan_get_pattern(plan, which, &n, &nnz, rp.data(), ci.data()), where);
  T.SetNumRows(n);
  T.SetNumCols(n);
  T.SetNumNz(nnz);
  T.SetNumPages(npages);
  T.AllocateMemory(LOCATION::GPU);
  ck(cudaMemcpy(T.GetPtrToGpuRowPtrs(), rp.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice), where);
  if (nnz) ck(cudaMemcpy(T.GetPtrToGpuColInd(), ci.data(), sizeof(int) * nnz, cudaMemcpyHostToDevice), where);
}

void check_batch(const char* where, const PagedCSRMatrices& A, const PagedVectors& b, const PagedVectors& x,
                 const SolverResults& res) {
  if (!A.ExistsGPU() || !b.ExistsGPU() || !x.ExistsGPU()) fail(where, "A, b and x must be allocated on the GPU");
  const int np = A.GetNumPages();
  if (b.GetNumPages() != np || x.GetNumPages() != np) fail(where, "A, b and x differ in their number of pages");
  if (A.GetNumRows() != A.GetNumCols()) fail(where, "matrices must be square");
  if (x.GetNumElements() != A.GetNumCols() || b.GetNumElements() != A.GetNumRows())
    fail(where, "vector length differs from the matrix size");
  if (!res.ExistsGPU() || res.GetNumPages() < np) fail(where, "SolverResults must hold one GPU entry per page");
}

// the timed part of the original helpers plus KernelFillTrueResNorms
void run_solver(const char* where, const PagedCSRMatrices& A, const PagedVectors& b, PagedVectors& x,
                SolverResults& res, const bilu_options& o, bool full_diagonal, double* PST, double* IST,
                double* OET) {
  check_batch(where, A, b, x, res);
  const int np = A.GetNumPages();
  std::lock_guard<std::mutex> lock(cache().mu);
  const auto t0 = std::chrono::high_resolution_clock::now();
  const Pattern p = device_pattern(A, where);
  bilu_plan* plan = cache().get(p, o, where);
  if (full_diagonal && info_of(plan, where).missing_diag > 0)
    fail(where, "the pattern lacks diagonal entries (the original asserts a full diagonal)");
  ck(bilu_plan_enable_timing(plan, 1), where);
  bilu_results R = {res.GetPtrToGpuIterCount(), res.GetPtrToGpuConvFlag(), res.GetPtrToGpuIterResNorm(),
                    nullptr, nullptr, nullptr, nullptr};
  ck(bilu_solve(plan, np, A.GetPtrToGpuValues(), b.GetPtrToGpuValues(), x.GetPtrToGpuValues(), &R, nullptr), where);
  ck(cudaDeviceSynchronize(), where);
  const auto t1 = std::chrono::high_resolution_clock::now();
  bilu_timing tm;
  ck(bilu_plan_last_timing(plan, &tm), where);
  const double oet = std::chrono::duration<double, std::milli>(t1 - t0).count();
  const double ist = std::min<double>(tm.solve_ms, oet);
  if (OET) *OET = oet;
  if (IST) *IST = ist;
  if (PST) *PST = oet - ist;
  res.SetTimeTaken(oet);
  std::cout << where << ": " << np << " systems solved in " << oet << " ms" << std::endl;
  ck(bilu_true_residual(plan, np, A.GetPtrToGpuValues(), b.GetPtrToGpuValues(), x.GetPtrToGpuValues(),
                        res.GetPtrToGpuTrueResNorm(), nullptr),
     where);
  ck(cudaDeviceSynchronize(), where);
}

void write_solution(const std::vector<std::string>& subdir, PagedVectors& x, const std::string& file) {
  x.CopyFromGpuToCpu();
  Print_ans(subdir, x, file);
  std::cout << "solutions written to " << file << " in each system directory" << std::endl;
}

}  // namespace

// ---------------------------------------------------------------- solvers
void Batched_ILU_Preconditioned_BiCGSTAB_Gpu(const std::vector<std::string>& subdir, const PagedCSRMatrices& A_pages,
                                             const PagedVectors& b_pages, PagedVectors& x_pages, const bool is_scaled,
                                             SolverResults& solver_results, const bool is_parilu,
                                             const int app_num_conv_ilu, const int num_iter_par_ilu, double& PST,
                                             double& IST, double& OET) {
  const char* where = "Batched_ILU_Preconditioned_BiCGSTAB_Gpu";
  if (!is_parilu && (app_num_conv_ilu < 1 || app_num_conv_ilu > 4)) fail(where, "ILU approach must be 1..4");
  if (is_parilu && num_iter_par_ilu < 0) fail(where, "negative number of ParILU sweeps");
  bilu_options o = base_options(is_parilu ? BILU_PRECOND_PARILU0 : BILU_PRECOND_ILU0_SPLIT);
  o.ilu_approach = is_parilu ? 1 : app_num_conv_ilu;
  o.parilu_sweeps = is_parilu ? num_iter_par_ilu : 0;
  run_solver(where, A_pages, b_pages, x_pages, solver_results, o, false, &PST, &IST, &OET);
  const std::string specifics = is_parilu ? "parILU_" + std::to_string(num_iter_par_ilu) + "_"
                                          : "conv_ILU_app_" + std::to_string(app_num_conv_ilu) + "_";
  write_solution(subdir, x_pages, (is_scaled ? "x_scaled_gpu_" : "x_gpu_") + specifics + "bicgstab.mtx");
}

void Batched_ILU_ISAI_Preconditioned_BiCGSTAB_Gpu(const std::vector<std::string>& subdir,
                                                  const PagedCSRMatrices& A_pages, const PagedVectors& b_pages,
                                                  PagedVectors& x_pages, const bool is_scaled,
                                                  SolverResults& solver_results, const bool is_parilu,
                                                  const int num_iter_par_ilu, double& PST, double& IST, double& OET) {
  const char* where = "Batched_ILU_ISAI_Preconditioned_BiCGSTAB_Gpu";
  if (is_parilu && num_iter_par_ilu < 0) fail(where, "negative number of ParILU sweeps");
  bilu_options o = base_options(is_parilu ? BILU_PRECOND_PARILU0_ISAI : BILU_PRECOND_ILU0_ISAI);
  o.ilu_approach = 3;
  o.parilu_sweeps = is_parilu ? num_iter_par_ilu : 0;
  o.isai_power = 2;
  run_solver(where, A_pages, b_pages, x_pages, solver_results, o, false, &PST, &IST, &OET);
  write_solution(subdir, x_pages, is_scaled ? "x_scaled_gpu_ilu_isai_bicgstab.mtx" : "x_gpu_ilu_isai_bicgstab.mtx");
}

void Batched_General_ISAI_Preconditioned_BiCGSTAB_Gpu(const std::vector<std::string>& subdir,
                                                      const PagedCSRMatrices& A_pages, const PagedVectors& b_pages,
                                                      PagedVectors& x_pages, const bool is_scaled,
                                                      SolverResults& solver_results, double& PST, double& IST,
                                                      double& OET) {
  bilu_options o = base_options(BILU_PRECOND_GENERAL_ISAI);
  o.isai_power = 1;
  run_solver("Batched_General_ISAI_Preconditioned_BiCGSTAB_Gpu", A_pages, b_pages, x_pages, solver_results, o, true,
             &PST, &IST, &OET);
  write_solution(subdir, x_pages,
                 is_scaled ? "x_scaled_gpu_general_isai_bicgstab.mtx" : "x_gpu_general_isai_bicgstab.mtx");
}

void Batched_conv_ILU_app1_Preconditioned_BiCGSTAB_merged_Gpu(const std::vector<std::string>& subdir,
                                                              const PagedCSRMatrices& A_pages,
                                                              const PagedVectors& b_pages, PagedVectors& x_pages,
                                                              const bool is_scaled, SolverResults& solver_results) {
  bilu_options o = base_options(BILU_PRECOND_ILU0);
  o.ilu_approach = 1;
  run_solver("Batched_conv_ILU_app1_Preconditioned_BiCGSTAB_merged_Gpu", A_pages, b_pages, x_pages, solver_results, o,
             true, nullptr, nullptr, nullptr);
  write_solution(subdir, x_pages,
                 is_scaled ? "x_scaled_gpu_conv_ilu_merged_app1_bicgstab.mtx" : "x_gpu_conv_ilu_merged_app1_bicgstab.mtx");
}

void Batched_conv_ILU_app1_Preconditioned_BiCGSTAB_segregated_Gpu(const std::vector<std::string>& subdir,
                                                                  const PagedCSRMatrices& A_pages,
                                                                  const PagedVectors& b_pages, PagedVectors& x_pages,
                                                                  const bool is_scaled,
                                                                  SolverResults& solver_results) {
  bilu_options o = base_options(BILU_PRECOND_ILU0_SPLIT);
  o.ilu_approach = 1;
  run_solver("Batched_conv_ILU_app1_Preconditioned_BiCGSTAB_segregated_Gpu", A_pages, b_pages, x_pages,
             solver_results, o, true, nullptr, nullptr, nullptr);
  write_solution(subdir, x_pages,
                 is_scaled ? "x_scaled_gpu_conv_ilu_segregated_app1_bicgstab.mtx"
                           : "x_gpu_conv_ilu_segregated_app1_bicgstab.mtx");
}

// ---------------------------------------------------------------- factorisations
namespace {

// in-place factors of `A` (factor pattern) -> reference L / U pages
void factor_to_pages(const char* where, const PagedCSRMatrices& A, bilu_plan* plan, const double* lu,
                     PagedCSRMatrices& L, PagedCSRMatrices& U) {
  const int np = A.GetNumPages();
  shape_pages(L, plan, 3, np, where);
  shape_pages(U, plan, 4, np, where);
  ck(bilu_split_lu(plan, np, lu, L.GetPtrToGpuValues(), U.GetPtrToGpuValues(), nullptr), where);
  ck(cudaDeviceSynchronize(), where);
}

}  // namespace

void ILU_0_Factorization_Gpu(const PagedCSRMatrices& A_pages, PagedCSRMatrices& L_pages, PagedCSRMatrices& U_pages,
                             const int approach_num) {
  const char* where = "ILU_0_Factorization_Gpu";
  if (approach_num < 1 || approach_num > 4) fail(where, "approach must be 1..4");
  bilu_options o = base_options(BILU_PRECOND_ILU0_SPLIT);
  o.ilu_approach = approach_num;
  std::lock_guard<std::mutex> lock(cache().mu);
  const Pattern p = device_pattern(A_pages, where);
  bilu_plan* plan = cache().get(p, o, where);
  const int np = A_pages.GetNumPages();
  DevBuf<double> lu((size_t)info_of(plan, where).nnz * np, where);
  ck(bilu_ilu0(plan, np, A_pages.GetPtrToGpuValues(), lu.p, approach_num, nullptr), where);
  factor_to_pages(where, A_pages, plan, lu.p, L_pages, U_pages);
}

void ComputeILU0Approach1(PagedCSRMatrices& Factored_Pages, const int* const /*diag_ptrs*/) {
  // diag_ptrs holds the diagonal positions of Factored_Pages' pattern; the plan
  // derives the same positions from the pattern itself.
  const char* where = "ComputeILU0Approach1";
  bilu_options o = base_options(BILU_PRECOND_ILU0_SPLIT);
  std::lock_guard<std::mutex> lock(cache().mu);
  const Pattern p = device_pattern(Factored_Pages, where);
  bilu_plan* plan = cache().get(p, o, where);
  if (info_of(plan, where).missing_diag > 0) fail(where, "the pattern lacks diagonal entries");
  double* v = Factored_Pages.GetPtrToGpuValues();
  ck(bilu_ilu0(plan, Factored_Pages.GetNumPages(), v, v, 1, nullptr), where);
  ck(cudaDeviceSynchronize(), where);
}

void ParILU_0_Factorization_Gpu(const PagedCSRMatrices& A_pages, PagedCSRMatrices& L_pages,
                                PagedCSRMatrices& U_pages, const int num_iterations) {
  const char* where = "ParILU_0_Factorization_Gpu";
  if (num_iterations < 0) fail(where, "negative number of sweeps");
  bilu_options o = base_options(BILU_PRECOND_PARILU0);
  o.parilu_sweeps = num_iterations;
  std::lock_guard<std::mutex> lock(cache().mu);
  const Pattern p = device_pattern(A_pages, where);
  bilu_plan* plan = cache().get(p, o, where);
  const int np = A_pages.GetNumPages();
  DevBuf<double> lu((size_t)info_of(plan, where).nnz * np, where);
  ck(bilu_parilu0(plan, np, A_pages.GetPtrToGpuValues(), nullptr, lu.p, num_iterations, nullptr), where);
  factor_to_pages(where, A_pages, plan, lu.p, L_pages, U_pages);
}

// ---------------------------------------------------------------- ISAI
void GenerateISAI_gpu(PagedCSRMatrices& aiA_pages, const PagedCSRMatrices& A_pages, const mat_type A_type,
                      const int power) {
  const char* where = "GenerateISAI_gpu";
  if (power < 1) fail(where, "power must be >= 1");
  std::lock_guard<std::mutex> lock(cache().mu);
  const Pattern p = device_pattern(A_pages, where);
  for (int i = 0; i < p.n; ++i) {
    const int b = p.rp[i], e = p.rp[i + 1];
    const bool has_diag = std::binary_search(p.ci.begin() + b, p.ci.begin() + e, i);
    if (!has_diag) fail(where, "row " + std::to_string(i) + " has no diagonal entry");
    if (A_type == mat_type::lower_tri && p.ci[e - 1] != i) fail(where, "lower_tri matrix with an entry above the diagonal");
    if (A_type == mat_type::upper_tri && p.ci[b] != i) fail(where, "upper_tri matrix with an entry below the diagonal");
  }
  const int np = A_pages.GetNumPages();
  const double* T = A_pages.GetPtrToGpuValues();
  if (A_type == mat_type::general) {
    bilu_options o = base_options(BILU_PRECOND_GENERAL_ISAI);
    o.isai_power = power;
    bilu_plan* plan = cache().get(p, o, where);
    shape_pages(aiA_pages, plan, 1, np, where);
    ck(bilu_isai(plan, np, T, aiA_pages.GetPtrToGpuValues(), nullptr, nullptr), where);
  } else {
    // ISAI(L) / ISAI(U) of a plan built on the triangular pattern itself: its
    // lower (upper) split is the matrix, the other split only its diagonal
    bilu_options o = base_options(BILU_PRECOND_ILU0_ISAI);
    o.isai_power = power;
    o.isai_lower_diag = A_type == mat_type::lower_tri ? 1 : 0;
    bilu_plan* plan = cache().get(p, o, where);
    const bilu_plan_info info = info_of(plan, where);
    if (A_type == mat_type::lower_tri) {
      shape_pages(aiA_pages, plan, 1, np, where);
      DevBuf<double> other((size_t)info.nnz_isai_U * np, where);
      ck(bilu_isai(plan, np, T, aiA_pages.GetPtrToGpuValues(), other.p, nullptr), where);
      ck(cudaDeviceSynchronize(), where);
    } else {
      shape_pages(aiA_pages, plan, 2, np, where);
      DevBuf<double> other((size_t)info.nnz_isai_L * np, where);
      ck(bilu_isai(plan, np, T, other.p, aiA_pages.GetPtrToGpuValues(), nullptr), where);
      ck(cudaDeviceSynchronize(), where);
    }
  }
  ck(cudaDeviceSynchronize(), where);
}
