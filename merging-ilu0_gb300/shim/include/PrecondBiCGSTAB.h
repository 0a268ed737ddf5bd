// Drop-in interface: the five batched solver entry points of the original
// code (PrecondBiCGSTAB.h:15-30 of Batched-ILU0-merged/ILU0_ISAI_bicgstab) and
// its iteration limit / absolute tolerance.  Implemented in shim/ref_api.cpp
// on the bilu C ABI (include/bilu.h).
#pragma once
#include <string>
#include <vector>

class PagedCSRMatrices;
class PagedVectors;
class SolverResults;

#define MAX_ITER 500
#define ATOL 0.00000000001

void Batched_ILU_Preconditioned_BiCGSTAB_Gpu(const std::vector<std::string>& subdir, const PagedCSRMatrices& A_pages,
                                             const PagedVectors& b_pages, PagedVectors& x_pages, const bool is_scaled,
                                             SolverResults& solver_results, const bool is_parilu,
                                             const int app_num_conv_ilu, const int num_iter_par_ilu, double& PST,
                                             double& IST, double& OET);

void Batched_ILU_ISAI_Preconditioned_BiCGSTAB_Gpu(const std::vector<std::string>& subdir,
                                                  const PagedCSRMatrices& A_pages, const PagedVectors& b_pages,
                                                  PagedVectors& x_pages, const bool is_scaled,
                                                  SolverResults& solver_results, const bool is_parilu,
                                                  const int num_iter_par_ilu, double& PST, double& IST, double& OET);

void Batched_General_ISAI_Preconditioned_BiCGSTAB_Gpu(const std::vector<std::string>& subdir,
                                                      const PagedCSRMatrices& A_pages, const PagedVectors& b_pages,
                                                      PagedVectors& x_pages, const bool is_scaled,
                                                      SolverResults& solver_results, double& PST, double& IST,
                                                      double& OET);

void Batched_conv_ILU_app1_Preconditioned_BiCGSTAB_merged_Gpu(const std::vector<std::string>& subdir,
                                                              const PagedCSRMatrices& A_pages,
                                                              const PagedVectors& b_pages, PagedVectors& x_pages,
                                                              const bool is_scaled, SolverResults& solver_results);

void Batched_conv_ILU_app1_Preconditioned_BiCGSTAB_segregated_Gpu(const std::vector<std::string>& subdir,
                                                                  const PagedCSRMatrices& A_pages,
                                                                  const PagedVectors& b_pages, PagedVectors& x_pages,
                                                                  const bool is_scaled,
                                                                  SolverResults& solver_results);
