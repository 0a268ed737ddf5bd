// Test driver for the drop-in C++ interface (libbilu_ref.so): reads a
// directory of Matrix Market systems the way the original drivers do
// (FillSubdir + ReadData), runs one entry point and dumps what it produced in
// binary form for the Python tests.
//
//   shim_driver <dir/> <problem_size> <is_scaled> <out_dir> <command> [args]
//     read                                   CSR of the pages only (no GPU)
//     ilu <is_parilu> <approach> <sweeps>    Batched_ILU_Preconditioned_BiCGSTAB_Gpu
//     ilu_isai <is_parilu> <sweeps>          Batched_ILU_ISAI_Preconditioned_BiCGSTAB_Gpu
//     general                                Batched_General_ISAI_Preconditioned_BiCGSTAB_Gpu
//     merged | segregated                    Batched_conv_ILU_app1_..._{merged,segregated}_Gpu
//     factor_ilu <approach>                  ILU_0_Factorization_Gpu  -> L.bin, U.bin
//     factor_parilu <sweeps>                 ParILU_0_Factorization_Gpu -> L.bin, U.bin
//     approach1                              ComputeILU0Approach1 on a copy of A -> F.bin
//     isai <0 general|1 lower|2 upper> <power>  GenerateISAI_gpu on A -> AI.bin
//
// Outputs in <out_dir>: subdirs.txt (page order), A.bin (CSR read), results.bin
// (per page: float iters, int conv, double iter_res, double true_res),
// timing.txt (PST IST OET time_taken), Results.txt (PrintSolverResults) and the
// entry point's own x_*.mtx files in every subdirectory.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "ILU_0.h"
#include "PrecondBiCGSTAB.h"
#include "ReadWriteData.h"
#include "SolverResults.h"
#include "isai.h"
#include "matrix.h"
#include "parILU_0.h"

namespace {

std::string out_dir;

FILE* open_out(const std::string& name) {
  FILE* f = std::fopen((out_dir + "/" + name).c_str(), "wb");
  if (!f) {
    std::perror(name.c_str());
    std::exit(2);
  }
  return f;
}

// n, nnz, npages, row_ptrs, col_idxs, values (host copy of the pages)
void dump_csr(PagedCSRMatrices& M, const std::string& name, bool from_gpu) {
  if (from_gpu) M.CopyFromGpuToCpu();
  FILE* f = open_out(name);
  const int hdr[3] = {M.GetNumRows(), M.GetNumNz(), M.GetNumPages()};
  std::fwrite(hdr, sizeof(int), 3, f);
  std::fwrite(M.GetPtrToCpuRowPtrs(), sizeof(int), M.GetNumRows() + 1, f);
  std::fwrite(M.GetPtrToCpuColInd(), sizeof(int), M.GetNumNz(), f);
  std::fwrite(M.GetPtrToCpuValues(), sizeof(double), (size_t)M.GetNumNz() * M.GetNumPages(), f);
  std::fclose(f);
}

void copy_pages(const PagedCSRMatrices& A, PagedCSRMatrices& B) {
  B.SetNumRows(A.GetNumRows());
  B.SetNumCols(A.GetNumCols());
  B.SetNumNz(A.GetNumNz());
  B.SetNumPages(A.GetNumPages());
  B.AllocateMemory(LOCATION::GPU);
  cudaMemcpy(B.GetPtrToGpuRowPtrs(), A.GetPtrToGpuRowPtrs(), sizeof(int) * (A.GetNumRows() + 1),
             cudaMemcpyDeviceToDevice);
  cudaMemcpy(B.GetPtrToGpuColInd(), A.GetPtrToGpuColInd(), sizeof(int) * A.GetNumNz(), cudaMemcpyDeviceToDevice);
  cudaMemcpy(B.GetPtrToGpuValues(), A.GetPtrToGpuValues(), sizeof(double) * A.GetNumNz() * A.GetNumPages(),
             cudaMemcpyDeviceToDevice);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 6) {
    std::fprintf(stderr, "usage: shim_driver <dir/> <problem_size> <is_scaled> <out_dir> <command> [args]\n");
    return 2;
  }
  const std::string dir = argv[1];
  const int problem_size = std::atoi(argv[2]);
  const bool is_scaled = std::atoi(argv[3]) == 1;
  out_dir = argv[4];
  const std::string cmd = argv[5];
  auto arg = [&](int k) { return k < argc ? std::atoi(argv[k]) : 0; };

  std::vector<std::string> subdir;
  FillSubdir(dir, subdir);
  PagedCSRMatrices A_pages;
  PagedVectors b_pages;
  ReadData(problem_size, subdir, A_pages, b_pages, is_scaled);
  {
    FILE* f = open_out("subdirs.txt");
    for (const auto& s : subdir) std::fprintf(f, "%s\n", s.c_str());
    std::fclose(f);
  }
  dump_csr(A_pages, "A.bin", false);
  {
    FILE* f = open_out("b.bin");
    std::fwrite(b_pages.GetPtrToCpuValues(), sizeof(double), (size_t)b_pages.GetNumPages() * b_pages.GetNumElements(),
                f);
    std::fclose(f);
  }
  if (cmd == "read") return 0;

  A_pages.AllocateMemory(LOCATION::GPU);
  A_pages.CopyFromCpuToGpu();
  b_pages.AllocateMemory(LOCATION::GPU);
  b_pages.CopyFromCpuToGpu();
  PagedVectors x_pages;
  x_pages.SetNumPages(A_pages.GetNumPages());
  x_pages.SetNumElements(A_pages.GetNumCols());
  x_pages.AllocateMemory(LOCATION::CPU);
  x_pages.AllocateMemory(LOCATION::GPU);
  SolverResults results(A_pages.GetNumPages(), ATOL, CPU_EXISTENCE::EXISTENT, GPU_EXISTENCE::EXISTENT);
  double PST = -1, IST = -1, OET = -1;

  if (cmd == "ilu") {
    for (int round = 0; round < 2; ++round)  // twice, as the drivers repeat calls: the second reuses the plan
      Batched_ILU_Preconditioned_BiCGSTAB_Gpu(subdir, A_pages, b_pages, x_pages, is_scaled, results, arg(6) == 1,
                                              arg(7), arg(8), PST, IST, OET);
  } else if (cmd == "ilu_isai") {
    Batched_ILU_ISAI_Preconditioned_BiCGSTAB_Gpu(subdir, A_pages, b_pages, x_pages, is_scaled, results, arg(6) == 1,
                                                 arg(7), PST, IST, OET);
  } else if (cmd == "general") {
    Batched_General_ISAI_Preconditioned_BiCGSTAB_Gpu(subdir, A_pages, b_pages, x_pages, is_scaled, results, PST, IST,
                                                     OET);
  } else if (cmd == "merged") {
    Batched_conv_ILU_app1_Preconditioned_BiCGSTAB_merged_Gpu(subdir, A_pages, b_pages, x_pages, is_scaled, results);
  } else if (cmd == "segregated") {
    Batched_conv_ILU_app1_Preconditioned_BiCGSTAB_segregated_Gpu(subdir, A_pages, b_pages, x_pages, is_scaled,
                                                                 results);
  } else if (cmd == "factor_ilu" || cmd == "factor_parilu") {
    PagedCSRMatrices L, U;
    if (cmd == "factor_ilu")
      ILU_0_Factorization_Gpu(A_pages, L, U, arg(6));
    else
      ParILU_0_Factorization_Gpu(A_pages, L, U, arg(6));
    dump_csr(L, "L.bin", true);
    dump_csr(U, "U.bin", true);
    return 0;
  } else if (cmd == "approach1") {
    PagedCSRMatrices F;
    copy_pages(A_pages, F);
    ComputeILU0Approach1(F, nullptr);
    dump_csr(F, "F.bin", true);
    return 0;
  } else if (cmd == "isai") {
    PagedCSRMatrices AI;
    const int t = arg(6);
    GenerateISAI_gpu(AI, A_pages, t == 0 ? mat_type::general : (t == 1 ? mat_type::lower_tri : mat_type::upper_tri),
                     arg(7));
    dump_csr(AI, "AI.bin", true);
    return 0;
  } else {
    std::fprintf(stderr, "unknown command %s\n", cmd.c_str());
    return 2;
  }

  results.CopyFromGpuToCpu();
  PrintSolverResults(subdir, results, out_dir + "/Results.txt");
  FILE* f = open_out("results.bin");
  for (int p = 0; p < results.GetNumPages(); ++p) {
    std::fwrite(results.GetPtrToCpuIterCount() + p, sizeof(float), 1, f);
    std::fwrite(results.GetPtrToCpuConvFlag() + p, sizeof(int), 1, f);
    std::fwrite(results.GetPtrToCpuIterResNorm() + p, sizeof(double), 1, f);
    std::fwrite(results.GetPtrToCpuTrueResNorm() + p, sizeof(double), 1, f);
  }
  std::fclose(f);
  FILE* t = open_out("timing.txt");
  std::fprintf(t, "%.6f %.6f %.6f %.6f\n", PST, IST, OET, results.GetTimeTaken());
  std::fclose(t);
  return 0;
}
