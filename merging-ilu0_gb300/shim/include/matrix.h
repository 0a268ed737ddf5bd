// Drop-in interface: the paged (system-major) batch containers of the
// original code (matrix.h:6-325 of Batched-ILU0-merged/ILU0_ISAI_bicgstab).
// Member order and types are those of the original classes, so objects
// created by its drivers can be passed to this library unchanged; the
// out-of-line methods are implemented in shim/ref_containers.cpp on the CUDA runtime.
#pragma once
#include "location_enums.h"

class PagedCSRMatrices {
 private:
  int nrows = 0;
  int ncols = 0;
  int nnz = 0;
  int npages = 0;
  CPU_EXISTENCE cpu_exists = CPU_EXISTENCE::NON_EXISTENT;
  GPU_EXISTENCE gpu_exists = GPU_EXISTENCE::NON_EXISTENT;
  int* col_ind_cpu = nullptr;
  int* row_ptrs_cpu = nullptr;
  double* values_cpu = nullptr;
  int* col_ind_gpu = nullptr;
  int* row_ptrs_gpu = nullptr;
  double* values_gpu = nullptr;

 public:
  bool ExistsCPU() const { return cpu_exists == CPU_EXISTENCE::EXISTENT; }
  bool ExistsGPU() const { return gpu_exists == GPU_EXISTENCE::EXISTENT; }
  void SetNumPages(const int pages) { npages = pages; }
  int GetNumPages() const { return npages; }
  void SetNumRows(const int rows) { nrows = rows; }
  int GetNumRows() const { return nrows; }
  void SetNumCols(const int cols) { ncols = cols; }
  int GetNumCols() const { return ncols; }
  void SetNumNz(const int nz) { nnz = nz; }
  int GetNumNz() const { return nnz; }
  void AllocateMemory(const LOCATION loc);
  void DeallocateMemory(const LOCATION loc);
  double* GetPtrToCpuValues() const { return values_cpu; }
  int* GetPtrToCpuColInd() const { return col_ind_cpu; }
  int* GetPtrToCpuRowPtrs() const { return row_ptrs_cpu; }
  double* GetPtrToGpuValues() const { return values_gpu; }
  int* GetPtrToGpuColInd() const { return col_ind_gpu; }
  int* GetPtrToGpuRowPtrs() const { return row_ptrs_gpu; }
  ~PagedCSRMatrices();
  PagedCSRMatrices();
  void CopyFromCpuToGpu();
  void CopyFromGpuToCpu();
  PagedCSRMatrices(const PagedCSRMatrices&) = delete;
  PagedCSRMatrices(const PagedCSRMatrices&&) = delete;
  PagedCSRMatrices& operator=(const PagedCSRMatrices&) = delete;
  PagedCSRMatrices& operator=(const PagedCSRMatrices&&) = delete;
};

class PagedCOOMatrices {
 private:
  int nrows = 0;
  int ncols = 0;
  int nnz = 0;
  int npages = 0;
  CPU_EXISTENCE cpu_exists = CPU_EXISTENCE::NON_EXISTENT;
  GPU_EXISTENCE gpu_exists = GPU_EXISTENCE::NON_EXISTENT;
  int* col_ind_cpu = nullptr;
  int* row_ind_cpu = nullptr;
  double* values_cpu = nullptr;
  int* col_ind_gpu = nullptr;
  int* row_ind_gpu = nullptr;
  double* values_gpu = nullptr;

 public:
  bool ExistsCPU() const { return cpu_exists == CPU_EXISTENCE::EXISTENT; }
  bool ExistsGPU() const { return gpu_exists == GPU_EXISTENCE::EXISTENT; }
  void SetNumPages(const int pages) { npages = pages; }
  int GetNumPages() const { return npages; }
  void SetNumRows(const int rows) { nrows = rows; }
  int GetNumRows() const { return nrows; }
  void SetNumCols(const int cols) { ncols = cols; }
  int GetNumCols() const { return ncols; }
  void SetNumNz(const int nz) { nnz = nz; }
  int GetNumNz() const { return nnz; }
  void AllocateMemory(const LOCATION loc);
  void DeallocateMemory(const LOCATION loc);
  double* GetPtrToCpuValues() const { return values_cpu; }
  int* GetPtrToCpuColInd() const { return col_ind_cpu; }
  int* GetPtrToCpuRowInd() const { return row_ind_cpu; }
  double* GetPtrToGpuValues() const { return values_gpu; }
  int* GetPtrToGpuColInd() const { return col_ind_gpu; }
  int* GetPtrToGpuRowInd() const { return row_ind_gpu; }
  ~PagedCOOMatrices();
  PagedCOOMatrices();
  void CopyFromCpuToGpu();
  void CopyFromGpuToCpu();
  PagedCOOMatrices(const PagedCOOMatrices&) = delete;
  PagedCOOMatrices(const PagedCOOMatrices&&) = delete;
  PagedCOOMatrices& operator=(const PagedCOOMatrices&) = delete;
  PagedCOOMatrices& operator=(const PagedCOOMatrices&&) = delete;
};

class PagedVectors {
 private:
  int npages = 0;
  int nelements = 0;
  CPU_EXISTENCE cpu_exists = CPU_EXISTENCE::NON_EXISTENT;
  GPU_EXISTENCE gpu_exists = GPU_EXISTENCE::NON_EXISTENT;
  double* values_cpu = nullptr;
  double* values_gpu = nullptr;

 public:
  bool ExistsCPU() const { return cpu_exists == CPU_EXISTENCE::EXISTENT; }
  bool ExistsGPU() const { return gpu_exists == GPU_EXISTENCE::EXISTENT; }
  void SetNumPages(const int pages) { npages = pages; }
  int GetNumPages() const { return npages; }
  void SetNumElements(const int eles) { nelements = eles; }
  int GetNumElements() const { return nelements; }
  void AllocateMemory(const LOCATION loc);
  void DeallocateMemory(const LOCATION loc);
  ~PagedVectors();
  PagedVectors();
  double* GetPtrToCpuValues() const { return values_cpu; }
  double* GetPtrToGpuValues() const { return values_gpu; }
  void CopyFromCpuToGpu();
  void CopyFromGpuToCpu();
  PagedVectors(const PagedVectors&) = delete;
  PagedVectors(const PagedVectors&&) = delete;
  PagedVectors& operator=(const PagedVectors&) = delete;
  PagedVectors& operator=(const PagedVectors&&) = delete;
};
