// Drop-in batch containers: the out-of-line methods of PagedCSRMatrices,
// PagedCOOMatrices, PagedVectors (matrix.h:6-325, matrix.cu) and SolverResults
// (SolverResults.h, SolverResults.cu) of Batched-ILU0-merged/ILU0_ISAI_bicgstab.
//
// Semantics kept from the original: AllocateMemory replaces an existing
// allocation at that location; CopyFromCpuToGpu / CopyFromGpuToCpu reallocate
// the destination before copying; destructors free both locations.  Two
// deliberate differences: a failed CUDA call throws std::runtime_error instead
// of printing and continuing with a null pointer, and a copy from a location
// that holds nothing throws std::logic_error instead of calling exit(1).
// SolverResults frees all four arrays (the original leaks the two residual
// norm arrays on deallocation).
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "SolverResults.h"
#include "matrix.h"

namespace {

void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
T* dev_alloc(size_t count, const char* what) {
  void* p = nullptr;
  if (count) check(cudaMalloc(&p, count * sizeof(T)), what);
  return static_cast<T*>(p);
}

template <typename T>
void dev_free(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

template <typename T>
void host_free(T*& p) {
  delete[] p;
  p = nullptr;
}

template <typename T>
void copy(T* dst, const T* src, size_t count, cudaMemcpyKind kind, const char* what) {
  if (count) check(cudaMemcpy(dst, src, count * sizeof(T), kind), what);
}

[[noreturn]] void absent(const char* where) { throw std::logic_error(std::string(" Not present on ") + where); }

}  // namespace

// ---------------------------------------------------------------- PagedCSRMatrices
PagedCSRMatrices::PagedCSRMatrices() {}

PagedCSRMatrices::~PagedCSRMatrices() {
  DeallocateMemory(LOCATION::CPU);
  DeallocateMemory(LOCATION::GPU);
}

void PagedCSRMatrices::AllocateMemory(const LOCATION loc) {
  const size_t nv = (size_t)npages * nnz;
  DeallocateMemory(loc);
  if (loc == LOCATION::CPU) {
    values_cpu = new double[nv];
    row_ptrs_cpu = new int[nrows + 1];
    col_ind_cpu = new int[nnz];
    cpu_exists = CPU_EXISTENCE::EXISTENT;
  } else {
    values_gpu = dev_alloc<double>(nv, "PagedCSRMatrices values");
    row_ptrs_gpu = dev_alloc<int>(nrows + 1, "PagedCSRMatrices row_ptrs");
    col_ind_gpu = dev_alloc<int>(nnz, "PagedCSRMatrices col_idxs");
    gpu_exists = GPU_EXISTENCE::EXISTENT;
  }
}

void PagedCSRMatrices::DeallocateMemory(const LOCATION loc) {
  if (loc == LOCATION::CPU) {
    if (!ExistsCPU()) return;
    host_free(values_cpu);
    host_free(row_ptrs_cpu);
    host_free(col_ind_cpu);
    cpu_exists = CPU_EXISTENCE::NON_EXISTENT;
  } else {
    if (!ExistsGPU()) return;
    dev_free(values_gpu);
    dev_free(row_ptrs_gpu);
    dev_free(col_ind_gpu);
    gpu_exists = GPU_EXISTENCE::NON_EXISTENT;
  }
}

void PagedCSRMatrices::CopyFromCpuToGpu() {
  if (!ExistsCPU()) absent("CPU");
  AllocateMemory(LOCATION::GPU);
  copy(values_gpu, values_cpu, (size_t)npages * nnz, cudaMemcpyHostToDevice, "PagedCSRMatrices H2D");
  copy(row_ptrs_gpu, row_ptrs_cpu, (size_t)nrows + 1, cudaMemcpyHostToDevice, "PagedCSRMatrices H2D");
  copy(col_ind_gpu, col_ind_cpu, (size_t)nnz, cudaMemcpyHostToDevice, "PagedCSRMatrices H2D");
}

void PagedCSRMatrices::CopyFromGpuToCpu() {
  if (!ExistsGPU()) absent("GPU");
  AllocateMemory(LOCATION::CPU);
  copy(values_cpu, values_gpu, (size_t)npages * nnz, cudaMemcpyDeviceToHost, "PagedCSRMatrices D2H");
  copy(row_ptrs_cpu, row_ptrs_gpu, (size_t)nrows + 1, cudaMemcpyDeviceToHost, "PagedCSRMatrices D2H");
  copy(col_ind_cpu, col_ind_gpu, (size_t)nnz, cudaMemcpyDeviceToHost, "PagedCSRMatrices D2H");
}

// ---------------------------------------------------------------- PagedCOOMatrices
PagedCOOMatrices::PagedCOOMatrices() {}

PagedCOOMatrices::~PagedCOOMatrices() {
  DeallocateMemory(LOCATION::CPU);
  DeallocateMemory(LOCATION::GPU);
}

void PagedCOOMatrices::AllocateMemory(const LOCATION loc) {
  const size_t nv = (size_t)npages * nnz;
  DeallocateMemory(loc);
  if (loc == LOCATION::CPU) {
    values_cpu = new double[nv];
    row_ind_cpu = new int[nnz];
    col_ind_cpu = new int[nnz];
    cpu_exists = CPU_EXISTENCE::EXISTENT;
  } else {
    values_gpu = dev_alloc<double>(nv, "PagedCOOMatrices values");
    row_ind_gpu = dev_alloc<int>(nnz, "PagedCOOMatrices row_idxs");
    col_ind_gpu = dev_alloc<int>(nnz, "PagedCOOMatrices col_idxs");
    gpu_exists = GPU_EXISTENCE::EXISTENT;
  }
}

void PagedCOOMatrices::DeallocateMemory(const LOCATION loc) {
  if (loc == LOCATION::CPU) {
    if (!ExistsCPU()) return;
    host_free(values_cpu);
    host_free(row_ind_cpu);
    host_free(col_ind_cpu);
    cpu_exists = CPU_EXISTENCE::NON_EXISTENT;
  } else {
    if (!ExistsGPU()) return;
    dev_free(values_gpu);
    dev_free(row_ind_gpu);
    dev_free(col_ind_gpu);
    gpu_exists = GPU_EXISTENCE::NON_EXISTENT;
  }
}

void PagedCOOMatrices::CopyFromCpuToGpu() {
  if (!ExistsCPU()) absent("CPU");
  AllocateMemory(LOCATION::GPU);
  copy(values_gpu, values_cpu, (size_t)npages * nnz, cudaMemcpyHostToDevice, "PagedCOOMatrices H2D");
  copy(row_ind_gpu, row_ind_cpu, (size_t)nnz, cudaMemcpyHostToDevice, "PagedCOOMatrices H2D");
  copy(col_ind_gpu, col_ind_cpu, (size_t)nnz, cudaMemcpyHostToDevice, "PagedCOOMatrices H2D");
}

void PagedCOOMatrices::CopyFromGpuToCpu() {
  if (!ExistsGPU()) absent("GPU");
  AllocateMemory(LOCATION::CPU);
  copy(values_cpu, values_gpu, (size_t)npages * nnz, cudaMemcpyDeviceToHost, "PagedCOOMatrices D2H");
  copy(row_ind_cpu, row_ind_gpu, (size_t)nnz, cudaMemcpyDeviceToHost, "PagedCOOMatrices D2H");
  copy(col_ind_cpu, col_ind_gpu, (size_t)nnz, cudaMemcpyDeviceToHost, "PagedCOOMatrices D2H");
}

// ---------------------------------------------------------------- PagedVectors
PagedVectors::PagedVectors() {}

PagedVectors::~PagedVectors() {
  DeallocateMemory(LOCATION::CPU);
  DeallocateMemory(LOCATION::GPU);
}

void PagedVectors::AllocateMemory(const LOCATION loc) {
  const size_t nv = (size_t)npages * nelements;
  DeallocateMemory(loc);
  if (loc == LOCATION::CPU) {
    values_cpu = new double[nv];
    cpu_exists = CPU_EXISTENCE::EXISTENT;
  } else {
    values_gpu = dev_alloc<double>(nv, "PagedVectors values");
    gpu_exists = GPU_EXISTENCE::EXISTENT;
  }
}

void PagedVectors::DeallocateMemory(const LOCATION loc) {
  if (loc == LOCATION::CPU) {
    if (!ExistsCPU()) return;
    host_free(values_cpu);
    cpu_exists = CPU_EXISTENCE::NON_EXISTENT;
  } else {
    if (!ExistsGPU()) return;
    dev_free(values_gpu);
    gpu_exists = GPU_EXISTENCE::NON_EXISTENT;
  }
}

void PagedVectors::CopyFromCpuToGpu() {
  if (!ExistsCPU()) absent("CPU");
  AllocateMemory(LOCATION::GPU);
  copy(values_gpu, values_cpu, (size_t)npages * nelements, cudaMemcpyHostToDevice, "PagedVectors H2D");
}

void PagedVectors::CopyFromGpuToCpu() {
  if (!ExistsGPU()) absent("GPU");
  AllocateMemory(LOCATION::CPU);
  copy(values_cpu, values_gpu, (size_t)npages * nelements, cudaMemcpyDeviceToHost, "PagedVectors D2H");
}

// ---------------------------------------------------------------- SolverResults
SolverResults::SolverResults() {}

SolverResults::SolverResults(const int num_pages, const double atol, const CPU_EXISTENCE to_allocate_on_cpu,
                             const GPU_EXISTENCE to_allocate_on_gpu) {
  SetNumPages(num_pages);
  SetATOL(atol);
  if (to_allocate_on_cpu == CPU_EXISTENCE::EXISTENT) AllocateMemory(LOCATION::CPU);
  if (to_allocate_on_gpu == GPU_EXISTENCE::EXISTENT) AllocateMemory(LOCATION::GPU);
}

SolverResults::~SolverResults() {
  DeallocateMemory(LOCATION::CPU);
  DeallocateMemory(LOCATION::GPU);
}

void SolverResults::AllocateMemory(const LOCATION loc) {
  const size_t n = (size_t)npages;
  DeallocateMemory(loc);
  if (loc == LOCATION::CPU) {
    true_residual_norm_cpu = new double[n];
    iter_residual_norm_cpu = new double[n];
    iter_count_cpu = new float[n];
    conv_flag_cpu = new int[n];
    cpu_exists = CPU_EXISTENCE::EXISTENT;
  } else {
    true_residual_norm_gpu = dev_alloc<double>(n, "SolverResults true residuals");
    iter_residual_norm_gpu = dev_alloc<double>(n, "SolverResults iteration residuals");
    iter_count_gpu = dev_alloc<float>(n, "SolverResults iteration counts");
    conv_flag_gpu = dev_alloc<int>(n, "SolverResults convergence flags");
    gpu_exists = GPU_EXISTENCE::EXISTENT;
  }
}

void SolverResults::DeallocateMemory(const LOCATION loc) {
  if (loc == LOCATION::CPU) {
    if (!ExistsCPU()) return;
    host_free(iter_count_cpu);
    host_free(conv_flag_cpu);
    host_free(true_residual_norm_cpu);
    host_free(iter_residual_norm_cpu);
    cpu_exists = CPU_EXISTENCE::NON_EXISTENT;
  } else {
    if (!ExistsGPU()) return;
    dev_free(iter_count_gpu);
    dev_free(conv_flag_gpu);
    dev_free(true_residual_norm_gpu);
    dev_free(iter_residual_norm_gpu);
    gpu_exists = GPU_EXISTENCE::NON_EXISTENT;
  }
}

void SolverResults::CopyFromCpuToGpu() {
  if (!ExistsCPU()) absent("CPU");
  AllocateMemory(LOCATION::GPU);
  const size_t n = (size_t)npages;
  copy(iter_count_gpu, iter_count_cpu, n, cudaMemcpyHostToDevice, "SolverResults H2D");
  copy(conv_flag_gpu, conv_flag_cpu, n, cudaMemcpyHostToDevice, "SolverResults H2D");
  copy(true_residual_norm_gpu, true_residual_norm_cpu, n, cudaMemcpyHostToDevice, "SolverResults H2D");
  copy(iter_residual_norm_gpu, iter_residual_norm_cpu, n, cudaMemcpyHostToDevice, "SolverResults H2D");
}

void SolverResults::CopyFromGpuToCpu() {
  if (!ExistsGPU()) absent("GPU");
  AllocateMemory(LOCATION::CPU);
  const size_t n = (size_t)npages;
  copy(iter_count_cpu, iter_count_gpu, n, cudaMemcpyDeviceToHost, "SolverResults D2H");
  copy(conv_flag_cpu, conv_flag_gpu, n, cudaMemcpyDeviceToHost, "SolverResults D2H");
  copy(true_residual_norm_cpu, true_residual_norm_gpu, n, cudaMemcpyDeviceToHost, "SolverResults D2H");
  copy(iter_residual_norm_cpu, iter_residual_norm_gpu, n, cudaMemcpyDeviceToHost, "SolverResults D2H");
}
