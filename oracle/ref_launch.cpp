// ORACLE -- test infrastructure only.
//
// Launches the reference's own kernels (compiled from its sources into the
// cubins of oracle/_ref by oracle/build_ref.py) through the CUDA driver API,
// in the primary context that PyTorch also uses, so that tests can hand in
// device pointers of torch tensors.  Kernels live in anonymous namespaces of
// the reference's translation units; they are found by enumerating a module's
// functions and matching the length-prefixed identifier inside the exported
// (mangled) name.  Launch shapes follow the reference's host helpers:
//   merged solver      PrecondBiCGSTAB_exact_ilu0_app1_merged_gpu.cu:568-577  (npages x 512, 11 n doubles)
//   true residual      ..._merged_gpu.cu:593                                   (npages x 512)
//   split ILU solver   PrecondBiCGSTAB_ilu_gpu.cu:474-485                      (npages x 512, 10 n doubles)
//   ILU-ISAI solver    PrecondBiCGSTAB_ilu_isai_gpu.cu:305-314                 (npages x 512, static)
//   ILU(0) approach 1  ILU_0_gpu.cu:175-186                                    (npages x 512, 2 n doubles)
//   ILU(0) approach 4  ILU_0_gpu.cu:1211-1222                                  (npages x 512)
//   ParILU(0)          parILU_0_gpu.cu:274-282                                 (npages x 512, (nL+nU) doubles)
//   ISAI extraction    isai_gpu.cu:312-317                                     (n x 512)
//   ISAI fill / solve  isai_gpu.cu:668-675                                     (ceil(32 n npages / 512) x 512)
//   general ISAI solver PrecondBiCGSTAB_general_isai_gpu.cu:266-274             (npages x 512, static)
// The spin-waiting ILU approaches 2 and 3 are never launched.
#include <cuda.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

const char* kUnits[] = {"merged", "ilu_split", "ilu_isai", "ilu0", "parilu", "isai", "general_isai"};
enum { U_MERGED, U_SPLIT, U_ISAI_SOLVER, U_ILU0, U_PARILU, U_ISAI, U_GENERAL, U_COUNT };
CUmodule g_mod[U_COUNT] = {};
char g_err[512] = "";

int fail(const char* what, CUresult r) {
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  std::snprintf(g_err, sizeof(g_err), "%s: %s", what, s ? s : "?");
  return (int)r ? (int)r : -1;
}

// exported name contains "<len><identifier>" (Itanium mangling of a nested name)
CUfunction find(int unit, const char* ident) {
  unsigned cnt = 0;
  if (cuModuleGetFunctionCount(&cnt, g_mod[unit]) != CUDA_SUCCESS) return nullptr;
  std::vector<CUfunction> fs(cnt);
  if (cuModuleEnumerateFunctions(fs.data(), cnt, g_mod[unit]) != CUDA_SUCCESS) return nullptr;
  const std::string key = std::to_string(std::strlen(ident)) + ident;
  for (CUfunction f : fs) {
    const char* nm = nullptr;
    if (cuFuncGetName(&nm, f) == CUDA_SUCCESS && nm && std::strstr(nm, key.c_str())) return f;
  }
  return nullptr;
}

int launch(int unit, const char* ident, unsigned grid, unsigned block, unsigned smem, void** args) {
  CUfunction f = find(unit, ident);
  if (!f) {
    std::snprintf(g_err, sizeof(g_err), "kernel %s not found in %s.cubin", ident, kUnits[unit]);
    return -2;
  }
  CUresult r;
  if (smem > 48 * 1024) {
    r = cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem);
    if (r != CUDA_SUCCESS) return fail("cuFuncSetAttribute", r);
  }
  r = cuLaunchKernel(f, grid, 1, 1, block, 1, 1, smem, nullptr, args, nullptr);
  if (r != CUDA_SUCCESS) return fail("cuLaunchKernel", r);
  r = cuCtxSynchronize();
  if (r != CUDA_SUCCESS) return fail("cuCtxSynchronize", r);
  return 0;
}

}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_err; }

// Loads the six cubins from `dir` into the primary context of `device`.
int ref_load(const char* dir, int device) {
  CUresult r = cuInit(0);
  if (r != CUDA_SUCCESS) return fail("cuInit", r);
  CUdevice dev;
  r = cuDeviceGet(&dev, device);
  if (r != CUDA_SUCCESS) return fail("cuDeviceGet", r);
  CUcontext ctx;
  r = cuDevicePrimaryCtxRetain(&ctx, dev);
  if (r != CUDA_SUCCESS) return fail("cuDevicePrimaryCtxRetain", r);
  r = cuCtxSetCurrent(ctx);
  if (r != CUDA_SUCCESS) return fail("cuCtxSetCurrent", r);
  for (int u = 0; u < U_COUNT; ++u) {
    if (g_mod[u]) continue;
    std::string path = std::string(dir) + "/" + kUnits[u] + ".cubin";
    FILE* fp = std::fopen(path.c_str(), "rb");
    if (!fp) {
      std::snprintf(g_err, sizeof(g_err), "cannot open %s", path.c_str());
      return -3;
    }
    std::fseek(fp, 0, SEEK_END);
    long sz = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    std::vector<char> img(sz);
    size_t got = std::fread(img.data(), 1, sz, fp);
    std::fclose(fp);
    if ((long)got != sz) return -3;
    r = cuModuleLoadData(&g_mod[u], img.data());
    if (r != CUDA_SUCCESS) return fail("cuModuleLoadData", r);
  }
  return 0;
}

int ref_merged(int n, int nnz, int npages, const int* rp, const int* ci, const double* vals, const double* rhs,
               double* ans, double* factored, const int* diag, float* iters, int* conv, double* res) {
  void* a[] = {&n, &nnz, &npages, &rp, &ci, &vals, &rhs, &ans, &factored, &diag, &iters, &conv, &res};
  return launch(U_MERGED, "KernelBatchedPreconditionedBiCGSTAB_ILU", npages, 512, 11 * n * 8, a);
}

int ref_true_residual(int n, int nnz, int npages, const int* rp, const int* ci, const double* vals,
                      const double* rhs, const double* ans, double* out) {
  void* a[] = {&n, &nnz, &npages, &rp, &ci, &vals, &rhs, &ans, &out};
  return launch(U_MERGED, "KernelFillTrueResNorms", npages, 512, 0, a);
}

int ref_split_solve(int n, int nnz, int npages, const int* rp, const int* ci, const double* vals, const double* rhs,
                    double* ans, int lnnz, const int* lrp, const int* lci, const double* lv, int unnz, const int* urp,
                    const int* uci, const double* uv, float* iters, int* conv, double* res) {
  void* a[] = {&n, &nnz, &npages, &rp, &ci, &vals, &rhs, &ans, &lnnz, &lrp, &lci, &lv, &unnz, &urp, &uci, &uv,
               &iters, &conv, &res};
  return launch(U_SPLIT, "KernelBatchedPreconditionedBiCGSTAB_ILU", npages, 512, 10 * n * 8, a);
}

int ref_isai_solve(int n, int nnz, int npages, const int* rp, const int* ci, const double* vals, const double* rhs,
                   double* ans, int lnnz, const int* lrp, const int* lci, const double* lv, int unnz, const int* urp,
                   const int* uci, const double* uv, float* iters, int* conv, double* res) {
  void* a[] = {&n, &nnz, &npages, &rp, &ci, &vals, &rhs, &ans, &lnnz, &lrp, &lci, &lv, &unnz, &urp, &uci, &uv,
               &iters, &conv, &res};
  return launch(U_ISAI_SOLVER, "KernelBatchedPreconditionedBiCGSTAB_ILU_ISAI", npages, 512, 0, a);
}

int ref_ilu0_app1(int npages, int n, int nnz, const int* rp, const int* ci, double* values, const int* diag) {
  void* a[] = {&npages, &n, &nnz, &rp, &ci, &values, &diag};
  return launch(U_ILU0, "compute_ilu_0_approach1_kernel", npages, 512, 2 * n * 8, a);
}

int ref_ilu0_app4(int npages, int nnz, double* values, const int* deps, const int* diag_starters, const int* eras,
                  int era_len, int dep_len) {
  void* a[] = {&npages, &nnz, &values, &deps, &diag_starters, &eras, &era_len, &dep_len};
  return launch(U_ILU0, "compute_ilu_0_approach4_kernel", npages, 512, 0, a);
}

int ref_parilu(int npages, int n, int nnz, const double* values, int lnnz, double* lv, int unnz, double* uv,
               int sweeps, const int* deps, const int* nz_ptrs) {
  void* a[] = {&npages, &n, &nnz, &values, &lnnz, &lv, &unnz, &uv, &sweeps, &deps, &nz_ptrs};
  return launch(U_PARILU, "compute_parilu_0_approach2_kernel", npages, 512, (lnnz + unnz) * 8, a);
}

int ref_isai_extract(int n, const int* arp, const int* aci, int annz, const int* irp, const int* ici, int innz,
                     int* dense, int* rhs_one, int* sizes) {
  void* a[] = {&n, &arp, &aci, &annz, &irp, &ici, &innz, &dense, &rhs_one, &sizes};
  return launch(U_ISAI, "Extract_pattern_kernel_approach1", n, 512, 0, a);
}

int ref_isai_fill(int npages, int n, int* irp, int* ici, double* ivals, int innz, const int* arp, const int* aci,
                  const double* avals, int annz, const int* dense, const int* rhs_one, const int* sizes,
                  int matrix_type) {
  void* a[] = {&npages, &n, &irp, &ici, &ivals, &innz, &arp, &aci, &avals, &annz, &dense, &rhs_one, &sizes,
               &matrix_type};
  const unsigned grid = (unsigned)((32LL * n * npages + 511) / 512);
  return launch(U_ISAI, "fill_values_and_solve_kernel_approach1", grid, 512, 0, a);
}

int ref_general_isai_solve(int n, int nnz, int npages, const int* rp, const int* ci, const double* vals,
                           const double* rhs, double* ans, int innz, const int* irp, const int* ici, const double* iv,
                           float* iters, int* conv, double* res) {
  void* a[] = {&n, &nnz, &npages, &rp, &ci, &vals, &rhs, &ans, &innz, &irp, &ici, &iv, &iters, &conv, &res};
  return launch(U_GENERAL, "KernelBatchedPreconditionedBiCGSTABGeneralISAI", npages, 512, 0, a);
}

}  // extern "C"
