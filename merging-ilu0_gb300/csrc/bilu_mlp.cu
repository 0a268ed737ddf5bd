// Host side of the learned ParILU(0) warm start (kernels in k_mlp.cu): model
// object, GPU training loop (Adam on FP32 master weights, BF16 compute
// copies), gradient / forward probes for checking against the oracle, the
// warm-start generator with its ILU-residual gate, and save / load.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "bilu.h"
#include "bilu_internal.h"

using namespace bilu;

struct bilu_mlp {
  float* p = nullptr;   // FP32 master parameters
  float* m = nullptr;   // Adam moments
  float* v = nullptr;
  float* g = nullptr;   // gradient accumulator
  void* pbf = nullptr;  // BF16 compute copy
  float* loss = nullptr;
  int step = 0;
  float* stats = nullptr;  // row statistics scratch (3 * nsys * n floats)
  size_t stats_cap = 0;
  int* idx = nullptr;      // sample-index scratch
  size_t idx_cap = 0;
};

namespace {

bilu_status fail(cudaError_t e, const char* what) {
  return set_error(BILU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bilu_status check_plan(const bilu_plan* P) {
  if (!P) return set_error(BILU_ERR_INVALID, "NULL plan");
  if (P->missing) return set_error(BILU_ERR_PATTERN, "the learned warm start needs every diagonal in the pattern");
  return BILU_OK;
}

bilu_status ensure_stats(bilu_mlp* M, const bilu_plan* P, int nsys, float** rown, float** coln, float** corr) {
  const size_t need = (size_t)3 * nsys * P->n;
  if (need > M->stats_cap) {
    if (M->stats) cudaFree(M->stats);
    M->stats = nullptr;
    M->stats_cap = 0;
    cudaError_t e = cudaMalloc((void**)&M->stats, need * sizeof(float));
    if (e != cudaSuccess) return set_error(BILU_ERR_ALLOC, "mlp row statistics");
    M->stats_cap = need;
  }
  *rown = M->stats;
  *coln = M->stats + (size_t)nsys * P->n;
  *corr = M->stats + (size_t)2 * nsys * P->n;
  return BILU_OK;
}

bilu_status ensure_idx(bilu_mlp* M, size_t count) {
  if (count > M->idx_cap) {
    if (M->idx) cudaFree(M->idx);
    M->idx = nullptr;
    M->idx_cap = 0;
    cudaError_t e = cudaMalloc((void**)&M->idx, count * sizeof(int));
    if (e != cudaSuccess) return set_error(BILU_ERR_ALLOC, "mlp sample indices");
    M->idx_cap = count;
  }
  return BILU_OK;
}

}  // namespace

extern "C" {

bilu_status bilu_mlp_create(bilu_mlp** out, uint64_t seed) {
  if (!out) return set_error(BILU_ERR_INVALID, "bilu_mlp_create: out is NULL");
  *out = nullptr;
  if (bilu_device_count() == 0) return set_error(BILU_ERR_NO_DEVICE, "no CUDA device");
  const int F = kMlpFeatures, H = kMlpHidden, NP = kMlpParams;
  // Xavier-uniform weights from splitmix64, zero biases; the output layer is
  // scaled by 0.1 so the untrained model starts near the first-order estimate
  std::vector<float> h(NP, 0.0f);
  uint64_t s = seed ^ 0x5DEECE66DULL;
  auto next = [&]() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
  };
  const float a1 = std::sqrt(6.0f / (F + H)), a2 = std::sqrt(6.0f / (H + H)), a3 = std::sqrt(6.0f / (H + 1));
  int o = 0;
  for (int k = 0; k < H * F; ++k) h[o + k] = (float)(a1 * next());
  o += H * F + H;
  for (int k = 0; k < H * H; ++k) h[o + k] = (float)(a2 * next());
  o += H * H + H;
  for (int k = 0; k < H; ++k) h[o + k] = (float)(0.1 * a3 * next());
  bilu_mlp* M = new bilu_mlp();
  cudaError_t e = cudaMalloc((void**)&M->p, NP * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->m, NP * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->v, NP * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->g, NP * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&M->pbf, NP * 2);
  if (e == cudaSuccess) e = cudaMalloc((void**)&M->loss, sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(M->p, h.data(), NP * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(M->m, 0, NP * sizeof(float));
  if (e == cudaSuccess) e = cudaMemset(M->v, 0, NP * sizeof(float));
  if (e == cudaSuccess) e = launch_mlp_to_bf16(M->p, M->pbf, NP, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    bilu_status st = fail(e, "bilu_mlp_create");
    bilu_mlp_destroy(M);
    return st;
  }
  *out = M;
  return BILU_OK;
}

bilu_status bilu_mlp_destroy(bilu_mlp* M) {
  if (!M) return BILU_OK;
  cudaFree(M->p);
  cudaFree(M->m);
  cudaFree(M->v);
  cudaFree(M->g);
  cudaFree(M->pbf);
  cudaFree(M->loss);
  cudaFree(M->stats);
  cudaFree(M->idx);
  delete M;
  return BILU_OK;
}

int bilu_mlp_param_count(void) { return kMlpParams; }

bilu_status bilu_mlp_get_params(const bilu_mlp* M, float* h_params) {
  if (!M || !h_params) return set_error(BILU_ERR_INVALID, "bilu_mlp_get_params: NULL argument");
  cudaError_t e = cudaMemcpy(h_params, M->p, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? BILU_OK : fail(e, "bilu_mlp_get_params");
}

bilu_status bilu_mlp_set_params(bilu_mlp* M, const float* h_params) {
  if (!M || !h_params) return set_error(BILU_ERR_INVALID, "bilu_mlp_set_params: NULL argument");
  cudaError_t e = cudaMemcpy(M->p, h_params, kMlpParams * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = launch_mlp_to_bf16(M->p, M->pbf, kMlpParams, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return e == cudaSuccess ? BILU_OK : fail(e, "bilu_mlp_set_params");
}

bilu_status bilu_mlp_train(bilu_mlp* M, const bilu_plan* P, int nsys, const double* d_values,
                           const double* d_lu_target, int steps, int batch, float lr, uint64_t seed,
                           float* h_losses, void* stream) {
  if (!M || nsys <= 0 || steps < 0 || batch <= 0 || !d_values || !d_lu_target || !(lr > 0.0f))
    return set_error(BILU_ERR_INVALID, "bilu_mlp_train: bad arguments");
  bilu_status st = check_plan(P);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  float *rown, *coln, *corr;
  st = ensure_stats(M, P, nsys, &rown, &coln, &corr);
  if (st) return st;
  cudaError_t e = launch_mlp_rowstats(P->dp, nsys, d_values, rown, coln, corr, s);
  std::vector<float> losses(steps, 0.0f);
  float* d_losses = nullptr;
  if (e == cudaSuccess && steps > 0) e = cudaMalloc((void**)&d_losses, steps * sizeof(float));
  if (e == cudaSuccess && steps > 0) e = cudaMemsetAsync(d_losses, 0, steps * sizeof(float), s);
  for (int t = 0; t < steps && e == cudaSuccess; ++t) {
    e = cudaMemsetAsync(M->g, 0, kMlpParams * sizeof(float), s);
    if (e == cudaSuccess)
      e = launch_mlp_train(P->dp, nsys, d_values, d_lu_target, rown, coln, corr, M->pbf, batch, nullptr,
                           seed ^ (0xA24BAED4963EE407ull * (uint64_t)(M->step + 1)), M->g, d_losses + t, s);
    if (e == cudaSuccess) {
      ++M->step;
      // cosine decay from lr to lr / 20 over the call's steps
      const float lrt = lr * (0.05f + 0.95f * 0.5f * (1.0f + std::cos(3.14159265358979f * (float)t / (float)steps)));
      e = launch_mlp_adam(M->p, M->m, M->v, M->g, M->pbf, kMlpParams, lrt, M->step, s);
    }
  }
  if (e == cudaSuccess && steps > 0 && h_losses)
    e = cudaMemcpyAsync(h_losses, d_losses, steps * sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(d_losses);
  return e == cudaSuccess ? BILU_OK : fail(e, "bilu_mlp_train");
}

bilu_status bilu_mlp_loss_grad(bilu_mlp* M, const bilu_plan* P, int nsys, const double* d_values,
                               const double* d_lu_target, int nsample, const int* h_idx, float* h_loss,
                               float* h_grad, void* stream) {
  if (!M || nsys <= 0 || nsample <= 0 || !h_idx || !h_loss || !h_grad)
    return set_error(BILU_ERR_INVALID, "bilu_mlp_loss_grad: bad arguments");
  bilu_status st = check_plan(P);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  float *rown, *coln, *corr;
  st = ensure_stats(M, P, nsys, &rown, &coln, &corr);
  if (!st) st = ensure_idx(M, nsample);
  if (st) return st;
  cudaError_t e = cudaMemcpyAsync(M->idx, h_idx, nsample * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = launch_mlp_rowstats(P->dp, nsys, d_values, rown, coln, corr, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(M->g, 0, kMlpParams * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(M->loss, 0, sizeof(float), s);
  if (e == cudaSuccess)
    e = launch_mlp_train(P->dp, nsys, d_values, d_lu_target, rown, coln, corr, M->pbf, nsample, M->idx, 0, M->g,
                         M->loss, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_grad, M->g, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_loss, M->loss, sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? BILU_OK : fail(e, "bilu_mlp_loss_grad");
}

bilu_status bilu_mlp_eval(bilu_mlp* M, const bilu_plan* P, int nsys, const double* d_values, int nsample,
                          const int* h_idx, float* h_features, float* h_out, double* h_base, void* stream) {
  if (!M || nsys <= 0 || nsample <= 0 || !h_idx || !h_features || !h_out || !h_base)
    return set_error(BILU_ERR_INVALID, "bilu_mlp_eval: bad arguments");
  bilu_status st = check_plan(P);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  float *rown, *coln, *corr;
  st = ensure_stats(M, P, nsys, &rown, &coln, &corr);
  if (!st) st = ensure_idx(M, nsample);
  if (st) return st;
  float *feat = nullptr, *out = nullptr;
  double* base = nullptr;
  cudaError_t e = cudaMalloc((void**)&feat, sizeof(float) * nsample * kMlpFeatures);
  if (e == cudaSuccess) e = cudaMalloc((void**)&out, sizeof(float) * nsample);
  if (e == cudaSuccess) e = cudaMalloc((void**)&base, sizeof(double) * nsample);
  if (e == cudaSuccess) e = cudaMemcpyAsync(M->idx, h_idx, nsample * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = launch_mlp_rowstats(P->dp, nsys, d_values, rown, coln, corr, s);
  if (e == cudaSuccess)
    e = launch_mlp_eval(P->dp, nsys, d_values, rown, coln, corr, M->pbf, nsample, M->idx, feat, out, base, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h_features, feat, sizeof(float) * nsample * kMlpFeatures, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_out, out, sizeof(float) * nsample, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_base, base, sizeof(double) * nsample, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(feat);
  cudaFree(out);
  cudaFree(base);
  return e == cudaSuccess ? BILU_OK : fail(e, "bilu_mlp_eval");
}

bilu_status bilu_mlp_warm_start(bilu_mlp* M, const bilu_plan* P, int nsys, const double* d_values, double* d_lu0,
                                double threshold, double* d_ilu_res, int* d_used, void* stream) {
  if (!M || nsys < 0 || (nsys > 0 && (!d_values || !d_lu0)))
    return set_error(BILU_ERR_INVALID, "bilu_mlp_warm_start: bad arguments");
  if (nsys == 0) return BILU_OK;
  bilu_status st = check_plan(P);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  float *rown, *coln, *corr;
  st = ensure_stats(M, P, nsys, &rown, &coln, &corr);
  if (st) return st;
  cudaError_t e = launch_mlp_rowstats(P->dp, nsys, d_values, rown, coln, corr, s);
  if (e == cudaSuccess)
    e = launch_mlp_warm(P->dp, nsys, d_values, rown, coln, corr, M->pbf, threshold, d_lu0, d_ilu_res, d_used, s);
  return e == cudaSuccess ? BILU_OK : fail(e, "bilu_mlp_warm_start");
}

bilu_status bilu_mlp_save(const bilu_mlp* M, const char* path) {
  if (!M || !path) return set_error(BILU_ERR_INVALID, "bilu_mlp_save: NULL argument");
  std::vector<float> h(kMlpParams);
  bilu_status st = bilu_mlp_get_params(M, h.data());
  if (st) return st;
  FILE* f = std::fopen(path, "wb");
  if (!f) return set_error(BILU_ERR_INVALID, std::string("cannot write ") + path);
  const char magic[8] = {'B', 'I', 'L', 'U', 'M', 'L', 'P', '1'};
  const int dims[3] = {kMlpFeatures, kMlpHidden, kMlpParams};
  bool ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(dims, sizeof(int), 3, f) == 3 &&
            std::fwrite(h.data(), sizeof(float), kMlpParams, f) == (size_t)kMlpParams;
  std::fclose(f);
  return ok ? BILU_OK : set_error(BILU_ERR_INVALID, std::string("short write to ") + path);
}

bilu_status bilu_mlp_load(bilu_mlp* M, const char* path) {
  if (!M || !path) return set_error(BILU_ERR_INVALID, "bilu_mlp_load: NULL argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return set_error(BILU_ERR_INVALID, std::string("cannot read ") + path);
  char magic[8];
  int dims[3];
  std::vector<float> h(kMlpParams);
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "BILUMLP1", 8) == 0 &&
            std::fread(dims, sizeof(int), 3, f) == 3 && dims[0] == kMlpFeatures && dims[1] == kMlpHidden &&
            dims[2] == kMlpParams && std::fread(h.data(), sizeof(float), kMlpParams, f) == (size_t)kMlpParams;
  std::fclose(f);
  if (!ok) return set_error(BILU_ERR_INVALID, std::string("not a bilu MLP file: ") + path);
  return bilu_mlp_set_params(M, h.data());
}

}  // extern "C"
