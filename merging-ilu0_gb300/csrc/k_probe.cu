// FP64 FMA throughput of the device: the denominator of the FP64 roofline
// that the benchmark quotes for the solver kernels (FP64 issue, not HBM,
// bounds them on GB300).  No reference counterpart.
//
// Every thread runs kChains independent DFMA chains, so the 64-cycle latency
// of a dependent DFMA is covered by the chains of one thread and the 8
// resident CTAs of 256 threads per SM; the rate is the number of lane FMAs
// over the CUDA-event time of the launch, the best of several launches.
#include <cuda_runtime.h>

#include <string>

#include "bilu.h"
#include "bilu_internal.h"

namespace bilu {
namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_dfma_rate(double* __restrict__ sink, int iters, double s) {
  double a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = 1e-3 * threadIdx.x + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], s, 1e-9);
  }
  double r = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) r += a[k];
  if (r == -1.0 && sink) sink[0] = r;  // never true (every a[k] stays >= 0): keeps every chain live
}

}  // namespace
}  // namespace bilu

extern "C" bilu_status bilu_probe_fp64_rate(double* h_gflops, void* stream) {
  using namespace bilu;
  if (!h_gflops) return set_error(BILU_ERR_INVALID, "bilu_probe_fp64_rate: NULL output");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return set_error(BILU_ERR_CUDA, std::string("bilu_probe_fp64_rate: ") + cudaGetErrorString(e));
  const int grid = sms * 8, iters = 4096;
  cudaEvent_t ev[2];
  if (cudaEventCreate(&ev[0]) != cudaSuccess || cudaEventCreate(&ev[1]) != cudaSuccess)
    return set_error(BILU_ERR_CUDA, "bilu_probe_fp64_rate: cudaEventCreate");
  float best = -1.0f;
  for (int rep = 0; rep < 7 && e == cudaSuccess; ++rep) {
    cudaEventRecord(ev[0], st);
    k_dfma_rate<<<grid, kThreads, 0, st>>>(nullptr, iters, 0.9999999);
    e = cudaGetLastError();
    cudaEventRecord(ev[1], st);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
    float ms = 0.0f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, ev[0], ev[1]);
    if (rep >= 2 && (best < 0.0f || ms < best)) best = ms;  // the first two launches warm up
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (e != cudaSuccess) return set_error(BILU_ERR_CUDA, std::string("bilu_probe_fp64_rate: ") + cudaGetErrorString(e));
  const double fmas = (double)grid * kThreads * iters * kChains;
  *h_gflops = 2.0 * fmas / (best * 1e-3) / 1e9;  // two FLOPs per FMA
  return BILU_OK;
}
