// Device diagnostics, no reference counterpart: the FP64 FMA throughput of
// the device, the denominator of the FP64 roofline that the benchmark quotes
// for the solver kernels (FP64 issue, not HBM, bounds them on GB300); and a
// check of the kernels' integer FP64 <-> FP32 conversions against the
// hardware's and of the integer reciprocal against __drcp_rn.
//
// Every thread runs CH independent DFMA chains (the loop unrolled 4 times), so
// the 64-cycle latency of a dependent DFMA is covered many times over by the
// chains of the SM's resident threads; the rate is the number of lane FMAs
// over the CUDA-event time of the launch.  Three launch shapes (4, 8 and 16
// chains per thread at full occupancy) each run 5 times after 2 warm-up
// launches, and the best rate is kept.  Thread 0 of CTA 0 also reads the SM
// cycle counter and the global nanosecond timer at its start and end, which
// gives the SM clock during the launch.
#include <cuda_runtime.h>

#include <string>

#include "bilu.h"
#include "bilu_internal.h"
#include "k_intfp.cuh"

namespace bilu {
namespace {

constexpr int kThreads = 256;

template <int CH>
__global__ void __launch_bounds__(kThreads) k_dfma_rate(long long* __restrict__ clk, int iters, double s) {
  long long c0 = 0, t0 = 0;
  const bool probe = blockIdx.x == 0 && threadIdx.x == 0;
  if (probe) {
    c0 = clock64();
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  }
  double a[CH];
#pragma unroll
  for (int k = 0; k < CH; ++k) a[k] = 1e-3 * threadIdx.x + k;
  for (int i = 0; i < iters; i += 4) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
#pragma unroll
      for (int k = 0; k < CH; ++k) a[k] = fma(a[k], s, 1e-9);
    }
  }
  double r = 0.0;
#pragma unroll
  for (int k = 0; k < CH; ++k) r += a[k];
  if (probe) {
    long long t1;
    const long long c1 = clock64();
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t1));
    clk[0] = c1 - c0;
    clk[1] = t1 - t0;
    clk[2] = r == -1.0 ? 1 : 0;  // never true (every a[k] stays >= 0): keeps every chain live
  }
}

template <int CH>
cudaError_t best_rate(cudaStream_t st, int sms, long long* d_clk, cudaEvent_t* ev, double* gflops, double* mhz) {
  int occ = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_dfma_rate<CH>, kThreads, 0);
  if (e != cudaSuccess) return e;
  const int grid = sms * (occ > 0 ? occ : 1), iters = 32768 / CH;
  for (int rep = 0; rep < 7 && e == cudaSuccess; ++rep) {
    cudaEventRecord(ev[0], st);
    k_dfma_rate<CH><<<grid, kThreads, 0, st>>>(d_clk, iters, 0.9999999);
    e = cudaGetLastError();
    cudaEventRecord(ev[1], st);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
    float ms = 0.0f;
    long long h[3] = {0, 0, 0};
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev[0], ev[1]);
    if (e == cudaSuccess) e = cudaMemcpy(h, d_clk, sizeof(h), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess || rep < 2 || ms <= 0.0f) continue;  // the first two launches warm up
    const double g = 2.0 * (double)grid * kThreads * iters * CH / (ms * 1e-3) / 1e9;  // two FLOPs per FMA
    if (g > *gflops) {
      *gflops = g;
      *mhz = h[1] > 0 ? 1e3 * (double)h[0] / (double)h[1] : 0.0;
    }
  }
  return e;
}

// The kernels' integer FP64 operations (k_intfp.cuh: integer forms with the
// hardware's for what they leave) against the hardware, on n bit patterns per
// thread.  Conversions, three kinds of double in turn: any 64-bit pattern;
// doubles whose exponent sweeps [860, 1165] and 2047 (float subnormal
// results, the zero / normal / overflow boundaries, infinities, NaNs) with
// random mantissas, every fourth of them with the 29 bits that rounding drops
// set to exactly half (ties); any 32-bit pattern for the widening.
// Reciprocals (against __drcp_rn): any 64-bit pattern, every other one with
// its mantissa reduced to its low 20 bits or its high 32 bits set, every
// eighth a power of two.  bad[0] counts roundings, bad[1] widenings, bad[2]
// reciprocals that differ in any bit (NaNs compare by being NaN: both sides
// are NaN or neither).
__global__ void k_intfp_check(unsigned long long seed, int n, unsigned long long* __restrict__ bad) {
  const unsigned long long tid = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  unsigned long long s = seed ^ (0x9e3779b97f4a7c15ull * (tid + 1));
  unsigned long long nd = 0, nw = 0, nr = 0;
  for (int i = 0; i < n; ++i) {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    unsigned long long u = s;
    if (i % 3 == 1) {
      const unsigned e = (unsigned)((s >> 53) % 307u);
      u = (s & 0x800fffffffffffffull) | ((unsigned long long)(e == 306u ? 0x7ffu : 860u + e) << 52);
      if ((s & 0x3000000000000ull) == 0) u = (u & ~0x1fffffffull) | 0x10000000ull;
    }
    const double d = __longlong_as_double((long long)u);
    const float a = __double2float_rn(d), b = ifp::f32(d);
    if (__float_as_uint(a) != __float_as_uint(b) && !(a != a && b != b)) ++nd;
    const float y = __uint_as_float((unsigned)(s >> 17));
    const double c = (double)y, w = ifp::f64(y);
    if (__double_as_longlong(c) != __double_as_longlong(w) && !(c != c && w != w)) ++nw;
    unsigned long long v = s * 0x2545f4914f6cdd1dull;
    if ((i & 3) == 1) v &= 0x80000000000fffffull | (0x7ffull << 52);
    if ((i & 3) == 3) v |= 0x000ffffffff00000ull;
    if ((i & 7) == 2) v &= 0xfff0000000000000ull;
    const double dv = __longlong_as_double((long long)v);
    const double ra = __drcp_rn(dv), rr = ifp::rcp(dv);
    if (__double_as_longlong(ra) != __double_as_longlong(rr) && !(ra != ra && rr != rr)) ++nr;
  }
  if (nd) atomicAdd(bad, nd);
  if (nw) atomicAdd(bad + 1, nw);
  if (nr) atomicAdd(bad + 2, nr);
}

}  // namespace
}  // namespace bilu

extern "C" bilu_status bilu_check_integer_fp(int n_per_thread, uint64_t seed, unsigned long long* h_mismatch,
                                             void* stream) {
  using namespace bilu;
  if (!h_mismatch || n_per_thread < 0) return set_error(BILU_ERR_INVALID, "bilu_check_integer_fp: bad arguments");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return set_error(BILU_ERR_CUDA, std::string("bilu_check_integer_fp: ") + cudaGetErrorString(e));
  unsigned long long* d_bad = nullptr;
  if (cudaMalloc(&d_bad, 3 * sizeof(unsigned long long)) != cudaSuccess)
    return set_error(BILU_ERR_ALLOC, "bilu_check_integer_fp: cudaMalloc");
  e = cudaMemsetAsync(d_bad, 0, 3 * sizeof(unsigned long long), st);
  if (e == cudaSuccess) {
    k_intfp_check<<<sms * 4, kThreads, 0, st>>>(seed, n_per_thread, d_bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h_mismatch, d_bad, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_bad);
  if (e != cudaSuccess) return set_error(BILU_ERR_CUDA, std::string("bilu_check_integer_fp: ") + cudaGetErrorString(e));
  return BILU_OK;
}

extern "C" bilu_status bilu_probe_fp64_rate(double* h_gflops, double* h_sm_mhz, void* stream) {
  using namespace bilu;
  if (!h_gflops) return set_error(BILU_ERR_INVALID, "bilu_probe_fp64_rate: NULL output");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return set_error(BILU_ERR_CUDA, std::string("bilu_probe_fp64_rate: ") + cudaGetErrorString(e));
  long long* d_clk = nullptr;
  if (cudaMalloc(&d_clk, 4 * sizeof(long long)) != cudaSuccess)
    return set_error(BILU_ERR_ALLOC, "bilu_probe_fp64_rate: cudaMalloc");
  cudaEvent_t ev[2] = {nullptr, nullptr};
  e = cudaEventCreate(&ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
  double gflops = 0.0, mhz = 0.0;
  if (e == cudaSuccess) e = best_rate<4>(st, sms, d_clk, ev, &gflops, &mhz);
  if (e == cudaSuccess) e = best_rate<8>(st, sms, d_clk, ev, &gflops, &mhz);
  if (e == cudaSuccess) e = best_rate<16>(st, sms, d_clk, ev, &gflops, &mhz);
  for (cudaEvent_t x : ev)
    if (x) cudaEventDestroy(x);
  cudaFree(d_clk);
  if (e != cudaSuccess) return set_error(BILU_ERR_CUDA, std::string("bilu_probe_fp64_rate: ") + cudaGetErrorString(e));
  *h_gflops = gflops;
  if (h_sm_mhz) *h_sm_mhz = mhz;
  return BILU_OK;
}
