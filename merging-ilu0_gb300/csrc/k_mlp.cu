// Learned ParILU(0) warm start: a per-nonzero MLP (9 -> 64 -> 64 -> 1, GELU in
// its tanh form, BF16 weights, FP32 accumulation) that predicts the converged
// ParILU factors, trained on the GPU by these kernels.  No counterpart in the
// reference.  Training runs on CUDA cores with an accurate tanh; inference
// (k_mlp_warm) runs the 64x64 layer on the tensor cores (mma.sync BF16 with
// FP32 accumulation, activations split into BF16 high + low parts so the
// products keep FP32-level precision) and the hardware tanh approximation.
//
// Features of nonzero (i, j) of system s, all scaled by d = |a_ii|:
//   a_ij, a_ii, a_jj, ||A(i,:)||_2, ||A(:,j)||_2 (column over the structurally
//   symmetric part), level(i) / (levels-1), sign(j - i), and the first-order
//   Schur corrections c_i, c_j with c_r = sum_{k<r} a_rk a_kr / a_kk.
// Output y is a relative correction of a first-order estimate of the factor
// ratio lu_ij / a_ij:  below the diagonal 1 / (a_jj - c_j), on it
// (a_ii - c_i) / a_ii, above it 1;  warm start lu0_ij = a_ij * base * (1 + y).
// Training target: y* = lu*_ij / (a_ij * base) - 1 with lu* the converged
// ParILU(0) factors the solver generates; loss = mean (y - y*)^2.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "bilu_internal.h"

namespace bilu {
namespace {

constexpr int NF = kMlpFeatures;
constexpr int H = kMlpHidden;
constexpr int OW1 = 0, OB1 = H * NF, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H, OB3 = OW3 + H;
static_assert(OB3 + 1 == kMlpParams, "parameter layout");

constexpr unsigned kFull = 0xffffffffu;

// GELU, tanh form: 0.5 x (1 + tanh(k (x + c x^3))), k = sqrt(2/pi), c = 0.044715
constexpr float kGk = 0.7978845608028654f, kGc = 0.044715f;
__device__ __forceinline__ float gelu(float x) {
  const float t = tanhf(kGk * fmaf(kGc * x, x * x, x));
  return 0.5f * x * (1.0f + t);
}
__device__ __forceinline__ float gelu_d(float x) {
  const float t = tanhf(kGk * fmaf(kGc * x, x * x, x));
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * kGk * fmaf(3.0f * kGc, x * x, 1.0f);
}
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu_fast(float x) {
  return 0.5f * x * (1.0f + tanh_approx(kGk * fmaf(kGc * x, x * x, x)));
}

// per (system, row): row 2-norm, column 2-norm, first-order Schur correction
__global__ void k_rowstats(const DevPattern P, int nsys, const double* __restrict__ A, float* __restrict__ rown,
                           float* __restrict__ coln, float* __restrict__ corr) {
  const int s = blockIdx.x;
  if (s >= nsys) return;
  // FP32 throughout (the features are FP32): FP64 division and square root
  // are long instruction sequences on this part's FP64 pipe
  const double* As = A + (size_t)s * P.nnz;
  for (int i = threadIdx.x; i < P.n; i += blockDim.x) {
    const int b = P.rp[i], e = P.rp[i + 1], d = P.diag[i];
    float rn = 0.0f, cn = 0.0f, c = 0.0f;
    for (int k = b; k < e; ++k) {
      const float a = (float)As[k];
      rn = fmaf(a, a, rn);
      const int t = P.tpos[k];
      if (t >= 0) {
        const float at = (float)As[t];
        cn = fmaf(at, at, cn);
        if (k < d) c = fmaf(a, at / (float)As[P.diag[P.ci[k]]], c);
      }
    }
    rown[(size_t)s * P.n + i] = sqrtf(rn);
    coln[(size_t)s * P.n + i] = sqrtf(cn);
    corr[(size_t)s * P.n + i] = c;
  }
}

struct Feat {
  float f[NF];
  float base;
  double a;
};

// Features in FP32 from one reciprocal (FP64 divisions are expensive on this
// part); base = first-order estimate of the factor ratio (FP32).
__device__ __forceinline__ Feat features(const DevPattern& P, int s, int e, const double* __restrict__ A,
                                         const float* __restrict__ rown, const float* __restrict__ coln,
                                         const float* __restrict__ corr) {
  Feat r;
  const int i = P.row_of[e], j = P.ci[e];
  const double* As = A + (size_t)s * P.nnz;
  const double aij = As[e];
  const float fij = (float)aij, fii = (float)As[P.diag[i]], fjj = (float)As[P.diag[j]];
  const float inv = 1.0f / (fii != 0.0f ? fabsf(fii) : 1.0f);
  const float ci_ = corr[(size_t)s * P.n + i], cj = corr[(size_t)s * P.n + j];
  r.f[0] = fij * inv;
  r.f[1] = fii * inv;
  r.f[2] = fjj * inv;
  r.f[3] = rown[(size_t)s * P.n + i] * inv;
  r.f[4] = coln[(size_t)s * P.n + j] * inv;
  r.f[5] = P.nlev_lo > 1 ? (float)P.row_lev[i] / (float)(P.nlev_lo - 1) : 0.0f;
  r.f[6] = j < i ? -1.0f : (j > i ? 1.0f : 0.0f);
  r.f[7] = ci_ * inv;
  r.f[8] = cj * inv;
  r.a = aij;
  float base = 1.0f;
  if (j < i) {
    const float den = fjj - cj;
    base = den != 0.0f ? 1.0f / den : (fjj != 0.0f ? 1.0f / fjj : 1.0f);
  } else if (j == i) {
    base = fii != 0.0f ? (fii - ci_) / fii : 1.0f;
  }
  r.base = base;
  return r;
}

// parameters (BF16) staged into shared memory as FP32
__device__ __forceinline__ void stage_params(const __nv_bfloat16* __restrict__ pbf, float* sp) {
  for (int k = threadIdx.x; k < kMlpParams; k += blockDim.x) sp[k] = __bfloat162float(pbf[k]);
}

// forward of one sample on CUDA cores; h1 / g1 / pre2 optionally stored (row of stride 65)
__device__ __forceinline__ float mlp_forward(const float* sp, const float* x, float* h1row, float* g1row,
                                             float* p2row) {
  float h[H];
#pragma unroll 4
  for (int u = 0; u < H; ++u) {
    float acc = sp[OB1 + u];
#pragma unroll
    for (int k = 0; k < NF; ++k) acc = fmaf(sp[OW1 + u * NF + k], x[k], acc);
    h[u] = gelu(acc);
    if (h1row) {
      h1row[u] = h[u];
      g1row[u] = gelu_d(acc);
    }
  }
  float out = sp[OB3];
  for (int u = 0; u < H; ++u) {
    float acc = sp[OB2 + u];
    const float4* w = reinterpret_cast<const float4*>(sp + OW2 + u * H);
#pragma unroll
    for (int v4 = 0; v4 < H / 4; ++v4) {
      const float4 q = w[v4];
      acc = fmaf(q.x, h[4 * v4 + 0], acc);
      acc = fmaf(q.y, h[4 * v4 + 1], acc);
      acc = fmaf(q.z, h[4 * v4 + 2], acc);
      acc = fmaf(q.w, h[4 * v4 + 3], acc);
    }
    if (p2row) p2row[u] = acc;
    out = fmaf(sp[OW3 + u], gelu(acc), out);
  }
  return out;
}

uint64_t __host__ __device__ __forceinline__ mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

constexpr int TB = 128;  // samples (threads) per training block
constexpr int LD = H + 1;

// One forward + backward pass over a block of samples; weight gradients are
// reduced over the block and added to `grad` (FP32 atomics), the summed
// squared error to `loss`.  Samples: explicit global entry indices (s*nnz+e)
// or, when idx == NULL, hashed from (seed, sample number).
__global__ void __launch_bounds__(TB) k_mlp_train(const DevPattern P, int nsys, const double* __restrict__ A,
                                                  const double* __restrict__ LUt, const float* __restrict__ rown,
                                                  const float* __restrict__ coln, const float* __restrict__ corr,
                                                  const __nv_bfloat16* __restrict__ pbf, int nsample,
                                                  const int* __restrict__ idx, uint64_t seed, float scale,
                                                  float* __restrict__ grad, float* __restrict__ loss) {
  extern __shared__ __align__(16) float sm[];
  float* sp = sm;                          // kMlpParams (padded to 4)
  float* X = sp + ((kMlpParams + 3) & ~3);  // TB * NF
  float* H1 = X + TB * NF;                 // TB * LD
  float* G1 = H1 + TB * LD;                // TB * LD (gelu', then dpre1)
  float* P2 = G1 + TB * LD;                // TB * LD (pre2, then d*h2)
  float* D2 = P2 + TB * LD;                // TB * LD (dpre2)
  float* DO = D2 + TB * LD;                // TB
  __shared__ float s_loss[TB / 32];
  stage_params(pbf, sp);
  __syncthreads();
  const int t = threadIdx.x;
  const long long q = (long long)blockIdx.x * TB + t;
  const bool live = q < nsample;
  float err2 = 0.0f;
  float* xr = X + t * NF;
  if (live) {
    long long g;
    if (idx) {
      g = idx[q];
    } else {  // a random system and a random entry among those the network predicts
      const uint64_t h = mix64(seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(q + 1)));
      g = (long long)(h % (uint64_t)nsys) * P.nnz + P.mlp_ent[(h >> 32) % (uint64_t)P.n_mlp];
    }
    const int s = (int)(g / P.nnz), e = (int)(g % P.nnz);
    const Feat ft = features(P, s, e, A, rown, coln, corr);
#pragma unroll
    for (int k = 0; k < NF; ++k) xr[k] = ft.f[k];
    const double denom = ft.a * (double)ft.base;
    const float ytrue = denom != 0.0 ? (float)(LUt[g] / denom - 1.0) : 0.0f;
    const float out = mlp_forward(sp, xr, H1 + t * LD, G1 + t * LD, P2 + t * LD);
    const float diff = out - ytrue;
    err2 = diff * diff;
    const float dout = 2.0f * diff * scale;
    DO[t] = dout;
    // layer 3 and 2
    float* p2 = P2 + t * LD;
    float* d2 = D2 + t * LD;
    for (int u = 0; u < H; ++u) {
      const float pre = p2[u];
      d2[u] = dout * sp[OW3 + u] * gelu_d(pre);
      p2[u] = dout * gelu(pre);  // contribution to dW3
    }
    // dh1 = W2^T dpre2, dpre1 = dh1 * gelu'(pre1)
    float dp[H];
#pragma unroll
    for (int u = 0; u < H; ++u) dp[u] = d2[u];
    float* g1 = G1 + t * LD;
    for (int v = 0; v < H; ++v) {
      float acc = 0.0f;
#pragma unroll
      for (int u = 0; u < H; ++u) acc = fmaf(sp[OW2 + u * H + v], dp[u], acc);
      g1[v] = acc * g1[v];
    }
  } else {
    DO[t] = 0.0f;
    for (int k = 0; k < NF; ++k) xr[k] = 0.0f;
    for (int u = 0; u < H; ++u) {
      H1[t * LD + u] = 0.0f;
      G1[t * LD + u] = 0.0f;
      P2[t * LD + u] = 0.0f;
      D2[t * LD + u] = 0.0f;
    }
  }
  // loss
  float l = err2;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) l += __shfl_down_sync(kFull, l, off);
  if ((t & 31) == 0) s_loss[t >> 5] = l;
  __syncthreads();
  if (t == 0) {
    float sum = 0.0f;
    for (int w = 0; w < TB / 32; ++w) sum += s_loss[w];
    atomicAdd(loss, sum * scale);
  }
  // block-reduced weight gradients
  for (int k = t; k < H * H; k += TB) {  // dW2[u][v] = sum_t dpre2[t][u] * h1[t][v]
    const int u = k / H, v = k % H;
    float acc = 0.0f;
    for (int r = 0; r < TB; ++r) acc = fmaf(D2[r * LD + u], H1[r * LD + v], acc);
    atomicAdd(grad + OW2 + k, acc);
  }
  for (int k = t; k < H * NF; k += TB) {  // dW1[u][f] = sum_t dpre1[t][u] * x[t][f]
    const int u = k / NF, f = k % NF;
    float acc = 0.0f;
    for (int r = 0; r < TB; ++r) acc = fmaf(G1[r * LD + u], X[r * NF + f], acc);
    atomicAdd(grad + OW1 + k, acc);
  }
  if (t < H) {
    float a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
    for (int r = 0; r < TB; ++r) {
      a1 += G1[r * LD + t];
      a2 += D2[r * LD + t];
      a3 += P2[r * LD + t];
    }
    atomicAdd(grad + OB1 + t, a1);
    atomicAdd(grad + OB2 + t, a2);
    atomicAdd(grad + OW3 + t, a3);
  }
  if (t == H) {
    float a = 0.0f;
    for (int r = 0; r < TB; ++r) a += DO[r];
    atomicAdd(grad + OB3, a);
  }
}

// Adam on the FP32 master parameters; refreshes the BF16 copy.
__global__ void k_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ g, __nv_bfloat16* __restrict__ pbf, int count, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const float gk = g[k];
  const float mk = b1 * m[k] + (1.0f - b1) * gk;
  const float vk = b2 * v[k] + (1.0f - b2) * gk * gk;
  m[k] = mk;
  v[k] = vk;
  const float pk = p[k] - lr * (mk / c1) / (sqrtf(vk / c2) + eps);
  p[k] = pk;
  pbf[k] = __float2bfloat16_rn(pk);
}

__global__ void k_to_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ pbf, int count) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < count) pbf[k] = __float2bfloat16_rn(p[k]);
}

// Features and forward outputs of given samples (checks against the oracle).
__global__ void k_mlp_eval(const DevPattern P, int nsys, const double* __restrict__ A, const float* __restrict__ rown,
                           const float* __restrict__ coln, const float* __restrict__ corr,
                           const __nv_bfloat16* __restrict__ pbf, int nsample, const int* __restrict__ idx,
                           float* __restrict__ feat, float* __restrict__ out, double* __restrict__ base) {
  extern __shared__ __align__(16) float sm[];
  stage_params(pbf, sm);
  __syncthreads();
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nsample) return;
  const long long g = idx[q];
  const Feat ft = features(P, (int)(g / P.nnz), (int)(g % P.nnz), A, rown, coln, corr);
  for (int k = 0; k < NF; ++k) feat[(size_t)q * NF + k] = ft.f[k];
  base[q] = ft.base;
  out[q] = mlp_forward(sm, ft.f, nullptr, nullptr, nullptr);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo_elem, float hi_elem) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo_elem, hi_elem);  // .x = first (low 16 bits)
  return *reinterpret_cast<const uint32_t*>(&v);
}

// d += a * b, m16n8k16, BF16 operands, FP32 accumulators
__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Warm start: persistent CTAs over the systems (the network's weights are
// staged once per CTA).  Entries with no dependency pairs on or above the
// diagonal converge to a_ij exactly and are copied.  The others go through the
// network in tiles of 32 per warp: every lane forms one entry's features, then
// each 16-entry half runs as m16n8k16 MMAs -- every lane forms the first-layer
// activations it needs for its A fragments (rows g and g+8, k = 2t, 2t+1,
// 2t+8, 2t+9 of each 16-wide chunk; g = lane/4, t = lane%4), split into BF16
// high and low parts; layer 2 is 2 x 4 x 8 MMAs against W2 (BF16); GELU and
// the output layer reduce over the 4 lanes of a quad.  The ILU residual
// ||(A - L0 U0)|_S||_F / ||A||_F then decides between the prediction and the
// plain initialisation lu0 = A.
//
// Shared-memory weight layout, arranged so that each lane fetches its operands
// with 128-bit loads (the kernel is bound by shared-memory traffic otherwise):
//   w1p [64][12]     hidden unit v: W1[v][0..8], b1[v], 0, 0
//   bw  [8][4] x 4   slice ut, quad index t: b2[u], b2[u+1], w3[u], w3[u+1], u = 8 ut + 2 t
//   b3  [4]          b3, 0, 0, 0
//   w2f [8][32][8]   slice ut, lane: its B fragments of the 4 k-chunks, (W2 row 8 ut + g,
//                    words 8 ch + t and 8 ch + 4 + t) for ch = 0..3
constexpr int WARM_THREADS = 256;
constexpr int WP_W1 = 0, WP_BW = H * 12, WP_B3 = WP_BW + 8 * 4 * 4, WP_W2 = WP_B3 + 4;
constexpr int WP_WORDS = WP_W2 + 8 * 32 * 8;
static_assert(WP_W2 % 4 == 0 && WP_WORDS % 4 == 0, "16-byte aligned weight blocks");

__global__ void __launch_bounds__(WARM_THREADS) k_mlp_warm(const DevPattern P, int nsys,
                                                           const double* __restrict__ A,
                                                           const float* __restrict__ rown,
                                                           const float* __restrict__ coln,
                                                           const float* __restrict__ corr,
                                                           const __nv_bfloat16* __restrict__ pbf, double threshold,
                                                           double* __restrict__ LU0, double* __restrict__ res_out,
                                                           int* __restrict__ used) {
  extern __shared__ __align__(16) unsigned char smraw[];
  float* wp = reinterpret_cast<float*>(smraw);
  uint32_t* w2f = reinterpret_cast<uint32_t*>(wp + WP_W2);
  double* lu = reinterpret_cast<double*>(wp + WP_WORDS);
  __shared__ double s_num[WARM_THREADS / 32], s_den[WARM_THREADS / 32];
  __shared__ int s_ok;
  for (int k = threadIdx.x; k < H * 12; k += blockDim.x) {
    const int v = k / 12, c = k % 12;
    wp[WP_W1 + k] = c < NF ? __bfloat162float(pbf[OW1 + v * NF + c]) : (c == NF ? __bfloat162float(pbf[OB1 + v]) : 0.0f);
  }
  for (int k = threadIdx.x; k < 8 * 4 * 4; k += blockDim.x) {
    const int ut = k >> 4, t = (k >> 2) & 3, c = k & 3, u = ut * 8 + 2 * t + (c & 1);
    wp[WP_BW + k] = __bfloat162float(pbf[(c < 2 ? OB2 : OW3) + u]);
  }
  if (threadIdx.x < 4) wp[WP_B3 + threadIdx.x] = threadIdx.x == 0 ? __bfloat162float(pbf[OB3]) : 0.0f;
  const uint32_t* w2g = reinterpret_cast<const uint32_t*>(pbf + OW2);  // row u: 32 words of 2 BF16
  for (int k = threadIdx.x; k < 8 * 32 * 8; k += blockDim.x) {
    const int ut = k >> 8, ln = (k >> 3) & 31, c = k & 7, ch = c >> 1;
    const int g = ln >> 2, t = ln & 3;
    w2f[k] = w2g[(ut * 8 + g) * (H / 2) + ch * 8 + (c & 1) * 4 + t];
  }
  __syncthreads();  // staged weights visible to every warp before b3 is read below
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const float4* w1v = reinterpret_cast<const float4*>(wp + WP_W1);
  const float4* bwv = reinterpret_cast<const float4*>(wp + WP_BW);
  const uint4* w2v = reinterpret_cast<const uint4*>(w2f);
  const float b3 = wp[WP_B3];
  const int ntile = (P.n_mlp + 31) >> 5;
  for (int s = blockIdx.x; s < nsys; s += gridDim.x) {
    __syncthreads();  // the previous system's lu and s_ok no longer read
    const double* As = A + (size_t)s * P.nnz;
    for (int e = threadIdx.x; e < P.nnz; e += blockDim.x) lu[e] = As[e];  // exact for the copied entries
    __syncthreads();
    for (int tile = warp; tile < ntile; tile += nwarp) {
      // features of entry tile*32 + lane
      const int q = tile * 32 + lane;
      const bool live = q < P.n_mlp;
      float f[NF];
      double ab = 0.0;
      int e = -1;
      if (live) {
        e = P.mlp_ent[q];
        const Feat ft = features(P, s, e, A, rown, coln, corr);
#pragma unroll
        for (int k = 0; k < NF; ++k) f[k] = ft.f[k];
        ab = ft.a * (double)ft.base;
      } else {
#pragma unroll
        for (int k = 0; k < NF; ++k) f[k] = 0.0f;
      }
#pragma unroll 1
      for (int half = 0; half < 2; ++half) {
        float xa[NF], xb[NF];  // rows g and g+8 of this half
#pragma unroll
        for (int k = 0; k < NF; ++k) {
          xa[k] = __shfl_sync(kFull, f[k], 16 * half + g);
          xb[k] = __shfl_sync(kFull, f[k], 16 * half + g + 8);
        }
        // first layer on CUDA cores, straight into A fragments (high and low parts)
        uint32_t ahi[4][4], alo[4][4];
#pragma unroll
        for (int ch = 0; ch < 4; ++ch) {
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {  // k = 2t, 2t+1 (hh 0) and 2t+8, 2t+9 (hh 1)
            const int v0 = ch * 16 + 2 * t + 8 * hh;
            float ha[2], hb[2];
#pragma unroll
            for (int d = 0; d < 2; ++d) {
              const float4 wa = w1v[(v0 + d) * 3], wb = w1v[(v0 + d) * 3 + 1], wc = w1v[(v0 + d) * 3 + 2];
              const float w[NF] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w, wc.x};
              float pa = wc.y, pb = wc.y;  // b1
#pragma unroll
              for (int k = 0; k < NF; ++k) {
                pa = fmaf(w[k], xa[k], pa);
                pb = fmaf(w[k], xb[k], pb);
              }
              ha[d] = gelu_fast(pa);
              hb[d] = gelu_fast(pb);
            }
            const float ha0h = __bfloat162float(__float2bfloat16_rn(ha[0]));
            const float ha1h = __bfloat162float(__float2bfloat16_rn(ha[1]));
            const float hb0h = __bfloat162float(__float2bfloat16_rn(hb[0]));
            const float hb1h = __bfloat162float(__float2bfloat16_rn(hb[1]));
            ahi[ch][2 * hh + 0] = pack_bf16(ha0h, ha1h);
            ahi[ch][2 * hh + 1] = pack_bf16(hb0h, hb1h);
            alo[ch][2 * hh + 0] = pack_bf16(ha[0] - ha0h, ha[1] - ha1h);
            alo[ch][2 * hh + 1] = pack_bf16(hb[0] - hb0h, hb[1] - hb1h);
          }
        }
        // register order of the A fragment: a0 (row g, k 2t..), a1 (row g+8, k 2t..), a2 (row g, k 2t+8..),
        // a3 (row g+8, k 2t+8..)
        float outa = 0.0f, outb = 0.0f;
#pragma unroll
        for (int ut = 0; ut < 8; ++ut) {
          float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
          const uint4 q0 = w2v[(ut * 32 + lane) * 2], q1 = w2v[(ut * 32 + lane) * 2 + 1];
          const uint32_t bfr[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
#pragma unroll
          for (int ch = 0; ch < 4; ++ch) {
            const uint32_t ah[4] = {ahi[ch][0], ahi[ch][1], ahi[ch][2], ahi[ch][3]};
            const uint32_t al[4] = {alo[ch][0], alo[ch][1], alo[ch][2], alo[ch][3]};
            mma_bf16(c, ah, bfr[2 * ch], bfr[2 * ch + 1]);
            mma_bf16(c, al, bfr[2 * ch], bfr[2 * ch + 1]);
          }
          const float4 bw = bwv[ut * 4 + t];  // b2[u], b2[u+1], w3[u], w3[u+1]
          outa = fmaf(bw.z, gelu_fast(c[0] + bw.x), outa);
          outa = fmaf(bw.w, gelu_fast(c[1] + bw.y), outa);
          outb = fmaf(bw.z, gelu_fast(c[2] + bw.x), outb);
          outb = fmaf(bw.w, gelu_fast(c[3] + bw.y), outb);
        }
        outa += __shfl_xor_sync(kFull, outa, 1);
        outa += __shfl_xor_sync(kFull, outa, 2);
        outb += __shfl_xor_sync(kFull, outb, 1);
        outb += __shfl_xor_sync(kFull, outb, 2);
        // the entry of row r (0..15) of this half lives on lane 16*half + r; rows r < 8
        // were reduced on lane 4r (outa), rows 8..15 on lane 4(r-8) (outb)
        const int r = lane & 15;
        const float ya = __shfl_sync(kFull, outa, (r & 7) << 2);
        const float yb = __shfl_sync(kFull, outb, (r & 7) << 2);
        if (live && (lane >> 4) == half) {
          const float y = (r < 8 ? ya : yb) + b3;
          lu[e] = ab * (1.0 + (double)y);
        }
      }
    }
    __syncthreads();
    // residual of the warm start: (A - LU)_ij = a_ij - sum_{k<min(i,j)} l_ik u_kj - (l_ij u_jj | u_ij)
    double num = 0.0, den = 0.0;
    for (int e = threadIdx.x; e < P.nnz; e += blockDim.x) {
      const int i = P.row_of[e], j = P.ci[e];
      double acc = 0.0;
      for (int q = P.dep_ptr[e]; q < P.dep_ptr[e + 1]; ++q) {
        const int2 d = P.dep[q];
        acc = fma(lu[d.x], lu[d.y], acc);
      }
      acc = (j < i) ? fma(lu[e], lu[P.diag[j]], acc) : acc + lu[e];
      const double rr = As[e] - acc;
      num = fma(rr, rr, num);
      den = fma(As[e], As[e], den);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      num += __shfl_down_sync(kFull, num, off);
      den += __shfl_down_sync(kFull, den, off);
    }
    if (lane == 0) {
      s_num[warp] = num;
      s_den[warp] = den;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0.0, b = 0.0;
      for (int w = 0; w < nwarp; ++w) {
        a += s_num[w];
        b += s_den[w];
      }
      const double res = b > 0.0 ? sqrt(a / b) : sqrt(a);
      s_ok = (res <= threshold) ? 1 : 0;  // NaN fails the test: fallback
      if (res_out) res_out[s] = res;
      if (used) used[s] = s_ok;
    }
    __syncthreads();
    const int ok = s_ok;
    for (int e = threadIdx.x; e < P.nnz; e += blockDim.x) LU0[(size_t)s * P.nnz + e] = ok ? lu[e] : As[e];
  }
}

}  // namespace

cudaError_t launch_mlp_rowstats(const DevPattern& p, int nsys, const double* A, float* rown, float* coln, float* corr,
                                cudaStream_t st) {
  if (nsys == 0) return cudaSuccess;
  k_rowstats<<<nsys, 256, 0, st>>>(p, nsys, A, rown, coln, corr);
  return cudaGetLastError();
}

size_t mlp_train_smem() {
  return sizeof(float) * (((kMlpParams + 3) & ~3) + TB * NF + 4 * TB * LD + TB);
}

cudaError_t launch_mlp_train(const DevPattern& p, int nsys, const double* A, const double* LUt, const float* rown,
                             const float* coln, const float* corr, const void* pbf, int nsample, const int* idx,
                             uint64_t seed, float* grad, float* loss, cudaStream_t st) {
  if (nsample == 0) return cudaSuccess;
  const size_t smem = mlp_train_smem();
  cudaError_t e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_mlp_train<<<(nsample + TB - 1) / TB, TB, smem, st>>>(p, nsys, A, LUt, rown, coln, corr,
                                                         (const __nv_bfloat16*)pbf, nsample, idx, seed,
                                                         1.0f / (float)nsample, grad, loss);
  return cudaGetLastError();
}

cudaError_t launch_mlp_adam(float* p, float* m, float* v, const float* g, void* pbf, int count, float lr, int step,
                            cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
  k_adam<<<(count + 255) / 256, 256, 0, st>>>(p, m, v, g, (__nv_bfloat16*)pbf, count, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

cudaError_t launch_mlp_to_bf16(const float* p, void* pbf, int count, cudaStream_t st) {
  k_to_bf16<<<(count + 255) / 256, 256, 0, st>>>(p, (__nv_bfloat16*)pbf, count);
  return cudaGetLastError();
}

cudaError_t launch_mlp_eval(const DevPattern& p, int nsys, const double* A, const float* rown, const float* coln,
                            const float* corr, const void* pbf, int nsample, const int* idx, float* feat, float* out,
                            double* base, cudaStream_t st) {
  if (nsample == 0) return cudaSuccess;
  const size_t smem = sizeof(float) * ((kMlpParams + 3) & ~3);
  k_mlp_eval<<<(nsample + 127) / 128, 128, smem, st>>>(p, nsys, A, rown, coln, corr, (const __nv_bfloat16*)pbf,
                                                       nsample, idx, feat, out, base);
  return cudaGetLastError();
}

cudaError_t launch_mlp_warm(const DevPattern& p, int nsys, const double* A, const float* rown, const float* coln,
                            const float* corr, const void* pbf, double threshold, double* lu0, double* res, int* used,
                            cudaStream_t st) {
  if (nsys == 0) return cudaSuccess;
  const size_t smem = sizeof(float) * WP_WORDS + sizeof(double) * p.nnz;
  cudaError_t e = cudaFuncSetAttribute(k_mlp_warm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mlp_warm, WARM_THREADS, smem);
  if (e != cudaSuccess) return e;
  const int grid = nsys < nsm * (occ > 0 ? occ : 1) ? nsys : nsm * (occ > 0 ? occ : 1);
  k_mlp_warm<<<grid, WARM_THREADS, smem, st>>>(p, nsys, A, rown, coln, corr, (const __nv_bfloat16*)pbf, threshold,
                                               lu0, res, used);
  return cudaGetLastError();
}

}  // namespace bilu
