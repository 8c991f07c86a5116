// Branch-survival MLP on the 5th-generation tensor cores (sm_103a).
//
// Network: x (16 features) -> 128 ReLU -> 128 ReLU -> 1 logit. Weights are
// bfloat16 (PyTorch Linear layout: (out, in)), biases float32; every product
// accumulates in float32 in tensor memory.
//
// Each CTA (128 threads, one per sample row) works on tiles of 128 samples:
//   Z1 = X W1^T           tcgen05.mma M128 N128 K16      -> TMEM cols [0, 128)
//   H1 = relu(Z1 + b1)    tcgen05.ld, rounded to bf16 into shared memory
//   Z2 = H1 W2^T          M128 N128 K128                 -> TMEM cols [128, 256)
//   logit = relu(Z2 + b2) . w3 + b3                      (per thread, registers)
// and, for training (weighted binary cross-entropy with logits),
//   g     = scale * wt * (sigmoid(logit) - y)
//   dZ2   = g w3 * [H2 > 0]                              (bf16 into shared)
//   dH1   = dZ2 W2           M128 N128 K128              -> TMEM cols [0, 128)
//   dW2  += dZ2^T H1         M128 N128 K128 (over samples) TMEM cols [256, 384)
//   dZ1   = dH1 * [H1 > 0]                               (bf16 into shared)
//   dW1  += dZ1^T X          M128 N16  K128               TMEM cols [384, 400)
// Bias and w3 gradients are summed in shared memory; each CTA adds its
// partial sums to the global float32 gradients once at the end.
//
// Operands are staged by the threads in the canonical no-swizzle K-major
// layout: 8-row x 16-byte core matrices, core matrices adjacent along K
// (leading byte offset 128) and 8-row groups K/8 * 128 bytes apart (stride
// byte offset). One thread issues the MMAs and commits them to an mbarrier;
// every wait on it is bounded and a timeout sets LOKI_DEVERR_TIMEOUT in the
// error word, frees the tensor memory and returns.
#include <algorithm>
#include <cuda_bf16.h>

#include "loki_common.cuh"

namespace loki {

constexpr int kF = LOKI_MLP_FEATURES;  // 16
constexpr int kH = LOKI_MLP_HIDDEN;    // 128
constexpr int kTile = 128;             // samples per tile = threads per CTA
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kColZ1 = 0, kColZ2 = 128, kColDW2 = 256, kColDW1 = 384;
constexpr long long kSpinLimit = 1LL << 20;  // mbarrier polls before giving up

// ---- PTX wrappers -----------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the mbarrier phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (long long i = 0; i < kSpinLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy shared-memory writes become visible to the tensor cores.
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, bf16 inputs, f32 accumulate.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// 16 consecutive f32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor, no swizzle (layout type 0), version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor, kind::f16: D f32, A and B bf16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}

// Byte offset of element (r, k) of an R x K bf16 K-major no-swizzle tile.
__host__ __device__ __forceinline__ uint32_t kmaj_off(int r, int k, int K) {
  return (uint32_t)((r >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// C (tmem) (+)= A (rows x K) * B (n x K)^T, K a multiple of 16; issued by one thread.
__device__ __forceinline__ void mma_tile(uint32_t d_tmem, const void* a, const void* b, int K,
                                         int M, int N, bool accumulate) {
  const uint32_t sa = smem_u32(a), sb = smem_u32(b);
  const uint32_t sbo = (uint32_t)(K / 8) * 128;
  const uint32_t idesc = idesc_bf16(M, N);
  for (int kk = 0; kk < K / 16; ++kk) {
    const uint64_t ad = smem_desc(sa + kk * 256, 128, sbo);
    const uint64_t bd = smem_desc(sb + kk * 256, 128, sbo);
    mma_bf16(d_tmem, ad, bd, idesc, (accumulate || kk > 0) ? 1u : 0u);
  }
}

__device__ __forceinline__ void st_bf16(unsigned char* tile, int r, int k, int K, float v) {
  *reinterpret_cast<__nv_bfloat16*>(tile + kmaj_off(r, k, K)) = __float2bfloat16_rn(v);
}

// ---- shared-memory plan -----------------------------------------------------
struct MlpSmem {
  alignas(128) unsigned char w1[kH * kF * 2];   // B of Z1: rows j, K = f
  alignas(128) unsigned char w2[kH * kH * 2];   // B of Z2: rows j, K = i
  alignas(128) unsigned char w2t[kH * kH * 2];  // B of dH1: rows i, K = j
  alignas(128) unsigned char x[kTile * kF * 2];   // A of Z1: rows n, K = f
  alignas(128) unsigned char xt[kF * kTile * 2];  // B of dW1: rows f, K = n
  alignas(128) unsigned char r1[kTile * kH * 2];  // H1 (A of Z2), dZ2 (A of dH1), dZ1^T
  alignas(128) unsigned char h1t[kH * kTile * 2];  // B of dW2: rows i, K = n
  alignas(128) unsigned char dz2t[kH * kTile * 2];  // A of dW2: rows j, K = n
  float b1[kH], b2[kH], w3[kH];
  float gb1[kH], gb2[kH], gw3[kH];
  float gb3, loss;
  alignas(8) uint64_t bar;
  uint32_t tmem;
  int failed;
};

// Stage the weights (bf16 from global) into the operand tiles.
__device__ void stage_weights(MlpSmem& S, const LokiMLP& W, bool backward) {
  const __nv_bfloat16* w1 = static_cast<const __nv_bfloat16*>(W.w1);
  const __nv_bfloat16* w2 = static_cast<const __nv_bfloat16*>(W.w2);
  const __nv_bfloat16* w3 = static_cast<const __nv_bfloat16*>(W.w3);
  for (int t = threadIdx.x; t < kH * kF; t += blockDim.x) {
    const int j = t / kF, f = t % kF;
    *reinterpret_cast<__nv_bfloat16*>(S.w1 + kmaj_off(j, f, kF)) = w1[t];
  }
  for (int t = threadIdx.x; t < kH * kH; t += blockDim.x) {
    const int j = t / kH, i = t % kH;
    const __nv_bfloat16 v = w2[t];
    *reinterpret_cast<__nv_bfloat16*>(S.w2 + kmaj_off(j, i, kH)) = v;
    if (backward) *reinterpret_cast<__nv_bfloat16*>(S.w2t + kmaj_off(i, j, kH)) = v;
  }
  for (int t = threadIdx.x; t < kH; t += blockDim.x) {
    S.b1[t] = W.b1[t];
    S.b2[t] = W.b2[t];
    S.w3[t] = __bfloat162float(w3[t]);
    S.gb1[t] = S.gb2[t] = S.gw3[t] = 0.0f;
  }
  if (threadIdx.x == 0) {
    S.gb3 = 0.0f;
    S.loss = 0.0f;
  }
}

// Test hook (loki_mlp_force_timeout): when set, an MMA wait that completed is
// treated as one that gave up. The commit has landed, so no tensor-core work
// is left in flight; the kernel then takes its timeout path (TMEM freed,
// LOKI_DEVERR_TIMEOUT reported) exactly as after a real bounded-wait expiry.
__device__ int g_mlp_force_timeout = 0;

// One MMA group: thread 0 issues, commits; everyone waits (bounded).
template <typename F>
__device__ __forceinline__ bool mma_sync(MlpSmem& S, uint32_t& phase, F issue) {
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x == 0) {
    issue();
    mma_commit(&S.bar);
  }
  const bool ok = mbar_wait(&S.bar, phase) && !g_mlp_force_timeout;
  phase ^= 1u;
  tc_fence_after();
  if (!ok) S.failed = 1;
  __syncthreads();
  return !S.failed;
}

// Forward of one tile up to the logit; leaves H1 (bf16) in S.r1 and returns
// this thread's logit. relu masks of H1 and H2 are returned as bit sets.
__device__ bool forward_tile(MlpSmem& S, const LokiMLP& W, const float* __restrict__ x,
                             int64_t row0, int64_t n, uint32_t& phase, bool keep_t,
                             float& logit, uint32_t (&m1)[4], uint32_t (&m2)[4]) {
  const int t = threadIdx.x;
  const int64_t row = row0 + t;
  const uint32_t lane_base = (uint32_t)((t & ~31) << 16);
  // X tile (and X^T for dW1): zero rows past n
  for (int f = 0; f < kF; ++f) {
    const float v = row < n ? x[row * kF + f] : 0.0f;
    st_bf16(S.x, t, f, kF, v);
    if (keep_t) st_bf16(S.xt, f, t, kTile, v);
  }
  if (!mma_sync(S, phase, [&] { mma_tile(S.tmem + kColZ1, S.x, S.w1, kF, kTile, kH, false); }))
    return false;
  for (int c0 = 0; c0 < kH; c0 += 16) {
    float z[16];
    tmem_ld16(S.tmem + lane_base + kColZ1 + c0, z);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const float h = fmaxf(__fadd_rn(z[i], S.b1[c0 + i]), 0.0f);
      const __nv_bfloat16 hb = __float2bfloat16_rn(h);
      const int c = c0 + i;
      if (__bfloat162float(hb) > 0.0f) m1[c >> 5] |= 1u << (c & 31);
      *reinterpret_cast<__nv_bfloat16*>(S.r1 + kmaj_off(t, c, kH)) = hb;
      if (keep_t) *reinterpret_cast<__nv_bfloat16*>(S.h1t + kmaj_off(c, t, kTile)) = hb;
    }
  }
  if (!mma_sync(S, phase, [&] { mma_tile(S.tmem + kColZ2, S.r1, S.w2, kH, kTile, kH, false); }))
    return false;
  float acc = W.b3[0];
  for (int c0 = 0; c0 < kH; c0 += 16) {
    float z[16];
    tmem_ld16(S.tmem + lane_base + kColZ2 + c0, z);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const float h = fmaxf(__fadd_rn(z[i], S.b2[c0 + i]), 0.0f);
      const int c = c0 + i;
      if (h > 0.0f) m2[c >> 5] |= 1u << (c & 31);
      acc = fmaf(h, S.w3[c], acc);
    }
  }
  logit = acc;
  return true;
}

__device__ void finish(MlpSmem& S, int32_t* err) {
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x < 32) tmem_dealloc(S.tmem, kTmemCols);
  if (threadIdx.x == 0 && S.failed) atomicOr(err, LOKI_DEVERR_TIMEOUT);
}

__device__ void setup(MlpSmem& S) {
  if (threadIdx.x == 0) {
    mbar_init(&S.bar, 1);
    S.failed = 0;
  }
  if (threadIdx.x < 32) tmem_alloc(&S.tmem, kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
}

__global__ void __launch_bounds__(kTile, 1)
mlp_forward_kernel(LokiMLP W, const float* __restrict__ x, int64_t n, float* __restrict__ logits,
                   int32_t* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  MlpSmem& S = *reinterpret_cast<MlpSmem*>(smem_raw);
  setup(S);
  stage_weights(S, W, false);
  uint32_t phase = 0;
  const int64_t ntiles = (n + kTile - 1) / kTile;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    uint32_t m1[4] = {0, 0, 0, 0}, m2[4] = {0, 0, 0, 0};
    float logit;
    if (!forward_tile(S, W, x, tile * kTile, n, phase, false, logit, m1, m2)) break;
    const int64_t row = tile * kTile + threadIdx.x;
    if (row < n) logits[row] = logit;
  }
  finish(S, err);
}

__device__ __forceinline__ float softplus(float z) {
  return z > 0.0f ? z + log1pf(expf(-z)) : log1pf(expf(z));
}

__global__ void __launch_bounds__(kTile, 1)
mlp_backward_kernel(LokiMLP W, const float* __restrict__ x, const float* __restrict__ y,
                    const float* __restrict__ wt, int64_t n, float scale, LokiMLPGrad G,
                    float* __restrict__ logits, int32_t* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  MlpSmem& S = *reinterpret_cast<MlpSmem*>(smem_raw);
  setup(S);
  stage_weights(S, W, true);
  uint32_t phase = 0;
  const int t = threadIdx.x;
  const uint32_t lane_base = (uint32_t)((t & ~31) << 16);
  const int64_t ntiles = (n + kTile - 1) / kTile;
  bool first = true;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    uint32_t m1[4] = {0, 0, 0, 0}, m2[4] = {0, 0, 0, 0};
    float logit;
    if (!forward_tile(S, W, x, tile * kTile, n, phase, true, logit, m1, m2)) break;
    const int64_t row = tile * kTile + t;
    float g = 0.0f;
    if (row < n) {
      const float yy = y[row], ww = wt ? wt[row] : 1.0f;
      const float p = 1.0f / (1.0f + expf(-logit));
      g = scale * ww * (p - yy);
      atomicAdd(&S.loss, scale * ww * (softplus(logit) - yy * logit));
      atomicAdd(&S.gb3, g);
      if (logits) logits[row] = logit;
    }
    // dZ2 = g * w3 * [H2 > 0] into r1 (A of dH1) and dz2t (A of dW2); w3 grads
    // need H2, recomputed from TMEM
    for (int c0 = 0; c0 < kH; c0 += 16) {
      float z[16];
      tmem_ld16(S.tmem + lane_base + kColZ2 + c0, z);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int c = c0 + i;
        const float h2 = fmaxf(__fadd_rn(z[i], S.b2[c]), 0.0f);
        const bool on = (m2[c >> 5] >> (c & 31)) & 1u;
        const float d = on ? g * S.w3[c] : 0.0f;
        if (g != 0.0f) {
          atomicAdd(&S.gw3[c], g * h2);
          if (on) atomicAdd(&S.gb2[c], d);
        }
        const __nv_bfloat16 db = __float2bfloat16_rn(d);
        *reinterpret_cast<__nv_bfloat16*>(S.r1 + kmaj_off(t, c, kH)) = db;
        *reinterpret_cast<__nv_bfloat16*>(S.dz2t + kmaj_off(c, t, kTile)) = db;
      }
    }
    // dH1 = dZ2 W2 and dW2 += dZ2^T H1 in one commit group
    const bool acc = !first;
    if (!mma_sync(S, phase, [&] {
          mma_tile(S.tmem + kColZ1, S.r1, S.w2t, kH, kTile, kH, false);
          mma_tile(S.tmem + kColDW2, S.dz2t, S.h1t, kTile, kH, kH, acc);
        }))
      break;
    // dZ1 = dH1 * [H1 > 0], transposed into r1 (A of dW1: rows j, K = n)
    for (int c0 = 0; c0 < kH; c0 += 16) {
      float z[16];
      tmem_ld16(S.tmem + lane_base + kColZ1 + c0, z);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int c = c0 + i;
        const bool on = (m1[c >> 5] >> (c & 31)) & 1u;
        const float d = on ? z[i] : 0.0f;
        if (d != 0.0f) atomicAdd(&S.gb1[c], d);
        *reinterpret_cast<__nv_bfloat16*>(S.r1 + kmaj_off(c, t, kTile)) =
            __float2bfloat16_rn(d);
      }
    }
    if (!mma_sync(S, phase, [&] {
          mma_tile(S.tmem + kColDW1, S.r1, S.xt, kTile, kH, kF, acc);
        }))
      break;
    first = false;
  }
  if (!S.failed && !first) {
    // this CTA's weight-gradient partial sums: lane j holds row j
    for (int c0 = 0; c0 < kH; c0 += 16) {
      float v[16];
      tmem_ld16(S.tmem + lane_base + kColDW2 + c0, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) atomicAdd(&G.w2[t * kH + c0 + i], v[i]);
    }
    float v[16];
    tmem_ld16(S.tmem + lane_base + kColDW1, v);
#pragma unroll
    for (int i = 0; i < kF; ++i) atomicAdd(&G.w1[t * kF + i], v[i]);
  }
  __syncthreads();
  if (!S.failed) {
    atomicAdd(&G.b1[t], S.gb1[t]);
    atomicAdd(&G.b2[t], S.gb2[t]);
    atomicAdd(&G.w3[t], S.gw3[t]);
    if (t == 0) {
      atomicAdd(G.b3, S.gb3);
      atomicAdd(G.loss, S.loss);
    }
  }
  finish(S, err);
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, int64_t n, float lr,
                            float beta1, float beta2, float eps, float c1, float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = beta1 * m[i] + (1.0f - beta1) * gi;
    const float vi = beta2 * v[i] + (1.0f - beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// Branch statistics of n parents (warp per parent): score against the
// threshold passed and the next one, level, score z within the level, and the
// shape of the normalised fold e / sqrt(v) (peak, mean, spread, peak
// significance, fraction of bins above mean + 2 sigma). Approximate math: the
// statistics only rank branches for the network.
__global__ void branch_features_kernel(const float* __restrict__ scores,
                                       const float* __restrict__ folds, int64_t n, int nbins,
                                       float thr_prev, float thr_next, float level_frac,
                                       float inv_sqrt_level, float log_n,
                                       const float* __restrict__ score_stats,
                                       float* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (p >= n) return;
  const float* e = folds + p * 2 * nbins;
  const float* v = e + nbins;
  float mx = -INFINITY, sum = 0.0f, sq = 0.0f;
  for (int j = lane; j < nbins; j += 32) {
    const float x = e[j] * rsqrtf(fmaxf(v[j], 1e-30f));
    mx = fmaxf(mx, x);
    sum += x;
    sq += x * x;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
    sum += __shfl_xor_sync(0xFFFFFFFFu, sum, o);
    sq += __shfl_xor_sync(0xFFFFFFFFu, sq, o);
  }
  const float mean = sum / nbins;
  const float sd = sqrtf(fmaxf(sq / nbins - mean * mean, 1e-12f));
  int above = 0;
  for (int j = lane; j < nbins; j += 32) {
    const float x = e[j] * rsqrtf(fmaxf(v[j], 1e-30f));
    above += x > mean + 2.0f * sd;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) above += __shfl_xor_sync(0xFFFFFFFFu, above, o);
  if (lane == 0) {
    const float s = scores[p];
    float f[kF];
    f[0] = s;
    f[1] = s - thr_prev;
    f[2] = thr_next - s;
    f[3] = level_frac;
    f[4] = s * inv_sqrt_level;
    f[5] = mx;
    f[6] = mean;
    f[7] = sd;
    f[8] = (mx - mean) / sd;
    f[9] = (s - score_stats[0]) / fmaxf(score_stats[1], 1e-6f);
    f[10] = log_n;
    f[11] = thr_next;
    f[12] = (float)above / nbins;
    f[13] = f[14] = f[15] = 0.0f;
    float4* o = reinterpret_cast<float4*>(out + p * kF);
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = make_float4(f[4 * q], f[4 * q + 1], f[4 * q + 2],
                                                   f[4 * q + 3]);
  }
}

static int check_mlp(const LokiMLP* W) {
  if (!W || !W->w1 || !W->b1 || !W->w2 || !W->b2 || !W->w3 || !W->b3)
    return set_error(LOKI_ERR_INVALID, "null MLP parameter pointer");
  return LOKI_OK;
}

static int mlp_grid(int64_t n) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + kTile - 1) / kTile, sms));
}

}  // namespace loki

using namespace loki;

extern "C" int64_t loki_mlp_smem_bytes(void) { return (int64_t)sizeof(MlpSmem); }

extern "C" int loki_mlp_force_timeout(int32_t on) {
  const int v = on ? 1 : 0;
  if (cudaMemcpyToSymbol(g_mlp_force_timeout, &v, sizeof(v)) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaMemcpyToSymbol failed");
  return LOKI_OK;
}

extern "C" int loki_mlp_forward(const LokiMLP* w, const float* x, int64_t n, float* logits,
                                int32_t* dev_err, void* stream) {
  int rc = check_mlp(w);
  if (rc) return rc;
  if (n < 0) return set_error(LOKI_ERR_INVALID, "n < 0");
  if (n == 0) return LOKI_OK;
  if (!x || !logits || !dev_err) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const int smem = (int)sizeof(MlpSmem);
  if (set_smem_limit(mlp_forward_kernel, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  note_launch();
  mlp_forward_kernel<<<mlp_grid(n), kTile, smem, (cudaStream_t)stream>>>(*w, x, n, logits,
                                                                       dev_err);
  return check_launch("mlp_forward");
}

extern "C" int loki_mlp_backward(const LokiMLP* w, const float* x, const float* y,
                                 const float* wt, int64_t n, float scale,
                                 const LokiMLPGrad* grad, float* logits, int32_t* dev_err,
                                 void* stream) {
  int rc = check_mlp(w);
  if (rc) return rc;
  if (n < 0) return set_error(LOKI_ERR_INVALID, "n < 0");
  if (n == 0) return LOKI_OK;
  if (!x || !y || !grad || !dev_err || !grad->w1 || !grad->b1 || !grad->w2 || !grad->b2 ||
      !grad->w3 || !grad->b3 || !grad->loss)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const int smem = (int)sizeof(MlpSmem);
  if (set_smem_limit(mlp_backward_kernel, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  note_launch();
  mlp_backward_kernel<<<mlp_grid(n), kTile, smem, (cudaStream_t)stream>>>(
      *w, x, y, wt, n, scale, *grad, logits, dev_err);
  return check_launch("mlp_backward");
}

extern "C" int loki_mlp_adam(float* params, const float* grads, float* m, float* v, int64_t n,
                             float lr, float beta1, float beta2, float eps, int64_t step,
                             void* stream) {
  if (!params || !grads || !m || !v) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (n < 0 || step < 1) return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (n == 0) return LOKI_OK;
  const float c1 = 1.0f - (float)pow((double)beta1, (double)step);
  const float c2 = 1.0f - (float)pow((double)beta2, (double)step);
  note_launch();
  adam_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 1024), 256, 0,
                (cudaStream_t)stream>>>(params, grads, m, v, n, lr, beta1, beta2, eps, c1, c2);
  return check_launch("mlp_adam");
}

extern "C" int loki_branch_features(const float* scores, const float* folds, int64_t n,
                                    int32_t nbins, float thr_prev, float thr_next,
                                    float level_frac, float inv_sqrt_level,
                                    const float* score_stats, float* features, void* stream) {
  if (n < 0 || nbins < 1) return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (n == 0) return LOKI_OK;
  if (!scores || !folds || !score_stats || !features)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if ((reinterpret_cast<uintptr_t>(features) & 15) != 0)
    return set_error(LOKI_ERR_INVALID, "features must be 16-byte aligned");
  const float log_n = (float)(log2((double)n) / 20.0);
  const int64_t threads = n * 32;
  note_launch();
  branch_features_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      scores, folds, n, nbins, thr_prev, thr_next, level_frac, inv_sqrt_level, log_n,
      score_stats, features);
  return check_launch("branch_features");
}
