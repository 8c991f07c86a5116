// FFA dynamic-programming kernels: per-level plan, DP level, the final level
// fused with normalisation and boxcar scoring, and the banded driver.
//
// Data layout in HBM (identical to pyloki): fold (nseg, P, 2, nbins) float32,
// C-contiguous, P = flattened parameter grid with the frequency axis fastest.
// With LokiFFALevel.storage = 1 the folds are stored as bfloat16 instead:
// every add and every score is still evaluated in float32, each stored
// profile value is rounded once to bfloat16 (round to nearest even).
#include <cuda_bf16.h>

#include <algorithm>

#include "loki_common.cuh"
#include "resolve.cuh"
#include "score.cuh"

namespace loki {

// Element access of a fold stored as S (float or bfloat16), in float32.
template <typename S>
struct Store;

template <>
struct Store<float> {
  // four consecutive values, g = index of the 16-byte group
  static __device__ __forceinline__ float4 load4(const float* p, size_t g) {
    return __ldg(reinterpret_cast<const float4*>(p) + g);
  }
  static __device__ __forceinline__ void store4(float* p, size_t g, float4 v) {
    reinterpret_cast<float4*>(p)[g] = v;
  }
  static __device__ __forceinline__ float load(const float* p) { return __ldg(p); }
  static __device__ __forceinline__ void store(float* p, float v) { *p = v; }
};

template <>
struct Store<__nv_bfloat16> {
  static __device__ __forceinline__ float4 load4(const __nv_bfloat16* p, size_t g) {
    const uint2 u = __ldg(reinterpret_cast<const uint2*>(p) + g);
    const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u.x));
    const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&u.y));
    return make_float4(a.x, a.y, b.x, b.y);
  }
  static __device__ __forceinline__ void store4(__nv_bfloat16* p, size_t g, float4 v) {
    const __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y);
    const __nv_bfloat162 b = __floats2bfloat162_rn(v.z, v.w);
    uint2 u;
    u.x = *reinterpret_cast<const unsigned*>(&a);
    u.y = *reinterpret_cast<const unsigned*>(&b);
    reinterpret_cast<uint2*>(p)[g] = u;
  }
  static __device__ __forceinline__ float load(const __nv_bfloat16* p) {
    return __bfloat162float(p[0]);
  }
  static __device__ __forceinline__ void store(__nv_bfloat16* p, float v) {
    *p = __float2bfloat16_rn(v);
  }
};

// ---------------------------------------------------------------------------
// Plan table (exact FP64 path; the f32 shift is part of the output)
// ---------------------------------------------------------------------------

__device__ __forceinline__ void out_param(const LokiFFALevel& L, int64_t q, double* pset) {
  const int n = L.nparams;
  const int64_t last = L.out_start + q % L.out_width;
  int64_t rest = q / L.out_width;
  pset[n - 1] = L.param_arr[n - 1][last];
  for (int d = n - 2; d >= 0; --d) {
    const int64_t c = L.counts_cur[d];
    pset[d] = L.param_arr[d][rest % c];
    rest /= c;
  }
}

__device__ __forceinline__ int64_t flat_in(const LokiFFALevel& L, const int64_t* idx, bool* ok) {
  const int n = L.nparams;
  int64_t flat = 0;
  for (int d = 0; d < n - 1; ++d) flat = flat * L.counts_prev[d] + idx[d];
  const int64_t il = idx[n - 1] - L.in_start;
  if (il < 0 || il >= L.in_width) *ok = false;
  return flat * L.in_width + il;
}

__host__ __device__ __forceinline__ int64_t n_out_params(const LokiFFALevel& L) {
  int64_t q = L.out_width;
  for (int d = 0; d < L.nparams - 1; ++d) q *= L.counts_cur[d];
  return q;
}

__host__ __device__ __forceinline__ int64_t n_in_params(const LokiFFALevel& L) {
  int64_t q = L.in_width;
  for (int d = 0; d < L.nparams - 1; ++d) q *= L.counts_prev[d];
  return q;
}

__global__ void ffa_plan_kernel(LokiFFALevel L, LokiFFACoord* __restrict__ coords,
                                int32_t* __restrict__ err) {
  const int64_t Q = n_out_params(L);
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < Q;
       q += (int64_t)gridDim.x * blockDim.x) {
    double pset[LOKI_MAX_PARAMS];
    int64_t idx[LOKI_MAX_PARAMS];
    out_param(L, q, pset);
    bool ok = true;
    const double pt = ffa_resolve(pset, L.nparams, L.level, 0, L.tseg_brute, L.nbins,
                                  L.counts_prev, L.limits, idx);
    const int64_t it = flat_in(L, idx, &ok);
    const double ph = ffa_resolve(pset, L.nparams, L.level, 1, L.tseg_brute, L.nbins,
                                  L.counts_prev, L.limits, idx);
    const int64_t ih = flat_in(L, idx, &ok);
    if (!ok) atomicOr(err, LOKI_DEVERR_WINDOW);
    LokiFFACoord c;
    c.i_tail = (uint32_t)it;
    c.shift_tail = __double2float_rn(pt);
    c.i_head = (uint32_t)ih;
    c.shift_head = __double2float_rn(ph);
    coords[q] = c;
  }
}

// ---------------------------------------------------------------------------
// Trial resolution shared by the level kernels
// ---------------------------------------------------------------------------

// Each lane resolves one output parameter (q0 + lane) using the block's
// table of per-other quantities (or computes them itself when the block
// spans too many others).
struct LaneTrial {
  int64_t t, h;
  int st, sh;
  bool ok;
};

__device__ __forceinline__ LaneTrial lane_trial(const LokiFFALevel& L, const LevelK& K,
                                                const OtherTable& T, bool tab,
                                                const OtherRes* __restrict__ gtab,
                                                int64_t n_other, int64_t q, int64_t Q,
                                                int32_t* err) {
  LaneTrial r{0, 0, 0, 0, false};
  if (q >= Q) return r;
  int64_t other, off;
  q_split(L, K, q, other, off);
  TrialRes tr;
  if (gtab) {
    tr = resolve_trial(L, K, gtab[other], gtab[n_other + other], off);
  } else if (tab) {
    const int oi = (int)(other - T.first);
    tr = resolve_trial(L, K, T.e[0][oi], T.e[1][oi], off);
  } else {
    const OtherRes ot = make_other(L, K, other, 0);
    const OtherRes oh = make_other(L, K, other, 1);
    tr = resolve_trial(L, K, ot, oh, off);
  }
  r.t = tr.in_tail;
  r.h = tr.in_head;
  r.st = tr.s_tail;
  r.sh = tr.s_head;
  r.ok = tr.ok;
  if (!tr.ok) atomicOr(err, LOKI_DEVERR_WINDOW);
  return r;
}

// Roll of one (2, 64) profile row held as one float4 per lane (lane l holds
// component l >> 4, bins 4 (l & 15) .. + 3): out[j] = in[(j - s) mod 64] per
// component, assembled from two neighbouring lanes by shuffles.
__device__ __forceinline__ float4 roll64(const float4 x, int s, int lane) {
  const int q = s >> 2, r = s & 3;
  const int base = lane & 16, l16 = lane & 15;
  const int srcA = base | ((l16 - q) & 15);
  const float a0 = __shfl_sync(0xFFFFFFFFu, x.x, srcA);
  const float a1 = __shfl_sync(0xFFFFFFFFu, x.y, srcA);
  const float a2 = __shfl_sync(0xFFFFFFFFu, x.z, srcA);
  const float a3 = __shfl_sync(0xFFFFFFFFu, x.w, srcA);
  if (r == 0) return make_float4(a0, a1, a2, a3);
  const int srcB = base | ((l16 - q - 1) & 15);
  const float b1 = __shfl_sync(0xFFFFFFFFu, x.y, srcB);
  const float b2 = __shfl_sync(0xFFFFFFFFu, x.z, srcB);
  const float b3 = __shfl_sync(0xFFFFFFFFu, x.w, srcB);
  if (r == 1) return make_float4(b3, a0, a1, a2);
  if (r == 2) return make_float4(b2, b3, a0, a1);
  return make_float4(b1, b2, b3, a0);
}

__device__ __forceinline__ float4 add4(const float4 a, const float4 b) {
  return make_float4(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z),
                     __fadd_rn(a.w, b.w));
}

// ---------------------------------------------------------------------------
// DP level (unify_fold, dynamic/dyn_pffa.py:435-489 + shift_add
// core/common.py:304-324). Each warp owns 32 consecutive output parameters;
// lane k resolves parameter k once, then the warp streams the roll-add of
// every segment pair, pair-major, so neighbouring parameters (neighbouring
// frequencies) are read and written together.
// ---------------------------------------------------------------------------

constexpr int kLevelWarps = 8;
constexpr int kBatch = 4;

// nbins == 64: one float4 per lane per row, four rows in flight per lane.
// One warp's work: output parameters [q0, q0 + 32).
template <typename S>
__device__ __forceinline__ void level64_warp(const LokiFFALevel& L, const LevelK& K,
                                             const S* __restrict__ in, S* __restrict__ out,
                                             int32_t* err, const OtherTable& T, bool tab,
                                             const OtherRes* __restrict__ gtab,
                                             int64_t n_other, int64_t q0) {
  const int lane = threadIdx.x & 31;
  const int64_t Q = n_out_params(L), P_in = n_in_params(L);
  if (q0 >= Q) return;
  const LaneTrial me = lane_trial(L, K, T, tab, gtab, n_other, q0 + lane, Q, err);
  const int kmax = (int)std::min<int64_t>(32, Q - q0);
  const int64_t nseg_out = L.nseg_in / 2;
  for (int64_t ip = 0; ip < nseg_out; ++ip) {
    // rows of 32 four-value groups
    const size_t g_t = (size_t)(2 * ip) * P_in * 32;
    const size_t g_h = (size_t)(2 * ip + 1) * P_in * 32;
    const size_t g_o = ((size_t)ip * Q + q0) * 32;
    for (int k0 = 0; k0 < kmax; k0 += kBatch) {
      float4 tv[kBatch], hv[kBatch];
      int st[kBatch], sh[kBatch];
      bool ok[kBatch];
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        const int k = k0 + u;
        const int src = k < kmax ? k : 0;
        const int64_t it = __shfl_sync(0xFFFFFFFFu, me.t, src);
        const int64_t ih = __shfl_sync(0xFFFFFFFFu, me.h, src);
        st[u] = __shfl_sync(0xFFFFFFFFu, me.st, src);
        sh[u] = __shfl_sync(0xFFFFFFFFu, me.sh, src);
        ok[u] = __shfl_sync(0xFFFFFFFFu, me.ok, src) && k < kmax;
        if (ok[u]) {
          tv[u] = Store<S>::load4(in, g_t + (size_t)it * 32 + lane);
          hv[u] = Store<S>::load4(in, g_h + (size_t)ih * 32 + lane);
        }
      }
#pragma unroll
      for (int u = 0; u < kBatch; ++u) {
        if (!ok[u]) continue;  // uniform across the warp
        const float4 a = roll64(tv[u], st[u], lane);
        const float4 b = roll64(hv[u], sh[u], lane);
        Store<S>::store4(out, g_o + (size_t)(k0 + u) * 32 + lane, add4(a, b));
      }
    }
  }
}

template <typename S>
__global__ void __launch_bounds__(kLevelWarps * 32, 4)
ffa_level64_kernel(LokiFFALevel L, LevelK K, const S* __restrict__ in, S* __restrict__ out,
                   int32_t* __restrict__ err, const OtherRes* __restrict__ gtab,
                   int64_t n_other) {
  __shared__ OtherTable T;
  const int warp = threadIdx.x >> 5;
  const int64_t Q = n_out_params(L);
  const int64_t qb = (int64_t)blockIdx.x * kLevelWarps * 32;
  bool tab = false;
  if (!gtab) {  // uniform: the whole block takes the same branch
    tab = build_table(T, L, K, qb, std::min<int64_t>(qb + kLevelWarps * 32, Q) - 1);
    __syncthreads();
  }
  level64_warp(L, K, in, out, err, T, tab, gtab, n_other, qb + warp * 32);
}

// Any nbins: scalar, lane j handles bins j, j + 32, ...
template <typename S>
__global__ void __launch_bounds__(kLevelWarps * 32, 4)
ffa_level_kernel(LokiFFALevel L, LevelK K, const S* __restrict__ in, S* __restrict__ out,
                 int32_t* __restrict__ err, const OtherRes* __restrict__ gtab,
                 int64_t n_other) {
  __shared__ OtherTable T;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t Q = n_out_params(L), P_in = n_in_params(L);
  const int64_t qb = (int64_t)blockIdx.x * kLevelWarps * 32;
  bool tab = false;
  if (!gtab) {  // uniform: the whole block takes the same branch
    tab = build_table(T, L, K, qb, std::min<int64_t>(qb + kLevelWarps * 32, Q) - 1);
    __syncthreads();
  }
  const int64_t q0 = qb + warp * 32;
  if (q0 >= Q) return;
  const LaneTrial me = lane_trial(L, K, T, tab, gtab, n_other, q0 + lane, Q, err);
  const int nb = L.nbins;
  const int kmax = (int)std::min<int64_t>(32, Q - q0);
  const int64_t nseg_out = L.nseg_in / 2;
  const size_t row = (size_t)2 * nb;
  for (int64_t ip = 0; ip < nseg_out; ++ip) {
    const S* in_t = in + (size_t)(2 * ip) * P_in * row;
    const S* in_h = in + (size_t)(2 * ip + 1) * P_in * row;
    S* o_base = out + ((size_t)ip * Q + q0) * row;
    for (int k = 0; k < kmax; ++k) {
      const int64_t it = __shfl_sync(0xFFFFFFFFu, me.t, k);
      const int64_t ih = __shfl_sync(0xFFFFFFFFu, me.h, k);
      const int st = __shfl_sync(0xFFFFFFFFu, me.st, k);
      const int sh = __shfl_sync(0xFFFFFFFFu, me.sh, k);
      const bool ok = __shfl_sync(0xFFFFFFFFu, me.ok, k);
      if (!ok) continue;
      const S* t = in_t + (size_t)it * row;
      const S* h = in_h + (size_t)ih * row;
      S* o = o_base + (size_t)k * row;
      for (int j = lane; j < nb; j += 32) {
        int jt = j - st;
        jt += (jt < 0) ? nb : 0;
        int jh = j - sh;
        jh += (jh < 0) ? nb : 0;
        Store<S>::store(o + j, __fadd_rn(Store<S>::load(t + jt), Store<S>::load(h + jh)));
        Store<S>::store(o + nb + j,
                        __fadd_rn(Store<S>::load(t + nb + jt), Store<S>::load(h + nb + jh)));
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Final level fused with get_fold_norm (ffa.py:382-411) and boxcar scoring
// (detection/scoring.py:99-165), segment 0 only: the warp builds 32
// normalised profiles in its shared tile, then lane k scores row k.
// ---------------------------------------------------------------------------

constexpr int kScoreWarps = 4;

// Segments scored by one fused final-level launch: spec.nseg output segments
// (0 means 1: segment 0 only), S/N rows segment-major.
__host__ __device__ __forceinline__ int64_t n_score_segs(const LokiScoreSpec& sp) {
  return sp.nseg > 1 ? sp.nseg : 1;
}

__host__ __device__ __forceinline__ int64_t n_full_params(const LokiFFALevel& L) {
  int64_t q = 1;
  for (int d = 0; d < L.nparams; ++d) q *= L.counts_cur[d];
  return q;
}

__device__ __forceinline__ void score_out(const LokiFFALevel& L, const LevelK& K,
                                          const LokiScoreSpec& sp, const ScoreK& SK,
                                          float* tile, int stride, int lane, int64_t q0,
                                          int kmax, float* snr, int64_t seg) {
  __syncwarp();
  if (lane < kmax) {
    int64_t other, off;
    q_split(L, K, q0 + lane, other, off);
    const int64_t full = seg * n_full_params(L) + other * L.counts_cur[L.nparams - 1] +
                         L.out_start + off;
    const int nout = sp.mode == 0 ? sp.nwidths : 1;
    float* row = tile + lane * stride;
    if (SK.pow2_64) score_row64_pow2(row, sp, SK, snr + (size_t)full * nout);
    else score_row(row, L.nbins, sp, snr + (size_t)full * nout);
  }
}

// One warp's work of the fused final level: parameters [q0, q0 + 32).
template <typename S>
__device__ __forceinline__ void score64_warp(const LokiFFALevel& L, const LevelK& K,
                                             const S* __restrict__ in,
                                             const LokiScoreSpec& sp, const ScoreK& SK,
                                             float* __restrict__ snr, int32_t* err,
                                             const OtherTable& T, bool tab,
                                             const OtherRes* __restrict__ gtab,
                                             int64_t n_other, int64_t q0, float* tile,
                                             int64_t seg) {
  const int lane = threadIdx.x & 31;
  const int stride = score_stride(64, sp.wmax);
  const int64_t Q = n_out_params(L), P_in = n_in_params(L);
  if (q0 >= Q) return;
  const LaneTrial me = lane_trial(L, K, T, tab, gtab, n_other, q0 + lane, Q, err);
  const int kmax = (int)std::min<int64_t>(32, Q - q0);
  const S* in_t = in + (size_t)(2 * seg) * P_in * 128;  // segment 2 seg of fold_in
  const S* in_h = in_t + (size_t)P_in * 128;            // segment 2 seg + 1
  // Lane j gathers bins j and j + 32 of both components at the rolled
  // positions, so it owns e and v of its two output bins.
  for (int k0 = 0; k0 < kmax; k0 += kBatch) {
    float te[kBatch][2], tv[kBatch][2], he[kBatch][2], hv[kBatch][2];
    bool ok[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int k = k0 + u;
      const int src = k < kmax ? k : 0;
      const int64_t it = __shfl_sync(0xFFFFFFFFu, me.t, src);
      const int64_t ih = __shfl_sync(0xFFFFFFFFu, me.h, src);
      const int st = __shfl_sync(0xFFFFFFFFu, me.st, src);
      const int sh = __shfl_sync(0xFFFFFFFFu, me.sh, src);
      ok[u] = __shfl_sync(0xFFFFFFFFu, me.ok, src) && k < kmax;
      if (ok[u]) {
        const S* t = in_t + (size_t)it * 128;
        const S* h = in_h + (size_t)ih * 128;
        const int jt0 = (lane - st) & 63, jt1 = (lane + 32 - st) & 63;
        const int jh0 = (lane - sh) & 63, jh1 = (lane + 32 - sh) & 63;
        te[u][0] = Store<S>::load(t + jt0);
        te[u][1] = Store<S>::load(t + jt1);
        tv[u][0] = Store<S>::load(t + 64 + jt0);
        tv[u][1] = Store<S>::load(t + 64 + jt1);
        he[u][0] = Store<S>::load(h + jh0);
        he[u][1] = Store<S>::load(h + jh1);
        hv[u][0] = Store<S>::load(h + 64 + jh0);
        hv[u][1] = Store<S>::load(h + 64 + jh1);
      }
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      const int k = k0 + u;
      if (k >= kmax) break;
      float* trow = tile + k * stride;
      if (!ok[u]) {
        trow[lane] = 0.0f;
        trow[lane + 32] = 0.0f;
        continue;
      }
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const float e = __fadd_rn(te[u][c], he[u][c]);
        const float v = __fadd_rn(tv[u][c], hv[u][c]);
        trow[lane + 32 * c] = __fdiv_rn(e, __fsqrt_rn(v));
      }
    }
  }
  score_out(L, K, sp, SK, tile, stride, lane, q0, kmax, snr, seg);
}

template <typename S>
__global__ void __launch_bounds__(kScoreWarps * 32)
ffa_level_score64_kernel(LokiFFALevel L, LevelK K, const S* __restrict__ in,
                         LokiScoreSpec sp, ScoreK SK, float* __restrict__ snr,
                         int32_t* __restrict__ err, const OtherRes* __restrict__ gtab,
                         int64_t n_other) {
  __shared__ OtherTable T;
  extern __shared__ float tiles[];
  const int warp = threadIdx.x >> 5;
  float* tile = tiles + (size_t)warp * 32 * score_stride(64, sp.wmax);
  const int64_t Q = n_out_params(L);
  const int64_t nblk = (Q + blockDim.x - 1) / blockDim.x;  // blocks per segment
  const int64_t seg = blockIdx.x / nblk;
  const int64_t qb = (blockIdx.x - seg * nblk) * blockDim.x;
  bool tab = false;
  if (!gtab) {  // uniform: the whole block takes the same branch
    tab = build_table(T, L, K, qb, std::min<int64_t>(qb + blockDim.x, Q) - 1);
    __syncthreads();
  }
  score64_warp(L, K, in, sp, SK, snr, err, T, tab, gtab, n_other, qb + warp * 32, tile, seg);
}

// Banded pipeline step (nbins == 64): blocks [0, nblk_f) score final band k
// from scratch buffer k % 2 while the remaining blocks build the penultimate
// band k + 1 into the other buffer, so the small penultimate-level work fills
// the SMs the scoring leaves idle. Launch order alone orders the buffers:
// step k + 1 starts after step k has finished both halves.
// Five resident blocks per SM (<= 102 registers): measured 12 % faster than
// the register-limited four, though ptxas then spills 64 bytes per thread.
template <typename S>
__global__ void __launch_bounds__(kScoreWarps * 32, 5)
band_union64_kernel(LokiFFALevel F, LevelK KF, const S* __restrict__ in_f,
                    LokiScoreSpec sp, ScoreK SK, float* __restrict__ snr,
                    const OtherRes* __restrict__ tab_f, int64_t no_f, int64_t nblk_f,
                    LokiFFALevel P, LevelK KP, const S* __restrict__ in_p,
                    S* __restrict__ out_p, const OtherRes* __restrict__ tab_p,
                    int64_t no_p, int32_t* __restrict__ err) {
  extern __shared__ float tiles[];
  __shared__ OtherTable T;  // unused: both levels come with global tables
  const int warp = threadIdx.x >> 5;
  const int64_t nsc = nblk_f * n_score_segs(sp);  // scoring blocks, segment-major
  if (blockIdx.x < nsc) {
    float* tile = tiles + (size_t)warp * 32 * score_stride(64, sp.wmax);
    const int64_t seg = blockIdx.x / nblk_f;
    score64_warp(F, KF, in_f, sp, SK, snr, err, T, false, tab_f, no_f,
                 (blockIdx.x - seg * nblk_f) * blockDim.x + warp * 32, tile, seg);
  } else {
    level64_warp(P, KP, in_p, out_p, err, T, false, tab_p, no_p,
                 (int64_t)(blockIdx.x - nsc) * blockDim.x + warp * 32);
  }
}

template <typename S>
__global__ void __launch_bounds__(kScoreWarps * 32)
ffa_level_score_kernel(LokiFFALevel L, LevelK K, const S* __restrict__ in,
                       LokiScoreSpec sp, ScoreK SK, float* __restrict__ snr,
                       int32_t* __restrict__ err, const OtherRes* __restrict__ gtab,
                       int64_t n_other) {
  __shared__ OtherTable T;
  extern __shared__ float tiles[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nb = L.nbins;
  const int stride = score_stride(nb, sp.wmax);
  float* tile = tiles + (size_t)warp * 32 * stride;
  const int64_t Q = n_out_params(L), P_in = n_in_params(L);
  const int64_t nblk = (Q + blockDim.x - 1) / blockDim.x;  // blocks per segment
  const int64_t seg = blockIdx.x / nblk;
  const int64_t qb = (blockIdx.x - seg * nblk) * blockDim.x;
  bool tab = false;
  if (!gtab) {  // uniform: the whole block takes the same branch
    tab = build_table(T, L, K, qb, std::min<int64_t>(qb + blockDim.x, Q) - 1);
    __syncthreads();
  }
  const int64_t q0 = qb + warp * 32;
  if (q0 >= Q) return;
  const LaneTrial me = lane_trial(L, K, T, tab, gtab, n_other, q0 + lane, Q, err);
  const int kmax = (int)std::min<int64_t>(32, Q - q0);
  const size_t row = (size_t)2 * nb;
  const S* in_t = in + (size_t)(2 * seg) * P_in * row;
  const S* in_h = in_t + (size_t)P_in * row;
  for (int k = 0; k < kmax; ++k) {
    const int64_t it = __shfl_sync(0xFFFFFFFFu, me.t, k);
    const int64_t ih = __shfl_sync(0xFFFFFFFFu, me.h, k);
    const int st = __shfl_sync(0xFFFFFFFFu, me.st, k);
    const int sh = __shfl_sync(0xFFFFFFFFu, me.sh, k);
    const bool ok = __shfl_sync(0xFFFFFFFFu, me.ok, k);
    float* trow = tile + k * stride;
    if (!ok) {
      for (int j = lane; j < nb; j += 32) trow[j] = 0.0f;
      continue;
    }
    const S* t = in_t + (size_t)it * row;
    const S* h = in_h + (size_t)ih * row;
    for (int j = lane; j < nb; j += 32) {
      int jt = j - st;
      jt += (jt < 0) ? nb : 0;
      int jh = j - sh;
      jh += (jh < 0) ? nb : 0;
      const float e = __fadd_rn(Store<S>::load(t + jt), Store<S>::load(h + jh));
      const float v = __fadd_rn(Store<S>::load(t + nb + jt), Store<S>::load(h + nb + jh));
      trow[j] = __fdiv_rn(e, __fsqrt_rn(v));
    }
  }
  score_out(L, K, sp, SK, tile, stride, lane, q0, kmax, snr, seg);
}

// ---------------------------------------------------------------------------
// Last two levels fused per tile (nbins == 64, widths 1, 2, 4, ..., 2^(NW-1)).
//
// A tile is (output segment b, group of final "others", block of kTileF final
// frequencies). A group is a run of consecutive final others (every parameter
// but frequency) whose tail and head resolve to the same penultimate others,
// so its trials read one run of penultimate rows for the tail (penultimate
// segment 2b) and one for the head (segment 2b + 1). The CTA builds those rows
// in shared memory from the materialised level before them (the penultimate
// unify_fold, dynamic/dyn_pffa.py:435-489, restricted to the tile's window),
// then scores every final trial of the tile lane-per-trial from shared memory:
// the final shift-add, get_fold_norm (ffa.py:382-411) and the boxcar S/N
// (detection/scoring.py:99-165). Neither of the last two levels is written to
// global memory. Tiles are ordered frequency-block-major, so CTAs in flight
// share the rows of the level before (L2 hits) and each of its profiles comes
// from DRAM about once.
//
// Shared row layout: 64 float2 (e, v) per penultimate row (512 bytes, rows
// 512-byte aligned), so a trial rolled by shift s reads bin (j - s) mod 64 at
// byte (8 * (64 - s + j)) mod 512 of the row: one add and one and-or per load.
// Compact rows let six 4-warp CTAs share an SM (36 rows per side: one final
// other's 64 frequencies span at most 34 penultimate rows), and a chunk of two
// final others (the usual group size of an acceleration search) is exactly
// one 32-trial task per warp, so no warp idles while the others score.
// Consecutive lanes hold consecutive final frequencies, whose rows and shifts
// advance by about half a row and half a bin per lane, so the lanes of a warp
// spread over the banks.
//
// FAST: the profile is normalised as e * rsqrtf(v) (at most a few ulp from the
// reference's e / sqrt(v)); otherwise with correctly rounded division and
// square root, which makes the S/N bit-identical to the reference.
// ---------------------------------------------------------------------------

constexpr int kTileF = 64;        // final frequencies per tile
constexpr int kTileWarps = 4;
constexpr int kTileRows = 36;     // shared penultimate rows per side (tail, head)
constexpr int kTileMembers = 8;   // final others per chunk of a group
constexpr int kTileRowBytes = 64 * (int)sizeof(float2);

// Final others grouped by their (tail, head) penultimate other: groups[0] is
// the group count G, groups[1 + g] the first other of group g, groups[1 + G] =
// n_other. One block; a block-wide scan of the boundary flags.
__global__ void __launch_bounds__(1024) tile_groups_kernel(const OtherRes* __restrict__ tab,
                                                           int64_t n_other,
                                                           int32_t* __restrict__ groups) {
  __shared__ int warp_tot[32];
  __shared__ int carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < n_other; base += blockDim.x) {
    const int64_t o = base + threadIdx.x;
    bool flag = false;
    if (o < n_other)
      flag = o == 0 || tab[o].prefix != tab[o - 1].prefix ||
             tab[n_other + o].prefix != tab[n_other + o - 1].prefix;
    const unsigned bal = __ballot_sync(0xFFFFFFFFu, flag);
    if (lane == 0) warp_tot[warp] = __popc(bal);
    __syncthreads();
    if (warp == 0) {
      int v = lane < nwarps ? warp_tot[lane] : 0;
      for (int d = 1; d < 32; d <<= 1) {
        const int u = __shfl_up_sync(0xFFFFFFFFu, v, d);
        if (lane >= d) v += u;
      }
      if (lane < nwarps) warp_tot[lane] = v;  // inclusive
    }
    __syncthreads();
    const int before = (warp ? warp_tot[warp - 1] : 0) + __popc(bal & lanemask_lt());
    if (flag) groups[1 + carry + before] = (int32_t)o;
    __syncthreads();
    if (threadIdx.x == 0) carry += warp_tot[nwarps - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    groups[0] = carry;
    groups[1 + carry] = (int32_t)n_other;
  }
}

// Previous-level index (of the last, frequency, dimension; window not
// applied) of final frequency fidx for one other.
__device__ __forceinline__ int64_t tile_index(const LokiFFALevel& L, const LevelK& K,
                                              const OtherRes& o, int64_t fidx) {
  const double f = L.param_arr[L.nparams - 1][fidx];
  float f_hi, f_lo;
  if (L.last_split) {
    const float2 fs = reinterpret_cast<const float2*>(L.last_split)[fidx];
    f_hi = fs.x;
    f_lo = fs.y;
  } else {
    split2(f, &f_hi, &f_lo);
  }
  return trial_index(o, f, f_hi, f_lo, L, K);
}

template <typename S>
__device__ __forceinline__ float round_store(float x) {
  return x;
}
template <>
__device__ __forceinline__ float round_store<__nv_bfloat16>(float x) {
  return __bfloat162float(__float2bfloat16_rn(x));
}

// Builds the tile's penultimate rows (row r < nt: tail side, frequency lo_t + r
// of penultimate other pt in segment s_t; else head side) into shared memory.
// Warp w owns a contiguous run of rows; lane k resolves row k of the run and
// the warp then gathers row by row.
template <typename S>
__device__ __forceinline__ void tile_build(const LokiFFALevel& P, const LevelK& KP,
                                           const S* __restrict__ fold_pp,
                                           const OtherRes* __restrict__ tab_p, int64_t no_p,
                                           float2* rows, int nt, int nh, int64_t lo_t,
                                           int64_t lo_h, int64_t pt, int64_t ph, int64_t s_t,
                                           int64_t s_h, int32_t* err) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int R = nt + nh;
  const int per = (R + kTileWarps - 1) / kTileWarps;  // <= 2 * kTileRows / 4 = 20
  const int r0 = warp * per;
  const int r1 = std::min(R, r0 + per);
  const int64_t P_in = n_in_params(P);
  // lane k: row r0 + k
  int32_t my_t = 0, my_h = 0, my_sh = 0;
  bool my_ok = false;
  if (r0 + lane < r1) {
    const int r = r0 + lane;
    const bool tail = r < nt;
    const int64_t po = tail ? pt : ph;
    const int64_t f8 = tail ? lo_t + r : lo_h + (r - nt);
    const TrialRes tr = resolve_trial(P, KP, tab_p[po], tab_p[no_p + po], f8);
    my_t = (int32_t)tr.in_tail;
    my_h = (int32_t)tr.in_head;
    my_sh = tr.s_tail | (tr.s_head << 8);
    my_ok = tr.ok;
    if (!tr.ok) atomicOr(err, LOKI_DEVERR_WINDOW);
  }
  for (int r = r0; r < r1; ++r) {
    const int k = r - r0;
    const int32_t it = __shfl_sync(0xFFFFFFFFu, my_t, k);
    const int32_t ih = __shfl_sync(0xFFFFFFFFu, my_h, k);
    const int32_t sh2 = __shfl_sync(0xFFFFFFFFu, my_sh, k);
    const bool ok = __shfl_sync(0xFFFFFFFFu, my_ok, k);
    float2* dst = rows + (size_t)(r < nt ? r : kTileRows + (r - nt)) * 64;
    if (!ok) {
      dst[lane] = dst[lane + 32] = make_float2(0.f, 0.f);
      continue;
    }
    const int64_t seg8 = r < nt ? s_t : s_h;
    const S* t = fold_pp + ((size_t)(2 * seg8) * P_in + it) * 128;
    const S* h = fold_pp + ((size_t)(2 * seg8 + 1) * P_in + ih) * 128;
    const int st = sh2 & 0xFF, shh = sh2 >> 8;
    const int jt0 = (lane - st) & 63, jt1 = (lane + 32 - st) & 63;
    const int jh0 = (lane - shh) & 63, jh1 = (lane + 32 - shh) & 63;
    const float e0 = round_store<S>(__fadd_rn(Store<S>::load(t + jt0), Store<S>::load(h + jh0)));
    const float e1 = round_store<S>(__fadd_rn(Store<S>::load(t + jt1), Store<S>::load(h + jh1)));
    const float v0 =
        round_store<S>(__fadd_rn(Store<S>::load(t + 64 + jt0), Store<S>::load(h + 64 + jh0)));
    const float v1 =
        round_store<S>(__fadd_rn(Store<S>::load(t + 64 + jt1), Store<S>::load(h + 64 + jh1)));
    dst[lane] = make_float2(e0, v0);
    dst[lane + 32] = make_float2(e1, v1);
  }
}

// (e, v) of bin j of a compact row whose roll starts at byte offset `off`
// (= 8 * ((64 - s) mod 64)); `base` is the row's 512-aligned shared address.
__device__ __forceinline__ float2 tile_ld(uint32_t base, uint32_t off, int j) {
  const uint32_t a = base | ((off + 8u * (uint32_t)j) & 511u);
  float2 r;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(r.x), "=f"(r.y) : "r"(a));
  return r;
}

// The same bin as one 64-bit word: pack2(e, v) (e in the low half).
__device__ __forceinline__ unsigned long long tile_ld64(uint32_t base, uint32_t off, int j) {
  const uint32_t a = base | ((off + 8u * (uint32_t)j) & 511u);
  unsigned long long r;
  asm volatile("ld.shared.b64 %0, [%1];" : "=l"(r) : "r"(a));
  return r;
}

// S/N of one final trial from its tail and head rows (lane-per-trial). The
// prefix sum runs sequentially in float32 as circular_prefix_sum does and is
// kept as register pairs P2[k] = (P[2k], P[2k + 1]); every even width's
// window differences are packed f32x2 subtractions of two pairs, folded into
// the running maximum three at a time. The differences and the maximum are
// the reference's, so the S/N is unchanged.
template <bool FAST, int NW>
__device__ __forceinline__ void tile_score_trial(uint32_t bt, uint32_t ot, uint32_t bh,
                                                 uint32_t oh, const LokiScoreSpec& sp,
                                                 const ScoreK& SK, float* __restrict__ out) {
  constexpr int WMAX = 1 << (NW - 1);
  unsigned long long P2[32];
  float m[NW];
#pragma unroll
  for (int iw = 0; iw < NW; ++iw) m[iw] = -FLT_MAX;
  float s = 0.0f, prev = 0.0f;
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    float nv[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      // tail + head, e and v in one packed add (each half rounded as __fadd_rn)
      unsigned long long ev;
      asm("add.rn.f32x2 %0, %1, %2;"
          : "=l"(ev)
          : "l"(tile_ld64(bt, ot, 2 * k + q)), "l"(tile_ld64(bh, oh, 2 * k + q)));
      float e, v;
      unpack2(ev, e, v);
      nv[q] = FAST ? __fmul_rn(e, rsqrtf(v)) : __fdiv_rn(e, __fsqrt_rn(v));
    }
    const float s0 = k == 0 ? nv[0] : __fadd_rn(s, nv[0]);
    s = __fadd_rn(s0, nv[1]);
    P2[k] = pack2(s0, s);
    // width 1: P[2k] - P[2k - 1] and P[2k + 1] - P[2k]
    if (k == 0) m[0] = fmaxf(m[0], __fsub_rn(s, s0));
    else m[0] = max3(m[0], __fsub_rn(s0, prev), __fsub_rn(s, s0));
    prev = s;
#pragma unroll
    for (int iw = 1; iw < NW; ++iw) {
      const int H = 1 << (iw - 1);  // width 2H
      if (k >= H) {
        unsigned long long d;
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(P2[k]), "l"(P2[k - H]));
        float d0, d1;
        unpack2(d, d0, d1);
        m[iw] = max3(m[iw], d0, d1);
      }
    }
  }
  const float total = s;
  // circular extension P[64 + i] = P[i] + total (scoring.py:42-71)
  {
    float p0, p1;
    unpack2(P2[0], p0, p1);
    m[0] = fmaxf(m[0], __fsub_rn(__fadd_rn(p0, total), prev));  // P[64] - P[63]
  }
  const unsigned long long tt = pack2(total, total);
#pragma unroll
  for (int k = 0; k < WMAX / 2; ++k) {
    unsigned long long ext;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(ext) : "l"(P2[k]), "l"(tt));
#pragma unroll
    for (int iw = 1; iw < NW; ++iw) {
      const int H = 1 << (iw - 1);
      if (k < H) {
        unsigned long long d;
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(ext), "l"(P2[32 - H + k]));
        float d0, d1;
        unpack2(d, d0, d1);
        m[iw] = max3(m[iw], d0, d1);
      }
    }
  }
  float best = -FLT_MAX;
#pragma unroll
  for (int iw = 0; iw < NW; ++iw) {
    float r;
    if (SK.inv_one) {
      r = snr_fast(m[iw], total, SK.hb_hi[iw], SK.hb_lo[iw], SK.b_hi[iw], SK.b_lo[iw],
                   sp.hb[iw], sp.b[iw]);
    } else {
      const double x = __dsub_rn(__dmul_rn(sp.hb[iw], (double)m[iw]),
                                 __dmul_rn(sp.b[iw], (double)total));
      r = __double2float_rn(__dmul_rn(x, sp.inv_stdnoise));
    }
    if (sp.mode == 0) out[iw] = r;
    else if (r > best) best = r;
  }
  if (sp.mode != 0) out[0] = best;
}

template <typename S, bool FAST, int NW>
__global__ void __launch_bounds__(kTileWarps * 32, 6)
ffa_final_tiled64_kernel(LokiFFALevel P, LevelK KP, const S* __restrict__ fold_pp,
                         const OtherRes* __restrict__ tab_p, int64_t no_p, LokiFFALevel F,
                         LevelK KF, const OtherRes* __restrict__ tab_f, int64_t no_f,
                         const int32_t* __restrict__ groups, LokiScoreSpec sp, ScoreK SK,
                         float* __restrict__ snr, int32_t* __restrict__ err) {
  __shared__ __align__(512) float2 rows[2 * kTileRows * 64];  // [side][row][bin]
  __shared__ int64_t win[4];  // tail lo, tail hi, head lo, head hi
  const uint32_t rows_sh = (uint32_t)__cvta_generic_to_shared(rows);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n = F.nparams;
  const int64_t nlast = F.counts_cur[n - 1];
  const int64_t nfb = (nlast + kTileF - 1) / kTileF;
  const int64_t ngroups = groups[0];
  const int64_t nseg_out = n_score_segs(sp);
  const int64_t total = nseg_out * nfb * ngroups;
  const int64_t n_full = n_full_params(F);
  const int nout = sp.mode == 0 ? NW : 1;
  for (int64_t t = blockIdx.x; t < total; t += gridDim.x) {
    const int64_t g = t % ngroups;
    const int64_t rest = t / ngroups;
    const int64_t fb = rest % nfb;
    const int64_t b = rest / nfb;
    const int64_t o0 = groups[1 + g], o1 = groups[2 + g];
    const int64_t f0 = fb * kTileF;
    const int nf = (int)std::min<int64_t>(kTileF, nlast - f0);
    const int64_t pt = tab_f[o0].prefix, ph = tab_f[no_f + o0].prefix;
    int64_t c0 = o0;
    int step = kTileMembers;
    while (c0 < o1) {
      const int64_t c1 = std::min<int64_t>(c0 + step, o1);
      const int m = (int)(c1 - c0);
      __syncthreads();  // the previous chunk's rows and windows are no longer read
      if (threadIdx.x == 0) {
        win[0] = INT64_MAX;  // minima; indices are >= 0, so the maxima start at 0
        win[1] = 0;
        win[2] = INT64_MAX;
        win[3] = 0;
      }
      __syncthreads();
      if (threadIdx.x < 4 * m) {  // corners: (member, tail|head, first|last frequency)
        const int i = threadIdx.x >> 2, side = (threadIdx.x >> 1) & 1, last = threadIdx.x & 1;
        const int64_t o = c0 + i;
        const int64_t idx = tile_index(F, KF, tab_f[side * no_f + o], last ? f0 + nf - 1 : f0);
        atomicMin(reinterpret_cast<unsigned long long*>(&win[2 * side]),
                  (unsigned long long)idx);
        atomicMax(reinterpret_cast<unsigned long long*>(&win[2 * side + 1]),
                  (unsigned long long)idx);
      }
      __syncthreads();
      const int64_t lo_t = win[0], lo_h = win[2];
      const int nt = (int)(win[1] - win[0] + 1), nh = (int)(win[3] - win[2] + 1);
      if (nt > kTileRows || nh > kTileRows) {  // uniform across the block
        if (step > 1) {
          step = 1;  // redo this chunk one member at a time
          continue;
        }
        if (threadIdx.x == 0) atomicOr(err, LOKI_DEVERR_WINDOW);
        c0 = c1;
        continue;
      }
      tile_build<S>(P, KP, fold_pp, tab_p, no_p, rows, nt, nh, lo_t, lo_h, pt, ph, 2 * b,
                    2 * b + 1, err);
      __syncthreads();
      // trials: member-major, 32 consecutive frequencies per warp task
      const int tasks = m * (kTileF / 32);
      for (int q = warp; q < tasks; q += kTileWarps) {
        const int i = q / (kTileF / 32);
        const int fi = (q % (kTileF / 32)) * 32 + lane;
        if (fi >= nf) continue;
        const int64_t o = c0 + i;
        const int64_t fidx = f0 + fi;
        const OtherRes ot = tab_f[o], oh = tab_f[no_f + o];
        const TrialRes tr = resolve_trial(F, KF, ot, oh, fidx);
        const int64_t rt = tr.in_tail - ot.prefix * F.in_width - lo_t;
        const int64_t rh = tr.in_head - oh.prefix * F.in_width - lo_h;
        float* out = snr + (size_t)(b * n_full + o * nlast + fidx) * nout;
        if (!tr.ok || rt < 0 || rt >= nt || rh < 0 || rh >= nh) {
          atomicOr(err, LOKI_DEVERR_WINDOW);
          for (int k = 0; k < nout; ++k) out[k] = __int_as_float(0x7fc00000);
          continue;
        }
        const uint32_t bt = rows_sh + (uint32_t)rt * kTileRowBytes;
        const uint32_t bh = rows_sh + (uint32_t)(kTileRows + rh) * kTileRowBytes;
        const uint32_t offt = 8u * (uint32_t)((64 - tr.s_tail) & 63);
        const uint32_t offh = 8u * (uint32_t)((64 - tr.s_head) & 63);
        tile_score_trial<FAST, NW>(bt, offt, bh, offh, sp, SK, out);
      }
      c0 = c1;
    }
  }
}

// Previous-level frequency window needed by each band of current-level
// frequencies. The resolved frequency index is monotone in the current
// frequency for fixed other parameters (f_new = f * (1 - v/c)), so a band
// [g0, g1) needs [min idx at g0, max idx at g1 - 1] over every other-parameter
// combination, tail and head. One thread per (band, other combination).
__global__ void ffa_band_window_kernel(LokiFFALevel L, int64_t band_width, int64_t nbands,
                                       unsigned long long* __restrict__ lo,
                                       unsigned long long* __restrict__ hi) {
  const int n = L.nparams;
  int64_t n_other = 1;
  for (int d = 0; d < n - 1; ++d) n_other *= L.counts_cur[d];
  const int64_t nf = L.counts_cur[n - 1];
  const int64_t total = nbands * n_other;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t band = t / n_other;
    const int64_t other = t - band * n_other;
    const int64_t g0 = band * band_width;
    const int64_t g1 = min(g0 + band_width, nf) - 1;
    double pset[LOKI_MAX_PARAMS];
    int64_t idx[LOKI_MAX_PARAMS];
    int64_t rest = other;
    for (int d = n - 2; d >= 0; --d) {
      const int64_t c = L.counts_cur[d];
      pset[d] = L.param_arr[d][rest % c];
      rest /= c;
    }
    int64_t mn = INT64_MAX, mx = -1;
    for (int side = 0; side < 2; ++side) {
      pset[n - 1] = L.param_arr[n - 1][side ? g1 : g0];
      for (int latter = 0; latter < 2; ++latter) {
        ffa_resolve(pset, n, L.level, latter, L.tseg_brute, L.nbins, L.counts_prev, L.limits,
                    idx);
        mn = min(mn, idx[n - 1]);
        mx = max(mx, idx[n - 1]);
      }
    }
    atomicMin(lo + band, (unsigned long long)mn);
    atomicMax(hi + band, (unsigned long long)mx);
  }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------

static int check_level(const LokiFFALevel* L) {
  if (!L) return set_error(LOKI_ERR_INVALID, "null level descriptor");
  if (L->nparams < 1 || L->nparams > LOKI_MAX_PARAMS)
    return set_error(LOKI_ERR_INVALID, "nparams %d out of range", L->nparams);
  if (L->nbins < 2) return set_error(LOKI_ERR_INVALID, "nbins %d < 2", L->nbins);
  if (L->level < 1 || L->level > 62)
    return set_error(LOKI_ERR_INVALID, "level %d out of range", L->level);
  if (L->out_width <= 0 || L->in_width <= 0 || L->out_start < 0 || L->in_start < 0)
    return set_error(LOKI_ERR_INVALID, "empty or negative window");
  const int n = L->nparams;
  if (L->out_start + L->out_width > L->counts_cur[n - 1])
    return set_error(LOKI_ERR_INVALID, "output window beyond the grid");
  if (L->in_start + L->in_width > L->counts_prev[n - 1])
    return set_error(LOKI_ERR_INVALID, "input window beyond the grid");
  for (int d = 0; d < n; ++d) {
    if (!L->param_arr[d]) return set_error(LOKI_ERR_INVALID, "null param_arr[%d]", d);
    if (L->counts_cur[d] < 1 || L->counts_prev[d] < 1)
      return set_error(LOKI_ERR_INVALID, "grid count < 1 in dim %d", d);
  }
  if (L->nseg_in < 2 || (L->nseg_in & 1))
    return set_error(LOKI_ERR_INVALID, "nseg_in %lld must be even and >= 2",
                     (long long)L->nseg_in);
  return LOKI_OK;
}

static int check_spec(const LokiScoreSpec* sp, int nbins) {
  if (!sp) return set_error(LOKI_ERR_INVALID, "null score spec");
  if (sp->nwidths < 1 || sp->nwidths > LOKI_MAX_WIDTHS)
    return set_error(LOKI_ERR_INVALID, "nwidths %d out of range", sp->nwidths);
  int wmax = 0;
  for (int i = 0; i < sp->nwidths; ++i) {
    if (sp->widths[i] < 1) return set_error(LOKI_ERR_INVALID, "width < 1");
    wmax = std::max(wmax, (int)sp->widths[i]);
  }
  if (wmax != sp->wmax) return set_error(LOKI_ERR_INVALID, "wmax != max(widths)");
  if (nbins + wmax > 2048)
    return set_error(LOKI_ERR_UNSUPPORTED, "nbins + wmax = %d above 2048", nbins + wmax);
  if (sp->nseg < 0) return set_error(LOKI_ERR_INVALID, "spec nseg < 0");
  return LOKI_OK;
}

// The fused final level scores segments [0, nseg) of its output.
static int check_score_segs(const LokiFFALevel* L, const LokiScoreSpec* sp) {
  if (n_score_segs(*sp) > L->nseg_in / 2)
    return set_error(LOKI_ERR_INVALID, "spec nseg %d above the %lld output segments",
                     sp->nseg, (long long)(L->nseg_in / 2));
  return LOKI_OK;
}

int score_smem_bytes(int nbins, int wmax, int warps) {
  return warps * 32 * score_stride(nbins, wmax) * (int)sizeof(float);
}

int score_warps_per_block(int nbins, int wmax) {
  int w = kScoreWarps;
  while (w > 1 && score_smem_bytes(nbins, wmax, w) > 200 * 1024) w >>= 1;
  return w;
}

// Aligned float4 rows are required by the nbins == 64 kernels.
static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

template <typename S>
static int launch_level_t(const LokiFFALevel& L, const LevelK& K, const S* in, S* out,
                          int32_t* err, cudaStream_t s, const OtherRes* gtab, int64_t n_other) {
  const int64_t Q = n_out_params(L);
  const int64_t blocks = (Q + kLevelWarps * 32 - 1) / (kLevelWarps * 32);
  if (blocks > 0x7FFFFFFF) return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
  note_launch();
  if (L.nbins == 64 && aligned16(in) && aligned16(out))
    ffa_level64_kernel<S><<<(unsigned)blocks, kLevelWarps * 32, 0, s>>>(L, K, in, out, err,
                                                                        gtab, n_other);
  else
    ffa_level_kernel<S><<<(unsigned)blocks, kLevelWarps * 32, 0, s>>>(L, K, in, out, err, gtab,
                                                                      n_other);
  return LOKI_OK;
}

// Folds are float32 (storage 0) or bfloat16 (storage 1).
static int launch_level(const LokiFFALevel& L, const LevelK& K, const void* in, void* out,
                        int32_t* err, cudaStream_t s, const OtherRes* gtab = nullptr,
                        int64_t n_other = 0) {
  if (L.storage == 1)
    return launch_level_t(L, K, static_cast<const __nv_bfloat16*>(in),
                          static_cast<__nv_bfloat16*>(out), err, s, gtab, n_other);
  return launch_level_t(L, K, static_cast<const float*>(in), static_cast<float*>(out), err, s,
                        gtab, n_other);
}

template <typename S>
static int launch_level_score_t(const LokiFFALevel& L, const LevelK& K, const S* in,
                                const LokiScoreSpec& sp, const ScoreK& SK, float* snr,
                                int32_t* err, cudaStream_t s, const OtherRes* gtab,
                                int64_t n_other) {
  const bool fast = L.nbins == 64;
  const int warps = fast ? kScoreWarps : score_warps_per_block(L.nbins, sp.wmax);
  const int smem = score_smem_bytes(L.nbins, sp.wmax, warps);
  auto kern = fast ? ffa_level_score64_kernel<S> : ffa_level_score_kernel<S>;
  if (smem > 48 * 1024 &&
      set_smem_limit(kern, smem) !=
          cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  const int64_t Q = n_out_params(L);
  const int64_t blocks = (Q + warps * 32 - 1) / (warps * 32) * n_score_segs(sp);
  if (blocks > 0x7FFFFFFF) return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
  note_launch();
  kern<<<(unsigned)blocks, warps * 32, smem, s>>>(L, K, in, sp, SK, snr, err, gtab, n_other);
  return LOKI_OK;
}

static int launch_level_score(const LokiFFALevel& L, const LevelK& K, const void* in,
                              const LokiScoreSpec& sp, const ScoreK& SK, float* snr,
                              int32_t* err, cudaStream_t s, const OtherRes* gtab = nullptr,
                              int64_t n_other = 0) {
  if (L.storage == 1)
    return launch_level_score_t(L, K, static_cast<const __nv_bfloat16*>(in), sp, SK, snr, err,
                                s, gtab, n_other);
  return launch_level_score_t(L, K, static_cast<const float*>(in), sp, SK, snr, err, s, gtab,
                              n_other);
}

// Per-level table of the exact per-(latter, other) resolve quantities,
// entry [latter * n_other + other].
__global__ void other_table_kernel(LokiFFALevel L, LevelK K, OtherRes* __restrict__ tab,
                                   int64_t n_other) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 2 * n_other;
       t += (int64_t)gridDim.x * blockDim.x)
    tab[t] = make_other(L, K, t % n_other, (int)(t / n_other));
}

static int64_t n_other_of(const LokiFFALevel& L) {
  int64_t n = 1;
  for (int d = 0; d < L.nparams - 1; ++d) n *= L.counts_cur[d];
  return n;
}

// Floats of OtherRes table for one level (rounded up to 64-byte units).
static int64_t table_floats(const LokiFFALevel& L) {
  const int64_t bytes = 2 * n_other_of(L) * (int64_t)sizeof(OtherRes);
  return ((bytes + 63) / 64) * 16;
}

}  // namespace loki

using namespace loki;

extern "C" int loki_ffa_plan(const LokiFFALevel* lvl, LokiFFACoord* coords, int32_t* dev_err,
                             void* stream) {
  int rc = check_level(lvl);
  if (rc) return rc;
  if (!coords || !dev_err) return set_error(LOKI_ERR_INVALID, "null output pointer");
  const int64_t Q = n_out_params(*lvl);
  const int blocks = (int)std::min<int64_t>((Q + 255) / 256, 152 * 32);
  note_launch();
  ffa_plan_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(*lvl, coords, dev_err);
  return check_launch("ffa_plan");
}

extern "C" int loki_ffa_level(const LokiFFALevel* lvl, const void* fold_in, void* fold_out,
                              int32_t* dev_err, void* stream) {
  int rc = check_level(lvl);
  if (rc) return rc;
  if (!fold_in || !fold_out || !dev_err)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const LevelK K = make_level_k(*lvl);
  rc = launch_level(*lvl, K, fold_in, fold_out, dev_err, (cudaStream_t)stream);
  if (rc) return rc;
  return check_launch("ffa_level");
}

extern "C" int loki_ffa_level_score(const LokiFFALevel* lvl, const void* fold_in,
                                    const LokiScoreSpec* spec, float* snr, int32_t* dev_err,
                                    void* stream) {
  int rc = check_level(lvl);
  if (rc) return rc;
  rc = check_spec(spec, lvl->nbins);
  if (rc) return rc;
  rc = check_score_segs(lvl, spec);
  if (rc) return rc;
  if (!fold_in || !snr || !dev_err) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const LevelK K = make_level_k(*lvl);
  const ScoreK SK = make_score_k(*spec, lvl->nbins);
  rc = launch_level_score(*lvl, K, fold_in, *spec, SK, snr, dev_err, (cudaStream_t)stream);
  if (rc) return rc;
  return check_launch("ffa_level_score");
}

extern "C" int loki_ffa_band_windows(const LokiFFALevel* lvl, int64_t band_width,
                                     int64_t* win_lo, int64_t* win_hi, void* stream) {
  int rc = check_level(lvl);
  if (rc) return rc;
  if (band_width < 1) return set_error(LOKI_ERR_INVALID, "band_width < 1");
  if (!win_lo || !win_hi) return set_error(LOKI_ERR_INVALID, "null window pointer");
  const int64_t nf = lvl->counts_cur[lvl->nparams - 1];
  const int64_t nbands = (nf + band_width - 1) / band_width;
  int64_t n_other = 1;
  for (int d = 0; d < lvl->nparams - 1; ++d) n_other *= lvl->counts_cur[d];
  cudaStream_t s = (cudaStream_t)stream;
  // lo starts at all-ones (max unsigned), hi at zero.
  if (cudaMemsetAsync(win_lo, 0xFF, nbands * sizeof(int64_t), s) != cudaSuccess ||
      cudaMemsetAsync(win_hi, 0x00, nbands * sizeof(int64_t), s) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaMemsetAsync failed");
  const int64_t total = nbands * n_other;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 32);
  note_launch();
  ffa_band_window_kernel<<<blocks, 256, 0, s>>>(*lvl, band_width, nbands,
                                                (unsigned long long*)win_lo,
                                                (unsigned long long*)win_hi);
  return check_launch("ffa_band_windows");
}

extern "C" int loki_ffa_final_banded(const LokiFFALevel* pen, const LokiFFALevel* fin,
                                     int64_t band_width, const int64_t* win_lo,
                                     const int64_t* win_hi, const void* fold_pp, float* scratch,
                                     int64_t scratch_floats, const LokiScoreSpec* spec,
                                     float* snr, int32_t* dev_err, void* stream) {
  int rc = check_level(pen);
  if (rc) return rc;
  rc = check_level(fin);
  if (rc) return rc;
  rc = check_spec(spec, fin->nbins);
  if (rc) return rc;
  rc = check_score_segs(fin, spec);
  if (rc) return rc;
  if (!win_lo || !win_hi || !fold_pp || !scratch || !snr || !dev_err)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (band_width < 1) return set_error(LOKI_ERR_INVALID, "band_width < 1");
  if (fin->level != pen->level + 1 || pen->nseg_in != 2 * fin->nseg_in ||
      fin->nparams != pen->nparams || fin->storage != pen->storage)
    return set_error(LOKI_ERR_INVALID, "pen/fin descriptors are not consecutive levels");
  cudaStream_t s = (cudaStream_t)stream;
  const int n = fin->nparams;
  const int64_t nf = fin->counts_cur[n - 1];
  const int64_t nbands = (nf + band_width - 1) / band_width;
  int64_t other_pen = 1;
  for (int d = 0; d < n - 1; ++d) other_pen *= pen->counts_cur[d];
  const int64_t prof_floats = 2 * (int64_t)fin->nbins;
  LevelK KP = make_level_k(*pen);
  LevelK KF = make_level_k(*fin);
  const ScoreK SK = make_score_k(*spec, fin->nbins);
  // The per-other tables of both levels are the same for every band: build
  // them once at the end of the scratch buffer.
  const int64_t tab_floats = table_floats(*pen) + table_floats(*fin);
  if (tab_floats >= scratch_floats)
    return set_error(LOKI_ERR_CAPACITY, "scratch too small for the resolve tables");
  const int64_t band_floats = ((scratch_floats - tab_floats) / 16) * 16;
  OtherRes* tab_p = reinterpret_cast<OtherRes*>(scratch + band_floats);
  OtherRes* tab_f = reinterpret_cast<OtherRes*>(scratch + band_floats + table_floats(*pen));
  const int64_t no_p = n_other_of(*pen), no_f = n_other_of(*fin);
  note_launch();
  note_launch();
  other_table_kernel<<<(unsigned)std::min<int64_t>((2 * no_p + 127) / 128, 1024), 128, 0, s>>>(
      *pen, KP, tab_p, no_p);
  other_table_kernel<<<(unsigned)std::min<int64_t>((2 * no_f + 127) / 128, 1024), 128, 0, s>>>(
      *fin, KF, tab_f, no_f);
  LokiFFALevel P = *pen, F = *fin;
  for (int64_t k = 0; k < nbands; ++k) {
    const int64_t h0 = win_lo[k], wh = win_hi[k] - win_lo[k] + 1;
    if (wh < 1 || h0 < 0 || h0 + wh > pen->counts_cur[n - 1])
      return set_error(LOKI_ERR_INVALID, "band %lld has an invalid window", (long long)k);
    if (fin->nseg_in * other_pen * wh * prof_floats > band_floats)
      return set_error(LOKI_ERR_CAPACITY, "band %lld needs more scratch", (long long)k);
  }
  const int64_t half = ((band_floats / 2) / 16) * 16;
  int64_t wmax_win = 0;
  for (int64_t k = 0; k < nbands; ++k) wmax_win = std::max(wmax_win, win_hi[k] - win_lo[k] + 1);
  const bool pipelined = fin->nbins == 64 && aligned16(fold_pp) && aligned16(scratch) &&
                         fin->nseg_in * other_pen * wmax_win * prof_floats <= half;
  if (pipelined) {
    // Software pipeline over bands with two scratch buffers.
    float* buf[2] = {scratch, scratch + half};
    const int smem = score_smem_bytes(64, spec->wmax, kScoreWarps);
    const bool bf16 = fin->storage == 1;
    if (smem > 48 * 1024 &&
        (bf16 ? set_smem_limit(band_union64_kernel<__nv_bfloat16>, smem)
              : set_smem_limit(band_union64_kernel<float>, smem)) !=
            cudaSuccess)
      return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
    P.out_start = win_lo[0];
    P.out_width = win_hi[0] - win_lo[0] + 1;
    set_out_width(KP, P);
    rc = launch_level(P, KP, fold_pp, buf[0], dev_err, s, tab_p, no_p);
    if (rc) return rc;
    for (int64_t k = 0; k < nbands; ++k) {
      F.out_start = k * band_width;
      F.out_width = std::min(band_width, nf - F.out_start);
      F.in_start = win_lo[k];
      F.in_width = win_hi[k] - win_lo[k] + 1;
      set_out_width(KF, F);
      const int64_t nblk_f = (n_out_params(F) + kScoreWarps * 32 - 1) / (kScoreWarps * 32);
      int64_t nblk_p = 0;
      if (k + 1 < nbands) {
        P.out_start = win_lo[k + 1];
        P.out_width = win_hi[k + 1] - win_lo[k + 1] + 1;
        set_out_width(KP, P);
        nblk_p = (n_out_params(P) + kScoreWarps * 32 - 1) / (kScoreWarps * 32);
      }
      if (nblk_f * n_score_segs(*spec) + nblk_p > 0x7FFFFFFF)
        return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
      note_launch();
      const unsigned grid = (unsigned)(nblk_f * n_score_segs(*spec) + nblk_p);
      if (bf16)
        band_union64_kernel<__nv_bfloat16><<<grid, kScoreWarps * 32, smem, s>>>(
            F, KF, reinterpret_cast<const __nv_bfloat16*>(buf[k & 1]), *spec, SK, snr, tab_f,
            no_f, nblk_f, P, KP, static_cast<const __nv_bfloat16*>(fold_pp),
            reinterpret_cast<__nv_bfloat16*>(buf[(k + 1) & 1]), tab_p, no_p, dev_err);
      else
        band_union64_kernel<float><<<grid, kScoreWarps * 32, smem, s>>>(
            F, KF, buf[k & 1], *spec, SK, snr, tab_f, no_f, nblk_f, P, KP,
            static_cast<const float*>(fold_pp), buf[(k + 1) & 1], tab_p, no_p, dev_err);
    }
    return check_launch("ffa_final_banded");
  }
  for (int64_t k = 0; k < nbands; ++k) {
    const int64_t h0 = win_lo[k], wh = win_hi[k] - win_lo[k] + 1;
    P.out_start = h0;
    P.out_width = wh;
    set_out_width(KP, P);
    rc = launch_level(P, KP, fold_pp, scratch, dev_err, s, tab_p, no_p);
    if (rc) return rc;
    F.out_start = k * band_width;
    F.out_width = std::min(band_width, nf - F.out_start);
    F.in_start = h0;
    F.in_width = wh;
    set_out_width(KF, F);
    rc = launch_level_score(F, KF, scratch, *spec, SK, snr, dev_err, s, tab_f, no_f);
    if (rc) return rc;
  }
  return check_launch("ffa_final_banded");
}

extern "C" int64_t loki_ffa_final_banded_scratch(const LokiFFALevel* pen, const LokiFFALevel* fin,
                                                 int64_t max_window) {
  if (check_level(pen) || check_level(fin) || max_window < 1) return -1;
  // two band buffers (the banded pipeline double-buffers) plus the tables
  const int64_t band = fin->nseg_in * n_other_of(*pen) * max_window * 2 * (int64_t)fin->nbins;
  return 2 * (((band + 15) / 16) * 16) + table_floats(*pen) + table_floats(*fin);
}

namespace loki {

// ---- fused tiled last two levels --------------------------------------------

template <typename S, bool FAST, int NW>
static int launch_tiled_t(const LokiFFALevel& P, const LevelK& KP, const void* fold_pp,
                          const OtherRes* tab_p, int64_t no_p, const LokiFFALevel& F,
                          const LevelK& KF, const OtherRes* tab_f, int64_t no_f,
                          const int32_t* groups, const LokiScoreSpec& sp, const ScoreK& SK,
                          float* snr, int32_t* err, cudaStream_t s) {
  auto kern = ffa_final_tiled64_kernel<S, FAST, NW>;
  int dev = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTileWarps * 32, 0) !=
          cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "occupancy query failed");
  const int grid = std::max(1, nsm * std::max(1, per_sm));
  note_launch();
  kern<<<grid, kTileWarps * 32, 0, s>>>(P, KP, static_cast<const S*>(fold_pp), tab_p, no_p, F,
                                        KF, tab_f, no_f, groups, sp, SK, snr, err);
  return LOKI_OK;
}

template <typename S, bool FAST>
static int launch_tiled_nw(int nw, const LokiFFALevel& P, const LevelK& KP, const void* pp,
                           const OtherRes* tp, int64_t np_, const LokiFFALevel& F,
                           const LevelK& KF, const OtherRes* tf, int64_t nf_,
                           const int32_t* groups, const LokiScoreSpec& sp, const ScoreK& SK,
                           float* snr, int32_t* err, cudaStream_t s) {
  switch (nw) {
    case 1: return launch_tiled_t<S, FAST, 1>(P, KP, pp, tp, np_, F, KF, tf, nf_, groups, sp, SK, snr, err, s);
    case 2: return launch_tiled_t<S, FAST, 2>(P, KP, pp, tp, np_, F, KF, tf, nf_, groups, sp, SK, snr, err, s);
    case 3: return launch_tiled_t<S, FAST, 3>(P, KP, pp, tp, np_, F, KF, tf, nf_, groups, sp, SK, snr, err, s);
    case 4: return launch_tiled_t<S, FAST, 4>(P, KP, pp, tp, np_, F, KF, tf, nf_, groups, sp, SK, snr, err, s);
    case 5: return launch_tiled_t<S, FAST, 5>(P, KP, pp, tp, np_, F, KF, tf, nf_, groups, sp, SK, snr, err, s);
    default: return launch_tiled_t<S, FAST, 6>(P, KP, pp, tp, np_, F, KF, tf, nf_, groups, sp, SK, snr, err, s);
  }
}

static int64_t tiled_scratch_bytes(const LokiFFALevel& pen, const LokiFFALevel& fin) {
  return (int64_t)sizeof(float) * (table_floats(pen) + table_floats(fin)) +
         (int64_t)sizeof(int32_t) * (n_other_of(fin) + 2);
}

}  // namespace loki

extern "C" int64_t loki_ffa_final_tiled_scratch(const LokiFFALevel* pen,
                                                const LokiFFALevel* fin) {
  if (check_level(pen) || check_level(fin)) return -1;
  return tiled_scratch_bytes(*pen, *fin);
}

extern "C" int loki_ffa_final_tiled(const LokiFFALevel* pen, const LokiFFALevel* fin,
                                    const void* fold_pp, void* scratch, int64_t scratch_bytes,
                                    const LokiScoreSpec* spec, int32_t fast_norm, float* snr,
                                    int32_t* dev_err, void* stream) {
  int rc = check_level(pen);
  if (rc) return rc;
  rc = check_level(fin);
  if (rc) return rc;
  rc = check_spec(spec, fin->nbins);
  if (rc) return rc;
  rc = check_score_segs(fin, spec);
  if (rc) return rc;
  if (!fold_pp || !scratch || !snr || !dev_err)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (fin->level != pen->level + 1 || pen->nseg_in != 2 * fin->nseg_in ||
      fin->nparams != pen->nparams || fin->storage != pen->storage)
    return set_error(LOKI_ERR_INVALID, "pen/fin descriptors are not consecutive levels");
  const int n = fin->nparams;
  if (pen->out_start != 0 || pen->out_width != pen->counts_cur[n - 1] || pen->in_start != 0 ||
      pen->in_width != pen->counts_prev[n - 1] || fin->out_start != 0 ||
      fin->out_width != fin->counts_cur[n - 1] || fin->in_start != 0 ||
      fin->in_width != pen->counts_cur[n - 1])
    return set_error(LOKI_ERR_INVALID, "the tiled final levels take full (unwindowed) grids");
  if (fin->nbins != 64)
    return set_error(LOKI_ERR_UNSUPPORTED, "the tiled final levels need nbins == 64");
  const ScoreK SK = make_score_k(*spec, fin->nbins);
  if (!SK.pow2_64)
    return set_error(LOKI_ERR_UNSUPPORTED, "the tiled final levels need widths 1, 2, 4, ... 32");
  if (n_in_params(*pen) >= (int64_t(1) << 31) || n_other_of(*fin) >= (int64_t(1) << 31))
    return set_error(LOKI_ERR_UNSUPPORTED, "grids above 2^31 parameter sets per segment");
  if (scratch_bytes < tiled_scratch_bytes(*pen, *fin))
    return set_error(LOKI_ERR_CAPACITY, "scratch of %lld bytes below the %lld needed",
                     (long long)scratch_bytes, (long long)tiled_scratch_bytes(*pen, *fin));
  if ((reinterpret_cast<uintptr_t>(scratch) & 63) != 0)
    return set_error(LOKI_ERR_INVALID, "scratch must be 64-byte aligned");
  cudaStream_t s = (cudaStream_t)stream;
  const LevelK KP = make_level_k(*pen);
  const LevelK KF = make_level_k(*fin);
  float* sc = static_cast<float*>(scratch);
  OtherRes* tab_p = reinterpret_cast<OtherRes*>(sc);
  OtherRes* tab_f = reinterpret_cast<OtherRes*>(sc + table_floats(*pen));
  int32_t* groups = reinterpret_cast<int32_t*>(sc + table_floats(*pen) + table_floats(*fin));
  const int64_t no_p = n_other_of(*pen), no_f = n_other_of(*fin);
  note_launch();
  note_launch();
  note_launch();
  other_table_kernel<<<(unsigned)std::min<int64_t>((2 * no_p + 127) / 128, 1024), 128, 0, s>>>(
      *pen, KP, tab_p, no_p);
  other_table_kernel<<<(unsigned)std::min<int64_t>((2 * no_f + 127) / 128, 1024), 128, 0, s>>>(
      *fin, KF, tab_f, no_f);
  tile_groups_kernel<<<1, 1024, 0, s>>>(tab_f, no_f, groups);
  const int nw = spec->nwidths;
  if (fin->storage == 1)
    rc = fast_norm ? launch_tiled_nw<__nv_bfloat16, true>(nw, *pen, KP, fold_pp, tab_p, no_p,
                                                          *fin, KF, tab_f, no_f, groups, *spec,
                                                          SK, snr, dev_err, s)
                   : launch_tiled_nw<__nv_bfloat16, false>(nw, *pen, KP, fold_pp, tab_p, no_p,
                                                           *fin, KF, tab_f, no_f, groups, *spec,
                                                           SK, snr, dev_err, s);
  else
    rc = fast_norm ? launch_tiled_nw<float, true>(nw, *pen, KP, fold_pp, tab_p, no_p, *fin, KF,
                                                  tab_f, no_f, groups, *spec, SK, snr, dev_err, s)
                   : launch_tiled_nw<float, false>(nw, *pen, KP, fold_pp, tab_p, no_p, *fin, KF,
                                                   tab_f, no_f, groups, *spec, SK, snr, dev_err,
                                                   s);
  if (rc) return rc;
  return check_launch("ffa_final_tiled");
}

namespace loki {
__global__ void f32_to_bf16_kernel(const float* __restrict__ in, int64_t n,
                                   __nv_bfloat16* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16_rn(in[i]);
}
}  // namespace loki

extern "C" int loki_f32_to_bf16(const float* in, int64_t n, void* out, void* stream) {
  if (n < 0) return set_error(LOKI_ERR_INVALID, "n < 0");
  if (n == 0) return LOKI_OK;
  if (!in || !out) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  note_launch();
  f32_to_bf16_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 64), 256, 0,
                       (cudaStream_t)stream>>>(in, n, static_cast<__nv_bfloat16*>(out));
  return check_launch("f32_to_bf16");
}
