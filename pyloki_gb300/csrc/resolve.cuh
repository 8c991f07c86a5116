// FFA resolve, split into a per-"other parameter" part and a per-trial part.
//
// The reference resolves every parameter set independently
// (core/fold.py:617-671): shift the Taylor vector by dt, re-reference the
// frequency f_new = f * (1 - v/c), find the previous-level grid index, and the
// relative phase frac((dt - delay) * f) * nbins. Everything except the last
// (frequency) coordinate depends only on the other parameters, so it is
// computed once per (latter, other-index) in exact FP64 (OtherRes) and shared.
//
// Per trial only two quantities remain: the frequency index
//   trunc(RN(RN(n * RN(RN(f * om) - fmin)) / range) + 1e-6)
// and the rounded shift of frac(RN(g * f)) * nbins. Both are first estimated
// in two-float FP32 arithmetic (~2^-46 relative); when the estimate is more
// than 1e-4 (index or bin units) away from the next rounding boundary the
// integer is certain, otherwise the exact FP64 chain is evaluated. The result
// is therefore identical to the FP64 reference for every trial.
#pragma once

#include "loki_common.cuh"

namespace loki {

constexpr int kMaxOthersPerBlock = 16;

// Per-level constants computed on the host with the device's exact rules.
struct LevelK {
  double dt[2];
  double tmat[2][LOKI_MAX_PARAMS + 1][LOKI_MAX_PARAMS + 1];  // RN(dt^(i-j) / (i-j)!)
  double scale_last;  // counts_prev[n-1] / (vmax - vmin), for the estimate only
  float B_hi, B_lo;   // fmin * scale_last - 1e-6 as a two-float
  FastDiv32 wdiv;     // division by out_width (valid when use_fd)
  int use_fd;         // all output indices fit in 32 bits
};

// Output parameter q of the windowed grid -> (other index, offset in window).
__host__ __device__ inline void set_out_width(LevelK& K, const LokiFFALevel& L) {
  int64_t q = L.out_width;
  for (int d = 0; d < L.nparams - 1; ++d) q *= L.counts_cur[d];
  K.use_fd = (q < (1ll << 32) && L.out_width < (1ll << 32)) ? 1 : 0;
  K.wdiv = FastDiv32::make(K.use_fd ? (uint32_t)L.out_width : 1u);
}

__device__ __forceinline__ void q_split(const LokiFFALevel& L, const LevelK& K, int64_t q,
                                        int64_t& other, int64_t& off) {
  if (K.use_fd) {
    const uint32_t o = K.wdiv.div((uint32_t)q);
    other = o;
    off = (int64_t)((uint32_t)q - o * (uint32_t)L.out_width);
  } else {
    other = q / L.out_width;
    off = q - other * L.out_width;
  }
}

struct OtherRes {
  double om;       // f multiplier: RN(1 - RN(v'/c)); exactly 1 for one parameter
  double g;        // RN(dt - delay)
  int64_t prefix;  // flattened previous-level index over dims 0..n-2
  float A_hi, A_lo;  // om * scale_last (two-float)
  float g_hi, g_lo;  // g (two-float)
};

__host__ __device__ inline double host_pow_rn(double x, int p) {
  if (p == 0) return 1.0;
  if (p == 1) return x;
  if (p == 2) return x * x;
  double hi = x * x;
  double lo = fma(x, x, -hi);
  for (int k = 3; k <= p; ++k) {
    double nh = hi * x;
    double nl = fma(hi, x, -nh);
    nl = fma(lo, x, nl);
    hi = nh + nl;
    lo = nl - (hi - nh);
  }
  return hi;
}

// Host: per-level constants (requires -ffp-contract=off in the host compiler).
inline LevelK make_level_k(const LokiFFALevel& L) {
  LevelK K;
  const int n = L.nparams;
  const double two_pow = (double)(1LL << (L.level - 1));
  const double fact[8] = {1.0, 1.0, 2.0, 6.0, 24.0, 120.0, 720.0, 5040.0};
  for (int latter = 0; latter < 2; ++latter) {
    K.dt[latter] = (n == 1) ? ((double)latter * two_pow) * L.tseg_brute
                            : (((double)latter - 0.5) * two_pow) * L.tseg_brute;
    for (int i = 0; i <= LOKI_MAX_PARAMS; ++i)
      for (int j = 0; j <= LOKI_MAX_PARAMS; ++j)
        K.tmat[latter][i][j] =
            (j <= i) ? host_pow_rn(K.dt[latter], i - j) / fact[i - j] : 0.0;
  }
  const double vmin = L.limits[n - 1][0], vmax = L.limits[n - 1][1];
  K.scale_last = (double)L.counts_prev[n - 1] / (vmax - vmin);
  const double B = vmin * K.scale_last - LOKI_FLOAT_EPSILON;
  K.B_hi = (float)B;
  K.B_lo = (float)(B - (double)K.B_hi);
  set_out_width(K, L);
  return K;
}

__device__ __forceinline__ void split2(double x, float* hi, float* lo) {
  *hi = __double2float_rn(x);
  *lo = __double2float_rn(__dsub_rn(x, (double)*hi));
}

// Exact per-(latter, other) part of ffa_resolve (same operations and order).
__device__ inline OtherRes make_other(const LokiFFALevel& L, const LevelK& K, int64_t other,
                                      int latter) {
  const int n = L.nparams;
  OtherRes o;
  o.prefix = 0;
  if (n == 1) {
    o.om = 1.0;
    o.g = K.dt[latter];
  } else {
    double tv[LOKI_MAX_PARAMS + 1];
    int64_t rest = other;
    for (int d = n - 2; d >= 0; --d) {
      const int64_t c = L.counts_cur[d];
      tv[d] = L.param_arr[d][rest % c];
      rest /= c;
    }
    double out[LOKI_MAX_PARAMS + 1];
    for (int i = 0; i <= n; ++i) {
      const int jmax = i < n - 2 ? i : n - 2;
      double acc = __dmul_rn(tv[0], K.tmat[latter][i][0]);
      for (int j = 1; j <= jmax; ++j) acc = __dadd_rn(acc, __dmul_rn(tv[j], K.tmat[latter][i][j]));
      out[i] = acc;
    }
    int64_t flat = 0;
    for (int d = 0; d < n - 1; ++d)
      flat = flat * L.counts_prev[d] +
             nearest_index(out[d], L.counts_prev[d], L.limits[d][0], L.limits[d][1]);
    o.prefix = flat;
    o.om = __dsub_rn(1.0, __ddiv_rn(out[n - 1], LOKI_C_VAL));
    const double delay = __ddiv_rn(out[n], LOKI_C_VAL);
    o.g = __dsub_rn(K.dt[latter], delay);
  }
  split2(__dmul_rn(o.om, K.scale_last), &o.A_hi, &o.A_lo);
  split2(o.g, &o.g_hi, &o.g_lo);
  return o;
}

// Exact FP64 chains, out of line so they only run when the estimate is
// inconclusive (the compiler must not evaluate them speculatively).
static __device__ __noinline__ int64_t trial_index_exact(double f, double om, int64_t n_grid,
                                                  double vmin, double vmax) {
  return nearest_index(__dmul_rn(f, om), n_grid, vmin, vmax);
}

static __device__ __noinline__ int trial_shift_exact(double g, double f, int nbins) {
  const double x = __dmul_rn(g, f);
  const double ph = __dsub_rn(x, floor(x));
  double ip = __dmul_rn(ph, (double)nbins);
  if (ip >= (double)nbins) ip = 0.0;
  return round_shift(ip, nbins);
}

// Previous-level index of the frequency coordinate. Returns it exactly.
__device__ __forceinline__ int64_t trial_index(const OtherRes& o, double f, float f_hi,
                                               float f_lo, const LokiFFALevel& L,
                                               const LevelK& K) {
  const int n = L.nparams;
  const int64_t n_grid = L.counts_prev[n - 1];
  if (n_grid <= 1) return 0;
  // estimate t = f * A - B  (~ raw + 1e-6)
  const float p = f_hi * o.A_hi;
  float e = fmaf(f_hi, o.A_hi, -p);
  e = fmaf(f_hi, o.A_lo, e);
  e = fmaf(f_lo, o.A_hi, e);
  const float s = p - K.B_hi;
  const float bb = s - p;
  const float err = (p - (s - bb)) + (-K.B_hi - bb);
  const float r = (err + e) - K.B_lo;
  const float fs = floorf(s);
  const float fr = (s - fs) + r;
  const float fl = floorf(fr);
  const float frac = fr - fl;
  if (frac > 1e-4f && frac < 1.0f - 1e-4f && fabsf(p) < 1.0e9f && fabsf(s) < 2.0e9f) {
    // fs and fl (in {-1, 0, 1, 2}) fit 32-bit integers, whose conversions
    // avoid the slow 64-bit conversion path
    int64_t idx = (int64_t)((int)fs + (int)fl);
    if (idx < 0) idx = 0;
    else if (idx >= n_grid) idx = n_grid - 1;
    return idx;
  }
  return trial_index_exact(f, o.om, n_grid, L.limits[n - 1][0], L.limits[n - 1][1]);
}

// Rounded relative shift in bins. Returns it exactly.
__device__ __forceinline__ int trial_shift(const OtherRes& o, double f, float f_hi, float f_lo,
                                           int nbins) {
  const float p = o.g_hi * f_hi;
  float e = fmaf(o.g_hi, f_hi, -p);
  e = fmaf(o.g_hi, f_lo, e);
  e = fmaf(o.g_lo, f_hi, e);
  float fr = (p - floorf(p)) + e;
  fr -= floorf(fr);
  const float u = fmaf(fr, (float)nbins, 0.5f);
  const float k = floorf(u);
  const float rem = u - k;
  if (rem > 1e-4f && rem < 1.0f - 1e-4f && fabsf(p) < 4.0e6f) {
    int s = (int)k;
    return s >= nbins ? s - nbins : s;
  }
  return trial_shift_exact(o.g, f, nbins);
}

// The others spanned by a block's consecutive output parameters, tabulated in
// shared memory (both latters). Returns false when they do not fit.
struct OtherTable {
  OtherRes e[2][kMaxOthersPerBlock];
  int64_t first;
  int count;
};

__device__ __forceinline__ bool build_table(OtherTable& T, const LokiFFALevel& L,
                                            const LevelK& K, int64_t q_first, int64_t q_last) {
  const int64_t o0 = q_first / L.out_width;
  const int64_t o1 = q_last / L.out_width;
  const int64_t cnt = o1 - o0 + 1;
  if (cnt > kMaxOthersPerBlock) return false;
  if (threadIdx.x == 0) {
    T.first = o0;
    T.count = (int)cnt;
  }
  if (threadIdx.x < 2 * cnt) {
    const int latter = threadIdx.x / (int)cnt;
    const int oi = threadIdx.x % (int)cnt;
    T.e[latter][oi] = make_other(L, K, o0 + oi, latter);
  }
  return true;
}

// Exact result of one trial (parameter q of the windowed current grid).
struct TrialRes {
  int64_t in_tail, in_head;  // flattened previous-level index (window applied)
  int s_tail, s_head;        // rounded shifts
  bool ok;                   // both indices inside the input window
};

__device__ __forceinline__ TrialRes resolve_trial(const LokiFFALevel& L, const LevelK& K,
                                                  const OtherRes& ot, const OtherRes& oh,
                                                  int64_t off) {
  const int n = L.nparams;
  const int64_t last = L.out_start + off;
  const double f = L.param_arr[n - 1][last];
  float f_hi, f_lo;
  if (L.last_split) {
    const float2 fs = reinterpret_cast<const float2*>(L.last_split)[last];
    f_hi = fs.x;
    f_lo = fs.y;
  } else {
    split2(f, &f_hi, &f_lo);
  }
  TrialRes r;
  const int64_t it = trial_index(ot, f, f_hi, f_lo, L, K) - L.in_start;
  const int64_t ih = trial_index(oh, f, f_hi, f_lo, L, K) - L.in_start;
  r.ok = it >= 0 && it < L.in_width && ih >= 0 && ih < L.in_width;
  r.in_tail = ot.prefix * L.in_width + it;
  r.in_head = oh.prefix * L.in_width + ih;
  r.s_tail = trial_shift(ot, f, f_hi, f_lo, L.nbins);
  r.s_head = trial_shift(oh, f, f_hi, f_lo, L.nbins);
  return r;
}

}  // namespace loki
