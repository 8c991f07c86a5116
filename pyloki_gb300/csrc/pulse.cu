// Synthetic pulsar series on the device: PulseSignalConfig.generate
// (simulation/pulse.py:310-406) for a batch of injections.
//
// Per sample (all float64, IEEE operations in the reference's order):
//   proper time   modulation model (simulation/modulate.py:36-50 derivative,
//                 77-82 series, 136-140 circular, 208-213 circular_t0,
//                 226-236 keplerian with kepler.py:63-101,104-140)
//   template      CDF-table difference over [t, t + dt) of the pulse phase
//                 (generate_pulse_template, pulse.py:38-68)
//   noise         standard normal from the counter-based stream of rng.cuh
//                 (or a caller-supplied array)
//   fold bin      get_phase_idx_int at 1 / period (utils/psr_utils.py:12-56)
// Three passes: the calibration folds (noise, samples per bin, template), the
// calibration on the folds in one block per injection (pulse.py:380-400 and
// calibrate_scale_on_folds 71-118, float32 where the reference is float32),
// and the emitted series, which regenerates noise and template rather than
// storing them.
#include <algorithm>
#include <cmath>

#include "loki_common.cuh"
#include "rng.cuh"

namespace loki {

constexpr uint32_t kPulseNoiseDomain = 0x50C5u;
constexpr int kPulseThreads = 256;
constexpr int kCalibThreads = 256;

// Python's float %: remainder with the sign of the divisor (numpy npy_divmod).
__device__ __forceinline__ double pymod(double a, double b) {
  double m = fmod(a, b);
  if (m != 0.0) {
    if ((b < 0.0) != (m < 0.0)) m = __dadd_rn(m, b);
  } else {
    m = copysign(0.0, b);
  }
  return m;
}

// a mod b for b > 0 as Python's float %. For a >= 0 the remainder
// a - k b (k = floor(a / b)) is exactly representable (the property that
// makes fmod exact), so one fused multiply-add returns it exactly once k is
// right; k from the rounded quotient is off by at most one, which the sign
// and range of the remainder reveal. Negative a (and NaN) take the
// fmod-and-adjust route of pymod, whose final addition rounds as numpy's does.
__device__ __forceinline__ double floor_mod_pos(double a, double b, double inv_b) {
  if (!(a >= 0.0)) return pymod(a, b);
  double k = floor(__dmul_rn(a, inv_b));
  double r = __fma_rn(-k, b, a);
  if (r < 0.0) {
    k -= 1.0;
    r = __fma_rn(-k, b, a);
  } else if (r >= b) {
    k += 1.0;
    r = __fma_rn(-k, b, a);
  }
  return r;
}

__device__ __forceinline__ int64_t floor_mod(int64_t a, int64_t n) {
  const int64_t m = a % n;
  return m < 0 ? m + n : m;
}

__device__ double proper_time_at(const LokiPulseSpec& s, int64_t i, const double* table,
                                 int64_t row) {
  const LokiModulation& m = s.mod;
  const double t = __dmul_rn((double)i, s.dt);
  switch (m.kind) {
    case LOKI_MOD_DERIVATIVE: {
      // shift + d (vel + d (acc / 2 + d (jerk / 6 + d snap / 24)))
      const double d = __dsub_rn(t, m.t_ref);
      double in = __dmul_rn(__dmul_rn(d, m.c[4]), 1.0 / 24.0);
      in = __dadd_rn(__dmul_rn(m.c[3], 1.0 / 6.0), in);
      in = __dadd_rn(__dmul_rn(m.c[2], 0.5), __dmul_rn(d, in));
      in = __dadd_rn(m.c[1], __dmul_rn(d, in));
      const double delay = __dadd_rn(m.c[0], __dmul_rn(d, in));
      return __dsub_rn(t, __ddiv_rn(delay, LOKI_C_VAL));
    }
    case LOKI_MOD_SERIES: {
      // sum_k c[k] d^k, summed in order k = 0, 1, ...
      const double d = __dsub_rn(t, m.t_ref);
      double delay = 0.0;
      for (int k = 0; k < m.ncoeff; ++k) delay = __dadd_rn(delay, __dmul_rn(m.c[k], pow_rn(d, k)));
      return __dsub_rn(t, __ddiv_rn(delay, LOKI_C_VAL));
    }
    case LOKI_MOD_CIRCULAR: {
      const double arg = __dadd_rn(__dmul_rn(m.c[1], __dsub_rn(t, m.t_ref)), m.c[2]);
      return __dsub_rn(t, __dmul_rn(m.c[0], sin(arg)));
    }
    case LOKI_MOD_CIRCULAR_T0: {
      const double arg = __dadd_rn(__dmul_rn(m.c[1], __dsub_rn(t, m.t_ref)), m.c[2]);
      return __dsub_rn(t, __ddiv_rn(__dmul_rn(m.c[0], sin(arg)), LOKI_C_VAL));
    }
    case LOKI_MOD_KEPLERIAN: {
      // mean anomaly, 8 Newton steps on Kepler's equation, true anomaly, z
      const double p_orb = m.c[0], ecc = m.c[1];
      const double tt = __dsub_rn(t, m.t_ref);
      const double tn = __ddiv_rn(floor_mod_pos(tt, p_orb, m.c[7]), p_orb);
      const double ma = __dadd_rn(__dmul_rn(2.0 * M_PI, tn), m.c[2]);
      double e = ma;
      for (int it = 0; it < 8; ++it) {
        const double num = __dsub_rn(__dadd_rn(ma, __dmul_rn(ecc, sin(e))), e);
        const double den = __dsub_rn(1.0, __dmul_rn(ecc, cos(e)));
        e = __dadd_rn(e, __ddiv_rn(num, den));
      }
      const double nu = __dmul_rn(2.0, atan(__dmul_rn(m.c[6], tan(__ddiv_rn(e, 2.0)))));
      const double r = __ddiv_rn(m.c[3], __dadd_rn(1.0, __dmul_rn(ecc, cos(nu))));
      const double z = __dmul_rn(__dmul_rn(r, sin(__dadd_rn(nu, m.c[4]))), m.c[5]);
      return __dsub_rn(t, __ddiv_rn(z, LOKI_C_VAL));
    }
    default:  // LOKI_MOD_TABLE
      return table[row + i];
  }
}

// Linear interpolation of the CDF table at phase p in [0, 1).
__device__ __forceinline__ double cdf_at(const float* lut, int ngrid, double p) {
  const double x = __dmul_rn(p, (double)ngrid);
  int i = (int)x;
  i = min(max(i, 0), ngrid - 1);  // p rounds to 1 only for proper times just below 0
  const double f = __dsub_rn(x, (double)i);
  return __dadd_rn(__dmul_rn(__dsub_rn(1.0, f), (double)lut[i]),
                   __dmul_rn(f, (double)lut[i + 1]));
}

__device__ __forceinline__ float template_at(const LokiPulseSpec& s, const float* lut,
                                             double inv_period, double pt) {
  const double p0 = __dmul_rn(floor_mod_pos(pt, s.period, inv_period), inv_period);
  const double p1 = __dmul_rn(floor_mod_pos(__dadd_rn(pt, s.dt), s.period, inv_period),
                              inv_period);
  if (!(p1 > p0)) return 0.0f;
  return __double2float_rn(__dsub_rn(cdf_at(lut, s.ngrid, p1), cdf_at(lut, s.ngrid, p0)));
}

// Fields every pass reads; the fold and calibration also need nbins.
__device__ __forceinline__ bool gen_ok(const LokiPulseSpec& s) {
  return s.ngrid >= 1 && s.lut_off >= 0 && s.period > 0.0 && s.dt > 0.0 &&
         s.mod.kind >= LOKI_MOD_DERIVATIVE && s.mod.kind <= LOKI_MOD_TABLE &&
         s.mod.ncoeff >= 0 && s.mod.ncoeff <= LOKI_MOD_MAX_COEFFS;
}

__device__ __forceinline__ bool spec_ok(const LokiPulseSpec& s, int stride) {
  return gen_ok(s) && s.nbins >= 4 && s.nbins <= stride;
}

__device__ __forceinline__ void load_spec(const LokiPulseSpec* specs, LokiPulseSpec* sh) {
  if (threadIdx.x == 0) *sh = specs[blockIdx.y];
  __syncthreads();
}

__global__ void __launch_bounds__(kPulseThreads)
pulse_template_kernel(const LokiPulseSpec* __restrict__ specs, int64_t nsamps,
                      int64_t per_block, const float* __restrict__ luts,
                      const double* __restrict__ table, float* __restrict__ tmpl,
                      double* __restrict__ pt_out) {
  __shared__ LokiPulseSpec s;
  load_spec(specs, &s);
  const int64_t row = (int64_t)blockIdx.y * nsamps;
  const bool ok = gen_ok(s);
  const double inv_period = __ddiv_rn(1.0, s.period);
  const float* lut = luts + s.lut_off;
  const int64_t end = min(nsamps, (int64_t)(blockIdx.x + 1) * per_block);
  for (int64_t i = blockIdx.x * per_block + threadIdx.x; i < end; i += blockDim.x) {
    if (!ok) {
      tmpl[row + i] = nanf("");
      if (pt_out) pt_out[row + i] = nan("");
      continue;
    }
    const double pt = proper_time_at(s, i, table, row);
    tmpl[row + i] = template_at(s, lut, inv_period, pt);
    if (pt_out) pt_out[row + i] = pt;
  }
}

// The folds accumulate in 64-bit fixed point (2^-32 units; counts as plain
// integers), so a fold is exact and independent of the order in which
// samples land: the same seed gives the same series on every run. Partial
// folds live in shared memory when 20 bytes per bin fit, else the atomics go
// to the output directly. A finishing pass turns the integers into float64 in
// place.
constexpr double kFix = 4294967296.0;  // 2^32
constexpr int kFoldSmemBins = 8192;

__device__ __forceinline__ unsigned long long to_fix(float v) {
  return (unsigned long long)__double2ll_rn(__dmul_rn((double)v, kFix));
}

__global__ void __launch_bounds__(kPulseThreads)
pulse_fold_kernel(const LokiPulseSpec* __restrict__ specs, int64_t nsamps, int64_t per_block,
                  const float* __restrict__ luts, const double* __restrict__ table,
                  const float* __restrict__ noise, unsigned long long* __restrict__ folds,
                  int stride, int use_smem, float* __restrict__ z_out,
                  float* __restrict__ t_out) {
  extern __shared__ unsigned long long part[];  // noise (nb), template (nb), counts (nb x 32 bit)
  __shared__ LokiPulseSpec s;
  load_spec(specs, &s);
  if (!spec_ok(s, stride)) return;
  const int nb = s.nbins;
  unsigned long long* f = folds + (size_t)blockIdx.y * 3 * stride;
  unsigned long long* pz = use_smem ? part : f;
  unsigned long long* pt_sum = use_smem ? part + nb : f + 2 * stride;
  unsigned int* pc = reinterpret_cast<unsigned int*>(part + 2 * nb);
  if (use_smem) {
    for (int b = threadIdx.x; b < 2 * nb; b += blockDim.x) part[b] = 0ull;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) pc[b] = 0u;
  }
  __syncthreads();
  const int64_t row = (int64_t)blockIdx.y * nsamps;
  const double inv_period = __ddiv_rn(1.0, s.period);
  const float* lut = luts + s.lut_off;
  const int64_t end = min(nsamps, (int64_t)(blockIdx.x + 1) * per_block);
  for (int64_t i = blockIdx.x * per_block + threadIdx.x; i < end; i += blockDim.x) {
    const double pt = proper_time_at(s, i, table, row);
    const float tv = template_at(s, lut, inv_period, pt);
    const float z = noise ? noise[row + i] : normal_at(s.seed, i, 0, kPulseNoiseDomain);
    const int bin = round_shift(phase_idx(pt, inv_period, nb, 0.0), nb);
    if (z_out) {
      z_out[row + i] = z;
      t_out[row + i] = tv;
    }
    atomicAdd(&pz[bin], to_fix(z));
    atomicAdd(&pt_sum[bin], to_fix(tv));
    if (use_smem) atomicAdd(&pc[bin], 1u);
    else atomicAdd(&f[stride + bin], 1ull);
  }
  if (!use_smem) return;
  __syncthreads();
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    if (pc[b] != 0u) {
      atomicAdd(&f[b], part[b]);
      atomicAdd(&f[stride + b], (unsigned long long)pc[b]);
      atomicAdd(&f[2 * stride + b], part[nb + b]);
    }
  }
}

// In place: rows 0 and 2 from 2^-32 fixed point, row 1 from an integer count.
__global__ void fold_finish_kernel(unsigned long long* folds, int64_t ninj, int stride) {
  const int64_t n = ninj * 3 * stride;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)((i / stride) % 3);
    const unsigned long long u = folds[i];
    const double v = r == 1 ? (double)u : __dmul_rn((double)(long long)u, 1.0 / kFix);
    reinterpret_cast<double*>(folds)[i] = v;
  }
}

__global__ void zero_folds_kernel(unsigned long long* folds, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    folds[i] = 0ull;
}

__device__ __forceinline__ float block_max(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xFFFFFFFFu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  v = red[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = fmaxf(v, red[w]);
  return v;
}

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  v = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w];
  return v;
}

// Max over widths 1 .. n/2 - 1 of the boxcar S/N of x (boxcar_snr_1d,
// detection/scoring.py:43-140, stdnoise 1): float32 circular prefix sums
// (thread 0, sequential as the reference), float32 window differences,
// float64 height and offset, float32 S/N per width.
__device__ float boxcar_max_all(const float* x, int n, float* P, float* redf) {
  const int wmax = n / 2 - 1;
  if (threadIdx.x == 0) {
    P[0] = x[0];
    for (int i = 1; i < n; ++i) P[i] = __fadd_rn(P[i - 1], x[i]);
    const float last = P[n - 1];
    for (int j = 0; j < wmax; ++j) P[n + j] = __fadd_rn(P[j], last);
  }
  __syncthreads();
  const double total = (double)P[n - 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  float best = -INFINITY;
  for (int w = 1 + warp; w <= wmax; w += nw) {
    float dm = -3.4028234663852886e38f;
    for (int j = lane; j < n; j += 32) dm = fmaxf(dm, __fsub_rn(P[j + w], P[j]));
    for (int o = 16; o > 0; o >>= 1) dm = fmaxf(dm, __shfl_xor_sync(0xFFFFFFFFu, dm, o));
    const double size_w = (double)(float)(n - w);
    const double h = __dsqrt_rn(__ddiv_rn(size_w, (double)((int64_t)n * w)));
    const double b = __ddiv_rn(__dmul_rn((double)w, h), size_w);
    const double snr = __dsub_rn(__dmul_rn(__dadd_rn(h, b), (double)dm), __dmul_rn(b, total));
    best = fmaxf(best, __double2float_rn(snr));
  }
  const float r = block_max(best, redf);
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kCalibThreads)
pulse_calibrate_kernel(const LokiPulseSpec* __restrict__ specs, const double* __restrict__ folds,
                       int stride, int max_iter, double tol, double* __restrict__ out) {
  extern __shared__ float sm[];  // nn (n), tn (n), prefix (n + n / 2)
  __shared__ LokiPulseSpec s;
  __shared__ double redd[kCalibThreads / 32];
  __shared__ float redf[kCalibThreads / 32];
  load_spec(specs, &s);
  double* o = out + (size_t)blockIdx.y * 4;
  if (!spec_ok(s, stride)) {
    if (threadIdx.x < 4) o[threadIdx.x] = nan("");
    return;
  }
  const int n = s.nbins;
  // the folds as the reference holds them: float32
  const double* fd = folds + (size_t)blockIdx.y * 3 * stride;
  auto vals = [&](int b) { return __double2float_rn(fd[b]); };
  auto var = [&](int b) { return __double2float_rn(fd[stride + b]); };
  auto tsum = [&](int b) { return __double2float_rn(fd[2 * stride + b]); };
  float* nn = sm;
  float* tn = sm + n;
  float* P = sm + 2 * n;
  // on-pulse window: width_bins bins centred on round(phi0 * nbins)
  const int64_t center = floor_mod((int64_t)rint(__dmul_rn(s.phi0, (double)n)), n);
  const int64_t width = max((int64_t)1, (int64_t)rint(__dmul_rn(s.ducy, (double)n)));
  const int64_t first = center - width / 2;
  auto off_pulse = [&](int b) {
    return width < n ? floor_mod((int64_t)b - first, n) >= width : false;
  };
  double sum = 0.0, cnt = 0.0;
  for (int b = threadIdx.x; b < n; b += blockDim.x)
    if (off_pulse(b)) { sum += (double)vals(b); cnt += 1.0; }
  sum = block_sum(sum, redd);
  cnt = block_sum(cnt, redd);
  const double mean = sum / cnt;
  double sq = 0.0;
  for (int b = threadIdx.x; b < n; b += blockDim.x)
    if (off_pulse(b)) {
      const double d = (double)vals(b) - mean;
      sq += d * d;
    }
  sq = block_sum(sq, redd);
  const float sd = __double2float_rn(sqrt(sq / cnt));
  const float ns = __fdiv_rn(1.0f, sd);
  const float ns2 = __fmul_rn(ns, ns);
  for (int b = threadIdx.x; b < n; b += blockDim.x) {
    const float root = __fsqrt_rn(__fmul_rn(var(b), ns2));
    nn[b] = __fdiv_rn(__fmul_rn(vals(b), ns), root);
    tn[b] = __fdiv_rn(tsum(b), root);
  }
  __syncthreads();
  const float snr_t = boxcar_max_all(tn, n, P, redf);
  // first guess (snr / snr_template) * noise_scale in float32, then the
  // damped Newton steps in float64 on float32 combined profiles
  double cur = (double)__fmul_rn(__fdiv_rn((float)s.snr, snr_t), ns);
  double meas = nan("");
  for (int it = 0; it < max_iter; ++it) {
    float* comb = P + n + n / 2;  // n floats past the prefix
    for (int b = threadIdx.x; b < n; b += blockDim.x)
      comb[b] = __double2float_rn(__dadd_rn((double)nn[b], __dmul_rn(cur, (double)tn[b])));
    __syncthreads();
    meas = (double)boxcar_max_all(comb, n, P, redf);
    const double diff = __dsub_rn(meas, s.snr);
    if (__dmul_rn(diff, diff) < __dmul_rn(tol, tol)) break;
    cur = __dsub_rn(cur, __ddiv_rn(__dmul_rn(0.8, diff), (double)snr_t));
  }
  if (threadIdx.x == 0) {
    o[0] = (double)ns;
    o[1] = cur;
    o[2] = (double)snr_t;
    o[3] = meas;
  }
}

__global__ void __launch_bounds__(kPulseThreads)
pulse_emit_kernel(const LokiPulseSpec* __restrict__ specs, int64_t nsamps, int64_t per_block,
                  const float* __restrict__ luts, const double* __restrict__ table,
                  const float* __restrict__ noise, const double* __restrict__ scales,
                  float* __restrict__ ts_e, float* __restrict__ ts_v) {
  __shared__ LokiPulseSpec s;
  load_spec(specs, &s);
  const int64_t row = (int64_t)blockIdx.y * nsamps;
  const float ns = (float)scales[blockIdx.y * 4 + 0];
  const float sc = __double2float_rn(scales[blockIdx.y * 4 + 1]);
  const float nv = __fmul_rn(ns, ns);
  const bool ok = gen_ok(s);
  const double inv_period = __ddiv_rn(1.0, s.period);
  const float* lut = luts + s.lut_off;
  const int64_t end = min(nsamps, (int64_t)(blockIdx.x + 1) * per_block);
  for (int64_t i = blockIdx.x * per_block + threadIdx.x; i < end; i += blockDim.x) {
    if (!ok) {
      ts_e[row + i] = nanf("");
      ts_v[row + i] = nanf("");
      continue;
    }
    const double pt = proper_time_at(s, i, table, row);
    const float tv = template_at(s, lut, inv_period, pt);
    const float z = noise ? noise[row + i] : normal_at(s.seed, i, 0, kPulseNoiseDomain);
    ts_e[row + i] = __fadd_rn(__fmul_rn(ns, z), __fmul_rn(sc, tv));
    ts_v[row + i] = nv;
  }
}

// In place: (ts_e, ts_v) hold (unit noise, template) from the fold pass and
// become (noise_scale * noise + scale * template, noise_scale^2). Four
// samples per thread when rows are 16-byte aligned.
__global__ void __launch_bounds__(kPulseThreads)
pulse_apply_kernel(int64_t nsamps, const double* __restrict__ scales, float* __restrict__ ts_e,
                   float* __restrict__ ts_v, int vec4) {
  const int64_t row = (int64_t)blockIdx.y * nsamps;
  const float ns = (float)scales[blockIdx.y * 4 + 0];
  const float sc = __double2float_rn(scales[blockIdx.y * 4 + 1]);
  const float nv = __fmul_rn(ns, ns);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if (vec4) {
    float4* e4 = reinterpret_cast<float4*>(ts_e + row);
    float4* v4 = reinterpret_cast<float4*>(ts_v + row);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nsamps / 4;
         i += stride) {
      const float4 z = e4[i], t = v4[i];
      e4[i] = make_float4(__fadd_rn(__fmul_rn(ns, z.x), __fmul_rn(sc, t.x)),
                          __fadd_rn(__fmul_rn(ns, z.y), __fmul_rn(sc, t.y)),
                          __fadd_rn(__fmul_rn(ns, z.z), __fmul_rn(sc, t.z)),
                          __fadd_rn(__fmul_rn(ns, z.w), __fmul_rn(sc, t.w)));
      v4[i] = make_float4(nv, nv, nv, nv);
    }
    return;
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nsamps; i += stride) {
    ts_e[row + i] = __fadd_rn(__fmul_rn(ns, ts_e[row + i]), __fmul_rn(sc, ts_v[row + i]));
    ts_v[row + i] = nv;
  }
}

int64_t pulse_per_block(int64_t nsamps, int32_t ninj, int64_t min_per_block) {
  // about four waves of 152 SMs x 8 blocks over all injections
  const int64_t want_blocks = std::max<int64_t>(1, (152 * 8 * 4 + ninj - 1) / ninj);
  int64_t pb = (nsamps + want_blocks - 1) / want_blocks;
  pb = std::max<int64_t>(pb, min_per_block);
  return (pb + kPulseThreads - 1) / kPulseThreads * kPulseThreads;
}

int check_pulse_args(const LokiPulseSpec* specs, int32_t ninj, int64_t nsamps,
                     const float* luts) {
  if (ninj < 0 || nsamps < 0) return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (ninj > 65535) return set_error(LOKI_ERR_UNSUPPORTED, "more than 65535 injections");
  if (ninj > 0 && nsamps > 0 && (!specs || !luts))
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  return LOKI_OK;
}

}  // namespace loki

using namespace loki;

extern "C" int loki_pulse_template(const LokiPulseSpec* specs, int32_t ninj, int64_t nsamps,
                                   const float* luts, const double* pt_table, float* tmpl,
                                   double* proper_time, void* stream) {
  int rc = check_pulse_args(specs, ninj, nsamps, luts);
  if (rc) return rc;
  if (ninj == 0 || nsamps == 0) return LOKI_OK;
  if (!tmpl) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const int64_t pb = pulse_per_block(nsamps, ninj, kPulseThreads);
  const dim3 grid((unsigned)((nsamps + pb - 1) / pb), (unsigned)ninj);
  note_launch();
  pulse_template_kernel<<<grid, kPulseThreads, 0, (cudaStream_t)stream>>>(
      specs, nsamps, pb, luts, pt_table, tmpl, proper_time);
  return check_launch("pulse_template");
}

extern "C" int loki_pulse_fold(const LokiPulseSpec* specs, int32_t ninj, int64_t nsamps,
                               const float* luts, const double* pt_table, const float* noise,
                               double* folds, int32_t fold_stride, float* noise_out,
                               float* tmpl_out, void* stream) {
  int rc = check_pulse_args(specs, ninj, nsamps, luts);
  if (rc) return rc;
  if (fold_stride < 4 || fold_stride > LOKI_PULSE_MAX_NBINS)
    return set_error(LOKI_ERR_UNSUPPORTED, "fold_stride outside [4, %d]", LOKI_PULSE_MAX_NBINS);
  if (ninj == 0) return LOKI_OK;
  if (!folds || (!noise_out) != (!tmpl_out))
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  auto* acc = reinterpret_cast<unsigned long long*>(folds);
  const int64_t nf = (int64_t)ninj * 3 * fold_stride;
  const unsigned fgrid = (unsigned)std::min<int64_t>((nf + 255) / 256, 152 * 8);
  note_launch();
  zero_folds_kernel<<<fgrid, 256, 0, (cudaStream_t)stream>>>(acc, nf);
  rc = check_launch("pulse_fold (zero)");
  if (rc) return rc;
  if (nsamps > 0) {
    const int use_smem = fold_stride <= kFoldSmemBins;
    const int smem = use_smem ? 20 * fold_stride : 0;
    if (smem > 48 * 1024 &&
        set_smem_limit(pulse_fold_kernel, smem) != cudaSuccess)
      return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
    // enough samples per block that the flush (3 * nbins atomics) stays small
    const int64_t pb =
        pulse_per_block(nsamps, ninj, std::max<int64_t>(4096, 16LL * fold_stride));
    const dim3 grid((unsigned)((nsamps + pb - 1) / pb), (unsigned)ninj);
    note_launch();
    pulse_fold_kernel<<<grid, kPulseThreads, smem, (cudaStream_t)stream>>>(
        specs, nsamps, pb, luts, pt_table, noise, acc, fold_stride, use_smem, noise_out,
        tmpl_out);
    rc = check_launch("pulse_fold");
    if (rc) return rc;
  }
  note_launch();
  fold_finish_kernel<<<fgrid, 256, 0, (cudaStream_t)stream>>>(acc, ninj, fold_stride);
  return check_launch("pulse_fold (finish)");
}

extern "C" int loki_pulse_calibrate(const LokiPulseSpec* specs, int32_t ninj, const double* folds,
                                    int32_t fold_stride, int32_t max_iter, double tol,
                                    double* out, void* stream) {
  if (ninj < 0 || max_iter < 0 || !(tol >= 0.0))
    return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (ninj > 65535) return set_error(LOKI_ERR_UNSUPPORTED, "more than 65535 injections");
  if (fold_stride < 4 || fold_stride > LOKI_PULSE_MAX_NBINS)
    return set_error(LOKI_ERR_UNSUPPORTED, "fold_stride outside [4, %d]", LOKI_PULSE_MAX_NBINS);
  if (ninj == 0) return LOKI_OK;
  if (!specs || !folds || !out) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  // nn, tn, prefix (n + n / 2) and the combined profile (n)
  const int smem = (4 * fold_stride + fold_stride / 2) * (int)sizeof(float);
  if (smem > 48 * 1024 &&
      set_smem_limit(pulse_calibrate_kernel, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  note_launch();
  pulse_calibrate_kernel<<<dim3(1, (unsigned)ninj), kCalibThreads, smem,
                           (cudaStream_t)stream>>>(specs, folds, fold_stride, max_iter, tol, out);
  return check_launch("pulse_calibrate");
}

extern "C" int loki_pulse_emit(const LokiPulseSpec* specs, int32_t ninj, int64_t nsamps,
                               const float* luts, const double* pt_table, const float* noise,
                               const double* scales, float* ts_e, float* ts_v, void* stream) {
  int rc = check_pulse_args(specs, ninj, nsamps, luts);
  if (rc) return rc;
  if (ninj == 0 || nsamps == 0) return LOKI_OK;
  if (!scales || !ts_e || !ts_v) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const int64_t pb = pulse_per_block(nsamps, ninj, kPulseThreads);
  const dim3 grid((unsigned)((nsamps + pb - 1) / pb), (unsigned)ninj);
  note_launch();
  pulse_emit_kernel<<<grid, kPulseThreads, 0, (cudaStream_t)stream>>>(
      specs, nsamps, pb, luts, pt_table, noise, scales, ts_e, ts_v);
  return check_launch("pulse_emit");
}

extern "C" int loki_pulse_apply(const double* scales, int32_t ninj, int64_t nsamps, float* ts_e,
                                float* ts_v, void* stream) {
  if (ninj < 0 || nsamps < 0) return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (ninj > 65535) return set_error(LOKI_ERR_UNSUPPORTED, "more than 65535 injections");
  if (ninj == 0 || nsamps == 0) return LOKI_OK;
  if (!scales || !ts_e || !ts_v) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const int vec4 = nsamps % 4 == 0 && ((uintptr_t)ts_e % 16) == 0 && ((uintptr_t)ts_v % 16) == 0;
  const int64_t work = vec4 ? nsamps / 4 : nsamps;
  const int64_t per_row = std::max<int64_t>(1, (152 * 8 + ninj - 1) / ninj);
  const unsigned gx = (unsigned)std::min<int64_t>(
      per_row, (work + kPulseThreads - 1) / kPulseThreads);
  note_launch();
  pulse_apply_kernel<<<dim3(gx, (unsigned)ninj), kPulseThreads, 0, (cudaStream_t)stream>>>(
      nsamps, scales, ts_e, ts_v, vec4);
  return check_launch("pulse_apply");
}

// ---------------------------------------------------------------------------
// TimeSeries.fold_ephem (io/timeseries.py:45-83): the series folded at one
// frequency over the proper times of a modulation model, in nsub
// subintegrations (core/fold.py:57-105 brutefold): every (subint, bin) sum
// in sample order in float32, so the fold is the reference's bit for bit.
// Pass 1 bins every sample; pass 2 gives each (subint, bin) one thread that
// walks its subint in order.
// ---------------------------------------------------------------------------
namespace loki {

__global__ void ephem_bins_kernel(LokiPulseSpec s, const double* __restrict__ table,
                                  int64_t n, double freq, int nbins,
                                  uint32_t* __restrict__ bins) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double pt = proper_time_at(s, i, table, 0);
    bins[i] = (uint32_t)round_shift(phase_idx(pt, freq, nbins, 0.0), nbins);
  }
}

__global__ void __launch_bounds__(256)
ephem_fold_kernel(const float* __restrict__ ts_e, const float* __restrict__ ts_v,
                  const uint32_t* __restrict__ bins, int64_t seg_len, int nbins,
                  float* __restrict__ fold, float* __restrict__ norm) {
  const int64_t seg = blockIdx.y;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t i0 = seg * seg_len;
  float e = 0.0f, v = 0.0f;
  if (b < nbins) {
    for (int64_t i = i0; i < i0 + seg_len; ++i) {
      if (bins[i] == (uint32_t)b) {
        e = __fadd_rn(e, ts_e[i]);
        v = __fadd_rn(v, ts_v[i]);
      }
    }
    fold[(seg * 2) * nbins + b] = e;
    fold[(seg * 2 + 1) * nbins + b] = v;
    if (norm)  // zero where the variance is within 1e-5 of zero (np.isclose)
      norm[seg * nbins + b] = fabsf(v) <= 1e-5f ? 0.0f : __fdiv_rn(e, __fsqrt_rn(v));
  }
}

// Mean of each group of `factor` samples (np_utils.downsample_1d).
__global__ void downsample_kernel(const float* __restrict__ x, int64_t nout, int factor,
                                  float* __restrict__ out) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nout;
       k += (int64_t)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j < factor; ++j) acc += (double)x[k * factor + j];
    out[k] = __double2float_rn(acc / factor);
  }
}

}  // namespace loki

extern "C" int loki_fold_ephem(const float* ts_e, const float* ts_v, int64_t nsamps, double dt,
                               const LokiModulation* mod, const double* pt_table, double freq,
                               int32_t nbins, int32_t nsubints, uint32_t* bins, float* fold,
                               float* norm, void* stream) {
  if (nsamps < 1 || !(dt > 0.0) || !(freq > 0.0) || nbins < 1 || nsubints < 1 ||
      nsubints > nsamps)
    return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (nsubints > 65535) return set_error(LOKI_ERR_UNSUPPORTED, "more than 65535 subints");
  if (!ts_e || !ts_v || !mod || !bins || !fold)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (mod->kind < LOKI_MOD_DERIVATIVE || mod->kind > LOKI_MOD_TABLE ||
      (mod->kind == LOKI_MOD_TABLE && !pt_table) || mod->ncoeff < 0 ||
      mod->ncoeff > LOKI_MOD_MAX_COEFFS)
    return set_error(LOKI_ERR_INVALID, "bad modulation");
  LokiPulseSpec s{};
  s.dt = dt;
  s.mod = *mod;
  const int64_t seg_len = nsamps / nsubints;
  const int64_t nfold = seg_len * nsubints;  // trailing samples are not folded
  note_launch();
  ephem_bins_kernel<<<(unsigned)std::min<int64_t>((nfold + 255) / 256, 152 * 16), 256, 0,
                      (cudaStream_t)stream>>>(s, pt_table, nfold, freq, nbins, bins);
  int rc = check_launch("fold_ephem (bins)");
  if (rc) return rc;
  note_launch();
  ephem_fold_kernel<<<dim3((unsigned)((nbins + 255) / 256), (unsigned)nsubints), 256, 0,
                      (cudaStream_t)stream>>>(ts_e, ts_v, bins, seg_len, nbins, fold, norm);
  return check_launch("fold_ephem");
}

extern "C" int loki_downsample(const float* x, int64_t n, int32_t factor, float* out,
                               void* stream) {
  if (n < 0 || factor < 1) return set_error(LOKI_ERR_INVALID, "bad sizes");
  const int64_t nout = n / factor;
  if (nout == 0) return LOKI_OK;
  if (!x || !out) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  note_launch();
  downsample_kernel<<<(unsigned)std::min<int64_t>((nout + 255) / 256, 152 * 16), 256, 0,
                      (cudaStream_t)stream>>>(x, nout, factor, out);
  return check_launch("downsample");
}
