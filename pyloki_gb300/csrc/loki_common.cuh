// Shared device helpers for the loki_gb300 kernels (sm_103a).
//
// Exactness: every FP64/FP32 expression that feeds an integer result (phase
// bin, grid index, rounded shift) is written with explicit round-to-nearest
// intrinsics in the reference's operation order, and the library is built with
// --fmad=false, so no multiply-add is contracted. This reproduces pyloki's
// numpy semantics bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/loki_gb300.h"

#define LOKI_C_VAL 299792458.0
#define LOKI_FLOAT_EPSILON 1e-6
#define LOKI_MAX_PARAMS 5

namespace loki {

// Host-side error recording (defined in capi.cu).
int set_error(int code, const char* fmt, ...);
int check_launch(const char* what);
// Counts one kernel launch of this host thread (read by loki_launch_count).
void note_launch();
// Raises (never lowers) a kernel's dynamic shared-memory limit on the current
// device to at least `bytes`; thread-safe (defined in capi.cu).
cudaError_t raise_smem_limit(const void* func, int bytes);
template <typename F>
inline cudaError_t set_smem_limit(F* func, int bytes) {
  return raise_smem_limit(reinterpret_cast<const void*>(func), bytes);
}

// Division by a runtime-constant 32-bit divisor d >= 1 with a precomputed
// multiplier (Granlund & Montgomery 1994): q = (t + ((n - t) >> 1)) >> (l - 1),
// t = umulhi(m, n), l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1.
// Exact for every 32-bit n.
struct FastDiv32 {
  uint32_t d, m, s;  // s = l - 1 (unused when d == 1)

  __host__ __device__ static FastDiv32 make(uint32_t dv) {
    FastDiv32 f;
    f.d = dv;
    uint32_t l = 0;
    while (l < 32 && (1ull << l) < dv) ++l;
    f.m = (uint32_t)((((1ull << l) - dv) << 32) / dv + 1);
    f.s = l ? l - 1 : 0;
    return f;
  }
  __device__ __forceinline__ uint32_t div(uint32_t n) const {
    if (d == 1) return n;
    const uint32_t t = __umulhi(m, n);
    return (t + ((n - t) >> 1)) >> s;
  }
};

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Phase bin of a periodic signal as a float in [0, nbins)
// (utils/psr_utils.py:12-46 get_phase_idx).
__device__ __forceinline__ double phase_idx(double proper_time, double freq,
                                            int nbins, double delay) {
  double phase = __dmul_rn(__dsub_rn(proper_time, delay), freq);
  phase = __dsub_rn(phase, floor(phase));
  double iphase = __dmul_rn(phase, (double)nbins);
  if (iphase >= (double)nbins) iphase = 0.0;
  return iphase;
}

// Integer bin with float32 half-up rounding (utils/psr_utils.py:49-56 and the
// shift rounding of core/common.py:313-318).
__device__ __forceinline__ int round_shift(double phase, int nbins) {
  int ibin = (int)__fadd_rn(__double2float_rn(phase), 0.5f);
  return ibin == nbins ? 0 : ibin;
}

__device__ __forceinline__ int round_shift_f32(float phase, int nbins) {
  int ibin = (int)__fadd_rn(phase, 0.5f);
  return ibin == nbins ? 0 : ibin;
}

// dt**p rounded to nearest for p = 0..5. p <= 2 is exact with one rounding;
// larger p uses a double-double product so the result is correctly rounded
// (the reference evaluates numpy's pow, which is correctly rounded up to
// rare last-ulp cases that depend on the platform's libm).
__device__ __forceinline__ double pow_rn(double x, int p) {
  if (p == 0) return 1.0;
  if (p == 1) return x;
  if (p == 2) return __dmul_rn(x, x);
  double hi = __dmul_rn(x, x);
  double lo = __fma_rn(x, x, -hi);
  for (int k = 3; k <= p; ++k) {
    double nh = __dmul_rn(hi, x);
    double nl = __fma_rn(hi, x, -nh);
    nl = __fma_rn(lo, x, nl);
    hi = __dadd_rn(nh, nl);
    lo = __dsub_rn(nl, __dsub_rn(hi, nh));
  }
  return hi;
}

__device__ __forceinline__ double fact_d(int p) {
  const double f[8] = {1.0, 1.0, 2.0, 6.0, 24.0, 120.0, 720.0, 5040.0};
  return f[p];
}

// Nearest grid index by truncation (utils/psr_utils.py:466-514).
__device__ __forceinline__ int64_t nearest_index(double val, int64_t n_grid,
                                                 double vmin, double vmax) {
  if (n_grid <= 1) return 0;
  double raw = __ddiv_rn(__dmul_rn((double)n_grid, __dsub_rn(val, vmin)),
                         __dsub_rn(vmax, vmin));
  int64_t idx = (int64_t)__dadd_rn(raw, LOKI_FLOAT_EPSILON);
  if (idx < 0) idx = 0;
  else if (idx >= n_grid) idx = n_grid - 1;
  return idx;
}

// FFA resolve of one parameter set against the previous level's grid
// (core/fold.py:617-671 ffa_taylor_resolve, utils/transforms.py:140-171
// shift_taylor_params_d_f). pset is ordered [..., jerk, accel, freq].
// Writes the previous-level multi-index and returns the relative phase.
__device__ __forceinline__ double ffa_resolve(const double* pset, int n, int level,
                                              int latter, double tseg_brute,
                                              int nbins, const int64_t* counts_prev,
                                              const double (*limits)[2],
                                              int64_t* idx_out) {
  const double f = pset[n - 1];
  double dt, delay;
  double pnew[LOKI_MAX_PARAMS];
  const double two_pow = (double)(1LL << (level - 1));
  if (n == 1) {
    dt = __dmul_rn((double)latter * two_pow, tseg_brute);
    delay = 0.0;
    pnew[0] = f;
  } else {
    dt = __dmul_rn(__dmul_rn((double)latter - 0.5, two_pow), tseg_brute);
    // Taylor vector [p_0 .. p_{n-2}, 0, 0]; new[i] = sum_j tv[j] * t[i][j],
    // t[i][j] = dt^(i-j) / (i-j)! for j <= i, summed left to right.
    double tv[LOKI_MAX_PARAMS + 1];
    for (int j = 0; j <= n; ++j) tv[j] = (j < n - 1) ? pset[j] : 0.0;
    double out[LOKI_MAX_PARAMS + 1];
    for (int i = 0; i <= n; ++i) {
      double acc = 0.0;
      bool first = true;
      for (int j = 0; j <= i; ++j) {
        double tij = __ddiv_rn(pow_rn(dt, i - j), fact_d(i - j));
        double term = __dmul_rn(tv[j], tij);
        acc = first ? term : __dadd_rn(acc, term);
        first = false;
      }
      out[i] = acc;
    }
    for (int i = 0; i < n - 1; ++i) pnew[i] = out[i];
    pnew[n - 1] = __dmul_rn(f, __dsub_rn(1.0, __ddiv_rn(out[n - 1], LOKI_C_VAL)));
    delay = __ddiv_rn(out[n], LOKI_C_VAL);
  }
  for (int ip = 0; ip < n; ++ip)
    idx_out[ip] = nearest_index(pnew[ip], counts_prev[ip], limits[ip][0], limits[ip][1]);
  return phase_idx(dt, f, nbins, delay);
}

}  // namespace loki
