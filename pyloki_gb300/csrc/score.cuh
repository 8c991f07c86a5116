// Boxcar matched-filter scoring of one warp-tile of profiles held in shared
// memory (detection/scoring.py:42-165, 249-282).
//
// Layout: row r of the tile starts at tile + r * stride and holds the
// normalised profile in [0, nbins); the circular prefix sum is built in place
// and extended to nbins + wmax entries. stride is odd so that the 32 lanes,
// each walking its own row, hit 32 different banks.
//
// Each lane owns one row and runs the prefix sum sequentially in float32,
// exactly as circular_prefix_sum does, so the sums (and the S/N derived from
// them in float64) are bit-identical to the reference.
#pragma once

#include <float.h>

#include "loki_common.cuh"

namespace loki {

__host__ __device__ __forceinline__ int score_stride(int nbins, int wmax) {
  int s = nbins + (wmax > 0 ? wmax : 1);
  return (s & 1) ? s : s + 1;
}

// Circular prefix sum of length nbins + wmax, in place (scoring.py:42-71).
__device__ __forceinline__ float prefix_row(float* row, int nbins, int wmax) {
  float s = row[0];
  for (int i = 1; i < nbins; ++i) {
    s = __fadd_rn(s, row[i]);
    row[i] = s;
  }
  const float last = s;
  const int nsum = nbins + wmax;
  if (nsum > nbins) {
    const int n_wraps = nsum / nbins;
    const int extra = nsum % nbins;
    for (int w = 1; w < n_wraps; ++w) {
      const float add = __fmul_rn((float)w, last);
      for (int j = 0; j < nbins; ++j) row[w * nbins + j] = __fadd_rn(row[j], add);
    }
    if (extra > 0) {
      const float add = __fmul_rn((float)n_wraps, last);
      for (int j = 0; j < extra; ++j) row[n_wraps * nbins + j] = __fadd_rn(row[j], add);
    }
  }
  return last;  // prefix_sum[nbins - 1] == total
}

// S/N for one width given the prefix row (scoring.py:131-138).
__device__ __forceinline__ double snr_width(const float* row, int nbins, int w,
                                            double hb, double b, float total) {
  float dmax = -FLT_MAX;
  for (int i = 0; i < nbins; ++i) {
    const float d = __fsub_rn(row[i + w], row[i]);
    if (d > dmax) dmax = d;
  }
  return __dsub_rn(__dmul_rn(hb, (double)dmax), __dmul_rn(b, (double)total));
}

// ---- fast path: nbins == 64, widths 1, 2, 4, ..., 2^(nw-1) -----------------
//
// The reference's S/N of one width is RN32(RN64(RN64(hb*d) - RN64(b*T))) with
// d = max prefix difference and T = total (both float32). It is estimated in
// two-float FP32 (hb, b split into hi/lo floats, exact products by FMA, exact
// two-sum); when the estimate is farther than 2^-40 * max(|hb d|, |b T|) from
// an f32 rounding midpoint the rounding of the FP64 chain is certain,
// otherwise the FP64 chain is evaluated.
struct ScoreK {
  float hb_hi[LOKI_MAX_WIDTHS], hb_lo[LOKI_MAX_WIDTHS];
  float b_hi[LOKI_MAX_WIDTHS], b_lo[LOKI_MAX_WIDTHS];
  int pow2_64;  // nbins == 64 and widths == 1, 2, 4, ... (<= 32)
  int inv_one;  // inv_stdnoise == 1
};

inline ScoreK make_score_k(const LokiScoreSpec& sp, int nbins) {
  ScoreK k;
  bool pow2 = nbins == 64 && sp.nwidths <= 6;
  for (int i = 0; i < sp.nwidths; ++i) {
    k.hb_hi[i] = (float)sp.hb[i];
    k.hb_lo[i] = (float)(sp.hb[i] - (double)k.hb_hi[i]);
    k.b_hi[i] = (float)sp.b[i];
    k.b_lo[i] = (float)(sp.b[i] - (double)k.b_hi[i]);
    if (sp.widths[i] != (1 << i)) pow2 = false;
  }
  k.pow2_64 = pow2 ? 1 : 0;
  k.inv_one = sp.inv_stdnoise == 1.0 ? 1 : 0;
  return k;
}

// Exact FP64 chain; out of line so the compiler cannot evaluate it
// speculatively on the (common) fast path.
static __device__ __noinline__ float snr_exact(float d, float T, double hb, double b) {
  return __double2float_rn(__dsub_rn(__dmul_rn(hb, (double)d), __dmul_rn(b, (double)T)));
}

__device__ __forceinline__ float snr_fast(float d, float T, float hbh, float hbl, float bh,
                                          float bl, double hb, double b) {
  const float p1 = hbh * d;
  float e1 = fmaf(hbh, d, -p1);
  e1 = fmaf(hbl, d, e1);
  const float p2 = bh * T;
  float e2 = fmaf(bh, T, -p2);
  e2 = fmaf(bl, T, e2);
  const float s = p1 - p2;
  const float bb = s - p1;
  const float es = (p1 - (s - bb)) + (-p2 - bb);
  const float lo = (e1 - e2) + es;
  const float r = s + lo;
  const float res = (s - r) + lo;
  const unsigned bits = __float_as_uint(fabsf(r));
  const unsigned expo = bits >> 23;
  if (expo > 30 && expo < 255 && (bits & 0x7FFFFFu) != 0u) {
    const float half_ulp = __uint_as_float((expo - 24u) << 23);
    const float margin = fmaxf(fabsf(p1), fabsf(p2)) * 9.094947e-13f;  // 2^-40
    if (fabsf(res) < half_ulp - margin) return r;
  }
  return snr_exact(d, T, hb, b);
}

// Two IEEE round-to-nearest subtractions in one instruction (sm_100+ f32x2).
__device__ __forceinline__ void sub2(float a0, float a1, float b0, float b1, float& d0,
                                     float& d1) {
  unsigned long long a, b, d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(a) : "f"(a0), "f"(a1));
  asm("mov.b64 %0, {%1, %2};" : "=l"(b) : "f"(b0), "f"(b1));
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  asm("mov.b64 {%0, %1}, %2;" : "=f"(d0), "=f"(d1) : "l"(d));
}

// max of three; a NaN input is ignored like Python's max(acc, nan) == acc.
__device__ __forceinline__ float max3(float a, float b, float c) {
  float m;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(m) : "f"(a), "f"(b), "f"(c));
  return m;
}

__device__ __forceinline__ unsigned long long pack2(float a, float b) {
  unsigned long long x;
  asm("mov.b64 %0, {%1, %2};" : "=l"(x) : "f"(a), "f"(b));
  return x;
}

__device__ __forceinline__ void unpack2(unsigned long long x, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(x));
}

// The prefix is held as 48 register pairs P2[k] = (P[2k], P[2k+1]); for even
// widths both operands of the packed subtraction are register pairs already.
template <int H>  // width W = 2H
__device__ __forceinline__ float dmax64_even(const unsigned long long (&P2)[48]) {
  float m = -FLT_MAX;
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(P2[k + H]), "l"(P2[k]));
    float d0, d1;
    unpack2(d, d0, d1);
    m = max3(m, d0, d1);
  }
  return m;
}

__device__ __forceinline__ float dmax64_w1(const unsigned long long (&P2)[48]) {
  float m = -FLT_MAX;
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    float a0, a1, b0, b1;
    unpack2(P2[k], a0, a1);
    unpack2(P2[k + 1], b0, b1);
    m = max3(m, __fsub_rn(a1, a0), __fsub_rn(b0, a1));
  }
  return m;
}

// Sequential prefix in registers, then the width scans with compile-time
// indices (no shared-memory traffic after the row is read once).
__device__ __forceinline__ void score_row64_pow2(const float* row, const LokiScoreSpec& sp,
                                                 const ScoreK& K, float* out) {
  unsigned long long P2[48];
  float s = row[0];
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    const float s0 = k == 0 ? s : __fadd_rn(s, row[2 * k]);
    s = __fadd_rn(s0, row[2 * k + 1]);
    P2[k] = pack2(s0, s);
  }
  const float total = s;
  const unsigned long long tt = pack2(total, total);
#pragma unroll
  for (int k = 0; k < 16; ++k)  // circular extension: P[64 + j] = P[j] + total
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(P2[32 + k]) : "l"(P2[k]), "l"(tt));
  float best = -FLT_MAX;
  for (int iw = 0; iw < sp.nwidths; ++iw) {
    float dm;
    switch (iw) {
      case 0: dm = dmax64_w1(P2); break;
      case 1: dm = dmax64_even<1>(P2); break;
      case 2: dm = dmax64_even<2>(P2); break;
      case 3: dm = dmax64_even<4>(P2); break;
      case 4: dm = dmax64_even<8>(P2); break;
      default: dm = dmax64_even<16>(P2); break;
    }
    float s;
    if (K.inv_one) {
      s = snr_fast(dm, total, K.hb_hi[iw], K.hb_lo[iw], K.b_hi[iw], K.b_lo[iw], sp.hb[iw],
                   sp.b[iw]);
    } else {
      const double x = __dsub_rn(__dmul_rn(sp.hb[iw], (double)dm),
                                 __dmul_rn(sp.b[iw], (double)total));
      s = __double2float_rn(__dmul_rn(x, sp.inv_stdnoise));
    }
    if (sp.mode == 0) out[iw] = s;
    else if (s > best) best = s;
  }
  if (sp.mode != 0) out[0] = best;
}

// Score the row owned by this lane. mode 0 writes nwidths values at out,
// mode 1 writes the max over widths at out[0].
__device__ __forceinline__ void score_row(float* row, int nbins, const LokiScoreSpec& sp,
                                          float* out) {
  const float total = prefix_row(row, nbins, sp.wmax);
  // (generic path: any nbins and width list, prefix in shared memory)
  if (sp.mode == 0) {
    for (int iw = 0; iw < sp.nwidths; ++iw) {
      double s = snr_width(row, nbins, sp.widths[iw], sp.hb[iw], sp.b[iw], total);
      out[iw] = __double2float_rn(__dmul_rn(s, sp.inv_stdnoise));
    }
  } else {
    double best = -(double)FLT_MAX;
    for (int iw = 0; iw < sp.nwidths; ++iw) {
      double s = __dmul_rn(
          snr_width(row, nbins, sp.widths[iw], sp.hb[iw], sp.b[iw], total),
          sp.inv_stdnoise);
      if (s > best) best = s;
    }
    out[0] = __double2float_rn(best);
  }
}

}  // namespace loki
