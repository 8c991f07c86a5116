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

// Score the row owned by this lane. mode 0 writes nwidths values at out,
// mode 1 writes the max over widths at out[0].
__device__ __forceinline__ void score_row(float* row, int nbins, const LokiScoreSpec& sp,
                                          float* out) {
  const float total = prefix_row(row, nbins, sp.wmax);
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
