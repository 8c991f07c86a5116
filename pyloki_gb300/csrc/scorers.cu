// Alternative profile scorers of detection/scoring.py. No search path of the
// reference calls them (its FFA and pruning score with the boxcar S/N); they
// are offered for users who score candidate profiles themselves.
//
//   kadane_kernel     kadane_circular_normalized_1d (scoring.py:675-755):
//                     float64 sequential, bit-identical to the reference
//   mf_kernel         the matched-filter bank (MatchedFilter, scoring.py:
//                     295-357, compute_snr_e_mat_2d 491-524): projections on
//                     every (template, circular shift), max per template
//   mf_double         _compute_snr_double (scoring.py:561-627): the best
//                     single or two-filter chi-square score among the top
//                     n_corr filters, mapped to a normal S/N
//   harmonic_kernel   harmonic_summing_score_func (scoring.py:630-642)
// The chi-square survival and normal ISF lookups interpolate the reference's
// tables (utils/maths.py:55-101), which the host builds with scipy.
#include <cfloat>

#include "loki_common.cuh"

namespace loki {

constexpr int kMfWarps = 4;

__global__ void __launch_bounds__(128)
kadane_kernel(const float* __restrict__ prof, int64_t n, int nb, const float* __restrict__ biases,
              int nbias, double* __restrict__ snr_out, int64_t* __restrict__ width_out,
              int64_t* __restrict__ start_out) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const float* x = prof + p * nb;
  double total = 0.0;
  for (int i = 0; i < nb; ++i) total = __dadd_rn(total, (double)x[i]);
  const double mean = __ddiv_rn(total, (double)nb);
  double best = -DBL_MAX;
  int best_w = 1, best_s = 0;
  for (int k = 0; k < nbias; ++k) {
    const double bias = (double)biases[k];
    double max_sum = -DBL_MAX, cur_max = 0.0, min_sum = DBL_MAX, cur_min = 0.0;
    int start_max = 0, end_max = 0, tmp_max = 0, start_min = 0, end_min = 0, tmp_min = 0;
    for (int i = 0; i < nb; ++i) {
      const double val = __dsub_rn(__dsub_rn((double)x[i], mean), bias);
      cur_max = __dadd_rn(cur_max, val);
      if (cur_max > max_sum) {
        max_sum = cur_max;
        start_max = tmp_max;
        end_max = i;
      }
      if (cur_max < 0.0) {
        cur_max = 0.0;
        tmp_max = i + 1;
      }
      cur_min = __dadd_rn(cur_min, val);
      if (cur_min < min_sum) {
        min_sum = cur_min;
        start_min = tmp_min;
        end_min = i;
      }
      if (cur_min > 0.0) {
        cur_min = 0.0;
        tmp_min = i + 1;
      }
    }
    double biased = max_sum;
    int s = start_max, w = end_max - start_max + 1;
    const int wrapped_w = nb - (end_min - start_min + 1);
    if (wrapped_w > 0) {  // the wrapped maximum excludes the minimum block
      const double wrapped = __dsub_rn(__dmul_rn(-(double)nb, bias), min_sum);
      if (wrapped > biased) {
        biased = wrapped;
        s = (end_min + 1) % nb;
        w = wrapped_w;
      }
    }
    const double unbiased = __dadd_rn(biased, __dmul_rn((double)w, bias));
    double snr = 0.0;
    if (w > 0 && w < nb)
      snr = __dmul_rn(unbiased, __dsqrt_rn(__ddiv_rn((double)nb, (double)((int64_t)w * (nb - w)))));
    if (snr > best) {
      best = snr;
      best_w = w;
      best_s = s;
    }
  }
  snr_out[p] = best;
  width_out[p] = best_w;
  start_out[p] = best_s;
}

// Projections of one profile on every filter row of e_mat (warp per profile,
// lane per filter, fused multiply-add in bin order) into the warp's scores.
__device__ __forceinline__ void mf_project(const float* __restrict__ x, const float* __restrict__ e,
                                           int nb, int nfilt, float* xs, float* scores) {
  const int lane = threadIdx.x & 31;
  for (int j = lane; j < nb; j += 32) xs[j] = x[j];
  __syncwarp();
  for (int f = lane; f < nfilt; f += 32) {
    const float* row = e + (size_t)f * nb;
    float acc = 0.0f;
    for (int j = 0; j < nb; ++j) acc = __fmaf_rn(row[j], xs[j], acc);
    scores[f] = acc;
  }
  __syncwarp();
}

__global__ void __launch_bounds__(kMfWarps * 32)
mf_kernel(const float* __restrict__ prof, int64_t n, int nb, const float* __restrict__ e_mat,
          int nfilt, int nsh, float stdnoise, float* __restrict__ snr, float* __restrict__ proj) {
  extern __shared__ float sm[];  // per warp: profile (nb) + scores (nfilt)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t p = (int64_t)blockIdx.x * kMfWarps + warp;
  if (p >= n) return;
  float* xs = sm + (size_t)warp * (nb + nfilt);
  float* scores = xs + nb;
  mf_project(prof + p * nb, e_mat, nb, nfilt, xs, scores);
  if (proj)
    for (int f = lane; f < nfilt; f += 32) proj[p * nfilt + f] = scores[f];
  const int ntemp = nfilt / nsh;
  for (int t = lane; t < ntemp; t += 32) {
    float m = scores[t * nsh];
    for (int k = 1; k < nsh; ++k) m = fmaxf(m, scores[t * nsh + k]);
    snr[p * ntemp + t] = __fdiv_rn(m, stdnoise);
  }
}

// chi_sq_minus_logsf_func (utils/maths.py:92-101) on a (df_max + 1, nchi)
// table, read flat as the reference's compiled code reads it: the entry
// after a row's last is the next row's first (a trailing zero row is
// appended so the last row has one).
__device__ __forceinline__ double chi_minus_logsf(const double* tab, int nchi, double x, int df,
                                                  double res, double xmax) {
  const double* row = tab + (size_t)df * nchi;
  if (x < xmax) {
    const double pos = __ddiv_rn(x, res);
    double fr = fmod(pos, 1.0);
    if (fr < 0.0) fr = __dadd_rn(fr, 1.0);
    const int64_t i = (int64_t)pos;
    return __dadd_rn(__dmul_rn(row[i], __dsub_rn(1.0, fr)), __dmul_rn(row[i + 1], fr));
  }
  return __ddiv_rn(__dmul_rn(row[nchi - 1], x), xmax);
}

// norm_isf_func (utils/maths.py:80-89) on the reference's nisf-entry table
// plus one repeated entry (tab[nisf]) for the read one past the end. A
// negative position (a score whose chi-square term is below its look-
// elsewhere penalty) wraps to the end of the table, as the reference's
// array indexing does.
__device__ __forceinline__ double norm_isf(const double* tab, int nisf, double m, double res,
                                           double mmax) {
  if (m < mmax) {
    const double pos = __ddiv_rn(m, res);
    double fr = fmod(pos, 1.0);
    if (fr < 0.0) fr = __dadd_rn(fr, 1.0);
    int64_t i = (int64_t)pos;
    int64_t j = i + 1;
    if (i < 0) i += nisf;
    if (j < 0) j += nisf;
    i = i < 0 ? 0 : (i > nisf ? nisf : i);  // stay in the nisf + 1 entries
    j = j < 0 ? 0 : (j > nisf ? nisf : j);
    return __dadd_rn(__dmul_rn(tab[i], __dsub_rn(1.0, fr)), __dmul_rn(tab[j], fr));
  }
  return __dmul_rn(tab[nisf - 1], sqrt(__ddiv_rn(m, mmax)));
}

struct ScoreTables {
  const double* chi;
  int nchi;
  double chi_res, chi_max;
  const double* isf;
  int nisf;
  double isf_res, isf_max;
};

__global__ void __launch_bounds__(kMfWarps * 32)
mf_double_kernel(const float* __restrict__ prof, int64_t n, int nb,
                 const float* __restrict__ e_mat, int nfilt, const float* __restrict__ inner,
                 int n_corr, ScoreTables T, double lee_single, double lee_double,
                 float* __restrict__ out) {
  extern __shared__ float sm[];  // per warp: profile, scores, n_corr indices
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t p = (int64_t)blockIdx.x * kMfWarps + warp;
  if (p >= n) return;
  float* xs = sm + (size_t)warp * (nb + nfilt + n_corr);
  float* scores = xs + nb;
  int* good = reinterpret_cast<int*>(scores + nfilt);
  mf_project(prof + p * nb, e_mat, nb, nfilt, xs, scores);
  if (lane != 0) return;
  // indices of the n_corr largest scores in ascending order of score (ties:
  // lower index first), as np.argsort(scores)[-n_corr:]; f only grows, so a
  // new filter ranks below an earlier one only on a strictly smaller score
  int cnt = 0;
  for (int f = 0; f < nfilt; ++f) {
    const float v = scores[f];
    int pos;
    if (cnt < n_corr) {
      pos = cnt++;
    } else {
      if (v < scores[good[0]]) continue;
      for (int k = 0; k + 1 < n_corr; ++k) good[k] = good[k + 1];
      pos = n_corr - 1;
    }
    while (pos > 0 && v < scores[good[pos - 1]]) {
      good[pos] = good[pos - 1];
      --pos;
    }
    good[pos] = f;
  }
  float smax = scores[0];
  for (int f = 1; f < nfilt; ++f) smax = fmaxf(smax, scores[f]);
  const double single = (double)smax * (double)smax;
  double dbl = single, s = 0.0;
  for (int i = 0; i + 1 < cnt; ++i)
    for (int j = i + 1; j < cnt; ++j) {
      const int a = good[i], b = good[j];
      const double g = (double)inner[(size_t)a * nfilt + b];
      if (fabs(g) < 0.99) {
        const double sa = (double)scores[a], sb = (double)scores[b];
        s = __ddiv_rn(__dsub_rn(__dadd_rn(__dmul_rn(sa, sa), __dmul_rn(sb, sb)),
                                __dmul_rn(__dmul_rn(__dmul_rn(2.0, g), sa), sb)),
                      __dsub_rn(1.0, __dmul_rn(g, g)));
      }
      dbl = fmax(s, dbl);  // an earlier s carries over, as in the reference
    }
  const double x1 = __dsub_rn(chi_minus_logsf(T.chi, T.nchi, single, 1, T.chi_res, T.chi_max),
                              lee_single);
  const double x2 = __dsub_rn(chi_minus_logsf(T.chi, T.nchi, dbl, 2, T.chi_res, T.chi_max),
                              lee_double);
  out[p] = __double2float_rn(norm_isf(T.isf, T.nisf, fmax(x1, x2), T.isf_res, T.isf_max));
}

__global__ void __launch_bounds__(128)
harmonic_kernel(const float* __restrict__ folds, int64_t n, int nb, int nh, ScoreTables T,
                double* __restrict__ out) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const float* e = folds + p * 2 * nb;
  const float* v = e + nb;
  const double scale = __dsqrt_rn((double)nb);
  double best = -INFINITY, raw = 0.0;
  for (int k = 1; k <= nh; ++k) {
    double re = 0.0, im = 0.0;
    for (int j = 0; j < nb; ++j) {
      const double x = (double)__fdiv_rn(e[j], __fsqrt_rn(v[j]));
      const int m = (int)(((int64_t)j * k) % nb);  // exact angle reduction
      double sn, cs;
      sincospi(__ddiv_rn(2.0 * m, (double)nb), &sn, &cs);
      re = __dadd_rn(re, __dmul_rn(x, cs));
      im = __dsub_rn(im, __dmul_rn(x, sn));
    }
    re = __ddiv_rn(re, scale);
    im = __ddiv_rn(im, scale);
    raw = __dadd_rn(raw, __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im)));
    best = fmax(best, chi_minus_logsf(T.chi, T.nchi, __dmul_rn(raw, 2.0), 2 * k, T.chi_res,
                                      T.chi_max));
  }
  out[p] = norm_isf(T.isf, T.nisf, best, T.isf_res, T.isf_max);
}

// _compute_snr_fft (scoring.py:527-558): the profile circularly padded to
// the next power of two N (np_utils.cpadpow2), the template zero-padded to N,
// their circular convolution c[k] = sum_m t[m] x[(k - m) mod N] (what the
// reference's irfft(rfft(x) rfft(t)) computes), max over k < nbins. Direct
// float64 sums; thread per (profile, template).
__global__ void __launch_bounds__(128)
mf_conv_kernel(const float* __restrict__ prof, int64_t n, int nb, int npad,
               const float* __restrict__ templates, int ntemp, float* __restrict__ out) {
  const int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q >= n * ntemp) return;
  const int64_t p = q / ntemp;
  const int t = (int)(q - p * ntemp);
  const float* x = prof + p * nb;
  const float* tm = templates + (size_t)t * nb;
  double best = -INFINITY;
  for (int k = 0; k < nb; ++k) {
    double c = 0.0;
    for (int m = 0; m < nb; ++m) {
      int j = k - m;
      j += j < 0 ? npad : 0;              // index into the padded profile
      c += (double)tm[m] * (double)x[j < nb ? j : j - nb];
    }
    best = fmax(best, c);
  }
  out[q] = __double2float_rn(best);
}

ScoreTables tables_of(const double* chi, int32_t nchi, double chi_res, double chi_max,
                      const double* isf, int32_t nisf, double isf_res, double isf_max) {
  return ScoreTables{chi, nchi, chi_res, chi_max, isf, nisf, isf_res, isf_max};
}

}  // namespace loki

using namespace loki;

extern "C" int loki_kadane_circular(const float* profiles, int64_t n, int32_t nbins,
                                    const float* biases, int32_t nbias, double* snr,
                                    int64_t* width, int64_t* start, void* stream) {
  if (n < 0 || nbins < 1 || nbias < 1) return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (n == 0) return LOKI_OK;
  if (!profiles || !biases || !snr || !width || !start)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  note_launch();
  kadane_kernel<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
      profiles, n, nbins, biases, nbias, snr, width, start);
  return check_launch("kadane_circular");
}

extern "C" int loki_matched_filter(const float* profiles, int64_t n, int32_t nbins,
                                   const float* e_mat, int32_t nfilt, int32_t shifts_per_template,
                                   float stdnoise, float* snr, float* projections, void* stream) {
  if (n < 0 || nbins < 1 || nfilt < 1 || shifts_per_template < 1 ||
      nfilt % shifts_per_template != 0 || !(stdnoise > 0.0f))
    return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (n == 0) return LOKI_OK;
  if (!profiles || !e_mat || !snr) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const int smem = kMfWarps * (nbins + nfilt) * (int)sizeof(float);
  if (smem > 200 * 1024) return set_error(LOKI_ERR_UNSUPPORTED, "nbins + filters too large");
  if (smem > 48 * 1024 &&
      set_smem_limit(mf_kernel, smem) !=
          cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  note_launch();
  mf_kernel<<<(unsigned)((n + kMfWarps - 1) / kMfWarps), kMfWarps * 32, smem,
              (cudaStream_t)stream>>>(profiles, n, nbins, e_mat, nfilt, shifts_per_template,
                                      stdnoise, snr, projections);
  return check_launch("matched_filter");
}

extern "C" int loki_matched_filter_double(const float* profiles, int64_t n, int32_t nbins,
                                          const float* e_mat, int32_t nfilt, const float* inner,
                                          int32_t n_corr, const double* chi_table, int32_t nchi,
                                          double chi_res, double chi_max,
                                          const double* isf_table, int32_t nisf, double isf_res,
                                          double isf_max, float* out, void* stream) {
  if (n < 0 || nbins < 1 || nfilt < 2 || n_corr < 2 || n_corr > nfilt || nchi < 2 || nisf < 2)
    return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (n == 0) return LOKI_OK;
  if (!profiles || !e_mat || !inner || !chi_table || !isf_table || !out)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const int smem = kMfWarps * (nbins + nfilt + n_corr) * (int)sizeof(float);
  if (smem > 200 * 1024) return set_error(LOKI_ERR_UNSUPPORTED, "nbins + filters too large");
  if (smem > 48 * 1024 &&
      set_smem_limit(mf_double_kernel, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  const double lee_double = log2(((double)nfilt * nfilt - 1.0) / 2.0);
  const double lee_single = log2((double)nfilt);
  note_launch();
  mf_double_kernel<<<(unsigned)((n + kMfWarps - 1) / kMfWarps), kMfWarps * 32, smem,
                     (cudaStream_t)stream>>>(
      profiles, n, nbins, e_mat, nfilt, inner, n_corr,
      tables_of(chi_table, nchi, chi_res, chi_max, isf_table, nisf, isf_res, isf_max),
      lee_single, lee_double, out);
  return check_launch("matched_filter_double");
}

extern "C" int loki_harmonic_sum(const float* folds, int64_t n, int32_t nbins,
                                 int32_t n_harmonics, const double* chi_table, int32_t chi_rows,
                                 int32_t nchi, double chi_res, double chi_max,
                                 const double* isf_table, int32_t nisf, double isf_res,
                                 double isf_max, double* out, void* stream) {
  if (n < 0 || nbins < 2 || n_harmonics < 1 || n_harmonics >= nbins || nchi < 2 || nisf < 2)
    return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (2 * n_harmonics >= chi_rows)
    return set_error(LOKI_ERR_UNSUPPORTED, "2 * n_harmonics above the chi-square table");
  if (n == 0) return LOKI_OK;
  if (!folds || !chi_table || !isf_table || !out)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  note_launch();
  harmonic_kernel<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
      folds, n, nbins, n_harmonics,
      tables_of(chi_table, nchi, chi_res, chi_max, isf_table, nisf, isf_res, isf_max), out);
  return check_launch("harmonic_sum");
}

extern "C" int loki_matched_filter_conv(const float* profiles, int64_t n, int32_t nbins,
                                        const float* templates, int32_t ntemp, float* out,
                                        void* stream) {
  if (n < 0 || nbins < 1 || ntemp < 1) return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (n == 0) return LOKI_OK;
  if (!profiles || !templates || !out) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  int npad = 1;
  while (npad < nbins) npad <<= 1;
  const int64_t work = n * ntemp;
  note_launch();
  mf_conv_kernel<<<(unsigned)((work + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
      profiles, n, nbins, npad, templates, ntemp, out);
  return check_launch("matched_filter_conv");
}
