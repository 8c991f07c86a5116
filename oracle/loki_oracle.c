/*
 * CPU oracle for the FFA / scoring hot path: a plain-C restatement of pyloki's
 * numba loops, used ONLY as test infrastructure (parity checker in tests/,
 * __graft_entry__.smoke(), and the CPU baseline leg of bench.py). The product
 * path never links or calls this file.
 *
 * Every function follows the reference's loop nest and floating-point
 * operation order (numpy semantics; build with -ffp-contract=off so no
 * multiply-add is fused). OpenMP parallelises the same axes the reference's
 * numba prange does. Pinned against fixtures produced by the reference itself
 * (tests/golden/*.npz, see tests/golden/make_fixtures.py).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define C_VAL 299792458.0
#define FLOAT_EPSILON 1e-6
#define MAXP 5

static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* utils/psr_utils.py:12-46 get_phase_idx */
static double phase_idx(double proper_time, double freq, int nbins, double delay) {
  double phase = (proper_time - delay) * freq;
  phase -= floor(phase);
  double iphase = phase * (double)nbins;
  if (iphase >= (double)nbins) iphase = 0.0;
  return iphase;
}

/* utils/psr_utils.py:49-56 get_phase_idx_int; core/common.py:313-318 rounding */
static int round_shift(double phase, int nbins) {
  float s = (float)phase;
  int ibin = (int)(s + 0.5f);
  return ibin == nbins ? 0 : ibin;
}

/* dt**p correctly rounded (numpy pow on the reference side). */
static double pow_rn(double x, int p) {
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

static const double FACT[8] = {1.0, 1.0, 2.0, 6.0, 24.0, 120.0, 720.0, 5040.0};

/* utils/psr_utils.py:466-514 get_nearest_indices_analytical (one dimension) */
static int64_t nearest_index(double val, int64_t n_grid, double vmin, double vmax) {
  if (n_grid <= 1) return 0;
  double raw = (double)n_grid * (val - vmin) / (vmax - vmin);
  int64_t idx = (int64_t)(raw + FLOAT_EPSILON);
  if (idx < 0) idx = 0;
  else if (idx >= n_grid) idx = n_grid - 1;
  return idx;
}

/* core/fold.py:617-671 ffa_taylor_resolve with utils/transforms.py:140-171
 * shift_taylor_params_d_f (matrix product summed left to right). */
double oracle_ffa_resolve(const double* pset, int n, const int64_t* counts_prev,
                          const double* limits, int level, int latter, double tseg_brute,
                          int nbins, int64_t* idx_out) {
  const double f = pset[n - 1];
  const double two_pow = (double)(1LL << (level - 1));
  double dt, delay, pnew[MAXP];
  if (n == 1) {
    dt = ((double)latter * two_pow) * tseg_brute;
    delay = 0.0;
    pnew[0] = f;
  } else {
    double tv[MAXP + 1], out[MAXP + 1];
    dt = (((double)latter - 0.5) * two_pow) * tseg_brute;
    for (int j = 0; j <= n; ++j) tv[j] = (j < n - 1) ? pset[j] : 0.0;
    for (int i = 0; i <= n; ++i) {
      double acc = 0.0;
      for (int j = 0; j <= i; ++j) {
        double term = tv[j] * (pow_rn(dt, i - j) / FACT[i - j]);
        acc = (j == 0) ? term : acc + term;
      }
      out[i] = acc;
    }
    for (int i = 0; i < n - 1; ++i) pnew[i] = out[i];
    pnew[n - 1] = f * (1.0 - out[n - 1] / C_VAL);
    delay = out[n] / C_VAL;
  }
  for (int ip = 0; ip < n; ++ip)
    idx_out[ip] = nearest_index(pnew[ip], counts_prev[ip], limits[2 * ip], limits[2 * ip + 1]);
  return phase_idx(dt, f, nbins, delay);
}

/* core/fold.py:108-171 brutefold_start. fold is (nseg, nfreq, 2, nbins). */
void oracle_brutefold(const float* ts_e, const float* ts_v, int64_t nsamps,
                      const double* freqs, int64_t nfreq, int64_t seg_len, int nbins,
                      double tsamp, double t_ref, float* fold, int nthreads) {
  set_threads(nthreads);
  const int64_t nseg = (nsamps + seg_len - 1) / seg_len;
  int32_t* pmap = (int32_t*)malloc((size_t)nfreq * seg_len * sizeof(int32_t));
#pragma omp parallel for schedule(static)
  for (int64_t f = 0; f < nfreq; ++f)
    for (int64_t i = 0; i < seg_len; ++i) {
      const double pt = (double)i * tsamp - t_ref;
      pmap[f * seg_len + i] = round_shift(phase_idx(pt, freqs[f], nbins, 0.0), nbins);
    }
  memset(fold, 0, (size_t)nseg * nfreq * 2 * nbins * sizeof(float));
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t s = 0; s < nseg; ++s) {
    const int64_t start = s * seg_len;
    const int64_t len = (start + seg_len <= nsamps) ? seg_len : nsamps - start;
    for (int64_t f = 0; f < nfreq; ++f) {
      float* fe = fold + ((size_t)s * nfreq + f) * 2 * nbins;
      float* fv = fe + nbins;
      const int32_t* m = pmap + f * seg_len;
      for (int64_t i = 0; i < len; ++i) {
        fe[m[i]] += ts_e[start + i];
        fv[m[i]] += ts_v[start + i];
      }
    }
  }
  free(pmap);
}

typedef struct {
  int n, nbins, level;
  double tseg_brute;
  const int64_t* counts_cur;
  const int64_t* counts_prev;
  const double* limits;        /* (n, 2) */
  const double* const* params; /* current-level grid per dim */
} OracleLevel;

static void decode_q(const OracleLevel* L, int64_t q, double* pset) {
  int64_t rest = q;
  for (int d = L->n - 1; d >= 0; --d) {
    const int64_t c = L->counts_cur[d];
    pset[d] = L->params[d][rest % c];
    rest /= c;
  }
}

static int64_t flat_prev(const OracleLevel* L, const int64_t* idx) {
  int64_t flat = 0;
  for (int d = 0; d < L->n; ++d) flat = flat * L->counts_prev[d] + idx[d];
  return flat;
}

/* Per-level plan (the resolve calls of dynamic/dyn_pffa.py:462-475). */
void oracle_ffa_plan(int n, int nbins, int level, double tseg_brute, const int64_t* counts_cur,
                     const int64_t* counts_prev, const double* limits,
                     const double* const* params, int64_t* i_tail, double* ph_tail,
                     int64_t* i_head, double* ph_head, int nthreads) {
  set_threads(nthreads);
  OracleLevel L = {n, nbins, level, tseg_brute, counts_cur, counts_prev, limits, params};
  int64_t Q = 1;
  for (int d = 0; d < n; ++d) Q *= counts_cur[d];
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < Q; ++q) {
    double pset[MAXP];
    int64_t idx[MAXP];
    decode_q(&L, q, pset);
    ph_tail[q] = oracle_ffa_resolve(pset, n, counts_prev, limits, level, 0, tseg_brute, nbins, idx);
    i_tail[q] = flat_prev(&L, idx);
    ph_head[q] = oracle_ffa_resolve(pset, n, counts_prev, limits, level, 1, tseg_brute, nbins, idx);
    i_head[q] = flat_prev(&L, idx);
  }
}

/* dynamic/dyn_pffa.py:435-489 unify_fold with core/common.py:304-324 shift_add.
 * fold_in (nseg_in, P_prev, 2, nbins) -> fold_out (nseg_in/2, P_cur, 2, nbins). */
void oracle_ffa_level(const float* fold_in, int64_t nseg_in, int n, int nbins, int level,
                      double tseg_brute, const int64_t* counts_cur, const int64_t* counts_prev,
                      const double* limits, const double* const* params, float* fold_out,
                      int nthreads) {
  set_threads(nthreads);
  OracleLevel L = {n, nbins, level, tseg_brute, counts_cur, counts_prev, limits, params};
  int64_t Q = 1, Pp = 1;
  for (int d = 0; d < n; ++d) {
    Q *= counts_cur[d];
    Pp *= counts_prev[d];
  }
  const int64_t nseg_out = nseg_in / 2;
  const size_t row = (size_t)2 * nbins;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t q = 0; q < Q; ++q) {
    double pset[MAXP];
    int64_t idx[MAXP];
    decode_q(&L, q, pset);
    const double pht =
        oracle_ffa_resolve(pset, n, counts_prev, limits, level, 0, tseg_brute, nbins, idx);
    const int64_t it = flat_prev(&L, idx);
    const double phh =
        oracle_ffa_resolve(pset, n, counts_prev, limits, level, 1, tseg_brute, nbins, idx);
    const int64_t ih = flat_prev(&L, idx);
    const int st = round_shift(pht, nbins);
    const int sh = round_shift(phh, nbins);
    for (int64_t ip = 0; ip < nseg_out; ++ip) {
      const float* t = fold_in + ((size_t)(2 * ip) * Pp + it) * row;
      const float* h = fold_in + ((size_t)(2 * ip + 1) * Pp + ih) * row;
      float* o = fold_out + ((size_t)ip * Q + q) * row;
      for (int j = 0; j < nbins; ++j) {
        const int i1 = ((j - st) % nbins + nbins) % nbins;
        const int i2 = ((j - sh) % nbins + nbins) % nbins;
        o[j] = t[i1] + h[i2];
        o[nbins + j] = t[nbins + i1] + h[nbins + i2];
      }
    }
  }
}

/* detection/scoring.py:42-71 circular_prefix_sum */
static void circular_prefix_sum(const float* x, int nbins, float* out, int nsum) {
  out[0] = x[0];
  for (int i = 1; i < nbins && i < nsum; ++i) out[i] = out[i - 1] + x[i];
  if (nsum <= nbins) return;
  const float last = out[nbins - 1];
  const int n_wraps = nsum / nbins, extra = nsum % nbins;
  for (int w = 1; w < n_wraps; ++w) {
    const float add = (float)w * last;
    for (int j = 0; j < nbins; ++j) out[w * nbins + j] = out[j] + add;
  }
  if (extra > 0) {
    const float add = (float)n_wraps * last;
    for (int j = 0; j < extra; ++j) out[n_wraps * nbins + j] = out[j] + add;
  }
}

static double snr_one(const float* prefix, int nbins, int64_t width, float total) {
  const int64_t size_w = nbins - width;
  const double height = sqrt((double)size_w / (double)(nbins * width));
  const double b = (double)width * height / (double)size_w;
  float dmax = -FLT_MAX;
  for (int i = 0; i < nbins; ++i) {
    const float d = prefix[i + width] - prefix[i];
    if (d > dmax) dmax = d;
  }
  return (height + b) * (double)dmax - (b * (double)total);
}

/* detection/scoring.py:99-153 boxcar_snr_1d / boxcar_snr_2d */
void oracle_boxcar_snr(const float* prof, int64_t nprof, int nbins, const int64_t* widths,
                       int nw, double stdnoise, float* out, int nthreads) {
  set_threads(nthreads);
  int64_t wmax = 0;
  for (int i = 0; i < nw; ++i) wmax = widths[i] > wmax ? widths[i] : wmax;
  const double inv = 1.0 / stdnoise;
#pragma omp parallel
  {
    float* prefix = (float*)malloc((nbins + wmax) * sizeof(float));
#pragma omp for schedule(static)
    for (int64_t p = 0; p < nprof; ++p) {
      circular_prefix_sum(prof + p * nbins, nbins, prefix, (int)(nbins + wmax));
      const float total = prefix[nbins - 1];
      for (int iw = 0; iw < nw; ++iw)
        out[p * nw + iw] = (float)(snr_one(prefix, nbins, widths[iw], total) * inv);
    }
    free(prefix);
  }
}

/* detection/scoring.py:249-282 snr_score_batch_func: folds (n, 2, nbins). */
void oracle_snr_score_batch(const float* folds, int64_t n, int nbins, const int64_t* widths,
                            int nw, float* out, int nthreads) {
  set_threads(nthreads);
  int64_t wmax = 0;
  for (int i = 0; i < nw; ++i) wmax = widths[i] > wmax ? widths[i] : wmax;
#pragma omp parallel
  {
    float* prefix = (float*)malloc((nbins + wmax) * sizeof(float));
    float* norm = (float*)malloc(nbins * sizeof(float));
#pragma omp for schedule(static)
    for (int64_t p = 0; p < n; ++p) {
      const float* e = folds + p * 2 * nbins;
      const float* v = e + nbins;
      for (int j = 0; j < nbins; ++j) norm[j] = e[j] / sqrtf(v[j]);
      circular_prefix_sum(norm, nbins, prefix, (int)(nbins + wmax));
      const float total = prefix[nbins - 1];
      double best = -(double)FLT_MAX;
      for (int iw = 0; iw < nw; ++iw) {
        const double s = snr_one(prefix, nbins, widths[iw], total);
        if (s > best) best = s;
      }
      out[p] = (float)best;
    }
    free(prefix);
    free(norm);
  }
}

/* ffa.py:382-411 get_fold_norm (real): (n, 2, nbins) -> (n, nbins) */
void oracle_fold_norm(const float* folds, int64_t n, int nbins, float* out) {
  for (int64_t p = 0; p < n; ++p)
    for (int j = 0; j < nbins; ++j)
      out[p * nbins + j] = folds[p * 2 * nbins + j] / sqrtf(folds[p * 2 * nbins + nbins + j]);
}

/* ---------------------------------------------------------------------------
 * Single-trial recursion: the fold of one parameter set at FFA level `level`,
 * segment `seg`, obtained by walking the resolve tree of unify_fold
 * (dynamic/dyn_pffa.py:462-489) down to level-0 brute folds of one segment at
 * one frequency (core/fold.py:150-170, same sequential sums). Costs one pass
 * over the series per trial, so any trial of a full-size search can be
 * checked without materialising a level.
 * ------------------------------------------------------------------------- */
typedef struct {
  const float* ts_e;
  const float* ts_v;
  int64_t nsamps;
  double tsamp;
  int64_t bseg_brute;
  int n, nbins;
  double tseg_brute;
  const double* limits;
  const int64_t* counts;        /* (nlevels, n) */
  const double* const* params;  /* (nlevels * n) pointers: params[l * n + d] */
} OracleSeries;

static void profile_rec(const OracleSeries* S, int level, int64_t seg, const int64_t* idx,
                        float* out) {
  const int n = S->n, nb = S->nbins;
  if (level == 0) {
    const double f = S->params[n - 1][idx[n - 1]];
    const double t_ref = (n == 1) ? 0.0 : (double)S->bseg_brute * S->tsamp / 2;
    memset(out, 0, 2 * nb * sizeof(float));
    const int64_t start = seg * S->bseg_brute;
    for (int64_t i = 0; i < S->bseg_brute && start + i < S->nsamps; ++i) {
      const double pt = (double)i * S->tsamp - t_ref;
      const int b = round_shift(phase_idx(pt, f, nb, 0.0), nb);
      out[b] += S->ts_e[start + i];
      out[nb + b] += S->ts_v[start + i];
    }
    return;
  }
  double pset[MAXP];
  int64_t it[MAXP], ih[MAXP];
  for (int d = 0; d < n; ++d) pset[d] = S->params[level * n + d][idx[d]];
  const int64_t* cprev = S->counts + (size_t)(level - 1) * n;
  const double pht = oracle_ffa_resolve(pset, n, cprev, S->limits, level, 0, S->tseg_brute, nb, it);
  const double phh = oracle_ffa_resolve(pset, n, cprev, S->limits, level, 1, S->tseg_brute, nb, ih);
  float* t = (float*)malloc(4 * nb * sizeof(float));
  float* h = t + 2 * nb;
  profile_rec(S, level - 1, 2 * seg, it, t);
  profile_rec(S, level - 1, 2 * seg + 1, ih, h);
  const int st = round_shift(pht, nb), sh = round_shift(phh, nb);
  for (int j = 0; j < nb; ++j) {
    const int i1 = ((j - st) % nb + nb) % nb;
    const int i2 = ((j - sh) % nb + nb) % nb;
    out[j] = t[i1] + h[i2];
    out[nb + j] = t[nb + i1] + h[nb + i2];
  }
  free(t);
}

/* Profiles (ntrials, 2, nbins) of segment `seg` at `level` for the given
 * flattened parameter indices of that level's grid. */
void oracle_ffa_trials(const float* ts_e, const float* ts_v, int64_t nsamps, double tsamp,
                       int64_t bseg_brute, int n, int nbins, const double* limits,
                       const int64_t* counts, const double* const* params, int level,
                       int64_t seg, const int64_t* flat_idx, int64_t ntrials, float* out,
                       int nthreads) {
  set_threads(nthreads);
  OracleSeries S = {ts_e, ts_v, nsamps, tsamp, bseg_brute, n, nbins,
                    (double)bseg_brute * tsamp, limits, counts, params};
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < ntrials; ++k) {
    int64_t idx[MAXP];
    int64_t rest = flat_idx[k];
    for (int d = n - 1; d >= 0; --d) {
      const int64_t c = counts[(size_t)level * n + d];
      idx[d] = rest % c;
      rest /= c;
    }
    profile_rec(&S, level, seg, idx, out + (size_t)k * 2 * nbins);
  }
}

/* The same single-trial recursion with every profile held and summed in
 * float64 (level-0 brute folds of the float32 samples, then the shift-adds):
 * the FP64 reference for reduced-precision fold storage. */
static void profile_rec_f64(const OracleSeries* S, int level, int64_t seg, const int64_t* idx,
                            double* out) {
  const int n = S->n, nb = S->nbins;
  if (level == 0) {
    const double f = S->params[n - 1][idx[n - 1]];
    const double t_ref = (n == 1) ? 0.0 : (double)S->bseg_brute * S->tsamp / 2;
    memset(out, 0, 2 * nb * sizeof(double));
    const int64_t start = seg * S->bseg_brute;
    for (int64_t i = 0; i < S->bseg_brute && start + i < S->nsamps; ++i) {
      const double pt = (double)i * S->tsamp - t_ref;
      const int b = round_shift(phase_idx(pt, f, nb, 0.0), nb);
      out[b] += (double)S->ts_e[start + i];
      out[nb + b] += (double)S->ts_v[start + i];
    }
    return;
  }
  double pset[MAXP];
  int64_t it[MAXP], ih[MAXP];
  for (int d = 0; d < n; ++d) pset[d] = S->params[level * n + d][idx[d]];
  const int64_t* cprev = S->counts + (size_t)(level - 1) * n;
  const double pht = oracle_ffa_resolve(pset, n, cprev, S->limits, level, 0, S->tseg_brute, nb, it);
  const double phh = oracle_ffa_resolve(pset, n, cprev, S->limits, level, 1, S->tseg_brute, nb, ih);
  double* t = (double*)malloc(4 * nb * sizeof(double));
  double* h = t + 2 * nb;
  profile_rec_f64(S, level - 1, 2 * seg, it, t);
  profile_rec_f64(S, level - 1, 2 * seg + 1, ih, h);
  const int st = round_shift(pht, nb), sh = round_shift(phh, nb);
  for (int j = 0; j < nb; ++j) {
    const int i1 = ((j - st) % nb + nb) % nb;
    const int i2 = ((j - sh) % nb + nb) % nb;
    out[j] = t[i1] + h[i2];
    out[nb + j] = t[nb + i1] + h[nb + i2];
  }
  free(t);
}

void oracle_ffa_trials_f64(const float* ts_e, const float* ts_v, int64_t nsamps, double tsamp,
                           int64_t bseg_brute, int n, int nbins, const double* limits,
                           const int64_t* counts, const double* const* params, int level,
                           int64_t seg, const int64_t* flat_idx, int64_t ntrials, double* out,
                           int nthreads) {
  set_threads(nthreads);
  OracleSeries S = {ts_e, ts_v, nsamps, tsamp, bseg_brute, n, nbins,
                    (double)bseg_brute * tsamp, limits, counts, params};
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t k = 0; k < ntrials; ++k) {
    int64_t idx[MAXP];
    int64_t rest = flat_idx[k];
    for (int d = n - 1; d >= 0; --d) {
      const int64_t c = counts[(size_t)level * n + d];
      idx[d] = rest % c;
      rest /= c;
    }
    profile_rec_f64(&S, level, seg, idx, out + (size_t)k * 2 * nbins);
  }
}
