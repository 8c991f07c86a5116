/*
 * CPU oracle for the Taylor and Chebyshev enumerate-prune levels (test
 * infrastructure only:
 * the parity checker in tests/ and the CPU baseline of bench.py; the product
 * never links or calls this file).
 *
 * One call runs one level of prune.py:165-332 pruning_iteration_batched with
 * the PrunePolyTaylorDPFuncts plugin (dynamic/dyn_poly_taylor.py:447-628):
 *   branch    core/taylor.py:68-169 (+ utils/psr_utils.py:131-143,227-248,
 *             347-379 and utils/np_utils.py:174-238 cartesian_prod_padded)
 *   resolve   core/taylor.py:172-277 (+ utils/transforms.py:10-48,
 *             utils/psr_utils.py:12-46,517-554)
 *   shift-add core/common.py:375-400 shift_add_batch
 *   score     detection/scoring.py:249-282 snr_score_batch_func
 *   threshold prune.py:271-276, transform core/taylor.py:323-339 with
 *             utils/transforms.py:93-138, backtrack prune.py:298-304
 *   add       utils/world_tree.py:482-551 add_batch / prune_on_overload,
 *             600-614 keep
 * With basis = 1 the level is the PrunePolyChebyshevDPFuncts plugin
 * (dynamic/dyn_poly_cheby.py:537-840): the parents are first shifted from
 * the previous to the current Chebyshev domain (core/chebyshev.py:75-179
 * with utils/transforms.py:661-710 shift_cheby_full), then branched with
 * the Chebyshev steps (utils/psr_utils.py:259-278), resolved through
 * cheby_to_taylor_param_shift (core/chebyshev.py:182-251,
 * utils/transforms.py:713-738 and 554-579) and transformed to the next
 * domain (core/chebyshev.py:340-356).
 * Batches of parents are processed in order exactly as the reference does;
 * inside a batch the children are independent and are resolved, folded and
 * scored in parallel (OpenMP), like the numba prange loops.
 *
 * Arithmetic follows the shimmed reference: IEEE double/float, numpy matmul
 * accumulated with forward fused multiply-adds (OpenBLAS dgemm order),
 * float32 scores compared with float64 thresholds (numba typing).
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
#define M6 (MAXP + 1)

typedef struct {
  int poly_order, nbins, nparams_ffa, moving, tiling, branch_max;
  double eta;
  double dparams_f[MAXP]; /* poly_taylor_step_f(P, tobs, nbins, eta, 0) */
  double factors[MAXP];   /* poly_taylor_shift_d_vec factors (before f/c) */
  double tm_add[M6][M6];  /* moving: t0_add - t0_cur; fixed: t0_add - t0_init */
  double tm_init[M6][M6]; /* moving: t0_init - t0_cur */
  double tm_next[M6][M6]; /* moving: t0_next - t0_cur */
  double dt_phase;        /* t0_add - t0_init */
  int64_t n_accel, n_freq;
  double accel_min, accel_max, freq_min, freq_max;
  /* Chebyshev basis (basis = 1). Matrices in row-product form: row k of
   * M is column k of the reference's matrix, so x @ A is mat_row(x, M, k). */
  int basis;
  double cm_prev[M6][M6]; /* shift_cheby_full coord_prev -> coord_cur (branch) */
  double cm_add[M6][M6];  /* coord_cur domain re-centred at t0_add (fixed: t0_init domain) */
  double cm_init[M6][M6]; /* coord_cur domain re-centred at t0_init (moving resolve) */
  double cm_next[M6][M6]; /* shift_cheby_full coord_cur -> coord_next (transform) */
  double r_mat[M6][M6];   /* compute_connection_matrix_r, row-product form */
  double k_fact[M6];      /* k! */
  double k_tspow[M6];     /* ts^k, ts the scale of the resolve domain */
  /* circular-orbit tree (basis = 2, poly_order 5) */
  double sig_prop;        /* propagator_significance */
  double sig_val;         /* validation_significance */
  double omega_max_sq;    /* (2 pi / p_orb_min)^2 */
  double x_mass_const;
  double dt_add;          /* moving: t0_add - t0_cur; fixed: t0_add - t0_init */
  double dt_init;         /* moving: t0_init - t0_cur */
  double dt_next;         /* moving: t0_next - t0_cur */
} OPruneLevel;

static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/* x @ T.T, row i: forward fused multiply-adds over j. */
static double mat_row(const double* x, const double T[M6][M6], int i, int m) {
  double acc = 0.0;
  for (int j = 0; j < m; ++j) acc = fma(x[j], T[i][j], acc);
  return acc;
}

/* utils/psr_utils.py:12-46 */
static double phase_idx(double proper_time, double freq, int nbins, double delay) {
  double phase = (proper_time - delay) * freq;
  phase -= floor(phase);
  double iphase = phase * (double)nbins;
  if (iphase >= (double)nbins) iphase = 0.0;
  return iphase;
}

/* core/common.py:389-391 */
static int round_shift(double phase, int nbins) {
  int s = (int)((float)phase + 0.5f);
  return s == nbins ? 0 : s;
}

/* utils/psr_utils.py:517-554, one axis */
static int64_t nearest(double v, double vmin, double vmax, int64_t n) {
  const double inv = vmax > vmin ? (double)n / (vmax - vmin) : 0.0;
  if (!(inv > 0.0)) return 0;
  int64_t idx = (int64_t)((v - vmin) * inv + FLOAT_EPSILON);
  if (idx < 0) idx = 0;
  else if (idx >= n) idx = n - 1;
  return idx;
}

/* detection/scoring.py:42-71 + 249-282 for one (2, nbins) fold */
static float score_fold(const float* f, int nbins, const int64_t* widths, int nw, float* norm,
                        float* prefix) {
  int64_t wmax = 0;
  for (int i = 0; i < nw; ++i) wmax = widths[i] > wmax ? widths[i] : wmax;
  for (int j = 0; j < nbins; ++j) norm[j] = f[j] / sqrtf(f[nbins + j]);
  const int nsum = (int)(nbins + wmax);
  prefix[0] = norm[0];
  for (int i = 1; i < nbins && i < nsum; ++i) prefix[i] = prefix[i - 1] + norm[i];
  if (nsum > nbins) {
    const float last = prefix[nbins - 1];
    const int n_wraps = nsum / nbins, extra = nsum % nbins;
    for (int w = 1; w < n_wraps; ++w) {
      const float add = (float)w * last;
      for (int j = 0; j < nbins; ++j) prefix[w * nbins + j] = prefix[j] + add;
    }
    const float add = (float)n_wraps * last;
    for (int j = 0; j < extra; ++j) prefix[n_wraps * nbins + j] = prefix[j] + add;
  }
  const float total = prefix[nbins - 1];
  double best = -(double)FLT_MAX;
  for (int iw = 0; iw < nw; ++iw) {
    const int64_t width = widths[iw];
    const int64_t size_w = nbins - width;
    const double height = sqrt((double)size_w / (double)(nbins * width));
    const double b = (double)width * height / (double)size_w;
    float dmax = -FLT_MAX;
    for (int i = 0; i < nbins; ++i) {
      const float d = prefix[i + width] - prefix[i];
      if (d > dmax) dmax = d;
    }
    const double snr = (height + b) * (double)dmax - (b * (double)total);
    if (snr > best) best = snr;
  }
  return (float)best;
}

typedef struct {
  int64_t count[MAXP];
  double first[MAXP], dact[MAXP];
  int branched[MAXP];
  int64_t total;
} Branch;

/* core/taylor.py:68-169 for one parent; returns 0 or -1 (branch_max). */
static int branch_parent(const OPruneLevel* L, const double* lf, Branch* B) {
  const int P = L->poly_order;
  const double f0 = lf[(P + 1) * 2];
  const double tol = L->eta - FLOAT_EPSILON;
  int rc = 0;
  B->total = 1;
  for (int j = 0; j < P; ++j) {
    const double pcur = lf[2 * j], dcur = lf[2 * j + 1];
    const double dnew = L->dparams_f[j] * C_VAL / f0;
    const double shift = fabs(dcur - dnew) * (L->factors[j] * (f0 / C_VAL));
    int64_t num = 1;
    double dact = dcur, first = pcur;
    int branched = 1;
    if (!(dcur > 0.0) || !(dnew > 0.0)) {
      rc = -1;
    } else {
      const double ratio = dcur / dnew;
      num = (int64_t)ceil(ratio - FLOAT_EPSILON);
      if (num < 1) num = 1;
      if (num > L->branch_max) rc = -1;
      dact = dcur / (double)num;
      first = (pcur - dcur / 2.0) + dact / 2.0;
    }
    if (shift < tol) {
      num = 1;
      dact = dcur;
      first = pcur;
      branched = 0;
    }
    B->branched[j] = branched;
    B->count[j] = num;
    B->first[j] = first;
    B->dact[j] = dact;
    B->total *= num;
  }
  return rc;
}

typedef struct {
  double leaf[2 * (MAXP + 2)];
  float fold[2 * 512];
  float score;
  int64_t parent;
  int32_t ia, iff;
  double phase;
  int cls; /* circular tree: 1 snap, 2 crackle, 0 Taylor */
} Child;

/* Child k (C-order odometer, last parameter fastest) of parent lf. */
static void make_child(const OPruneLevel* L, const double* lf, const Branch* B, int64_t k,
                       double* out) {
  const int P = L->poly_order;
  memset(out, 0, sizeof(double) * 2 * (P + 2));
  for (int j = P - 1; j >= 0; --j) {
    const int64_t c = B->count[j];
    const int64_t i = k % c;
    k /= c;
    /* branched: first_center + i * dact; kept: the parent's value itself */
    out[2 * j] = B->branched[j] ? B->first[j] + (double)i * B->dact[j] : B->first[j];
    out[2 * j + 1] = B->dact[j];
  }
  out[2 * P] = lf[2 * P];              /* d0 (error stays 0) */
  out[2 * (P + 1)] = lf[2 * (P + 1)];  /* f0 */
  out[2 * (P + 1) + 1] = lf[2 * (P + 1) + 1];
}

static void resolve(const OPruneLevel* L, Child* ch) {
  const int P = L->poly_order, m = P + 1;
  double pv[M6];
  for (int i = 0; i < m; ++i) pv[i] = ch->leaf[2 * i];
  const double f0 = ch->leaf[2 * m];
  double accel, vel, dd;
  if (L->moving) {
    accel = mat_row(pv, L->tm_add, P - 2, m);
    vel = mat_row(pv, L->tm_add, P - 1, m) - mat_row(pv, L->tm_init, P - 1, m);
    dd = mat_row(pv, L->tm_add, P, m) - mat_row(pv, L->tm_init, P, m);
  } else {
    accel = mat_row(pv, L->tm_add, P - 2, m);
    vel = mat_row(pv, L->tm_add, P - 1, m);
    dd = mat_row(pv, L->tm_add, P, m);
  }
  const double freq = f0 * (1 - vel / C_VAL);
  const double delay = dd / C_VAL;
  ch->phase = phase_idx(L->dt_phase, f0, L->nbins, delay);
  ch->ia = (int32_t)nearest(accel, L->accel_min, L->accel_max, L->n_accel);
  ch->iff = (int32_t)nearest(freq, L->freq_min, L->freq_max, L->n_freq);
}

/* core/taylor.py:323-339 + utils/transforms.py:93-138 */
static void transform(const OPruneLevel* L, const double* in, double* out) {
  const int P = L->poly_order, m = P + 1;
  memcpy(out, in, sizeof(double) * 2 * (P + 2));
  if (!L->moving) return;
  double v[M6], e[M6];
  for (int i = 0; i < m; ++i) {
    v[i] = in[2 * i];
    e[i] = in[2 * i + 1];
  }
  for (int i = 0; i < m; ++i) out[2 * i] = mat_row(v, L->tm_next, i, m);
  if (L->tiling == 0) {
    for (int i = 0; i < m; ++i) out[2 * i + 1] = e[i] * fabs(L->tm_next[i][i]);
  } else if (L->tiling == 2) {
    double A[M6][M6];
    for (int i = 0; i < M6; ++i)
      for (int j = 0; j < M6; ++j) A[i][j] = fabs(L->tm_next[i][j]);
    for (int i = 0; i < m; ++i) out[2 * i + 1] = mat_row(e, A, i, m);
  } else {
    double A[M6][M6], e2[M6];
    for (int i = 0; i < M6; ++i)
      for (int j = 0; j < M6; ++j) A[i][j] = L->tm_next[i][j] * L->tm_next[i][j];
    for (int j = 0; j < m; ++j) e2[j] = e[j] * e[j];
    for (int i = 0; i < m; ++i) out[2 * i + 1] = sqrt(mat_row(e2, A, i, m));
  }
  out[2 * m] = in[2 * m];
  out[2 * m + 1] = in[2 * m + 1];
}

/* utils/transforms.py:661-710 shift_cheby_full of rows 0..P (values and
 * errors; the tiling strategy propagates the errors). */
static void cheby_shift(const OPruneLevel* L, const double M[M6][M6], const double* in,
                        double* out) {
  const int m = L->poly_order + 1;
  double v[M6], e[M6];
  for (int i = 0; i < m; ++i) {
    v[i] = in[2 * i];
    e[i] = in[2 * i + 1];
  }
  for (int k = 0; k < m; ++k) out[2 * k] = mat_row(v, M, k, m);
  if (L->tiling == 0) {
    for (int k = 0; k < m; ++k) out[2 * k + 1] = e[k] * fabs(M[k][k]);
  } else if (L->tiling == 2) {
    double A[M6][M6];
    for (int i = 0; i < M6; ++i)
      for (int j = 0; j < M6; ++j) A[i][j] = fabs(M[i][j]);
    for (int k = 0; k < m; ++k) out[2 * k + 1] = mat_row(e, A, k, m);
  } else {
    double A[M6][M6], e2[M6];
    for (int i = 0; i < M6; ++i)
      for (int j = 0; j < M6; ++j) A[i][j] = M[i][j] * M[i][j];
    for (int j = 0; j < m; ++j) e2[j] = e[j] * e[j];
    for (int k = 0; k < m; ++k) out[2 * k + 1] = sqrt(mat_row(e2, A, k, m));
  }
}

/* utils/transforms.py:713-738 cheby_to_taylor_param_shift: the Chebyshev
 * values re-centred by M, then cheby_to_taylor (554-579): ascending power
 * coefficients d[k] = (alpha_asc @ R)[k] * k! / ts^k. */
static void cheby_taylor(const OPruneLevel* L, const double M[M6][M6], const double* alpha,
                         double* d) {
  const int m = L->poly_order + 1;
  double a[M6], asc[M6];
  for (int k = 0; k < m; ++k) a[k] = mat_row(alpha, M, k, m);
  for (int k = 0; k < m; ++k) asc[k] = a[m - 1 - k];
  for (int k = 0; k < m; ++k) d[k] = mat_row(asc, L->r_mat, k, m) * L->k_fact[k] / L->k_tspow[k];
}

/* core/chebyshev.py:182-282 (moving and fixed grid) */
static void resolve_cheby(const OPruneLevel* L, Child* ch) {
  const int m = L->poly_order + 1;
  double alpha[M6], da[M6];
  for (int i = 0; i < m; ++i) alpha[i] = ch->leaf[2 * i];
  const double f0 = ch->leaf[2 * m];
  cheby_taylor(L, L->cm_add, alpha, da);
  double accel = da[2], vel = da[1], dd = da[0];
  if (L->moving) {
    double di[M6];
    cheby_taylor(L, L->cm_init, alpha, di);
    vel = da[1] - di[1];
    dd = da[0] - di[0];
  }
  const double freq = f0 * (1 - vel / C_VAL);
  const double delay = dd / C_VAL;
  ch->phase = phase_idx(L->dt_phase, f0, L->nbins, delay);
  ch->ia = (int32_t)nearest(accel, L->accel_min, L->accel_max, L->n_accel);
  ch->iff = (int32_t)nearest(freq, L->freq_min, L->freq_max, L->n_freq);
}

/* core/chebyshev.py:340-356 (moving grid; the fixed grid keeps the leaf) */
static void transform_cheby(const OPruneLevel* L, const double* in, double* out) {
  const int P = L->poly_order;
  memcpy(out, in, sizeof(double) * 2 * (P + 2));
  if (L->moving) cheby_shift(L, L->cm_next, in, out);
}

/* core/circular.py:14-81 get_circ_mask for one leaf (values v, errors e,
 * rows [crackle, snap, jerk, accel, ...]): 1 circular by snap-accel, 2 by
 * crackle-jerk (the hole), 0 Taylor. */
static int circ_class(const double* v, const double* e, double sig) {
  const int sig_snap = fabs(v[1]) > sig * e[1];
  const int sig_accel = fabs(v[3]) > sig * e[3];
  const int sig_jerk = fabs(v[2]) > sig * e[2];
  if (sig_snap && sig_accel && (-v[1] * v[3]) > 0) return 1;
  if (sig_jerk && (-v[0] * v[2]) > 0) return 2;
  return 0;
}

/* utils/transforms.py:248-310 shift_taylor_circular_params of one leaf's
 * values [d5 .. d0] by dt (in_hole: omega from crackle-jerk). */
static void circ_shift(const double* v, double dt, int in_hole, double* o) {
  const double d5 = v[0], d4 = v[1], d3 = v[2], d2 = v[3], d1 = v[4], d0 = v[5];
  const double w2 = in_hole ? -d5 / d3 : -d4 / d2;
  const double w = sqrt(w2);
  const double wdt = w * dt;
  const double c = cos(wdt), sn = sin(wdt);
  const double d2j = d2 * c + (d3 / w) * sn;
  const double d3j = d3 * c - (d2 * w) * sn;
  const double d1ci = -d3 / w2, d1cj = -d3j / w2;
  const double d0cj = -d2j / w2, d0ci = -d2 / w2;
  o[0] = -w2 * d3j;
  o[1] = -w2 * d2j;
  o[2] = d3j;
  o[3] = d2j;
  o[4] = d1cj + (d1 - d1ci);
  o[5] = d0cj + (d0 - d0ci) + (d1 - d1ci) * dt;
}

/* core/circular.py:83-125 circ_validate_batch for one leaf */
static int circ_valid(const OPruneLevel* L, const double* v, const double* e) {
  const double vs = L->sig_val;
  const int sig_snap = fabs(v[1]) > vs * e[1];
  const int sig_accel = fabs(v[3]) > vs * e[3];
  const int phys = (-v[1] * v[3]) > 0.0;
  if (!(sig_snap && sig_accel)) return 1; /* the hole is never validated */
  if (!phys) return 0;
  const double w2 = -v[1] / v[3];
  const double limit = L->x_mass_const * pow(w2, 2.0 / 3.0);
  return w2 <= L->omega_max_sq && fabs(v[3]) <= limit;
}

/* core/circular.py:444-597 (moving and fixed grid) for one child; sets its class */
static void resolve_circ(const OPruneLevel* L, Child* ch) {
  const int P = 5, m = 6;
  double v[M6], e[M6];
  for (int i = 0; i < m; ++i) {
    v[i] = ch->leaf[2 * i];
    e[i] = ch->leaf[2 * i + 1];
  }
  ch->cls = circ_class(v, e, L->sig_prop);
  if (ch->cls == 0) {
    resolve(L, ch);
    return;
  }
  const double f0 = ch->leaf[2 * (P + 1)];
  double a[M6];
  circ_shift(v, L->dt_add, ch->cls == 2, a);
  double accel = a[3], vel = a[4], dd = a[5];
  if (L->moving) {
    double b[M6];
    circ_shift(v, L->dt_init, ch->cls == 2, b);
    vel = a[4] - b[4];
    dd = a[5] - b[5];
  }
  const double freq = f0 * (1 - vel / C_VAL);
  const double delay = dd / C_VAL;
  ch->phase = phase_idx(L->dt_phase, f0, L->nbins, delay);
  ch->ia = (int32_t)nearest(accel, L->accel_min, L->accel_max, L->n_accel);
  ch->iff = (int32_t)nearest(freq, L->freq_min, L->freq_max, L->n_freq);
}

/* core/circular.py:670-706 (moving grid): closed-form shift of the values
 * (errors unchanged) for the circular classes, the Taylor transform else */
static void transform_circ(const OPruneLevel* L, const Child* ch, double* out) {
  const int P = 5;
  if (!L->moving) {
    memcpy(out, ch->leaf, sizeof(double) * 2 * (P + 2));
    return;
  }
  if (ch->cls == 0) {
    transform(L, ch->leaf, out);
    return;
  }
  memcpy(out, ch->leaf, sizeof(double) * 2 * (P + 2));
  double v[M6], o[M6];
  for (int i = 0; i < P + 1; ++i) v[i] = ch->leaf[2 * i];
  circ_shift(v, L->dt_next, ch->cls == 2, o);
  for (int i = 0; i < P + 1; ++i) out[2 * i] = o[i];
}

/* core/circular.py:205-395 circ_taylor_branch_batch over parents [b0, b1)
 * then circ_taylor_validate_batch (398-441): the validated children in the
 * reference's order (the kept children of every parent, then each
 * expanded cell's crackle children). Returns the validated count, or -1
 * when a parameter needs more than branch_max children; *n_branch gets the
 * count before validation. */
static int64_t circ_children(const OPruneLevel* L, const double* leaves, int64_t b0,
                             int64_t b1, Child** out, int64_t* n_branch) {
  const int P = 5;
  const int64_t nbat = b1 - b0;
  Branch* br = (Branch*)malloc(sizeof(Branch) * nbat);
  int* needs0 = (int*)malloc(sizeof(int) * nbat);
  double* d0new = (double*)malloc(sizeof(double) * nbat);
  int64_t total = 0;
  int rc = 0;
  for (int64_t i = 0; i < nbat && !rc; ++i) {
    const double* lf = leaves + (b0 + i) * 2 * (P + 2);
    rc = branch_parent(L, lf, &br[i]);
    /* crackle: held at the parent value with the would-be child step
     * (psr_utils.py:383-398), or the parent step when it needs no branching */
    const double f0 = lf[2 * (P + 1)];
    const double dcur = lf[1], dnew = L->dparams_f[0] * C_VAL / f0;
    const double shift = fabs(dcur - dnew) * (L->factors[0] * (f0 / C_VAL));
    needs0[i] = !(shift < L->eta - FLOAT_EPSILON);
    d0new[i] = dnew;
    double dact = dcur;
    if (needs0[i] && dcur > 0.0 && dnew > 0.0) {
      int64_t num = (int64_t)ceil(dcur / dnew - FLOAT_EPSILON);
      if (num < 1) num = 1;
      dact = dcur / (double)num;
    }
    br[i].total /= br[i].count[0];
    br[i].count[0] = 1;
    br[i].branched[0] = 0;
    br[i].first[0] = lf[0];
    br[i].dact[0] = dact;
    total += br[i].total;
  }
  if (rc) {
    free(br);
    free(needs0);
    free(d0new);
    return -1;
  }
  /* first product; cells in the hole whose crackle step is too coarse expand */
  typedef struct {
    double leaf[2 * (MAXP + 2)];
    int64_t parent;
  } Cell;
  Cell* first = (Cell*)malloc(sizeof(Cell) * (total > 0 ? total : 1));
  int* expand = (int*)malloc(sizeof(int) * (total > 0 ? total : 1));
  int64_t n_keep = 0, n_exp_children = 0, c = 0;
  for (int64_t i = 0; i < nbat; ++i) {
    const double* lf = leaves + (b0 + i) * 2 * (P + 2);
    for (int64_t k = 0; k < br[i].total; ++k, ++c) {
      make_child(L, lf, &br[i], k, first[c].leaf);
      first[c].parent = b0 + i;
      double v[M6], e[M6];
      for (int j = 0; j < P + 1; ++j) {
        v[j] = first[c].leaf[2 * j];
        e[j] = first[c].leaf[2 * j + 1];
      }
      const double sg = L->sig_prop;
      const int snap = fabs(v[1]) > sg * e[1] && fabs(v[3]) > sg * e[3] && (-v[1] * v[3]) > 0;
      expand[c] = !snap && fabs(v[2]) > sg * e[2] && needs0[i];
      if (!expand[c]) {
        ++n_keep;
      } else {
        const double dcur = lf[1];
        int64_t num = (int64_t)ceil(dcur / d0new[i] - FLOAT_EPSILON);
        if (num < 1) num = 1;
        if (num > L->branch_max) rc = -1;
        n_exp_children += num;
      }
    }
  }
  *n_branch = n_keep + n_exp_children;
  Child* ch = (Child*)malloc(sizeof(Child) * (*n_branch > 0 ? *n_branch : 1));
  int64_t w = 0;
  for (int pass = 0; pass < 2 && !rc; ++pass) {
    for (int64_t q = 0; q < total; ++q) {
      if (expand[q] != pass) continue;
      const Cell* src = &first[q];
      if (!pass) {
        memcpy(ch[w].leaf, src->leaf, sizeof(src->leaf));
        ch[w++].parent = src->parent;
        continue;
      }
      /* psr_utils.py:347-380 branch_param_padded of the crackle */
      const double* lf = leaves + src->parent * 2 * (P + 2);
      const double pcur = src->leaf[0], dcur = lf[1];
      const double dnew = d0new[src->parent - b0];
      int64_t num = (int64_t)ceil(dcur / dnew - FLOAT_EPSILON);
      if (num < 1) num = 1;
      const double dact = dcur / (double)num;
      const double first_center = (pcur - dcur / 2.0) + dact / 2.0;
      for (int64_t k = 0; k < num; ++k) {
        memcpy(ch[w].leaf, src->leaf, sizeof(src->leaf));
        ch[w].parent = src->parent;
        ch[w].leaf[0] = first_center + (double)k * dact;
        ch[w].leaf[1] = dact;
        ++w;
      }
    }
  }
  free(first);
  free(expand);
  free(br);
  free(needs0);
  free(d0new);
  if (rc) {
    free(ch);
    return -1;
  }
  /* validation keeps the order */
  int64_t nv = 0;
  for (int64_t q = 0; q < w; ++q) {
    double v[M6], e[M6];
    for (int j = 0; j < P + 1; ++j) {
      v[j] = ch[q].leaf[2 * j];
      e[j] = ch[q].leaf[2 * j + 1];
    }
    if (!circ_valid(L, v, e)) continue;
    if (nv != q) {
      memcpy(ch[nv].leaf, ch[q].leaf, sizeof(ch[q].leaf));
      ch[nv].parent = ch[q].parent;
    }
    ++nv;
  }
  *out = ch;
  return nv;
}

/* np.partition order: ascending, NaN last. */
static int cmp_float(const void* a, const void* b) {
  const float x = *(const float*)a, y = *(const float*)b;
  const int nx = x != x, ny = y != y;
  if (nx || ny) return nx - ny;
  return (x > y) - (x < y);
}

typedef struct {
  double* leaves;
  float *folds, *scores;
  int32_t* bt;
  int64_t valid, size;
  int P, nbins;
} Tree;

static void tree_put(Tree* T, int64_t pos, const double* leaf, const float* fold, float score,
                     const int32_t* bt) {
  const int P = T->P;
  memcpy(T->leaves + pos * 2 * (P + 2), leaf, sizeof(double) * 2 * (P + 2));
  memcpy(T->folds + pos * 2 * T->nbins, fold, sizeof(float) * 2 * T->nbins);
  T->scores[pos] = score;
  memcpy(T->bt + pos * (P + 2), bt, sizeof(int32_t) * (P + 2));
}

static void tree_move(Tree* T, int64_t dst, int64_t src) {
  if (dst == src) return;
  tree_put(T, dst, T->leaves + src * 2 * (T->P + 2), T->folds + src * 2 * T->nbins,
           T->scores[src], T->bt + src * (T->P + 2));
}

/* utils/world_tree.py:482-551 add_batch (+ prune_on_overload, keep). */
static double add_batch(Tree* T, int64_t n, double* const* leaves, float* const* folds,
                        const float* scores, int32_t* const* bts, double current) {
  if (n == 0) return current;
  if (n <= T->size - T->valid) {
    for (int64_t i = 0; i < n; ++i) tree_put(T, T->valid + i, leaves[i], folds[i], scores[i], bts[i]);
    T->valid += n;
    return current;
  }
  const int64_t total = T->valid + n;
  float* scratch = (float*)malloc(sizeof(float) * total);
  memcpy(scratch, T->scores, sizeof(float) * T->valid);
  memcpy(scratch + T->valid, scores, sizeof(float) * n);
  qsort(scratch, total, sizeof(float), cmp_float);
  const float kth = scratch[total - T->size];
  const float mid = scratch[total - total / 2 - 1];
  free(scratch);
  const double topk = nextafter((double)kth, INFINITY);
  const double med = nextafter((double)mid, INFINITY);
  double eff = current;
  if (topk > eff) eff = topk;
  if (med > eff) eff = med;
  int64_t w = 0;
  for (int64_t r = 0; r < T->valid; ++r)
    if ((double)T->scores[r] >= eff) tree_move(T, w++, r);
  T->valid = w;
  for (int64_t i = 0; i < n && T->valid < T->size; ++i)
    if ((double)scores[i] >= eff) {
      tree_put(T, T->valid, leaves[i], folds[i], scores[i], bts[i]);
      T->valid += 1;
    }
  return eff;
}

/* core/common.py:375-400 shift_add_batch + scoring.py:249-282 for one child */
static void fold_score(const OPruneLevel* L, Child* c, const float* folds, const float* seg,
                       const int64_t* widths, int nw, float* norm, float* prefix) {
  const int nb = L->nbins;
  const int s = round_shift(c->phase, nb);
  const float* pf = folds + c->parent * 2 * nb;
  const float* sf = seg + ((int64_t)c->ia * L->n_freq + c->iff) * 2 * nb;
  int src = (nb - s) % nb;
  for (int j = 0; j < nb; ++j) {
    c->fold[j] = pf[j] + sf[src];
    c->fold[nb + j] = pf[nb + j] + sf[nb + src];
    if (++src == nb) src = 0;
  }
  c->score = score_fold(c->fold, nb, widths, nw, norm, prefix);
}

/* prune.py:276-323 for one batch's scored children: score range,
 * threshold, transform of the survivors, backtracks, add_batch. */
static void select_add(const OPruneLevel* L, Child* ch, int64_t nch, double threshold,
                       double* current, Tree* T, double* smin, double* smax) {
  const int P = L->poly_order;
  /* np.min/np.max over the batch; Python min/max then skip a NaN batch value */
  float bmin = ch[0].score, bmax = ch[0].score;
  int has_nan = 0;
  for (int64_t c = 0; c < nch; ++c) {
    const float s = ch[c].score;
    if (s != s) has_nan = 1;
    if (s < bmin) bmin = s;
    if (s > bmax) bmax = s;
  }
  if (!has_nan) {
    if ((double)bmin < *smin) *smin = bmin;
    if ((double)bmax > *smax) *smax = bmax;
  }
  const double thr = threshold > *current ? threshold : *current;
  int64_t npass = 0;
  for (int64_t c = 0; c < nch; ++c) npass += (double)ch[c].score >= thr;
  if (npass == 0) return;
  double** pl = (double**)malloc(sizeof(double*) * npass);
  float** pfo = (float**)malloc(sizeof(float*) * npass);
  int32_t** pbt = (int32_t**)malloc(sizeof(int32_t*) * npass);
  float* ps = (float*)malloc(sizeof(float) * npass);
  double* tl = (double*)malloc(sizeof(double) * npass * 2 * (P + 2));
  int32_t* tb = (int32_t*)malloc(sizeof(int32_t) * npass * (P + 2));
  int64_t w = 0;
  for (int64_t c = 0; c < nch; ++c) {
    if (!((double)ch[c].score >= thr)) continue;
    double* out = tl + w * 2 * (P + 2);
    if (L->basis == 2) transform_circ(L, &ch[c], out);
    else if (L->basis == 1) transform_cheby(L, ch[c].leaf, out);
    else transform(L, ch[c].leaf, out);
    int32_t* bt = tb + w * (P + 2);
    memset(bt, 0, sizeof(int32_t) * (P + 2));
    bt[0] = (int32_t)ch[c].parent;
    bt[L->nparams_ffa - 1] = ch[c].ia;
    bt[L->nparams_ffa] = ch[c].iff;
    bt[P + 1] = (int32_t)ch[c].phase;
    pl[w] = out;
    pfo[w] = ch[c].fold;
    pbt[w] = bt;
    ps[w] = ch[c].score;
    ++w;
  }
  *current = add_batch(T, npass, pl, pfo, ps, pbt, *current);
  free(pl);
  free(pfo);
  free(pbt);
  free(ps);
  free(tl);
  free(tb);
}

/*
 * One pruning level. leaves (n_par, P+2, 2) f64, folds (n_par, 2, nbins) f32,
 * seg = FFA fold of the added segment (n_accel*n_freq rows of (2, nbins)).
 * Output tree of capacity max_sugg. stats = {n_leaves, n_leaves_phy};
 * smm = {score_min, score_max}. Returns the new tree size, or -1 when a
 * parent needs more than branch_max children.
 */
int64_t oracle_prune_level(const OPruneLevel* L, const double* leaves, const float* folds,
                           int64_t n_par, const float* seg, const int64_t* widths, int nw,
                           double threshold, int64_t max_sugg, int64_t batch_size,
                           double* lout, float* fout, float* sout, int32_t* bout,
                           int64_t* stats, double* smm, int nthreads) {
  set_threads(nthreads);
  const int P = L->poly_order, nb = L->nbins;
  if (nb > 256 || P < 2 || P > MAXP || (L->basis == 2 && P != 5)) return -2;
  Tree T = {lout, fout, sout, bout, 0, max_sugg, P, nb};
  double current = threshold;
  int64_t n_leaves = 0, n_phy = 0;
  double smin = INFINITY, smax = -INFINITY;
  if (batch_size > n_par) batch_size = n_par;
  if (batch_size < 1) batch_size = 1;
  const int cheby = L->basis == 1, circ = L->basis == 2;
  Branch* br = (Branch*)malloc(sizeof(Branch) * batch_size);
  int64_t* off = (int64_t*)malloc(sizeof(int64_t) * (batch_size + 1));
  /* Chebyshev: the batch's parents shifted to the current domain */
  double* shifted = cheby ? (double*)malloc(sizeof(double) * batch_size * 2 * (P + 2)) : NULL;
  int rc = 0;
  for (int64_t b0 = 0; b0 < n_par && !rc; b0 += batch_size) {
    const int64_t b1 = b0 + batch_size < n_par ? b0 + batch_size : n_par;
    const int64_t nbat = b1 - b0;
    Child* ch = NULL;
    int64_t nch = 0;
    if (circ) {
      int64_t nbr = 0;
      nch = circ_children(L, leaves, b0, b1, &ch, &nbr);
      if (nch < 0) {
        rc = -1;
        break;
      }
      n_leaves += nbr;
      n_phy += nch;
#pragma omp parallel
      {
        float norm[512], prefix[1024];
#pragma omp for schedule(static)
        for (int64_t c = 0; c < nch; ++c) {
          resolve_circ(L, &ch[c]);
          fold_score(L, &ch[c], folds, seg, widths, nw, norm, prefix);
        }
      }
      if (L->moving) { /* core/circular.py:478-509: the basis flag of the batch */
        int has_taylor = 0;
        for (int64_t c = 0; c < nch; ++c) has_taylor |= ch[c].cls == 0;
        for (int64_t c = 0; c < nch; ++c) {
          double* flag = &ch[c].leaf[2 * (P + 1) + 1];
          if (ch[c].cls == 1) *flag = 1.0;
          else if (ch[c].cls == 2) *flag = has_taylor ? 0.0 : 2.0;
        }
      }
    } else {
      off[0] = 0;
      for (int64_t i = 0; i < nbat && !rc; ++i) {
        const double* lf = leaves + (b0 + i) * 2 * (P + 2);
        if (cheby) {
          double* sh = shifted + i * 2 * (P + 2);
          memcpy(sh, lf, sizeof(double) * 2 * (P + 2));
          cheby_shift(L, L->cm_prev, lf, sh);
          lf = sh;
        }
        rc = branch_parent(L, lf, &br[i]);
        off[i + 1] = off[i] + br[i].total;
      }
      if (rc) break;
      nch = off[nbat];
      n_leaves += nch;
      n_phy += nch;
      if (nch > 0) ch = (Child*)malloc(sizeof(Child) * nch);
#pragma omp parallel
      {
        float norm[512], prefix[1024];
#pragma omp for schedule(static)
        for (int64_t i = 0; i < nbat; ++i) {
          const double* lf =
              cheby ? shifted + i * 2 * (P + 2) : leaves + (b0 + i) * 2 * (P + 2);
          for (int64_t k = 0; k < br[i].total; ++k) {
            Child* c = &ch[off[i] + k];
            make_child(L, lf, &br[i], k, c->leaf);
            c->parent = b0 + i;
            if (cheby) resolve_cheby(L, c);
            else resolve(L, c);
            fold_score(L, c, folds, seg, widths, nw, norm, prefix);
          }
        }
      }
    }
    if (nch > 0) select_add(L, ch, nch, threshold, &current, &T, &smin, &smax);
    free(ch);
  }
  free(br);
  free(off);
  free(shifted);
  if (rc) return -1;
  stats[0] = n_leaves;
  stats[1] = n_phy;
  smm[0] = isfinite(smin) ? smin : 0.0;
  smm[1] = isfinite(smax) ? smax : 0.0;
  return T.valid;
}

/*
 * dynamic/dyn_poly_taylor.py:587-628 ascend_func with core/taylor.py:280-320
 * and core/common.py:432-459: re-fold every survivor over the segments so far
 * (in the given order) and re-score. tm (nseg, 6, 6) Taylor matrices for
 * t0_seg - t0_cur, dt (nseg) = t0_seg - t0_cur, seg_rows (nseg) pointers to
 * the FFA fold of each segment. folds/scores are rewritten, scores_ep gets
 * the old scores.
 */
void oracle_prune_ascend(const OPruneLevel* L, const double* leaves, float* folds,
                         float* scores, float* scores_ep, int64_t n, int nseg,
                         const double* tm, const double* dt, const float* const* seg_folds,
                         const int64_t* widths, int nw, int nthreads) {
  set_threads(nthreads);
  const int P = L->poly_order, m = P + 1, nb = L->nbins;
#pragma omp parallel
  {
    float norm[512], prefix[1024];
#pragma omp for schedule(static)
    for (int64_t r = 0; r < n; ++r) {
      const double* lf = leaves + r * 2 * (P + 2);
      double pv[M6];
      for (int i = 0; i < m; ++i) pv[i] = lf[2 * i];
      const double f0 = lf[2 * m];
      int cls = 0;
      if (L->basis == 2) {
        double ev[M6];
        for (int i = 0; i < m; ++i) ev[i] = lf[2 * i + 1];
        cls = circ_class(pv, ev, L->sig_prop);
      }
      float* acc = folds + r * 2 * nb;
      for (int j = 0; j < 2 * nb; ++j) acc[j] = 0.0f;
      for (int s = 0; s < nseg; ++s) {
        const double(*T)[M6] = (const double(*)[M6])(tm + s * M6 * M6);
        double accel, freq, delay;
        if (L->basis == 2 && cls != 0) {  /* core/circular.py:598-667 */
          double o[M6];
          circ_shift(pv, dt[s], cls == 2, o);
          accel = o[3];
          freq = f0 * (1 - o[4] / C_VAL);
          delay = o[5] / C_VAL;
        } else if (L->basis == 1) {  /* core/chebyshev.py:254-300: tm holds the re-centring */
          double d[M6];
          cheby_taylor(L, T, pv, d);
          accel = d[2];
          freq = f0 * (1 - d[1] / C_VAL);
          delay = d[0] / C_VAL;
        } else {
          accel = mat_row(pv, T, P - 2, m);
          freq = f0 * (1 - mat_row(pv, T, P - 1, m) / C_VAL);
          delay = mat_row(pv, T, P, m) / C_VAL;
        }
        const double ph = phase_idx(dt[s], f0, nb, delay);
        const int64_t ia = nearest(accel, L->accel_min, L->accel_max, L->n_accel);
        const int64_t iff = nearest(freq, L->freq_min, L->freq_max, L->n_freq);
        const float* sf = seg_folds[s] + (ia * L->n_freq + iff) * 2 * nb;
        const int sh = round_shift(ph, nb);
        int src = (nb - sh) % nb;
        for (int j = 0; j < nb; ++j) {
          acc[j] += sf[src];
          acc[nb + j] += sf[nb + src];
          if (++src == nb) src = 0;
        }
      }
      scores_ep[r] = scores[r];
      scores[r] = score_fold(acc, nb, widths, nw, norm, prefix);
    }
  }
}

/* out[r] = x[r] @ A for n rows of m values, with M the row-product form of
 * A (forward fused multiply-adds, the dgemm order of the reference's numpy
 * matmul); used for the Chebyshev seed (utils/transforms.py:458-487). */
void oracle_rowprod(const double* x, int64_t n, int m, const double* M, double* out) {
  const double(*T)[M6] = (const double(*)[M6])M;
  for (int64_t r = 0; r < n; ++r)
    for (int k = 0; k < m; ++k) out[r * m + k] = mat_row(x + r * m, T, k, m);
}
