/*
 * loki_gb300 — C ABI of the GB300 (sm_103a) FFA / scoring / pruning kernels.
 *
 * Every entry point takes device pointers that the caller allocated, plain
 * sizes, and a CUDA stream (as void*; NULL = legacy default stream). Nothing
 * here allocates device memory. Calls are asynchronous on the given stream
 * and return a status code (LOKI_OK or a negative LOKI_ERR_*); a readable
 * message for the last failure on the calling thread is available from
 * loki_last_error(). Kernels never trap: range violations found on the device
 * are written to the caller's int32 error word (0 = no error), which the
 * caller reads after synchronising.
 *
 * Array layouts follow pyloki exactly (C-contiguous):
 *   fold     float32 (nsegments, *param_counts, 2, nbins)   [2 = (ts_e, ts_v) sums]
 *   fold_c   complex64 (nsegments, *param_counts, 2, nbins/2+1) [Fourier domain]
 *   snr      float32 (nprofiles, nwidths)
 */
#ifndef LOKI_GB300_H
#define LOKI_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LOKI_OK 0
#define LOKI_ERR_INVALID -1     /* bad argument (size, null pointer, layout) */
#define LOKI_ERR_CUDA -2        /* a CUDA launch or runtime call failed */
#define LOKI_ERR_UNSUPPORTED -3 /* valid but not handled (e.g. nbins too large) */
#define LOKI_ERR_CAPACITY -4    /* output capacity too small (e.g. branch_max) */

/* Device-side error word values. */
#define LOKI_DEVERR_NONE 0
#define LOKI_DEVERR_WINDOW 1   /* resolved index outside the input window */
#define LOKI_DEVERR_BRANCH 2   /* branch count above branch_max */
#define LOKI_DEVERR_TIMEOUT 4  /* a bounded wait on the tensor cores gave up */
#define LOKI_DEVERR_CAPACITY 8 /* a device-counted run outgrew a workspace */

#define LOKI_MAX_PARAMS 5
#define LOKI_MAX_WIDTHS 64
#define LOKI_MAX_RESCORE_LEVELS 24

/* One FFA dynamic-programming level: the current grid (optionally a window of
 * its last, frequency, dimension) resolved against the previous level's grid
 * (optionally a window of its last dimension). */
typedef struct {
  int32_t nparams;          /* 1..5, order [..., jerk, accel, freq] */
  int32_t nbins;            /* profile bins */
  int32_t level;            /* current FFA level, >= 1 */
  int32_t storage;          /* fold element type: 0 float32, 1 bfloat16 (adds and
                               scores in float32; each stored value rounded once) */
  double tseg_brute;        /* seconds, bseg_brute * tsamp */
  int64_t counts_cur[LOKI_MAX_PARAMS];   /* full grid counts, current level */
  int64_t counts_prev[LOKI_MAX_PARAMS];  /* full grid counts, previous level */
  double limits[LOKI_MAX_PARAMS][2];     /* param_limits (min, max) */
  const double* param_arr[LOKI_MAX_PARAMS]; /* device: current-level grid per dim */
  int64_t out_start;        /* first current-level frequency index computed */
  int64_t out_width;        /* number of current-level frequency indices */
  int64_t in_start;         /* first previous-level frequency index held in fold_in */
  int64_t in_width;         /* previous-level frequency indices held in fold_in */
  int64_t nseg_in;          /* segments in fold_in; output has nseg_in / 2 */
  /* Optional (may be NULL): device float2 array, counts_cur[nparams-1]
   * entries, of the last-dimension grid split as (float(f), float(f - float(f))).
   * Lets the kernels skip one FP64 operation per parameter set. */
  const float* last_split;
} LokiFFALevel;

/* Packed plan entry, identical to pyloki's ffacoord_dtype (ffa.py:36-43). */
typedef struct {
  uint32_t i_tail;
  float shift_tail;
  uint32_t i_head;
  float shift_head;
} LokiFFACoord;

/* Boxcar scoring constants. hb[w] = height + b and b[w] as float64, computed
 * by the host with the reference's expressions (detection/scoring.py:99-140). */
typedef struct {
  int32_t nwidths;
  int32_t wmax;             /* max(widths) */
  int32_t mode;             /* 0: one S/N per width; 1: max over widths */
  int32_t nseg;             /* fused final level only: output segments scored,
                               0 or 1 = segment 0; S/N rows are segment-major
                               (nseg, full grid, nout). Ignored elsewhere. */
  double inv_stdnoise;
  int32_t widths[LOKI_MAX_WIDTHS];
  double hb[LOKI_MAX_WIDTHS];
  double b[LOKI_MAX_WIDTHS];
} LokiScoreSpec;

/* ---- library ---------------------------------------------------------- */
int loki_version(void);
const char* loki_last_error(void);
/* Kernels this library has enqueued from the calling host thread so far
 * (monotone). No reference counterpart: it lets a caller count launches. */
int64_t loki_launch_count(void);

/* ---- FFA (time domain, float32) --------------------------------------- */

/* Brute fold of a series into (nsegments, nfreqs, 2, nbins) at the start of
 * the FFA. Replaces core/fold.py:108-171 brutefold_start (called through
 * ffa_taylor_init, core/fold.py:527-569). Per (segment, freq, bin) the sum is
 * taken in sample order, so the result is bit-identical to the reference.
 * phase_scratch holds the (freq, sample) phase-bin map; it may be smaller
 * than nfreqs * segment_len bytes (nbins <= 256) or 2x that (nbins > 256),
 * in which case the frequencies are processed in chunks. */
int loki_brutefold(const float* ts_e, const float* ts_v, int64_t nsamps,
                   const double* freqs, int64_t nfreqs, int64_t segment_len,
                   int32_t nbins, double tsamp, double t_ref,
                   void* phase_scratch, int64_t scratch_bytes,
                   float* fold_out, void* stream);

/* Scratch bytes with which loki_brutefold / loki_brutefold_unit_variance fold
 * all nfreqs frequencies in one pass. With nbins <= 256 that is the phase
 * map plus the chain layout (per frequency: segment_len bytes of map, then
 * per 512-sample time chunk the chunk's positions sorted by bin, 1 KiB, and
 * the bin starts); a smaller scratch folds in frequency chunks, and one too
 * small for a single frequency of the chain layout uses the map alone. No
 * reference counterpart. */
int64_t loki_brutefold_scratch_bytes(int64_t nfreqs, int64_t segment_len, int32_t nbins);

/* loki_brutefold for a series whose ts_v is all ones (the normalised series
 * io/timeseries.py:198-236 from_tim produces). Every variance sum of the
 * reference is then the bin's sample count, exact in float32, and the same
 * for every full segment: it is written from one histogram of the phase map
 * per frequency, and only the ts_e sums run sample by sample (half the
 * shared memory per thread). The fold is bit-identical to loki_brutefold's
 * with ts_v = 1. segment_len < 2^24. No reference counterpart as an entry
 * point. */
int loki_brutefold_unit_variance(const float* ts_e, int64_t nsamps, const double* freqs,
                                 int64_t nfreqs, int64_t segment_len, int32_t nbins,
                                 double tsamp, double t_ref, void* phase_scratch,
                                 int64_t scratch_bytes, float* fold_out, void* stream);

/* loki_brutefold without a caller-supplied phase scratch and without any
 * device allocation: no counterpart in the reference. For callers that may
 * not allocate device memory: cudaMalloc and cudaFree synchronise the whole
 * device, stalling a host pipeline that keeps other streams busy, and a host
 * that holds a fixed device-memory budget has nothing left to hand out.
 * The map lives in a fixed 16 MiB device array of the library (its size is
 * returned by loki_brutefold_noalloc_scratch_bytes), so segment_len is
 * limited to 16 Mi samples for nbins <= 256 and 8 Mi for nbins > 256;
 * beyond that it returns LOKI_ERR_CAPACITY. The array is shared by all calls
 * on one device: calls that overlap on the GPU (different streams, no
 * ordering between them) race on it; calls on one stream are ordered. */
int loki_brutefold_noalloc(const float* ts_e, const float* ts_v, int64_t nsamps,
                           const double* freqs, int64_t nfreqs, int64_t segment_len,
                           int32_t nbins, double tsamp, double t_ref,
                           float* fold_out, void* stream);
int64_t loki_brutefold_noalloc_scratch_bytes(void);

/* Plan table of one FFA level (one entry per current-level parameter set in
 * the output window). Replaces the per-parameter resolve inside unify_fold
 * (dynamic/dyn_pffa.py:462-475 -> core/fold.py:617-671) and
 * FFAPlan.resolve_coordinates[_freq] (ffa.py:105-193). */
int loki_ffa_plan(const LokiFFALevel* lvl, LokiFFACoord* coords, int32_t* dev_err,
                  void* stream);

/* One FFA DP level: fold_out[ipair, p] = roll(fold_in[2 ipair, tail(p)], s_t)
 * + roll(fold_in[2 ipair + 1, head(p)], s_h). Replaces unify_fold
 * (dynamic/dyn_pffa.py:435-489) with shift_add (core/common.py:304-324). */
int loki_ffa_level(const LokiFFALevel* lvl, const void* fold_in, void* fold_out,
                   int32_t* dev_err, void* stream);

/* Final FFA level fused with normalisation and boxcar scoring of segment 0:
 * the unify_fold of the last level, get_fold_norm (ffa.py:382-411) and
 * boxcar_snr_nd (detection/scoring.py:156-165) in one pass; the final fold is
 * never written. snr is the full-grid array (P_full, nwidths), or (P_full,)
 * in mode 1; a frequency window writes only its own rows. */
int loki_ffa_level_score(const LokiFFALevel* lvl, const void* fold_in,
                         const LokiScoreSpec* spec, float* snr, int32_t* dev_err,
                         void* stream);

/* Band windows for the banded final levels: for bands of band_width
 * current-level frequency indices, the [lo, hi] range of previous-level
 * frequency indices that their tail and head resolve to (over every other
 * parameter). win_lo / win_hi hold ceil(counts_cur[-1] / band_width) int64.
 * Host-side planning helper with no reference counterpart; it lets the last
 * two levels of a large FFA run in memory-bounded frequency bands. */
int loki_ffa_band_windows(const LokiFFALevel* lvl, int64_t band_width,
                          int64_t* win_lo, int64_t* win_hi, void* stream);

/* Banded last two levels: for each band k of band_width final frequencies,
 * compute the penultimate level restricted to the host window
 * [win_lo[k], win_hi[k]] into scratch (loki_ffa_level), then the final level
 * of the band fused with scoring (loki_ffa_level_score). pen / fin describe
 * the full penultimate and final levels (their windows are overwritten per
 * band); fold_pp is the materialised level before the penultimate. Together
 * these replace the last two unify_fold calls (dynamic/dyn_pffa.py:435-489)
 * plus get_fold_norm and boxcar_snr_nd without materialising either level.
 * win_lo / win_hi are HOST arrays (from loki_ffa_band_windows). */
int loki_ffa_final_banded(const LokiFFALevel* pen, const LokiFFALevel* fin,
                          int64_t band_width, const int64_t* win_lo, const int64_t* win_hi,
                          const void* fold_pp, float* scratch, int64_t scratch_floats,
                          const LokiScoreSpec* spec, float* snr, int32_t* dev_err,
                          void* stream);

/* Floats of scratch loki_ffa_final_banded needs for penultimate windows of at
 * most max_window frequencies: the band fold plus two small per-level resolve
 * tables. Returns -1 for invalid descriptors. */
int64_t loki_ffa_final_banded_scratch(const LokiFFALevel* pen, const LokiFFALevel* fin,
                                      int64_t max_window);

/* Last two FFA levels fused in one persistent launch: the penultimate and the
 * final unify_fold (dynamic/dyn_pffa.py:435-489) plus get_fold_norm
 * (ffa.py:382-411) and boxcar_snr_nd (detection/scoring.py:156-165), with
 * neither level written to global memory. Each CTA takes a tile (output
 * segment, run of final "other" parameter sets that resolve to the same
 * penultimate others, 64 final frequencies), builds the penultimate rows the
 * tile reads in shared memory from fold_pp (the materialised level before the
 * penultimate), and scores the tile's trials from there. pen / fin describe
 * the full (unwindowed) penultimate and final levels. nbins must be 64 and the
 * widths 1, 2, 4, ..., 2^(nw-1) with nw <= 6 (else LOKI_ERR_UNSUPPORTED: use
 * loki_ffa_final_banded). fast_norm 0 normalises with correctly rounded
 * division and square root (S/N bit-identical to the reference); 1 uses
 * e * rsqrt(v) (S/N within 1e-5 of the reference relative to max(|S/N|, 1)).
 * scratch (64-byte aligned, loki_ffa_final_tiled_scratch bytes) holds the
 * per-level resolve tables and the tile groups. */
int loki_ffa_final_tiled(const LokiFFALevel* pen, const LokiFFALevel* fin, const void* fold_pp,
                         void* scratch, int64_t scratch_bytes, const LokiScoreSpec* spec,
                         int32_t fast_norm, float* snr, int32_t* dev_err, void* stream);
/* Bytes of scratch loki_ffa_final_tiled needs; -1 for invalid descriptors. */
int64_t loki_ffa_final_tiled_scratch(const LokiFFALevel* pen, const LokiFFALevel* fin);

/* Round n float32 values to bfloat16 (nearest even): the brute fold, summed
 * in float32, enters a bfloat16-stored FFA (LokiFFALevel.storage = 1).
 * No reference counterpart: the reference stores float32 only. */
int loki_f32_to_bf16(const float* in, int64_t n, void* out, void* stream);

/* FP64 re-scoring of FFA candidates. levels[l - 1] describes FFA level l
 * (full grids, l = 1 .. nlevels, the last being the candidates' level); the
 * series (ts_e, ts_v, device float32, nsamps samples) and the level-0
 * frequency grid freqs0 (device, nfreq0 values) are those of the search;
 * cand holds ncand flat parameter indices of the last level (device) and
 * segs, if not NULL, each candidate's segment of that level (device; NULL:
 * every candidate in segment seg). Each candidate's fold is rebuilt from the
 * samples: the resolve
 * tree (dynamic/dyn_pffa.py:462-489) gives every level-0 segment's frequency
 * and accumulated shift, its samples are binned as in the brute fold
 * (core/fold.py:108-171) and everything is summed in float64. snr receives
 * (ncand, nwidths) boxcar S/N (detection/scoring.py:99-140) in float64 and
 * prof, if not NULL, the float64 profiles (ncand, 2, nbins). A candidate
 * index outside the last level's grid, or a segment without all its level-0
 * segments, yields NaN rows.
 * No reference counterpart: it backs bfloat16 fold storage, whose retained
 * candidates are re-scored here. */
int loki_ffa_rescore(const LokiFFALevel* levels, int32_t nlevels, const float* ts_e,
                     const float* ts_v, int64_t nsamps, double tsamp, int64_t bseg_brute,
                     const double* freqs0, int64_t nfreq0, const int64_t* cand,
                     const int64_t* segs, int64_t ncand, int64_t seg,
                     const LokiScoreSpec* spec, double* snr, double* prof, void* stream);

/* ---- FFA (Fourier domain, complex64 = 2 x float32 per coefficient) ----
 * Folds are (nseg, nparams..., 2, nbins / 2 + 1) complex64, nbins even.
 * The float32 / complex64 arithmetic follows the reference's expressions;
 * its BLAS, numpy cos/sin and pocketfft are not reproduced bit for bit. */

/* Complex brute fold (core/fold.py:395-481 brutefold_start_complex_opt, via
 * ffa_taylor_init_complex 572-614): the DFT of every segment at the
 * harmonics h * f, h = 0 .. nbins / 2, with the t_ref phase correction.
 * nsamps must be a multiple of segment_len. ts_v may be NULL, meaning all
 * ones: the variance sums are then the same for every segment and are taken
 * once (the same values). */
int loki_brutefold_complex(const float* ts_e, const float* ts_v, int64_t nsamps,
                           const double* freqs, int64_t nfreqs, int64_t segment_len,
                           int32_t nbins, double tsamp, double t_ref, void* fold_out,
                           void* stream);

/* One complex DP level (dynamic/dyn_pffa.py:435-489 with shift_add_complex,
 * core/common.py:344-372): out[ipair, p] = tail * e^{-2 pi i k s_t / nbins}
 * + head * e^{-2 pi i k s_h / nbins} by phasor recurrence over k, the rows
 * and float32 shifts taken from the level's plan (loki_ffa_plan). Whole
 * levels only (no frequency window). */
int loki_ffa_level_complex(const LokiFFALevel* lvl, const LokiFFACoord* plan,
                           const void* fold_in, void* fold_out, void* stream);

/* Normalised profiles of complex folds (ffa.py:401-411): irfft of both
 * components to nbins samples, then e / sqrt(v); folds (n, 2, nbins / 2 + 1)
 * complex64 -> out (n, nbins) float32. */
int loki_fold_norm_complex(const void* folds, int64_t n, int32_t nbins, float* out,
                           void* stream);

/* ---- enumerate-prune (Taylor / Chebyshev basis, float32 folds) -------- */

/* Constants of one pruning level, computed by the host with the reference's
 * numpy expressions (prune.py:165-332 with core/taylor.py:68-339):
 * leaves are (P + 2, 2) float64 rows [d_P .. d_1, d_0, (f0, flag)] x (value,
 * error); backtracks are (P + 2) int32 [parent, ffa param idx.., phase]. */
typedef struct {
  int32_t poly_order;     /* P (number of Taylor parameters d_P..d_1), <= 5 */
  int32_t nbins;
  int32_t nparams_ffa;    /* parameters of the FFA grid (backtrack columns) */
  int32_t moving;         /* 1: moving grid, 0: fixed grid */
  int32_t tiling;         /* 0 aggressive, 1 quadrature, 2 conservative */
  int32_t branch_max;
  double eta_m;           /* eta - FLOAT_EPSILON */
  double dfc[LOKI_MAX_PARAMS];      /* poly_taylor_step_f(...) * C, order d_P..d_1 */
  double fac[LOKI_MAX_PARAMS];      /* bin-shift factors (psr_utils.py:227-248) */
  double tm_a[LOKI_MAX_PARAMS + 1][LOKI_MAX_PARAMS + 1]; /* Taylor shift to t0_add */
  double tm_i[LOKI_MAX_PARAMS + 1][LOKI_MAX_PARAMS + 1]; /* ... to t0_init (moving) */
  double tm_n[LOKI_MAX_PARAMS + 1][LOKI_MAX_PARAMS + 1]; /* transform to t0_next */
  double tm_e[LOKI_MAX_PARAMS + 1][LOKI_MAX_PARAMS + 1]; /* |tm_n| or tm_n**2 */
  double dt_phase;        /* t0_add - t0_init */
  int64_t n_accel, n_freq;          /* FFA grid counts of the accel / freq axes */
  double accel_min, accel_inv;      /* accel_inv = n_accel / range, 0 if flat */
  double freq_min, freq_inv;
  /* Chebyshev basis (core/chebyshev.py; basis = 1). Leaves then hold
   * coefficients [alpha_P .. alpha_0]; every matrix M below is applied as
   * y_i = sum_j x_j M[i][j] with forward fused multiply-adds, i.e. the host
   * passes the transpose of the reference's right-hand matrix:
   *   tm_b  = C(prev -> cur)^T        parent shift before branching
   *   tm_be = |C|^T or (C**2)^T       its error matrix (tiling 2 / 1)
   *   tm_a, tm_i = C(cur -> t_add / t_init, same scale)^T   (resolve)
   *   tm_n, tm_e = C(cur -> next)^T and its error matrix   (transform)
   *   tm_r  = R^T (Chebyshev -> power series connection matrix)
   * and the Taylor value of order k is (d_k * cfact[k]) / ctsk[k]. For the
   * Taylor basis (basis = 0) these fields are ignored. */
  int32_t basis;
  int32_t reserved2;
  double tm_b[LOKI_MAX_PARAMS + 1][LOKI_MAX_PARAMS + 1];
  double tm_be[LOKI_MAX_PARAMS + 1][LOKI_MAX_PARAMS + 1];
  double tm_r[LOKI_MAX_PARAMS + 1][LOKI_MAX_PARAMS + 1];
  double cfact[LOKI_MAX_PARAMS + 1];  /* k! */
  double ctsk[LOKI_MAX_PARAMS + 1];   /* scale**k */
  /* Circular-orbit Taylor tree (core/circular.py; basis = 2, poly_order 5):
   * significance levels of the circular classification and of the physical
   * validation, (2 pi / p_orb_min)**2, the mass constant, and the time
   * offsets of the closed-form circular propagation. On the moving grid
   * circ_dt_add / circ_dt_init / circ_dt_next are t0_add / t0_init /
   * t0_next minus t0_cur; on the fixed grid circ_dt_add is t0_add - t0_init. */
  double circ_sig_prop, circ_sig_valid, circ_omega_max_sq, circ_x_mass;
  double circ_dt_add, circ_dt_init, circ_dt_next;
} LokiPruneLevel;

/* Per-parent branching result. */
typedef struct {
  double first[LOKI_MAX_PARAMS];  /* first child centre (or the parent value) */
  double dact[LOKI_MAX_PARAMS];   /* actual child step (or the parent step) */
  int32_t count[LOKI_MAX_PARAMS];
  int32_t reserved;
  double d0;                      /* the children's lowest-order value */
} LokiBranchInfo;

/* Branch every parent (core/taylor.py:68-169 poly_taylor_branch_batch):
 * info[i] and the exclusive child offsets (n_parents + 1 int64; the last is
 * the number of leaves). scan_scratch needs loki_scan_scratch_bytes(n + 1). */
int loki_prune_branch(const LokiPruneLevel* lvl, const double* leaves, int64_t n_parents,
                      LokiBranchInfo* info, int64_t* offsets, void* scan_scratch,
                      int64_t scan_scratch_bytes, int32_t* dev_err, void* stream);

/* Resolve, gather, shift-add and score every child leaf (core/taylor.py:
 * 172-277, core/common.py:375-400, detection/scoring.py:249-282). Writes the
 * child score, its (accel, freq) FFA indices and its phase; score_minmax
 * (2 floats, min then max) is atomically folded over all children. */
int loki_prune_score(const LokiPruneLevel* lvl, const double* leaves, const float* folds,
                     int64_t n_parents, const LokiBranchInfo* info, const int64_t* offsets,
                     int64_t n_children, const float* fold_segment,
                     const LokiScoreSpec* spec, float* child_scores, int32_t* child_idx,
                     double* child_phase, float* score_minmax, int32_t* dev_err,
                     void* stream);

/* Ids of the children whose score >= threshold, in order (no overflow). */
int loki_prune_select(const float* child_scores, int64_t n_children, double threshold,
                      int64_t* surv_ids, int64_t* n_surv, void* scan_scratch,
                      int64_t scan_scratch_bytes, void* stream);

/* Exact batch-sequential selection with the overflow rule of
 * WorldTree.add_batch / prune_on_overload (utils/world_tree.py:482-551), for
 * when more than capacity children pass. One block walks the parent batches
 * in order; ids (capacity + 16 * batch children) int64 and keys (same count)
 * float32 are scratch. Writes the survivor ids, their count and the final
 * threshold (float64). */
int loki_prune_select_overflow(const float* child_scores, const int64_t* offsets,
                               int64_t n_parents, int64_t batch_size, double threshold,
                               int64_t capacity, int64_t* surv_ids, int64_t* n_surv,
                               double* thr_out, int64_t* scratch_ids, float* scratch_keys,
                               int64_t scratch_len, void* stream);

/* Write the new tree from the survivors (transform core/taylor.py:323-339,
 * backtrack prune.py:307-312): leaves, folds, scores, scores_ep, backtracks. */
int loki_prune_emit(const LokiPruneLevel* lvl, const double* leaves, const float* folds,
                    const LokiBranchInfo* info, const int64_t* offsets, int64_t n_parents,
                    const float* fold_segment, const int64_t* surv_ids, int64_t n_surv,
                    const float* child_scores, const int32_t* child_idx,
                    const double* child_phase, double* leaves_out, float* folds_out,
                    float* scores_out, float* scores_ep_out, int32_t* bt_out,
                    void* stream);

/* Re-fold every survivor over all segments so far and re-score it
 * (dynamic/dyn_poly_taylor.py:587-628 ascend_func). Device arrays, one entry
 * per segment in accumulation order: tm_seg the Taylor shift matrices
 * ((P+1)^2 doubles each, to t0_seg - t0_cur), dt_seg the phase time offsets,
 * seg_idx the segment index into ffa_fold (nseg_ffa, *counts, 2, nbins) whose
 * segments are seg_stride floats apart. Overwrites folds and scores and copies
 * the old scores to scores_ep. */
int loki_prune_ascend(const LokiPruneLevel* lvl, const double* leaves, float* folds,
                      float* scores, float* scores_ep, int64_t n, int32_t nseg,
                      const double* tm_seg, const double* dt_seg, const int32_t* seg_idx,
                      const float* ffa_fold, int64_t seg_stride, const LokiScoreSpec* spec,
                      int32_t* dev_err, void* stream);

/* loki_prune_ascend with the survivor count on the device (*n_dev <= n_cap),
 * for a run whose counts never reach the host (loki_prune_run); Taylor and
 * Chebyshev trees. Same reference function as loki_prune_ascend. */
int loki_prune_ascend_dev(const LokiPruneLevel* lvl, const double* leaves, float* folds,
                          float* scores, float* scores_ep, const int64_t* n_dev, int64_t n_cap,
                          int32_t nseg, const double* tm_seg, const double* dt_seg,
                          const int32_t* seg_idx, const float* ffa_fold, int64_t seg_stride,
                          const LokiScoreSpec* spec, int32_t* dev_err, void* stream);

/* ---- complex (Fourier) folds ---------------------------------------------
 * The same steps for trees over Fourier-domain FFA folds
 * (PrunePolyTaylorComplexDPFuncts / PrunePolyChebyshevComplexDPFuncts):
 * folds and FFA segment rows are (2, nbins / 2 + 1) complex64, the segment
 * row is rotated by the phasor recurrence of shift_add_complex_batch
 * (core/common.py:403-429) and scored through its irfft
 * (detection/scoring.py:285-292); the ascend sums rotated rows
 * (core/common.py:460-490). Taylor and Chebyshev bases; nbins even. */
int loki_prune_score_complex(const LokiPruneLevel* lvl, const double* leaves, const void* folds,
                             int64_t n_parents, const LokiBranchInfo* info,
                             const int64_t* offsets, int64_t n_children,
                             const void* fold_segment, const LokiScoreSpec* spec,
                             float* child_scores, int32_t* child_idx, double* child_phase,
                             float* score_minmax, int32_t* dev_err, void* stream);
int loki_prune_emit_complex(const LokiPruneLevel* lvl, const double* leaves, const void* folds,
                            const LokiBranchInfo* info, const int64_t* offsets,
                            int64_t n_parents, const void* fold_segment,
                            const int64_t* surv_ids, int64_t n_surv, const float* child_scores,
                            const int32_t* child_idx, const double* child_phase,
                            double* leaves_out, void* folds_out, float* scores_out,
                            float* scores_ep_out, int32_t* bt_out, void* stream);
int loki_prune_ascend_complex(const LokiPruneLevel* lvl, const double* leaves, void* folds,
                              float* scores, float* scores_ep, int64_t n, int32_t nseg,
                              const double* tm_seg, const double* dt_seg,
                              const int32_t* seg_idx, const void* ffa_fold, int64_t seg_stride,
                              const LokiScoreSpec* spec, int32_t* dev_err, void* stream);

/* ---- circular-orbit tree (basis = 2, poly_order 5) ---------------------
 * One level of prune.py:165-332 with the PruneCircTaylorDPFuncts plugin
 * (dynamic/dyn_circular_taylor.py:444-740, core/circular.py:13-705):
 *   loki_prune_circ_branch  circ_taylor_branch_batch: per-parent branching
 *       info, and exclusive scans (n + 1 int64 each) of the children that keep
 *       the parent crackle (keep_off) and of those from crackle expansion
 *       (exp_off); children total = keep_off[n] + exp_off[n].
 *   loki_prune_circ_map     every child at its batch-ordered position in
 *       child_map (16 bytes each) and its circ_taylor_validate_batch result
 *       as 1.0 / 0.0 in valid_flags; compact with loki_prune_select
 *       (threshold 0.5) to the valid children (n_leaves_phy of them).
 *   loki_prune_circ_score   resolve (circular or Taylor propagation by
 *       get_circ_mask class), gather, shift-add and score of every valid
 *       child; child_class (int8) and batch_taylor (int32 per parent batch)
 *       feed the basis flag; batch_offsets (n + 1 int64) are the valid-child
 *       offsets at parent-batch boundaries, for loki_prune_select_overflow.
 *   loki_prune_circ_emit    circ_taylor_transform_batch, basis flags,
 *       backtracks and folds of the survivors (ids into the valid list).
 * The ascend is loki_prune_ascend with basis 2. */
int loki_prune_circ_branch(const LokiPruneLevel* lvl, const double* leaves,
                           int64_t n_parents, LokiBranchInfo* info, int64_t* keep_off,
                           int64_t* exp_off, void* scan_scratch, int64_t scan_scratch_bytes,
                           int32_t* dev_err, void* stream);
int loki_prune_circ_map(const LokiPruneLevel* lvl, const double* leaves, int64_t n_parents,
                        int64_t batch_size, const LokiBranchInfo* info,
                        const int64_t* keep_off, const int64_t* exp_off, void* child_map,
                        float* valid_flags, void* stream);
int loki_prune_circ_score(const LokiPruneLevel* lvl, const double* leaves, const float* folds,
                          int64_t n_parents, int64_t batch_size, const LokiBranchInfo* info,
                          const void* child_map, const int64_t* keep_off,
                          const int64_t* exp_off, const int64_t* valid_ids, int64_t n_valid,
                          const float* fold_segment, const LokiScoreSpec* spec,
                          float* child_scores, int32_t* child_idx, double* child_phase,
                          int8_t* child_class, int32_t* batch_taylor, int64_t* batch_offsets,
                          float* score_minmax, int32_t* dev_err, void* stream);
int loki_prune_circ_emit(const LokiPruneLevel* lvl, const double* leaves, const float* folds,
                         int64_t batch_size, const LokiBranchInfo* info, const void* child_map,
                         const int64_t* valid_ids, const float* fold_segment,
                         const int64_t* surv_ids, int64_t n_surv, const float* child_scores,
                         const int32_t* child_idx, const double* child_phase,
                         const int8_t* child_class, const int32_t* batch_taylor,
                         double* leaves_out, float* folds_out, float* scores_out,
                         float* scores_ep_out, int32_t* bt_out, void* stream);

/* loki_prune_circ_score / loki_prune_circ_emit over complex folds
 * (PruneCircTaylorComplexDPFuncts, dynamic/dyn_circular_taylor.py:168-330):
 * tree folds and segment rows are (2, nbins / 2 + 1) complex64; the children's
 * folds are the phasor-rotated segment row plus the parent fold
 * (core/common.py:403-429), scored through their irfft
 * (detection/scoring.py:285-292). nbins must be even. */
int loki_prune_circ_score_complex(
    const LokiPruneLevel* lvl, const double* leaves, const void* folds, int64_t n_parents,
    int64_t batch_size, const LokiBranchInfo* info, const void* child_map,
    const int64_t* keep_off, const int64_t* exp_off, const int64_t* valid_ids, int64_t n_valid,
    const void* fold_segment, const LokiScoreSpec* spec, float* child_scores,
    int32_t* child_idx, double* child_phase, int8_t* child_class, int32_t* batch_taylor,
    int64_t* batch_offsets, float* score_minmax, int32_t* dev_err, void* stream);
int loki_prune_circ_emit_complex(
    const LokiPruneLevel* lvl, const double* leaves, const void* folds, int64_t batch_size,
    const LokiBranchInfo* info, const void* child_map, const int64_t* valid_ids,
    const void* fold_segment, const int64_t* surv_ids, int64_t n_surv,
    const float* child_scores, const int32_t* child_idx, const double* child_phase,
    const int8_t* child_class, const int32_t* batch_taylor, double* leaves_out,
    void* folds_out, float* scores_out, float* scores_ep_out, int32_t* bt_out, void* stream);

/* loki_prune_branch restricted to the parents with parent_mask[i] != 0
 * (device uint8): the others get no children (their offsets repeat), so the
 * score, select and emit calls of the level skip them while backtracks keep
 * the full tree's parent indices. No reference counterpart: it backs the
 * learned branch proposal; with every mask byte set it is loki_prune_branch. */
int loki_prune_branch_masked(const LokiPruneLevel* lvl, const double* leaves,
                             int64_t n_parents, const uint8_t* parent_mask,
                             LokiBranchInfo* info, int64_t* offsets, void* scan_scratch,
                             int64_t scan_scratch_bytes, int32_t* dev_err, void* stream);

/* ---- native level driver ---------------------------------------------- */

/* A pruning tree on the device: n rows in use of cap. */
typedef struct {
  double* leaves;      /* (cap, poly_order + 2, 2) */
  float* folds;        /* (cap, 2, nbins) */
  float* scores;       /* (cap,) */
  float* scores_ep;    /* (cap,) */
  int32_t* backtracks; /* (cap, poly_order + 2) */
  int64_t n;
  int64_t cap;
} LokiPruneTree;

/* Caller-owned workspace of loki_prune_level (device unless noted). */
typedef struct {
  void* info;              /* par_cap LokiBranchInfo */
  int64_t* offsets;        /* par_cap + 1 */
  void* scan;              /* loki_scan_scratch_bytes(par_cap + 1) */
  int64_t scan_bytes;
  int64_t par_cap;
  float* child_scores;     /* child_cap */
  int32_t* child_idx;      /* 2 * child_cap */
  double* child_phase;     /* child_cap */
  int64_t* surv;           /* child_cap */
  void* sscan;             /* loki_scan_scratch_bytes(child_cap) + 8 (child_cap + 1) */
  int64_t sscan_bytes;
  int64_t child_cap;
  int64_t* n_surv;         /* 1 */
  float* minmax;           /* 2 */
  int64_t* ovf_ids;        /* ovf_cap */
  float* ovf_keys;         /* ovf_cap */
  double* ovf_thr;         /* 1 */
  int64_t ovf_cap;
  int64_t* host_words;     /* pinned host memory, 4 words */
  void* ev_score_begin;    /* optional cudaEvent_t recorded before / after the */
  void* ev_score_end;      /* score launch (NULL: none) */
} LokiPruneWork;

/* What one level did; need_* > 0 names the capacity to grow to after a
 * LOKI_ERR_CAPACITY return (the level can then be run again as is). */
typedef struct {
  int64_t n_parents;
  int64_t n_children;
  int64_t n_surv;
  float score_min;
  float score_max;
  int32_t overflow;        /* the overflow rule ran */
  int32_t dev_err;         /* non-zero: error word set by branch (nothing else ran) */
  int64_t need_par_cap;
  int64_t need_child_cap;
  int64_t need_ovf_cap;
  int64_t need_tree_cap;
} LokiPruneLevelResult;

/* One pruning level of the Taylor or Chebyshev plugin on real folds
 * (prune.py:165-332): branch (restricted to parent_mask when not NULL),
 * score, select with the overflow rule at max_sugg survivors, emit into out.
 * The same calls as loki_prune_branch / _score / _select / _select_overflow /
 * _emit in sequence, with two host waits on w->host_words. */
int loki_prune_level(const LokiPruneLevel* lvl, const LokiPruneTree* in, LokiPruneTree* out,
                     const LokiPruneWork* w, const float* fold_segment,
                     const LokiScoreSpec* spec, double threshold, int64_t max_sugg,
                     int64_t batch_size, const uint8_t* parent_mask, LokiPruneLevelResult* res,
                     int32_t* dev_err, void* stream);

/* Per-level record of a device-resident run (loki_prune_run). n_children is
 * the count the level asked for, also when it exceeded the workspace. */
typedef struct {
  int64_t n_parents;
  int64_t n_children;
  int64_t n_valid;         /* children past validation (the circular tree); n_children otherwise */
  int64_t n_surv;
  float score_min;
  float score_max;
  int32_t overflow;        /* the overflow rule ran */
  int32_t reserved;
} LokiPruneLevelStats;

/* Buffers of loki_prune_run (device unless noted; all caller-owned). */
typedef struct {
  LokiPruneTree trees[2];       /* ping-pong trees, cap >= max_sugg; trees[0] holds the seed */
  LokiPruneWork work;           /* par_cap >= max_sugg, ovf_cap >= max_sugg + child_cap + 1;
                                   host_words and the events are not used */
  int64_t* counts;              /* 8 words: parents, children, survivors, backtrack rows,
                                   valid children of the level */
  int32_t* ovf_flag;            /* 1 word */
  LokiPruneLevelStats* stats;   /* nlevels records */
  double* best_leaves;          /* nlevels rows of (poly_order + 2) * 2, or NULL */
  float* best_scores;           /* nlevels, or NULL */
  int32_t* bt_hist;             /* bt_rows x (poly_order + 2): every level's survivors'
                                   backtracks in level order, or NULL */
  int64_t bt_rows;
  /* circular-orbit tree only (basis 2), else NULL: */
  int64_t* exp_off;             /* par_cap + 1: crackle-expansion children per parent */
  void* child_map;              /* child_cap x 16 B: the children in batch order */
  float* valid_flags;           /* child_cap */
  int64_t* valid_ids;           /* child_cap */
  int8_t* child_class;          /* child_cap */
  int32_t* batch_taylor;        /* par_cap / batch_size + 1 */
  int64_t* batch_offsets;       /* par_cap + 1 */
} LokiPruneRun;

/* Every level of one reference segment (prune.py:526-613 Pruning.execute
 * without the ascend; the same kernels as loki_prune_level) enqueued on the
 * stream with all counts kept on the device: no host wait, so a whole run
 * can be captured in a CUDA graph and replayed. Level l (1-based) reads
 * trees[(l - 1) & 1], writes trees[l & 1], adds segment seg_idx[l - 1] of
 * ffa_folds (segment stride seg_stride floats) at threshold
 * thresholds[l - 1]; stats[l - 1] records it, best_* its best leaf and
 * bt_hist its survivors' backtracks (after those of the levels before). A
 * level without survivors leaves every later level empty. A workspace that
 * is too small sets LOKI_DEVERR_CAPACITY in *dev_err (the run's results are
 * then void: grow work.child_cap to the largest stats[].n_children, or
 * bt_rows to the sum of stats[].n_surv, and run again); a branch count above
 * branch_max sets LOKI_DEVERR_BRANCH. No reference counterpart
 * as one call: it replaces the per-level loop of Pruning.execute. */
int loki_prune_run(const LokiPruneLevel* lvls, int32_t nlevels, const float* ffa_folds,
                   int64_t seg_stride, const int32_t* seg_idx, const double* thresholds,
                   const LokiScoreSpec* spec, int64_t seed_n, int64_t max_sugg,
                   int64_t batch_size, const LokiPruneRun* run, int32_t* dev_err,
                   void* stream);

/* One job of loki_prune_run_blocks: a reference segment of a fold, its
 * buffers and its device error word. */
typedef struct {
  const float* ffa_fold;   /* segment rows of this job's FFA fold */
  int64_t seg_stride;      /* floats between segments */
  int64_t seed_n;          /* parents already in run.trees[0] (leaves, folds, scores) */
  LokiPruneRun run;        /* as for loki_prune_run (circular fields for basis 2 only) */
  int32_t* dev_err;        /* device error word */
} LokiPruneJob;

/* loki_prune_run for njobs jobs at once: one thread block per job runs every
 * level with block barriers between the steps (the same branch, score,
 * select, overflow and emit code), so the whole batch is one launch. Job j's
 * level l uses levels[j * nlevels + l - 1], seg_idx[j * nlevels + l - 1] and
 * thresholds[j * nlevels + l - 1] (host arrays, checked and copied with the
 * jobs into dev_scratch of loki_prune_run_blocks_scratch_bytes bytes).
 * Results, counters and LOKI_DEVERR_* flags per job as loki_prune_run
 * writes them. Taylor and Chebyshev trees (not basis 2). No reference
 * counterpart as one call: it replaces the per-segment loop of
 * prune_dyp_tree (prune.py:696-780) over Pruning.execute. */
int loki_prune_run_blocks(const LokiPruneJob* jobs, int32_t njobs, const LokiPruneLevel* levels,
                          const int32_t* seg_idx, const double* thresholds, int32_t nlevels,
                          const LokiScoreSpec* spec, int64_t max_sugg, int64_t batch_size,
                          void* dev_scratch, int64_t dev_scratch_bytes, void* stream);
int64_t loki_prune_run_blocks_scratch_bytes(int32_t njobs, int32_t nlevels);

/* The same jobs, arguments and results as loki_prune_run_blocks, run level
 * by level over all jobs at once: every step of a level (branch, the two
 * scans, score, select, overflow rule, emit, backtrack history, best leaf
 * and record) is one launch whose blocks cover every job (grid y = job), so
 * a batch costs the launches of a single run and each step spreads over the
 * whole GPU; no host wait, so the enqueue can be captured in a CUDA graph.
 * dev_scratch of loki_prune_run_blocks_scratch_bytes bytes; njobs <= 65535.
 * Taylor and Chebyshev trees, and the circular-orbit tree (basis 2,
 * poly_order 5, the jobs' runs with their circular fields): its level adds
 * the crackle-expansion scan, the batch-ordered child map, the validity
 * compaction and the valid-child batch offsets of loki_prune_run's circular
 * level, each one launch over every job. */
int loki_prune_run_batch(const LokiPruneJob* jobs, int32_t njobs, const LokiPruneLevel* levels,
                         const int32_t* seg_idx, const double* thresholds, int32_t nlevels,
                         const LokiScoreSpec* spec, int64_t max_sugg, int64_t batch_size,
                         void* dev_scratch, int64_t dev_scratch_bytes, void* stream);

/* loki_prune_run_batch in two halves, so that the kernels can be captured
 * in a CUDA graph once and replayed: loki_prune_batch_tables checks the jobs
 * and copies the tables into dev_scratch (host memory is read: not inside a
 * capture) and writes the batch's shape (6 words: nbins, poly_order, largest
 * par_cap, largest child_cap, fourier, circular-orbit tree);
 * loki_prune_batch_enqueue enqueues the kernels
 * over the tables in dev_scratch for that shape. A replay after
 * loki_prune_batch_tables with new jobs of the same count, levels and shape
 * runs the new jobs. fourier != 0: complex (Fourier-domain) trees, the
 * jobs' tree folds (cap, 2, nbins / 2 + 1) complex64, fold rows and
 * seg_stride in complex elements (the complex level kernels' per-child code,
 * prune.py:165-332 with PrunePolyTaylorComplexDPFuncts, the Chebyshev
 * counterpart and PruneCircTaylorComplexDPFuncts). */
int loki_prune_batch_tables(const LokiPruneJob* jobs, int32_t njobs,
                            const LokiPruneLevel* levels, const int32_t* seg_idx,
                            const double* thresholds, int32_t nlevels,
                            const LokiScoreSpec* spec, int64_t max_sugg, int64_t batch_size,
                            int32_t fourier, void* dev_scratch, int64_t dev_scratch_bytes,
                            int64_t* shape_out, void* stream);
int loki_prune_batch_enqueue(void* dev_scratch, int32_t njobs, int32_t nlevels,
                             const LokiScoreSpec* spec, int64_t max_sugg, int64_t batch_size,
                             const int64_t* shape_in, void* stream);

/* loki_prune_batch_enqueue with CUDA events around every level's score
 * launch; waits for the stream and writes the score kernel's time of each
 * level (ms) to score_ms (host, nlevels). For measurement. */
int loki_prune_batch_score_times(void* dev_scratch, int32_t njobs, int32_t nlevels,
                                 const LokiScoreSpec* spec, int64_t max_sugg,
                                 int64_t batch_size, const int64_t* shape_in, float* score_ms,
                                 void* stream);

/* One job of loki_prune_seed_batch: the seed tree of a run (the
 * reference segment's n grid points, core/taylor.py:14-65 seeds): its leaves
 * and fold rows are copied into the run's first tree and scored. */
typedef struct {
  const double* seed_leaves;  /* n x (poly_order + 2) x 2 */
  const float* fold_rows;     /* n x 2 x nbins: the reference segment of the FFA fold */
  int64_t n;
  double* leaves_out;
  float* folds_out;
  float* scores_out;
  float* scores_ep_out;
  float* seed_scores_out;     /* the level-0 record */
  int32_t* bt_out;            /* n x (poly_order + 2), cleared */
  int32_t* dev_err;           /* cleared */
} LokiSeedJob;

/* The seeds of njobs runs in one launch (grid y = job); jobs (host array)
 * are checked and copied into dev_scratch of at least
 * njobs * sizeof(LokiSeedJob) bytes. */
int loki_prune_seed_batch(const LokiSeedJob* jobs, int32_t njobs, int32_t nbins,
                          int32_t poly_order, const LokiScoreSpec* spec, void* dev_scratch,
                          int64_t dev_scratch_bytes, void* stream);

/* One job of loki_prune_ascend_batch: the ascend of loki_prune_ascend_dev
 * (its level descriptor, final tree, device survivor count and per-segment
 * tables) for one run. */
typedef struct {
  LokiPruneLevel lvl;
  const double* leaves;
  float* folds;
  float* scores;
  float* scores_ep;
  const int64_t* n_dev;    /* survivors (device), <= n_cap */
  const double* tm_seg;
  const double* dt_seg;
  const int32_t* seg_idx;
  const float* ffa_fold;
  int64_t seg_stride;
  int32_t* dev_err;
} LokiAscendJob;

/* loki_prune_ascend_dev for njobs runs in one launch (grid y = job): the
 * jobs (host array) are checked and copied into dev_scratch of at least
 * njobs * sizeof(LokiAscendJob) bytes. Every job has nseg segments and at
 * most n_cap survivors. Taylor, Chebyshev and circular-orbit trees;
 * fourier != 0: complex trees as loki_prune_ascend_complex (folds and
 * seg_stride in complex elements). */
int loki_prune_ascend_batch(const LokiAscendJob* jobs, int32_t njobs, int32_t nseg,
                            const LokiScoreSpec* spec, int64_t n_cap, int32_t fourier,
                            void* dev_scratch, int64_t dev_scratch_bytes, void* stream);

/* A device byte range and its place in a packed destination. */
typedef struct {
  const void* src;
  int64_t bytes;
  int64_t dst_off;
} LokiGatherPart;

/* Copy every part into dst (device, dst_bytes) at its offset in one launch
 * (the parts, a host array, are checked and copied into dev_scratch of at
 * least nparts * sizeof(LokiGatherPart) bytes): many small device ranges
 * become one packed buffer for a single device-to-host copy. */
int loki_gather_parts(const LokiGatherPart* parts, int32_t nparts, void* dst, int64_t dst_bytes,
                      void* dev_scratch, int64_t dev_scratch_bytes, void* stream);

/* Best leaf of a tree (utils/world_tree.py:441-459 get_best_k with k = 1):
 * the leaf row (row_len float64) and score of the maximum score, first index
 * on ties; nothing is written for n = 0. */
int loki_prune_best(const float* scores, int64_t n, const double* leaves, int32_t row_len,
                    double* leaf_out, float* score_out, void* stream);

/* Scratch bytes for the internal scans over n elements. */
int64_t loki_scan_scratch_bytes(int64_t n);

/* ---- scoring ---------------------------------------------------------- */

/* Boxcar S/N of normalised profiles (nprof, nbins) -> (nprof, nwidths) or
 * (nprof,) in mode 1. Replaces boxcar_snr_2d / boxcar_snr_1d
 * (detection/scoring.py:99-153). */
int loki_boxcar_snr(const float* profiles, int64_t nprof, int32_t nbins,
                    const LokiScoreSpec* spec, float* snr, void* stream);

/* Score of (n, 2, nbins) folds: boxcar S/N of e / sqrt(v), max over widths
 * (detection/scoring.py:249-282 snr_score_batch_func). spec->mode is ignored. */
int loki_snr_score_batch(const float* folds, int64_t n, int32_t nbins,
                         const LokiScoreSpec* spec, float* scores, void* stream);

/* Normalised profiles out[p, j] = folds[p, 0, j] / sqrt(folds[p, 1, j]) for
 * (n, 2, nbins) folds. Replaces get_fold_norm (ffa.py:382-411, real case). */
int loki_fold_norm(const float* folds, int64_t n, int32_t nbins, float* out,
                   void* stream);

/* ---- threshold-scheme design (Monte-Carlo folds) ------------------------ */

/* simulate_folds + fold_max_scores (detection/thresholding.py:46-96, 484-500)
 * for nrows rows at once: folds_out[r] = folds_in[src_row[r]] (zeros when
 * folds_in is NULL) + bias[r] * profile + N(0, noise_std^2) per bin, from a
 * Philox-4x32-10 stream keyed by seed and (r, bin); scores[r] = max over the
 * spec's widths of the boxcar S/N of folds_out[r] / sqrt_var (float32
 * division, as prune_folds normalises, thresholding.py:99-135). spec->mode
 * must be 1. */
int loki_sim_score_folds(const float* folds_in, const int64_t* src_row, const float* bias,
                         int64_t nrows, const float* profile, int32_t nbins, float noise_std,
                         float sqrt_var, uint64_t seed, const LokiScoreSpec* spec,
                         float* folds_out, float* scores, void* stream);

/* dst[i] = src[idx[i]] for n rows of row_len float32 (survivor compaction). */
int loki_gather_rows(const float* src, const int64_t* idx, int64_t n, int64_t row_len,
                     float* dst, void* stream);

/* ---- learned branch proposal (tensor cores) ----------------------------
 * A 16 -> 128 -> 128 -> 1 MLP (ReLU) scoring per-branch statistics of the
 * pruning tree. No reference counterpart: the reference has no learned
 * part; these entry points back the optional branch-survival model. */
#define LOKI_MLP_FEATURES 16
#define LOKI_MLP_HIDDEN 128

/* Device pointers. Weights bfloat16 in (out, in) layout: w1 (128, 16),
 * w2 (128, 128), w3 (128,); biases float32: b1 (128,), b2 (128,), b3 (1,). */
typedef struct {
  const void* w1;
  const float* b1;
  const void* w2;
  const float* b2;
  const void* w3;
  const float* b3;
} LokiMLP;

/* Device float32 gradient sums with the shapes of LokiMLP, plus the loss sum.
 * loki_mlp_backward adds to them (the caller zeroes them per step). */
typedef struct {
  float* w1;
  float* b1;
  float* w2;
  float* b2;
  float* w3;
  float* b3;
  float* loss;
} LokiMLPGrad;

/* Shared memory one MLP block uses (bytes). */
int64_t loki_mlp_smem_bytes(void);

/* Test hook for the bounded tensor-core waits of the MLP kernels: with on != 0
 * (current device) every completed MMA wait is treated as expired, so the
 * kernels take their timeout path (tensor memory freed, LOKI_DEVERR_TIMEOUT in
 * the error word) with nothing left in flight; 0 restores normal operation.
 * Synchronous. No reference counterpart (error-path testing only). */
int loki_mlp_force_timeout(int32_t on);

/* logits[i] for features x (n, 16) float32 (rounded to bfloat16 on load). */
int loki_mlp_forward(const LokiMLP* w, const float* x, int64_t n, float* logits,
                     int32_t* dev_err, void* stream);

/* Forward plus backward of the weighted binary cross-entropy with logits,
 * scale * sum_i wt[i] * (softplus(z_i) - y_i z_i) (wt NULL: all ones): adds the
 * loss and the parameter gradients to grad; logits, if not NULL, receives z. */
int loki_mlp_backward(const LokiMLP* w, const float* x, const float* y, const float* wt,
                      int64_t n, float scale, const LokiMLPGrad* grad, float* logits,
                      int32_t* dev_err, void* stream);

/* Branch statistics of n pruning-tree parents into features (n, 16) float32
 * (16-byte aligned): scores (n,), folds (n, 2, nbins) float32; thresholds the
 * parents passed and their children face; level / levels; 1 / sqrt(level + 1);
 * score_stats = device (mean, std) of the scores. */
int loki_branch_features(const float* scores, const float* folds, int64_t n, int32_t nbins,
                         float thr_prev, float thr_next, float level_frac,
                         float inv_sqrt_level, const float* score_stats, float* features,
                         void* stream);

/* One Adam step over n float32 parameters (bias-corrected, step >= 1). */
int loki_mlp_adam(float* params, const float* grads, float* m, float* v, int64_t n, float lr,
                  float beta1, float beta2, float eps, int64_t step, void* stream);

/* ---- synthetic pulsar series (injection generator) -----------------------
 * PulseSignalConfig.generate (simulation/pulse.py:310-406) for many
 * injections at once: proper time of a modulation model
 * (simulation/modulate.py), a CDF-lookup pulse template
 * (generate_pulse_template, pulse.py:38-68), white noise, the calibration
 * folds at the pulse period and the S/N calibration on those folds
 * (calibrate_scale_on_folds, pulse.py:71-118). */
#define LOKI_MOD_MAX_COEFFS 16
#define LOKI_MOD_DERIVATIVE 0  /* c = shift, vel, acc, jerk, snap (m / s^k) */
#define LOKI_MOD_SERIES 1      /* c[k] = d^(k) / k! for k < ncoeff */
#define LOKI_MOD_CIRCULAR 2    /* c = x_orb (lt-s), omega (rad/s), psi (rad) */
#define LOKI_MOD_CIRCULAR_T0 3 /* c = a, omega (rad/s), phi (rad) */
#define LOKI_MOD_KEPLERIAN 4   /* c = p_orb, |ecc|, phi, a (1-ecc^2), aop, sin(inc),
                                  sqrt((1+ecc)/(1-ecc)), 1 / p_orb */
#define LOKI_MOD_TABLE 5       /* proper times read from a device table */
#define LOKI_PULSE_MAX_NBINS 12288 /* calibration fold bins (shared-memory bound) */

typedef struct {
  int32_t kind;   /* LOKI_MOD_* */
  int32_t ncoeff; /* used terms of c (LOKI_MOD_SERIES) */
  double t_ref;   /* reference epoch (s) */
  double c[LOKI_MOD_MAX_COEFFS];
} LokiModulation;

/* One injection. Sample i is at t = i * dt; its proper time comes from mod
 * (or pt_table[inj * nsamps + i] for LOKI_MOD_TABLE). */
typedef struct {
  double dt;        /* sample spacing (s) */
  double period;    /* pulse period (s) */
  double snr;       /* target folded S/N */
  double ducy;      /* duty cycle (on-pulse window of the calibration) */
  double phi0;      /* pulse phase */
  int32_t nbins;    /* calibration fold bins, int(period / dt) */
  int32_t ngrid;    /* CDF table intervals; the table holds ngrid + 1 values */
  int64_t lut_off;  /* offset of this injection's CDF table in luts */
  uint64_t seed;    /* noise stream */
  LokiModulation mod;
} LokiPulseSpec;

/* specs: device array of ninj LokiPulseSpec. luts: float32 CDF tables.
 * pt_table: float64 (ninj, nsamps) proper times, or NULL when no spec is
 * LOKI_MOD_TABLE. noise: float32 (ninj, nsamps) standard normals, or NULL to
 * draw them from each spec's seed (Philox-4x32-10, Box-Muller). */

/* Template (ninj, nsamps) float32 and, if proper_time is not NULL, the
 * proper times (ninj, nsamps) float64. */
int loki_pulse_template(const LokiPulseSpec* specs, int32_t ninj, int64_t nsamps,
                        const float* luts, const double* pt_table, float* tmpl,
                        double* proper_time, void* stream);

/* Calibration folds (ninj, 3, fold_stride) float64, overwritten by the call:
 * [0] sum of noise, [1] samples per bin (unit variance), [2] sum of template,
 * binned by get_phase_idx_int (utils/psr_utils.py:50-56) at 1 / period.
 * Sums are exact in 2^-32 fixed point (independent of summation order;
 * caller noise must stay below 2^20 in magnitude). noise_out and tmpl_out
 * (both or neither, (ninj, nsamps) float32) receive the unit noise and the
 * template for loki_pulse_apply. */
int loki_pulse_fold(const LokiPulseSpec* specs, int32_t ninj, int64_t nsamps,
                    const float* luts, const double* pt_table, const float* noise,
                    double* folds, int32_t fold_stride, float* noise_out, float* tmpl_out,
                    void* stream);

/* Noise scale and calibrated signal scale per injection from the folds
 * (ninj, 3, fold_stride) float64, rounded to float32 as the reference holds them:
 * out (ninj, 4) float64 = noise_scale, signal scale, template S/N, last
 * measured S/N. Stops when |S/N - snr| < tol or after max_iter steps. */
int loki_pulse_calibrate(const LokiPulseSpec* specs, int32_t ninj, const double* folds,
                         int32_t fold_stride, int32_t max_iter, double tol, double* out,
                         void* stream);

/* In place on the noise_out / tmpl_out arrays of loki_pulse_fold:
 * ts_e = noise_scale * noise + scale * template, ts_v = noise_scale^2
 * (float32 arithmetic, as pulse.py:402-405), scales from loki_pulse_calibrate. */
int loki_pulse_apply(const double* scales, int32_t ninj, int64_t nsamps, float* ts_e,
                     float* ts_v, void* stream);

/* The same series as fold + calibrate + apply, regenerating noise and
 * template instead of reading them back (no (ninj, nsamps) buffers needed
 * before the scales are known). */
int loki_pulse_emit(const LokiPulseSpec* specs, int32_t ninj, int64_t nsamps,
                    const float* luts, const double* pt_table, const float* noise,
                    const double* scales, float* ts_e, float* ts_v, void* stream);

/* TimeSeries.fold_ephem (io/timeseries.py:45-83): the series folded at freq
 * over the proper times of mod (t = i dt; pt_table for LOKI_MOD_TABLE) into
 * fold (nsubints, 2, nbins) float32, each (subint, bin) summed in sample
 * order as core/fold.py:57-105 brutefold does (bit-identical); norm
 * (nsubints, nbins), if not NULL, = e / sqrt(v), or 0 where |v| <= 1e-5.
 * bins: nsamps uint32 scratch. Trailing samples past nsubints whole
 * subints are not folded. */
int loki_fold_ephem(const float* ts_e, const float* ts_v, int64_t nsamps, double dt,
                    const LokiModulation* mod, const double* pt_table, double freq,
                    int32_t nbins, int32_t nsubints, uint32_t* bins, float* fold, float* norm,
                    void* stream);

/* Mean of each group of factor samples, n / factor outputs
 * (utils/np_utils.py:119-122 downsample_1d). */
int loki_downsample(const float* x, int64_t n, int32_t factor, float* out, void* stream);

/* ---- series conditioning (io/timeseries.py:198-236 TimeSeries.from_tim) ---
 * from_tim dereddens the series with sigpyproc's median filter and
 * normalises it with sigpyproc's location and scale estimates. sigpyproc is
 * a git dependency of the reference (pyproject.toml:41) outside its tree, so
 * the steps are defined here:
 * loki_running_median: out[i] = the order statistic of rank window / 2 of
 * x[i - window/2 .. i - window/2 + window - 1] with half-sample symmetric
 * reflection at the ends (scipy.ndimage.median_filter, mode "reflect"), or
 * x[i] minus it when subtract != 0. 1 <= window <= 32768; x finite (no NaN).
 * No allocation. */
int loki_running_median(const float* x, int64_t n, int32_t window, int32_t subtract,
                        float* out, void* stream);

/* k-th smallest element (0-based) of x into *out (device), by a radix select
 * over the float order; scratch of loki_select_scratch_bytes() device bytes. */
int loki_select_kth(const float* x, int64_t n, int64_t k, float* out, void* scratch,
                    int64_t scratch_bytes, void* stream);
int64_t loki_select_scratch_bytes(void);

/* Sum of x (square == 0) or of x^2 (square != 0) accumulated in float64 into
 * *out (device); scratch of at least min(ceil(n / 256), 1024) doubles. */
int loki_sum_f64(const float* x, int64_t n, int32_t square, double* out, void* scratch,
                 int64_t scratch_bytes, void* stream);

/* y = (x - loc) / scale in float32, or y = |x - loc| when scale == 0 (the
 * absolute deviations of a median-absolute-deviation scale). */
int loki_affine(const float* x, int64_t n, float loc, float scale, float* y, void* stream);

/* ---- alternative profile scorers (detection/scoring.py) ------------------
 * None of these is on a search path of the reference; they score candidate
 * profiles (n, nbins) float32 on request. */

/* kadane_circular_normalized_1d (scoring.py:675-755) per profile: the best
 * mean-subtracted circular window over the biases, float64, with its width
 * and start. Bit-identical to the reference. */
int loki_kadane_circular(const float* profiles, int64_t n, int32_t nbins, const float* biases,
                         int32_t nbias, double* snr, int64_t* width, int64_t* start,
                         void* stream);

/* The matched-filter bank (MatchedFilter + compute_snr_e_mat_2d,
 * scoring.py:295-357,491-524): e_mat (nfilt, nbins) holds, per template,
 * shifts_per_template circularly shifted rows; snr (n, nfilt /
 * shifts_per_template) = max projection / stdnoise; projections (n, nfilt)
 * is optional (NULL: not written). */
int loki_matched_filter(const float* profiles, int64_t n, int32_t nbins, const float* e_mat,
                        int32_t nfilt, int32_t shifts_per_template, float stdnoise, float* snr,
                        float* projections, void* stream);

/* MatchedFilter.compute_fft (_compute_snr_fft, scoring.py:527-558): per
 * (profile, template) the max over the first nbins lags of the circular
 * convolution of the profile, circularly padded to the next power of two,
 * with the zero-padded template (ntemp, nbins). out (n, ntemp). */
int loki_matched_filter_conv(const float* profiles, int64_t n, int32_t nbins,
                             const float* templates, int32_t ntemp, float* out, void* stream);

/* _compute_snr_double (scoring.py:561-627): per profile, the larger of the
 * single-filter and the best two-filter chi-square score among the n_corr
 * largest projections, less its look-elsewhere penalty, mapped to a normal
 * S/N. inner = e_mat e_mat^T (nfilt, nfilt). chi_table is the
 * (df_max + 2, nchi) table of -log sf of chi-square (utils/maths.py:61-77,
 * a zero row appended), isf_table the normal ISF of exp(-x): the reference's
 * nisf entries plus the last repeated once (nisf + 1 values). */
int loki_matched_filter_double(const float* profiles, int64_t n, int32_t nbins,
                               const float* e_mat, int32_t nfilt, const float* inner,
                               int32_t n_corr, const double* chi_table, int32_t nchi,
                               double chi_res, double chi_max, const double* isf_table,
                               int32_t nisf, double isf_res, double isf_max, float* out,
                               void* stream);

/* harmonic_summing_score_func (scoring.py:630-642) per fold (n, 2, nbins):
 * cumulative power of harmonics 1..n_harmonics of e / sqrt(v), best
 * chi-square score over the prefix, as a normal S/N (float64). chi_rows =
 * rows of chi_table; tables as for loki_matched_filter_double. */
int loki_harmonic_sum(const float* folds, int64_t n, int32_t nbins, int32_t n_harmonics,
                      const double* chi_table, int32_t chi_rows, int32_t nchi, double chi_res,
                      double chi_max, const double* isf_table, int32_t nisf, double isf_res,
                      double isf_max, double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* LOKI_GB300_H */
