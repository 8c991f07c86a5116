// FP64 re-scoring of FFA candidates.
//
// A candidate is one parameter set of an FFA level (one segment). Its fold is
// the sum, over the level-0 segments below it, of each segment's brute fold
// at the level-0 frequency that the resolves along the path select
// (dynamic/dyn_pffa.py:462-489, core/fold.py:617-671), rolled by the sum of
// the rounded shifts met on the way down: at level l the shift-add writes
// o[j] = t[(j - s_t) mod nbins] + h[(j - s_h) mod nbins] (core/common.py:
// 304-324), and rolls compose by adding their shifts. The kernel walks every
// path with the same FP64 resolve as the level kernels, folds each level-0
// segment's samples straight from the series with the brute fold's FP64
// phase bins (core/fold.py:108-171), sums everything in FP64, and scores the
// FP64 profile with the boxcar S/N of detection/scoring.py:99-140 in FP64.
//
// This is what keeps reduced-precision fold storage honest: the DP levels may
// store bfloat16, but the S/N reported for retained candidates is recomputed
// here from the samples with FP64 sums.
#include <algorithm>

#include "loki_common.cuh"

namespace loki {

constexpr int kRescoreThreads = 256;
constexpr int kRescoreChunk = 256;  // leaves resolved per pass

struct LevelChain {
  LokiFFALevel L[LOKI_MAX_RESCORE_LEVELS];  // L[l - 1] describes level l
};

struct SeriesArgs {
  const float* ts_e;
  const float* ts_v;
  int64_t nsamps;
  int64_t bseg;
  double tsamp;
  double t_ref;
  const double* freqs0;  // level-0 frequency grid
};

__global__ void __launch_bounds__(kRescoreThreads)
rescore_kernel(const LevelChain C, int nlev, const SeriesArgs A,
               const int64_t* __restrict__ cand, const int64_t* __restrict__ segs,
               int64_t ncand, int64_t Qtop, int64_t seg_default, int64_t nseg_top,
               LokiScoreSpec sp, double* __restrict__ snr, double* __restrict__ prof) {
  extern __shared__ double sm[];
  const int n = C.L[0].nparams;
  const int nb = C.L[0].nbins;
  const int W = 2 * nb;
  double* acc = sm;                                   // W: e bins then v bins
  double* pre = acc + W;                              // nb + wmax
  double* lfreq = pre + nb + sp.wmax;                 // chunk
  int64_t* lseg = reinterpret_cast<int64_t*>(lfreq + kRescoreChunk);  // chunk
  int* lshift = reinterpret_cast<int*>(lseg + kRescoreChunk);          // chunk
  const int64_t nleaf = 1LL << nlev;
  const LokiFFALevel& top = C.L[nlev - 1];
  for (int64_t c = blockIdx.x; c < ncand; c += gridDim.x) {
    const int64_t q = cand[c];
    const int64_t seg = segs ? segs[c] : seg_default;
    if (q < 0 || q >= Qtop || seg < 0 || seg >= nseg_top) {  // not a trial: NaN, no access
      for (int iw = threadIdx.x; iw < sp.nwidths; iw += blockDim.x)
        snr[(size_t)c * sp.nwidths + iw] = NAN;
      if (prof)
        for (int j = threadIdx.x; j < W; j += blockDim.x) prof[(size_t)c * W + j] = NAN;
      continue;
    }
    int64_t idx_top[LOKI_MAX_PARAMS];
    {
      int64_t rest = q;
      for (int d = n - 1; d >= 0; --d) {
        idx_top[d] = rest % top.counts_cur[d];
        rest /= top.counts_cur[d];
      }
    }
    for (int k = threadIdx.x; k < W; k += blockDim.x) acc[k] = 0.0;
    for (int64_t base = 0; base < nleaf; base += kRescoreChunk) {
      const int cn = (int)min((int64_t)kRescoreChunk, nleaf - base);
      for (int k = threadIdx.x; k < cn; k += blockDim.x) {
        const int64_t leaf = base + k;
        int64_t idx[LOKI_MAX_PARAMS];
        for (int d = 0; d < n; ++d) idx[d] = idx_top[d];
        int shift = 0;
        for (int l = nlev; l >= 1; --l) {
          const LokiFFALevel& L = C.L[l - 1];
          double pset[LOKI_MAX_PARAMS];
          for (int d = 0; d < n; ++d) pset[d] = L.param_arr[d][idx[d]];
          const int latter = (int)((leaf >> (l - 1)) & 1);
          const double ph = ffa_resolve(pset, n, l, latter, L.tseg_brute, nb, L.counts_prev,
                                        L.limits, idx);
          shift += round_shift(ph, nb);
        }
        lfreq[k] = A.freqs0[idx[n - 1]];  // level 0 has one value in every other dim
        lseg[k] = (seg << nlev) + leaf;
        lshift[k] = shift % nb;
      }
      __syncthreads();
      for (int k = 0; k < cn; ++k) {
        const double f = lfreq[k];
        const int sft = lshift[k];
        const int64_t start = lseg[k] * A.bseg;
        const int64_t len = min(A.bseg, A.nsamps - start);
        for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
          const double pt = __dsub_rn(__dmul_rn((double)i, A.tsamp), A.t_ref);
          int b = round_shift(phase_idx(pt, f, nb, 0.0), nb) + sft;
          if (b >= nb) b -= nb;
          atomicAdd(acc + b, (double)__ldg(A.ts_e + start + i));
          atomicAdd(acc + nb + b, (double)__ldg(A.ts_v + start + i));
        }
      }
      __syncthreads();
    }
    if (prof)
      for (int j = threadIdx.x; j < W; j += blockDim.x) prof[(size_t)c * W + j] = acc[j];
    if (threadIdx.x == 0) {
      // circular prefix of e / sqrt(v) (detection/scoring.py:42-71), FP64
      double run = 0.0;
      for (int j = 0; j < nb; ++j) {
        run += acc[j] / sqrt(acc[nb + j]);
        pre[j] = run;
      }
      for (int i = nb; i < nb + sp.wmax; ++i)
        pre[i] = pre[i % nb] + (double)(i / nb) * run;
    }
    __syncthreads();
    for (int iw = threadIdx.x; iw < sp.nwidths; iw += blockDim.x) {
      const int w = sp.widths[iw];
      double dmax = -INFINITY;
      for (int i = 0; i < nb; ++i) dmax = fmax(dmax, pre[i + w] - pre[i]);
      snr[(size_t)c * sp.nwidths + iw] =
          (sp.hb[iw] * dmax - sp.b[iw] * pre[nb - 1]) * sp.inv_stdnoise;
    }
    __syncthreads();
  }
}

static int rescore_smem(int nbins, int wmax) {
  return (int)((size_t)(3 * nbins + wmax) * sizeof(double) +
               kRescoreChunk * (sizeof(double) + sizeof(int64_t) + sizeof(int)));
}

}  // namespace loki

using namespace loki;

extern "C" int loki_ffa_rescore(const LokiFFALevel* levels, int32_t nlevels, const float* ts_e,
                                const float* ts_v, int64_t nsamps, double tsamp,
                                int64_t bseg_brute, const double* freqs0, int64_t nfreq0,
                                const int64_t* cand, const int64_t* segs, int64_t ncand,
                                int64_t seg, const LokiScoreSpec* spec, double* snr,
                                double* prof, void* stream) {
  if (!levels || !ts_e || !ts_v || !freqs0 || !cand || !spec || !snr)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (nlevels < 1 || nlevels > LOKI_MAX_RESCORE_LEVELS)
    return set_error(LOKI_ERR_INVALID, "nlevels %d outside 1..%d", nlevels,
                     LOKI_MAX_RESCORE_LEVELS);
  if (ncand < 0 || seg < 0 || nsamps < 1 || bseg_brute < 1 || !(tsamp > 0.0))
    return set_error(LOKI_ERR_INVALID, "bad sizes");
  const int n = levels[0].nparams, nb = levels[0].nbins;
  if (n < 1 || n > LOKI_MAX_PARAMS || nb < 2 || nb > 1024)
    return set_error(LOKI_ERR_INVALID, "nparams or nbins out of range");
  for (int l = 0; l < nlevels; ++l) {
    const LokiFFALevel& L = levels[l];
    if (L.level != l + 1 || L.nparams != n || L.nbins != nb)
      return set_error(LOKI_ERR_INVALID, "levels[%d] is not level %d of one search", l, l + 1);
    for (int d = 0; d < n; ++d) {
      if (!L.param_arr[d] || L.counts_cur[d] < 1 || L.counts_prev[d] < 1)
        return set_error(LOKI_ERR_INVALID, "levels[%d] has an empty grid", l);
      if (l > 0 && L.counts_prev[d] != levels[l - 1].counts_cur[d])
        return set_error(LOKI_ERR_INVALID, "levels %d and %d do not chain", l, l + 1);
    }
  }
  for (int d = 0; d < n - 1; ++d)
    if (levels[0].counts_prev[d] != 1)
      return set_error(LOKI_ERR_INVALID, "level 0 must hold one value in every non-frequency "
                                         "dimension");
  if (levels[0].counts_prev[n - 1] != nfreq0)
    return set_error(LOKI_ERR_INVALID, "freqs0 does not match the level-0 grid");
  if (spec->nwidths < 1 || spec->nwidths > LOKI_MAX_WIDTHS || spec->wmax < 1)
    return set_error(LOKI_ERR_INVALID, "bad score spec");
  for (int i = 0; i < spec->nwidths; ++i)
    if (spec->widths[i] < 1 || spec->widths[i] > spec->wmax)
      return set_error(LOKI_ERR_INVALID, "score width outside 1..wmax");
  // segments of the last level whose level-0 segments all exist
  const int64_t nseg0 = (nsamps + bseg_brute - 1) / bseg_brute;
  const int64_t nseg_top = nseg0 >> nlevels;
  if (!segs && seg >= nseg_top)
    return set_error(LOKI_ERR_INVALID, "segment %lld needs level-0 segments beyond %lld",
                     (long long)seg, (long long)nseg0);
  if (ncand == 0) return LOKI_OK;
  int64_t Qtop = 1;
  for (int d = 0; d < n; ++d) Qtop *= levels[nlevels - 1].counts_cur[d];
  LevelChain C;
  for (int l = 0; l < nlevels; ++l) C.L[l] = levels[l];
  SeriesArgs A;
  A.ts_e = ts_e;
  A.ts_v = ts_v;
  A.nsamps = nsamps;
  A.bseg = bseg_brute;
  A.tsamp = tsamp;
  A.t_ref = n == 1 ? 0.0 : (double)bseg_brute * tsamp / 2.0;  // ffa.py t_ref of the brute fold
  A.freqs0 = freqs0;
  const int smem = rescore_smem(nb, spec->wmax);
  if (smem > 48 * 1024 && set_smem_limit(rescore_kernel, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  const unsigned grid = (unsigned)std::min<int64_t>(ncand, 152 * 8);
  note_launch();
  rescore_kernel<<<grid, kRescoreThreads, smem, (cudaStream_t)stream>>>(
      C, nlevels, A, cand, segs, ncand, Qtop, seg, nseg_top, *spec, snr, prof);
  return check_launch("ffa_rescore");
}
