// FFA kernels: brute fold, per-level plan, DP level, fused final level+score.
//
// Data layout in HBM (identical to pyloki): fold (nseg, P, 2, nbins) float32,
// C-contiguous, P = flattened parameter grid with the frequency axis fastest.
#include <algorithm>

#include "loki_common.cuh"
#include "score.cuh"

namespace loki {

// ---------------------------------------------------------------------------
// Brute fold (core/fold.py:108-171 brutefold_start)
// ---------------------------------------------------------------------------

// Phase-bin map of one segment: map[f][i] = get_phase_idx_int(i*tsamp - t_ref,
// freq[f], nbins, 0). Depends only on (freq, sample-in-segment), so one map
// serves every segment (and every series with the same grid).
template <typename T>
__global__ void phase_map_kernel(const double* __restrict__ freqs, int64_t nfreq,
                                 int64_t seg_len, int nbins, double tsamp,
                                 double t_ref, T* __restrict__ map) {
  const int64_t total = nfreq * seg_len;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = k / seg_len;
    const int64_t i = k - f * seg_len;
    const double pt = __dsub_rn(__dmul_rn((double)i, tsamp), t_ref);
    map[k] = (T)round_shift(phase_idx(pt, freqs[f], nbins, 0.0), nbins);
  }
}

// One warp per (segment, frequency). Samples are consumed in chunks of 32 in
// time order; inside a chunk the lanes that hit the same bin are ranked by
// lane index (match_any + popc) and added rank by rank, so every bin receives
// its samples in exactly the sequential order of the reference loop.
// Accumulators live in shared memory (2 * nbins floats per warp).
template <typename T, int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
brutefold_kernel(const float* __restrict__ ts_e, const float* __restrict__ ts_v,
                 int64_t nsamps, const T* __restrict__ map, int64_t nfreq_chunk,
                 int64_t f_offset, int64_t nfreq_total, int64_t seg_len,
                 int64_t nseg, int nbins, float* __restrict__ fold) {
  extern __shared__ float acc_all[];
  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t seg = blockIdx.x % nseg;
  const int64_t fi = (blockIdx.x / nseg) * WARPS + warp;
  float* acc_e = acc_all + (size_t)warp * 2 * nbins;
  float* acc_v = acc_e + nbins;
  for (int j = lane; j < 2 * nbins; j += 32) acc_e[j] = 0.0f;
  __syncwarp();
  if (fi >= nfreq_chunk) return;
  const int64_t start = seg * seg_len;
  const int64_t len = std::min<int64_t>(seg_len, nsamps - start);
  const T* mrow = map + fi * seg_len;
  const float* se = ts_e + start;
  const float* sv = ts_v + start;
  const unsigned lt = lanemask_lt();
  for (int64_t base = 0; base < len; base += 32) {
    const int64_t i = base + lane;
    const bool valid = i < len;
    const unsigned bin = valid ? (unsigned)mrow[i] : 0xFFFFFFFFu;
    const float e = valid ? se[i] : 0.0f;
    const float v = valid ? sv[i] : 0.0f;
    const unsigned peers = __match_any_sync(0xFFFFFFFFu, bin);
    const int rank = __popc(peers & lt);
    const int maxrank = (int)__reduce_max_sync(0xFFFFFFFFu, valid ? (unsigned)rank : 0u);
    for (int r = 0; r <= maxrank; ++r) {
      if (valid && rank == r) {
        acc_e[bin] = __fadd_rn(acc_e[bin], e);
        acc_v[bin] = __fadd_rn(acc_v[bin], v);
      }
      __syncwarp();
    }
  }
  float* out = fold + ((size_t)seg * nfreq_total + f_offset + fi) * 2 * nbins;
  for (int j = lane; j < 2 * nbins; j += 32) out[j] = acc_e[j];
}

// ---------------------------------------------------------------------------
// Plan / level helpers
// ---------------------------------------------------------------------------

struct Resolved {
  int64_t in_tail;  // flattened index into fold_in's parameter axis (window applied)
  int64_t in_head;
  double ph_tail;
  double ph_head;
  bool ok;
};

// Decompose output parameter q of the (windowed) current grid into values.
__device__ __forceinline__ void out_param(const LokiFFALevel& L, int64_t q, double* pset) {
  const int n = L.nparams;
  int64_t last = L.out_start + q % L.out_width;
  int64_t rest = q / L.out_width;
  pset[n - 1] = L.param_arr[n - 1][last];
  for (int d = n - 2; d >= 0; --d) {
    const int64_t c = L.counts_cur[d];
    pset[d] = L.param_arr[d][rest % c];
    rest /= c;
  }
}

__device__ __forceinline__ int64_t flat_in(const LokiFFALevel& L, const int64_t* idx,
                                           bool* ok) {
  const int n = L.nparams;
  int64_t flat = 0;
  for (int d = 0; d < n - 1; ++d) flat = flat * L.counts_prev[d] + idx[d];
  const int64_t il = idx[n - 1] - L.in_start;
  if (il < 0 || il >= L.in_width) *ok = false;
  return flat * L.in_width + il;
}

__device__ __forceinline__ Resolved resolve_q(const LokiFFALevel& L, int64_t q) {
  double pset[LOKI_MAX_PARAMS];
  int64_t idx[LOKI_MAX_PARAMS];
  out_param(L, q, pset);
  Resolved r;
  r.ok = true;
  r.ph_tail = ffa_resolve(pset, L.nparams, L.level, 0, L.tseg_brute, L.nbins,
                          L.counts_prev, L.limits, idx);
  r.in_tail = flat_in(L, idx, &r.ok);
  r.ph_head = ffa_resolve(pset, L.nparams, L.level, 1, L.tseg_brute, L.nbins,
                          L.counts_prev, L.limits, idx);
  r.in_head = flat_in(L, idx, &r.ok);
  return r;
}

__host__ __device__ __forceinline__ int64_t n_out_params(const LokiFFALevel& L) {
  int64_t q = L.out_width;
  for (int d = 0; d < L.nparams - 1; ++d) q *= L.counts_cur[d];
  return q;
}

__host__ __device__ __forceinline__ int64_t n_in_params(const LokiFFALevel& L) {
  int64_t q = L.in_width;
  for (int d = 0; d < L.nparams - 1; ++d) q *= L.counts_prev[d];
  return q;
}

__global__ void ffa_plan_kernel(LokiFFALevel L, LokiFFACoord* __restrict__ coords,
                                int32_t* __restrict__ err) {
  const int64_t Q = n_out_params(L);
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < Q;
       q += (int64_t)gridDim.x * blockDim.x) {
    Resolved r = resolve_q(L, q);
    if (!r.ok) atomicOr(err, LOKI_DEVERR_WINDOW);
    LokiFFACoord c;
    c.i_tail = (uint32_t)r.in_tail;
    c.shift_tail = __double2float_rn(r.ph_tail);
    c.i_head = (uint32_t)r.in_head;
    c.shift_head = __double2float_rn(r.ph_head);
    coords[q] = c;
  }
}

// Each warp owns 32 consecutive output parameters: lane k resolves parameter
// k (FP64, once per level), then the warp streams the roll-add of every
// segment pair for the 32 parameters, pair-major so that neighbouring
// parameters (neighbouring frequencies) are read and written together.
__global__ void __launch_bounds__(256)
ffa_level_kernel(LokiFFALevel L, const float* __restrict__ in, float* __restrict__ out,
                 int32_t* __restrict__ err) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t Q = n_out_params(L);
  const int64_t P_in = n_in_params(L);
  const int64_t q0 = gw * 32;
  if (q0 >= Q) return;
  const int nb = L.nbins;
  int64_t my_t = 0, my_h = 0;
  int my_st = 0, my_sh = 0;
  bool my_ok = false;
  if (q0 + lane < Q) {
    Resolved r = resolve_q(L, q0 + lane);
    my_ok = r.ok;
    my_t = r.in_tail;
    my_h = r.in_head;
    my_st = round_shift(r.ph_tail, nb);
    my_sh = round_shift(r.ph_head, nb);
    if (!r.ok) atomicOr(err, LOKI_DEVERR_WINDOW);
  }
  const int kmax = (int)std::min<int64_t>(32, Q - q0);
  const int64_t nseg_out = L.nseg_in / 2;
  const size_t row = (size_t)2 * nb;
  for (int64_t ip = 0; ip < nseg_out; ++ip) {
    const float* in_t = in + (size_t)(2 * ip) * P_in * row;
    const float* in_h = in + (size_t)(2 * ip + 1) * P_in * row;
    float* o_base = out + ((size_t)ip * Q + q0) * row;
    for (int k = 0; k < kmax; ++k) {
      const int64_t it = __shfl_sync(0xFFFFFFFFu, my_t, k);
      const int64_t ih = __shfl_sync(0xFFFFFFFFu, my_h, k);
      const int st = __shfl_sync(0xFFFFFFFFu, my_st, k);
      const int sh = __shfl_sync(0xFFFFFFFFu, my_sh, k);
      const bool ok = __shfl_sync(0xFFFFFFFFu, my_ok, k);
      if (!ok) continue;
      const float* t = in_t + (size_t)it * row;
      const float* h = in_h + (size_t)ih * row;
      float* o = o_base + (size_t)k * row;
      for (int j = lane; j < nb; j += 32) {
        int jt = j - st;
        jt += (jt < 0) ? nb : 0;
        int jh = j - sh;
        jh += (jh < 0) ? nb : 0;
        o[j] = __fadd_rn(t[jt], h[jh]);
        o[nb + j] = __fadd_rn(t[nb + jt], h[nb + jh]);
      }
    }
  }
}

// Final level fused with get_fold_norm and boxcar scoring, segment 0 only.
// Lane k resolves parameter k; the warp builds the 32 normalised profiles in
// its shared tile, then lane k scores row k.
__global__ void __launch_bounds__(128)
ffa_level_score_kernel(LokiFFALevel L, const float* __restrict__ in, LokiScoreSpec sp,
                       float* __restrict__ snr, int32_t* __restrict__ err) {
  extern __shared__ float tiles[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nb = L.nbins;
  const int stride = score_stride(nb, sp.wmax);
  float* tile = tiles + (size_t)warp * 32 * stride;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t Q = n_out_params(L);
  const int64_t P_in = n_in_params(L);
  const int64_t q0 = gw * 32;
  if (q0 >= Q) return;
  int64_t my_t = 0, my_h = 0;
  int my_st = 0, my_sh = 0;
  bool my_ok = false;
  if (q0 + lane < Q) {
    Resolved r = resolve_q(L, q0 + lane);
    my_ok = r.ok;
    my_t = r.in_tail;
    my_h = r.in_head;
    my_st = round_shift(r.ph_tail, nb);
    my_sh = round_shift(r.ph_head, nb);
    if (!r.ok) atomicOr(err, LOKI_DEVERR_WINDOW);
  }
  const int kmax = (int)std::min<int64_t>(32, Q - q0);
  const size_t row = (size_t)2 * nb;
  const float* in_t = in;                      // segment 0 of fold_in
  const float* in_h = in + (size_t)P_in * row;  // segment 1 of fold_in
  for (int k = 0; k < kmax; ++k) {
    const int64_t it = __shfl_sync(0xFFFFFFFFu, my_t, k);
    const int64_t ih = __shfl_sync(0xFFFFFFFFu, my_h, k);
    const int st = __shfl_sync(0xFFFFFFFFu, my_st, k);
    const int sh = __shfl_sync(0xFFFFFFFFu, my_sh, k);
    const bool ok = __shfl_sync(0xFFFFFFFFu, my_ok, k);
    float* trow = tile + k * stride;
    if (!ok) {
      for (int j = lane; j < nb; j += 32) trow[j] = 0.0f;
      continue;
    }
    const float* t = in_t + (size_t)it * row;
    const float* h = in_h + (size_t)ih * row;
    for (int j = lane; j < nb; j += 32) {
      int jt = j - st;
      jt += (jt < 0) ? nb : 0;
      int jh = j - sh;
      jh += (jh < 0) ? nb : 0;
      const float e = __fadd_rn(t[jt], h[jh]);
      const float v = __fadd_rn(t[nb + jt], h[nb + jh]);
      trow[j] = __fdiv_rn(e, __fsqrt_rn(v));
    }
  }
  __syncwarp();
  if (lane < kmax) {
    // Output row = full-grid flattened index of this parameter set, so that a
    // frequency window writes its rows in place in the (P_full, nout) array.
    const int64_t q = q0 + lane;
    const int64_t full = (q / L.out_width) * L.counts_cur[L.nparams - 1] + L.out_start +
                         q % L.out_width;
    const int nout = sp.mode == 0 ? sp.nwidths : 1;
    score_row(tile + lane * stride, nb, sp, snr + (size_t)full * nout);
  }
}

// Previous-level frequency window needed by each band of current-level
// frequencies. The resolved frequency index is monotone in the current
// frequency for fixed other parameters (f_new = f * (1 - v/c)), so a band
// [g0, g1) needs [min idx at g0, max idx at g1 - 1] over every other-parameter
// combination, tail and head. One thread per (band, other combination).
__global__ void ffa_band_window_kernel(LokiFFALevel L, int64_t band_width, int64_t nbands,
                                       unsigned long long* __restrict__ lo,
                                       unsigned long long* __restrict__ hi) {
  const int n = L.nparams;
  int64_t n_other = 1;
  for (int d = 0; d < n - 1; ++d) n_other *= L.counts_cur[d];
  const int64_t nf = L.counts_cur[n - 1];
  const int64_t total = nbands * n_other;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t band = t / n_other;
    const int64_t other = t - band * n_other;
    const int64_t g0 = band * band_width;
    const int64_t g1 = min(g0 + band_width, nf) - 1;
    double pset[LOKI_MAX_PARAMS];
    int64_t idx[LOKI_MAX_PARAMS];
    int64_t rest = other;
    for (int d = n - 2; d >= 0; --d) {
      const int64_t c = L.counts_cur[d];
      pset[d] = L.param_arr[d][rest % c];
      rest /= c;
    }
    int64_t mn = INT64_MAX, mx = -1;
    for (int side = 0; side < 2; ++side) {
      pset[n - 1] = L.param_arr[n - 1][side ? g1 : g0];
      for (int latter = 0; latter < 2; ++latter) {
        ffa_resolve(pset, n, L.level, latter, L.tseg_brute, L.nbins, L.counts_prev,
                    L.limits, idx);
        mn = min(mn, idx[n - 1]);
        mx = max(mx, idx[n - 1]);
      }
    }
    atomicMin(lo + band, (unsigned long long)mn);
    atomicMax(hi + band, (unsigned long long)mx);
  }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------

static int check_level(const LokiFFALevel* L) {
  if (!L) return set_error(LOKI_ERR_INVALID, "null level descriptor");
  if (L->nparams < 1 || L->nparams > LOKI_MAX_PARAMS)
    return set_error(LOKI_ERR_INVALID, "nparams %d out of range", L->nparams);
  if (L->nbins < 2) return set_error(LOKI_ERR_INVALID, "nbins %d < 2", L->nbins);
  if (L->level < 1 || L->level > 62)
    return set_error(LOKI_ERR_INVALID, "level %d out of range", L->level);
  if (L->out_width <= 0 || L->in_width <= 0 || L->out_start < 0 || L->in_start < 0)
    return set_error(LOKI_ERR_INVALID, "empty or negative window");
  const int n = L->nparams;
  if (L->out_start + L->out_width > L->counts_cur[n - 1])
    return set_error(LOKI_ERR_INVALID, "output window beyond the grid");
  if (L->in_start + L->in_width > L->counts_prev[n - 1])
    return set_error(LOKI_ERR_INVALID, "input window beyond the grid");
  for (int d = 0; d < n; ++d) {
    if (!L->param_arr[d]) return set_error(LOKI_ERR_INVALID, "null param_arr[%d]", d);
    if (L->counts_cur[d] < 1 || L->counts_prev[d] < 1)
      return set_error(LOKI_ERR_INVALID, "grid count < 1 in dim %d", d);
  }
  if (L->nseg_in < 2 || (L->nseg_in & 1))
    return set_error(LOKI_ERR_INVALID, "nseg_in %lld must be even and >= 2",
                     (long long)L->nseg_in);
  return LOKI_OK;
}

static int fill_spec_check(const LokiScoreSpec* sp, int nbins) {
  if (!sp) return set_error(LOKI_ERR_INVALID, "null score spec");
  if (sp->nwidths < 1 || sp->nwidths > LOKI_MAX_WIDTHS)
    return set_error(LOKI_ERR_INVALID, "nwidths %d out of range", sp->nwidths);
  int wmax = 0;
  for (int i = 0; i < sp->nwidths; ++i) {
    if (sp->widths[i] < 1) return set_error(LOKI_ERR_INVALID, "width < 1");
    wmax = std::max(wmax, (int)sp->widths[i]);
  }
  if (wmax != sp->wmax) return set_error(LOKI_ERR_INVALID, "wmax != max(widths)");
  if (nbins + wmax > 2048)
    return set_error(LOKI_ERR_UNSUPPORTED, "nbins + wmax = %d above 2048", nbins + wmax);
  return LOKI_OK;
}

int score_smem_bytes(int nbins, int wmax, int warps) {
  return warps * 32 * score_stride(nbins, wmax) * (int)sizeof(float);
}

int score_warps_per_block(int nbins, int wmax) {
  int w = 4;
  while (w > 1 && score_smem_bytes(nbins, wmax, w) > 200 * 1024) w >>= 1;
  return w;
}

}  // namespace loki

using namespace loki;

extern "C" int loki_brutefold(const float* ts_e, const float* ts_v, int64_t nsamps,
                              const double* freqs, int64_t nfreqs, int64_t segment_len,
                              int32_t nbins, double tsamp, double t_ref,
                              void* phase_scratch, int64_t scratch_bytes,
                              float* fold_out, void* stream) {
  if (!ts_e || !ts_v || !freqs || !phase_scratch || !fold_out)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (nsamps <= 0 || nfreqs <= 0 || segment_len <= 0)
    return set_error(LOKI_ERR_INVALID, "nsamps, nfreqs and segment_len must be > 0");
  if (nbins < 1 || nbins > 4096)
    return set_error(LOKI_ERR_UNSUPPORTED, "nbins %d outside [1, 4096]", nbins);
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t nseg = (nsamps + segment_len - 1) / segment_len;
  const int elem = nbins <= 256 ? 1 : 2;
  int64_t chunk = scratch_bytes / (segment_len * elem);
  if (chunk < 1)
    return set_error(LOKI_ERR_CAPACITY, "phase scratch of %lld bytes holds no frequency",
                     (long long)scratch_bytes);
  chunk = std::min(chunk, nfreqs);
  constexpr int WARPS = 8;
  const size_t smem = (size_t)WARPS * 2 * nbins * sizeof(float);
  if (smem > 48 * 1024) {
    cudaError_t e1 = cudaFuncSetAttribute(brutefold_kernel<uint8_t, WARPS>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaError_t e2 = cudaFuncSetAttribute(brutefold_kernel<uint16_t, WARPS>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e1 != cudaSuccess || e2 != cudaSuccess)
      return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  }
  for (int64_t f0 = 0; f0 < nfreqs; f0 += chunk) {
    const int64_t nf = std::min(chunk, nfreqs - f0);
    const int64_t total = nf * segment_len;
    const int mblocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 64);
    const int64_t fblocks = (nf + WARPS - 1) / WARPS;
    const int64_t blocks = nseg * fblocks;
    if (blocks > 0x7FFFFFFF) return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
    if (elem == 1) {
      uint8_t* map = (uint8_t*)phase_scratch;
      phase_map_kernel<uint8_t><<<mblocks, 256, 0, s>>>(freqs + f0, nf, segment_len, nbins,
                                                       tsamp, t_ref, map);
      brutefold_kernel<uint8_t, WARPS><<<(unsigned)blocks, WARPS * 32, smem, s>>>(
          ts_e, ts_v, nsamps, map, nf, f0, nfreqs, segment_len, nseg, nbins, fold_out);
    } else {
      uint16_t* map = (uint16_t*)phase_scratch;
      phase_map_kernel<uint16_t><<<mblocks, 256, 0, s>>>(freqs + f0, nf, segment_len, nbins,
                                                        tsamp, t_ref, map);
      brutefold_kernel<uint16_t, WARPS><<<(unsigned)blocks, WARPS * 32, smem, s>>>(
          ts_e, ts_v, nsamps, map, nf, f0, nfreqs, segment_len, nseg, nbins, fold_out);
    }
    int rc = check_launch("brutefold");
    if (rc) return rc;
  }
  return LOKI_OK;
}

extern "C" int loki_ffa_final_banded(const LokiFFALevel* pen, const LokiFFALevel* fin,
                                     int64_t band_width, const int64_t* win_lo,
                                     const int64_t* win_hi, const float* fold_pp,
                                     float* scratch, int64_t scratch_floats,
                                     const LokiScoreSpec* spec, float* snr, int32_t* dev_err,
                                     void* stream) {
  int rc = check_level(pen);
  if (rc) return rc;
  rc = check_level(fin);
  if (rc) return rc;
  rc = fill_spec_check(spec, fin->nbins);
  if (rc) return rc;
  if (!win_lo || !win_hi || !fold_pp || !scratch || !snr || !dev_err)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (band_width < 1) return set_error(LOKI_ERR_INVALID, "band_width < 1");
  if (fin->level != pen->level + 1 || pen->nseg_in != 2 * fin->nseg_in ||
      fin->nparams != pen->nparams)
    return set_error(LOKI_ERR_INVALID, "pen/fin descriptors are not consecutive levels");
  cudaStream_t s = (cudaStream_t)stream;
  const int warps = score_warps_per_block(fin->nbins, spec->wmax);
  const int smem = score_smem_bytes(fin->nbins, spec->wmax, warps);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(ffa_level_score_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  const int n = fin->nparams;
  const int64_t nf = fin->counts_cur[n - 1];
  const int64_t nbands = (nf + band_width - 1) / band_width;
  int64_t other_pen = 1;
  for (int d = 0; d < n - 1; ++d) other_pen *= pen->counts_cur[d];
  const int64_t prof_floats = 2 * (int64_t)fin->nbins;
  LokiFFALevel P = *pen, F = *fin;
  for (int64_t k = 0; k < nbands; ++k) {
    const int64_t h0 = win_lo[k], wh = win_hi[k] - win_lo[k] + 1;
    if (wh < 1 || h0 < 0 || h0 + wh > pen->counts_cur[n - 1])
      return set_error(LOKI_ERR_INVALID, "band %lld has an invalid window", (long long)k);
    if (fin->nseg_in * other_pen * wh * prof_floats > scratch_floats)
      return set_error(LOKI_ERR_CAPACITY, "band %lld needs more scratch", (long long)k);
    P.out_start = h0;
    P.out_width = wh;
    const int64_t Qp = n_out_params(P);
    const int64_t bp = ((Qp + 31) / 32 + 7) / 8;
    ffa_level_kernel<<<(unsigned)bp, 256, 0, s>>>(P, fold_pp, scratch, dev_err);
    F.out_start = k * band_width;
    F.out_width = std::min(band_width, nf - F.out_start);
    F.in_start = h0;
    F.in_width = wh;
    const int64_t Qf = n_out_params(F);
    const int64_t bf = ((Qf + 31) / 32 + warps - 1) / warps;
    ffa_level_score_kernel<<<(unsigned)bf, warps * 32, smem, s>>>(F, scratch, *spec, snr,
                                                                  dev_err);
  }
  return check_launch("ffa_final_banded");
}

extern "C" int loki_ffa_plan(const LokiFFALevel* lvl, LokiFFACoord* coords,
                             int32_t* dev_err, void* stream) {
  int rc = check_level(lvl);
  if (rc) return rc;
  if (!coords || !dev_err) return set_error(LOKI_ERR_INVALID, "null output pointer");
  const int64_t Q = n_out_params(*lvl);
  const int blocks = (int)std::min<int64_t>((Q + 255) / 256, 152 * 32);
  ffa_plan_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(*lvl, coords, dev_err);
  return check_launch("ffa_plan");
}

extern "C" int loki_ffa_level(const LokiFFALevel* lvl, const float* fold_in,
                              float* fold_out, int32_t* dev_err, void* stream) {
  int rc = check_level(lvl);
  if (rc) return rc;
  if (!fold_in || !fold_out || !dev_err)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const int64_t Q = n_out_params(*lvl);
  const int64_t warps = (Q + 31) / 32;
  const int64_t blocks = (warps + 7) / 8;
  if (blocks > 0x7FFFFFFF) return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
  ffa_level_kernel<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(*lvl, fold_in, fold_out,
                                                                       dev_err);
  return check_launch("ffa_level");
}

extern "C" int loki_ffa_level_score(const LokiFFALevel* lvl, const float* fold_in,
                                    const LokiScoreSpec* spec, float* snr,
                                    int32_t* dev_err, void* stream) {
  int rc = check_level(lvl);
  if (rc) return rc;
  rc = fill_spec_check(spec, lvl->nbins);
  if (rc) return rc;
  if (!fold_in || !snr || !dev_err) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const int warps = score_warps_per_block(lvl->nbins, spec->wmax);
  const int smem = score_smem_bytes(lvl->nbins, spec->wmax, warps);
  if (smem > 48 * 1024) {
    if (cudaFuncSetAttribute(ffa_level_score_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess)
      return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  }
  const int64_t Q = n_out_params(*lvl);
  const int64_t nw = (Q + 31) / 32;
  const int64_t blocks = (nw + warps - 1) / warps;
  if (blocks > 0x7FFFFFFF) return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
  ffa_level_score_kernel<<<(unsigned)blocks, warps * 32, smem, (cudaStream_t)stream>>>(
      *lvl, fold_in, *spec, snr, dev_err);
  return check_launch("ffa_level_score");
}

extern "C" int loki_ffa_band_windows(const LokiFFALevel* lvl, int64_t band_width,
                                     int64_t* win_lo, int64_t* win_hi, void* stream) {
  int rc = check_level(lvl);
  if (rc) return rc;
  if (band_width < 1) return set_error(LOKI_ERR_INVALID, "band_width < 1");
  if (!win_lo || !win_hi) return set_error(LOKI_ERR_INVALID, "null window pointer");
  const int64_t nf = lvl->counts_cur[lvl->nparams - 1];
  const int64_t nbands = (nf + band_width - 1) / band_width;
  int64_t n_other = 1;
  for (int d = 0; d < lvl->nparams - 1; ++d) n_other *= lvl->counts_cur[d];
  cudaStream_t s = (cudaStream_t)stream;
  // lo starts at all-ones (max unsigned), hi at zero.
  if (cudaMemsetAsync(win_lo, 0xFF, nbands * sizeof(int64_t), s) != cudaSuccess ||
      cudaMemsetAsync(win_hi, 0x00, nbands * sizeof(int64_t), s) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaMemsetAsync failed");
  const int64_t total = nbands * n_other;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 32);
  ffa_band_window_kernel<<<blocks, 256, 0, s>>>(*lvl, band_width, nbands,
                                                (unsigned long long*)win_lo,
                                                (unsigned long long*)win_hi);
  return check_launch("ffa_band_windows");
}
