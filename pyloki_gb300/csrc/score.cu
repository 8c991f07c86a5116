// Standalone boxcar scoring kernels (detection/scoring.py:99-165, 249-282).
#include <algorithm>

#include "loki_common.cuh"
#include "score.cuh"

namespace loki {

int score_smem_bytes(int nbins, int wmax, int warps);
int score_warps_per_block(int nbins, int wmax);

// Each warp scores 32 profiles: rows are staged into the warp's tile with
// coalesced loads (normalising e / sqrt(v) first when FROM_EV), then lane k
// runs the sequential prefix sum and the width scan of row k.
template <bool FROM_EV>
__global__ void __launch_bounds__(128)
score_kernel(const float* __restrict__ in, int64_t nprof, int nb, LokiScoreSpec sp, ScoreK SK,
             float* __restrict__ out) {
  extern __shared__ float tiles[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int stride = score_stride(nb, sp.wmax);
  float* tile = tiles + (size_t)warp * 32 * stride;
  const int64_t p0 = ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * 32;
  if (p0 >= nprof) return;
  const int kmax = (int)min((int64_t)32, nprof - p0);
  for (int k = 0; k < kmax; ++k) {
    float* trow = tile + k * stride;
    if (FROM_EV) {
      const float* src = in + (size_t)(p0 + k) * 2 * nb;
      for (int j = lane; j < nb; j += 32) trow[j] = __fdiv_rn(src[j], __fsqrt_rn(src[nb + j]));
    } else {
      const float* src = in + (size_t)(p0 + k) * nb;
      for (int j = lane; j < nb; j += 32) trow[j] = src[j];
    }
  }
  __syncwarp();
  if (lane < kmax) {
    const int nout = sp.mode == 0 ? sp.nwidths : 1;
    float* row = tile + lane * stride;
    if (SK.pow2_64) score_row64_pow2(row, sp, SK, out + (size_t)(p0 + lane) * nout);
    else score_row(row, nb, sp, out + (size_t)(p0 + lane) * nout);
  }
}

static int check_spec(const LokiScoreSpec* sp, int nbins) {
  if (!sp) return set_error(LOKI_ERR_INVALID, "null score spec");
  if (nbins < 2) return set_error(LOKI_ERR_INVALID, "nbins %d < 2", nbins);
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

template <bool FROM_EV>
static int launch_score(const float* in, int64_t nprof, int nbins, LokiScoreSpec sp,
                        float* out, cudaStream_t s, const char* what) {
  const int warps = score_warps_per_block(nbins, sp.wmax);
  const int smem = score_smem_bytes(nbins, sp.wmax, warps);
  if (smem > 48 * 1024 &&
      set_smem_limit(score_kernel<FROM_EV>, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  const int64_t nw = (nprof + 31) / 32;
  const int64_t blocks = (nw + warps - 1) / warps;
  if (blocks > 0x7FFFFFFF) return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
  const ScoreK SK = make_score_k(sp, nbins);
  note_launch();
  score_kernel<FROM_EV><<<(unsigned)blocks, warps * 32, smem, s>>>(in, nprof, nbins, sp, SK, out);
  return check_launch(what);
}

}  // namespace loki

using namespace loki;

extern "C" int loki_boxcar_snr(const float* profiles, int64_t nprof, int32_t nbins,
                               const LokiScoreSpec* spec, float* snr, void* stream) {
  int rc = check_spec(spec, nbins);
  if (rc) return rc;
  if (nprof < 0) return set_error(LOKI_ERR_INVALID, "nprof < 0");
  if (nprof == 0) return LOKI_OK;
  if (!profiles || !snr) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  return launch_score<false>(profiles, nprof, nbins, *spec, snr, (cudaStream_t)stream,
                             "boxcar_snr");
}

extern "C" int loki_snr_score_batch(const float* folds, int64_t n, int32_t nbins,
                                    const LokiScoreSpec* spec, float* scores, void* stream) {
  int rc = check_spec(spec, nbins);
  if (rc) return rc;
  if (n < 0) return set_error(LOKI_ERR_INVALID, "n < 0");
  if (n == 0) return LOKI_OK;
  if (!folds || !scores) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  LokiScoreSpec sp = *spec;
  sp.mode = 1;
  return launch_score<true>(folds, n, nbins, sp, scores, (cudaStream_t)stream,
                            "snr_score_batch");
}

namespace loki {
// norm[p, j] = fold[p, 0, j] / sqrt(fold[p, 1, j])  (ffa.py:382-411 get_fold_norm)
__global__ void fold_norm_kernel(const float* __restrict__ folds, int64_t n, int nb,
                                 float* __restrict__ out) {
  const int64_t total = n * nb;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = k / nb;
    const int64_t j = k - p * nb;
    const float* src = folds + p * 2 * nb;
    out[k] = __fdiv_rn(src[j], __fsqrt_rn(src[nb + j]));
  }
}
}  // namespace loki

extern "C" int loki_fold_norm(const float* folds, int64_t n, int32_t nbins, float* out,
                              void* stream) {
  if (n < 0 || nbins < 1) return set_error(LOKI_ERR_INVALID, "bad fold_norm sizes");
  if (n == 0) return LOKI_OK;
  if (!folds || !out) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const int64_t total = n * nbins;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 32);
  note_launch();
  fold_norm_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(folds, n, nbins, out);
  return check_launch("fold_norm");
}
