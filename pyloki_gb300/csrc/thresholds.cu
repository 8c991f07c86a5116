// Monte-Carlo fold simulation and scoring for the threshold-scheme designer
// (detection/thresholding.py:46-96 simulate_folds, 484-500 fold_max_scores).
//
// Output row r is input row src_row[r] plus bias[r] * profile plus Gaussian
// noise of standard deviation noise_std; its score is the max over widths of
// the boxcar S/N (detection/scoring.py:99-153) of row / sqrt_var (float32
// division, as prune_folds normalises), with the
// same scoring code as the FFA and pruning scorers. Noise of (row, bin) comes
// from a Philox-4x32-10 counter-based generator (Salmon, Moraes, Dror and
// Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC 2011) keyed by the
// seed, counter (row, bin), and a Box-Muller transform, so it does not depend
// on the launch shape.
#include <algorithm>

#include "loki_common.cuh"
#include "rng.cuh"
#include "score.cuh"

namespace loki {

int score_smem_bytes(int nbins, int wmax, int warps);
int score_warps_per_block(int nbins, int wmax);

// A warp per 32 output rows: the warp builds each row with coalesced stores
// (and the normalised copy in its shared tile), then lane k scores row k.
__global__ void __launch_bounds__(128)
sim_score_kernel(const float* __restrict__ in, const int64_t* __restrict__ src_row,
                 const float* __restrict__ bias, int64_t nrows,
                 const float* __restrict__ profile, int nb, float noise_std,
                 float sqrt_var, uint64_t seed, LokiScoreSpec sp, ScoreK SK,
                 float* __restrict__ out, float* __restrict__ scores) {
  extern __shared__ float tiles[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int stride = score_stride(nb, sp.wmax);
  float* tile = tiles + (size_t)warp * 32 * stride;
  const int64_t r0 = ((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * 32;
  if (r0 >= nrows) return;
  const int kmax = (int)min((int64_t)32, nrows - r0);
  for (int k = 0; k < kmax; ++k) {
    const int64_t r = r0 + k;
    const float* src = in ? in + src_row[r] * nb : nullptr;
    const float b = bias[r];
    float* dst = out + r * nb;
    float* trow = tile + k * stride;
    for (int j = lane; j < nb; j += 32) {
      const float base = src ? src[j] : 0.0f;
      const float x = base + normal_at(seed, r, j) * noise_std + profile[j] * b;
      dst[j] = x;
      trow[j] = __fdiv_rn(x, sqrt_var);
    }
  }
  __syncwarp();
  if (lane < kmax) {
    float* row = tile + lane * stride;
    if (SK.pow2_64) score_row64_pow2(row, sp, SK, scores + r0 + lane);
    else score_row(row, nb, sp, scores + r0 + lane);
  }
}

__global__ void gather_rows_kernel(const float* __restrict__ src, const int64_t* __restrict__ idx,
                                   int64_t n, int64_t row_len, float* __restrict__ dst) {
  const int64_t total = n * row_len;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / row_len, j = t - i * row_len;
    dst[t] = src[idx[i] * row_len + j];
  }
}

}  // namespace loki

using namespace loki;

extern "C" int loki_sim_score_folds(const float* folds_in, const int64_t* src_row,
                                    const float* bias, int64_t nrows, const float* profile,
                                    int32_t nbins, float noise_std, float sqrt_var,
                                    uint64_t seed, const LokiScoreSpec* spec, float* folds_out,
                                    float* scores, void* stream) {
  if (nrows < 0 || nbins < 2) return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (!spec || spec->nwidths < 1 || spec->nwidths > LOKI_MAX_WIDTHS || spec->mode != 1)
    return set_error(LOKI_ERR_INVALID, "spec must be a mode-1 (max over widths) spec");
  if (nbins + spec->wmax > 2048)
    return set_error(LOKI_ERR_UNSUPPORTED, "nbins + wmax above 2048");
  if (nrows == 0) return LOKI_OK;
  if (!bias || !profile || !folds_out || !scores || (folds_in && !src_row))
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const int warps = score_warps_per_block(nbins, spec->wmax);
  const int smem = score_smem_bytes(nbins, spec->wmax, warps);
  if (smem > 48 * 1024 &&
      set_smem_limit(sim_score_kernel, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  const ScoreK SK = make_score_k(*spec, nbins);
  const int64_t blocks = (nrows + warps * 32 - 1) / (warps * 32);
  if (blocks > 0x7FFFFFFF) return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
  note_launch();
  sim_score_kernel<<<(unsigned)blocks, warps * 32, smem, (cudaStream_t)stream>>>(
      folds_in, src_row, bias, nrows, profile, nbins, noise_std, sqrt_var, seed, *spec, SK,
      folds_out, scores);
  return check_launch("sim_score_folds");
}

extern "C" int loki_gather_rows(const float* src, const int64_t* idx, int64_t n,
                                int64_t row_len, float* dst, void* stream) {
  if (n < 0 || row_len < 1) return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (n == 0) return LOKI_OK;
  if (!src || !idx || !dst) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  note_launch();
  gather_rows_kernel<<<(unsigned)std::min<int64_t>((n * row_len + 255) / 256, 152 * 32), 256, 0,
                       (cudaStream_t)stream>>>(src, idx, n, row_len, dst);
  return check_launch("gather_rows");
}
