// Enumerate-prune kernels for the Taylor basis with float32 folds
// (prune.py:165-332 pruning_iteration_batched with the PrunePolyTaylorDPFuncts
// plugin, dynamic/dyn_poly_taylor.py:396-690).
//
// One level = branch (per parent) -> exclusive scan of child counts -> score
// (per child: branch value, FP64 resolve, gather + roll + add, boxcar S/N) ->
// selection (in child order, with the exact overflow rule when needed) ->
// emit (transform the survivors, write the new tree). Child order is parent
// order then the C-order odometer over the branched parameters, which is the
// order the reference appends survivors in.
//
// FP64 arithmetic follows the reference's numpy operations with round-to-
// nearest intrinsics (no contraction); the batched Taylor shifts reproduce
// the BLAS matrix product, which accumulates each output with forward fused
// multiply-adds (acc = fma(x_j, T_ij, acc), j = 0..P).
#include <algorithm>
#include <vector>

#include "loki_common.cuh"
#include "score.cuh"

namespace loki {

int score_smem_bytes(int nbins, int wmax, int warps);

// ---------------------------------------------------------------------------
// exclusive scan of int64 (counts) or of score >= threshold flags
// ---------------------------------------------------------------------------

constexpr int kScanBlock = 1024;

template <bool FLAGS>
__device__ __forceinline__ int64_t scan_in(const void* in, int64_t i, int64_t n, double thr) {
  if (i >= n) return 0;
  if (FLAGS) return ((double)reinterpret_cast<const float*>(in)[i] >= thr) ? 1 : 0;
  return reinterpret_cast<const int64_t*>(in)[i];
}

// One kScanBlock-element tile of the scan: exclusive within the tile, the
// tile's total in sums[tile].
template <bool FLAGS>
__device__ __forceinline__ void scan_tile(const void* in, int64_t n, double thr, int64_t* out,
                                          int64_t* sums, int64_t tile, int64_t* warp_tot) {
  const int64_t i = tile * kScanBlock + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t x = scan_in<FLAGS>(in, i, n, thr);
  int64_t v = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xFFFFFFFFu, v, o);
    if (lane >= o) v += y;
  }
  if (lane == 31) warp_tot[warp] = v;
  __syncthreads();
  if (warp == 0) {
    int64_t w = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
      if (lane >= o) w += y;
    }
    warp_tot[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  const int64_t incl = v + (warp ? warp_tot[warp - 1] : 0);
  if (i < n) out[i] = incl - x;  // exclusive within the block
  if (threadIdx.x == kScanBlock - 1) sums[tile] = incl;
  __syncthreads();  // warp_tot is reused by the next tile
}

// n_dev, when not null, holds the element count on the device: the blocks
// then stride over its tiles.
template <bool FLAGS>
__global__ void __launch_bounds__(kScanBlock)
scan_block_kernel(const void* in, int64_t n, const int64_t* n_dev, double thr, int64_t* out,
                  int64_t* sums) {
  __shared__ int64_t warp_tot[32];
  if (!n_dev) {
    scan_tile<FLAGS>(in, n, thr, out, sums, blockIdx.x, warp_tot);
    return;
  }
  n = *n_dev;
  const int64_t ntiles = (n + kScanBlock - 1) / kScanBlock;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x)  // uniform over the block
    scan_tile<FLAGS>(in, n, thr, out, sums, t, warp_tot);
}

// Single block: exclusive scan of the block sums (any count), carry-chained.
// With n_dev the block count and the total's slot (out + n) come from the
// device count.
__global__ void __launch_bounds__(kScanBlock)
scan_sums_kernel(int64_t* sums, int64_t nblocks, int64_t* total, const int64_t* n_dev,
                 int64_t* out) {
  __shared__ int64_t warp_tot[32];
  __shared__ int64_t carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (n_dev) {
    const int64_t n = *n_dev;
    nblocks = (n + kScanBlock - 1) / kScanBlock;
    total = out + n;
  }
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < nblocks; base += kScanBlock) {
    const int64_t i = base + threadIdx.x;
    const int64_t x = i < nblocks ? sums[i] : 0;
    int64_t v = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xFFFFFFFFu, v, o);
      if (lane >= o) v += y;
    }
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    if (warp == 0) {
      int64_t w = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
        if (lane >= o) w += y;
      }
      warp_tot[lane] = w;
    }
    __syncthreads();
    const int64_t incl = v + (warp ? warp_tot[warp - 1] : 0);
    const int64_t c = carry;
    if (i < nblocks) sums[i] = c + incl - x;
    __syncthreads();
    if (threadIdx.x == kScanBlock - 1) carry = c + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void scan_add_kernel(int64_t* out, int64_t n, const int64_t* n_dev,
                                const int64_t* sums) {
  if (!n_dev) {
    const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] += sums[blockIdx.x];
    return;
  }
  n = *n_dev;
  for (int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kScanBlock)
    out[i] += sums[i / kScanBlock];
}

// out[0..n) exclusive scan, out[n] = total.
template <bool FLAGS>
static int exclusive_scan(const void* in, int64_t n, double thr, int64_t* out, void* scratch,
                          int64_t scratch_bytes, cudaStream_t s) {
  const int64_t nblocks = std::max<int64_t>(1, (n + kScanBlock - 1) / kScanBlock);
  if (scratch_bytes < nblocks * (int64_t)sizeof(int64_t))
    return set_error(LOKI_ERR_CAPACITY, "scan scratch too small");
  int64_t* sums = reinterpret_cast<int64_t*>(scratch);
  if (n == 0) {
    if (cudaMemsetAsync(out, 0, sizeof(int64_t), s) != cudaSuccess)
      return set_error(LOKI_ERR_CUDA, "cudaMemsetAsync failed");
    return LOKI_OK;
  }
  for (int i = 0; i < 3; ++i) note_launch();
  scan_block_kernel<FLAGS><<<(unsigned)nblocks, kScanBlock, 0, s>>>(in, n, nullptr, thr, out,
                                                                    sums);
  scan_sums_kernel<<<1, kScanBlock, 0, s>>>(sums, nblocks, out + n, nullptr, nullptr);
  scan_add_kernel<<<(unsigned)nblocks, kScanBlock, 0, s>>>(out, n, nullptr, sums);
  return check_launch("exclusive_scan");
}

// The same scan over a device-held count *n_dev <= n_cap (no host wait):
// out[0..n) exclusive scan, out[n] = total. At most `grid` blocks stride over
// the tiles.
template <bool FLAGS>
static int exclusive_scan_dev(const void* in, int64_t n_cap, const int64_t* n_dev, double thr,
                              int64_t* out, void* scratch, int64_t scratch_bytes, int grid,
                              cudaStream_t s) {
  const int64_t ntiles = std::max<int64_t>(1, (n_cap + kScanBlock - 1) / kScanBlock);
  if (scratch_bytes < ntiles * (int64_t)sizeof(int64_t))
    return set_error(LOKI_ERR_CAPACITY, "scan scratch too small");
  const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ntiles, grid));
  int64_t* sums = reinterpret_cast<int64_t*>(scratch);
  for (int i = 0; i < 3; ++i) note_launch();
  scan_block_kernel<FLAGS><<<blocks, kScanBlock, 0, s>>>(in, n_cap, n_dev, thr, out, sums);
  scan_sums_kernel<<<1, kScanBlock, 0, s>>>(sums, ntiles, nullptr, n_dev, out);
  scan_add_kernel<<<blocks, kScanBlock, 0, s>>>(out, n_cap, n_dev, sums);
  return check_launch("exclusive_scan_dev");
}

// ---------------------------------------------------------------------------
// shared FP64 pieces
// ---------------------------------------------------------------------------

// y_i = sum_j x_j T_ij accumulated with forward fused multiply-adds.
__device__ __forceinline__ double tdot(const double* x, const double (*T)[LOKI_MAX_PARAMS + 1],
                                       int i, int m) {
  double acc = 0.0;
  for (int j = 0; j < m; ++j) acc = __fma_rn(x[j], T[i][j], acc);
  return acc;
}

// get_nearest_indices_2d_batch for one axis (utils/psr_utils.py:517-554).
__device__ __forceinline__ int64_t axis_index(double v, double vmin, double inv, int64_t n) {
  if (!(inv > 0.0)) return 0;
  const double raw = __dmul_rn(__dsub_rn(v, vmin), inv);
  int64_t idx = (int64_t)__dadd_rn(raw, LOKI_FLOAT_EPSILON);
  if (idx < 0) idx = 0;
  else if (idx >= n) idx = n - 1;
  return idx;
}

// Child leaf parameters [d_P .. d_1] from the parent's branching info.
__device__ __forceinline__ void child_params(const LokiBranchInfo& B, int P, int64_t local,
                                             double* pv) {
  for (int j = P - 1; j >= 0; --j) {
    const int64_t c = B.count[j];
    const int64_t k = local % c;
    local /= c;
    pv[j] = (c == 1 && k == 0) ? B.first[j]
                               : __dadd_rn(B.first[j], __dmul_rn((double)k, B.dact[j]));
  }
}

struct ChildRes {
  int32_t ia, iff;  // (accel, freq) FFA grid indices
  double phase;
};

// cheby_to_taylor (utils/transforms.py:556-583) of coefficients a[0..P]
// (alpha_P..alpha_0), lowest three Taylor orders only: d_k =
// ((rev(a) @ R)[k] * k!) / scale**k for k = 2 (accel), 1 (velocity), 0 (delay).
__device__ __forceinline__ void cheby_low3(const LokiPruneLevel& D, const double* a, int m,
                                           double* d2, double* d1, double* d0) {
  double ar[LOKI_MAX_PARAMS + 1];
  for (int i = 0; i < m; ++i) ar[i] = a[m - 1 - i];
  double d[3];
  for (int k = 0; k < 3; ++k)
    d[k] = __ddiv_rn(__dmul_rn(tdot(ar, D.tm_r, k, m), D.cfact[k]), D.ctsk[k]);
  *d0 = d[0];
  *d1 = d[1];
  *d2 = d[2];
}

// Chebyshev resolve (core/chebyshev.py:180-277): shift the coefficients to
// t_add (and t_init on the moving grid) at the current scale, then read the
// Taylor accel / velocity / delay there.
__device__ __forceinline__ void cheby_kinematics(const LokiPruneLevel& D, const double* pv,
                                                 double* accel, double* vel, double* dd) {
  const int m = D.poly_order + 1;
  double a[LOKI_MAX_PARAMS + 1];
  for (int i = 0; i < m; ++i) a[i] = tdot(pv, D.tm_a, i, m);
  double a2, a1, a0;
  cheby_low3(D, a, m, &a2, &a1, &a0);
  *accel = a2;
  if (D.moving) {
    for (int i = 0; i < m; ++i) a[i] = tdot(pv, D.tm_i, i, m);
    double i2, i1, i0;
    cheby_low3(D, a, m, &i2, &i1, &i0);
    *vel = __dsub_rn(a1, i1);
    *dd = __dsub_rn(a0, i0);
  } else {
    *vel = a1;
    *dd = a0;
  }
}

// poly_taylor_resolve_batch (moving) / poly_taylor_fixed_resolve_batch
// (core/taylor.py:172-277) for one child with params pv[0..P] (d_P..d_1, d_0).
__device__ __forceinline__ ChildRes resolve_child(const LokiPruneLevel& D, const double* pv,
                                                  double f0) {
  const int P = D.poly_order, m = P + 1;
  double accel, vel, dd;
  if (D.basis == 1) {
    cheby_kinematics(D, pv, &accel, &vel, &dd);
  } else if (D.moving) {
    accel = tdot(pv, D.tm_a, P - 2, m);
    vel = __dsub_rn(tdot(pv, D.tm_a, P - 1, m), tdot(pv, D.tm_i, P - 1, m));
    dd = __dsub_rn(tdot(pv, D.tm_a, P, m), tdot(pv, D.tm_i, P, m));
  } else {
    accel = tdot(pv, D.tm_a, P - 2, m);
    vel = tdot(pv, D.tm_a, P - 1, m);
    dd = tdot(pv, D.tm_a, P, m);
  }
  const double freq = __dmul_rn(f0, __dsub_rn(1.0, __ddiv_rn(vel, LOKI_C_VAL)));
  const double delay = __ddiv_rn(dd, LOKI_C_VAL);
  ChildRes r;
  r.phase = phase_idx(D.dt_phase, f0, D.nbins, delay);
  r.ia = (int32_t)axis_index(accel, D.accel_min, D.accel_inv, D.n_accel);
  r.iff = (int32_t)axis_index(freq, D.freq_min, D.freq_inv, D.n_freq);
  return r;
}

// ---------------------------------------------------------------------------
// branch
// ---------------------------------------------------------------------------

// Parent i: per-parameter child counts, steps and first values (info[i]) and
// its child count (counts[i]).
__device__ __forceinline__ void branch_one(const LokiPruneLevel& D,
                                           const double* __restrict__ leaves, int64_t i,
                                           LokiBranchInfo* __restrict__ info,
                                           int64_t* __restrict__ counts,
                                           int32_t* __restrict__ err,
                                           const uint8_t* __restrict__ mask) {
  const int P = D.poly_order, m = P + 1;
  const double* lf = leaves + i * (P + 2) * 2;
  const double f0 = lf[(P + 1) * 2];
  const double fscale = __ddiv_rn(f0, LOKI_C_VAL);
  // Parent values and errors in the current domain: as stored (Taylor), or
  // shifted from the previous to the current Chebyshev domain with
  // shift_cheby_full (utils/transforms.py:650-701).
  double pval[LOKI_MAX_PARAMS + 1], perr[LOKI_MAX_PARAMS + 1];
  if (D.basis == 1) {
    double raw[LOKI_MAX_PARAMS + 1], rawe[LOKI_MAX_PARAMS + 1];
    for (int k = 0; k < m; ++k) {
      raw[k] = lf[2 * k];
      rawe[k] = lf[2 * k + 1];
    }
    for (int k = 0; k < m; ++k) pval[k] = tdot(raw, D.tm_b, k, m);
    if (D.tiling == 0) {
      for (int k = 0; k < m; ++k) perr[k] = __dmul_rn(rawe[k], fabs(D.tm_b[k][k]));
    } else if (D.tiling == 2) {
      for (int k = 0; k < m; ++k) perr[k] = tdot(rawe, D.tm_be, k, m);
    } else {
      double e2[LOKI_MAX_PARAMS + 1];
      for (int k = 0; k < m; ++k) e2[k] = __dmul_rn(rawe[k], rawe[k]);
      for (int k = 0; k < m; ++k) perr[k] = __dsqrt_rn(tdot(e2, D.tm_be, k, m));
    }
  } else {
    for (int k = 0; k < m; ++k) {
      pval[k] = lf[2 * k];
      perr[k] = lf[2 * k + 1];
    }
  }
  // Halving is exact, so x / 2 is computed as x * 0.5 (the same rounded
  // value as the reference's division).
  LokiBranchInfo B;
  B.d0 = pval[P];
  int64_t total = 1;
  for (int j = 0; j < P; ++j) {
    const double pcur = pval[j], dcur = perr[j];
    const double dnew = __ddiv_rn(D.dfc[j], f0);
    const double fb = __dmul_rn(D.fac[j], fscale);
    const double shift = __dmul_rn(fabs(__dsub_rn(dcur, dnew)), fb);
    const bool split = !(shift < D.eta_m);
    int64_t num = 1;
    double dact = dcur, first = pcur;
    if (!(dcur > 0.0) || !(dnew > 0.0)) {
      atomicOr(err, LOKI_DEVERR_BRANCH);
    } else if (split || dcur > __dmul_rn(dnew, 0.5 * (double)D.branch_max)) {
      // The child count is needed for a split, and for the reference's
      // branch_max check of every parameter; a parameter that does not
      // split and whose step is at most half of branch_max new steps cannot
      // exceed branch_max (ratio <= branch_max / 2 up to rounding), so its
      // division is skipped.
      const double ratio = __ddiv_rn(dcur, dnew);
      num = (int64_t)ceil(__dsub_rn(ratio, LOKI_FLOAT_EPSILON));
      if (num < 1) num = 1;
      if (num > D.branch_max) {
        atomicOr(err, LOKI_DEVERR_BRANCH);
        num = D.branch_max;
      }
      if (split) {  // division by 1 or a power of two is exact scaling
        dact = num == 1                ? dcur
               : (num & (num - 1)) == 0 ? __dmul_rn(dcur, 1.0 / (double)num)
                                        : __ddiv_rn(dcur, (double)num);
        const double pmin = __dsub_rn(pcur, __dmul_rn(dcur, 0.5));
        first = __dadd_rn(pmin, __dmul_rn(dact, 0.5));
      }
    }
    if (!split) {
      num = 1;
      dact = dcur;
      first = pcur;
    }
    B.first[j] = first;
    B.dact[j] = dact;
    B.count[j] = (int32_t)num;
    total *= num;
  }
  info[i] = B;
  counts[i] = (mask && !mask[i]) ? 0 : total;  // a masked-out parent has no children
}

__global__ void prune_branch_kernel(LokiPruneLevel D, const double* __restrict__ leaves,
                                    int64_t n, LokiBranchInfo* __restrict__ info,
                                    int64_t* __restrict__ counts, int32_t* __restrict__ err,
                                    const uint8_t* __restrict__ mask,
                                    const int64_t* __restrict__ n_dev) {
  if (n_dev) n = *n_dev;  // parent count held on the device
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  branch_one(D, leaves, i, info, counts, err, mask);
}

// ---------------------------------------------------------------------------
// score: warp per 32 children
// ---------------------------------------------------------------------------

constexpr int kPruneWarps = 4;

__device__ __forceinline__ int64_t find_parent(const int64_t* offsets, int64_t n, int64_t c) {
  int64_t lo = 0, hi = n;  // offsets[lo] <= c < offsets[hi]
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (offsets[mid] <= c) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ unsigned float_key(float x) {
  const unsigned u = __float_as_uint(x);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ float key_float(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// Children c0 .. c0 + 31 (those below n_children) of one warp.
__device__ __forceinline__ void score_tile(const LokiPruneLevel& D, const double* __restrict__ leaves,
                   const float* __restrict__ folds, int64_t n_parents,
                   const LokiBranchInfo* __restrict__ info, const int64_t* __restrict__ offsets,
                   int64_t n_children, const float* __restrict__ seg, const LokiScoreSpec& sp,
                   const ScoreK& SK, float* __restrict__ scores, int32_t* __restrict__ cidx,
                   double* __restrict__ cphase, unsigned* __restrict__ minmax_keys,
                   float* tile, int64_t c0) {
  const int lane = threadIdx.x & 31;
  const int nb = D.nbins, P = D.poly_order;
  const int stride = score_stride(nb, sp.wmax);
  const int kmax = (int)std::min<int64_t>(32, n_children - c0);
  // lane k resolves child c0 + k
  int64_t my_par = 0, my_row = 0;
  int my_shift = 0;
  if (lane < kmax) {
    const int64_t c = c0 + lane;
    const int64_t par = find_parent(offsets, n_parents, c);
    const LokiBranchInfo B = info[par];
    const double* lf = leaves + par * (P + 2) * 2;
    double pv[LOKI_MAX_PARAMS + 1];
    child_params(B, P, c - offsets[par], pv);
    pv[P] = B.d0;  // d_0 (alpha_0 in the current domain for Chebyshev)
    const ChildRes r = resolve_child(D, pv, lf[(P + 1) * 2]);
    cidx[2 * c] = r.ia;
    cidx[2 * c + 1] = r.iff;
    cphase[c] = r.phase;
    my_par = par;
    my_row = (int64_t)r.ia * D.n_freq + r.iff;
    my_shift = round_shift(r.phase, nb);
  }
  if (nb == 64) {
    // eight children's rows in flight per lane (bins lane and lane + 32)
    constexpr int kU = 8;
    for (int k0 = 0; k0 < kmax; k0 += kU) {
      float pe[kU][2], pw[kU][2], se[kU][2], sw[kU][2];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int k = k0 + u;
        const int src = k < kmax ? k : 0;
        const int64_t par = __shfl_sync(0xFFFFFFFFu, my_par, src);
        const int64_t row = __shfl_sync(0xFFFFFFFFu, my_row, src);
        const int sh = __shfl_sync(0xFFFFFFFFu, my_shift, src);
        if (k < kmax) {
          const float* pf = folds + par * 128;
          const float* sf = seg + row * 128;
#pragma unroll
          for (int c = 0; c < 2; ++c) {
            const int j = lane + 32 * c;
            const int js = (j - sh) & 63;
            pe[u][c] = __ldg(pf + j);
            pw[u][c] = __ldg(pf + 64 + j);
            se[u][c] = __ldg(sf + js);
            sw[u][c] = __ldg(sf + 64 + js);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int k = k0 + u;
        if (k >= kmax) break;
        float* trow = tile + k * stride;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const float e = __fadd_rn(pe[u][c], se[u][c]);
          const float v = __fadd_rn(pw[u][c], sw[u][c]);
          trow[lane + 32 * c] = __fdiv_rn(e, __fsqrt_rn(v));
        }
      }
    }
  } else {
    for (int k = 0; k < kmax; ++k) {
      const int64_t par = __shfl_sync(0xFFFFFFFFu, my_par, k);
      const int64_t row = __shfl_sync(0xFFFFFFFFu, my_row, k);
      const int sh = __shfl_sync(0xFFFFFFFFu, my_shift, k);
      const float* pf = folds + par * 2 * nb;
      const float* sf = seg + row * 2 * nb;
      float* trow = tile + k * stride;
      for (int j = lane; j < nb; j += 32) {
        int js = j - sh;
        js += (js < 0) ? nb : 0;
        const float e = __fadd_rn(pf[j], sf[js]);
        const float v = __fadd_rn(pf[nb + j], sf[nb + js]);
        trow[j] = __fdiv_rn(e, __fsqrt_rn(v));
      }
    }
  }
  __syncwarp();
  if (lane < kmax) {
    float* row = tile + lane * stride;
    float s;
    if (SK.pow2_64) score_row64_pow2(row, sp, SK, &s);
    else score_row(row, nb, sp, &s);
    scores[c0 + lane] = s;
    if (s == s) {  // NaN scores do not enter min/max (like np.min on finite data)
      atomicMin(minmax_keys, float_key(s));
      atomicMax(minmax_keys + 1, float_key(s));
    }
  }
}

__global__ void __launch_bounds__(kPruneWarps * 32)
prune_score_kernel(LokiPruneLevel D, const double* __restrict__ leaves,
                   const float* __restrict__ folds, int64_t n_parents,
                   const LokiBranchInfo* __restrict__ info, const int64_t* __restrict__ offsets,
                   int64_t n_children, const float* __restrict__ seg, LokiScoreSpec sp,
                   ScoreK SK, float* __restrict__ scores, int32_t* __restrict__ cidx,
                   double* __restrict__ cphase, unsigned* __restrict__ minmax_keys,
                   int64_t* cnt_dev, int64_t child_cap, LokiPruneLevelStats* st,
                   int32_t* err) {
  extern __shared__ float tiles[];
  const int warp = threadIdx.x >> 5;
  float* tile = tiles + (size_t)warp * 32 * score_stride(D.nbins, sp.wmax);
  if (!cnt_dev) {
    const int64_t c0 = ((int64_t)blockIdx.x * kPruneWarps + warp) * 32;
    if (c0 < n_children)
      score_tile(D, leaves, folds, n_parents, info, offsets, n_children, seg, sp, SK, scores,
                 cidx, cphase, minmax_keys, tile, c0);
    return;
  }
  // device counts: cnt_dev[0] parents; the children are offsets[parents],
  // none when they exceed the workspace (the run is then flagged). Block 0
  // records them for the later kernels of the level. Warps stride over the
  // 32-child tiles.
  n_parents = cnt_dev[0];
  const int64_t total = offsets[n_parents];
  n_children = total > child_cap ? 0 : total;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cnt_dev[1] = n_children;
    st->n_parents = n_parents;
    st->n_children = total;
    st->n_valid = total;
    if (total > child_cap) atomicOr(err, LOKI_DEVERR_CAPACITY);
  }
  for (int64_t t = (int64_t)blockIdx.x * kPruneWarps + warp; t * 32 < n_children;
       t += (int64_t)gridDim.x * kPruneWarps) {
    score_tile(D, leaves, folds, n_parents, info, offsets, n_children, seg, sp, SK, scores,
               cidx, cphase, minmax_keys, tile, t * 32);
    __syncwarp();  // the tile rows are rewritten by the next tile
  }
}

__global__ void minmax_init_kernel(unsigned* keys) {
  keys[0] = 0xFFFFFFFFu;
  keys[1] = 0u;
}

__global__ void minmax_finish_kernel(const unsigned* keys, float* out) {
  if (keys[0] == 0xFFFFFFFFu) {  // no finite score
    out[0] = 0.0f;
    out[1] = 0.0f;
  } else {
    out[0] = key_float(keys[0]);
    out[1] = key_float(keys[1]);
  }
}

// ---------------------------------------------------------------------------
// selection without overflow
// ---------------------------------------------------------------------------

__global__ void select_scatter_kernel(const float* __restrict__ scores, int64_t n, double thr,
                                      const int64_t* __restrict__ pos, int64_t* __restrict__ ids,
                                      const int64_t* __restrict__ n_dev) {
  if (n_dev) {  // device count: grid-stride walk
    n = *n_dev;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
      if ((double)scores[i] >= thr) ids[pos[i]] = i;
    return;
  }
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n && (double)scores[i] >= thr) ids[pos[i]] = i;
}

// ---------------------------------------------------------------------------
// selection with the overflow rule (single block, sequential over batches)
// ---------------------------------------------------------------------------

constexpr int kSelThreads = 1024;

// Block-wide exclusive scan of one flag per thread; returns the offset of this
// thread and writes the block total.
__device__ __forceinline__ int block_scan_flag(int f, int* total, int* wsum) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned b = __ballot_sync(0xFFFFFFFFu, f);
  const int before = __popc(b & lanemask_lt());
  if (lane == 0) wsum[warp] = __popc(b);
  __syncthreads();
  if (warp == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
    int v = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xFFFFFFFFu, v, o);
      if (lane >= o) v += y;
    }
    wsum[lane] = v - w;  // exclusive
    if (lane == 31) wsum[32] = v;
  }
  __syncthreads();
  const int off = wsum[warp] + before;
  *total = wsum[32];
  __syncthreads();
  return off;
}

// Value of ascending rank r among keys[0..n) (radix select, 4 x 8 bits).
__device__ unsigned block_select(const unsigned* keys, int64_t n, int64_t r, unsigned* hist) {
  unsigned prefix = 0, mask = 0;
  for (int shift = 24; shift >= 0; shift -= 8) {
    for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0;
    __syncthreads();
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
      const unsigned k = keys[i];
      if ((k & mask) == prefix) atomicAdd(&hist[(k >> shift) & 0xFF], 1u);
    }
    __syncthreads();
    __shared__ unsigned sel_digit;
    __shared__ long long sel_r;
    if (threadIdx.x == 0) {
      long long acc = 0;
      int d = 0;
      for (; d < 256; ++d) {
        if (acc + hist[d] > r) break;
        acc += hist[d];
      }
      sel_digit = (unsigned)(d < 256 ? d : 255);
      sel_r = r - acc;
    }
    __syncthreads();
    prefix |= sel_digit << shift;
    mask |= 0xFFu << shift;
    r = sel_r;
    __syncthreads();
  }
  return prefix;
}

// The overflow rule over the whole selection, by one block (any multiple of
// 32 threads up to 1024): batch by batch of parents, the passing children are
// appended while they fit, otherwise prune_on_overload raises the threshold.
// Writes ids[0 .. *n_out) and the final threshold.
__device__ void select_overflow_block(const float* __restrict__ scores,
                                      const int64_t* __restrict__ offsets, int64_t n_parents,
                                      int64_t batch, double thr, int64_t cap,
                                      int64_t* __restrict__ ids, int64_t* n_out,
                                      double* __restrict__ thr_out,
                                      int64_t* __restrict__ tmp_ids,
                                      unsigned* __restrict__ keys) {
  __shared__ int wsum[33];
  __shared__ unsigned hist[256];
  __shared__ long long vs_sh;
  __shared__ double cur_sh;
  const int nthr = blockDim.x;  // the loops stride by the block
  if (threadIdx.x == 0) {
    vs_sh = 0;
    cur_sh = thr;
  }
  __syncthreads();
  for (int64_t p0 = 0; p0 < n_parents; p0 += batch) {
    const int64_t p1 = std::min(p0 + batch, n_parents);
    const int64_t c_lo = offsets[p0], c_hi = offsets[p1];
    if (c_hi == c_lo) continue;
    const double eff_in = fmax(thr, cur_sh);
    // pass 1: count passing children of the batch
    int64_t m = 0;
    for (int64_t base = c_lo; base < c_hi; base += nthr) {
      const int64_t c = base + threadIdx.x;
      const int f = (c < c_hi && (double)scores[c] >= eff_in) ? 1 : 0;
      int tot;
      block_scan_flag(f, &tot, wsum);
      m += tot;
    }
    int64_t vs = vs_sh;
    if (m <= cap - vs) {  // fast path: append in order
      int64_t w = vs;
      for (int64_t base = c_lo; base < c_hi; base += nthr) {
        const int64_t c = base + threadIdx.x;
        const int f = (c < c_hi && (double)scores[c] >= eff_in) ? 1 : 0;
        int tot;
        const int off = block_scan_flag(f, &tot, wsum);
        if (f) ids[w + off] = c;
        w += tot;
      }
      if (threadIdx.x == 0) vs_sh = vs + m;
      __syncthreads();
      continue;
    }
    // prune_on_overload: keys of the current tree and of the passing batch
    int64_t w = vs;
    for (int64_t i = threadIdx.x; i < vs; i += nthr) keys[i] = float_key(scores[ids[i]]);
    for (int64_t base = c_lo; base < c_hi; base += nthr) {
      const int64_t c = base + threadIdx.x;
      const int f = (c < c_hi && (double)scores[c] >= eff_in) ? 1 : 0;
      int tot;
      const int off = block_scan_flag(f, &tot, wsum);
      if (f) {
        keys[w + off] = float_key(scores[c]);
        tmp_ids[w - vs + off] = c;
      }
      w += tot;
    }
    __syncthreads();
    const int64_t total = vs + m;
    const unsigned kth = block_select(keys, total, total - cap, hist);
    const unsigned mid = block_select(keys, total, total - total / 2 - 1, hist);
    double eff = cur_sh;
    const double tk = nextafter((double)key_float(kth), INFINITY);
    const double tm = nextafter((double)key_float(mid), INFINITY);
    eff = fmax(eff, fmax(tk, tm));
    // keep tree entries >= eff (stable)
    int64_t kept = 0;
    for (int64_t base = 0; base < vs; base += nthr) {
      const int64_t i = base + threadIdx.x;
      int64_t id = 0;
      int f = 0;
      if (i < vs) {
        id = ids[i];
        f = (double)scores[id] >= eff ? 1 : 0;
      }
      int tot;
      const int off = block_scan_flag(f, &tot, wsum);
      if (f) keys[kept + off] = (unsigned)(id & 0xFFFFFFFFu), tmp_ids[m + kept + off] = id;
      kept += tot;
    }
    __syncthreads();
    for (int64_t i = threadIdx.x; i < kept; i += nthr) ids[i] = tmp_ids[m + i];
    __syncthreads();
    // pending batch entries >= eff, in order, up to the free space
    const int64_t space = cap - kept;
    int64_t added = 0;
    for (int64_t base = 0; base < m; base += nthr) {
      const int64_t i = base + threadIdx.x;
      int64_t id = 0;
      int f = 0;
      if (i < m) {
        id = tmp_ids[i];
        f = (double)scores[id] >= eff ? 1 : 0;
      }
      int tot;
      const int off = block_scan_flag(f, &tot, wsum);
      if (f && added + off < space) ids[kept + added + off] = id;
      added += tot;
    }
    if (threadIdx.x == 0) {
      vs_sh = kept + std::min(added, space);
      cur_sh = eff;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *n_out = vs_sh;
    *thr_out = cur_sh;
  }
  __syncthreads();
}

// With cnt_dev (device counts: [0] parents) the plain selection's survivor
// count is pos[*n_in] (n_in: its inputs, the children): it is stored at
// *n_out, and the kernel does nothing more unless it exceeds cap (then
// *ovf_flag is set and the overflow rule rewrites the selection and *n_out).
// n_out points into the same counters, so neither pointer is restrict.
__global__ void __launch_bounds__(kSelThreads)
select_overflow_kernel(const float* __restrict__ scores, const int64_t* __restrict__ offsets,
                       int64_t n_parents, int64_t batch, double thr, int64_t cap,
                       int64_t* __restrict__ ids, int64_t* n_out,
                       double* __restrict__ thr_out, int64_t* __restrict__ tmp_ids,
                       unsigned* __restrict__ keys, const int64_t* cnt_dev,
                       int32_t* __restrict__ ovf_flag, const int64_t* __restrict__ pos,
                       const int64_t* n_in) {
  if (cnt_dev) {
    const int64_t n_sel = pos[*n_in];  // the selection's total over its n_in inputs
    n_parents = cnt_dev[0];
    __syncthreads();  // every thread has read the counters
    if (threadIdx.x == 0) *n_out = n_sel;
    if (n_sel <= cap) return;  // uniform over the block
    if (threadIdx.x == 0) *ovf_flag = 1;
  }
  select_overflow_block(scores, offsets, n_parents, batch, thr, cap, ids, n_out, thr_out, tmp_ids,
                        keys);
}

// ---------------------------------------------------------------------------
// emit: thread per survivor for the leaf, warp per 32 survivors for folds
// ---------------------------------------------------------------------------

// Survivors s0 .. s0 + 31 (those below n_surv) of one warp.
__device__ __forceinline__ void emit_tile(const LokiPruneLevel& D, const double* __restrict__ leaves,
                  const float* __restrict__ folds, const LokiBranchInfo* __restrict__ info,
                  const int64_t* __restrict__ offsets, int64_t n_parents,
                  const float* __restrict__ seg, const int64_t* __restrict__ surv,
                  int64_t n_surv, const float* __restrict__ cscores,
                  const int32_t* __restrict__ cidx, const double* __restrict__ cphase,
                  double* __restrict__ lout, float* __restrict__ fout,
                  float* __restrict__ sout, float* __restrict__ seout,
                  int32_t* __restrict__ bout, int64_t s0) {
  const int lane = threadIdx.x & 31;
  const int nb = D.nbins, P = D.poly_order, m = P + 1;
  const int kmax = (int)std::min<int64_t>(32, n_surv - s0);
  int64_t my_par = 0, my_row = 0;
  int my_shift = 0;
  if (lane < kmax) {
    const int64_t s = s0 + lane;
    const int64_t c = surv[s];
    const int64_t par = find_parent(offsets, n_parents, c);
    const LokiBranchInfo B = info[par];
    const double* lf = leaves + par * (P + 2) * 2;
    double pv[LOKI_MAX_PARAMS + 1], ev[LOKI_MAX_PARAMS + 1];
    child_params(B, P, c - offsets[par], pv);
    pv[P] = B.d0;
    for (int j = 0; j < P; ++j) ev[j] = B.dact[j];
    ev[P] = 0.0;
    double* lo = lout + s * (P + 2) * 2;
    if (D.moving) {
      for (int i = 0; i < m; ++i) lo[2 * i] = tdot(pv, D.tm_n, i, m);
      if (D.tiling == 0) {
        for (int i = 0; i < m; ++i) lo[2 * i + 1] = __dmul_rn(ev[i], fabs(D.tm_n[i][i]));
      } else if (D.tiling == 2) {
        for (int i = 0; i < m; ++i) lo[2 * i + 1] = tdot(ev, D.tm_e, i, m);
      } else {
        double e2[LOKI_MAX_PARAMS + 1];
        for (int j = 0; j < m; ++j) e2[j] = __dmul_rn(ev[j], ev[j]);
        for (int i = 0; i < m; ++i) lo[2 * i + 1] = __dsqrt_rn(tdot(e2, D.tm_e, i, m));
      }
    } else {
      for (int i = 0; i < m; ++i) {
        lo[2 * i] = pv[i];
        lo[2 * i + 1] = ev[i];
      }
    }
    lo[2 * m] = lf[2 * m];          // f0
    lo[2 * m + 1] = lf[2 * m + 1];  // basis flag
    const float sc = cscores[c];
    sout[s] = sc;
    seout[s] = sc;
    int32_t* bt = bout + s * (P + 2);
    const int ia = cidx[2 * c], iff = cidx[2 * c + 1];
    bt[0] = (int32_t)par;
    for (int j = 1; j < P + 1; ++j) bt[j] = 0;
    bt[D.nparams_ffa - 1] = ia;  // column 1 + (nparams_ffa - 2)
    bt[D.nparams_ffa] = iff;     // column 1 + (nparams_ffa - 1)
    bt[P + 1] = (int32_t)cphase[c];
    my_par = par;
    my_row = (int64_t)ia * D.n_freq + iff;
    my_shift = round_shift(cphase[c], nb);
  }
  if (nb == 64) {
    // four survivors' rows in flight per lane (bins lane and lane + 32)
    constexpr int kU = 4;
    for (int k0 = 0; k0 < kmax; k0 += kU) {
      float pe[kU][2], pw[kU][2], se[kU][2], sw[kU][2];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int k = k0 + u;
        const int src = k < kmax ? k : 0;
        const int64_t par = __shfl_sync(0xFFFFFFFFu, my_par, src);
        const int64_t row = __shfl_sync(0xFFFFFFFFu, my_row, src);
        const int sh = __shfl_sync(0xFFFFFFFFu, my_shift, src);
        if (k < kmax) {
          const float* pf = folds + par * 128;
          const float* sf = seg + row * 128;
#pragma unroll
          for (int c = 0; c < 2; ++c) {
            const int j = lane + 32 * c;
            const int js = (j - sh) & 63;
            pe[u][c] = __ldg(pf + j);
            pw[u][c] = __ldg(pf + 64 + j);
            se[u][c] = __ldg(sf + js);
            sw[u][c] = __ldg(sf + 64 + js);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int k = k0 + u;
        if (k >= kmax) break;
        float* o = fout + (s0 + k) * 128;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          o[lane + 32 * c] = __fadd_rn(pe[u][c], se[u][c]);
          o[64 + lane + 32 * c] = __fadd_rn(pw[u][c], sw[u][c]);
        }
      }
    }
    return;
  }
  for (int k = 0; k < kmax; ++k) {
    const int64_t par = __shfl_sync(0xFFFFFFFFu, my_par, k);
    const int64_t row = __shfl_sync(0xFFFFFFFFu, my_row, k);
    const int sh = __shfl_sync(0xFFFFFFFFu, my_shift, k);
    const float* pf = folds + par * 2 * nb;
    const float* sf = seg + row * 2 * nb;
    float* o = fout + (s0 + k) * 2 * nb;
    for (int j = lane; j < nb; j += 32) {
      int js = j - sh;
      js += (js < 0) ? nb : 0;
      o[j] = __fadd_rn(pf[j], sf[js]);
      o[nb + j] = __fadd_rn(pf[nb + j], sf[nb + js]);
    }
  }
}

__global__ void __launch_bounds__(kPruneWarps * 32)
prune_emit_kernel(LokiPruneLevel D, const double* __restrict__ leaves,
                  const float* __restrict__ folds, const LokiBranchInfo* __restrict__ info,
                  const int64_t* __restrict__ offsets, int64_t n_parents,
                  const float* __restrict__ seg, const int64_t* __restrict__ surv,
                  int64_t n_surv, const float* __restrict__ cscores,
                  const int32_t* __restrict__ cidx, const double* __restrict__ cphase,
                  double* __restrict__ lout, float* __restrict__ fout,
                  float* __restrict__ sout, float* __restrict__ seout,
                  int32_t* __restrict__ bout, const int64_t* __restrict__ cnt_dev) {
  const int warp = threadIdx.x >> 5;
  if (!cnt_dev) {
    const int64_t s0 = ((int64_t)blockIdx.x * kPruneWarps + warp) * 32;
    if (s0 < n_surv)
      emit_tile(D, leaves, folds, info, offsets, n_parents, seg, surv, n_surv, cscores, cidx,
                cphase, lout, fout, sout, seout, bout, s0);
    return;
  }
  // device counts: cnt_dev[0] parents, cnt_dev[2] survivors
  n_parents = cnt_dev[0];
  n_surv = cnt_dev[2];
  for (int64_t t = (int64_t)blockIdx.x * kPruneWarps + warp; t * 32 < n_surv;
       t += (int64_t)gridDim.x * kPruneWarps)
    emit_tile(D, leaves, folds, info, offsets, n_parents, seg, surv, n_surv, cscores, cidx,
              cphase, lout, fout, sout, seout, bout, t * 32);
}

// ---------------------------------------------------------------------------
// circular-orbit propagation, shared by the circular tree and its ascend
// ---------------------------------------------------------------------------

// get_circ_mask (core/circular.py:13-79): 1 snap-circular, 2 crackle-circular
// (the snap/accel hole), 0 Taylor.
__device__ __forceinline__ int circ_class(const double* v, const double* e, double sig) {
  const double crackle = v[0], snap = v[1], jerk = v[2], accel = v[3];
  const bool sig_snap = fabs(snap) > __dmul_rn(sig, e[1]);
  const bool sig_accel = fabs(accel) > __dmul_rn(sig, e[3]);
  const bool sig_jerk = fabs(jerk) > __dmul_rn(sig, e[2]);
  const bool snap_circ = sig_snap && sig_accel && __dmul_rn(-snap, accel) > 0.0;
  if (snap_circ) return 1;
  if (sig_jerk && __dmul_rn(-crackle, jerk) > 0.0) return 2;
  return 0;
}

// shift_taylor_circular_params (utils/transforms.py:246-299): closed-form
// circular-orbit propagation of [d5 .. d0] by dt (values only). cos and sin
// are CUDA's double-precision functions.
__device__ __forceinline__ void circ_shift(const double* p, double dt, bool hole, double* out) {
  const double d5 = p[0], d4 = p[1], d3 = p[2], d2 = p[3], d1 = p[4], d0 = p[5];
  const double wsq = hole ? __ddiv_rn(-d5, d3) : __ddiv_rn(-d4, d2);
  const double w = __dsqrt_rn(wsq);
  const double wdt = __dmul_rn(w, dt);
  const double c = cos(wdt), s = sin(wdt);
  const double d2j = __dadd_rn(__dmul_rn(d2, c), __dmul_rn(__ddiv_rn(d3, w), s));
  const double d3j = __dsub_rn(__dmul_rn(d3, c), __dmul_rn(__dmul_rn(d2, w), s));
  const double d1ci = __ddiv_rn(-d3, wsq);
  const double d1cj = __ddiv_rn(-d3j, wsq);
  const double e1 = __dsub_rn(d1, d1ci);
  const double d0cj = __ddiv_rn(-d2j, wsq);
  const double d0ci = __ddiv_rn(-d2, wsq);
  out[0] = __dmul_rn(-wsq, d3j);
  out[1] = __dmul_rn(-wsq, d2j);
  out[2] = d3j;
  out[3] = d2j;
  out[4] = __dadd_rn(d1cj, e1);
  out[5] = __dadd_rn(__dadd_rn(d0cj, __dsub_rn(d0, d0ci)), __dmul_rn(e1, dt));
}

// ---------------------------------------------------------------------------
// ascend: warp per 32 survivors, segments accumulated in order
// ---------------------------------------------------------------------------

// Survivors s0 .. s0 + 31 (those below n) of one warp; acc and tile are the
// warp's accumulators (32 x 2 nb) and score tile.
__device__ __forceinline__ void ascend_tile(const LokiPruneLevel& D, const double* __restrict__ leaves,
                    float* __restrict__ folds, float* __restrict__ scores,
                    float* __restrict__ scores_ep, int64_t n, int nseg,
                    const double* __restrict__ tm_seg, const double* __restrict__ dt_seg,
                    const int32_t* __restrict__ seg_idx, const float* __restrict__ ffa,
                    int64_t seg_stride, const LokiScoreSpec& sp, const ScoreK& SK, float* acc,
                    float* tile, int64_t s0) {
  const int lane = threadIdx.x & 31;
  const int nb = D.nbins, P = D.poly_order, m = P + 1;
  const int stride = score_stride(nb, sp.wmax);
  const int kmax = (int)std::min<int64_t>(32, n - s0);
  for (int k = 0; k < kmax; ++k)
    for (int j = lane; j < 2 * nb; j += 32) acc[k * 2 * nb + j] = 0.0f;
  double pv[LOKI_MAX_PARAMS + 1];
  double f0 = 1.0;
  int cls = 0;  // circular tree: class of the survivor (core/circular.py:597-666)
  if (lane < kmax) {
    const double* lf = leaves + (s0 + lane) * (P + 2) * 2;
    double ev[LOKI_MAX_PARAMS + 1];
    for (int i = 0; i < m; ++i) {
      pv[i] = lf[2 * i];
      ev[i] = lf[2 * i + 1];
    }
    f0 = lf[2 * m];
    if (D.basis == 2) cls = circ_class(pv, ev, D.circ_sig_prop);
  }
  __syncwarp();
  for (int sg = 0; sg < nseg; ++sg) {
    const double(*T)[LOKI_MAX_PARAMS + 1] =
        reinterpret_cast<const double(*)[LOKI_MAX_PARAMS + 1]>(tm_seg + sg * 36);
    int64_t my_row = 0;
    int my_shift = 0;
    if (lane < kmax) {
      double accel, vel, dd;
      if (D.basis == 1) {  // core/chebyshev.py:280-320: shift to t0_seg, then Taylor
        double a[LOKI_MAX_PARAMS + 1];
        for (int i = 0; i < m; ++i) a[i] = tdot(pv, T, i, m);
        cheby_low3(D, a, m, &accel, &vel, &dd);
      } else if (cls != 0) {  // circular survivors: closed-form propagation
        double a[6];
        circ_shift(pv, dt_seg[sg], cls == 2, a);
        accel = a[3];
        vel = a[4];
        dd = a[5];
      } else {
        accel = tdot(pv, T, P - 2, m);
        vel = tdot(pv, T, P - 1, m);
        dd = tdot(pv, T, P, m);
      }
      const double freq = __dmul_rn(f0, __dsub_rn(1.0, __ddiv_rn(vel, LOKI_C_VAL)));
      const double delay = __ddiv_rn(dd, LOKI_C_VAL);
      const double ph = phase_idx(dt_seg[sg], f0, nb, delay);
      const int64_t ia = axis_index(accel, D.accel_min, D.accel_inv, D.n_accel);
      const int64_t iff = axis_index(freq, D.freq_min, D.freq_inv, D.n_freq);
      my_row = ia * D.n_freq + iff;
      my_shift = round_shift(ph, nb);
    }
    const float* fseg = ffa + (int64_t)seg_idx[sg] * seg_stride;
    if (nb == 64) {
      // eight survivors' segment rows in flight per lane (bins lane, lane + 32)
      constexpr int kU = 8;
      for (int k0 = 0; k0 < kmax; k0 += kU) {
        float se[kU][2], sw[kU][2];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int k = k0 + u;
          const int src = k < kmax ? k : 0;
          const int64_t row = __shfl_sync(0xFFFFFFFFu, my_row, src);
          const int sh = __shfl_sync(0xFFFFFFFFu, my_shift, src);
          if (k < kmax) {
            const float* sf = fseg + row * 128;
#pragma unroll
            for (int c = 0; c < 2; ++c) {
              const int js = (lane + 32 * c - sh) & 63;
              se[u][c] = __ldg(sf + js);
              sw[u][c] = __ldg(sf + 64 + js);
            }
          }
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int k = k0 + u;
          if (k >= kmax) break;
          float* a = acc + k * 128;
#pragma unroll
          for (int c = 0; c < 2; ++c) {
            const int j = lane + 32 * c;
            a[j] = __fadd_rn(a[j], se[u][c]);
            a[64 + j] = __fadd_rn(a[64 + j], sw[u][c]);
          }
        }
      }
      continue;
    }
    for (int k = 0; k < kmax; ++k) {
      const int64_t row = __shfl_sync(0xFFFFFFFFu, my_row, k);
      const int sh = __shfl_sync(0xFFFFFFFFu, my_shift, k);
      const float* sf = fseg + row * 2 * nb;
      float* a = acc + k * 2 * nb;
      for (int j = lane; j < nb; j += 32) {
        int js = j - sh;
        js += (js < 0) ? nb : 0;
        a[j] = __fadd_rn(a[j], sf[js]);
        a[nb + j] = __fadd_rn(a[nb + j], sf[nb + js]);
      }
    }
  }
  __syncwarp();
  for (int k = 0; k < kmax; ++k) {
    const float* a = acc + k * 2 * nb;
    float* o = folds + (s0 + k) * 2 * nb;
    float* trow = tile + k * stride;
    for (int j = lane; j < nb; j += 32) {
      o[j] = a[j];
      o[nb + j] = a[nb + j];
      trow[j] = __fdiv_rn(a[j], __fsqrt_rn(a[nb + j]));
    }
  }
  __syncwarp();
  if (lane < kmax) {
    scores_ep[s0 + lane] = scores[s0 + lane];
    float s;
    float* row = tile + lane * stride;
    if (SK.pow2_64) score_row64_pow2(row, sp, SK, &s);
    else score_row(row, nb, sp, &s);
    scores[s0 + lane] = s;
  }
}

__global__ void __launch_bounds__(kPruneWarps * 32)
prune_ascend_kernel(LokiPruneLevel D, const double* __restrict__ leaves,
                    float* __restrict__ folds, float* __restrict__ scores,
                    float* __restrict__ scores_ep, int64_t n, int nseg,
                    const double* __restrict__ tm_seg, const double* __restrict__ dt_seg,
                    const int32_t* __restrict__ seg_idx, const float* __restrict__ ffa,
                    int64_t seg_stride, LokiScoreSpec sp, ScoreK SK,
                    const int64_t* __restrict__ n_dev) {
  extern __shared__ float tiles[];
  const int warp = threadIdx.x >> 5;
  // per warp: the 32 accumulators (2 * nb each) followed by the score tile
  const int stride = score_stride(D.nbins, sp.wmax);
  float* acc = tiles + (size_t)warp * 32 * (2 * D.nbins + stride);
  float* tile = acc + 32 * 2 * D.nbins;
  if (!n_dev) {
    const int64_t s0 = ((int64_t)blockIdx.x * kPruneWarps + warp) * 32;
    if (s0 < n)
      ascend_tile(D, leaves, folds, scores, scores_ep, n, nseg, tm_seg, dt_seg, seg_idx, ffa,
                  seg_stride, sp, SK, acc, tile, s0);
    return;
  }
  n = *n_dev;  // survivors held on the device: warps stride over their tiles
  for (int64_t t = (int64_t)blockIdx.x * kPruneWarps + warp; t * 32 < n;
       t += (int64_t)gridDim.x * kPruneWarps) {
    ascend_tile(D, leaves, folds, scores, scores_ep, n, nseg, tm_seg, dt_seg, seg_idx, ffa,
                seg_stride, sp, SK, acc, tile, t * 32);
    __syncwarp();  // the accumulators are reused by the next tile
  }
}

// ---------------------------------------------------------------------------
// circular-orbit Taylor tree (core/circular.py, dynamic/dyn_circular_taylor.py)
//
// Leaves are [d5 (crackle), d4 (snap), d3, d2, d1, d0, (f0, flag)]. Children
// of one parent batch are ordered as the reference builds them: first every
// child that keeps the parent's crackle (cartesian order over the batch),
// then the children whose crackle is expanded, each expansion in crackle
// order. Physical validation drops children before scoring, so the scored
// list is the compacted list of valid children.
// ---------------------------------------------------------------------------

// One child of the circular tree: parent, index in the parent's cartesian
// product over d4..d1, and the crackle sub-index (-1: parent crackle kept).
struct CircChild {
  int32_t parent, cart, crackle, pad;
};

// circ_validate_batch (core/circular.py:82-124) for one child.
__device__ __forceinline__ bool circ_valid(const LokiPruneLevel& D, const double* v,
                                           const double* e) {
  const double snap = v[1], accel = v[3], sig = D.circ_sig_valid;
  const bool sig_snap = fabs(snap) > __dmul_rn(sig, e[1]);
  const bool sig_accel = fabs(accel) > __dmul_rn(sig, e[3]);
  if (!(sig_snap && sig_accel)) return true;
  if (!(__dmul_rn(-snap, accel) > 0.0)) return false;
  const double wsq = __ddiv_rn(-snap, accel);
  const double limit = __dmul_rn(D.circ_x_mass, pow(wsq, 2.0 / 3.0));
  return wsq <= D.circ_omega_max_sq && fabs(accel) <= limit;
}

// Parameters and errors of one circular child (core/circular.py:204-394).
__device__ __forceinline__ void circ_child(const LokiBranchInfo& B, const double* lf,
                                           const CircChild& ch, double* pv, double* ev) {
  const int P = 5;
  child_params(B, P, ch.cart, pv);
  pv[P] = B.d0;
  for (int j = 0; j < P; ++j) ev[j] = B.dact[j];
  ev[P] = 0.0;
  if (ch.crackle >= 0) {  // branch_param_padded on the parent crackle cell
    const double dact = B.dact[0];
    const double first = __dadd_rn(__dsub_rn(lf[0], __dmul_rn(lf[1], 0.5)),
                                   __dmul_rn(dact, 0.5));
    pv[0] = __dadd_rn(first, __dmul_rn((double)ch.crackle, dact));
  }
}

// Branch every parent (circ_taylor_branch_batch): per-parameter branching of
// d4..d1 as in the Taylor tree, crackle deferred; counts the children that
// keep the parent crackle and those produced by crackle expansion.
__device__ __forceinline__ void circ_branch_one(const LokiPruneLevel& D,
                                                const double* __restrict__ leaves, int64_t i,
                                                LokiBranchInfo* __restrict__ info,
                                                int64_t* __restrict__ n_keep,
                                                int64_t* __restrict__ n_exp,
                                                int32_t* __restrict__ err);

// n_dev, when not null, holds the parent count on the device (grid-stride).
__global__ void circ_branch_kernel(LokiPruneLevel D, const double* __restrict__ leaves,
                                   int64_t n, LokiBranchInfo* __restrict__ info,
                                   int64_t* __restrict__ n_keep, int64_t* __restrict__ n_exp,
                                   int32_t* __restrict__ err, const int64_t* __restrict__ n_dev) {
  if (n_dev) {
    n = *n_dev;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
      circ_branch_one(D, leaves, i, info, n_keep, n_exp, err);
    return;
  }
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) circ_branch_one(D, leaves, i, info, n_keep, n_exp, err);
}

__device__ __forceinline__ void circ_branch_one(const LokiPruneLevel& D,
                                                const double* __restrict__ leaves, int64_t i,
                                                LokiBranchInfo* __restrict__ info,
                                                int64_t* __restrict__ n_keep,
                                                int64_t* __restrict__ n_exp,
                                                int32_t* __restrict__ err) {
  const int P = 5;
  const double* lf = leaves + i * (P + 2) * 2;
  const double f0 = lf[(P + 1) * 2];
  const double fscale = __ddiv_rn(f0, LOKI_C_VAL);
  LokiBranchInfo B;
  B.d0 = lf[2 * P];
  bool needs0 = false;
  int64_t num_c = 1;
  int64_t total = 1;
  for (int j = 0; j < P; ++j) {
    const double pcur = lf[2 * j], dcur = lf[2 * j + 1];
    const double dnew = __ddiv_rn(D.dfc[j], f0);
    const double fb = __dmul_rn(D.fac[j], fscale);
    const double shift = __dmul_rn(fabs(__dsub_rn(dcur, dnew)), fb);
    const bool needs = shift >= D.eta_m;
    int64_t num = 1;
    double dact = dcur, first = pcur;
    if (!(dcur > 0.0) || !(dnew > 0.0)) {
      atomicOr(err, LOKI_DEVERR_BRANCH);
    } else {
      const double ratio = __ddiv_rn(dcur, dnew);
      num = (int64_t)ceil(__dsub_rn(ratio, LOKI_FLOAT_EPSILON));
      if (num < 1) num = 1;
      if (num > D.branch_max) {
        atomicOr(err, LOKI_DEVERR_BRANCH);
        num = D.branch_max;
      }
      dact = __ddiv_rn(dcur, (double)num);
      first = __dadd_rn(__dsub_rn(pcur, __dmul_rn(dcur, 0.5)), __dmul_rn(dact, 0.5));
    }
    if (j == 0) {  // crackle keeps the parent value; its step is the would-be child step
      needs0 = needs;
      num_c = num;
      first = pcur;
      num = 1;
    }
    if (!needs) {
      num = 1;
      dact = dcur;
      first = pcur;
    }
    B.first[j] = first;
    B.dact[j] = dact;
    B.count[j] = (int32_t)num;
    total *= num;
  }
  B.reserved = needs0 ? (int32_t)num_c : 0;
  // first cartesian product: which children fall in the hole and expand crackle
  const double sig = D.circ_sig_prop;
  int64_t keep = 0, exp = 0;
  double pv[LOKI_MAX_PARAMS + 1];
  for (int64_t k = 0; k < total; ++k) {
    child_params(B, P, k, pv);
    const double snap = pv[1], jerk = pv[2], accel = pv[3];
    const bool snap_circ = fabs(snap) > __dmul_rn(sig, B.dact[1]) &&
                           fabs(accel) > __dmul_rn(sig, B.dact[3]) &&
                           __dmul_rn(-snap, accel) > 0.0;
    const bool expand = !snap_circ && fabs(jerk) > __dmul_rn(sig, B.dact[2]) && needs0;
    if (expand) exp += num_c;
    else ++keep;
  }
  info[i] = B;
  n_keep[i] = keep;
  n_exp[i] = exp;
}

// Children of every parent at their batch-ordered positions, plus a validity
// flag (1.0 / 0.0) per child for the compaction.
__device__ __forceinline__ void circ_map_one(const LokiPruneLevel& D,
                                             const double* __restrict__ leaves, int64_t n,
                                             int64_t batch, const LokiBranchInfo* __restrict__ info,
                                             const int64_t* __restrict__ keep_off,
                                             const int64_t* __restrict__ exp_off,
                                             CircChild* __restrict__ map,
                                             float* __restrict__ validf, int64_t i);

// With cnt (device counts) the parents are cnt[0] and the children
// keep_off[n] + exp_off[n]; block 0 records the children in cnt[1] and the
// level's statistics, and above child_cap the level gets none (flagged).
__global__ void circ_map_kernel(LokiPruneLevel D, const double* __restrict__ leaves, int64_t n,
                                int64_t batch, const LokiBranchInfo* __restrict__ info,
                                const int64_t* __restrict__ keep_off,
                                const int64_t* __restrict__ exp_off,
                                CircChild* __restrict__ map, float* __restrict__ validf,
                                int64_t* cnt, int64_t child_cap, LokiPruneLevelStats* st,
                                int32_t* err) {
  if (cnt) {
    n = cnt[0];
    const int64_t total = keep_off[n] + exp_off[n];
    const bool fits = total <= child_cap;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      cnt[1] = fits ? total : 0;
      st->n_parents = n;
      st->n_children = total;
      if (!fits) atomicOr(err, LOKI_DEVERR_CAPACITY);
    }
    if (!fits) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
      circ_map_one(D, leaves, n, batch, info, keep_off, exp_off, map, validf, i);
    return;
  }
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) circ_map_one(D, leaves, n, batch, info, keep_off, exp_off, map, validf, i);
}

__device__ __forceinline__ void circ_map_one(const LokiPruneLevel& D,
                                             const double* __restrict__ leaves, int64_t n,
                                             int64_t batch, const LokiBranchInfo* __restrict__ info,
                                             const int64_t* __restrict__ keep_off,
                                             const int64_t* __restrict__ exp_off,
                                             CircChild* __restrict__ map,
                                             float* __restrict__ validf, int64_t i) {
  const int P = 5;
  const int64_t b0 = (i / batch) * batch, b1 = std::min(b0 + batch, n);
  int64_t pk = keep_off[i] + exp_off[b0];
  int64_t pe = keep_off[b1] + exp_off[i];
  const LokiBranchInfo B = info[i];
  const double* lf = leaves + i * (P + 2) * 2;
  const int64_t num_c = B.reserved;
  int64_t total = 1;
  for (int j = 0; j < P; ++j) total *= B.count[j];
  const double sig = D.circ_sig_prop;
  double pv[LOKI_MAX_PARAMS + 1], ev[LOKI_MAX_PARAMS + 1];
  for (int64_t k = 0; k < total; ++k) {
    CircChild ch = {(int32_t)i, (int32_t)k, -1, 0};
    circ_child(B, lf, ch, pv, ev);
    const double snap = pv[1], jerk = pv[2], accel = pv[3];
    const bool snap_circ = fabs(snap) > __dmul_rn(sig, ev[1]) &&
                           fabs(accel) > __dmul_rn(sig, ev[3]) &&
                           __dmul_rn(-snap, accel) > 0.0;
    const bool expand = !snap_circ && fabs(jerk) > __dmul_rn(sig, ev[2]) && num_c > 0;
    const float ok = circ_valid(D, pv, ev) ? 1.0f : 0.0f;  // crackle does not enter
    if (!expand) {
      map[pk] = ch;
      validf[pk] = ok;
      ++pk;
    } else {
      for (int64_t c = 0; c < num_c; ++c) {
        ch.crackle = (int32_t)c;
        map[pe] = ch;
        validf[pe] = ok;
        ++pe;
      }
    }
  }
}

// Position of the first valid child at or after child index c.
__device__ __forceinline__ int64_t lower_bound64(const int64_t* a, int64_t n, int64_t c) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (a[mid] < c) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Valid-child offsets at parent-batch boundaries (for the overflow rule).
__global__ void circ_boff_kernel(const int64_t* __restrict__ keep_off,
                                 const int64_t* __restrict__ exp_off, int64_t n,
                                 const int64_t* __restrict__ valid_ids, int64_t n_valid,
                                 int64_t* __restrict__ boff, const int64_t* __restrict__ cnt) {
  if (cnt) {  // device counts: cnt[0] parents, cnt[4] valid children
    n = cnt[0];
    n_valid = cnt[4];
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p <= n;
         p += (int64_t)gridDim.x * blockDim.x)
      boff[p] = lower_bound64(valid_ids, n_valid, keep_off[p] + exp_off[p]);
    return;
  }
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p > n) return;
  boff[p] = lower_bound64(valid_ids, n_valid, keep_off[p] + exp_off[p]);
}

// Resolve (circ_taylor_resolve_batch / circ_taylor_fixed_resolve_batch) of
// one valid child; returns its class.
__device__ __forceinline__ int circ_resolve(const LokiPruneLevel& D, const double* pv,
                                            const double* ev, double f0, ChildRes* r) {
  const int m = 6;
  const int cls = circ_class(pv, ev, D.circ_sig_prop);
  double accel, vel, dd;
  if (cls != 0) {
    double a[6], b[6];
    circ_shift(pv, D.circ_dt_add, cls == 2, a);
    accel = a[3];
    if (D.moving) {
      circ_shift(pv, D.circ_dt_init, cls == 2, b);
      vel = __dsub_rn(a[4], b[4]);
      dd = __dsub_rn(a[5], b[5]);
    } else {
      vel = a[4];
      dd = a[5];
    }
  } else if (D.moving) {
    accel = tdot(pv, D.tm_a, 3, m);
    vel = __dsub_rn(tdot(pv, D.tm_a, 4, m), tdot(pv, D.tm_i, 4, m));
    dd = __dsub_rn(tdot(pv, D.tm_a, 5, m), tdot(pv, D.tm_i, 5, m));
  } else {
    accel = tdot(pv, D.tm_a, 3, m);
    vel = tdot(pv, D.tm_a, 4, m);
    dd = tdot(pv, D.tm_a, 5, m);
  }
  const double freq = __dmul_rn(f0, __dsub_rn(1.0, __ddiv_rn(vel, LOKI_C_VAL)));
  const double delay = __ddiv_rn(dd, LOKI_C_VAL);
  r->phase = phase_idx(D.dt_phase, f0, D.nbins, delay);
  r->ia = (int32_t)axis_index(accel, D.accel_min, D.accel_inv, D.n_accel);
  r->iff = (int32_t)axis_index(freq, D.freq_min, D.freq_inv, D.n_freq);
  return cls;
}

// Valid children v0 .. v0 + 31 (those below n_valid) of one warp.
__device__ __forceinline__ void circ_score_tile(const LokiPruneLevel& D, const double* __restrict__ leaves,
                  const float* __restrict__ folds, int64_t batch,
                  const LokiBranchInfo* __restrict__ info, const CircChild* __restrict__ map,
                  const int64_t* __restrict__ valid_ids, int64_t n_valid,
                  const float* __restrict__ seg, const LokiScoreSpec& sp, const ScoreK& SK,
                  float* __restrict__ scores, int32_t* __restrict__ cidx,
                  double* __restrict__ cphase, int8_t* __restrict__ ccls,
                  int32_t* __restrict__ batch_taylor, unsigned* __restrict__ minmax_keys,
                  float* tile, int64_t v0) {
  const int lane = threadIdx.x & 31;
  const int nb = D.nbins, P = 5;
  const int stride = score_stride(nb, sp.wmax);
  const int kmax = (int)std::min<int64_t>(32, n_valid - v0);
  int64_t my_par = 0, my_row = 0;
  int my_shift = 0;
  if (lane < kmax) {
    const int64_t v = v0 + lane;
    const CircChild ch = map[valid_ids[v]];
    const LokiBranchInfo B = info[ch.parent];
    const double* lf = leaves + (int64_t)ch.parent * (P + 2) * 2;
    double pv[6], ev[6];
    circ_child(B, lf, ch, pv, ev);
    ChildRes r;
    const int cls = circ_resolve(D, pv, ev, lf[(P + 1) * 2], &r);
    if (cls == 0) atomicOr(batch_taylor + ch.parent / batch, 1);
    cidx[2 * v] = r.ia;
    cidx[2 * v + 1] = r.iff;
    cphase[v] = r.phase;
    ccls[v] = (int8_t)cls;
    my_par = ch.parent;
    my_row = (int64_t)r.ia * D.n_freq + r.iff;
    my_shift = round_shift(r.phase, nb);
  }
  for (int k = 0; k < kmax; ++k) {
    const int64_t par = __shfl_sync(0xFFFFFFFFu, my_par, k);
    const int64_t row = __shfl_sync(0xFFFFFFFFu, my_row, k);
    const int sh = __shfl_sync(0xFFFFFFFFu, my_shift, k);
    const float* pf = folds + par * 2 * nb;
    const float* sf = seg + row * 2 * nb;
    float* trow = tile + k * stride;
    for (int j = lane; j < nb; j += 32) {
      int js = j - sh;
      js += (js < 0) ? nb : 0;
      const float e = __fadd_rn(pf[j], sf[js]);
      const float vv = __fadd_rn(pf[nb + j], sf[nb + js]);
      trow[j] = __fdiv_rn(e, __fsqrt_rn(vv));
    }
  }
  __syncwarp();
  if (lane < kmax) {
    float* row = tile + lane * stride;
    float s;
    if (SK.pow2_64) score_row64_pow2(row, sp, SK, &s);
    else score_row(row, nb, sp, &s);
    scores[v0 + lane] = s;
    if (s == s) {
      atomicMin(minmax_keys, float_key(s));
      atomicMax(minmax_keys + 1, float_key(s));
    }
  }
}

// With cnt (device counts) the valid children are pos_v[cnt[1]] (the
// validity compaction's total); block 0 records them in cnt[4] and st.
__global__ void __launch_bounds__(kPruneWarps * 32)
circ_score_kernel(LokiPruneLevel D, const double* __restrict__ leaves,
                  const float* __restrict__ folds, int64_t batch,
                  const LokiBranchInfo* __restrict__ info, const CircChild* __restrict__ map,
                  const int64_t* __restrict__ valid_ids, int64_t n_valid,
                  const float* __restrict__ seg, LokiScoreSpec sp, ScoreK SK,
                  float* __restrict__ scores, int32_t* __restrict__ cidx,
                  double* __restrict__ cphase, int8_t* __restrict__ ccls,
                  int32_t* __restrict__ batch_taylor, unsigned* __restrict__ minmax_keys,
                  int64_t* cnt, const int64_t* __restrict__ pos_v, LokiPruneLevelStats* st) {
  extern __shared__ float tiles[];
  const int warp = threadIdx.x >> 5;
  float* tile = tiles + (size_t)warp * 32 * score_stride(D.nbins, sp.wmax);
  if (!cnt) {
    const int64_t v0 = ((int64_t)blockIdx.x * kPruneWarps + warp) * 32;
    if (v0 < n_valid)
      circ_score_tile(D, leaves, folds, batch, info, map, valid_ids, n_valid, seg, sp, SK,
                      scores, cidx, cphase, ccls, batch_taylor, minmax_keys, tile, v0);
    return;
  }
  n_valid = pos_v[cnt[1]];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cnt[4] = n_valid;
    st->n_valid = n_valid;
  }
  for (int64_t t = (int64_t)blockIdx.x * kPruneWarps + warp; t * 32 < n_valid;
       t += (int64_t)gridDim.x * kPruneWarps) {
    circ_score_tile(D, leaves, folds, batch, info, map, valid_ids, n_valid, seg, sp, SK, scores,
                    cidx, cphase, ccls, batch_taylor, minmax_keys, tile, t * 32);
    __syncwarp();
  }
}

// New tree from the survivors: circ_taylor_transform_batch
// (core/circular.py:669-705, moving grid), the basis flag written by the
// moving-grid resolve (core/circular.py:478-509: 1 snap, 2 crackle, and 0 for
// the crackle children of a batch that also holds Taylor children), backtracks
// and folds.
// Survivors s0 .. s0 + 31 (those below n_surv) of one warp.
__device__ __forceinline__ void circ_emit_tile(const LokiPruneLevel& D, const double* __restrict__ leaves,
                 const float* __restrict__ folds, int64_t batch,
                 const LokiBranchInfo* __restrict__ info, const CircChild* __restrict__ map,
                 const int64_t* __restrict__ valid_ids, const float* __restrict__ seg,
                 const int64_t* __restrict__ surv, int64_t n_surv,
                 const float* __restrict__ cscores, const int32_t* __restrict__ cidx,
                 const double* __restrict__ cphase, const int8_t* __restrict__ ccls,
                 const int32_t* __restrict__ batch_taylor, double* __restrict__ lout,
                 float* __restrict__ fout, float* __restrict__ sout,
                 float* __restrict__ seout, int32_t* __restrict__ bout, int64_t s0) {
  const int lane = threadIdx.x & 31;
  const int nb = D.nbins, P = 5, m = 6;
  const int kmax = (int)std::min<int64_t>(32, n_surv - s0);
  int64_t my_par = 0, my_row = 0;
  int my_shift = 0;
  if (lane < kmax) {
    const int64_t s = s0 + lane;
    const int64_t v = surv[s];
    const CircChild ch = map[valid_ids[v]];
    const LokiBranchInfo B = info[ch.parent];
    const double* lf = leaves + (int64_t)ch.parent * (P + 2) * 2;
    double pv[6], ev[6];
    circ_child(B, lf, ch, pv, ev);
    const int cls = ccls[v];
    double* lo = lout + s * (P + 2) * 2;
    double flag = lf[2 * m + 1];
    if (D.moving) {
      if (cls == 1) flag = 1.0;
      else if (cls == 2) flag = batch_taylor[ch.parent / batch] ? 0.0 : 2.0;
      if (cls != 0) {
        double o[6];
        circ_shift(pv, D.circ_dt_next, cls == 2, o);
        for (int i = 0; i < m; ++i) {
          lo[2 * i] = o[i];
          lo[2 * i + 1] = ev[i];
        }
      } else {
        for (int i = 0; i < m; ++i) lo[2 * i] = tdot(pv, D.tm_n, i, m);
        if (D.tiling == 0) {
          for (int i = 0; i < m; ++i) lo[2 * i + 1] = __dmul_rn(ev[i], fabs(D.tm_n[i][i]));
        } else if (D.tiling == 2) {
          for (int i = 0; i < m; ++i) lo[2 * i + 1] = tdot(ev, D.tm_e, i, m);
        } else {
          double e2[6];
          for (int j = 0; j < m; ++j) e2[j] = __dmul_rn(ev[j], ev[j]);
          for (int i = 0; i < m; ++i) lo[2 * i + 1] = __dsqrt_rn(tdot(e2, D.tm_e, i, m));
        }
      }
    } else {
      for (int i = 0; i < m; ++i) {
        lo[2 * i] = pv[i];
        lo[2 * i + 1] = ev[i];
      }
    }
    lo[2 * m] = lf[2 * m];
    lo[2 * m + 1] = flag;
    const float sc = cscores[v];
    sout[s] = sc;
    seout[s] = sc;
    int32_t* bt = bout + s * (P + 2);
    const int ia = cidx[2 * v], iff = cidx[2 * v + 1];
    bt[0] = ch.parent;
    for (int j = 1; j < P + 1; ++j) bt[j] = 0;
    bt[D.nparams_ffa - 1] = ia;
    bt[D.nparams_ffa] = iff;
    bt[P + 1] = (int32_t)cphase[v];
    my_par = ch.parent;
    my_row = (int64_t)ia * D.n_freq + iff;
    my_shift = round_shift(cphase[v], nb);
  }
  for (int k = 0; k < kmax; ++k) {
    const int64_t par = __shfl_sync(0xFFFFFFFFu, my_par, k);
    const int64_t row = __shfl_sync(0xFFFFFFFFu, my_row, k);
    const int sh = __shfl_sync(0xFFFFFFFFu, my_shift, k);
    const float* pf = folds + par * 2 * nb;
    const float* sf = seg + row * 2 * nb;
    float* o = fout + (s0 + k) * 2 * nb;
    for (int j = lane; j < nb; j += 32) {
      int js = j - sh;
      js += (js < 0) ? nb : 0;
      o[j] = __fadd_rn(pf[j], sf[js]);
      o[nb + j] = __fadd_rn(pf[nb + j], sf[nb + js]);
    }
  }
}

__global__ void __launch_bounds__(kPruneWarps * 32)
circ_emit_kernel(LokiPruneLevel D, const double* __restrict__ leaves,
                 const float* __restrict__ folds, int64_t batch,
                 const LokiBranchInfo* __restrict__ info, const CircChild* __restrict__ map,
                 const int64_t* __restrict__ valid_ids, const float* __restrict__ seg,
                 const int64_t* __restrict__ surv, int64_t n_surv,
                 const float* __restrict__ cscores, const int32_t* __restrict__ cidx,
                 const double* __restrict__ cphase, const int8_t* __restrict__ ccls,
                 const int32_t* __restrict__ batch_taylor, double* __restrict__ lout,
                 float* __restrict__ fout, float* __restrict__ sout,
                 float* __restrict__ seout, int32_t* __restrict__ bout,
                 const int64_t* __restrict__ cnt) {
  const int warp = threadIdx.x >> 5;
  if (!cnt) {
    const int64_t s0 = ((int64_t)blockIdx.x * kPruneWarps + warp) * 32;
    if (s0 < n_surv)
      circ_emit_tile(D, leaves, folds, batch, info, map, valid_ids, seg, surv, n_surv, cscores,
                     cidx, cphase, ccls, batch_taylor, lout, fout, sout, seout, bout, s0);
    return;
  }
  n_surv = cnt[2];  // device counts: warps stride over the survivors' tiles
  for (int64_t t = (int64_t)blockIdx.x * kPruneWarps + warp; t * 32 < n_surv;
       t += (int64_t)gridDim.x * kPruneWarps)
    circ_emit_tile(D, leaves, folds, batch, info, map, valid_ids, seg, surv, n_surv, cscores,
                   cidx, cphase, ccls, batch_taylor, lout, fout, sout, seout, bout, t * 32);
}

// ---------------------------------------------------------------------------
// complex (Fourier) folds: PrunePolyTaylorComplexDPFuncts and the Chebyshev
// counterpart. Tree folds and FFA segment rows are (2, nbf) complex64, nbf =
// nbins / 2 + 1 (float2 re, im). One lane owns one child: it rotates the
// segment row with the phasor recurrence of shift_add_complex_batch
// (core/common.py:403-429), adds the parent fold, and scores the irfft of the
// sum (detection/scoring.py:285-292).
// ---------------------------------------------------------------------------

// Phasor step exp(-2 pi i shift / nbins) with the reference's float32 angle
// float32(-2 * float32(pi)) * float32(shift) / nbins.
__device__ __forceinline__ float2 prune_phasor(double phase, int nbins) {
  const float m2pi = -2.0f * (float)3.14159265358979323846;
  const float ang = __fdiv_rn(__fmul_rn(m2pi, (float)phase), (float)nbins);
  float sn, cs;
  sincosf(ang, &sn, &cs);
  return make_float2(cs, sn);
}

__device__ __forceinline__ float2 cmul_rn(float2 a, float2 b) {
  return make_float2(__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                     __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}

// comb = seg * phasor^k + par, both components (par may be null: seg only).
__device__ __forceinline__ void rotate_add(const float2* __restrict__ seg,
                                           const float2* __restrict__ par, float2 delta, int nbf,
                                           float2* __restrict__ comb) {
  for (int c = 0; c < 2; ++c) {
    float2 ph = make_float2(1.0f, 0.0f);
    for (int k = 0; k < nbf; ++k) {
      const float2 r = cmul_rn(seg[c * nbf + k], ph);
      const float2 p = par ? par[c * nbf + k] : make_float2(0.0f, 0.0f);
      comb[c * nbf + k] = make_float2(__fadd_rn(r.x, p.x), __fadd_rn(r.y, p.y));
      ph = cmul_rn(ph, delta);
    }
  }
}

// irfft (n = nbins, even) of both components, then e / sqrt(v) into row.
// tw holds cos, then sin, of 2 pi t / nbins (float32 of the exact value).
__device__ __forceinline__ void irfft_norm(const float2* __restrict__ comb, int nbins, int nbf,
                                           const float* __restrict__ tw, float* row) {
  const float inv = 1.0f / (float)nbins;
  for (int j = 0; j < nbins; ++j) {
    float x[2];
    for (int c = 0; c < 2; ++c) {
      const float2* X = comb + c * nbf;
      float acc = X[0].x;
      const float nyq = X[nbf - 1].x;
      acc = (j & 1) ? __fsub_rn(acc, nyq) : __fadd_rn(acc, nyq);
      int idx = 0;
      for (int m = 1; m < nbf - 1; ++m) {
        idx += j;
        if (idx >= nbins) idx -= nbins;
        const float t = __fsub_rn(__fmul_rn(X[m].x, tw[idx]), __fmul_rn(X[m].y, tw[nbins + idx]));
        acc = __fadd_rn(acc, __fmul_rn(2.0f, t));
      }
      x[c] = __fmul_rn(acc, inv);
    }
    row[j] = __fdiv_rn(x[0], __fsqrt_rn(x[1]));
  }
}

__device__ __forceinline__ void load_twiddles(float* tw, int nbins) {
  for (int t = threadIdx.x; t < nbins; t += blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)t / (double)nbins, &s, &c);
    tw[t] = (float)c;
    tw[nbins + t] = (float)s;
  }
}

// Per-warp shared memory of the complex kernels: 32 lanes x (2, nbf) float2
// sums, then the 32-row score tile.
__host__ __device__ inline size_t cplx_warp_floats(int nbins, int stride) {
  return (size_t)32 * 2 * (nbins / 2 + 1) * 2 + (size_t)32 * stride;
}

// One child of the complex tree: resolve, rotate-add the segment row onto the
// parent fold, score the sum through its irfft (comb and trow: this lane's
// scratch, tw: the block's twiddles).
__device__ __forceinline__ void score_child_complex(
    const LokiPruneLevel& D, const double* __restrict__ leaves, const float2* __restrict__ folds,
    int64_t n_parents, const LokiBranchInfo* __restrict__ info,
    const int64_t* __restrict__ offsets, const float2* __restrict__ seg, const LokiScoreSpec& sp,
    float* __restrict__ scores, int32_t* __restrict__ cidx, double* __restrict__ cphase,
    unsigned* __restrict__ minmax_keys, const float* tw, float2* comb, float* trow, int64_t c) {
  const int nb = D.nbins, nbf = nb / 2 + 1, P = D.poly_order;
  const int64_t par = find_parent(offsets, n_parents, c);
  const LokiBranchInfo B = info[par];
  const double* lf = leaves + par * (P + 2) * 2;
  double pv[LOKI_MAX_PARAMS + 1];
  child_params(B, P, c - offsets[par], pv);
  pv[P] = B.d0;
  const ChildRes r = resolve_child(D, pv, lf[(P + 1) * 2]);
  cidx[2 * c] = r.ia;
  cidx[2 * c + 1] = r.iff;
  cphase[c] = r.phase;
  const int64_t row = (int64_t)r.ia * D.n_freq + r.iff;
  rotate_add(seg + row * 2 * nbf, folds + par * 2 * nbf, prune_phasor(r.phase, nb), nbf, comb);
  irfft_norm(comb, nb, nbf, tw, trow);
  float s;
  score_row(trow, nb, sp, &s);
  scores[c] = s;
  if (s == s) {
    atomicMin(minmax_keys, float_key(s));
    atomicMax(minmax_keys + 1, float_key(s));
  }
}

__global__ void __launch_bounds__(kPruneWarps * 32)
prune_score_complex_kernel(LokiPruneLevel D, const double* __restrict__ leaves,
                           const float2* __restrict__ folds, int64_t n_parents,
                           const LokiBranchInfo* __restrict__ info,
                           const int64_t* __restrict__ offsets, int64_t n_children,
                           const float2* __restrict__ seg, LokiScoreSpec sp, ScoreK SK,
                           float* __restrict__ scores, int32_t* __restrict__ cidx,
                           double* __restrict__ cphase, unsigned* __restrict__ minmax_keys) {
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nb = D.nbins, nbf = nb / 2 + 1;
  const int stride = score_stride(nb, sp.wmax);
  float* tw = smem;
  load_twiddles(tw, nb);
  __syncthreads();
  float* wbase = smem + 2 * nb + (size_t)warp * cplx_warp_floats(nb, stride);
  float2* comb = reinterpret_cast<float2*>(wbase) + (size_t)lane * 2 * nbf;
  float* tile = wbase + (size_t)32 * 2 * nbf * 2;
  const int64_t c = ((int64_t)blockIdx.x * kPruneWarps + warp) * 32 + lane;
  if (c >= n_children) return;
  score_child_complex(D, leaves, folds, n_parents, info, offsets, seg, sp, scores, cidx, cphase,
                      minmax_keys, tw, comb, tile + lane * stride, c);
}

// Survivors of the complex tree: transform / backtrack exactly as
// prune_emit_kernel, the fold written as the complex sum.
// One survivor of the complex tree: transform, backtrack and the complex
// sum of its fold.
__device__ __forceinline__ void emit_one_complex(
    const LokiPruneLevel& D, const double* __restrict__ leaves, const float2* __restrict__ folds,
    const LokiBranchInfo* __restrict__ info, const int64_t* __restrict__ offsets,
    int64_t n_parents, const float2* __restrict__ seg, const int64_t* __restrict__ surv,
    const float* __restrict__ cscores, const int32_t* __restrict__ cidx,
    const double* __restrict__ cphase, double* __restrict__ lout, float2* __restrict__ fout,
    float* __restrict__ sout, float* __restrict__ seout, int32_t* __restrict__ bout,
    int64_t s) {
  const int nb = D.nbins, nbf = nb / 2 + 1, P = D.poly_order, m = P + 1;
  const int64_t c = surv[s];
  const int64_t par = find_parent(offsets, n_parents, c);
  const LokiBranchInfo B = info[par];
  const double* lf = leaves + par * (P + 2) * 2;
  double pv[LOKI_MAX_PARAMS + 1], ev[LOKI_MAX_PARAMS + 1];
  child_params(B, P, c - offsets[par], pv);
  pv[P] = B.d0;
  for (int j = 0; j < P; ++j) ev[j] = B.dact[j];
  ev[P] = 0.0;
  double* lo = lout + s * (P + 2) * 2;
  if (D.moving) {
    for (int i = 0; i < m; ++i) lo[2 * i] = tdot(pv, D.tm_n, i, m);
    if (D.tiling == 0) {
      for (int i = 0; i < m; ++i) lo[2 * i + 1] = __dmul_rn(ev[i], fabs(D.tm_n[i][i]));
    } else if (D.tiling == 2) {
      for (int i = 0; i < m; ++i) lo[2 * i + 1] = tdot(ev, D.tm_e, i, m);
    } else {
      double e2[LOKI_MAX_PARAMS + 1];
      for (int j = 0; j < m; ++j) e2[j] = __dmul_rn(ev[j], ev[j]);
      for (int i = 0; i < m; ++i) lo[2 * i + 1] = __dsqrt_rn(tdot(e2, D.tm_e, i, m));
    }
  } else {
    for (int i = 0; i < m; ++i) {
      lo[2 * i] = pv[i];
      lo[2 * i + 1] = ev[i];
    }
  }
  lo[2 * m] = lf[2 * m];
  lo[2 * m + 1] = lf[2 * m + 1];
  sout[s] = cscores[c];
  seout[s] = cscores[c];
  int32_t* bt = bout + s * (P + 2);
  const int ia = cidx[2 * c], iff = cidx[2 * c + 1];
  bt[0] = (int32_t)par;
  for (int j = 1; j < P + 1; ++j) bt[j] = 0;
  bt[D.nparams_ffa - 1] = ia;
  bt[D.nparams_ffa] = iff;
  bt[P + 1] = (int32_t)cphase[c];
  const int64_t row = (int64_t)ia * D.n_freq + iff;
  rotate_add(seg + row * 2 * nbf, folds + par * 2 * nbf, prune_phasor(cphase[c], nb), nbf,
             fout + s * 2 * nbf);
}

__global__ void __launch_bounds__(kPruneWarps * 32)
prune_emit_complex_kernel(LokiPruneLevel D, const double* __restrict__ leaves,
                          const float2* __restrict__ folds,
                          const LokiBranchInfo* __restrict__ info,
                          const int64_t* __restrict__ offsets, int64_t n_parents,
                          const float2* __restrict__ seg, const int64_t* __restrict__ surv,
                          int64_t n_surv, const float* __restrict__ cscores,
                          const int32_t* __restrict__ cidx, const double* __restrict__ cphase,
                          double* __restrict__ lout, float2* __restrict__ fout,
                          float* __restrict__ sout, float* __restrict__ seout,
                          int32_t* __restrict__ bout) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n_surv) return;
  emit_one_complex(D, leaves, folds, info, offsets, n_parents, seg, surv, cscores, cidx, cphase,
                   lout, fout, sout, seout, bout, s);
}

// Ascend of the complex tree (dyn_poly_taylor.py:632-679 with
// core/common.py:460-490): per survivor the rotated segment rows are summed
// over the segments in order, then the sum is scored through its irfft.
// Ascend of one survivor of the complex tree.
__device__ __forceinline__ void ascend_one_complex(
    const LokiPruneLevel& D, const double* __restrict__ leaves, float2* __restrict__ folds,
    float* __restrict__ scores, float* __restrict__ scores_ep, int nseg,
    const double* __restrict__ tm_seg, const double* __restrict__ dt_seg,
    const int32_t* __restrict__ seg_idx, const float2* __restrict__ ffa, int64_t seg_stride,
    const LokiScoreSpec& sp, const float* tw, float2* comb, float* trow, int64_t r) {
  const int nb = D.nbins, nbf = nb / 2 + 1, P = D.poly_order, m = P + 1;
  const double* lf = leaves + r * (P + 2) * 2;
  double pv[LOKI_MAX_PARAMS + 1], ev[LOKI_MAX_PARAMS + 1];
  for (int i = 0; i < m; ++i) {
    pv[i] = lf[2 * i];
    ev[i] = lf[2 * i + 1];
  }
  const double f0 = lf[2 * m];
  // circular tree: class of the survivor (core/circular.py:597-666)
  const int cls = D.basis == 2 ? circ_class(pv, ev, D.circ_sig_prop) : 0;
  for (int k = 0; k < 2 * nbf; ++k) comb[k] = make_float2(0.0f, 0.0f);
  for (int sg = 0; sg < nseg; ++sg) {
    const double(*T)[LOKI_MAX_PARAMS + 1] =
        reinterpret_cast<const double(*)[LOKI_MAX_PARAMS + 1]>(tm_seg + sg * 36);
    double accel, vel, dd;
    if (D.basis == 1) {
      double a[LOKI_MAX_PARAMS + 1];
      for (int i = 0; i < m; ++i) a[i] = tdot(pv, T, i, m);
      cheby_low3(D, a, m, &accel, &vel, &dd);
    } else if (cls != 0) {  // circular survivors: closed-form propagation
      double a[6];
      circ_shift(pv, dt_seg[sg], cls == 2, a);
      accel = a[3];
      vel = a[4];
      dd = a[5];
    } else {
      accel = tdot(pv, T, P - 2, m);
      vel = tdot(pv, T, P - 1, m);
      dd = tdot(pv, T, P, m);
    }
    const double freq = __dmul_rn(f0, __dsub_rn(1.0, __ddiv_rn(vel, LOKI_C_VAL)));
    const double delay = __ddiv_rn(dd, LOKI_C_VAL);
    const double ph = phase_idx(dt_seg[sg], f0, nb, delay);
    const int64_t ia = axis_index(accel, D.accel_min, D.accel_inv, D.n_accel);
    const int64_t iff = axis_index(freq, D.freq_min, D.freq_inv, D.n_freq);
    const float2* row = ffa + (int64_t)seg_idx[sg] * seg_stride + (ia * D.n_freq + iff) * 2 * nbf;
    const float2 delta = prune_phasor(ph, nb);
    for (int c = 0; c < 2; ++c) {  // res += row * phasor^k
      float2 p = make_float2(1.0f, 0.0f);
      for (int k = 0; k < nbf; ++k) {
        const float2 t = cmul_rn(row[c * nbf + k], p);
        float2& a = comb[c * nbf + k];
        a = make_float2(__fadd_rn(a.x, t.x), __fadd_rn(a.y, t.y));
        p = cmul_rn(p, delta);
      }
    }
  }
  float2* o = folds + r * 2 * nbf;
  for (int k = 0; k < 2 * nbf; ++k) o[k] = comb[k];
  irfft_norm(comb, nb, nbf, tw, trow);
  scores_ep[r] = scores[r];
  float s;
  score_row(trow, nb, sp, &s);
  scores[r] = s;
}

__global__ void __launch_bounds__(kPruneWarps * 32)
prune_ascend_complex_kernel(LokiPruneLevel D, const double* __restrict__ leaves,
                            float2* __restrict__ folds, float* __restrict__ scores,
                            float* __restrict__ scores_ep, int64_t n, int nseg,
                            const double* __restrict__ tm_seg,
                            const double* __restrict__ dt_seg,
                            const int32_t* __restrict__ seg_idx,
                            const float2* __restrict__ ffa, int64_t seg_stride,
                            LokiScoreSpec sp, ScoreK SK) {
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nb = D.nbins, nbf = nb / 2 + 1;
  const int stride = score_stride(nb, sp.wmax);
  float* tw = smem;
  load_twiddles(tw, nb);
  __syncthreads();
  float* wbase = smem + 2 * nb + (size_t)warp * cplx_warp_floats(nb, stride);
  float2* comb = reinterpret_cast<float2*>(wbase) + (size_t)lane * 2 * nbf;
  float* tile = wbase + (size_t)32 * 2 * nbf * 2;
  const int64_t r = ((int64_t)blockIdx.x * kPruneWarps + warp) * 32 + lane;
  if (r >= n) return;
  ascend_one_complex(D, leaves, folds, scores, scores_ep, nseg, tm_seg, dt_seg, seg_idx, ffa,
                     seg_stride, sp, tw, comb, tile + lane * stride, r);
}

// ---------------------------------------------------------------------------
// circular-orbit tree over complex folds (PruneCircTaylorComplexDPFuncts,
// dynamic/dyn_circular_taylor.py:168-330): the circular branch, validation,
// resolve and transform of the real-fold circular kernels, with the complex
// shift-add (core/common.py:403-429) and irfft scoring
// (detection/scoring.py:285-292) of the complex Taylor kernels.
// ---------------------------------------------------------------------------

// Valid child v of the complex circular tree: resolve, rotate + add into
// the lane's comb buffer, irfft into trow, score (tw: the block's twiddles).
__device__ __forceinline__ void circ_score_one_complex(
    const LokiPruneLevel& D, const double* __restrict__ leaves, const float2* __restrict__ folds,
    int64_t batch, const LokiBranchInfo* __restrict__ info, const CircChild* __restrict__ map,
    const int64_t* __restrict__ valid_ids, const float2* __restrict__ seg,
    const LokiScoreSpec& sp, const float* tw, float2* comb, float* trow,
    float* __restrict__ scores, int32_t* __restrict__ cidx, double* __restrict__ cphase,
    int8_t* __restrict__ ccls, int32_t* __restrict__ batch_taylor,
    unsigned* __restrict__ minmax_keys, int64_t v) {
  const int nb = D.nbins, nbf = nb / 2 + 1, P = 5;
  const CircChild ch = map[valid_ids[v]];
  const LokiBranchInfo B = info[ch.parent];
  const double* lf = leaves + (int64_t)ch.parent * (P + 2) * 2;
  double pv[6], ev[6];
  circ_child(B, lf, ch, pv, ev);
  ChildRes r;
  const int cls = circ_resolve(D, pv, ev, lf[(P + 1) * 2], &r);
  if (cls == 0) atomicOr(batch_taylor + ch.parent / batch, 1);
  cidx[2 * v] = r.ia;
  cidx[2 * v + 1] = r.iff;
  cphase[v] = r.phase;
  ccls[v] = (int8_t)cls;
  const int64_t row = (int64_t)r.ia * D.n_freq + r.iff;
  rotate_add(seg + row * 2 * nbf, folds + (int64_t)ch.parent * 2 * nbf,
             prune_phasor(r.phase, nb), nbf, comb);
  irfft_norm(comb, nb, nbf, tw, trow);
  float s;
  score_row(trow, nb, sp, &s);
  scores[v] = s;
  if (s == s) {
    atomicMin(minmax_keys, float_key(s));
    atomicMax(minmax_keys + 1, float_key(s));
  }
}

__global__ void __launch_bounds__(kPruneWarps * 32)
circ_score_complex_kernel(LokiPruneLevel D, const double* __restrict__ leaves,
                          const float2* __restrict__ folds, int64_t batch,
                          const LokiBranchInfo* __restrict__ info,
                          const CircChild* __restrict__ map,
                          const int64_t* __restrict__ valid_ids, int64_t n_valid,
                          const float2* __restrict__ seg, LokiScoreSpec sp, ScoreK SK,
                          float* __restrict__ scores, int32_t* __restrict__ cidx,
                          double* __restrict__ cphase, int8_t* __restrict__ ccls,
                          int32_t* __restrict__ batch_taylor,
                          unsigned* __restrict__ minmax_keys) {
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nb = D.nbins, nbf = nb / 2 + 1;
  const int stride = score_stride(nb, sp.wmax);
  float* tw = smem;
  load_twiddles(tw, nb);
  __syncthreads();
  float* wbase = smem + 2 * nb + (size_t)warp * cplx_warp_floats(nb, stride);
  float2* comb = reinterpret_cast<float2*>(wbase) + (size_t)lane * 2 * nbf;
  float* tile = wbase + (size_t)32 * 2 * nbf * 2;
  const int64_t v = ((int64_t)blockIdx.x * kPruneWarps + warp) * 32 + lane;
  if (v >= n_valid) return;
  circ_score_one_complex(D, leaves, folds, batch, info, map, valid_ids, seg, sp, tw, comb,
                         tile + lane * stride, scores, cidx, cphase, ccls, batch_taylor,
                         minmax_keys, v);
}

// Survivor s of the complex circular tree (circ_emit_one's leaves, basis
// flag and backtracks; the fold written as the complex sum).
__device__ __forceinline__ void circ_emit_one_complex(
    const LokiPruneLevel& D, const double* __restrict__ leaves, const float2* __restrict__ folds,
    int64_t batch, const LokiBranchInfo* __restrict__ info, const CircChild* __restrict__ map,
    const int64_t* __restrict__ valid_ids, const float2* __restrict__ seg,
    const int64_t* __restrict__ surv, const float* __restrict__ cscores,
    const int32_t* __restrict__ cidx, const double* __restrict__ cphase,
    const int8_t* __restrict__ ccls, const int32_t* __restrict__ batch_taylor,
    double* __restrict__ lout, float2* __restrict__ fout, float* __restrict__ sout,
    float* __restrict__ seout, int32_t* __restrict__ bout, int64_t s) {
  const int nb = D.nbins, nbf = nb / 2 + 1, P = 5, m = 6;
  const int64_t v = surv[s];
  const CircChild ch = map[valid_ids[v]];
  const LokiBranchInfo B = info[ch.parent];
  const double* lf = leaves + (int64_t)ch.parent * (P + 2) * 2;
  double pv[6], ev[6];
  circ_child(B, lf, ch, pv, ev);
  const int cls = ccls[v];
  double* lo = lout + s * (P + 2) * 2;
  double flag = lf[2 * m + 1];
  if (D.moving) {
    if (cls == 1) flag = 1.0;
    else if (cls == 2) flag = batch_taylor[ch.parent / batch] ? 0.0 : 2.0;
    if (cls != 0) {
      double o[6];
      circ_shift(pv, D.circ_dt_next, cls == 2, o);
      for (int i = 0; i < m; ++i) {
        lo[2 * i] = o[i];
        lo[2 * i + 1] = ev[i];
      }
    } else {
      for (int i = 0; i < m; ++i) lo[2 * i] = tdot(pv, D.tm_n, i, m);
      if (D.tiling == 0) {
        for (int i = 0; i < m; ++i) lo[2 * i + 1] = __dmul_rn(ev[i], fabs(D.tm_n[i][i]));
      } else if (D.tiling == 2) {
        for (int i = 0; i < m; ++i) lo[2 * i + 1] = tdot(ev, D.tm_e, i, m);
      } else {
        double e2[6];
        for (int j = 0; j < m; ++j) e2[j] = __dmul_rn(ev[j], ev[j]);
        for (int i = 0; i < m; ++i) lo[2 * i + 1] = __dsqrt_rn(tdot(e2, D.tm_e, i, m));
      }
    }
  } else {
    for (int i = 0; i < m; ++i) {
      lo[2 * i] = pv[i];
      lo[2 * i + 1] = ev[i];
    }
  }
  lo[2 * m] = lf[2 * m];
  lo[2 * m + 1] = flag;
  sout[s] = cscores[v];
  seout[s] = cscores[v];
  int32_t* bt = bout + s * (P + 2);
  const int ia = cidx[2 * v], iff = cidx[2 * v + 1];
  bt[0] = ch.parent;
  for (int j = 1; j < P + 1; ++j) bt[j] = 0;
  bt[D.nparams_ffa - 1] = ia;
  bt[D.nparams_ffa] = iff;
  bt[P + 1] = (int32_t)cphase[v];
  const int64_t row = (int64_t)ia * D.n_freq + iff;
  rotate_add(seg + row * 2 * nbf, folds + (int64_t)ch.parent * 2 * nbf,
             prune_phasor(cphase[v], nb), nbf, fout + s * 2 * nbf);
}

// Survivors of the complex circular tree: leaves, basis flag and backtracks as
// circ_emit_kernel, the fold written as the complex sum.
__global__ void __launch_bounds__(kPruneWarps * 32)
circ_emit_complex_kernel(LokiPruneLevel D, const double* __restrict__ leaves,
                         const float2* __restrict__ folds, int64_t batch,
                         const LokiBranchInfo* __restrict__ info,
                         const CircChild* __restrict__ map,
                         const int64_t* __restrict__ valid_ids, const float2* __restrict__ seg,
                         const int64_t* __restrict__ surv, int64_t n_surv,
                         const float* __restrict__ cscores, const int32_t* __restrict__ cidx,
                         const double* __restrict__ cphase, const int8_t* __restrict__ ccls,
                         const int32_t* __restrict__ batch_taylor, double* __restrict__ lout,
                         float2* __restrict__ fout, float* __restrict__ sout,
                         float* __restrict__ seout, int32_t* __restrict__ bout) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n_surv) return;
  circ_emit_one_complex(D, leaves, folds, batch, info, map, valid_ids, seg, surv, cscores, cidx,
                        cphase, ccls, batch_taylor, lout, fout, sout, seout, bout, s);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

static int check_prune(const LokiPruneLevel* D) {
  if (!D) return set_error(LOKI_ERR_INVALID, "null prune level descriptor");
  if (D->poly_order < 2 || D->poly_order > LOKI_MAX_PARAMS)
    return set_error(LOKI_ERR_INVALID, "poly_order %d outside [2, %d]", D->poly_order,
                     LOKI_MAX_PARAMS);
  if (D->nbins < 2) return set_error(LOKI_ERR_INVALID, "nbins < 2");
  if (D->nparams_ffa < 2 || D->nparams_ffa > D->poly_order)
    return set_error(LOKI_ERR_INVALID, "nparams_ffa %d outside [2, poly_order]",
                     D->nparams_ffa);
  if (D->n_accel < 1 || D->n_freq < 1) return set_error(LOKI_ERR_INVALID, "empty FFA grid");
  if (D->tiling < 0 || D->tiling > 2) return set_error(LOKI_ERR_INVALID, "bad tiling");
  return LOKI_OK;
}

static int prune_spec_check(const LokiScoreSpec* sp, int nbins) {
  if (!sp || sp->nwidths < 1 || sp->nwidths > LOKI_MAX_WIDTHS)
    return set_error(LOKI_ERR_INVALID, "bad score spec");
  if (nbins + sp->wmax > 1024)
    return set_error(LOKI_ERR_UNSUPPORTED, "nbins + wmax above 1024 for pruning");
  return LOKI_OK;
}

}  // namespace loki

using namespace loki;

extern "C" int64_t loki_scan_scratch_bytes(int64_t n) {
  return std::max<int64_t>(1, (n + kScanBlock - 1) / kScanBlock) * (int64_t)sizeof(int64_t);
}

static int prune_branch_impl(const LokiPruneLevel* lvl, const double* leaves,
                             int64_t n_parents, const uint8_t* mask, LokiBranchInfo* info,
                             int64_t* offsets, void* scan_scratch, int64_t scan_scratch_bytes,
                             int32_t* dev_err, void* stream);

// End of a device-resident level (single thread): the level's record (score
// range from the ordered keys, as minmax_finish_kernel), then the survivors
// become the next level's parents and the keys restart.
__device__ __forceinline__ void level_end(int64_t* cnt, unsigned* keys, int32_t* ovf_flag,
                                          LokiPruneLevelStats* st) {
  st->n_surv = cnt[2];
  const bool none = keys[0] == 0xFFFFFFFFu;  // no finite score
  st->score_min = none ? 0.0f : key_float(keys[0]);
  st->score_max = none ? 0.0f : key_float(keys[1]);
  st->overflow = *ovf_flag;
  st->reserved = 0;
  *ovf_flag = 0;
  keys[0] = 0xFFFFFFFFu;
  keys[1] = 0u;
  cnt[3] += cnt[2];  // backtrack history rows
  cnt[0] = cnt[2];
}

// Best leaf of a tree (max score, first index on ties, as torch.argmax):
// one block reduces (score, index), then copies the leaf row and its score.
__device__ void block_best(const float* __restrict__ scores, int64_t n,
                           const double* __restrict__ leaves, int row,
                           double* __restrict__ leaf_out, float* __restrict__ score_out) {
  __shared__ float sv[32];
  __shared__ int64_t si[32];
  float bv = -INFINITY;
  int64_t bi = -1;
  // each thread visits its elements in increasing index order, so it keeps
  // its first maximum; float4 loads, four in flight, when the scores are
  // 16-byte aligned
  int64_t head = 0;
  if ((reinterpret_cast<uintptr_t>(scores) & 15) == 0) {
    const float4* s4 = reinterpret_cast<const float4*>(scores);
    const int64_t n4 = n >> 2;
    const int64_t step = blockDim.x;
    int64_t q = threadIdx.x;
    for (; q + 3 * step < n4; q += 4 * step) {
      float4 a[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = s4[q + u * step];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float c[4] = {a[u].x, a[u].y, a[u].z, a[u].w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (bi < 0 || c[k] > bv) {
            bv = c[k];
            bi = 4 * (q + u * step) + k;
          }
        }
      }
    }
    for (; q < n4; q += step) {
      const float4 a = s4[q];
      const float c[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (bi < 0 || c[k] > bv) {
          bv = c[k];
          bi = 4 * q + k;
        }
      }
    }
    head = n4 << 2;
  }
  for (int64_t i = head + threadIdx.x; i < n; i += blockDim.x) {
    const float v = scores[i];
    if (bi < 0 || v > bv) {
      bv = v;
      bi = i;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const float ov = __shfl_down_sync(0xFFFFFFFFu, bv, o);
    const int64_t oi = __shfl_down_sync(0xFFFFFFFFu, bi, o);
    if (oi >= 0 && (bi < 0 || ov > bv || (ov == bv && oi < bi))) {
      bv = ov;
      bi = oi;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    sv[warp] = bv;
    si[warp] = bi;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    bv = lane < nw ? sv[lane] : -INFINITY;
    bi = lane < nw ? si[lane] : -1;
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_down_sync(0xFFFFFFFFu, bv, o);
      const int64_t oi = __shfl_down_sync(0xFFFFFFFFu, bi, o);
      if (oi >= 0 && (bi < 0 || ov > bv || (ov == bv && oi < bi))) {
        bv = ov;
        bi = oi;
      }
    }
    bi = __shfl_sync(0xFFFFFFFFu, bi, 0);
    if (bi >= 0)
      for (int j = lane; j < row; j += 32) leaf_out[j] = leaves[bi * row + j];
    if (lane == 0 && bi >= 0) *score_out = scores[bi];
  }
}

__global__ void __launch_bounds__(1024)
prune_best_kernel(const float* __restrict__ scores, int64_t n, const double* __restrict__ leaves,
                  int row, double* __restrict__ leaf_out, float* __restrict__ score_out,
                  int64_t* lvl_cnt, unsigned* lvl_keys, int32_t* lvl_ovf,
                  LokiPruneLevelStats* lvl_st) {
  if (lvl_cnt) n = lvl_cnt[2];  // the level's survivors; 0 writes nothing
  block_best(scores, n, leaves, row, leaf_out, score_out);
  // every thread read the count before block_best's barrier
  if (threadIdx.x == 0 && lvl_cnt) level_end(lvl_cnt, lvl_keys, lvl_ovf, lvl_st);
}

extern "C" int loki_prune_best(const float* scores, int64_t n, const double* leaves,
                               int32_t row_len, double* leaf_out, float* score_out,
                               void* stream) {
  if (n < 0 || row_len < 1) return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (n == 0) return LOKI_OK;
  if (!scores || !leaves || !leaf_out || !score_out)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  note_launch();
  prune_best_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(scores, n, leaves, row_len, leaf_out,
                                                         score_out, nullptr, nullptr, nullptr,
                                                         nullptr);
  return check_launch("prune_best");
}

extern "C" int loki_prune_branch(const LokiPruneLevel* lvl, const double* leaves,
                                 int64_t n_parents, LokiBranchInfo* info, int64_t* offsets,
                                 void* scan_scratch, int64_t scan_scratch_bytes,
                                 int32_t* dev_err, void* stream) {
  return prune_branch_impl(lvl, leaves, n_parents, nullptr, info, offsets, scan_scratch,
                           scan_scratch_bytes, dev_err, stream);
}

extern "C" int loki_prune_branch_masked(const LokiPruneLevel* lvl, const double* leaves,
                                        int64_t n_parents, const uint8_t* parent_mask,
                                        LokiBranchInfo* info, int64_t* offsets,
                                        void* scan_scratch, int64_t scan_scratch_bytes,
                                        int32_t* dev_err, void* stream) {
  if (n_parents > 0 && !parent_mask) return set_error(LOKI_ERR_INVALID, "null parent mask");
  return prune_branch_impl(lvl, leaves, n_parents, parent_mask, info, offsets, scan_scratch,
                           scan_scratch_bytes, dev_err, stream);
}

static int prune_branch_impl(const LokiPruneLevel* lvl, const double* leaves,
                             int64_t n_parents, const uint8_t* mask, LokiBranchInfo* info,
                             int64_t* offsets, void* scan_scratch, int64_t scan_scratch_bytes,
                             int32_t* dev_err, void* stream) {
  int rc = check_prune(lvl);
  if (rc) return rc;
  if (n_parents < 0) return set_error(LOKI_ERR_INVALID, "n_parents < 0");
  if (!offsets || !dev_err || (n_parents && (!leaves || !info)))
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  cudaStream_t s = (cudaStream_t)stream;
  if (n_parents > 0) {
    // child counts go to offsets[0..n), scanned in place
    note_launch();
    prune_branch_kernel<<<(unsigned)((n_parents + 255) / 256), 256, 0, s>>>(
        *lvl, leaves, n_parents, info, offsets, dev_err, mask, nullptr);
    rc = check_launch("prune_branch");
    if (rc) return rc;
  }
  return exclusive_scan<false>(offsets, n_parents, 0.0, offsets, scan_scratch,
                               scan_scratch_bytes, s);
}

extern "C" int loki_prune_score(const LokiPruneLevel* lvl, const double* leaves,
                                const float* folds, int64_t n_parents,
                                const LokiBranchInfo* info, const int64_t* offsets,
                                int64_t n_children, const float* fold_segment,
                                const LokiScoreSpec* spec, float* child_scores,
                                int32_t* child_idx, double* child_phase, float* score_minmax,
                                int32_t* dev_err, void* stream) {
  int rc = check_prune(lvl);
  if (rc) return rc;
  rc = prune_spec_check(spec, lvl->nbins);
  if (rc) return rc;
  if (!score_minmax || !dev_err) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned* keys = reinterpret_cast<unsigned*>(score_minmax);  // reused as ordered keys
  note_launch();
  minmax_init_kernel<<<1, 1, 0, s>>>(keys);
  if (n_children > 0) {
    if (!leaves || !folds || !info || !offsets || !fold_segment || !child_scores ||
        !child_idx || !child_phase)
      return set_error(LOKI_ERR_INVALID, "null pointer argument");
    LokiScoreSpec sp = *spec;
    sp.mode = 1;
    const ScoreK SK = make_score_k(sp, lvl->nbins);
    const int smem = score_smem_bytes(lvl->nbins, sp.wmax, kPruneWarps);
    if (smem > 200 * 1024)
      return set_error(LOKI_ERR_UNSUPPORTED, "nbins + wmax too large for pruning");
    if (smem > 48 * 1024 &&
        set_smem_limit(prune_score_kernel, smem) != cudaSuccess)
      return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
    const int64_t blocks = (n_children + kPruneWarps * 32 - 1) / (kPruneWarps * 32);
    if (blocks > 0x7FFFFFFF) return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
    note_launch();
    prune_score_kernel<<<(unsigned)blocks, kPruneWarps * 32, smem, s>>>(
        *lvl, leaves, folds, n_parents, info, offsets, n_children, fold_segment, sp, SK,
        child_scores, child_idx, child_phase, keys, nullptr, 0, nullptr, nullptr);
  }
  note_launch();
  minmax_finish_kernel<<<1, 1, 0, s>>>(keys, score_minmax);
  return check_launch("prune_score");
}

extern "C" int loki_prune_select(const float* child_scores, int64_t n_children,
                                 double threshold, int64_t* surv_ids, int64_t* n_surv,
                                 void* scan_scratch, int64_t scan_scratch_bytes, void* stream) {
  if (n_children < 0 || !n_surv) return set_error(LOKI_ERR_INVALID, "bad select arguments");
  if (n_children > 0 && (!child_scores || !surv_ids))
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  cudaStream_t s = (cudaStream_t)stream;
  // positions are scanned into surv_ids' tail-free temp: reuse surv_ids is not
  // possible (scatter reads positions), so positions live in the scratch
  // after the block sums.
  const int64_t sums_bytes = loki_scan_scratch_bytes(n_children);
  const int64_t need = sums_bytes + (n_children + 1) * (int64_t)sizeof(int64_t);
  if (scan_scratch_bytes < need)
    return set_error(LOKI_ERR_CAPACITY, "select scratch needs %lld bytes", (long long)need);
  int64_t* pos = reinterpret_cast<int64_t*>(reinterpret_cast<char*>(scan_scratch) + sums_bytes);
  int rc = exclusive_scan<true>(child_scores, n_children, threshold, pos, scan_scratch,
                                sums_bytes, s);
  if (rc) return rc;
  if (n_children > 0) note_launch();
  if (n_children > 0)
    select_scatter_kernel<<<(unsigned)((n_children + 255) / 256), 256, 0, s>>>(
        child_scores, n_children, threshold, pos, surv_ids, nullptr);
  if (cudaMemcpyAsync(n_surv, pos + n_children, sizeof(int64_t), cudaMemcpyDeviceToDevice, s) !=
      cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaMemcpyAsync failed");
  return check_launch("prune_select");
}

extern "C" int loki_prune_select_overflow(const float* child_scores, const int64_t* offsets,
                                          int64_t n_parents, int64_t batch_size,
                                          double threshold, int64_t capacity,
                                          int64_t* surv_ids, int64_t* n_surv, double* thr_out,
                                          int64_t* scratch_ids, float* scratch_keys,
                                          int64_t scratch_len, void* stream) {
  if (batch_size < 1 || capacity < 1 || n_parents < 0)
    return set_error(LOKI_ERR_INVALID, "bad overflow selection arguments");
  if (!child_scores || !offsets || !surv_ids || !n_surv || !thr_out || !scratch_ids ||
      !scratch_keys)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  note_launch();
  select_overflow_kernel<<<1, kSelThreads, 0, (cudaStream_t)stream>>>(
      child_scores, offsets, n_parents, batch_size, threshold, capacity, surv_ids, n_surv,
      thr_out, scratch_ids, reinterpret_cast<unsigned*>(scratch_keys), nullptr, nullptr,
      nullptr, nullptr);
  (void)scratch_len;
  return check_launch("prune_select_overflow");
}

extern "C" int loki_prune_emit(const LokiPruneLevel* lvl, const double* leaves,
                               const float* folds, const LokiBranchInfo* info,
                               const int64_t* offsets, int64_t n_parents,
                               const float* fold_segment, const int64_t* surv_ids,
                               int64_t n_surv, const float* child_scores,
                               const int32_t* child_idx, const double* child_phase,
                               double* leaves_out, float* folds_out, float* scores_out,
                               float* scores_ep_out, int32_t* bt_out, void* stream) {
  int rc = check_prune(lvl);
  if (rc) return rc;
  if (n_surv <= 0) return LOKI_OK;
  if (!leaves || !folds || !info || !offsets || !fold_segment || !surv_ids || !child_scores ||
      !child_idx || !child_phase || !leaves_out || !folds_out || !scores_out ||
      !scores_ep_out || !bt_out)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const int64_t blocks = (n_surv + kPruneWarps * 32 - 1) / (kPruneWarps * 32);
  note_launch();
  prune_emit_kernel<<<(unsigned)blocks, kPruneWarps * 32, 0, (cudaStream_t)stream>>>(
      *lvl, leaves, folds, info, offsets, n_parents, fold_segment, surv_ids, n_surv,
      child_scores, child_idx, child_phase, leaves_out, folds_out, scores_out, scores_ep_out,
      bt_out, nullptr);
  return check_launch("prune_emit");
}

extern "C" int loki_prune_ascend(const LokiPruneLevel* lvl, const double* leaves, float* folds,
                                 float* scores, float* scores_ep, int64_t n, int32_t nseg,
                                 const double* tm_seg, const double* dt_seg,
                                 const int32_t* seg_idx, const float* ffa_fold,
                                 int64_t seg_stride, const LokiScoreSpec* spec,
                                 int32_t* dev_err, void* stream) {
  int rc = check_prune(lvl);
  if (rc) return rc;
  rc = prune_spec_check(spec, lvl->nbins);
  if (rc) return rc;
  if (n <= 0) return LOKI_OK;
  if (nseg < 1 || !leaves || !folds || !scores || !scores_ep || !tm_seg || !dt_seg ||
      !seg_idx || !ffa_fold || !dev_err)
    return set_error(LOKI_ERR_INVALID, "bad ascend arguments");
  LokiScoreSpec sp = *spec;
  sp.mode = 1;
  const ScoreK SK = make_score_k(sp, lvl->nbins);
  const int nb = lvl->nbins;
  const int smem = kPruneWarps * 32 * (2 * nb + score_stride(nb, sp.wmax)) * (int)sizeof(float);
  if (smem > 200 * 1024) return set_error(LOKI_ERR_UNSUPPORTED, "nbins too large for ascend");
  if (smem > 48 * 1024 &&
      set_smem_limit(prune_ascend_kernel, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  const int64_t blocks = (n + kPruneWarps * 32 - 1) / (kPruneWarps * 32);
  note_launch();
  prune_ascend_kernel<<<(unsigned)blocks, kPruneWarps * 32, smem, (cudaStream_t)stream>>>(
      *lvl, leaves, folds, scores, scores_ep, n, nseg, tm_seg, dt_seg, seg_idx, ffa_fold,
      seg_stride, sp, SK, nullptr);
  return check_launch("prune_ascend");
}

extern "C" int loki_prune_ascend_dev(const LokiPruneLevel* lvl, const double* leaves,
                                     float* folds, float* scores, float* scores_ep,
                                     const int64_t* n_dev, int64_t n_cap, int32_t nseg,
                                     const double* tm_seg, const double* dt_seg,
                                     const int32_t* seg_idx, const float* ffa_fold,
                                     int64_t seg_stride, const LokiScoreSpec* spec,
                                     int32_t* dev_err, void* stream) {
  int rc = check_prune(lvl);
  if (rc) return rc;
  rc = prune_spec_check(spec, lvl->nbins);
  if (rc) return rc;
  if (n_cap < 1 || nseg < 1 || !n_dev || !leaves || !folds || !scores || !scores_ep ||
      !tm_seg || !dt_seg || !seg_idx || !ffa_fold || !dev_err)
    return set_error(LOKI_ERR_INVALID, "bad ascend arguments");
  LokiScoreSpec sp = *spec;
  sp.mode = 1;
  const ScoreK SK = make_score_k(sp, lvl->nbins);
  const int nb = lvl->nbins;
  const int smem = kPruneWarps * 32 * (2 * nb + score_stride(nb, sp.wmax)) * (int)sizeof(float);
  if (smem > 200 * 1024) return set_error(LOKI_ERR_UNSUPPORTED, "nbins too large for ascend");
  if (smem > 48 * 1024 && set_smem_limit(prune_ascend_kernel, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  int dev = 0, nsm = 0, occ = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, prune_ascend_kernel,
                                                    kPruneWarps * 32, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "occupancy query failed");
  const int64_t need = (n_cap + kPruneWarps * 32 - 1) / (kPruneWarps * 32);
  const unsigned blocks = (unsigned)std::max<int64_t>(
      1, std::min<int64_t>(need, (int64_t)nsm * std::max(1, occ)));
  note_launch();
  prune_ascend_kernel<<<blocks, kPruneWarps * 32, smem, (cudaStream_t)stream>>>(
      *lvl, leaves, folds, scores, scores_ep, 0, nseg, tm_seg, dt_seg, seg_idx, ffa_fold,
      seg_stride, sp, SK, n_dev);
  return check_launch("prune_ascend_dev");
}

// ---- circular-orbit tree --------------------------------------------------

static int check_circ(const LokiPruneLevel* lvl) {
  int rc = check_prune(lvl);
  if (rc) return rc;
  if (lvl->basis != 2 || lvl->poly_order != 5)
    return set_error(LOKI_ERR_INVALID, "the circular tree needs basis 2 and poly_order 5");
  return LOKI_OK;
}

extern "C" int loki_prune_circ_branch(const LokiPruneLevel* lvl, const double* leaves,
                                      int64_t n_parents, LokiBranchInfo* info,
                                      int64_t* keep_off, int64_t* exp_off, void* scan_scratch,
                                      int64_t scan_scratch_bytes, int32_t* dev_err,
                                      void* stream) {
  int rc = check_circ(lvl);
  if (rc) return rc;
  if (n_parents < 0) return set_error(LOKI_ERR_INVALID, "n_parents < 0");
  if (!keep_off || !exp_off || !dev_err || (n_parents && (!leaves || !info)))
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  cudaStream_t s = (cudaStream_t)stream;
  if (n_parents > 0) {
    note_launch();
    circ_branch_kernel<<<(unsigned)((n_parents + 255) / 256), 256, 0, s>>>(
        *lvl, leaves, n_parents, info, keep_off, exp_off, dev_err, nullptr);
    rc = check_launch("prune_circ_branch");
    if (rc) return rc;
  }
  rc = exclusive_scan<false>(keep_off, n_parents, 0.0, keep_off, scan_scratch,
                             scan_scratch_bytes, s);
  if (rc) return rc;
  return exclusive_scan<false>(exp_off, n_parents, 0.0, exp_off, scan_scratch,
                               scan_scratch_bytes, s);
}

extern "C" int loki_prune_circ_map(const LokiPruneLevel* lvl, const double* leaves,
                                   int64_t n_parents, int64_t batch_size,
                                   const LokiBranchInfo* info, const int64_t* keep_off,
                                   const int64_t* exp_off, void* child_map, float* valid_flags,
                                   void* stream) {
  int rc = check_circ(lvl);
  if (rc) return rc;
  if (batch_size < 1 || n_parents < 0) return set_error(LOKI_ERR_INVALID, "bad batch size");
  if (n_parents == 0) return LOKI_OK;
  if (!leaves || !info || !keep_off || !exp_off || !child_map || !valid_flags)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  note_launch();
  circ_map_kernel<<<(unsigned)((n_parents + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      *lvl, leaves, n_parents, batch_size, info, keep_off, exp_off,
      reinterpret_cast<CircChild*>(child_map), valid_flags, nullptr, 0, nullptr, nullptr);
  return check_launch("prune_circ_map");
}

extern "C" int loki_prune_circ_score(const LokiPruneLevel* lvl, const double* leaves,
                                     const float* folds, int64_t n_parents, int64_t batch_size,
                                     const LokiBranchInfo* info, const void* child_map,
                                     const int64_t* keep_off, const int64_t* exp_off,
                                     const int64_t* valid_ids, int64_t n_valid,
                                     const float* fold_segment, const LokiScoreSpec* spec,
                                     float* child_scores, int32_t* child_idx,
                                     double* child_phase, int8_t* child_class,
                                     int32_t* batch_taylor, int64_t* batch_offsets,
                                     float* score_minmax, int32_t* dev_err, void* stream) {
  int rc = check_circ(lvl);
  if (rc) return rc;
  rc = prune_spec_check(spec, lvl->nbins);
  if (rc) return rc;
  if (batch_size < 1 || n_parents < 0 || n_valid < 0)
    return set_error(LOKI_ERR_INVALID, "bad circular score arguments");
  if (!score_minmax || !dev_err || !batch_taylor || !batch_offsets || !keep_off || !exp_off)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t nbatch = (n_parents + batch_size - 1) / batch_size;
  if (nbatch > 0 && cudaMemsetAsync(batch_taylor, 0, nbatch * sizeof(int32_t), s) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaMemsetAsync failed");
  unsigned* keys = reinterpret_cast<unsigned*>(score_minmax);
  note_launch();
  minmax_init_kernel<<<1, 1, 0, s>>>(keys);
  if (n_valid > 0) {
    if (!leaves || !folds || !info || !child_map || !valid_ids || !fold_segment ||
        !child_scores || !child_idx || !child_phase || !child_class)
      return set_error(LOKI_ERR_INVALID, "null pointer argument");
    LokiScoreSpec sp = *spec;
    sp.mode = 1;
    const ScoreK SK = make_score_k(sp, lvl->nbins);
    const int smem = score_smem_bytes(lvl->nbins, sp.wmax, kPruneWarps);
    if (smem > 200 * 1024)
      return set_error(LOKI_ERR_UNSUPPORTED, "nbins + wmax too large for pruning");
    if (smem > 48 * 1024 &&
        set_smem_limit(circ_score_kernel, smem) != cudaSuccess)
      return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
    const int64_t blocks = (n_valid + kPruneWarps * 32 - 1) / (kPruneWarps * 32);
    if (blocks > 0x7FFFFFFF) return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
    note_launch();
    circ_score_kernel<<<(unsigned)blocks, kPruneWarps * 32, smem, s>>>(
        *lvl, leaves, folds, batch_size, info, reinterpret_cast<const CircChild*>(child_map),
        valid_ids, n_valid, fold_segment, sp, SK, child_scores, child_idx, child_phase,
        child_class, batch_taylor, keys, nullptr, nullptr, nullptr);
  }
  note_launch();
  minmax_finish_kernel<<<1, 1, 0, s>>>(keys, score_minmax);
  note_launch();
  circ_boff_kernel<<<(unsigned)((n_parents + 1 + 255) / 256), 256, 0, s>>>(
      keep_off, exp_off, n_parents, valid_ids, n_valid, batch_offsets, nullptr);
  return check_launch("prune_circ_score");
}

extern "C" int loki_prune_circ_emit(const LokiPruneLevel* lvl, const double* leaves,
                                    const float* folds, int64_t batch_size,
                                    const LokiBranchInfo* info, const void* child_map,
                                    const int64_t* valid_ids, const float* fold_segment,
                                    const int64_t* surv_ids, int64_t n_surv,
                                    const float* child_scores, const int32_t* child_idx,
                                    const double* child_phase, const int8_t* child_class,
                                    const int32_t* batch_taylor, double* leaves_out,
                                    float* folds_out, float* scores_out, float* scores_ep_out,
                                    int32_t* bt_out, void* stream) {
  int rc = check_circ(lvl);
  if (rc) return rc;
  if (n_surv <= 0) return LOKI_OK;
  if (batch_size < 1) return set_error(LOKI_ERR_INVALID, "bad batch size");
  if (!leaves || !folds || !info || !child_map || !valid_ids || !fold_segment || !surv_ids ||
      !child_scores || !child_idx || !child_phase || !child_class || !batch_taylor ||
      !leaves_out || !folds_out || !scores_out || !scores_ep_out || !bt_out)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const int64_t blocks = (n_surv + kPruneWarps * 32 - 1) / (kPruneWarps * 32);
  note_launch();
  circ_emit_kernel<<<(unsigned)blocks, kPruneWarps * 32, 0, (cudaStream_t)stream>>>(
      *lvl, leaves, folds, batch_size, info, reinterpret_cast<const CircChild*>(child_map),
      valid_ids, fold_segment, surv_ids, n_surv, child_scores, child_idx, child_phase,
      child_class, batch_taylor, leaves_out, folds_out, scores_out, scores_ep_out, bt_out,
      nullptr);
  return check_launch("prune_circ_emit");
}

static int cplx_smem(const LokiPruneLevel* lvl, const LokiScoreSpec& sp, int* smem);

extern "C" int loki_prune_circ_score_complex(
    const LokiPruneLevel* lvl, const double* leaves, const void* folds, int64_t n_parents,
    int64_t batch_size, const LokiBranchInfo* info, const void* child_map,
    const int64_t* keep_off, const int64_t* exp_off, const int64_t* valid_ids, int64_t n_valid,
    const void* fold_segment, const LokiScoreSpec* spec, float* child_scores,
    int32_t* child_idx, double* child_phase, int8_t* child_class, int32_t* batch_taylor,
    int64_t* batch_offsets, float* score_minmax, int32_t* dev_err, void* stream) {
  int rc = check_circ(lvl);
  if (rc) return rc;
  rc = prune_spec_check(spec, lvl->nbins);
  if (rc) return rc;
  if (batch_size < 1 || n_parents < 0 || n_valid < 0)
    return set_error(LOKI_ERR_INVALID, "bad circular score arguments");
  if (!score_minmax || !dev_err || !batch_taylor || !batch_offsets || !keep_off || !exp_off)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t nbatch = (n_parents + batch_size - 1) / batch_size;
  if (nbatch > 0 && cudaMemsetAsync(batch_taylor, 0, nbatch * sizeof(int32_t), s) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaMemsetAsync failed");
  unsigned* keys = reinterpret_cast<unsigned*>(score_minmax);
  note_launch();
  minmax_init_kernel<<<1, 1, 0, s>>>(keys);
  if (n_valid > 0) {
    if (!leaves || !folds || !info || !child_map || !valid_ids || !fold_segment ||
        !child_scores || !child_idx || !child_phase || !child_class)
      return set_error(LOKI_ERR_INVALID, "null pointer argument");
    LokiScoreSpec sp = *spec;
    sp.mode = 1;
    const ScoreK SK = make_score_k(sp, lvl->nbins);
    int smem = 0;
    rc = cplx_smem(lvl, sp, &smem);
    if (rc) return rc;
    if (smem > 48 * 1024 &&
        set_smem_limit(circ_score_complex_kernel, smem) != cudaSuccess)
      return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
    const int64_t blocks = (n_valid + kPruneWarps * 32 - 1) / (kPruneWarps * 32);
    if (blocks > 0x7FFFFFFF) return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
    note_launch();
    circ_score_complex_kernel<<<(unsigned)blocks, kPruneWarps * 32, smem, s>>>(
        *lvl, leaves, static_cast<const float2*>(folds), batch_size, info,
        reinterpret_cast<const CircChild*>(child_map), valid_ids, n_valid,
        static_cast<const float2*>(fold_segment), sp, SK, child_scores, child_idx,
        child_phase, child_class, batch_taylor, keys);
  }
  note_launch();
  minmax_finish_kernel<<<1, 1, 0, s>>>(keys, score_minmax);
  note_launch();
  circ_boff_kernel<<<(unsigned)((n_parents + 1 + 255) / 256), 256, 0, s>>>(
      keep_off, exp_off, n_parents, valid_ids, n_valid, batch_offsets, nullptr);
  return check_launch("prune_circ_score_complex");
}

extern "C" int loki_prune_circ_emit_complex(
    const LokiPruneLevel* lvl, const double* leaves, const void* folds, int64_t batch_size,
    const LokiBranchInfo* info, const void* child_map, const int64_t* valid_ids,
    const void* fold_segment, const int64_t* surv_ids, int64_t n_surv,
    const float* child_scores, const int32_t* child_idx, const double* child_phase,
    const int8_t* child_class, const int32_t* batch_taylor, double* leaves_out,
    void* folds_out, float* scores_out, float* scores_ep_out, int32_t* bt_out, void* stream) {
  int rc = check_circ(lvl);
  if (rc) return rc;
  if (lvl->nbins % 2) return set_error(LOKI_ERR_INVALID, "complex folds need an even nbins");
  if (n_surv <= 0) return LOKI_OK;
  if (batch_size < 1) return set_error(LOKI_ERR_INVALID, "bad batch size");
  if (!leaves || !folds || !info || !child_map || !valid_ids || !fold_segment || !surv_ids ||
      !child_scores || !child_idx || !child_phase || !child_class || !batch_taylor ||
      !leaves_out || !folds_out || !scores_out || !scores_ep_out || !bt_out)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  note_launch();
  circ_emit_complex_kernel<<<(unsigned)((n_surv + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
      *lvl, leaves, static_cast<const float2*>(folds), batch_size, info,
      reinterpret_cast<const CircChild*>(child_map), valid_ids,
      static_cast<const float2*>(fold_segment), surv_ids, n_surv, child_scores, child_idx,
      child_phase, child_class, batch_taylor, leaves_out, static_cast<float2*>(folds_out),
      scores_out, scores_ep_out, bt_out);
  return check_launch("prune_circ_emit_complex");
}

// ---- complex (Fourier) folds -----------------------------------------------

static int cplx_smem(const LokiPruneLevel* lvl, const LokiScoreSpec& sp, int* smem) {
  if (lvl->nbins % 2) return set_error(LOKI_ERR_INVALID, "complex folds need an even nbins");
  const size_t bytes = ((size_t)2 * lvl->nbins +
                        kPruneWarps * cplx_warp_floats(lvl->nbins,
                                                       score_stride(lvl->nbins, sp.wmax))) *
                       sizeof(float);
  if (bytes > 200 * 1024)
    return set_error(LOKI_ERR_UNSUPPORTED, "nbins too large for complex pruning");
  *smem = (int)bytes;
  return LOKI_OK;
}

extern "C" int loki_prune_score_complex(const LokiPruneLevel* lvl, const double* leaves,
                                        const void* folds, int64_t n_parents,
                                        const LokiBranchInfo* info, const int64_t* offsets,
                                        int64_t n_children, const void* fold_segment,
                                        const LokiScoreSpec* spec, float* child_scores,
                                        int32_t* child_idx, double* child_phase,
                                        float* score_minmax, int32_t* dev_err, void* stream) {
  int rc = check_prune(lvl);
  if (rc) return rc;
  rc = prune_spec_check(spec, lvl->nbins);
  if (rc) return rc;
  if (!score_minmax || !dev_err) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned* keys = reinterpret_cast<unsigned*>(score_minmax);
  note_launch();
  minmax_init_kernel<<<1, 1, 0, s>>>(keys);
  if (n_children > 0) {
    if (!leaves || !folds || !info || !offsets || !fold_segment || !child_scores ||
        !child_idx || !child_phase)
      return set_error(LOKI_ERR_INVALID, "null pointer argument");
    LokiScoreSpec sp = *spec;
    sp.mode = 1;
    const ScoreK SK = make_score_k(sp, lvl->nbins);
    int smem = 0;
    rc = cplx_smem(lvl, sp, &smem);
    if (rc) return rc;
    if (set_smem_limit(prune_score_complex_kernel, smem) != cudaSuccess)
      return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
    const int64_t blocks = (n_children + kPruneWarps * 32 - 1) / (kPruneWarps * 32);
    if (blocks > 0x7FFFFFFF) return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
    note_launch();
    prune_score_complex_kernel<<<(unsigned)blocks, kPruneWarps * 32, smem, s>>>(
        *lvl, leaves, reinterpret_cast<const float2*>(folds), n_parents, info, offsets,
        n_children, reinterpret_cast<const float2*>(fold_segment), sp, SK, child_scores,
        child_idx, child_phase, keys);
  }
  note_launch();
  minmax_finish_kernel<<<1, 1, 0, s>>>(keys, score_minmax);
  return check_launch("prune_score_complex");
}

extern "C" int loki_prune_emit_complex(const LokiPruneLevel* lvl, const double* leaves,
                                       const void* folds, const LokiBranchInfo* info,
                                       const int64_t* offsets, int64_t n_parents,
                                       const void* fold_segment, const int64_t* surv_ids,
                                       int64_t n_surv, const float* child_scores,
                                       const int32_t* child_idx, const double* child_phase,
                                       double* leaves_out, void* folds_out, float* scores_out,
                                       float* scores_ep_out, int32_t* bt_out, void* stream) {
  int rc = check_prune(lvl);
  if (rc) return rc;
  if (n_surv <= 0) return LOKI_OK;
  if (!leaves || !folds || !info || !offsets || !fold_segment || !surv_ids || !child_scores ||
      !child_idx || !child_phase || !leaves_out || !folds_out || !scores_out ||
      !scores_ep_out || !bt_out)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  note_launch();
  prune_emit_complex_kernel<<<(unsigned)((n_surv + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
      *lvl, leaves, reinterpret_cast<const float2*>(folds), info, offsets, n_parents,
      reinterpret_cast<const float2*>(fold_segment), surv_ids, n_surv, child_scores, child_idx,
      child_phase, leaves_out, reinterpret_cast<float2*>(folds_out), scores_out, scores_ep_out,
      bt_out);
  return check_launch("prune_emit_complex");
}

extern "C" int loki_prune_ascend_complex(const LokiPruneLevel* lvl, const double* leaves,
                                         void* folds, float* scores, float* scores_ep,
                                         int64_t n, int32_t nseg, const double* tm_seg,
                                         const double* dt_seg, const int32_t* seg_idx,
                                         const void* ffa_fold, int64_t seg_stride,
                                         const LokiScoreSpec* spec, int32_t* dev_err,
                                         void* stream) {
  int rc = check_prune(lvl);
  if (rc) return rc;
  rc = prune_spec_check(spec, lvl->nbins);
  if (rc) return rc;
  if (n <= 0) return LOKI_OK;
  if (nseg < 1 || !leaves || !folds || !scores || !scores_ep || !tm_seg || !dt_seg ||
      !seg_idx || !ffa_fold || !dev_err)
    return set_error(LOKI_ERR_INVALID, "bad ascend arguments");
  LokiScoreSpec sp = *spec;
  sp.mode = 1;
  const ScoreK SK = make_score_k(sp, lvl->nbins);
  int smem = 0;
  rc = cplx_smem(lvl, sp, &smem);
  if (rc) return rc;
  if (set_smem_limit(prune_ascend_complex_kernel, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  const int64_t blocks = (n + kPruneWarps * 32 - 1) / (kPruneWarps * 32);
  note_launch();
  prune_ascend_complex_kernel<<<(unsigned)blocks, kPruneWarps * 32, smem,
                                (cudaStream_t)stream>>>(
      *lvl, leaves, reinterpret_cast<float2*>(folds), scores, scores_ep, n, nseg, tm_seg, dt_seg,
      seg_idx, reinterpret_cast<const float2*>(ffa_fold), seg_stride, sp, SK);
  return check_launch("prune_ascend_complex");
}

// ---------------------------------------------------------------------------
// device-resident run: every level of one reference segment with the counts
// kept on the device (counts[0] parents, [1] children, [2] survivors)
// ---------------------------------------------------------------------------

namespace loki {

__global__ void run_seed_kernel(int64_t* cnt, int64_t n, unsigned* keys) {
  cnt[0] = n;
  for (int k = 1; k < 8; ++k) cnt[k] = 0;
  keys[0] = 0xFFFFFFFFu;  // score min / max keys of the first level
  keys[1] = 0u;
}

__global__ void run_level_end_kernel(int64_t* cnt, unsigned* keys, int32_t* ovf_flag,
                                     LokiPruneLevelStats* st) {
  level_end(cnt, keys, ovf_flag, st);
}

// survivors' backtracks appended to the history at row counts[3]
__global__ void run_bt_copy_kernel(const int32_t* __restrict__ bt, const int64_t* cnt, int row,
                                   int32_t* __restrict__ hist, int64_t hist_rows,
                                   int32_t* err) {
  const int64_t start = cnt[3], rows = cnt[2];
  if (start + rows > hist_rows) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(err, LOKI_DEVERR_CAPACITY);
    return;
  }
  int32_t* out = hist + start * row;
  const int64_t n = rows * row;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = bt[i];
}

}  // namespace loki

// One circular-orbit level with device counts (counts[4] = valid children):
// branch (kept and crackle-expanded children per parent), the two scans, the
// batch-ordered child map, validation compaction, resolve + score, batch
// offsets of the valid children, selection with the overflow rule, emit.
static int circ_level_dev(const LokiPruneLevel& D, const LokiPruneTree& in,
                          const LokiPruneTree& out, const LokiPruneWork& w,
                          const LokiPruneRun* run, const float* seg, double thr,
                          const LokiScoreSpec& sp, const ScoreK& SK, int smem, int64_t max_sugg,
                          int64_t batch, unsigned g_par, unsigned g_flat, unsigned g_score,
                          unsigned g_emit, int scan_grid, int64_t* cnt, int64_t* pos,
                          int64_t sums_bytes, unsigned* keys, LokiPruneLevelStats* st,
                          int32_t* dev_err, cudaStream_t s) {
  LokiBranchInfo* info = reinterpret_cast<LokiBranchInfo*>(w.info);
  CircChild* map = reinterpret_cast<CircChild*>(run->child_map);
  note_launch();
  circ_branch_kernel<<<g_par, 256, 0, s>>>(D, in.leaves, 0, info, w.offsets, run->exp_off,
                                           dev_err, cnt);
  int rc = exclusive_scan_dev<false>(w.offsets, w.par_cap, cnt, 0.0, w.offsets, w.scan,
                                     w.scan_bytes, scan_grid, s);
  if (rc) return rc;
  rc = exclusive_scan_dev<false>(run->exp_off, w.par_cap, cnt, 0.0, run->exp_off, w.scan,
                                 w.scan_bytes, scan_grid, s);
  if (rc) return rc;
  note_launch();
  circ_map_kernel<<<g_par, 256, 0, s>>>(D, in.leaves, 0, batch, info, w.offsets, run->exp_off,
                                        map, run->valid_flags, cnt, w.child_cap, st, dev_err);
  // validation compaction: valid flags are 1.0 / 0.0
  rc = exclusive_scan_dev<true>(run->valid_flags, w.child_cap, cnt + 1, 0.5, pos, w.sscan,
                                sums_bytes, scan_grid, s);
  if (rc) return rc;
  for (int i = 0; i < 3; ++i) note_launch();
  select_scatter_kernel<<<g_flat, 256, 0, s>>>(run->valid_flags, 0, 0.5, pos, run->valid_ids,
                                               cnt + 1);
  if (cudaMemsetAsync(run->batch_taylor, 0,
                      (size_t)(w.par_cap / batch + 1) * sizeof(int32_t), s) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaMemsetAsync failed");
  circ_score_kernel<<<g_score, kPruneWarps * 32, smem, s>>>(
      D, in.leaves, in.folds, batch, info, map, run->valid_ids, 0, seg, sp, SK, w.child_scores,
      w.child_idx, w.child_phase, run->child_class, run->batch_taylor, keys, cnt, pos, st);
  circ_boff_kernel<<<g_par, 256, 0, s>>>(w.offsets, run->exp_off, 0, run->valid_ids, 0,
                                         run->batch_offsets, cnt);
  rc = exclusive_scan_dev<true>(w.child_scores, w.child_cap, cnt + 4, thr, pos, w.sscan,
                                sums_bytes, scan_grid, s);
  if (rc) return rc;
  for (int i = 0; i < 3; ++i) note_launch();
  select_scatter_kernel<<<g_flat, 256, 0, s>>>(w.child_scores, 0, thr, pos, w.surv, cnt + 4);
  select_overflow_kernel<<<1, kSelThreads, 0, s>>>(
      w.child_scores, run->batch_offsets, 0, batch, thr, max_sugg, w.surv, cnt + 2, w.ovf_thr,
      w.ovf_ids, reinterpret_cast<unsigned*>(w.ovf_keys), cnt, run->ovf_flag, pos, cnt + 4);
  circ_emit_kernel<<<g_emit, kPruneWarps * 32, 0, s>>>(
      D, in.leaves, in.folds, batch, info, map, run->valid_ids, seg, w.surv, 0, w.child_scores,
      w.child_idx, w.child_phase, run->child_class, run->batch_taylor, out.leaves, out.folds,
      out.scores, out.scores_ep, out.backtracks, cnt);
  return LOKI_OK;
}

extern "C" int loki_prune_run(const LokiPruneLevel* lvls, int32_t nlevels, const float* ffa_folds,
                              int64_t seg_stride, const int32_t* seg_idx,
                              const double* thresholds, const LokiScoreSpec* spec,
                              int64_t seed_n, int64_t max_sugg, int64_t batch_size,
                              const LokiPruneRun* run, int32_t* dev_err, void* stream) {
  if (!lvls || nlevels < 1 || !ffa_folds || !seg_idx || !thresholds || !spec || !run ||
      !dev_err)
    return set_error(LOKI_ERR_INVALID, "null pointer or no level");
  if (max_sugg < 1 || batch_size < 1 || seed_n < 0 || seed_n > max_sugg || seg_stride < 1)
    return set_error(LOKI_ERR_INVALID, "bad sizes");
  const LokiPruneWork& w = run->work;
  const LokiPruneTree* tr = run->trees;
  if (tr[0].cap < max_sugg || tr[1].cap < max_sugg || w.par_cap < max_sugg || w.child_cap < 1 ||
      w.ovf_cap < max_sugg + w.child_cap + 1)
    return set_error(LOKI_ERR_CAPACITY, "run workspace below max_sugg / child_cap");
  if (!run->counts || !run->ovf_flag || !run->stats || !w.info || !w.offsets || !w.scan ||
      !w.child_scores || !w.child_idx || !w.child_phase || !w.surv || !w.sscan || !w.minmax ||
      !w.ovf_ids || !w.ovf_keys || !w.ovf_thr)
    return set_error(LOKI_ERR_INVALID, "null workspace pointer");
  for (int l = 0; l < nlevels; ++l) {
    int rc = check_prune(&lvls[l]);
    if (rc) return rc;
    if (lvls[l].basis != lvls[0].basis || lvls[l].poly_order != lvls[0].poly_order ||
        lvls[l].nbins != lvls[0].nbins)
      return set_error(LOKI_ERR_INVALID, "levels of different trees");
  }
  const bool circ = lvls[0].basis == 2;
  if (circ && (lvls[0].poly_order != 5 || !run->exp_off || !run->child_map ||
               !run->valid_flags || !run->valid_ids || !run->child_class ||
               !run->batch_taylor || !run->batch_offsets))
    return set_error(LOKI_ERR_INVALID, "the circular-orbit tree needs poly_order 5 and its "
                                       "workspace");
  int rc = prune_spec_check(spec, lvls[0].nbins);
  if (rc) return rc;
  const int64_t sums_bytes = loki_scan_scratch_bytes(w.child_cap);
  if (w.scan_bytes < loki_scan_scratch_bytes(w.par_cap + 1) ||
      w.sscan_bytes < sums_bytes + (w.child_cap + 1) * (int64_t)sizeof(int64_t))
    return set_error(LOKI_ERR_CAPACITY, "scan scratch below par_cap / child_cap");
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = lvls[0].nbins, P = lvls[0].poly_order;
  LokiScoreSpec sp = *spec;
  sp.mode = 1;
  const ScoreK SK = make_score_k(sp, nb);
  const int smem = score_smem_bytes(nb, sp.wmax, kPruneWarps);
  if (smem > 200 * 1024)
    return set_error(LOKI_ERR_UNSUPPORTED, "nbins + wmax too large for pruning");
  if (smem > 48 * 1024 && (set_smem_limit(prune_score_kernel, smem) != cudaSuccess ||
                           set_smem_limit(circ_score_kernel, smem) != cudaSuccess))
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  int dev = 0, nsm = 0, occ_s = 0, occ_e = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      (circ ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, circ_score_kernel,
                                                            kPruneWarps * 32, smem)
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_s, prune_score_kernel,
                                                            kPruneWarps * 32, smem)) !=
          cudaSuccess ||
      (circ ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_e, circ_emit_kernel,
                                                            kPruneWarps * 32, 0)
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_e, prune_emit_kernel,
                                                            kPruneWarps * 32, 0)) !=
          cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "occupancy query failed");
  // grids: one full wave of the score / emit kernels, and enough blocks for
  // the parent-sized and child-sized passes to stride through
  const unsigned g_score = (unsigned)std::max(1, nsm * std::max(1, occ_s));
  const unsigned g_emit = (unsigned)std::max(1, nsm * std::max(1, occ_e));
  const unsigned g_par = (unsigned)std::min<int64_t>((w.par_cap + 255) / 256, 8 * nsm);
  const unsigned g_flat = (unsigned)(4 * nsm);
  const int scan_grid = 2 * nsm;
  int64_t* cnt = run->counts;
  int64_t* pos = reinterpret_cast<int64_t*>(reinterpret_cast<char*>(w.sscan) + sums_bytes);
  unsigned* keys = reinterpret_cast<unsigned*>(w.minmax);
  const int row_bt = P + 2, row_leaf = (P + 2) * 2;
  note_launch();
  run_seed_kernel<<<1, 1, 0, s>>>(cnt, seed_n, keys);
  for (int l = 1; l <= nlevels; ++l) {
    const LokiPruneLevel& D = lvls[l - 1];
    const LokiPruneTree& in = tr[(l - 1) & 1];
    const LokiPruneTree& out = tr[l & 1];
    const float* seg = ffa_folds + (int64_t)seg_idx[l - 1] * seg_stride;
    const double thr = thresholds[l - 1];
    LokiPruneLevelStats* st = run->stats + (l - 1);
    LokiBranchInfo* info = reinterpret_cast<LokiBranchInfo*>(w.info);
    if (circ) {
      rc = circ_level_dev(D, in, out, w, run, seg, thr, sp, SK, smem, max_sugg, batch_size,
                          g_par, g_flat, g_score, g_emit, scan_grid, cnt, pos, sums_bytes, keys,
                          st, dev_err, s);
      if (rc) return rc;
    } else {
    note_launch();
    prune_branch_kernel<<<g_par, 256, 0, s>>>(D, in.leaves, w.par_cap, info, w.offsets, dev_err,
                                              nullptr, cnt);
    rc = exclusive_scan_dev<false>(w.offsets, w.par_cap, cnt, 0.0, w.offsets, w.scan,
                                   w.scan_bytes, scan_grid, s);
    if (rc) return rc;
    note_launch();
    prune_score_kernel<<<g_score, kPruneWarps * 32, smem, s>>>(
        D, in.leaves, in.folds, 0, info, w.offsets, 0, seg, sp, SK, w.child_scores, w.child_idx,
        w.child_phase, keys, cnt, w.child_cap, st, dev_err);
    rc = exclusive_scan_dev<true>(w.child_scores, w.child_cap, cnt + 1, thr, pos, w.sscan,
                                  sums_bytes, scan_grid, s);
    if (rc) return rc;
    for (int i = 0; i < 3; ++i) note_launch();
    select_scatter_kernel<<<g_flat, 256, 0, s>>>(w.child_scores, 0, thr, pos, w.surv, cnt + 1);
    select_overflow_kernel<<<1, kSelThreads, 0, s>>>(
        w.child_scores, w.offsets, 0, batch_size, thr, max_sugg, w.surv, cnt + 2, w.ovf_thr,
        w.ovf_ids, reinterpret_cast<unsigned*>(w.ovf_keys), cnt, run->ovf_flag, pos, cnt + 1);
    prune_emit_kernel<<<g_emit, kPruneWarps * 32, 0, s>>>(
        D, in.leaves, in.folds, info, w.offsets, 0, seg, w.surv, 0, w.child_scores, w.child_idx,
        w.child_phase, out.leaves, out.folds, out.scores, out.scores_ep, out.backtracks, cnt);
    }
    if (run->bt_hist) {  // before the level end moves the counters on
      note_launch();
      run_bt_copy_kernel<<<g_flat, 256, 0, s>>>(out.backtracks, cnt, row_bt, run->bt_hist,
                                                run->bt_rows, dev_err);
    }
    note_launch();
    if (run->best_leaves && run->best_scores) {  // best leaf, then the level end
      prune_best_kernel<<<1, 1024, 0, s>>>(out.scores, 0, out.leaves, row_leaf,
                                           run->best_leaves + (int64_t)(l - 1) * row_leaf,
                                           run->best_scores + (l - 1), cnt, keys,
                                           run->ovf_flag, st);
    } else {
      run_level_end_kernel<<<1, 1, 0, s>>>(cnt, keys, run->ovf_flag, st);
    }
    rc = check_launch("prune_run");
    if (rc) return rc;
  }
  return LOKI_OK;
}

// ---------------------------------------------------------------------------
// block-per-run driver: one thread block runs every level of one job (a
// reference segment of a fold) with block barriers between the steps, so a
// batch of jobs is one launch instead of ~13 dependent launches per level
// and job. The steps are those of loki_prune_run (Taylor and Chebyshev
// trees): branch, scan, score, select (with the overflow rule), emit,
// backtrack history, best leaf and level record.
// ---------------------------------------------------------------------------

namespace loki {

constexpr int kRunThreads = 512;  // 16 warps a job

// Exclusive scan of in[0..n) (int64 counts, or score >= thr flags) into
// out[0..n), out[n] = total, by one block; in may be out. Returns the total.
template <bool FLAGS>
__device__ int64_t block_scan64(const void* in, int64_t n, double thr, int64_t* out,
                                int64_t* warp_tot) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int64_t carry = 0;
  for (int64_t base = 0; base < n; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const int64_t x = scan_in<FLAGS>(in, i, n, thr);
    int64_t v = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xFFFFFFFFu, v, o);
      if (lane >= o) v += y;
    }
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    if (warp == 0) {
      int64_t w = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
        if (lane >= o) w += y;
      }
      warp_tot[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const int64_t incl = v + (warp ? warp_tot[warp - 1] : 0);
    if (i < n) out[i] = carry + incl - x;
    carry += warp_tot[nw - 1];
    __syncthreads();  // warp_tot is rewritten by the next tile
  }
  if (threadIdx.x == 0) out[n] = carry;
  __syncthreads();
  return carry;
}

__global__ void __launch_bounds__(kRunThreads, 1)
prune_block_run_kernel(const LokiPruneJob* __restrict__ jobs,
                       const LokiPruneLevel* __restrict__ levels,
                       const int32_t* __restrict__ seg_idx, const double* __restrict__ thr_all,
                       int32_t nlevels, LokiScoreSpec sp, ScoreK SK, int64_t max_sugg,
                       int64_t batch) {
  extern __shared__ float tiles[];
  __shared__ int64_t warp_tot[32];
  __shared__ int64_t n_sh;
  const LokiPruneJob& J = jobs[blockIdx.x];
  const LokiPruneRun& R = J.run;
  const LokiPruneWork& w = R.work;
  const int tid = threadIdx.x, warp = tid >> 5, nwarps = blockDim.x >> 5;
  float* tile = tiles + (size_t)warp * 32 * score_stride(levels[0].nbins, sp.wmax);
  int64_t* cnt = R.counts;
  unsigned* keys = reinterpret_cast<unsigned*>(w.minmax);
  LokiBranchInfo* info = reinterpret_cast<LokiBranchInfo*>(w.info);
  // selection positions after the scan sums, as loki_prune_run places them
  const int64_t sums_bytes = (int64_t)max((int64_t)1, (w.child_cap + kScanBlock - 1) / kScanBlock) * 8;
  int64_t* pos = reinterpret_cast<int64_t*>(reinterpret_cast<char*>(w.sscan) + sums_bytes);
  const int P = levels[0].poly_order;
  const int row_bt = P + 2, row_leaf = (P + 2) * 2;
  if (tid == 0) {
    cnt[0] = J.seed_n;
    for (int k = 1; k < 8; ++k) cnt[k] = 0;
    keys[0] = 0xFFFFFFFFu;
    keys[1] = 0u;
    *R.ovf_flag = 0;
  }
  __syncthreads();
  int64_t n_par = J.seed_n;
  for (int l = 1; l <= nlevels; ++l) {
    const LokiPruneLevel& D = levels[(size_t)blockIdx.x * nlevels + (l - 1)];
    const LokiPruneTree& in = R.trees[(l - 1) & 1];
    const LokiPruneTree& out = R.trees[l & 1];
    const float* seg = J.ffa_fold + (int64_t)seg_idx[(size_t)blockIdx.x * nlevels + (l - 1)] *
                                        J.seg_stride;
    const double thr = thr_all[(size_t)blockIdx.x * nlevels + (l - 1)];
    LokiPruneLevelStats* st = R.stats + (l - 1);
    // branch and the child offsets
    for (int64_t i = tid; i < n_par; i += blockDim.x)
      branch_one(D, in.leaves, i, info, w.offsets, J.dev_err, nullptr);
    __syncthreads();
    const int64_t total = block_scan64<false>(w.offsets, n_par, 0.0, w.offsets, warp_tot);
    const int64_t n_child = total > w.child_cap ? 0 : total;
    if (tid == 0) {
      cnt[1] = n_child;
      st->n_parents = n_par;
      st->n_children = total;
      st->n_valid = total;
      if (total > w.child_cap) atomicOr(J.dev_err, LOKI_DEVERR_CAPACITY);
    }
    // score every child
    for (int64_t t = warp; t * 32 < n_child; t += nwarps) {
      score_tile(D, in.leaves, in.folds, n_par, info, w.offsets, n_child, seg, sp, SK,
                 w.child_scores, w.child_idx, w.child_phase, keys, tile, t * 32);
      __syncwarp();  // the tile rows are rewritten by the next tile
    }
    __syncthreads();
    // select: survivors in order, then the overflow rule when they exceed max_sugg
    const int64_t n_sel = block_scan64<true>(w.child_scores, n_child, thr, pos, warp_tot);
    for (int64_t i = tid; i < n_child; i += blockDim.x)
      if ((double)w.child_scores[i] >= thr) w.surv[pos[i]] = i;
    if (tid == 0) n_sh = n_sel;
    __syncthreads();
    if (n_sel > max_sugg) {  // uniform over the block
      if (tid == 0) *R.ovf_flag = 1;
      select_overflow_block(w.child_scores, w.offsets, n_par, batch, thr, max_sugg, w.surv,
                            &n_sh, w.ovf_thr, w.ovf_ids, reinterpret_cast<unsigned*>(w.ovf_keys));
    }
    const int64_t n_surv = n_sh;
    // the next tree
    for (int64_t t = warp; t * 32 < n_surv; t += nwarps)
      emit_tile(D, in.leaves, in.folds, info, w.offsets, n_par, seg, w.surv, n_surv,
                w.child_scores, w.child_idx, w.child_phase, out.leaves, out.folds, out.scores,
                out.scores_ep, out.backtracks, t * 32);
    __syncthreads();
    // backtrack history, best leaf, level record
    if (R.bt_hist) {
      const int64_t start = cnt[3];
      if (start + n_surv > R.bt_rows) {
        if (tid == 0) atomicOr(J.dev_err, LOKI_DEVERR_CAPACITY);
      } else {
        int32_t* h = R.bt_hist + start * row_bt;
        for (int64_t i = tid; i < n_surv * row_bt; i += blockDim.x) h[i] = out.backtracks[i];
      }
    }
    if (R.best_leaves && R.best_scores)
      block_best(out.scores, n_surv, out.leaves, row_leaf,
                 R.best_leaves + (int64_t)(l - 1) * row_leaf, R.best_scores + (l - 1));
    __syncthreads();
    if (tid == 0) {
      cnt[2] = n_surv;
      level_end(cnt, keys, R.ovf_flag, st);
    }
    __syncthreads();
    n_par = n_surv;
  }
}

}  // namespace loki

extern "C" int64_t loki_prune_run_blocks_scratch_bytes(int32_t njobs, int32_t nlevels) {
  if (njobs < 1 || nlevels < 1) return 0;
  const int64_t nl = (int64_t)njobs * nlevels;
  return ((int64_t)njobs * sizeof(LokiPruneJob) + 255) / 256 * 256 +
         (nl * (int64_t)sizeof(LokiPruneLevel) + 255) / 256 * 256 +
         (nl * 4 + 255) / 256 * 256 + nl * 8;
}

extern "C" int loki_prune_run_blocks(const LokiPruneJob* jobs, int32_t njobs,
                                     const LokiPruneLevel* levels, const int32_t* seg_idx,
                                     const double* thresholds, int32_t nlevels,
                                     const LokiScoreSpec* spec, int64_t max_sugg,
                                     int64_t batch_size, void* dev_scratch,
                                     int64_t dev_scratch_bytes, void* stream) {
  if (!jobs || njobs < 1 || !levels || !seg_idx || !thresholds || nlevels < 1 || !spec ||
      !dev_scratch)
    return set_error(LOKI_ERR_INVALID, "null pointer, no job or no level");
  if (max_sugg < 1 || batch_size < 1)
    return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (dev_scratch_bytes < loki_prune_run_blocks_scratch_bytes(njobs, nlevels))
    return set_error(LOKI_ERR_CAPACITY, "job scratch below %lld bytes",
                     (long long)loki_prune_run_blocks_scratch_bytes(njobs, nlevels));
  const int nb = levels[0].nbins;
  for (int64_t k = 0; k < (int64_t)njobs * nlevels; ++k) {
    int rc = check_prune(&levels[k]);
    if (rc) return rc;
    if (levels[k].basis != levels[0].basis || levels[k].poly_order != levels[0].poly_order ||
        levels[k].nbins != nb)
      return set_error(LOKI_ERR_INVALID, "levels of different trees");
  }
  if (levels[0].basis == 2)
    return set_error(LOKI_ERR_UNSUPPORTED, "the circular-orbit tree runs in loki_prune_run");
  for (int j = 0; j < njobs; ++j) {
    const LokiPruneJob& J = jobs[j];
    const LokiPruneRun& R = J.run;
    const LokiPruneWork& w = R.work;
    if (!J.ffa_fold || J.seg_stride < 1 || !J.dev_err || J.seed_n < 0 || J.seed_n > max_sugg)
      return set_error(LOKI_ERR_INVALID, "job %d: bad fold, error word or seed", j);
    if (R.trees[0].cap < max_sugg || R.trees[1].cap < max_sugg || w.par_cap < max_sugg ||
        w.child_cap < 1 || w.ovf_cap < max_sugg + w.child_cap + 1)
      return set_error(LOKI_ERR_CAPACITY, "job %d: workspace below max_sugg / child_cap", j);
    if (!R.counts || !R.ovf_flag || !R.stats || !w.info || !w.offsets || !w.child_scores ||
        !w.child_idx || !w.child_phase || !w.surv || !w.sscan || !w.minmax || !w.ovf_ids ||
        !w.ovf_keys || !w.ovf_thr)
      return set_error(LOKI_ERR_INVALID, "job %d: null workspace pointer", j);
    if (w.sscan_bytes <
        loki_scan_scratch_bytes(w.child_cap) + (w.child_cap + 1) * (int64_t)sizeof(int64_t))
      return set_error(LOKI_ERR_CAPACITY, "job %d: selection scratch below child_cap", j);
    for (int t = 0; t < 2; ++t)
      if (!R.trees[t].leaves || !R.trees[t].folds || !R.trees[t].scores ||
          !R.trees[t].scores_ep || !R.trees[t].backtracks)
        return set_error(LOKI_ERR_INVALID, "job %d: null tree pointer", j);
  }
  int rc = prune_spec_check(spec, nb);
  if (rc) return rc;
  LokiScoreSpec sp = *spec;
  sp.mode = 1;
  const ScoreK SK = make_score_k(sp, nb);
  const int smem = (kRunThreads / 32) * 32 * score_stride(nb, sp.wmax) * (int)sizeof(float);
  if (smem > 200 * 1024)
    return set_error(LOKI_ERR_UNSUPPORTED, "nbins + wmax too large for the block driver");
  if (set_smem_limit(prune_block_run_kernel, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  const int64_t nl = (int64_t)njobs * nlevels;
  char* base = reinterpret_cast<char*>(dev_scratch);
  const int64_t o_lv = ((int64_t)njobs * sizeof(LokiPruneJob) + 255) / 256 * 256;
  const int64_t o_si = o_lv + (nl * (int64_t)sizeof(LokiPruneLevel) + 255) / 256 * 256;
  const int64_t o_th = o_si + (nl * 4 + 255) / 256 * 256;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(base, jobs, njobs * sizeof(LokiPruneJob), cudaMemcpyHostToDevice, s) !=
          cudaSuccess ||
      cudaMemcpyAsync(base + o_lv, levels, nl * sizeof(LokiPruneLevel), cudaMemcpyHostToDevice,
                      s) != cudaSuccess ||
      cudaMemcpyAsync(base + o_si, seg_idx, nl * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(base + o_th, thresholds, nl * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "copy of the job tables failed");
  note_launch();
  prune_block_run_kernel<<<(unsigned)njobs, kRunThreads, smem, s>>>(
      reinterpret_cast<const LokiPruneJob*>(base),
      reinterpret_cast<const LokiPruneLevel*>(base + o_lv),
      reinterpret_cast<const int32_t*>(base + o_si), reinterpret_cast<const double*>(base + o_th),
      nlevels, sp, SK, max_sugg, batch_size);
  return check_launch("prune_block_run");
}

// ---------------------------------------------------------------------------
// level-synchronous batch: every step of a level is one launch over all jobs
// (blockIdx.y = job), so a batch of jobs costs the launches of one run and
// each step spreads over the whole GPU. The device code is that of
// loki_prune_run; the counters, records and results of job j are those a
// loki_prune_run of job j writes.
// ---------------------------------------------------------------------------

namespace loki {

struct BatchTabs {
  const LokiPruneJob* jobs;
  const LokiPruneLevel* levels;  // [job][level]
  const int32_t* seg_idx;        // [job][level]
  const double* thr;             // [job][level]
  int32_t nlevels;
};

__device__ __forceinline__ int64_t* job_pos(const LokiPruneWork& w) {
  const int64_t sums = (int64_t)max((int64_t)1, (w.child_cap + kScanBlock - 1) / kScanBlock) * 8;
  return reinterpret_cast<int64_t*>(reinterpret_cast<char*>(w.sscan) + sums);
}

__global__ void bj_seed_kernel(BatchTabs T) {
  const LokiPruneJob& J = T.jobs[blockIdx.x];
  int64_t* cnt = J.run.counts;
  cnt[0] = J.seed_n;
  for (int k = 1; k < 8; ++k) cnt[k] = 0;
  unsigned* keys = reinterpret_cast<unsigned*>(J.run.work.minmax);
  keys[0] = 0xFFFFFFFFu;
  keys[1] = 0u;
  *J.run.ovf_flag = 0;
}

__global__ void bj_branch_kernel(BatchTabs T, int l) {
  const LokiPruneJob& J = T.jobs[blockIdx.y];
  const LokiPruneLevel& D = T.levels[(size_t)blockIdx.y * T.nlevels + (l - 1)];
  const LokiPruneWork& w = J.run.work;
  const int64_t n = J.run.counts[0];
  const double* leaves = J.run.trees[(l - 1) & 1].leaves;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    branch_one(D, leaves, i, reinterpret_cast<LokiBranchInfo*>(w.info), w.offsets, J.dev_err,
               nullptr);
}

// The scans of a level, per job. Counts (in place, scratch w.scan): mode 0
// the parents' child counts (offsets), mode 2 the circular tree's crackle
// expansion counts (exp_off), both over counts[0] parents. Flags (into the
// positions after w.sscan's sums): mode 1 score >= threshold over counts[1]
// children, mode 3 the circular tree's validity flags over counts[1]
// children, mode 4 score >= threshold over counts[4] valid children.
__device__ __forceinline__ void bj_scan_args(const BatchTabs& T, int l, int mode,
                                             const void** in, int64_t** out, int64_t** sums,
                                             int64_t* n, double* thr) {
  const LokiPruneJob& J = T.jobs[blockIdx.y];
  const LokiPruneWork& w = J.run.work;
  if (mode == 0 || mode == 2) {
    int64_t* a = mode == 0 ? w.offsets : J.run.exp_off;
    *in = a;
    *out = a;
    *sums = reinterpret_cast<int64_t*>(w.scan);
    *n = J.run.counts[0];
    *thr = 0.0;
  } else {
    *in = mode == 3 ? static_cast<const void*>(J.run.valid_flags)
                    : static_cast<const void*>(w.child_scores);
    *out = job_pos(w);
    *sums = reinterpret_cast<int64_t*>(w.sscan);
    *n = J.run.counts[mode == 4 ? 4 : 1];
    *thr = mode == 3 ? 0.5 : T.thr[(size_t)blockIdx.y * T.nlevels + (l - 1)];
  }
}

template <bool FLAGS>
__global__ void __launch_bounds__(kScanBlock) bj_scan_block_kernel(BatchTabs T, int l, int mode) {
  __shared__ int64_t warp_tot[32];
  const void* in;
  int64_t *out, *sums, n;
  double thr;
  bj_scan_args(T, l, mode, &in, &out, &sums, &n, &thr);
  const int64_t ntiles = (n + kScanBlock - 1) / kScanBlock;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x)
    scan_tile<FLAGS>(in, n, thr, out, sums, t, warp_tot);
}

template <bool FLAGS>
__global__ void __launch_bounds__(kScanBlock) bj_scan_sums_kernel(BatchTabs T, int l, int mode) {
  __shared__ int64_t warp_tot[32];
  __shared__ int64_t carry;
  const void* in;
  int64_t *out, *sums, n;
  double thr;
  bj_scan_args(T, l, mode, &in, &out, &sums, &n, &thr);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t nblocks = (n + kScanBlock - 1) / kScanBlock;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < nblocks; base += kScanBlock) {
    const int64_t i = base + threadIdx.x;
    const int64_t x = i < nblocks ? sums[i] : 0;
    int64_t v = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xFFFFFFFFu, v, o);
      if (lane >= o) v += y;
    }
    if (lane == 31) warp_tot[warp] = v;
    __syncthreads();
    if (warp == 0) {
      int64_t w = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xFFFFFFFFu, w, o);
        if (lane >= o) w += y;
      }
      warp_tot[lane] = w;
    }
    __syncthreads();
    const int64_t incl = v + (warp ? warp_tot[warp - 1] : 0);
    const int64_t c = carry;
    if (i < nblocks) sums[i] = c + incl - x;
    __syncthreads();
    if (threadIdx.x == kScanBlock - 1) carry = c + incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) out[n] = carry;
}

template <bool FLAGS>
__global__ void __launch_bounds__(kScanBlock) bj_scan_add_kernel(BatchTabs T, int l, int mode) {
  const void* in;
  int64_t *out, *sums, n;
  double thr;
  bj_scan_args(T, l, mode, &in, &out, &sums, &n, &thr);
  for (int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kScanBlock)
    out[i] += sums[i / kScanBlock];
}

__global__ void __launch_bounds__(kPruneWarps * 32, 4)
bj_score_kernel(BatchTabs T, int l, LokiScoreSpec sp, ScoreK SK) {
  extern __shared__ float tiles[];
  const LokiPruneJob& J = T.jobs[blockIdx.y];
  const size_t li = (size_t)blockIdx.y * T.nlevels + (l - 1);
  const LokiPruneLevel& D = T.levels[li];
  const LokiPruneRun& R = J.run;
  const LokiPruneWork& w = R.work;
  const LokiPruneTree& in = R.trees[(l - 1) & 1];
  const float* seg = J.ffa_fold + (int64_t)T.seg_idx[li] * J.seg_stride;
  const int warp = threadIdx.x >> 5;
  float* tile = tiles + (size_t)warp * 32 * score_stride(D.nbins, sp.wmax);
  int64_t* cnt = R.counts;
  const int64_t n_par = cnt[0];
  const int64_t total = w.offsets[n_par];
  const int64_t n_child = total > w.child_cap ? 0 : total;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cnt[1] = n_child;
    LokiPruneLevelStats* st = R.stats + (l - 1);
    st->n_parents = n_par;
    st->n_children = total;
    st->n_valid = total;
    if (total > w.child_cap) atomicOr(J.dev_err, LOKI_DEVERR_CAPACITY);
  }
  for (int64_t t = (int64_t)blockIdx.x * kPruneWarps + warp; t * 32 < n_child;
       t += (int64_t)gridDim.x * kPruneWarps) {
    score_tile(D, in.leaves, in.folds, n_par, reinterpret_cast<LokiBranchInfo*>(w.info),
               w.offsets, n_child, seg, sp, SK, w.child_scores, w.child_idx, w.child_phase,
               reinterpret_cast<unsigned*>(w.minmax), tile, t * 32);
    __syncwarp();
  }
}

// mode 1: survivors among counts[1] children; mode 3: the circular tree's
// valid children (valid_ids) among counts[1]; mode 4: survivors among
// counts[4] valid children.
__global__ void bj_scatter_kernel(BatchTabs T, int l, int mode) {
  const LokiPruneJob& J = T.jobs[blockIdx.y];
  const LokiPruneWork& w = J.run.work;
  const double thr = mode == 3 ? 0.5 : T.thr[(size_t)blockIdx.y * T.nlevels + (l - 1)];
  const float* f = mode == 3 ? J.run.valid_flags : w.child_scores;
  int64_t* ids = mode == 3 ? J.run.valid_ids : w.surv;
  const int64_t n = J.run.counts[mode == 4 ? 4 : 1];
  const int64_t* pos = job_pos(w);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if ((double)f[i] >= thr) ids[pos[i]] = i;
}

// one block per job: the survivor count, and the overflow rule when it
// exceeds max_sugg
__global__ void __launch_bounds__(kSelThreads)
bj_overflow_kernel(BatchTabs T, int l, int64_t max_sugg, int64_t batch, int circ) {
  const LokiPruneJob& J = T.jobs[blockIdx.x];
  const LokiPruneRun& R = J.run;
  const LokiPruneWork& w = R.work;
  int64_t* cnt = R.counts;
  const int64_t n_sel = job_pos(w)[cnt[circ ? 4 : 1]];
  const int64_t n_par = cnt[0];
  __syncthreads();  // every thread has read the counters
  if (threadIdx.x == 0) cnt[2] = n_sel;
  if (n_sel <= max_sugg) return;  // uniform over the block
  if (threadIdx.x == 0) *R.ovf_flag = 1;
  // the circular tree's batches are over its valid children
  select_overflow_block(w.child_scores, circ ? R.batch_offsets : w.offsets, n_par, batch,
                        T.thr[(size_t)blockIdx.x * T.nlevels + (l - 1)], max_sugg, w.surv,
                        cnt + 2, w.ovf_thr, w.ovf_ids, reinterpret_cast<unsigned*>(w.ovf_keys));
}

__global__ void __launch_bounds__(kPruneWarps * 32) bj_emit_kernel(BatchTabs T, int l) {
  const LokiPruneJob& J = T.jobs[blockIdx.y];
  const size_t li = (size_t)blockIdx.y * T.nlevels + (l - 1);
  const LokiPruneLevel& D = T.levels[li];
  const LokiPruneRun& R = J.run;
  const LokiPruneWork& w = R.work;
  const LokiPruneTree& in = R.trees[(l - 1) & 1];
  const LokiPruneTree& out = R.trees[l & 1];
  const float* seg = J.ffa_fold + (int64_t)T.seg_idx[li] * J.seg_stride;
  const int warp = threadIdx.x >> 5;
  const int64_t n_par = R.counts[0], n_surv = R.counts[2];
  for (int64_t t = (int64_t)blockIdx.x * kPruneWarps + warp; t * 32 < n_surv;
       t += (int64_t)gridDim.x * kPruneWarps)
    emit_tile(D, in.leaves, in.folds, reinterpret_cast<LokiBranchInfo*>(w.info), w.offsets,
              n_par, seg, w.surv, n_surv, w.child_scores, w.child_idx, w.child_phase,
              out.leaves, out.folds, out.scores, out.scores_ep, out.backtracks, t * 32);
}

// complex (Fourier-domain) trees: the per-child functions of the complex
// level kernels, grid-stride over each job's device counts. The jobs' fold
// rows and segment strides are in complex (float2) units.
__global__ void __launch_bounds__(kPruneWarps * 32)
bj_score_complex_kernel(BatchTabs T, int l, LokiScoreSpec sp) {
  extern __shared__ float smem[];
  const LokiPruneJob& J = T.jobs[blockIdx.y];
  const size_t li = (size_t)blockIdx.y * T.nlevels + (l - 1);
  const LokiPruneLevel& D = T.levels[li];
  const LokiPruneRun& R = J.run;
  const LokiPruneWork& w = R.work;
  const LokiPruneTree& in = R.trees[(l - 1) & 1];
  const float2* seg = reinterpret_cast<const float2*>(J.ffa_fold) + (int64_t)T.seg_idx[li] *
                                                                        J.seg_stride;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nb = D.nbins, nbf = nb / 2 + 1;
  const int stride = score_stride(nb, sp.wmax);
  float* tw = smem;
  load_twiddles(tw, nb);
  __syncthreads();
  float* wbase = smem + 2 * nb + (size_t)warp * cplx_warp_floats(nb, stride);
  float2* comb = reinterpret_cast<float2*>(wbase) + (size_t)lane * 2 * nbf;
  float* trow = wbase + (size_t)32 * 2 * nbf * 2 + lane * stride;
  int64_t* cnt = R.counts;
  const int64_t n_par = cnt[0];
  const int64_t total = w.offsets[n_par];
  const int64_t n_child = total > w.child_cap ? 0 : total;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cnt[1] = n_child;
    LokiPruneLevelStats* st = R.stats + (l - 1);
    st->n_parents = n_par;
    st->n_children = total;
    st->n_valid = total;
    if (total > w.child_cap) atomicOr(J.dev_err, LOKI_DEVERR_CAPACITY);
  }
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n_child;
       c += (int64_t)gridDim.x * blockDim.x)
    score_child_complex(D, in.leaves, reinterpret_cast<const float2*>(in.folds), n_par,
                        reinterpret_cast<LokiBranchInfo*>(w.info), w.offsets, seg, sp,
                        w.child_scores, w.child_idx, w.child_phase,
                        reinterpret_cast<unsigned*>(w.minmax), tw, comb, trow, c);
}

__global__ void __launch_bounds__(kPruneWarps * 32) bj_emit_complex_kernel(BatchTabs T, int l) {
  const LokiPruneJob& J = T.jobs[blockIdx.y];
  const size_t li = (size_t)blockIdx.y * T.nlevels + (l - 1);
  const LokiPruneLevel& D = T.levels[li];
  const LokiPruneRun& R = J.run;
  const LokiPruneWork& w = R.work;
  const LokiPruneTree& in = R.trees[(l - 1) & 1];
  const LokiPruneTree& out = R.trees[l & 1];
  const float2* seg = reinterpret_cast<const float2*>(J.ffa_fold) + (int64_t)T.seg_idx[li] *
                                                                        J.seg_stride;
  const int64_t n_par = R.counts[0], n_surv = R.counts[2];
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n_surv;
       s += (int64_t)gridDim.x * blockDim.x)
    emit_one_complex(D, in.leaves, reinterpret_cast<const float2*>(in.folds),
                     reinterpret_cast<LokiBranchInfo*>(w.info), w.offsets, n_par, seg, w.surv,
                     w.child_scores, w.child_idx, w.child_phase, out.leaves,
                     reinterpret_cast<float2*>(out.folds), out.scores, out.scores_ep,
                     out.backtracks, s);
}

// circular-orbit tree (real folds): the steps of circ_level_dev per job
__global__ void bj_circ_branch_kernel(BatchTabs T, int l) {
  const LokiPruneJob& J = T.jobs[blockIdx.y];
  const LokiPruneLevel& D = T.levels[(size_t)blockIdx.y * T.nlevels + (l - 1)];
  const LokiPruneRun& R = J.run;
  const int64_t n = R.counts[0];
  const double* leaves = R.trees[(l - 1) & 1].leaves;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    circ_branch_one(D, leaves, i, reinterpret_cast<LokiBranchInfo*>(R.work.info),
                    R.work.offsets, R.exp_off, J.dev_err);
}

// the batch-ordered child map and validity flags; counts[1] = every child,
// or 0 above the workspace (flagged)
__global__ void bj_circ_map_kernel(BatchTabs T, int l, int64_t batch) {
  const LokiPruneJob& J = T.jobs[blockIdx.y];
  const LokiPruneLevel& D = T.levels[(size_t)blockIdx.y * T.nlevels + (l - 1)];
  const LokiPruneRun& R = J.run;
  const LokiPruneWork& w = R.work;
  int64_t* cnt = R.counts;
  const int64_t n = cnt[0];
  const int64_t total = w.offsets[n] + R.exp_off[n];
  const bool fits = total <= w.child_cap;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cnt[1] = fits ? total : 0;
    LokiPruneLevelStats* st = R.stats + (l - 1);
    st->n_parents = n;
    st->n_children = total;
    if (!fits) atomicOr(J.dev_err, LOKI_DEVERR_CAPACITY);
  }
  if (!fits) return;
  const double* leaves = R.trees[(l - 1) & 1].leaves;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    circ_map_one(D, leaves, n, batch, reinterpret_cast<const LokiBranchInfo*>(w.info),
                 w.offsets, R.exp_off, reinterpret_cast<CircChild*>(R.child_map),
                 R.valid_flags, i);
}

// the per-batch "holds Taylor children" flags of the current parents
__global__ void bj_circ_clear_kernel(BatchTabs T, int64_t batch) {
  const LokiPruneRun& R = T.jobs[blockIdx.y].run;
  const int64_t nb = R.counts[0] / batch + 1;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nb;
       i += (int64_t)gridDim.x * blockDim.x)
    R.batch_taylor[i] = 0;
}

__global__ void __launch_bounds__(kPruneWarps * 32)
bj_circ_score_kernel(BatchTabs T, int l, LokiScoreSpec sp, ScoreK SK, int64_t batch) {
  extern __shared__ float tiles[];
  const LokiPruneJob& J = T.jobs[blockIdx.y];
  const size_t li = (size_t)blockIdx.y * T.nlevels + (l - 1);
  const LokiPruneLevel& D = T.levels[li];
  const LokiPruneRun& R = J.run;
  const LokiPruneWork& w = R.work;
  const LokiPruneTree& in = R.trees[(l - 1) & 1];
  const float* seg = J.ffa_fold + (int64_t)T.seg_idx[li] * J.seg_stride;
  const int warp = threadIdx.x >> 5;
  float* tile = tiles + (size_t)warp * 32 * score_stride(D.nbins, sp.wmax);
  int64_t* cnt = R.counts;
  const int64_t n_valid = job_pos(w)[cnt[1]];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cnt[4] = n_valid;
    R.stats[l - 1].n_valid = n_valid;
  }
  for (int64_t t = (int64_t)blockIdx.x * kPruneWarps + warp; t * 32 < n_valid;
       t += (int64_t)gridDim.x * kPruneWarps) {
    circ_score_tile(D, in.leaves, in.folds, batch,
                    reinterpret_cast<const LokiBranchInfo*>(w.info),
                    reinterpret_cast<const CircChild*>(R.child_map), R.valid_ids, n_valid, seg,
                    sp, SK, w.child_scores, w.child_idx, w.child_phase, R.child_class,
                    R.batch_taylor, reinterpret_cast<unsigned*>(w.minmax), tile, t * 32);
    __syncwarp();
  }
}

// valid-child offsets at the parents (the overflow rule reads those at
// batch boundaries)
__global__ void bj_circ_boff_kernel(BatchTabs T) {
  const LokiPruneRun& R = T.jobs[blockIdx.y].run;
  const int64_t n = R.counts[0], n_valid = R.counts[4];
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p <= n;
       p += (int64_t)gridDim.x * blockDim.x)
    R.batch_offsets[p] = lower_bound64(R.valid_ids, n_valid, R.work.offsets[p] + R.exp_off[p]);
}

__global__ void __launch_bounds__(kPruneWarps * 32)
bj_circ_emit_kernel(BatchTabs T, int l, int64_t batch) {
  const LokiPruneJob& J = T.jobs[blockIdx.y];
  const size_t li = (size_t)blockIdx.y * T.nlevels + (l - 1);
  const LokiPruneLevel& D = T.levels[li];
  const LokiPruneRun& R = J.run;
  const LokiPruneWork& w = R.work;
  const LokiPruneTree& in = R.trees[(l - 1) & 1];
  const LokiPruneTree& out = R.trees[l & 1];
  const float* seg = J.ffa_fold + (int64_t)T.seg_idx[li] * J.seg_stride;
  const int warp = threadIdx.x >> 5;
  const int64_t n_surv = R.counts[2];
  for (int64_t t = (int64_t)blockIdx.x * kPruneWarps + warp; t * 32 < n_surv;
       t += (int64_t)gridDim.x * kPruneWarps)
    circ_emit_tile(D, in.leaves, in.folds, batch,
                   reinterpret_cast<const LokiBranchInfo*>(w.info),
                   reinterpret_cast<const CircChild*>(R.child_map), R.valid_ids, seg, w.surv,
                   n_surv, w.child_scores, w.child_idx, w.child_phase, R.child_class,
                   R.batch_taylor, out.leaves, out.folds, out.scores, out.scores_ep,
                   out.backtracks, t * 32);
}

// the circular tree over complex folds: lane per valid child / survivor
__global__ void __launch_bounds__(kPruneWarps * 32)
bj_circ_score_complex_kernel(BatchTabs T, int l, LokiScoreSpec sp, int64_t batch) {
  extern __shared__ float smem[];
  const LokiPruneJob& J = T.jobs[blockIdx.y];
  const size_t li = (size_t)blockIdx.y * T.nlevels + (l - 1);
  const LokiPruneLevel& D = T.levels[li];
  const LokiPruneRun& R = J.run;
  const LokiPruneWork& w = R.work;
  const LokiPruneTree& in = R.trees[(l - 1) & 1];
  const float2* seg =
      reinterpret_cast<const float2*>(J.ffa_fold) + (int64_t)T.seg_idx[li] * J.seg_stride;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nb = D.nbins, nbf = nb / 2 + 1;
  const int stride = score_stride(nb, sp.wmax);
  float* tw = smem;
  load_twiddles(tw, nb);
  __syncthreads();
  float* wbase = smem + 2 * nb + (size_t)warp * cplx_warp_floats(nb, stride);
  float2* comb = reinterpret_cast<float2*>(wbase) + (size_t)lane * 2 * nbf;
  float* trow = wbase + (size_t)32 * 2 * nbf * 2 + lane * stride;
  int64_t* cnt = R.counts;
  const int64_t n_valid = job_pos(w)[cnt[1]];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cnt[4] = n_valid;
    R.stats[l - 1].n_valid = n_valid;
  }
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n_valid;
       v += (int64_t)gridDim.x * blockDim.x)
    circ_score_one_complex(D, in.leaves, reinterpret_cast<const float2*>(in.folds), batch,
                           reinterpret_cast<const LokiBranchInfo*>(w.info),
                           reinterpret_cast<const CircChild*>(R.child_map), R.valid_ids, seg, sp,
                           tw, comb, trow, w.child_scores, w.child_idx, w.child_phase,
                           R.child_class, R.batch_taylor, reinterpret_cast<unsigned*>(w.minmax),
                           v);
}

__global__ void __launch_bounds__(kPruneWarps * 32)
bj_circ_emit_complex_kernel(BatchTabs T, int l, int64_t batch) {
  const LokiPruneJob& J = T.jobs[blockIdx.y];
  const size_t li = (size_t)blockIdx.y * T.nlevels + (l - 1);
  const LokiPruneLevel& D = T.levels[li];
  const LokiPruneRun& R = J.run;
  const LokiPruneWork& w = R.work;
  const LokiPruneTree& in = R.trees[(l - 1) & 1];
  const LokiPruneTree& out = R.trees[l & 1];
  const float2* seg =
      reinterpret_cast<const float2*>(J.ffa_fold) + (int64_t)T.seg_idx[li] * J.seg_stride;
  const int64_t n_surv = R.counts[2];
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n_surv;
       s += (int64_t)gridDim.x * blockDim.x)
    circ_emit_one_complex(D, in.leaves, reinterpret_cast<const float2*>(in.folds), batch,
                          reinterpret_cast<const LokiBranchInfo*>(w.info),
                          reinterpret_cast<const CircChild*>(R.child_map), R.valid_ids, seg,
                          w.surv, w.child_scores, w.child_idx, w.child_phase, R.child_class,
                          R.batch_taylor, out.leaves, reinterpret_cast<float2*>(out.folds),
                          out.scores, out.scores_ep, out.backtracks, s);
}

__global__ void bj_bt_kernel(BatchTabs T, int l, int row) {
  const LokiPruneJob& J = T.jobs[blockIdx.y];
  const LokiPruneRun& R = J.run;
  if (!R.bt_hist) return;
  const int64_t start = R.counts[3], rows = R.counts[2];
  if (start + rows > R.bt_rows) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(J.dev_err, LOKI_DEVERR_CAPACITY);
    return;
  }
  const int32_t* bt = R.trees[l & 1].backtracks;
  int32_t* h = R.bt_hist + start * row;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < rows * row;
       i += (int64_t)gridDim.x * blockDim.x)
    h[i] = bt[i];
}

// one block per job: the best leaf of the new tree, then the level's end
__global__ void __launch_bounds__(1024) bj_best_kernel(BatchTabs T, int l, int row_leaf) {
  const LokiPruneJob& J = T.jobs[blockIdx.x];
  const LokiPruneRun& R = J.run;
  int64_t* cnt = R.counts;
  const int64_t n = cnt[2];
  if (R.best_leaves && R.best_scores)
    block_best(R.trees[l & 1].scores, n, R.trees[l & 1].leaves, row_leaf,
               R.best_leaves + (int64_t)(l - 1) * row_leaf, R.best_scores + (l - 1));
  __syncthreads();  // every thread has read the count
  if (threadIdx.x == 0)
    level_end(cnt, reinterpret_cast<unsigned*>(R.work.minmax), R.ovf_flag, R.stats + (l - 1));
}

}  // namespace loki

// Host checks of a batch and the copy of its tables into dev_scratch; fills
// the grid sizes of the enqueue.
struct BatchShape {
  int nbins, poly_order;
  int64_t max_par, max_child;
  int fourier;  // complex (Fourier-domain) folds
  int circ;     // circular-orbit tree (real folds, poly_order 5)
};

static int batch_tables(const LokiPruneJob* jobs, int32_t njobs, const LokiPruneLevel* levels,
                        const int32_t* seg_idx, const double* thresholds, int32_t nlevels,
                        const LokiScoreSpec* spec, int64_t max_sugg, int64_t batch_size,
                        void* dev_scratch, int64_t dev_scratch_bytes, cudaStream_t s,
                        BatchShape* shape, int fourier = 0) {
  if (!jobs || njobs < 1 || njobs > 65535 || !levels || !seg_idx || !thresholds ||
      nlevels < 1 || !spec || !dev_scratch)
    return set_error(LOKI_ERR_INVALID, "null pointer, no job (or above 65535) or no level");
  if (max_sugg < 1 || batch_size < 1) return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (dev_scratch_bytes < loki_prune_run_blocks_scratch_bytes(njobs, nlevels))
    return set_error(LOKI_ERR_CAPACITY, "job scratch below %lld bytes",
                     (long long)loki_prune_run_blocks_scratch_bytes(njobs, nlevels));
  const int nb = levels[0].nbins, P = levels[0].poly_order;
  int64_t max_par = 0, max_child = 0;
  for (int64_t k = 0; k < (int64_t)njobs * nlevels; ++k) {
    int rc = check_prune(&levels[k]);
    if (rc) return rc;
    if (levels[k].basis != levels[0].basis || levels[k].poly_order != P ||
        levels[k].nbins != nb)
      return set_error(LOKI_ERR_INVALID, "levels of different trees");
  }
  const bool circ = levels[0].basis == 2;
  if (circ && P != 5)
    return set_error(LOKI_ERR_UNSUPPORTED, "the circular-orbit tree has poly_order 5");
  for (int j = 0; j < njobs; ++j) {
    const LokiPruneJob& J = jobs[j];
    const LokiPruneRun& R = J.run;
    const LokiPruneWork& w = R.work;
    if (!J.ffa_fold || J.seg_stride < 1 || !J.dev_err || J.seed_n < 0 || J.seed_n > max_sugg)
      return set_error(LOKI_ERR_INVALID, "job %d: bad fold, error word or seed", j);
    if (circ && (!R.exp_off || !R.child_map || !R.valid_flags || !R.valid_ids ||
                 !R.child_class || !R.batch_taylor || !R.batch_offsets))
      return set_error(LOKI_ERR_INVALID, "job %d: no circular-orbit workspace", j);
    if (R.trees[0].cap < max_sugg || R.trees[1].cap < max_sugg || w.par_cap < max_sugg ||
        w.child_cap < 1 || w.ovf_cap < max_sugg + w.child_cap + 1)
      return set_error(LOKI_ERR_CAPACITY, "job %d: workspace below max_sugg / child_cap", j);
    if (!R.counts || !R.ovf_flag || !R.stats || !w.info || !w.offsets || !w.scan ||
        !w.child_scores || !w.child_idx || !w.child_phase || !w.surv || !w.sscan || !w.minmax ||
        !w.ovf_ids || !w.ovf_keys || !w.ovf_thr)
      return set_error(LOKI_ERR_INVALID, "job %d: null workspace pointer", j);
    if (w.scan_bytes < loki_scan_scratch_bytes(w.par_cap + 1) ||
        w.sscan_bytes <
            loki_scan_scratch_bytes(w.child_cap) + (w.child_cap + 1) * (int64_t)sizeof(int64_t))
      return set_error(LOKI_ERR_CAPACITY, "job %d: scan scratch below par_cap / child_cap", j);
    for (int t = 0; t < 2; ++t)
      if (!R.trees[t].leaves || !R.trees[t].folds || !R.trees[t].scores ||
          !R.trees[t].scores_ep || !R.trees[t].backtracks)
        return set_error(LOKI_ERR_INVALID, "job %d: null tree pointer", j);
    max_par = std::max(max_par, w.par_cap);
    max_child = std::max(max_child, w.child_cap);
  }
  int rc = prune_spec_check(spec, nb);
  if (rc) return rc;
  const int64_t nl = (int64_t)njobs * nlevels;
  char* base = reinterpret_cast<char*>(dev_scratch);
  const int64_t o_lv = ((int64_t)njobs * sizeof(LokiPruneJob) + 255) / 256 * 256;
  const int64_t o_si = o_lv + (nl * (int64_t)sizeof(LokiPruneLevel) + 255) / 256 * 256;
  const int64_t o_th = o_si + (nl * 4 + 255) / 256 * 256;
  if (cudaMemcpyAsync(base, jobs, njobs * sizeof(LokiPruneJob), cudaMemcpyHostToDevice, s) !=
          cudaSuccess ||
      cudaMemcpyAsync(base + o_lv, levels, nl * sizeof(LokiPruneLevel), cudaMemcpyHostToDevice,
                      s) != cudaSuccess ||
      cudaMemcpyAsync(base + o_si, seg_idx, nl * 4, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(base + o_th, thresholds, nl * 8, cudaMemcpyHostToDevice, s) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "copy of the job tables failed");
  shape->nbins = nb;
  shape->poly_order = P;
  shape->max_par = max_par;
  shape->max_child = max_child;
  shape->fourier = fourier ? 1 : 0;
  shape->circ = circ ? 1 : 0;
  return LOKI_OK;
}

// The kernels of a batch over tables already in dev_scratch (no host
// access to them: the enqueue can be captured in a CUDA graph and replayed
// after new tables of the same shape are copied in).
static int batch_enqueue(void* dev_scratch, int32_t njobs, int32_t nlevels,
                         const LokiScoreSpec* spec, int64_t max_sugg, int64_t batch_size,
                         const BatchShape& shape, cudaStream_t s,
                         cudaEvent_t* ev_score = nullptr) {
  const int nb = shape.nbins, P = shape.poly_order;
  const bool cplx = shape.fourier != 0;
  LokiScoreSpec sp = *spec;
  sp.mode = 1;
  const ScoreK SK = make_score_k(sp, nb);
  const int smem =
      cplx ? (int)((2 * nb + kPruneWarps * cplx_warp_floats(nb, score_stride(nb, sp.wmax))) *
                   sizeof(float))
           : score_smem_bytes(nb, sp.wmax, kPruneWarps);
  if (smem > 200 * 1024)
    return set_error(LOKI_ERR_UNSUPPORTED, "nbins + wmax too large for pruning");
  if (smem > 48 * 1024 &&
      (cplx ? (shape.circ ? set_smem_limit(bj_circ_score_complex_kernel, smem)
                          : set_smem_limit(bj_score_complex_kernel, smem))
            : shape.circ ? set_smem_limit(bj_circ_score_kernel, smem)
                         : set_smem_limit(bj_score_kernel, smem)) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "device query failed");
  const int64_t nl = (int64_t)njobs * nlevels;
  char* base = reinterpret_cast<char*>(dev_scratch);
  const int64_t o_lv = ((int64_t)njobs * sizeof(LokiPruneJob) + 255) / 256 * 256;
  const int64_t o_si = o_lv + (nl * (int64_t)sizeof(LokiPruneLevel) + 255) / 256 * 256;
  const int64_t o_th = o_si + (nl * 4 + 255) / 256 * 256;
  BatchTabs T;
  T.jobs = reinterpret_cast<const LokiPruneJob*>(base);
  T.levels = reinterpret_cast<const LokiPruneLevel*>(base + o_lv);
  T.seg_idx = reinterpret_cast<const int32_t*>(base + o_si);
  T.thr = reinterpret_cast<const double*>(base + o_th);
  T.nlevels = nlevels;
  // Per-job grids. The jobs' sizes differ from level to level, so every job
  // gets enough blocks for several times an even share of the GPU: blocks
  // past a job's work retire at once, and the block scheduler spreads the
  // busy jobs' blocks over the whole GPU.
  auto per_job = [&](int64_t waves_blocks, int64_t cap_blocks) {
    return (unsigned)std::max<int64_t>(
        1, std::min<int64_t>(cap_blocks, (waves_blocks + njobs - 1) / njobs));
  };
  const int64_t max_par = shape.max_par, max_child = shape.max_child;
  const int64_t spread = std::min<int64_t>(njobs, 16);
  const unsigned g_par = per_job(8 * nsm * spread, (max_par + 255) / 256);
  const unsigned g_scan_p = per_job(2 * nsm, (max_par + 1 + kScanBlock - 1) / kScanBlock);
  const unsigned g_scan_c = per_job(2 * nsm, (max_child + kScanBlock - 1) / kScanBlock);
  const unsigned g_score =
      per_job(6 * nsm * spread, (max_child + kPruneWarps * 32 - 1) / (kPruneWarps * 32));
  const unsigned g_flat = per_job(8 * nsm, (max_child + 255) / 256);
  const unsigned g_emit =
      per_job(6 * nsm * spread, (max_par + kPruneWarps * 32 - 1) / (kPruneWarps * 32));
  const int row_bt = P + 2, row_leaf = (P + 2) * 2;
  int l_cur = 1;
  auto scan = [&](int mode, unsigned g) {
    if (mode == 0 || mode == 2) {
      bj_scan_block_kernel<false><<<dim3(g, njobs), kScanBlock, 0, s>>>(T, l_cur, mode);
      bj_scan_sums_kernel<false><<<dim3(1, njobs), kScanBlock, 0, s>>>(T, l_cur, mode);
      bj_scan_add_kernel<false><<<dim3(g, njobs), kScanBlock, 0, s>>>(T, l_cur, mode);
    } else {
      bj_scan_block_kernel<true><<<dim3(g, njobs), kScanBlock, 0, s>>>(T, l_cur, mode);
      bj_scan_sums_kernel<true><<<dim3(1, njobs), kScanBlock, 0, s>>>(T, l_cur, mode);
      bj_scan_add_kernel<true><<<dim3(g, njobs), kScanBlock, 0, s>>>(T, l_cur, mode);
    }
  };
  note_launch();
  bj_seed_kernel<<<(unsigned)njobs, 1, 0, s>>>(T);
  for (int l = 1; l <= nlevels; ++l) {
    l_cur = l;
    if (shape.circ) {
      // circ_level_dev's steps for every job at once
      for (int i = 0; i < 21; ++i) note_launch();
      bj_circ_branch_kernel<<<dim3(g_par, njobs), 256, 0, s>>>(T, l);
      scan(0, g_scan_p);
      scan(2, g_scan_p);
      bj_circ_map_kernel<<<dim3(g_par, njobs), 256, 0, s>>>(T, l, batch_size);
      scan(3, g_scan_c);
      bj_scatter_kernel<<<dim3(g_flat, njobs), 256, 0, s>>>(T, l, 3);
      bj_circ_clear_kernel<<<dim3(g_par, njobs), 256, 0, s>>>(T, batch_size);
      if (ev_score) cudaEventRecord(ev_score[2 * (l - 1)], s);
      if (cplx)
        bj_circ_score_complex_kernel<<<dim3(g_score, njobs), kPruneWarps * 32, smem, s>>>(
            T, l, sp, batch_size);
      else
        bj_circ_score_kernel<<<dim3(g_score, njobs), kPruneWarps * 32, smem, s>>>(T, l, sp, SK,
                                                                                 batch_size);
      if (ev_score) cudaEventRecord(ev_score[2 * (l - 1) + 1], s);
      bj_circ_boff_kernel<<<dim3(g_par, njobs), 256, 0, s>>>(T);
      scan(4, g_scan_c);
      bj_scatter_kernel<<<dim3(g_flat, njobs), 256, 0, s>>>(T, l, 4);
      bj_overflow_kernel<<<(unsigned)njobs, kSelThreads, 0, s>>>(T, l, max_sugg, batch_size,
                                                                 1);
      if (cplx)
        bj_circ_emit_complex_kernel<<<dim3(g_emit, njobs), kPruneWarps * 32, 0, s>>>(
            T, l, batch_size);
      else
        bj_circ_emit_kernel<<<dim3(g_emit, njobs), kPruneWarps * 32, 0, s>>>(T, l, batch_size);
    } else {
      for (int i = 0; i < 11; ++i) note_launch();
      bj_branch_kernel<<<dim3(g_par, njobs), 256, 0, s>>>(T, l);
      scan(0, g_scan_p);
      if (ev_score) cudaEventRecord(ev_score[2 * (l - 1)], s);
      if (cplx)
        bj_score_complex_kernel<<<dim3(g_score, njobs), kPruneWarps * 32, smem, s>>>(T, l, sp);
      else
        bj_score_kernel<<<dim3(g_score, njobs), kPruneWarps * 32, smem, s>>>(T, l, sp, SK);
      if (ev_score) cudaEventRecord(ev_score[2 * (l - 1) + 1], s);
      scan(1, g_scan_c);
      bj_scatter_kernel<<<dim3(g_flat, njobs), 256, 0, s>>>(T, l, 1);
      bj_overflow_kernel<<<(unsigned)njobs, kSelThreads, 0, s>>>(T, l, max_sugg, batch_size,
                                                                 0);
      if (cplx)
        bj_emit_complex_kernel<<<dim3(g_emit, njobs), kPruneWarps * 32, 0, s>>>(T, l);
      else
        bj_emit_kernel<<<dim3(g_emit, njobs), kPruneWarps * 32, 0, s>>>(T, l);
    }
    note_launch();
    note_launch();
    bj_bt_kernel<<<dim3(g_flat, njobs), 256, 0, s>>>(T, l, row_bt);
    bj_best_kernel<<<(unsigned)njobs, 1024, 0, s>>>(T, l, row_leaf);
    int rc = check_launch("prune_run_batch");
    if (rc) return rc;
  }
  return LOKI_OK;
}

extern "C" int loki_prune_run_batch(const LokiPruneJob* jobs, int32_t njobs,
                                    const LokiPruneLevel* levels, const int32_t* seg_idx,
                                    const double* thresholds, int32_t nlevels,
                                    const LokiScoreSpec* spec, int64_t max_sugg,
                                    int64_t batch_size, void* dev_scratch,
                                    int64_t dev_scratch_bytes, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  BatchShape shape;
  int rc = batch_tables(jobs, njobs, levels, seg_idx, thresholds, nlevels, spec, max_sugg,
                        batch_size, dev_scratch, dev_scratch_bytes, s, &shape);
  if (rc) return rc;
  return batch_enqueue(dev_scratch, njobs, nlevels, spec, max_sugg, batch_size, shape, s);
}

extern "C" int loki_prune_batch_tables(const LokiPruneJob* jobs, int32_t njobs,
                                       const LokiPruneLevel* levels, const int32_t* seg_idx,
                                       const double* thresholds, int32_t nlevels,
                                       const LokiScoreSpec* spec, int64_t max_sugg,
                                       int64_t batch_size, int32_t fourier, void* dev_scratch,
                                       int64_t dev_scratch_bytes, int64_t* shape_out,
                                       void* stream) {
  if (!shape_out) return set_error(LOKI_ERR_INVALID, "null shape pointer");
  BatchShape shape;
  int rc = batch_tables(jobs, njobs, levels, seg_idx, thresholds, nlevels, spec, max_sugg,
                        batch_size, dev_scratch, dev_scratch_bytes, (cudaStream_t)stream,
                        &shape, fourier);
  if (rc) return rc;
  shape_out[0] = shape.nbins;
  shape_out[1] = shape.poly_order;
  shape_out[2] = shape.max_par;
  shape_out[3] = shape.max_child;
  shape_out[4] = shape.fourier;
  shape_out[5] = shape.circ;
  return LOKI_OK;
}

extern "C" int loki_prune_batch_score_times(void* dev_scratch, int32_t njobs, int32_t nlevels,
                                            const LokiScoreSpec* spec, int64_t max_sugg,
                                            int64_t batch_size, const int64_t* shape_in,
                                            float* score_ms, void* stream) {
  if (!dev_scratch || !spec || !shape_in || !score_ms || njobs < 1 || njobs > 65535 ||
      nlevels < 1 || max_sugg < 1 || batch_size < 1)
    return set_error(LOKI_ERR_INVALID, "bad batch timing arguments");
  BatchShape shape;
  shape.nbins = (int)shape_in[0];
  shape.poly_order = (int)shape_in[1];
  shape.max_par = shape_in[2];
  shape.max_child = shape_in[3];
  shape.fourier = shape_in[4] != 0;
  shape.circ = shape_in[5] != 0;
  if (shape.nbins < 1 || shape.poly_order < 1 || shape.poly_order > LOKI_MAX_PARAMS ||
      shape.max_par < 1 || shape.max_child < 1 ||
      (shape.circ && shape.poly_order != 5))
    return set_error(LOKI_ERR_INVALID, "bad batch shape");
  int rc = prune_spec_check(spec, shape.nbins);
  if (rc) return rc;
  std::vector<cudaEvent_t> ev(2 * (size_t)nlevels, nullptr);
  for (auto& e : ev)
    if (cudaEventCreate(&e) != cudaSuccess) {
      for (auto& f : ev)
        if (f) cudaEventDestroy(f);
      return set_error(LOKI_ERR_CUDA, "cudaEventCreate failed");
    }
  cudaStream_t s = (cudaStream_t)stream;
  rc = batch_enqueue(dev_scratch, njobs, nlevels, spec, max_sugg, batch_size, shape, s,
                     ev.data());
  if (!rc && cudaStreamSynchronize(s) != cudaSuccess)
    rc = set_error(LOKI_ERR_CUDA, "cudaStreamSynchronize failed");
  for (int l = 0; l < nlevels && !rc; ++l)
    if (cudaEventElapsedTime(&score_ms[l], ev[2 * l], ev[2 * l + 1]) != cudaSuccess)
      rc = set_error(LOKI_ERR_CUDA, "cudaEventElapsedTime failed");
  for (auto& e : ev) cudaEventDestroy(e);
  return rc;
}

extern "C" int loki_prune_batch_enqueue(void* dev_scratch, int32_t njobs, int32_t nlevels,
                                        const LokiScoreSpec* spec, int64_t max_sugg,
                                        int64_t batch_size, const int64_t* shape_in,
                                        void* stream) {
  if (!dev_scratch || !spec || !shape_in || njobs < 1 || njobs > 65535 || nlevels < 1 ||
      max_sugg < 1 || batch_size < 1)
    return set_error(LOKI_ERR_INVALID, "bad batch enqueue arguments");
  BatchShape shape;
  shape.nbins = (int)shape_in[0];
  shape.poly_order = (int)shape_in[1];
  shape.max_par = shape_in[2];
  shape.max_child = shape_in[3];
  shape.fourier = shape_in[4] != 0;
  shape.circ = shape_in[5] != 0;
  if (shape.nbins < 1 || shape.poly_order < 1 || shape.poly_order > LOKI_MAX_PARAMS ||
      shape.max_par < 1 || shape.max_child < 1 ||
      (shape.circ && shape.poly_order != 5))
    return set_error(LOKI_ERR_INVALID, "bad batch shape");
  int rc = prune_spec_check(spec, shape.nbins);
  if (rc) return rc;
  return batch_enqueue(dev_scratch, njobs, nlevels, spec, max_sugg, batch_size, shape,
                       (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// batched ascend and read-back of many jobs' final trees
// ---------------------------------------------------------------------------

namespace loki {

__global__ void __launch_bounds__(kPruneWarps * 32)
prune_ascend_batch_kernel(const LokiAscendJob* __restrict__ jobs, int nseg, LokiScoreSpec sp,
                          ScoreK SK) {
  extern __shared__ float tiles[];
  const LokiAscendJob& J = jobs[blockIdx.y];
  const LokiPruneLevel& D = J.lvl;
  const int warp = threadIdx.x >> 5;
  const int stride = score_stride(D.nbins, sp.wmax);
  float* acc = tiles + (size_t)warp * 32 * (2 * D.nbins + stride);
  float* tile = acc + 32 * 2 * D.nbins;
  const int64_t n = *J.n_dev;
  for (int64_t t = (int64_t)blockIdx.x * kPruneWarps + warp; t * 32 < n;
       t += (int64_t)gridDim.x * kPruneWarps) {
    ascend_tile(D, J.leaves, J.folds, J.scores, J.scores_ep, n, nseg, J.tm_seg, J.dt_seg,
                J.seg_idx, J.ffa_fold, J.seg_stride, sp, SK, acc, tile, t * 32);
    __syncwarp();  // the accumulators are reused by the next tile
  }
}

// The same over complex trees (folds and segment strides in float2 units).
__global__ void __launch_bounds__(kPruneWarps * 32)
prune_ascend_batch_complex_kernel(const LokiAscendJob* __restrict__ jobs, int nseg,
                                  LokiScoreSpec sp) {
  extern __shared__ float smem[];
  const LokiAscendJob& J = jobs[blockIdx.y];
  const LokiPruneLevel& D = J.lvl;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nb = D.nbins, nbf = nb / 2 + 1;
  const int stride = score_stride(nb, sp.wmax);
  float* tw = smem;
  load_twiddles(tw, nb);
  __syncthreads();
  float* wbase = smem + 2 * nb + (size_t)warp * cplx_warp_floats(nb, stride);
  float2* comb = reinterpret_cast<float2*>(wbase) + (size_t)lane * 2 * nbf;
  float* trow = wbase + (size_t)32 * 2 * nbf * 2 + lane * stride;
  const int64_t n = *J.n_dev;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x)
    ascend_one_complex(D, J.leaves, reinterpret_cast<float2*>(J.folds), J.scores, J.scores_ep,
                       nseg, J.tm_seg, J.dt_seg, J.seg_idx,
                       reinterpret_cast<const float2*>(J.ffa_fold), J.seg_stride, sp, tw, comb,
                       trow, r);
}

// Block y copies part y: src[y][0 .. bytes[y]) to dst + off[y] (16-byte
// words where both ends allow, else bytes).
__global__ void gather_parts_kernel(const LokiGatherPart* __restrict__ parts,
                                    char* __restrict__ dst) {
  const LokiGatherPart& P = parts[blockIdx.y];
  const char* src = reinterpret_cast<const char*>(P.src);
  char* d = dst + P.dst_off;
  const int64_t nb = P.bytes;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(d)) & 15) == 0) {
    const int64_t n16 = nb >> 4;
    for (int64_t i = i0; i < n16; i += step)
      reinterpret_cast<uint4*>(d)[i] = reinterpret_cast<const uint4*>(src)[i];
    for (int64_t i = (n16 << 4) + i0; i < nb; i += step) d[i] = src[i];
  } else {
    for (int64_t i = i0; i < nb; i += step) d[i] = src[i];
  }
}

}  // namespace loki

extern "C" int loki_prune_ascend_batch(const LokiAscendJob* jobs, int32_t njobs, int32_t nseg,
                                       const LokiScoreSpec* spec, int64_t n_cap,
                                       int32_t fourier, void* dev_scratch,
                                       int64_t dev_scratch_bytes, void* stream) {
  if (!jobs || njobs < 1 || njobs > 65535 || nseg < 1 || !spec || n_cap < 1 || !dev_scratch)
    return set_error(LOKI_ERR_INVALID, "bad batched ascend arguments");
  if (dev_scratch_bytes < (int64_t)njobs * (int64_t)sizeof(LokiAscendJob))
    return set_error(LOKI_ERR_CAPACITY, "ascend job scratch below %lld bytes",
                     (long long)njobs * (long long)sizeof(LokiAscendJob));
  const int nb = jobs[0].lvl.nbins;
  for (int j = 0; j < njobs; ++j) {
    const LokiAscendJob& J = jobs[j];
    int rc = check_prune(&J.lvl);
    if (rc) return rc;
    if (J.lvl.nbins != nb || J.lvl.basis != jobs[0].lvl.basis)
      return set_error(LOKI_ERR_INVALID, "ascend jobs of different trees");
    if (!J.n_dev || !J.leaves || !J.folds || !J.scores || !J.scores_ep || !J.tm_seg ||
        !J.dt_seg || !J.seg_idx || !J.ffa_fold || J.seg_stride < 1 || !J.dev_err)
      return set_error(LOKI_ERR_INVALID, "ascend job %d: null pointer or bad stride", j);
  }
  int rc = prune_spec_check(spec, nb);
  if (rc) return rc;
  LokiScoreSpec sp = *spec;
  sp.mode = 1;
  const ScoreK SK = make_score_k(sp, nb);
  const int stride = score_stride(nb, sp.wmax);
  const int smem =
      fourier ? (int)((2 * nb + kPruneWarps * cplx_warp_floats(nb, stride)) * sizeof(float))
              : kPruneWarps * 32 * (2 * nb + stride) * (int)sizeof(float);
  if (smem > 200 * 1024) return set_error(LOKI_ERR_UNSUPPORTED, "nbins too large for ascend");
  if (smem > 48 * 1024 && (fourier ? set_smem_limit(prune_ascend_batch_complex_kernel, smem)
                                   : set_smem_limit(prune_ascend_batch_kernel, smem)) !=
                              cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  int dev = 0, nsm = 0, occ = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      (fourier ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                     &occ, prune_ascend_batch_complex_kernel, kPruneWarps * 32, smem)
               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, prune_ascend_batch_kernel,
                                                               kPruneWarps * 32, smem)) !=
          cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "occupancy query failed");
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(dev_scratch, jobs, njobs * sizeof(LokiAscendJob), cudaMemcpyHostToDevice,
                      s) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "copy of the ascend jobs failed");
  const int64_t need = (n_cap + kPruneWarps * 32 - 1) / (kPruneWarps * 32);
  const int64_t wave = ((int64_t)nsm * std::max(1, occ) + njobs - 1) / njobs;
  const unsigned bx = (unsigned)std::max<int64_t>(1, std::min<int64_t>(need, wave));
  note_launch();
  if (fourier)
    prune_ascend_batch_complex_kernel<<<dim3(bx, njobs), kPruneWarps * 32, smem, s>>>(
        reinterpret_cast<const LokiAscendJob*>(dev_scratch), nseg, sp);
  else
    prune_ascend_batch_kernel<<<dim3(bx, njobs), kPruneWarps * 32, smem, s>>>(
        reinterpret_cast<const LokiAscendJob*>(dev_scratch), nseg, sp, SK);
  return check_launch("prune_ascend_batch");
}

extern "C" int loki_gather_parts(const LokiGatherPart* parts, int32_t nparts, void* dst,
                                 int64_t dst_bytes, void* dev_scratch,
                                 int64_t dev_scratch_bytes, void* stream) {
  if (!parts || nparts < 1 || nparts > 65535 || !dst || !dev_scratch)
    return set_error(LOKI_ERR_INVALID, "bad gather arguments");
  if (dev_scratch_bytes < (int64_t)nparts * (int64_t)sizeof(LokiGatherPart))
    return set_error(LOKI_ERR_CAPACITY, "gather scratch below %lld bytes",
                     (long long)nparts * (long long)sizeof(LokiGatherPart));
  int64_t maxb = 0;
  for (int i = 0; i < nparts; ++i) {
    if (parts[i].bytes < 0 || parts[i].dst_off < 0 ||
        parts[i].dst_off + parts[i].bytes > dst_bytes || (parts[i].bytes > 0 && !parts[i].src))
      return set_error(LOKI_ERR_INVALID, "gather part %d outside the destination", i);
    maxb = std::max(maxb, parts[i].bytes);
  }
  if (maxb == 0) return LOKI_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(dev_scratch, parts, nparts * sizeof(LokiGatherPart),
                      cudaMemcpyHostToDevice, s) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "copy of the gather parts failed");
  const unsigned bx = (unsigned)std::max<int64_t>(1, std::min<int64_t>(64, (maxb / 16 + 255) / 256));
  note_launch();
  gather_parts_kernel<<<dim3(bx, nparts), 256, 0, s>>>(
      reinterpret_cast<const LokiGatherPart*>(dev_scratch), reinterpret_cast<char*>(dst));
  return check_launch("gather_parts");
}

namespace loki {

// Block y seeds job y: leaves copied, the segment rows copied into the tree
// and scored (normalised e / sqrt(v), boxcar S/N as loki_snr_score_batch),
// scores_ep and the seed record set, backtracks and the error word cleared.
__global__ void __launch_bounds__(kPruneWarps * 32)
prune_seed_batch_kernel(const LokiSeedJob* __restrict__ jobs, int nb, int P, LokiScoreSpec sp,
                        ScoreK SK) {
  extern __shared__ float tiles[];
  const LokiSeedJob& J = jobs[blockIdx.y];
  const int64_t n = J.n;
  const int row_leaf = (P + 2) * 2, row_bt = P + 2;
  const int64_t gtid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t gstep = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = gtid; i < n * row_leaf; i += gstep) J.leaves_out[i] = J.seed_leaves[i];
  for (int64_t i = gtid; i < n * 2 * nb; i += gstep) J.folds_out[i] = J.fold_rows[i];
  for (int64_t i = gtid; i < n * row_bt; i += gstep) J.bt_out[i] = 0;
  if (gtid == 0) *J.dev_err = 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int stride = score_stride(nb, sp.wmax);
  float* tile = tiles + (size_t)warp * 32 * stride;
  for (int64_t p0 = ((int64_t)blockIdx.x * kPruneWarps + warp) * 32; p0 < n;
       p0 += (int64_t)gridDim.x * kPruneWarps * 32) {
    const int kmax = (int)min((int64_t)32, n - p0);
    for (int k = 0; k < kmax; ++k) {
      const float* src = J.fold_rows + (p0 + k) * 2 * nb;
      float* trow = tile + k * stride;
      for (int j = lane; j < nb; j += 32) trow[j] = __fdiv_rn(src[j], __fsqrt_rn(src[nb + j]));
    }
    __syncwarp();
    if (lane < kmax) {
      float s;
      float* row = tile + lane * stride;
      if (SK.pow2_64) score_row64_pow2(row, sp, SK, &s);
      else score_row(row, nb, sp, &s);
      J.scores_out[p0 + lane] = s;
      J.scores_ep_out[p0 + lane] = s;
      J.seed_scores_out[p0 + lane] = s;
    }
    __syncwarp();
  }
}

}  // namespace loki

extern "C" int loki_prune_seed_batch(const LokiSeedJob* jobs, int32_t njobs, int32_t nbins,
                                     int32_t poly_order, const LokiScoreSpec* spec,
                                     void* dev_scratch, int64_t dev_scratch_bytes,
                                     void* stream) {
  if (!jobs || njobs < 1 || njobs > 65535 || !spec || !dev_scratch || nbins < 2 ||
      poly_order < 1 || poly_order > LOKI_MAX_PARAMS)
    return set_error(LOKI_ERR_INVALID, "bad seed batch arguments");
  if (dev_scratch_bytes < (int64_t)njobs * (int64_t)sizeof(LokiSeedJob))
    return set_error(LOKI_ERR_CAPACITY, "seed job scratch below %lld bytes",
                     (long long)njobs * (long long)sizeof(LokiSeedJob));
  int64_t maxn = 0;
  for (int j = 0; j < njobs; ++j) {
    const LokiSeedJob& J = jobs[j];
    if (J.n < 0 || (J.n > 0 && (!J.seed_leaves || !J.fold_rows || !J.leaves_out ||
                                !J.folds_out || !J.scores_out || !J.scores_ep_out ||
                                !J.seed_scores_out || !J.bt_out)) ||
        !J.dev_err)
      return set_error(LOKI_ERR_INVALID, "seed job %d: null pointer or negative size", j);
    maxn = std::max(maxn, J.n);
  }
  int rc = prune_spec_check(spec, nbins);
  if (rc) return rc;
  LokiScoreSpec sp = *spec;
  sp.mode = 1;
  const ScoreK SK = make_score_k(sp, nbins);
  const int smem = score_smem_bytes(nbins, sp.wmax, kPruneWarps);
  if (smem > 200 * 1024) return set_error(LOKI_ERR_UNSUPPORTED, "nbins + wmax too large");
  if (smem > 48 * 1024 && set_smem_limit(prune_seed_batch_kernel, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(dev_scratch, jobs, njobs * sizeof(LokiSeedJob), cudaMemcpyHostToDevice,
                      s) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "copy of the seed jobs failed");
  const unsigned bx =
      (unsigned)std::max<int64_t>(1, std::min<int64_t>(32, (maxn + kPruneWarps * 32 - 1) /
                                                               (kPruneWarps * 32)));
  note_launch();
  prune_seed_batch_kernel<<<dim3(bx, njobs), kPruneWarps * 32, smem, s>>>(
      reinterpret_cast<const LokiSeedJob*>(dev_scratch), nbins, poly_order, sp, SK);
  return check_launch("prune_seed_batch");
}
