// Input conditioning of a time series: the running-median deredden, order
// statistics, the mean and the normalisation that io/timeseries.py:198-236
// (TimeSeries.from_tim) applies through sigpyproc's TimeSeries.deredden and
// TimeSeries.normalise before a search.
//
// Definitions (sigpyproc is not part of the reference tree, so its filters are
// restated here with these semantics):
// - running median over `window` samples: output i is the order statistic of
//   rank window / 2 (the upper median for an even window) of the samples at
//   i - window/2 .. i - window/2 + window - 1, with half-sample symmetric
//   reflection at the ends (scipy.ndimage.median_filter, mode "reflect");
// - k-th order statistic of a float32 array (0-based, ascending);
// - the mean accumulated in float64.
#include <algorithm>

#include "loki_common.cuh"

namespace loki {

constexpr int kMedThreads = 512;
constexpr int kMedMaxWindow = 32768;

// Index of position j in [0, n) after half-sample symmetric reflection
// (period 2n).
__device__ __forceinline__ int64_t reflect_idx(int64_t j, int64_t n) {
  const int64_t p = 2 * n;
  int64_t m = j % p;
  if (m < 0) m += p;
  return m < n ? m : p - 1 - m;
}

// Number of entries of the ascending window s[0..w) below v (lower bound),
// found by warp `lane`s with a 32-way search.
__device__ __forceinline__ int warp_lower_bound(const float* s, int w, float v, int lane) {
  int lo = 0, hi = w;  // answer in [lo, hi]
  while (hi - lo > 32) {
    const int step = (hi - lo + 31) / 32;
    const int idx = lo + (lane + 1) * step - 1;  // last element of lane's slice
    const bool below = idx < hi && s[idx] < v;
    const unsigned m = __ballot_sync(0xFFFFFFFFu, below);
    const int nb = __popc(m);  // slices entirely below v
    lo = lo + nb * step;
    hi = min(hi, lo + step);
  }
  const int idx = lo + lane;
  const bool below = idx < hi && s[idx] < v;
  return lo + __popc(__ballot_sync(0xFFFFFFFFu, below));
}

// Block b computes outputs [b * chunk, min((b + 1) * chunk, n)). The window is
// kept sorted in shared memory: a bitonic sort of the first window, then per
// output one removal and one insertion (two warp searches and a shift).
__global__ void __launch_bounds__(kMedThreads)
running_median_kernel(const float* __restrict__ x, int64_t n, int w, int pw, int64_t chunk,
                      int subtract, float* __restrict__ out) {
  extern __shared__ float s[];  // [pw]
  __shared__ int pos[2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t i0 = (int64_t)blockIdx.x * chunk;
  if (i0 >= n) return;  // uniform over the block
  const int64_t i1 = min(i0 + chunk, n);
  const int half = w / 2;
  for (int k = tid; k < pw; k += kMedThreads)
    s[k] = k < w ? x[reflect_idx(i0 - half + k, n)] : __int_as_float(0x7F800000);
  __syncthreads();
  for (int size = 2; size <= pw; size <<= 1) {  // bitonic sort, ascending
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int k = tid; k < pw / 2; k += kMedThreads) {
        const int a = 2 * k - (k & (stride - 1));
        const int b = a + stride;
        const bool up = (a & size) == 0;
        const float va = s[a], vb = s[b];
        if ((va > vb) == up) {
          s[a] = vb;
          s[b] = va;
        }
      }
      __syncthreads();
    }
  }
  // the samples leaving and entering the window for output i + 1, loaded one
  // output ahead
  float vo = x[reflect_idx(i0 - half, n)];
  float vn = x[reflect_idx(i0 - half + w, n)];
  for (int64_t i = i0;; ++i) {
    if (tid == 0) {
      const float m = s[half];
      out[i] = subtract ? __fsub_rn(x[i], m) : m;
    }
    if (i + 1 >= i1) break;
    const float co = vo, cn = vn;
    if (i + 2 < i1) {
      vo = x[reflect_idx(i + 1 - half, n)];
      vn = x[reflect_idx(i + 1 - half + w, n)];
    }
    if (co == cn) continue;  // the window's sorted content is unchanged
    if (warp < 2) {
      const int r = warp_lower_bound(s, w, warp == 0 ? co : cn, lane);
      if (lane == 0) pos[warp] = r;
    }
    __syncthreads();
    const int p = pos[0], q = pos[1];
    // cn > co: s[p+1 .. q-1] move down one and cn lands at q - 1;
    // cn < co: s[q .. p-1] move up one and cn lands at q
    const int src = cn > co ? p + 1 : q;
    const int dst = cn > co ? p : q + 1;
    const int len = cn > co ? q - 1 - p : p - q;
    constexpr int kPer = kMedMaxWindow / kMedThreads;
    float v[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      if (j * kMedThreads >= len) break;  // uniform over the block
      const int k = tid + j * kMedThreads;
      if (k < len) v[j] = s[src + k];
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      if (j * kMedThreads >= len) break;
      const int k = tid + j * kMedThreads;
      if (k < len) s[dst + k] = v[j];
    }
    if (tid == 0) s[cn > co ? q - 1 : q] = cn;
    __syncthreads();
  }
}

// Order-preserving map of a float to an unsigned key (NaN after +inf).
__device__ __forceinline__ unsigned f2key(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key2f(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// Radix select state: st[0] = key prefix, st[1] = prefix mask, st[2] = rank k
// within the matching keys (int64 in words 2-3).
struct SelState {
  unsigned prefix, mask;
  long long k;
};

__global__ void select_init_kernel(SelState* st, unsigned* hist, int64_t k) {
  st->prefix = 0;
  st->mask = 0;
  st->k = k;
  for (int d = threadIdx.x; d < 256; d += blockDim.x) hist[d] = 0;
}

// Histogram of the digit at `shift` among keys that match the prefix.
__global__ void __launch_bounds__(256)
select_hist_kernel(const float* __restrict__ x, int64_t n, int shift, const SelState* st,
                   unsigned* __restrict__ hist) {
  __shared__ unsigned h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const unsigned prefix = st->prefix, mask = st->mask;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned key = f2key(x[i]);
    if ((key & mask) == prefix) atomicAdd(&h[(key >> shift) & 0xFFu], 1u);
  }
  __syncthreads();
  if (h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], h[threadIdx.x]);
}

// Choose the digit holding rank k, move the prefix on, clear the histogram;
// after the last digit write the value.
__global__ void select_pick_kernel(SelState* st, unsigned* hist, int shift, float* out) {
  if (threadIdx.x != 0) return;
  long long k = st->k;
  int d = 0;
  for (; d < 255; ++d) {
    if (k < (long long)hist[d]) break;
    k -= hist[d];
  }
  st->k = k;
  st->prefix |= (unsigned)d << shift;
  st->mask |= 0xFFu << shift;
  for (int j = 0; j < 256; ++j) hist[j] = 0;
  if (shift == 0) *out = key2f(st->prefix);
}

// sum of x (or of x^2) in float64: per-block partial sums, then one block
// adds them
__global__ void __launch_bounds__(256)
sum_f64_kernel(const float* __restrict__ x, int64_t n, int square, double* __restrict__ part) {
  __shared__ double w[8];
  double a = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = (double)x[i];
    a += square ? v * v : v;
  }
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xFFFFFFFFu, a, o);
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < 8; ++k) t += w[k];
    part[blockIdx.x] = t;
  }
}

__global__ void sum_parts_kernel(const double* __restrict__ part, int nparts,
                                 double* __restrict__ out) {
  __shared__ double w[32];
  double a = 0.0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) a += part[k];
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xFFFFFFFFu, a, o);
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x + 31) / 32; ++k) t += w[k];
    *out = t;
  }
}

// y = (x - loc) / scale, float32 arithmetic, or |x - loc| when scale == 0
__global__ void affine_kernel(const float* __restrict__ x, int64_t n, float loc, float scale,
                              float* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float d = __fsub_rn(x[i], loc);
    y[i] = scale == 0.0f ? fabsf(d) : __fdiv_rn(d, scale);
  }
}

}  // namespace loki

using namespace loki;

extern "C" int loki_running_median(const float* x, int64_t n, int32_t window,
                                   int32_t subtract, float* out, void* stream) {
  if (!x || !out) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (n <= 0) return set_error(LOKI_ERR_INVALID, "n must be > 0");
  if (window < 1) return set_error(LOKI_ERR_INVALID, "window %d must be >= 1", window);
  if (window > kMedMaxWindow)
    return set_error(LOKI_ERR_UNSUPPORTED, "window %d above %d", window, kMedMaxWindow);
  int pw = 1;
  while (pw < window) pw <<= 1;
  pw = std::max(pw, 2);
  const int smem = pw * (int)sizeof(float);
  if (set_smem_limit(running_median_kernel, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "device query failed");
  // one block per SM (registers and the window's shared memory), each output
  // chunk long enough to pay for its sort
  const int64_t blocks = std::max<int64_t>(
      1, std::min<int64_t>((int64_t)nsm, (n + 4 * (int64_t)window - 1) / (4 * window)));
  const int64_t chunk = (n + blocks - 1) / blocks;
  note_launch();
  running_median_kernel<<<(unsigned)blocks, kMedThreads, smem, (cudaStream_t)stream>>>(
      x, n, window, pw, chunk, subtract, out);
  return check_launch("running_median");
}

extern "C" int64_t loki_select_scratch_bytes(void) { return 256 * 4 + 64; }

extern "C" int loki_select_kth(const float* x, int64_t n, int64_t k, float* out,
                               void* scratch, int64_t scratch_bytes, void* stream) {
  if (!x || !out || !scratch) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (n <= 0 || k < 0 || k >= n) return set_error(LOKI_ERR_INVALID, "need 0 <= k < n");
  if (scratch_bytes < loki_select_scratch_bytes())
    return set_error(LOKI_ERR_CAPACITY, "select scratch below %lld bytes",
                     (long long)loki_select_scratch_bytes());
  cudaStream_t s = (cudaStream_t)stream;
  unsigned* hist = reinterpret_cast<unsigned*>(scratch);
  SelState* st = reinterpret_cast<SelState*>(reinterpret_cast<char*>(scratch) + 256 * 4);
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 1024);
  for (int i = 0; i < 9; ++i) note_launch();
  select_init_kernel<<<1, 256, 0, s>>>(st, hist, k);
  for (int shift = 24; shift >= 0; shift -= 8) {
    select_hist_kernel<<<blocks, 256, 0, s>>>(x, n, shift, st, hist);
    select_pick_kernel<<<1, 32, 0, s>>>(st, hist, shift, out);
  }
  return check_launch("select_kth");
}

extern "C" int loki_sum_f64(const float* x, int64_t n, int32_t square, double* out,
                            void* scratch, int64_t scratch_bytes, void* stream) {
  if (!x || !out || !scratch) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (n < 0) return set_error(LOKI_ERR_INVALID, "n must be >= 0");
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 1024));
  if (scratch_bytes < blocks * (int64_t)sizeof(double))
    return set_error(LOKI_ERR_CAPACITY, "sum scratch below %d doubles", blocks);
  cudaStream_t s = (cudaStream_t)stream;
  double* part = reinterpret_cast<double*>(scratch);
  note_launch();
  note_launch();
  sum_f64_kernel<<<blocks, 256, 0, s>>>(x, n, square, part);
  sum_parts_kernel<<<1, 256, 0, s>>>(part, blocks, out);
  return check_launch("sum_f64");
}

extern "C" int loki_affine(const float* x, int64_t n, float loc, float scale, float* y,
                           void* stream) {
  if (!x || !y) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (n <= 0) return LOKI_OK;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
  note_launch();
  affine_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(x, n, loc, scale, y);
  return check_launch("affine");
}
