// Brute fold at the start of the FFA (core/fold.py:108-171 brutefold_start).
//
// The reference computes a phase-bin map per (frequency, sample in segment)
// and then, per segment and frequency, adds every sample into its bin in time
// order. Here the map is built once per frequency chunk (phase_map_kernel, FP64
// with the reference's rounding) and shared by all segments; the fold kernel
// gives each thread one (segment, frequency) and walks the samples in time
// order exactly like the reference loop, so every bin sum is bit-identical.
//
// Per thread the running sums of the current bin stay in registers; all 2 x
// nbins sums live in shared memory laid out [bin][thread] (conflict-free).
// The map row is read 16 bytes at a time and the series 4 samples at a time
// (the 8 threads' series loads of one block are broadcasts of the same
// addresses). Blocks are ordered segment-fastest so that the map rows of the
// frequencies in flight stay in L2 while every segment consumes them.
#include <algorithm>

#include "loki_common.cuh"

namespace loki {

template <typename T>
__global__ void phase_map_kernel(const double* __restrict__ freqs, int64_t nfreq,
                                 int64_t seg_len, int nbins, double tsamp, double t_ref,
                                 T* __restrict__ map) {
  const int64_t total = nfreq * seg_len;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = k / seg_len;
    const int64_t i = k - f * seg_len;
    const double pt = __dsub_rn(__dmul_rn((double)i, tsamp), t_ref);
    int b = round_shift(phase_idx(pt, freqs[f], nbins, 0.0), nbins);
    // Only a non-finite frequency can leave [0, nbins); keep every
    // accumulator index in bounds (the host rejects such grids up front).
    if (b < 0 || b >= nbins) b = 0;
    map[k] = (T)b;
  }
}

template <typename T>
struct MapVec;
template <>
struct MapVec<uint8_t> {
  static constexpr int N = 16;
  __device__ static int get(const uint4& v, int k) {
    const unsigned w = k < 4 ? v.x : k < 8 ? v.y : k < 12 ? v.z : v.w;
    return (w >> (8 * (k & 3))) & 0xFF;
  }
};
template <>
struct MapVec<uint16_t> {
  static constexpr int N = 8;
  __device__ static int get(const uint4& v, int k) {
    const unsigned w = k < 2 ? v.x : k < 4 ? v.y : k < 6 ? v.z : v.w;
    return (w >> (16 * (k & 1))) & 0xFFFF;
  }
};

__device__ __forceinline__ float f4get(const float4& v, int k) {
  return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
}

// kUnit: ts_v is all ones, so only the ts_e sums are taken here (half the
// shared memory per thread); brutefold_count_kernel writes the variance rows.
template <typename T, bool kUnit>
__global__ void __launch_bounds__(128)
brutefold_seq_kernel(const float* __restrict__ ts_e, const float* __restrict__ ts_v,
                     int64_t nsamps, const T* __restrict__ map, int64_t nfreq_chunk,
                     int64_t f_offset, int64_t nfreq_total, int64_t seg_len, int64_t nseg,
                     int nbins, float* __restrict__ fold) {
  extern __shared__ float acc[];  // [NC * nbins][blockDim.x]
  constexpr int NC = kUnit ? 1 : 2;
  const int BS = blockDim.x;
  const int t = threadIdx.x;
  const int64_t seg = blockIdx.x % nseg;
  const int64_t fi = (blockIdx.x / nseg) * BS + t;
  if (fi >= nfreq_chunk) return;  // no block-level synchronisation follows
  for (int b = 0; b < NC * nbins; ++b) acc[b * BS + t] = 0.0f;
  const int64_t start = seg * seg_len;
  const int64_t len = std::min<int64_t>(seg_len, nsamps - start);
  const T* m = map + fi * seg_len;
  const float* e = ts_e + start;
  const float* v = kUnit ? e : ts_v + start;
  int cur = 0;
  float ae = 0.0f, av = 0.0f;
  constexpr int VN = MapVec<T>::N;
  int64_t i = 0;
  const bool aligned = ((reinterpret_cast<uintptr_t>(m) | reinterpret_cast<uintptr_t>(e) |
                         reinterpret_cast<uintptr_t>(v)) & 15) == 0;
  if (aligned && len >= VN) {
    // software pipeline: the map word and series of the next VN samples are
    // loaded while the current VN samples are added
    uint4 mv = *reinterpret_cast<const uint4*>(m);
    float4 ev[VN / 4], vv[VN / 4];
#pragma unroll
    for (int q = 0; q < VN / 4; ++q) {
      ev[q] = __ldg(reinterpret_cast<const float4*>(e) + q);
      if constexpr (!kUnit) vv[q] = __ldg(reinterpret_cast<const float4*>(v) + q);
    }
    for (; i + VN <= len; i += VN) {
      const bool more = i + 2 * VN <= len;
      uint4 mv_n = mv;
      float4 ev_n[VN / 4], vv_n[VN / 4];
#pragma unroll
      for (int q = 0; q < VN / 4; ++q) {
        ev_n[q] = ev[q];
        if constexpr (!kUnit) vv_n[q] = vv[q];
      }
      if (more) {
        mv_n = *reinterpret_cast<const uint4*>(m + i + VN);
#pragma unroll
        for (int q = 0; q < VN / 4; ++q) {
          ev_n[q] = __ldg(reinterpret_cast<const float4*>(e + i + VN) + q);
          if constexpr (!kUnit) vv_n[q] = __ldg(reinterpret_cast<const float4*>(v + i + VN) + q);
        }
      }
#pragma unroll
      for (int k = 0; k < VN; ++k) {
        const int b = MapVec<T>::get(mv, k);
        if (b != cur) {
          acc[cur * BS + t] = ae;
          ae = acc[b * BS + t];
          if constexpr (!kUnit) {
            acc[(nbins + cur) * BS + t] = av;
            av = acc[(nbins + b) * BS + t];
          }
          cur = b;
        }
        ae = __fadd_rn(ae, f4get(ev[k >> 2], k & 3));
        if constexpr (!kUnit) av = __fadd_rn(av, f4get(vv[k >> 2], k & 3));
      }
      mv = mv_n;
#pragma unroll
      for (int q = 0; q < VN / 4; ++q) {
        ev[q] = ev_n[q];
        if constexpr (!kUnit) vv[q] = vv_n[q];
      }
    }
  }
  for (; i < len; ++i) {
    const int b = (int)m[i];
    if (b != cur) {
      acc[cur * BS + t] = ae;
      ae = acc[b * BS + t];
      if constexpr (!kUnit) {
        acc[(nbins + cur) * BS + t] = av;
        av = acc[(nbins + b) * BS + t];
      }
      cur = b;
    }
    ae = __fadd_rn(ae, e[i]);
    if constexpr (!kUnit) av = __fadd_rn(av, v[i]);
  }
  acc[cur * BS + t] = ae;
  if constexpr (!kUnit) acc[(nbins + cur) * BS + t] = av;
  float* out = fold + ((size_t)seg * nfreq_total + f_offset + fi) * 2 * nbins;
  if ((reinterpret_cast<uintptr_t>(out) & 15) == 0 && ((NC * nbins) & 3) == 0) {
    for (int b = 0; b < NC * nbins; b += 4)
      *reinterpret_cast<float4*>(out + b) =
          make_float4(acc[b * BS + t], acc[(b + 1) * BS + t], acc[(b + 2) * BS + t],
                      acc[(b + 3) * BS + t]);
  } else {
    for (int b = 0; b < NC * nbins; ++b) out[b] = acc[b * BS + t];
  }
}

// Variance rows of a unit-variance fold: with ts_v all ones every (segment,
// frequency, bin) sum of the reference is the bin's sample count (exact in
// float32 below 2^24 samples per segment). The map depends only on the sample
// position within a segment, so every full segment has the same counts: one
// histogram per frequency (and one more for a shorter last segment).
template <typename T>
__global__ void __launch_bounds__(256)
brutefold_count_kernel(const T* __restrict__ map, int64_t nfreq_chunk, int64_t f_offset,
                       int64_t nfreq_total, int64_t seg_len, int64_t nsamps, int64_t nseg,
                       int nbins, float* __restrict__ fold) {
  extern __shared__ int hist[];  // [2][nbins]: full segments, last segment
  const int64_t fi = blockIdx.x;
  if (fi >= nfreq_chunk) return;
  const T* m = map + fi * seg_len;
  const int64_t last_len = nsamps - (nseg - 1) * seg_len;
  for (int b = threadIdx.x; b < 2 * nbins; b += blockDim.x) hist[b] = 0;
  __syncthreads();
  for (int64_t i = threadIdx.x; i < seg_len; i += blockDim.x) {
    const int b = (int)m[i];
    atomicAdd(&hist[b], 1);
    if (i < last_len) atomicAdd(&hist[nbins + b], 1);
  }
  __syncthreads();
  for (int64_t k = threadIdx.x; k < nseg * nbins; k += blockDim.x) {
    const int64_t seg = k / nbins;
    const int b = (int)(k - seg * nbins);
    const int c = seg == nseg - 1 ? hist[nbins + b] : hist[b];
    fold[((size_t)seg * nfreq_total + f_offset + fi) * 2 * nbins + nbins + b] = (float)c;
  }
}


}  // namespace loki

using namespace loki;

namespace loki {

// unit: ts_v is all ones (ts_v may be NULL); the ts_e sums come from the
// sequential kernel and the variance rows from the per-frequency counts.
static int brutefold_impl(const float* ts_e, const float* ts_v, bool unit, int64_t nsamps,
                          const double* freqs, int64_t nfreqs, int64_t segment_len,
                          int32_t nbins, double tsamp, double t_ref, void* phase_scratch,
                          int64_t scratch_bytes, float* fold_out, void* stream) {
  if (!ts_e || (!ts_v && !unit) || !freqs || !phase_scratch || !fold_out)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (nsamps <= 0 || nfreqs <= 0 || segment_len <= 0)
    return set_error(LOKI_ERR_INVALID, "nsamps, nfreqs and segment_len must be > 0");
  if (nbins < 1 || nbins > 768)
    return set_error(LOKI_ERR_UNSUPPORTED, "nbins %d outside [1, 768]", nbins);
  if (unit && segment_len >= (int64_t(1) << 24))
    return set_error(LOKI_ERR_UNSUPPORTED, "unit-variance counts need segments below 2^24");
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t nseg = (nsamps + segment_len - 1) / segment_len;
  const int elem = nbins <= 256 ? 1 : 2;
  int64_t chunk = scratch_bytes / (segment_len * elem);
  if (chunk < 1)
    return set_error(LOKI_ERR_CAPACITY, "phase scratch of %lld bytes holds no frequency",
                     (long long)scratch_bytes);
  chunk = std::min(chunk, nfreqs);
  const int nc = unit ? 1 : 2;
  int bs = 128;  // nc * nbins floats of shared memory per thread, <= 200 KB a block
  while (bs > 32 && (size_t)bs * nc * nbins * sizeof(float) > 200 * 1024) bs >>= 1;
  const size_t smem = (size_t)bs * nc * nbins * sizeof(float);
  if (smem > 200 * 1024) return set_error(LOKI_ERR_UNSUPPORTED, "nbins too large");
  auto k8 = unit ? brutefold_seq_kernel<uint8_t, true> : brutefold_seq_kernel<uint8_t, false>;
  auto k16 =
      unit ? brutefold_seq_kernel<uint16_t, true> : brutefold_seq_kernel<uint16_t, false>;
  if (set_smem_limit(k8, (int)smem) != cudaSuccess ||
      set_smem_limit(k16, (int)smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  const int hsmem = 2 * nbins * (int)sizeof(int);
  for (int64_t f0 = 0; f0 < nfreqs; f0 += chunk) {
    const int64_t nf = std::min(chunk, nfreqs - f0);
    const int64_t total = nf * segment_len;
    const int mblocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 64);
    const int64_t blocks = nseg * ((nf + bs - 1) / bs);
    if (blocks > 0x7FFFFFFF || nf > 0x7FFFFFFF)
      return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
    note_launch();
    note_launch();
    if (unit) note_launch();
    if (elem == 1) {
      uint8_t* map = (uint8_t*)phase_scratch;
      phase_map_kernel<uint8_t><<<mblocks, 256, 0, s>>>(freqs + f0, nf, segment_len, nbins,
                                                       tsamp, t_ref, map);
      k8<<<(unsigned)blocks, bs, smem, s>>>(ts_e, ts_v, nsamps, map, nf, f0, nfreqs,
                                            segment_len, nseg, nbins, fold_out);
      if (unit)
        brutefold_count_kernel<uint8_t><<<(unsigned)nf, 256, hsmem, s>>>(
            map, nf, f0, nfreqs, segment_len, nsamps, nseg, nbins, fold_out);
    } else {
      uint16_t* map = (uint16_t*)phase_scratch;
      phase_map_kernel<uint16_t><<<mblocks, 256, 0, s>>>(freqs + f0, nf, segment_len, nbins,
                                                        tsamp, t_ref, map);
      k16<<<(unsigned)blocks, bs, smem, s>>>(ts_e, ts_v, nsamps, map, nf, f0, nfreqs,
                                             segment_len, nseg, nbins, fold_out);
      if (unit)
        brutefold_count_kernel<uint16_t><<<(unsigned)nf, 256, hsmem, s>>>(
            map, nf, f0, nfreqs, segment_len, nsamps, nseg, nbins, fold_out);
    }
    int rc = check_launch("brutefold");
    if (rc) return rc;
  }
  return LOKI_OK;
}

}  // namespace loki

extern "C" int loki_brutefold(const float* ts_e, const float* ts_v, int64_t nsamps,
                              const double* freqs, int64_t nfreqs, int64_t segment_len,
                              int32_t nbins, double tsamp, double t_ref, void* phase_scratch,
                              int64_t scratch_bytes, float* fold_out, void* stream) {
  return brutefold_impl(ts_e, ts_v, false, nsamps, freqs, nfreqs, segment_len, nbins, tsamp,
                        t_ref, phase_scratch, scratch_bytes, fold_out, stream);
}

extern "C" int loki_brutefold_unit_variance(const float* ts_e, int64_t nsamps,
                                            const double* freqs, int64_t nfreqs,
                                            int64_t segment_len, int32_t nbins, double tsamp,
                                            double t_ref, void* phase_scratch,
                                            int64_t scratch_bytes, float* fold_out,
                                            void* stream) {
  return brutefold_impl(ts_e, nullptr, true, nsamps, freqs, nfreqs, segment_len, nbins, tsamp,
                        t_ref, phase_scratch, scratch_bytes, fold_out, stream);
}

// Fixed phase-map scratch of loki_brutefold_noalloc. 16 MiB holds the map of
// one frequency for segments of up to 16 Mi samples (nbins <= 256, one byte a
// sample) or 8 Mi samples (nbins > 256, two bytes); larger frequency grids are
// processed in chunks of as many frequencies as the array holds.
static constexpr int64_t kNoAllocScratchBytes = int64_t(16) << 20;
static __device__ __align__(256) unsigned char g_noalloc_phase_scratch[kNoAllocScratchBytes];

namespace {
// Device address of the array in the current context. Looked up on every call
// (the lookup allocates nothing): an address cached per device ordinal would
// go stale after cudaDeviceReset or under a non-primary context.
int noalloc_scratch(void** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_phase_scratch);
  if (e != cudaSuccess || !p)
    return set_error(LOKI_ERR_CUDA, "cudaGetSymbolAddress of the phase scratch failed: %s",
                     cudaGetErrorString(e));
  *out = p;
  return LOKI_OK;
}
}  // namespace

extern "C" int64_t loki_brutefold_noalloc_scratch_bytes(void) { return kNoAllocScratchBytes; }

extern "C" int loki_brutefold_noalloc(const float* ts_e, const float* ts_v, int64_t nsamps,
                                      const double* freqs, int64_t nfreqs, int64_t segment_len,
                                      int32_t nbins, double tsamp, double t_ref, float* fold_out,
                                      void* stream) {
  if (!ts_e || !ts_v || !freqs || !fold_out)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (nsamps <= 0 || nfreqs <= 0 || segment_len <= 0)
    return set_error(LOKI_ERR_INVALID, "nsamps, nfreqs and segment_len must be > 0");
  if (nbins < 1 || nbins > 768)
    return set_error(LOKI_ERR_UNSUPPORTED, "nbins %d outside [1, 768]", nbins);
  const int64_t elem = nbins <= 256 ? 1 : 2;
  if (segment_len > kNoAllocScratchBytes / elem)
    return set_error(LOKI_ERR_CAPACITY,
                     "segment_len %lld above the no-alloc limit of %lld samples for nbins %d "
                     "(fixed %lld-byte phase scratch)",
                     (long long)segment_len, (long long)(kNoAllocScratchBytes / elem), nbins,
                     (long long)kNoAllocScratchBytes);
  void* scratch = nullptr;
  const int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  // Every map entry a fold reads is written by the phase-map launch of the same
  // chunk, and every fold_out element by one fold thread: nothing is cleared.
  return loki_brutefold(ts_e, ts_v, nsamps, freqs, nfreqs, segment_len, nbins, tsamp, t_ref,
                        scratch, kNoAllocScratchBytes, fold_out, stream);
}
