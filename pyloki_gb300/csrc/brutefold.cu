// Brute fold at the start of the FFA (core/fold.py:108-171 brutefold_start).
//
// Two paths give the same bit-identical sums. With nbins <= 256 and room for
// the chain layout in the scratch, the chain path below (chain_order_kernel,
// brutefold_chain_kernel). Otherwise the per-thread walk described next.
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


// ---------------------------------------------------------------------------
// Chain layout (nbins <= 256). Each (segment, frequency, bin) sum is a chain
// of adds in sample order. The order in which a frequency's samples reach its
// bins depends only on the sample position within a segment, so it is built
// once per frequency (chain_order_kernel): the segment is cut into time
// chunks of kChunk samples, and within a chunk the samples are listed bin by
// bin, in time order, as byte offsets into a shared-memory row. Each bin's run
// is padded to a multiple of 4 entries with the offset of a zero column, so a
// 16-byte load yields 4 entries and adding the zeros leaves a sum unchanged
// (a sum that starts at +0 and adds finite or infinite values is never -0, and
// x + 0 = x for every other x). Walking a bin's entries chunk after chunk
// visits its samples in the reference's order.
//
// brutefold_chain_kernel gives each lane one segment (32 segments per block)
// and each warp a set of (frequency, bin) chains: all lanes step through the
// same chain at once, so the entries are broadcasts, there is no divergence,
// and the 32 segments' samples sit in 32 different shared-memory banks (rows
// of kChunk + 1 floats, the last one the zero column). The chain sums live in
// shared memory between chunks.
// ---------------------------------------------------------------------------

constexpr int kChunk = 512;        // samples per time chunk
constexpr int kChainWarps = 16;    // warps per fold block
constexpr int kChainRow = kChunk + 1;
constexpr uint32_t kZeroOff = kChunk * 4;  // byte offset of the zero column

__host__ __device__ inline int chain_nbp(int nbins) { return (nbins + 1 + 7) & ~7; }
// groups of 4 entries per (frequency, chunk): sum of ceil(n_b / 4) <= C/4 + nbins
__host__ __device__ inline int chain_groups(int nbins) { return kChunk / 4 + nbins; }

// One warp per (frequency, time chunk): order[f][t] = groups of 4 byte
// offsets sorted by bin (stable, padded per bin); offs[f][t][b] = first group
// of bin b, offs[f][t][nbins] = groups in use.
__global__ void __launch_bounds__(256)
chain_order_kernel(const uint8_t* __restrict__ map, int64_t nfreq, int64_t seg_len, int nbins,
                   uint32_t* __restrict__ order, uint16_t* __restrict__ offs) {
  __shared__ int cnt_all[8][256];
  __shared__ int pos_all[8][256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t nch = (seg_len + kChunk - 1) / kChunk;
  const int64_t item = (int64_t)blockIdx.x * 8 + warp;
  if (item >= nfreq * nch) return;  // no block-level synchronisation follows
  const int64_t f = item / nch, t = item - f * nch;
  const int nbp = chain_nbp(nbins), gc = chain_groups(nbins);
  const int clen = (int)min((int64_t)kChunk, seg_len - t * kChunk);
  const uint8_t* m = map + f * seg_len + t * kChunk;
  int* cnt = cnt_all[warp];
  int* pos = pos_all[warp];
  for (int b = lane; b < nbins; b += 32) cnt[b] = 0;
  __syncwarp();
  const unsigned lt = (1u << lane) - 1u;
  for (int s0 = 0; s0 < clen; s0 += 32) {  // counts per bin
    const int s = s0 + lane;
    const bool ok = s < clen;
    const int b = ok ? (int)m[s] : -1 - lane;
    const unsigned grp = __match_any_sync(0xFFFFFFFFu, b);
    if (ok && (grp & lt) == 0) cnt[b] += __popc(grp);
    __syncwarp();
  }
  // exclusive scan of the padded group counts: lane l owns bins [l*per, (l+1)*per)
  const int per = (nbins + 31) / 32;
  int local = 0;
  for (int q = 0; q < per; ++q) {
    const int b = lane * per + q;
    if (b < nbins) local += (cnt[b] + 3) >> 2;
  }
  int incl = local;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o) incl += y;
  }
  const int total = __shfl_sync(0xFFFFFFFFu, incl, 31);
  int run = incl - local;
  uint16_t* of = offs + (f * nch + t) * nbp;
  uint32_t* od = order + (f * nch + t) * (int64_t)gc * 4;
  for (int q = 0; q < per; ++q) {
    const int b = lane * per + q;
    if (b < nbins) {
      const int c = cnt[b], g = (c + 3) >> 2;
      of[b] = (uint16_t)run;
      pos[b] = 4 * run;  // the next free entry of bin b
      for (int k = c; k < 4 * g; ++k) od[4 * run + k] = kZeroOff;  // padding
      run += g;
    }
  }
  for (int b = nbins + lane; b < nbp; b += 32) of[b] = (uint16_t)total;
  __syncwarp();
  for (int s0 = 0; s0 < clen; s0 += 32) {  // stable scatter
    const int s = s0 + lane;
    const bool ok = s < clen;
    const int b = ok ? (int)m[s] : -1 - lane;
    const unsigned grp = __match_any_sync(0xFFFFFFFFu, b);
    if (ok) od[pos[b] + __popc(grp & lt)] = (uint32_t)s * 4u;
    __syncwarp();
    if (ok && (grp >> lane) == 1u) pos[b] += __popc(grp);  // highest lane of the group
    __syncwarp();
  }
}

__device__ __forceinline__ float lds_f32(uint32_t addr) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
  return v;
}

__device__ __forceinline__ uint4 lds_u32x4(uint32_t addr) {
  uint4 v;
  asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "r"(addr));
  return v;
}

// Block: 32 segments (lanes) x F frequencies; chain c = f * nbins + b, warp w
// walks chains w, w + 16, ... NC = 2 also sums ts_v. Shared memory, in order:
// series rows [NC][32][kChainRow] f32, chain sums [NC][F * nbins][33] f32,
// order groups [F][gc] uint4, chain table [F * nbins] u32, bin starts
// [F][nbp] u16.
template <int NC>
__global__ void __launch_bounds__(kChainWarps * 32, NC == 1 ? 2 : 1)
brutefold_chain_kernel(const float* __restrict__ ts_e, const float* __restrict__ ts_v,
                       int64_t nsamps, const uint32_t* __restrict__ order,
                       const uint16_t* __restrict__ offs, int64_t nfreq_chunk, int64_t f_offset,
                       int64_t nfreq_total, int64_t seg_len, int64_t nseg, int nbins, int F,
                       float* __restrict__ fold) {
  extern __shared__ __align__(16) float csm[];
  const int nbp = chain_nbp(nbins), gc = chain_groups(nbins);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t nsg = (nseg + 31) / 32;
  const int64_t sg = blockIdx.x % nsg, fg = blockIdx.x / nsg;
  const int64_t f0 = fg * F;
  const int nfb = (int)min((int64_t)F, nfreq_chunk - f0);
  const int nchains = nfb * nbins;
  const int nct = F * nbins;  // chain slots
  static_assert(kChunk == kChainWarps * 32, "one series sample per thread and row");
  float* xs = csm;                        // [NC][32][kChainRow]
  float* acc = xs + NC * 32 * kChainRow;  // [NC][nct][33]
  const int fl = (NC * 32 * kChainRow + NC * nct * 33 + 3) & ~3;
  uint4* ord_s = reinterpret_cast<uint4*>(csm + fl);
  uint32_t* tab = reinterpret_cast<uint32_t*>(ord_s + F * gc);
  uint16_t* off_s = reinterpret_cast<uint16_t*>(tab + nct);
  const int64_t nch = (seg_len + kChunk - 1) / kChunk;
  for (int r = tid; r < NC * 32; r += kChainWarps * 32) xs[r * kChainRow + kChunk] = 0.0f;
  for (int i = tid; i < NC * nct * 33; i += kChainWarps * 32) acc[i] = 0.0f;
  for (int c = tid; c < nchains; c += kChainWarps * 32) {
    const int f = c / nbins, b = c - f * nbins;
    tab[c] = (uint32_t)(f * gc) | ((uint32_t)(f * nbp + b) << 16);
  }
  // 32-bit shared addresses: the lane's series row, the order groups
  const uint32_t xb = (uint32_t)__cvta_generic_to_shared(xs + lane * kChainRow);
  const uint32_t ob = (uint32_t)__cvta_generic_to_shared(ord_s);
  constexpr uint32_t kV = 32 * kChainRow * 4;  // ts_v rows follow the ts_e rows
  const bool interior = sg * 32 + 32 < nseg;  // 32 full segments, none of them the last
  for (int64_t t = 0; t < nch; ++t) {
    const int clen = (int)min((int64_t)kChunk, seg_len - t * kChunk);
    __syncthreads();  // the previous chunk's rows are consumed (and the setup is done)
    // series rows: row r = segment sg * 32 + r; samples beyond nsamps (and
    // rows beyond the last segment) are 0
    const int64_t p0 = sg * 32 * seg_len + t * kChunk;
    if (interior && clen == kChunk) {  // one sample of every row a thread, no checks
      const float* pe = ts_e + p0 + tid;
#pragma unroll 8
      for (int r = 0; r < 32; ++r) {
        xs[r * kChainRow + tid] = __ldg(pe + (int64_t)r * seg_len);
        if constexpr (NC == 2)
          xs[(32 + r) * kChainRow + tid] = __ldg(ts_v + p0 + tid + (int64_t)r * seg_len);
      }
    } else if (tid < clen) {
      for (int r = 0; r < 32; ++r) {
        const int64_t p = p0 + (int64_t)r * seg_len + tid;
        const bool in = sg * 32 + r < nseg && p < nsamps;
        xs[r * kChainRow + tid] = in ? __ldg(ts_e + p) : 0.0f;
        if constexpr (NC == 2) xs[(32 + r) * kChainRow + tid] = in ? __ldg(ts_v + p) : 0.0f;
      }
    }
    // this chunk's order groups and bin starts of the block's frequencies
    for (int i = tid; i < nfb * gc; i += kChainWarps * 32) {
      const int f = i / gc, q = i - f * gc;
      ord_s[i] = __ldg(reinterpret_cast<const uint4*>(order + ((f0 + f) * nch + t) * gc * 4) + q);
    }
    for (int i = tid; i < nfb * nbp; i += kChainWarps * 32) {
      const int f = i / nbp, q = i - f * nbp;
      off_s[i] = offs[((f0 + f) * nch + t) * nbp + q];
    }
    __syncthreads();
    for (int c = warp; c < nchains; c += kChainWarps) {
      const uint32_t tb = tab[c];
      const int oi = (int)(tb >> 16);
      const uint32_t g0 = off_s[oi], g1 = off_s[oi + 1];
      float a = acc[c * 33 + lane];
      float v = NC == 2 ? acc[(nct + c) * 33 + lane] : 0.0f;
      const uint32_t gend = ob + ((tb & 0xFFFFu) + g1) * 16u;
      for (uint32_t ga = ob + ((tb & 0xFFFFu) + g0) * 16u; ga < gend; ga += 16u) {
        const uint4 e = lds_u32x4(ga);
        a = __fadd_rn(a, lds_f32(xb + e.x));
        a = __fadd_rn(a, lds_f32(xb + e.y));
        a = __fadd_rn(a, lds_f32(xb + e.z));
        a = __fadd_rn(a, lds_f32(xb + e.w));
        if constexpr (NC == 2) {
          v = __fadd_rn(v, lds_f32(xb + kV + e.x));
          v = __fadd_rn(v, lds_f32(xb + kV + e.y));
          v = __fadd_rn(v, lds_f32(xb + kV + e.z));
          v = __fadd_rn(v, lds_f32(xb + kV + e.w));
        }
      }
      acc[c * 33 + lane] = a;
      if constexpr (NC == 2) acc[(nct + c) * 33 + lane] = v;
    }
  }
  __syncthreads();
  // the block's sums, whole rows to the fold
  for (int r = 0; r < 32; ++r) {
    const int64_t g = sg * 32 + r;
    if (g >= nseg) break;
    for (int c = tid; c < nchains; c += kChainWarps * 32) {
      const int f = c / nbins, b = c - f * nbins;
      float* out = fold + ((size_t)g * nfreq_total + f_offset + f0 + f) * 2 * nbins;
      out[b] = acc[c * 33 + r];
      if constexpr (NC == 2) out[nbins + b] = acc[(nct + c) * 33 + r];
    }
  }
}

}  // namespace loki

using namespace loki;

namespace loki {

// Bytes per frequency of the chain layout: map, order groups, bin starts.
static int64_t chain_bytes_per_freq(int64_t seg_len, int nbins) {
  const int64_t nch = (seg_len + kChunk - 1) / kChunk;
  return seg_len + nch * chain_groups(nbins) * 16 + nch * chain_nbp(nbins) * 2;
}

static int64_t round256(int64_t x) { return (x + 255) & ~int64_t(255); }

static int chain_smem(int nbins, int nc, int F) {
  const int nct = F * nbins;
  const int fl = (nc * 32 * kChainRow + nc * nct * 33 + 3) & ~3;  // 16-byte aligned groups
  return fl * 4 + F * chain_groups(nbins) * 16 + nct * 4 + F * chain_nbp(nbins) * 2;
}

// Frequencies per fold block (F) and its shared memory; F = 0: the chain
// kernel does not apply. Unit variance: two blocks per SM.
static void chain_shape(int nbins, int nc, int* F, int* smem) {
  *F = 0;
  *smem = 0;
  if (nbins < 1 || nbins > 256) return;
  // unit variance: two blocks in the 228 KB of an SM (1 KB reserved per block)
  const int limit = nc == 1 ? 114 * 1024 - 1024 : 220 * 1024;
  int f = 16;
  while (f > 0 && chain_smem(nbins, nc, f) > limit) --f;
  *F = f;
  *smem = f > 0 ? chain_smem(nbins, nc, f) : 0;
}

// Frequencies of the chain layout that fit in the scratch (0: none).
static int64_t chain_chunk(int64_t scratch_bytes, int64_t seg_len, int nbins) {
  const int64_t per = chain_bytes_per_freq(seg_len, nbins);
  return std::max<int64_t>(0, (scratch_bytes - 3 * 256) / per);
}

// The chain path: per frequency chunk, the phase map, the chain order, the
// chain fold and (unit) the count rows.
static int brutefold_chain(const float* ts_e, const float* ts_v, bool unit, int64_t nsamps,
                           const double* freqs, int64_t nfreqs, int64_t seg_len, int nbins,
                           double tsamp, double t_ref, char* scratch, int64_t chunk, int F,
                           int smem, float* fold_out, cudaStream_t s) {
  const int64_t nseg = (nsamps + seg_len - 1) / seg_len;
  const int64_t nch = (seg_len + kChunk - 1) / kChunk;
  auto kf = unit ? brutefold_chain_kernel<1> : brutefold_chain_kernel<2>;
  if (set_smem_limit(kf, smem) != cudaSuccess)
    return set_error(LOKI_ERR_CUDA, "cudaFuncSetAttribute failed");
  uint8_t* map = reinterpret_cast<uint8_t*>(scratch);
  uint32_t* order = reinterpret_cast<uint32_t*>(scratch + round256(chunk * seg_len));
  uint16_t* offs = reinterpret_cast<uint16_t*>(
      scratch + round256(chunk * seg_len) + round256(chunk * nch * chain_groups(nbins) * 16));
  const int hsmem = 2 * nbins * (int)sizeof(int);
  const int64_t nsg = (nseg + 31) / 32;
  for (int64_t f0 = 0; f0 < nfreqs; f0 += chunk) {
    const int64_t nf = std::min(chunk, nfreqs - f0);
    const int64_t total = nf * seg_len;
    const int mblocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 64);
    const int64_t oblocks = (nf * nch + 7) / 8;
    const int64_t blocks = nsg * ((nf + F - 1) / F);
    if (blocks > 0x7FFFFFFF || oblocks > 0x7FFFFFFF)
      return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
    for (int i = 0; i < (unit ? 4 : 3); ++i) note_launch();
    phase_map_kernel<uint8_t><<<mblocks, 256, 0, s>>>(freqs + f0, nf, seg_len, nbins, tsamp,
                                                     t_ref, map);
    chain_order_kernel<<<(unsigned)oblocks, 256, 0, s>>>(map, nf, seg_len, nbins, order, offs);
    kf<<<(unsigned)blocks, kChainWarps * 32, smem, s>>>(ts_e, ts_v, nsamps, order, offs, nf, f0,
                                                        nfreqs, seg_len, nseg, nbins, F,
                                                        fold_out);
    if (unit)
      brutefold_count_kernel<uint8_t><<<(unsigned)nf, 256, hsmem, s>>>(
          map, nf, f0, nfreqs, seg_len, nsamps, nseg, nbins, fold_out);
    int rc = check_launch("brutefold_chain");
    if (rc) return rc;
  }
  return LOKI_OK;
}

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
  const int nc = unit ? 1 : 2;
  {  // the chain layout when it applies and one frequency of it fits
    int F = 0, csmem = 0;
    chain_shape(nbins, nc, &F, &csmem);
    const int64_t cchunk = std::min(chain_chunk(scratch_bytes, segment_len, nbins), nfreqs);
    if (F > 0 && cchunk > 0)
      return brutefold_chain(ts_e, ts_v, unit, nsamps, freqs, nfreqs, segment_len, nbins, tsamp,
                             t_ref, reinterpret_cast<char*>(phase_scratch), cchunk, F, csmem,
                             fold_out, s);
  }
  const int64_t nseg = (nsamps + segment_len - 1) / segment_len;
  const int elem = nbins <= 256 ? 1 : 2;
  int64_t chunk = scratch_bytes / (segment_len * elem);
  if (chunk < 1)
    return set_error(LOKI_ERR_CAPACITY, "phase scratch of %lld bytes holds no frequency",
                     (long long)scratch_bytes);
  chunk = std::min(chunk, nfreqs);
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

extern "C" int64_t loki_brutefold_scratch_bytes(int64_t nfreqs, int64_t segment_len,
                                                int32_t nbins) {
  if (nfreqs <= 0 || segment_len <= 0 || nbins < 1) return 0;
  int F = 0, smem = 0;
  chain_shape(nbins, 1, &F, &smem);
  if (F > 0) return 3 * 256 + nfreqs * chain_bytes_per_freq(segment_len, nbins);
  return nfreqs * segment_len * (nbins <= 256 ? 1 : 2);
}

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
