// Fourier-domain FFA (use_fourier=True): complex brute fold, complex DP level
// with fractional phase shifts, and the inverse-FFT fold norm.
//
// Profiles are (2, nbins_f) complex64 rows, nbins_f = nbins / 2 + 1, stored
// as float2 (re, im). The arithmetic follows the reference's float32 /
// complex64 expressions; its BLAS sgemm, numpy cos/sin and pocketfft inverse
// transform are not reproduced bit for bit, so this path is compared with the
// reference to a stated float32 tolerance.
#include <algorithm>

#include "loki_common.cuh"

namespace loki {

// brutefold_start_complex_opt (core/fold.py:395-481): for every (segment,
// frequency, harmonic h) the DFT sum_t x[t] exp(-2 pi i f_h t tsamp) of both
// components, f_h = float32(f * h), the angle formed in float32 as
// f_h * float32(t * float32(-2 pi tsamp)); then the t_ref phase correction
// exp(i float32(2 pi t_ref) f_h). One thread owns one (frequency, harmonic)
// and kSegs segments, so each basis value serves kSegs segments.
constexpr int kSegs = 16;

// sin and cos of a float32 angle by Cody and Waite's additive reduction
// ("Software Manual for the Elementary Functions", 1980): 2 pi split into
// three float32 parts, the first two with 8 significant bits so that k times
// them is exact for |k| < 2^15 (angles up to about 2e5 rad), subtracted with
// fused multiply-adds; sincosf of the reduced angle then stays on its short
// path. The parts come from 2 pi to 60 digits: 0x1.92p+2 + 0x1.fbp-10 +
// 0x1.5110b4p-20 (their sum is 2 pi to 2e-14).
__device__ __forceinline__ void sincos_reduced(float a, float* s, float* c) {
  constexpr float kC1 = 0x1.92p+2f, kC2 = 0x1.fbp-10f, kC3 = 0x1.5110b4p-20f;
  const float k = rintf(__fmul_rn(a, 0.15915494f));
  if (fabsf(k) < 32768.0f) {
    float r = __fmaf_rn(-k, kC1, a);
    r = __fmaf_rn(-k, kC2, r);
    r = __fmaf_rn(-k, kC3, r);
    sincosf(r, s, c);
  } else {
    sincosf(a, s, c);
  }
}

__global__ void __launch_bounds__(128)
brutefold_complex_kernel(const float* __restrict__ ts_e, const float* __restrict__ ts_v,
                         const double* __restrict__ freqs, int64_t nfreq, int64_t seg_len,
                         int64_t nseg, int nbf, float tfac, float corr_factor,
                         float2* __restrict__ fold) {
  const int64_t ncomb = nfreq * nbf;
  const int64_t comb = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t s0 = (int64_t)blockIdx.y * kSegs;
  if (comb >= ncomb) return;
  const int64_t fi = comb / nbf;
  const int h = (int)(comb - fi * nbf);
  const float fh = (float)(freqs[fi] * (double)h);
  const int ns = (int)std::min<int64_t>(kSegs, nseg - s0);
  float er[kSegs], ei[kSegs], vr[kSegs], vi[kSegs];
#pragma unroll
  for (int k = 0; k < kSegs; ++k) er[k] = ei[k] = vr[k] = vi[k] = 0.0f;
  // ts_v NULL: all ones, so every segment's variance sums are the running sums
  // of the basis values (fmaf(1, c, acc) = acc + c), taken once in vr[0]/vi[0]
  const bool unit = ts_v == nullptr;
  int64_t t = 0;
  // four samples per step with 16-byte (broadcast) loads of each segment;
  // every accumulator still takes its terms in sample order
  const bool vec = (seg_len & 3) == 0 &&
                   ((reinterpret_cast<uintptr_t>(ts_e) | reinterpret_cast<uintptr_t>(ts_v)) &
                    15) == 0;
  if (unit && vec) {
    for (; t < seg_len; t += 4) {
      float sn[4], cs[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float tv = __fmul_rn((float)(t + q), tfac);
        sincos_reduced(__fmul_rn(fh, tv), &sn[q], &cs[q]);
        vr[0] = fmaf(1.0f, cs[q], vr[0]);
        vi[0] = fmaf(1.0f, sn[q], vi[0]);
      }
#pragma unroll
      for (int k = 0; k < kSegs; ++k) {
        if (k < ns) {
          const float4 xe =
              __ldg(reinterpret_cast<const float4*>(ts_e + (s0 + k) * seg_len + t));
          const float e4[4] = {xe.x, xe.y, xe.z, xe.w};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            er[k] = fmaf(e4[q], cs[q], er[k]);
            ei[k] = fmaf(e4[q], sn[q], ei[k]);
          }
        }
      }
    }
  }
  if (vec && !unit) {
    for (; t < seg_len; t += 4) {
      float sn[4], cs[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float tv = __fmul_rn((float)(t + q), tfac);
        sincos_reduced(__fmul_rn(fh, tv), &sn[q], &cs[q]);
      }
#pragma unroll
      for (int k = 0; k < kSegs; ++k) {
        if (k < ns) {
          const int64_t at = (s0 + k) * seg_len + t;
          const float4 xe = __ldg(reinterpret_cast<const float4*>(ts_e + at));
          const float4 xv = __ldg(reinterpret_cast<const float4*>(ts_v + at));
          const float e4[4] = {xe.x, xe.y, xe.z, xe.w}, v4[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            er[k] = fmaf(e4[q], cs[q], er[k]);
            ei[k] = fmaf(e4[q], sn[q], ei[k]);
            vr[k] = fmaf(v4[q], cs[q], vr[k]);
            vi[k] = fmaf(v4[q], sn[q], vi[k]);
          }
        }
      }
    }
  }
  for (; t < seg_len; ++t) {
    const float tv = __fmul_rn((float)t, tfac);
    const float ang = __fmul_rn(fh, tv);
    float sn, cs;
    sincos_reduced(ang, &sn, &cs);
    if (unit) {
      vr[0] = fmaf(1.0f, cs, vr[0]);
      vi[0] = fmaf(1.0f, sn, vi[0]);
    }
#pragma unroll
    for (int k = 0; k < kSegs; ++k) {
      if (k < ns) {
        const int64_t at = (s0 + k) * seg_len + t;
        const float xe = __ldg(ts_e + at);
        er[k] = fmaf(xe, cs, er[k]);
        ei[k] = fmaf(xe, sn, ei[k]);
        if (!unit) {
          const float xv = __ldg(ts_v + at);
          vr[k] = fmaf(xv, cs, vr[k]);
          vi[k] = fmaf(xv, sn, vi[k]);
        }
      }
    }
  }
  if (unit) {
#pragma unroll
    for (int k = 1; k < kSegs; ++k) {
      vr[k] = vr[0];
      vi[k] = vi[0];
    }
  }
  // correction phasor exp(i * float32(corr_factor * f_h)), complex64 multiply
  const float th = __fmul_rn(corr_factor, fh);
  float cs_c, sn_c;
  sincos_reduced(th, &sn_c, &cs_c);
#pragma unroll
  for (int k = 0; k < kSegs; ++k) {  // constant indices keep the sums in registers
    if (k >= ns) break;
    float2* row = fold + ((s0 + k) * nfreq + fi) * 2 * nbf;
    row[h] = make_float2(__fsub_rn(__fmul_rn(er[k], cs_c), __fmul_rn(ei[k], sn_c)),
                         __fadd_rn(__fmul_rn(er[k], sn_c), __fmul_rn(ei[k], cs_c)));
    row[nbf + h] = make_float2(__fsub_rn(__fmul_rn(vr[k], cs_c), __fmul_rn(vi[k], sn_c)),
                               __fadd_rn(__fmul_rn(vr[k], sn_c), __fmul_rn(vi[k], cs_c)));
  }
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                     __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}

// Rotation step of shift_add_complex (core/common.py:344-372): the angle
// float32(float32(-2 pi) * shift) / nbins and its unit phasor.
__device__ __forceinline__ float2 shift_phasor(float shift, int nbins) {
  const float step = __fdiv_rn(__fmul_rn((float)(-2.0 * 3.14159265358979323846), shift),
                               (float)nbins);
  float sn, cs;
  sincosf(step, &sn, &cs);
  return make_float2(cs, sn);
}

// One complex DP level (dynamic/dyn_pffa.py:435-489 with shift_add_complex):
// thread per (output segment, parameter set, component); the plan gives the
// tail / head rows and their float32 phase shifts.
__global__ void ffa_level_complex_kernel(const LokiFFACoord* __restrict__ plan, int64_t Q,
                                         int64_t P_in, int64_t nseg_out, int nbins, int nbf,
                                         const float2* __restrict__ in,
                                         float2* __restrict__ out) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t total = nseg_out * Q * 2;
  if (k >= total) return;
  const int c = (int)(k & 1);
  const int64_t q = (k >> 1) % Q;
  const int64_t ip = (k >> 1) / Q;
  const LokiFFACoord co = plan[q];
  const float2* t = in + (((2 * ip) * P_in + co.i_tail) * 2 + c) * nbf;
  const float2* h = in + (((2 * ip + 1) * P_in + co.i_head) * 2 + c) * nbf;
  float2* o = out + ((ip * Q + q) * 2 + c) * nbf;
  const float2 dt = shift_phasor(co.shift_tail, nbins);
  const float2 dh = shift_phasor(co.shift_head, nbins);
  float2 pt = make_float2(1.0f, 0.0f), ph = make_float2(1.0f, 0.0f);
  for (int j = 0; j < nbf; ++j) {
    const float2 a = cmul(t[j], pt), b = cmul(h[j], ph);
    o[j] = make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
    pt = cmul(pt, dt);
    ph = cmul(ph, dh);
  }
}

// get_fold_norm for Fourier folds (ffa.py:401-411): irfft of each component
// (nbins real samples from nbins_f coefficients, computed in float64 with
// exact twiddles and rounded to float32), then e / sqrt(v).
// irfft (numpy, n = nbins) of each component, then e / sqrt(v). Twiddle
// factors cos/sin(2 pi r / nbins) depend only on r = (m j) mod nbins: a block
// fills a float32 table of nbins entries (float64 sincospi, rounded once) and
// every term reads it; the sums run in float32 with fused multiply-adds, as
// numpy's float32 transform of a complex64 fold does (float64 sums would
// leave the FP64 pipe, a small fraction of GB300's float32 rate, the limit).
__global__ void fold_norm_complex_kernel(const float2* __restrict__ folds, int64_t n, int nbins,
                                         int nbf, float* __restrict__ out) {
  extern __shared__ float tw[];  // [nbins] cos, [nbins] sin
  for (int r = threadIdx.x; r < nbins; r += blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)r / (double)nbins, &s, &c);
    tw[r] = (float)c;
    tw[nbins + r] = (float)s;
  }
  __syncthreads();
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n * nbins) return;
  const int64_t p = k / nbins;
  const int j = (int)(k - p * nbins);
  float val[2];
  for (int c = 0; c < 2; ++c) {
    const float2* x = folds + (p * 2 + c) * nbf;
    float acc = x[0].x;
    int r = 0;
    for (int m = 1; m < nbf; ++m) {
      // the imaginary parts of the DC and (for even nbins) Nyquist terms are
      // ignored; other terms count twice
      r += j;
      if (r >= nbins) r -= nbins;
      const float cth = tw[r], s = tw[nbins + r];
      const float2 xm = x[m];
      if (2 * m == nbins) {
        acc = __fmaf_rn(xm.x, cth, acc);
      } else {
        acc = __fmaf_rn(2.0f * xm.x, cth, acc);
        acc = __fmaf_rn(-2.0f * xm.y, s, acc);
      }
    }
    val[c] = __fdiv_rn(acc, (float)nbins);
  }
  out[k] = __fdiv_rn(val[0], __fsqrt_rn(val[1]));
}

}  // namespace loki

using namespace loki;

extern "C" int loki_brutefold_complex(const float* ts_e, const float* ts_v, int64_t nsamps,
                                      const double* freqs, int64_t nfreqs, int64_t segment_len,
                                      int32_t nbins, double tsamp, double t_ref, void* fold_out,
                                      void* stream) {
  if (!ts_e || !freqs || !fold_out)  // ts_v NULL: all ones
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  if (nsamps <= 0 || nfreqs <= 0 || segment_len <= 0 || nbins < 2)
    return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (nsamps % segment_len != 0)
    return set_error(LOKI_ERR_INVALID,
                     "the Fourier brute fold needs nsamps a multiple of segment_len");
  const int nbf = nbins / 2 + 1;
  const int64_t nseg = nsamps / segment_len;
  const int64_t ncomb = nfreqs * nbf;
  const float tfac = (float)(-2.0 * 3.14159265358979323846 * tsamp);
  const float corr = (float)(2.0 * 3.14159265358979323846 * t_ref);
  const int64_t gx = (ncomb + 127) / 128, gy = (nseg + kSegs - 1) / kSegs;
  if (gx > 0x7FFFFFFF || gy > 65535) return set_error(LOKI_ERR_UNSUPPORTED, "grid too large");
  note_launch();
  brutefold_complex_kernel<<<dim3((unsigned)gx, (unsigned)gy), 128, 0, (cudaStream_t)stream>>>(
      ts_e, ts_v, freqs, nfreqs, segment_len, nseg, nbf, tfac, corr,
      reinterpret_cast<float2*>(fold_out));
  return check_launch("brutefold_complex");
}

extern "C" int loki_ffa_level_complex(const LokiFFALevel* lvl, const LokiFFACoord* plan,
                                      const void* fold_in, void* fold_out, void* stream) {
  if (!lvl || !plan || !fold_in || !fold_out)
    return set_error(LOKI_ERR_INVALID, "null pointer argument");
  int64_t Q = 1, P_in = 1;
  for (int d = 0; d < lvl->nparams; ++d) {
    Q *= lvl->counts_cur[d];
    P_in *= lvl->counts_prev[d];
  }
  if (lvl->out_start != 0 || lvl->out_width != lvl->counts_cur[lvl->nparams - 1] ||
      lvl->in_start != 0 || lvl->in_width != lvl->counts_prev[lvl->nparams - 1])
    return set_error(LOKI_ERR_UNSUPPORTED, "Fourier levels are materialised whole");
  if (lvl->nseg_in < 2 || lvl->nseg_in % 2)
    return set_error(LOKI_ERR_INVALID, "nseg_in must be even");
  const int nbf = lvl->nbins / 2 + 1;
  const int64_t nseg_out = lvl->nseg_in / 2;
  const int64_t total = nseg_out * Q * 2;
  note_launch();
  ffa_level_complex_kernel<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      plan, Q, P_in, nseg_out, lvl->nbins, nbf, reinterpret_cast<const float2*>(fold_in),
      reinterpret_cast<float2*>(fold_out));
  return check_launch("ffa_level_complex");
}

extern "C" int loki_fold_norm_complex(const void* folds, int64_t n, int32_t nbins, float* out,
                                      void* stream) {
  if (n < 0 || nbins < 2) return set_error(LOKI_ERR_INVALID, "bad sizes");
  if (n == 0) return LOKI_OK;
  if (!folds || !out) return set_error(LOKI_ERR_INVALID, "null pointer argument");
  const int64_t total = n * nbins;
  if (nbins > 8192) return set_error(LOKI_ERR_UNSUPPORTED, "nbins above 8192");
  note_launch();
  fold_norm_complex_kernel<<<(unsigned)((total + 255) / 256), 256, 8 * nbins,
                             (cudaStream_t)stream>>>(
      reinterpret_cast<const float2*>(folds), n, nbins, nbins / 2 + 1, out);
  return check_launch("fold_norm_complex");
}
