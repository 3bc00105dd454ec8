// Fused multi-stage polyphase upsampling FIR for sm_103a, with the engine glue
// around it (reference src/engine.c:608-717, src/fir.c:523-725):
//
//   PCM float  -> boxcar running mean over `taps` samples (optional)
//              -> S upsampling stages (2x half-band 63/127 taps, or a 4x
//                 quarter-band 127-tap stage), FP32 FMA polyphase
//              -> gain ramp g_start + step * i and the soft clip's threshold
//                 test in FP32, the tanh knee above +-0.95 in FP64 (optional)
//              -> double output for the trellis SDM
//
// Two kernels, either way one read of the PCM input and one write of the
// output in HBM:
//   fir_poly_kernel   chains of five to eight 63-tap half-band stages (factor
//                     32 to 256: the PCM rates into DSD64 / DSD128 / DSD256)
//                     as one polyphase stage of the chain's combined response,
//                     register-tiled (below);
//   fir_chain_kernel  every other chain as a cascade: one CTA produces a tile
//                     of final outputs for one channel, walks the chain
//                     backwards to find the input range each stage needs,
//                     stages the PCM window (with its history halo) and every
//                     intermediate signal in shared memory, and writes only
//                     the final tile, two outputs per 16-byte store.
//
// Stream continuity: a call may be one block of a longer stream.  The last
// kHistory PCM samples of the previous block are kept per channel and stand in
// for negative input indices, so the chain is the same LTI system as one long
// run (the delay lines of ippsFIRMR, src/fir.c:319-329).
//
// Half-band taps at even offsets from the centre are sin(k pi)/(k pi) ~ 1e-17
// in the FP64 design; they are dropped from the FP32 polyphase because their
// products are below FP32 resolution of any output.
#include "api_context.h"
#include "fir_internal.h"
#include "fp_convert.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace dsdgpu {

// floor division for possibly negative numerators.  Stage ratios are powers
// of two (2 or 4): an arithmetic shift, since a 64-bit integer division runs
// through the FP64 pipe's reciprocal on this part.
__device__ __forceinline__ long long fdiv(long long a, int b) {
  if (b > 0 && (b & (b - 1)) == 0) return a >> (__ffs(b) - 1);
  return a >= 0 ? a / b : -((-a + b - 1) / b);
}

// One 63-tap half-band 2x stage (the chain's common stage): outputs m in
// [mlo, mhi) of the signal whose input window in shared memory is [ilo, ihi).
// out[2i] = sum_t h'[2t] x[i - t] (32 taps), out[2i + 1] = h'[31] x[i - 15].
// A thread computes kHbR consecutive input indices from a register window of
// kHbR + 31 inputs (each input read once from shared memory for up to 32
// products); kHbR is odd, so the warp's window loads, kHbR floats apart per
// lane, fall in distinct banks.
constexpr int kHbR = 9;
constexpr int kHbTaps = 32;

__device__ __forceinline__ void halfband_stage(const FirChainConst& F, const float* in,
                                               long long ilo, long long ihi, float* out,
                                               long long mlo, long long mhi) {
  // indices relative to the stage's windows in shared memory (32-bit)
  const long long i0 = fdiv(mlo, 2);
  const int n_in = (int)(ihi - ilo);
  const int n_out = (int)(mhi - mlo);
  const int i0r = (int)(i0 - ilo);           // >= 31: the stage's halo
  const int moff = (int)(2 * ilo - mlo);     // out index of input index r: 2 r + moff
  const int nb = (int)((fdiv(mhi - 1, 2) + 1 - i0 + kHbR - 1) / kHbR);
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    const int ib = i0r + b * kHbR;
    float w[kHbR + kHbTaps - 1];
    if (ib + kHbR - 1 < n_in) {
#pragma unroll
      for (int j = 0; j < kHbR + kHbTaps - 1; j++) w[j] = in[ib - (kHbTaps - 1) + j];
    } else {
#pragma unroll
      for (int j = 0; j < kHbR + kHbTaps - 1; j++) {
        const int idx = ib - (kHbTaps - 1) + j;
        w[j] = idx < n_in ? in[idx] : 0.0f;
      }
    }
#pragma unroll
    for (int q = 0; q < kHbR; q++) {
      float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
      for (int t = 0; t < kHbTaps; t += 2) {
        a0 = fmaf(F.hb[t], w[q + kHbTaps - 1 - t], a0);
        a1 = fmaf(F.hb[t + 1], w[q + kHbTaps - 2 - t], a1);
      }
      const int m = 2 * (ib + q) + moff;
      if ((unsigned)m < (unsigned)n_out) out[m] = a0 + a1;
      if ((unsigned)(m + 1) < (unsigned)n_out) out[m + 1] = F.hb_center * w[q + kHbTaps - 16];
    }
  }
}

// A merged stage (factor U = 8 or 16, kPolyTaps taps per branch, its branch r
// at taps[r * kPolyTaps] whatever its place in the chain): out[U*i + r] =
// sum_j hm[U*j + r] x[i - j].  A work item is (branch group g, input index i): the inputs
// x[i - j], streamed through registers kPolyChunk at a time, feed the
// group's kPolyGroup branches.  Items run i fastest, so a warp's lanes share
// the group, whose taps are compile-time constant operands (one instance per
// group), and read consecutive inputs.
constexpr int kPolyChunk = 12;
static_assert(kPolyTaps % kPolyChunk == 0 && kPolyChunk % 2 == 0, "chunked taps");

template <int G>
__device__ __forceinline__ void poly_item(const FirChainConst& F, const float* in, int base,
                                          float (&a)[kPolyGroup]) {
  float a0[kPolyGroup], a1[kPolyGroup];
#pragma unroll
  for (int rr = 0; rr < kPolyGroup; rr++) a0[rr] = a1[rr] = 0.0f;
#pragma unroll
  for (int c = 0; c < kPolyTaps; c += kPolyChunk) {
    float w[kPolyChunk];
#pragma unroll
    for (int jj = 0; jj < kPolyChunk; jj++) w[jj] = in[base - c - jj];
#pragma unroll
    for (int rr = 0; rr < kPolyGroup; rr++) {
      constexpr int kRow = G * kPolyGroup * kPolyTaps;
#pragma unroll
      for (int jj = 0; jj < kPolyChunk; jj += 2) {
        a0[rr] = fmaf(F.taps[kRow + rr * kPolyTaps + c + jj], w[jj], a0[rr]);
        a1[rr] = fmaf(F.taps[kRow + rr * kPolyTaps + c + jj + 1], w[jj + 1], a1[rr]);
      }
    }
  }
#pragma unroll
  for (int rr = 0; rr < kPolyGroup; rr++) a[rr] = a0[rr] + a1[rr];
}

__device__ __forceinline__ void poly_stage(const FirChainConst& F, int k, const float* in,
                                           long long ilo, float* out, long long mlo,
                                           long long mhi) {
  const int U = F.U[k];
  const long long i0 = fdiv(mlo, U), i1 = fdiv(mhi - 1, U) + 1;
  const int ni = (int)(i1 - i0);
  const int groups = U / kPolyGroup;
  for (int it = threadIdx.x; it < groups * ni; it += blockDim.x) {
    const int g = it / ni;
    const int il = it - g * ni;
    const int base = (int)(i0 + il - ilo);   // >= kPolyTaps - 1: the stage's halo
    float a[kPolyGroup];
    switch (g) {
      case 0: poly_item<0>(F, in, base, a); break;
      case 1: poly_item<1>(F, in, base, a); break;
      case 2: poly_item<2>(F, in, base, a); break;
      default: poly_item<3>(F, in, base, a); break;
    }
    const long long mb = (long long)U * (i0 + il) + g * kPolyGroup;
#pragma unroll
    for (int rr = 0; rr < kPolyGroup; rr++) {
      const long long m = mb + rr;
      if (m >= mlo && m < mhi) out[m - mlo] = a[rr];
    }
  }
}

// Any other stage (the 127-tap first stage into DSD512, the 4x quarter-band
// stage): one thread per input index i, outputs U*i + r.
__device__ __forceinline__ void generic_stage(const FirChainConst& F, int k, const float* in,
                                              long long ilo, float* out, long long mlo,
                                              long long mhi) {
  const int U = F.U[k];
  const long long i0 = fdiv(mlo, U), i1 = fdiv(mhi - 1, U) + 1;
  for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    for (int r = 0; r < U; r++) {
      const long long m = (long long)U * i + r;
      if (m < mlo || m >= mhi) continue;
      const int nt = F.nphase[k][r];
      const int toff = F.phase_off[k][r];
      float acc0 = 0.0f, acc1 = 0.0f;
      int t = 0;
      for (; t + 1 < nt; t += 2) {
        acc0 = fmaf(F.taps[toff + t], in[i - F.lag[toff + t] - ilo], acc0);
        acc1 = fmaf(F.taps[toff + t + 1], in[i - F.lag[toff + t + 1] - ilo], acc1);
      }
      if (t < nt) acc0 = fmaf(F.taps[toff + t], in[i - F.lag[toff + t] - ilo], acc0);
      out[m - mlo] = acc0 + acc1;
    }
  }
}

// 0 <= p < 2^23 as a float, exactly, without a conversion instruction: the
// integer placed in the significand of 2^23, minus 2^23.
__device__ __forceinline__ float small_to_float(int p) {
  return __fsub_rn(__int_as_float(0x4B000000 | p), 8388608.0f);
}

// The engine's epilogue of one output (src/engine.c:646-651, 704-717): gain
// ramp and the soft clip's threshold test in FP32 (within the chain's 1e-6
// contract), the tanh knee in FP64 on the rare samples above the threshold,
// one widening per output (integer operations).  The ramp is
// gb + step * p, with gb = g_start + step * (tile start) formed once per
// thread and p the output's offset in the tile: no per-output conversion.
__device__ __forceinline__ double fir_epilogue(float v, int p, float gb, float gstep,
                                               int apply_gain, int soft_clip) {
  const float y = apply_gain ? v * fmaf(gstep, small_to_float(p), gb) : v;
  if (soft_clip && fabsf(y) > 0.95f) return soft_clip_095((double)y);
  return widen_normal_fast(y);
}

// The same output for a consumer that reads FP32 (the PreCorr walk narrows
// its input to FP32): y itself, which equals narrowing its exact widening;
// the rare knee value narrowed as that consumer would.
__device__ __forceinline__ float fir_epilogue_f32(float v, int p, float gb, float gstep,
                                                  int apply_gain, int soft_clip) {
  const float y = apply_gain ? v * fmaf(gstep, small_to_float(p), gb) : v;
  if (soft_clip && fabsf(y) > 0.95f) return __double2float_rn(soft_clip_095((double)y));
  return y;
}

template <typename OutT>
__device__ __forceinline__ OutT fir_out(float v, int p, float gb, float gstep, int apply_gain,
                                        int soft_clip);
template <>
__device__ __forceinline__ double fir_out<double>(float v, int p, float gb, float gstep,
                                                  int apply_gain, int soft_clip) {
  return fir_epilogue(v, p, gb, gstep, apply_gain, soft_clip);
}
template <>
__device__ __forceinline__ float fir_out<float>(float v, int p, float gb, float gstep,
                                                int apply_gain, int soft_clip) {
  return fir_epilogue_f32(v, p, gb, gstep, apply_gain, soft_clip);
}

// The epilogue's last part for an output whose gain is applied: the knee or
// the widening (or, for FP32 consumers, the value itself).
template <typename OutT>
__device__ __forceinline__ OutT fir_finish(float y, bool knee);
template <>
__device__ __forceinline__ double fir_finish<double>(float y, bool knee) {
  return knee ? soft_clip_095((double)y) : widen_normal_fast(y);
}
template <>
__device__ __forceinline__ float fir_finish<float>(float y, bool knee) {
  return knee ? __double2float_rn(soft_clip_095((double)y)) : y;
}

template <typename T> struct Pair2;
template <> struct Pair2<double> { using type = double2; };
template <> struct Pair2<float> { using type = float2; };

// The chain description is a by-value kernel parameter (constant bank, about
// 8.7 KB): every launch carries its own chain, so contexts and batch streams
// with different rate pairs never share mutable device constants.
template <typename OutT>
__global__ void __launch_bounds__(kFirThreads, 2)
fir_chain_kernel(const __grid_constant__ FirChainConst F, const float* __restrict__ pcm,
                 size_t pcm_stride, long long count, const float* __restrict__ hist,
                 OutT* __restrict__ out, size_t out_stride, float g_start, float g_step,
                 int apply_gain, int soft_clip, int vec2) {
  extern __shared__ float sm[];
  const int ch = blockIdx.y;
  const long long total_out = count * F.ratio;
  const long long o_lo = (long long)blockIdx.x * F.tile;
  if (o_lo >= total_out) return;
  const long long o_hi = min(o_lo + (long long)F.tile, total_out);

  // ranges of every signal: sig[S] is the output, sig[0] the boxcar output
  long long lo[kMaxStages + 1], hi[kMaxStages + 1];
  lo[F.S] = o_lo;
  hi[F.S] = o_hi;
  for (int k = F.S - 1; k >= 0; k--) {
    lo[k] = fdiv(lo[k + 1] - (F.L[k] - 1), F.U[k]);
    hi[k] = fdiv(hi[k + 1] - 1, F.U[k]) + 1;
  }
  const int bt = F.boxcar;
  const long long p_lo = lo[0] - (bt > 0 ? bt - 1 : 0);

  // shared layout: [pcm window][sig 0][sig 1]...[sig S-1][final tile]
  float* buf[kMaxStages + 1];
  float* pw = sm;
  int off = (int)(hi[0] - p_lo);
  for (int k = 0; k < F.S; k++) {
    buf[k] = sm + off;
    off += (int)(hi[k] - lo[k]);
  }
  buf[F.S] = sm + ((off + 3) & ~3);

  const float* x = pcm + (size_t)ch * pcm_stride;
  const float* hx = hist + (size_t)ch * kHistory;
  for (long long i = p_lo + threadIdx.x; i < hi[0]; i += blockDim.x) {
    float v;
    if (i >= 0) v = x[i];
    else if (i >= -kHistory) v = hx[kHistory + i];
    else v = 0.0f;
    pw[i - p_lo] = v;
  }
  __syncthreads();

  // boxcar: mean of the last `bt` samples (the reference keeps a running FP64
  // sum; the direct sum differs only in rounding)
  for (long long i = lo[0] + threadIdx.x; i < hi[0]; i += blockDim.x) {
    float v;
    if (bt > 0) {
      float s = 0.0f;
      for (int j = 0; j < bt; j++) s += pw[i - j - p_lo];
      v = s * F.inv_boxcar;
    } else {
      v = pw[i - p_lo];
    }
    buf[0][i - lo[0]] = v;
  }
  __syncthreads();

  for (int k = 0; k < F.S; k++) {
    if (F.poly_stage[k])
      poly_stage(F, k, buf[k], lo[k], buf[k + 1], lo[k + 1], hi[k + 1]);
    else if (F.hb_stage[k])
      halfband_stage(F, buf[k], lo[k], hi[k], buf[k + 1], lo[k + 1], hi[k + 1]);
    else
      generic_stage(F, k, buf[k], lo[k], buf[k + 1], lo[k + 1], hi[k + 1]);
    __syncthreads();
  }

  // the final tile to HBM: consecutive threads write consecutive outputs,
  // two per 16-byte store where the row allows it
  const float* fin = buf[F.S];
  const int n = (int)(o_hi - o_lo);   // <= tile < 2^23
  OutT* dst = out + (size_t)ch * out_stride + o_lo;
  const float gb = fmaf(g_step, (float)o_lo, g_start);
  if (vec2) {
    using P2 = typename Pair2<OutT>::type;
    for (int p = 2 * (int)threadIdx.x; p < n; p += 2 * (int)blockDim.x) {
      const OutT y0 = fir_out<OutT>(fin[p], p, gb, g_step, apply_gain, soft_clip);
      if (p + 1 < n) {
        const OutT y1 = fir_out<OutT>(fin[p + 1], p + 1, gb, g_step, apply_gain, soft_clip);
        P2 v;
        v.x = y0;
        v.y = y1;
        *reinterpret_cast<P2*>(dst + p) = v;
      } else {
        dst[p] = y0;
      }
    }
  } else {
    for (int p = threadIdx.x; p < n; p += blockDim.x)
      dst[p] = fir_out<OutT>(fin[p], p, gb, g_step, apply_gain, soft_clip);
  }
}

// The whole chain as one polyphase stage (chains of five to eight 63-tap
// half-band stages: factor U = 32, 64, 128 or 256): out[U*i + r] = sum_k
// h_r[k] b[i - k], b the boxcar output, h_r[k] = hm[U*k + r] the chain's
// combined response (length 62 (U - 1) + 1, at most 62 taps per branch,
// zero-padded to kPolyK).  For fixed k this is an outer product of a column
// of inputs and a row of taps, so each thread holds an 8 x 8 block of outputs
// (8 consecutive input indices x 8 branches, in pairs spread so that a row's
// pair stores from neighbouring lanes are contiguous) in registers and per
// tap row does 64 FMAs from 8 inputs (a register window sliding along k) and
// 8 taps (four broadcast 8-byte shared loads), as 32 packed FMAs.  No intermediate signal,
// no stage barrier; the combined filter's FP32 result differs from the
// stage-by-stage cascade only in rounding.  A warp holds (32 / RT) x 8 input
// indices and RT x 8 branches; a CTA covers kPolyOut outputs.
template <int RT, typename OutT>
__global__ void __launch_bounds__(kFirThreads, 2)
fir_poly_kernel(const __grid_constant__ FirChainConst F, const float* __restrict__ taps,
                const float* __restrict__ pcm, size_t pcm_stride, long long count,
                const float* __restrict__ hist, OutT* __restrict__ out, size_t out_stride,
                float g_start, float g_step, int apply_gain, int soft_clip, int vec2, int nch) {
  constexpr int IT = 32 / RT;
  constexpr int halo = kPolyK - 1;
  extern __shared__ __align__(16) float smp[];
  const int U = F.poly_U;
  const int rows = kPolyOut / U;           // input indices per tile
  const int bt = F.boxcar;
  // shared: taps [kPolyK][U] (k-major, loaded once: the CTAs are persistent
  // and take tiles in turn), b[i0 - halo + t] for t < rows + halo, then the
  // PCM window behind it
  float* ts = smp;
  float* bw = ts + kPolyK * U;
  const int nb = rows + halo;
  float* pw = bw + nb;
  const int np = nb + (bt > 0 ? bt - 1 : 0);
  for (int t = threadIdx.x; t < kPolyK * U; t += blockDim.x) ts[t] = taps[t];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int per_rb = U / (8 * RT);        // warps across the branches of a row block
  const int rb = warp / per_rb, pb = warp - rb * per_rb;
  const int it = lane / RT, rt = lane - it * RT;
  const int row0 = rb * (8 * IT) + it * 8;   // local input index of q = 0
  // the thread's 8 branches: rb0 + 2 RT j + {0, 1}, j < 4, rb0 = block + 2 rt,
  // so that for each j the RT lanes of a row write one contiguous run
  const int rbase = pb * (8 * RT) + 2 * rt;
  const long long tiles = (count + rows - 1) / rows;

  for (long long wi = blockIdx.x; wi < tiles * nch; wi += gridDim.x) {
    const int ch = (int)(wi / tiles);
    const long long i0 = (wi - (long long)ch * tiles) * rows;
    const float* x = pcm + (size_t)ch * pcm_stride;
    const float* hx = hist + (size_t)ch * kHistory;
    const long long p0 = i0 - halo - (bt > 0 ? bt - 1 : 0);
    __syncthreads();                       // the previous tile's window is read
    for (int t = threadIdx.x; t < np; t += blockDim.x) {
      const long long i = p0 + t;
      float v = 0.0f;                      // beyond the block: read by no kept output
      if (i >= 0 && i < count) v = x[i];
      else if (i < 0 && i >= -kHistory) v = hx[kHistory + i];
      pw[t] = v;
    }
    __syncthreads();
    // boxcar: mean of the last `bt` samples, newest first
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
      float v;
      if (bt > 0) {
        float sum = 0.0f;
        for (int j = 0; j < bt; j++) sum += pw[t + bt - 1 - j];
        v = sum * F.inv_boxcar;
      } else {
        v = pw[t];
      }
      bw[t] = v;
    }
    __syncthreads();

    // acc[q][j] = outputs (row0 + q, branches rbase + 2 RT j + {0, 1}) as a
    // pair, accumulated with packed FP32 FMAs (two FMAs per instruction, each
    // rounded as a scalar fmaf)
    float2 acc[8][4];
#pragma unroll
    for (int q = 0; q < 8; q++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[q][j] = make_float2(0.0f, 0.0f);
    // b[row0 + q - k] = bb[q - k]; for the tap rows k0 .. k0 + 7 the window
    // w[m] = bb[m - 7 - k0] (m < 15) holds every input they need:
    // b[row0 + q - (k0 + kk)] = w[7 + q - kk] (each held twice, as a pair)
    const float* bb = bw + halo + row0;
    float2 w[15];
#pragma unroll
    for (int m = 0; m < 15; m++) {
      const float v = bb[m - 7];
      w[m] = make_float2(v, v);
    }
#pragma unroll 1
    for (int k0 = 0; k0 < kPolyK; k0 += 8) {
      if (k0 > 0) {
#pragma unroll
        for (int m = 14; m >= 8; m--) w[m] = w[m - 8];
#pragma unroll
        for (int m = 0; m < 8; m++) {
          const float v = bb[m - 7 - k0];
          w[m] = make_float2(v, v);
        }
      }
#pragma unroll
      for (int kk = 0; kk < 8; kk++) {
        const float* tr = ts + (k0 + kk) * U + rbase;
        float2 h[4];
#pragma unroll
        for (int j = 0; j < 4; j++) h[j] = *reinterpret_cast<const float2*>(tr + 2 * RT * j);
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const float2 xv = w[7 + q - kk];
#pragma unroll
          for (int j = 0; j < 4; j++) acc[q][j] = __ffma2_rn(h[j], xv, acc[q][j]);
        }
      }
    }

    // epilogue: the gain ramp in place, then the knee test: a tile whose
    // outputs all stay within the threshold (the usual case) takes the short
    // path, and the unrolled code with the inlined FP64 tanh runs only for a
    // warp where some output needs it
    const float gb = fmaf(g_step, (float)(i0 * U), g_start);
    bool over = false;
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int pq = (row0 + q) * U + rbase;   // offset from the tile's first output (< 2^23)
#pragma unroll
      for (int j = 0; j < 4; j++)
#pragma unroll
        for (int e = 0; e < 2; e++) {
          float& y = e ? acc[q][j].y : acc[q][j].x;
          if (apply_gain) y *= fmaf(g_step, small_to_float(pq + 2 * RT * j + e), gb);
          over |= fabsf(y) > 0.95f;
        }
    }
    over = soft_clip && __any_sync(0xffffffffu, over);
    OutT* dst = out + (size_t)ch * out_stride;
    if (!over) {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const long long i = i0 + row0 + q;
        if (i >= count) break;
        OutT* d = dst + (size_t)i * U + rbase;
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const OutT y0 = fir_finish<OutT>(acc[q][j].x, false);
          const OutT y1 = fir_finish<OutT>(acc[q][j].y, false);
          if (vec2) {
            typename Pair2<OutT>::type v;
            v.x = y0;
            v.y = y1;
            *reinterpret_cast<typename Pair2<OutT>::type*>(d + 2 * RT * j) = v;
          } else {
            d[2 * RT * j] = y0;
            d[2 * RT * j + 1] = y1;
          }
        }
      }
    } else {
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const long long i = i0 + row0 + q;
        if (i >= count) break;
        OutT* d = dst + (size_t)i * U + rbase;
#pragma unroll
        for (int j = 0; j < 4; j++) {
          const float a = acc[q][j].x, b = acc[q][j].y;
          const OutT y0 = fir_finish<OutT>(a, fabsf(a) > 0.95f);
          const OutT y1 = fir_finish<OutT>(b, fabsf(b) > 0.95f);
          if (vec2) {
            typename Pair2<OutT>::type v;
            v.x = y0;
            v.y = y1;
            *reinterpret_cast<typename Pair2<OutT>::type*>(d + 2 * RT * j) = v;
          } else {
            d[2 * RT * j] = y0;
            d[2 * RT * j + 1] = y1;
          }
        }
      }
    }
  }
}

// Keep the last kHistory PCM samples of this block (for the next one).
__global__ void fir_history_kernel(const float* __restrict__ pcm, size_t pcm_stride,
                                   long long count, float* __restrict__ hist) {
  const int ch = blockIdx.x;
  float* h = hist + (size_t)ch * kHistory;
  const float* x = pcm + (size_t)ch * pcm_stride;
  // new history = last kHistory samples of (old history ++ block)
  __shared__ float tmp[kHistory];
  for (int j = threadIdx.x; j < kHistory; j += blockDim.x) {
    const long long src = count - kHistory + j;   // index into the block
    tmp[j] = src >= 0 ? x[src] : h[kHistory + src];
  }
  __syncthreads();
  for (int j = threadIdx.x; j < kHistory; j += blockDim.x) h[j] = tmp[j];
}

// FP64 design of the reference's half-band / quarter-band taps (src/fir.c:65-121).
double bessel_i0(double x) {
  double sum = 1.0, term = 1.0;
  const double q = (x / 2.0) * (x / 2.0);
  for (int k = 1; k <= 25; k++) {
    term *= q / ((double)k * (double)k);
    sum += term;
    if (term < 1e-20 * sum) break;
  }
  return sum;
}

void design_taps(int ntaps, bool quarter, double* h) {
  const int c = (ntaps - 1) / 2;
  const double beta = 12.0, pi = 3.14159265358979323846;
  const double i0b = bessel_i0(beta);
  double sum = 0.0;
  for (int n = 0; n < ntaps; n++) {
    const double x = quarter ? (double)(n - c) * 0.25 : (double)(n - c) / 2.0;
    const double sinc = (std::fabs(x) < 1e-15) ? 1.0 : std::sin(pi * x) / (pi * x);
    const double t = (double)(n - c) / c;
    const double arg = 1.0 - t * t;
    const double w = bessel_i0(beta * std::sqrt(arg > 0.0 ? arg : 0.0)) / i0b;
    h[n] = quarter ? 0.25 * sinc * w : sinc * w;
    sum += h[n];
  }
  for (int n = 0; n < ntaps; n++) h[n] /= sum;
}

// Stage plan of fir_chain_init_ex for upsampling (src/fir.c:523-611, 131-150).
int plan_chain(unsigned fs_in, unsigned fs_out, int* U, int* L) {
  if (fs_in == 0 || fs_out < fs_in || fs_out % fs_in) return -1;
  const unsigned ratio = fs_out / fs_in;
  if (ratio & (ratio - 1)) return -1;
  int S = 0;
  for (unsigned r = ratio; r > 1; r >>= 1) S++;
  if (S > kMaxStages) return -1;
  const bool to512 = (fs_out == 22579200u || fs_out == 24576000u);
  if (ratio == 8 && to512) {
    U[0] = 4; L[0] = 127;
    U[1] = 2; L[1] = 63;
    return 2;
  }
  for (int i = 0; i < S; i++) {
    U[i] = 2;
    L[i] = (S >= 2 && i == 0 && to512) ? 127 : 63;
  }
  return S;
}

// The run of stages a chain merges into one polyphase stage: the 63-tap
// half-band 2x stages from k0 (0, or 1 behind the 127-tap first stage of the
// chains into DSD512), all but the last three, at most four (U <= 16) and at
// least three (a shorter run leaves too much zero padding).  Their cascade is
// one LTI filter: stage k maps y_k = h'_k * (up2 y_{k-1}), so the run is
// hm * (up 2^M y) with hm = h'_{M-1} * up2(h'_{M-2} * up2(... h'_0)), of length
// 1 + 62 (2^M - 1).  Its FP32 form differs from the stage-by-stage FP32
// cascade only in rounding (both within the chain's 1e-6 of the FP64
// restatement), and its branches keep every thread busy where those stages,
// 1/16 to 1/2 of a tile's width, left most of them idle at the barrier.
int merged_stages(int S, const int* U, const int* L, int* k0) {
  *k0 = (S > 0 && (U[0] != 2 || L[0] != 63)) ? 1 : 0;
  int M = S - *k0 - 3;
  if (M > 4) M = 4;
  if (M < 3) return 0;
  for (int k = *k0; k < *k0 + M; k++)
    if (U[k] != 2 || L[k] != 63) return 0;
  return M;
}

// The combined impulse response of M cascaded 63-tap half-band 2x stages
// (h'_k = 2 h_k): hm = h'_{M-1} * up2(h'_{M-2} * up2(... h'_0)), in FP64.
static std::vector<double> cascade_response(int M) {
  std::vector<double> g(63), t;
  design_taps(63, false, g.data());
  for (double& v : g) v *= 2.0;
  double h[63];
  design_taps(63, false, h);
  for (int k = 1; k < M; k++) {
    const size_t n = 2 * (g.size() - 1) + 1;     // up2(g)
    t.assign(n + 62, 0.0);
    for (size_t a = 0; a < g.size(); a++)
      for (int b = 0; b < 63; b++) t[2 * a + (size_t)b] += g[a] * (2.0 * h[b]);
    g.swap(t);
  }
  return g;
}

// The chains run whole as one polyphase stage: five to eight 63-tap
// half-band 2x stages (factor 32 to 256, at most 62 taps per branch).
static int whole_chain_factor(int S, const int* U, const int* L) {
  if (S < 5 || S > 8) return 0;
  for (int k = 0; k < S; k++)
    if (U[k] != 2 || L[k] != 63) return 0;
  return 1 << S;
}

// Branch taps of the whole-chain stage of factor U, k-major: t[k * U + r] =
// hm[U * k + r] as FP32 (zero past the response).
static std::vector<float> whole_chain_taps(int U) {
  int S = 0;
  for (int u = U; u > 1; u >>= 1) S++;
  const std::vector<double> g = cascade_response(S);
  std::vector<float> t((size_t)kPolyK * U, 0.0f);
  for (int k = 0; k < kPolyK; k++)
    for (int r = 0; r < U; r++) {
      const size_t tap = (size_t)U * k + r;
      if (tap < g.size()) t[(size_t)k * U + r] = (float)g[tap];
    }
  return t;
}

int build_chain_const(unsigned fs_in, unsigned fs_out, int boxcar, FirChainConst* F) {
  memset(F, 0, sizeof *F);
  int U[kMaxStages], L[kMaxStages];
  const int S0 = plan_chain(fs_in, fs_out, U, L);
  if (S0 < 0) return -1;
  int U0[kMaxStages], L0[kMaxStages];
  for (int k = 0; k < S0; k++) {
    U0[k] = U[k];
    L0[k] = L[k];
  }
  int k0 = 0;
  const int M = merged_stages(S0, U, L, &k0);
  F->S = M ? S0 - M + 1 : S0;
  F->ratio = (int)(fs_out / fs_in);
  F->boxcar = boxcar;
  F->inv_boxcar = boxcar > 0 ? (float)(1.0 / boxcar) : 1.0f;
  int toff = 0;
  if (M) {
    // the merged stage's taps first (offset 0: the kernel addresses them
    // as constants), branch r at r * kPolyTaps
    const std::vector<double> g = cascade_response(M);
    const int Um = 1 << M;
    if ((int)g.size() > Um * kPolyTaps || Um * kPolyTaps > kMaxChainTaps) return -1;
    F->U[k0] = Um;
    F->L[k0] = Um * kPolyTaps;
    F->poly_stage[k0] = 1;
    for (int r = 0; r < Um; r++) {
      F->phase_off[k0][r] = r * kPolyTaps;
      F->nphase[k0][r] = kPolyTaps;
      for (int j = 0; j < kPolyTaps; j++) {
        const size_t tap = (size_t)Um * j + r;
        F->taps[r * kPolyTaps + j] = tap < g.size() ? (float)g[tap] : 0.0f;
        F->lag[r * kPolyTaps + j] = j;
      }
    }
    toff = Um * kPolyTaps;
    // the stages behind the run move up to follow the merged one
    for (int k = k0 + M; k < S0; k++) {
      U[k - M + 1] = U[k];
      L[k - M + 1] = L[k];
    }
  }
  const int S = F->S;
  for (int k = 0; k < S; k++) {
    if (F->poly_stage[k]) continue;
    F->U[k] = U[k];
    F->L[k] = L[k];
    double h[255];
    design_taps(L[k], U[k] == 4, h);
    for (int r = 0; r < U[k]; r++) {
      F->phase_off[k][r] = toff;
      int n = 0;
      for (int j = 0; U[k] * j + r < L[k]; j++) {
        const int tap = U[k] * j + r;
        const double hv = h[tap] * (double)U[k];
        if (std::fabs(hv) < 1e-12) continue;     // half-band zero taps
        if (toff + n >= kMaxChainTaps) return -1;
        F->taps[toff + n] = (float)hv;
        F->lag[toff + n] = j;
        n++;
      }
      F->nphase[k][r] = n;
      toff += n;
    }
    if (U[k] == 2 && L[k] == 63 && F->nphase[k][0] == 32 && F->nphase[k][1] == 1) {
      F->hb_stage[k] = 1;
      for (int t = 0; t < 32; t++) F->hb[t] = F->taps[F->phase_off[k][0] + t];
      F->hb_center = F->taps[F->phase_off[k][1]];
    }
  }
  // output tile: 8,192 final samples per CTA (measured on the 10 s DSD128 stereo
  // chain: 4,096 / 6,144 / 8,192 / 12,288 / 16,384 ran 1.03 / 0.83 / 0.75 / 0.84 / 1.26 ms;
  // 256 threads with at least 2 CTAs per SM; 3 fit by registers and shared memory)
  F->tile = 8192;
  F->poly_U = whole_chain_factor(S0, U0, L0);
  if (F->poly_U) F->tile = kPolyOut;
  return 0;
}

size_t chain_smem_bytes(const FirChainConst& F) {
  if (F.poly_U) {
    // taps [kPolyK][U], the boxcar output with its halo, the PCM window
    const size_t rows = (size_t)(kPolyOut / F.poly_U);
    const size_t nb = rows + kPolyK - 1;
    return ((size_t)kPolyK * F.poly_U + nb + nb + (F.boxcar > 0 ? F.boxcar - 1 : 0) + 16) *
           sizeof(float);
  }
  // worst-case extents of every signal for a tile, plus the PCM window
  long long lo[kMaxStages + 1], hi[kMaxStages + 1];
  size_t best = 0;
  for (int phase = 0; phase < 4; phase++) {
    lo[F.S] = (long long)phase * F.tile + 1000003LL * F.ratio;   // a generic offset
    hi[F.S] = lo[F.S] + F.tile;
    for (int k = F.S - 1; k >= 0; k--) {
      auto fd = [](long long a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); };
      lo[k] = fd(lo[k + 1] - (F.L[k] - 1), F.U[k]);
      hi[k] = fd(hi[k + 1] - 1, F.U[k]) + 1;
    }
    size_t tot = (size_t)(hi[0] - lo[0] + (F.boxcar > 0 ? F.boxcar - 1 : 0));
    for (int k = 0; k < F.S; k++) tot += (size_t)(hi[k] - lo[k]);
    tot = ((tot + 3) & ~(size_t)3) + (size_t)F.tile;   // the final tile
    if (tot > best) best = tot;
  }
  return (best + 16) * sizeof(float);
}

// Device copies of the whole-chain taps (factor 32, 64, 128, 256), per
// device, made by fir_chain_prepare (outside any stream capture).
constexpr int kWholeFactors = 4;
static float* g_whole_taps[64][kWholeFactors] = {};

static const float* whole_taps_device(int dev, int U) {
  const int slot = U == 32 ? 0 : (U == 64 ? 1 : (U == 128 ? 2 : (U == 256 ? 3 : -1)));
  return (slot < 0 || dev < 0 || dev >= 64) ? nullptr : g_whole_taps[dev][slot];
}

int fir_chain_prepare() {
  // the shared-memory opt-in is a per-device function attribute
  static bool attr_set[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return -1;
  if (!g_whole_taps[dev][0]) {
    for (int slot = 0; slot < kWholeFactors; slot++) {
      const int U = 32 << slot;
      const std::vector<float> t = whole_chain_taps(U);
      float* d = nullptr;
      if (cudaMalloc(&d, sizeof(float) * t.size()) != cudaSuccess) return -1;
      if (cudaMemcpy(d, t.data(), sizeof(float) * t.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(d);
        return -1;
      }
      g_whole_taps[dev][slot] = d;
    }
  }
  if (!attr_set[dev]) {
    if (cudaFuncSetAttribute(fir_chain_kernel<double>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, kFirMaxSmem) != cudaSuccess ||
        cudaFuncSetAttribute(fir_chain_kernel<double>,
                             cudaFuncAttributePreferredSharedMemoryCarveout, 100) != cudaSuccess ||
        cudaFuncSetAttribute(fir_chain_kernel<float>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, kFirMaxSmem) != cudaSuccess ||
        cudaFuncSetAttribute(fir_chain_kernel<float>,
                             cudaFuncAttributePreferredSharedMemoryCarveout, 100) != cudaSuccess ||
        cudaFuncSetAttribute(fir_poly_kernel<8, double>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, kFirMaxSmem) != cudaSuccess ||
        cudaFuncSetAttribute(fir_poly_kernel<8, float>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, kFirMaxSmem) != cudaSuccess ||
        cudaFuncSetAttribute(fir_poly_kernel<4, double>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, kFirMaxSmem) != cudaSuccess ||
        cudaFuncSetAttribute(fir_poly_kernel<4, float>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, kFirMaxSmem) != cudaSuccess)
      return -1;
    attr_set[dev] = true;
  }
  return 0;
}

template <typename OutT>
static int launch_fir_chain_t(const FirChainConst& F, size_t smem, const float* pcm,
                              size_t pcm_stride, long long count, const float* hist, OutT* out,
                              size_t out_stride, double g_start, double g_step, int apply_gain,
                              int soft_clip, int nch, cudaStream_t stream) {
  const long long n_out = count * (long long)F.ratio;
  if (n_out <= 0) return 0;
  if (fir_chain_prepare() != 0) return -1;
  if (smem > (size_t)kFirMaxSmem) return -1;
  const dim3 grid((unsigned)((n_out + F.tile - 1) / F.tile), (unsigned)nch);
  // pair stores (16 bytes of doubles, 8 of floats): tiles start at even
  // outputs, so the rows and the base have to be aligned to a pair
  const int vec2 = ((reinterpret_cast<uintptr_t>(out) & (2 * sizeof(OutT) - 1)) == 0 &&
                    (out_stride & 1) == 0 && (F.tile & 1) == 0) ? 1 : 0;
  if (F.poly_U) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const float* taps = whole_taps_device(dev, F.poly_U);
    if (!taps) return -1;
    // persistent CTAs, two per SM (the register bound), taking tiles in turn
    const long long work = (long long)grid.x * nch;
    const unsigned ctas = (unsigned)std::min<long long>(work, 2ll * (sms > 0 ? sms : 148));
    if (F.poly_U == 32)
      fir_poly_kernel<4, OutT><<<ctas, kFirThreads, smem, stream>>>(
          F, taps, pcm, pcm_stride, count, hist, out, out_stride, (float)g_start, (float)g_step,
          apply_gain, soft_clip, vec2, nch);
    else
      fir_poly_kernel<8, OutT><<<ctas, kFirThreads, smem, stream>>>(
          F, taps, pcm, pcm_stride, count, hist, out, out_stride, (float)g_start, (float)g_step,
          apply_gain, soft_clip, vec2, nch);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
  }
  fir_chain_kernel<OutT><<<grid, kFirThreads, smem, stream>>>(F, pcm, pcm_stride, count, hist,
                                                              out, out_stride, (float)g_start,
                                                              (float)g_step, apply_gain,
                                                              soft_clip, vec2);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_fir_chain(const FirChainConst& F, size_t smem, const float* pcm, size_t pcm_stride,
                     long long count, const float* hist, double* out, size_t out_stride,
                     double g_start, double g_step, int apply_gain, int soft_clip, int nch,
                     cudaStream_t stream) {
  return launch_fir_chain_t(F, smem, pcm, pcm_stride, count, hist, out, out_stride, g_start,
                            g_step, apply_gain, soft_clip, nch, stream);
}

int launch_fir_chain(const FirChainConst& F, size_t smem, const float* pcm, size_t pcm_stride,
                     long long count, const float* hist, float* out, size_t out_stride,
                     double g_start, double g_step, int apply_gain, int soft_clip, int nch,
                     cudaStream_t stream) {
  return launch_fir_chain_t(F, smem, pcm, pcm_stride, count, hist, out, out_stride, g_start,
                            g_step, apply_gain, soft_clip, nch, stream);
}

int launch_fir_history(const float* pcm, size_t pcm_stride, long long count, float* hist, int nch,
                       cudaStream_t stream) {
  fir_history_kernel<<<nch, 128, 0, stream>>>(pcm, pcm_stride, count, hist);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace dsdgpu

using namespace dsdgpu;

extern "C" {

int dsdgpu_fir_setup(dsdgpu_context_t* c, const dsdgpu_fir_params_t* p, int num_channels) {
  if (!c || !p || num_channels < 1) return DSDGPU_ERR_ARG;
  if (p->boxcar_taps < 0 || p->boxcar_taps > 64) return c->fail(DSDGPU_ERR_ARG, "boxcar taps out of range");
  cudaSetDevice(c->device);
  FirChainConst F;
  if (build_chain_const(p->fs_in, p->fs_out, p->boxcar_taps, &F) != 0)
    return c->fail(DSDGPU_ERR_ARG, "unsupported rate pair (upsampling by a power of two only)");
  if (c->d_fir_hist) cudaFree(c->d_fir_hist);
  c->d_fir_hist = nullptr;
  cudaError_t e = cudaMalloc(&c->d_fir_hist, sizeof(float) * kHistory * (size_t)num_channels);
  if (e != cudaSuccess) return c->cuda_fail(e, "fir history allocation");
  cudaMemsetAsync(c->d_fir_hist, 0, sizeof(float) * kHistory * (size_t)num_channels, c->stream);
  c->fir = F;
  c->fir_params = *p;
  c->fir_channels = num_channels;
  c->fir_smem = chain_smem_bytes(F);
  if (c->fir_smem > (size_t)kFirMaxSmem) return c->fail(DSDGPU_ERR_UNSUPPORTED, "fir tile does not fit shared memory");
  c->fir_ready = true;
  return c->check_status();
}

int dsdgpu_fir_reset(dsdgpu_context_t* c) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->fir_ready) return c->fail(DSDGPU_ERR_STATE, "fir not set up");
  cudaSetDevice(c->device);
  cudaMemsetAsync(c->d_fir_hist, 0, sizeof(float) * kHistory * (size_t)c->fir_channels, c->stream);
  return c->check_status();
}

}  // extern "C"

namespace dsdgpu {

// dsdgpu_fir_process_async for either output type (FP64 for the trellis SDM,
// FP32 for the pipeline's PreCorr mode)
template <typename OutT>
int fir_process_async_t(dsdgpu_context_t* c, int first, int nch, const float* d_in,
                        size_t in_stride, size_t count, OutT* d_out, size_t out_stride,
                        double gain_start, double gain_end, size_t* out_count) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->fir_ready) return c->fail(DSDGPU_ERR_STATE, "fir not set up");
  if (first < 0 || nch < 1 || first + nch > c->fir_channels) return c->fail(DSDGPU_ERR_ARG, "bad channel range");
  const size_t n_out = count * (size_t)c->fir.ratio;
  if (out_count) *out_count = n_out;
  if (count == 0) return DSDGPU_OK;
  if (!d_in || !d_out) return c->fail(DSDGPU_ERR_ARG, "null buffer");
  if (out_stride < n_out) return c->fail(DSDGPU_ERR_ARG, "output stride too small");
  cudaSetDevice(c->device);
  // gain ramp of engine_process_block (src/engine.c:609-651)
  double gs = gain_start, ge = gain_end;
  if (gs == 0.0) gs = ge;
  const int apply = (gs != 1.0 || ge != 1.0) ? 1 : 0;
  const double step = (n_out > 1) ? (ge - gs) / (double)(n_out - 1) : 0.0;
  float* hist = c->d_fir_hist + (size_t)first * kHistory;
  if (launch_fir_chain(c->fir, c->fir_smem, d_in, in_stride, (long long)count, hist, d_out,
                       out_stride, gs, step, apply, c->fir_params.soft_clip, nch, c->stream) != 0)
    return c->cuda_fail(cudaGetLastError(), "fir launch");
  c->launches++;
  if (launch_fir_history(d_in, in_stride, (long long)count, hist, nch, c->stream) != 0)
    return c->cuda_fail(cudaGetLastError(), "fir history launch");
  c->launches++;
  return DSDGPU_OK;
}

}  // namespace dsdgpu

int fir_process_async_f32(dsdgpu_context* c, int nch, const float* d_in, size_t in_stride,
                          size_t count, float* d_out, size_t out_stride, double gain_start,
                          double gain_end, size_t* out_count) {
  return dsdgpu::fir_process_async_t(c, 0, nch, d_in, in_stride, count, d_out, out_stride,
                                     gain_start, gain_end, out_count);
}

extern "C" {

int dsdgpu_fir_process_async(dsdgpu_context_t* c, int first, int nch, const float* d_in,
                             size_t in_stride, size_t count, double* d_out, size_t out_stride,
                             double gain_start, double gain_end, size_t* out_count) {
  return dsdgpu::fir_process_async_t(c, first, nch, d_in, in_stride, count, d_out, out_stride,
                                     gain_start, gain_end, out_count);
}

int dsdgpu_fir_process(dsdgpu_context_t* c, int first, int nch, const float* d_in,
                       size_t in_stride, size_t count, double* d_out, size_t out_stride,
                       double gain_start, double gain_end, size_t* out_count) {
  int rc = dsdgpu_fir_process_async(c, first, nch, d_in, in_stride, count, d_out, out_stride,
                                    gain_start, gain_end, out_count);
  if (rc) return rc;
  return c->check_status();
}

}  // extern "C"
