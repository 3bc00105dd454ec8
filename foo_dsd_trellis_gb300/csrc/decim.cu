// DSD -> PCM decimation on sm_103a: the reference's FIR-only engine branch
// (src/engine.c:566-577; chain src/fir.c:523-611 with 63-tap half-band /2
// stages, ipp_downsample_d src/fir.c:467-487; gain ramp src/engine.c:879-889).
//
// Every stage is one launch, FP64, y[m] = sum_k h[k] x[2m - k] (the delay
// line of the previous call stands in for negative indices), followed by a
// small launch that keeps the stage's last 62 consumed inputs.  A stage
// consumes floor(count / 2) * 2 inputs, as the reference's numIters =
// in_count / factor.  IPP's summation order and use of FMA are not known, so
// the stages take the cheapest exact-enough form:
//   * the 63-tap half-band's taps at odd k other than the centre are the
//     design's zeros (|h| < 2e-17: they move an output by ~1e-17 of full scale), so
//     only the 32 even taps and the centre tap are applied;
//   * FP64 stages: those 33 taps as FMAs in ascending tap order;
//   * the first stage reads +-1 decisions: the 32 even taps form 4 groups of
//     8, each group's sum for every pattern of its 8 decisions is a table
//     entry (4 x 256 FP64 values, sums in tap order), so an output is 4 table
//     reads, the centre tap's +-h[31] and 4 adds.
// The result differs from a tap-order sum of separately rounded products by
// a few FP64 ulps (float32 output within 2e-7 of full scale).
#include "api_context.h"
#include "fir_internal.h"

#include <cstring>

using namespace dsdgpu;

namespace {

constexpr int kDecTaps = 63;

struct DecTaps {
  double h[kDecTaps];
};

// nonzero taps: even k and the centre
constexpr int kNzTaps = 33;
struct DecNz {
  double h[kNzTaps];
  int k[kNzTaps];
};

constexpr int kLutGroups = 4;   // 32 even taps in groups of 8

// FP64 stage: the 33 nonzero taps as FMAs in ascending tap order
__global__ void decim_stage_kernel(const __grid_constant__ DecNz T, const double* __restrict__ in,
                                   size_t in_stride, long long m_out,
                                   const double* __restrict__ dly, double* __restrict__ out,
                                   size_t out_stride, int nch) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m_out * nch) return;
  const long long c = i / m_out, m = i % m_out;
  const double* dl = dly + (size_t)c * (kDecTaps - 1);
  const double* xc = in + (size_t)c * in_stride;
  double acc = 0.0;
#pragma unroll
  for (int q = 0; q < kNzTaps; q++) {
    const long long j = 2 * m - T.k[q];
    const double x = j >= 0 ? xc[j] : dl[kDecTaps - 1 + j];
    acc = __fma_rn(T.h[q], x, acc);
  }
  out[(size_t)c * out_stride + m] = acc;
}

// first stage, decision bytes in: 4 group-table reads + the centre tap
__global__ void __launch_bounds__(256) decim_bits_kernel(const __grid_constant__ DecNz T,
                                                         const double* __restrict__ lut, double h31,
                                                         const uint8_t* __restrict__ bits,
                                                         size_t in_stride, long long m_out,
                                                         const double* __restrict__ dly,
                                                         double* __restrict__ out,
                                                         size_t out_stride, int nch) {
  __shared__ double tab[kLutGroups * 256];
  for (int q = threadIdx.x; q < kLutGroups * 256; q += blockDim.x) tab[q] = lut[q];
  __syncthreads();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m_out * nch) return;
  const long long c = i / m_out, m = i % m_out;
  const double* dl = dly + (size_t)c * (kDecTaps - 1);
  const uint8_t* bc = bits + (size_t)c * in_stride;
  double acc = 0.0;
  if (2 * m < kDecTaps - 1) {
    // the window reaches the delay line, whose values are zero before the
    // first call: the 33 taps directly
#pragma unroll
    for (int q = 0; q < kNzTaps; q++) {
      const long long j = 2 * m - T.k[q];
      const double x = j >= 0 ? (bc[j] & 1u ? 1.0 : -1.0) : dl[kDecTaps - 1 + j];
      acc = __fma_rn(T.h[q], x, acc);
    }
  } else {
#pragma unroll
    for (int g = 0; g < kLutGroups; g++) {
      unsigned p = 0;
#pragma unroll
      for (int u = 0; u < 8; u++) p |= (unsigned)(bc[2 * m - 16 * g - 2 * u] & 1u) << u;
      acc = __dadd_rn(acc, tab[g * 256 + p]);
    }
    acc = __dadd_rn(acc, (bc[2 * m - 31] & 1u) ? h31 : -h31);
  }
  out[(size_t)c * out_stride + m] = acc;
}

// delay line <- the last 62 consumed inputs of (delay line ++ stage input)
template <bool kBits>
__global__ void decim_dly_kernel(const uint8_t* __restrict__ bits, const double* __restrict__ in,
                                 size_t in_stride, long long used, double* __restrict__ dly,
                                 int nch) {
  const int c = blockIdx.x;
  if (c >= nch) return;
  __shared__ double tmp[kDecTaps - 1];
  double* dl = dly + (size_t)c * (kDecTaps - 1);
  for (int k = threadIdx.x; k < kDecTaps - 1; k += blockDim.x) {
    const long long j = used - (kDecTaps - 1) + k;
    double v;
    if (j >= 0) v = kBits ? (bits[(size_t)c * in_stride + j] ? 1.0 : -1.0) : in[(size_t)c * in_stride + j];
    else v = dl[kDecTaps - 1 + j];
    tmp[k] = v;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kDecTaps - 1; k += blockDim.x) dl[k] = tmp[k];
}

__global__ void decim_gain_kernel(const double* __restrict__ y, size_t y_stride, long long n,
                                  int nch, double g_start, double g_step, int apply,
                                  float* __restrict__ out, size_t out_stride) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * nch) return;
  const long long c = i / n, t = i % n;
  double v = y[(size_t)c * y_stride + t];
  if (apply) v = __dmul_rn(v, __dadd_rn(g_start, __dmul_rn(g_step, (double)t)));
  out[(size_t)c * out_stride + t] = (float)v;
}

// FP64 output of the rate-conversion branch (src/engine.c:640-717): gain ramp
// (when either end differs from 1), then the optional soft clip
__global__ void decim_gain_f64_kernel(const double* __restrict__ y, size_t y_stride, long long n,
                                      int nch, double g_start, double g_step, int apply,
                                      int soft_clip, double* __restrict__ out, size_t out_stride) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * nch) return;
  const long long c = i / n, t = i % n;
  double v = y[(size_t)c * y_stride + t];
  if (apply) v = __dmul_rn(v, __dadd_rn(g_start, __dmul_rn(g_step, (double)t)));
  if (soft_clip) v = soft_clip_095(v);
  out[(size_t)c * out_stride + t] = v;
}

unsigned nb(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

struct dsdgpu_decim_state {
  int stages = 0;
  int nch = 0;
  DecTaps taps{};
  DecNz nz{};
  double* d_lut = nullptr;      // [group][pattern] sums of the first stage
  double* d_dly = nullptr;      // [stage][nch][62]
  double* d_buf = nullptr;      // ping-pong [2][nch][row]
  size_t row = 0;
  ~dsdgpu_decim_state() {
    if (d_lut) cudaFree(d_lut);
    if (d_dly) cudaFree(d_dly);
    if (d_buf) cudaFree(d_buf);
  }
};

void decim_free(dsdgpu_decim_state* s) { delete s; }

// The FP64 chain from fresh state without a context (the batch plan's DSD
// input to a lower rate): `stages` 63-tap half-band /2 stages over `count`
// inputs through the ping-pong rows of `buf` (2 x nch rows of `row` doubles,
// row >= count / 2 + 1), with the zero delay lines `zero_dly` (nch x 62
// zeros, read only: a fresh stream has nothing before its first sample), then
// gain and the optional soft clip into `out`.  *out_count = count >> stages.
// out32 non-null: FP32 output instead (the gain, no clip, narrowed to
// nearest: the PreCorr walk's input), `out` unused.
int launch_decim_f64_fresh(const double* in, size_t in_stride, long long count, int stages,
                           int nch, double* buf, size_t row, const double* zero_dly,
                           double g_start, double g_step, int apply, int soft_clip, double* out,
                           size_t out_stride, cudaStream_t st, float* out32) {
  if (count < 2 || stages < 1) return 0;
  DecTaps taps{};
  DecNz nz{};
  design_taps(kDecTaps, false, taps.h);
  for (int q = 0, k = 0; k < kDecTaps; k++)
    if ((k & 1) == 0 || k == kDecTaps / 2) { nz.h[q] = taps.h[k]; nz.k[q] = k; q++; }
  double* pp[2] = {buf, buf + row * (size_t)nch};
  long long cur = count;
  const double* x = in;
  size_t xs = in_stride;
  for (int k = 0; k < stages; k++) {
    const long long m = cur / 2;
    if (m > 0)
      decim_stage_kernel<<<nb(m * nch, 256), 256, 0, st>>>(nz, x, xs, m, zero_dly, pp[k & 1], row,
                                                           nch);
    x = pp[k & 1];
    xs = row;
    cur = m;
  }
  if (cur > 0 && out32)
    decim_gain_kernel<<<nb(cur * nch, 256), 256, 0, st>>>(x, xs, cur, nch, g_start, g_step, apply,
                                                          out32, out_stride);
  else if (cur > 0)
    decim_gain_f64_kernel<<<nb(cur * nch, 256), 256, 0, st>>>(x, xs, cur, nch, g_start, g_step,
                                                              apply, soft_clip ? 1 : 0, out,
                                                              out_stride);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

extern "C" {

int dsdgpu_decim_setup(dsdgpu_context_t* c, unsigned fs_in, unsigned fs_out, int nch) {
  if (!c || nch < 1) return DSDGPU_ERR_ARG;
  if (fs_out == 0 || fs_in <= fs_out || fs_in % fs_out) return c->fail(DSDGPU_ERR_ARG, "decimation needs fs_in = fs_out * 2^k");
  unsigned r = fs_in / fs_out;
  if (r & (r - 1)) return c->fail(DSDGPU_ERR_ARG, "decimation ratio must be a power of two");
  int S = 0;
  while (r > 1) { S++; r >>= 1; }
  if (S > kMaxStages) return c->fail(DSDGPU_ERR_ARG, "too many stages");
  cudaSetDevice(c->device);
  dsdgpu_decim_state* s = new (std::nothrow) dsdgpu_decim_state();
  if (!s) return DSDGPU_ERR_NOMEM;
  s->stages = S;
  s->nch = nch;
  design_taps(kDecTaps, false, s->taps.h);
  for (int q = 0, k = 0; k < kDecTaps; k++)
    if ((k & 1) == 0 || k == kDecTaps / 2) { s->nz.h[q] = s->taps.h[k]; s->nz.k[q] = k; q++; }
  // group g, pattern p: sum over u = 0..7 of h[16 g + 2 u] * (bit u of p ? 1 : -1)
  double lut[kLutGroups * 256];
  for (int g = 0; g < kLutGroups; g++)
    for (int p = 0; p < 256; p++) {
      double acc = 0.0;
      for (int u = 0; u < 8; u++) {
        const double h = s->taps.h[16 * g + 2 * u];
        acc += ((p >> u) & 1) ? h : -h;
      }
      lut[g * 256 + p] = acc;
    }
  const size_t dbytes = sizeof(double) * (size_t)S * nch * (kDecTaps - 1);
  if (cudaMalloc(&s->d_dly, dbytes) != cudaSuccess || cudaMalloc(&s->d_lut, sizeof lut) != cudaSuccess) {
    delete s;
    return c->cuda_fail(cudaGetLastError(), "decimation buffers");
  }
  cudaMemcpyAsync(s->d_lut, lut, sizeof lut, cudaMemcpyHostToDevice, c->stream);
  cudaMemsetAsync(s->d_dly, 0, dbytes, c->stream);
  decim_free(c->decim);
  c->decim = s;
  return c->check_status();
}

int dsdgpu_decim_reset(dsdgpu_context_t* c) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->decim) return c->fail(DSDGPU_ERR_STATE, "decimation not set up");
  cudaSetDevice(c->device);
  dsdgpu_decim_state* s = c->decim;
  cudaMemsetAsync(s->d_dly, 0, sizeof(double) * (size_t)s->stages * s->nch * (kDecTaps - 1), c->stream);
  return c->check_status();
}

int dsdgpu_decim_process_async(dsdgpu_context_t* c, int nch, const uint8_t* d_bits,
                               size_t bits_stride, size_t count, float* d_pcm, size_t pcm_stride,
                               double gain_start, double gain_end, size_t* out_count) {
  if (!c) return DSDGPU_ERR_ARG;
  dsdgpu_decim_state* s = c->decim;
  if (!s) return c->fail(DSDGPU_ERR_STATE, "decimation not set up");
  if (nch != s->nch) return c->fail(DSDGPU_ERR_ARG, "channel count differs from the setup");
  size_t n = count;
  for (int k = 0; k < s->stages; k++) n /= 2;
  if (out_count) *out_count = n;
  if (count < 2) return DSDGPU_OK;
  if (!d_bits || !d_pcm) return c->fail(DSDGPU_ERR_ARG, "null buffer");
  if (pcm_stride < n) return c->fail(DSDGPU_ERR_ARG, "output stride too small");
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  const size_t row = ((count / 2 + 1) + 31) & ~(size_t)31;
  if (s->row < row) {
    if (s->d_buf) cudaFree(s->d_buf);
    s->d_buf = nullptr;
    s->row = 0;
    if (cudaMalloc(&s->d_buf, sizeof(double) * 2 * row * (size_t)nch) != cudaSuccess)
      return c->cuda_fail(cudaGetLastError(), "decimation buffers");
    s->row = row;
  }
  double* buf[2] = {s->d_buf, s->d_buf + s->row * (size_t)nch};
  size_t cur = count;
  const double* in = nullptr;
  for (int k = 0; k < s->stages; k++) {
    const long long m = (long long)(cur / 2);
    double* out = buf[k & 1];
    double* dly = s->d_dly + (size_t)k * nch * (kDecTaps - 1);
    if (m > 0) {
      if (k == 0) {
        decim_bits_kernel<<<nb(m * nch, 256), 256, 0, st>>>(s->nz, s->d_lut, s->taps.h[kDecTaps / 2], d_bits,
                                                            bits_stride, m, dly, out, s->row, nch);
        decim_dly_kernel<true><<<nch, 64, 0, st>>>(d_bits, nullptr, bits_stride, 2 * m, dly, nch);
      } else {
        decim_stage_kernel<<<nb(m * nch, 256), 256, 0, st>>>(s->nz, in, s->row, m, dly, out, s->row,
                                                             nch);
        decim_dly_kernel<false><<<nch, 64, 0, st>>>(nullptr, in, s->row, 2 * m, dly, nch);
      }
      c->launches += 2;
    }
    in = out;
    cur = (size_t)m;
  }
  // gain ramp of engine_process_fir_gain (src/engine.c:879-889), then float
  double gs = gain_start;
  if (gs == 0.0) gs = gain_end;
  const int apply = (gs != 1.0 || gain_end != 1.0) ? 1 : 0;
  const double step = n > 1 ? (gain_end - gs) / (double)(n - 1) : 0.0;
  if (n > 0) {
    decim_gain_kernel<<<nb((long long)n * nch, 256), 256, 0, st>>>(in, s->row, (long long)n, nch, gs,
                                                                 step, apply, d_pcm, pcm_stride);
    c->launches++;
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? DSDGPU_OK : c->cuda_fail(e, "decimation launch");
}

int dsdgpu_decim_process_f64_async(dsdgpu_context_t* c, int nch, const double* d_in,
                                   size_t in_stride, size_t count, double* d_out,
                                   size_t out_stride, double gain_start, double gain_end,
                                   int soft_clip, size_t* out_count) {
  if (!c) return DSDGPU_ERR_ARG;
  dsdgpu_decim_state* s = c->decim;
  if (!s) return c->fail(DSDGPU_ERR_STATE, "decimation not set up");
  if (nch != s->nch) return c->fail(DSDGPU_ERR_ARG, "channel count differs from the setup");
  size_t n = count;
  for (int k = 0; k < s->stages; k++) n /= 2;
  if (out_count) *out_count = n;
  if (count < 2) return DSDGPU_OK;
  if (!d_in || !d_out) return c->fail(DSDGPU_ERR_ARG, "null buffer");
  if (nch > 1 && (in_stride < count || out_stride < n))
    return c->fail(DSDGPU_ERR_ARG, "row stride shorter than the count");
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  const size_t row = ((count / 2 + 1) + 31) & ~(size_t)31;
  if (s->row < row) {
    if (s->d_buf) cudaFree(s->d_buf);
    s->d_buf = nullptr;
    s->row = 0;
    if (cudaMalloc(&s->d_buf, sizeof(double) * 2 * row * (size_t)nch) != cudaSuccess)
      return c->cuda_fail(cudaGetLastError(), "decimation buffers");
    s->row = row;
  }
  double* buf[2] = {s->d_buf, s->d_buf + s->row * (size_t)nch};
  size_t cur = count;
  const double* in = d_in;
  size_t istride = in_stride;
  for (int k = 0; k < s->stages; k++) {
    const long long m = (long long)(cur / 2);
    double* out = buf[k & 1];
    double* dly = s->d_dly + (size_t)k * nch * (kDecTaps - 1);
    if (m > 0) {
      decim_stage_kernel<<<nb(m * nch, 256), 256, 0, st>>>(s->nz, in, istride, m, dly, out, s->row, nch);
      decim_dly_kernel<false><<<nch, 64, 0, st>>>(nullptr, in, istride, 2 * m, dly, nch);
      c->launches += 2;
    }
    in = out;
    istride = s->row;
    cur = (size_t)m;
  }
  // gain ramp of the rate-conversion branch (src/engine.c:646-651), soft clip (:704-717)
  double gs = gain_start;
  if (gs == 0.0) gs = gain_end;
  const int apply = (gs != 1.0 || gain_end != 1.0) ? 1 : 0;
  const double step = n > 1 ? (gain_end - gs) / (double)(n - 1) : 0.0;
  if (n > 0) {
    decim_gain_f64_kernel<<<nb((long long)n * nch, 256), 256, 0, st>>>(
        in, istride, (long long)n, nch, gs, step, apply, soft_clip ? 1 : 0, d_out, out_stride);
    c->launches++;
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? DSDGPU_OK : c->cuda_fail(e, "decimation launch");
}

int dsdgpu_decim_process_f64(dsdgpu_context_t* c, int nch, const double* d_in, size_t in_stride,
                             size_t count, double* d_out, size_t out_stride, double gain_start,
                             double gain_end, int soft_clip, size_t* out_count) {
  const int rc = dsdgpu_decim_process_f64_async(c, nch, d_in, in_stride, count, d_out, out_stride,
                                                gain_start, gain_end, soft_clip, out_count);
  return rc ? rc : c->check_status();
}

int dsdgpu_decim_process(dsdgpu_context_t* c, int nch, const uint8_t* d_bits, size_t bits_stride,
                         size_t count, float* d_pcm, size_t pcm_stride, double gain_start,
                         double gain_end, size_t* out_count) {
  const int rc = dsdgpu_decim_process_async(c, nch, d_bits, bits_stride, count, d_pcm, pcm_stride,
                                            gain_start, gain_end, out_count);
  return rc ? rc : c->check_status();
}

}  // extern "C"
