// Same-rate FIR lowpass on sm_103a: the engine's FIR_MODE_FIR alternative to
// the same-rate boxcar (reference src/engine.c:168-181, :505-523), i.e.
// fir_lowpass_init_ex / fir_lowpass_process (src/fir.c:795-872): a Kaiser
// (beta 10) windowed sinc, 127 taps at 50 kHz by default, FP64, applied to the
// +-1 decisions of the DSD input with its delay line carried across calls
// (zero at setup), then the engine's linear gain ramp.
//
// The inputs are +-1, so every product h[k] * x is exact and an output is a
// sum of +-h[k].  The taps are padded with zeros to W = 32 * ceil(ntaps / 32)
// and split into W / 8 groups of 8; for every group the sum of its taps under
// each of the 256 sign patterns is precomputed on the host (accumulated from
// 0.0 in tap order within the group), so an output is W / 8 table reads and
// W / 8 FP64 adds (16 at 127 taps) instead of 127.  IPP's summation order is
// closed; the order here (group j = taps W-1-8j .. W-8-8j, oldest sample
// first, groups added in j order) is the one the oracle restates.
//
//   lowpass_kernel        persistent CTAs of 256 threads, group tables in
//                         shared memory; a tile is 256 consecutive outputs
//                         of one channel, whose input window (the tile plus
//                         the 256 samples before it) is turned into bit words
//                         with warp ballots; each thread funnel-shifts its own
//                         W-bit window out of those words
//   lowpass_hist_kernel   keeps the last 256 decisions per channel as bits,
//                         with the count of samples seen (outputs whose window
//                         reaches before the first sample treat it as 0, the
//                         reference's zeroed delay line)
#include "api_context.h"
#include "fir_internal.h"

#include <cmath>
#include <cstring>
#include <vector>

using dsdgpu::bessel_i0;

namespace {

constexpr int kLpMaxTaps = 255;               // IPP_HB_NTAPS_MAX (include/fir.h:18)
constexpr int kLpTile = 256;                  // outputs per tile = threads per CTA
constexpr int kLpWords = (2 * kLpTile) / 32 + 1;   // tile + 256 history bits + 1 overread word
constexpr int kLpHistWords = 8;               // 256 history bits per channel

struct LpHist {
  uint32_t w[kLpHistWords];   // bit b of word q: sample -256 + 32q + b (relative to the next block)
  int32_t valid;              // samples seen so far, at most 256
  int32_t pad[3];
};

// fir_lowpass_init_ex's design (src/fir.c:795-825), its expression order kept
int design_lowpass(unsigned fs, double cutoff_hz, int ntaps, double* h) {
  if (ntaps < 3) ntaps = 3;
  if (ntaps > kLpMaxTaps) ntaps = kLpMaxTaps;
  if (ntaps % 2 == 0) ntaps++;
  double fc = cutoff_hz / ((double)fs / 2.0);
  if (fc > 0.5) fc = 0.5;
  const int M = ntaps - 1;
  const double kPi = 3.14159265358979323846;
  const double i0b = bessel_i0(10.0);
  for (int n = 0; n <= M; n++) {
    const double x = (double)n - (double)M / 2.0;
    const double s = (std::fabs(x) < 1e-10) ? 2.0 * fc : std::sin(2.0 * kPi * fc * x) / (kPi * x);
    const double t = 2.0 * n / M - 1.0;
    const double arg = 1.0 - t * t;
    h[n] = s * (bessel_i0(10.0 * std::sqrt(std::fabs(arg))) / i0b);
  }
  double sum = 0.0;
  for (int n = 0; n < ntaps; n++) sum += h[n];
  if (sum > 0.0)
    for (int n = 0; n < ntaps; n++) h[n] /= sum;
  return ntaps;
}

// bit v of a group's pattern is the sample at window position 8j + v, i.e.
// tap W-1-8j-v; a set bit is +1
void build_tables(const double* h, int ntaps, int W, double* tab) {
  for (int j = 0; j < W / 8; j++)
    for (int p = 0; p < 256; p++) {
      double g = 0.0;
      for (int v = 0; v < 8; v++) {
        const int k = W - 1 - 8 * j - v;
        if (k < ntaps) g += (p >> v & 1) ? h[k] : -h[k];
      }
      tab[j * 256 + p] = g;
    }
}

// sample p of the block (0/1), or of the history words hw for p in [-256, 0)
__device__ __forceinline__ uint32_t window_bit(const uint8_t* x, const uint32_t* hw, long long p,
                                               long long count) {
  if (p >= count) return 0u;
  if (p >= 0) return x[p] & 1u;
  const int q = (int)(p + 256);
  return hw[q >> 5] >> (q & 31) & 1u;
}

// OutT = float: the FP64 output narrowed to nearest (the PreCorr walk's input)
template <typename OutT>
__global__ void __launch_bounds__(kLpTile) lowpass_kernel(
    const double* __restrict__ lut, const double* __restrict__ taps, int ntaps, int W,
    const uint8_t* __restrict__ bits, size_t bits_stride, long long count,
    const LpHist* __restrict__ hist, int nch, double g_start, double g_step,
    OutT* __restrict__ out, size_t out_stride) {
  extern __shared__ double smem[];
  double* tab = smem;
  uint32_t* words = reinterpret_cast<uint32_t*>(smem + (W / 8) * 256);
  const int G = W / 8;
  for (int q = threadIdx.x; q < G * 256; q += blockDim.x) tab[q] = lut[q];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long tiles_per_ch = (count + kLpTile - 1) / kLpTile;
  const long long ntiles = tiles_per_ch * nch;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int c = (int)(tile / tiles_per_ch);
    const long long i0 = (tile % tiles_per_ch) * kLpTile;
    const uint8_t* x = bits + (size_t)c * bits_stride;
    const long long valid = hist[c].valid;
    __syncthreads();   // the previous tile's words are consumed (and the tables loaded)
    // word q holds samples i0 - 256 + 32q + b
    for (int q = warp; q < kLpWords; q += kLpTile / 32) {
      const uint32_t b = window_bit(x, hist[c].w, i0 - 256 + 32 * q + lane, count);
      const uint32_t wv = __ballot_sync(0xffffffffu, b);
      if (lane == 0) words[q] = wv;
    }
    __syncthreads();
    const long long i = i0 + threadIdx.x;
    if (i >= count) continue;
    // this output's window: samples i - W + 1 .. i, from bit o of the words
    const int o = (int)threadIdx.x + 257 - W;
    const int q0 = o >> 5, sh = o & 31;
    double acc = 0.0;
    if (i - W + 1 >= -valid) {
#pragma unroll 4
      for (int j4 = 0; j4 < G / 4; j4++) {
        const uint32_t v = __funnelshift_r(words[q0 + j4], words[q0 + j4 + 1], sh);
#pragma unroll
        for (int u = 0; u < 4; u++) acc = __dadd_rn(acc, tab[(4 * j4 + u) * 256 + (v >> (8 * u) & 0xffu)]);
      }
    } else {
      // the window reaches before the first sample (zero there): the
      // groups' sums in the tables' order with the unseen samples skipped
      for (int j = 0; j < G; j++) {
        double g = 0.0;
        for (int v = 0; v < 8; v++) {
          const int k = W - 1 - 8 * j - v;
          const long long p = i - k;
          if (k >= ntaps || p < -valid) continue;
          const int pos = o + 8 * j + v;
          const bool one = words[pos >> 5] >> (pos & 31) & 1u;
          g = __dadd_rn(g, one ? taps[k] : -taps[k]);
        }
        acc = __dadd_rn(acc, g);
      }
    }
    out[(size_t)c * out_stride + i] =
        (OutT)__dmul_rn(acc, __dadd_rn(g_start, __dmul_rn(g_step, (double)i)));
  }
}

// history <- the last 256 samples of (history ++ block); valid += count (cap 256)
__global__ void lowpass_hist_kernel(const uint8_t* __restrict__ bits, size_t bits_stride,
                                    long long count, LpHist* __restrict__ hist, int nch) {
  const int c = blockIdx.x;
  if (c >= nch) return;
  __shared__ uint32_t nw[kLpHistWords];
  const long long valid = hist[c].valid;
  const uint8_t* x = bits + (size_t)c * bits_stride;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;   // 256 threads: one word per warp
  const uint32_t b = window_bit(x, hist[c].w, count - 256 + 32 * warp + lane, count);
  const uint32_t wv = __ballot_sync(0xffffffffu, b);
  if (lane == 0) nw[warp] = wv;
  __syncthreads();
  if (threadIdx.x < kLpHistWords) hist[c].w[threadIdx.x] = nw[threadIdx.x];
  if (threadIdx.x == 0) {
    const long long v = valid + count;
    hist[c].valid = (int32_t)(v > 256 ? 256 : v);
  }
}

}  // namespace

// Context-free form (the batch plan's same-rate DSD streams, fresh state):
// the design and group tables on the host, the kernel with a zeroed history
// (valid = 0: every window starts at the stream's first sample).
int lowpass_tables(unsigned fs, double cutoff_hz, int ntaps_req, std::vector<double>& lut,
                   std::vector<double>& taps, int* W) {
  double h[kLpMaxTaps + 1];
  const int n = design_lowpass(fs, cutoff_hz, ntaps_req, h);
  *W = 32 * ((n + 31) / 32);
  taps.assign(h, h + n);
  lut.assign((size_t)(*W / 8) * 256, 0.0);
  build_tables(h, n, *W, lut.data());
  return n;
}

size_t lowpass_hist_bytes(int nch) { return (size_t)nch * sizeof(LpHist); }

static size_t lowpass_smem(int W) {
  return (size_t)(W / 8) * 256 * sizeof(double) + kLpWords * sizeof(uint32_t);
}

int lowpass_prepare(int W) {
  const int smem = (int)lowpass_smem(W);
  if (cudaFuncSetAttribute(lowpass_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           smem) != cudaSuccess ||
      cudaFuncSetAttribute(lowpass_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           smem) != cudaSuccess)
    return -1;
  return 0;
}

template <typename OutT>
static int launch_lowpass_fresh_t(const double* lut, const double* taps, int ntaps, int W,
                                  const uint8_t* bits, size_t bits_stride, long long count,
                                  const void* zero_hist, int nch, double g_start, double g_step,
                                  OutT* out, size_t out_stride, int num_sms, cudaStream_t stream) {
  if (count <= 0) return 0;
  const size_t smem = lowpass_smem(W);
  const long long tiles = (count + kLpTile - 1) / kLpTile * nch;
  const long long cap = (long long)(num_sms > 0 ? num_sms : 152) * (smem > 50 * 1024 ? 3 : 4);
  lowpass_kernel<OutT><<<(unsigned)(tiles < cap ? tiles : cap), kLpTile, smem, stream>>>(
      lut, taps, ntaps, W, bits, bits_stride, count, (const LpHist*)zero_hist, nch, g_start,
      g_step, out, out_stride);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_lowpass_fresh(const double* lut, const double* taps, int ntaps, int W,
                         const uint8_t* bits, size_t bits_stride, long long count,
                         const void* zero_hist, int nch, double g_start, double g_step,
                         double* out, size_t out_stride, int num_sms, cudaStream_t stream) {
  return launch_lowpass_fresh_t(lut, taps, ntaps, W, bits, bits_stride, count, zero_hist, nch,
                                g_start, g_step, out, out_stride, num_sms, stream);
}

int launch_lowpass_fresh(const double* lut, const double* taps, int ntaps, int W,
                         const uint8_t* bits, size_t bits_stride, long long count,
                         const void* zero_hist, int nch, double g_start, double g_step,
                         float* out, size_t out_stride, int num_sms, cudaStream_t stream) {
  return launch_lowpass_fresh_t(lut, taps, ntaps, W, bits, bits_stride, count, zero_hist, nch,
                                g_start, g_step, out, out_stride, num_sms, stream);
}

struct dsdgpu_lowpass_state {
  int ntaps = 0;
  int W = 0;
  int nch = 0;
  double* d_lut = nullptr;
  double* d_taps = nullptr;
  LpHist* d_hist = nullptr;
  std::vector<double> taps;
};

void lowpass_free(dsdgpu_lowpass_state* s) {
  if (!s) return;
  if (s->d_lut) cudaFree(s->d_lut);
  if (s->d_taps) cudaFree(s->d_taps);
  if (s->d_hist) cudaFree(s->d_hist);
  delete s;
}

extern "C" {

int dsdgpu_lowpass_setup(dsdgpu_context_t* c, unsigned fs, double cutoff_hz, int ntaps, int nch) {
  if (!c || nch < 1) return DSDGPU_ERR_ARG;
  if (fs == 0 || !(cutoff_hz > 0.0)) return c->fail(DSDGPU_ERR_ARG, "lowpass needs fs > 0 and cutoff > 0");
  cudaSetDevice(c->device);
  lowpass_free(c->lowpass);
  c->lowpass = nullptr;
  auto* s = new dsdgpu_lowpass_state;
  double h[kLpMaxTaps + 1];
  s->ntaps = design_lowpass(fs, cutoff_hz, ntaps, h);
  s->W = 32 * ((s->ntaps + 31) / 32);
  s->nch = nch;
  s->taps.assign(h, h + s->ntaps);
  std::vector<double> tab((size_t)(s->W / 8) * 256);
  build_tables(h, s->ntaps, s->W, tab.data());
  cudaError_t e = cudaMalloc(&s->d_lut, tab.size() * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_taps, (size_t)s->ntaps * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&s->d_hist, (size_t)nch * sizeof(LpHist));
  if (e != cudaSuccess) {
    lowpass_free(s);
    return c->cuda_fail(e, "lowpass allocation");
  }
  cudaMemcpyAsync(s->d_lut, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(s->d_taps, h, (size_t)s->ntaps * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  cudaMemsetAsync(s->d_hist, 0, (size_t)nch * sizeof(LpHist), c->stream);
  const size_t smem = (size_t)(s->W / 8) * 256 * sizeof(double) + kLpWords * sizeof(uint32_t);
  e = cudaFuncSetAttribute(lowpass_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) {
    lowpass_free(s);
    return c->cuda_fail(e, "lowpass shared memory");
  }
  c->lowpass = s;
  return c->check_status();   // the host table is freed on return: wait for its copy
}

int dsdgpu_lowpass_design(unsigned fs, double cutoff_hz, int ntaps, double* taps, int cap,
                          int* out_ntaps) {
  if (fs == 0 || !(cutoff_hz > 0.0) || !taps || !out_ntaps) return DSDGPU_ERR_ARG;
  double h[kLpMaxTaps + 1];
  const int n = design_lowpass(fs, cutoff_hz, ntaps, h);
  if (cap < n) return DSDGPU_ERR_ARG;
  memcpy(taps, h, (size_t)n * sizeof(double));
  *out_ntaps = n;
  return DSDGPU_OK;
}

int dsdgpu_lowpass_taps(const dsdgpu_context_t* c, double* taps, int cap, int* ntaps) {
  if (!c || !ntaps) return DSDGPU_ERR_ARG;
  if (!c->lowpass) return DSDGPU_ERR_STATE;
  *ntaps = c->lowpass->ntaps;
  if (taps) {
    if (cap < c->lowpass->ntaps) return DSDGPU_ERR_ARG;
    memcpy(taps, c->lowpass->taps.data(), (size_t)c->lowpass->ntaps * sizeof(double));
  }
  return DSDGPU_OK;
}

int dsdgpu_lowpass_reset(dsdgpu_context_t* c) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->lowpass) return c->fail(DSDGPU_ERR_STATE, "lowpass not set up");
  cudaSetDevice(c->device);
  cudaMemsetAsync(c->lowpass->d_hist, 0, (size_t)c->lowpass->nch * sizeof(LpHist), c->stream);
  return c->check_status();
}

int dsdgpu_lowpass_process_async(dsdgpu_context_t* c, int first, int nch, const uint8_t* d_bits,
                                 size_t bits_stride, size_t count, double* d_out, size_t out_stride,
                                 double gain_start, double gain_end) {
  if (!c) return DSDGPU_ERR_ARG;
  dsdgpu_lowpass_state* s = c->lowpass;
  if (!s) return c->fail(DSDGPU_ERR_STATE, "lowpass not set up");
  if (first < 0 || nch < 1 || first + nch > s->nch) return c->fail(DSDGPU_ERR_ARG, "bad channel range");
  if (count == 0) return DSDGPU_OK;
  if (!d_bits || !d_out) return c->fail(DSDGPU_ERR_ARG, "null buffer");
  if (nch > 1 && (bits_stride < count || out_stride < count))
    return c->fail(DSDGPU_ERR_ARG, "row stride shorter than the count");
  cudaSetDevice(c->device);
  // gain ramp of engine_process_block's same-rate branch (src/engine.c:518-523)
  double gs = gain_start;
  if (gs == 0.0) gs = gain_end;
  const double step = count > 1 ? (gain_end - gs) / (double)(count - 1) : 0.0;
  const long long tiles = (long long)((count + kLpTile - 1) / kLpTile) * nch;
  const size_t smem = (size_t)(s->W / 8) * 256 * sizeof(double) + kLpWords * sizeof(uint32_t);
  const int per_sm = smem > 50 * 1024 ? 3 : 4;   // 4 x 32 KB (127 taps), 3 x 64 KB (255)
  const long long cap = (long long)(c->num_sms > 0 ? c->num_sms : 152) * per_sm;
  const unsigned grid = (unsigned)(tiles < cap ? tiles : cap);
  LpHist* hist = s->d_hist + first;
  lowpass_kernel<double><<<grid, kLpTile, smem, c->stream>>>(s->d_lut, s->d_taps, s->ntaps, s->W, d_bits,
                                                     bits_stride, (long long)count, hist, nch, gs,
                                                     step, d_out, out_stride);
  lowpass_hist_kernel<<<nch, 256, 0, c->stream>>>(d_bits, bits_stride, (long long)count, hist, nch);
  c->launches += 2;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? DSDGPU_OK : c->cuda_fail(e, "lowpass launch");
}

int dsdgpu_lowpass_process(dsdgpu_context_t* c, int first, int nch, const uint8_t* d_bits,
                           size_t bits_stride, size_t count, double* d_out, size_t out_stride,
                           double gain_start, double gain_end) {
  const int rc = dsdgpu_lowpass_process_async(c, first, nch, d_bits, bits_stride, count, d_out,
                                              out_stride, gain_start, gain_end);
  return rc ? rc : c->check_status();
}

}  // extern "C"
