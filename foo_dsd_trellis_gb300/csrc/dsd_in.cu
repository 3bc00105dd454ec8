// Same-rate DSD input on sm_103a: DoP unpack and the engine's boxcar
// pre-smooth with gain ramp (the DSD-Wide re-encode path of
// engine_process_block, reference src/engine.c:487-563, with dop_unpack
// src/dop.c:74-87).
//
//   dop_unpack_kernel  one thread per DoP sample: the float is rounded to its
//                      24-bit integer (f * 2^23, half away from zero) and the
//                      low 16 bits become 16 decision bytes, MSB first
//   boxcar_kernel      one thread per output: the window sum of the last
//                      `taps` +-1 values (the reference's running FP64 sum is
//                      an exact integer count, so a direct count is
//                      identical), then (sum * (1/taps)) * (g_start + g_step*i)
//                      in the reference's operation order
//   boxcar_hist_kernel keeps the last taps - 1 values per channel for the
//                      next block (the reference's ring), 0 before the start
#include "api_context.h"

#include <cstring>

using namespace dsdgpu;

namespace {

constexpr int kMaxBoxcar = 256;

__global__ void dop_unpack_kernel(const float* __restrict__ dop, size_t dop_stride, long long frames,
                                  int nch, uint8_t* __restrict__ bits, size_t bits_stride) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= frames * nch) return;
  const long long c = i / frames, f = i % frames;
  const double d = (double)dop[(size_t)c * dop_stride + f] * 8388608.0;
  const int v = d >= 0.0 ? (int)(d + 0.5) : (int)(d - 0.5);
  const unsigned w = (unsigned)v & 0xFFFFu;
  uint8_t* o = bits + (size_t)c * bits_stride + 16 * (size_t)f;
#pragma unroll
  for (int b = 0; b < 16; b++) o[b] = (uint8_t)((w >> (15 - b)) & 1u);
}

// the reference's own output form of dop_unpack: +-1.0f per decision
__global__ void dop_unpack_f32_kernel(const float* __restrict__ dop, size_t dop_stride,
                                      long long frames, int nch, float* __restrict__ out,
                                      size_t out_stride) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= frames * nch) return;
  const long long c = i / frames, f = i % frames;
  const double d = (double)dop[(size_t)c * dop_stride + f] * 8388608.0;
  const int v = d >= 0.0 ? (int)(d + 0.5) : (int)(d - 0.5);
  const unsigned w = (unsigned)v & 0xFFFFu;
  float* o = out + (size_t)c * out_stride + 16 * (size_t)f;
#pragma unroll
  for (int b = 0; b < 16; b++) o[b] = ((w >> (15 - b)) & 1u) ? 1.0f : -1.0f;
}

// OutT = float: the FP64 value narrowed to nearest (the PreCorr walk's input)
template <typename OutT>
__global__ void boxcar_kernel(const uint8_t* __restrict__ bits, size_t bits_stride, long long count,
                              const int8_t* __restrict__ hist, int taps, int nch,
                              double g_start, double g_step, OutT* __restrict__ out,
                              size_t out_stride) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count * nch) return;
  const long long c = i / count, t = i % count;
  const uint8_t* x = bits + (size_t)c * bits_stride;
  const int8_t* h = hist + (size_t)c * (kMaxBoxcar - 1);
  int sum = 0;
  for (int k = 0; k < taps; k++) {
    const long long j = t - k;
    sum += j >= 0 ? (x[j] ? 1 : -1) : h[kMaxBoxcar - 1 + j];
  }
  const double inv_n = 1.0 / (double)taps;
  out[(size_t)c * out_stride + t] = (OutT)
      __dmul_rn(__dmul_rn((double)sum, inv_n), __dadd_rn(g_start, __dmul_rn(g_step, (double)t)));
}

// new history = the last taps - 1 values of (old history ++ block)
__global__ void boxcar_hist_kernel(const uint8_t* __restrict__ bits, size_t bits_stride,
                                   long long count, int8_t* __restrict__ hist, int nch) {
  const int c = blockIdx.x;
  if (c >= nch) return;
  __shared__ int8_t tmp[kMaxBoxcar - 1];
  int8_t* h = hist + (size_t)c * (kMaxBoxcar - 1);
  const uint8_t* x = bits + (size_t)c * bits_stride;
  for (int k = threadIdx.x; k < kMaxBoxcar - 1; k += blockDim.x) {
    const long long j = count - (kMaxBoxcar - 1) + k;      // index into the block
    tmp[k] = j >= 0 ? (int8_t)(x[j] ? 1 : -1) : h[kMaxBoxcar - 1 + j];
  }
  __syncthreads();
  for (int k = threadIdx.x; k < kMaxBoxcar - 1; k += blockDim.x) h[k] = tmp[k];
}

unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// Launchers without a context (the batch plan's DSD-input streams, fresh
// state: `zero_hist` holds nch x (kMaxBoxcar - 1) zero bytes).
size_t boxcar_hist_bytes(int nch) { return (size_t)nch * (kMaxBoxcar - 1); }

int launch_dop_unpack(const float* dop, size_t dop_stride, long long frames, int nch,
                      uint8_t* bits, size_t bits_stride, cudaStream_t stream) {
  if (frames <= 0) return 0;
  dop_unpack_kernel<<<nblk(frames * nch, 256), 256, 0, stream>>>(dop, dop_stride, frames, nch,
                                                                  bits, bits_stride);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_dop_unpack_f32(const float* dop, size_t dop_stride, long long frames, int nch,
                          float* out, size_t out_stride, cudaStream_t stream) {
  if (frames <= 0) return 0;
  dop_unpack_f32_kernel<<<nblk(frames * nch, 256), 256, 0, stream>>>(dop, dop_stride, frames,
                                                                      nch, out, out_stride);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_boxcar_fresh(const uint8_t* bits, size_t bits_stride, long long count,
                        const int8_t* zero_hist, int taps, int nch, double g_start, double g_step,
                        double* out, size_t out_stride, cudaStream_t stream) {
  if (count <= 0) return 0;
  if (taps < 1 || taps > kMaxBoxcar) return -1;
  boxcar_kernel<double><<<nblk(count * nch, 256), 256, 0, stream>>>(
      bits, bits_stride, count, zero_hist, taps, nch, g_start, g_step, out, out_stride);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_boxcar_fresh_f32(const uint8_t* bits, size_t bits_stride, long long count,
                            const int8_t* zero_hist, int taps, int nch, double g_start,
                            double g_step, float* out, size_t out_stride, cudaStream_t stream) {
  if (count <= 0) return 0;
  if (taps < 1 || taps > kMaxBoxcar) return -1;
  boxcar_kernel<float><<<nblk(count * nch, 256), 256, 0, stream>>>(
      bits, bits_stride, count, zero_hist, taps, nch, g_start, g_step, out, out_stride);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Same-rate boxcar taps of engine_init (src/engine.c:130-147): DSD512 and up
// 16, DSD128/256 64, DSD64 32.
int samerate_boxcar_taps(unsigned fs) {
  if (fs >= 22579200u) return 16;
  if (fs >= 5644800u) return 64;
  return 32;
}

extern "C" {

int dsdgpu_dop_unpack(dsdgpu_context_t* c, int nch, const float* d_dop, size_t dop_stride,
                      size_t frames, uint8_t* d_bits, size_t bits_stride) {
  if (!c || nch < 1 || (frames > 0 && (!d_dop || !d_bits))) return DSDGPU_ERR_ARG;
  if (bits_stride < 16 * frames) return c->fail(DSDGPU_ERR_ARG, "bit row shorter than 16 x frames");
  if (frames == 0) return DSDGPU_OK;
  cudaSetDevice(c->device);
  dop_unpack_kernel<<<nblk((long long)frames * nch, 256), 256, 0, c->stream>>>(
      d_dop, dop_stride, (long long)frames, nch, d_bits, bits_stride);
  c->launches++;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? DSDGPU_OK : c->cuda_fail(e, "dop unpack launch");
}

int dsdgpu_dop_unpack_f32(dsdgpu_context_t* c, int nch, const float* d_dop, size_t dop_stride,
                          size_t frames, float* d_out, size_t out_stride) {
  if (!c || nch < 1 || (frames > 0 && (!d_dop || !d_out))) return DSDGPU_ERR_ARG;
  if (out_stride < 16 * frames) return c->fail(DSDGPU_ERR_ARG, "output row shorter than 16 x frames");
  if (frames == 0) return DSDGPU_OK;
  cudaSetDevice(c->device);
  dop_unpack_f32_kernel<<<nblk((long long)frames * nch, 256), 256, 0, c->stream>>>(
      d_dop, dop_stride, (long long)frames, nch, d_out, out_stride);
  c->launches++;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? DSDGPU_OK : c->cuda_fail(e, "dop unpack launch");
}

int dsdgpu_boxcar_setup(dsdgpu_context_t* c, int taps, int nch) {
  if (!c || nch < 1) return DSDGPU_ERR_ARG;
  if (taps < 1 || taps > kMaxBoxcar) return c->fail(DSDGPU_ERR_ARG, "boxcar taps out of range (1..256)");
  cudaSetDevice(c->device);
  if (c->d_box_hist) cudaFree(c->d_box_hist);
  c->d_box_hist = nullptr;
  const size_t bytes = (size_t)nch * (kMaxBoxcar - 1);
  cudaError_t e = cudaMalloc(&c->d_box_hist, bytes);
  if (e != cudaSuccess) return c->cuda_fail(e, "boxcar history allocation");
  cudaMemsetAsync(c->d_box_hist, 0, bytes, c->stream);
  c->box_taps = taps;
  c->box_nch = nch;
  return c->check_status();
}

int dsdgpu_boxcar_reset(dsdgpu_context_t* c) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->d_box_hist) return c->fail(DSDGPU_ERR_STATE, "boxcar not set up");
  cudaSetDevice(c->device);
  cudaMemsetAsync(c->d_box_hist, 0, (size_t)c->box_nch * (kMaxBoxcar - 1), c->stream);
  return c->check_status();
}

int dsdgpu_boxcar_process_async(dsdgpu_context_t* c, int first, int nch, const uint8_t* d_bits,
                                size_t bits_stride, size_t count, double* d_out,
                                size_t out_stride, double gain_start, double gain_end) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->d_box_hist) return c->fail(DSDGPU_ERR_STATE, "boxcar not set up");
  if (first < 0 || nch < 1 || first + nch > c->box_nch) return c->fail(DSDGPU_ERR_ARG, "bad channel range");
  if (count == 0) return DSDGPU_OK;
  if (!d_bits || !d_out) return c->fail(DSDGPU_ERR_ARG, "null buffer");
  cudaSetDevice(c->device);
  // gain ramp of engine_process_block's same-rate branch (src/engine.c:530-535)
  double gs = gain_start;
  if (gs == 0.0) gs = gain_end;
  const double step = count > 1 ? (gain_end - gs) / (double)(count - 1) : 0.0;
  int8_t* hist = c->d_box_hist + (size_t)first * (kMaxBoxcar - 1);
  boxcar_kernel<double><<<nblk((long long)count * nch, 256), 256, 0, c->stream>>>(
      d_bits, bits_stride, (long long)count, hist, c->box_taps, nch, gs, step, d_out, out_stride);
  boxcar_hist_kernel<<<nch, 256, 0, c->stream>>>(d_bits, bits_stride, (long long)count, hist, nch);
  c->launches += 2;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? DSDGPU_OK : c->cuda_fail(e, "boxcar launch");
}

int dsdgpu_boxcar_process(dsdgpu_context_t* c, int first, int nch, const uint8_t* d_bits,
                          size_t bits_stride, size_t count, double* d_out, size_t out_stride,
                          double gain_start, double gain_end) {
  const int rc = dsdgpu_boxcar_process_async(c, first, nch, d_bits, bits_stride, count, d_out,
                                             out_stride, gain_start, gain_end);
  return rc ? rc : c->check_status();
}

}  // extern "C"
