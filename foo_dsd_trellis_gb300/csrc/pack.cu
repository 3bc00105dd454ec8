// DSD bit packing on sm_103a (reference src/dop.c:114-184, the plugin's pack
// stage src/threadpool.c:329-345, and the DSF/DFF byte orders of
// tools/dsd_encode.c:80-98).
//
//   DoP      16 decisions per 24-bit frame, MSB first, stored little-endian
//            [bits 7..0, bits 15..8, marker]; the marker alternates 0x05/0xFA
//            from the caller's phase; channels interleaved frame by frame.
//   native   8 decisions per byte, MSB first (bits_pack); a trailing partial
//            byte is left-aligned.
//
// Decisions arrive as one byte per sample (0/1).  Each thread packs whole
// frames/bytes from 16/8 consecutive decision bytes; both kernels are pure
// HBM streams (read n bytes, write 3n/16 or n/8).
#include "api_context.h"

namespace dsdgpu {

__global__ void pack_dop_kernel(const uint8_t* __restrict__ bits, size_t stride, int nch,
                                size_t frames, int phase, uint8_t* __restrict__ out) {
  const size_t total = frames * (size_t)nch;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t f = t / (size_t)nch;
    const int ch = (int)(t % (size_t)nch);
    const uint8_t* b = bits + (size_t)ch * stride + 16 * f;
    unsigned w = 0;
#pragma unroll
    for (int i = 0; i < 16; i++) w = (w << 1) | (b[i] & 1u);
    uint8_t* o = out + 3 * t;
    o[0] = (uint8_t)(w & 0xffu);
    o[1] = (uint8_t)(w >> 8);
    o[2] = ((f + (size_t)phase) & 1u) ? 0xFAu : 0x05u;
  }
}

__global__ void pack_native_kernel(const uint8_t* __restrict__ bits, size_t stride, int nch,
                                   size_t n, uint8_t* __restrict__ out, size_t out_stride) {
  const size_t nbytes = (n + 7) / 8;
  const size_t total = nbytes * (size_t)nch;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int ch = (int)(t / nbytes);
    const size_t i = t % nbytes;
    const uint8_t* b = bits + (size_t)ch * stride + 8 * i;
    unsigned v = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const unsigned bit = (8 * i + k < n) ? (b[k] & 1u) : 0u;
      v |= bit << (7 - k);
    }
    out[(size_t)ch * out_stride + i] = (uint8_t)v;
  }
}

static unsigned grid_for_sms(int num_sms, size_t items) {
  size_t g = (items + 255) / 256;
  const size_t cap = (size_t)(num_sms > 0 ? num_sms : 148) * 16;
  if (g > cap) g = cap;
  return (unsigned)(g ? g : 1);
}

static unsigned grid_for(dsdgpu_context* c, size_t items) { return grid_for_sms(c->num_sms, items); }

int launch_pack_dop(const uint8_t* bits, size_t stride, int nch, size_t frames, int phase,
                    uint8_t* out, int num_sms, cudaStream_t stream) {
  if (frames == 0) return 0;
  pack_dop_kernel<<<grid_for_sms(num_sms, frames * nch), 256, 0, stream>>>(bits, stride, nch,
                                                                           frames, phase, out);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_pack_native(const uint8_t* bits, size_t stride, int nch, size_t n, uint8_t* out,
                       size_t out_stride, int num_sms, cudaStream_t stream) {
  if (n == 0) return 0;
  pack_native_kernel<<<grid_for_sms(num_sms, ((n + 7) / 8) * nch), 256, 0, stream>>>(
      bits, stride, nch, n, out, out_stride);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace dsdgpu

using namespace dsdgpu;

extern "C" {

int dsdgpu_pack_dop(dsdgpu_context_t* c, int nch, const uint8_t* d_bits, size_t bits_stride,
                    size_t n, uint8_t* d_out, int phase, int* next_phase) {
  if (!c || nch < 1 || phase < 0 || phase > 1) return DSDGPU_ERR_ARG;
  const size_t frames = n / 16;
  if (next_phase) *next_phase = (int)((frames + (size_t)phase) & 1u);
  if (frames == 0) return DSDGPU_OK;
  if (!d_bits || !d_out) return c->fail(DSDGPU_ERR_ARG, "null buffer");
  cudaSetDevice(c->device);
  pack_dop_kernel<<<grid_for(c, frames * nch), 256, 0, c->stream>>>(d_bits, bits_stride, nch,
                                                                    frames, phase, d_out); c->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "pack launch");
  return c->check_status();
}

int dsdgpu_pack_native(dsdgpu_context_t* c, int nch, const uint8_t* d_bits, size_t bits_stride,
                       size_t n, uint8_t* d_out, size_t out_stride) {
  if (!c || nch < 1) return DSDGPU_ERR_ARG;
  if (n == 0) return DSDGPU_OK;
  if (!d_bits || !d_out) return c->fail(DSDGPU_ERR_ARG, "null buffer");
  if (out_stride < (n + 7) / 8) return c->fail(DSDGPU_ERR_ARG, "output stride too small");
  cudaSetDevice(c->device);
  pack_native_kernel<<<grid_for(c, ((n + 7) / 8) * nch), 256, 0, c->stream>>>(
      d_bits, bits_stride, nch, n, d_out, out_stride); c->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "pack launch");
  return c->check_status();
}

}  // extern "C"
