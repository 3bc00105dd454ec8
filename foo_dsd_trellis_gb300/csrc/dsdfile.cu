// DSF / DSDIFF file layout: header bytes on the host, payload packing on the
// device (reference tools/dsd_encode.c:80-98 packers, :164-292 writers).
//
// The reference's offline encoder writes mono files only; the multichannel
// layouts here follow the two formats' published specifications with the
// reference's choices kept where it makes one:
//   DSF   DSD chunk (28 B) | fmt chunk (52 B) | data chunk header (12 B) |
//         payload [block][channel][4096 B], decisions LSB first in a byte,
//         the last block zero-padded; metadata offset 0.
//   DFF   FRM8 | "DSD " | FVER 1.5.0.0 | PROP { "SND " | FS | CHNL } | "DSD "
//         chunk header | payload: bytes interleaved by channel, decisions
//         MSB first, a trailing partial byte zero-filled; no CMPR chunk and
//         no pad byte after an odd-length payload (as the reference writes).
#include "api_context.h"

#include <cstring>

namespace {

// DSF channel types (DSF specification): 1 mono, 2 stereo, 3 three channels,
// 4 quad, 6 five channels, 7 5.1.
int dsf_channel_type(int nch) {
  static const int t[7] = {0, 1, 2, 3, 4, 6, 7};
  return (nch >= 1 && nch <= 6) ? t[nch] : 0;
}

// DSDIFF channel IDs (specification 1.5, CHNL chunk).
const char* dff_channel_id(int nch, int ch) {
  static const char* ids[7][6] = {
      {},
      {"SLFT"},
      {"SLFT", "SRGT"},
      {"MLFT", "MRGT", "C   "},
      {"MLFT", "MRGT", "LS  ", "RS  "},
      {"MLFT", "MRGT", "C   ", "LS  ", "RS  "},
      {"MLFT", "MRGT", "C   ", "LFE ", "LS  ", "RS  "},
  };
  return ids[nch][ch];
}

struct Writer {
  uint8_t* p;
  size_t n = 0;
  size_t cap;
  bool ok = true;
  void put(const void* src, size_t len) {
    if (n + len > cap) { ok = false; return; }
    memcpy(p + n, src, len);
    n += len;
  }
  void id(const char* s) { put(s, 4); }
  void le(uint64_t v, int bytes) {
    uint8_t b[8];
    for (int i = 0; i < bytes; i++) b[i] = (uint8_t)(v >> (8 * i));
    put(b, (size_t)bytes);
  }
  void be(uint64_t v, int bytes) {
    uint8_t b[8];
    for (int i = 0; i < bytes; i++) b[i] = (uint8_t)(v >> (8 * (bytes - 1 - i)));
    put(b, (size_t)bytes);
  }
};

constexpr uint32_t kDsfBlock = 4096;

uint64_t dsf_payload(int nch, uint64_t samples) {
  const uint64_t bytes = (samples + 7) / 8;
  const uint64_t blocks = (bytes + kDsfBlock - 1) / kDsfBlock;
  return blocks * kDsfBlock * (uint64_t)nch;
}

uint64_t dff_payload(int nch, uint64_t samples) { return (samples + 7) / 8 * (uint64_t)nch; }

// [block][channel][kDsfBlock] bytes, LSB first (pack_dsd_lsb,
// tools/dsd_encode.c:90-98, per channel)
__global__ void pack_dsf_kernel(const uint8_t* __restrict__ bits, size_t stride, int nch, size_t n,
                                size_t total, uint8_t* __restrict__ out) {
  const size_t row = (size_t)nch * kDsfBlock;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t blk = t / row, r = t % row;
    const int ch = (int)(r / kDsfBlock);
    const size_t i = blk * kDsfBlock + r % kDsfBlock;   // byte index within the channel
    const uint8_t* b = bits + (size_t)ch * stride + 8 * i;
    unsigned v = 0;
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (8 * i + k < n) v |= (b[k] & 1u) << k;
    out[t] = (uint8_t)v;
  }
}

// [byte][channel], MSB first (pack_dsd_msb, tools/dsd_encode.c:80-88, per channel)
__global__ void pack_dff_kernel(const uint8_t* __restrict__ bits, size_t stride, int nch, size_t n,
                                size_t total, uint8_t* __restrict__ out) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t i = t / (size_t)nch;
    const int ch = (int)(t % (size_t)nch);
    const uint8_t* b = bits + (size_t)ch * stride + 8 * i;
    unsigned v = 0;
#pragma unroll
    for (int k = 0; k < 8; k++)
      if (8 * i + k < n) v |= (b[k] & 1u) << (7 - k);
    out[t] = (uint8_t)v;
  }
}

}  // namespace

extern "C" {

int dsdgpu_file_header(int format, int nch, unsigned fs, uint64_t samples, uint8_t* hdr,
                       size_t cap, size_t* hdr_len, uint64_t* payload_bytes) {
  if (!hdr || nch < 1 || fs == 0) return DSDGPU_ERR_ARG;
  if (nch > 6) return DSDGPU_ERR_UNSUPPORTED;
  Writer w{hdr, 0, cap};
  uint64_t pay = 0;
  if (format == DSDGPU_FILE_DSF) {
    // write_dsf (tools/dsd_encode.c:238-292)
    pay = dsf_payload(nch, samples);
    const uint64_t data_chunk = 12 + pay, fmt_chunk = 52, dsd_chunk = 28;
    w.id("DSD ");
    w.le(dsd_chunk, 8);
    w.le(dsd_chunk + fmt_chunk + data_chunk, 8);
    w.le(0, 8);                         // metadata offset: none
    w.id("fmt ");
    w.le(fmt_chunk, 8);
    w.le(1, 4);                         // format version
    w.le(0, 4);                         // format ID: DSD raw
    w.le((uint64_t)dsf_channel_type(nch), 4);
    w.le((uint64_t)nch, 4);
    w.le(fs, 4);
    w.le(1, 4);                         // bits per sample (LSB first)
    w.le(samples, 8);                   // sample count per channel
    w.le(kDsfBlock, 4);                 // block size per channel
    w.le(0, 4);                         // reserved
    w.id("data");
    w.le(data_chunk, 8);
  } else if (format == DSDGPU_FILE_DFF) {
    // write_dff (tools/dsd_encode.c:168-232), CHNL with one ID per channel
    pay = dff_payload(nch, samples);
    const uint64_t chnl_payload = 2 + 4 * (uint64_t)nch;
    const uint64_t prop_payload = 4 + (12 + 4) + (12 + chnl_payload);
    const uint64_t frm8_payload = 4 + (12 + 4) + (12 + prop_payload) + (12 + pay);
    w.id("FRM8");
    w.be(frm8_payload, 8);
    w.id("DSD ");
    w.id("FVER");
    w.be(4, 8);
    w.be(0x01050000u, 4);               // version 1.5.0.0
    w.id("PROP");
    w.be(prop_payload, 8);
    w.id("SND ");
    w.id("FS  ");
    w.be(4, 8);
    w.be(fs, 4);
    w.id("CHNL");
    w.be(chnl_payload, 8);
    w.be((uint64_t)nch, 2);
    for (int c = 0; c < nch; c++) w.id(dff_channel_id(nch, c));
    w.id("DSD ");
    w.be(pay, 8);
  } else {
    return DSDGPU_ERR_ARG;
  }
  if (!w.ok) return DSDGPU_ERR_ARG;
  if (hdr_len) *hdr_len = w.n;
  if (payload_bytes) *payload_bytes = pay;
  return DSDGPU_OK;
}

int dsdgpu_pack_file(dsdgpu_context_t* c, int format, int nch, const uint8_t* d_bits,
                     size_t bits_stride, size_t n, uint8_t* d_out, uint64_t* payload_bytes) {
  if (!c || nch < 1) return DSDGPU_ERR_ARG;
  if (nch > 6) return c->fail(DSDGPU_ERR_UNSUPPORTED, "DSF/DFF layouts cover 1..6 channels");
  if (format != DSDGPU_FILE_DSF && format != DSDGPU_FILE_DFF)
    return c->fail(DSDGPU_ERR_ARG, "bad file format");
  const uint64_t pay = format == DSDGPU_FILE_DSF ? dsf_payload(nch, n) : dff_payload(nch, n);
  if (payload_bytes) *payload_bytes = pay;
  if (pay == 0) return DSDGPU_OK;
  if (!d_bits || !d_out) return c->fail(DSDGPU_ERR_ARG, "null buffer");
  if (nch > 1 && bits_stride < n) return c->fail(DSDGPU_ERR_ARG, "row stride shorter than the count");
  cudaSetDevice(c->device);
  size_t g = (pay + 255) / 256;
  const size_t cap = (size_t)(c->num_sms > 0 ? c->num_sms : 152) * 16;
  if (g > cap) g = cap;
  if (format == DSDGPU_FILE_DSF)
    pack_dsf_kernel<<<(unsigned)g, 256, 0, c->stream>>>(d_bits, bits_stride, nch, n, (size_t)pay, d_out);
  else
    pack_dff_kernel<<<(unsigned)g, 256, 0, c->stream>>>(d_bits, bits_stride, nch, n, (size_t)pay, d_out);
  c->launches++;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "file pack launch");
  return c->check_status();
}

}  // extern "C"
