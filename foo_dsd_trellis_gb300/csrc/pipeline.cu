// Whole-path entry points: PCM -> FIR chain + engine glue -> segment-parallel
// trellis SDM with Density-Aligned Stitching -> DoP / native / decision bytes.
// This is the GPU counterpart of the plugin's PCM path with DAS (reference
// src/dsp_plugin.c:2990-3216 for PCM in / DoP out, src/dsp_plugin.c:1283-2945
// for the DAS phases), one chunk per call.  Stage timings are taken with CUDA
// events on the context's stream.
#include "api_context.h"

#include <cstring>

namespace {
constexpr unsigned kDsd64Rate = 2822400u;   // DSD_RATE_64: inputs at or above it are DSD
}  // namespace

extern "C" {

int dsdgpu_pipeline_setup(dsdgpu_context_t* c, const dsdgpu_pipeline_params_t* p, int nch) {
  if (!c || !p || nch < 1) return DSDGPU_ERR_ARG;
  if (p->output_format < DSDGPU_OUT_BITS || p->output_format > DSDGPU_OUT_PCM)
    return c->fail(DSDGPU_ERR_ARG, "bad output format");
  c->pipe_pcm_out = p->output_format == DSDGPU_OUT_PCM;
  if (c->pipe_pcm_out) {
    // DSD -> PCM: DoP unpack and the decimation chain, no SDM (src/engine.c:566-577)
    if (p->fir.fs_out >= p->fir.fs_in) return c->fail(DSDGPU_ERR_ARG, "PCM output needs fs_out < fs_in");
    const int rc = dsdgpu_decim_setup(c, p->fir.fs_in, p->fir.fs_out, nch);
    if (rc) return rc;
    c->pipe = *p;
    c->pipe_nch = nch;
    c->pipe_ready = true;
    c->pipe_same_rate = false;
    c->pipe_precorr = false;
    c->pipe_lowpass = false;
    c->pipe_dsd_up = false;
    c->pipe_dsd_down = false;
    if (!c->ev_ready) {
      for (int i = 0; i < dsdgpu_context::kEvents; i++) cudaEventCreate(&c->ev[i]);
      c->ev_ready = true;
    }
    return DSDGPU_OK;
  }
  if (p->sdm_mode != DSDGPU_SDM_TRELLIS && p->sdm_mode != DSDGPU_SDM_PRECORR)
    return c->fail(DSDGPU_ERR_ARG, "bad sdm mode");
  c->pipe_precorr = p->sdm_mode == DSDGPU_SDM_PRECORR;
  int rc = c->pipe_precorr ? dsdgpu_precorr_setup(c, p->sdm.order, p->sdm.a, p->sdm.g,
                                                  p->sdm.state_limit, nch)
                           : dsdgpu_sdm_setup(c, &p->sdm, nch);
  if (rc) return rc;
  c->pipe_same_rate = p->fir.fs_in == p->fir.fs_out;
  if (p->samerate_filter != DSDGPU_SAMERATE_BOXCAR && p->samerate_filter != DSDGPU_SAMERATE_LOWPASS)
    return c->fail(DSDGPU_ERR_ARG, "bad same-rate filter");
  c->pipe_lowpass = c->pipe_same_rate && p->samerate_filter == DSDGPU_SAMERATE_LOWPASS;
  // DSD input at another DSD rate (the engine's rate-conversion branch with DSD
  // in, src/engine.c:600-729: boxcar at the input rate, FIR up or down, gain,
  // soft clip unless PreCorr)
  const bool dsd_in = p->fir.fs_in >= kDsd64Rate;
  c->pipe_dsd_up = dsd_in && p->fir.fs_out > p->fir.fs_in;
  c->pipe_dsd_down = dsd_in && p->fir.fs_out < p->fir.fs_in;
  c->pipe_down_stages = 0;
  dsdgpu_fir_params_t fp = p->fir;
  if (c->pipe_precorr) fp.soft_clip = 0;   // the engine does not clip ahead of PreCorr
  if (c->pipe_dsd_down) {
    // boxcar_taps 0: no pre-smooth, as the plugin's DAS FIR phase
    // (engine_process_fir_gain, src/engine.c:789-900); a one-tap mean is the
    // identity on the +-1 input
    const int taps = p->fir.boxcar_taps > 0 ? p->fir.boxcar_taps : 1;
    rc = dsdgpu_boxcar_setup(c, taps, nch);
    if (!rc) rc = dsdgpu_decim_setup(c, p->fir.fs_in, p->fir.fs_out, nch);
    if (!rc)
      for (unsigned r = p->fir.fs_in / p->fir.fs_out; r > 1; r >>= 1) c->pipe_down_stages++;
  } else if (c->pipe_lowpass) {
    // DSD in at the output rate: DoP unpack + FIR lowpass (fir_lowpass_init,
    // src/engine.c:168-181, 505-523)
    rc = dsdgpu_lowpass_setup(c, p->fir.fs_in, 50000.0, 127, nch);
  } else if (c->pipe_same_rate) {
    // DSD in at the output rate: DoP unpack + boxcar (src/engine.c:487-563)
    const int taps = p->fir.boxcar_taps > 0 ? p->fir.boxcar_taps : samerate_boxcar_taps(p->fir.fs_in);
    rc = dsdgpu_boxcar_setup(c, taps, nch);
  } else {
    rc = dsdgpu_fir_setup(c, &fp, nch);
  }
  if (rc) return rc;
  c->pipe = *p;
  c->pipe.fir = fp;
  c->pipe_nch = nch;
  c->pipe_ready = true;
  c->dop_phase = 0;
  if (!c->ev_ready) {
    for (int i = 0; i < dsdgpu_context::kEvents; i++) cudaEventCreate(&c->ev[i]);
    c->ev_ready = true;
  }
  return DSDGPU_OK;
}

// plugin_flush (src/dsp_plugin.c:3622-3653): every channel's SDM (or PreCorr)
// state, the filters' histories and the DoP marker phase start over, so the
// next chunk converts as the first chunk of a new stream.
int dsdgpu_pipeline_flush(dsdgpu_context_t* c) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->pipe_ready) return c->fail(DSDGPU_ERR_STATE, "pipeline not set up");
  int rc = DSDGPU_OK;
  if (c->pipe_pcm_out) {
    rc = dsdgpu_decim_reset(c);
  } else {
    rc = c->pipe_precorr ? dsdgpu_precorr_reset(c) : dsdgpu_sdm_reset(c, -1);
    if (!rc) {
      if (c->pipe_dsd_down) {
        rc = dsdgpu_boxcar_reset(c);
        if (!rc) rc = dsdgpu_decim_reset(c);
      } else if (c->pipe_lowpass) {
        rc = dsdgpu_lowpass_reset(c);
      } else if (c->pipe_same_rate) {
        rc = dsdgpu_boxcar_reset(c);
      } else {
        rc = dsdgpu_fir_reset(c);
      }
    }
    if (!rc && c->conv) rc = dsdgpu_conv_reset(c);
  }
  c->dop_phase = 0;
  return rc;
}

int dsdgpu_pipeline_process(dsdgpu_context_t* c, const float* d_pcm, size_t pcm_stride,
                            size_t frames, double gain_start, double gain_end, uint8_t* d_out,
                            size_t out_stride, size_t* out_samples, size_t* out_bytes) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->pipe_ready) return c->fail(DSDGPU_ERR_STATE, "pipeline not set up");
  if (frames > 0 && (!d_pcm || !d_out)) return c->fail(DSDGPU_ERR_ARG, "null buffer");
  if (frames == 0) {   // an empty block: no output, no state change
    if (out_samples) *out_samples = 0;
    if (out_bytes) *out_bytes = 0;
    return DSDGPU_OK;
  }
  cudaSetDevice(c->device);
  const int nch = c->pipe_nch;
  if (c->pipe_pcm_out) {
    // DSD -> PCM: DoP unpack into decision bytes, decimation to float rows
    const size_t n_in = 16 * frames;
    const size_t bit_row = (n_in + 255) & ~(size_t)255;
    int rc = c->ensure_scratch(bit_row * (size_t)nch + 256);
    if (rc) return rc;
    uint8_t* d_bits = (uint8_t*)c->d_scratch;
    cudaEventRecord(c->ev[0], c->stream);
    rc = dsdgpu_dop_unpack(c, nch, d_pcm, pcm_stride, frames, d_bits, bit_row);
    if (rc) return rc;
    size_t n = 0;
    rc = dsdgpu_decim_process_async(c, nch, d_bits, bit_row, n_in, (float*)d_out, out_stride,
                                    gain_start, gain_end, &n);
    if (rc) return rc;
    cudaEventRecord(c->ev[5], c->stream);
    rc = c->check_status();
    if (rc) return rc;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[5]);
    c->stage_ms[0] = ms;
    c->stage_ms[1] = c->stage_ms[2] = c->stage_ms[3] = 0.0f;
    c->stage_ms[4] = ms;
    if (out_samples) *out_samples = n;
    if (out_bytes) *out_bytes = n * sizeof(float) * (size_t)nch;
    return DSDGPU_OK;
  }
  // DoP input (same rate, DSD up or down): 16 decisions per frame
  const bool dop_in = c->pipe_same_rate || c->pipe_dsd_up || c->pipe_dsd_down;
  const size_t n_in = dop_in ? 16 * frames : frames;
  size_t n_fir = c->pipe_same_rate ? n_in : n_in * (size_t)c->fir.ratio;
  if (c->pipe_dsd_down) {
    n_fir = n_in;
    for (int k = 0; k < c->pipe_down_stages; k++) n_fir /= 2;
  }
  // device work buffers: FIR output (double), stitched decisions, and for DSD
  // rate conversion the unpacked input (+-1 floats up; decisions and their
  // boxcar mean down)
  const size_t fir_bytes = (n_fir * sizeof(double) + 255) & ~(size_t)255;
  const size_t bit_row = (n_fir + 255) & ~(size_t)255;
  const size_t in_f32 = c->pipe_dsd_up ? ((n_in * sizeof(float) + 255) & ~(size_t)255) : 0;
  const size_t in_bits = c->pipe_dsd_down ? ((n_in + 255) & ~(size_t)255) : 0;
  const size_t in_f64 = c->pipe_dsd_down ? ((n_in * sizeof(double) + 255) & ~(size_t)255) : 0;
  int rc = c->ensure_scratch((fir_bytes + bit_row + in_f32 + in_bits + in_f64) * (size_t)nch + 256);
  if (rc) return rc;
  double* d_fir = (double*)c->d_scratch;
  uint8_t* d_bits = (uint8_t*)c->d_scratch + fir_bytes * (size_t)nch;
  uint8_t* d_extra = d_bits + bit_row * (size_t)nch;
  const size_t fir_stride = fir_bytes / sizeof(double);

  // PCM into PreCorr without a convolution: the chain writes FP32, the
  // values the walk would narrow its FP64 input to (the FP32 chain's outputs
  // widen exactly, and PreCorr has no soft clip ahead of it), so the walk
  // reads them as they are; the rows keep their FP64 stride in elements
  const bool f32_precorr = c->pipe_precorr && !c->conv && !c->pipe_same_rate &&
                           !c->pipe_dsd_up && !c->pipe_dsd_down;
  cudaEventRecord(c->ev[0], c->stream);
  size_t fo = 0;
  if (c->pipe_same_rate) {
    // the decision buffer holds the unpacked input until the DAS writes it
    rc = dsdgpu_dop_unpack(c, nch, d_pcm, pcm_stride, frames, d_bits, bit_row);
    if (rc) return rc;
    rc = c->pipe_lowpass
             ? dsdgpu_lowpass_process_async(c, 0, nch, d_bits, bit_row, n_fir, d_fir, fir_stride,
                                            gain_start, gain_end)
             : dsdgpu_boxcar_process_async(c, 0, nch, d_bits, bit_row, n_fir, d_fir, fir_stride,
                                           gain_start, gain_end);
    fo = n_fir;
  } else if (c->pipe_dsd_up) {
    // +-1.0 floats at the input DSD rate, then the FIR chain with its boxcar
    float* d_f = (float*)d_extra;
    const size_t f_stride = in_f32 / sizeof(float);
    rc = dsdgpu_dop_unpack_f32(c, nch, d_pcm, pcm_stride, frames, d_f, f_stride);
    if (rc) return rc;
    rc = dsdgpu_fir_process_async(c, 0, nch, d_f, f_stride, n_in, d_fir, fir_stride, gain_start,
                                  gain_end, &fo);
  } else if (c->pipe_dsd_down) {
    // decisions, their boxcar mean (gain 1: the sum times 1/taps exactly as
    // the engine forms it), then the FP64 decimation chain, gain and clip
    uint8_t* d_in_bits = d_extra;
    double* d_box = (double*)(d_extra + in_bits * (size_t)nch);
    const size_t box_stride = in_f64 / sizeof(double);
    rc = dsdgpu_dop_unpack(c, nch, d_pcm, pcm_stride, frames, d_in_bits, in_bits);
    if (rc) return rc;
    rc = dsdgpu_boxcar_process_async(c, 0, nch, d_in_bits, in_bits, n_in, d_box, box_stride, 1.0, 1.0);
    if (rc) return rc;
    rc = dsdgpu_decim_process_f64_async(c, nch, d_box, box_stride, n_in, d_fir, fir_stride,
                                        gain_start, gain_end, c->pipe.fir.soft_clip, &fo);
  } else if (f32_precorr) {
    rc = fir_process_async_f32(c, nch, d_pcm, pcm_stride, frames, (float*)d_fir,
                               fir_stride, gain_start, gain_end, &fo);
  } else {
    rc = dsdgpu_fir_process_async(c, 0, nch, d_pcm, pcm_stride, frames, d_fir, fir_stride,
                                  gain_start, gain_end, &fo);
  }
  if (rc) return rc;
  if (c->conv) {
    // room-correction convolution at the SDM rate (src/gpu_cuda.c:3432-3492)
    rc = conv_run(c, nch, d_fir, fir_stride, fo, d_fir, fir_stride);
    if (rc) return rc;
  }
  cudaEventRecord(c->ev[1], c->stream);
  size_t n = 0;
  if (c->pipe_precorr) {
    // PreCorr: sequential per channel, no latency (src/engine.c:557-559, 723-726)
    cudaEventRecord(c->ev[2], c->stream);
    rc = f32_precorr ? precorr_run(c, 0, nch, (const float*)d_fir, fir_stride, fo, d_bits, bit_row)
                     : precorr_run(c, 0, nch, d_fir, fir_stride, fo, d_bits, bit_row);
    cudaEventRecord(c->ev[3], c->stream);
    n = fo;
  } else {
    c->timing_das = true;
    rc = dsdgpu_das_process(c, &c->pipe.das, nch, d_fir, fir_stride, fo, d_bits, bit_row, &n,
                            nullptr, 0);
    c->timing_das = false;
  }
  if (rc) return rc;
  cudaEventRecord(c->ev[4], c->stream);
  size_t nbytes = 0;
  if (c->pipe.output_format == DSDGPU_OUT_DOP) {
    int next = 0;
    rc = dsdgpu_pack_dop(c, nch, d_bits, bit_row, n, d_out, c->dop_phase, &next);
    if (rc) return rc;
    c->dop_phase = next;
    nbytes = (n / 16) * 3 * (size_t)nch;
  } else if (c->pipe.output_format == DSDGPU_OUT_NATIVE) {
    rc = dsdgpu_pack_native(c, nch, d_bits, bit_row, n, d_out, out_stride);
    if (rc) return rc;
    nbytes = ((n + 7) / 8) * (size_t)nch;
  } else {
    if (out_stride < n) return c->fail(DSDGPU_ERR_ARG, "output stride too small");
    cudaMemcpy2DAsync(d_out, out_stride, d_bits, bit_row, n, (size_t)nch,
                      cudaMemcpyDeviceToDevice, c->stream);
    nbytes = n * (size_t)nch;
  }
  cudaEventRecord(c->ev[5], c->stream);
  rc = c->check_status();
  if (rc) return rc;
  float ms[5] = {0, 0, 0, 0, 0};
  cudaEventElapsedTime(&ms[0], c->ev[0], c->ev[1]);   // FIR
  cudaEventElapsedTime(&ms[1], c->ev[2], c->ev[3]);   // segment SDM (last launch)
  cudaEventElapsedTime(&ms[2], c->ev[1], c->ev[4]);   // DAS total
  cudaEventElapsedTime(&ms[3], c->ev[4], c->ev[5]);   // pack
  cudaEventElapsedTime(&ms[4], c->ev[0], c->ev[5]);   // whole step
  memcpy(c->stage_ms, ms, sizeof ms);
  if (out_samples) *out_samples = n;
  if (out_bytes) *out_bytes = nbytes;
  return DSDGPU_OK;
}

int dsdgpu_pipeline_process_host(dsdgpu_context_t* c, const float* h_pcm, size_t frames,
                                 double gain_start, double gain_end, uint8_t* h_out,
                                 size_t out_capacity, size_t* out_samples, size_t* out_bytes) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->pipe_ready) return c->fail(DSDGPU_ERR_STATE, "pipeline not set up");
  if (frames > 0 && (!h_pcm || !h_out)) return c->fail(DSDGPU_ERR_ARG, "null buffer");
  if (frames == 0) {
    if (out_samples) *out_samples = 0;
    if (out_bytes) *out_bytes = 0;
    return DSDGPU_OK;
  }
  cudaSetDevice(c->device);
  const int nch = c->pipe_nch;
  size_t n_fir = frames * (c->pipe_same_rate || c->pipe_pcm_out ? (size_t)16 : (size_t)c->fir.ratio);
  if (c->pipe_dsd_up) n_fir = 16 * frames * (size_t)c->fir.ratio;
  if (c->pipe_dsd_down) {
    n_fir = 16 * frames;
    for (int k = 0; k < c->pipe_down_stages; k++) n_fir /= 2;
  }
  if (c->pipe_pcm_out) n_fir = n_fir * sizeof(float);   // output rows hold floats (fewer of them)
  // staging for the input and output on the device, kept across calls
  const size_t in_bytes = (frames * (size_t)nch * sizeof(float) + 255) & ~(size_t)255;
  const size_t out_row = (n_fir + 255) & ~(size_t)255;
  const size_t need = in_bytes + out_row * (size_t)nch;
  if (c->io_bytes < need) {
    if (c->d_io) cudaFree(c->d_io);
    c->d_io = nullptr;
    c->io_bytes = 0;
    cudaError_t e = cudaMalloc(&c->d_io, need);
    if (e != cudaSuccess) return c->cuda_fail(e, "io staging allocation");
    c->io_bytes = need;
  }
  float* d_pcm = (float*)c->d_io;
  uint8_t* d_out = (uint8_t*)c->d_io + in_bytes;
  cudaError_t e = cudaMemcpyAsync(d_pcm, h_pcm, frames * (size_t)nch * sizeof(float),
                                  cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "pcm upload");
  size_t n = 0, nb = 0;
  int rc = dsdgpu_pipeline_process(c, d_pcm, frames, frames, gain_start, gain_end, d_out,
                                   c->pipe_pcm_out ? out_row / sizeof(float) : out_row, &n, &nb);
  if (rc) return rc;
  if (nb > out_capacity) return c->fail(DSDGPU_ERR_ARG, "host output buffer too small");
  if (c->pipe.output_format == DSDGPU_OUT_PCM) {
    // the rows were written with a stride of out_row bytes / 4 floats
    e = cudaMemcpy2DAsync(h_out, n * sizeof(float), d_out, out_row, n * sizeof(float), (size_t)nch,
                          cudaMemcpyDeviceToHost, c->stream);
  } else if (c->pipe.output_format == DSDGPU_OUT_NATIVE) {
    const size_t rowb = (n + 7) / 8;
    e = cudaMemcpy2DAsync(h_out, rowb, d_out, out_row, rowb, (size_t)nch, cudaMemcpyDeviceToHost,
                          c->stream);
  } else if (c->pipe.output_format == DSDGPU_OUT_BITS) {
    e = cudaMemcpy2DAsync(h_out, n, d_out, out_row, n, (size_t)nch, cudaMemcpyDeviceToHost,
                          c->stream);
  } else {
    e = cudaMemcpyAsync(h_out, d_out, nb, cudaMemcpyDeviceToHost, c->stream);
  }
  if (e != cudaSuccess) return c->cuda_fail(e, "output download");
  rc = c->check_status();
  if (rc) return rc;
  if (out_samples) *out_samples = n;
  if (out_bytes) *out_bytes = nb;
  return DSDGPU_OK;
}

int dsdgpu_stage_times(const dsdgpu_context_t* c, float* ms5) {
  if (!c || !ms5) return DSDGPU_ERR_ARG;
  memcpy(ms5, c->stage_ms, sizeof c->stage_ms);
  return DSDGPU_OK;
}

int dsdgpu_get_stream(const dsdgpu_context_t* c, void** stream) {
  if (!c || !stream) return DSDGPU_ERR_ARG;
  *stream = (void*)c->stream;
  return DSDGPU_OK;
}

}  // extern "C"
