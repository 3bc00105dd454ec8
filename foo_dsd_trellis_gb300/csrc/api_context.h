// The opaque dsdgpu_context of include/dsdgpu.h, shared by the host-side
// translation units of libdsdgpu.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/dsdgpu.h"
#include "sdm_internal.h"
#include "fir_internal.h"
#include "das_internal.h"

// Validated copy of the ABI's trellis parameters (sdm_context_init's limits,
// src/trellis.c:977-1011, plus the library's register-ring latency bound).
int sdm_params_from_abi(const dsdgpu_sdm_params_t* p, dsdgpu::SdmParams* P, const char** err);

namespace dsdgpu {
int launch_sdm_jobs(const SdmParams& P, const SdmJob* d_jobs, int njobs, int* d_counter,
                    SdmCtx* d_ctxs, int* d_status, int max_blocks, cudaStream_t stream);
int init_contexts(SdmCtx* d_ctxs, int first, int count, int keep_counters, cudaStream_t stream);
int sdm_jobs_per_cta(const SdmParams& P);   // 32 / lanes_per_job(P)
// Balanced launches (sdm_trellis.cu): warps per SM sub-partition, or 0 for a
// plain launch; the queue entries the parts need; the launch itself.
int sdm_balanced_warps(const SdmParams& P, const SdmJob* jobs, int njobs, int sms,
                       long long part_len);
long long sdm_parts_total(const SdmJob* jobs, int njobs, long long part_len);
const char* sdm_last_kernel();   // kernel of this host thread's last SDM launch
int launch_sdm_parts(const SdmParams& P, const SdmJob* d_jobs, int njobs, long long part_len,
                     unsigned long long* d_queue, long long total, int warps_per_pipe, int sms,
                     SdmCtx* d_ctxs, int* d_status, cudaStream_t stream);
int lanes_per_job(const SdmParams& P);      // the fixed width of capped launches
int launch_pack_dop(const uint8_t* bits, size_t stride, int nch, size_t frames, int phase,
                    uint8_t* out, int num_sms, cudaStream_t stream);
int launch_pack_native(const uint8_t* bits, size_t stride, int nch, size_t n, uint8_t* out,
                       size_t out_stride, int num_sms, cudaStream_t stream);
}  // namespace dsdgpu

struct dsdgpu_conv_state;   // UPOLS convolution (conv.cu)
struct dsdgpu_decim_state;  // DSD -> PCM decimation (decim.cu)
void decim_free(dsdgpu_decim_state* s);
struct dsdgpu_lowpass_state;  // same-rate FIR lowpass (lowpass.cu)
void lowpass_free(dsdgpu_lowpass_state* s);
struct dsdgpu_precorr_state;  // PreCorr greedy SDM (precorr.cu)
// PreCorr rows of the batch plan: one channel of a stream, walked from fresh state
struct PcBatchRow {
  const float* in;
  long long count;
  uint8_t* out;
};
size_t precorr_table_floats();
int precorr_batch_train(int order, const double* a, const double* g, double limit, float* d_table,
                        cudaStream_t stream);
int launch_precorr_batch(int order, const double* a, const double* g, double limit,
                         const float* d_table, const PcBatchRow* d_rows, int nrows,
                         cudaStream_t stream);
void precorr_free(dsdgpu_precorr_state* s);
struct dsdgpu_context;
// PreCorr decisions for channels [first, first + nch) of the context's state
// (FP64 input, narrowed per sample as the reference's float walk reads it, or
// input already in FP32).
int precorr_run(dsdgpu_context* c, int first, int nch, const double* d_in, size_t in_stride,
                size_t count, uint8_t* d_bits, size_t bits_stride);
int precorr_run(dsdgpu_context* c, int first, int nch, const float* d_in, size_t in_stride,
                size_t count, uint8_t* d_bits, size_t bits_stride);
// The FIR chain of channels [0, nch) writing FP32 outputs (for PreCorr).
int fir_process_async_f32(dsdgpu_context* c, int nch, const float* d_in, size_t in_stride,
                          size_t count, float* d_out, size_t out_stride, double gain_start,
                          double gain_end, size_t* out_count);
// Convolve a chunk of `nch` channels with the context's IRs (history carried).
int conv_run(dsdgpu_context* c, int nch, const double* d_in, size_t in_stride, size_t count,
             double* d_out, size_t out_stride);
void conv_free(dsdgpu_conv_state* s);
int samerate_boxcar_taps(unsigned fs);   // engine_init's same-rate boxcar length
// context-free launchers of the DSD-input kernels (dsd_in.cu), fresh state
size_t boxcar_hist_bytes(int nch);
int launch_dop_unpack(const float* dop, size_t dop_stride, long long frames, int nch,
                      uint8_t* bits, size_t bits_stride, cudaStream_t stream);
int launch_dop_unpack_f32(const float* dop, size_t dop_stride, long long frames, int nch,
                          float* out, size_t out_stride, cudaStream_t stream);
int launch_boxcar_fresh(const uint8_t* bits, size_t bits_stride, long long count,
                        const int8_t* zero_hist, int taps, int nch, double g_start, double g_step,
                        double* out, size_t out_stride, cudaStream_t stream);
int launch_boxcar_fresh_f32(const uint8_t* bits, size_t bits_stride, long long count,
                            const int8_t* zero_hist, int taps, int nch, double g_start,
                            double g_step, float* out, size_t out_stride, cudaStream_t stream);
// the same-rate FIR lowpass without a context (lowpass.cu): host tables,
// the shared-memory attribute (outside capture), fresh-state launches
int lowpass_tables(unsigned fs, double cutoff_hz, int ntaps_req, std::vector<double>& lut,
                   std::vector<double>& taps, int* W);
size_t lowpass_hist_bytes(int nch);
int lowpass_prepare(int W);
int launch_lowpass_fresh(const double* lut, const double* taps, int ntaps, int W,
                         const uint8_t* bits, size_t bits_stride, long long count,
                         const void* zero_hist, int nch, double g_start, double g_step,
                         double* out, size_t out_stride, int num_sms, cudaStream_t stream);
int launch_lowpass_fresh(const double* lut, const double* taps, int ntaps, int W,
                         const uint8_t* bits, size_t bits_stride, long long count,
                         const void* zero_hist, int nch, double g_start, double g_step,
                         float* out, size_t out_stride, int num_sms, cudaStream_t stream);
// the FP64 decimation chain from fresh state without a context (decim.cu);
// out32 non-null: FP32 output (gain, no clip) there instead of `out`
int launch_decim_f64_fresh(const double* in, size_t in_stride, long long count, int stages,
                           int nch, double* buf, size_t row, const double* zero_dly,
                           double g_start, double g_step, int apply, int soft_clip, double* out,
                           size_t out_stride, cudaStream_t st, float* out32 = nullptr);

struct dsdgpu_context {
  int device = 0;
  int num_sms = 0;
  int max_blocks = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  unsigned long long launches = 0;   // kernels this context has launched
  unsigned long long sdm_samples = 0;       // SDM input samples run so far
  unsigned long long sdm_last_samples = 0;  // ... by the last SDM launch
  std::string sdm_last_kernel;              // ... and its kernel

  int* d_counter = nullptr;   // persistent-kernel job counter
  int* d_status = nullptr;    // device status word (bounded walks/waits)

  // trellis SDM
  bool sdm_ready = false;
  dsdgpu::SdmParams sdm{};
  int sdm_mode = 0;               // selection strategy (DSDGPU_OPT_SDM_SELECT)
  int sdm_lanes = 0;              // lanes per SDM job (DSDGPU_OPT_SDM_LANES), 0 = automatic
  int sdm_balance = 1;            // balanced launches allowed (DSDGPU_OPT_SDM_BALANCE)
  int failure_test = 0;           // DSDGPU_OPT_FAILURE_TEST bits
  int nctx = 0;
  dsdgpu::SdmCtx* d_ctx = nullptr;
  std::vector<int64_t> pending;   // latency fill per context (host mirror)
  std::vector<int> draining;
  dsdgpu::SdmJob* d_jobs = nullptr;
  int jobs_cap = 0;
  unsigned long long* d_parts = nullptr;   // part queue of balanced SDM launches
  long long parts_cap = 0;

  // FIR chain
  bool fir_ready = false;
  dsdgpu::FirChainConst fir{};
  dsdgpu_fir_params_t fir_params{};
  int fir_channels = 0;
  size_t fir_smem = 0;
  float* d_fir_hist = nullptr;   // last PCM samples per channel

  // DAS (device plan buffers, grown on demand)
  int das_persistent = 0;          // contexts [0, das_persistent) are the channels' own
  int das_last_segments = 0;
  uint8_t* d_das_bits = nullptr;   size_t das_bits_cap = 0;
  double* d_das_est = nullptr;     size_t das_est_cap = 0;
  long long* d_das_i64 = nullptr;  size_t das_i64_cap = 0;
  double* d_das_f64 = nullptr;     size_t das_f64_cap = 0;
  int* d_das_bp = nullptr;         size_t das_bp_cap = 0;
  dsdgpu::SeamTask* d_das_tasks = nullptr;        size_t das_tasks_cap = 0;
  dsdgpu::AssemblePiece* d_das_pieces = nullptr;  size_t das_pieces_cap = 0;
  dsdgpu::SegBuf* d_das_segbuf = nullptr;         size_t das_segbuf_cap = 0;
  double* d_das_qfir = nullptr;    size_t das_qfir_cap = 0;
  unsigned char* d_das_seam_scr = nullptr;  size_t das_seam_scr_cap = 0;   // overlaps > 16,384
  bool das_qfir_ready = false;
  cudaStream_t das_side = nullptr;      // seg0-first: the estimator beside seg1's trellis run
  cudaEvent_t das_side_ev[2] = {};

  // whole-path pipeline
  bool pipe_ready = false;
  dsdgpu_pipeline_params_t pipe{};
  int pipe_nch = 0;
  int dop_phase = 0;
  static constexpr int kEvents = 6;
  cudaEvent_t ev[kEvents] = {};
  bool ev_ready = false;
  bool timing_das = false;        // record events around the segment SDM launch
  float stage_ms[5] = {0, 0, 0, 0, 0};
  void* d_io = nullptr;           // device staging of the host-buffer entry point
  size_t io_bytes = 0;

  // same-rate DSD input: boxcar ring (last 255 values per channel)
  int8_t* d_box_hist = nullptr;
  int box_taps = 0;
  int box_nch = 0;
  bool pipe_same_rate = false;    // pipeline input is DoP: unpack + boxcar instead of the FIR
  // DSD -> DSD rate conversion (DoP in at a DSD rate other than the output's):
  // up through the FIR chain on +-1 floats, down through the FP64 decimation chain
  bool pipe_dsd_up = false;
  bool pipe_dsd_down = false;
  int pipe_down_stages = 0;
  // same-rate FIR lowpass (FIR_MODE_FIR), used instead of the boxcar when set up
  dsdgpu_lowpass_state* lowpass = nullptr;
  bool pipe_lowpass = false;

  // DSD -> PCM decimation chain (pipeline output format DSDGPU_OUT_PCM)
  dsdgpu_decim_state* decim = nullptr;
  bool pipe_pcm_out = false;

  // PreCorr SDM (pipeline sdm_mode DSDGPU_SDM_PRECORR)
  dsdgpu_precorr_state* precorr = nullptr;
  bool pipe_precorr = false;

  // UPOLS convolution applied after the FIR chain when set up
  dsdgpu_conv_state* conv = nullptr;

  // reusable device scratch for the host-buffer entry points
  void* d_scratch = nullptr;
  size_t scratch_bytes = 0;

  int fail(int code, const char* what);
  int cuda_fail(cudaError_t e, const char* what);
  int ensure_scratch(size_t bytes);
  int check_status();
  int run_jobs(const std::vector<dsdgpu::SdmJob>& jobs);
  void plan_steps(int64_t pend, int64_t count, int64_t discard, int64_t* skip, int64_t* out,
                  int64_t* new_pend) const;
  void release_all() {
    conv_free(conv);
    conv = nullptr;
    decim_free(decim);
    decim = nullptr;
    precorr_free(precorr);
    precorr = nullptr;
    lowpass_free(lowpass);
    lowpass = nullptr;
    if (d_box_hist) cudaFree(d_box_hist);
    d_box_hist = nullptr;
    if (d_ctx) cudaFree(d_ctx);
    if (d_jobs) cudaFree(d_jobs);
    if (d_parts) cudaFree(d_parts);
    d_parts = nullptr;
    parts_cap = 0;
    if (d_scratch) cudaFree(d_scratch);
    if (d_fir_hist) cudaFree(d_fir_hist);
    d_fir_hist = nullptr;
    if (d_io) cudaFree(d_io);
    d_io = nullptr;
    io_bytes = 0;
    if (ev_ready)
      for (int i = 0; i < kEvents; i++) cudaEventDestroy(ev[i]);
    ev_ready = false;
    for (cudaEvent_t& e : das_side_ev)
      if (e) cudaEventDestroy(e);
    das_side_ev[0] = das_side_ev[1] = nullptr;
    if (das_side) cudaStreamDestroy(das_side);
    das_side = nullptr;
    void* das[] = {d_das_bits, d_das_est, d_das_i64, d_das_f64, d_das_bp, d_das_tasks,
                   d_das_pieces, d_das_segbuf, d_das_qfir, d_das_seam_scr};
    for (void* p : das)
      if (p) cudaFree(p);
    d_das_bits = nullptr; d_das_est = nullptr; d_das_i64 = nullptr; d_das_f64 = nullptr;
    d_das_bp = nullptr; d_das_tasks = nullptr; d_das_pieces = nullptr; d_das_segbuf = nullptr;
    d_das_qfir = nullptr;
    d_das_seam_scr = nullptr;
    das_bits_cap = das_est_cap = das_i64_cap = das_f64_cap = das_bp_cap = 0;
    das_tasks_cap = das_pieces_cap = das_segbuf_cap = das_qfir_cap = das_seam_scr_cap = 0;
    das_qfir_ready = false;
    d_ctx = nullptr;
    d_jobs = nullptr;
    d_scratch = nullptr;
  }
};
