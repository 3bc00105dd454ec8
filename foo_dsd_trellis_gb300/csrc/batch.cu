// Batched multi-stream conversion: the dsdgpu_plan_* entry points of
// include/dsdgpu.h.
//
// A plan converts many whole PCM streams (uneven lengths, mixed rates and
// trellis settings) in one pass:
//
//   graph 1   one fused FIR-chain launch per stream (each with its own chain
//             as a kernel parameter), then one RMS launch over every stream's
//             DAS boundaries, copied to pinned host memory;
//   host      reposition of quiet boundaries (rare; src/dsp_plugin.c:1959-2024)
//             and, only for streams whose layout moved, a rewrite of their
//             rows of the device tables;
//   graph 2   one persistent SDM launch per trellis parameter set over all DAS
//             segments of all its streams (sets run concurrently on forked
//             streams, their grids split in proportion to their work);
//   graph 3   one seam-search launch over every boundary of every stream, then
//             per stream the assembly gather and the packing.
//
// Every segment run starts from one shared fresh context (full-parallel DAS
// seeding of a stream that starts from sdm_context_init, src/dsp_plugin.c:
// 2264-2283) and keeps its working state in a per-CTA scratch context, so the
// plan holds no per-segment SDM state.  Table sizes do not depend on the
// reposition (every segment is used and every boundary is stitched in
// full-parallel mode), so the graphs are captured once and replayed (the tables'
// contents, including every buffer pointer the kernels follow, live in device
// memory that the host rewrites between graph launches).
//
// The autotuner (seg_len = 0) measures the SDM kernel's aggregate throughput
// at several resident-warp counts for each parameter set (short launches on a
// synthetic signal, cached in the context) and picks the DAS segment length
// and resident warps per SM that minimise its model of the SDM phase:
// total segment samples / throughput at the resident warp count, plus the
// tail of the longest segment run.
#include "api_context.h"
#include "das_plan.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

using namespace dsdgpu;

namespace {

constexpr int kBatchMaxChannels = 8;     // MAX_CHANNELS of the reference plugin
constexpr long long kTuneSegLens[] = {32768, 49152, 65536, 98304, 131072};
constexpr int kTuneBps[] = {8, 12, 16};  // resident SDM warps per SM (16 = register limit)
constexpr int kTuneWarpLevels[] = {1, 4, 8, 12, 16};
constexpr long long kTuneSamples = 1024;
constexpr int kDsd64Rate = 2822400;   // input at this rate or above is DoP (DSD)

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct StreamPlan {
  dsdgpu_stream_desc_t d;
  FirChainConst F;
  size_t fir_smem = 0;
  size_t n_fir = 0;                     // FIR output samples per channel
  size_t pcm_off = 0, pcm_stride = 0;   // floats
  size_t fir_off = 0, fir_stride = 0;   // doubles
  size_t seg_off0 = 0, seg_row = 0;     // segment decision buffers: base, bytes per channel
  std::vector<size_t> seg_off;          // per segment, within a channel's row
  size_t bits_off = 0, bits_stride = 0; // stitched decision rows
  size_t out_off = 0, out_stride = 0, out_bytes = 0;
  int cls = 0;                          // trellis parameter class (-1: a PreCorr stream)
  bool precorr = false;
  int pc_cls = -1;                      // PreCorr parameter class
  // DoP input (fs_in a DSD rate): 1 = same rate (unpack, boxcar of box_taps),
  // 2 = to a higher DSD rate (unpack to +-1 floats, the FIR chain), 3 = to a
  // lower one (unpack, boxcar of box_taps, down_stages FP64 half-band /2
  // stages); 0 = PCM
  int dsd_mode = 0;
  int box_taps = 0;
  int down_stages = 0;
  int lp = -1;                          // same-rate DSD through the FIR lowpass: its table set
  size_t f32_off = 0, f32_stride = 0;   // FP32 rows: a PreCorr stream's walk input, or a
                                        // DSD-up trellis stream's unpacked +-1 input (floats)
  size_t f32in_off = 0;                 // a DSD-up PreCorr stream's unpacked input (f32_stride
                                        // is its walk rows'; these rows are 16 x frames long)
  int lat = 0;
  size_t overlap = 0;
  int S = 0;
  std::vector<long long> nom_start, nom_size;
  std::vector<long long> start, size;   // layout the device tables hold
  std::vector<long long> in_start, in_cnt, discard;
  std::vector<int64_t> seg_out;
  long long final_count = 0;
  std::vector<int> job_index;           // [ch * S + s] -> job table row
  int bp_base = 0;
  int task_first = 0, ntasks = 0;
  int piece_first = 0, npieces = 0;
  int segbuf_first = 0;
  int center_first = 0;
  std::vector<long long> centers;       // reposition windows (nominal layout)
  std::vector<int> which;
};

struct SdmClass {
  SdmParams P;
  int job_first = 0, njobs = 0;
  long long samples = 0;
  long long max_job = 0;
  int grid = 0;
  int scratch_first = 0;                // its CTAs' scratch contexts
  cudaStream_t side = nullptr;
  cudaEvent_t join = nullptr;
};

// The same-rate FIR lowpass of one input rate (fir_lowpass_init: 127 taps at
// 50 kHz): taps and group tables in the arena.
struct LpSet {
  unsigned fs = 0;
  int ntaps = 0, W = 0;
  std::vector<double> lut, taps;
  size_t lut_off = 0, taps_off = 0;     // doubles into d_lp
};

// Streams in PreCorr mode with one NTF and limit: one table, one launch.
struct PcClass {
  int order = 0;
  double a[kMaxOrder] = {}, g[kMaxOrder] = {};
  double limit = 0.0;
  int row_first = 0, nrows = 0;
  long long samples = 0;
  cudaStream_t side = nullptr;
  cudaEvent_t join = nullptr;
};

// Layout of one stream for a given segment length: the segment inputs and the
// kept-decision counts of a run from fresh state.
void layout_stream(StreamPlan& s, long long seg_len) {
  das_nominal_layout(s.n_fir, seg_len, 0, s.overlap, s.nom_start, s.nom_size);
  s.S = (int)s.nom_start.size();
  s.start = s.nom_start;
  s.size = s.nom_size;
}

void segment_io(StreamPlan& s) {
  das_segment_io(s.start, s.size, s.n_fir, s.overlap, s.lat, false, s.in_start, s.in_cnt,
                 s.discard);
  s.seg_out.assign(s.S, 0);
  for (int k = 0; k < s.S; k++) {
    int64_t skip, out, np;
    // seg0 runs from the persistent context (nothing pending, no discard);
    // the others from the snapshot of it (nothing pending) with a discard
    sdm_plan_steps(s.lat, 0, s.in_cnt[k], s.discard[k], &skip, &out, &np);
    s.seg_out[k] = out;
  }
}

}  // namespace

struct dsdgpu_plan {
  dsdgpu_context* c = nullptr;
  int fmt = 0;
  long long seg_len = 0;
  int bps = 16;
  double predicted_ms = 0;
  std::vector<StreamPlan> st;
  std::vector<SdmClass> cls;
  std::vector<PcClass> pcls;
  std::vector<LpSet> lps;
  std::vector<PcBatchRow> pcrows;
  long long pc_samples = 0;
  std::vector<SdmJob> jobs;
  std::vector<SeamTask> tasks;
  std::vector<AssemblePiece> pieces;
  std::vector<SegBuf> segbuf;
  std::vector<long long> centers;       // absolute FIR indices (channel-0 rows)
  int max_ovl = 0;
  int nbp = 0;
  int nscratch = 0;
  long long sdm_samples = 0, out_samples = 0;
  // device memory: one arena
  void* d_arena = nullptr;
  size_t arena_bytes = 0;
  float* d_pcm = nullptr;
  double* d_fir = nullptr;
  float* d_f32 = nullptr;              // FP32 chain outputs of the PreCorr streams
  float* d_pctab = nullptr;            // PreCorr tables, one per class
  PcBatchRow* d_pcrows = nullptr;
  int8_t* d_boxhist = nullptr;         // zero boxcar history of the DSD streams
  double* d_lp = nullptr;              // lowpass taps and tables
  void* d_lphist = nullptr;            // zero lowpass history (fresh streams)
  // scratch of the DSD streams to a lower rate, shared (graph 1 runs its
  // streams in order): unpacked decisions, boxcar output, the chain's
  // ping-pong rows, the chain's zero delay lines
  uint8_t* d_dn_bits = nullptr;
  double* d_dn_box = nullptr;
  double* d_dn_pp = nullptr;
  double* d_dn_dly = nullptr;
  cudaEvent_t fork = nullptr;          // graph 2's fork point (several launches)
  uint8_t* d_seg = nullptr;
  uint8_t* d_bits = nullptr;
  uint8_t* d_out = nullptr;
  SdmCtx* d_ctx = nullptr;             // [0] fresh, then scratch contexts
  SdmJob* d_jobs = nullptr;
  SeamTask* d_tasks = nullptr;
  AssemblePiece* d_pieces = nullptr;
  SegBuf* d_segbuf = nullptr;
  int* d_bp = nullptr;
  unsigned char* d_seam_scr = nullptr;   // per-boundary seam scratch (overlaps > 16,384)
  int* d_counters = nullptr;
  double* d_seed = nullptr;
  float* d_hist = nullptr;
  double* d_qfir = nullptr;
  long long* d_centers = nullptr;
  double* d_rms = nullptr;
  double* h_rms = nullptr;             // pinned
  long long* d_cand = nullptr;         // candidate windows of one boundary
  double* d_cand_rms = nullptr;
  size_t cand_cap = 0;
  cudaGraphExec_t g1 = nullptr, g2 = nullptr, g3 = nullptr;
  cudaEvent_t ev[5] = {};
  float ms[4] = {0, 0, 0, 0};
  bool ran = false;

  int fail(int code, const char* what) { return c->fail(code, what); }
  ~dsdgpu_plan();
};

dsdgpu_plan::~dsdgpu_plan() {
  if (c) cudaSetDevice(c->device);
  if (g1) cudaGraphExecDestroy(g1);
  if (g2) cudaGraphExecDestroy(g2);
  if (g3) cudaGraphExecDestroy(g3);
  for (auto& k : cls) {
    if (k.side) cudaStreamDestroy(k.side);
    if (k.join) cudaEventDestroy(k.join);
  }
  for (auto& k : pcls) {
    if (k.side) cudaStreamDestroy(k.side);
    if (k.join) cudaEventDestroy(k.join);
  }
  if (fork) cudaEventDestroy(fork);
  for (cudaEvent_t e : ev)
    if (e) cudaEventDestroy(e);
  if (h_rms) cudaFreeHost(h_rms);
  if (d_cand) cudaFree(d_cand);
  if (d_cand_rms) cudaFree(d_cand_rms);
  if (d_arena) cudaFree(d_arena);
}

namespace {

// ---- autotuner -------------------------------------------------------------

struct TuneCurve {
  std::vector<int> warps;       // resident jobs (all SMs)
  std::vector<double> rate;     // SDM input samples per second
  double at(double w) const {
    if (warps.empty()) return 1.0;
    if (w <= warps.front()) return rate.front() * w / warps.front();
    for (size_t i = 1; i < warps.size(); i++)
      if (w <= warps[i]) {
        const double f = (w - warps[i - 1]) / (double)(warps[i] - warps[i - 1]);
        return rate[i - 1] + f * (rate[i] - rate[i - 1]);
      }
    return rate.back();
  }
};

std::map<std::string, TuneCurve>& tune_cache() {
  static std::map<std::string, TuneCurve> m;
  return m;
}
std::mutex& tune_mutex() {
  static std::mutex m;
  return m;
}

std::string class_key(const SdmParams& P, int device) {
  std::string k(reinterpret_cast<const char*>(&P), sizeof P);
  k += std::to_string(device);
  return k;
}

// Aggregate SDM throughput of one parameter set at the tuner's warp levels:
// short launches of identical synthetic jobs (a two-tone signal at -6 dBFS).
int measure_curve(dsdgpu_context* c, const SdmParams& P, TuneCurve* out) {
  const int sms = c->num_sms > 0 ? c->num_sms : 1;
  const int jpc = sdm_jobs_per_cta(P);
  const int maxw = kTuneWarpLevels[sizeof(kTuneWarpLevels) / sizeof(int) - 1] * sms * jpc;
  std::vector<double> x(kTuneSamples);
  for (long long i = 0; i < kTuneSamples; i++)
    x[i] = 0.3 * std::sin(0.0021 * (double)i) + 0.2 * std::sin(0.037 * (double)i + 1.0);
  double* d_x = nullptr;
  uint8_t* d_o = nullptr;
  SdmCtx* d_c = nullptr;
  SdmJob* d_j = nullptr;
  int* d_cnt = nullptr;
  int rc = DSDGPU_OK;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaMalloc(&d_x, sizeof(double) * kTuneSamples) != cudaSuccess ||
      cudaMalloc(&d_o, (size_t)maxw * kTuneSamples) != cudaSuccess ||
      cudaMalloc(&d_c, sizeof(SdmCtx) * (size_t)(2 + maxw)) != cudaSuccess ||
      cudaMalloc(&d_j, sizeof(SdmJob) * (size_t)maxw) != cudaSuccess ||
      cudaMalloc(&d_cnt, sizeof(int)) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    rc = c->cuda_fail(cudaGetLastError(), "tuner allocation");
  }
  if (!rc) {
    cudaMemcpyAsync(d_x, x.data(), sizeof(double) * kTuneSamples, cudaMemcpyHostToDevice, c->stream);
    init_contexts(d_c, 0, 1, 0, c->stream);
    std::vector<SdmJob> jobs(maxw);
    for (int i = 0; i < maxw; i++) {
      SdmJob& j = jobs[i];
      j.in = d_x;
      j.out = d_o + (size_t)i * kTuneSamples;
      j.n_in = kTuneSamples;
      j.skip_out = 0;
      j.ctx = -(1 + 1);        // scratch bank at context 1
      j.copy_from = 0;
      j.seed_state = nullptr;
      j.flags = kJobNoStore;
    }
    cudaMemcpyAsync(d_j, jobs.data(), sizeof(SdmJob) * jobs.size(), cudaMemcpyHostToDevice, c->stream);
    SdmParams Q = P;
    Q.mode = c->sdm_mode;
    Q.lanes = lanes_per_job(P);   // the width the plan's capped launches use
    // warm-up
    if (launch_sdm_jobs(Q, d_j, sms * jpc, d_cnt, d_c, c->d_status, 0, c->stream) != 0)
      rc = c->cuda_fail(cudaGetLastError(), "tuner launch");
    for (int lv : kTuneWarpLevels) {
      if (rc) break;
      const int w = lv * sms * jpc;            // resident jobs (lv warps per SM)
      cudaEventRecord(e0, c->stream);
      if (launch_sdm_jobs(Q, d_j, w, d_cnt, d_c, c->d_status, 0, c->stream) != 0) {
        rc = c->cuda_fail(cudaGetLastError(), "tuner launch");
        break;
      }
      cudaEventRecord(e1, c->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        rc = c->cuda_fail(cudaGetLastError(), "tuner run");
        break;
      }
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      c->launches++;
      out->warps.push_back(w);
      out->rate.push_back((double)w * (double)kTuneSamples / (ms > 0 ? ms * 1e-3 : 1e-9));
    }
    if (!rc) rc = c->check_status();
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (d_x) cudaFree(d_x);
  if (d_o) cudaFree(d_o);
  if (d_c) cudaFree(d_c);
  if (d_j) cudaFree(d_j);
  if (d_cnt) cudaFree(d_cnt);
  return rc;
}

// Modelled SDM-phase seconds of the plan's classes at one segment length and
// resident-warp budget.
double model_seconds(const std::vector<StreamPlan>& st, const std::vector<SdmClass>& cls,
                     const std::vector<const TuneCurve*>& curves, long long seg_len, int slots) {
  const size_t nc = cls.size();
  std::vector<double> W(nc, 0.0), Lmax(nc, 0.0);
  long long J = 0;
  for (const StreamPlan& s0 : st) {
    if (s0.precorr) continue;
    StreamPlan s = s0;
    layout_stream(s, seg_len);
    segment_io(s);
    for (int k = 0; k < s.S; k++) {
      W[s.cls] += (double)s.in_cnt[k] * s.d.channels;
      Lmax[s.cls] = std::max(Lmax[s.cls], (double)s.in_cnt[k]);
    }
    J += (long long)s.S * s.d.channels;
  }
  long long cap = slots;
  for (size_t k = 0; k < nc; k++) cap = std::max<long long>(cap, (long long)slots * sdm_jobs_per_cta(cls[k].P));
  const double w = (double)std::min<long long>(J, cap);   // resident jobs
  double work = 0.0, tail = 0.0;
  for (size_t k = 0; k < nc; k++) {
    const double R = curves[k]->at(w);
    const double per_job = R / w;
    work += W[k] / R;
    const double longest = Lmax[k] / per_job;
    tail = std::max(tail, J > cap ? 0.5 * longest : longest);
  }
  return J > cap ? work + tail : std::max(work, tail);
}

// ---- plan construction -----------------------------------------------------

int upload_stream_rows(dsdgpu_plan* pl, StreamPlan& s, cudaStream_t stream);

int capture_graphs(dsdgpu_plan* pl) {
  dsdgpu_context* c = pl->c;
  cudaStream_t m = c->stream;
  cudaGraph_t g = nullptr;
  // graph 1: FIR chains and boundary RMS
  if (cudaStreamBeginCapture(m, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return c->cuda_fail(cudaGetLastError(), "graph capture");
  int rc = DSDGPU_OK;
  for (StreamPlan& s : pl->st) {
    const double gain = s.d.gain;
    const int apply = gain != 1.0 ? 1 : 0;
    const int nch = s.d.channels;
    int r = 0;
    if (s.precorr && s.dsd_mode) {
      // PreCorr on DoP input: the same stages with FP32 output, no clip
      // (the pipeline narrows their FP64 output ahead of the walk)
      float* w = pl->d_f32 + s.f32_off;
      const long long cnt = 16 * s.d.frames;
      if (s.dsd_mode == 1) {
        r = launch_dop_unpack(pl->d_pcm + s.pcm_off, s.pcm_stride, s.d.frames, nch,
                              pl->d_bits + s.bits_off, s.bits_stride, m);
        if (!r && s.lp >= 0) {
          const LpSet& L = pl->lps[s.lp];
          r = launch_lowpass_fresh(pl->d_lp + L.lut_off, pl->d_lp + L.taps_off, L.ntaps, L.W,
                                   pl->d_bits + s.bits_off, s.bits_stride, (long long)s.n_fir,
                                   pl->d_lphist, nch, gain, 0.0, w, s.f32_stride, c->num_sms, m);
        } else if (!r) {
          r = launch_boxcar_fresh_f32(pl->d_bits + s.bits_off, s.bits_stride, (long long)s.n_fir,
                                      pl->d_boxhist, s.box_taps, nch, gain, 0.0, w, s.f32_stride,
                                      m);
        }
      } else if (s.dsd_mode == 2) {
        const size_t in_stride = align_up((size_t)cnt, 64);
        r = launch_dop_unpack_f32(pl->d_pcm + s.pcm_off, s.pcm_stride, s.d.frames, nch,
                                  pl->d_f32 + s.f32in_off, in_stride, m);
        if (!r)
          r = launch_fir_chain(s.F, s.fir_smem, pl->d_f32 + s.f32in_off, in_stride, cnt,
                               pl->d_hist, w, s.f32_stride, gain, 0.0, apply, 0, nch, m);
      } else {
        const size_t bs = align_up((size_t)cnt, 256), fs = align_up((size_t)cnt, 32);
        const size_t row = align_up((size_t)cnt / 2 + 1, 32);
        r = launch_dop_unpack(pl->d_pcm + s.pcm_off, s.pcm_stride, s.d.frames, nch,
                              pl->d_dn_bits, bs, m);
        if (!r)
          r = launch_boxcar_fresh(pl->d_dn_bits, bs, cnt, pl->d_boxhist, s.box_taps, nch, 1.0,
                                  0.0, pl->d_dn_box, fs, m);
        if (!r)
          r = launch_decim_f64_fresh(pl->d_dn_box, fs, cnt, s.down_stages, nch, pl->d_dn_pp, row,
                                     pl->d_dn_dly, gain, 0.0, apply, 0, nullptr, s.f32_stride, m,
                                     w);
      }
    } else if (s.dsd_mode == 1) {
      // same-rate DSD: DoP unpack into the decision rows (free until the
      // assembly writes them), the boxcar with the constant gain
      r = launch_dop_unpack(pl->d_pcm + s.pcm_off, s.pcm_stride, s.d.frames, nch,
                            pl->d_bits + s.bits_off, s.bits_stride, m);
      if (!r && s.lp >= 0) {
        const LpSet& L = pl->lps[s.lp];
        r = launch_lowpass_fresh(pl->d_lp + L.lut_off, pl->d_lp + L.taps_off, L.ntaps, L.W,
                                 pl->d_bits + s.bits_off, s.bits_stride, (long long)s.n_fir,
                                 pl->d_lphist, nch, gain, 0.0, pl->d_fir + s.fir_off,
                                 s.fir_stride, c->num_sms, m);
      } else if (!r) {
        r = launch_boxcar_fresh(pl->d_bits + s.bits_off, s.bits_stride, (long long)s.n_fir,
                                pl->d_boxhist, s.box_taps, nch, gain, 0.0, pl->d_fir + s.fir_off,
                                s.fir_stride, m);
      }
    } else if (s.dsd_mode == 2) {
      // DSD up: +-1 floats at the input rate through the FIR chain
      r = launch_dop_unpack_f32(pl->d_pcm + s.pcm_off, s.pcm_stride, s.d.frames, nch,
                                pl->d_f32 + s.f32_off, s.f32_stride, m);
      if (!r)
        r = launch_fir_chain(s.F, s.fir_smem, pl->d_f32 + s.f32_off, s.f32_stride,
                             16 * s.d.frames, pl->d_hist, pl->d_fir + s.fir_off, s.fir_stride,
                             gain, 0.0, apply, s.d.soft_clip, nch, m);
    } else if (s.dsd_mode == 3) {
      // DSD down (the pipeline's rate-conversion branch with DSD in): unpack,
      // the boxcar at gain 1, the FP64 chain with the gain and the clip
      const long long cnt = 16 * s.d.frames;
      const size_t bs = align_up((size_t)cnt, 256), fs = align_up((size_t)cnt, 32);
      const size_t row = align_up((size_t)cnt / 2 + 1, 32);
      r = launch_dop_unpack(pl->d_pcm + s.pcm_off, s.pcm_stride, s.d.frames, nch, pl->d_dn_bits,
                            bs, m);
      if (!r)
        r = launch_boxcar_fresh(pl->d_dn_bits, bs, cnt, pl->d_boxhist, s.box_taps, nch, 1.0, 0.0,
                                pl->d_dn_box, fs, m);
      if (!r)
        r = launch_decim_f64_fresh(pl->d_dn_box, fs, cnt, s.down_stages, nch, pl->d_dn_pp, row,
                                   pl->d_dn_dly, gain, 0.0, apply, s.d.soft_clip,
                                   pl->d_fir + s.fir_off, s.fir_stride, m);
    } else if (s.precorr) {
      // PreCorr streams: FP32 out (the values the walk reads), no soft clip
      // ahead of PreCorr (the pipeline in that mode, src/engine.c:557-559)
      r = launch_fir_chain(s.F, s.fir_smem, pl->d_pcm + s.pcm_off, s.pcm_stride, s.d.frames,
                           pl->d_hist, pl->d_f32 + s.f32_off, s.f32_stride, gain, 0.0, apply, 0,
                           nch, m);
    } else {
      r = launch_fir_chain(s.F, s.fir_smem, pl->d_pcm + s.pcm_off, s.pcm_stride, s.d.frames,
                           pl->d_hist, pl->d_fir + s.fir_off, s.fir_stride, gain, 0.0, apply,
                           s.d.soft_clip, nch, m);
    }
    if (r != 0) {
      rc = DSDGPU_ERR_CUDA;
      break;
    }
  }
  if (!rc && !pl->centers.empty()) {
    if (launch_das_rms(pl->d_fir, pl->d_centers, (int)pl->centers.size(), pl->d_rms, m) != 0)
      rc = DSDGPU_ERR_CUDA;
    else if (cudaMemcpyAsync(pl->h_rms, pl->d_rms, sizeof(double) * pl->centers.size(),
                             cudaMemcpyDeviceToHost, m) != cudaSuccess)
      rc = DSDGPU_ERR_CUDA;
  }
  cudaError_t e = cudaStreamEndCapture(m, &g);
  if (rc || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return c->cuda_fail(cudaGetLastError(), "graph 1 capture");
  }
  e = cudaGraphInstantiate(&pl->g1, g, 0);
  cudaGraphDestroy(g);
  g = nullptr;
  if (e != cudaSuccess) return c->cuda_fail(e, "graph 1 instantiate");

  // graph 2: SDM per class, concurrent on forked streams (every side stream
  // waits on one fork point; the main stream joins them all at the end)
  if (cudaStreamBeginCapture(m, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return c->cuda_fail(cudaGetLastError(), "graph capture");
  const bool forked = pl->cls.size() + pl->pcls.size() > 1;
  if (forked) {
    cudaEventRecord(pl->fork, m);
    for (SdmClass& K : pl->cls) cudaStreamWaitEvent(K.side, pl->fork, 0);
    for (PcClass& Q : pl->pcls) cudaStreamWaitEvent(Q.side, pl->fork, 0);
  }
  for (size_t k = 0; k < pl->cls.size() && !rc; k++) {
    SdmClass& K = pl->cls[k];
    SdmParams P = K.P;   // its lanes: the option's, or the width chosen with the job slots
    P.mode = c->sdm_mode;
    if (launch_sdm_jobs(P, pl->d_jobs + K.job_first, K.njobs, pl->d_counters + k, pl->d_ctx,
                        c->d_status, K.grid, forked ? K.side : m) != 0)
      rc = DSDGPU_ERR_CUDA;
  }
  for (size_t q = 0; q < pl->pcls.size() && !rc; q++) {
    PcClass& Q = pl->pcls[q];
    if (launch_precorr_batch(Q.order, Q.a, Q.g, Q.limit, pl->d_pctab + q * precorr_table_floats(),
                             pl->d_pcrows + Q.row_first, Q.nrows, forked ? Q.side : m) != 0)
      rc = DSDGPU_ERR_CUDA;
  }
  if (forked) {
    for (SdmClass& K : pl->cls) {
      cudaEventRecord(K.join, K.side);
      cudaStreamWaitEvent(m, K.join, 0);
    }
    for (PcClass& Q : pl->pcls) {
      cudaEventRecord(Q.join, Q.side);
      cudaStreamWaitEvent(m, Q.join, 0);
    }
  }
  e = cudaStreamEndCapture(m, &g);
  if (rc || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return c->cuda_fail(cudaGetLastError(), "graph 2 capture");
  }
  e = cudaGraphInstantiate(&pl->g2, g, 0);
  cudaGraphDestroy(g);
  g = nullptr;
  if (e != cudaSuccess) return c->cuda_fail(e, "graph 2 instantiate");

  // graph 3: seams over all boundaries, then per stream assembly and packing
  if (cudaStreamBeginCapture(m, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return c->cuda_fail(cudaGetLastError(), "graph capture");
  if (!rc && !pl->tasks.empty()) {
    const int r = launch_das_seams(pl->d_tasks, (int)pl->tasks.size(), pl->max_ovl, pl->d_qfir,
                                   pl->d_bp, pl->d_seam_scr, m);
    if (r) rc = DSDGPU_ERR_CUDA;
  }
  for (StreamPlan& s : pl->st) {
    if (rc) break;
    const int nch = s.d.channels;
    // PreCorr streams wrote their decision rows directly
    if (!s.precorr &&
        launch_das_assemble(pl->d_pieces + s.piece_first, s.npieces, pl->d_bp + s.bp_base,
                            pl->d_bits + s.bits_off, s.bits_stride, nch, s.S,
                            pl->d_segbuf + s.segbuf_first, m) != 0) {
      rc = DSDGPU_ERR_CUDA;
      break;
    }
    const size_t n = (size_t)s.final_count;
    if (pl->fmt == DSDGPU_OUT_DOP) {
      if (launch_pack_dop(pl->d_bits + s.bits_off, s.bits_stride, nch, n / 16, 0,
                          pl->d_out + s.out_off, c->num_sms, m) != 0)
        rc = DSDGPU_ERR_CUDA;
    } else if (pl->fmt == DSDGPU_OUT_NATIVE) {
      if (launch_pack_native(pl->d_bits + s.bits_off, s.bits_stride, nch, n,
                             pl->d_out + s.out_off, s.out_stride, c->num_sms, m) != 0)
        rc = DSDGPU_ERR_CUDA;
    }
  }
  e = cudaStreamEndCapture(m, &g);
  if (rc || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return c->cuda_fail(cudaGetLastError(), "graph 3 capture");
  }
  e = cudaGraphInstantiate(&pl->g3, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return c->cuda_fail(e, "graph 3 instantiate");
  return DSDGPU_OK;
}

// Every buffer range the stream's rows let a kernel touch lies inside the
// stream's own part of the arena: FIR rows, segment rows, stitched rows.
bool rows_in_bounds(const dsdgpu_plan* pl, const StreamPlan& s) {
  for (int k = 0; k < s.S; k++) {
    if (s.in_start[k] < 0 || s.in_cnt[k] < 0 || (size_t)(s.in_start[k] + s.in_cnt[k]) > s.n_fir)
      return false;
    if (s.seg_off[k] + (size_t)s.in_cnt[k] > s.seg_row) return false;
  }
  for (int i = 0; i < s.ntasks; i++) {
    const SeamTask& t = pl->tasks[s.task_first + i];
    const int b = t.boundary - s.bp_base;
    if (b < 1 || b >= s.S || t.prev_seg < 0 || t.prev_seg >= s.S || t.ovl_len < 0) return false;
    if (t.prev_off < 0 || t.prev_off + t.ovl_len > s.in_cnt[t.prev_seg]) return false;
    if (t.ovl_len > s.in_cnt[b] || t.ovl_len > pl->max_ovl) return false;
  }
  for (int i = 0; i < s.npieces; i++) {
    const AssemblePiece& p = pl->pieces[s.piece_first + i];
    if (p.seg < 0 || p.seg >= s.S || p.base < 0 || p.end_base > (long long)s.bits_stride)
      return false;
    if (p.next_stitched &&
        (p.next_seg < 0 || p.next_seg >= s.S || p.next_base < 0 ||
         (size_t)p.next_base + s.overlap > s.bits_stride))
      return false;
  }
  return s.final_count >= 0 && (size_t)s.final_count <= s.bits_stride;
}

// Job, seam-task, piece and segment-buffer rows of one stream for its current
// layout (the rows' positions in the tables are fixed at plan creation).
// Returns false when a row would reach outside the stream's buffers.
bool fill_stream_rows(dsdgpu_plan* pl, StreamPlan& s) {
  if (s.precorr) return true;   // no segments: its rows are the PreCorr rows
  segment_io(s);
  const int nch = s.d.channels;
  s.seg_off.assign(s.S, 0);
  size_t row = 0;
  for (int k = 0; k < s.S; k++) {
    s.seg_off[k] = row;
    row += align_up((size_t)s.in_cnt[k], 256);
  }
  for (int ch = 0; ch < nch; ch++)
    for (int k = 0; k < s.S; k++)
      pl->segbuf[s.segbuf_first + (size_t)ch * s.S + k].ptr =
          pl->d_seg + s.seg_off0 + (size_t)ch * s.seg_row + s.seg_off[k];
  // segment buffer offsets inside each channel row
  for (int k = 0; k < s.S; k++) {
    for (int ch = 0; ch < nch; ch++) {
      SdmJob& j = pl->jobs[s.job_index[ch * s.S + k]];
      j.in = pl->d_fir + s.fir_off + (size_t)ch * s.fir_stride + s.in_start[k];
      j.out = pl->d_seg + s.seg_off0 + (size_t)ch * s.seg_row + s.seg_off[k];
      j.n_in = s.in_cnt[k];
      int64_t skip, out, np;
      sdm_plan_steps(s.lat, 0, s.in_cnt[k], s.discard[k], &skip, &out, &np);
      j.skip_out = skip;
      j.ctx = -(1 + pl->cls[s.cls].scratch_first);
      j.copy_from = 0;
      j.seed_state = k == 0 ? nullptr : pl->d_seed;
      j.flags = kJobNoStore;
    }
  }
  std::vector<SeamPlan> sp;
  std::vector<AssemblePiece> pc;
  const char* err = nullptr;
  if (das_stream_plan(s.S, s.seg_out.data(), s.size, s.overlap, false, sp, pc, &s.final_count,
                      &err) != 0)
    return false;
  for (size_t i = 0; i < sp.size(); i++) {
    SeamTask& t = pl->tasks[s.task_first + i];
    t.boundary = s.bp_base + sp[i].boundary;
    t.ovl_len = sp[i].ovl_len;
    t.prev_seg = sp[i].prev_seg;
    t.prev_off = sp[i].prev_off;
    t.lat = s.lat;
    t.prev = pl->d_seg + s.seg_off0 + s.seg_off[sp[i].prev_seg] + sp[i].prev_off;
    t.next = pl->d_seg + s.seg_off0 + s.seg_off[sp[i].boundary];
  }
  for (size_t i = 0; i < pc.size(); i++) pl->pieces[s.piece_first + i] = pc[i];
  return sp.size() == (size_t)s.ntasks && pc.size() == (size_t)s.npieces && rows_in_bounds(pl, s);
}

}  // namespace

extern "C" {

int dsdgpu_plan_create(dsdgpu_context_t* c, const dsdgpu_stream_desc_t* streams, int nstreams,
                       int64_t seg_len, int output_format, uint64_t max_device_bytes,
                       dsdgpu_plan_t** out) {
  if (!c || !streams || nstreams < 1 || !out) return DSDGPU_ERR_ARG;
  *out = nullptr;
  if (output_format < DSDGPU_OUT_BITS || output_format > DSDGPU_OUT_NATIVE)
    return c->fail(DSDGPU_ERR_ARG, "bad output format");
  if (seg_len < 0) return c->fail(DSDGPU_ERR_ARG, "negative segment length");
  cudaSetDevice(c->device);
  dsdgpu_plan* pl = new (std::nothrow) dsdgpu_plan();
  if (!pl) return DSDGPU_ERR_NOMEM;
  pl->c = c;
  pl->fmt = output_format;
  auto bail = [&](int rc) {
    delete pl;
    return rc;
  };

  // ---- streams and parameter classes ----
  pl->st.resize(nstreams);
  for (int i = 0; i < nstreams; i++) {
    StreamPlan& s = pl->st[i];
    s.d = streams[i];
    const dsdgpu_stream_desc_t& d = s.d;
    if (d.channels < 1 || d.channels > kBatchMaxChannels)
      return bail(c->fail(DSDGPU_ERR_ARG, "stream channels out of range (1..8)"));
    if (d.frames < 1) return bail(c->fail(DSDGPU_ERR_ARG, "stream without frames"));
    if (d.sdm_mode != DSDGPU_SDM_TRELLIS && d.sdm_mode != DSDGPU_SDM_PRECORR)
      return bail(c->fail(DSDGPU_ERR_ARG, "bad sdm mode"));
    s.precorr = d.sdm_mode == DSDGPU_SDM_PRECORR;
    if (d.fs_in <= 0 || d.fs_out <= 0) return bail(c->fail(DSDGPU_ERR_ARG, "bad rate"));
    // DoP input at a DSD rate (the pipeline's rule): the same-rate re-encode
    // or the FIR chain on +-1 floats to a higher DSD rate
    if (d.fs_in >= kDsd64Rate) {
      s.dsd_mode = d.fs_out == d.fs_in ? 1 : (d.fs_out > d.fs_in ? 2 : 3);
    }
    if (d.samerate_filter != DSDGPU_SAMERATE_BOXCAR && d.samerate_filter != DSDGPU_SAMERATE_LOWPASS)
      return bail(c->fail(DSDGPU_ERR_ARG, "bad same-rate filter"));
    if (s.dsd_mode == 1 && d.samerate_filter == DSDGPU_SAMERATE_LOWPASS) {
      // the pipeline's same-rate FIR mode (src/engine.c:168-181, 505-523)
      int k = -1;
      for (size_t j = 0; j < pl->lps.size() && k < 0; j++)
        if (pl->lps[j].fs == (unsigned)d.fs_in) k = (int)j;
      if (k < 0) {
        LpSet L;
        L.fs = (unsigned)d.fs_in;
        L.ntaps = lowpass_tables(L.fs, 50000.0, 127, L.lut, L.taps, &L.W);
        pl->lps.push_back(std::move(L));
        k = (int)pl->lps.size() - 1;
      }
      s.lp = k;
    }
    if (s.dsd_mode == 3) {
      // the decimation chain's plan (dsdgpu_decim_setup); boxcar 0 = a one-tap
      // mean, the identity on +-1 input (the plugin's DAS FIR phase has none)
      unsigned r = (unsigned)d.fs_in / (unsigned)d.fs_out;
      if ((unsigned)d.fs_in % (unsigned)d.fs_out || (r & (r - 1)))
        return bail(c->fail(DSDGPU_ERR_ARG, "decimation needs fs_in = fs_out * 2^k"));
      while (r > 1) {
        s.down_stages++;
        r >>= 1;
      }
      if (s.down_stages > kMaxStages) return bail(c->fail(DSDGPU_ERR_ARG, "too many stages"));
      s.box_taps = d.boxcar_taps > 0 ? d.boxcar_taps : 1;
      if (d.boxcar_taps < 0 || s.box_taps > 256)
        return bail(c->fail(DSDGPU_ERR_ARG, "boxcar taps out of range (1..256)"));
      s.n_fir = (16 * (size_t)d.frames) >> s.down_stages;
    } else if (s.dsd_mode == 1) {
      // engine_init's same-rate boxcar (src/engine.c:130-147), 0 = the rate's default
      s.box_taps = d.boxcar_taps > 0 ? d.boxcar_taps : samerate_boxcar_taps((unsigned)d.fs_in);
      if (d.boxcar_taps < 0 || s.box_taps > 256)
        return bail(c->fail(DSDGPU_ERR_ARG, "boxcar taps out of range (1..256)"));
      s.n_fir = 16 * (size_t)d.frames;
    } else {
      if (d.boxcar_taps < 0 || d.boxcar_taps > 64)
        return bail(c->fail(DSDGPU_ERR_ARG, "boxcar taps out of range"));
      if (build_chain_const((unsigned)d.fs_in, (unsigned)d.fs_out, d.boxcar_taps, &s.F) != 0)
        return bail(c->fail(DSDGPU_ERR_ARG, "unsupported rate pair (upsampling by a power of two only)"));
      s.fir_smem = chain_smem_bytes(s.F);
      if (s.fir_smem > (size_t)kFirMaxSmem)
        return bail(c->fail(DSDGPU_ERR_UNSUPPORTED, "fir tile does not fit shared memory"));
      s.n_fir = (size_t)d.frames * (s.dsd_mode == 2 ? 16 : 1) * (size_t)s.F.ratio;
    }
    if (s.precorr) {
      // the checks of dsdgpu_precorr_setup; K, depth and lat are not used
      const dsdgpu_sdm_params_t& q = d.sdm;
      if (q.order < 2 || q.order > kMaxOrder)
        return bail(c->fail(DSDGPU_ERR_ARG, "NTF order out of range (2..10)"));
      if (!(q.state_limit >= 0.0)) return bail(c->fail(DSDGPU_ERR_ARG, "state limit must be >= 0"));
      s.cls = -1;
      int k = -1;
      for (size_t j = 0; j < pl->pcls.size() && k < 0; j++) {
        const PcClass& Q = pl->pcls[j];
        bool same = Q.order == q.order && Q.limit == q.state_limit;
        for (int i = 0; same && i < q.order; i++) same = Q.a[i] == q.a[i] && Q.g[i] == q.g[i];
        if (same) k = (int)j;
      }
      if (k < 0) {
        PcClass Q;
        Q.order = q.order;
        for (int i = 0; i < q.order; i++) {
          Q.a[i] = q.a[i];
          Q.g[i] = q.g[i];
        }
        Q.limit = q.state_limit;
        pl->pcls.push_back(Q);
        k = (int)pl->pcls.size() - 1;
      }
      s.pc_cls = k;
      continue;
    }
    SdmParams P;
    const char* err = nullptr;
    const int prc = sdm_params_from_abi(&d.sdm, &P, &err);
    if (prc) return bail(c->fail(prc, err));
    P.lanes = c->sdm_lanes;   // part of the class: the plan's job slots depend on it
    s.lat = P.lat;
    s.overlap = 64 * (size_t)P.lat;
    int k = -1;
    for (size_t q = 0; q < pl->cls.size(); q++)
      if (memcmp(&pl->cls[q].P, &P, sizeof P) == 0) { k = (int)q; break; }
    if (k < 0) {
      SdmClass K;
      K.P = P;
      pl->cls.push_back(K);
      k = (int)pl->cls.size() - 1;
    }
    s.cls = k;
  }

  const int sms = c->num_sms > 0 ? c->num_sms : 1;
  // ---- segment length and launch shape ----
  if (seg_len > 0) {
    pl->seg_len = seg_len;
    pl->bps = 16;
  } else {
    std::lock_guard<std::mutex> lock(tune_mutex());
    std::vector<const TuneCurve*> curves;
    for (SdmClass& K : pl->cls) {
      const std::string key = class_key(K.P, c->device) + "#" + std::to_string(c->sdm_mode);
      auto it = tune_cache().find(key);
      if (it == tune_cache().end()) {
        TuneCurve tc;
        const int rc = measure_curve(c, K.P, &tc);
        if (rc) return bail(rc);
        it = tune_cache().emplace(key, tc).first;
      }
      curves.push_back(&it->second);
    }
    double best = 1e300;
    for (long long sl : kTuneSegLens)
      for (int b : kTuneBps) {
        const double t = model_seconds(pl->st, pl->cls, curves, sl, b * sms);
        if (t < best * 0.999) {
          best = t;
          pl->seg_len = sl;
          pl->bps = b;
        }
      }
    pl->predicted_ms = best * 1e3;
  }

  // ---- layouts, sizes, table positions ----
  size_t pcm_total = 0, fir_total = 0, seg_total = 0, bits_total = 0, out_total = 0;
  size_t f32_total = 0;
  for (StreamPlan& s : pl->st) {
    const int nch = s.d.channels;
    s.pcm_stride = align_up((size_t)s.d.frames, 64);
    s.pcm_off = pcm_total;
    pcm_total += s.pcm_stride * nch;
    std::vector<SeamPlan> sp;
    std::vector<AssemblePiece> pc;
    if (s.precorr) {
      s.S = 0;
      s.f32_stride = align_up(s.n_fir, 64);
      s.f32_off = f32_total;
      f32_total += s.f32_stride * nch;
      if (s.dsd_mode == 2) {
        s.f32in_off = f32_total;
        f32_total += align_up(16 * (size_t)s.d.frames, 64) * nch;
      }
      s.bits_stride = align_up(s.n_fir, 256);
      s.bits_off = bits_total;
      bits_total += s.bits_stride * nch;
      s.final_count = (long long)s.n_fir;   // one decision per input, no latency
    } else {
      if (s.dsd_mode == 2) {
        s.f32_stride = align_up(16 * (size_t)s.d.frames, 64);
        s.f32_off = f32_total;
        f32_total += s.f32_stride * nch;
      }
      layout_stream(s, pl->seg_len);
      segment_io(s);
      s.fir_stride = align_up(s.n_fir, 32);
      s.fir_off = fir_total;
      fir_total += s.fir_stride * nch;
      // a reposition moves samples between neighbouring segments but keeps their
      // sum: 256 bytes of slack per segment cover the per-segment alignment
      size_t row = 0;
      for (int k = 0; k < s.S; k++) row += align_up((size_t)s.in_cnt[k], 256);
      s.seg_row = row + 256 * (size_t)s.S;
      s.seg_off0 = seg_total;
      seg_total += s.seg_row * nch;
      s.bits_stride = align_up(s.n_fir, 256);
      s.bits_off = bits_total;
      bits_total += s.bits_stride * nch;
      // final count does not depend on the seams or on the reposition
      const char* err = nullptr;
      if (das_stream_plan(s.S, s.seg_out.data(), s.size, s.overlap, false, sp, pc, &s.final_count,
                          &err) != 0)
        return bail(c->fail(DSDGPU_ERR_UNSUPPORTED, err));
    }
    const size_t n = (size_t)s.final_count;
    if (pl->fmt == DSDGPU_OUT_DOP) {
      s.out_stride = (n / 16) * 3 * (size_t)nch;
      s.out_bytes = s.out_stride;
    } else if (pl->fmt == DSDGPU_OUT_NATIVE) {
      s.out_stride = (n + 7) / 8;
      s.out_bytes = s.out_stride * (size_t)nch;
    } else {
      s.out_stride = s.bits_stride;
      s.out_bytes = n * (size_t)nch;
    }
    if (pl->fmt != DSDGPU_OUT_BITS) {
      s.out_off = out_total;
      out_total += align_up(s.out_stride * (pl->fmt == DSDGPU_OUT_NATIVE ? nch : 1), 256);
    }
    s.ntasks = (int)sp.size();
    s.npieces = (int)pc.size();
    for (const SeamPlan& t : sp) pl->max_ovl = std::max(pl->max_ovl, t.ovl_len);
    pl->out_samples += (long long)n * nch;
    if (!s.precorr && s.d.reposition && s.S > 2)
      das_reposition_centers(s.nom_start, s.n_fir, s.centers, s.which);
  }
  // PreCorr rows: class-major, then stream, channel (pointers set with the arena)
  for (size_t q = 0; q < pl->pcls.size(); q++) {
    PcClass& Q = pl->pcls[q];
    Q.row_first = (int)pl->pcrows.size();
    for (StreamPlan& s : pl->st) {
      if (!s.precorr || s.pc_cls != (int)q) continue;
      for (int ch = 0; ch < s.d.channels; ch++) pl->pcrows.push_back(PcBatchRow{nullptr, 0, nullptr});
      Q.samples += (long long)s.n_fir * s.d.channels;
    }
    Q.nrows = (int)pl->pcrows.size() - Q.row_first;
    pl->pc_samples += Q.samples;
  }
  // jobs: class-major, then stream, segment, channel
  int njobs = 0;
  for (size_t k = 0; k < pl->cls.size(); k++) {
    SdmClass& K = pl->cls[k];
    K.job_first = njobs;
    for (StreamPlan& s : pl->st) {
      if (s.cls != (int)k) continue;
      s.job_index.assign((size_t)s.S * s.d.channels, -1);
      for (int q = 0; q < s.S; q++)
        for (int ch = 0; ch < s.d.channels; ch++) {
          s.job_index[(size_t)ch * s.S + q] = njobs++;
          K.samples += s.in_cnt[q];
          K.max_job = std::max<long long>(K.max_job, s.in_cnt[q]);
        }
    }
    K.njobs = njobs - K.job_first;
    pl->sdm_samples += K.samples;
  }
  // resident-warp budget split over the classes in proportion to their work
  const int slots = pl->bps * sms;
  int nscratch = 0;
  for (SdmClass& K : pl->cls) {
    int gsz = (int)std::llround((double)slots * (double)K.samples / (double)std::max(1LL, pl->sdm_samples));
    gsz = std::max(1, gsz);
    // lanes per job (unless the option fixes them): the default half-warp
    // while the class's jobs fit one wave of its warps (a small trellis's
    // step is a chain of dependent operations, and an FP64 warp instruction
    // costs the same with 2 lanes active as with 32, so the fewest jobs a
    // warp that still fit win); beyond one wave the widest width that fits,
    // else the narrowest (K = 2 over 30,058 jobs: 569 -> 1,510 DSD Msamples/s
    // at 2 lanes)
    if (K.P.lanes == 0 && (long long)K.njobs > (long long)gsz * sdm_jobs_per_cta(K.P)) {
      int best = 0;
      for (int l = 16; l >= 2; l /= 2) {
        SdmParams Q = K.P;
        Q.lanes = l;
        const int jpc = sdm_jobs_per_cta(Q);
        if (32 / jpc != l) continue;            // below the trellis's own width
        best = l;
        if ((long long)K.njobs <= (long long)gsz * jpc) break;
      }
      if (best) K.P.lanes = best;
    }
    const int jpc = sdm_jobs_per_cta(K.P);
    gsz = std::min(gsz, (K.njobs + jpc - 1) / jpc);
    K.grid = gsz;
    K.scratch_first = 1 + nscratch;
    nscratch += gsz * jpc;       // one scratch context per job slot of the launch
  }
  pl->nscratch = nscratch;
  int ntasks = 0, npieces = 0, nseg = 0, ncen = 0, nbp = 0;
  for (StreamPlan& s : pl->st) {
    s.task_first = ntasks;
    ntasks += s.ntasks;
    s.piece_first = npieces;
    npieces += s.npieces;
    s.segbuf_first = nseg;
    nseg += s.S * s.d.channels;
    s.bp_base = nbp;
    nbp += s.S;
    s.center_first = ncen;
    for (long long b : s.centers) pl->centers.push_back((long long)s.fir_off + b);
    ncen += (int)s.centers.size();
  }
  pl->nbp = nbp;
  pl->jobs.resize(njobs);
  pl->tasks.resize(ntasks);
  pl->pieces.resize(npieces);
  pl->segbuf.resize(nseg);

  // shared scratch of the DSD streams to a lower rate (the largest one's)
  size_t dn_bits = 0, dn_box = 0, dn_pp = 0;
  for (const StreamPlan& s : pl->st) {
    if (s.dsd_mode != 3) continue;
    const size_t cnt = 16 * (size_t)s.d.frames, nch = (size_t)s.d.channels;
    dn_bits = std::max(dn_bits, align_up(cnt, 256) * nch);
    dn_box = std::max(dn_box, align_up(cnt, 32) * nch);
    dn_pp = std::max(dn_pp, 2 * align_up(cnt / 2 + 1, 32) * nch);
  }

  size_t lp_total = 0;
  for (LpSet& L : pl->lps) {
    L.lut_off = lp_total;
    lp_total += L.lut.size();
    L.taps_off = lp_total;
    lp_total += L.taps.size();
  }

  // ---- device arena ----
  struct Part { void** p; size_t bytes; };
  const size_t nctx = 1 + (size_t)nscratch;
  std::vector<Part> parts = {
      {(void**)&pl->d_pcm, sizeof(float) * pcm_total},
      {(void**)&pl->d_fir, sizeof(double) * fir_total},
      {(void**)&pl->d_f32, sizeof(float) * f32_total},
      {(void**)&pl->d_pctab, sizeof(float) * precorr_table_floats() * pl->pcls.size()},
      {(void**)&pl->d_pcrows, sizeof(PcBatchRow) * pl->pcrows.size()},
      {(void**)&pl->d_boxhist, boxcar_hist_bytes(kBatchMaxChannels)},
      {(void**)&pl->d_dn_bits, dn_bits},
      {(void**)&pl->d_dn_box, sizeof(double) * dn_box},
      {(void**)&pl->d_dn_pp, sizeof(double) * dn_pp},
      {(void**)&pl->d_dn_dly, sizeof(double) * 62 * kBatchMaxChannels},
      {(void**)&pl->d_lp, sizeof(double) * lp_total},
      {(void**)&pl->d_lphist, lowpass_hist_bytes(kBatchMaxChannels)},
      {(void**)&pl->d_seg, seg_total},
      {(void**)&pl->d_bits, bits_total},
      {(void**)&pl->d_out, out_total},
      {(void**)&pl->d_ctx, sizeof(SdmCtx) * nctx},
      {(void**)&pl->d_jobs, sizeof(SdmJob) * (size_t)njobs},
      {(void**)&pl->d_tasks, sizeof(SeamTask) * (size_t)std::max(1, ntasks)},
      {(void**)&pl->d_pieces, sizeof(AssemblePiece) * (size_t)std::max(1, npieces)},
      {(void**)&pl->d_segbuf, sizeof(SegBuf) * (size_t)nseg},
      {(void**)&pl->d_bp, sizeof(int) * (size_t)nbp},
      {(void**)&pl->d_counters, sizeof(int) * pl->cls.size()},
      {(void**)&pl->d_seed, sizeof(double) * kMaxOrder},
      {(void**)&pl->d_hist, sizeof(float) * kHistory * kBatchMaxChannels},
      {(void**)&pl->d_qfir, sizeof(double) * 255},
      {(void**)&pl->d_centers, sizeof(long long) * (size_t)std::max(1, ncen)},
      {(void**)&pl->d_rms, sizeof(double) * (size_t)std::max(1, ncen)},
      {(void**)&pl->d_seam_scr, das_seam_global_bytes(pl->max_ovl) * (size_t)ntasks},
  };
  size_t total = 0;
  for (const Part& p : parts) total += align_up(p.bytes, 256);
  pl->arena_bytes = total;
  if (max_device_bytes && total > max_device_bytes)
    return bail(c->fail(DSDGPU_ERR_TOO_LARGE, "plan exceeds the device-memory limit"));
  cudaError_t e = cudaMalloc(&pl->d_arena, total);
  if (e != cudaSuccess) return bail(c->cuda_fail(e, "plan arena allocation"));
  {
    size_t off = 0;
    for (const Part& p : parts) {
      *p.p = (uint8_t*)pl->d_arena + off;
      off += align_up(p.bytes, 256);
    }
  }
  if (pl->fmt == DSDGPU_OUT_BITS) pl->d_out = pl->d_bits;
  if (!pl->centers.empty() &&
      cudaMallocHost(&pl->h_rms, sizeof(double) * pl->centers.size()) != cudaSuccess)
    return bail(c->cuda_fail(cudaGetLastError(), "pinned rms buffer"));

  // ---- tables ----
  for (StreamPlan& s : pl->st)
    if (!fill_stream_rows(pl, s))
      return bail(c->fail(DSDGPU_ERR_STATE, "plan rows out of the stream's buffers"));
  cudaStream_t m = c->stream;
  double q2[255];
  pop_fir_times_two(q2);
  cudaMemcpyAsync(pl->d_qfir, q2, sizeof q2, cudaMemcpyHostToDevice, m);
  cudaMemsetAsync(pl->d_seed, 0, sizeof(double) * kMaxOrder, m);
  cudaMemsetAsync(pl->d_hist, 0, sizeof(float) * kHistory * kBatchMaxChannels, m);
  cudaMemsetAsync(pl->d_boxhist, 0, boxcar_hist_bytes(kBatchMaxChannels), m);
  cudaMemsetAsync(pl->d_dn_dly, 0, sizeof(double) * 62 * kBatchMaxChannels, m);
  cudaMemsetAsync(pl->d_lphist, 0, lowpass_hist_bytes(kBatchMaxChannels), m);
  for (const LpSet& L : pl->lps) {
    cudaMemcpyAsync(pl->d_lp + L.lut_off, L.lut.data(), sizeof(double) * L.lut.size(),
                    cudaMemcpyHostToDevice, m);
    cudaMemcpyAsync(pl->d_lp + L.taps_off, L.taps.data(), sizeof(double) * L.taps.size(),
                    cudaMemcpyHostToDevice, m);
    if (lowpass_prepare(L.W) != 0) return bail(c->cuda_fail(cudaGetLastError(), "lowpass attributes"));
  }
  cudaMemsetAsync(pl->d_bp, 0, sizeof(int) * (size_t)nbp, m);
  cudaMemsetAsync(pl->d_pcm, 0, sizeof(float) * pcm_total, m);
  if (!pl->jobs.empty())
    cudaMemcpyAsync(pl->d_jobs, pl->jobs.data(), sizeof(SdmJob) * pl->jobs.size(),
                    cudaMemcpyHostToDevice, m);
  if (!pl->tasks.empty())
    cudaMemcpyAsync(pl->d_tasks, pl->tasks.data(), sizeof(SeamTask) * pl->tasks.size(),
                    cudaMemcpyHostToDevice, m);
  if (!pl->pieces.empty())
    cudaMemcpyAsync(pl->d_pieces, pl->pieces.data(), sizeof(AssemblePiece) * pl->pieces.size(),
                    cudaMemcpyHostToDevice, m);
  cudaMemcpyAsync(pl->d_segbuf, pl->segbuf.data(), sizeof(SegBuf) * pl->segbuf.size(),
                  cudaMemcpyHostToDevice, m);
  if (!pl->centers.empty())
    cudaMemcpyAsync(pl->d_centers, pl->centers.data(), sizeof(long long) * pl->centers.size(),
                    cudaMemcpyHostToDevice, m);
  if (init_contexts(pl->d_ctx, 0, 1, 0, m) != 0)
    return bail(c->cuda_fail(cudaGetLastError(), "context init"));
  c->launches++;
  {
    size_t r = 0;
    for (size_t q = 0; q < pl->pcls.size(); q++)
      for (StreamPlan& s : pl->st) {
        if (!s.precorr || s.pc_cls != (int)q) continue;
        for (int ch = 0; ch < s.d.channels; ch++)
          pl->pcrows[r++] = PcBatchRow{pl->d_f32 + s.f32_off + (size_t)ch * s.f32_stride,
                                       (long long)s.n_fir,
                                       pl->d_bits + s.bits_off + (size_t)ch * s.bits_stride};
      }
    if (!pl->pcrows.empty())
      cudaMemcpyAsync(pl->d_pcrows, pl->pcrows.data(), sizeof(PcBatchRow) * pl->pcrows.size(),
                      cudaMemcpyHostToDevice, m);
    for (size_t q = 0; q < pl->pcls.size(); q++) {
      const PcClass& Q = pl->pcls[q];
      if (precorr_batch_train(Q.order, Q.a, Q.g, Q.limit, pl->d_pctab + q * precorr_table_floats(),
                              m) != 0)
        return bail(c->cuda_fail(cudaGetLastError(), "precorr table"));
      c->launches++;
    }
  }
  if (pl->cls.size() + pl->pcls.size() > 1) {
    // graph 2 forks one side stream per launch
    bool ok = cudaEventCreateWithFlags(&pl->fork, cudaEventDisableTiming) == cudaSuccess;
    for (SdmClass& K : pl->cls)
      ok = ok && cudaStreamCreateWithFlags(&K.side, cudaStreamNonBlocking) == cudaSuccess &&
           cudaEventCreateWithFlags(&K.join, cudaEventDisableTiming) == cudaSuccess;
    for (PcClass& Q : pl->pcls)
      ok = ok && cudaStreamCreateWithFlags(&Q.side, cudaStreamNonBlocking) == cudaSuccess &&
           cudaEventCreateWithFlags(&Q.join, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) return bail(c->cuda_fail(cudaGetLastError(), "class streams"));
  }
  for (cudaEvent_t& ev : pl->ev)
    if (cudaEventCreate(&ev) != cudaSuccess) return bail(c->cuda_fail(cudaGetLastError(), "events"));
  // function attributes are set outside the capture
  if (fir_chain_prepare() != 0 || (pl->max_ovl > 0 && das_seam_prepare(pl->max_ovl) != 0))
    return bail(c->cuda_fail(cudaGetLastError(), "kernel attributes"));
  int rc = c->check_status();
  if (rc) return bail(rc);
  rc = capture_graphs(pl);
  if (rc) return bail(rc);
  *out = pl;
  return DSDGPU_OK;
}

void dsdgpu_plan_destroy(dsdgpu_plan_t* pl) {
  if (!pl) return;
  if (pl->c) {
    cudaSetDevice(pl->c->device);
    cudaStreamSynchronize(pl->c->stream);
  }
  delete pl;
}

int dsdgpu_plan_info(const dsdgpu_plan_t* pl, dsdgpu_plan_info_t* info) {
  if (!pl || !info) return DSDGPU_ERR_ARG;
  memset(info, 0, sizeof *info);
  info->seg_len = pl->seg_len;
  info->jobs = (int64_t)pl->jobs.size();
  info->sdm_samples = pl->sdm_samples;
  info->out_samples = pl->out_samples;
  info->device_bytes = (int64_t)pl->arena_bytes;
  info->classes = (int32_t)pl->cls.size();
  info->blocks_per_sm = pl->bps;
  info->predicted_ms = pl->predicted_ms;
  return DSDGPU_OK;
}

int dsdgpu_plan_stream(const dsdgpu_plan_t* pl, int i, float** d_pcm, size_t* pcm_stride,
                       uint8_t** d_out, size_t* out_stride, size_t* out_samples,
                       size_t* out_bytes) {
  if (!pl || i < 0 || i >= (int)pl->st.size()) return DSDGPU_ERR_ARG;
  const StreamPlan& s = pl->st[i];
  if (d_pcm) *d_pcm = pl->d_pcm + s.pcm_off;
  if (pcm_stride) *pcm_stride = s.pcm_stride;
  if (d_out) *d_out = pl->fmt == DSDGPU_OUT_BITS ? pl->d_bits + s.bits_off : pl->d_out + s.out_off;
  if (out_stride) *out_stride = s.out_stride;
  if (out_samples) *out_samples = (size_t)s.final_count;
  if (out_bytes) *out_bytes = s.out_bytes;
  return DSDGPU_OK;
}

int dsdgpu_plan_run(dsdgpu_plan_t* pl) {
  if (!pl) return DSDGPU_ERR_ARG;
  dsdgpu_context* c = pl->c;
  cudaSetDevice(c->device);
  cudaStream_t m = c->stream;
  cudaEventRecord(pl->ev[0], m);
  cudaError_t e = cudaGraphLaunch(pl->g1, m);
  if (e != cudaSuccess) return c->cuda_fail(e, "graph 1 launch");
  cudaEventRecord(pl->ev[3], m);
  for (const StreamPlan& s : pl->st)
    c->launches += s.dsd_mode == 3 ? 3 + s.down_stages : (s.dsd_mode ? 2 : 1);
  c->launches += pl->centers.empty() ? 0 : 1;
  int rc = DSDGPU_OK;
  if (!pl->centers.empty()) {
    // the boundary RMS values are needed on the host
    e = cudaStreamSynchronize(m);
    if (e != cudaSuccess) return c->cuda_fail(e, "graph 1 run");
    std::vector<int> dirty;
    for (size_t i = 0; i < pl->st.size(); i++) {
      StreamPlan& s = pl->st[i];
      std::vector<long long> start = s.nom_start, size = s.nom_size;
      if (!s.centers.empty()) {
        std::vector<double> cur(pl->h_rms + s.center_first,
                                pl->h_rms + s.center_first + s.centers.size());
        bool quiet = false;
        for (double r : cur) quiet |= (r <= 0.005);
        if (quiet) {
          const double* row0 = pl->d_fir + s.fir_off;
          RmsEval ev = [&](const std::vector<long long>& cand, std::vector<double>& out) -> int {
            if (cand.size() > pl->cand_cap) {
              if (pl->d_cand) cudaFree(pl->d_cand);
              if (pl->d_cand_rms) cudaFree(pl->d_cand_rms);
              pl->d_cand = nullptr;
              pl->d_cand_rms = nullptr;
              pl->cand_cap = 0;
              if (cudaMalloc(&pl->d_cand, sizeof(long long) * cand.size()) != cudaSuccess ||
                  cudaMalloc(&pl->d_cand_rms, sizeof(double) * cand.size()) != cudaSuccess)
                return c->cuda_fail(cudaGetLastError(), "rms candidates");
              pl->cand_cap = cand.size();
            }
            cudaMemcpyAsync(pl->d_cand, cand.data(), sizeof(long long) * cand.size(),
                            cudaMemcpyHostToDevice, m);
            if (launch_das_rms(row0, pl->d_cand, (int)cand.size(), pl->d_cand_rms, m) != 0)
              return c->cuda_fail(cudaGetLastError(), "rms launch");
            c->launches++;
            out.resize(cand.size());
            cudaMemcpyAsync(out.data(), pl->d_cand_rms, sizeof(double) * out.size(),
                            cudaMemcpyDeviceToHost, m);
            return c->check_status();
          };
          rc = das_reposition_apply(start, size, s.n_fir, s.overlap, s.which, cur, ev);
          if (rc) return rc;
        }
      }
      if (start != s.start) {
        s.start = start;
        s.size = size;
        if (!fill_stream_rows(pl, s))
          return c->fail(DSDGPU_ERR_STATE, "repositioned rows out of the stream's buffers");
        dirty.push_back((int)i);
      }
    }
    for (int i : dirty) {
      rc = upload_stream_rows(pl, pl->st[i], m);
      if (rc) return rc;
    }
  }
  cudaEventRecord(pl->ev[1], m);
  e = cudaGraphLaunch(pl->g2, m);
  if (e != cudaSuccess) return c->cuda_fail(e, "graph 2 launch");
  cudaEventRecord(pl->ev[2], m);
  e = cudaGraphLaunch(pl->g3, m);
  if (e != cudaSuccess) return c->cuda_fail(e, "graph 3 launch");
  cudaEventRecord(pl->ev[4], m);
  size_t npc = 0;
  for (const StreamPlan& s : pl->st) npc += s.precorr ? 1 : 0;
  // per stream: assembly (trellis streams) and packing (unless BITS)
  c->launches += pl->cls.size() + pl->pcls.size() + (pl->tasks.empty() ? 0 : 1) +
                 (pl->st.size() - npc) + (pl->fmt == DSDGPU_OUT_BITS ? 0 : pl->st.size());
  c->sdm_samples += (unsigned long long)pl->sdm_samples;
  c->sdm_last_samples = (unsigned long long)pl->sdm_samples;
  rc = c->check_status();
  if (rc) return rc;
  const int pairs[4][2] = {{0, 3}, {1, 2}, {2, 4}, {0, 4}};
  for (int i = 0; i < 4; i++) {
    float t = 0.0f;
    if (cudaEventElapsedTime(&t, pl->ev[pairs[i][0]], pl->ev[pairs[i][1]]) != cudaSuccess)
      return c->cuda_fail(cudaGetLastError(), "run timing");
    pl->ms[i] = t;
  }
  pl->ran = true;
  return DSDGPU_OK;
}

int dsdgpu_plan_run_host(dsdgpu_plan_t* pl, const float* const* h_pcm, uint8_t* const* h_out) {
  if (!pl || !h_pcm || !h_out) return DSDGPU_ERR_ARG;
  dsdgpu_context* c = pl->c;
  cudaSetDevice(c->device);
  cudaStream_t m = c->stream;
  for (size_t i = 0; i < pl->st.size(); i++) {
    const StreamPlan& s = pl->st[i];
    if (!h_pcm[i] || !h_out[i]) return c->fail(DSDGPU_ERR_ARG, "null host buffer");
    const size_t fr = (size_t)s.d.frames;
    cudaError_t e = cudaMemcpy2DAsync(pl->d_pcm + s.pcm_off, s.pcm_stride * sizeof(float), h_pcm[i],
                                      fr * sizeof(float), fr * sizeof(float),
                                      (size_t)s.d.channels, cudaMemcpyHostToDevice, m);
    if (e != cudaSuccess) return c->cuda_fail(e, "pcm upload");
  }
  int rc = dsdgpu_plan_run(pl);
  if (rc) return rc;
  for (size_t i = 0; i < pl->st.size(); i++) {
    const StreamPlan& s = pl->st[i];
    const size_t n = (size_t)s.final_count;
    cudaError_t e;
    if (pl->fmt == DSDGPU_OUT_DOP) {
      e = cudaMemcpyAsync(h_out[i], pl->d_out + s.out_off, s.out_bytes, cudaMemcpyDeviceToHost, m);
    } else if (pl->fmt == DSDGPU_OUT_NATIVE) {
      e = cudaMemcpyAsync(h_out[i], pl->d_out + s.out_off, s.out_bytes, cudaMemcpyDeviceToHost, m);
    } else {
      e = cudaMemcpy2DAsync(h_out[i], n, pl->d_bits + s.bits_off, s.bits_stride, n,
                            (size_t)s.d.channels, cudaMemcpyDeviceToHost, m);
    }
    if (e != cudaSuccess) return c->cuda_fail(e, "output download");
  }
  return c->check_status();
}

int dsdgpu_plan_times(const dsdgpu_plan_t* pl, float* ms4) {
  if (!pl || !ms4) return DSDGPU_ERR_ARG;
  memcpy(ms4, pl->ms, sizeof pl->ms);
  return DSDGPU_OK;
}

int dsdgpu_plan_time_plain(dsdgpu_plan_t* pl, int njobs, int64_t* samples, double* seconds) {
  if (!pl || njobs < 1 || !samples || !seconds) return DSDGPU_ERR_ARG;
  dsdgpu_context* c = pl->c;
  if (!pl->ran) return c->fail(DSDGPU_ERR_STATE, "run the plan first (the FIR output is its input)");
  cudaSetDevice(c->device);
  cudaStream_t m = c->stream;
  njobs = std::min<int>(njobs, (int)pl->jobs.size());
  // the first njobs rows of the job table, each its own launch of one CTA
  std::vector<int> cls_of(pl->jobs.size(), 0);
  for (size_t k = 0; k < pl->cls.size(); k++)
    for (int j = 0; j < pl->cls[k].njobs; j++) cls_of[pl->cls[k].job_first + j] = (int)k;
  int64_t smp = 0;
  cudaStreamSynchronize(m);
  const auto t0 = std::chrono::steady_clock::now();
  for (int j = 0; j < njobs; j++) {
    SdmParams P = pl->cls[cls_of[j]].P;   // the class's width, as the batched launch
    P.mode = c->sdm_mode;
    if (launch_sdm_jobs(P, pl->d_jobs + j, 1, pl->d_counters, pl->d_ctx, c->d_status, 1, m) != 0)
      return c->cuda_fail(cudaGetLastError(), "plain launch");
    c->launches++;
    smp += pl->jobs[j].n_in;
  }
  const cudaError_t e = cudaStreamSynchronize(m);
  const auto t1 = std::chrono::steady_clock::now();
  if (e != cudaSuccess) return c->cuda_fail(e, "plain run");
  *samples = smp;
  *seconds = std::chrono::duration<double>(t1 - t0).count();
  return c->check_status();
}

}  // extern "C"

namespace {

int upload_stream_rows(dsdgpu_plan* pl, StreamPlan& s, cudaStream_t m) {
  dsdgpu_context* c = pl->c;
  // job rows of this stream are contiguous: [ch * S + k] indices in order
  int lo = 1 << 30, hi = -1;
  for (int j : s.job_index) { lo = std::min(lo, j); hi = std::max(hi, j); }
  cudaError_t e = cudaSuccess;
  if (hi >= lo)
    e = cudaMemcpyAsync(pl->d_jobs + lo, pl->jobs.data() + lo, sizeof(SdmJob) * (size_t)(hi - lo + 1),
                        cudaMemcpyHostToDevice, m);
  if (e == cudaSuccess && s.ntasks > 0)
    e = cudaMemcpyAsync(pl->d_tasks + s.task_first, pl->tasks.data() + s.task_first,
                        sizeof(SeamTask) * (size_t)s.ntasks, cudaMemcpyHostToDevice, m);
  if (e == cudaSuccess && s.npieces > 0)
    e = cudaMemcpyAsync(pl->d_pieces + s.piece_first, pl->pieces.data() + s.piece_first,
                        sizeof(AssemblePiece) * (size_t)s.npieces, cudaMemcpyHostToDevice, m);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(pl->d_segbuf + s.segbuf_first, pl->segbuf.data() + s.segbuf_first,
                        sizeof(SegBuf) * (size_t)s.S * s.d.channels, cudaMemcpyHostToDevice, m);
  if (e != cudaSuccess) return c->cuda_fail(e, "table upload");
  // the host tables must stay valid until the copies ran
  return c->check_status();
}

}  // namespace
