/*
 * dsdgpu — GB300 (sm_103a) implementation of the foo_dsd_trellis PCM/DSD -> DSD
 * hot path behind a C ABI: FIR upsampling chain with the engine glue, the
 * trellis sigma-delta modulator, Density-Aligned Stitching of parallel
 * segments, and bit packing / DoP framing.
 *
 * Conventions (those of the reference's include/gpu_compute.h:1-9):
 *   - every call returns an int status: 0 (DSDGPU_OK) on success, a negative
 *     DSDGPU_ERR_* code on failure; the caller decides what to do next;
 *   - an opaque context owns the device, a CUDA stream and all device state;
 *     it is not thread-safe: drive one context from one thread;
 *   - setup calls are separate from per-block calls;
 *   - buffers named d_* are device pointers owned by the caller; buffers named
 *     h_* are host pointers (pinned or pageable);
 *   - a per-block call with zero samples or frames returns DSDGPU_OK with no
 *     output, changes no stream state, and accepts null buffers;
 *   - dsdgpu_destroy(NULL) does nothing.
 * Decisions are exchanged as one byte per DSD sample (1 = +1.0, 0 = -1.0)
 * unless a function says otherwise.
 */
#ifndef DSDGPU_H
#define DSDGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DSDGPU_OK                0
#define DSDGPU_ERR_ARG          (-1)  /* invalid argument; the reference's -1 */
#define DSDGPU_ERR_CUDA         (-2)  /* a CUDA runtime call failed */
#define DSDGPU_ERR_NOMEM        (-3)  /* device or host allocation failed */
#define DSDGPU_ERR_STATE        (-4)  /* call out of order (not set up, ...) */
#define DSDGPU_ERR_DEVICE       (-5)  /* a kernel reported a bounded-wait or
                                         bounded-walk failure in its status word */
#define DSDGPU_ERR_UNSUPPORTED  (-6)  /* parameters valid for the reference but
                                         not built in this library */
#define DSDGPU_ERR_TOO_LARGE    (-7)  /* request exceeds the fixed scratch of the
                                         allocation-free entry point */

typedef struct dsdgpu_context dsdgpu_context_t;

/* Trellis SDM parameters: the arguments of sdm_context_init plus the NTF
 * coefficients of the ntf_filter_t it is given and the state limiter
 * (reference include/trellis.h:62-63, include/ntf.h:14-20,
 * include/trellis.h:57). */
typedef struct {
    int    order;        /* NTF order, 2..10 */
    double a[10];        /* ntf_filter_t.a (first `order` used) */
    double g[10];        /* ntf_filter_t.g */
    int    depth;        /* path-dedup mask width, 1..64 (the reference
                            accepts 1..32; 33..64 follow its arithmetic with a
                            64-bit path) */
    int    cands;        /* candidates kept per sample K, 1..32 */
    int    lat;          /* traceback latency in samples, 1..2048 */
    double state_limit;  /* integrator clamp, 0 = off */
} dsdgpu_sdm_params_t;

/* One segment of work for dsdgpu_sdm_segments: sdm_segment_process
 * (reference src/engine.c:915-938) on context `channel`, optionally after
 * sdm_context_copy_state from `seed_from` (src/trellis.c:1064) and seeding of
 * the live candidates with `d_seed_state` and zero cost
 * (src/dsp_plugin.c:2316-2326). */
typedef struct {
    const double *d_in;          /* device, `count` doubles */
    uint8_t      *d_out;         /* device, room for `count` decision bytes */
    int64_t       count;         /* input samples */
    int64_t       discard;       /* warm-up decisions to drop after latency fill */
    int           channel;       /* context the segment runs on and leaves its state in */
    int           seed_from;     /* context to copy first, or -1 */
    const double *d_seed_state;  /* device, `order` doubles, or NULL */
    int64_t       out_count;     /* written: decisions produced */
} dsdgpu_segment_t;

/* FIR chain + engine glue parameters: fir_chain_init_ex(fs_in, fs_out) for an
 * upsampling power-of-two ratio (reference src/fir.c:523-611) and the
 * engine's per-channel pre/post processing around it (src/engine.c:608-717). */
typedef struct {
    unsigned fs_in;       /* input rate (PCM or DSD), Hz */
    unsigned fs_out;      /* output DSD rate, fs_in * 2^k, k = 1..9 */
    int      boxcar_taps; /* running-mean pre-smooth at the input rate: 8 on the
                             engine's rate-conversion path (engine_process_block),
                             0 = off (the plugin's DAS FIR phase,
                             engine_process_fir_gain, src/engine.c:789-900) */
    int      soft_clip;   /* 1: tanh knee above +-0.95 before the SDM
                             (engine_process_block); 0 in the DAS FIR phase */
} dsdgpu_fir_params_t;

/* DAS seeding modes (reference src/dsp_plugin.c:2185-2283). */
#define DSDGPU_DAS_FULL_PARALLEL 0  /* every segment from the chunk-start state
                                       (the reference's mode at DSD512 and up) */
#define DSDGPU_DAS_SEG0_FIRST    1  /* seg0 on the channel's context, seg1 DIRECT
                                       from its end state, seg2+ seeded by the
                                       16-level greedy estimate (below DSD512) */

/* Density-Aligned Stitching parameters for one chunk.  The overlap is
 * 64 * lat of the SDM setup (src/dsp_plugin.c:1343). */
typedef struct {
    int64_t seg_len;     /* nominal segment length in FIR samples; 0: use nsegs */
    int     nsegs;       /* segment count when seg_len is 0 */
    int     seed_mode;   /* DSDGPU_DAS_FULL_PARALLEL or DSDGPU_DAS_SEG0_FIRST */
    int     reposition;  /* 1: move quiet boundaries of seg >= 2 (RMS search) */
} dsdgpu_das_params_t;

/* Output formats of the whole-path pipeline. */
#define DSDGPU_OUT_BITS    0   /* one byte per decision, [channel][sample] */
#define DSDGPU_OUT_DOP     1   /* DoP 24-bit frames, [frame][channel][3] */
#define DSDGPU_OUT_NATIVE  2   /* MSB-first DSD bytes, [channel][byte] */
#define DSDGPU_OUT_PCM     3   /* DSD -> PCM: float32 rows [channel][sample], stride in floats */

/* SDM of the whole-path pipeline: the reference's sdm_mode_t
 * (include/dsd_types.h:50-53), numbered so that a zero-filled parameter block
 * keeps the trellis (the reference numbers PreCorr 0). */
#define DSDGPU_SDM_TRELLIS 0   /* trellis SDM with DAS */
#define DSDGPU_SDM_PRECORR 1   /* PreCorr greedy SDM, sequential per channel */

/* Whole-path parameters: the FIR chain with its glue, the trellis SDM, DAS,
 * and the output format.  The input is PCM below DSD64's 2,822,400 Hz and DoP
 * at or above it, as the engine decides (src/engine.c:156-164):
 *   PCM in                   boxcar, FIR upsampling chain, gain, soft clip
 *   DSD in, same rate        DoP unpack, boxcar or lowpass (samerate_filter)
 *   DSD in, higher DSD rate  DoP unpack to +-1, boxcar, FIR upsampling chain,
 *                            gain, soft clip (the engine's rate-conversion
 *                            branch; fir.boxcar_taps 8 as the engine sets it)
 *   DSD in, lower DSD rate   DoP unpack, boxcar, FP64 decimation chain, gain,
 *                            soft clip (the same branch, downsampling)
 *   DSD in, PCM out          DoP unpack, decimation chain, float32
 * then the SDM and packing.  The soft clip is never applied ahead of PreCorr
 * (src/engine.c:704-717). */
/* Pre-SDM filter of the same-rate DSD path: the reference's fir_mode
 * (FIR_MODE_BOXCAR 0 / FIR_MODE_FIR 1, include/dsd_types.h:436-438; the
 * engine's default is the boxcar, src/engine.c:168-181). */
#define DSDGPU_SAMERATE_BOXCAR  0   /* rate-adaptive running mean (fir.boxcar_taps) */
#define DSDGPU_SAMERATE_LOWPASS 1   /* 127-tap FP64 lowpass at 50 kHz (fir_lowpass_init) */

typedef struct {
    dsdgpu_fir_params_t fir;
    dsdgpu_sdm_params_t sdm;
    dsdgpu_das_params_t das;
    int                 output_format;   /* DSDGPU_OUT_* */
    int                 sdm_mode;        /* DSDGPU_SDM_*; 0 = trellis */
    int                 samerate_filter; /* DSDGPU_SAMERATE_*; same-rate input only */
} dsdgpu_pipeline_params_t;

/* ---- lifecycle (replaces gpu_create / gpu_destroy, include/gpu_compute.h:52-55) ---- */

/* Create a context on CUDA device `device`.  *out is NULL on failure. */
int  dsdgpu_create(int device, dsdgpu_context_t **out);
void dsdgpu_destroy(dsdgpu_context_t *ctx);
/* Human-readable description of the last failure on this context. */
const char *dsdgpu_last_error(const dsdgpu_context_t *ctx);
/* Options (dsdgpu_set_option). */
#define DSDGPU_OPT_SDM_SELECT   1   /* survivor selection of the trellis SDM: */
#define DSDGPU_SELECT_FAST      0   /*   parallel ranks where provably equal to the
                                         reference's serial order, serial otherwise
                                         (default) */
#define DSDGPU_SELECT_EXACT     1   /*   always the serial reference order */
#define DSDGPU_SELECT_VERIFY    2   /*   serial, and the parallel result is checked
                                         against it every sample (a disagreement
                                         returns DSDGPU_ERR_DEVICE) */
#define DSDGPU_OPT_SDM_LANES    2   /* lanes of a warp per trellis job: 0 = automatic
                                         (default), or 2, 4, 8, 16, 32 (raised to the
                                         next power of two >= K); 32 / lanes jobs share
                                         a warp.  Results do not depend on it. */
#define DSDGPU_OPT_SDM_BALANCE  3   /* 1 (default): an uncapped launch of many long K > 16
                                         jobs slightly above a whole number of warps per
                                         FP64 pipe cuts the jobs into 1,024-sample parts
                                         queued over an even number of warps per pipe;
                                         0: one job per warp from start to end.  Results
                                         do not depend on it. */
#define DSDGPU_OPT_FAILURE_TEST 4   /* failure-path tests only (default 0): bits that
                                         make the kernels' bounded waits and walks give
                                         up early, so a test can check that the call
                                         returns DSDGPU_ERR_DEVICE and the context stays
                                         usable.  No fault is raised; no wait is
                                         unbounded. */
#define DSDGPU_FAIL_PART_WAIT   1   /*   a balanced launch's part queue gets one entry
                                         that no part publishes, and the wait for it
                                         gives up after ~1 ms instead of ~4 s */
#define DSDGPU_FAIL_CHAIN_WALK  2   /*   the serial selection's path-hash chain walk
                                         gives up after one hop */
int  dsdgpu_set_option(dsdgpu_context_t *ctx, int option, int value);

/* Number of kernels this context has launched so far. */
int  dsdgpu_launch_count(const dsdgpu_context_t *ctx, uint64_t *count);
/* Input samples the trellis SDM has stepped through: in total, and in the
 * last SDM launch (warm-up and overlap samples of DAS segments included). */
int  dsdgpu_sdm_work(const dsdgpu_context_t *ctx, uint64_t *total_samples, uint64_t *last_launch);
/* Name of the kernel the context's last trellis SDM launch ran, with its
 * template arguments (e.g. "sdm_parts_kernel<7>", "sdm_jobs_kernel<7,32>",
 * "sdm_split_kernel<6,8,2>"); "" before the first. */
int  dsdgpu_sdm_last_kernel(const dsdgpu_context_t *ctx, char *name, size_t cap);
/* Wait for all work queued on the context's stream. */
int  dsdgpu_synchronize(dsdgpu_context_t *ctx);

/* ---- trellis SDM (replaces sdm_context_init / sdm_process_block /
 *      sdm_drain / sdm_context_copy_state / sdm_context_reset,
 *      include/trellis.h:62-88; and gpu_cuda_trellis_setup / gpu_cuda_trellis,
 *      include/gpu_compute.h:246-256) ---- */

/* Allocate and initialise `num_contexts` device SDM contexts with one
 * parameter set (sdm_context_init on each).  Replaces any previous setup. */
int dsdgpu_sdm_setup(dsdgpu_context_t *ctx, const dsdgpu_sdm_params_t *p, int num_contexts);

/* sdm_context_reset on context `channel`, or on all contexts when -1. */
int dsdgpu_sdm_reset(dsdgpu_context_t *ctx, int channel);

/* sdm_process_block on contexts [first, first + nch): channel c reads
 * d_in[c * in_stride ...] (count doubles) and writes its decisions to
 * d_out[c * out_stride ...].  out_counts[c] receives the decisions of channel
 * c (count minus what is still filling the latency); may be NULL.  With more
 * than one channel, in_stride must be at least count and out_stride at least
 * the decisions a channel writes (DSDGPU_ERR_ARG otherwise). */
int dsdgpu_sdm_process(dsdgpu_context_t *ctx, int first, int nch,
                       const double *d_in, size_t in_stride, size_t count,
                       uint8_t *d_out, size_t out_stride, size_t *out_counts);

/* Host-buffer form with the reference's float +-1.0 output: h_in is
 * [nch][count] doubles, h_out [nch][count] floats.  Copies in, runs, copies
 * out (sdm_process_block's own signature, per channel). */
int dsdgpu_sdm_process_host(dsdgpu_context_t *ctx, int first, int nch,
                            const double *h_in, size_t count, float *h_out,
                            size_t *out_counts);

/* sdm_drain on contexts [first, first + nch). */
int dsdgpu_sdm_drain(dsdgpu_context_t *ctx, int first, int nch, uint8_t *d_out,
                     size_t out_stride, size_t max_out, size_t *out_counts);

/* sdm_context_copy_state(dst, src). */
int dsdgpu_sdm_copy_state(dsdgpu_context_t *ctx, int dst, int src);

/* Run many segments in one persistent launch (the batched form).  Segments
 * whose `channel` is the same must not appear twice in one call, and no
 * segment may name as `seed_from` a context another segment of the call runs
 * on (copy it beforehand with dsdgpu_sdm_copy_state). */
int dsdgpu_sdm_segments(dsdgpu_context_t *ctx, dsdgpu_segment_t *segs, int nseg);

/* ---- FIR chain (replaces fir_chain_init_ex / fir_chain_process_d /
 *      fir_chain_reset, include/fir.h:55-83, and gpu_cuda_fir_chain_f64,
 *      include/gpu_compute.h) ---- */

/* Plan the chain and allocate per-channel history for `num_channels`. */
int dsdgpu_fir_setup(dsdgpu_context_t *ctx, const dsdgpu_fir_params_t *p, int num_channels);
/* Clear the per-channel history (fir_chain_reset plus the boxcar reset). */
int dsdgpu_fir_reset(dsdgpu_context_t *ctx);
/* One block per channel: d_in[c * in_stride ...] holds `count` float PCM
 * samples; d_out[c * out_stride ...] receives count * fs_out / fs_in doubles:
 * boxcar, FIR chain, gain ramp from gain_start to gain_end over the block
 * (a gain_start of 0 means gain_end; no ramp when both are 1), soft clip.
 * History carries over to the next call, as the reference's delay lines do. */
int dsdgpu_fir_process(dsdgpu_context_t *ctx, int first, int nch,
                       const float *d_in, size_t in_stride, size_t count,
                       double *d_out, size_t out_stride,
                       double gain_start, double gain_end, size_t *out_count);
/* Same, queued on the context's stream without waiting. */
int dsdgpu_fir_process_async(dsdgpu_context_t *ctx, int first, int nch,
                             const float *d_in, size_t in_stride, size_t count,
                             double *d_out, size_t out_stride,
                             double gain_start, double gain_end, size_t *out_count);

/* ---- Density-Aligned Stitching (replaces the DAS block of plugin_process,
 *      src/dsp_plugin.c:1283-2762, and gpu_cuda_trellis_das,
 *      include/gpu_compute.h) ---- */

/* One chunk of `nch` channels through segment-parallel SDM and stitching.
 * Requires dsdgpu_sdm_setup with num_contexts >= nch: contexts [0, nch) are
 * the channels' persistent SDM states, used and carried like the reference's
 * (the last segment's state is copied back).  d_fir[c * fir_stride ...] holds
 * `count` doubles of channel c; the stitched decisions go to
 * d_out[c * out_stride ...] and *out_count receives their number.  When
 * h_stitch_pos is not NULL it receives up to max_segs seam offsets (entry s
 * for boundary s; 0 where there is none). */
int dsdgpu_das_process(dsdgpu_context_t *ctx, const dsdgpu_das_params_t *p, int nch,
                       const double *d_fir, size_t fir_stride, size_t count,
                       uint8_t *d_out, size_t out_stride, size_t *out_count,
                       int *h_stitch_pos, int max_segs);

/* ---- bit packing (replaces dop_pack_i24 / bits_pack, include/dop.h:38-46) ---- */

/* DoP: `n` decisions per channel (d_bits[c * bits_stride ...]) become n / 16
 * frames of 3 bytes [bits 7..0, bits 15..8, marker] per channel, channels
 * interleaved frame by frame in d_out ([frame][channel][3], the plugin's
 * output layout); the marker starts at 0x05 for phase 0, 0xFA for phase 1.
 * *next_phase receives the phase for the following block. */
int dsdgpu_pack_dop(dsdgpu_context_t *ctx, int nch, const uint8_t *d_bits, size_t bits_stride,
                    size_t n, uint8_t *d_out, int phase, int *next_phase);

/* Native DSD bytes, MSB first: d_out[c * out_stride ...] receives (n + 7) / 8
 * bytes per channel. */
int dsdgpu_pack_native(dsdgpu_context_t *ctx, int nch, const uint8_t *d_bits, size_t bits_stride,
                       size_t n, uint8_t *d_out, size_t out_stride);

/* ---- whole path: PCM -> FIR + glue -> segment SDM + DAS -> pack (the PCM
 *      conversion of plugin_process_pcm with the DAS phases of
 *      plugin_process, src/dsp_plugin.c:2990-3216, 1283-2945) ---- */

/* Set up the FIR chain, `nch` persistent SDM contexts and the packer. */
int dsdgpu_pipeline_setup(dsdgpu_context_t *ctx, const dsdgpu_pipeline_params_t *p, int nch);
/* One chunk from device buffers: d_pcm[c * pcm_stride ...] holds `frames`
 * float samples of channel c.  The output layout follows the format (rows of
 * out_stride bytes for BITS and NATIVE).  The DoP marker phase carries over
 * between calls.  *out_samples receives the decisions per channel,
 * *out_bytes the bytes written. */
int dsdgpu_pipeline_process(dsdgpu_context_t *ctx, const float *d_pcm, size_t pcm_stride,
                            size_t frames, double gain_start, double gain_end,
                            uint8_t *d_out, size_t out_stride,
                            size_t *out_samples, size_t *out_bytes);
/* The same from host buffers: h_pcm is planar [nch][frames]; h_out receives
 * the packed output (rows of (n + 7) / 8 bytes for NATIVE, n for BITS).
 * Includes the host<->device copies. */
int dsdgpu_pipeline_process_host(dsdgpu_context_t *ctx, const float *h_pcm, size_t frames,
                                 double gain_start, double gain_end, uint8_t *h_out,
                                 size_t out_capacity, size_t *out_samples, size_t *out_bytes);
/* plugin_flush (src/dsp_plugin.c:3622-3653): reset every channel's SDM or
 * PreCorr state, the FIR / boxcar / lowpass / decimation / convolution
 * histories and the DoP marker phase, so that the next
 * dsdgpu_pipeline_process call starts a new stream (seek, track change). */
int dsdgpu_pipeline_flush(dsdgpu_context_t *ctx);
/* Milliseconds of the last pipeline call, measured with CUDA events on the
 * context's stream: [FIR, segment SDM launch, DAS total, pack, whole call]. */
int dsdgpu_stage_times(const dsdgpu_context_t *ctx, float *ms5);
/* The CUDA stream (cudaStream_t) the context queues its work on. */
int dsdgpu_get_stream(const dsdgpu_context_t *ctx, void **stream);

/* Allocation-free trellis SDM (no counterpart in the reference; added for
 * callers that cannot allocate device memory, such as a player's real-time
 * audio callback, where an allocation can block and cause a dropout, or a host
 * that grants a fixed device-memory budget).  With keep_state 0 it runs
 * sdm_context_init and then sdm_process_block on up to 8 channels; with
 * keep_state 1 it continues from the contexts the previous call on this
 * device left behind (same parameters and channel count, else
 * DSDGPU_ERR_STATE), so successive callback blocks form one stream per
 * channel, the latency fill applying to the first block only.  All of its
 * scratch (context bank, job table, counter, status word) is in a fixed
 * device array of about 110 KB that every GPU which loads the library keeps
 * until exit; it calls no cudaMalloc, cudaFree or allocating library routine.
 * More than 8 channels is rejected with DSDGPU_ERR_TOO_LARGE; parameters are
 * checked as for dsdgpu_sdm_setup (lat up to 2048).  With more than one
 * channel, in_stride must be at least count and out_stride at least the
 * decisions a channel writes (DSDGPU_ERR_ARG otherwise).
 * The first call on a device looks up the array's device address; the
 * address is not valid across cudaDeviceReset.  CUDA loads kernels lazily, so make one warm-up call with
 * the same parameters and channel count outside the real-time path (or set
 * CUDA_MODULE_LOADING=EAGER): the first use of a kernel variant can allocate
 * inside the driver.  Calls share the array: two calls whose work overlaps on
 * the GPU race and must not be issued.  Work is queued on `stream` (a
 * cudaStream_t, NULL for the default stream) and the call waits for it to
 * finish before returning.  Inputs, outputs and out_counts are as for
 * dsdgpu_sdm_process. */
int dsdgpu_sdm_process_noalloc(const dsdgpu_sdm_params_t *p, int nch, int keep_state,
                               const double *d_in, size_t in_stride, size_t count,
                               uint8_t *d_out, size_t out_stride, size_t *out_counts,
                               void *stream);

/* Measured FP64 add/multiply issue rate of the device in Gop/s (separate
 * DADD and DMUL, the operations the trellis SDM is made of). */
int dsdgpu_probe_fp64(dsdgpu_context_t *ctx, double *gops);

/* Self-check of the library's float -> double widening on the integer pipe
 * (the FIR chain's output conversion) against the hardware conversion, on the
 * binary32 patterns seed + i * 0x9E3779B1 (mod 2^32) for i < n: n = 2^32
 * checks every pattern.  *mismatches counts differing results (0 expected).
 * No counterpart in the reference. */
int dsdgpu_selftest_convert(dsdgpu_context_t *ctx, uint64_t n, uint64_t seed,
                            uint64_t *mismatches);

/* Best candidate's integrator state (sdm_state_distance's input,
 * src/trellis.c:1094-1109) and the counters conv_fail, cands_collapse,
 * next_filter_drops, total_children (include/trellis.h:53-56), plus
 * num_cands, pending.  best_state may be NULL; info may be NULL (6 values). */
int dsdgpu_sdm_query(dsdgpu_context_t *ctx, int channel, double *best_state, uint64_t *info);

/* sdm_state_distance(a, b) (src/trellis.c:1094-1109): sum of the squared
 * differences of the two contexts' best-candidate states. */
int dsdgpu_sdm_state_distance(dsdgpu_context_t *ctx, int a, int b, double *dist);

/* sdm_estimate_state / sdm_estimate_state_multibit (src/trellis.c:1118-1187),
 * many at once (one GPU warp each): the NTF loop of `p` (order, a, g,
 * state_limit; K, depth and lat are not used) run greedily from init_state
 * over `count` samples of d_in (device) with a num_levels quantiser (2 = the
 * 1-bit sign rule, 16 = sdm_estimate_state's default); out_state receives the
 * state after the last sample.  Waits for completion. */
typedef struct {
    const double *d_in;          /* device, `count` doubles */
    int64_t       count;
    double        init_state[10];
    double        out_state[10]; /* written */
} dsdgpu_estimate_t;
int dsdgpu_sdm_estimate_state(dsdgpu_context_t *ctx, const dsdgpu_sdm_params_t *p,
                              int num_levels, dsdgpu_estimate_t *items, int n);

/* ---- Batched multi-stream plan -------------------------------------------
 * Many independent PCM streams of uneven length and mixed rates converted in
 * one pass: per-stream FIR chains, then every DAS segment of every stream in
 * one persistent SDM launch per trellis parameter set (streams whose NTF, K,
 * depth and lat agree share a launch; different sets run concurrently),
 * one seam-search launch over all boundaries, and per-stream assembly and
 * packing.  The device work of a run is replayed from CUDA graphs captured
 * at the first run.  This has no single counterpart in the reference, which
 * converts one stream per plugin instance; each stream's output equals
 * dsdgpu_pipeline_process on a fresh context with the same parameters
 * (constant gain, full-parallel DAS seeding, src/dsp_plugin.c:2185-2283).
 * A stream with sdm_mode DSDGPU_SDM_PRECORR runs the PreCorr greedy SDM
 * instead (src/precorr.c:20-287; K, depth and lat unused, no soft clip
 * ahead of it, as the pipeline in that mode): its chain writes FP32 and one
 * launch per PreCorr parameter set walks every such channel of every stream,
 * one thread each, beside the trellis launches.
 * A stream whose fs_in is a DSD rate takes DoP floats (planar, 16 DSD samples
 * per frame) as the pipeline does: at fs_out == fs_in the same-rate
 * re-encode (unpack, boxcar or the 127-tap FIR lowpass, DAS trellis), above it the FIR chain on the
 * unpacked +-1 values, below it the boxcar and the FP64 half-band /2 chain
 * (in PreCorr mode each with FP32 output and no clip).
 * Each run converts whole streams from fresh state. */
typedef struct {
    int32_t fs_in;             /* PCM rate, Hz; a DSD rate (2,822,400 and up): DoP input */
    int32_t fs_out;            /* DSD rate, Hz: fs_in times a power of two */
    int32_t channels;          /* 1..8 */
    int32_t boxcar_taps;       /* 0 = off (engine default 8); same-rate DSD: 0 = the rate's
                                  default (32 / 64 / 16), up to 256; DSD down: up to 256 */
    int64_t frames;            /* PCM frames per channel (DoP frames for DSD input) */
    double gain;               /* FIR output gain, constant over the stream */
    int32_t soft_clip;         /* tanh soft clip above +-0.95 */
    int32_t reposition;        /* RMS reposition of quiet DAS boundaries */
    dsdgpu_sdm_params_t sdm;   /* NTF, K, depth, lat, state limit */
    int32_t sdm_mode;          /* DSDGPU_SDM_TRELLIS (DAS trellis) or DSDGPU_SDM_PRECORR */
    int32_t samerate_filter;   /* DSDGPU_SAMERATE_*: same-rate DSD input only */
} dsdgpu_stream_desc_t;

typedef struct {
    int64_t seg_len;           /* DAS segment length in use */
    int64_t jobs;              /* SDM segment runs per batch run */
    int64_t sdm_samples;       /* SDM input samples per run (incl. warm-up) */
    int64_t out_samples;       /* output DSD samples per run, all channels */
    int64_t device_bytes;      /* device memory held by the plan */
    int32_t classes;           /* trellis parameter sets (SDM launches) */
    int32_t blocks_per_sm;     /* resident SDM warps per SM the launches use */
    double predicted_ms;       /* autotuner's model of the SDM phase */
} dsdgpu_plan_info_t;

typedef struct dsdgpu_plan dsdgpu_plan_t;

/* seg_len 0 = pick the DAS segment length (32,768 .. 131,072) and the SDM
 * launch shape by measurement (the autotuner, cached in the context).
 * output_format is DSDGPU_OUT_BITS / DOP / NATIVE.  DSDGPU_ERR_TOO_LARGE
 * when the plan's device buffers would exceed max_device_bytes (0 = no
 * limit). */
int dsdgpu_plan_create(dsdgpu_context_t *ctx, const dsdgpu_stream_desc_t *streams,
                       int nstreams, int64_t seg_len, int output_format,
                       uint64_t max_device_bytes, dsdgpu_plan_t **plan);
void dsdgpu_plan_destroy(dsdgpu_plan_t *plan);
int dsdgpu_plan_info(const dsdgpu_plan_t *plan, dsdgpu_plan_info_t *info);
/* Device buffers the plan owns for stream i: planar float PCM
 * [channels][pcm_stride] in, and the packed output (DoP: interleaved
 * frames; NATIVE: per-channel rows of out_stride bytes; BITS: per-channel
 * rows of decision bytes, out_stride apart).  out_samples is the stream's
 * DSD samples per channel; out_bytes the packed size of all channels. */
int dsdgpu_plan_stream(const dsdgpu_plan_t *plan, int stream, float **d_pcm, size_t *pcm_stride,
                       uint8_t **d_out, size_t *out_stride, size_t *out_samples,
                       size_t *out_bytes);
/* One batch run on the device buffers (waits for completion). */
int dsdgpu_plan_run(dsdgpu_plan_t *plan);
/* The same with host buffers: h_pcm[i] planar [channels][frames] floats,
 * h_out[i] receives out_bytes (contiguous rows for NATIVE / BITS); copies
 * are inside the call. */
int dsdgpu_plan_run_host(dsdgpu_plan_t *plan, const float *const *h_pcm, uint8_t *const *h_out);
/* Milliseconds of the last run: [FIR + RMS, SDM launches, seams + assembly
 * + packing, whole run]. */
int dsdgpu_plan_times(const dsdgpu_plan_t *plan, float *ms4);
/* The one-segment-per-launch form over the first `njobs` segment runs of the
 * last run (same kernel, one job per launch, launched back to back); returns
 * the SDM input samples processed and the seconds taken. */
int dsdgpu_plan_time_plain(dsdgpu_plan_t *plan, int njobs, int64_t *samples, double *seconds);

/* ---- Same-rate DSD input (DSD -> DSD re-encode) ----------------------------
 * dop_unpack (src/dop.c:74-87) and the engine's same-rate boxcar with gain ramp
 * (engine_process_block, src/engine.c:487-563).  A pipeline set up with
 * fir.fs_in == fir.fs_out takes DoP floats (planar [nch][frames], 16 DSD
 * samples per frame) and runs unpack -> boxcar (fir.boxcar_taps, 0 = the
 * engine's rate default: 32 at DSD64, 64 at DSD128/256, 16 at DSD512) or,
 * with samerate_filter DSDGPU_SAMERATE_LOWPASS, the FIR lowpass below ->
 * DAS SDM (or PreCorr) -> packing. */
/* DoP floats [nch][dop_stride] -> 0/1 decision bytes [nch][bits_stride],
 * 16 per frame, MSB first. */
int dsdgpu_dop_unpack(dsdgpu_context_t *ctx, int nch, const float *d_dop, size_t dop_stride,
                      size_t frames, uint8_t *d_bits, size_t bits_stride);
/* The same unpack in dop_unpack's own output form: +-1.0f floats
 * [nch][out_stride], 16 per frame. */
int dsdgpu_dop_unpack_f32(dsdgpu_context_t *ctx, int nch, const float *d_dop, size_t dop_stride,
                          size_t frames, float *d_out, size_t out_stride);
int dsdgpu_boxcar_setup(dsdgpu_context_t *ctx, int taps, int nch);   /* taps 1..256 */
int dsdgpu_boxcar_reset(dsdgpu_context_t *ctx);
/* Decision bytes -> (window count / taps) * (gain ramp), the window carried
 * across calls; gain_start 0 means gain_end (the first chunk). */
int dsdgpu_boxcar_process(dsdgpu_context_t *ctx, int first, int nch, const uint8_t *d_bits,
                          size_t bits_stride, size_t count, double *d_out, size_t out_stride,
                          double gain_start, double gain_end);
int dsdgpu_boxcar_process_async(dsdgpu_context_t *ctx, int first, int nch,
                                const uint8_t *d_bits, size_t bits_stride, size_t count,
                                double *d_out, size_t out_stride, double gain_start,
                                double gain_end);

/* Same-rate FIR lowpass (fir_lowpass_init_ex / fir_lowpass_process /
 * fir_lowpass_reset, src/fir.c:795-877; the engine's FIR_MODE_FIR branch,
 * src/engine.c:505-523, and the plugin's gpu_fir_lowpass_setup /
 * gpu_fir_lowpass_f64, include/gpu_compute.h:88-103): Kaiser (beta 10)
 * windowed sinc, ntaps clamped to 3..255 and made odd, cutoff_hz / (fs / 2)
 * capped at 0.5, normalised to unit sum, FP64; applied to +-1 decisions with
 * the delay line carried across calls (zero at setup and reset), then the
 * gain ramp of the boxcar.  fir_lowpass_init is cutoff 50,000 Hz, 127 taps. */
int dsdgpu_lowpass_setup(dsdgpu_context_t *ctx, unsigned fs, double cutoff_hz, int ntaps,
                         int nch);
/* The design alone (host code, no context): taps[0 .. *ntaps). */
int dsdgpu_lowpass_design(unsigned fs, double cutoff_hz, int ntaps, double *taps, int cap,
                          int *out_ntaps);
/* The designed taps (the FP64 coeffs_d of fir_lowpass_t); *ntaps receives the
 * count, taps may be NULL. */
int dsdgpu_lowpass_taps(const dsdgpu_context_t *ctx, double *taps, int cap, int *ntaps);
int dsdgpu_lowpass_reset(dsdgpu_context_t *ctx);
int dsdgpu_lowpass_process(dsdgpu_context_t *ctx, int first, int nch, const uint8_t *d_bits,
                           size_t bits_stride, size_t count, double *d_out, size_t out_stride,
                           double gain_start, double gain_end);
int dsdgpu_lowpass_process_async(dsdgpu_context_t *ctx, int first, int nch,
                                 const uint8_t *d_bits, size_t bits_stride, size_t count,
                                 double *d_out, size_t out_stride, double gain_start,
                                 double gain_end);

/* ---- DSD -> PCM decimation (FIR-only engine branch, src/engine.c:566-577) ---
 * FP64 chain of 63-tap half-band /2 stages (src/fir.c:467-487,523-611), delay
 * lines carried across calls, gain ramp, narrowed to float32.  A pipeline with
 * output_format DSDGPU_OUT_PCM (fir.fs_out < fir.fs_in) takes DoP floats and
 * returns PCM: unpack -> decimation -> float. */
int dsdgpu_decim_setup(dsdgpu_context_t *ctx, unsigned fs_in, unsigned fs_out, int nch);
/* The same chain on FP64 input with FP64 output: the downsampling half of the
 * engine's rate-conversion branch (fir_chain_process_d, then the gain ramp
 * when either end differs from 1 and, when soft_clip, the tanh clip above
 * +-0.95; src/engine.c:600-717). */
int dsdgpu_decim_process_f64(dsdgpu_context_t *ctx, int nch, const double *d_in,
                             size_t in_stride, size_t count, double *d_out, size_t out_stride,
                             double gain_start, double gain_end, int soft_clip,
                             size_t *out_count);
int dsdgpu_decim_process_f64_async(dsdgpu_context_t *ctx, int nch, const double *d_in,
                                   size_t in_stride, size_t count, double *d_out,
                                   size_t out_stride, double gain_start, double gain_end,
                                   int soft_clip, size_t *out_count);
int dsdgpu_decim_reset(dsdgpu_context_t *ctx);
/* 0/1 decision bytes [nch][bits_stride] (count per channel) -> float PCM
 * [nch][pcm_stride]; *out_count = count / (fs_in / fs_out) (each stage keeps
 * floor(count / 2) outputs). */
int dsdgpu_decim_process(dsdgpu_context_t *ctx, int nch, const uint8_t *d_bits,
                         size_t bits_stride, size_t count, float *d_pcm, size_t pcm_stride,
                         double gain_start, double gain_end, size_t *out_count);
int dsdgpu_decim_process_async(dsdgpu_context_t *ctx, int nch, const uint8_t *d_bits,
                               size_t bits_stride, size_t count, float *d_pcm,
                               size_t pcm_stride, double gain_start, double gain_end,
                               size_t *out_count);

/* ---- DSF / DSDIFF files (the offline encoder's writers) -------------------
 * Replace write_dsf / write_dff and their packers pack_dsd_lsb / pack_dsd_msb
 * (reference tools/dsd_encode.c:80-98, :164-292), which write mono files; the
 * same layouts extend to 1..6 channels per the formats' specifications.
 * DSF: 92-byte header (DSD, fmt, data chunk headers), payload
 * [block][channel][4096 B], decisions LSB first, last block zero-padded.
 * DFF: FRM8 / FVER 1.5 / PROP (SND, FS, CHNL) / DSD chunk header, payload
 * bytes interleaved by channel, MSB first (no CMPR chunk, no pad byte after
 * an odd payload: the reference's bytes).  A file is the header followed by
 * the payload. */
#define DSDGPU_FILE_DSF 1
#define DSDGPU_FILE_DFF 2
/* Host only (no device work): the header of a file of `samples` decisions per
 * channel at fs Hz into hdr (capacity cap >= 128); *payload_bytes = the size
 * of the payload that follows it. */
int dsdgpu_file_header(int format, int nch, unsigned fs, uint64_t samples, uint8_t *hdr,
                       size_t cap, size_t *hdr_len, uint64_t *payload_bytes);
/* 0/1 decision bytes [nch][bits_stride] (n per channel) -> the payload in the
 * file's layout at d_out (*payload_bytes bytes). */
int dsdgpu_pack_file(dsdgpu_context_t *ctx, int format, int nch, const uint8_t *d_bits,
                     size_t bits_stride, size_t n, uint8_t *d_out, uint64_t *payload_bytes);

/* ---- PreCorr greedy SDM (src/precorr.c, include/precorr.h:49-61) ----------
 * Replaces precorr_context_init / precorr_process_block /
 * precorr_context_reset (src/precorr.c:198-287) and the reference's GPU entry
 * points gpu_cuda_precorr_setup / gpu_cuda_precorr (src/gpu_cuda.c:822-850,
 * 2933-2974; gpu_precorr_process, include/gpu_compute.h:140-144).  Setup
 * trains the 256 x 8 correction table on the device (65,536 LCG samples at
 * amplitude 0.1, cells with fewer than 4 hits zero) and resets `nch`
 * per-channel states; the coefficients are used as float copies, as the
 * reference's context does.  Decisions equal the reference's CPU build bit for
 * bit.  A pipeline with sdm_mode DSDGPU_SDM_PRECORR runs this instead of the
 * trellis (src/engine.c:557-559, 723-726), with its sdm.order/a/g/state_limit. */
int dsdgpu_precorr_setup(dsdgpu_context_t *ctx, int order, const double *a, const double *g,
                         double state_limit, int nch);
/* Zero state, history 0x69, phase 0, previous output 0; the table is kept. */
int dsdgpu_precorr_reset(dsdgpu_context_t *ctx);
/* Copy the trained table out: host floats [256][8] (history, phase). */
int dsdgpu_precorr_table(dsdgpu_context_t *ctx, float *h_table);
/* FP64 samples [nch][in_stride] (count per channel) for channels
 * [first, first + nch) -> 0/1 decision bytes [nch][bits_stride]; no latency,
 * state carried across calls. */
int dsdgpu_precorr_process(dsdgpu_context_t *ctx, int first, int nch, const double *d_in,
                           size_t in_stride, size_t count, uint8_t *d_bits, size_t bits_stride);
int dsdgpu_precorr_process_async(dsdgpu_context_t *ctx, int first, int nch,
                                 const double *d_in, size_t in_stride, size_t count,
                                 uint8_t *d_bits, size_t bits_stride);

/* ---- UPOLS convolution at the SDM rate ------------------------------------
 * Uniformly partitioned overlap-save convolution of every channel with its
 * own IR (the reference's room-correction convolver: IR partitioning
 * src/convolution.c:355-405, GPU block processing src/gpu_cuda.c:3432-3492,
 * partition multiply-accumulate src/kernels/conv_kernels.cu:62-84), FP32,
 * whole chunks at a time with the input history carried between calls.  Once
 * set up, dsdgpu_pipeline_process applies it between the FIR chain and the
 * SDM (the pipeline's channel count must equal nch). */
/* ir: host floats [nch][ir_len]; partition: power of two (FFT size 2x); at
 * most 32 partitions. */
int dsdgpu_conv_setup(dsdgpu_context_t *ctx, const float *ir, size_t ir_len, int nch,
                      int partition);
int dsdgpu_conv_reset(dsdgpu_context_t *ctx);   /* zero the input history */
int dsdgpu_conv_clear(dsdgpu_context_t *ctx);   /* free; the pipeline stops convolving */
/* d_in / d_out: device doubles [nch][stride]; d_out may equal d_in. */
int dsdgpu_conv_process(dsdgpu_context_t *ctx, int nch, const double *d_in, size_t in_stride,
                        size_t count, double *d_out, size_t out_stride);

/* ---- Differentiable path: STE adjoint of FIR chain + NTF loop ------------
 * Training support with no counterpart in the reference's C code (its
 * training_pipeline/diff_sdm.py runs a soft greedy SDM in PyTorch).  Clips of
 * PCM go through a pre-emphasis FIR (taps are parameters), the linear FP64
 * upsampling chain (fir_chain_process_d without boxcar or clip, times a
 * constant gain), and the exact trellis SDM (one sequential run per clip
 * plus a drain, so decision t belongs to input sample t).  The loss is the
 * mean square of a decimating low-pass of (decisions - reference), the
 * reference being the chain output of the clip without pre-emphasis.
 * The gradient uses a straight-through surrogate: with the forward decisions
 * y^ and loop-filter outputs v^ frozen, y = y^ + kappa (v - v^) and the NTF
 * loop is the linear recurrence driven by y.  The surrogate equals the loss at
 * the forward's parameters and its exact gradient is what backward returns
 * (taps, a[], g[]); dsdgpu_diff_surrogate evaluates it anywhere, for finite
 * differences.  Loop state is checkpointed every `checkpoint` samples and
 * recomputed in the backward pass. */
typedef struct {
    int32_t fs_in;             /* PCM rate, Hz */
    int32_t fs_out;            /* SDM rate, Hz (fs_in times a power of two) */
    int32_t nclips;            /* clips per batch */
    int32_t preemph_taps;      /* pre-emphasis FIR length, 1..255 */
    int64_t frames;            /* PCM frames per clip */
    int32_t decim;             /* loss decimation factor */
    int32_t lpf_taps;          /* loss low-pass length (odd, <= 511) */
    double lpf_cutoff_hz;      /* loss low-pass cutoff */
    double kappa;              /* straight-through slope of the quantiser */
    double gain;               /* chain output gain */
    int32_t checkpoint;        /* loop-state checkpoint interval (power of two) */
    int32_t pad;
    dsdgpu_sdm_params_t sdm;   /* trellis (K, depth, lat) and the NTF order */
} dsdgpu_diff_params_t;

typedef struct dsdgpu_diff dsdgpu_diff_t;

int dsdgpu_diff_create(dsdgpu_context_t *ctx, const dsdgpu_diff_params_t *p, dsdgpu_diff_t **out);
void dsdgpu_diff_destroy(dsdgpu_diff_t *d);
/* Clip PCM, float [nclips][frames] on the device (copied; the reference
 * signal is computed here). */
int dsdgpu_diff_set_input(dsdgpu_diff_t *d, const float *d_pcm);
/* Forward at (taps[preemph_taps], a[order], g[order]) (host arrays): exact
 * decisions, checkpoints and the loss. */
int dsdgpu_diff_forward(dsdgpu_diff_t *d, const double *taps, const double *a, const double *g,
                        double *loss);
/* Gradient of the surrogate at the last forward (host arrays out). */
int dsdgpu_diff_backward(dsdgpu_diff_t *d, double *grad_taps, double *grad_a, double *grad_g);
/* The surrogate loss at other parameters, decisions of the last forward frozen. */
int dsdgpu_diff_surrogate(dsdgpu_diff_t *d, const double *taps, const double *a, const double *g,
                          double *loss);
/* Milliseconds of the last calls: [forward, exact SDM inside it, backward, surrogate]. */
int dsdgpu_diff_times(const dsdgpu_diff_t *d, float *ms4);
/* Device buffers of the last forward: SDM input [nclips][n] doubles and the
 * decisions [nclips][n] (0/1 bytes); n = frames * fs_out / fs_in. */
int dsdgpu_diff_buffers(const dsdgpu_diff_t *d, const double **d_sdm_in, const uint8_t **d_bits,
                        int64_t *n);

#ifdef __cplusplus
}
#endif

#endif /* DSDGPU_H */
