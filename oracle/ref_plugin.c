/*
 * ORACLE — test infrastructure only (see oracle.h).
 *
 * Compiles the reference's DSP plugin core, src/dsp_plugin.c, where it lies
 * (the Makefile passes its path as REF_PLUGIN_C) together with the
 * reference's own src/engine.c, src/fir.c, src/trellis.c, src/trellis_fast.c,
 * src/ntf.c, src/dop.c, src/precorr.c and src/preemph.c, so that
 * plugin_process (src/dsp_plugin.c:1146-2990) — DoP unpack, the engine's FIR
 * phase, DAS layout, reposition, seeding, segment SDM, seam search, assembly,
 * state carry and DoP packing — runs here on known input.  What is not the
 * reference's own code:
 *
 *  - oracle/ref_shim/windows.h: the Win32 names those files use, on POSIX;
 *  - oracle/ref_shim/ipps.h, ippcore.h and oracle/ref_ipp.c: Intel IPP's FIR
 *    functions from their published semantics (IPP is closed and absent);
 *  - below: the thread pool runs every submitted block inline, in submission
 *    order, with the block dispatch of the reference's worker
 *    (src/threadpool.c:279-358); the plugin waits for its blocks before
 *    using them, so inline execution gives the pool's results.  The GPU,
 *    ONNX, CPU-set, resampler, convolution and capture subsystems are
 *    absent (their constructors fail or report nothing available), which the
 *    plugin handles as a CPU-only host with no ML model.
 *
 * The harness initialises the engine itself and clears the first-chunk
 * warm-up mute (src/dsp_plugin.c:2830-2841), so the first chunk's decisions
 * are visible, and keeps a copy of each channel's FIR output of the last
 * chunk (the input of the DAS phase) for the checker.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include REF_PLUGIN_C

/* ── subsystems that are absent here ── */

void trellis_log_c(const char *msg) { (void)msg; }

volatile LONG g_gpu_sdm_override = 0;
volatile LONG g_gpu_sdm_override_valid = 0;
audio_capture_t g_audio_capture;
void capture_write_dsd(float **ch_data, size_t count, int channels, uint32_t dsd_rate)
{
    (void)ch_data; (void)count; (void)channels; (void)dsd_rate;
}

bool gpu_available(gpu_backend_t preferred) { (void)preferred; return false; }
void gpu_get_info(gpu_info_t *info) { memset(info, 0, sizeof *info); }
gpu_context_t *gpu_create(gpu_backend_t backend) { (void)backend; return NULL; }
void gpu_destroy(gpu_context_t *ctx) { (void)ctx; }
void gpu_reset_chunk(gpu_context_t *ctx) { (void)ctx; }
bool gpu_dx12_probe(void) { return false; }
int gpu_fir_setup(gpu_context_t *ctx, const float *taps, int ntaps, int num_stages, bool upsample)
{
    (void)ctx; (void)taps; (void)ntaps; (void)num_stages; (void)upsample;
    return -1;
}
int gpu_fir_chain_process(gpu_context_t *ctx, const float *in, float *out, size_t count,
                          size_t *out_count, const float *delay_in, float *delay_out)
{
    (void)ctx; (void)in; (void)out; (void)count; (void)out_count; (void)delay_in; (void)delay_out;
    return -1;
}
int gpu_fir_chain_process_f64(gpu_context_t *ctx, const float *in, double *out, size_t count,
                              size_t *out_count)
{
    (void)ctx; (void)in; (void)out; (void)count; (void)out_count;
    return -1;
}
int gpu_fir_lowpass_setup(gpu_context_t *ctx, const float *taps, int ntaps)
{
    (void)ctx; (void)taps; (void)ntaps;
    return -1;
}
int gpu_fir_lowpass_f64(gpu_context_t *ctx, const float *in, double *out, size_t count,
                        double gain)
{
    (void)ctx; (void)in; (void)out; (void)count; (void)gain;
    return -1;
}
int gpu_dx11_trellis_setup(void *ctx, int num_cands, int order, int trellis_lat,
                           const double *a, const double *g, double state_limit)
{
    (void)ctx; (void)num_cands; (void)order; (void)a; (void)g; (void)trellis_lat; (void)state_limit;
    return -1;
}
int gpu_cuda_trellis_setup(void *ctx, int num_cands, int order, int trellis_lat,
                           const double *a, const double *g, double state_limit, int depth)
{
    (void)ctx; (void)num_cands; (void)order; (void)a; (void)g; (void)trellis_lat;
    (void)state_limit; (void)depth;
    return -1;
}
int gpu_dx12_trellis_setup_full(void *ctx, int nc, int ord, int lat, const double *a,
                                const double *g, double state_limit)
{
    (void)ctx; (void)nc; (void)ord; (void)lat; (void)a; (void)g; (void)state_limit;
    return -1;
}
int gpu_cuda_precorr_setup(void *ctx, int order, const float *a, const float *g,
                           const float *table, float state_limit)
{
    (void)ctx; (void)order; (void)a; (void)g; (void)table; (void)state_limit;
    return -1;
}
int gpu_cuda_precorr(void *ctx, const float *in, float *out, size_t count,
                     const gpu_precorr_state_t *init, gpu_precorr_state_t *final_state)
{
    (void)ctx; (void)in; (void)out; (void)count; (void)init; (void)final_state;
    return -1;
}
int gpu_conv_max_partitions(gpu_context_t *ctx, uint32_t signal_rate, int partition_size,
                            int budget_level)
{
    (void)ctx; (void)signal_rate; (void)partition_size; (void)budget_level;
    return 0;
}
gpu_conv_state_t *gpu_conv_init(gpu_context_t *ctx, int num_partitions, int partition_size,
                                int fft_size, const void *ir_freq, int channel_idx)
{
    (void)ctx; (void)num_partitions; (void)partition_size; (void)fft_size; (void)ir_freq;
    (void)channel_idx;
    return NULL;
}

bool onnx_runtime_available(void) { return false; }
void onnx_filter_free(onnx_filter_t *f) { (void)f; }
void onnx_filter_reset(onnx_filter_t *f) { (void)f; }
void onnx_filter_predict_taps(onnx_filter_t *f, const float features[3], float taps_out[3])
{
    (void)f; (void)features;
    taps_out[0] = taps_out[1] = taps_out[2] = 0.0f;
}

int cpuset_detect(cpu_topology_t *topo) { memset(topo, 0, sizeof *topo); return -1; }
void cpuset_benchmark(cpu_topology_t *topo) { (void)topo; }
void cpuset_update_load(cpu_topology_t *topo) { (void)topo; }
int cpuset_select(const cpu_topology_t *topo, smt_mode_t smt, ccd_mode_t ccd, ecore_mode_t ec,
                  int max_threads, uint32_t *out_ids, uint8_t *out_lps, uint16_t *out_groups,
                  int max_out)
{
    (void)topo; (void)smt; (void)ccd; (void)ec; (void)max_threads; (void)out_ids;
    (void)out_lps; (void)out_groups; (void)max_out;
    return 0;
}
cpuset_monitor_t *cpuset_monitor_create(cpu_topology_t *topo, int interval_ms, int hysteresis)
{
    (void)topo; (void)interval_ms; (void)hysteresis;
    return NULL;
}
void cpuset_monitor_destroy(cpuset_monitor_t *mon) { (void)mon; }
void cpuset_monitor_read(const cpuset_monitor_t *mon, cpu_topology_t *out) { (void)mon; (void)out; }
bool cpuset_monitor_changed(cpuset_monitor_t *mon, uint64_t *new_mask)
{
    (void)mon; (void)new_mask;
    return false;
}

resample_ctx_t *resample_create(uint32_t fs_in, uint32_t fs_out, int engine, int quality)
{
    (void)fs_in; (void)fs_out; (void)engine; (void)quality;
    return NULL;
}
size_t resample_process(resample_ctx_t *ctx, const float *in, float *out, size_t in_count)
{
    (void)ctx; (void)in; (void)out; (void)in_count;
    return 0;
}
void resample_free(resample_ctx_t *ctx) { (void)ctx; }

int conv_init(conv_state_t *state, uint32_t signal_rate, uint32_t conv_rate)
{
    (void)state; (void)signal_rate; (void)conv_rate;
    return -1;
}
int conv_load_ir(conv_state_t *state, const char *wav_path) { (void)state; (void)wav_path; return -1; }
void conv_process(conv_state_t *state, double *buf, size_t count) { (void)state; (void)buf; (void)count; }
void conv_launch(conv_state_t *state, double *buf, size_t count) { (void)state; (void)buf; (void)count; }
void conv_finalize(conv_state_t *state, double *buf, size_t count) { (void)state; (void)buf; (void)count; }
void conv_reset(conv_state_t *state) { (void)state; }
void conv_free(conv_state_t *state) { (void)state; }

/* ── the thread pool: blocks run inline ── */

struct threadpool {
    int threads;
};

static int g_pool_threads = 16;
#define REF_MAX_CH 8
static double *g_fir[REF_MAX_CH];
static size_t g_fir_n[REF_MAX_CH], g_fir_cap[REF_MAX_CH];

/* The block dispatch of src/threadpool.c:279-358. */
static void run_block(channel_block_t *b)
{
    if (b->mode == BLOCK_MODE_SDM) {
        b->out_count = sdm_segment_process(b->sdm_ctx, b->in, b->out, b->count, b->discard);
    } else if (b->mode == BLOCK_MODE_FIR) {
        b->out_count = engine_process_fir_gain(b->eng, b->in_f32, b->count, b->cfg, &b->fir_out);
        int ch = b->channel;
        if (ch >= 0 && ch < REF_MAX_CH && b->fir_out) {
            if (g_fir_cap[ch] < b->out_count) {
                free(g_fir[ch]);
                g_fir[ch] = (double *)malloc((b->out_count ? b->out_count : 1) * sizeof(double));
                g_fir_cap[ch] = g_fir[ch] ? b->out_count : 0;
            }
            if (g_fir[ch]) {
                memcpy(g_fir[ch], b->fir_out, b->out_count * sizeof(double));
                g_fir_n[ch] = b->out_count;
            }
        }
    } else if (b->mode == BLOCK_MODE_UNPACK) {
        float *tmp = (float *)malloc((b->pcm_frames ? b->pcm_frames : 1) * sizeof(float));
        for (size_t f = 0; f < b->pcm_frames; f++)
            tmp[f] = b->pcm_interleaved[f * (size_t)b->num_channels + (size_t)b->channel];
        dop_unpack(tmp, b->dsd_channel, b->pcm_frames);
        free(tmp);
        b->out_count = b->pcm_frames * DOP_BITS_PER_FRAME;
    } else if (b->mode == BLOCK_MODE_PACK) {
        size_t frames = b->count / DOP_BITS_PER_FRAME;
        uint8_t *tmp = (uint8_t *)b->pcm_temp;
        dop_pack_i24(b->dsd_channel, tmp, b->count, (int)b->discard);
        uint8_t *dst = (uint8_t *)b->pcm_interleaved;
        for (size_t f = 0; f < frames; f++) {
            size_t d = (f * (size_t)b->num_channels + (size_t)b->channel) * 3;
            dst[d] = tmp[3 * f];
            dst[d + 1] = tmp[3 * f + 1];
            dst[d + 2] = tmp[3 * f + 2];
        }
        b->out_count = frames;
    } else if (b->mode == BLOCK_MODE_ESTIMATE) {
        const ntf_filter_t *f = b->est_filter;
        if (f) {
            double st[MAX_NTF_ORDER];
            for (int i = 0; i < f->order; i++) st[i] = b->est_init[i];
            size_t pos = 0;
            for (int seg = 1; seg < b->est_num_segs; seg++) {
                size_t bnd = b->est_boundaries[seg];
                if (bnd > pos && bnd <= b->count) {
                    sdm_estimate_state(f, st, b->in + pos, bnd - pos, b->est_state_limit, st);
                    pos = bnd;
                }
                for (int i = 0; i < f->order; i++) b->est_result[seg][i] = st[i];
            }
        }
        b->out_count = 0;
    } else {
        b->out_count = engine_process_block(b->eng, b->in, b->out, b->count, b->cfg);
    }
}

threadpool_t *threadpool_create(int thread_count, DWORD affinity_mask)
{
    (void)affinity_mask;
    threadpool_t *p = (threadpool_t *)calloc(1, sizeof *p);
    if (p) p->threads = thread_count > 0 ? thread_count : g_pool_threads;
    return p;
}
threadpool_t *threadpool_create_cpuset(const uint32_t *ids, const uint8_t *lps,
                                       const uint16_t *groups, int count)
{
    (void)ids; (void)lps; (void)groups;
    return threadpool_create(count, 0);
}
void threadpool_set_reserved(threadpool_t *pool, int reserved_count) { (void)pool; (void)reserved_count; }
int threadpool_submit(threadpool_t *pool, channel_block_t *block)
{
    (void)pool;
    run_block(block);
    return 0;
}
int threadpool_submit_to(threadpool_t *pool, int worker_index, channel_block_t *block)
{
    (void)worker_index;
    return threadpool_submit(pool, block);
}
void threadpool_wait(threadpool_t *pool) { (void)pool; }
void threadpool_destroy(threadpool_t *pool) { free(pool); }
int threadpool_get_thread_count(threadpool_t *pool) { return pool ? pool->threads : 0; }
void threadpool_reset_log(threadpool_t *pool) { (void)pool; }
int threadpool_get_stressed_thread(threadpool_t *pool, double *ratio)
{
    (void)pool;
    if (ratio) *ratio = 0.0;
    return -1;
}
int threadpool_migrate_thread(threadpool_t *pool, int index, uint32_t id)
{
    (void)pool; (void)index; (void)id;
    return -1;
}
uint32_t threadpool_get_worker_cpuset(threadpool_t *pool, int index) { (void)pool; (void)index; return 0; }
double threadpool_get_worker_self_load(threadpool_t *pool, int index) { (void)pool; (void)index; return 0.0; }

/* ── the checker's interface ── */

typedef struct {
    unsigned fs_out;       /* DSD output rate */
    int cands, depth, lat; /* trellis */
    int ntf_filter;        /* ntf_filter_id_t, -1 = the engine's choice */
    int par_mode;          /* rate_parallel of the input rate: -1 auto, 0 sequential, 2..8 */
    int threads;           /* compute-pool size seen by the plugin */
    int fir_prec;          /* -1 auto (FP64), 0 FP32, 1 FP64 */
    int fir_mode;          /* same rate: -1 auto (boxcar), 0 boxcar, 1 FIR lowpass */
    float state_limit;     /* -1 = the engine's choice */
} ref_plugin_cfg_t;

void *ref_plugin_new(const ref_plugin_cfg_t *c, int nch, unsigned dsd_rate_in)
{
    if (nch < 1 || nch > REF_MAX_CH) return NULL;
    g_pool_threads = c->threads > 0 ? c->threads : 16;
    plugin_state_t *s = plugin_create();
    if (!s) return NULL;
    dsd_config_t *cfg = &s->config;
    cfg->fs_in = dsd_rate_in;
    cfg->fs_out = c->fs_out;
    cfg->sdm_mode = SDM_MODE_TRELLIS;
    cfg->trellis_cands = c->cands;
    cfg->trellis_depth = c->depth;
    cfg->trellis_lat = c->lat;
    cfg->ntf_filter = c->ntf_filter;
    cfg->fir_prec = c->fir_prec;
    cfg->fir_mode = c->fir_mode;
    cfg->state_limit = c->state_limit;
    int idx = rate_map_index(dsd_rate_in);
    if (idx >= 0 && idx < RATE_MAP_COUNT) cfg->rate_parallel[idx] = (int8_t)c->par_mode;
    if (plugin_init_engine(s, nch, dsd_rate_in) != 0) {
        plugin_destroy(s);
        return NULL;
    }
    s->needs_warmup = false;
    return s;
}

size_t ref_plugin_process(void *h, const float *dop, uint8_t *out_i24, size_t frames, int nch,
                          unsigned pcm_rate)
{
    plugin_state_t *s = (plugin_state_t *)h;
    for (int c = 0; c < REF_MAX_CH; c++) g_fir_n[c] = 0;
    return plugin_process(s, dop, out_i24, frames, nch, pcm_rate);
}

size_t ref_plugin_fir(void *h, int ch, double *out, size_t cap)
{
    (void)h;
    if (ch < 0 || ch >= REF_MAX_CH || !g_fir[ch]) return 0;
    size_t n = g_fir_n[ch] < cap ? g_fir_n[ch] : cap;
    memcpy(out, g_fir[ch], n * sizeof(double));
    return g_fir_n[ch];
}

int ref_plugin_segments(void *h) { return ((plugin_state_t *)h)->last_segments_per_ch; }

/* The trellis parameters the engine resolved for channel ch (path table,
 * NTF choice, limiter); returns its sdm_mode_t, -1 for a bad channel. */
int ref_plugin_engine_state(void *h, int ch, int *cands, int *depth, int *lat, int *order,
                            double *a, double *g, double *state_limit, float *fir_gain)
{
    plugin_state_t *s = (plugin_state_t *)h;
    if (ch < 0 || ch >= s->num_channels) return -1;
    engine_channel_t *e = &s->channels[ch];
    *cands = (int)e->sdm.trellis_num;
    *depth = s->config.trellis_depth;
    *lat = (int)e->sdm.trellis_lat;
    *order = e->sdm.filter ? e->sdm.filter->order : 0;
    for (int i = 0; i < *order; i++) {
        a[i] = e->sdm.filter->a[i];
        g[i] = e->sdm.filter->g[i];
    }
    *state_limit = e->sdm.state_limit;
    *fir_gain = e->fir_gain;
    return e->sdm_mode;
}

void ref_plugin_free(void *h) { plugin_destroy((plugin_state_t *)h); }
