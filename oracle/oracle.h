/*
 * ORACLE — test infrastructure only.
 *
 * CPU restatement of the foo_dsd_trellis PCM/DSD -> DSD hot path, used as the
 * checker for the CUDA kernels in foo_dsd_trellis_gb300/csrc and as the timed
 * CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs
 * may load it; the product library never links or calls it.
 *
 * Pinning:
 *   sdm_oracle.c  bit-identical to the reference src/trellis.c (scalar build,
 *                 gcc -ffp-contract=off), checked by tests/test_oracle_ref.py
 *                 against oracle/_ref/libref.so (depth <= 32) and
 *                 oracle/_ref/libref_wide.so (depth 33..64), and by the
 *                 committed golden SHA-256 digests in tests/golden/.
 *   pack_oracle.c bit-identical to src/dop.c (same checks).
 *   fir_oracle.c  FP64 restatement of src/fir.c + the engine glue; the
 *                 reference computes the FIR with Intel IPP, which is absent,
 *                 so FIR parity is unpinned beyond the reference's own
 *                 magnitude tests (passband, image rejection, counts).
 *   das_oracle.c  restatement of the DAS block of src/dsp_plugin.c; it drives
 *                 the pinned SDM restatement, but the stitch logic itself has
 *                 no reference golden vectors (parity unpinned for the seam
 *                 search; see the header of das_oracle.c).
 */
#ifndef DSD_ORACLE_H
#define DSD_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORA_MAX_ORDER 10     /* MAX_NTF_ORDER, include/ntf.h:11 */
#define ORA_MAX_K     32     /* SDM_TRELLIS_MAX_NUM, include/trellis.h:12 */
#define ORA_MAX_LAT   2048   /* SDM_TRELLIS_MAX_LAT, include/trellis.h:13 */
#define ORA_MAX_DEPTH 64     /* widened; the reference caps at 32 */
#define ORA_SLOTS     (2 * ORA_MAX_K)
#define ORA_NBUCKET   128    /* PATH_HASH_SIZE, include/trellis.h:14 */

/* One candidate slot of a trellis bank (the reference's sdm_state_t). */
typedef struct {
    double   s[ORA_MAX_ORDER];
    double   cost;
    uint64_t path;
    int16_t  link;       /* hash-chain successor: slot of the same bank, -1 none */
    int16_t  parent;     /* slot in the other bank this child was expanded from */
    uint8_t  next;       /* traceback bit carried by the candidate */
    uint8_t  ring;       /* history ring id */
    uint8_t  ring_taken; /* a child already took this parent's ring */
} ora_slot_t;

typedef struct {
    int      order;
    double   a[ORA_MAX_ORDER], g[ORA_MAX_ORDER];
    int      K, lat, depth;
    uint64_t mask;
    double   state_limit;

    ora_slot_t slot[2][ORA_SLOTS];
    int8_t     act[2][ORA_MAX_K];
    int16_t    heads[ORA_NBUCKET];
    int        n, bank;
    unsigned   pos, pending, draining;
    uint8_t    free_ring[2 * ORA_MAX_K];
    unsigned   nfree;
    uint8_t    rings[2 * ORA_MAX_K][ORA_MAX_LAT / 8];

    uint64_t conv_fail, cands_collapse, next_filter_drops, total_children;
} ora_sdm_t;

/* ---- trellis SDM (src/trellis.c) ---- */
ora_sdm_t *ora_sdm_new(int order, const double *a, const double *g, int depth,
                       int cands, int lat, double state_limit);
void   ora_sdm_free(ora_sdm_t *c);
size_t ora_sdm_process(ora_sdm_t *c, const double *in, float *out, size_t count);
size_t ora_sdm_process_bits(ora_sdm_t *c, const double *in, uint8_t *bits, size_t count);
size_t ora_sdm_drain(ora_sdm_t *c, float *out, size_t max_out);
void   ora_sdm_copy(ora_sdm_t *dst, const ora_sdm_t *src);
void   ora_sdm_reset(ora_sdm_t *c);
size_t ora_sdm_segment(ora_sdm_t *c, const double *in, float *out, size_t count,
                       size_t discard);
size_t ora_sdm_segment_bits(ora_sdm_t *c, const double *in, uint8_t *bits,
                            size_t count, size_t discard);
void   ora_sdm_seed(ora_sdm_t *c, const double *state);
void   ora_sdm_best_state(const ora_sdm_t *c, double *out);
void   ora_sdm_info(const ora_sdm_t *c, uint64_t *info);
int    ora_sdm_cand(const ora_sdm_t *c, unsigned i, double *state, double *cost,
                    uint64_t *path, unsigned *next);
void   ora_estimate_state(int order, const double *a, const double *g,
                          const double *init, const double *in, size_t count,
                          double state_limit, int levels, double *out);

/* Many independent segments on a thread pool (the CPU baseline). */
typedef struct {
    const double *in;
    uint8_t      *bits;
    size_t        count;
    size_t        discard;
    size_t        out_count;   /* written */
    const ora_sdm_t *seed;     /* context to copy before running (NULL: fresh) */
    const double *seed_state;  /* if non-NULL: seed active candidates */
    ora_sdm_t    *final_ctx;   /* if non-NULL: receives the context after the job */
} ora_seg_job_t;
int ora_sdm_run_jobs(int order, const double *a, const double *g, int depth,
                     int cands, int lat, double state_limit,
                     ora_seg_job_t *jobs, int njobs, int nthreads);

/* ---- DoP / bit packing (src/dop.c) ---- */
int  ora_dop_pack_i24(const float *bits, uint8_t *out, size_t n, int phase);
void ora_bits_pack(const float *src, uint8_t *dst, size_t n);
int  ora_dop_pack_u8(const uint8_t *bits, uint8_t *out, size_t n, int phase);
void ora_bits_pack_u8(const uint8_t *bits, uint8_t *dst, size_t n);
size_t ora_pack_dsf_u8(const uint8_t *bits, size_t stride, int nch, size_t n, uint8_t *out);
size_t ora_pack_dff_u8(const uint8_t *bits, size_t stride, int nch, size_t n, uint8_t *out);

/* ---- FIR chain + engine glue (src/fir.c, src/engine.c) ---- */
int  ora_fir_design(int ntaps, int quarter, double *h);
int  ora_fir_plan(unsigned fs_in, unsigned fs_out, int *factors, int *ntaps);
size_t ora_fir_upsample(unsigned fs_in, unsigned fs_out, const double *in,
                        size_t n, double *out);
void ora_boxcar(const double *in, double *out, size_t n, int taps);
void ora_gain_ramp(double *buf, size_t n, double g_start, double g_end);
void ora_soft_clip(double *buf, size_t n);
size_t ora_engine_fir(unsigned fs_in, unsigned fs_out, const float *in, size_t n,
                      int boxcar_taps, double g_start, double g_end, int soft_clip,
                      double *out);

/* ---- Same-rate DSD input (src/dop.c:74-87, src/engine.c:527-543) ---- */
typedef struct ora_boxcar ora_boxcar_t;
void ora_dop_unpack(const float *pcm24, float *bits, size_t frames);
ora_boxcar_t *ora_boxcar_new(int taps);
void ora_boxcar_free(ora_boxcar_t *b);
void ora_boxcar_gain(ora_boxcar_t *b, const float *in, double *out, size_t count,
                     double g_start, double g_end);

/* ---- Same-rate FIR lowpass (src/fir.c:795-872, src/engine.c:505-523) ---- */
typedef struct ora_lowpass ora_lowpass_t;
int  ora_lowpass_design(unsigned fs, double cutoff_hz, int ntaps, double *h);
ora_lowpass_t *ora_lowpass_new(unsigned fs, double cutoff_hz, int ntaps);
void ora_lowpass_free(ora_lowpass_t *lp);
int  ora_lowpass_taps(const ora_lowpass_t *lp, double *h);
void ora_lowpass_process(ora_lowpass_t *lp, const float *in, double *out, size_t count,
                         double g_start, double g_end);

/* ---- PreCorr greedy SDM (src/precorr.c) ---- */
typedef struct ora_precorr ora_precorr_t;
ora_precorr_t *ora_precorr_new(int order, const double *a, const double *g, double state_limit);
void ora_precorr_free(ora_precorr_t *p);
void ora_precorr_table(const ora_precorr_t *p, float *tab);
size_t ora_precorr_process(ora_precorr_t *p, const double *in, uint8_t *bits, size_t n);

/* ---- DSD -> PCM decimation (src/fir.c:467-487,523-611) ---- */
typedef struct ora_decim ora_decim_t;
ora_decim_t *ora_decim_new(unsigned fs_in, unsigned fs_out);
void ora_decim_free(ora_decim_t *d);
size_t ora_decim_process(ora_decim_t *d, const double *in, size_t n, double *out);
/* DSD -> DSD downsampling branch (src/engine.c:600-717, downsampling chain) */
size_t ora_engine_down(ora_boxcar_t *bc, ora_decim_t *d, const float *in, size_t n,
                       double g_start, double g_end, int soft_clip, double *out);

/* ---- DAS (src/dsp_plugin.c DAS block) ---- */
typedef struct {
    int    seg_len;        /* nominal segment length in FIR samples (0: from nsegs) */
    int    nsegs;          /* used when seg_len == 0 */
    int    seed_mode;      /* 0 = full-parallel (persistent seed), 1 = seg0-first */
    int    reposition;     /* apply the RMS boundary reposition for seg >= 2 */
} ora_das_cfg_t;
size_t ora_das_run(int order, const double *a, const double *g, int depth,
                   int cands, int lat, double state_limit,
                   const ora_das_cfg_t *cfg, const double *const *fir, size_t count,
                   int nch, uint8_t *const *out_bits, int *stitch_pos,
                   size_t *seg_starts, int nthreads);
/* The same for one chunk of a stream: carry[ch] is the channel's persistent
 * context (fresh for the first chunk), continued by seg0 and replaced by the
 * last segment's final context when the chunk has more than one segment
 * (src/dsp_plugin.c:2714-2721). */
size_t ora_das_run_carry(int order, const double *a, const double *g, int depth,
                         int cands, int lat, double state_limit,
                         const ora_das_cfg_t *cfg, const double *const *fir, size_t count,
                         int nch, uint8_t *const *out_bits, int *stitch_pos,
                         size_t *seg_starts, int nthreads, ora_sdm_t *const *carry);

#ifdef __cplusplus
}
#endif
#endif
