/*
 * Test infrastructure only (oracle): a thin driver around the reference's own
 * trellis SDM, NTF table, DoP packers and PreCorr SDM, compiled from the
 * reference sources in place (src/trellis.c, src/ntf.c, src/dop.c,
 * src/precorr.c) by oracle/Makefile into
 * oracle/_ref/.  Nothing here is shipped or measured; the product never links
 * it.  It exists so that the C restatement in oracle/sdm_oracle.c and the CUDA
 * kernels can be checked against the reference's real code.
 *
 * Built twice:
 *   libref.so       the reference types, unmodified (depth <= 32).
 *   libref_wide.so  the same sources compiled with ref_widen.h force-included,
 *                   which widens every uint32_t (path, trellis_mask) to 64
 *                   bits.  sdm_context_init (src/trellis.c:984-987) still caps
 *                   the depth argument at SDM_TRELLIS_MAX_ORDER = 32, so for a
 *                   depth above 32 this driver initialises with depth 32 and
 *                   then writes the widened mask itself (a shift by 64 is
 *                   undefined in C, so depth 64 is spelled as all ones).
 */
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include "trellis.h"
#include "ntf.h"
#include "dop.h"
#include "precorr.h"

typedef struct {
    ntf_filter_t  filt;     /* the context keeps a pointer to its filter */
    sdm_context_t ctx;
} ref_sdm_t;

int ref_path_bits(void) { return (int)(8 * sizeof(((sdm_state_t *)0)->path)); }

int ref_ntf_count(void) { return ntf_get_filter_count(); }

/* Copy table entry `idx` out (src/ntf.c:16-790). */
int ref_ntf_entry(int idx, double *a, double *g, int *order, unsigned *freq,
                  char *name, int name_len)
{
    const ntf_filter_t *f = ntf_get_by_index(idx);
    if (!f) return -1;
    memcpy(a, f->a, sizeof(f->a));
    memcpy(g, f->g, sizeof(f->g));
    *order = f->order;
    *freq = f->freq;
    strncpy(name, f->name, (size_t)name_len - 1);
    name[name_len - 1] = 0;
    return 0;
}

/* Index of ntf_get_filter(id, rate) in the table, -1 if none (src/ntf.c:814-832). */
int ref_ntf_lookup(int id, unsigned rate)
{
    const ntf_filter_t *f = ntf_get_filter((ntf_filter_id_t)id, rate);
    if (!f) return -1;
    for (int i = 0; i < ntf_get_filter_count(); i++)
        if (ntf_get_by_index(i) == f) return i;
    return -1;
}

int ref_ntf_auto(unsigned rate)
{
    const ntf_filter_t *f = ntf_auto_select(rate);
    if (!f) return -1;
    for (int i = 0; i < ntf_get_filter_count(); i++)
        if (ntf_get_by_index(i) == f) return i;
    return -1;
}

void *ref_sdm_new(int order, const double *a, const double *g, int depth,
                  int cands, int lat, double state_limit)
{
    ref_sdm_t *r = (ref_sdm_t *)calloc(1, sizeof(ref_sdm_t));
    if (!r) return NULL;
    memcpy(r->filt.a, a, sizeof(r->filt.a));
    memcpy(r->filt.g, g, sizeof(r->filt.g));
    r->filt.order = order;
    r->filt.name = "driver";
    int init_depth = depth;
    if (8 * sizeof(r->ctx.trellis_mask) > 32 && depth > 32)
        init_depth = 32;
    if (sdm_context_init(&r->ctx, &r->filt, init_depth, cands, lat) != 0) {
        free(r);
        return NULL;
    }
    if (init_depth != depth) {
        if (depth >= 64) r->ctx.trellis_mask = ~(uint64_t)0;
        else             r->ctx.trellis_mask = ((uint64_t)1 << depth) - 1;
    }
    r->ctx.state_limit = state_limit;
    return r;
}

void ref_sdm_free(void *p)
{
    ref_sdm_t *r = (ref_sdm_t *)p;
    if (!r) return;
    sdm_context_free(&r->ctx);
    free(r);
}

size_t ref_sdm_process(void *p, const double *in, float *out, size_t count)
{
    return sdm_process_block(&((ref_sdm_t *)p)->ctx, in, out, count);
}

size_t ref_sdm_drain(void *p, float *out, size_t max_out)
{
    return sdm_drain(&((ref_sdm_t *)p)->ctx, out, max_out);
}

void ref_sdm_reset(void *p) { sdm_context_reset(&((ref_sdm_t *)p)->ctx); }

/* dst must have been created with the same parameters. */
void ref_sdm_copy(void *dst, const void *src)
{
    ref_sdm_t *d = (ref_sdm_t *)dst;
    const ref_sdm_t *s = (const ref_sdm_t *)src;
    sdm_context_copy_state(&d->ctx, &s->ctx);
    d->ctx.filter = &d->filt;   /* the copy points at src's filter; same values */
}

/* The warmup/discard wrapper of src/engine.c:915-938, restated (engine.c
 * itself needs Windows and IPP).  A NULL-free scratch buffer is used for the
 * discarded part. */
size_t ref_sdm_segment(void *p, const double *in, float *out, size_t count,
                       size_t discard)
{
    sdm_context_t *c = &((ref_sdm_t *)p)->ctx;
    if (discard == 0)
        return sdm_process_block(c, in, out, count);
    size_t warm = (size_t)c->trellis_lat + discard;
    float *trash = (float *)malloc((warm > count ? count : warm) * sizeof(float) + 4);
    if (!trash) return 0;
    if (warm > count) {
        sdm_process_block(c, in, trash, count);
        free(trash);
        return 0;
    }
    sdm_process_block(c, in, trash, warm);
    free(trash);
    return sdm_process_block(c, in + warm, out, count - warm);
}

/* Seed every active candidate of the current bank with `state` and zero
 * cost, as the DAS dispatch does for temp contexts (src/dsp_plugin.c:2316-2326). */
void ref_sdm_seed(void *p, const double *state)
{
    sdm_context_t *c = &((ref_sdm_t *)p)->ctx;
    int bank = c->idx & 1;
    for (unsigned i = 0; i < c->num_cands; i++) {
        sdm_state_t *st = c->trellis[bank].act[i];
        if (st) {
            for (int k = 0; k < c->filter->order; k++)
                st->state[k] = state[k];
            st->cost = 0.0;
        }
    }
}

/* Best candidate's integrator state (act[0] of the current bank). */
void ref_sdm_best_state(const void *p, double *out)
{
    const sdm_context_t *c = &((const ref_sdm_t *)p)->ctx;
    const sdm_state_t *s = c->trellis[c->idx & 1].act[0];
    for (int k = 0; k < c->filter->order; k++)
        out[k] = s->state[k];
}

/* Scalar fields: num_cands, pos, pending, idx, draining and the four counters. */
void ref_sdm_info(const void *p, uint64_t *info)
{
    const sdm_context_t *c = &((const ref_sdm_t *)p)->ctx;
    info[0] = c->num_cands;
    info[1] = c->pos;
    info[2] = c->pending;
    info[3] = c->idx;
    info[4] = c->draining;
    info[5] = c->conv_fail;
    info[6] = c->cands_collapse;
    info[7] = c->next_filter_drops;
    info[8] = c->total_children;
}

/* Candidate `i` of the current bank: state[0..order-1], cost, path, next. */
int ref_sdm_cand(const void *p, unsigned i, double *state, double *cost,
                 uint64_t *path, unsigned *next)
{
    const sdm_context_t *c = &((const ref_sdm_t *)p)->ctx;
    if (i >= c->num_cands) return -1;
    const sdm_state_t *s = c->trellis[c->idx & 1].act[i];
    for (int k = 0; k < c->filter->order; k++) state[k] = s->state[k];
    *cost = s->cost;
    *path = s->path;
    *next = s->next;
    return 0;
}

void ref_estimate_state(int order, const double *a, const double *g,
                        const double *init, const double *in, size_t count,
                        double state_limit, int levels, double *out)
{
    ntf_filter_t f;
    memset(&f, 0, sizeof(f));
    memcpy(f.a, a, sizeof(f.a));
    memcpy(f.g, g, sizeof(f.g));
    f.order = order;
    sdm_estimate_state_multibit(&f, init, in, count, state_limit, levels, out);
}

int ref_dop_pack_i24(const float *bits, uint8_t *out, size_t n, int phase)
{
    return dop_pack_i24(bits, out, n, phase);
}

void ref_bits_pack(const float *src, uint8_t *dst, size_t n) { bits_pack(src, dst, n); }
void ref_bits_unpack(const uint8_t *src, float *dst, size_t n) { bits_unpack(src, dst, n); }
void ref_dop_unpack(const float *pcm, float *bits, size_t frames) { dop_unpack(pcm, bits, frames); }
void ref_dop_pack(const float *bits, float *pcm, size_t n) { dop_pack(bits, pcm, n); }

/* ---- PreCorr (src/precorr.c) ---- */
typedef struct {
    ntf_filter_t filt;
    precorr_context_t ctx;
} ref_precorr_t;

void *ref_precorr_new(int order, const double *a, const double *g, double state_limit)
{
    ref_precorr_t *p = (ref_precorr_t *)calloc(1, sizeof *p);
    if (!p) return NULL;
    p->filt.order = order;
    for (int i = 0; i < order; i++) { p->filt.a[i] = a[i]; p->filt.g[i] = g[i]; }
    if (precorr_context_init(&p->ctx, &p->filt) != 0) { free(p); return NULL; }
    p->ctx.state_limit = (float)state_limit;
    return p;
}

void ref_precorr_free(void *h) { free(h); }

size_t ref_precorr_process(void *h, const double *in, float *out, size_t n)
{
    return precorr_process_block(&((ref_precorr_t *)h)->ctx, in, out, n);
}

void ref_precorr_table(void *h, float *tab)
{
    memcpy(tab, ((ref_precorr_t *)h)->ctx.pred_table, sizeof(float) * PRECORR_HIST_SIZE * PRECORR_PHASES);
}
