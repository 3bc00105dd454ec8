/*
 * ORACLE — test infrastructure only (see oracle.h).  Not shipped, not measured
 * as the product; the CUDA path never calls it.
 *
 * Restatement of the reference trellis (Viterbi look-ahead) 1-bit SDM,
 * src/trellis.c, in the scalar form gcc builds (the MSVC/AVX2 branches at
 * src/trellis.c:882-928 are compiled out there).  It is written against an
 * explicit slot-memory model so that the GPU kernel can follow the same model:
 *
 *  - each of the two trellis banks has 2K candidate slots; a parent at act
 *    rank i expands into slots 2i (decision bit 0, state[0] + 1) and 2i + 1
 *    (bit 1, state[0] - 1)                      (src/trellis.c:153-191, 735-746)
 *  - costs are ordered by their IEEE-754 bit patterns read as int64
 *                                               (src/trellis.c:582-597)
 *  - path dedup is a 128-bucket chained hash keyed by path & 127 whose chains
 *    run through a per-slot link that survives from sort to sort
 *                                               (src/trellis.c:601-617)
 *  - at K = 32 the reference's first insertion loop stores act[32], one past
 *    the array (src/trellis.c:668-673).  In the reference layout that word is
 *    trellis[1].sdm[0].state[0] when bank 0 is being sorted (never read before
 *    it is rewritten) and path_hash[0] when bank 1 is being sorted.  The
 *    restatement reproduces the second effect exactly (heads[0] = evicted slot)
 *    because it changes which duplicates the dedup finds.
 *  - links, parents and act entries are slot indices, so a copy of the
 *    context (sdm_context_copy_state) keeps them pointing into the copy.  In
 *    the reference a copied path_list still points into the source context;
 *    the two agree unless a corrupted bucket-0 chain (K = 32 only) walks into
 *    a link inherited from a copy.
 */
#include "oracle.h"
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define NIL (-1)

static inline int64_t cost_key(double c)
{
    int64_t k;
    memcpy(&k, &c, sizeof k);
    return k;
}

/* NTF advance with y = 0 for one parent (src/trellis.c:37-151): writes the
 * shared child state d[] and returns the filter output v.  Operation order is
 * left to right, no contraction. */
static inline double ntf_advance(const ora_sdm_t *c, const double *s, double *d, double x)
{
    const int N = c->order;
    const double *a = c->a, *g = c->g;
    double v;
    d[0] = s[0] - g[0] * s[1] + x;
    v = x + a[0] * d[0];
    int i;
    for (i = 1; i < N - 1; i++) {
        d[i] = s[i] + s[i - 1] - g[i] * s[i + 1];
        v += a[i] * d[i];
    }
    d[i] = s[i] + s[i - 1];
    v += a[i] * d[i];
    return v;
}

static inline double clamp_state(double v, double lim)
{
    if (v > lim) return lim;
    if (v < -lim) return -lim;
    return v;
}

static inline unsigned ring_get(const uint8_t *r, unsigned i) { return (r[i >> 3] >> (i & 7)) & 1u; }
static inline void ring_put(uint8_t *r, unsigned i, unsigned v)
{
    r[i >> 3] = (uint8_t)((r[i >> 3] & ~(1u << (i & 7))) | (v << (i & 7)));
}

static void sdm_init_fields(ora_sdm_t *c)
{
    memset(c->slot, 0, sizeof c->slot);
    /* the reference zeroes its slots, so every path_list starts as NULL */
    for (int b = 0; b < 2; b++)
        for (int i = 0; i < ORA_SLOTS; i++) c->slot[b][i].link = c->slot[b][i].parent = NIL;
    memset(c->act, 0, sizeof c->act);
    for (int i = 0; i < ORA_NBUCKET; i++) c->heads[i] = NIL;
    memset(c->rings, 0, sizeof c->rings);
    c->n = 1;
    c->bank = 0;
    c->pos = c->pending = c->draining = 0;
    c->nfree = 0;
    for (int i = 0; i < 2 * c->K; i++) c->free_ring[c->nfree++] = (uint8_t)i;
    /* the first candidate takes the ring popped last from the free list */
    c->slot[0][0].ring = c->free_ring[--c->nfree];
    c->slot[0][0].path = 0;
    c->act[0][0] = 0;
}

ora_sdm_t *ora_sdm_new(int order, const double *a, const double *g, int depth,
                       int cands, int lat, double state_limit)
{
    /* parameter limits of sdm_context_init (src/trellis.c:981-990), depth widened */
    if (!a || !g || order < 2 || order > ORA_MAX_ORDER) return NULL;
    if (depth < 1 || depth > ORA_MAX_DEPTH || cands < 1 || cands > ORA_MAX_K ||
        lat < 1 || lat > ORA_MAX_LAT)
        return NULL;
    ora_sdm_t *c = (ora_sdm_t *)calloc(1, sizeof *c);
    if (!c) return NULL;
    c->order = order;
    memcpy(c->a, a, sizeof c->a);
    memcpy(c->g, g, sizeof c->g);
    c->K = cands;
    c->lat = lat;
    c->depth = depth;
    c->mask = depth >= 64 ? ~(uint64_t)0 : (((uint64_t)1 << depth) - 1);
    c->state_limit = state_limit;
    for (int i = 0; i < ORA_NBUCKET; i++) c->heads[i] = NIL;
    sdm_init_fields(c);
    return c;
}

void ora_sdm_free(ora_sdm_t *c) { free(c); }

/* Hash lookup-or-insert of child slot `si` of bank `b` (src/trellis.c:601-617). */
static int path_lookup(ora_sdm_t *c, int b, int si)
{
    ora_slot_t *S = c->slot[b];
    unsigned h = (unsigned)(S[si].path & (ORA_NBUCKET - 1));
    for (int t = c->heads[h]; t != NIL; t = S[t].link)
        if (S[t].path == S[si].path)
            return t;
    S[si].link = c->heads[h];
    c->heads[h] = (int16_t)si;
    return NIL;
}

/* Store into act position j of bank b.  Position K == 32 is one past the
 * reference's array; see the file header for what that store hits. */
static inline void act_store(ora_sdm_t *c, int b, unsigned j, int slot)
{
    if (j < ORA_MAX_K) c->act[b][j] = (int8_t)slot;
    else if (b == 1) c->heads[0] = (int16_t)slot;
}

/* Survivor selection over the 2n children of bank b (src/trellis.c:621-731). */
static unsigned select_survivors(ora_sdm_t *c, int b, unsigned nchild)
{
    ora_slot_t *S = c->slot[b];
    int8_t *act = c->act[b];
    const unsigned K = (unsigned)c->K;
    int min = NIL;

    for (unsigned i = 0; i < nchild; i++) {
        c->heads[S[i].path & (ORA_NBUCKET - 1)] = NIL;
        if (min == NIL || cost_key(S[i].cost) < cost_key(S[min].cost))
            min = (int)i;
    }
    c->total_children += nchild;

    unsigned votes1 = 0;
    for (unsigned i = 0; i < nchild; i++) votes1 += S[i].next & 1u;
    unsigned majority = (votes1 > nchild - votes1) ? 1u : 0u;
    if (S[min].next != majority) {
        int bm = NIL;
        for (unsigned i = 0; i < nchild; i++)
            if (S[i].next == majority && (bm == NIL || cost_key(S[i].cost) < cost_key(S[bm].cost)))
                bm = (int)i;
        if (bm != NIL && S[bm].cost < S[min].cost * 1.1)
            min = bm;
    }
    const unsigned want = S[min].next;

    unsigned n = 0;
    for (unsigned i = 0; i < nchild; i++) {
        const int s = (int)i;
        const int64_t ks = cost_key(S[s].cost);
        if (S[s].next != want) { c->next_filter_drops++; continue; }
        if (n == K && cost_key(S[act[n - 1]].cost) <= ks) continue;

        int t = path_lookup(c, b, s);
        unsigned j;
        if (t == NIL) {
            for (j = n; j > 0; j--) {
                int r = act[j - 1];
                if (cost_key(S[r].cost) <= ks) break;
                act_store(c, b, j, r);
            }
            if (j < K) act[j] = (int8_t)s;
            if (n < K) n++;
            continue;
        }
        if (cost_key(S[t].cost) <= ks) continue;

        unsigned tp;
        for (tp = 0; tp < n; tp++)
            if (act[tp] == t) break;
        if (tp == n) {
            /* t was already evicted: insert s as if new */
            for (j = n; j > 0; j--) {
                int r = act[j - 1];
                if (cost_key(S[r].cost) <= ks) break;
                if (j < K) act[j] = (int8_t)r;
            }
            if (j < K) act[j] = (int8_t)s;
            if (n < K) n++;
            continue;
        }
        /* replace t by s */
        for (j = tp; j + 1 < n; j++) act[j] = act[j + 1];
        n--;
        for (j = n; j > 0; j--) {
            int r = act[j - 1];
            if (cost_key(S[r].cost) <= ks) break;
            if (j < K) act[j] = (int8_t)r;
        }
        if (j < K) act[j] = (int8_t)s;
        n++;
    }
    return n;
}

/* One input sample (src/trellis.c:868-973).  Returns the traceback bit. */
static unsigned sdm_step_sample(ora_sdm_t *c, double x)
{
    const int cb = c->bank, nb = cb ^ 1;
    ora_slot_t *P = c->slot[cb], *C = c->slot[nb];
    const int N = c->order;
    const double a0 = c->a[0];
    const double lim = c->state_limit;
    unsigned next_pos = c->pos + 1;
    if (next_pos == (unsigned)c->lat) next_pos = 0;

    for (int i = 0; i < c->n; i++) {
        const int ps = c->act[cb][i];
        ora_slot_t *p = &P[ps];
        ora_slot_t *c0 = &C[2 * i], *c1 = &C[2 * i + 1];
        double d[ORA_MAX_ORDER];
        double v = ntf_advance(c, p->s, d, x);
        for (int k = 0; k < N; k++) { c0->s[k] = d[k]; c1->s[k] = d[k]; }
        c0->s[0] += 1.0;
        c1->s[0] -= 1.0;
        if (lim > 0.0) {
            for (int k = 0; k < N; k++) {
                c0->s[k] = clamp_state(c0->s[k], lim);
                c1->s[k] = clamp_state(c1->s[k], lim);
            }
        }
        double e0 = v + a0, e1 = v - a0;
        c0->cost = p->cost + e0 * e0;
        c1->cost = p->cost + e1 * e1;
        c0->path = ((p->path << 1) | 0u) & c->mask;
        c1->path = ((p->path << 1) | 1u) & c->mask;
        c0->ring = c1->ring = p->ring;
        c0->next = c1->next = p->next;
        c0->parent = c1->parent = (int16_t)ps;
        p->next = (uint8_t)ring_get(c->rings[p->ring], next_pos);
        p->ring_taken = 0;
    }

    const unsigned n_old = (unsigned)c->n;
    unsigned n_new = select_survivors(c, nb, 2u * n_old);
    const int8_t *act = c->act[nb];
    const double min_cost = C[act[0]].cost;
    const unsigned out = C[act[0]].next;

    for (unsigned i = 0; i < n_new; i++) {
        ora_slot_t *s = &C[act[i]];
        ora_slot_t *p = &P[s->parent];
        if (p->ring_taken) {
            uint8_t h = c->free_ring[--c->nfree];
            memcpy(c->rings[h], c->rings[s->ring], (size_t)(c->lat + 7) / 8);
            s->ring = h;
        } else {
            p->ring_taken = 1;
        }
        s->cost -= min_cost;
        s->next = p->next;
        ring_put(c->rings[s->ring], c->pos, (unsigned)(s->path & 1u));
    }
    for (unsigned i = 0; i < n_old; i++) {
        ora_slot_t *p = &P[c->act[cb][i]];
        if (!p->ring_taken) c->free_ring[c->nfree++] = p->ring;
    }
    if (n_new < n_old) { c->conv_fail++; c->cands_collapse++; }
    c->n = (int)n_new;
    c->pos = next_pos;
    c->bank = nb;
    return out;
}

/* sdm_process_block (src/trellis.c:1013-1040). */
size_t ora_sdm_process(ora_sdm_t *c, const double *in, float *out, size_t count)
{
    size_t len = count, produced = 0;
    if (c->pending < (unsigned)c->lat) {
        size_t pre = (size_t)c->lat - c->pending;
        if (pre > len) pre = len;
        c->pending += (unsigned)pre;
        len -= pre;
        while (pre--) sdm_step_sample(c, *in++);
    }
    while (len--) out[produced++] = sdm_step_sample(c, *in++) ? 1.0f : -1.0f;
    return produced;
}

size_t ora_sdm_process_bits(ora_sdm_t *c, const double *in, uint8_t *bits, size_t count)
{
    size_t len = count, produced = 0;
    if (c->pending < (unsigned)c->lat) {
        size_t pre = (size_t)c->lat - c->pending;
        if (pre > len) pre = len;
        c->pending += (unsigned)pre;
        len -= pre;
        while (pre--) sdm_step_sample(c, *in++);
    }
    while (len--) bits[produced++] = (uint8_t)sdm_step_sample(c, *in++);
    return produced;
}

/* sdm_drain (src/trellis.c:1042-1062). */
size_t ora_sdm_drain(ora_sdm_t *c, float *out, size_t max_out)
{
    size_t len = c->pending;
    if (len > max_out) len = max_out;
    if (!c->draining && c->pending < (unsigned)c->lat) {
        unsigned flush = (unsigned)c->lat - c->pending;
        while (flush--) sdm_step_sample(c, 0.0);
    }
    c->draining = 1;
    c->pending -= (unsigned)len;
    for (size_t i = 0; i < len; i++) out[i] = sdm_step_sample(c, 0.0) ? 1.0f : -1.0f;
    return len;
}

/* sdm_context_copy_state (src/trellis.c:1064-1092). */
void ora_sdm_copy(ora_sdm_t *dst, const ora_sdm_t *src)
{
    memcpy(dst, src, sizeof *dst);
    for (int i = 0; i < ORA_NBUCKET; i++) dst->heads[i] = NIL;
    dst->conv_fail = dst->cands_collapse = dst->next_filter_drops = dst->total_children = 0;
}

/* sdm_context_reset (src/trellis.c:1189-1224): only conv_fail of the counters
 * is cleared there. */
void ora_sdm_reset(ora_sdm_t *c)
{
    sdm_init_fields(c);
    c->conv_fail = 0;
}

/* The warmup/discard wrapper sdm_segment_process (src/engine.c:915-938). */
static size_t segment_common(ora_sdm_t *c, const double *in, float *out, uint8_t *bits,
                             size_t count, size_t discard)
{
    if (discard == 0)
        return out ? ora_sdm_process(c, in, out, count) : ora_sdm_process_bits(c, in, bits, count);
    size_t warm = (size_t)c->lat + discard;
    size_t feed = warm > count ? count : warm;
    /* the discarded part: run the trellis, drop the decisions */
    size_t len = feed;
    if (c->pending < (unsigned)c->lat) {
        size_t pre = (size_t)c->lat - c->pending;
        if (pre > len) pre = len;
        c->pending += (unsigned)pre;
        len -= pre;
        while (pre--) sdm_step_sample(c, *in++);
    }
    while (len--) sdm_step_sample(c, *in++);
    if (warm > count) return 0;
    return out ? ora_sdm_process(c, in, out, count - warm)
               : ora_sdm_process_bits(c, in, bits, count - warm);
}

size_t ora_sdm_segment(ora_sdm_t *c, const double *in, float *out, size_t count, size_t discard)
{
    return segment_common(c, in, out, NULL, count, discard);
}

size_t ora_sdm_segment_bits(ora_sdm_t *c, const double *in, uint8_t *bits, size_t count,
                            size_t discard)
{
    return segment_common(c, in, NULL, bits, count, discard);
}

/* DAS temp seeding (src/dsp_plugin.c:2316-2326). */
void ora_sdm_seed(ora_sdm_t *c, const double *state)
{
    for (int i = 0; i < c->n; i++) {
        ora_slot_t *s = &c->slot[c->bank][c->act[c->bank][i]];
        for (int k = 0; k < c->order; k++) s->s[k] = state[k];
        s->cost = 0.0;
    }
}

void ora_sdm_best_state(const ora_sdm_t *c, double *out)
{
    const ora_slot_t *s = &c->slot[c->bank][c->act[c->bank][0]];
    for (int k = 0; k < c->order; k++) out[k] = s->s[k];
}

void ora_sdm_info(const ora_sdm_t *c, uint64_t *info)
{
    info[0] = (uint64_t)c->n;
    info[1] = c->pos;
    info[2] = c->pending;
    info[3] = (uint64_t)c->bank;
    info[4] = c->draining;
    info[5] = c->conv_fail;
    info[6] = c->cands_collapse;
    info[7] = c->next_filter_drops;
    info[8] = c->total_children;
}

int ora_sdm_cand(const ora_sdm_t *c, unsigned i, double *state, double *cost,
                 uint64_t *path, unsigned *next)
{
    if ((int)i >= c->n) return -1;
    const ora_slot_t *s = &c->slot[c->bank][c->act[c->bank][i]];
    for (int k = 0; k < c->order; k++) state[k] = s->s[k];
    *cost = s->cost;
    *path = s->path;
    *next = s->next;
    return 0;
}

/* Greedy multi-level state estimator (src/trellis.c:1125-1187). */
void ora_estimate_state(int order, const double *a, const double *g,
                        const double *init, const double *in, size_t count,
                        double state_limit, int levels, double *out)
{
    double st[ORA_MAX_ORDER], ns[ORA_MAX_ORDER];
    const double step = 2.0 / (double)(levels - 1);
    for (int i = 0; i < order; i++) st[i] = init[i];
    for (size_t n = 0; n < count; n++) {
        const double x = in[n];
        ns[0] = st[0] - g[0] * st[1] + x;
        double v = x + a[0] * ns[0];
        for (int i = 1; i < order - 1; i++) {
            ns[i] = st[i] + st[i - 1] - g[i] * st[i + 1];
            v += a[i] * ns[i];
        }
        ns[order - 1] = st[order - 1] + st[order - 2];
        v += a[order - 1] * ns[order - 1];
        double y;
        if (levels <= 2) {
            y = (v * a[0] > 0.0) ? 1.0 : -1.0;
        } else {
            double yi = v / a[0];
            int idx = (int)((yi + 1.0) / step + 0.5);
            if (idx < 0) idx = 0;
            if (idx > levels - 1) idx = levels - 1;
            y = -1.0 + (double)idx * step;
        }
        ns[0] -= y;
        if (state_limit > 0.0)
            for (int i = 0; i < order; i++) ns[i] = clamp_state(ns[i], state_limit);
        for (int i = 0; i < order; i++) st[i] = ns[i];
    }
    for (int i = 0; i < order; i++) out[i] = st[i];
}

/* ---- thread pool over independent segments (CPU baseline) ---- */

typedef struct {
    ora_seg_job_t *jobs;
    int njobs;
    int next;
    pthread_mutex_t mu;
    const ora_sdm_t *proto;
} pool_t;

static void *pool_worker(void *arg)
{
    pool_t *p = (pool_t *)arg;
    ora_sdm_t *c = (ora_sdm_t *)malloc(sizeof *c);
    if (!c) return NULL;
    for (;;) {
        pthread_mutex_lock(&p->mu);
        int j = p->next++;
        pthread_mutex_unlock(&p->mu);
        if (j >= p->njobs) break;
        ora_seg_job_t *jb = &p->jobs[j];
        if (jb->seed) ora_sdm_copy(c, jb->seed);
        else memcpy(c, p->proto, sizeof *c);
        if (jb->seed_state) ora_sdm_seed(c, jb->seed_state);
        jb->out_count = ora_sdm_segment_bits(c, jb->in, jb->bits, jb->count, jb->discard);
        if (jb->final_ctx) ora_sdm_copy(jb->final_ctx, c);
    }
    free(c);
    return NULL;
}

int ora_sdm_run_jobs(int order, const double *a, const double *g, int depth,
                     int cands, int lat, double state_limit,
                     ora_seg_job_t *jobs, int njobs, int nthreads)
{
    ora_sdm_t *proto = ora_sdm_new(order, a, g, depth, cands, lat, state_limit);
    if (!proto) return -1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > njobs) nthreads = njobs > 0 ? njobs : 1;
    pool_t p;
    p.jobs = jobs;
    p.njobs = njobs;
    p.next = 0;
    p.proto = proto;
    pthread_mutex_init(&p.mu, NULL);
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof *th);
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, pool_worker, &p);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&p.mu);
    ora_sdm_free(proto);
    return 0;
}
