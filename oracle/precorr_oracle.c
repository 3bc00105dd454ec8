/*
 * ORACLE — test infrastructure only (see oracle.h).
 *
 * Restatement of the reference's PreCorr SDM (src/precorr.c, header
 * include/precorr.h): a greedy 1-bit quantiser after the same NTF loop as the
 * trellis but in single precision (the reference builds it with precise
 * floating point: every operation rounded separately, left to right), with a
 * prediction table of 256 output histories x 8 phases trained at init on
 * 65,536 samples of LCG noise at amplitude 0.1 (mean quantiser residual per
 * cell, cells with fewer than 4 hits zero), then per sample:
 *   v = NTF(x, previous output); y = sign(v); state <- d (clamped if a limit);
 *   out = sign(y - table[history][phase]); history <- history << 1 | out.
 */
#include "oracle.h"

#include <stdlib.h>
#include <string.h>

#define PC_HIST 256
#define PC_PHASES 8
#define PC_TRAIN 65536
#define PC_AMP 0.1f
#define PC_MIN_HITS 4

struct ora_precorr {
    int order;
    float a[10], g[10];
    float state[10];
    float table[PC_HIST][PC_PHASES];
    unsigned history;
    int phase;
    float prev_y;
    float limit;
};

static float pc_filter(const float *s, float *d, const float *a, const float *g, int order,
                       float x, float y)
{
    d[0] = s[0] - g[0] * s[1] + x - y;
    float v = x + a[0] * d[0];
    int i;
    for (i = 1; i < order - 1; i++) {
        d[i] = s[i] + s[i - 1] - g[i] * s[i + 1];
        v += a[i] * d[i];
    }
    d[i] = s[i] + s[i - 1];
    v += a[i] * d[i];
    return v;
}

ora_precorr_t *ora_precorr_new(int order, const double *a, const double *g, double state_limit)
{
    if (order < 2 || order > 10) return NULL;
    ora_precorr_t *p = (ora_precorr_t *)calloc(1, sizeof *p);
    if (!p) return NULL;
    p->order = order;
    for (int i = 0; i < order; i++) { p->a[i] = (float)a[i]; p->g[i] = (float)g[i]; }
    p->limit = (float)state_limit;
    /* training (the limiter is not applied) */
    static float accum[PC_HIST][PC_PHASES];
    static int hits[PC_HIST][PC_PHASES];
    memset(accum, 0, sizeof accum);
    memset(hits, 0, sizeof hits);
    float st[10] = {0}, d[10];
    unsigned hist = 0x69;
    int ph = 0;
    float py = 0.0f;
    uint32_t rng = 0xDEADBEEFu;
    for (int i = 0; i < PC_TRAIN; i++) {
        rng = rng * 1664525u + 1013904223u;
        float x = PC_AMP * ((float)(int32_t)rng / 2147483648.0f);
        float v = pc_filter(st, d, p->a, p->g, order, x, py);
        float y = v >= 0.0f ? 1.0f : -1.0f;
        memcpy(st, d, (size_t)order * sizeof(float));
        accum[hist][ph] += y - v;
        hits[hist][ph]++;
        hist = ((hist << 1) | (y > 0.0f ? 1u : 0u)) & 0xFFu;
        ph = (ph + 1) & (PC_PHASES - 1);
        py = y;
    }
    for (int h = 0; h < PC_HIST; h++)
        for (int q = 0; q < PC_PHASES; q++)
            p->table[h][q] = hits[h][q] >= PC_MIN_HITS ? accum[h][q] / (float)hits[h][q] : 0.0f;
    p->history = 0x69;
    return p;
}

void ora_precorr_free(ora_precorr_t *p) { free(p); }

void ora_precorr_table(const ora_precorr_t *p, float *tab)
{
    memcpy(tab, p->table, sizeof p->table);
}

size_t ora_precorr_process(ora_precorr_t *p, const double *in, uint8_t *bits, size_t n)
{
    float d[10];
    for (size_t i = 0; i < n; i++) {
        float x = (float)in[i];
        float v = pc_filter(p->state, d, p->a, p->g, p->order, x, p->prev_y);
        float y = v >= 0.0f ? 1.0f : -1.0f;
        if (p->limit > 0.0f)
            for (int k = 0; k < p->order; k++) {
                if (d[k] > p->limit) d[k] = p->limit;
                else if (d[k] < -p->limit) d[k] = -p->limit;
            }
        memcpy(p->state, d, (size_t)p->order * sizeof(float));
        float yc = y - p->table[p->history][p->phase];
        float out = yc >= 0.0f ? 1.0f : -1.0f;
        bits[i] = out > 0.0f ? 1u : 0u;
        p->history = ((p->history << 1) | bits[i]) & 0xFFu;
        p->phase = (p->phase + 1) & (PC_PHASES - 1);
        p->prev_y = out;
    }
    return n;
}
