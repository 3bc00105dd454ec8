/*
 * ORACLE — test infrastructure only (see oracle.h).
 *
 * Restatement of the reference's same-rate DSD input path:
 *   - dop_unpack (src/dop.c:74-87): each float DoP sample is rounded to a
 *     24-bit integer (f * 2^23, half away from zero, src/dop.c:19-25) and its
 *     low 16 bits are 16 DSD bits, MSB first, written as +-1.0f;
 *   - the same-rate boxcar of engine_process_block (src/engine.c:527-543):
 *     a running FP64 sum over `taps` +-1 values (ring, initially zero), times
 *     1/taps, times the linear gain ramp g_start + g_step * i (the first
 *     chunk's g_start of 0 means g_end), in the reference's operation order.
 * The ring state is carried across calls through ora_boxcar_t.
 */
#include "oracle.h"

#include <stdlib.h>
#include <string.h>

static int32_t to_int24(float f)
{
    double d = (double)f * 8388608.0;
    return d >= 0.0 ? (int32_t)(d + 0.5) : (int32_t)(d - 0.5);
}

void ora_dop_unpack(const float *pcm24, float *bits, size_t frames)
{
    for (size_t i = 0; i < frames; i++) {
        uint16_t w = (uint16_t)(to_int24(pcm24[i]) & 0xFFFF);
        for (int b = 15; b >= 0; b--) *bits++ = ((w >> b) & 1u) ? 1.0f : -1.0f;
    }
}

struct ora_boxcar {
    int taps;
    int pos;
    double sum;
    double *ring;
};

ora_boxcar_t *ora_boxcar_new(int taps)
{
    ora_boxcar_t *b = (ora_boxcar_t *)calloc(1, sizeof *b);
    if (!b) return NULL;
    b->taps = taps;
    b->ring = (double *)calloc((size_t)taps, sizeof(double));
    if (!b->ring) { free(b); return NULL; }
    return b;
}

void ora_boxcar_free(ora_boxcar_t *b)
{
    if (b) { free(b->ring); free(b); }
}

void ora_boxcar_gain(ora_boxcar_t *bc, const float *in, double *out, size_t count,
                     double g_start, double g_end)
{
    const double inv_n = 1.0 / (double)bc->taps;
    if (g_start == 0.0) g_start = g_end;
    const double g_step = (count > 1) ? (g_end - g_start) / (double)(count - 1) : 0.0;
    for (size_t i = 0; i < count; i++) {
        double s = in[i] >= 0.0f ? 1.0 : -1.0;
        bc->sum -= bc->ring[bc->pos];
        bc->ring[bc->pos] = s;
        bc->sum += s;
        bc->pos = (bc->pos + 1) % bc->taps;
        out[i] = bc->sum * inv_n * (g_start + g_step * (double)i);
    }
}
