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

/*
 * DSD -> PCM decimation (fir_chain_init_ex downsampling, src/fir.c:523-611;
 * ipp_downsample_d, src/fir.c:467-487; the FIR-only engine branch,
 * src/engine.c:566-577 with the gain ramp of src/engine.c:879-889): every
 * stage is the 63-tap half-band (src/fir.c:65-95) with IPP FIRMR semantics
 * for a down factor of 2 and phase 0, y[m] = sum_k h[k] x[2m - k], its delay
 * line holding the previous inputs; a call consumes floor(count / 2) * 2
 * inputs per stage (the remainder is not seen by the stage, as the
 * reference's numIters = in_count / factor).
 */
#define ORA_DEC_TAPS 63

struct ora_decim {
    int stages;
    double h[ORA_DEC_TAPS];
    double dly[9][ORA_DEC_TAPS - 1];   /* previous inputs of each stage, oldest first */
};

ora_decim_t *ora_decim_new(unsigned fs_in, unsigned fs_out)
{
    if (fs_out == 0 || fs_in <= fs_out || fs_in % fs_out) return NULL;
    unsigned r = fs_in / fs_out;
    if (r & (r - 1)) return NULL;
    ora_decim_t *d = (ora_decim_t *)calloc(1, sizeof *d);
    if (!d) return NULL;
    while (r > 1) { d->stages++; r >>= 1; }
    if (d->stages > 9) { free(d); return NULL; }
    ora_fir_design(ORA_DEC_TAPS, 0, d->h);
    return d;
}

void ora_decim_free(ora_decim_t *d) { free(d); }

size_t ora_decim_process(ora_decim_t *d, const double *in, size_t n, double *out)
{
    double *a = (double *)malloc((n + 1) * sizeof(double));
    double *b = (double *)malloc((n / 2 + 1) * sizeof(double));
    if (!a || !b) { free(a); free(b); return 0; }
    memcpy(a, in, n * sizeof(double));
    size_t cur = n;
    const int L = ORA_DEC_TAPS;
    for (int s = 0; s < d->stages; s++) {
        size_t m = cur / 2;
        double *dl = d->dly[s];
        for (size_t o = 0; o < m; o++) {
            double acc = 0.0;
            for (int k = 0; k < L; k++) {
                long long j = 2 * (long long)o - k;
                double x = j >= 0 ? a[j] : dl[L - 1 + j];
                acc += d->h[k] * x;
            }
            b[o] = acc;
        }
        /* delay line <- the last L - 1 consumed inputs */
        size_t used = 2 * m;
        double tmp[ORA_DEC_TAPS - 1];
        for (int k = 0; k < L - 1; k++) {
            long long j = (long long)used - (L - 1) + k;
            tmp[k] = j >= 0 ? a[j] : dl[L - 1 + j];
        }
        memcpy(dl, tmp, sizeof tmp);
        double *t = a; a = b; b = t;
        cur = m;
    }
    memcpy(out, a, cur * sizeof(double));
    free(a);
    free(b);
    return cur;
}
