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

/*
 * The rate-conversion branch of engine_process_block for DSD input at a higher
 * rate than the output (src/engine.c:600-717 with fir_chain_init_ex's
 * downsampling chain): the +-1 input widened, the boxcar's running FP64 mean
 * (ring carried in bc), the FP64 decimation chain (delay lines carried in d),
 * the gain ramp when either end differs from 1 (a g_start of 0 means g_end),
 * and the tanh soft clip when asked (the engine skips it ahead of PreCorr).
 */
size_t ora_engine_down(ora_boxcar_t *bc, ora_decim_t *d, const float *in, size_t n,
                       double g_start, double g_end, int soft_clip, double *out)
{
    double *w = (double *)malloc((n + 1) * sizeof(double));
    if (!w) return 0;
    ora_boxcar_gain(bc, in, w, n, 1.0, 1.0);
    const size_t m = ora_decim_process(d, w, n, out);
    free(w);
    if (g_start == 0.0) g_start = g_end;
    ora_gain_ramp(out, m, g_start, g_end);
    if (soft_clip) ora_soft_clip(out, m);
    return m;
}

/*
 * Same-rate FIR lowpass (the engine's FIR_MODE_FIR alternative to the boxcar,
 * src/engine.c:168-181 and :505-523):
 *   - design of fir_lowpass_init_ex (src/fir.c:795-857): ntaps clamped to
 *     3..255 and made odd, fc = cutoff / (fs / 2) capped at 0.5, Kaiser
 *     (beta 10) windowed sinc, normalised to unit sum, FP64 throughout, in the
 *     reference's expression order; fir_lowpass_init uses 50 kHz, 127 taps;
 *   - filtering (fir_lowpass_process, src/fir.c:863-872, IPP ippsFIRSR_64f):
 *     y[i] = sum_k h[k] x[i - k] on +-1.0 inputs, delay line zero at init and
 *     carried across calls, then the gain ramp of src/engine.c:518-523.
 * IPP's summation order is closed; this restatement fixes one: the taps are
 * padded with zeros to W = 32 * ceil(ntaps / 32) and summed as W / 8 partial
 * sums, group j holding taps k = W-1-8j-v for v = 0..7 (oldest sample
 * first), each partial sum accumulated from 0.0 in v order and the partial
 * sums added in j order.  Samples before the first input are 0.
 */
#include <math.h>

#define ORA_LP_MAX_TAPS 255
#define ORA_LP_BETA 10.0
#define ORA_LP_PI 3.14159265358979323846

struct ora_lowpass {
    int ntaps;
    int W;
    double h[ORA_LP_MAX_TAPS + 1];
    double hist[256];        /* the last 256 inputs, oldest first (0 = not seen) */
};

static double lp_bessel_i0(double x)
{
    double sum = 1.0, term = 1.0;
    const double q = (x / 2.0) * (x / 2.0);
    for (int k = 1; k <= 25; k++) {
        term *= q / ((double)k * (double)k);
        sum += term;
        if (term < 1e-20 * sum) break;
    }
    return sum;
}

int ora_lowpass_design(unsigned fs, double cutoff_hz, int ntaps, double *h)
{
    if (ntaps < 3) ntaps = 3;
    if (ntaps > ORA_LP_MAX_TAPS) ntaps = ORA_LP_MAX_TAPS;
    if (ntaps % 2 == 0) ntaps++;
    double fc = cutoff_hz / ((double)fs / 2.0);
    if (fc > 0.5) fc = 0.5;
    const int M = ntaps - 1;
    const double i0b = lp_bessel_i0(ORA_LP_BETA);
    for (int n = 0; n <= M; n++) {
        const double x = (double)n - (double)M / 2.0;
        const double s = (fabs(x) < 1e-10) ? 2.0 * fc : sin(2.0 * ORA_LP_PI * fc * x) / (ORA_LP_PI * x);
        const double t = 2.0 * n / M - 1.0;
        const double arg = 1.0 - t * t;
        h[n] = s * (lp_bessel_i0(ORA_LP_BETA * sqrt(fabs(arg))) / i0b);
    }
    double sum = 0.0;
    for (int n = 0; n < ntaps; n++) sum += h[n];
    if (sum > 0.0)
        for (int n = 0; n < ntaps; n++) h[n] /= sum;
    return ntaps;
}

ora_lowpass_t *ora_lowpass_new(unsigned fs, double cutoff_hz, int ntaps)
{
    ora_lowpass_t *lp = (ora_lowpass_t *)calloc(1, sizeof *lp);
    if (!lp) return NULL;
    lp->ntaps = ora_lowpass_design(fs, cutoff_hz, ntaps, lp->h);
    lp->W = 32 * ((lp->ntaps + 31) / 32);
    return lp;
}

void ora_lowpass_free(ora_lowpass_t *lp) { free(lp); }

int ora_lowpass_taps(const ora_lowpass_t *lp, double *h)
{
    memcpy(h, lp->h, (size_t)lp->ntaps * sizeof(double));
    return lp->ntaps;
}

void ora_lowpass_process(ora_lowpass_t *lp, const float *in, double *out, size_t count,
                         double g_start, double g_end)
{
    double *x = (double *)malloc((count + 256) * sizeof(double));
    if (!x) return;
    memcpy(x, lp->hist, sizeof lp->hist);
    for (size_t i = 0; i < count; i++) x[256 + i] = in[i] >= 0.0f ? 1.0 : -1.0;
    if (g_start == 0.0) g_start = g_end;
    const double g_step = (count > 1) ? (g_end - g_start) / (double)(count - 1) : 0.0;
    const int W = lp->W;
    for (size_t i = 0; i < count; i++) {
        double acc = 0.0;
        for (int j = 0; j < W / 8; j++) {
            double grp = 0.0;
            for (int v = 0; v < 8; v++) {
                const int k = W - 1 - 8 * j - v;
                if (k < lp->ntaps) grp += x[256 + i - k] * lp->h[k];
            }
            acc += grp;
        }
        out[i] = acc * (g_start + g_step * (double)i);
    }
    memcpy(lp->hist, x + count, sizeof lp->hist);
    free(x);
}
