/*
 * ORACLE — test infrastructure only (see oracle.h).
 *
 * FP64 restatement of the reference's upsampling FIR chain and the engine glue
 * around it.  The reference evaluates the chain with Intel IPP ippsFIRMR_64f
 * (src/fir.c:455-465), which is closed and absent; this file states the
 * published FIRMR semantics in direct form instead:
 *     zero-stuff by U with the input sample at phase 0, then
 *     y[m] = sum_k h'[k] * z[m - k],  h' = U * h,  delay line starting at zero
 * (src/fir.c:175-179, 386-390).  The summation runs k = 0..ntaps-1 over the
 * non-zero terms.  FIR parity is therefore unpinned at the IPP boundary and is
 * checked against the reference's own magnitude tests instead (passband flat,
 * images rejected, output counts; test/test_fir.c:204-257).
 *
 * Design (src/fir.c:65-150):
 *   half-band: Kaiser beta 12, sinc((n - c) / 2), normalised to unit sum
 *   quarter-band (the 4x stage): 0.25 * sinc(0.25 (n - c)), 127 taps
 *   taps per stage: 127 for a 4x stage and for stage 0 of a >= 2-stage chain
 *   into DSD512 (44.1k or 48k family); 63 otherwise.
 *   chain: power-of-two ratio, 2x stages, except ratio 8 into DSD512 = 4x + 2x
 *   (src/fir.c:523-611).
 * Glue (src/engine.c:629-651, 704-717): boxcar running mean over `taps` input
 * samples, linear gain ramp, tanh soft clip above +-0.95.
 */
#include "oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define KAISER_BETA 12.0
#define ORA_PI 3.14159265358979323846

static double bessel_i0(double x)
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

int ora_fir_design(int ntaps, int quarter, double *h)
{
    if (ntaps < 3 || (ntaps & 1) == 0) return -1;
    const int c = (ntaps - 1) / 2;
    const double i0b = bessel_i0(KAISER_BETA);
    double sum = 0.0;
    for (int n = 0; n < ntaps; n++) {
        double x = quarter ? (double)(n - c) * 0.25 : (double)(n - c) / 2.0;
        double sinc = (fabs(x) < 1e-15) ? 1.0 : sin(ORA_PI * x) / (ORA_PI * x);
        double t = (double)(n - c) / c;
        double arg = 1.0 - t * t;
        double w = bessel_i0(KAISER_BETA * sqrt(arg > 0.0 ? arg : 0.0)) / i0b;
        h[n] = quarter ? 0.25 * sinc * w : sinc * w;
        sum += h[n];
    }
    for (int n = 0; n < ntaps; n++) h[n] /= sum;
    return 0;
}

/* Stage factors and tap counts for fs_in -> fs_out (upsampling only).
 * Returns the number of stages (0 for equal rates), -1 if unsupported. */
int ora_fir_plan(unsigned fs_in, unsigned fs_out, int *factors, int *ntaps)
{
    if (fs_in == 0 || fs_out < fs_in) return -1;
    if (fs_in == fs_out) return 0;
    if (fs_out % fs_in) return -1;
    unsigned ratio = fs_out / fs_in;
    if (ratio & (ratio - 1)) return -1;
    int stages = 0;
    for (unsigned r = ratio; r > 1; r >>= 1) stages++;
    if (stages > 9) return -1;
    const int to512 = (fs_out == 22579200u || fs_out == 24576000u);
    if (ratio == 8 && to512) {
        factors[0] = 4; ntaps[0] = 127;
        factors[1] = 2; ntaps[1] = 63;
        return 2;
    }
    for (int i = 0; i < stages; i++) {
        factors[i] = 2;
        ntaps[i] = (stages >= 2 && i == 0 && to512) ? 127 : 63;
    }
    return stages;
}

/* One upsampling stage, fresh delay line.  Output m = U*i + r sums
 * h[k] * z[m - k] over k = r, r + U, ... (ascending), and z[m - k] is the
 * input sample in[i - j] for k = r + U*j; terms before the stream start
 * (j > i) are the zero delay line and are skipped. */
static void upsample_stage(const double *in, size_t n, int U, const double *h, int ntaps,
                           double *out)
{
    for (size_t i = 0; i < n; i++) {
        const size_t jmax = i;
        for (int r = 0; r < U; r++) {
            double acc = 0.0;
            size_t j = 0;
            for (int k = r; k < ntaps && j <= jmax; k += U, j++)
                acc += h[k] * in[i - j];
            out[i * (size_t)U + (size_t)r] = acc;
        }
    }
}

size_t ora_fir_upsample(unsigned fs_in, unsigned fs_out, const double *in, size_t n,
                        double *out)
{
    int fac[9], nt[9];
    int stages = ora_fir_plan(fs_in, fs_out, fac, nt);
    if (stages < 0) return 0;
    if (stages == 0) { memcpy(out, in, n * sizeof(double)); return n; }
    size_t total = n;
    for (int i = 0; i < stages; i++) total *= (size_t)fac[i];
    double *a = (double *)malloc(total * sizeof(double));
    double *b = (double *)malloc(total * sizeof(double));
    if (!a || !b) { free(a); free(b); return 0; }
    memcpy(a, in, n * sizeof(double));
    size_t cur = n;
    double h[255];
    for (int i = 0; i < stages; i++) {
        ora_fir_design(nt[i], fac[i] == 4, h);
        for (int k = 0; k < nt[i]; k++) h[k] *= (double)fac[i];
        upsample_stage(a, cur, fac[i], h, nt[i], b);
        cur *= (size_t)fac[i];
        double *t = a; a = b; b = t;
    }
    memcpy(out, a, cur * sizeof(double));
    free(a);
    free(b);
    return cur;
}

/* Running mean over `taps` samples with a zeroed history (src/engine.c:629-642). */
void ora_boxcar(const double *in, double *out, size_t n, int taps)
{
    if (taps <= 0) { if (out != in) memmove(out, in, n * sizeof(double)); return; }
    double *ring = (double *)calloc((size_t)taps, sizeof(double));
    double sum = 0.0;
    const double inv = 1.0 / (double)taps;
    int pos = 0;
    for (size_t i = 0; i < n; i++) {
        double s = in[i];
        sum -= ring[pos];
        ring[pos] = s;
        sum += s;
        pos = (pos + 1) % taps;
        out[i] = sum * inv;
    }
    free(ring);
}

/* buf[i] *= g_start + step * i (src/engine.c:646-651). */
void ora_gain_ramp(double *buf, size_t n, double g_start, double g_end)
{
    if (g_start == 1.0 && g_end == 1.0) return;
    double step = (n > 1) ? (g_end - g_start) / (double)(n - 1) : 0.0;
    for (size_t i = 0; i < n; i++) buf[i] *= g_start + step * (double)i;
}

/* tanh knee above |0.95| (src/engine.c:704-717). */
void ora_soft_clip(double *buf, size_t n)
{
    const double th = 0.95, inv_knee = 1.0 / (1.0 - th);
    for (size_t i = 0; i < n; i++) {
        double x = buf[i];
        if (x > th) buf[i] = th + (1.0 - th) * tanh((x - th) * inv_knee);
        else if (x < -th) buf[i] = -th - (1.0 - th) * tanh((-x - th) * inv_knee);
    }
}

/* Rate-conversion branch of engine_process_block, FP64 (src/engine.c:613-717):
 * widen, boxcar, FIR chain, gain ramp, optional soft clip. */
size_t ora_engine_fir(unsigned fs_in, unsigned fs_out, const float *in, size_t n,
                      int boxcar_taps, double g_start, double g_end, int soft_clip,
                      double *out)
{
    double *w = (double *)malloc((n ? n : 1) * sizeof(double));
    if (!w) return 0;
    for (size_t i = 0; i < n; i++) w[i] = (double)in[i];
    ora_boxcar(w, w, n, boxcar_taps);
    size_t m = ora_fir_upsample(fs_in, fs_out, w, n, out);
    free(w);
    if (g_start == 0.0) g_start = g_end;
    ora_gain_ramp(out, m, g_start, g_end);
    if (soft_clip) ora_soft_clip(out, m);
    return m;
}
