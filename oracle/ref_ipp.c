/*
 * ORACLE — test infrastructure only.  Stand-ins for the Intel IPP functions
 * that the reference's src/fir.c and src/engine.c call (declared in
 * oracle/ref_shim/ipps.h and ippcore.h), so those files compile and run here
 * with the rest of the reference's code.  IPP is closed and absent; these
 * follow its published semantics:
 *
 *   FIRMR  the input is zero-stuffed by upFactor (sample i at position
 *          upFactor * i + upPhase), filtered by the taps, and every
 *          downFactor-th filtered sample from downPhase is kept; one
 *          iteration consumes downFactor inputs and writes upFactor outputs
 *          (the reference uses phases 0, src/fir.c:195, 413)
 *   FIRSR  a direct-form FIR, one output per input
 *
 * Both carry the previous inputs in the caller's delay line (the reference
 * allocates tapsLen - 1 elements and passes it as source and destination,
 * src/fir.c:206-215, 322-340); here it holds the last tapsLen - 1 inputs,
 * oldest first, zero at start.  Output j sums h[k] * x[...] over the taps
 * k = 0 .. tapsLen-1 in ascending order, skipping the zero-stuffed terms, in
 * the precision of the function (Ipp32f or Ipp64f accumulators).  This is
 * the same arithmetic as oracle/fir_oracle.c's and oracle/dsd_oracle.c's
 * restatements; IPP's own summation order is closed.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "ref_shim/ippcore.h"

#define ORA_IPP_MAX_TAPS 1024

struct ora_ipp_fir_spec {
    int taps, up, down, single_rate, is64;
    double h[ORA_IPP_MAX_TAPS];
    float hf[ORA_IPP_MAX_TAPS];
};

static void *ipp_alloc(size_t bytes)
{
    void *p = NULL;
    if (posix_memalign(&p, 64, bytes ? bytes : 64) != 0) return NULL;
    return p;
}

Ipp8u *ippsMalloc_8u(int len) { return (Ipp8u *)ipp_alloc((size_t)len); }
Ipp32f *ippsMalloc_32f(int len) { return (Ipp32f *)ipp_alloc((size_t)len * sizeof(Ipp32f)); }
Ipp64f *ippsMalloc_64f(int len) { return (Ipp64f *)ipp_alloc((size_t)len * sizeof(Ipp64f)); }
void ippsFree(void *p) { free(p); }
IppStatus ippsZero_8u(Ipp8u *p, int len) { memset(p, 0, (size_t)len); return ippStsNoErr; }
IppStatus ippsZero_32f(Ipp32f *p, int len) { memset(p, 0, (size_t)len * 4); return ippStsNoErr; }
IppStatus ippsZero_64f(Ipp64f *p, int len) { memset(p, 0, (size_t)len * 8); return ippStsNoErr; }

IppStatus ippsConvert_64f32f(const Ipp64f *src, Ipp32f *dst, int len)
{
    for (int i = 0; i < len; i++) dst[i] = (Ipp32f)src[i];
    return ippStsNoErr;
}

IppStatus ippsConvert_32f64f(const Ipp32f *src, Ipp64f *dst, int len)
{
    for (int i = 0; i < len; i++) dst[i] = (Ipp64f)src[i];
    return ippStsNoErr;
}

IppStatus ippsFIRMRGetSize(int tapsLen, int upFactor, int downFactor, IppDataType tapsType,
                           int *pSpecSize, int *pBufSize)
{
    (void)tapsType;
    if (tapsLen < 1 || tapsLen > ORA_IPP_MAX_TAPS) return ippStsSizeErr;
    if (upFactor < 1 || downFactor < 1) return ippStsFIRMRFactorErr;
    *pSpecSize = (int)sizeof(struct ora_ipp_fir_spec);
    *pBufSize = 64;
    return ippStsNoErr;
}

IppStatus ippsFIRSRGetSize(int tapsLen, IppDataType tapsType, int *pSpecSize, int *pBufSize)
{
    return ippsFIRMRGetSize(tapsLen, 1, 1, tapsType, pSpecSize, pBufSize);
}

static IppStatus spec_init(struct ora_ipp_fir_spec *s, const double *hd, const float *hf,
                           int taps, int up, int up_phase, int down, int down_phase, int sr)
{
    if (!s || (!hd && !hf)) return ippStsNullPtrErr;
    if (taps < 1 || taps > ORA_IPP_MAX_TAPS) return ippStsSizeErr;
    if (up < 1 || down < 1 || up_phase != 0 || down_phase != 0) return ippStsFIRMRFactorErr;
    memset(s, 0, sizeof *s);
    s->taps = taps;
    s->up = up;
    s->down = down;
    s->single_rate = sr;
    s->is64 = hd != NULL;
    for (int k = 0; k < taps; k++) {
        s->h[k] = hd ? hd[k] : (double)hf[k];
        s->hf[k] = hf ? hf[k] : (float)hd[k];
    }
    return ippStsNoErr;
}

IppStatus ippsFIRMRInit_32f(const Ipp32f *pTaps, int tapsLen, int upFactor, int upPhase,
                            int downFactor, int downPhase, IppsFIRSpec_32f *pSpec)
{
    return spec_init(pSpec, NULL, pTaps, tapsLen, upFactor, upPhase, downFactor, downPhase, 0);
}

IppStatus ippsFIRMRInit_64f(const Ipp64f *pTaps, int tapsLen, int upFactor, int upPhase,
                            int downFactor, int downPhase, IppsFIRSpec_64f *pSpec)
{
    return spec_init(pSpec, pTaps, NULL, tapsLen, upFactor, upPhase, downFactor, downPhase, 0);
}

IppStatus ippsFIRSRInit_32f(const Ipp32f *pTaps, int tapsLen, IppAlgType algType,
                            IppsFIRSpec_32f *pSpec)
{
    (void)algType;
    return spec_init(pSpec, NULL, pTaps, tapsLen, 1, 0, 1, 0, 1);
}

IppStatus ippsFIRSRInit_64f(const Ipp64f *pTaps, int tapsLen, IppAlgType algType,
                            IppsFIRSpec_64f *pSpec)
{
    (void)algType;
    return spec_init(pSpec, pTaps, NULL, tapsLen, 1, 0, 1, 0, 1);
}

/* One multi-rate call in double or float arithmetic.  x(i) for i < 0 reads
 * the delay line (dly[L + i], L = taps - 1). */
#define FIRMR_BODY(T, H)                                                              \
    const int L = s->taps - 1, U = s->up, D = s->down;                               \
    const long long n_in = (long long)iters * D, n_out = (long long)iters * U;      \
    for (long long j = 0; j < n_out; j++) {                                          \
        T acc = (T)0;                                                                \
        const long long pos = j * D; /* position in the zero-stuffed stream */       \
        for (int k = 0; k < s->taps; k++) {                                          \
            long long q = pos - k;                                                   \
            if (((q % U) + U) % U != 0) continue;                                    \
            long long i = q >= 0 ? q / U : -((-q + U - 1) / U);                      \
            T x;                                                                     \
            if (i >= 0) x = src[i];                                                  \
            else if (-i <= L) x = dsrc[L + i];                                       \
            else x = (T)0;                                                           \
            acc += s->H[k] * x;                                                      \
        }                                                                            \
        dst[j] = acc;                                                                \
    }                                                                                \
    if (L > 0) {                                                                     \
        T *tmp = (T *)malloc((size_t)L * sizeof(T));                                 \
        for (int k = 0; k < L; k++) {                                                \
            long long i = n_in - L + k;                                              \
            tmp[k] = i >= 0 ? src[i] : dsrc[L + i];                                  \
        }                                                                            \
        memcpy(ddst, tmp, (size_t)L * sizeof(T));                                    \
        free(tmp);                                                                   \
    }                                                                                \
    return ippStsNoErr;

IppStatus ippsFIRMR_64f(const Ipp64f *src, Ipp64f *dst, int iters, IppsFIRSpec_64f *s,
                        const Ipp64f *dsrc, Ipp64f *ddst, Ipp8u *buf)
{
    (void)buf;
    if (!s || iters < 0) return ippStsNullPtrErr;
    FIRMR_BODY(double, h)
}

IppStatus ippsFIRMR_32f(const Ipp32f *src, Ipp32f *dst, int iters, IppsFIRSpec_32f *s,
                        const Ipp32f *dsrc, Ipp32f *ddst, Ipp8u *buf)
{
    (void)buf;
    if (!s || iters < 0) return ippStsNullPtrErr;
    FIRMR_BODY(float, hf)
}

IppStatus ippsFIRSR_64f(const Ipp64f *src, Ipp64f *dst, int n, IppsFIRSpec_64f *s,
                        const Ipp64f *dsrc, Ipp64f *ddst, Ipp8u *buf)
{
    return ippsFIRMR_64f(src, dst, n, s, dsrc, ddst, buf);
}

IppStatus ippsFIRSR_32f(const Ipp32f *src, Ipp32f *dst, int n, IppsFIRSpec_32f *s,
                        const Ipp32f *dsrc, Ipp32f *ddst, Ipp8u *buf)
{
    return ippsFIRMR_32f(src, dst, n, s, dsrc, ddst, buf);
}

static Ipp64u g_features = ippCPUID_SSE42 | ippCPUID_AVX | ippCPUID_AVX2;

IppStatus ippGetCpuFeatures(Ipp64u *pFeaturesMask, Ipp32u pCpuidInfoRegs[4])
{
    if (pFeaturesMask) *pFeaturesMask = g_features;
    if (pCpuidInfoRegs) memset(pCpuidInfoRegs, 0, 4 * sizeof(Ipp32u));
    return ippStsNoErr;
}

IppStatus ippSetCpuFeatures(Ipp64u features)
{
    g_features = features;
    return ippStsNoErr;
}

const IppLibraryVersion *ippGetLibVersion(void)
{
    static const IppLibraryVersion v = {0, 0, 0, 0, {0}, "ippstandin", "restatement", "-"};
    return &v;
}

IppStatus ippInit(void) { return ippStsNoErr; }
