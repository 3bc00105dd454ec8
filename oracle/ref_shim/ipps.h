/*
 * ORACLE — test infrastructure only.  The subset of Intel IPP's signal
 * processing API that the reference's src/fir.c and src/engine.c call, with
 * IPP's published signatures.  IPP itself is closed and absent; the
 * functions are implemented in oracle/ref_ipp.c from the published
 * semantics (FIRMR: zero-stuff by upFactor at upPhase, filter, keep every
 * downFactor-th sample from downPhase; FIRSR: direct-form FIR; both with a
 * caller-held delay line of previous inputs), so the reference's own FIR
 * chain, lowpass and engine code can run here.  Their summation order is
 * this repository's choice, not IPP's.
 */
#ifndef ORACLE_REF_IPPS_H
#define ORACLE_REF_IPPS_H

#include <stdint.h>

typedef float Ipp32f;
typedef double Ipp64f;
typedef uint8_t Ipp8u;
typedef uint32_t Ipp32u;
typedef uint64_t Ipp64u;
typedef int IppStatus;
typedef struct { double re, im; } Ipp64fc;
typedef enum { ipp32f = 13, ipp64f = 19 } IppDataType;
typedef enum { ippAlgAuto = 0, ippAlgDirect = 1, ippAlgFFT = 2 } IppAlgType;
typedef enum { ippAlgHintNone = 0, ippAlgHintFast = 1, ippAlgHintAccurate = 2 } IppHintAlgorithm;
typedef struct ora_ipp_fir_spec IppsFIRSpec_32f;
typedef struct ora_ipp_fir_spec IppsFIRSpec_64f;
typedef struct ora_ipp_dft_spec IppsDFTSpec_C_64fc;

#define ippStsNoErr 0
#define ippStsSizeErr (-6)
#define ippStsNullPtrErr (-8)
#define ippStsFIRMRFactorErr (-28)

Ipp8u *ippsMalloc_8u(int len);
Ipp32f *ippsMalloc_32f(int len);
Ipp64f *ippsMalloc_64f(int len);
void ippsFree(void *p);
IppStatus ippsZero_8u(Ipp8u *p, int len);
IppStatus ippsZero_32f(Ipp32f *p, int len);
IppStatus ippsZero_64f(Ipp64f *p, int len);
IppStatus ippsConvert_64f32f(const Ipp64f *src, Ipp32f *dst, int len);
IppStatus ippsConvert_32f64f(const Ipp32f *src, Ipp64f *dst, int len);

IppStatus ippsFIRMRGetSize(int tapsLen, int upFactor, int downFactor, IppDataType tapsType,
                           int *pSpecSize, int *pBufSize);
IppStatus ippsFIRMRInit_32f(const Ipp32f *pTaps, int tapsLen, int upFactor, int upPhase,
                            int downFactor, int downPhase, IppsFIRSpec_32f *pSpec);
IppStatus ippsFIRMRInit_64f(const Ipp64f *pTaps, int tapsLen, int upFactor, int upPhase,
                            int downFactor, int downPhase, IppsFIRSpec_64f *pSpec);
IppStatus ippsFIRMR_32f(const Ipp32f *pSrc, Ipp32f *pDst, int numIters, IppsFIRSpec_32f *pSpec,
                        const Ipp32f *pDlySrc, Ipp32f *pDlyDst, Ipp8u *pBuf);
IppStatus ippsFIRMR_64f(const Ipp64f *pSrc, Ipp64f *pDst, int numIters, IppsFIRSpec_64f *pSpec,
                        const Ipp64f *pDlySrc, Ipp64f *pDlyDst, Ipp8u *pBuf);
IppStatus ippsFIRSRGetSize(int tapsLen, IppDataType tapsType, int *pSpecSize, int *pBufSize);
IppStatus ippsFIRSRInit_32f(const Ipp32f *pTaps, int tapsLen, IppAlgType algType,
                            IppsFIRSpec_32f *pSpec);
IppStatus ippsFIRSRInit_64f(const Ipp64f *pTaps, int tapsLen, IppAlgType algType,
                            IppsFIRSpec_64f *pSpec);
IppStatus ippsFIRSR_32f(const Ipp32f *pSrc, Ipp32f *pDst, int numIters, IppsFIRSpec_32f *pSpec,
                        const Ipp32f *pDlySrc, Ipp32f *pDlyDst, Ipp8u *pBuf);
IppStatus ippsFIRSR_64f(const Ipp64f *pSrc, Ipp64f *pDst, int numIters, IppsFIRSpec_64f *pSpec,
                        const Ipp64f *pDlySrc, Ipp64f *pDlyDst, Ipp8u *pBuf);

#endif
