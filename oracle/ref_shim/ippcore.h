/*
 * ORACLE — test infrastructure only.  The subset of Intel IPP's core API that
 * the reference's src/fir.c calls (CPU dispatch queries and the version
 * string), implemented in oracle/ref_ipp.c as inert stand-ins.
 */
#ifndef ORACLE_REF_IPPCORE_H
#define ORACLE_REF_IPPCORE_H

#include "ipps.h"

typedef struct {
    int major, minor, majorBuild, build;
    char targetCpu[4];
    const char *Name, *Version, *BuildDate;
} IppLibraryVersion;

#define ippCPUID_SSE42   0x00000100ull
#define ippCPUID_AVX     0x00000200ull
#define ippCPUID_AVX2    0x00008000ull
#define ippCPUID_AVX512F 0x00010000ull

IppStatus ippGetCpuFeatures(Ipp64u *pFeaturesMask, Ipp32u pCpuidInfoRegs[4]);
IppStatus ippSetCpuFeatures(Ipp64u features);
const IppLibraryVersion *ippGetLibVersion(void);
IppStatus ippInit(void);

/* MSVC's CPUID intrinsic, named by src/fir.c's dispatch override */
static inline void __cpuidex(int info[4], int leaf, int sub)
{
    (void)leaf;
    (void)sub;
    info[0] = info[1] = info[2] = info[3] = 0;
}

#endif
