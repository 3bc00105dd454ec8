/* ORACLE — test infrastructure only (see oracle.h).  DAS restatement: filled in below. */
#include "oracle.h"
size_t ora_das_run(int order, const double *a, const double *g, int depth,
                   int cands, int lat, double state_limit,
                   const ora_das_cfg_t *cfg, const double *const *fir, size_t count,
                   int nch, uint8_t *const *out_bits, int *stitch_pos,
                   size_t *seg_starts, int nthreads)
{
    (void)order; (void)a; (void)g; (void)depth; (void)cands; (void)lat; (void)state_limit;
    (void)cfg; (void)fir; (void)count; (void)nch; (void)out_bits; (void)stitch_pos;
    (void)seg_starts; (void)nthreads;
    return 0;
}
