// Constant-memory description of a fused upsampling FIR chain.
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

namespace dsdgpu {

constexpr int kMaxStages = 9;         // FIR_MAX_STAGES (reference include/fir.h:14)
constexpr int kMaxChainTaps = 2048;   // polyphase taps over all stages
constexpr int kMaxPhases = 16;        // polyphase branches of one stage (a merged stage: 8 or 16)
constexpr int kPolyTaps = 60;         // taps per branch of a merged stage (zero-padded)
constexpr int kPolyGroup = 4;         // branches per work item of a merged stage
constexpr int kPolyK = 64;            // taps per branch of a whole-chain stage (zero-padded)
constexpr int kPolyOut = 16384;       // outputs per CTA of a whole-chain stage
constexpr int kHistory = 256;         // PCM samples kept between blocks per channel
constexpr int kFirThreads = 256;
constexpr int kFirMaxSmem = 200 * 1024;   // dynamic shared memory cap of one FIR tile

// The engine's tanh soft clip above +-0.95 (src/engine.c:704-717), its
// constants formed as the reference forms them (1 - 0.95 and 1 / (1 - 0.95)
// in FP64, not the decimal literals 0.05 and 20).
__device__ __forceinline__ double soft_clip_095(double x) {
  const double thresh = 0.95;
  const double knee = 1.0 - thresh;
  const double inv_knee = 1.0 / knee;
  if (x > thresh) return __dadd_rn(thresh, __dmul_rn(knee, tanh(__dmul_rn(__dsub_rn(x, thresh), inv_knee))));
  if (x < -thresh)
    return __dsub_rn(-thresh, __dmul_rn(knee, tanh(__dmul_rn(__dsub_rn(-x, thresh), inv_knee))));
  return x;
}

struct FirChainConst {
  int S;                               // number of stages
  int ratio;                           // total upsampling factor
  int boxcar;                          // boxcar taps, 0 = off
  float inv_boxcar;
  int tile;                            // final output samples per CTA
  int U[kMaxStages];                   // stage factors (2 or 4; 8 or 16 for a merged stage)
  int L[kMaxStages];                   // stage tap counts (63 or 127; U * kPolyTaps merged)
  int nphase[kMaxStages][kMaxPhases];  // non-zero taps per polyphase branch
  int phase_off[kMaxStages][kMaxPhases];   // offset into taps[] / lag[]
  float taps[kMaxChainTaps];           // h'[U*j + r] = U * h[U*j + r]
  int lag[kMaxChainTaps];              // j
  // a merged stage: the leading 63-tap half-band stages of a long chain as
  // one polyphase stage of factor U = 2^M, branch r holding the kPolyTaps
  // taps hm[U*j + r] (lag j, zero-padded) of the stages' combined response
  int poly_stage[kMaxStages];
  // > 0: the whole chain (only 63-tap half-band 2x stages, factor 32 to 256)
  // as one polyphase stage of this factor, run by fir_poly_kernel
  int poly_U;
  // the 63-tap half-band 2x stage (every stage but a 127-tap first stage and
  // the 4x quarter-band one): its 32 even-phase taps and the centre tap, at
  // fixed offsets so that the unrolled kernel reads them as constant operands
  int hb_stage[kMaxStages];            // 1: stage k is a 63-tap half-band 2x stage
  float hb[32];                        // h'[2t], lag t
  float hb_center;                     // h'[31], lag 15
};

// Chain construction (fir_chain_init_ex's stage plan and tap design) and the
// launchers of the fused chain kernel and its history update.
int build_chain_const(unsigned fs_in, unsigned fs_out, int boxcar, FirChainConst* F);
void design_taps(int ntaps, bool quarter, double* h);      // Kaiser half/quarter-band design
double bessel_i0(double x);   // the reference's 25-term I0 series (src/fir.c:65-77)
int plan_chain(unsigned fs_in, unsigned fs_out, int* U, int* L);   // stage factors and lengths
size_t chain_smem_bytes(const FirChainConst& F);
int fir_chain_prepare();   // kernel attributes (call outside stream capture)
int launch_fir_chain(const FirChainConst& F, size_t smem, const float* pcm, size_t pcm_stride,
                     long long count, const float* hist, double* out, size_t out_stride,
                     double g_start, double g_step, int apply_gain, int soft_clip, int nch,
                     cudaStream_t stream);
// the same chain writing FP32 outputs (for a consumer that reads FP32)
int launch_fir_chain(const FirChainConst& F, size_t smem, const float* pcm, size_t pcm_stride,
                     long long count, const float* hist, float* out, size_t out_stride,
                     double g_start, double g_step, int apply_gain, int soft_clip, int nch,
                     cudaStream_t stream);
int launch_fir_history(const float* pcm, size_t pcm_stride, long long count, float* hist, int nch,
                       cudaStream_t stream);

}  // namespace dsdgpu
