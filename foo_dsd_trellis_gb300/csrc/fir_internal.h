// Constant-memory description of a fused upsampling FIR chain.
#pragma once

namespace dsdgpu {

constexpr int kMaxStages = 9;         // FIR_MAX_STAGES (reference include/fir.h:14)
constexpr int kMaxChainTaps = 1024;   // non-zero polyphase taps over all stages
constexpr int kHistory = 256;         // PCM samples kept between blocks per channel
constexpr int kFirThreads = 256;

struct FirChainConst {
  int S;                               // number of stages
  int ratio;                           // total upsampling factor
  int boxcar;                          // boxcar taps, 0 = off
  float inv_boxcar;
  int tile;                            // final output samples per CTA
  int U[kMaxStages];                   // stage factors (2 or 4)
  int L[kMaxStages];                   // stage tap counts (63 or 127)
  int nphase[kMaxStages][4];           // non-zero taps per polyphase branch
  int phase_off[kMaxStages][4];        // offset into taps[] / lag[]
  float taps[kMaxChainTaps];           // h'[U*j + r] = U * h[U*j + r]
  int lag[kMaxChainTaps];              // j
};

}  // namespace dsdgpu
