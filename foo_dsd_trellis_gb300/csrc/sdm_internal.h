// Internal layouts shared by the trellis SDM kernels and the C-ABI host layer.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace dsdgpu {

constexpr int kMaxOrder = 10;    // MAX_NTF_ORDER (reference include/ntf.h:11)
constexpr int kMaxCands = 32;    // SDM_TRELLIS_MAX_NUM (include/trellis.h:12)
constexpr int kMaxLat = 2048;    // SDM_TRELLIS_MAX_LAT (include/trellis.h:13)
constexpr int kSlots = 2 * kMaxCands;
constexpr int kRingWords = kMaxLat / 32;
constexpr int kBuckets = 128;    // PATH_HASH_SIZE (include/trellis.h:14)

// The reference's state limiter (if v > lim: lim; else if v < -lim: -lim,
// src/trellis.c:180-186) for a positive finite lim, on the integer pipe:
// magnitudes of doubles order like their bit patterns; NaN (magnitude above
// +inf's) passes through as in C.  Shared by every trellis kernel.
__device__ __forceinline__ double clamp_state(double v, double lim) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned long long mag = b & 0x7FFFFFFFFFFFFFFFull;
  const unsigned long long lb = (unsigned long long)__double_as_longlong(lim);
  if (mag > lb && mag <= 0x7FF0000000000000ull)
    return __longlong_as_double((long long)((b & 0x8000000000000000ull) | lb));
  return v;
}

// Uniform trellis parameters (one NTF and one (K, depth, lat) per launch).
struct SdmParams {
  double a[kMaxOrder];
  double g[kMaxOrder];
  double state_limit;     // 0 = limiter off
  unsigned long long mask;  // (1 << depth) - 1, all ones for depth 64
  int order;
  int cands;              // K
  int lat;
  int depth;
  int mode;               // kModeFast, kModeExact or kModeVerify
  int lanes;              // lanes per job (2..32, a power of two >= K); 0 = automatic
  // bounds of the kernels' waits and walks; 0 = the built-in bound (shortened
  // only by the failure-path tests, DSDGPU_OPT_FAILURE_TEST)
  int hop_limit;                // path-hash chain walk, hops
  long long part_wait_cycles;   // balanced launch: wait for an unpublished part
};

// Survivor selection strategy of the SDM kernel.
enum : int {
  kModeFast = 0,     // parallel rank selection where it is provably equal, serial otherwise
  kModeExact = 1,    // always the serial (reference-order) selection
  kModeVerify = 2,   // serial selection, with the fast one computed and compared
};

// Device-resident SDM context: the state of one reference sdm_context_t that
// can influence future decisions.  Candidates are kept in rank (act) order.
// The slot memory (spath/skey/slink for both banks) is the part of the
// reference's sdm_state_t array that a path-hash chain walk can read: it is
// only consulted by the K = 32 bucket-0 case, but it has to be carried so
// that case stays exact.
struct alignas(16) SdmCtx {
  double s[kMaxCands][kMaxOrder];
  double cost[kMaxCands];
  unsigned long long path[kMaxCands];
  uint32_t ring[kMaxCands][kRingWords];   // traceback ring: bit p at word p>>5, bit p&31
  unsigned long long spath[2][kSlots];
  unsigned long long skey[2][kSlots];     // cost bit patterns
  int8_t slink[2][kSlots];                // hash-chain links, -1 = none
  uint8_t next[kMaxCands];
  uint8_t slot[kMaxCands];                // slot index of the candidate in bank `bank`
  int32_t n;                              // live candidates
  int32_t bank;                           // idx & 1
  int32_t pos;                            // ring write position
  int32_t pad;
  unsigned long long conv_fail, cands_collapse, next_filter_drops, total_children;
};

// One unit of work for the persistent SDM kernel: run `n_in` input samples
// through context `ctx`, dropping the decisions of the first `skip_out` steps
// and writing the rest as 0/1 bytes to `out`.  Optionally the context is
// first copied from `copy_from` (sdm_context_copy_state) and its live
// candidates seeded with `seed_state` and zero cost (DAS temp seeding).
struct SdmJob {
  const double* in;       // nullptr: zeros (drain)
  uint8_t* out;
  long long n_in;
  long long skip_out;
  int ctx;                // < 0: per-CTA scratch bank starting at -ctx - 1
  int copy_from;          // -1: none
  const double* seed_state;  // nullptr: none (kMaxOrder doubles)
  int flags;              // kJobNoStore: leave the context unwritten at the end
};

enum : int {
  kJobNoStore = 1,        // the run's final state is not needed (whole-stream batch runs)
};

// Device status word: 0 ok, else an error code from dsdgpu.h.
enum : int {
  kStatusOk = 0,
  kStatusChainLimit = 1,   // a path-hash chain walk exceeded its bound
  kStatusVerifyMismatch = 2,  // verify mode: the fast selection disagreed with the serial one
  kStatusQueueWait = 3,    // a balanced launch's wait for a queued job part gave up
};

}  // namespace dsdgpu
