// Density-Aligned Stitching on sm_103a (reference src/dsp_plugin.c:1283-2762).
//
// One chunk per call.  The host plans the segment layout (and the RMS-driven
// reposition of quiet boundaries, whose window RMS values come from a kernel);
// the segments run as one persistent SDM launch; then
//
//   das_seam_kernel     one CTA per boundary: match density by block prefix
//                       sum, the reference's candidate scan and the run
//                       nearest the density peak (from match bitmasks, in
//                       parallel), and the 255-tap pop metric of every
//                       candidate (an FP32 pass over all offsets, then the
//                       reference's FP64 sum, in its tap order, for the
//                       offsets that can hold the maximum);
//   das_assemble_kernel gathers the final stream for every channel.
//
// The stitch search of a boundary only reads the last `overlap` decisions of
// the previous segment's copied region and the first `overlap` decisions of
// the new segment, and the write positions do not depend on the chosen seams
// (the stitch point moves only which side of the overlap a sample comes from),
// so every boundary is searched in parallel and the assembly is a gather.
#include "api_context.h"
#include "das_internal.h"
#include "das_plan.h"

#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace dsdgpu {

int launch_sdm_jobs(const SdmParams& P, const SdmJob* d_jobs, int njobs, int* d_counter,
                    SdmCtx* d_ctxs, int* d_status, int max_blocks, cudaStream_t stream);

constexpr int kMaxQ = 32;

// ---- window RMS (src/dsp_plugin.c:1975-1978): serial FP64 sum of squares ----
__global__ void das_rms_kernel(const double* __restrict__ x, const long long* __restrict__ centers,
                               int n, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long long win = kRmsWindow;
  const long long c = centers[i];
  double s = 0.0;
  for (long long k = c - win / 2; k < c + win / 2; k++) s = __dadd_rn(s, __dmul_rn(x[k], x[k]));
  out[i] = sqrt(__ddiv_rn(s, (double)win));
}

// ---- greedy multi-level state estimator (src/trellis.c:1125-1187) ----
// One sample of sdm_estimate_state_multibit: the NTF advance with y = 0, the
// quantiser (levels <= 2: the sign of v * a0; else v / a0 rounded to the
// nearest of `levels` values in [-1, 1]), y subtracted from state 0, clamp.
//
// The estimate is one serial chain per channel.  Every FP64 warp instruction
// holds its sub-partition's FP64 pipe for ~64 cycles however many lanes it
// runs, so the chain costs its count of FP64 instructions, and the step is
// written in warp form: lane i (< order) holds state[i], and the state update
// is four warp instructions
//     p  = g[i] * state[i+1]
//     r  = state[i] + (i == 0 ? -p : state[i-1])
//     ns = r + (i == 0 ? x : i == order-1 ? -0.0 : -p)
//     q  = a[i] * ns
// that are the reference's expressions operand for operand (a - b == a + (-b)
// and r + (-0.0) == r in IEEE arithmetic, signed zeros included); the sum
// v = x + q[0] + q[1] + ... keeps the reference's order on broadcast q.
//
// The quantiser's index idx = trunc((v / a0 + 1) / step + 0.5), clamped to
// [0, levels - 1], comes from u = fma(v, 1/(a0 step), 1/step) and integer
// work on u's bits.  While |u| < 1024, u is within 1e-12 of the reference's
// rounded (v / a0 + 1) / step (three roundings in the two constants and the
// fma against three in the reference's divisions and sum), so floor(u + 0.5)
// is the index unless u + 0.5 lies within 1e-9 of an integer; those samples,
// |u| >= 1024 and non-finite u take the reference's divisions.  The 1-bit
// sign test and the limiter compare bit patterns as integers.  A step is
// order + 6 FP64 instructions (order + 8 above 32 levels).
constexpr unsigned kFullMask = 0xffffffffu;
constexpr unsigned kNearHalf = 1100;   // 1e-9 in units of 2^-40, rounded up

struct EstConst {
  double c1;                 // (1 / a0) * (1 / step), rounded
  double rstep;              // 1 / step, rounded
  double step;               // 2 / (levels - 1)
  double lim;                // state_limit
  unsigned long long lim_bits;  // bits of state_limit when it is > 0, else 0 (limiter off)
  int levels;
};

// Per-lane constants of the warp form.
struct EstLane {
  double g, a;   // g[lane], a[lane]; 0 for lanes >= order
  double a0;
  double ylev;   // -1 + lane * step (the level table, one level per lane)
  int lane;
};

template <int N>
__device__ __forceinline__ EstLane est_lane(const SdmParams& P, const EstConst& E) {
  EstLane W;
  W.lane = threadIdx.x & 31;
  W.g = 0.0;
  W.a = 0.0;
#pragma unroll
  for (int i = 0; i < N; i++)
    if (W.lane == i) {
      W.g = P.g[i];
      W.a = P.a[i];
    }
  W.a0 = P.a[0];
  W.ylev = __dadd_rn(-1.0, __dmul_rn((double)W.lane, E.step));
  return W;
}

// The reference's quantiser expression, for the blocks the product form
// leaves undecided.
__device__ __forceinline__ int quant_exact(double v, double a0, double step, int levels) {
  const double yi = __ddiv_rn(v, a0);
  int idx = __double2int_rz(__dadd_rn(__ddiv_rn(__dadd_rn(yi, 1.0), step), 0.5));
  if (idx < 0) idx = 0;
  if (idx > levels - 1) idx = levels - 1;
  return idx;
}

// floor(u + 0.5) clamped to [0, levels - 1] from u's bits, without branches;
// `bad` is set where the reference's divisions must decide (|u| >= 1024, inf,
// NaN, or u + 0.5 within 1e-9 of an integer).
__device__ __forceinline__ int quant_fast(double u, int levels, bool& bad) {
  const unsigned hi = (unsigned)__double2hiint(u);
  const unsigned lo = (unsigned)__double2loint(u);
  const unsigned ex = (hi >> 20) & 0x7ffu;             // biased exponent
  const unsigned sh = 1035u - min(max(ex, 1021u), 1032u);  // 3..14: F = floor(u * 2^40) = fh:fl
  const unsigned mh = (hi & 0xfffffu) | 0x100000u;
  const unsigned fl = __funnelshift_r(lo, mh, sh);
  const unsigned fh = mh >> sh;
  const unsigned f8 = fh & 0xffu;                      // fraction bits 39..32
  const bool near = (f8 == 0x80u && fl <= kNearHalf) || (f8 == 0x7fu && fl >= 0u - kNearHalf);
  const bool low = (hi >> 31) != 0u || ex < 1021u;     // u < 0.25: w < 1 however it rounds
  bad |= ex >= 1033u || (!low && near);
  const int k = min((int)((fh + 0x80u) >> 8), levels - 1);  // (F + 2^39) >> 40
  return low ? 0 : k;
}

__device__ __forceinline__ double neg(double p) {
  return __longlong_as_double(__double_as_longlong(p) ^ (long long)0x8000000000000000ull);
}

// One estimator step in warp form; s is this lane's state.  Q: 0 = the 1-bit
// sign rule, 1 = 3..32 levels (the level comes from the lane holding it),
// 2 = more levels (y = -1 + idx * step as the reference forms it).  EXACT
// takes the reference's divisions for the index; otherwise the product form,
// which sets `bad` for a sample it cannot decide.
template <int N, int Q, bool LIM, bool EXACT>
__device__ __forceinline__ double est_step(double s, double x, const EstLane& W, const EstConst& E,
                                           bool& bad) {
  const double sn = __shfl_down_sync(kFullMask, s, 1);
  const double sp = __shfl_up_sync(kFullMask, s, 1);
  const double np = neg(__dmul_rn(W.g, sn));
  const double r = __dadd_rn(s, W.lane == 0 ? np : sp);
  double ns = __dadd_rn(r, W.lane == 0 ? x : (W.lane == N - 1 ? -0.0 : np));
  const double q = __dmul_rn(W.a, ns);
  double v = __dadd_rn(x, __shfl_sync(kFullMask, q, 0));
#pragma unroll
  for (int i = 1; i < N; i++) v = __dadd_rn(v, __shfl_sync(kFullMask, q, i));
  double y;
  if (Q == 0) {
    const long long b = __double_as_longlong(__dmul_rn(v, W.a0));
    y = (b > 0 && b <= 0x7ff0000000000000LL) ? 1.0 : -1.0;   // v * a0 > 0
  } else {
    const int idx = EXACT ? quant_exact(v, W.a0, E.step, E.levels)
                          : quant_fast(__fma_rn(v, E.c1, E.rstep), E.levels, bad);
    y = Q == 1 ? __shfl_sync(kFullMask, W.ylev, idx)
               : __dadd_rn(-1.0, __dmul_rn((double)idx, E.step));
  }
  ns = __dsub_rn(ns, W.lane == 0 ? y : 0.0);
  if (LIM) {   // ns > lim -> lim; ns < -lim -> -lim; NaN stays
    const long long b = __double_as_longlong(ns);
    const unsigned long long ab = (unsigned long long)b & 0x7fffffffffffffffull;
    if (ab > E.lim_bits && ab <= 0x7ff0000000000000ull) ns = b < 0 ? -E.lim : E.lim;
  }
  return W.lane < N ? ns : 0.0;
}

// n samples of x (any 8-byte alignment) through the estimator: 32 inputs per
// coalesced load, the next block's load in flight while this block runs.  A
// block with a sample the product form could not decide runs again from its
// starting state with the reference's divisions.
template <int N, int Q, bool LIM>
__device__ double est_walk(double s, const EstLane& W, const EstConst& E,
                           const double* __restrict__ x, long long n) {
  if (n <= 0) return s;
  double xl = W.lane < n ? __ldg(x + W.lane) : 0.0;
  for (long long b = 0; b < n; b += 32) {
    const long long nx = b + 32 + W.lane;
    const double xn = nx < n ? __ldg(x + nx) : 0.0;
    const int m = (int)min(32LL, n - b);
    const double s0 = s;
    bool bad = false;
    if (m == 32) {
#pragma unroll 4
      for (int j = 0; j < 32; j++)
        s = est_step<N, Q, LIM, false>(s, __shfl_sync(kFullMask, xl, j), W, E, bad);
    } else {
      for (int j = 0; j < m; j++)
        s = est_step<N, Q, LIM, false>(s, __shfl_sync(kFullMask, xl, j), W, E, bad);
    }
    if (Q != 0 && __any_sync(kFullMask, bad)) {
      s = s0;
      for (int j = 0; j < m; j++)
        s = est_step<N, Q, LIM, true>(s, __shfl_sync(kFullMask, xl, j), W, E, bad);
    }
    xl = xn;
  }
  return s;
}

EstConst make_est_const(const SdmParams& P, int levels) {
  EstConst E;
  memset(&E, 0, sizeof E);
  E.levels = levels;
  E.step = 2.0 / (double)(levels - 1);
  E.rstep = 1.0 / E.step;
  E.c1 = (1.0 / P.a[0]) * E.rstep;
  E.lim = P.state_limit;
  if (P.state_limit > 0.0) memcpy(&E.lim_bits, &P.state_limit, sizeof E.lim_bits);
  return E;
}

int est_kind(int levels) { return levels <= 2 ? 0 : levels <= 32 ? 1 : 2; }

// One warp per estimate (sdm_estimate_state(_multibit) on its own input).
constexpr int kEstWarps = 4;
template <int N, int Q, bool LIM>
__global__ void __launch_bounds__(32 * kEstWarps)
estimate_kernel(SdmParams P, EstConst E, const dsdgpu_estimate_t* __restrict__ items, int n,
                double* __restrict__ out /* [n][kMaxOrder] */) {
  const int j = blockIdx.x * kEstWarps + (int)(threadIdx.x >> 5);
  if (j >= n) return;
  const EstLane W = est_lane<N>(P, E);
  double s = W.lane < N ? items[j].init_state[W.lane] : 0.0;
  s = est_walk<N, Q, LIM>(s, W, E, items[j].d_in, items[j].count);
  if (W.lane < kMaxOrder) out[(size_t)j * kMaxOrder + W.lane] = W.lane < N ? s : 0.0;
}

// DAS seeding: one warp per channel walks the chunk from seg1's start with
// the 16-level estimator and records the state at every later segment start.
template <int N, bool LIM>
__global__ void __launch_bounds__(32)
das_estimate_kernel(SdmParams P, EstConst E, const double* __restrict__ fir, size_t fir_stride,
                    const SdmCtx* __restrict__ pers, int pers_first,
                    const long long* __restrict__ starts, int S, long long count,
                    double* __restrict__ est /* [nch][S][kMaxOrder] */, int nch) {
  const int ch = blockIdx.x;
  if (ch >= nch) return;
  const EstLane W = est_lane<N>(P, E);
  double s = W.lane < N ? pers[pers_first + ch].s[0][W.lane] : 0.0;
  const double* x = fir + (size_t)ch * fir_stride;
  const long long est_start = starts[1];
  long long pos = 0;
  for (int sg = 1; sg < S; sg++) {
    const long long bnd = sg >= 2 ? starts[sg] - est_start : 0;
    if (bnd > pos && bnd <= count - est_start) {
      s = est_walk<N, 1, LIM>(s, W, E, x + est_start + pos, bnd - pos);
      pos = bnd;
    }
    double* o = est + ((size_t)ch * S + sg) * kMaxOrder;
    if (W.lane < kMaxOrder) o[W.lane] = W.lane < N ? s : 0.0;
  }
}

template <int N, bool LIM>
void launch_estimate_n(const SdmParams& P, const EstConst& E, int kind,
                       const dsdgpu_estimate_t* d_items, int n, double* d_out, cudaStream_t stream) {
  const int blocks = (n + kEstWarps - 1) / kEstWarps;
  const int threads = 32 * kEstWarps;
  if (kind == 0) estimate_kernel<N, 0, LIM><<<blocks, threads, 0, stream>>>(P, E, d_items, n, d_out);
  else if (kind == 1) estimate_kernel<N, 1, LIM><<<blocks, threads, 0, stream>>>(P, E, d_items, n, d_out);
  else estimate_kernel<N, 2, LIM><<<blocks, threads, 0, stream>>>(P, E, d_items, n, d_out);
}

int launch_estimate(const SdmParams& P, int levels, const dsdgpu_estimate_t* d_items, int n,
                    double* d_out, cudaStream_t stream) {
  const EstConst E = make_est_const(P, levels);
  const int kind = est_kind(levels);
  switch (P.order) {
#define DSD_CASE(NN) \
  case NN:                                                                    \
    if (E.lim_bits) launch_estimate_n<NN, true>(P, E, kind, d_items, n, d_out, stream); \
    else launch_estimate_n<NN, false>(P, E, kind, d_items, n, d_out, stream);           \
    break;
    DSD_CASE(2) DSD_CASE(3) DSD_CASE(4) DSD_CASE(5) DSD_CASE(6)
    DSD_CASE(7) DSD_CASE(8) DSD_CASE(9) DSD_CASE(10)
#undef DSD_CASE
    default: return -1;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_das_estimate(const SdmParams& P, const double* fir, size_t fir_stride, const SdmCtx* pers,
                        int pers_first, const long long* starts, int S, long long count, double* est,
                        int nch, cudaStream_t stream) {
  const EstConst E = make_est_const(P, 16);
  switch (P.order) {
#define DSD_CASE(NN)                                                                 \
  case NN:                                                                           \
    if (E.lim_bits)                                                                  \
      das_estimate_kernel<NN, true><<<nch, 32, 0, stream>>>(P, E, fir, fir_stride, pers, \
                                                            pers_first, starts, S,   \
                                                            count, est, nch);        \
    else                                                                             \
      das_estimate_kernel<NN, false><<<nch, 32, 0, stream>>>(P, E, fir, fir_stride,  \
                                                             pers, pers_first, starts, \
                                                             S, count, est, nch);    \
    break;
    DSD_CASE(2) DSD_CASE(3) DSD_CASE(4) DSD_CASE(5) DSD_CASE(6)
    DSD_CASE(7) DSD_CASE(8) DSD_CASE(9) DSD_CASE(10)
#undef DSD_CASE
    default: return -1;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// Best-candidate state of the persistent contexts, replicated per segment
// (full-parallel seeding, src/dsp_plugin.c:2268-2283).
__global__ void das_seed_from_best_kernel(const SdmCtx* __restrict__ ctxs, int first, int S,
                                          double* __restrict__ est, int nch, int order) {
  const int ch = blockIdx.x;
  const SdmCtx* c = &ctxs[first + ch];
  for (int i = threadIdx.x; i < S * kMaxOrder; i += blockDim.x) {
    const int k = i % kMaxOrder;
    est[(size_t)ch * S * kMaxOrder + i] = k < order ? c->s[0][k] : 0.0;
  }
}

// ---- seam search, one CTA per boundary (src/dsp_plugin.c:2455-2652) ----
// kGlobal: overlaps above kMaxSeamOverlap (traceback latencies above 256) keep
// the match flags, the prefix sums, the density map and the search scratch in
// a global slice per boundary (das_seam_global_bytes) instead of shared memory.
//
// The reference's scans are restated in parallel, with the same results:
//  - candidate runs: a run start is the first position of a maximal run of
//    matches whose density reaches the floor (the serial scan stops there and
//    jumps to the run's end); the starts with runs of at least 4 are listed
//    in order from match / floor bitmasks, and the spacing rule is applied
//    greedily over that list;
//  - the run near the density peak: the first hit in the scan order
//    (r = 0, 1, ..., pp - r before pp + r) of a run of 8, else of 4, else the
//    LAST single match in that order (the serial loop keeps overwriting its
//    pick below 4), else the peak itself;
//  - pop metric: max over 639 offsets of |sum of +-q2[k]| in tap order.  Every
//    offset is first summed in FP32 together with a rigorous bound E on
//    |v32 - v64|: the running error of recursive summation (Higham, Accuracy
//    and Stability of Numerical Algorithms, 2nd ed., section 4.2:
//    |s^ - s| <= u/(1-u) sum_i |s^_i| over the computed partial sums, taken
//    twice here), plus u * sum|q2| for the taps rounded to FP32, plus 2^-40
//    for the FP64 sum's own rounding.  LB = max_j (|v32_j| - E_j) bounds the
//    FP64 maximum from below, so an offset with |v32_j| + E_j < LB cannot hold
//    it; the rest (about one per candidate) are summed in FP64 in the
//    reference's order.  Bounds are formed with directed rounding.  If more
//    than kPopList offsets qualify, every offset is summed in FP64.
constexpr int kPopJlo = -127, kPopJhi = 512, kPopJ = kPopJhi - kPopJlo;
constexpr int kPopR = 4;                                     // offsets per screening thread
constexpr int kPopBlocks = (kPopJ + kPopR - 1) / kPopR;
constexpr int kPopList = 512;
constexpr int kPopTaps = 256;                                // 255 taps and a zero

__host__ __device__ inline size_t seam_scratch_bytes(int L) {
  const size_t W = ((size_t)L + 31) / 32;
  const size_t runs = 4 * ((size_t)L / 5 + 8);
  const size_t pop = 4 * (size_t)(kMaxQ + 1) * kPopBlocks + 4 * (size_t)kPopList;
  return 8 * W + (runs > pop ? runs : pop);
}

// block-wide exclusive scans (blockDim a multiple of 32, at most 1024)
__device__ __forceinline__ int block_excl_sum(int v, int* red, int* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int n = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += n;
  }
  __syncthreads();
  if (lane == 31) red[w] = x;
  __syncthreads();
  if (w == 0) {
    int y = lane < nw ? red[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int n = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += n;
    }
    red[lane] = y;
  }
  __syncthreads();
  const int r = x - v + (w > 0 ? red[w - 1] : 0);
  if (total) *total = red[nw - 1];
  __syncthreads();
  return r;
}

__device__ __forceinline__ int block_excl_max(int v, int* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int n = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x = max(x, n);
  }
  int ex = __shfl_up_sync(0xffffffffu, x, 1);
  if (lane == 0) ex = -1;
  __syncthreads();
  if (lane == 31) red[w] = x;
  __syncthreads();
  if (w == 0) {
    int y = lane < nw ? red[lane] : -1;
    for (int o = 1; o < 32; o <<= 1) {
      const int n = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y = max(y, n);
    }
    red[lane] = y;
  }
  __syncthreads();
  const int r = max(ex, w > 0 ? red[w - 1] : -1);
  __syncthreads();
  return r;
}

// Run starts of one thread's words [w0, w1) in order: fn(p) for every p that
// opens the serial scan's run (see above) with p < L - 3 and a run of >= 4.
// czf / cnz: last match-at-floor / last mismatch position before word w0.
template <class Fn>
__device__ __forceinline__ void seam_runs(const unsigned* zb, const unsigned* fb, int W, int L,
                                          int w0, int w1, int czf, int cnz, Fn fn) {
  for (int w = w0; w < w1; w++) {
    const unsigned z = zb[w], zfw = z & fb[w], nz = ~z;   // bits at >= L: mismatches
    unsigned zf = zfw;
    while (zf) {
      const int b = __ffs(zf) - 1;
      zf &= zf - 1u;
      const int p = (w << 5) + b;
      if (p >= L - 3) return;
      const unsigned below = (1u << b) - 1u;
      const unsigned zfb = zfw & below, nzb = nz & below;
      const int pzf = zfb ? (w << 5) + 31 - __clz(zfb) : czf;
      const int pnz = nzb ? (w << 5) + 31 - __clz(nzb) : cnz;
      if (pzf >= 0 && pnz < pzf) continue;          // same run as an earlier start
      const unsigned above = nz & ~below;           // bit b is a match
      int e;
      if (above) {
        e = (w << 5) + __ffs(above) - 1;
      } else {
        int w2 = w + 1;
        while (w2 < W && zb[w2] == 0xffffffffu) w2++;
        e = w2 < W ? (w2 << 5) + __ffs(~zb[w2]) - 1 : L;
      }
      if (e > L) e = L;
      if (e - p >= 4) fn(p);
    }
    if (zfw) czf = (w << 5) + 31 - __clz(zfw);
    if (nz) cnz = (w << 5) + 31 - __clz(nz);
  }
}

// mr consecutive matches from tp (tp + mr <= L)
__device__ __forceinline__ bool seam_zrun(const unsigned* zb, int W, int L, int tp, int mr) {
  if (tp < 0 || tp + mr > L) return false;
  const int w = tp >> 5, b = tp & 31;
  unsigned long long v = zb[w];
  if (w + 1 < W) v |= (unsigned long long)zb[w + 1] << 32;
  const unsigned long long m = ((1ull << mr) - 1ull) << b;
  return (v & m) == m;
}

// FP32 pop values of offsets j0 .. j0 + kPopR - 1 of a candidate at sp:
// v[r] = sum_k e[sp + j0 + r - 127 + k] * q2f[k], e = +-1 / 0 inside [sp, L),
// and mu[r] = the sum of |partial sums| (the running error bound's sum).
__device__ __forceinline__ float seam_e(const __half* ef, int i, int sp, int L) {
  return (i >= sp && i < L) ? __half2float(ef[i]) : 0.0f;
}

__device__ __forceinline__ void seam_screen(const __half* ef, const float* q2f, int L, int sp,
                                            int j0, float (&v)[kPopR], float (&mu)[kPopR]) {
  const int base = sp + j0 - 127;
  float w[2 * kPopR - 1];
#pragma unroll
  for (int r = 0; r < kPopR; r++) {
    v[r] = 0.0f;
    mu[r] = 0.0f;
  }
#pragma unroll
  for (int m = 0; m < kPopR - 1; m++) w[m] = seam_e(ef, base + m, sp, L);
  for (int c = 0; c < kPopTaps / kPopR; c++) {
    const int cb = base + c * kPopR;
#pragma unroll
    for (int t = 0; t < kPopR; t++) w[kPopR - 1 + t] = seam_e(ef, cb + kPopR - 1 + t, sp, L);
#pragma unroll
    for (int kk = 0; kk < kPopR; kk++) {
      const float q = q2f[c * kPopR + kk];
#pragma unroll
      for (int r = 0; r < kPopR; r++) {
        v[r] = fmaf(w[kk + r], q, v[r]);
        mu[r] += fabsf(v[r]);
      }
    }
#pragma unroll
    for (int m = 0; m < kPopR - 1; m++) w[m] = w[m + kPopR];
  }
}

// Error bound of one screened offset (rounded up): 2u * mu + c0.
__device__ __forceinline__ float seam_err(float mu, float c0) {
  return __fadd_ru(__fmul_ru(mu, 0x1p-23f), c0);
}

template <bool kGlobal>
__global__ void __launch_bounds__(kSeamThreads, 3)
das_seam_kernel(const SeamTask* __restrict__ tasks, int ntasks, const double* __restrict__ qfir2,
                int* __restrict__ bp_out, unsigned char* __restrict__ gscr, size_t gstride) {
  const int ti = blockIdx.x;
  if (ti >= ntasks) return;
  const SeamTask T = tasks[ti];
  const int lat = T.lat;
  const int L = T.ovl_len;
  extern __shared__ unsigned char smraw[];
  unsigned char* base = kGlobal ? gscr + (size_t)ti * gstride : smraw;
  int8_t* dif = (int8_t*)base;                        // next - prev in {-1, 0, 1} (x2 later)
  int* dmap = (int*)(base + ((L + 15) & ~15));        // prefix sums, then the density map
  int* win = kGlobal ? dmap + ((L + 1 + 3) & ~3) : dmap;   // density map (global form)
  unsigned char* scr = (unsigned char*)(kGlobal ? win + L : dmap + (L + 1));
  const int W = (L + 31) >> 5;
  unsigned* zb = (unsigned*)scr;                      // bit p: prev[p] == next[p]
  unsigned* fb = zb + W;                              // bit p: density >= floor
  int* runs = (int*)(fb + W);                         // run starts (then the pop scratch)
  float* pop_blk = (float*)(fb + W);
  int* pop_list = (int*)(pop_blk + (kMaxQ + 1) * kPopBlocks);
  __shared__ int red[32];
  __shared__ int s_peak, s_pp, s_nq, s_best, s_nruns, s_first8, s_first4, s_last1, s_nlist,
      s_overflow;
  __shared__ int qpos[kMaxQ + 1], qden[kMaxQ + 1];
  __shared__ double qmax[kMaxQ + 1];
  __shared__ unsigned s_lb[kMaxQ + 1];
  __shared__ double s_q2[255];
  __shared__ float s_q2f[kPopTaps];
  __shared__ float s_abs;

  for (int k = threadIdx.x; k < 255; k += blockDim.x) s_q2[k] = qfir2[k];
  // match flags: prev = T.prev[0..L), next = T.next[0..L)
  for (int i = threadIdx.x; i < L; i += blockDim.x) {
    const int a = T.prev[i], b = T.next[i];
    dif[i] = (int8_t)(b - a);          // bits 0/1: diff of the +-1 samples is 2 * (b - a)
  }
  if (threadIdx.x == 0) {
    s_first8 = s_first4 = 0x7fffffff;
    s_last1 = -1;
    s_nlist = 0;
    s_overflow = 0;
  }
  __syncthreads();

  int half_w = lat;
  if (half_w > L / 2) half_w = L / 2;
  if (half_w < 4) half_w = 4;

  // prefix sum of matches -> dmap[p] = matches in [max(0, p - hw), min(L, p + hw))
  // (the reference's incremental window, src/dsp_plugin.c:2483-2501)
  // inclusive scan into dmap[1..L], dmap[0] = 0
  {
    const int per = (L + blockDim.x - 1) / blockDim.x;
    const int b0 = threadIdx.x * per, b1 = min(L, b0 + per);
    int loc = 0;
    for (int i = b0; i < b1; i++) loc += (dif[i] == 0);
    int run = block_excl_sum(loc, red, nullptr);
    if (threadIdx.x == 0) dmap[0] = 0;
    for (int i = b0; i < b1; i++) {
      run += (dif[i] == 0);
      dmap[i + 1] = run;
    }
  }
  __syncthreads();
  // convert the prefix into window counts: in place via registers (shared
  // form, at most 32 per thread), or into their own array (global form)
  int* pref = dmap;
  if constexpr (kGlobal) {
    for (int p = threadIdx.x; p < L; p += blockDim.x) {
      const int hi = min(L, p + half_w), lo = max(0, p - half_w);
      win[p] = pref[hi] - pref[lo];
    }
    __syncthreads();
    dmap = win;
  } else {
    int myv[32];
    int cnt = 0;
    for (int p = threadIdx.x; p < L && cnt < 32; p += blockDim.x, cnt++) {
      const int hi = min(L, p + half_w), lo = max(0, p - half_w);
      myv[cnt] = pref[hi] - pref[lo];
    }
    __syncthreads();
    cnt = 0;
    for (int p = threadIdx.x; p < L && cnt < 32; p += blockDim.x, cnt++) dmap[p] = myv[cnt];
  }
  __syncthreads();

  // peak and its first position
  {
    int best = -1, bi = 0x7fffffff;
    for (int p = threadIdx.x; p < L; p += blockDim.x) {
      const int v = dmap[p];
      if (v > best || (v == best && p < bi)) { best = v; bi = p; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const int ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    __shared__ int wb[32], wi[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { wb[w] = best; wi[w] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
      int B = -1, I = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); i++)
        if (wb[i] > B || (wb[i] == B && wi[i] < I)) { B = wb[i]; I = wi[i]; }
      s_peak = L > 0 ? (B > 0 ? B : 0) : 0;
      s_pp = L > 0 ? I : 0;
    }
    __syncthreads();
  }
  const int floor_d = s_peak * 9 / 10;
  const int pp = s_pp;

  // match and floor bitmasks, one word per warp step
  {
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int w = threadIdx.x >> 5; w < W; w += nw) {
      const int p = (w << 5) + lane;
      const bool z = p < L && dif[p] == 0;
      const bool f = p < L && dmap[p] >= floor_d;
      const unsigned zm = __ballot_sync(0xffffffffu, z);
      const unsigned fm = __ballot_sync(0xffffffffu, f);
      if (lane == 0) {
        zb[w] = zm;
        fb[w] = fm;
      }
    }
  }
  __syncthreads();

  // run starts in order, and the scan-order hits around the peak
  {
    const int per = (W + blockDim.x - 1) / blockDim.x;
    const int w0 = min(W, (int)threadIdx.x * per), w1 = min(W, w0 + per);
    int lzf = -1, lnz = -1;
    for (int w = w0; w < w1; w++) {
      const unsigned zf = zb[w] & fb[w], nz = ~zb[w];
      if (zf) lzf = (w << 5) + 31 - __clz(zf);
      if (nz) lnz = (w << 5) + 31 - __clz(nz);
    }
    const int czf = block_excl_max(lzf, red);
    const int cnz = block_excl_max(lnz, red);
    int cnt = 0;
    seam_runs(zb, fb, W, L, w0, w1, czf, cnz, [&](int) { cnt++; });
    int total;
    int off = block_excl_sum(cnt, red, &total);
    seam_runs(zb, fb, W, L, w0, w1, czf, cnz, [&](int p) { runs[off++] = p; });
    if (threadIdx.x == 0) s_nruns = total;
    for (int o = threadIdx.x; o < 2 * (half_w + 1); o += blockDim.x) {
      const int r = o >> 1;
      const int tp = (o & 1) ? pp + r : pp - r;
      if (seam_zrun(zb, W, L, tp, 8)) atomicMin(&s_first8, o);
      if (seam_zrun(zb, W, L, tp, 4)) atomicMin(&s_first4, o);
      if (seam_zrun(zb, W, L, tp, 1)) atomicMax(&s_last1, o);
    }
  }
  __syncthreads();

  // candidates: spacing rule over the run starts, then the peak-run pick
  if (threadIdx.x == 0) {
    const int min_spacing = half_w;
    const int nr = s_nruns;
    int nq = 0, i = 0;
    while (i < nr && nq < kMaxQ) {
      const int rs = runs[i];
      if (nq > 0 && rs - qpos[nq - 1] < min_spacing) {
        const int target = qpos[nq - 1] + min_spacing;
        int lo = i + 1, hi = nr;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (runs[mid] < target) lo = mid + 1;
          else hi = mid;
        }
        i = lo;
        continue;
      }
      qpos[nq] = rs;
      qden[nq] = dmap[rs];
      nq++;
      i++;
    }
    int prp = pp;
    const int o = s_first8 != 0x7fffffff ? s_first8 : (s_first4 != 0x7fffffff ? s_first4 : s_last1);
    if (o >= 0) prp = (o & 1) ? pp + (o >> 1) : pp - (o >> 1);
    int dup = 0;
    for (int ci = 0; ci < nq; ci++)
      if (abs(qpos[ci] - prp) < min_spacing) { dup = 1; break; }
    if (!dup && nq < kMaxQ) {
      qpos[nq] = prp;
      qden[nq] = L > 0 ? dmap[prp] : 0;
      nq++;
    }
    if (nq == 0) { qpos[0] = 0; qden[0] = 0; nq = 1; }
    for (int ci = 0; ci < nq; ci++) {
      qmax[ci] = 0.0;
      s_lb[ci] = 0u;
    }
    s_nq = nq;
  }
  __syncthreads();
  const int nq = s_nq;

  // pop metric: |255-tap FIR of the stitched-minus-unstitched difference| over
  // j in [-127, 512) (offsets below -127 see no term: value 0); terms with
  // idx < sp (before the stitch) or with equal bits are zero and are skipped
  // (adding +-0 leaves the magnitude unchanged)
  if (nq > 1) {
    __half* ef = reinterpret_cast<__half*>(dmap);   // the density map is no longer read
    for (int i = threadIdx.x; i < L; i += blockDim.x) ef[i] = __int2half_rn((int)dif[i]);
    for (int k = threadIdx.x; k < kPopTaps; k += blockDim.x)
      s_q2f[k] = k < 255 ? __double2float_rn(s_q2[k]) : 0.0f;
    __syncthreads();
    if (threadIdx.x < 32) {
      float a = 0.0f;
      for (int k = threadIdx.x; k < kPopTaps; k += 32) a += fabsf(s_q2f[k]);
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if (threadIdx.x == 0) s_abs = a;
    }
    __syncthreads();
    // u * sum|q2| (the taps' rounding to FP32, with margin) + 2^-40, rounded up
    const float c0 = __fmaf_ru(s_abs, 0x1.04p-24f, 0x1p-40f);
    const int items = nq * kPopBlocks;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
      const int ci = it / kPopBlocks;
      const int j0 = kPopJlo + (it - ci * kPopBlocks) * kPopR;
      float v[kPopR], mu[kPopR];
      seam_screen(ef, s_q2f, L, qpos[ci], j0, v, mu);
      float hi = 0.0f, lo = 0.0f;
#pragma unroll
      for (int r = 0; r < kPopR; r++) {
        if (j0 + r >= kPopJhi) continue;
        const float e = seam_err(mu[r], c0);
        hi = fmaxf(hi, __fadd_ru(fabsf(v[r]), e));
        lo = fmaxf(lo, __fsub_rd(fabsf(v[r]), e));
      }
      pop_blk[it] = hi;
      atomicMax(&s_lb[ci], __float_as_uint(lo));   // lo >= 0: bit order is value order
    }
    __syncthreads();
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
      const int ci = it / kPopBlocks;
      const float lb = __uint_as_float(s_lb[ci]);
      if (pop_blk[it] < lb) continue;
      const int j0 = kPopJlo + (it - ci * kPopBlocks) * kPopR;
      float v[kPopR], mu[kPopR];
      seam_screen(ef, s_q2f, L, qpos[ci], j0, v, mu);
#pragma unroll
      for (int r = 0; r < kPopR; r++) {
        if (j0 + r >= kPopJhi || __fadd_ru(fabsf(v[r]), seam_err(mu[r], c0)) < lb) continue;
        const int slot = atomicAdd(&s_nlist, 1);
        if (slot < kPopList) pop_list[slot] = ci * kPopJ + (j0 + r - kPopJlo);
        else s_overflow = 1;
      }
    }
    __syncthreads();
    const bool all = s_overflow != 0;
    const int n = all ? nq * kPopJ : s_nlist;
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
      const int item = all ? e : pop_list[e];
      const int ci = item / kPopJ;
      const int j = kPopJlo + (item - ci * kPopJ);
      const int sp = qpos[ci];
      double val = 0.0;
      int k0 = 127 - j;
      if (k0 < 0) k0 = 0;
      for (int k = k0; k < 255; k++) {
        const int idx = sp + j - 127 + k;
        if (idx >= L) break;
        const int d = dif[idx];
        if (d) val = __dadd_rn(val, d > 0 ? s_q2[k] : -s_q2[k]);
      }
      const double ad = fabs(val);
      // max over j: atomicMax on the bit pattern of a non-negative double
      atomicMax((unsigned long long*)&qmax[ci], (unsigned long long)__double_as_longlong(ad));
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double q[kMaxQ + 1];
    const int peak = s_peak;
    for (int ci = 0; ci < nq; ci++) {
      if (nq == 1) { q[ci] = 0.0; continue; }
      double dr = __ddiv_rn((double)qden[ci], (double)(peak > 0 ? peak : 1));
      if (dr < 0.5) dr = 0.5;
      q[ci] = __ddiv_rn(qmax[ci], dr);
    }
    int best = 0;
    for (int ci = 1; ci < nq; ci++) {
      const double ratio = __ddiv_rn(q[ci], __dadd_rn(q[best], 1e-15));
      if (ratio < 0.8) best = ci;
      else if (ratio < 1.2 && qden[ci] > qden[best]) best = ci;
    }
    s_best = qpos[best];
    bp_out[T.boundary] = s_best;
  }
}

// ---- assembly: gather every channel's stream (src/dsp_plugin.c:2420-2714) ----
__global__ void das_assemble_kernel(const AssemblePiece* __restrict__ pieces, int npieces,
                                    const int* __restrict__ bp, uint8_t* __restrict__ out,
                                    size_t out_stride, int nch, int S, const SegBuf* __restrict__ segbuf) {
  const int pi = blockIdx.y;
  if (pi >= npieces) return;
  const AssemblePiece P = pieces[pi];
  // this piece covers stream [begin, end) taken from segment P.seg, whose
  // decision i sits at stream position P.base + i
  const long long begin = P.base + (P.stitched ? bp[P.seg] : 0);
  long long end = P.end_base;
  if (P.next_stitched) end = P.next_base + bp[P.next_seg];
  for (int ch = 0; ch < nch; ch++) {
    const uint8_t* src = segbuf[ch * S + P.seg].ptr;
    uint8_t* dst = out + (size_t)ch * out_stride;
    for (long long p = begin + blockIdx.x * (long long)blockDim.x + threadIdx.x; p < end;
         p += (long long)gridDim.x * blockDim.x)
      dst[p] = src[p - P.base];
  }
}

// The pop-metric low-pass, host side (src/dsp_plugin.c:2568-2600), times two:
// the difference of two +-1 samples is +-2, and doubling is exact.
void pop_fir_times_two(double* q2) {
  const int N = 255;
  const double fc = 20000.0 / (5644800.0 / 2.0);
  double q[255];
  double sum = 0;
  for (int i = 0; i < N; i++) {
    const double n = i - 127.0;
    if (n > -0.001 && n < 0.001) q[i] = 2.0 * fc;
    else q[i] = std::sin(2.0 * 3.14159265358979 * fc * n) / (3.14159265358979 * n);
    const double x = 2.0 * i / (N - 1) - 1.0;
    const double kb = 8.0;
    const double arg = kb * std::sqrt(1.0 - x * x > 0 ? 1.0 - x * x : 0);
    double i0a = 1.0, term = 1.0;
    for (int m = 1; m <= 20; m++) {
      term *= (arg / 2.0 / m) * (arg / 2.0 / m);
      i0a += term;
    }
    double i0k = 1.0;
    term = 1.0;
    for (int m = 1; m <= 20; m++) {
      term *= (kb / 2.0 / m) * (kb / 2.0 / m);
      i0k += term;
    }
    q[i] *= i0a / i0k;
    sum += q[i];
  }
  for (int i = 0; i < N; i++) q2[i] = 2.0 * (q[i] / sum);
}

int launch_das_rms(const double* x, const long long* d_centers, int n, double* d_out,
                   cudaStream_t stream) {
  if (n <= 0) return 0;
  das_rms_kernel<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(x, d_centers, n, d_out);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

size_t das_seam_smem(int max_ovl) {
  return ((size_t)(max_ovl + 15) & ~(size_t)15) + sizeof(int) * (size_t)(max_ovl + 1) +
         seam_scratch_bytes(max_ovl) + 64;
}

size_t das_seam_global_bytes(int max_ovl) {
  if (max_ovl <= kMaxSeamOverlap) return 0;
  const size_t L = (size_t)max_ovl;
  return (((L + 15) & ~(size_t)15) + sizeof(int) * (((L + 1 + 3) & ~(size_t)3) + L) +
          seam_scratch_bytes(max_ovl) + 255) & ~(size_t)255;
}

int das_seam_prepare(int max_ovl) {
  if (max_ovl > kMaxSeamOverlap) return 0;
  const size_t smem = das_seam_smem(max_ovl);
  // the largest carveout: three CTAs per SM hold ~70 KB each at overlap 8,192
  if (cudaFuncSetAttribute(das_seam_kernel<false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                           100) != cudaSuccess)
    return -1;
  if (smem <= 48 * 1024) return 0;
  return cudaFuncSetAttribute(das_seam_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem) == cudaSuccess ? 0 : -1;
}

int launch_das_seams(const SeamTask* d_tasks, int ntasks, int max_ovl, const double* d_qfir2,
                     int* d_bp, unsigned char* d_gscratch, cudaStream_t stream) {
  if (ntasks <= 0) return 0;
  if (max_ovl > kMaxSeamOverlap) {
    if (!d_gscratch) return -2;
    das_seam_kernel<true><<<(unsigned)ntasks, kSeamThreads, 0, stream>>>(
        d_tasks, ntasks, d_qfir2, d_bp, d_gscratch, das_seam_global_bytes(max_ovl));
  } else {
    const size_t smem = das_seam_smem(max_ovl);
    das_seam_kernel<false><<<(unsigned)ntasks, kSeamThreads, smem, stream>>>(d_tasks, ntasks,
                                                                             d_qfir2, d_bp, nullptr, 0);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_das_assemble(const AssemblePiece* d_pieces, int npieces, const int* d_bp, uint8_t* out,
                        size_t out_stride, int nch, int S, const SegBuf* d_segbuf,
                        cudaStream_t stream) {
  if (npieces <= 0) return 0;
  const dim3 grid(64, (unsigned)npieces);
  das_assemble_kernel<<<grid, 256, 0, stream>>>(d_pieces, npieces, d_bp, out, out_stride, nch, S,
                                                d_segbuf);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace dsdgpu

using namespace dsdgpu;

namespace {

template <typename T>
int ensure_dev(dsdgpu_context* c, T** p, size_t* cap, size_t n, const char* what) {
  if (*cap >= n) return DSDGPU_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (n ? n : 1));
  if (e != cudaSuccess) return c->cuda_fail(e, what);
  *cap = n;
  return DSDGPU_OK;
}

// The side stream and events of the seg0-first estimator, made on first use.
int ensure_das_side(dsdgpu_context* c) {
  if (c->das_side) return DSDGPU_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&c->das_side, cudaStreamNonBlocking);
  for (int i = 0; i < 2 && e == cudaSuccess; i++)
    e = cudaEventCreateWithFlags(&c->das_side_ev[i], cudaEventDisableTiming);
  if (e != cudaSuccess) return c->cuda_fail(e, "estimator stream");
  return DSDGPU_OK;
}

// Grow the SDM context bank to `need` contexts, keeping the existing ones.
int ensure_ctx_capacity(dsdgpu_context* c, int need) {
  if (c->nctx >= need) return DSDGPU_OK;
  SdmCtx* nd = nullptr;
  cudaError_t e = cudaMalloc(&nd, sizeof(SdmCtx) * (size_t)need);
  if (e != cudaSuccess) return c->cuda_fail(e, "context bank growth");
  if (c->nctx > 0) cudaMemcpyAsync(nd, c->d_ctx, sizeof(SdmCtx) * (size_t)c->nctx,
                                   cudaMemcpyDeviceToDevice, c->stream);
  cudaStreamSynchronize(c->stream);
  if (c->d_ctx) cudaFree(c->d_ctx);
  c->d_ctx = nd;
  c->pending.resize(need, 0);
  c->draining.resize(need, 0);
  c->nctx = need;
  return DSDGPU_OK;
}

}  // namespace

extern "C" {

int dsdgpu_sdm_estimate_state(dsdgpu_context_t* c, const dsdgpu_sdm_params_t* p, int num_levels,
                              dsdgpu_estimate_t* items, int n) {
  if (!c || !p || n < 0 || (n > 0 && !items)) return DSDGPU_ERR_ARG;
  if (p->order < 2 || p->order > kMaxOrder) return c->fail(DSDGPU_ERR_ARG, "NTF order out of range (2..10)");
  if (num_levels < 2) return c->fail(DSDGPU_ERR_ARG, "num_levels below 2");
  if (n == 0) return DSDGPU_OK;
  for (int j = 0; j < n; j++)
    if (items[j].count < 0 || (items[j].count > 0 && !items[j].d_in))
      return c->fail(DSDGPU_ERR_ARG, "bad estimate input");
  cudaSetDevice(c->device);
  SdmParams P{};
  P.order = p->order;
  for (int k = 0; k < p->order; k++) {
    P.a[k] = p->a[k];
    P.g[k] = p->g[k];
  }
  P.state_limit = p->state_limit;
  const size_t ib = sizeof(dsdgpu_estimate_t) * (size_t)n;
  const size_t ob = sizeof(double) * kMaxOrder * (size_t)n;
  int rc = c->ensure_scratch(ib + ob + 256);
  if (rc) return rc;
  auto* d_items = (dsdgpu_estimate_t*)c->d_scratch;
  auto* d_out = (double*)((char*)c->d_scratch + ((ib + 255) & ~(size_t)255));
  cudaMemcpyAsync(d_items, items, ib, cudaMemcpyHostToDevice, c->stream);
  if (launch_estimate(P, num_levels, d_items, n, d_out, c->stream) != 0)
    return c->cuda_fail(cudaGetLastError(), "estimate launch");
  c->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "estimate launch");
  std::vector<double> out((size_t)n * kMaxOrder);
  e = cudaMemcpyAsync(out.data(), d_out, ob, cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "estimate read");
  rc = c->check_status();
  if (rc) return rc;
  for (int j = 0; j < n; j++)
    for (int k = 0; k < kMaxOrder; k++) items[j].out_state[k] = out[(size_t)j * kMaxOrder + k];
  return DSDGPU_OK;
}

int dsdgpu_das_process(dsdgpu_context_t* c, const dsdgpu_das_params_t* dp, int nch,
                       const double* d_fir, size_t fir_stride, size_t count, uint8_t* d_out,
                       size_t out_stride, size_t* out_count, int* h_stitch_pos, int max_segs) {
  if (!c || !dp || nch < 1) return DSDGPU_ERR_ARG;
  if (!c->sdm_ready) return c->fail(DSDGPU_ERR_STATE, "sdm not set up");
  if (nch > c->das_persistent) {
    if (c->das_persistent == 0 && c->nctx >= nch) c->das_persistent = nch;
    else return c->fail(DSDGPU_ERR_STATE, "persistent contexts: call dsdgpu_sdm_setup with num_contexts >= channels");
  }
  if (count > 0 && (!d_fir || !d_out)) return c->fail(DSDGPU_ERR_ARG, "null buffer");
  if (count == 0) {   // an empty chunk: no decisions, the contexts unchanged
    if (out_count) *out_count = 0;
    return DSDGPU_OK;
  }
  cudaSetDevice(c->device);
  const int lat = c->sdm.lat;
  const size_t overlap = 64 * (size_t)lat;

  // ---- layout (src/dsp_plugin.c:1343-1366, 1936-1957) ----
  std::vector<long long> start, size;
  const int S = das_nominal_layout(count, dp->seg_len, dp->nsegs, overlap, start, size);
  int rc;
  // ---- reposition of quiet boundaries (src/dsp_plugin.c:1959-2024) ----
  if (dp->reposition && S > 2) {
    RmsEval rms = [&](const std::vector<long long>& centers, std::vector<double>& out) -> int {
      int r = ensure_dev(c, &c->d_das_i64, &c->das_i64_cap, centers.size(), "rms centers");
      if (r) return r;
      r = ensure_dev(c, &c->d_das_f64, &c->das_f64_cap, centers.size(), "rms values");
      if (r) return r;
      cudaMemcpyAsync(c->d_das_i64, centers.data(), sizeof(long long) * centers.size(),
                      cudaMemcpyHostToDevice, c->stream);
      if (launch_das_rms(d_fir, c->d_das_i64, (int)centers.size(), c->d_das_f64, c->stream) != 0)
        return c->cuda_fail(cudaGetLastError(), "rms launch");
      c->launches++;
      out.resize(centers.size());
      cudaMemcpyAsync(out.data(), c->d_das_f64, sizeof(double) * out.size(), cudaMemcpyDeviceToHost,
                      c->stream);
      return c->check_status();
    };
    std::vector<long long> centers;
    std::vector<int> which;
    das_reposition_centers(start, count, centers, which);
    if (!centers.empty()) {
      std::vector<double> cur;
      rc = rms(centers, cur);
      if (rc) return rc;
      rc = das_reposition_apply(start, size, count, overlap, which, cur, rms);
      if (rc) return rc;
    }
  }

  const bool seg0_first = dp->seed_mode == DSDGPU_DAS_SEG0_FIRST;
  // context bank: [0, P) persistent, then per channel S temps, then P snapshots
  const int P = c->das_persistent;
  const int temp0 = P;
  const int snap0 = P + nch * S;
  rc = ensure_ctx_capacity(c, snap0 + nch);
  if (rc) return rc;

  // segment output buffers
  std::vector<long long> seg_in_start, seg_in_count, seg_discard;
  das_segment_io(start, size, count, overlap, lat, seg0_first, seg_in_start, seg_in_count,
                 seg_discard);
  size_t buf_total = 0;
  std::vector<size_t> seg_off(S);
  for (int s = 0; s < S; s++) {
    seg_off[s] = buf_total;
    buf_total += ((size_t)seg_in_count[s] + 255) & ~(size_t)255;
  }
  rc = ensure_dev(c, &c->d_das_bits, &c->das_bits_cap, buf_total * (size_t)nch + 256, "segment buffers");
  if (rc) return rc;
  rc = ensure_dev(c, &c->d_das_est, &c->das_est_cap, (size_t)nch * S * kMaxOrder, "seed states");
  if (rc) return rc;

  // ---- segment SDM runs ----
  std::vector<int64_t> seg_out((size_t)nch * S, 0);
  auto seg_ptr = [&](int ch, int s) { return c->d_das_bits + (size_t)ch * buf_total + seg_off[s]; };
  auto add_job = [&](std::vector<SdmJob>& jobs, int ch, int s, int ctx, int copy_from, bool seed,
                     int pend_from) {
    int64_t skip, out, np;
    sdm_plan_steps(lat, c->pending[pend_from], seg_in_count[s], seg_discard[s], &skip, &out, &np);
    c->pending[ctx] = np;
    c->draining[ctx] = c->draining[pend_from];
    seg_out[(size_t)ch * S + s] = out;
    if (seg_in_count[s] == 0) return;
    SdmJob j;
    j.in = d_fir + (size_t)ch * fir_stride + seg_in_start[s];
    j.out = seg_ptr(ch, s);
    j.n_in = seg_in_count[s];
    j.skip_out = skip;
    j.ctx = ctx;
    j.copy_from = copy_from;
    j.seed_state = seed ? c->d_das_est + ((size_t)ch * S + s) * kMaxOrder : nullptr;
    j.flags = 0;
    jobs.push_back(j);
  };
  int first_par = 0;
  if (seg0_first) {
    std::vector<SdmJob> j0;
    for (int ch = 0; ch < nch; ch++) add_job(j0, ch, 0, ch, -1, false, ch);
    rc = c->run_jobs(j0);
    if (rc) return rc;
    // seg1 and the estimator both start from seg0's final state and neither
    // writes what the other reads: the estimator walks on a side stream
    // while seg1's trellis runs, and the segment launch waits for it
    if (S > 2) {
      rc = ensure_das_side(c);
      if (rc) return rc;
      std::vector<long long> st(start.begin(), start.end());
      rc = ensure_dev(c, &c->d_das_i64, &c->das_i64_cap, (size_t)S, "starts");
      if (rc) return rc;
      cudaEventRecord(c->das_side_ev[0], c->stream);
      cudaStreamWaitEvent(c->das_side, c->das_side_ev[0], 0);
      cudaMemcpyAsync(c->d_das_i64, st.data(), sizeof(long long) * S, cudaMemcpyHostToDevice, c->das_side);
      if (launch_das_estimate(c->sdm, d_fir, fir_stride, c->d_ctx, 0, c->d_das_i64, S,
                              (long long)count, c->d_das_est, nch, c->das_side) != 0)
        return c->cuda_fail(cudaGetLastError(), "estimate launch");
      c->launches++;
      cudaEventRecord(c->das_side_ev[1], c->das_side);
    }
    if (S > 1) {
      std::vector<SdmJob> j1;
      for (int ch = 0; ch < nch; ch++) add_job(j1, ch, 1, temp0 + ch * S + 1, ch, false, ch);
      rc = c->run_jobs(j1);
      if (rc) {
        if (S > 2) cudaStreamSynchronize(c->das_side);
        return rc;
      }
    }
    if (S > 2) cudaStreamWaitEvent(c->stream, c->das_side_ev[1], 0);
    // seg2+ copy the persistent context after seg0: snapshot it so the
    // parallel launch reads a context nothing writes
    for (int ch = 0; ch < nch; ch++) {
      cudaMemcpyAsync(c->d_ctx + snap0 + ch, c->d_ctx + ch, sizeof(SdmCtx), cudaMemcpyDeviceToDevice, c->stream);
      c->pending[snap0 + ch] = c->pending[ch];
      c->draining[snap0 + ch] = c->draining[ch];
    }
    first_par = 2;
  } else {
    for (int ch = 0; ch < nch; ch++) {
      cudaMemcpyAsync(c->d_ctx + snap0 + ch, c->d_ctx + ch, sizeof(SdmCtx), cudaMemcpyDeviceToDevice, c->stream);
      c->pending[snap0 + ch] = c->pending[ch];
      c->draining[snap0 + ch] = c->draining[ch];
    }
    das_seed_from_best_kernel<<<nch, 128, 0, c->stream>>>(c->d_ctx, snap0, S, c->d_das_est, nch,
                                                         c->sdm.order); c->launches++;
  }
  {
    std::vector<SdmJob> jp;
    for (int ch = 0; ch < nch; ch++)
      for (int s = first_par; s < S; s++) {
        if (s == 0) add_job(jp, ch, 0, ch, -1, false, ch);
        else add_job(jp, ch, s, temp0 + ch * S + s, snap0 + ch, true, snap0 + ch);
      }
    if (c->timing_das) cudaEventRecord(c->ev[2], c->stream);
    rc = c->run_jobs(jp);
    if (c->timing_das) cudaEventRecord(c->ev[3], c->stream);
    if (rc) return rc;
  }

  // ---- stream plan: write positions do not depend on the seams ----
  std::vector<SeamPlan> splan;
  std::vector<AssemblePiece> pieces;
  long long final_count = 0;
  {
    const char* err = nullptr;
    if (das_stream_plan(S, seg_out.data(), size, overlap, seg0_first, splan, pieces, &final_count,
                        &err) != 0)
      return c->fail(DSDGPU_ERR_UNSUPPORTED, err);
  }
  std::vector<SeamTask> tasks;
  for (const SeamPlan& sp : splan) {
    SeamTask t;
    t.boundary = sp.boundary;
    t.ovl_len = sp.ovl_len;
    t.prev_seg = sp.prev_seg;
    t.prev_off = sp.prev_off;
    t.lat = lat;
    t.prev = nullptr;
    t.next = nullptr;
    tasks.push_back(t);
  }
  if (out_count) *out_count = (size_t)final_count;
  if (out_stride < (size_t)final_count) return c->fail(DSDGPU_ERR_ARG, "output stride too small");

  // ---- seams (channel 0) ----
  rc = ensure_dev(c, &c->d_das_bp, &c->das_bp_cap, (size_t)S, "seam positions");
  if (rc) return rc;
  cudaMemsetAsync(c->d_das_bp, 0, sizeof(int) * S, c->stream);
  if (!tasks.empty()) {
    for (auto& t : tasks) {
      t.prev = seg_ptr(0, t.prev_seg) + t.prev_off;
      t.next = seg_ptr(0, t.boundary);
    }
    rc = ensure_dev(c, &c->d_das_tasks, &c->das_tasks_cap, tasks.size(), "seam tasks");
    if (rc) return rc;
    if (!c->das_qfir_ready) {
      double q2[255];
      pop_fir_times_two(q2);
      rc = ensure_dev(c, &c->d_das_qfir, &c->das_qfir_cap, 255, "pop filter");
      if (rc) return rc;
      cudaMemcpyAsync(c->d_das_qfir, q2, sizeof q2, cudaMemcpyHostToDevice, c->stream);
      cudaStreamSynchronize(c->stream);
      c->das_qfir_ready = true;
    }
    cudaMemcpyAsync(c->d_das_tasks, tasks.data(), sizeof(SeamTask) * tasks.size(),
                    cudaMemcpyHostToDevice, c->stream);
    int maxL = 0;
    for (auto& t : tasks) maxL = std::max(maxL, t.ovl_len);
    unsigned char* gscr = nullptr;
    const size_t gb = das_seam_global_bytes(maxL);
    if (gb) {
      // overlaps above the shared-memory form: per-boundary scratch in HBM
      rc = ensure_dev(c, &c->d_das_seam_scr, &c->das_seam_scr_cap, gb * tasks.size(), "seam scratch");
      if (rc) return rc;
      gscr = c->d_das_seam_scr;
    }
    if (das_seam_prepare(maxL) != 0) return c->cuda_fail(cudaGetLastError(), "seam kernel attributes");
    rc = launch_das_seams(c->d_das_tasks, (int)tasks.size(), maxL, c->d_das_qfir, c->d_das_bp,
                          gscr, c->stream);
    if (rc == -2) return c->fail(DSDGPU_ERR_UNSUPPORTED, "overlap too long for the seam kernel");
    if (rc) return c->cuda_fail(cudaGetLastError(), "seam launch");
    c->launches++;
  }

  // ---- assembly ----
  std::vector<SegBuf> sb((size_t)nch * S);
  for (int ch = 0; ch < nch; ch++)
    for (int s = 0; s < S; s++) sb[(size_t)ch * S + s].ptr = seg_ptr(ch, s);
  rc = ensure_dev(c, &c->d_das_pieces, &c->das_pieces_cap, pieces.size(), "assembly plan");
  if (rc) return rc;
  rc = ensure_dev(c, &c->d_das_segbuf, &c->das_segbuf_cap, sb.size(), "segment table");
  if (rc) return rc;
  cudaMemcpyAsync(c->d_das_pieces, pieces.data(), sizeof(AssemblePiece) * pieces.size(),
                  cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(c->d_das_segbuf, sb.data(), sizeof(SegBuf) * sb.size(), cudaMemcpyHostToDevice,
                  c->stream);
  if (!pieces.empty()) {
    if (launch_das_assemble(c->d_das_pieces, (int)pieces.size(), c->d_das_bp, d_out, out_stride, nch,
                            S, c->d_das_segbuf, c->stream) != 0)
      return c->cuda_fail(cudaGetLastError(), "assembly launch");
    c->launches++;
  }

  // ---- state carry: persistent <- last temp (src/dsp_plugin.c:2715-2725) ----
  if (S > 1) {
    for (int ch = 0; ch < nch; ch++) {
      const int last = temp0 + ch * S + (S - 1);
      cudaMemcpyAsync(c->d_ctx + ch, c->d_ctx + last, sizeof(SdmCtx), cudaMemcpyDeviceToDevice, c->stream);
      c->pending[ch] = c->pending[last];
      c->draining[ch] = c->draining[last];
    }
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "das launch");
  rc = c->check_status();
  if (rc) return rc;
  if (h_stitch_pos) {
    std::vector<int> bp(S);
    cudaMemcpy(bp.data(), c->d_das_bp, sizeof(int) * S, cudaMemcpyDeviceToHost);
    for (int s = 0; s < S && s < max_segs; s++) h_stitch_pos[s] = bp[s];
  }
  c->das_last_segments = S;
  return DSDGPU_OK;
}

}  // extern "C"
