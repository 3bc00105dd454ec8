// Differentiable path (dsdgpu_diff_* of include/dsdgpu.h): straight-through
// adjoint of the FP64 FIR chain and the linear NTF loop filter.
//
// Forward (per clip c, n = frames * ratio samples):
//   p = w (*) x                  pre-emphasis FIR at the PCM rate (FP64)
//   u = gain * chain(p)          FP64 upsampling chain (fir_chain_process_d
//                                semantics, src/fir.c:455-465, no boxcar/clip)
//   y^ = trellis SDM(u)          exact decisions, one sequential run + drain
//   s_t = M s_{t-1} + e0 (u_t - y^_t),  v^_t = u_t + a . (M s_{t-1} + e0 u_t)
//                                the NTF loop (src/trellis.c:37-151) driven by
//                                the decisions, from zero state
//   L = mean_m z_m^2,  z = decimating low-pass of (y^ - r), r = gain * chain(x)
//
// Surrogate (decisions frozen): y_t = y^_t + kappa (v_t - v^_t) with the loop
// driven by y; it equals L at the forward's parameters, and backward returns
// its exact gradient.
//
// The base trajectory (the loop driven by the decisions, open loop M) runs
// serially per clip in the trellis's own operation order: M has eigenvalues
// slightly outside the unit circle, so only the exact operation sequence
// reproduces the bounded states the trellis kept; it leaves a checkpoint
// every `checkpoint` samples.  The closed loop A = (I - kappa e0 a^T) M of the
// surrogate (and, transposed, of the adjoint) is stable, so those recurrences
// run as blocked scans: one thread per (clip, checkpoint block) runs its
// block from a zero start, a per-clip carry pass chains the blocks with the
// block-length matrix power, and a final pass reruns every block from its
// true start.  The backward pass recomputes base states inside a block from
// the checkpoints, in the same operation order (two levels: the block's
// sub-starts every 64 samples, then one 64-sample run at a time, both in a
// per-thread scratch area of device memory).
#include "api_context.h"
#include "fir_internal.h"

#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

using namespace dsdgpu;

namespace {

constexpr int kMaxPreTaps = 255;
constexpr int kMaxLpfTaps = 511;
constexpr int kSubLen = 64;               // samples per sub-block of the recompute
constexpr int kMaxSubs = 256;             // sub-blocks per checkpoint block (<= 16384 samples)
constexpr int kScanThreads = 64;
constexpr double kStateBound = 1e12;      // far above the loop's natural state range (~1e6)

struct LoopCoef {
  double a[kMaxOrder];
  double g[kMaxOrder];
  double kappa;
};

struct Mat {
  double m[kMaxOrder][kMaxOrder];
};

struct LossShape {
  int T;            // low-pass taps
  int D;            // decimation
  long long M;      // decimated outputs per clip
  double scale;     // dL/dz_m = scale * z_m
};

struct StageDesc {
  int U;
  int nph[4];
  int off[4];
};

// ---- NTF loop (reference operation order, src/trellis.c:104-118) ----
template <int N>
__device__ __forceinline__ void loop_d(const LoopCoef& C, const double* s, double x, double* d) {
  d[0] = __dadd_rn(__dsub_rn(s[0], __dmul_rn(C.g[0], s[1])), x);
#pragma unroll
  for (int i = 1; i < N - 1; i++) d[i] = __dsub_rn(__dadd_rn(s[i], s[i - 1]), __dmul_rn(C.g[i], s[i + 1]));
  d[N - 1] = __dadd_rn(s[N - 1], s[N - 2]);
}

template <int N>
__device__ __forceinline__ double loop_v(const LoopCoef& C, double x, const double* d) {
  double v = __dadd_rn(x, __dmul_rn(C.a[0], d[0]));
#pragma unroll
  for (int i = 1; i < N; i++) v = __dadd_rn(v, __dmul_rn(C.a[i], d[i]));
  return v;
}

// mu_{t-1} = M^T dbar
template <int N>
__device__ __forceinline__ void loop_mt(const LoopCoef& C, const double* db, double* mu) {
#pragma unroll
  for (int j = 0; j < N; j++) {
    double m = db[j];
    if (j + 1 < N) m += db[j + 1];
    if (j >= 1) m -= C.g[j - 1] * db[j - 1];
    mu[j] = m;
  }
}

// dL/dy_t from the decimated low-pass: sum over m with 0 <= t - m D < T
__device__ __forceinline__ double lam_at(const double* __restrict__ z, const double* __restrict__ h,
                                         const LossShape& S, long long t) {
  long long mhi = t / S.D;
  if (mhi > S.M - 1) mhi = S.M - 1;
  const long long lo = t - (S.T - 1);
  const long long mlo = lo <= 0 ? 0 : (lo + S.D - 1) / S.D;
  double acc = 0.0;
  for (long long m = mlo; m <= mhi; m++) acc += z[m] * h[t - m * S.D];
  return acc * S.scale;
}

// ---- blocked scans --------------------------------------------------------

// per-clip forward carry: starts[b] = state entering block b
template <int N>
__global__ void fwd_carry_kernel(Mat Q, const double* __restrict__ ends, int nb, int nclips,
                                 double* __restrict__ starts) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nclips) return;
  double S[N], T[N];
#pragma unroll
  for (int k = 0; k < N; k++) S[k] = 0.0;
  for (int b = 0; b < nb; b++) {
    const size_t o = ((size_t)c * nb + b) * N;
#pragma unroll
    for (int k = 0; k < N; k++) starts[o + k] = S[k];
#pragma unroll
    for (int i = 0; i < N; i++) {
      double acc = ends[o + i];
#pragma unroll
      for (int j = 0; j < N; j++) acc += Q.m[i][j] * S[j];
      T[i] = acc;
    }
#pragma unroll
    for (int k = 0; k < N; k++) S[k] = T[k];
  }
}

// surrogate (closed loop), block-local from zero state: end states
template <int N>
__global__ void sur_local_kernel(LoopCoef C, const double* __restrict__ u,
                                 const double* __restrict__ beta, long long n, int Lb, int nb,
                                 int nclips, double* __restrict__ ends) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= nclips * nb) return;
  const int c = id / nb, b = id % nb;
  const size_t base = (size_t)c * n + (size_t)b * Lb;
  double s[N], d[N];
#pragma unroll
  for (int k = 0; k < N; k++) s[k] = 0.0;
  for (int t = 0; t < Lb; t++) {
    const double x = u[base + t];
    loop_d<N>(C, s, x, d);
    const double y = C.kappa * loop_v<N>(C, x, d) + beta[base + t];
#pragma unroll
    for (int k = 0; k < N; k++) s[k] = d[k];
    s[0] -= y;
  }
#pragma unroll
  for (int k = 0; k < N; k++) ends[(size_t)id * N + k] = s[k];
}

// surrogate from its block starts: the outputs y_t
template <int N>
__global__ void sur_full_kernel(LoopCoef C, const double* __restrict__ u,
                                const double* __restrict__ beta, long long n, int Lb, int nb,
                                int nclips, const double* __restrict__ starts,
                                double* __restrict__ yout) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= nclips * nb) return;
  const int c = id / nb, b = id % nb;
  const size_t base = (size_t)c * n + (size_t)b * Lb;
  double s[N], d[N];
#pragma unroll
  for (int k = 0; k < N; k++) s[k] = starts[(size_t)id * N + k];
  for (int t = 0; t < Lb; t++) {
    const double x = u[base + t];
    loop_d<N>(C, s, x, d);
    const double y = C.kappa * loop_v<N>(C, x, d) + beta[base + t];
    yout[base + t] = y;
#pragma unroll
    for (int k = 0; k < N; k++) s[k] = d[k];
    s[0] -= y;
  }
}

// adjoint, block-local from a zero incoming adjoint: mu entering the previous block
template <int N>
__global__ void adj_local_kernel(LoopCoef C, const double* __restrict__ z,
                                 const double* __restrict__ h, LossShape S, long long n, int Lb,
                                 int nb, int nclips, double* __restrict__ loc) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= nclips * nb) return;
  const int c = id / nb, b = id % nb;
  const double* zc = z + (size_t)c * S.M;
  double mu[N], db[N];
#pragma unroll
  for (int k = 0; k < N; k++) mu[k] = 0.0;
  for (int t = Lb - 1; t >= 0; t--) {
    const double lam = lam_at(zc, h, S, (long long)b * Lb + t);
    const double vb = C.kappa * (lam - mu[0]);
#pragma unroll
    for (int i = 0; i < N; i++) db[i] = mu[i] + vb * C.a[i];
    loop_mt<N>(C, db, mu);
  }
#pragma unroll
  for (int k = 0; k < N; k++) loc[(size_t)id * N + k] = mu[k];
}

// per-clip adjoint carry: cin[b] = true adjoint of the block's last state
template <int N>
__global__ void adj_carry_kernel(Mat P, const double* __restrict__ loc, int nb, int nclips,
                                 double* __restrict__ cin) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nclips) return;
  double Cb[N], T[N];
#pragma unroll
  for (int k = 0; k < N; k++) Cb[k] = 0.0;
  for (int b = nb - 1; b >= 0; b--) {
    const size_t o = ((size_t)c * nb + b) * N;
#pragma unroll
    for (int k = 0; k < N; k++) cin[o + k] = Cb[k];
    // adjoint entering block b - 1: local part of block b plus P applied to cin[b]
#pragma unroll
    for (int i = 0; i < N; i++) {
      double acc = loc[o + i];
#pragma unroll
      for (int j = 0; j < N; j++) acc += P.m[i][j] * Cb[j];
      T[i] = acc;
    }
#pragma unroll
    for (int k = 0; k < N; k++) Cb[k] = T[k];
  }
}

// the adjoint proper: states recomputed from the checkpoints, ubar and the
// NTF coefficient gradients (per-thread partial sums)
template <int N>
__global__ void __launch_bounds__(kScanThreads)
adj_full_kernel(LoopCoef C, const double* __restrict__ u, const uint8_t* __restrict__ bits,
                const double* __restrict__ z, const double* __restrict__ h, LossShape S,
                long long n, int Lb, int nb, int nclips, const double* __restrict__ starts,
                const double* __restrict__ cin, double* __restrict__ scr,
                double* __restrict__ ubar, double* __restrict__ gpart) {
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= nclips * nb) return;
  const int c = id / nb, b = id % nb;
  const size_t base = (size_t)c * n + (size_t)b * Lb;
  const double* zc = z + (size_t)c * S.M;
  const int nsub = Lb / kSubLen;
  // this thread's scratch: the state entering each sub-block, then the
  // states entering each sample of the sub-block being reversed
  double* sub = scr + (size_t)id * (nsub + kSubLen) * N;
  double* st = sub + (size_t)nsub * N;
  double s[N], d[N];
#pragma unroll
  for (int k = 0; k < N; k++) s[k] = starts[(size_t)id * N + k];
  for (int j = 0; j < nsub; j++) {
#pragma unroll
    for (int k = 0; k < N; k++) sub[j * N + k] = s[k];
    for (int q = 0; q < kSubLen; q++) {
      const size_t t = base + (size_t)j * kSubLen + q;
      loop_d<N>(C, s, u[t], d);
#pragma unroll
      for (int k = 0; k < N; k++) s[k] = d[k];
      s[0] = __dsub_rn(s[0], bits[t] ? 1.0 : -1.0);
    }
  }
  double mu[N], db[N], ga[N], gg[N];
#pragma unroll
  for (int k = 0; k < N; k++) {
    mu[k] = cin[(size_t)id * N + k];
    ga[k] = 0.0;
    gg[k] = 0.0;
  }
  for (int j = nsub - 1; j >= 0; j--) {
#pragma unroll
    for (int k = 0; k < N; k++) s[k] = sub[j * N + k];
    for (int q = 0; q < kSubLen; q++) {
      const size_t t = base + (size_t)j * kSubLen + q;
#pragma unroll
      for (int k = 0; k < N; k++) st[q * N + k] = s[k];
      loop_d<N>(C, s, u[t], d);
#pragma unroll
      for (int k = 0; k < N; k++) s[k] = d[k];
      s[0] = __dsub_rn(s[0], bits[t] ? 1.0 : -1.0);
    }
    for (int q = kSubLen - 1; q >= 0; q--) {
      const size_t t = base + (size_t)j * kSubLen + q;
      double sp[N];
#pragma unroll
      for (int k = 0; k < N; k++) sp[k] = st[q * N + k];
      loop_d<N>(C, sp, u[t], d);
      const double lam = lam_at(zc, h, S, (long long)(t - (size_t)c * n));
      const double vb = C.kappa * (lam - mu[0]);
#pragma unroll
      for (int i = 0; i < N; i++) db[i] = mu[i] + vb * C.a[i];
      ubar[t] = db[0] + vb;
#pragma unroll
      for (int i = 0; i < N; i++) ga[i] += vb * d[i];
#pragma unroll
      for (int i = 0; i < N - 1; i++) gg[i] -= db[i] * sp[i + 1];
      loop_mt<N>(C, db, mu);
    }
  }
#pragma unroll
  for (int k = 0; k < N; k++) {
    gpart[(size_t)id * 2 * N + k] = ga[k];
    gpart[(size_t)id * 2 * N + N + k] = gg[k];
  }
}

// ---- the adjoint scans with one state component per lane ----------------
//
// An FP64 instruction costs this part's FP64 unit about the same for one
// active lane as for 32, so the serial chain of a scan item is its count of
// FP64 instructions.  These forms give each (clip, block) item a group of G
// lanes, lane k owning component k of the state and of the adjoint: the
// per-component operations of loop_d, the adjoint products and loop_mt run
// once for all k (neighbours by shuffles), with the same operations per
// component as the one-thread forms above, so the results are the same.
template <int G>
struct Lane {
  int k;
  unsigned hm;
};

template <int N, int G>
__device__ __forceinline__ double loop_d_lane(const LoopCoef& C, const Lane<G>& L, double gk,
                                              double s, double x) {
  const double s_prev = __shfl_up_sync(L.hm, s, 1, G);
  const double s_next = __shfl_down_sync(L.hm, s, 1, G);
  const double m = __dmul_rn(gk, s_next);
  const double u = __dadd_rn(s, L.k == 0 ? -m : s_prev);
  return __dadd_rn(u, L.k == 0 ? x : (L.k < N - 1 ? -m : -0.0));
}

// mu_j = db_j + db_{j+1} - g_{j-1} db_{j-1} (loop_mt, one component per lane)
template <int N, int G>
__device__ __forceinline__ double loop_mt_lane(const Lane<G>& L, double gkm1, double db) {
  const double dn = __shfl_down_sync(L.hm, db, 1, G);
  const double dp = __shfl_up_sync(L.hm, db, 1, G);
  double m = db;
  if (L.k + 1 < N) m += dn;
  if (L.k >= 1) m -= gkm1 * dp;
  return m;
}

template <int G>
__device__ __forceinline__ bool lane_setup(Lane<G>& L, long long& item) {
  const int wl = threadIdx.x & 31;
  L.k = wl & (G - 1);
  L.hm = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (wl - L.k));
  item = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / G;
  return true;
}

template <int N, int G>
__global__ void adj_local_lane_kernel(LoopCoef C, const double* __restrict__ z,
                                      const double* __restrict__ h, LossShape S, long long n, int Lb,
                                      int nb, int nclips, double* __restrict__ loc) {
  Lane<G> L;
  long long item;
  lane_setup<G>(L, item);
  if (item >= (long long)nclips * nb) return;          // whole groups leave together
  const int c = (int)(item / nb), b = (int)(item % nb);
  const double* zc = z + (size_t)c * S.M;
  const int k = L.k;
  const double ak = k < N ? C.a[k] : 0.0;
  const double gkm1 = (k >= 1 && k <= N) ? C.g[k - 1] : 0.0;
  double mu = 0.0;
  for (int t = Lb - 1; t >= 0; t--) {
    const double lam = lam_at(zc, h, S, (long long)b * Lb + t);
    const double mu0 = __shfl_sync(L.hm, mu, 0, G);
    const double vb = C.kappa * (lam - mu0);
    const double db = mu + vb * ak;
    mu = loop_mt_lane<N, G>(L, gkm1, db);
  }
  if (k < N) loc[(size_t)item * N + k] = mu;
}

template <int N, int G>
__global__ void __launch_bounds__(kScanThreads)
adj_full_lane_kernel(LoopCoef C, const double* __restrict__ u, const uint8_t* __restrict__ bits,
                     const double* __restrict__ z, const double* __restrict__ h, LossShape S,
                     long long n, int Lb, int nb, int nclips, const double* __restrict__ starts,
                     const double* __restrict__ cin, double* __restrict__ scr,
                     double* __restrict__ ubar, double* __restrict__ gpart) {
  Lane<G> L;
  long long item;
  lane_setup<G>(L, item);
  if (item >= (long long)nclips * nb) return;
  const int c = (int)(item / nb), b = (int)(item % nb);
  const size_t base = (size_t)c * n + (size_t)b * Lb;
  const double* zc = z + (size_t)c * S.M;
  const int nsub = Lb / kSubLen;
  const int k = L.k;
  const bool own = k < N;
  const double gk = own ? C.g[k] : 0.0;
  const double ak = own ? C.a[k] : 0.0;
  const double gkm1 = (k >= 1 && k <= N) ? C.g[k - 1] : 0.0;
  // the item's scratch: the state entering each sub-block, then the states
  // entering each sample of the sub-block being reversed (component k at k)
  double* sub = scr + (size_t)item * (nsub + kSubLen) * N;
  double* st = sub + (size_t)nsub * N;
  double s = own ? starts[(size_t)item * N + k] : 0.0;
  for (int j = 0; j < nsub; j++) {
    if (own) sub[j * N + k] = s;
    for (int q = 0; q < kSubLen; q++) {
      const size_t t = base + (size_t)j * kSubLen + q;
      s = loop_d_lane<N, G>(C, L, gk, s, u[t]);
      if (k == 0) s = __dsub_rn(s, bits[t] ? 1.0 : -1.0);
    }
  }
  double mu = own ? cin[(size_t)item * N + k] : 0.0, ga = 0.0, gg = 0.0;
  for (int j = nsub - 1; j >= 0; j--) {
    s = own ? sub[j * N + k] : 0.0;
    for (int q = 0; q < kSubLen; q++) {
      const size_t t = base + (size_t)j * kSubLen + q;
      if (own) st[q * N + k] = s;
      s = loop_d_lane<N, G>(C, L, gk, s, u[t]);
      if (k == 0) s = __dsub_rn(s, bits[t] ? 1.0 : -1.0);
    }
    __syncwarp(L.hm);
    for (int q = kSubLen - 1; q >= 0; q--) {
      const size_t t = base + (size_t)j * kSubLen + q;
      const double sp = own ? st[q * N + k] : 0.0;
      const double d = loop_d_lane<N, G>(C, L, gk, sp, u[t]);
      const double lam = lam_at(zc, h, S, (long long)(t - (size_t)c * n));
      const double mu0 = __shfl_sync(L.hm, mu, 0, G);
      const double vb = C.kappa * (lam - mu0);
      const double db = mu + vb * ak;
      if (k == 0) ubar[t] = db + vb;
      ga += vb * d;
      const double sp1 = __shfl_down_sync(L.hm, sp, 1, G);
      if (k < N - 1) gg -= db * sp1;
      mu = loop_mt_lane<N, G>(L, gkm1, db);
    }
    __syncwarp(L.hm);
  }
  if (own) {
    gpart[(size_t)item * 2 * N + k] = ga;
    gpart[(size_t)item * 2 * N + N + k] = gg;
  }
}

// base trajectory, serial per clip in the reference's operation order: the
// loop without quantiser feedback is slightly unstable (the delayed
// resonators have |eigenvalue| > 1), so only the exact operation sequence of
// the trellis reproduces its bounded states; a reordered evaluation would
// amplify rounding.  Writes the checkpoints, beta_t = y^_t - kappa v^_t and
// the largest |state| seen (a sanity bound the host checks).
//
// The |state| maximum is taken on the integer pipe (magnitudes of doubles
// order like their bit patterns; a NaN state reads as above every bound).
//
// One clip per group of G lanes, one state component per lane (the same
// operations per component as the reference's loop; v's sum stays left to
// right on the gathered products).
template <int N, int G>
__global__ void base_lane_kernel(LoopCoef C, const double* __restrict__ u,
                                 const uint8_t* __restrict__ bits, long long n, int Lb, int nclips,
                                 double* __restrict__ starts, double* __restrict__ beta,
                                 double* __restrict__ smax) {
  Lane<G> L;
  long long item;
  lane_setup<G>(L, item);
  if (item >= nclips) return;
  const int c = (int)item, k = L.k;
  const bool own = k < N;
  const double gk = own ? C.g[k] : 0.0;
  const double ak = own ? C.a[k] : 0.0;
  const size_t base = (size_t)c * n;
  const int nb = (int)(n / Lb);
  const double* uc = u + base;
  const uint8_t* bc = bits + base;
  double s = 0.0;
  unsigned long long mx = 0;
  for (long long t = 0; t < n; t++) {
    if ((t & (Lb - 1)) == 0 && own) starts[((size_t)c * nb + (size_t)(t / Lb)) * N + k] = s;
    const double x = __ldg(uc + t);
    const double d = loop_d_lane<N, G>(C, L, gk, s, x);
    const double p = __dmul_rn(ak, d);
    double v = __dadd_rn(x, __shfl_sync(L.hm, p, 0, G));
#pragma unroll
    for (int j = 1; j < N; j++) v = __dadd_rn(v, __shfl_sync(L.hm, p, j, G));
    const double yt = __ldg(bc + t) ? 1.0 : -1.0;
    if (k == 0) beta[base + t] = yt - C.kappa * v;
    s = k == 0 ? __dsub_rn(d, yt) : d;
    if (own) {
      const unsigned long long m = (unsigned long long)__double_as_longlong(s) & 0x7FFFFFFFFFFFFFFFull;
      mx = m > mx ? m : mx;
    }
  }
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_down_sync(L.hm, mx, o, G);
    mx = other > mx ? other : mx;
  }
  if (k == 0) smax[c] = __longlong_as_double((long long)mx);
}

// ---- loss: decimating low-pass of (y - r), block partial sums of z^2 ----
template <bool kBits>
__global__ void loss_z_kernel(const uint8_t* __restrict__ bits, const double* __restrict__ yv,
                              const double* __restrict__ r, long long n,
                              const double* __restrict__ h, LossShape S, int nclips,
                              double* __restrict__ z, double* __restrict__ partial) {
  __shared__ double red[256];
  const long long total = (long long)nclips * S.M;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double sq = 0.0;
  if (i < total) {
    const long long c = i / S.M, m = i % S.M;
    const size_t o = (size_t)c * n + (size_t)m * S.D;
    double acc = 0.0;
    for (int k = 0; k < S.T; k++) {
      const double y = kBits ? (bits[o + k] ? 1.0 : -1.0) : yv[o + k];
      acc += h[k] * (y - r[o + k]);
    }
    z[i] = acc;
    sq = acc * acc;
  }
  red[threadIdx.x] = sq;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// ---- pre-emphasis FIR and its tap gradient ----
__global__ void preemph_kernel(const float* __restrict__ x, long long frames, int nclips,
                               const double* __restrict__ w, int T, double* __restrict__ p) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= frames * nclips) return;
  const long long c = i / frames, f = i % frames;
  const float* xc = x + c * frames;
  double acc = 0.0;
  const int kmax = (int)(f < T - 1 ? f : T - 1);
  for (int k = 0; k <= kmax; k++) acc = fma(w[k], (double)xc[f - k], acc);
  p[i] = acc;
}

__global__ void float_to_double_kernel(const float* __restrict__ x, long long n, double* __restrict__ y) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = (double)x[i];
}

// grad_w[k] = sum_c sum_f pbar[c][f] x[c][f - k]; one CTA per tap, fixed order
__global__ void taps_grad_kernel(const double* __restrict__ pbar, const float* __restrict__ x,
                                 long long frames, int nclips, int T, double* __restrict__ gw) {
  __shared__ double red[256];
  const int k = blockIdx.x;
  if (k >= T) return;
  double acc = 0.0;
  const long long total = frames * nclips;
  for (long long i = threadIdx.x; i < total; i += blockDim.x) {
    const long long f = i % frames;
    if (f >= k) acc = fma(pbar[i], (double)x[i - k], acc);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) gw[k] = red[0];
}

// ---- FP64 upsampling stage and its transpose ----
// out[U i + r] = sum_t taps[off_r + t] in[i - lag_t]  (zero history)
__global__ void chain64_stage_kernel(const double* __restrict__ in, long long n_in,
                                     double* __restrict__ out, StageDesc D,
                                     const double* __restrict__ taps, const int* __restrict__ lag,
                                     int nclips, double scale) {
  const long long n_out = n_in * D.U;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_out * nclips) return;
  const long long c = i / n_out, m = i % n_out;
  const long long j = m / D.U;
  const int r = (int)(m % D.U);
  const double* x = in + c * n_in;
  double acc = 0.0;
  for (int t = 0; t < D.nph[r]; t++) {
    const long long src = j - lag[D.off[r] + t];
    if (src >= 0) acc = fma(taps[D.off[r] + t], x[src], acc);
  }
  out[i] = acc * scale;
}

// inbar[j] = sum_r sum_t taps[off_r + t] outbar[U (j + lag_t) + r]
__global__ void chain64_stage_adj_kernel(const double* __restrict__ obar, long long n_in,
                                         double* __restrict__ ibar, StageDesc D,
                                         const double* __restrict__ taps,
                                         const int* __restrict__ lag, int nclips, double scale) {
  const long long n_out = n_in * D.U;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_in * nclips) return;
  const long long c = i / n_in, j = i % n_in;
  const double* y = obar + c * n_out;
  double acc = 0.0;
  for (int r = 0; r < D.U; r++)
    for (int t = 0; t < D.nph[r]; t++) {
      const long long m = (long long)D.U * (j + lag[D.off[r] + t]) + r;
      if (m < n_out) acc = fma(taps[D.off[r] + t], y[m], acc);
    }
  ibar[i] = acc * scale;
}

unsigned grid_of(long long n, int threads) { return (unsigned)((n + threads - 1) / threads); }

void mat_mul(const Mat& A, const Mat& B, Mat& C, int N) {
  Mat T;
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) {
      double s = 0.0;
      for (int k = 0; k < N; k++) s += A.m[i][k] * B.m[k][j];
      T.m[i][j] = s;
    }
  C = T;
}

Mat mat_pow(const Mat& A, long long e, int N) {
  Mat R;
  memset(&R, 0, sizeof R);
  for (int i = 0; i < N; i++) R.m[i][i] = 1.0;
  Mat B = A;
  while (e > 0) {
    if (e & 1) mat_mul(R, B, R, N);
    mat_mul(B, B, B, N);
    e >>= 1;
  }
  return R;
}

// M of the NTF loop: d = M s + e0 x
Mat loop_matrix(const double* g, int N) {
  Mat M;
  memset(&M, 0, sizeof M);
  M.m[0][0] = 1.0;
  M.m[0][1] = -g[0];
  for (int i = 1; i < N - 1; i++) {
    M.m[i][i - 1] = 1.0;
    M.m[i][i] = 1.0;
    M.m[i][i + 1] = -g[i];
  }
  M.m[N - 1][N - 2] = 1.0;
  M.m[N - 1][N - 1] = 1.0;
  return M;
}

// closed loop A = (I - kappa e0 a^T) M
Mat closed_loop(const Mat& M, const double* a, double kappa, int N) {
  Mat A = M;
  for (int j = 0; j < N; j++) {
    double s = 0.0;
    for (int i = 0; i < N; i++) s += a[i] * M.m[i][j];
    A.m[0][j] = M.m[0][j] - kappa * s;
  }
  return A;
}

Mat transpose(const Mat& A, int N) {
  Mat T;
  memset(&T, 0, sizeof T);
  for (int i = 0; i < N; i++)
    for (int j = 0; j < N; j++) T.m[i][j] = A.m[j][i];
  return T;
}

}  // namespace

struct dsdgpu_diff {
  dsdgpu_context* c = nullptr;
  dsdgpu_diff_params_t p{};
  int N = 0;
  long long n = 0;          // samples per clip at the SDM rate
  int nb = 0;               // checkpoint blocks per clip
  LossShape S{};
  // chain
  int stages = 0;
  StageDesc sd[kMaxStages]{};
  double* d_taps = nullptr;
  int* d_lag = nullptr;
  // buffers
  float* d_x = nullptr;         // [C][frames]
  double* d_xd = nullptr;       // x as doubles (reference chain input)
  double* d_w = nullptr;        // pre-emphasis taps
  double* d_p = nullptr;        // [C][frames]
  double* d_ping = nullptr;     // chain intermediates [C][n]
  double* d_pong = nullptr;
  double* d_u = nullptr;        // SDM input [C][n]
  double* d_r = nullptr;        // reference [C][n]
  uint8_t* d_bits = nullptr;    // [C][n]
  double* d_beta = nullptr;     // [C][n]
  double* d_y = nullptr;        // surrogate outputs / adjoint scratch [C][n]
  double* d_ubar = nullptr;     // [C][n]
  double* d_h = nullptr;        // loss low-pass
  double* d_z = nullptr;        // [C][M]
  double* d_part = nullptr;     // loss partial sums
  double* d_ends = nullptr;     // [C][nb][N]
  double* d_starts = nullptr;   // checkpoints [C][nb][N]
  double* d_sstarts = nullptr;  // surrogate block starts
  double* d_cin = nullptr;      // adjoint carries
  double* d_gpart = nullptr;    // [C][nb][2N]
  double* d_gw = nullptr;       // taps gradient
  double* d_scr = nullptr;      // per-thread recompute states of the adjoint
  double* d_smax = nullptr;     // largest |state| of each clip's base trajectory
  SdmCtx* d_ctx = nullptr;
  SdmJob* d_jobs = nullptr;
  int* d_counter = nullptr;
  unsigned nparts = 0;
  bool have_input = false, have_forward = false;
  LoopCoef coef{};              // parameters of the last forward
  std::vector<double> taps;     // ditto
  float ms[4] = {0, 0, 0, 0};
  cudaEvent_t ev[4] = {};
  std::vector<void*> allocs;

  template <typename T>
  int alloc(T** p, size_t count) {
    if (cudaMalloc((void**)p, sizeof(T) * (count ? count : 1)) != cudaSuccess) return -1;
    allocs.push_back((void*)*p);
    return 0;
  }
  ~dsdgpu_diff() {
    if (c) cudaSetDevice(c->device);
    for (void* q : allocs) cudaFree(q);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
  }
};

namespace {

template <int N>
int launch_scan(const char* which, dsdgpu_diff* D, const LoopCoef& C, const Mat& carry,
                const double* u, const double* beta) {
  const int tot = D->p.nclips * D->nb;
  const unsigned g = grid_of(tot, kScanThreads);
  const unsigned gc = grid_of(D->p.nclips, 32);
  cudaStream_t s = D->c->stream;
  const int Lb = D->p.checkpoint;
  if (!strcmp(which, "base")) {
    // one clip per warp, one state component per lane
    constexpr int GB = N <= 8 ? 8 : 16;
    base_lane_kernel<N, GB><<<D->p.nclips, GB, 0, s>>>(C, u, D->d_bits, D->n, Lb, D->p.nclips,
                                                       D->d_starts, D->d_beta, D->d_smax);
    D->c->launches -= 2;
  } else if (!strcmp(which, "sur")) {
    sur_local_kernel<N><<<g, kScanThreads, 0, s>>>(C, u, beta, D->n, Lb, D->nb, D->p.nclips, D->d_ends);
    fwd_carry_kernel<N><<<gc, 32, 0, s>>>(carry, D->d_ends, D->nb, D->p.nclips, D->d_sstarts);
    sur_full_kernel<N><<<g, kScanThreads, 0, s>>>(C, u, beta, D->n, Lb, D->nb, D->p.nclips,
                                                  D->d_sstarts, D->d_y);
  } else {
    // one state component per lane: G = 8 lanes per item up to order 8
    constexpr int G = N <= 8 ? 8 : 16;
    const unsigned gl = grid_of((long long)tot * G, kScanThreads);
    adj_local_lane_kernel<N, G><<<gl, kScanThreads, 0, s>>>(C, D->d_z, D->d_h, D->S, D->n, Lb,
                                                           D->nb, D->p.nclips, D->d_ends);
    adj_carry_kernel<N><<<gc, 32, 0, s>>>(carry, D->d_ends, D->nb, D->p.nclips, D->d_cin);
    adj_full_lane_kernel<N, G><<<gl, kScanThreads, 0, s>>>(C, u, D->d_bits, D->d_z, D->d_h, D->S,
                                                          D->n, Lb, D->nb, D->p.nclips, D->d_starts,
                                                          D->d_cin, D->d_scr, D->d_ubar, D->d_gpart);
  }
  D->c->launches += 3;
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int scan(const char* which, dsdgpu_diff* D, const LoopCoef& C, const Mat& carry, const double* u,
         const double* beta) {
  switch (D->N) {
#define DIFF_CASE(NN) case NN: return launch_scan<NN>(which, D, C, carry, u, beta);
    DIFF_CASE(2) DIFF_CASE(3) DIFF_CASE(4) DIFF_CASE(5) DIFF_CASE(6)
    DIFF_CASE(7) DIFF_CASE(8) DIFF_CASE(9) DIFF_CASE(10)
#undef DIFF_CASE
    default: return -1;
  }
}

// u = gain * chain(src) for all clips (src: [C][frames] doubles)
int run_chain(dsdgpu_diff* D, const double* src, double* dst) {
  cudaStream_t s = D->c->stream;
  const int C = D->p.nclips;
  long long len = D->p.frames;
  const double* in = src;
  for (int k = 0; k < D->stages; k++) {
    double* out = (k == D->stages - 1) ? dst : ((k & 1) ? D->d_pong : D->d_ping);
    const double scale = (k == D->stages - 1) ? D->p.gain : 1.0;
    chain64_stage_kernel<<<grid_of(len * D->sd[k].U * C, 256), 256, 0, s>>>(
        in, len, out, D->sd[k], D->d_taps, D->d_lag, C, scale);
    D->c->launches++;
    in = out;
    len *= D->sd[k].U;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// pbar = chain^T(ubar) * gain, ending at the PCM rate in d_ping or d_pong
int run_chain_adj(dsdgpu_diff* D, const double* ubar, double** pbar) {
  cudaStream_t s = D->c->stream;
  const int C = D->p.nclips;
  long long len = D->n;
  const double* in = ubar;
  double* out = nullptr;
  for (int k = D->stages - 1; k >= 0; k--) {
    const long long n_in = len / D->sd[k].U;
    out = ((D->stages - 1 - k) & 1) ? D->d_pong : D->d_ping;
    const double scale = (k == D->stages - 1) ? D->p.gain : 1.0;
    chain64_stage_adj_kernel<<<grid_of(n_in * C, 256), 256, 0, s>>>(in, n_in, out, D->sd[k],
                                                                     D->d_taps, D->d_lag, C, scale);
    D->c->launches++;
    in = out;
    len = n_in;
  }
  *pbar = out;
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int loss_from(dsdgpu_diff* D, bool bits, double* loss) {
  cudaStream_t s = D->c->stream;
  const long long tot = (long long)D->p.nclips * D->S.M;
  if (bits)
    loss_z_kernel<true><<<D->nparts, 256, 0, s>>>(D->d_bits, nullptr, D->d_r, D->n, D->d_h, D->S,
                                                  D->p.nclips, D->d_z, D->d_part);
  else
    loss_z_kernel<false><<<D->nparts, 256, 0, s>>>(nullptr, D->d_y, D->d_r, D->n, D->d_h, D->S,
                                                   D->p.nclips, D->d_z, D->d_part);
  D->c->launches++;
  (void)tot;
  std::vector<double> part(D->nparts);
  cudaError_t e = cudaMemcpyAsync(part.data(), D->d_part, sizeof(double) * D->nparts,
                                  cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return D->c->cuda_fail(e, "loss");
  double acc = 0.0;
  for (double v : part) acc += v;
  *loss = acc / ((double)D->p.nclips * (double)D->S.M);
  return DSDGPU_OK;
}

LoopCoef coef_of(const dsdgpu_diff* D, const double* a, const double* g) {
  LoopCoef C;
  memset(&C, 0, sizeof C);
  for (int i = 0; i < D->N; i++) {
    C.a[i] = a[i];
    C.g[i] = g[i];
  }
  C.kappa = D->p.kappa;
  return C;
}

// pre-emphasis + chain at taps w -> d_u
int sdm_input(dsdgpu_diff* D, const double* w) {
  cudaStream_t s = D->c->stream;
  cudaMemcpyAsync(D->d_w, w, sizeof(double) * D->p.preemph_taps, cudaMemcpyHostToDevice, s);
  const long long tot = D->p.frames * D->p.nclips;
  preemph_kernel<<<grid_of(tot, 256), 256, 0, s>>>(D->d_x, D->p.frames, D->p.nclips, D->d_w,
                                                   D->p.preemph_taps, D->d_p);
  D->c->launches++;
  return run_chain(D, D->d_p, D->d_u);
}

}  // namespace

extern "C" {

int dsdgpu_diff_create(dsdgpu_context_t* c, const dsdgpu_diff_params_t* p, dsdgpu_diff_t** out) {
  if (!c || !p || !out) return DSDGPU_ERR_ARG;
  *out = nullptr;
  SdmParams P;
  const char* err = nullptr;
  int rc = sdm_params_from_abi(&p->sdm, &P, &err);
  if (rc) return c->fail(rc, err);
  if (p->nclips < 1 || p->frames < 1) return c->fail(DSDGPU_ERR_ARG, "no clips");
  if (p->preemph_taps < 1 || p->preemph_taps > kMaxPreTaps)
    return c->fail(DSDGPU_ERR_ARG, "pre-emphasis taps out of range (1..255)");
  if (p->lpf_taps < 1 || p->lpf_taps > kMaxLpfTaps || !(p->lpf_taps & 1))
    return c->fail(DSDGPU_ERR_ARG, "loss low-pass taps must be odd, <= 511");
  if (p->decim < 1) return c->fail(DSDGPU_ERR_ARG, "decimation < 1");
  const int L = p->checkpoint;
  if (L < kSubLen || L > kSubLen * kMaxSubs || (L & (L - 1)))
    return c->fail(DSDGPU_ERR_ARG, "checkpoint must be a power of two in 64..16384");
  int U[kMaxStages], Ls[kMaxStages];
  const int S = plan_chain((unsigned)p->fs_in, (unsigned)p->fs_out, U, Ls);
  if (S < 0) return c->fail(DSDGPU_ERR_ARG, "unsupported rate pair");
  dsdgpu_diff* D = new (std::nothrow) dsdgpu_diff();
  if (!D) return DSDGPU_ERR_NOMEM;
  D->c = c;
  D->p = *p;
  D->N = P.order;
  D->n = p->frames * (long long)(p->fs_out / p->fs_in);
  if (D->n % L != 0 || D->n <= P.lat || D->n < p->lpf_taps) {
    delete D;
    return c->fail(DSDGPU_ERR_ARG, "clip length (frames * ratio) must be a multiple of the checkpoint");
  }
  D->nb = (int)(D->n / L);
  D->S.T = p->lpf_taps;
  D->S.D = p->decim;
  D->S.M = (D->n - p->lpf_taps) / p->decim + 1;
  D->S.scale = 2.0 / ((double)p->nclips * (double)D->S.M);
  cudaSetDevice(c->device);
  // FP64 chain: the reference's tap design, every tap kept
  std::vector<double> taps;
  std::vector<int> lag;
  D->stages = S;
  for (int k = 0; k < S; k++) {
    double h[255];
    design_taps(Ls[k], U[k] == 4, h);
    D->sd[k].U = U[k];
    for (int r = 0; r < U[k]; r++) {
      D->sd[k].off[r] = (int)taps.size();
      int cnt = 0;
      for (int j = 0; U[k] * j + r < Ls[k]; j++) {
        taps.push_back(h[U[k] * j + r] * (double)U[k]);
        lag.push_back(j);
        cnt++;
      }
      D->sd[k].nph[r] = cnt;
    }
  }
  // loss low-pass: Kaiser-windowed sinc (beta 10), unit DC gain
  std::vector<double> hl(p->lpf_taps);
  {
    const int T = p->lpf_taps;
    const double fc = p->lpf_cutoff_hz / (double)p->fs_out;   // cycles per sample
    const double pi = 3.14159265358979323846;
    auto i0 = [](double x) {
      double s = 1.0, t = 1.0;
      for (int k = 1; k < 60; k++) {
        t *= (x / (2.0 * k)) * (x / (2.0 * k));
        s += t;
      }
      return s;
    };
    double sum = 0.0;
    for (int k = 0; k < T; k++) {
      const double m = k - (T - 1) / 2.0;
      const double sinc = m == 0.0 ? 2.0 * fc : std::sin(2.0 * pi * fc * m) / (pi * m);
      const double q = 2.0 * k / (double)(T - 1) - 1.0;
      const double w = T > 1 ? i0(10.0 * std::sqrt(std::fmax(0.0, 1.0 - q * q))) / i0(10.0) : 1.0;
      hl[k] = sinc * w;
      sum += hl[k];
    }
    for (double& v : hl) v /= sum;
  }
  const size_t Cn = (size_t)p->nclips * (size_t)D->n;
  const size_t Cf = (size_t)p->nclips * (size_t)p->frames;
  const size_t CbN = (size_t)p->nclips * D->nb * D->N;
  D->nparts = grid_of((long long)p->nclips * D->S.M, 256);
  bool ok = D->alloc(&D->d_taps, taps.size()) == 0 && D->alloc(&D->d_lag, lag.size()) == 0 &&
            D->alloc(&D->d_x, Cf) == 0 && D->alloc(&D->d_xd, Cf) == 0 &&
            D->alloc(&D->d_w, kMaxPreTaps) == 0 && D->alloc(&D->d_p, Cf) == 0 &&
            D->alloc(&D->d_ping, Cn / 2 + 1) == 0 && D->alloc(&D->d_pong, Cn / 2 + 1) == 0 &&
            D->alloc(&D->d_u, Cn) == 0 && D->alloc(&D->d_r, Cn) == 0 &&
            D->alloc(&D->d_bits, Cn) == 0 && D->alloc(&D->d_beta, Cn) == 0 &&
            D->alloc(&D->d_y, Cn) == 0 && D->alloc(&D->d_ubar, Cn) == 0 &&
            D->alloc(&D->d_h, hl.size()) == 0 &&
            D->alloc(&D->d_z, (size_t)p->nclips * D->S.M) == 0 &&
            D->alloc(&D->d_part, D->nparts) == 0 && D->alloc(&D->d_ends, CbN) == 0 &&
            D->alloc(&D->d_starts, CbN) == 0 && D->alloc(&D->d_sstarts, CbN) == 0 &&
            D->alloc(&D->d_cin, CbN) == 0 && D->alloc(&D->d_gpart, 2 * CbN) == 0 &&
            D->alloc(&D->d_gw, kMaxPreTaps) == 0 && D->alloc(&D->d_smax, (size_t)p->nclips) == 0 &&
            D->alloc(&D->d_scr, (size_t)p->nclips * D->nb * (L / kSubLen + kSubLen) * D->N) == 0 &&
            D->alloc(&D->d_ctx, (size_t)p->nclips) == 0 &&
            D->alloc(&D->d_jobs, (size_t)p->nclips) == 0 && D->alloc(&D->d_counter, 1) == 0;
  for (cudaEvent_t& e : D->ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
  if (!ok) {
    delete D;
    return c->cuda_fail(cudaGetLastError(), "diff allocation");
  }
  cudaStream_t s = c->stream;
  cudaMemcpyAsync(D->d_taps, taps.data(), sizeof(double) * taps.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(D->d_lag, lag.data(), sizeof(int) * lag.size(), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(D->d_h, hl.data(), sizeof(double) * hl.size(), cudaMemcpyHostToDevice, s);
  rc = c->check_status();
  if (rc) {
    delete D;
    return rc;
  }
  *out = D;
  return DSDGPU_OK;
}

void dsdgpu_diff_destroy(dsdgpu_diff_t* D) {
  if (!D) return;
  if (D->c) {
    cudaSetDevice(D->c->device);
    cudaStreamSynchronize(D->c->stream);
  }
  delete D;
}

int dsdgpu_diff_set_input(dsdgpu_diff_t* D, const float* d_pcm) {
  if (!D || !d_pcm) return DSDGPU_ERR_ARG;
  dsdgpu_context* c = D->c;
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const size_t Cf = (size_t)D->p.nclips * (size_t)D->p.frames;
  cudaError_t e = cudaMemcpyAsync(D->d_x, d_pcm, sizeof(float) * Cf, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return c->cuda_fail(e, "pcm copy");
  float_to_double_kernel<<<grid_of((long long)Cf, 256), 256, 0, s>>>(D->d_x, (long long)Cf, D->d_xd);
  c->launches++;
  if (run_chain(D, D->d_xd, D->d_r) != 0) return c->cuda_fail(cudaGetLastError(), "reference chain");
  D->have_input = true;
  D->have_forward = false;
  return c->check_status();
}

int dsdgpu_diff_forward(dsdgpu_diff_t* D, const double* taps, const double* a, const double* g,
                        double* loss) {
  if (!D || !taps || !a || !g || !loss) return DSDGPU_ERR_ARG;
  dsdgpu_context* c = D->c;
  if (!D->have_input) return c->fail(DSDGPU_ERR_STATE, "no input clips");
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const int N = D->N;
  cudaEventRecord(D->ev[0], s);
  if (sdm_input(D, taps) != 0) return c->cuda_fail(cudaGetLastError(), "sdm input");
  // exact decisions: every clip one sequential run, then a drain of lat zeros
  dsdgpu_sdm_params_t sp = D->p.sdm;
  for (int i = 0; i < N; i++) {
    sp.a[i] = a[i];
    sp.g[i] = g[i];
  }
  SdmParams P;
  const char* err = nullptr;
  int rc = sdm_params_from_abi(&sp, &P, &err);
  if (rc) return c->fail(rc, err);
  P.mode = c->sdm_mode;
  P.lanes = c->sdm_lanes;
  const int C = D->p.nclips;
  if (init_contexts(D->d_ctx, 0, C, 0, s) != 0) return c->cuda_fail(cudaGetLastError(), "context init");
  c->launches++;
  cudaEventRecord(D->ev[1], s);
  std::vector<SdmJob> jobs(C);
  for (int k = 0; k < 2; k++) {
    for (int i = 0; i < C; i++) {
      SdmJob& j = jobs[i];
      j.ctx = i;
      j.copy_from = -1;
      j.seed_state = nullptr;
      j.flags = 0;
      if (k == 0) {
        j.in = D->d_u + (size_t)i * D->n;
        j.n_in = D->n;
        j.skip_out = P.lat;
        j.out = D->d_bits + (size_t)i * D->n;
      } else {
        j.in = nullptr;
        j.n_in = P.lat;
        j.skip_out = 0;
        j.out = D->d_bits + (size_t)i * D->n + (D->n - P.lat);
      }
    }
    cudaMemcpyAsync(D->d_jobs, jobs.data(), sizeof(SdmJob) * C, cudaMemcpyHostToDevice, s);
    if (launch_sdm_jobs(P, D->d_jobs, C, D->d_counter, D->d_ctx, c->d_status, 0, s) != 0)
      return c->cuda_fail(cudaGetLastError(), "sdm launch");
    c->launches++;
    // the job table is rewritten for the drain: wait for the copy's source
    rc = c->check_status();
    if (rc) return rc;
  }
  c->sdm_samples += (unsigned long long)C * (unsigned long long)(D->n + P.lat);
  cudaEventRecord(D->ev[2], s);
  // base trajectory, checkpoints and beta
  const LoopCoef coef = coef_of(D, a, g);
  Mat none;
  memset(&none, 0, sizeof none);
  if (scan("base", D, coef, none, D->d_u, nullptr) != 0) return c->cuda_fail(cudaGetLastError(), "base pass");
  rc = loss_from(D, true, loss);
  if (rc) return rc;
  {
    // the decisions must form one bounded loop trajectory: a trellis output
    // that switched between unmerged paths drives the open loop off it
    std::vector<double> mx(C);
    cudaMemcpy(mx.data(), D->d_smax, sizeof(double) * C, cudaMemcpyDeviceToHost);
    for (int i = 0; i < C; i++)
      if (!(mx[i] < kStateBound))
        return c->fail(DSDGPU_ERR_UNSUPPORTED,
                       "decisions leave the loop's bounded trajectory (trellis paths did not merge within lat)");
  }
  cudaEventRecord(D->ev[3], s);
  cudaEventSynchronize(D->ev[3]);
  cudaEventElapsedTime(&D->ms[0], D->ev[0], D->ev[3]);
  cudaEventElapsedTime(&D->ms[1], D->ev[1], D->ev[2]);
  D->coef = coef;
  D->taps.assign(taps, taps + D->p.preemph_taps);
  D->have_forward = true;
  return c->check_status();
}

int dsdgpu_diff_backward(dsdgpu_diff_t* D, double* grad_taps, double* grad_a, double* grad_g) {
  if (!D || !grad_taps || !grad_a || !grad_g) return DSDGPU_ERR_ARG;
  dsdgpu_context* c = D->c;
  if (!D->have_forward) return c->fail(DSDGPU_ERR_STATE, "no forward to differentiate");
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const int N = D->N;
  cudaEventRecord(D->ev[0], s);
  // z of the last forward is in d_z (the loss pass over the decisions)
  const Mat A = closed_loop(loop_matrix(D->coef.g, N), D->coef.a, D->p.kappa, N);
  const Mat P = transpose(mat_pow(A, D->p.checkpoint, N), N);
  if (scan("adj", D, D->coef, P, D->d_u, nullptr) != 0) return c->cuda_fail(cudaGetLastError(), "adjoint scan");
  double* pbar = nullptr;
  if (run_chain_adj(D, D->d_ubar, &pbar) != 0) return c->cuda_fail(cudaGetLastError(), "chain adjoint");
  taps_grad_kernel<<<D->p.preemph_taps, 256, 0, s>>>(pbar, D->d_x, D->p.frames, D->p.nclips,
                                                     D->p.preemph_taps, D->d_gw);
  c->launches++;
  const size_t parts = (size_t)D->p.nclips * D->nb;
  std::vector<double> gp(parts * 2 * N);
  cudaMemcpyAsync(gp.data(), D->d_gpart, sizeof(double) * gp.size(), cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(grad_taps, D->d_gw, sizeof(double) * D->p.preemph_taps, cudaMemcpyDeviceToHost, s);
  cudaEventRecord(D->ev[1], s);
  const int rc = c->check_status();
  if (rc) return rc;
  for (int k = 0; k < N; k++) {
    double sa = 0.0, sg = 0.0;
    for (size_t q = 0; q < parts; q++) {
      sa += gp[q * 2 * N + k];
      sg += gp[q * 2 * N + N + k];
    }
    grad_a[k] = sa;
    grad_g[k] = sg;
  }
  cudaEventElapsedTime(&D->ms[2], D->ev[0], D->ev[1]);
  return DSDGPU_OK;
}

int dsdgpu_diff_surrogate(dsdgpu_diff_t* D, const double* taps, const double* a, const double* g,
                          double* loss) {
  if (!D || !taps || !a || !g || !loss) return DSDGPU_ERR_ARG;
  dsdgpu_context* c = D->c;
  if (!D->have_forward) return c->fail(DSDGPU_ERR_STATE, "no forward decisions to freeze");
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const int N = D->N;
  cudaEventRecord(D->ev[0], s);
  // the surrogate's SDM input goes to d_y's twin: reuse d_ubar as scratch
  double* u_keep = D->d_u;
  D->d_u = D->d_ubar;
  int rc = sdm_input(D, taps) != 0 ? DSDGPU_ERR_CUDA : DSDGPU_OK;
  D->d_u = u_keep;
  if (rc) return c->cuda_fail(cudaGetLastError(), "surrogate input");
  const LoopCoef coef = coef_of(D, a, g);
  const Mat A = mat_pow(closed_loop(loop_matrix(g, N), a, D->p.kappa, N), D->p.checkpoint, N);
  if (scan("sur", D, coef, A, D->d_ubar, D->d_beta) != 0) return c->cuda_fail(cudaGetLastError(), "surrogate scan");
  rc = loss_from(D, false, loss);
  // backward reads the forward's z: recompute it from the decisions
  double tmp;
  if (!rc) rc = loss_from(D, true, &tmp);
  cudaEventRecord(D->ev[1], s);
  cudaEventSynchronize(D->ev[1]);
  cudaEventElapsedTime(&D->ms[3], D->ev[0], D->ev[1]);
  // the surrogate's SDM input sat in d_ubar, which backward rewrites
  return rc ? rc : c->check_status();
}

int dsdgpu_diff_times(const dsdgpu_diff_t* D, float* ms4) {
  if (!D || !ms4) return DSDGPU_ERR_ARG;
  memcpy(ms4, D->ms, sizeof D->ms);
  return DSDGPU_OK;
}

int dsdgpu_diff_buffers(const dsdgpu_diff_t* D, const double** d_sdm_in, const uint8_t** d_bits,
                        int64_t* n) {
  if (!D) return DSDGPU_ERR_ARG;
  if (d_sdm_in) *d_sdm_in = D->d_u;
  if (d_bits) *d_bits = D->d_bits;
  if (n) *n = D->n;
  return DSDGPU_OK;
}

}  // extern "C"
