// Trellis (Viterbi look-ahead) 1-bit sigma-delta modulator for sm_103a.
//
// One warp runs one SDM job (a channel block or a DAS segment); a persistent
// grid pulls jobs from an atomic counter, so one launch covers any mix of
// channels, segments and streams.  Lane i owns the candidate at rank i
// (K <= 32): its NTF state, cost, path, traceback bit and a lat-bit traceback
// ring live in registers.  Each input sample:
//
//   1. expansion   every live lane advances its NTF (FP64, reference order,
//                  no contraction: __dadd_rn/__dmul_rn) and forms both
//                  children: slots 2i (bit 0, state[0] + 1) and 2i + 1
//                  (bit 1, state[0] - 1)          (reference src/trellis.c:37-191)
//   2. selection   warp argmin over the 2n children by int64 cost bits,
//                  majority vote on the traceback bit with the 1.1x override,
//                  then the reference's ordered insertion with path-hash
//                  dedup, emulated warp-cooperatively: the sorted act list is
//                  held one entry per lane and every insertion is a ballot +
//                  shuffle; the hash chains are walked in shared memory
//                                                  (src/trellis.c:582-731)
//   3. commit      survivors pull their parent's state, path, traceback bit
//                  and ring with shuffles, normalise cost by the new minimum
//                  and write their decision bit into the ring
//                                                  (src/trellis.c:938-972)
//
// The shared-memory slot arrays (path, cost bits, chain link for both banks)
// reproduce the reference's slot memory, including the K = 32 store one past
// act[] that lands on path_hash[0] while bank 1 is sorted (src/trellis.c:668-673).
#include "sdm_internal.h"

#include <climits>
#include <cstdio>

namespace dsdgpu {

// One warp per CTA (one job, or 32 / LPJ jobs side by side for K <= 16): a
// few thousand long-running jobs spread evenly over the SMs.  At 32 lanes the
// launch bound (32 threads, 13 CTAs per SM) holds the kernel at 128 registers
// (a 152-register build measured 50 % slower on the DSD128 DAS workload, with
// fewer warps per FP64 pipe); narrower widths take 10 CTAs per SM, which left
// the 16-lane order-8 kernel at 168 registers with 60 bytes of spills instead
// of 344 and ran the DSD512 workload 6.7 % faster (442.1 -> 471.5).
constexpr int kRegRingWords = 8;      // rings held in registers: lat <= 256
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ long long key_of(double c) { return __double_as_longlong(c); }

// A ring word kept opaque in a register: without it the word-select loops over
// a 64-word ring compile to an indexed local-memory array.
template <int RW>
__device__ __forceinline__ uint32_t reg_word(uint32_t v) {
  if constexpr (RW > kRegRingWords) asm volatile("" : "+r"(v));
  return v;
}

template <int LPJ>
__device__ __forceinline__ unsigned long long shfl64(unsigned long long v, int src, unsigned hm) {
  return (unsigned long long)__shfl_sync(hm, (long long)v, src, LPJ);
}

// ballot / match over the job's lanes, as bits of the job's lane numbers
#define BALLOT(p) (__ballot_sync(hm, (p)) >> sh)
#define MATCH(v) (__match_any_sync(hm, (v)) >> sh)

// The NTF advance with y = 0 (src/trellis.c:37-151; every order has the
// same shape): d[0] = (s0 - g0 s1) + x; d[i] = (s[i] + s[i-1]) - g[i] s[i+1];
// d[N-1] = s[N-1] + s[N-2]; v = ((x + a0 d0) + a1 d1) + ...  The two children
// of a candidate share s[1..N-1], so everything that does not involve s[0]
// (g0 s1, g1 s2, d[2..N-1] and a[i] d[i] for i >= 2) is the same for both
// siblings: it is computed once per parent, while the next selection runs,
// and handed to the surviving children as a Pack.  Each sample then keeps only
// the s[0]-dependent operations on its critical path.  Every operation is the
// reference's, in the reference's order, rounded separately (no contraction).
template <int N>
struct Pack {
  double G0;      // g0 * s1
  double G1;      // g1 * s2          (N >= 3)
  double D[N];    // d[i], i = 2..N-1
  double A[N];    // a[i] * d[i], i = 2..N-1
};

template <int N>
__host__ __device__ constexpr int shared_ops() { return N >= 3 ? 4 * N - 8 : 1; }

// Operation k of the shared part, inputs S[1..N-1] (a child's state), into
// np (with scratch tg/tu).  Orders respect the dependencies when k runs
// 0, 1, 2, ...
template <int N>
__device__ __forceinline__ void shared_op(int k, const SdmParams& P, const double (&S)[N],
                                          Pack<N>& np, double (&tg)[N], double (&tu)[N]) {
  if (N < 3) {
    if (k == 0) np.G0 = __dmul_rn(P.g[0], S[1]);
    return;
  }
  constexpr int M = N - 3;   // middle indices i = 2..N-2
  if (k == 0) { np.G0 = __dmul_rn(P.g[0], S[1]); return; }
  if (k == 1) { np.G1 = __dmul_rn(P.g[1], S[2]); return; }
  k -= 2;
  if (k < M) { const int i = 2 + k; tg[i] = __dmul_rn(P.g[i], S[i + 1]); return; }
  k -= M;
  if (k < M) { const int i = 2 + k; tu[i] = __dadd_rn(S[i], S[i - 1]); return; }
  k -= M;
  if (k == 0) { np.D[N - 1] = __dadd_rn(S[N - 1], S[N - 2]); return; }
  k -= 1;
  if (k < M) { const int i = 2 + k; np.D[i] = __dsub_rn(tu[i], tg[i]); return; }
  k -= M;
  if (k < N - 2) { const int i = 2 + k; np.A[i] = __dmul_rn(P.a[i], np.D[i]); return; }
}

template <int N>
__device__ __forceinline__ void shared_all(const SdmParams& P, const double (&S)[N], Pack<N>& np) {
  double tg[N], tu[N];
#pragma unroll
  for (int k = 0; k < shared_ops<N>(); k++) shared_op<N>(k, P, S, np, tg, tu);
}

// Shared memory of one job run by LPJ lanes: the slot memory of both banks
// for its 2 * LPJ children (K <= LPJ, so children 2K.. are never touched),
// the 128-bucket path hash and the selection scratch.
template <int LPJ>
struct WarpSmem {
  static constexpr int S = 2 * LPJ;
  unsigned long long path[2][S];
  long long key[2][S];
  int8_t link[2][S];
  int8_t heads[kBuckets];
  int8_t act[LPJ];             // scatter target of the fast selection
  uint8_t hashmark[S];         // children the serial path hashed (verify mode)
  uint8_t hashmark2[S];        // children the fast path deems hashed
  int8_t pos[S];               // sorted position of each child (serial path)
  int8_t idx_at[S];            // child at each sorted position (serial path)
};

// Lanes per job: the smallest power of two >= K (at least 2) is the tightest
// packing, 32 / LPJ jobs per warp; a requested width (SdmParams::lanes) is
// raised to it.
__host__ __device__ constexpr int min_lanes(int K) {
  return K > 16 ? 32 : K > 8 ? 16 : K > 4 ? 8 : K > 2 ? 4 : 2;
}

// Fixed rule (the batch plan sizes its job slots with it): a requested width,
// else a whole warp for K > 16 and a half-warp below.
int lanes_per_job(const SdmParams& P) {
  if (P.lat > 32 * kRegRingWords) return 32;   // the wide-ring kernel: one job per warp
  const int lo = min_lanes(P.cands);
  if (P.lanes > 0) return P.lanes > lo ? P.lanes : lo;
  return lo > 16 ? 32 : 16;
}

// Warp slots of the device: 16 one-warp CTAs per SM (128 registers a thread).
static int resident_warps() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 152 * 16;
  if (!cached[dev]) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = (sms > 0 ? sms : 152) * 16;
  }
  return cached[dev];
}

// Lanes for a launch of njobs jobs with no block cap: the widest width whose
// jobs all fit in one wave of resident warps.  The trellis step of a small-K
// job is bound by its serial selection chain rather than by FP64 issue, so
// fewer jobs per warp run faster as long as no job waits for a second wave
// (10 s stereo same-rate DSD128, 1722 jobs: K = 16 at 32 lanes 289 vs 256 at
// 16 lanes DSD Msamples/s; K = 2 at 2 lanes 174, at 16 lanes 309).
static int launch_lanes(const SdmParams& P, int njobs, int max_blocks) {
  if (P.lanes > 0 || max_blocks > 0 || P.lat > 32 * kRegRingWords) return lanes_per_job(P);
  const int lo = min_lanes(P.cands);
  int lanes = 32;
  // warp slots of a width: 16 one-warp CTAs per SM at 32 lanes (128 registers),
  // 10 below (their launch bound leaves up to 204 registers)
  while (lanes > lo &&
         (long long)njobs * lanes > (long long)resident_warps() / 16 * (lanes == 32 ? 16 : 10) * 32)
    lanes >>= 1;
  return lanes;
}

template <int LPJ>
__host__ __device__ constexpr unsigned job_mask(int sh) {
  return LPJ == 32 ? 0xffffffffu : (((1u << LPJ) - 1u) << sh);
}

// (key, index) order of the survivor selection: cost bits as int64, then slot.
__device__ __forceinline__ bool key_less(long long ka, int ia, long long kb, int ib) {
  return ka < kb || (ka == kb && ia < ib);
}

// Bitonic sort of the 2 * LPJ (key, index) pairs of one job, two per lane
// (sorted positions 2*lane and 2*lane + 1), ascending.  With LPJ = 16 each
// half-warp sorts its own job (exchange distances stay inside the half).
template <int LPJ, typename Hook>
__device__ __forceinline__ void bitonic_sort(long long& kA, int& iA, long long& kB, int& iB,
                                             int lane, unsigned hm, Hook&& hook) {
  int stage = 0;
#pragma unroll
  for (int k = 2; k <= 2 * LPJ; k <<= 1) {
    const bool asc = ((2 * lane) & k) == 0;
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      hook(stage++);
      if (j == 1) {
        const bool sw = asc ? key_less(kB, iB, kA, iA) : key_less(kA, iA, kB, iB);
        if (sw) {
          const long long tk = kA; kA = kB; kB = tk;
          const int ti = iA; iA = iB; iB = ti;
        }
      } else {
        const int lj = j >> 1;
        const bool keep_min = (((lane & lj) == 0) == asc);
        long long pk = __shfl_xor_sync(hm, kA, lj, LPJ);
        int pi = __shfl_xor_sync(hm, iA, lj, LPJ);
        if (keep_min == key_less(pk, pi, kA, iA)) { kA = pk; iA = pi; }
        pk = __shfl_xor_sync(hm, kB, lj, LPJ);
        pi = __shfl_xor_sync(hm, iB, lj, LPJ);
        if (keep_min == key_less(pk, pi, kB, iB)) { kB = pk; iB = pi; }
      }
    }
  }
}

// Stages of the bitonic sort of 2 * LPJ keys: log2(2 LPJ) (log2(2 LPJ) + 1) / 2
// (21 for 64 keys, 15 for 32, 10, 6, 3).
template <int LPJ>
__host__ __device__ constexpr int sort_stages() {
  return LPJ == 32 ? 21 : LPJ == 16 ? 15 : LPJ == 8 ? 10 : LPJ == 4 ? 6 : 3;
}

// LPJ lanes run one job (lanes_per_job(K)): a whole warp for K > 16, else
// 32 / LPJ jobs side by side in one warp, so small trellises do not leave
// most of every FP64 warp instruction idle.  `lane` is the lane within the
// job, `hm` the job's lanes; warp intrinsics use hm and width LPJ, ballots
// are shifted to the job's bits.
template <int N, int LPJ, int RW>
__device__ void run_job(const SdmParams& P, const SdmJob& job, SdmCtx* __restrict__ ctxs,
                        WarpSmem<LPJ>& sm, int* __restrict__ status) {
  constexpr int S = WarpSmem<LPJ>::S;
  const int wl = threadIdx.x & 31;
  const int lane = wl & (LPJ - 1);
  const unsigned sh = (unsigned)(wl - lane);
  const unsigned hm = job_mask<LPJ>((int)sh);
  // ctx < 0: the job's end state goes to a scratch context, one per job slot
  // of the launch, at (-ctx - 1) + slot (jobs whose end state nobody reads)
  const int slot_id = (int)blockIdx.x * (32 / LPJ) + wl / LPJ;
  const int dst_i = job.ctx >= 0 ? job.ctx : (-job.ctx - 1) + slot_id;
  const SdmCtx* src = &ctxs[job.copy_from >= 0 ? job.copy_from : dst_i];
  SdmCtx* dst = &ctxs[dst_i];
  const int K = P.cands;
  const int W = (P.lat + 31) >> 5;
  const unsigned long long mask = P.mask;

  int n = src->n, bank = src->bank, pos = src->pos;
  double s[N];
  double cost = 0.0;
  unsigned long long path = 0;
  uint32_t ring[RW];
  int nxt = 0, slot = 0;
#pragma unroll
  for (int k = 0; k < N; k++) s[k] = 0.0;
#pragma unroll
  for (int w = 0; w < RW; w++) ring[w] = 0;
  if (lane < n) {
#pragma unroll
    for (int k = 0; k < N; k++) s[k] = src->s[lane][k];
    cost = src->cost[lane];
    path = src->path[lane];
    nxt = src->next[lane];
    slot = src->slot[lane];
#pragma unroll
    for (int w = 0; w < RW; w++)
      if (w < W) ring[w] = src->ring[lane][w];
  }
  for (int i = lane; i < 2 * S; i += LPJ) {
    const int b = i / S, j = i % S;
    sm.path[b][j] = src->spath[b][j];
    sm.key[b][j] = (long long)src->skey[b][j];
    sm.link[b][j] = src->slink[b][j];
  }
  unsigned long long c_conv = 0, c_coll = 0, c_drop = 0, c_tot = 0;
  if (job.copy_from < 0) {
    c_conv = src->conv_fail;
    c_coll = src->cands_collapse;
    c_drop = src->next_filter_drops;
    c_tot = src->total_children;
  }
  __syncwarp(hm);
  if (job.seed_state) {
    // DAS temp seeding: every live candidate gets the estimated state, cost 0.
    if (lane < n) {
#pragma unroll
      for (int k = 0; k < N; k++) s[k] = job.seed_state[k];
      cost = 0.0;
      sm.key[bank][slot] = key_of(0.0);
    }
    __syncwarp(hm);
  }
  // the candidate as (s0, s1, shared part of its next advance)
  double cs0 = s[0], cs1 = s[1];
  Pack<N> pk;
  shared_all<N>(P, s, pk);

  const long long n_in = job.n_in;
  const double* __restrict__ in = job.in;
  double x_cur = 0.0, x_nxt = 0.0;
  if (in) {
    if (lane < n_in) x_cur = in[lane];
    if (LPJ + lane < n_in) x_nxt = in[LPJ + lane];
  }
  uint8_t obit = 0;
  int err = 0;
  const bool lim_on = P.state_limit > 0.0;

  for (long long t = 0; t < n_in; t++) {
    const int tl = (int)(t & (LPJ - 1));
    if (tl == 0 && t > 0) {
      x_cur = x_nxt;
      x_nxt = (in && t + LPJ + lane < n_in) ? in[t + LPJ + lane] : 0.0;
    }
    const double x = __shfl_sync(hm, x_cur, tl, LPJ);
    const int nb = bank ^ 1;
    int next_pos = pos + 1;
    if (next_pos == P.lat) next_pos = 0;
    const bool live = lane < n;

    // ---- 1. expansion: the s0-dependent part of the advance ----
    double S[N];          // the children's shared state s[1..N-1] (clamped)
#pragma unroll
    for (int k = 0; k < N; k++) S[k] = 0.0;
    double s00 = 0.0, s01 = 0.0;
    long long key0 = LLONG_MAX, key1 = LLONG_MAX;
    unsigned long long q = 0;
    int new_next = 0;
    const int old_next = nxt;
    if (live) {
      const double d0 = __dadd_rn(__dsub_rn(cs0, pk.G0), x);
      const double d1 = (N >= 3) ? __dsub_rn(__dadd_rn(cs1, cs0), pk.G1) : __dadd_rn(cs1, cs0);
      double v = __dadd_rn(x, __dmul_rn(P.a[0], d0));
      v = __dadd_rn(v, __dmul_rn(P.a[1], d1));
#pragma unroll
      for (int i = 2; i < N; i++) v = __dadd_rn(v, pk.A[i]);
      s00 = __dadd_rn(d0, 1.0);
      s01 = __dsub_rn(d0, 1.0);
      S[1] = d1;
#pragma unroll
      for (int i = 2; i < N; i++) S[i] = pk.D[i];
      if (lim_on) {
#pragma unroll
        for (int k = 1; k < N; k++) S[k] = clamp_state(S[k], P.state_limit);
        s00 = clamp_state(s00, P.state_limit);
        s01 = clamp_state(s01, P.state_limit);
      }
      const double e0 = __dadd_rn(v, P.a[0]);
      const double e1 = __dsub_rn(v, P.a[0]);
      key0 = key_of(__dadd_rn(cost, __dmul_rn(e0, e0)));
      key1 = key_of(__dadd_rn(cost, __dmul_rn(e1, e1)));
      q = (path << 1) & mask;
      uint32_t wv = 0;
#pragma unroll
      for (int w = 0; w < RW; w++) {
        const uint32_t r = reg_word<RW>(ring[w]);
        if (w == (next_pos >> 5)) wv = r;
      }
      new_next = (int)((wv >> (next_pos & 31)) & 1u);
      sm.path[nb][2 * lane] = q;
      sm.path[nb][2 * lane + 1] = q | 1ull;
      sm.key[nb][2 * lane] = key0;
      sm.key[nb][2 * lane + 1] = key1;
      sm.heads[q & (kBuckets - 1)] = -1;
      sm.heads[(q | 1ull) & (kBuckets - 1)] = -1;
    }
    __syncwarp(hm);

    // the children's shared part, one operation per stage of the sort below
    Pack<N> npk;
    double tg[N], tu[N];
    // ---- 2. selection ----
    // All 2n children sorted by (cost bits as int64, slot index): position 0
    // is the reference's minimum (first index among equal costs), the first
    // sorted child carrying the majority bit is its best_maj, and the
    // eligible children keep their (cost, index) order (src/trellis.c:628-652).
    long long sk0 = live ? key0 : LLONG_MAX, sk1 = live ? key1 : LLONG_MAX;
    int si0 = 2 * lane, si1 = 2 * lane + 1;
    // The shared-part operations ride on the sort stages, except the last
    // kDeferOps, which are issued at the start of the selection so that its
    // integer work runs while they occupy the FP64 unit.
    constexpr int kOps = shared_ops<N>();
    constexpr int kStages = sort_stages<LPJ>();
    constexpr int kDeferOps = 8;
    constexpr int kSortOps = (kOps < kStages ? kOps : kStages) > kDeferOps
                                 ? (kOps < kStages ? kOps : kStages) - kDeferOps : 0;
    bitonic_sort<LPJ>(sk0, si0, sk1, si1, lane, hm, [&](int st) {
      if (st < kSortOps) shared_op<N>(st, P, S, npk, tg, tu);
    });
    const int sn0 = __shfl_sync(hm, old_next, si0 >> 1, LPJ);   // traceback bit of each sorted child
    const int sn1 = __shfl_sync(hm, old_next, si1 >> 1, LPJ);
    const bool sl0 = (si0 >> 1) < n, sl1 = (si1 >> 1) < n;
    const unsigned nx1 = BALLOT(live && old_next);
    const int votes1 = 2 * __popc(nx1);
    const int majority = (votes1 > 2 * n - votes1) ? 1 : 0;
    const long long mk = __shfl_sync(hm, sk0, 0, LPJ);
    int want = __shfl_sync(hm, sn0, 0, LPJ);
    if (want != majority) {
      const unsigned mA = BALLOT(sl0 && sn0 == majority);
      const unsigned mB = BALLOT(sl1 && sn1 == majority);
      int pos = 1 << 20;
      if (mA) pos = 2 * (__ffs(mA) - 1);
      if (mB) pos = min(pos, 2 * (__ffs(mB) - 1) + 1);
      if (pos < (1 << 20)) {
        const long long bA = __shfl_sync(hm, sk0, pos >> 1, LPJ);
        const long long bB = __shfl_sync(hm, sk1, pos >> 1, LPJ);
        const double cbm = __longlong_as_double((pos & 1) ? bB : bA);
        if (cbm < __dmul_rn(__longlong_as_double(mk), 1.1)) want = majority;
      }
    }
#pragma unroll
    for (int k = kSortOps; k < kOps; k++) shared_op<N>(k, P, S, npk, tg, tu);
    unsigned elig = BALLOT(live && old_next == want);
    c_drop += 2ull * (unsigned)(n - __popc(elig));
    c_tot += 2ull * (unsigned)n;

    // ---- 2b. fast selection ----
    // With no two eligible children on the same path, the reference's ordered
    // insertion with path-hash dedup keeps exactly the first K eligible
    // children of the (cost, index) order: every insert is new to the hash,
    // evictions drop the largest, ties keep insertion (index) order, skips are
    // children that would not be among the K smallest.  A child is hashed iff
    // fewer than K eligible children with a lower index precede it in that
    // order; only at K = 32 while bank 1 is sorted can the stored chain links
    // be read in a later sample (through the act[32] store onto path_hash[0]),
    // so only then are they written, as "previous hashed child of the same
    // bucket".  Duplicate paths, or a bucket-0 child once the list can be full
    // at K = 32 in bank 1, take the serial path.
    const bool me = live && old_next == want;
    const bool e0 = sl0 && sn0 == want, e1 = sl1 && sn1 == want;
    const unsigned EA = BALLOT(e0), EB = BALLOT(e1);
    const int m2 = __popc(EA) + __popc(EB);
    const bool links_matter = (K == kMaxCands && nb == 1);
    bool fast_ok = (P.mode != kModeExact);
    int f_cnt = 0, f_Ls = -1, f_link0 = -1, f_link1 = -1;
    long long f_Lk = LLONG_MAX;
    bool f_h0 = false, f_h1 = false;
    if (fast_ok) {
      const unsigned mm = MATCH(q);
      if (__any_sync(hm, me && __popc(mm & elig) > 1)) fast_ok = false;
      if (links_matter && m2 > K && __any_sync(hm, me && (q & (kBuckets - 1)) == 0))
        fast_ok = false;
    }
    if (fast_ok) {
      const unsigned below = (1u << lane) - 1u;
      const int r0 = __popc(EA & below) + __popc(EB & below);
      const int r1 = r0 + (e0 ? 1 : 0);
      if (e0 && r0 < K) sm.act[r0] = (int8_t)si0;
      if (e1 && r1 < K) sm.act[r1] = (int8_t)si1;
      if (links_matter) {
        // eligible children sorted before, with a lower index: OR-scan of
        // one-hot index masks over the sorted positions
        const unsigned long long mine = (e0 ? (1ull << si0) : 0ull) | (e1 ? (1ull << si1) : 0ull);
        unsigned long long inc = mine;
#pragma unroll
        for (int o = 1; o < LPJ; o <<= 1) {
          const unsigned long long v = (unsigned long long)__shfl_up_sync(hm, (long long)inc, o, LPJ);
          if (lane >= o) inc |= v;
        }
        const unsigned long long before0 = inc & ~mine;
        const unsigned long long before1 = before0 | (e0 ? (1ull << si0) : 0ull);
        const int p0 = __popcll(before0 & ((1ull << si0) - 1ull));
        const int p1 = __popcll(before1 & ((1ull << si1) - 1ull));
        sm.hashmark2[si0] = (uint8_t)(e0 && p0 < K);
        sm.hashmark2[si1] = (uint8_t)(e1 && p1 < K);
      }
      __syncwarp(hm);
      f_cnt = m2 < K ? m2 : K;
      if (lane < f_cnt) {
        f_Ls = sm.act[lane];
        f_Lk = sm.key[nb][f_Ls];
      }
      if (links_matter) {
        f_h0 = live && sm.hashmark2[2 * lane] != 0;
        f_h1 = live && sm.hashmark2[2 * lane + 1] != 0;
        const unsigned H0 = BALLOT(f_h0), H1 = BALLOT(f_h1);
        const unsigned s0 = MATCH((unsigned)(q & (kBuckets - 1))) & H0 & below;
        const unsigned s1 = MATCH((unsigned)((q | 1ull) & (kBuckets - 1))) & H1 & below;
        f_link0 = s0 ? 2 * (31 - __clz(s0)) : -1;
        f_link1 = s1 ? 2 * (31 - __clz(s1)) + 1 : -1;
      }
      __syncwarp(hm);
    }

    // ---- 2c. serial selection (exact reference order) ----
    // The reference's act list is always ordered by (cost, index) (children are
    // inserted in index order, after every element of equal cost), so it is
    // held as a set of sorted positions: insertion, eviction of the worst,
    // replacement and the "list full and worst <= s" skip are bit operations.
    // Children are visited in index order and the path hash is walked in
    // shared memory exactly as sdm_check_path does, stale links included.
    int cnt = 0;
    long long Lk = LLONG_MAX;
    int Ls = -1;
    if (!fast_ok || P.mode == kModeVerify) {
      sm.pos[si0] = (int8_t)(2 * lane);
      sm.pos[si1] = (int8_t)(2 * lane + 1);
      sm.idx_at[2 * lane] = (int8_t)si0;
      sm.idx_at[2 * lane + 1] = (int8_t)si1;
      if (P.mode == kModeVerify && live) { sm.hashmark[2 * lane] = 0; sm.hashmark[2 * lane + 1] = 0; }
      __syncwarp(hm);
      const int nch = 2 * n;
      unsigned long long Lm = 0ull;   // the act list, as sorted positions
      unsigned el = elig;
      while (el) {
        const int p = __ffs(el) - 1;
        el &= el - 1;
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int c = 2 * p + h;
          const int ps = sm.pos[c];
          const long long sk = sm.key[nb][c];
          const unsigned long long sp = sm.path[nb][c];
          if (cnt == K && (63 - __clzll((long long)Lm)) < ps) continue;
          const int b = (int)(sp & (kBuckets - 1));
          int t = sm.heads[b];
          int hops = 0;
          const int hop_limit = P.hop_limit > 0 ? P.hop_limit : 4 * kSlots;
          while (t >= 0) {
            if (sm.path[nb][t] == sp) break;
            t = sm.link[nb][t];
            if (++hops > hop_limit) { err = kStatusChainLimit; t = -1; break; }
          }
          if (t < 0) {
            __syncwarp(hm);
            if (lane == 0) {
              sm.link[nb][c] = sm.heads[b];
              sm.heads[b] = (int8_t)c;
              sm.hashmark[c] = 1;
            }
            __syncwarp(hm);
            if (cnt == K) {
              const int wp = 63 - __clzll((long long)Lm);
              if (K == kMaxCands && nb == 1) {
                // the store to act[32] hits path_hash[0] in the reference layout
                if (lane == 0) sm.heads[0] = sm.idx_at[wp];
                __syncwarp(hm);
              }
              Lm = (Lm & ~(1ull << wp)) | (1ull << ps);
            } else {
              Lm |= 1ull << ps;
              cnt++;
            }
            continue;
          }
          if (sm.key[nb][t] <= sk) continue;
          const bool t_in = t < nch && ((Lm >> sm.pos[t]) & 1ull);
          if (t_in) {
            Lm = (Lm & ~(1ull << sm.pos[t])) | (1ull << ps);      // replace t by s
          } else if (cnt == K) {
            Lm = (Lm & ~(1ull << (63 - __clzll((long long)Lm)))) | (1ull << ps);
          } else {
            Lm |= 1ull << ps;
            cnt++;
          }
        }
      }
      // act[rank] = the child at the rank-th set position
      const unsigned long long lowA = (1ull << (2 * lane)) - 1ull;
      if ((Lm >> (2 * lane)) & 1ull) sm.act[__popcll(Lm & lowA)] = (int8_t)si0;
      if ((Lm >> (2 * lane + 1)) & 1ull) sm.act[__popcll(Lm & (lowA | (1ull << (2 * lane))))] = (int8_t)si1;
      __syncwarp(hm);
      if (lane < cnt) {
        Ls = sm.act[lane];
        Lk = sm.key[nb][Ls];
      }
      __syncwarp(hm);
    }

    if (fast_ok) {
      if (P.mode == kModeVerify) {
        bool bad = (cnt != f_cnt) || (lane < cnt && (Ls != f_Ls || Lk != f_Lk));
        if (links_matter) {
          if (live && (sm.hashmark[2 * lane] != 0) != f_h0) bad = true;
          if (live && (sm.hashmark[2 * lane + 1] != 0) != f_h1) bad = true;
          if (f_h0 && sm.link[nb][2 * lane] != f_link0) bad = true;
          if (f_h1 && sm.link[nb][2 * lane + 1] != f_link1) bad = true;
        }
        if (__any_sync(hm, bad)) err = max(err, (int)kStatusVerifyMismatch);
      } else {
        cnt = f_cnt;
        Ls = f_Ls;
        Lk = f_Lk;
        if (links_matter) {
          if (f_h0) sm.link[nb][2 * lane] = (int8_t)f_link0;
          if (f_h1) sm.link[nb][2 * lane + 1] = (int8_t)f_link1;
        }
        __syncwarp(hm);
      }
    }

    // ---- 3. commit ----
    const int n_old = n;
    const int n_new = cnt;
    const double min_cost = __longlong_as_double(__shfl_sync(hm, Lk, 0, LPJ));
    const bool surv = lane < n_new;
    const int pp = surv ? (Ls >> 1) : lane;
    const int hh = surv ? (Ls & 1) : 0;
    const double f00 = __shfl_sync(hm, s00, pp, LPJ);
    const double f01 = __shfl_sync(hm, s01, pp, LPJ);
    const double fS1 = __shfl_sync(hm, S[1], pp, LPJ);
    Pack<N> fp;
    fp.G0 = __shfl_sync(hm, npk.G0, pp, LPJ);
    if (N >= 3) fp.G1 = __shfl_sync(hm, npk.G1, pp, LPJ);
#pragma unroll
    for (int i = 2; i < N; i++) {
      fp.D[i] = __shfl_sync(hm, npk.D[i], pp, LPJ);
      fp.A[i] = __shfl_sync(hm, npk.A[i], pp, LPJ);
    }
    const bool last = (t == n_in - 1);
    double fs[N];
    if (last) {
      // the full child state is only needed when the context is stored
#pragma unroll
      for (int i = 2; i < N; i++) fs[i] = __shfl_sync(hm, S[i], pp, LPJ);
    }
    const unsigned long long npath = shfl64<LPJ>(q, pp, hm) | (unsigned long long)hh;
    const int nnext = __shfl_sync(hm, new_next, pp, LPJ);
    uint32_t nring[RW];
#pragma unroll
    for (int w = 0; w < RW; w++)
      nring[w] = (w < W) ? __shfl_sync(hm, ring[w], pp, LPJ) : 0u;
    if (surv) {
      cs0 = hh ? f01 : f00;
      cs1 = fS1;
      pk.G0 = fp.G0;
      if (N >= 3) pk.G1 = fp.G1;
#pragma unroll
      for (int i = 2; i < N; i++) { pk.D[i] = fp.D[i]; pk.A[i] = fp.A[i]; }
      if (last) {
        // the child state, stored now so no register holds it through the loop
        dst->s[lane][0] = cs0;
        dst->s[lane][1] = cs1;
#pragma unroll
        for (int i = 2; i < N; i++) dst->s[lane][i] = fs[i];
      }
      cost = __dsub_rn(__longlong_as_double(Lk), min_cost);
      path = npath;
      nxt = nnext;
      slot = Ls;
#pragma unroll
      for (int w = 0; w < RW; w++) {
        uint32_t v = reg_word<RW>(nring[w]);
        if (w == (pos >> 5)) v = (v & ~(1u << (pos & 31))) | ((uint32_t)hh << (pos & 31));
        ring[w] = v;
      }
      sm.key[nb][Ls] = key_of(cost);
    }
    __syncwarp(hm);
    if (n_new < n_old) { c_conv++; c_coll++; }
    n = n_new;
    bank = nb;
    pos = next_pos;

    // ---- output ----
    if (t >= job.skip_out) {
      const long long o = t - job.skip_out;
      const int ol = (int)(o & (LPJ - 1));
      if (lane == ol) obit = (uint8_t)want;
      if (ol == LPJ - 1 || t == n_in - 1) {
        if (lane <= ol) job.out[o - ol + lane] = obit;
      }
    }
  }

  // ---- store the context (the states were stored at the last sample) ----
  if (job.flags & kJobNoStore) {
    err = __reduce_max_sync(hm, err);
    if (err && lane == 0) atomicMax(status, err);
    return;
  }
  if (lane < n) {
    dst->cost[lane] = cost;
    dst->path[lane] = path;
    dst->next[lane] = (uint8_t)nxt;
    dst->slot[lane] = (uint8_t)slot;
#pragma unroll
    for (int w = 0; w < RW; w++)
      if (w < W) dst->ring[lane][w] = ring[w];
  }
  __syncwarp(hm);
  for (int i = lane; i < 2 * S; i += LPJ) {
    const int b = i / S, j = i % S;
    dst->spath[b][j] = sm.path[b][j];
    dst->skey[b][j] = (unsigned long long)sm.key[b][j];
    dst->slink[b][j] = sm.link[b][j];
  }
  if (lane == 0) {
    dst->n = n;
    dst->bank = bank;
    dst->pos = pos;
    dst->conv_fail = c_conv;
    dst->cands_collapse = c_coll;
    dst->next_filter_drops = c_drop;
    dst->total_children = c_tot;
  }
  err = __reduce_max_sync(hm, err);
  if (err && lane == 0) atomicMax(status, err);
}

template <int N, int LPJ>
__global__ void __launch_bounds__(32, LPJ == 32 ? 13 : 10)
sdm_jobs_kernel(SdmParams P, const SdmJob* __restrict__ jobs, int njobs,
                int* __restrict__ job_counter, SdmCtx* __restrict__ ctxs,
                int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char sdm_smem_raw[];
  const int wl = threadIdx.x & 31;
  const int lane = wl & (LPJ - 1);
  const unsigned hm = job_mask<LPJ>(wl - lane);
  WarpSmem<LPJ>& sm =
      reinterpret_cast<WarpSmem<LPJ>*>(sdm_smem_raw)[(threadIdx.x >> 5) * (32 / LPJ) + wl / LPJ];
  for (;;) {
    int j = 0;
    if (lane == 0) j = atomicAdd(job_counter, 1);
    j = __shfl_sync(hm, j, 0, LPJ);
    if (j >= njobs) break;
    const SdmJob job = jobs[j];
    run_job<N, LPJ, kRegRingWords>(P, job, ctxs, sm, status);
    __syncwarp(hm);
  }
}

// Traceback latencies above 256 (the reference allows up to 2048,
// include/trellis.h:13): the whole 2048-bit ring in registers, one job per
// warp; 8 CTAs per SM leave 255 registers a thread.
template <int N>
__global__ void __launch_bounds__(32, 8)
sdm_jobs_wide_kernel(SdmParams P, const SdmJob* __restrict__ jobs, int njobs,
                     int* __restrict__ job_counter, SdmCtx* __restrict__ ctxs,
                     int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char sdm_smem_raw[];
  WarpSmem<32>& sm = reinterpret_cast<WarpSmem<32>*>(sdm_smem_raw)[0];
  for (;;) {
    int j = 0;
    if ((threadIdx.x & 31) == 0) j = atomicAdd(job_counter, 1);
    j = __shfl_sync(kFull, j, 0);
    if (j >= njobs) break;
    const SdmJob job = jobs[j];
    run_job<N, 32, kRingWords>(P, job, ctxs, sm, status);
    __syncwarp();
  }
}

// The kernel (with its template arguments) of this host thread's last SDM
// launch, for callers that report what ran.
static thread_local char g_last_kernel[64] = "";

const char* sdm_last_kernel() { return g_last_kernel; }

static void note_kernel(const char* name, int a, int b = -1, int c = -1) {
  if (c >= 0) snprintf(g_last_kernel, sizeof g_last_kernel, "%s<%d,%d,%d>", name, a, b, c);
  else if (b >= 0) snprintf(g_last_kernel, sizeof g_last_kernel, "%s<%d,%d>", name, a, b);
  else snprintf(g_last_kernel, sizeof g_last_kernel, "%s<%d>", name, a);
}

// ---- balanced launches: jobs cut into parts, parts queued ----
// One job per warp pins a job to one SM sub-partition, and every FP64 warp
// instruction of the warps there shares its FP64 pipe.  1,874 DAS segments
// over 152 SMs put 4 warps on 50 sub-partitions and 3 on the rest, and the
// launch lasts as long as the slowest 4-warp pipe (measured: 1,824 jobs, 3 per
// sub-partition, ran at 0.86 of the FP64 rate, 1,874 at 0.79).  A balanced
// launch holds exactly w warps per sub-partition, cuts every job into parts
// of part_len samples, and queues the parts: a warp that finishes part p of
// job j stores the context (as a streamed block boundary does), publishes
// part p + 1 at the queue's tail, and takes the next entry at its head, so
// the jobs move between warps and every pipe stays loaded to the end.
// Queue layout: [0] head, [1] tail, [2 ..] entries (part << 32 | job; empty
// ~0).  A wait for an entry that is not yet published is bounded.
constexpr long long kPartWaitCycles = 8000000000ll;   // ~4 s at 2 GHz

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// The rare wait for an entry not yet published (out of line: inlined, its
// loop changes the register allocation of the step loop).
__device__ __noinline__ unsigned long long wait_entry(const unsigned long long* p, int* status,
                                                     long long limit) {
  unsigned long long e = ~0ull;
  const long long t0 = clock64();
  if (limit <= 0) limit = kPartWaitCycles;
  do {
    __nanosleep(1000);
    e = ld_acquire_u64(p);
  } while (e == ~0ull && clock64() - t0 < limit);
  if (e == ~0ull && (threadIdx.x & 31) == 0) atomicMax(status, kStatusQueueWait);
  return e;
}

template <int N>
__global__ void __launch_bounds__(32, 13)
sdm_parts_kernel(SdmParams P, const SdmJob* __restrict__ jobs, long long part_len,
                 unsigned long long* __restrict__ queue, long long total,
                 SdmCtx* __restrict__ ctxs, int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char sdm_smem_raw[];
  WarpSmem<32>& sm = reinterpret_cast<WarpSmem<32>*>(sdm_smem_raw)[0];
  const int lane = threadIdx.x & 31;
  unsigned long long* head = queue;
  unsigned long long* tail = queue + 1;
  unsigned long long* ent = queue + 2;
  for (;;) {
    unsigned long long idx = 0;
    if (lane == 0) idx = atomicAdd(head, 1ull);
    idx = __shfl_sync(kFull, idx, 0);
    if (idx >= (unsigned long long)total) break;
    // every lane reads the entry with acquire semantics (one transaction)
    unsigned long long e = ld_acquire_u64(ent + idx);
    if (e == ~0ull) e = wait_entry(ent + idx, status, P.part_wait_cycles);
    if (e == ~0ull) break;
    __threadfence();   // the previous part's context is read after the entry
    const int j = (int)(e & 0xffffffffull);
    const long long p = (long long)(e >> 32);
    const SdmJob jb = jobs[j];
    const long long off = p * part_len;
    const long long rem = jb.n_in - off;
    SdmJob pj = jb;
    pj.n_in = rem < part_len ? rem : part_len;
    if (jb.in) pj.in = jb.in + off;
    const long long sk = jb.skip_out - off;
    pj.skip_out = sk <= 0 ? 0 : (sk < pj.n_in ? sk : pj.n_in);
    pj.out = jb.out + (off > jb.skip_out ? off - jb.skip_out : 0);
    if (p > 0) {
      // later parts continue from the job's own context
      pj.copy_from = -1;
      pj.seed_state = nullptr;
    }
    const bool more = off + pj.n_in < jb.n_in;
    run_job<N, 32, kRegRingWords>(P, pj, ctxs, sm, status);
    __threadfence();   // this part's context and decisions before its successor's entry
    __syncwarp();
    if (lane == 0 && more) {
      const unsigned long long t = atomicAdd(tail, 1ull);
      atomicExch(ent + t, ((unsigned long long)(p + 1) << 32) | (unsigned long long)(unsigned)j);
    }
    __syncwarp();
  }
}

__global__ void parts_queue_init_kernel(unsigned long long* queue, long long total, int njobs) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    queue[0] = 0ull;
    queue[1] = (unsigned long long)njobs;
  }
  if (i < total) queue[2 + i] = i < njobs ? (unsigned long long)i : ~0ull;
}

// Warps per sub-partition of a balanced launch of these jobs on `sms` SMs, or
// 0 when the plain launch is kept: K > 16 (a whole warp per job), no width
// or block cap requested, every job on its own context with its state kept,
// and the jobs only slightly above a whole number of warps per pipe (the
// parts of the extra jobs are shared out; a plain launch would give those
// pipes one warp more than the rest for the whole launch).
int sdm_balanced_warps(const SdmParams& P, const SdmJob* jobs, int njobs, int sms,
                       long long part_len) {
  if (P.lanes != 0 || lanes_per_job(P) != 32 || P.lat > 32 * kRegRingWords || sms <= 0) return 0;
  const long long pipes = 4ll * sms;
  if (njobs <= pipes) return 0;
  const long long w = (njobs + pipes - 1) / pipes;   // warps per pipe of the plain launch
  if (w < 2 || w > 4 || njobs % pipes == 0) return 0;
  if ((double)njobs > 1.10 * (double)((w - 1) * pipes)) return 0;
  long long samples = 0;
  for (int i = 0; i < njobs; i++) {
    if (jobs[i].ctx < 0 || (jobs[i].flags & kJobNoStore)) return 0;
    samples += jobs[i].n_in;
  }
  if (samples < 8 * part_len * (long long)njobs) return 0;   // parts too coarse to share out
  return (int)(w - 1);
}

long long sdm_parts_total(const SdmJob* jobs, int njobs, long long part_len) {
  long long total = 0;
  for (int i = 0; i < njobs; i++)
    total += jobs[i].n_in > 0 ? (jobs[i].n_in + part_len - 1) / part_len : 1;
  return total;
}

int launch_sdm_parts(const SdmParams& P, const SdmJob* d_jobs, int njobs, long long part_len,
                     unsigned long long* d_queue, long long total, int warps_per_pipe, int sms,
                     SdmCtx* d_ctxs, int* d_status, cudaStream_t stream) {
  parts_queue_init_kernel<<<(unsigned)((total + 255) / 256), 256, 0, stream>>>(d_queue, total, njobs);
  note_kernel("sdm_parts_kernel", P.order);
  const dim3 grid((unsigned)(4 * warps_per_pipe * sms));
  const size_t smem = sizeof(WarpSmem<32>);
  switch (P.order) {
#define DSD_CASE(NN)                                                                        \
  case NN:                                                                                  \
    sdm_parts_kernel<NN><<<grid, 32, smem, stream>>>(P, d_jobs, part_len, d_queue, total,   \
                                                     d_ctxs, d_status);                     \
    break;
    DSD_CASE(2) DSD_CASE(3) DSD_CASE(4) DSD_CASE(5) DSD_CASE(6)
    DSD_CASE(7) DSD_CASE(8) DSD_CASE(9) DSD_CASE(10)
#undef DSD_CASE
    default: return -1;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int sdm_jobs_per_cta(const SdmParams& P) { return 32 / lanes_per_job(P); }

static int launch_wide(const SdmParams& P, dim3 grid, const SdmJob* d_jobs, int njobs,
                       int* d_counter, SdmCtx* d_ctxs, int* d_status, cudaStream_t stream) {
  const size_t smem = sizeof(WarpSmem<32>);
  switch (P.order) {
#define DSD_CASE(NN)                                                                          \
  case NN:                                                                                    \
    sdm_jobs_wide_kernel<NN><<<grid, 32, smem, stream>>>(P, d_jobs, njobs, d_counter, d_ctxs, \
                                                         d_status);                           \
    break;
    DSD_CASE(2) DSD_CASE(3) DSD_CASE(4) DSD_CASE(5) DSD_CASE(6)
    DSD_CASE(7) DSD_CASE(8) DSD_CASE(9) DSD_CASE(10)
#undef DSD_CASE
    default: return -1;
  }
  return 0;
}

template <int LPJ>
static int launch_lpj(const SdmParams& P, dim3 grid, const SdmJob* d_jobs, int njobs,
                      int* d_counter, SdmCtx* d_ctxs, int* d_status, cudaStream_t stream) {
  const size_t smem = sizeof(WarpSmem<LPJ>) * (size_t)(32 / LPJ);
  switch (P.order) {
#define DSD_CASE(NN)                                                                       \
  case NN:                                                                                 \
    sdm_jobs_kernel<NN, LPJ><<<grid, 32, smem, stream>>>(P, d_jobs, njobs, d_counter, d_ctxs, \
                                                         d_status);                        \
    break;
    DSD_CASE(2) DSD_CASE(3) DSD_CASE(4) DSD_CASE(5) DSD_CASE(6)
    DSD_CASE(7) DSD_CASE(8) DSD_CASE(9) DSD_CASE(10)
#undef DSD_CASE
    default: return -1;
  }
  return 0;
}

bool sdm_scalar_eligible(const SdmParams& P, int max_blocks);   // sdm_scalar.cu
int launch_sdm_scalar(const SdmParams& P, const SdmJob* d_jobs, int njobs, SdmCtx* d_ctxs,
                      cudaStream_t stream);
int sdm_split_jobs_per_warp(const SdmParams& P);                 // sdm_split.cu
bool sdm_split_supported(const SdmParams& P);
int launch_sdm_split(const SdmParams& P, const SdmJob* d_jobs, int njobs, SdmCtx* d_ctxs,
                     cudaStream_t stream);

// Host-side launcher: each warp-sized CTA runs 32 / LPJ jobs side by side
// (lanes_per_job); max_blocks caps the CTAs.  Uncapped launches of small
// trellises take their own kernels: while the jobs fit in two warps per
// scheduler, each candidate's NTF advance spread over lanes (sdm_split.cu,
// K <= 2, or K <= 4 up to order 8: the shortest step); beyond that, at
// K <= 2, one job per thread (sdm_scalar.cu, the fewest FP64 instructions per
// job).
int launch_sdm_jobs(const SdmParams& P, const SdmJob* d_jobs, int njobs, int* d_counter,
                    SdmCtx* d_ctxs, int* d_status, int max_blocks, cudaStream_t stream) {
  if (njobs <= 0) return 0;
  if (P.lanes == 0 && max_blocks == 0 && P.lat <= 32 * kRegRingWords) {
    const long long split_cap = (long long)sdm_split_jobs_per_warp(P) * 2 * 4 * (resident_warps() / 16);
    if (sdm_split_supported(P) && njobs <= split_cap) {
      if (P.order <= 8) note_kernel("sdm_split_kernel", P.order, 8, P.cands <= 2 ? 2 : 4);
      else note_kernel("sdm_split_kernel", P.order, 16, 2);
      return launch_sdm_split(P, d_jobs, njobs, d_ctxs, stream);
    }
    if (sdm_scalar_eligible(P, max_blocks)) {
      note_kernel("sdm_scalar_kernel", P.order);
      return launch_sdm_scalar(P, d_jobs, njobs, d_ctxs, stream);
    }
  }
  const int lanes = launch_lanes(P, njobs, max_blocks);
  const int jpc = 32 / lanes;
  int blocks = (njobs + jpc - 1) / jpc;
  if (max_blocks > 0 && blocks > max_blocks) blocks = max_blocks;
  cudaMemsetAsync(d_counter, 0, sizeof(int), stream);
  const dim3 grid(blocks);
  int rc = -1;
  if (P.lat > 32 * kRegRingWords) {
    note_kernel("sdm_jobs_wide_kernel", P.order);
    rc = launch_wide(P, grid, d_jobs, njobs, d_counter, d_ctxs, d_status, stream);
    if (rc) return rc;
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
  }
  note_kernel("sdm_jobs_kernel", P.order, lanes);
  switch (lanes) {
    case 32: rc = launch_lpj<32>(P, grid, d_jobs, njobs, d_counter, d_ctxs, d_status, stream); break;
    case 16: rc = launch_lpj<16>(P, grid, d_jobs, njobs, d_counter, d_ctxs, d_status, stream); break;
    case 8: rc = launch_lpj<8>(P, grid, d_jobs, njobs, d_counter, d_ctxs, d_status, stream); break;
    case 4: rc = launch_lpj<4>(P, grid, d_jobs, njobs, d_counter, d_ctxs, d_status, stream); break;
    default: rc = launch_lpj<2>(P, grid, d_jobs, njobs, d_counter, d_ctxs, d_status, stream); break;
  }
  if (rc) return rc;
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}


}  // namespace dsdgpu
