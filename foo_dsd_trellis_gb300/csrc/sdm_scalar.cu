// Trellis SDM for K <= 2 candidates (the reference engine's path-table default,
// src/engine.c:60-75): one thread runs one job, 32 jobs per warp.
//
// On this part an FP64 warp instruction occupies the FP64 unit about as long
// with 2 active lanes as with 32, so a warp-cooperative job at K = 2 (the
// kernel in sdm_trellis.cu) spends a full warp instruction on every
// operation of 2 candidates, and its sort, ballots and shuffles sit on the
// per-sample critical path.  Here every lane carries its own job: each FP64
// instruction advances 32 jobs, and the selection of at most 4 children is a
// few predicated integer operations in registers.
//
// The step is the reference's (src/trellis.c:868-973; selection :621-731):
// expansion of every candidate into children 2i (bit 0, state[0] + 1) and
// 2i + 1 (bit 1, state[0] - 1) with the FP64 NTF advance in the reference's
// operation order (no contraction); argmin by the int64 reading of the cost
// bits (first index among equals); majority vote of the traceback bits with
// the 1.1x override; then the ordered insertion over the children in index
// order with path dedup.  With at most 4 children the dedup hash reduces to a
// scan of the children hashed so far this sample (a path is hashed at most
// once, so the match is unique), and the act list to two registers.  The
// context format is SdmCtx's (rank order), so jobs, DAS seeding and copies
// work as with the warp kernel; the slot memory is only read by the K = 32
// case and is left as loaded.
#include "sdm_internal.h"

namespace dsdgpu {

namespace {

constexpr int kScalarRingWords = 8;   // lat <= 256

__device__ __forceinline__ long long ckey(double c) { return __double_as_longlong(c); }

// element i of a 4-entry register array, without dynamic indexing (which
// would put the array in local memory)
template <typename T>
__device__ __forceinline__ T pick4(const T (&a)[4], int i) {
  return i == 0 ? a[0] : i == 1 ? a[1] : i == 2 ? a[2] : a[3];
}

template <int N>
struct Cand {
  double s[N];
  double cost;
  unsigned long long path;
  uint32_t ring[kScalarRingWords];
  int next;
};

template <int N>
__global__ void __launch_bounds__(32) sdm_scalar_kernel(SdmParams P, const SdmJob* __restrict__ jobs,
                                                       int njobs, SdmCtx* __restrict__ ctxs) {
  const int jid = blockIdx.x * blockDim.x + threadIdx.x;
  if (jid >= njobs) return;
  const SdmJob job = jobs[jid];
  const int dst_i = job.ctx >= 0 ? job.ctx : (-job.ctx - 1) + jid;
  const SdmCtx* src = &ctxs[job.copy_from >= 0 ? job.copy_from : dst_i];
  SdmCtx* dst = &ctxs[dst_i];
  const int K = P.cands;
  const int W = (P.lat + 31) >> 5;
  const unsigned long long mask = P.mask;
  const bool lim_on = P.state_limit > 0.0;
  const double lim = P.state_limit;

  int n = src->n, bank = src->bank, pos = src->pos;
  Cand<N> c[2];
#pragma unroll
  for (int i = 0; i < 2; i++) {
#pragma unroll
    for (int k = 0; k < N; k++) c[i].s[k] = 0.0;
    c[i].cost = 0.0;
    c[i].path = 0;
    c[i].next = 0;
#pragma unroll
    for (int w = 0; w < kScalarRingWords; w++) c[i].ring[w] = 0;
    if (i < n) {
#pragma unroll
      for (int k = 0; k < N; k++) c[i].s[k] = src->s[i][k];
      c[i].cost = src->cost[i];
      c[i].path = src->path[i];
      c[i].next = src->next[i];
#pragma unroll
      for (int w = 0; w < kScalarRingWords; w++)
        if (w < W) c[i].ring[w] = src->ring[i][w];
    }
  }
  unsigned long long c_conv = 0, c_coll = 0, c_drop = 0, c_tot = 0;
  if (job.copy_from < 0) {
    c_conv = src->conv_fail;
    c_coll = src->cands_collapse;
    c_drop = src->next_filter_drops;
    c_tot = src->total_children;
  }
  if (job.seed_state) {
    // DAS temp seeding: every live candidate gets the estimated state, cost 0
#pragma unroll
    for (int i = 0; i < 2; i++)
      if (i < n) {
#pragma unroll
        for (int k = 0; k < N; k++) c[i].s[k] = job.seed_state[k];
        c[i].cost = 0.0;
      }
  }

  const long long n_in = job.n_in;
  const double* __restrict__ in = job.in;
  // one input line (16 samples) per L1 miss; a step is thousands of cycles
  for (long long t = 0; t < n_in; t++) {
    {
      const double x = in ? __ldg(in + t) : 0.0;
      int next_pos = pos + 1;
      if (next_pos == P.lat) next_pos = 0;

      // ---- expansion: per parent the shared child state d, s0 of both
      // children, both child costs, and the parent's new traceback bit ----
      double d[2][N], s00[2], s01[2], k0c[2], k1c[2];
      int newnext[2];
#pragma unroll
      for (int i = 0; i < 2; i++) {
        const double (&s)[N] = c[i].s;
        d[i][0] = __dadd_rn(__dsub_rn(s[0], __dmul_rn(P.g[0], s[1])), x);
        double v = __dadd_rn(x, __dmul_rn(P.a[0], d[i][0]));
#pragma unroll
        for (int q = 1; q < N - 1; q++) {
          d[i][q] = __dsub_rn(__dadd_rn(s[q], s[q - 1]), __dmul_rn(P.g[q], s[q + 1]));
          v = __dadd_rn(v, __dmul_rn(P.a[q], d[i][q]));
        }
        d[i][N - 1] = __dadd_rn(s[N - 1], s[N - 2]);
        v = __dadd_rn(v, __dmul_rn(P.a[N - 1], d[i][N - 1]));
        s00[i] = __dadd_rn(d[i][0], 1.0);
        s01[i] = __dsub_rn(d[i][0], 1.0);
        if (lim_on) {
#pragma unroll
          for (int q = 1; q < N; q++) d[i][q] = clamp_state(d[i][q], lim);
          s00[i] = clamp_state(s00[i], lim);
          s01[i] = clamp_state(s01[i], lim);
        }
        const double e0 = __dadd_rn(v, P.a[0]);
        const double e1 = __dsub_rn(v, P.a[0]);
        k0c[i] = __dadd_rn(c[i].cost, __dmul_rn(e0, e0));
        k1c[i] = __dadd_rn(c[i].cost, __dmul_rn(e1, e1));
        uint32_t wv = 0;
#pragma unroll
        for (int w = 0; w < kScalarRingWords; w++)
          if (w == (next_pos >> 5)) wv = c[i].ring[w];
        newnext[i] = (int)((wv >> (next_pos & 31)) & 1u);
      }

      // ---- selection over children ch = 0 .. 2n-1 (parent ch >> 1) ----
      const int nchild = 2 * n;
      c_tot += (unsigned long long)nchild;
      // per child: cost, key, traceback bit (the parent's old next), path
      double ccost[4];
      long long ckeyv[4];
      int cnext[4];
      unsigned long long cpath[4];
#pragma unroll
      for (int ch = 0; ch < 4; ch++) {
        const int p = ch >> 1;
        ccost[ch] = (ch & 1) ? k1c[p] : k0c[p];
        ckeyv[ch] = ckey(ccost[ch]);
        cnext[ch] = c[p].next;
        cpath[ch] = ((c[p].path << 1) | (unsigned long long)(ch & 1)) & mask;
      }
      int mn = 0;
      int votes1 = 0;
#pragma unroll
      for (int ch = 0; ch < 4; ch++)
        if (ch < nchild) {
          if (ckeyv[ch] < pick4(ckeyv, mn)) mn = ch;
          votes1 += cnext[ch] & 1;
        }
      const int majority = (votes1 > nchild - votes1) ? 1 : 0;
      if (pick4(cnext, mn) != majority) {
        int bm = -1;
#pragma unroll
        for (int ch = 0; ch < 4; ch++)
          if (ch < nchild && cnext[ch] == majority && (bm < 0 || ckeyv[ch] < pick4(ckeyv, bm)))
            bm = ch;
        if (bm >= 0 && pick4(ccost, bm) < __dmul_rn(pick4(ccost, mn), 1.1)) mn = bm;
      }
      const int want = pick4(cnext, mn);
      // ordered insertion with dedup; act holds child indices, na entries
      int act0 = 0, act1 = 0, na = 0;
      unsigned hashed = 0;   // children inserted into the dedup hash this sample
#pragma unroll
      for (int ch = 0; ch < 4; ch++) {
        if (ch >= nchild) continue;
        if (cnext[ch] != want) { c_drop++; continue; }
        const long long ks = ckeyv[ch];
        if (na == K && pick4(ckeyv, na == 2 ? act1 : act0) <= ks) continue;
        int tfound = -1;
#pragma unroll
        for (int h = 0; h < ch; h++)
          if (((hashed >> h) & 1u) && cpath[h] == cpath[ch]) tfound = h;
        if (tfound < 0) {
          hashed |= 1u << ch;
        } else {
          if (pick4(ckeyv, tfound) <= ks) continue;
          // t still in the act list: take it out, then insert ch in order
          if (na >= 1 && act0 == tfound) { act0 = act1; na--; }
          else if (na == 2 && act1 == tfound) { na--; }
        }
        // insertion after every entry with key <= ks; a full list (K
        // entries) drops its worst entry
        if (na == 0) {
          act0 = ch;
        } else if (na == 1) {
          if (pick4(ckeyv, act0) <= ks) { if (K >= 2) act1 = ch; }
          else { if (K >= 2) act1 = act0; act0 = ch; }
        } else {
          if (pick4(ckeyv, act0) <= ks) act1 = ch;
          else { act1 = act0; act0 = ch; }
        }
        if (na < K) na++;
      }
      const int n_new = na;

      // ---- commit: survivors take their parent's state, ring and new
      // traceback bit; costs are normalised by the new minimum ----
      const double min_cost = pick4(ccost, act0);
      const int out_bit = want;
      Cand<N> nc[2];
#pragma unroll
      for (int r = 0; r < 2; r++) {
        const int ch = r == 0 ? act0 : act1;
        const bool live = r < n_new;
        const int p = live ? (ch >> 1) : 0;
        const int b = live ? (ch & 1) : 0;
#pragma unroll
        for (int q = 1; q < N; q++) nc[r].s[q] = p ? d[1][q] : d[0][q];
        nc[r].s[0] = b ? (p ? s01[1] : s01[0]) : (p ? s00[1] : s00[0]);
        nc[r].cost = live ? __dsub_rn(pick4(ccost, ch), min_cost) : 0.0;
        nc[r].path = live ? pick4(cpath, ch) : 0ull;
        nc[r].next = p ? newnext[1] : newnext[0];
#pragma unroll
        for (int w = 0; w < kScalarRingWords; w++) {
          uint32_t v = p ? c[1].ring[w] : c[0].ring[w];
          if (w == (pos >> 5)) v = (v & ~(1u << (pos & 31))) | ((uint32_t)b << (pos & 31));
          nc[r].ring[w] = v;
        }
      }
#pragma unroll
      for (int r = 0; r < 2; r++) c[r] = nc[r];
      if (n_new < n) { c_conv++; c_coll++; }
      n = n_new;
      bank ^= 1;
      pos = next_pos;

      if (t >= job.skip_out) job.out[t - job.skip_out] = (uint8_t)out_bit;
    }
  }

  if (job.flags & kJobNoStore) return;
#pragma unroll
  for (int i = 0; i < 2; i++)
    if (i < n) {
#pragma unroll
      for (int k = 0; k < N; k++) dst->s[i][k] = c[i].s[k];
      dst->cost[i] = c[i].cost;
      dst->path[i] = c[i].path;
      dst->next[i] = (uint8_t)c[i].next;
      dst->slot[i] = (uint8_t)i;
#pragma unroll
      for (int w = 0; w < kScalarRingWords; w++)
        if (w < W) dst->ring[i][w] = c[i].ring[w];
    }
  if (job.copy_from >= 0) {
    // the rest of the context (slot memory) follows the copy, as the warp
    // kernel's store does
    for (int i = 0; i < 2 * kSlots; i++) {
      const int b = i / kSlots, q = i % kSlots;
      dst->spath[b][q] = src->spath[b][q];
      dst->skey[b][q] = src->skey[b][q];
      dst->slink[b][q] = src->slink[b][q];
    }
  }
  dst->n = n;
  dst->bank = bank;
  dst->pos = pos;
  dst->conv_fail = c_conv;
  dst->cands_collapse = c_coll;
  dst->next_filter_drops = c_drop;
  dst->total_children = c_tot;
}

}  // namespace

bool sdm_scalar_eligible(const SdmParams& P, int max_blocks) {
  return P.cands <= 2 && P.lanes == 0 && max_blocks == 0 && P.lat <= 32 * kScalarRingWords;
}

int launch_sdm_scalar(const SdmParams& P, const SdmJob* d_jobs, int njobs, SdmCtx* d_ctxs,
                      cudaStream_t stream) {
  if (njobs <= 0) return 0;
  const dim3 grid((njobs + 31) / 32), block(32);
  switch (P.order) {
#define DSD_CASE(NN) \
  case NN: sdm_scalar_kernel<NN><<<grid, block, 0, stream>>>(P, d_jobs, njobs, d_ctxs); break;
    DSD_CASE(2) DSD_CASE(3) DSD_CASE(4) DSD_CASE(5) DSD_CASE(6)
    DSD_CASE(7) DSD_CASE(8) DSD_CASE(9) DSD_CASE(10)
#undef DSD_CASE
    default: return -1;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace dsdgpu
