// Trellis SDM for K <= 4 with each candidate's NTF advance split over lanes
// (K <= 2: the engine's path-table default; K = 4: its default for paths the
// table does not list, include/dsd_types.h:479-481).
//
// An FP64 instruction occupies this part's FP64 unit for ~64 cycles per warp,
// dependent or not and whatever the number of active lanes, so the latency of
// one trellis step is its count of FP64 instructions.  With one candidate per
// lane (sdm_trellis.cu) or one job per lane (sdm_scalar.cu) a step issues all
// 5N + 6 (or twice that) operations one after another.  Here a candidate
// spans H lanes, lane q owning state component q, and every operation that
// does not depend on another component runs once for all q:
//
//   m = g_q s_{q+1};  u = s_q + (q == 0 ? -m : s_{q-1});
//   d_q = u + (q == 0 ? x : q < N-1 ? -m : -0.0);   p_q = a_q d_q
//
// which are exactly the reference's operations in its order ((s0 - g0 s1) + x,
// (s_q + s_{q-1}) - g_q s_{q+1}, s_{N-1} + s_{N-2}; adding -m is subtracting m,
// adding -0.0 leaves any value unchanged).  Only v = ((x + p_0) + p_1) + ...
// stays serial (N adds, the products gathered by shuffles).  A step is then
// about N + 9 FP64 instructions instead of 5N + 6.  Lanes q and q+1 of a
// candidate form its two children's costs; the selection of at most 8
// children runs redundantly in every lane of the job (the act list in KC
// registers, the dedup hash a scan of the children hashed this sample); the
// survivors pull state components, ring words and bits from their parent's
// lanes.  Reference: src/trellis.c:868-973 (step), :621-731 (selection).
//
// Layout: a job is G = KC H lanes (KC = 2 candidate slots for K <= 2, 4 for
// K <= 4; H = 8 for N <= 8, 16 above), 32 / G jobs per warp; candidate c owns
// lanes [c H, c H + H), lane q < N holds s_q, lane
// q < W ring word q; cost, path and next are held by every lane of the
// candidate.  The context format is SdmCtx's, as for the other kernels.
#include "sdm_internal.h"

namespace dsdgpu {

namespace {

// element i of a register array, without dynamic indexing (which would put
// the array in local memory)
template <typename T, int M>
__device__ __forceinline__ T pickn(const T (&a)[M], int i) {
  T r = a[0];
#pragma unroll
  for (int j = 1; j < M; j++)
    if (i == j) r = a[j];
  return r;
}

template <int N, int H, int KC>
__global__ void __launch_bounds__(32) sdm_split_kernel(SdmParams P, const SdmJob* __restrict__ jobs,
                                                      int njobs, SdmCtx* __restrict__ ctxs) {
  constexpr int G = KC * H;        // KC candidate slots of H lanes
  constexpr int NC = 2 * KC;       // children
  const int wl = threadIdx.x & 31;
  const int jl = wl & (G - 1);                 // lane within the job
  const unsigned sh = (unsigned)(wl - jl);
  const unsigned hm = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << sh);
  const int cand = jl / H, q = jl % H;
  const int jid = (int)((blockIdx.x * 32 + wl) / G);
  if (jid >= njobs) return;                    // whole jobs leave together
  const SdmJob job = jobs[jid];
  const SdmCtx* src = &ctxs[job.copy_from >= 0 ? job.copy_from : job.ctx];
  SdmCtx* dst = &ctxs[job.ctx];
  const int K = P.cands;
  const int W = (P.lat + 31) >> 5;
  const unsigned long long mask = P.mask;
  const bool lim_on = P.state_limit > 0.0;
  const double lim = P.state_limit;
  // this lane's coefficients (distinct per lane: held in registers)
  double gq = 0.0, aq = 0.0;
#pragma unroll
  for (int k = 0; k < N; k++)
    if (k == q) { gq = P.g[k]; aq = P.a[k]; }
  const double a0 = P.a[0];

  int n = src->n, bank = src->bank, pos = src->pos;
  double sq = 0.0, cost = 0.0;
  unsigned long long path = 0;
  int next = 0;
  uint32_t ringw = 0;
  if (cand < n) {
    if (q < N) sq = src->s[cand][q];
    cost = src->cost[cand];
    path = src->path[cand];
    next = src->next[cand];
    if (q < W) ringw = src->ring[cand][q];
    if (job.seed_state) {
      // DAS temp seeding: every live candidate gets the estimated state, cost 0
      if (q < N) sq = job.seed_state[q];
      cost = 0.0;
    }
  }
  unsigned long long c_conv = 0, c_coll = 0, c_drop = 0, c_tot = 0;
  if (job.copy_from < 0) {
    c_conv = src->conv_fail;
    c_coll = src->cands_collapse;
    c_drop = src->next_filter_drops;
    c_tot = src->total_children;
  }

  const long long n_in = job.n_in;
  const double* __restrict__ in = job.in;
  for (long long t = 0; t < n_in; t++) {
    const double x = in ? __ldg(in + t) : 0.0;
    int next_pos = pos + 1;
    if (next_pos == P.lat) next_pos = 0;

    // ---- NTF advance, one state component per lane ----
    const double s_prev = __shfl_up_sync(hm, sq, 1, H);
    const double s_next = __shfl_down_sync(hm, sq, 1, H);
    const double m = __dmul_rn(gq, s_next);
    const double u = __dadd_rn(sq, q == 0 ? -m : s_prev);
    const double d = __dadd_rn(u, q == 0 ? x : (q < N - 1 ? -m : -0.0));
    const double p = __dmul_rn(aq, d);
    double pj[N];
#pragma unroll
    for (int j = 0; j < N; j++) pj[j] = __shfl_sync(hm, p, cand * H + j, G);
    double v = __dadd_rn(x, pj[0]);
#pragma unroll
    for (int j = 1; j < N; j++) v = __dadd_rn(v, pj[j]);
    // lanes q = 0 / 1 of a candidate: its children with bit 0 / 1
    const double e = __dadd_rn(v, (q & 1) ? -a0 : a0);
    const double kc = __dadd_rn(cost, __dmul_rn(e, e));
    // the parent's traceback bit at next_pos
    const uint32_t wn = __shfl_sync(hm, ringw, cand * H + (next_pos >> 5), G);
    const int newnext = (int)((wn >> (next_pos & 31)) & 1u);

    // ---- selection over the children, in every lane of the job ----
    double ccost[NC];
    long long ckeyv[NC];
    int cnext[NC];
    unsigned long long cpath[NC];
    int nnext[KC];
#pragma unroll
    for (int ch = 0; ch < NC; ch++) ccost[ch] = __shfl_sync(hm, kc, (ch >> 1) * H + (ch & 1), G);
#pragma unroll
    for (int c = 0; c < KC; c++) {
      const int nx = __shfl_sync(hm, next, c * H, G);
      const unsigned long long pth =
          (unsigned long long)__shfl_sync(hm, (long long)path, c * H, G);
      nnext[c] = __shfl_sync(hm, newnext, c * H, G);
#pragma unroll
      for (int b = 0; b < 2; b++) {
        cnext[2 * c + b] = nx;
        cpath[2 * c + b] = ((pth << 1) | (unsigned long long)b) & mask;
      }
    }
#pragma unroll
    for (int ch = 0; ch < NC; ch++) ckeyv[ch] = __double_as_longlong(ccost[ch]);
    const int nchild = 2 * n;
    c_tot += (unsigned long long)nchild;
    int mn = 0, votes1 = 0;
#pragma unroll
    for (int ch = 0; ch < NC; ch++)
      if (ch < nchild) {
        if (ckeyv[ch] < pickn(ckeyv, mn)) mn = ch;
        votes1 += cnext[ch] & 1;
      }
    const int majority = (votes1 > nchild - votes1) ? 1 : 0;
    if (pickn(cnext, mn) != majority) {
      int bm = -1;
#pragma unroll
      for (int ch = 0; ch < NC; ch++)
        if (ch < nchild && cnext[ch] == majority && (bm < 0 || ckeyv[ch] < pickn(ckeyv, bm)))
          bm = ch;
      if (bm >= 0 && pickn(ccost, bm) < __dmul_rn(pickn(ccost, mn), 1.1)) mn = bm;
    }
    const int want = pickn(cnext, mn);
    // the act list: na child indices sorted by cost key, equal keys in
    // insertion order; inserting after every entry with key <= ks is the
    // reference's backwards shift, and a full list (K) drops its last entry
    int act[KC];
#pragma unroll
    for (int i = 0; i < KC; i++) act[i] = 0;
    int na = 0;
    unsigned hashed = 0;
#pragma unroll
    for (int ch = 0; ch < NC; ch++) {
      if (ch >= nchild) continue;
      if (cnext[ch] != want) { c_drop++; continue; }
      const long long ks = ckeyv[ch];
      if (na == K && pickn(ckeyv, pickn(act, na - 1)) <= ks) continue;
      int tfound = -1;
#pragma unroll
      for (int h = 0; h < ch; h++)
        if (((hashed >> h) & 1u) && cpath[h] == cpath[ch]) tfound = h;
      if (tfound < 0) {
        hashed |= 1u << ch;
      } else {
        if (pickn(ckeyv, tfound) <= ks) continue;
        // t still in the act list: take it out
        int tp = KC;
#pragma unroll
        for (int i = KC - 1; i >= 0; i--)
          if (i < na && act[i] == tfound) tp = i;
        if (tp < KC) {
#pragma unroll
          for (int i = 0; i < KC - 1; i++)
            if (i >= tp) act[i] = act[i + 1];
          na--;
        }
      }
      int jpos = 0;   // entries with key <= ks (a prefix: the list is sorted)
#pragma unroll
      for (int i = 0; i < KC; i++)
        if (i < na && pickn(ckeyv, act[i]) <= ks) jpos++;
      if (jpos < K) {
#pragma unroll
        for (int i = KC - 1; i >= 1; i--)
          if (i > jpos) act[i] = act[i - 1];
#pragma unroll
        for (int i = 0; i < KC; i++)
          if (i == jpos) act[i] = ch;
      }
      if (na < K) na++;
    }
    const int n_new = na;

    // ---- commit: the lanes of candidate slot `cand` take survivor `cand` ----
    const double min_cost = pickn(ccost, act[0]);
    const bool live = cand < n_new;
    const int ch = pickn(act, cand);
    const int par = live ? (ch >> 1) : 0;
    const int b = live ? (ch & 1) : 0;
    const double dpar = __shfl_sync(hm, d, par * H + q, G);
    const uint32_t rpar = __shfl_sync(hm, ringw, par * H + q, G);
    double snew = q == 0 ? __dadd_rn(dpar, b ? -1.0 : 1.0) : dpar;
    if (lim_on) snew = clamp_state(snew, lim);
    sq = q < N ? snew : 0.0;
    cost = live ? __dsub_rn(pickn(ccost, ch), min_cost) : 0.0;
    path = live ? pickn(cpath, ch) : 0ull;
    next = pickn(nnext, par);
    ringw = (q == (pos >> 5)) ? ((rpar & ~(1u << (pos & 31))) | ((uint32_t)b << (pos & 31))) : rpar;
    if (n_new < n) { c_conv++; c_coll++; }
    n = n_new;
    bank ^= 1;
    pos = next_pos;
    if (jl == 0 && t >= job.skip_out) job.out[t - job.skip_out] = (uint8_t)want;
  }

  if (job.flags & kJobNoStore) return;
  if (cand < n) {
    if (q < N) dst->s[cand][q] = sq;
    if (q < W) dst->ring[cand][q] = ringw;
    if (q == 0) {
      dst->cost[cand] = cost;
      dst->path[cand] = path;
      dst->next[cand] = (uint8_t)next;
      dst->slot[cand] = (uint8_t)cand;
    }
  }
  if (job.copy_from >= 0) {
    for (int i = jl; i < 2 * kSlots; i += G) {
      const int bk = i / kSlots, j = i % kSlots;
      dst->spath[bk][j] = src->spath[bk][j];
      dst->skey[bk][j] = src->skey[bk][j];
      dst->slink[bk][j] = src->slink[bk][j];
    }
  }
  if (jl == 0) {
    dst->n = n;
    dst->bank = bank;
    dst->pos = pos;
    dst->conv_fail = c_conv;
    dst->cands_collapse = c_coll;
    dst->next_filter_drops = c_drop;
    dst->total_children = c_tot;
  }
}

template <int H, int KC>
int launch_split(const SdmParams& P, const SdmJob* d_jobs, int njobs, SdmCtx* d_ctxs,
                 cudaStream_t stream) {
  const int jpw = 32 / (KC * H);
  const dim3 grid((njobs + jpw - 1) / jpw), block(32);
  switch (P.order) {
#define DSD_CASE(NN) \
  case NN: sdm_split_kernel<NN, H, KC><<<grid, block, 0, stream>>>(P, d_jobs, njobs, d_ctxs); break;
    DSD_CASE(2) DSD_CASE(3) DSD_CASE(4) DSD_CASE(5) DSD_CASE(6) DSD_CASE(7) DSD_CASE(8)
#undef DSD_CASE
    default: return -1;
  }
  return 0;
}

}  // namespace

// The split kernel takes K <= 2 at any order (2 slots of 8 lanes up to order
// 8, of 16 lanes above) and K = 3, 4 up to order 8 (4 slots of 8 lanes).
bool sdm_split_supported(const SdmParams& P) {
  return P.cands <= 2 || (P.cands <= 4 && P.order <= 8);
}

// Jobs per warp of the split kernel for these parameters.
int sdm_split_jobs_per_warp(const SdmParams& P) {
  return (P.cands <= 2 && P.order <= 8) ? 2 : 1;
}

int launch_sdm_split(const SdmParams& P, const SdmJob* d_jobs, int njobs, SdmCtx* d_ctxs,
                     cudaStream_t stream) {
  if (njobs <= 0) return 0;
  int rc = -1;
  if (P.cands <= 2 && P.order <= 8) {
    rc = launch_split<8, 2>(P, d_jobs, njobs, d_ctxs, stream);
  } else if (P.cands <= 4 && P.order <= 8) {
    rc = launch_split<8, 4>(P, d_jobs, njobs, d_ctxs, stream);
  } else if (P.cands <= 2) {
    const dim3 grid(njobs), block(32);
    switch (P.order) {
      case 9: sdm_split_kernel<9, 16, 2><<<grid, block, 0, stream>>>(P, d_jobs, njobs, d_ctxs); rc = 0; break;
      case 10: sdm_split_kernel<10, 16, 2><<<grid, block, 0, stream>>>(P, d_jobs, njobs, d_ctxs); rc = 0; break;
      default: rc = -1;
    }
  }
  if (rc) return rc;
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace dsdgpu
