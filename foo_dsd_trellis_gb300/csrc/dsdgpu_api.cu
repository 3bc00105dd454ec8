// C-ABI host layer of libdsdgpu (include/dsdgpu.h): context lifecycle and the
// trellis SDM entry points.  The FIR, DAS and packing entry points live in
// their own translation units and share the context defined in api_context.h.
#include "api_context.h"
#include "das_plan.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>

namespace dsdgpu {

int launch_sdm_jobs(const SdmParams& P, const SdmJob* d_jobs, int njobs, int* d_counter,
                    SdmCtx* d_ctxs, int* d_status, int max_blocks, cudaStream_t stream);

// (Re)initialise contexts [first, first + count) to the state sdm_context_init
// leaves (src/trellis.c:977-1011): one live candidate in slot 0 of bank 0,
// all state, cost, path and history zero, every hash-chain link empty.  With
// keep_counters, cands_collapse, next_filter_drops and total_children keep
// their values, as sdm_context_reset does (src/trellis.c:1189-1224).
__global__ void sdm_ctx_init_kernel(SdmCtx* ctxs, int first, int count, int keep_counters) {
  SdmCtx* c = &ctxs[first + blockIdx.x];
  if ((int)blockIdx.x >= count) return;
  const int t = threadIdx.x;
  double* s = &c->s[0][0];
  for (int i = t; i < kMaxCands * kMaxOrder; i += blockDim.x) s[i] = 0.0;
  uint32_t* r = &c->ring[0][0];
  for (int i = t; i < kMaxCands * kRingWords; i += blockDim.x) r[i] = 0u;
  for (int i = t; i < kMaxCands; i += blockDim.x) {
    c->cost[i] = 0.0;
    c->path[i] = 0ull;
    c->next[i] = 0;
    c->slot[i] = 0;
  }
  for (int i = t; i < 2 * kSlots; i += blockDim.x) {
    c->spath[i / kSlots][i % kSlots] = 0ull;
    c->skey[i / kSlots][i % kSlots] = 0ull;
    c->slink[i / kSlots][i % kSlots] = -1;
  }
  if (t == 0) {
    c->n = 1;
    c->bank = 0;
    c->pos = 0;
    c->conv_fail = 0;
    if (!keep_counters) {
      c->cands_collapse = 0;
      c->next_filter_drops = 0;
      c->total_children = 0;
    }
  }
}

int init_contexts(SdmCtx* d_ctxs, int first, int count, int keep_counters, cudaStream_t stream) {
  if (count <= 0) return 0;
  sdm_ctx_init_kernel<<<count, 256, 0, stream>>>(d_ctxs, first, count, keep_counters);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

__global__ void zero_counters_kernel(SdmCtx* ctxs, int idx) {
  SdmCtx* c = &ctxs[idx];
  c->conv_fail = c->cands_collapse = c->next_filter_drops = c->total_children = 0;
}

// Decision bytes -> the reference's float +-1.0 samples.
__global__ void bits_to_float_kernel(const uint8_t* __restrict__ bits, float* __restrict__ out,
                                     size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    out[i] = bits[i] ? 1.0f : -1.0f;
}

}  // namespace dsdgpu

using namespace dsdgpu;

int dsdgpu_context::fail(int code, const char* what) {
  last_error = what;
  return code;
}

int dsdgpu_context::cuda_fail(cudaError_t e, const char* what) {
  char buf[256];
  snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  last_error = buf;
  return DSDGPU_ERR_CUDA;
}

int dsdgpu_context::ensure_scratch(size_t bytes) {
  if (scratch_bytes >= bytes) return DSDGPU_OK;
  if (d_scratch) cudaFree(d_scratch);
  d_scratch = nullptr;
  scratch_bytes = 0;
  cudaError_t e = cudaMalloc(&d_scratch, bytes);
  if (e != cudaSuccess) return cuda_fail(e, "scratch allocation");
  scratch_bytes = bytes;
  return DSDGPU_OK;
}

int dsdgpu_context::check_status() {
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_fail(e, "stream synchronize");
  int st = 0;
  e = cudaMemcpy(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "status read");
  if (st != 0) {
    cudaMemset(d_status, 0, sizeof(int));
    char buf[128];
    snprintf(buf, sizeof buf, "device status word %d (bounded walk/wait gave up)", st);
    last_error = buf;
    return DSDGPU_ERR_DEVICE;
  }
  return DSDGPU_OK;
}

int dsdgpu_context::run_jobs(const std::vector<SdmJob>& jobs) {
  const int n = (int)jobs.size();
  if (n == 0) return DSDGPU_OK;
  if (n > jobs_cap) {
    if (d_jobs) cudaFree(d_jobs);
    d_jobs = nullptr;
    jobs_cap = 0;
    cudaError_t e = cudaMalloc(&d_jobs, sizeof(SdmJob) * (size_t)n);
    if (e != cudaSuccess) return cuda_fail(e, "job table allocation");
    jobs_cap = n;
  }
  unsigned long long steps = 0;
  for (const SdmJob& j : jobs) steps += (unsigned long long)j.n_in;
  sdm_samples += steps;
  sdm_last_samples = steps;
  cudaError_t e = cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(SdmJob) * (size_t)n,
                                  cudaMemcpyHostToDevice, stream);
  if (e != cudaSuccess) return cuda_fail(e, "job table upload");
  SdmParams P = sdm;
  P.mode = sdm_mode;
  P.lanes = sdm_lanes;
  // failure-path tests: waits and walks that give up early (see the option)
  P.hop_limit = (failure_test & DSDGPU_FAIL_CHAIN_WALK) ? 1 : 0;
  P.part_wait_cycles = (failure_test & DSDGPU_FAIL_PART_WAIT) ? 2000000ll : 0;
  // many long jobs a little above a whole number of warps per FP64 pipe: the
  // balanced launch (parts of 1,024 samples queued over w warps per pipe; on
  // the DSD128 headline 1,024 / 2,048 / 4,096 ran 270.1 / 268.8 / 265.4 DSD
  // Msamples/s: shorter parts leave a shorter tail)
  constexpr long long kPartLen = 1024;
  const int wpp = (max_blocks == 0 && sdm_balance)
                      ? sdm_balanced_warps(P, jobs.data(), n, num_sms, kPartLen) : 0;
  if (wpp > 0) {
    // with DSDGPU_FAIL_PART_WAIT the queue holds one entry that no part
    // publishes: the warp that takes it waits (bounded) and gives up
    const long long total = sdm_parts_total(jobs.data(), n, kPartLen) +
                            ((failure_test & DSDGPU_FAIL_PART_WAIT) ? 1 : 0);
    if (total + 2 > parts_cap) {
      if (d_parts) cudaFree(d_parts);
      d_parts = nullptr;
      parts_cap = 0;
      e = cudaMalloc(&d_parts, sizeof(unsigned long long) * (size_t)(total + 2));
      if (e != cudaSuccess) return cuda_fail(e, "part queue allocation");
      parts_cap = total + 2;
    }
    if (launch_sdm_parts(P, d_jobs, n, kPartLen, d_parts, total, wpp, num_sms, d_ctx, d_status,
                         stream) != 0)
      return cuda_fail(cudaGetLastError(), "sdm kernel launch");
    sdm_last_kernel = dsdgpu::sdm_last_kernel();
    launches += 2;
    return check_status();
  }
  if (launch_sdm_jobs(P, d_jobs, n, d_counter, d_ctx, d_status, max_blocks, stream) != 0)
    return cuda_fail(cudaGetLastError(), "sdm kernel launch");
  sdm_last_kernel = dsdgpu::sdm_last_kernel();
  launches++;
  return check_status();
}

// Segment bookkeeping of sdm_process_block / sdm_segment_process: how many
// leading steps produce no kept decision, and the pending count afterwards.
int sdm_params_from_abi(const dsdgpu_sdm_params_t* p, dsdgpu::SdmParams* P, const char** err) {
  if (p->order < 2 || p->order > kMaxOrder) { *err = "order out of range"; return DSDGPU_ERR_ARG; }
  if (p->depth < 1 || p->depth > 64) { *err = "depth out of range"; return DSDGPU_ERR_ARG; }
  if (p->cands < 1 || p->cands > kMaxCands) { *err = "cands out of range"; return DSDGPU_ERR_ARG; }
  if (p->lat < 1 || p->lat > kMaxLat) { *err = "lat out of range"; return DSDGPU_ERR_ARG; }
  memset(P, 0, sizeof *P);
  for (int i = 0; i < p->order; i++) { P->a[i] = p->a[i]; P->g[i] = p->g[i]; }
  P->state_limit = p->state_limit;
  P->mask = p->depth >= 64 ? ~0ull : ((1ull << p->depth) - 1ull);
  P->order = p->order;
  P->cands = p->cands;
  P->lat = p->lat;
  P->depth = p->depth;
  return DSDGPU_OK;
}

void dsdgpu_context::plan_steps(int64_t pend, int64_t count, int64_t discard, int64_t* skip,
                                int64_t* out, int64_t* new_pend) const {
  sdm_plan_steps(sdm.lat, pend, count, discard, skip, out, new_pend);
}

extern "C" {

int dsdgpu_create(int device, dsdgpu_context_t** out) {
  if (!out) return DSDGPU_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return DSDGPU_ERR_CUDA;
  if (cudaSetDevice(device) != cudaSuccess) return DSDGPU_ERR_CUDA;
  dsdgpu_context* c = new (std::nothrow) dsdgpu_context();
  if (!c) return DSDGPU_ERR_NOMEM;
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&c->d_counter, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&c->d_status, sizeof(int)) != cudaSuccess ||
      cudaMemset(c->d_status, 0, sizeof(int)) != cudaSuccess) {
    dsdgpu_destroy(c);
    return DSDGPU_ERR_CUDA;
  }
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, device);
  c->num_sms = prop.multiProcessorCount;
  c->max_blocks = 0;  // 0: as many blocks as jobs need
  *out = c;
  return DSDGPU_OK;
}

void dsdgpu_destroy(dsdgpu_context_t* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  c->release_all();
  if (c->d_counter) cudaFree(c->d_counter);
  if (c->d_status) cudaFree(c->d_status);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int dsdgpu_sdm_work(const dsdgpu_context_t* c, uint64_t* total_samples, uint64_t* last_launch) {
  if (!c) return DSDGPU_ERR_ARG;
  if (total_samples) *total_samples = c->sdm_samples;
  if (last_launch) *last_launch = c->sdm_last_samples;
  return DSDGPU_OK;
}

int dsdgpu_set_option(dsdgpu_context_t* c, int option, int value) {
  if (!c) return DSDGPU_ERR_ARG;
  switch (option) {
    case DSDGPU_OPT_SDM_SELECT:
      if (value < DSDGPU_SELECT_FAST || value > DSDGPU_SELECT_VERIFY)
        return c->fail(DSDGPU_ERR_ARG, "bad selection mode");
      c->sdm_mode = value;
      return DSDGPU_OK;
    case DSDGPU_OPT_SDM_LANES:
      if (value != 0 && (value < 2 || value > 32 || (value & (value - 1))))
        return c->fail(DSDGPU_ERR_ARG, "lanes per job must be 0 or a power of two in 2..32");
      c->sdm_lanes = value;
      return DSDGPU_OK;
    case DSDGPU_OPT_SDM_BALANCE:
      if (value != 0 && value != 1) return c->fail(DSDGPU_ERR_ARG, "balance must be 0 or 1");
      c->sdm_balance = value;
      return DSDGPU_OK;
    case DSDGPU_OPT_FAILURE_TEST:
      if (value & ~(DSDGPU_FAIL_PART_WAIT | DSDGPU_FAIL_CHAIN_WALK))
        return c->fail(DSDGPU_ERR_ARG, "unknown failure-test bits");
      c->failure_test = value;
      return DSDGPU_OK;
    default:
      return c->fail(DSDGPU_ERR_ARG, "unknown option");
  }
}

int dsdgpu_launch_count(const dsdgpu_context_t* c, uint64_t* count) {
  if (!c || !count) return DSDGPU_ERR_ARG;
  *count = c->launches;
  return DSDGPU_OK;
}

const char* dsdgpu_last_error(const dsdgpu_context_t* c) {
  return c ? c->last_error.c_str() : "no context";
}

int dsdgpu_synchronize(dsdgpu_context_t* c) {
  if (!c) return DSDGPU_ERR_ARG;
  return c->check_status();
}

int dsdgpu_sdm_setup(dsdgpu_context_t* c, const dsdgpu_sdm_params_t* p, int num_contexts) {
  if (!c || !p) return DSDGPU_ERR_ARG;
  if (num_contexts < 1) return c->fail(DSDGPU_ERR_ARG, "num_contexts < 1");
  SdmParams P;
  const char* err = nullptr;
  const int prc = sdm_params_from_abi(p, &P, &err);
  if (prc) return c->fail(prc, err);
  cudaSetDevice(c->device);
  if (c->d_ctx) cudaFree(c->d_ctx);
  c->d_ctx = nullptr;
  c->nctx = 0;
  cudaError_t e = cudaMalloc(&c->d_ctx, sizeof(SdmCtx) * (size_t)num_contexts);
  if (e != cudaSuccess) return c->cuda_fail(e, "context allocation");
  c->sdm = P;
  c->nctx = num_contexts;
  c->das_persistent = 0;
  c->pending.assign(num_contexts, 0);
  c->draining.assign(num_contexts, 0);
  sdm_ctx_init_kernel<<<num_contexts, 256, 0, c->stream>>>(c->d_ctx, 0, num_contexts, 0); c->launches++;
  e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "context init launch");
  c->sdm_ready = true;
  return c->check_status();
}

int dsdgpu_sdm_reset(dsdgpu_context_t* c, int channel) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->sdm_ready) return c->fail(DSDGPU_ERR_STATE, "sdm not set up");
  if (channel < -1 || channel >= c->nctx) return c->fail(DSDGPU_ERR_ARG, "bad channel");
  cudaSetDevice(c->device);
  const int first = channel < 0 ? 0 : channel;
  const int count = channel < 0 ? c->nctx : 1;
  sdm_ctx_init_kernel<<<count, 256, 0, c->stream>>>(c->d_ctx, first, count, 1); c->launches++;
  for (int i = first; i < first + count; i++) { c->pending[i] = 0; c->draining[i] = 0; }
  return c->check_status();
}

int dsdgpu_sdm_process(dsdgpu_context_t* c, int first, int nch, const double* d_in,
                       size_t in_stride, size_t count, uint8_t* d_out, size_t out_stride,
                       size_t* out_counts) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->sdm_ready) return c->fail(DSDGPU_ERR_STATE, "sdm not set up");
  if (first < 0 || nch < 1 || first + nch > c->nctx) return c->fail(DSDGPU_ERR_ARG, "bad channel range");
  if (count > 0 && (!d_in || !d_out)) return c->fail(DSDGPU_ERR_ARG, "null buffer");
  if (nch > 1 && count > 0) {
    // rows of different channels must not overlap
    int64_t max_out = 0;
    for (int ch = 0; ch < nch; ch++) {
      int64_t skip, out, np;
      c->plan_steps(c->pending[first + ch], (int64_t)count, 0, &skip, &out, &np);
      max_out = std::max(max_out, out);
    }
    if (in_stride < count || out_stride < (size_t)max_out)
      return c->fail(DSDGPU_ERR_ARG, "row stride shorter than a channel's rows");
  }
  cudaSetDevice(c->device);
  std::vector<SdmJob> jobs;
  for (int ch = 0; ch < nch; ch++) {
    const int idx = first + ch;
    int64_t skip, out, np;
    c->plan_steps(c->pending[idx], (int64_t)count, 0, &skip, &out, &np);
    if (out_counts) out_counts[ch] = (size_t)out;
    c->pending[idx] = np;
    if (count == 0) continue;
    SdmJob j;
    j.in = d_in + (size_t)ch * in_stride;
    j.out = d_out + (size_t)ch * out_stride;
    j.n_in = (long long)count;
    j.skip_out = skip;
    j.ctx = idx;
    j.copy_from = -1;
    j.seed_state = nullptr;
    j.flags = 0;
    jobs.push_back(j);
  }
  return c->run_jobs(jobs);
}

int dsdgpu_sdm_process_host(dsdgpu_context_t* c, int first, int nch, const double* h_in,
                            size_t count, float* h_out, size_t* out_counts) {
  if (!c || (count > 0 && (!h_in || !h_out))) return DSDGPU_ERR_ARG;
  if (!c->sdm_ready) return c->fail(DSDGPU_ERR_STATE, "sdm not set up");
  if (first < 0 || nch < 1 || first + nch > c->nctx) return c->fail(DSDGPU_ERR_ARG, "bad channel range");
  cudaSetDevice(c->device);
  const size_t tot = (size_t)nch * count;
  const size_t in_bytes = (tot * sizeof(double) + 255) & ~(size_t)255;
  const size_t bit_bytes = (tot + 255) & ~(size_t)255;
  int rc = c->ensure_scratch(in_bytes + bit_bytes + tot * sizeof(float) + 256);
  if (rc) return rc;
  double* d_in = (double*)c->d_scratch;
  uint8_t* d_bits = (uint8_t*)c->d_scratch + in_bytes;
  float* d_f = (float*)((uint8_t*)c->d_scratch + in_bytes + bit_bytes);
  cudaError_t e = cudaMemcpyAsync(d_in, h_in, tot * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "input upload");
  std::vector<size_t> oc(nch);
  rc = dsdgpu_sdm_process(c, first, nch, d_in, count, count, d_bits, count, oc.data());
  if (rc) return rc;
  // decisions are written at the start of each channel's row
  bits_to_float_kernel<<<256, 256, 0, c->stream>>>(d_bits, d_f, tot); c->launches++;
  for (int ch = 0; ch < nch; ch++) {
    if (out_counts) out_counts[ch] = oc[ch];
    if (oc[ch] == 0) continue;
    e = cudaMemcpyAsync(h_out + (size_t)ch * count, d_f + (size_t)ch * count,
                        oc[ch] * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "output download");
  }
  return c->check_status();
}

int dsdgpu_sdm_drain(dsdgpu_context_t* c, int first, int nch, uint8_t* d_out, size_t out_stride,
                     size_t max_out, size_t* out_counts) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->sdm_ready) return c->fail(DSDGPU_ERR_STATE, "sdm not set up");
  if (first < 0 || nch < 1 || first + nch > c->nctx) return c->fail(DSDGPU_ERR_ARG, "bad channel range");
  cudaSetDevice(c->device);
  std::vector<SdmJob> jobs;
  for (int ch = 0; ch < nch; ch++) {
    const int idx = first + ch;
    // sdm_drain (src/trellis.c:1042-1062)
    int64_t len = std::min<int64_t>(c->pending[idx], (int64_t)max_out);
    int64_t flush = 0;
    if (!c->draining[idx] && c->pending[idx] < c->sdm.lat) flush = c->sdm.lat - c->pending[idx];
    c->draining[idx] = 1;
    c->pending[idx] -= len;
    if (out_counts) out_counts[ch] = (size_t)len;
    if (flush + len == 0) continue;
    if (len > 0 && !d_out) return c->fail(DSDGPU_ERR_ARG, "null output");
    SdmJob j;
    j.in = nullptr;
    j.out = d_out ? d_out + (size_t)ch * out_stride : nullptr;
    j.n_in = flush + len;
    j.skip_out = flush;
    j.ctx = idx;
    j.copy_from = -1;
    j.seed_state = nullptr;
    j.flags = 0;
    jobs.push_back(j);
  }
  return c->run_jobs(jobs);
}

int dsdgpu_sdm_copy_state(dsdgpu_context_t* c, int dst, int src) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->sdm_ready) return c->fail(DSDGPU_ERR_STATE, "sdm not set up");
  if (dst < 0 || src < 0 || dst >= c->nctx || src >= c->nctx) return c->fail(DSDGPU_ERR_ARG, "bad context");
  if (dst == src) return DSDGPU_OK;
  cudaSetDevice(c->device);
  cudaError_t e = cudaMemcpyAsync(c->d_ctx + dst, c->d_ctx + src, sizeof(SdmCtx),
                                  cudaMemcpyDeviceToDevice, c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "context copy");
  zero_counters_kernel<<<1, 1, 0, c->stream>>>(c->d_ctx, dst); c->launches++;
  c->pending[dst] = c->pending[src];
  c->draining[dst] = c->draining[src];
  return c->check_status();
}

int dsdgpu_sdm_segments(dsdgpu_context_t* c, dsdgpu_segment_t* segs, int nseg) {
  if (!c || (nseg > 0 && !segs)) return DSDGPU_ERR_ARG;
  if (!c->sdm_ready) return c->fail(DSDGPU_ERR_STATE, "sdm not set up");
  cudaSetDevice(c->device);
  std::vector<char> runs(c->nctx, 0);
  for (int i = 0; i < nseg; i++) {
    const dsdgpu_segment_t& s = segs[i];
    if (s.channel < 0 || s.channel >= c->nctx) return c->fail(DSDGPU_ERR_ARG, "bad segment channel");
    if (s.seed_from < -1 || s.seed_from >= c->nctx) return c->fail(DSDGPU_ERR_ARG, "bad seed_from");
    if (s.count < 0 || s.discard < 0) return c->fail(DSDGPU_ERR_ARG, "negative count");
    if (runs[s.channel]) return c->fail(DSDGPU_ERR_ARG, "a context appears twice in one call");
    runs[s.channel] = 1;
  }
  for (int i = 0; i < nseg; i++)
    if (segs[i].seed_from >= 0 && segs[i].seed_from != segs[i].channel && runs[segs[i].seed_from])
      return c->fail(DSDGPU_ERR_ARG, "seed_from names a context that runs in the same call");
  std::vector<SdmJob> jobs;
  for (int i = 0; i < nseg; i++) {
    dsdgpu_segment_t& s = segs[i];
    const int from = s.seed_from >= 0 ? s.seed_from : s.channel;
    int64_t skip, out, np;
    c->plan_steps(c->pending[from], s.count, s.discard, &skip, &out, &np);
    c->draining[s.channel] = c->draining[from];
    c->pending[s.channel] = np;
    s.out_count = out;
    if (s.count == 0) {
      if (s.seed_from >= 0 && s.seed_from != s.channel) {
        int rc = dsdgpu_sdm_copy_state(c, s.channel, s.seed_from);
        if (rc) return rc;
        c->pending[s.channel] = np;
      }
      continue;
    }
    if (!s.d_in || (out > 0 && !s.d_out)) return c->fail(DSDGPU_ERR_ARG, "null segment buffer");
    SdmJob j;
    j.in = s.d_in;
    j.out = s.d_out;
    j.n_in = s.count;
    j.skip_out = skip;
    j.ctx = s.channel;
    j.copy_from = (s.seed_from >= 0 && s.seed_from != s.channel) ? s.seed_from : -1;
    j.seed_state = s.d_seed_state;
    j.flags = 0;
    jobs.push_back(j);
  }
  return c->run_jobs(jobs);
}

int dsdgpu_sdm_query(dsdgpu_context_t* c, int channel, double* best_state, uint64_t* info) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->sdm_ready) return c->fail(DSDGPU_ERR_STATE, "sdm not set up");
  if (channel < 0 || channel >= c->nctx) return c->fail(DSDGPU_ERR_ARG, "bad channel");
  cudaSetDevice(c->device);
  int rc = c->check_status();
  if (rc) return rc;
  SdmCtx* h = (SdmCtx*)malloc(sizeof(SdmCtx));
  if (!h) return DSDGPU_ERR_NOMEM;
  cudaError_t e = cudaMemcpy(h, c->d_ctx + channel, sizeof(SdmCtx), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) { free(h); return c->cuda_fail(e, "context read"); }
  if (best_state)
    for (int k = 0; k < c->sdm.order; k++) best_state[k] = h->s[0][k];
  if (info) {
    info[0] = h->conv_fail;
    info[1] = h->cands_collapse;
    info[2] = h->next_filter_drops;
    info[3] = h->total_children;
    info[4] = (uint64_t)h->n;
    info[5] = (uint64_t)c->pending[channel];
  }
  free(h);
  return DSDGPU_OK;
}

int dsdgpu_sdm_last_kernel(const dsdgpu_context_t* c, char* name, size_t cap) {
  if (!c || !name || cap == 0) return DSDGPU_ERR_ARG;
  snprintf(name, cap, "%s", c->sdm_last_kernel.c_str());
  return DSDGPU_OK;
}

int dsdgpu_sdm_state_distance(dsdgpu_context_t* c, int a, int b, double* dist) {
  // sdm_state_distance (src/trellis.c:1094-1109): the sum over the NTF order
  // of the squared differences of the two best candidates' states, in order
  if (!c || !dist) return DSDGPU_ERR_ARG;
  double sa[dsdgpu::kMaxOrder], sb[dsdgpu::kMaxOrder];
  int rc = dsdgpu_sdm_query(c, a, sa, nullptr);
  if (rc) return rc;
  rc = dsdgpu_sdm_query(c, b, sb, nullptr);
  if (rc) return rc;
  double d = 0.0;
  for (int i = 0; i < c->sdm.order; i++) {
    const double t = sa[i] - sb[i];
    d += t * t;
  }
  *dist = d;
  return DSDGPU_OK;
}

}  // extern "C"
