// Allocation-free trellis SDM entry point (dsdgpu_sdm_process_noalloc).
//
// Who needs it: code that converts audio inside a real-time audio callback
// (a player's DSP chain runs its per-chunk processing on the playback
// thread, where a device allocation can block on driver locks and
// synchronise the device long enough to cause a dropout), and hosts that give
// the converter a fixed device-memory budget up front.  Such callers cannot
// call cudaMalloc, so this entry point allocates nothing: every piece of
// scratch memory the SDM kernel needs beyond the caller's input and output
// (the per-channel context bank, the job table, the job counter and the
// status word) lives in one file-scope __device__ array of fixed size,
// kNoAllocScratchBytes, that every GPU which loads the library holds until
// the process exits.
//
// The array's name is only a host-side stand-in in host code, not a device
// address, so the first call on each device looks its address up with
// cudaGetSymbolAddress (with that device current) and caches it; that first
// call should therefore come before any stream capture.  All calls share the
// array and it keeps the last call's contents: the counter and status word
// are cleared on every call and the contexts are re-initialised, but two
// calls whose work overlaps on the GPU (for example on different streams)
// race on the same memory and must not be issued.
#include "api_context.h"

#include <cstring>
#include <mutex>

namespace dsdgpu {

int launch_sdm_jobs(const SdmParams& P, const SdmJob* d_jobs, int njobs, int* d_counter,
                    SdmCtx* d_ctxs, int* d_status, int max_blocks, cudaStream_t stream);
int init_contexts(SdmCtx* d_ctxs, int first, int count, int keep_counters, cudaStream_t stream);
int sdm_max_lat_in_registers();

constexpr int kNoAllocMaxChannels = 8;
constexpr size_t kCtxBytes = sizeof(SdmCtx) * kNoAllocMaxChannels;
constexpr size_t kJobOffset = (kCtxBytes + 255) & ~(size_t)255;
constexpr size_t kCounterOffset = (kJobOffset + sizeof(SdmJob) * kNoAllocMaxChannels + 255) & ~(size_t)255;
constexpr size_t kNoAllocScratchBytes = kCounterOffset + 256;

static __device__ __align__(256) unsigned char g_sdm_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
static unsigned char* g_scratch_addr[kMaxDevices];
static std::once_flag g_scratch_once[kMaxDevices];
static cudaError_t g_scratch_err[kMaxDevices];

}  // namespace dsdgpu

using namespace dsdgpu;

extern "C" int dsdgpu_sdm_process_noalloc(const dsdgpu_sdm_params_t* p, int nch, const double* d_in,
                                          size_t in_stride, size_t count, uint8_t* d_out,
                                          size_t out_stride, size_t* out_counts, void* stream) {
  if (!p) return DSDGPU_ERR_ARG;
  if (nch < 1) return DSDGPU_ERR_ARG;
  if (nch > kNoAllocMaxChannels) return DSDGPU_ERR_TOO_LARGE;   // fixed scratch: 8 channels
  if (p->order < 2 || p->order > kMaxOrder || p->depth < 1 || p->depth > 64 || p->cands < 1 ||
      p->cands > kMaxCands || p->lat < 1 || p->lat > kMaxLat)
    return DSDGPU_ERR_ARG;
  if (p->lat > sdm_max_lat_in_registers()) return DSDGPU_ERR_UNSUPPORTED;
  if (count > 0 && (!d_in || !d_out)) return DSDGPU_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return DSDGPU_ERR_CUDA;
  // one-time, per device: the device address of the scratch array
  std::call_once(g_scratch_once[dev], [dev] {
    void* ptr = nullptr;
    g_scratch_err[dev] = cudaGetSymbolAddress(&ptr, g_sdm_noalloc_scratch);
    g_scratch_addr[dev] = (unsigned char*)ptr;
  });
  if (g_scratch_err[dev] != cudaSuccess || !g_scratch_addr[dev]) return DSDGPU_ERR_CUDA;
  unsigned char* base = g_scratch_addr[dev];
  SdmCtx* d_ctx = (SdmCtx*)base;
  SdmJob* d_jobs = (SdmJob*)(base + kJobOffset);
  int* d_counter = (int*)(base + kCounterOffset);
  int* d_status = d_counter + 1;
  cudaStream_t s = (cudaStream_t)stream;

  // sdm_context_init on every channel, then sdm_process_block over the block
  const int64_t lat = p->lat;
  const int64_t pre = (int64_t)count < lat ? (int64_t)count : lat;
  SdmParams P;
  memset(&P, 0, sizeof P);
  for (int i = 0; i < p->order; i++) { P.a[i] = p->a[i]; P.g[i] = p->g[i]; }
  P.state_limit = p->state_limit;
  P.mask = p->depth >= 64 ? ~0ull : ((1ull << p->depth) - 1ull);
  P.order = p->order;
  P.cands = p->cands;
  P.lat = p->lat;
  P.depth = p->depth;
  SdmJob jobs[kNoAllocMaxChannels];
  for (int ch = 0; ch < nch; ch++) {
    if (out_counts) out_counts[ch] = (size_t)((int64_t)count - pre);
    jobs[ch].in = d_in + (size_t)ch * in_stride;
    jobs[ch].out = d_out + (size_t)ch * out_stride;
    jobs[ch].n_in = (long long)count;
    jobs[ch].skip_out = pre;
    jobs[ch].ctx = ch;
    jobs[ch].copy_from = -1;
    jobs[ch].seed_state = nullptr;
    jobs[ch].flags = 0;
  }
  if (count == 0) return DSDGPU_OK;
  if (cudaMemsetAsync(d_status, 0, sizeof(int), s) != cudaSuccess) return DSDGPU_ERR_CUDA;
  if (init_contexts(d_ctx, 0, nch, 0, s) != 0) return DSDGPU_ERR_CUDA;
  if (cudaMemcpyAsync(d_jobs, jobs, sizeof(SdmJob) * (size_t)nch, cudaMemcpyHostToDevice, s) !=
      cudaSuccess)
    return DSDGPU_ERR_CUDA;
  if (launch_sdm_jobs(P, d_jobs, nch, d_counter, d_ctx, d_status, 0, s) != 0) return DSDGPU_ERR_CUDA;
  int st = 0;
  if (cudaMemcpyAsync(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return DSDGPU_ERR_CUDA;
  return st ? DSDGPU_ERR_DEVICE : DSDGPU_OK;
}
