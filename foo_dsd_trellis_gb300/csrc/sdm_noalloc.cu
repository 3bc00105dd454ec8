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
// cudaGetSymbolAddress (with that device current) and caches it.  The cached address
// belongs to the device's primary context: after cudaDeviceReset the module
// is loaded again elsewhere and this entry point must not be used in that
// process any more.
//
// CUDA loads modules and kernels lazily by default, so the first call on a
// device, and the first call with each new kernel variant (NTF order, number
// of candidates, lat above 256), load code and may allocate inside the
// driver.  A real-time caller makes one warm-up call with the same parameters
// and channel count outside the callback (or runs with
// CUDA_MODULE_LOADING=EAGER); after that, calls allocate nothing.
//
// All calls share the array and it keeps the last call's contents: the
// status word is cleared on every call, and the contexts are re-initialised
// unless the caller asks to continue from them (keep_state).  Two calls whose
// work overlaps on the GPU (for example on different streams) race on the
// same memory and must not be issued.
#include "api_context.h"
#include "das_plan.h"

#include <cstring>
#include <mutex>

namespace dsdgpu {

int launch_sdm_jobs(const SdmParams& P, const SdmJob* d_jobs, int njobs, int* d_counter,
                    SdmCtx* d_ctxs, int* d_status, int max_blocks, cudaStream_t stream);
int init_contexts(SdmCtx* d_ctxs, int first, int count, int keep_counters, cudaStream_t stream);

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

// What the array's contexts hold after the last successful call on a device:
// the parameters and channel count they were run with and each channel's
// latency fill, so that a keep_state call continues one stream per channel.
struct NoAllocStream {
  std::mutex mu;
  bool valid = false;
  SdmParams P;
  int nch = 0;
  int64_t pending[kNoAllocMaxChannels] = {};
};
static NoAllocStream g_streams[kMaxDevices];

}  // namespace dsdgpu

using namespace dsdgpu;

extern "C" int dsdgpu_sdm_process_noalloc(const dsdgpu_sdm_params_t* p, int nch, int keep_state,
                                          const double* d_in, size_t in_stride, size_t count,
                                          uint8_t* d_out, size_t out_stride, size_t* out_counts,
                                          void* stream) {
  if (!p || nch < 1 || (keep_state != 0 && keep_state != 1)) return DSDGPU_ERR_ARG;
  if (nch > kNoAllocMaxChannels) return DSDGPU_ERR_TOO_LARGE;   // fixed scratch: 8 channels
  SdmParams P;
  const char* err = nullptr;
  const int prc = sdm_params_from_abi(p, &P, &err);
  if (prc != DSDGPU_OK) return prc;
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

  NoAllocStream& S = g_streams[dev];
  std::lock_guard<std::mutex> lock(S.mu);
  if (keep_state && (!S.valid || S.nch != nch || memcmp(&S.P, &P, sizeof P) != 0))
    return DSDGPU_ERR_STATE;

  // sdm_context_init on every channel (unless continuing), then
  // sdm_process_block over the block: the first lat inputs of a stream give
  // no output
  SdmJob jobs[kNoAllocMaxChannels];
  int64_t pend[kNoAllocMaxChannels];
  size_t max_out = 0;
  for (int ch = 0; ch < nch; ch++) {
    int64_t skip = 0, out = 0;
    sdm_plan_steps(P.lat, keep_state ? S.pending[ch] : 0, (int64_t)count, 0, &skip, &out,
                   &pend[ch]);
    if ((size_t)out > max_out) max_out = (size_t)out;
    jobs[ch].in = d_in + (size_t)ch * in_stride;
    jobs[ch].out = d_out + (size_t)ch * out_stride;
    jobs[ch].n_in = (long long)count;
    jobs[ch].skip_out = skip;
    jobs[ch].ctx = ch;
    jobs[ch].copy_from = -1;
    jobs[ch].seed_state = nullptr;
    jobs[ch].flags = 0;
  }
  // rows of different channels must not overlap
  if (nch > 1 && count > 0 && (in_stride < count || out_stride < max_out)) return DSDGPU_ERR_ARG;
  if (out_counts)
    for (int ch = 0; ch < nch; ch++) out_counts[ch] = (size_t)((int64_t)count - jobs[ch].skip_out);

  S.valid = false;   // until this call has completed
  if (!keep_state && init_contexts(d_ctx, 0, nch, 0, s) != 0) return DSDGPU_ERR_CUDA;
  if (count > 0) {
    if (cudaMemsetAsync(d_status, 0, sizeof(int), s) != cudaSuccess) return DSDGPU_ERR_CUDA;
    if (cudaMemcpyAsync(d_jobs, jobs, sizeof(SdmJob) * (size_t)nch, cudaMemcpyHostToDevice, s) !=
        cudaSuccess)
      return DSDGPU_ERR_CUDA;
    if (launch_sdm_jobs(P, d_jobs, nch, d_counter, d_ctx, d_status, 0, s) != 0)
      return DSDGPU_ERR_CUDA;
  }
  int st = 0;
  if (count > 0 &&
      cudaMemcpyAsync(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return DSDGPU_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return DSDGPU_ERR_CUDA;
  if (st) return DSDGPU_ERR_DEVICE;
  S.valid = true;
  memcpy(&S.P, &P, sizeof P);
  S.nch = nch;
  for (int ch = 0; ch < nch; ch++) S.pending[ch] = pend[ch];
  return DSDGPU_OK;
}
