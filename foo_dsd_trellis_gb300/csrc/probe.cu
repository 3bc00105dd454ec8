// FP64 issue-rate probe: the denominator of the trellis SDM roofline.  The
// SDM's FP64 work is separate adds and multiplies (the reference forbids
// contraction), so the peak that bounds it is the DADD/DMUL rate of the FP64
// pipe, measured here with independent chains of __dadd_rn / __dmul_rn
// (no memory traffic besides one store per thread).
#include "api_context.h"
#include "fp_convert.h"

namespace dsdgpu {

__global__ void fp64_probe_kernel(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = (k & 1) ? __dmul_rn(x[k], b) : __dadd_rn(x[k], a);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Conversion self-check: binary32 pattern (seed + i * 0x9E3779B1) mod 2^32
// for i < n (an odd multiplier: n = 2^32 visits every pattern once), widened
// by widen_exact, by widen_normal_fast and by the hardware; NaNs compare as NaN.
__global__ void convert_check_kernel(unsigned long long n, unsigned seed,
                                     unsigned long long* bad) {
  unsigned long long local = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const float f = __uint_as_float(seed + (unsigned)i * 0x9E3779B1u);
    const double a = widen_exact(f), a2 = widen_normal_fast(f), b = (double)f;
    const bool same = (f != f) ? (a != a && a2 != a2)
                               : (__double_as_longlong(a) == __double_as_longlong(b) &&
                                  __double_as_longlong(a2) == __double_as_longlong(b));
    local += same ? 0 : 1;
  }
  if (local) atomicAdd(bad, local);
}

}  // namespace dsdgpu

using namespace dsdgpu;

extern "C" int dsdgpu_selftest_convert(dsdgpu_context_t* c, uint64_t n, uint64_t seed,
                                       uint64_t* mismatches) {
  if (!c || !mismatches) return DSDGPU_ERR_ARG;
  cudaSetDevice(c->device);
  unsigned long long* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(unsigned long long));
  if (e != cudaSuccess) return c->cuda_fail(e, "self-check allocation");
  cudaMemsetAsync(d, 0, sizeof(unsigned long long), c->stream);
  const int blocks = (c->num_sms > 0 ? c->num_sms : 148) * 8;
  convert_check_kernel<<<blocks, 256, 0, c->stream>>>((unsigned long long)n, (unsigned)seed,
                                                      d);
  c->launches++;
  unsigned long long h = 0;
  cudaMemcpyAsync(&h, d, sizeof h, cudaMemcpyDeviceToHost, c->stream);
  e = cudaStreamSynchronize(c->stream);
  cudaFree(d);
  if (e != cudaSuccess) return c->cuda_fail(e, "self-check");
  *mismatches = h;
  return DSDGPU_OK;
}

extern "C" int dsdgpu_probe_fp64(dsdgpu_context_t* c, double* gops) {
  if (!c || !gops) return DSDGPU_ERR_ARG;
  cudaSetDevice(c->device);
  const int blocks = (c->num_sms > 0 ? c->num_sms : 148) * 8, threads = 256, iters = 2048;
  double* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(double) * (size_t)blocks * threads);
  if (e != cudaSuccess) return c->cuda_fail(e, "probe allocation");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; rep++) {
    cudaEventRecord(e0, c->stream);
    fp64_probe_kernel<<<blocks, threads, 0, c->stream>>>(d, iters, 1.0000001, 0.9999999);
    c->launches++;
    cudaEventRecord(e1, c->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "probe");
  *gops = (double)blocks * threads * iters * 8 / (best * 1e-3) / 1e9;
  return DSDGPU_OK;
}
