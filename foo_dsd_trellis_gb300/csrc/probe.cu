// FP64 issue-rate probe: the denominator of the trellis SDM roofline.  The
// SDM's FP64 work is separate adds and multiplies (the reference forbids
// contraction), so the peak that bounds it is the DADD/DMUL rate of the FP64
// pipe, measured here with independent chains of __dadd_rn / __dmul_rn
// (no memory traffic besides one store per thread).
#include "api_context.h"

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

}  // namespace dsdgpu

using namespace dsdgpu;

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
