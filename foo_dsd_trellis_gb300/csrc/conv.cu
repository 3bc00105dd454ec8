// Uniformly partitioned overlap-save (UPOLS) convolution at the SDM rate, FP32
// (reference src/convolution.c:355-405 partitions the IR; src/gpu_cuda.c:
// 3432-3492 and src/kernels/conv_kernels.cu:62-84 run it block by block with
// a frequency-domain delay line).
//
// Here a call convolves whole chunks of every channel at once:
//   1. forward   every window m of 2P samples (input distance P) of each
//                channel's stream [history of NP*P samples | chunk | zeros]
//                is read straight from the FP64 input and transformed by this
//                file's FFT (one CTA per window, shared memory): the 2P real
//                samples packed as P complex values, a mixed radix-2/4
//                Stockham FFT, and the split into the P + 1 bins of the real
//                transform
//   2. MAC       Y_b[f] = sum_k X_{b-k}[f] H_k[f]: one thread per (channel,
//                bin, run of blocks) streams the spectra once, holding the NP
//                partition spectra and NP running sums in registers
//   3. inverse   every output block: the real-transform bins folded back to P
//                complex values, the inverse FFT, and the second half of the
//                block, scaled by 1/(2P), written to the FP64 SDM input
//   4. history   the last NP*P input samples, for the next chunk
// Partitions above 8,192 samples (a transform beyond one CTA's shared memory)
// use cuFFT for the plain R2C / C2R transforms around the same MAC kernel.
#include "api_context.h"

#include <cufft.h>

#include <new>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <utility>
#include <vector>

using namespace dsdgpu;

namespace {

constexpr int kMaxParts = 32;        // IR up to 32 partitions (rounded up to 1/2/4/8/16/32)
constexpr int kMacRun = 256;         // output blocks per MAC thread

int round_parts(int np) {
  int r = 1;
  while (r < np) r <<= 1;
  return r;
}

// ---- framing: history + chunk (double -> float) + zero tail ----
__global__ void conv_frame_kernel(const double* __restrict__ in, size_t in_stride, long long count,
                                  const float* __restrict__ hist, long long hlen, long long L,
                                  int nch, float* __restrict__ w) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L * nch) return;
  const long long c = i / L, k = i % L;
  float v = 0.0f;
  if (k < hlen) v = hist[c * hlen + k];
  else if (k - hlen < count) v = (float)in[(size_t)c * in_stride + (k - hlen)];
  w[i] = v;
}

// new history = the last hlen samples of (old history ++ chunk), from the framed buffer
__global__ void conv_hist_kernel(const float* __restrict__ w, long long L, long long hlen,
                                 long long count, int nch, float* __restrict__ hist) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hlen * nch) return;
  const long long c = i / hlen, k = i % hlen;
  hist[i] = w[c * L + count + k];     // framed index hlen + count - hlen + k
}

// ---- partitioned complex multiply-accumulate ----
// Thread (c, f, run r): outputs b in [b0, b1) = [r kMacRun, ...), input blocks
// j from b0 - NP + 1; window of input block j is m = j + NP - 1.
template <int NP>
__global__ void __launch_bounds__(128)
conv_mac_kernel(const cufftComplex* __restrict__ X, const cufftComplex* __restrict__ H,
                cufftComplex* __restrict__ Y, int bins, long long B, long long wpc, int nch) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const long long r = blockIdx.y;
  const int c = blockIdx.z;
  if (f >= bins || c >= nch) return;
  const long long b0 = r * kMacRun;
  if (b0 >= B) return;
  const long long b1 = min(B, b0 + (long long)kMacRun);
  float hr[NP], hi[NP], ar[NP], ai[NP];
#pragma unroll
  for (int k = 0; k < NP; k++) {
    const cufftComplex h = H[((size_t)c * NP + k) * bins + f];
    hr[k] = h.x;
    hi[k] = h.y;
    ar[k] = 0.0f;
    ai[k] = 0.0f;
  }
  // ar[k] holds the running sum of output block j + k
  const cufftComplex* Xc = X + (size_t)c * wpc * bins;
  cufftComplex* Yc = Y + (size_t)c * B * bins;
  for (long long j = b0 - NP + 1; j < b1; j++) {
    const cufftComplex x = Xc[(size_t)(j + NP - 1) * bins + f];
#pragma unroll
    for (int k = 0; k < NP; k++) {
      ar[k] = fmaf(x.x, hr[k], fmaf(-x.y, hi[k], ar[k]));
      ai[k] = fmaf(x.x, hi[k], fmaf(x.y, hr[k], ai[k]));
    }
    if (j >= b0) Yc[(size_t)j * bins + f] = make_cuFloatComplex(ar[0], ai[0]);
#pragma unroll
    for (int k = 0; k < NP - 1; k++) {
      ar[k] = ar[k + 1];
      ai[k] = ai[k + 1];
    }
    ar[NP - 1] = 0.0f;
    ai[NP - 1] = 0.0f;
  }
}

// ---- gather the valid half of every output block ----
__global__ void conv_gather_kernel(const float* __restrict__ o, int P, long long B, long long count,
                                   int nch, float scale, double* __restrict__ out,
                                   size_t out_stride) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count * nch) return;
  const long long c = i / count, t = i % count;
  const long long b = t / P, k = t % P;
  out[(size_t)c * out_stride + t] = (double)(o[((size_t)c * B + b) * 2 * P + P + k] * scale);
}

// IR partition k of channel c, zero-padded to 2P
__global__ void conv_ir_frame_kernel(const float* __restrict__ ir, long long ir_len, int P, int NP,
                                     int nch, float* __restrict__ w) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long per = (long long)NP * 2 * P;
  if (i >= per * nch) return;
  const long long c = i / per, r = i % per;
  const long long k = r / (2 * P), q = r % (2 * P);
  const long long src = k * P + q;
  w[i] = (q < P && src < ir_len) ? ir[c * ir_len + src] : 0.0f;
}

unsigned blocks_of(long long n, int t) { return (unsigned)((n + t - 1) / t); }

// ---- the transforms (partitions P <= kOwnFftMaxP) ----
constexpr int kOwnFftMaxP = 8192;
constexpr int kFftThreads = 256;

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// e^{-2 pi i j / (2M)} (forward) or its conjugate (inverse), from the table
template <bool INV>
__device__ __forceinline__ float2 twid(const float2* __restrict__ tw2, int j) {
  const float2 w = __ldg(&tw2[j]);
  return INV ? make_float2(w.x, -w.y) : w;
}

// Complex FFT of M (a power of two, 32..8192) points in shared memory, a and b
// the ping-pong buffers; returns the buffer that holds the result.  Stockham
// autosort: a radix-2 stage first when log2 M is odd, then radix-4 stages;
// stage with span p: butterfly j reads x[j + q M/4], twiddles W_{4p}^{k q}
// (k = j mod p), writes y[4(j - k) + k + q p].  Unnormalised in both
// directions.
template <bool INV>
__device__ float2* fft_smem(float2* a, float2* b, int M, const float2* __restrict__ tw2) {
  int p = 1;
  if ((__ffs(M) - 1) & 1) {
    const int h = M / 2;
    for (int j = threadIdx.x; j < h; j += blockDim.x) {
      const float2 x0 = a[j], x1 = a[j + h];
      b[2 * j] = make_float2(x0.x + x1.x, x0.y + x1.y);
      b[2 * j + 1] = make_float2(x0.x - x1.x, x0.y - x1.y);
    }
    __syncthreads();
    float2* t = a; a = b; b = t;
    p = 2;
  }
  const int Q = M / 4;
  for (; p < M; p *= 4) {
    const int ts = M / (2 * p);          // table index of W_{4p}
    for (int j = threadIdx.x; j < Q; j += blockDim.x) {
      const int k = j & (p - 1);
      float2 a0 = a[j], a1 = a[j + Q], a2 = a[j + 2 * Q], a3 = a[j + 3 * Q];
      if (k) {
        a1 = cmul(a1, twid<INV>(tw2, k * ts));
        a2 = cmul(a2, twid<INV>(tw2, 2 * k * ts));
        a3 = cmul(a3, twid<INV>(tw2, 3 * k * ts));
      }
      const float2 t0 = make_float2(a0.x + a2.x, a0.y + a2.y);
      const float2 t1 = make_float2(a0.x - a2.x, a0.y - a2.y);
      const float2 t2 = make_float2(a1.x + a3.x, a1.y + a3.y);
      const float2 t3 = make_float2(a1.x - a3.x, a1.y - a3.y);
      // s * t3 with s = -i (forward) or +i (inverse)
      const float2 st3 = INV ? make_float2(-t3.y, t3.x) : make_float2(t3.y, -t3.x);
      const int base = 4 * (j - k) + k;
      b[base] = make_float2(t0.x + t2.x, t0.y + t2.y);
      b[base + p] = make_float2(t1.x + st3.x, t1.y + st3.y);
      b[base + 2 * p] = make_float2(t0.x - t2.x, t0.y - t2.y);
      b[base + 3 * p] = make_float2(t1.x - st3.x, t1.y - st3.y);
    }
    __syncthreads();
    float2* t = a; a = b; b = t;
  }
  return a;
}

// Real transform of 2M samples z[n] = x[2n] + i x[2n+1] already in `a`:
// X[k] = (Z_k + Z*_{M-k}) / 2 + e^{-i pi k / M} (Z_k - Z*_{M-k}) / (2i),
// k = 0..M, written to X (M + 1 bins).
__device__ void rfft_smem(float2* a, float2* b, int M, const float2* __restrict__ tw2,
                          float2* __restrict__ X) {
  const float2* Z = fft_smem<false>(a, b, M, tw2);
  for (int k = threadIdx.x; k <= M; k += blockDim.x) {
    const float2 zk = Z[k & (M - 1)];
    const float2 zm = Z[(M - k) & (M - 1)];
    const float2 e = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));   // (zk + conj zm) / 2
    const float2 d = make_float2(zk.x - zm.x, zk.y + zm.y);                     // zk - conj zm
    const float2 o = make_float2(0.5f * d.y, -0.5f * d.x);                      // d / (2i)
    const float2 w = __ldg(&tw2[k]);                                            // e^{-i pi k / M}
    const float2 wo = cmul(w, o);
    X[k] = make_float2(e.x + wo.x, e.y + wo.y);
  }
}

// One window of the framed input stream [history | chunk | zeros] per CTA.
__device__ __forceinline__ float framed_at(const double* __restrict__ in, size_t in_stride,
                                           long long count, const float* __restrict__ hist,
                                           long long hlen, int c, long long k) {
  if (k < hlen) return hist[(size_t)c * hlen + k];
  k -= hlen;
  return k < count ? (float)in[(size_t)c * in_stride + k] : 0.0f;
}

__global__ void __launch_bounds__(kFftThreads)
conv_fwd_kernel(const double* __restrict__ in, size_t in_stride, long long count,
                const float* __restrict__ hist, long long hlen, int P, long long wpc,
                const float2* __restrict__ tw2, float2* __restrict__ X) {
  extern __shared__ float2 fsm[];
  const long long m = blockIdx.x;
  const int c = blockIdx.y;
  float2* a = fsm;
  const long long k0 = m * P;
  for (int n = threadIdx.x; n < P; n += blockDim.x)
    a[n] = make_float2(framed_at(in, in_stride, count, hist, hlen, c, k0 + 2 * n),
                       framed_at(in, in_stride, count, hist, hlen, c, k0 + 2 * n + 1));
  __syncthreads();
  rfft_smem(a, fsm + P, P, tw2, X + ((size_t)c * wpc + m) * (P + 1));
}

// IR partition k of channel c (P samples, zero-padded to 2P) per CTA.
__global__ void __launch_bounds__(kFftThreads)
conv_ir_fft_kernel(const float* __restrict__ ir, long long ir_len, int P, int NP,
                   const float2* __restrict__ tw2, float2* __restrict__ H) {
  extern __shared__ float2 fsm[];
  const int k = blockIdx.x, c = blockIdx.y;
  float2* a = fsm;
  for (int n = threadIdx.x; n < P; n += blockDim.x) {
    float v[2];
    for (int h = 0; h < 2; h++) {
      const long long q = 2 * (long long)n + h;
      const long long src = (long long)k * P + q;
      v[h] = (q < P && src < ir_len) ? ir[(size_t)c * ir_len + src] : 0.0f;
    }
    a[n] = make_float2(v[0], v[1]);
  }
  __syncthreads();
  rfft_smem(a, fsm + P, P, tw2, H + ((size_t)c * NP + k) * (P + 1));
}

// One output block per CTA: Z_k = (Y_k + Y*_{M-k}) + i e^{i pi k / M}
// (Y_k - Y*_{M-k}), the inverse FFT, and x[P + t] = the second half of the
// 2P-sample block (x[2n] = Re z_n, x[2n+1] = Im z_n), scaled, to FP64.
__global__ void __launch_bounds__(kFftThreads)
conv_inv_kernel(const float2* __restrict__ Y, int P, long long B, long long count, float scale,
                const float2* __restrict__ tw2, double* __restrict__ out, size_t out_stride) {
  extern __shared__ float2 fsm[];
  const long long bblk = blockIdx.x;
  const int c = blockIdx.y;
  const float2* Yb = Y + ((size_t)c * B + bblk) * (P + 1);
  float2* a = fsm;
  for (int k = threadIdx.x; k < P; k += blockDim.x) {
    const float2 yk = Yb[k];
    const float2 ym = Yb[P - k];
    const float2 e = make_float2(yk.x + ym.x, yk.y - ym.y);    // yk + conj ym
    const float2 d = make_float2(yk.x - ym.x, yk.y + ym.y);    // yk - conj ym
    const float2 w = __ldg(&tw2[k]);
    const float2 o = cmul(make_float2(w.x, -w.y), d);          // e^{+i pi k / M} d
    a[k] = make_float2(e.x - o.y, e.y + o.x);                  // e + i o
  }
  __syncthreads();
  const float2* z = fft_smem<true>(a, fsm + P, P, tw2);
  const long long t0 = bblk * P;
  for (int t = threadIdx.x; t < P; t += blockDim.x) {
    if (t0 + t >= count) break;
    const int j = P + t;
    const float2 v = z[j >> 1];
    out[(size_t)c * out_stride + t0 + t] = (double)(((j & 1) ? v.y : v.x) * scale);
  }
}

// new history = the last hlen samples of (old history ++ chunk)
__global__ void conv_hist_direct_kernel(const double* __restrict__ in, size_t in_stride,
                                        long long count, const float* __restrict__ hist,
                                        long long hlen, int nch, float* __restrict__ nhist) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hlen * nch) return;
  const int c = (int)(i / hlen);
  const long long k = i % hlen;
  nhist[i] = framed_at(in, in_stride, count, hist, hlen, c, count + k);
}

size_t fft_smem_bytes(int P) { return 2 * (size_t)P * sizeof(float2); }

int fft_prepare(int P) {
  static int done[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return -1;
  if (done[dev]) return 0;
  const int bytes = (int)fft_smem_bytes(kOwnFftMaxP);
  if (cudaFuncSetAttribute(conv_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) !=
          cudaSuccess ||
      cudaFuncSetAttribute(conv_inv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) !=
          cudaSuccess ||
      cudaFuncSetAttribute(conv_ir_fft_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           bytes) != cudaSuccess)
    return -1;
  done[dev] = 1;
  (void)P;
  return 0;
}

}  // namespace

struct dsdgpu_conv_state {
  int nch = 0, P = 0, NP = 0;
  long long ir_len = 0;
  bool own_fft = false;             // this file's FFT (P <= 8192) or cuFFT
  cufftComplex* d_H = nullptr;      // [nch][NP][P + 1]
  float* d_hist = nullptr;          // [nch][NP * P]
  float* d_hist2 = nullptr;         // the next chunk's history (own FFT path)
  float2* d_tw2 = nullptr;          // e^{-2 pi i j / (2P)}, j < 2P
  float* d_w = nullptr;             // framed input / C2R output (cuFFT path)
  cufftComplex* d_X = nullptr;
  cufftComplex* d_Y = nullptr;
  size_t w_cap = 0, x_cap = 0, y_cap = 0;
  cufftHandle r2c = 0, c2r = 0;
  long long r2c_batch = -1, c2r_batch = -1;
  ~dsdgpu_conv_state() {
    if (r2c) cufftDestroy(r2c);
    if (c2r) cufftDestroy(c2r);
    for (void* p : {(void*)d_H, (void*)d_hist, (void*)d_hist2, (void*)d_tw2, (void*)d_w,
                    (void*)d_X, (void*)d_Y})
      if (p) cudaFree(p);
  }
};

namespace {

template <typename T>
int grow(T** p, size_t* cap, size_t n) {
  if (*cap >= n) return 0;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  if (cudaMalloc((void**)p, sizeof(T) * n) != cudaSuccess) return -1;
  *cap = n;
  return 0;
}

int plan_r2c(dsdgpu_conv_state* s, long long batch, cudaStream_t st) {
  if (s->r2c_batch == batch) return 0;
  if (s->r2c) cufftDestroy(s->r2c);
  s->r2c = 0;
  int n = 2 * s->P;
  int inembed = n, onembed = s->P + 1;
  if (cufftPlanMany(&s->r2c, 1, &n, &inembed, 1, s->P, &onembed, 1, s->P + 1, CUFFT_R2C,
                    (int)batch) != CUFFT_SUCCESS)
    return -1;
  cufftSetStream(s->r2c, st);
  s->r2c_batch = batch;
  return 0;
}

int plan_c2r(dsdgpu_conv_state* s, long long batch, cudaStream_t st) {
  if (s->c2r_batch == batch) return 0;
  if (s->c2r) cufftDestroy(s->c2r);
  s->c2r = 0;
  int n = 2 * s->P;
  int inembed = s->P + 1, onembed = n;
  if (cufftPlanMany(&s->c2r, 1, &n, &inembed, 1, s->P + 1, &onembed, 1, n, CUFFT_C2R,
                    (int)batch) != CUFFT_SUCCESS)
    return -1;
  cufftSetStream(s->c2r, st);
  s->c2r_batch = batch;
  return 0;
}

int launch_mac(int NP, const cufftComplex* X, const cufftComplex* H, cufftComplex* Y, int bins,
               long long B, long long wpc, int nch, cudaStream_t st) {
  const dim3 grid(blocks_of(bins, 128), (unsigned)((B + kMacRun - 1) / kMacRun), (unsigned)nch);
  switch (NP) {
#define MAC_CASE(K) case K: conv_mac_kernel<K><<<grid, 128, 0, st>>>(X, H, Y, bins, B, wpc, nch); break;
    MAC_CASE(1) MAC_CASE(2) MAC_CASE(4) MAC_CASE(8) MAC_CASE(16) MAC_CASE(32)
#undef MAC_CASE
    default: return -1;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace

void conv_free(dsdgpu_conv_state* s) { delete s; }

// Convolve chunk (in -> out, may alias) with the context's IRs; history carried.
int conv_run(dsdgpu_context* c, int nch, const double* d_in, size_t in_stride, size_t count,
             double* d_out, size_t out_stride) {
  dsdgpu_conv_state* s = c->conv;
  if (!s) return c->fail(DSDGPU_ERR_STATE, "convolution not set up");
  if (nch != s->nch) return c->fail(DSDGPU_ERR_ARG, "channel count differs from the IR set");
  if (count == 0) return DSDGPU_OK;
  cudaStream_t st = c->stream;
  const int P = s->P, NP = s->NP, bins = P + 1;
  const long long B = ((long long)count + P - 1) / P;
  const long long wpc = B + NP;                       // windows per channel (the last unused)
  const long long L = wpc * P;                        // framed samples per channel
  const long long hlen = (long long)NP * P;
  if (s->own_fft) {
    if (grow(&s->d_X, &s->x_cap, (size_t)(nch * wpc) * bins) ||
        grow(&s->d_Y, &s->y_cap, (size_t)(nch * B) * bins))
      return c->cuda_fail(cudaGetLastError(), "convolution buffers");
    if (fft_prepare(P)) return c->cuda_fail(cudaGetLastError(), "fft kernel attributes");
    const size_t smem = fft_smem_bytes(P);
    conv_fwd_kernel<<<dim3((unsigned)(wpc - 1), (unsigned)nch), kFftThreads, smem, st>>>(
        d_in, in_stride, (long long)count, s->d_hist, hlen, P, wpc, s->d_tw2,
        reinterpret_cast<float2*>(s->d_X));
    c->launches++;
    conv_hist_direct_kernel<<<blocks_of(hlen * nch, 256), 256, 0, st>>>(
        d_in, in_stride, (long long)count, s->d_hist, hlen, nch, s->d_hist2);
    c->launches++;
    std::swap(s->d_hist, s->d_hist2);
    if (launch_mac(NP, s->d_X, s->d_H, s->d_Y, bins, B, wpc, nch, st))
      return c->cuda_fail(cudaGetLastError(), "convolution MAC");
    c->launches++;
    conv_inv_kernel<<<dim3((unsigned)B, (unsigned)nch), kFftThreads, smem, st>>>(
        reinterpret_cast<const float2*>(s->d_Y), P, B, (long long)count, 1.0f / (float)(2 * P),
        s->d_tw2, d_out, out_stride);
    c->launches++;
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? DSDGPU_OK : c->cuda_fail(e, "convolution launch");
  }
  const size_t wlen = std::max((size_t)(L * nch), (size_t)(nch * B * 2 * P));
  if (grow(&s->d_w, &s->w_cap, wlen) || grow(&s->d_X, &s->x_cap, (size_t)(nch * wpc) * bins) ||
      grow(&s->d_Y, &s->y_cap, (size_t)(nch * B) * bins))
    return c->cuda_fail(cudaGetLastError(), "convolution buffers");
  conv_frame_kernel<<<blocks_of(L * nch, 256), 256, 0, st>>>(d_in, in_stride, (long long)count,
                                                             s->d_hist, hlen, L, nch, s->d_w);
  c->launches++;
  if (plan_r2c(s, (long long)nch * wpc - 1, st)) return c->fail(DSDGPU_ERR_CUDA, "cuFFT R2C plan");
  if (cufftExecR2C(s->r2c, s->d_w, s->d_X) != CUFFT_SUCCESS)
    return c->fail(DSDGPU_ERR_CUDA, "cuFFT R2C");
  // history for the next chunk (before the framed buffer is reused)
  conv_hist_kernel<<<blocks_of(hlen * nch, 256), 256, 0, st>>>(s->d_w, L, hlen, (long long)count,
                                                               nch, s->d_hist);
  c->launches++;
  if (launch_mac(NP, s->d_X, s->d_H, s->d_Y, bins, B, wpc, nch, st))
    return c->cuda_fail(cudaGetLastError(), "convolution MAC");
  c->launches++;
  if (plan_c2r(s, (long long)nch * B, st)) return c->fail(DSDGPU_ERR_CUDA, "cuFFT C2R plan");
  if (cufftExecC2R(s->c2r, s->d_Y, s->d_w) != CUFFT_SUCCESS)
    return c->fail(DSDGPU_ERR_CUDA, "cuFFT C2R");
  conv_gather_kernel<<<blocks_of((long long)count * nch, 256), 256, 0, st>>>(
      s->d_w, P, B, (long long)count, nch, 1.0f / (float)(2 * P), d_out, out_stride);
  c->launches++;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? DSDGPU_OK : c->cuda_fail(e, "convolution launch");
}

extern "C" {

int dsdgpu_conv_setup(dsdgpu_context_t* c, const float* ir, size_t ir_len, int nch, int partition) {
  if (!c || !ir || ir_len == 0 || nch < 1) return DSDGPU_ERR_ARG;
  if (partition < 64 || partition > (1 << 16) || (partition & (partition - 1)))
    return c->fail(DSDGPU_ERR_ARG, "partition must be a power of two in 64..65536");
  const long long np = ((long long)ir_len + partition - 1) / partition;
  if (np > kMaxParts) return c->fail(DSDGPU_ERR_UNSUPPORTED, "IR longer than 32 partitions");
  cudaSetDevice(c->device);
  dsdgpu_conv_state* s = new (std::nothrow) dsdgpu_conv_state();
  if (!s) return DSDGPU_ERR_NOMEM;
  s->nch = nch;
  s->P = partition;
  s->NP = round_parts((int)np);
  s->ir_len = (long long)ir_len;
  s->own_fft = partition <= kOwnFftMaxP;
  const int P = s->P, NP = s->NP, bins = P + 1;
  cudaStream_t st = c->stream;
  float* d_ir = nullptr;
  float* d_frame = nullptr;
  cufftHandle plan = 0;
  int rc = DSDGPU_OK;
  if (cudaMalloc(&s->d_H, sizeof(cufftComplex) * (size_t)nch * NP * bins) != cudaSuccess ||
      cudaMalloc(&s->d_hist, sizeof(float) * (size_t)nch * NP * P) != cudaSuccess ||
      cudaMalloc(&d_ir, sizeof(float) * (size_t)nch * ir_len) != cudaSuccess ||
      (!s->own_fft &&
       cudaMalloc(&d_frame, sizeof(float) * (size_t)nch * NP * 2 * P) != cudaSuccess)) {
    rc = c->cuda_fail(cudaGetLastError(), "convolution setup allocation");
  }
  if (!rc && s->own_fft) {
    // twiddle table in FP64 rounded to FP32, the IR partitions by the same FFT
    std::vector<float2> tw((size_t)2 * P);
    const double pi = 3.14159265358979323846;
    for (int j = 0; j < 2 * P; j++) {
      const double ang = -2.0 * pi * (double)j / (double)(2 * P);
      tw[j] = make_float2((float)std::cos(ang), (float)std::sin(ang));
    }
    if (cudaMalloc(&s->d_tw2, sizeof(float2) * tw.size()) != cudaSuccess ||
        cudaMalloc(&s->d_hist2, sizeof(float) * (size_t)nch * NP * P) != cudaSuccess ||
        fft_prepare(P) != 0) {
      rc = c->cuda_fail(cudaGetLastError(), "convolution setup allocation");
    } else {
      cudaMemsetAsync(s->d_hist, 0, sizeof(float) * (size_t)nch * NP * P, st);
      cudaMemcpyAsync(s->d_tw2, tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(d_ir, ir, sizeof(float) * (size_t)nch * ir_len, cudaMemcpyHostToDevice, st);
      conv_ir_fft_kernel<<<dim3((unsigned)NP, (unsigned)nch), kFftThreads, fft_smem_bytes(P), st>>>(
          d_ir, (long long)ir_len, P, NP, s->d_tw2, reinterpret_cast<float2*>(s->d_H));
      c->launches++;
      if (cudaGetLastError() != cudaSuccess) rc = c->fail(DSDGPU_ERR_CUDA, "IR partition FFT");
    }
  } else if (!rc) {
    cudaMemsetAsync(s->d_hist, 0, sizeof(float) * (size_t)nch * NP * P, st);
    cudaMemcpyAsync(d_ir, ir, sizeof(float) * (size_t)nch * ir_len, cudaMemcpyHostToDevice, st);
    const long long tot = (long long)nch * NP * 2 * P;
    conv_ir_frame_kernel<<<blocks_of(tot, 256), 256, 0, st>>>(d_ir, (long long)ir_len, P, NP, nch,
                                                              d_frame);
    c->launches++;
    int n = 2 * P;
    if (cufftPlan1d(&plan, n, CUFFT_R2C, nch * NP) != CUFFT_SUCCESS ||
        cufftSetStream(plan, st) != CUFFT_SUCCESS ||
        cufftExecR2C(plan, d_frame, s->d_H) != CUFFT_SUCCESS)
      rc = c->fail(DSDGPU_ERR_CUDA, "cuFFT of the IR partitions");
  }
  if (!rc) rc = c->check_status();
  if (plan) cufftDestroy(plan);
  if (d_ir) cudaFree(d_ir);
  if (d_frame) cudaFree(d_frame);
  if (rc) {
    delete s;
    return rc;
  }
  conv_free(c->conv);
  c->conv = s;
  return DSDGPU_OK;
}

int dsdgpu_conv_reset(dsdgpu_context_t* c) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->conv) return c->fail(DSDGPU_ERR_STATE, "convolution not set up");
  cudaSetDevice(c->device);
  dsdgpu_conv_state* s = c->conv;
  cudaMemsetAsync(s->d_hist, 0, sizeof(float) * (size_t)s->nch * s->NP * s->P, c->stream);
  return c->check_status();
}

int dsdgpu_conv_clear(dsdgpu_context_t* c) {
  if (!c) return DSDGPU_ERR_ARG;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  conv_free(c->conv);
  c->conv = nullptr;
  return DSDGPU_OK;
}

int dsdgpu_conv_process(dsdgpu_context_t* c, int nch, const double* d_in, size_t in_stride,
                        size_t count, double* d_out, size_t out_stride) {
  if (!c || nch < 1 || (count > 0 && (!d_in || !d_out))) return DSDGPU_ERR_ARG;
  cudaSetDevice(c->device);
  const int rc = conv_run(c, nch, d_in, in_stride, count, d_out, out_stride);
  return rc ? rc : c->check_status();
}

}  // extern "C"
