// PreCorr (predictive-correction) SDM on sm_103a: the reference's greedy
// single-precision quantiser with a trained correction table (reference
// src/precorr.c:141-287, include/precorr.h:49-61; its own GPU form is one
// thread per channel, src/kernels/sdm_kernels.cu:222-292).
//
//   precorr_train_kernel    one CTA: the 256 x 8 table of mean quantiser
//                           residuals over 65,536 samples of LCG noise at
//                           amplitude 0.1 (src/precorr.c:141-196) — the walk is
//                           serial, so one thread runs it with the sums in
//                           shared memory, then the CTA divides
//   narrow_rows_kernel      FP64 input rows narrowed to FP32 in one wide pass
//                           (the walk reads floats, as the reference's does;
//                           the pipeline's PCM path has the FIR chain write
//                           FP32 and skips this pass)
//   precorr_process_kernel  one thread per channel, the table in shared memory:
//                           NTF loop, greedy sign, state limiter, correction
//                           from table[history][phase], re-quantise
//                           (src/precorr.c:222-270)
//
// Every FP32 operation is an explicitly rounded intrinsic in the reference's
// order (left to right, no contraction), so the decisions equal the
// reference's CPU build bit for bit; the reference's own GPU kernel is built
// with contraction on and can differ from its CPU path.  Per channel the loop
// is a latency chain through the previous output (about fifteen dependent
// FP32 operations per sample), so throughput is one sample per chain latency
// per channel; the next 16 inputs and the next step's two candidate
// corrections are loaded ahead of the chain to keep load latency off it.
#include "api_context.h"

#include <algorithm>
#include <cstring>

using namespace dsdgpu;

namespace {

constexpr int kPcHist = 256;
constexpr int kPcPhases = 8;
constexpr int kPcTable = kPcHist * kPcPhases;
constexpr int kPcTrain = 65536;
constexpr int kPcMinHits = 4;
constexpr unsigned kPcHistInit = 0x69u;

struct PcCoef {
  float a[10];
  float g[10];
  int order;
  float limit;
};

// per-channel state carried between calls
struct PcState {
  float s[10];
  float prev_y;
  unsigned history;
  int phase;
  int pad;
};

// NTF filter step (src/precorr.c:20-126): d[] from the state, the input and
// the previous output; returns v.  `t0` = (s0 - g0*s1) + x is computed ahead
// of the previous output, so only d0 = t0 - y sits on the output chain.
template <int N>
__device__ __forceinline__ float pc_filter(const float (&s)[10], float (&d)[10], const PcCoef& C,
                                           float x, float y) {
  const float t0 = __fadd_rn(__fsub_rn(s[0], __fmul_rn(C.g[0], s[1])), x);
#pragma unroll
  for (int i = 1; i < N - 1; i++) d[i] = __fsub_rn(__fadd_rn(s[i], s[i - 1]), __fmul_rn(C.g[i], s[i + 1]));
  d[N - 1] = __fadd_rn(s[N - 1], s[N - 2]);
  d[0] = __fsub_rn(t0, y);
  float v = __fadd_rn(x, __fmul_rn(C.a[0], d[0]));
#pragma unroll
  for (int i = 1; i < N; i++) v = __fadd_rn(v, __fmul_rn(C.a[i], d[i]));
  return v;
}

// The reference's lcg_float (src/precorr.c:128-139): a * ((float)(int32)r / 2^31).
__device__ __forceinline__ float pc_lcg(uint32_t& r) {
  r = r * 1664525u + 1013904223u;
  return __fmul_rn(0.1f, __fdiv_rn(__int2float_rn((int)r), 2147483648.0f));
}

template <int N>
__device__ void pc_train(const PcCoef& C, float* acc, int* hits) {
  float s[10] = {0}, d[10] = {0};
  unsigned hist = kPcHistInit;
  int ph = 0;
  float py = 0.0f;
  uint32_t r = 0xDEADBEEFu;
  for (int i = 0; i < kPcTrain; i++) {
    const float x = pc_lcg(r);
    const float v = pc_filter<N>(s, d, C, x, py);
    const float y = v >= 0.0f ? 1.0f : -1.0f;
#pragma unroll
    for (int k = 0; k < N; k++) s[k] = d[k];
    const int cell = (int)hist * kPcPhases + ph;
    acc[cell] = __fadd_rn(acc[cell], __fsub_rn(y, v));
    hits[cell]++;
    hist = ((hist << 1) | (y > 0.0f ? 1u : 0u)) & 0xFFu;
    ph = (ph + 1) & (kPcPhases - 1);
    py = y;
  }
}

__global__ void __launch_bounds__(256) precorr_train_kernel(const __grid_constant__ PcCoef C,
                                                            float* __restrict__ table) {
  __shared__ float acc[kPcTable];
  __shared__ int hits[kPcTable];
  for (int i = threadIdx.x; i < kPcTable; i += blockDim.x) {
    acc[i] = 0.0f;
    hits[i] = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    switch (C.order) {
      case 2: pc_train<2>(C, acc, hits); break;
      case 3: pc_train<3>(C, acc, hits); break;
      case 4: pc_train<4>(C, acc, hits); break;
      case 5: pc_train<5>(C, acc, hits); break;
      case 6: pc_train<6>(C, acc, hits); break;
      case 7: pc_train<7>(C, acc, hits); break;
      case 8: pc_train<8>(C, acc, hits); break;
      case 9: pc_train<9>(C, acc, hits); break;
      default: pc_train<10>(C, acc, hits); break;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kPcTable; i += blockDim.x)
    table[i] = hits[i] >= kPcMinHits ? __fdiv_rn(acc[i], __int2float_rn(hits[i])) : 0.0f;
}

constexpr int kPcAhead = 16;

// The reference's limiter (if d > L: L; else if d < -L: -L) for L > 0.  NaN
// stays NaN (max/min with .NaN propagate it; comparisons with any NaN are
// false, so the decisions do not depend on its payload).
__device__ __forceinline__ float pc_clamp(float d, float lo, float hi) {
  float r;
  asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(d), "f"(lo));
  asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(r), "f"(hi));
  return r;
}

// Decision code of a table cell c: bit 0 = the output for v >= 0 (y = +1),
// bit 1 = the output for v < 0 (y = -1), out = (y - c >= 0)
// (src/precorr.c:252-256).  The walk reads the codes of a history's two
// successors at the next phase (histories 2h and 2h + 1, low 8 bits) as one
// byte: codes[phase][h] = code(2h & 0xFF) | code((2h + 1) & 0xFF) << 2, where
// `phase` is the successors' phase.
__device__ __forceinline__ unsigned pc_code(float c) {
  return (__fsub_rn(1.0f, c) >= 0.0f ? 1u : 0u) | (__fsub_rn(-1.0f, c) >= 0.0f ? 2u : 0u);
}

// Walk state of one channel in registers.  The previous output enters v only
// through d0 = t0 - y at the head of v's sum, so each step forms v for both
// y = +1 and y = -1 (two independent chains) and picks one with the previous
// bit: the serial dependence per sample is a select, a compare and a select.
template <int N, bool LIM>
struct PcWalk {
  PcCoef C;
  float L;
  float s[10];
  unsigned pbit;   // previous output bit (prev_y = +1 / -1)
  unsigned hist;   // last 8 output bits
  unsigned code;   // decision code of this step's cell

  // one sample with prev_y = +-1; `row` = codes of the next step's phase
  __device__ __forceinline__ unsigned step(const uint8_t* row, float x) {
    const unsigned pair = row[hist];
    float d[10];
    const float t0 = __fadd_rn(__fsub_rn(s[0], __fmul_rn(C.g[0], s[1])), x);
#pragma unroll
    for (int i = 1; i < N - 1; i++) d[i] = __fsub_rn(__fadd_rn(s[i], s[i - 1]), __fmul_rn(C.g[i], s[i + 1]));
    d[N - 1] = __fadd_rn(s[N - 1], s[N - 2]);
    const float dp = __fsub_rn(t0, 1.0f), dn = __fsub_rn(t0, -1.0f);
    float vp = __fadd_rn(x, __fmul_rn(C.a[0], dp));
    float vn = __fadd_rn(x, __fmul_rn(C.a[0], dn));
#pragma unroll
    for (int i = 1; i < N; i++) {
      const float p = __fmul_rn(C.a[i], d[i]);
      vp = __fadd_rn(vp, p);
      vn = __fadd_rn(vn, p);
    }
    d[0] = pbit ? dp : dn;
    const float v = pbit ? vp : vn;
    if (LIM) {
#pragma unroll
      for (int k = 0; k < N; k++) d[k] = pc_clamp(d[k], -L, L);
    }
#pragma unroll
    for (int k = 0; k < N; k++) s[k] = d[k];
    const unsigned bit = (v >= 0.0f ? code : code >> 1) & 1u;
    hist = ((hist << 1) | bit) & 0xFFu;
    pbit = bit;
    code = bit ? pair >> 2 : pair & 3u;
    return bit;
  }
};

// The first sample after a reset (prev_y = 0): the plain step.
template <int N, bool LIM>
__device__ __forceinline__ unsigned pc_first_step(PcWalk<N, LIM>& W, const uint8_t* row, float x) {
  const unsigned pair = row[W.hist];
  float d[10];
  const float v = pc_filter<N>(W.s, d, W.C, x, 0.0f);
  if (LIM) {
#pragma unroll
    for (int k = 0; k < N; k++) d[k] = pc_clamp(d[k], -W.L, W.L);
  }
#pragma unroll
  for (int k = 0; k < N; k++) W.s[k] = d[k];
  const unsigned bit = (v >= 0.0f ? W.code : W.code >> 1) & 1u;
  W.hist = ((W.hist << 1) | bit) & 0xFFu;
  W.pbit = bit;
  W.code = bit ? pair >> 2 : pair & 3u;
  return bit;
}

template <int N, bool LIM>
__device__ void pc_run(const PcCoef& Cg, const uint8_t* codes, PcState& st,
                       const float* __restrict__ x, long long count, uint8_t* __restrict__ out) {
  PcWalk<N, LIM> W;
#pragma unroll
  for (int k = 0; k < N; k++) {
    W.C.a[k] = Cg.a[k];
    W.C.g[k] = Cg.g[k];
  }
  W.L = Cg.limit;
#pragma unroll
  for (int k = 0; k < 10; k++) W.s[k] = st.s[k];
  W.pbit = st.prev_y > 0.0f ? 1u : 0u;
  W.hist = st.history;
  int ph0 = st.phase;   // phase of the next sample
  {
    // this step's code: successors of the previous history, at phase ph0
    const unsigned pair = codes[ph0 * kPcHist + (int)(W.hist >> 1)];
    W.code = (W.hist & 1u) ? pair >> 2 : pair & 3u;
  }
  const bool any = count > 0;
  if (any && st.prev_y == 0.0f) {
    *out++ = (uint8_t)pc_first_step(W, codes + ((ph0 + 1) & 7) * kPcHist, *x++);
    count--;
    ph0 = (ph0 + 1) & 7;
  }
  // codes row of the successors of step j of a chunk (chunks keep the phase)
  const uint8_t* rows[kPcPhases];
#pragma unroll
  for (int r = 0; r < kPcPhases; r++) rows[r] = codes + ((ph0 + r + 1) & 7) * kPcHist;
  const bool vec_out = ((uintptr_t)out & 15u) == 0;
  float xa[kPcAhead];
#pragma unroll
  for (int j = 0; j < kPcAhead; j++) xa[j] = j < count ? x[j] : 0.0f;
  long long base = 0;
  // whole chunks: straight-line code over kPcAhead samples, the next chunk's
  // inputs in flight meanwhile (converted when used)
  for (; base + kPcAhead <= count; base += kPcAhead) {
    float xb[kPcAhead];
    if (base + 2 * kPcAhead <= count) {
#pragma unroll
      for (int j = 0; j < kPcAhead; j++) xb[j] = x[base + kPcAhead + j];
    } else {
#pragma unroll
      for (int j = 0; j < kPcAhead; j++) {
        const long long i = base + kPcAhead + j;
        xb[j] = i < count ? x[i] : 0.0f;
      }
    }
    unsigned w[kPcAhead / 4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int j = 0; j < kPcAhead; j++) w[j >> 2] |= W.step(rows[j & 7], xa[j]) << (8 * (j & 3));
    if (vec_out) {
      *reinterpret_cast<uint4*>(out + base) = make_uint4(w[0], w[1], w[2], w[3]);
    } else {
#pragma unroll
      for (int j = 0; j < kPcAhead; j++) out[base + j] = (uint8_t)((w[j >> 2] >> (8 * (j & 3))) & 1u);
    }
#pragma unroll
    for (int j = 0; j < kPcAhead; j++) xa[j] = xb[j];
  }
  // the ragged tail
  const int m = (int)(count - base);
#pragma unroll
  for (int j = 0; j < kPcAhead; j++)
    if (j < m) out[base + j] = (uint8_t)W.step(rows[j & 7], xa[j]);
#pragma unroll
  for (int k = 0; k < 10; k++) st.s[k] = W.s[k];
  if (any) st.prev_y = W.pbit ? 1.0f : -1.0f;
  st.history = W.hist;
  st.phase = (int)((ph0 + count) & 7);
}

template <int N>
__device__ __forceinline__ void pc_run_lim(const PcCoef& C, const uint8_t* codes, PcState& st,
                                           const float* x, long long count, uint8_t* out) {
  if (C.limit > 0.0f) pc_run<N, true>(C, codes, st, x, count, out);
  else pc_run<N, false>(C, codes, st, x, count, out);
}

__global__ void __launch_bounds__(32) precorr_process_kernel(const __grid_constant__ PcCoef C,
                                                             const float* __restrict__ table,
                                                             PcState* __restrict__ states, int nch,
                                                             const float* __restrict__ in,
                                                             size_t in_stride, long long count,
                                                             uint8_t* __restrict__ bits,
                                                             size_t bits_stride) {
  __shared__ uint8_t codes[kPcPhases * kPcHist];
  for (int i = threadIdx.x; i < kPcPhases * kPcHist; i += blockDim.x) {
    const int ph = i / kPcHist, h2 = (2 * (i % kPcHist)) & 0xFF;
    codes[i] = (uint8_t)(pc_code(table[h2 * kPcPhases + ph]) |
                         (pc_code(table[(h2 + 1) * kPcPhases + ph]) << 2));
  }
  __syncthreads();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nch) return;
  PcState st = states[c];
  const float* x = in + (size_t)c * in_stride;
  uint8_t* o = bits + (size_t)c * bits_stride;
  switch (C.order) {
    case 2: pc_run_lim<2>(C, codes, st, x, count, o); break;
    case 3: pc_run_lim<3>(C, codes, st, x, count, o); break;
    case 4: pc_run_lim<4>(C, codes, st, x, count, o); break;
    case 5: pc_run_lim<5>(C, codes, st, x, count, o); break;
    case 6: pc_run_lim<6>(C, codes, st, x, count, o); break;
    case 7: pc_run_lim<7>(C, codes, st, x, count, o); break;
    case 8: pc_run_lim<8>(C, codes, st, x, count, o); break;
    case 9: pc_run_lim<9>(C, codes, st, x, count, o); break;
    default: pc_run_lim<10>(C, codes, st, x, count, o); break;
  }
  states[c] = st;
}

// precorr_context_reset (src/precorr.c:279-287): zero state, history 0x69,
// phase 0, previous output 0; the table is kept.
__global__ void precorr_reset_kernel(PcState* states, int nch) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nch) return;
  PcState st;
  for (int k = 0; k < 10; k++) st.s[k] = 0.0f;
  st.prev_y = 0.0f;
  st.history = kPcHistInit;
  st.phase = 0;
  st.pad = 0;
  states[c] = st;
}

// The batch plan's PreCorr streams: one thread per row (a channel of a
// stream), each from fresh state (precorr_context_init) over its own count,
// rows of one class (NTF and limit) per launch.
__global__ void __launch_bounds__(32) precorr_batch_kernel(const __grid_constant__ PcCoef C,
                                                           const float* __restrict__ table,
                                                           const PcBatchRow* __restrict__ rows,
                                                           int nrows) {
  __shared__ uint8_t codes[kPcPhases * kPcHist];
  for (int i = threadIdx.x; i < kPcPhases * kPcHist; i += blockDim.x) {
    const int ph = i / kPcHist, h2 = (2 * (i % kPcHist)) & 0xFF;
    codes[i] = (uint8_t)(pc_code(table[h2 * kPcPhases + ph]) |
                         (pc_code(table[(h2 + 1) * kPcPhases + ph]) << 2));
  }
  __syncthreads();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const PcBatchRow row = rows[r];
  PcState st;
  for (int k = 0; k < 10; k++) st.s[k] = 0.0f;
  st.prev_y = 0.0f;
  st.history = kPcHistInit;
  st.phase = 0;
  st.pad = 0;
  switch (C.order) {
    case 2: pc_run_lim<2>(C, codes, st, row.in, row.count, row.out); break;
    case 3: pc_run_lim<3>(C, codes, st, row.in, row.count, row.out); break;
    case 4: pc_run_lim<4>(C, codes, st, row.in, row.count, row.out); break;
    case 5: pc_run_lim<5>(C, codes, st, row.in, row.count, row.out); break;
    case 6: pc_run_lim<6>(C, codes, st, row.in, row.count, row.out); break;
    case 7: pc_run_lim<7>(C, codes, st, row.in, row.count, row.out); break;
    case 8: pc_run_lim<8>(C, codes, st, row.in, row.count, row.out); break;
    case 9: pc_run_lim<9>(C, codes, st, row.in, row.count, row.out); break;
    default: pc_run_lim<10>(C, codes, st, row.in, row.count, row.out); break;
  }
}

// FP64 rows narrowed to FP32 in one wide pass (all lanes of every warp
// busy), so the walk's loop carries no conversion: out[ch][j] =
// float(in[ch][j]), rounded to nearest as the walk would round them.
__global__ void narrow_rows_kernel(const double* __restrict__ in, size_t in_stride,
                                   long long count, float* __restrict__ out) {
  const int ch = blockIdx.y;
  const double* x = in + (size_t)ch * in_stride;
  float* y = out + (size_t)ch * (size_t)count;
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < count;
       j += (long long)gridDim.x * blockDim.x)
    y[j] = __double2float_rn(x[j]);
}

}  // namespace

struct dsdgpu_precorr_state {
  PcCoef coef{};
  int nch = 0;
  float* d_table = nullptr;
  PcState* d_states = nullptr;
  float* d_f32 = nullptr;   // FP64 input narrowed ahead of the walk
  size_t f32_cap = 0;
  ~dsdgpu_precorr_state() {
    if (d_table) cudaFree(d_table);
    if (d_states) cudaFree(d_states);
    if (d_f32) cudaFree(d_f32);
  }
};

void precorr_free(dsdgpu_precorr_state* s) { delete s; }

// precorr_context_init's float copies of the coefficients (src/precorr.c:198-220).
static PcCoef pc_coef(int order, const double* a, const double* g, double limit) {
  PcCoef C{};
  C.order = order;
  for (int i = 0; i < 10; i++) {
    C.a[i] = i < order ? (float)a[i] : 0.0f;
    C.g[i] = i < order ? (float)g[i] : 0.0f;
  }
  C.limit = (float)limit;
  return C;
}

size_t precorr_table_floats() { return (size_t)kPcTable; }

int precorr_batch_train(int order, const double* a, const double* g, double limit, float* d_table,
                        cudaStream_t stream) {
  precorr_train_kernel<<<1, 256, 0, stream>>>(pc_coef(order, a, g, limit), d_table);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

int launch_precorr_batch(int order, const double* a, const double* g, double limit,
                         const float* d_table, const PcBatchRow* d_rows, int nrows,
                         cudaStream_t stream) {
  if (nrows <= 0) return 0;
  precorr_batch_kernel<<<(nrows + 31) / 32, 32, 0, stream>>>(pc_coef(order, a, g, limit), d_table,
                                                            d_rows, nrows);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// The pipeline's SDM stage in PreCorr mode (src/engine.c:557-559, 723-726):
// FP32 input (the reference's walk reads floats).
int precorr_run(dsdgpu_context_t* c, int first, int nch, const float* d_in, size_t in_stride,
                size_t count, uint8_t* d_bits, size_t bits_stride) {
  dsdgpu_precorr_state* s = c->precorr;
  precorr_process_kernel<<<(nch + 31) / 32, 32, 0, c->stream>>>(
      s->coef, s->d_table, s->d_states + first, nch, d_in, in_stride, (long long)count, d_bits,
      bits_stride);
  c->launches++;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? DSDGPU_OK : c->cuda_fail(e, "precorr launch");
}

// FP64 input: narrowed to FP32 rows first (one wide pass), then the FP32
// walk.  A per-sample conversion inside the walk sits on its loop-carried
// chain (measured 4.0 s against 3.0 s per 10 s stereo call).
int precorr_run(dsdgpu_context_t* c, int first, int nch, const double* d_in, size_t in_stride,
                size_t count, uint8_t* d_bits, size_t bits_stride) {
  if (count == 0) return DSDGPU_OK;
  dsdgpu_precorr_state* s = c->precorr;
  const size_t need = (size_t)nch * count;
  if (need > s->f32_cap) {
    if (s->d_f32) cudaFree(s->d_f32);
    s->d_f32 = nullptr;
    s->f32_cap = 0;
    const cudaError_t e = cudaMalloc(&s->d_f32, sizeof(float) * need);
    if (e != cudaSuccess) return c->cuda_fail(e, "precorr narrowing buffer");
    s->f32_cap = need;
  }
  const int bx = (int)std::min<long long>((long long)(count + 255) / 256,
                                          (long long)(c->num_sms > 0 ? c->num_sms : 148) * 8);
  narrow_rows_kernel<<<dim3((unsigned)bx, (unsigned)nch), 256, 0, c->stream>>>(
      d_in, in_stride, (long long)count, s->d_f32);
  c->launches++;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "precorr narrowing launch");
  return precorr_run(c, first, nch, (const float*)s->d_f32, count, count, d_bits, bits_stride);
}

extern "C" {

int dsdgpu_precorr_setup(dsdgpu_context_t* c, int order, const double* a, const double* g,
                         double state_limit, int nch) {
  if (!c || !a || !g || nch < 1) return DSDGPU_ERR_ARG;
  if (order < 2 || order > 10) return c->fail(DSDGPU_ERR_ARG, "NTF order out of range (2..10)");
  if (!(state_limit >= 0.0)) return c->fail(DSDGPU_ERR_ARG, "state limit must be >= 0");
  cudaSetDevice(c->device);
  dsdgpu_precorr_state* s = new (std::nothrow) dsdgpu_precorr_state();
  if (!s) return DSDGPU_ERR_NOMEM;
  s->coef = pc_coef(order, a, g, state_limit);
  s->nch = nch;
  if (cudaMalloc(&s->d_table, sizeof(float) * kPcTable) != cudaSuccess ||
      cudaMalloc(&s->d_states, sizeof(PcState) * (size_t)nch) != cudaSuccess) {
    delete s;
    return c->cuda_fail(cudaGetLastError(), "precorr allocation");
  }
  precorr_train_kernel<<<1, 256, 0, c->stream>>>(s->coef, s->d_table);
  precorr_reset_kernel<<<(nch + 127) / 128, 128, 0, c->stream>>>(s->d_states, nch);
  c->launches += 2;
  precorr_free(c->precorr);
  c->precorr = s;
  return c->check_status();
}

int dsdgpu_precorr_reset(dsdgpu_context_t* c) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->precorr) return c->fail(DSDGPU_ERR_STATE, "precorr not set up");
  cudaSetDevice(c->device);
  precorr_reset_kernel<<<(c->precorr->nch + 127) / 128, 128, 0, c->stream>>>(c->precorr->d_states,
                                                                             c->precorr->nch);
  c->launches++;
  return c->check_status();
}

int dsdgpu_precorr_table(dsdgpu_context_t* c, float* h_table) {
  if (!c || !h_table) return DSDGPU_ERR_ARG;
  if (!c->precorr) return c->fail(DSDGPU_ERR_STATE, "precorr not set up");
  cudaSetDevice(c->device);
  const cudaError_t e = cudaMemcpyAsync(h_table, c->precorr->d_table, sizeof(float) * kPcTable,
                                        cudaMemcpyDeviceToHost, c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "precorr table download");
  return c->check_status();
}

int dsdgpu_precorr_process_async(dsdgpu_context_t* c, int first, int nch, const double* d_in,
                                 size_t in_stride, size_t count, uint8_t* d_bits,
                                 size_t bits_stride) {
  if (!c) return DSDGPU_ERR_ARG;
  if (!c->precorr) return c->fail(DSDGPU_ERR_STATE, "precorr not set up");
  if (first < 0 || nch < 1 || first + nch > c->precorr->nch)
    return c->fail(DSDGPU_ERR_ARG, "bad channel range");
  if (count == 0) return DSDGPU_OK;
  if (!d_in || !d_bits) return c->fail(DSDGPU_ERR_ARG, "null buffer");
  if (nch > 1 && (in_stride < count || bits_stride < count))
    return c->fail(DSDGPU_ERR_ARG, "row stride shorter than the count");
  cudaSetDevice(c->device);
  return precorr_run(c, first, nch, d_in, in_stride, count, d_bits, bits_stride);
}

int dsdgpu_precorr_process(dsdgpu_context_t* c, int first, int nch, const double* d_in,
                           size_t in_stride, size_t count, uint8_t* d_bits, size_t bits_stride) {
  const int rc = dsdgpu_precorr_process_async(c, first, nch, d_in, in_stride, count, d_bits,
                                              bits_stride);
  return rc ? rc : c->check_status();
}

}  // extern "C"
