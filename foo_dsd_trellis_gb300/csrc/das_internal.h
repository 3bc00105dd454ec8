// Device-side plan records of the DAS pipeline.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace dsdgpu {

// One seam search: boundary `boundary` compares prev[0..ovl_len) (the last
// decisions of the stream before the seam, inside segment prev_seg's buffer at
// prev_off) with next[0..ovl_len) (segment `boundary`'s first decisions).
struct SeamTask {
  const uint8_t* prev;
  const uint8_t* next;
  long long prev_off;
  int boundary;           // index into the seam-position array
  int ovl_len;
  int prev_seg;
  int lat;                // trellis latency of the stream (density window)
};

constexpr int kSeamThreads = 512;
constexpr int kMaxSeamOverlap = 32 * kSeamThreads;   // density values held per thread

// One gather range of the final stream: segment `seg` supplies stream
// positions [base + (stitched ? bp[seg] : 0), end), where end is the next
// piece's start (next_base + bp[next_seg] when that piece is stitched) or
// end_base; decision i of the segment sits at stream position base + i.
struct AssemblePiece {
  long long base;
  long long end_base;
  long long next_base;
  int seg;
  int stitched;
  int next_stitched;
  int next_seg;
};

struct SegBuf {
  const uint8_t* ptr;
};

// Launchers of the DAS kernels (das.cu); 0 on success.
int launch_das_rms(const double* x, const long long* d_centers, int n, double* d_out,
                   cudaStream_t stream);
size_t das_seam_smem(int max_ovl);
int das_seam_prepare(int max_ovl);   // kernel attributes (call outside stream capture)
// Overlaps above kMaxSeamOverlap need d_gscratch of ntasks x
// das_seam_global_bytes(max_ovl) bytes (-2 without it).
size_t das_seam_global_bytes(int max_ovl);
int launch_das_seams(const SeamTask* d_tasks, int ntasks, int max_ovl, const double* d_qfir2,
                     int* d_bp, unsigned char* d_gscratch, cudaStream_t stream);
int launch_das_assemble(const AssemblePiece* d_pieces, int npieces, const int* d_bp, uint8_t* out,
                        size_t out_stride, int nch, int S, const SegBuf* d_segbuf,
                        cudaStream_t stream);
void pop_fir_times_two(double* q2);

}  // namespace dsdgpu
