// Device-side plan records of the DAS pipeline.
#pragma once
#include <cstdint>

namespace dsdgpu {

// One seam search: boundary `boundary` compares prev[0..ovl_len) (the last
// decisions of the stream before the seam, inside segment prev_seg's buffer at
// prev_off) with next[0..ovl_len) (segment `boundary`'s first decisions).
struct SeamTask {
  const uint8_t* prev;
  const uint8_t* next;
  long long prev_off;
  int boundary;
  int ovl_len;
  int prev_seg;
  int pad;
};

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

}  // namespace dsdgpu
