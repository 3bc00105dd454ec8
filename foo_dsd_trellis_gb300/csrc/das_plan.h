// Host-side planning of Density-Aligned Stitching (reference
// src/dsp_plugin.c:1343-2725), shared by the single-stream entry point
// (dsdgpu_das_process) and the multi-stream batch plan.  Everything here is
// integer bookkeeping on the host; the RMS values that drive the reposition of
// quiet boundaries come from the device through a callback.
#pragma once
#include <cstdint>
#include <functional>
#include <vector>

#include "das_internal.h"

namespace dsdgpu {

// Segment bookkeeping of sdm_process_block / sdm_segment_process
// (src/trellis.c:1026-1062, src/engine.c:915-938): how many leading steps of a
// run of `count` inputs produce no kept decision, how many decisions are kept,
// and the context's pending (latency-fill) count afterwards.
void sdm_plan_steps(int64_t lat, int64_t pend, int64_t count, int64_t discard, int64_t* skip,
                    int64_t* out, int64_t* new_pend);

// Equal split of `count` samples into S segments (src/dsp_plugin.c:1343-1366,
// 1936-1957): S = count / seg_len (or nsegs), reduced until every segment
// holds at least max(4 * overlap, 256) samples.  Returns S.
int das_nominal_layout(size_t count, long long seg_len, int nsegs, size_t overlap,
                       std::vector<long long>& start, std::vector<long long>& size);

constexpr long long kRmsWindow = 2048;   // src/dsp_plugin.c:1963

// RMS of the FIR signal over windows [c - win/2, c + win/2) for every center.
using RmsEval = std::function<int(const std::vector<long long>& centers, std::vector<double>& rms)>;

// Boundaries the reposition looks at (s >= 2, window inside the chunk).
void das_reposition_centers(const std::vector<long long>& start, size_t count,
                            std::vector<long long>& centers, std::vector<int>& which);

// Reposition of quiet boundaries (src/dsp_plugin.c:1959-2024): a boundary
// whose window RMS `cur[i]` is <= 0.005 moves to the loudest offset found by
// the reference's outward scan (steps of win/2 up to min(40 %, 200,000)),
// subject to keeping 2 * overlap from its neighbours.  `rms` is called once,
// with the candidate windows of every quiet boundary.  Returns 0 or the callback's error.
int das_reposition_apply(std::vector<long long>& start, std::vector<long long>& size, size_t count,
                         size_t overlap, const std::vector<int>& which,
                         const std::vector<double>& cur, const RmsEval& rms);

// Input range and discard of every segment's SDM run
// (src/dsp_plugin.c:2185-2352): seg0 runs from the persistent context, later
// segments start `overlap` early and discard overlap - lat warm-up decisions;
// every segment but the last extends `overlap` past its end.
void das_segment_io(const std::vector<long long>& start, const std::vector<long long>& size,
                    size_t count, size_t overlap, int lat, bool seg0_first,
                    std::vector<long long>& in_start, std::vector<long long>& in_cnt,
                    std::vector<long long>& discard);

// One seam search of the stream plan (the device task adds the pointers).
struct SeamPlan {
  long long prev_off;
  int boundary;
  int ovl_len;
  int prev_seg;
};

// Stream plan from the segments' kept-decision counts (channel 0; every
// channel has the same counts): where each segment's decisions land in the
// stitched stream, which boundaries need a seam search, and the gather pieces
// (src/dsp_plugin.c:2414-2682).  Write positions do not depend on the seams.
// Returns 0, or -1 with `*err` set when a segment is shorter than the overlap.
int das_stream_plan(int S, const int64_t* seg_out, const std::vector<long long>& size,
                    size_t overlap, bool seg0_first, std::vector<SeamPlan>& tasks,
                    std::vector<AssemblePiece>& pieces, long long* final_count, const char** err);

}  // namespace dsdgpu
