// Host-side DAS planning (reference src/dsp_plugin.c:1343-2725); the contract
// of every function is in das_plan.h.
#include "das_plan.h"

#include <algorithm>

namespace dsdgpu {

void sdm_plan_steps(int64_t lat, int64_t pend, int64_t count, int64_t discard, int64_t* skip,
                    int64_t* out, int64_t* new_pend) {
  if (discard == 0) {
    int64_t pre = std::min<int64_t>(lat - pend, count);
    if (pre < 0) pre = 0;
    *skip = pre;
    *out = count - pre;
    *new_pend = pend + pre;
    return;
  }
  const int64_t warm = lat + discard;
  if (warm > count) {
    int64_t pre = std::min<int64_t>(lat - pend, count);
    if (pre < 0) pre = 0;
    *skip = count;
    *out = 0;
    *new_pend = pend + pre;
  } else {
    *skip = warm;
    *out = count - warm;
    *new_pend = lat;
  }
}

int das_nominal_layout(size_t count, long long seg_len, int nsegs, size_t overlap,
                       std::vector<long long>& start, std::vector<long long>& size) {
  int S = seg_len > 0 ? (int)(count / (size_t)seg_len) : nsegs;
  if (S < 1) S = 1;
  size_t min_seg = overlap * 4;
  if (min_seg < 256) min_seg = 256;
  while (S > 1 && count / (size_t)S < min_seg) S--;
  start.assign(S, 0);
  size.assign(S, 0);
  const size_t base = count / (size_t)S, rem = count % (size_t)S;
  size_t pos = 0;
  for (int s = 0; s < S; s++) {
    start[s] = (long long)pos;
    size[s] = (long long)((s == S - 1) ? count - pos : base + ((size_t)s < rem ? 1 : 0));
    pos += (size_t)size[s];
  }
  return S;
}

void das_reposition_centers(const std::vector<long long>& start, size_t count,
                            std::vector<long long>& centers, std::vector<int>& which) {
  centers.clear();
  which.clear();
  const int S = (int)start.size();
  for (int s = 2; s < S; s++) {
    const long long b = start[s];
    if (b < kRmsWindow || b + kRmsWindow >= (long long)count) continue;
    centers.push_back(b);
    which.push_back(s);
  }
}

int das_reposition_apply(std::vector<long long>& start, std::vector<long long>& size, size_t count,
                         size_t overlap, const std::vector<int>& which,
                         const std::vector<double>& cur, const RmsEval& rms_eval) {
  const int S = (int)start.size();
  const long long win = kRmsWindow;
  const size_t base = count / (size_t)S;
  long long max_shift = (long long)(base * 2 / 5);
  if (max_shift > 200000) max_shift = 200000;
  const long long step = win / 2;
  // Candidate windows of every quiet boundary, evaluated in one call.  A
  // boundary's candidates depend only on its own nominal start (each boundary
  // appears once in `which`, and only its own turn moves it), so they can all
  // be taken before the first move; the neighbour constraints, which do see
  // earlier moves, are applied in the scan below.  The RMS values are pure, so
  // evaluating offsets past the reference's early exit changes nothing.
  std::vector<long long> cand;
  std::vector<size_t> first(which.size() + 1, 0);
  for (size_t wi = 0; wi < which.size(); wi++) {
    first[wi] = cand.size();
    if (cur[wi] > 0.005) continue;
    const long long b = start[which[wi]];
    for (long long off = step; off <= max_shift; off += step)
      for (int dir = -1; dir <= 1; dir += 2) {
        const long long cc = dir < 0 ? (b > off ? b - off : 0) : b + off;
        if (cc < win / 2 || cc + win / 2 >= (long long)count) continue;
        cand.push_back(cc);
      }
  }
  first[which.size()] = cand.size();
  std::vector<double> rms(cand.size());
  if (!cand.empty()) {
    const int rc = rms_eval(cand, rms);
    if (rc) return rc;
  }
  for (size_t wi = 0; wi < which.size(); wi++) {
    if (cur[wi] > 0.005) continue;
    const int s = which[wi];
    const long long b = start[s];
    long long best_pos = b;
    double best_rms = cur[wi];
    size_t ci = first[wi];
    for (long long off = step; off <= max_shift; off += step) {
      for (int dir = -1; dir <= 1; dir += 2) {
        const long long cc = dir < 0 ? (b > off ? b - off : 0) : b + off;
        if (cc < win / 2 || cc + win / 2 >= (long long)count) continue;
        const double r = rms[ci++];
        if (s > 0 && cc <= start[s - 1] + (long long)overlap * 2) continue;
        if (s < S - 1 && start[s + 1] >= (long long)overlap * 2 &&
            cc >= start[s + 1] - (long long)overlap * 2)
          continue;
        if (r > best_rms) { best_rms = r; best_pos = cc; }
      }
      if (best_rms > 0.005) break;
    }
    if (best_pos != b) {
      start[s] = best_pos;
      size[s - 1] = best_pos - start[s - 1];
      size[s] = (s < S - 1) ? start[s + 1] - best_pos : (long long)count - best_pos;
    }
  }
  return 0;
}

void das_segment_io(const std::vector<long long>& start, const std::vector<long long>& size,
                    size_t count, size_t overlap, int lat, bool seg0_first,
                    std::vector<long long>& in_start, std::vector<long long>& in_cnt,
                    std::vector<long long>& discard) {
  const int S = (int)start.size();
  const long long ov = (long long)overlap;
  in_start.assign(S, 0);
  in_cnt.assign(S, 0);
  discard.assign(S, 0);
  for (int s = 0; s < S; s++) {
    const bool ext = s < S - 1;
    long long is, ic, disc = 0;
    if (s == 0) {
      is = 0;
      ic = size[0];
      if (!seg0_first && ext && size[0] + ov <= (long long)count) ic += ov;
    } else if (s == 1 && seg0_first) {
      is = start[1];
      ic = size[1];
      if (S > 2 && start[1] + size[1] + ov <= (long long)count) ic += ov;
    } else {
      is = start[s] >= ov ? start[s] - ov : 0;
      ic = start[s] + size[s] - is;
      if (ext && start[s] + size[s] + ov <= (long long)count) ic += ov;
      disc = start[s] >= ov ? ov - lat : 0;
    }
    in_start[s] = is;
    in_cnt[s] = ic;
    discard[s] = disc;
  }
}

int das_stream_plan(int S, const int64_t* seg_out, const std::vector<long long>& size,
                    size_t overlap, bool seg0_first, std::vector<SeamPlan>& tasks,
                    std::vector<AssemblePiece>& pieces, long long* final_count, const char** err) {
  const long long ov = (long long)overlap;
  std::vector<long long> cnt(S), ps(S, 0), wp(S, 0);
  std::vector<int> stitched(S, 0), used(S, 0);
  tasks.clear();
  pieces.clear();
  for (int s = 0; s < S; s++) cnt[s] = seg_out[s];
  if (!seg0_first && cnt[0] > size[0]) cnt[0] = size[0];
  long long w = cnt[0];
  wp[0] = w;
  used[0] = 1;
  int last_used = 0;
  for (int s = 1; s < S; s++) {
    const long long so = seg_out[s];
    if (so == 0) continue;
    used[s] = 1;
    if (s == 1 && seg0_first) {
      ps[s] = w;                  // DIRECT: appended as is
      w += so;
      wp[s] = w;
      last_used = s;
      continue;
    }
    if (w < ov) {
      *err = "stream shorter than the overlap before a seam";
      return -1;
    }
    const long long pstart = w - ov;
    long long ol = w - pstart;
    if (ol > so) ol = so;
    if (ol > ov) ol = ov;
    // the previous `overlap` stream decisions must all come from segment
    // last_used: its copied part starts at base (+ its seam, < overlap)
    const bool prev_stitched = stitched[last_used] != 0;
    const long long base_last = last_used == 0 ? 0 : ps[last_used];
    const long long prev_len = prev_stitched ? seg_out[last_used] : cnt[last_used];
    if (prev_stitched ? (prev_len < 2 * ov) : (prev_len < ov)) {
      *err = "segment shorter than the overlap";
      return -1;
    }
    SeamPlan t;
    t.boundary = s;
    t.ovl_len = (int)ol;
    t.prev_seg = last_used;
    t.prev_off = pstart - base_last;
    tasks.push_back(t);
    ps[s] = pstart;
    stitched[s] = 1;
    w = pstart + so;
    wp[s] = w;
    last_used = s;
  }
  *final_count = w;

  std::vector<int> order_used;
  for (int s = 0; s < S; s++)
    if (used[s]) order_used.push_back(s);
  for (size_t i = 0; i < order_used.size(); i++) {
    const int s = order_used[i];
    AssemblePiece p;
    p.seg = s;
    p.base = (s == 0) ? 0 : ps[s];
    p.stitched = stitched[s];
    p.end_base = wp[s];
    p.next_stitched = 0;
    p.next_seg = 0;
    p.next_base = 0;
    if (i + 1 < order_used.size()) {
      const int n = order_used[i + 1];
      if (stitched[n]) {
        p.next_stitched = 1;
        p.next_seg = n;
        p.next_base = ps[n];
      } else {
        p.end_base = ps[n];   // DIRECT follower starts at our end
      }
    }
    pieces.push_back(p);
  }
  return 0;
}

}  // namespace dsdgpu
