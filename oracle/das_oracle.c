/*
 * ORACLE — test infrastructure only (see oracle.h).
 *
 * Restatement of Density-Aligned Stitching as the reference runs it for one
 * chunk (src/dsp_plugin.c:1283-1367 and 1936-2762), driving the pinned SDM
 * restatement of sdm_oracle.c.  The reference computes the segment count
 * from its thread pool (at most 2 or 4 per channel); here the count comes
 * from a nominal segment length (or is given), and everything else follows
 * the reference per segment and per boundary:
 *
 *  layout    overlap = 64 * lat; equal split with the remainder spread over
 *            the first segments; fewer segments while a segment would be
 *            shorter than max(4 * overlap, 256)           (:1343-1366, 1936-1957)
 *  reposition for seg >= 2 when there are more than 2 segments: a boundary in
 *            a quiet region (2048-sample RMS <= 0.005 on channel 0) moves to
 *            the loudest point found at +-1024-sample steps within
 *            min(40 % of a segment, 200000), keeping 2*overlap clear of the
 *            neighbours                                     (:1959-2024)
 *  seeding   seg0-first (rates below DSD512): seg0 runs on the persistent
 *            context, seg1 on a copy of its final state ("DIRECT"), seg2+ on
 *            copies seeded with the 16-level greedy estimate at their start
 *            (:2185-2283); full-parallel (DSD512 and up): every segment starts
 *            from the persistent state of the chunk start, seg1+ seeded with its
 *            best candidate's state                        (:2268-2283)
 *  segments  seg >= 1 (seg >= 2 in seg0-first) start `overlap` early, run
 *            `overlap - lat` warm-up decisions that are dropped, and extend
 *            `overlap` past their end when they are not last (:2285-2340)
 *  stitch    on channel 0, per boundary: sliding match density, candidates of
 *            density >= 90 % of the peak with runs >= 4, plus the run nearest
 *            the density peak, each scored by the peak of a 255-tap Kaiser
 *            low-pass of the stitched-minus-unstitched difference over +-512
 *            samples divided by the clamped density ratio; the pick prefers a
 *            clearly lower pop (< 0.8x) or a similar pop (< 1.2x) at higher
 *            density                                       (:2414-2682)
 *  assembly  the same positions on every channel; in full-parallel mode seg0's
 *            output is cut back to its nominal length before the first
 *            overlap, exactly as the reference does        (:2420-2430, 2683-2714)
 *  carry     across the chunks of a stream, the persistent context continues
 *            in seg0 and is replaced by the last segment's final context
 *                                                          (:2714-2721)
 *
 * Parity: pinned to the reference's own plugin_process (src/dsp_plugin.c
 * compiled here with its engine, FIR chain and trellis by oracle/ref_plugin.c,
 * IPP and Win32 replaced by stand-ins): the DoP output of both seed modes,
 * explicit and automatic segment counts, same-rate and rate-converting paths
 * and chunk streams agree byte for byte (tests/test_oracle_ref.py).  The
 * reference's segment count comes from its thread pool (at most 8 per channel
 * per chunk); larger counts use the same per-segment and per-boundary rules.
 */
#include "oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define DSD_RATE_512_HZ 22579200u

/* The 255-tap pop-metric low-pass, computed the reference's way (:2568-2600). */
static void pop_fir(double *q)
{
    const int N = 255;
    const double fc = 20000.0 / (5644800.0 / 2.0);
    double sum = 0;
    for (int i = 0; i < N; i++) {
        double n = i - 127.0;
        if (n > -0.001 && n < 0.001)
            q[i] = 2.0 * fc;
        else
            q[i] = sin(2.0 * 3.14159265358979 * fc * n) / (3.14159265358979 * n);
        double x = 2.0 * i / (N - 1) - 1.0;
        double kb = 8.0;
        double arg = kb * sqrt(1.0 - x * x > 0 ? 1.0 - x * x : 0);
        double i0a = 1.0, term = 1.0;
        for (int m = 1; m <= 20; m++) {
            term *= (arg / 2.0 / m) * (arg / 2.0 / m);
            i0a += term;
        }
        double i0k = 1.0;
        term = 1.0;
        for (int m = 1; m <= 20; m++) {
            term *= (kb / 2.0 / m) * (kb / 2.0 / m);
            i0k += term;
        }
        q[i] *= i0a / i0k;
        sum += q[i];
    }
    for (int i = 0; i < N; i++) q[i] /= sum;
}

typedef struct { int pos, run, density; double quality; } qcand_t;

/* Seam search for one boundary.  prev/next are the decision bits (0/1) of the
 * last `ovl_len` stream samples and of the new segment's first samples. */
static int seam_search(const uint8_t *prev, const uint8_t *next, int ovl_len, int lat,
                       const double *qfir)
{
    int half_w = lat;
    if (half_w > ovl_len / 2) half_w = ovl_len / 2;
    if (half_w < 4) half_w = 4;

    int *dmap = (int *)calloc((size_t)(ovl_len > 0 ? ovl_len : 1), sizeof(int));
    int peak = 0;
    {
        int cur = 0;
        int ie = half_w < ovl_len ? half_w : ovl_len;
        for (int w = 0; w < ie; w++)
            if (prev[w] == next[w]) cur++;
        if (ovl_len > 0) dmap[0] = cur;
        if (cur > peak) peak = cur;
        for (int p = 1; p < ovl_len; p++) {
            int add = p + half_w - 1;
            if (add >= 0 && add < ovl_len && prev[add] == next[add]) cur++;
            int rem = p - half_w - 1;
            if (rem >= 0 && rem < ovl_len && prev[rem] == next[rem]) cur--;
            dmap[p] = cur;
            if (cur > peak) peak = cur;
        }
    }

    const int floor_d = peak * 9 / 10;
    const int min_spacing = half_w;
    qcand_t q[32];
    int nq = 0;
    for (int p = 0; p < ovl_len - 3 && nq < 32;) {
        if (prev[p] != next[p] || dmap[p] < floor_d) { p++; continue; }
        int rs = p, rl = 0;
        while (p < ovl_len && prev[p] == next[p]) { rl++; p++; }
        if (rl < 4) continue;
        if (nq > 0 && rs - q[nq - 1].pos < min_spacing) continue;
        q[nq].pos = rs;
        q[nq].run = rl;
        q[nq].density = dmap[rs];
        q[nq].quality = 1e30;
        nq++;
    }
    {
        int pp = 0;
        for (int p = 1; p < ovl_len; p++)
            if (dmap[p] > dmap[pp]) pp = p;
        int prp = pp, prl = 1;
        for (int mr = 8; mr >= 1 && prl < 4; mr >>= 1) {
            for (int r = 0; r <= half_w && prl < 4; r++) {
                int tryp[2] = { pp - r, pp + r };
                for (int t = 0; t < 2 && prl < 4; t++) {
                    int tp = tryp[t];
                    if (tp < 0 || tp + mr > ovl_len) continue;
                    int rl = 0;
                    for (int k = 0; k < mr; k++) {
                        if (prev[tp + k] == next[tp + k]) rl++;
                        else break;
                    }
                    if (rl >= mr) { prp = tp; prl = mr; }
                }
            }
        }
        int dup = 0;
        for (int ci = 0; ci < nq; ci++)
            if (abs(q[ci].pos - prp) < min_spacing) { dup = 1; break; }
        if (!dup && nq < 32) {
            q[nq].pos = prp;
            q[nq].run = prl;
            q[nq].density = ovl_len > 0 ? dmap[prp] : 0;
            q[nq].quality = 1e30;
            nq++;
        }
    }
    if (nq == 0) {
        q[0].pos = 0; q[0].run = 1; q[0].density = 0; q[0].quality = 0;
        nq = 1;
    }
    if (nq == 1) q[0].quality = 0;
    if (nq > 1) {
        const int fh = 127, er = 512;
        for (int ci = 0; ci < nq; ci++) {
            const int sp = q[ci].pos;
            double max_d = 0;
            for (int j = -er; j < er; j++) {
                double val = 0;
                for (int k = 0; k < 255; k++) {
                    int idx = sp + j - fh + k;
                    if (idx >= sp && idx >= 0 && idx < ovl_len) {
                        double diff = (double)(next[idx] ? 1.0f : -1.0f) - (double)(prev[idx] ? 1.0f : -1.0f);
                        val += qfir[k] * diff;
                    }
                }
                double ad = fabs(val);
                if (ad > max_d) max_d = ad;
            }
            double dr = (double)q[ci].density / (double)(peak > 0 ? peak : 1);
            if (dr < 0.5) dr = 0.5;
            q[ci].quality = max_d / dr;
        }
    }
    int best = 0;
    for (int ci = 1; ci < nq; ci++) {
        double ratio = q[ci].quality / (q[best].quality + 1e-15);
        if (ratio < 0.8) best = ci;
        else if (ratio < 1.2 && q[ci].density > q[best].density) best = ci;
    }
    free(dmap);
    return q[best].pos;
}

static double window_rms(const double *x, size_t c, size_t w)
{
    double s = 0.0;
    for (size_t i = c - w / 2; i < c + w / 2; i++) s += x[i] * x[i];
    return sqrt(s / (double)w);
}

size_t ora_das_run(int order, const double *a, const double *g, int depth,
                   int cands, int lat, double state_limit,
                   const ora_das_cfg_t *cfg, const double *const *fir, size_t count,
                   int nch, uint8_t *const *out_bits, int *stitch_pos,
                   size_t *seg_starts, int nthreads)
{
    return ora_das_run_carry(order, a, g, depth, cands, lat, state_limit, cfg, fir, count, nch,
                             out_bits, stitch_pos, seg_starts, nthreads, NULL);
}

size_t ora_das_run_carry(int order, const double *a, const double *g, int depth,
                         int cands, int lat, double state_limit,
                         const ora_das_cfg_t *cfg, const double *const *fir, size_t count,
                         int nch, uint8_t *const *out_bits, int *stitch_pos,
                         size_t *seg_starts, int nthreads, ora_sdm_t *const *carry)
{
    const size_t overlap = 64 * (size_t)lat;
    int S = cfg->seg_len > 0 ? (int)(count / (size_t)cfg->seg_len) : cfg->nsegs;
    if (S < 1) S = 1;
    size_t min_seg = overlap * 4;
    if (min_seg < 256) min_seg = 256;
    while (S > 1 && count / (size_t)S < min_seg) S--;

    size_t *start = (size_t *)calloc((size_t)S, sizeof(size_t));
    size_t *size = (size_t *)calloc((size_t)S, sizeof(size_t));
    {
        size_t base = count / (size_t)S, rem = count % (size_t)S, pos = 0;
        for (int s = 0; s < S; s++) {
            start[s] = pos;
            size[s] = (s == S - 1) ? count - pos : base + ((size_t)s < rem ? 1 : 0);
            pos += size[s];
        }
    }
    if (cfg->reposition && S > 2) {
        const size_t base = count / (size_t)S;
        size_t max_shift = base * 2 / 5;
        if (max_shift > 200000) max_shift = 200000;
        const size_t win = 2048;
        const double loud = 0.005;
        for (int s = 2; s < S; s++) {
            size_t b = start[s];
            if (b < win || b + win >= count) continue;
            double cur = window_rms(fir[0], b, win);
            if (cur > loud) continue;
            size_t best_pos = b;
            double best_rms = cur;
            const size_t step = win / 2;
            for (size_t off = step; off <= max_shift; off += step) {
                for (int dir = -1; dir <= 1; dir += 2) {
                    size_t c = (dir < 0) ? (b > off ? b - off : 0) : b + off;
                    if (c < win / 2 || c + win / 2 >= count) continue;
                    if (s > 0 && c <= start[s - 1] + overlap * 2) continue;
                    if (s < S - 1 && start[s + 1] >= overlap * 2 && c >= start[s + 1] - overlap * 2)
                        continue;
                    double r = window_rms(fir[0], c, win);
                    if (r > best_rms) { best_rms = r; best_pos = c; }
                }
                if (best_rms > loud) break;
            }
            if (best_pos != b) {
                start[s] = best_pos;
                size[s - 1] = best_pos - start[s - 1];
                size[s] = (s < S - 1) ? start[s + 1] - best_pos : count - best_pos;
            }
        }
    }
    if (seg_starts)
        for (int s = 0; s < S; s++) seg_starts[s] = start[s];

    const int seg0_first = cfg->seed_mode == 1;
    ora_sdm_t **pers = (ora_sdm_t **)calloc((size_t)nch, sizeof(void *));
    uint8_t **buf = (uint8_t **)calloc((size_t)nch * (size_t)S, sizeof(void *));
    size_t *cnt = (size_t *)calloc((size_t)nch * (size_t)S, sizeof(size_t));
    double (*est)[ORA_MAX_ORDER] = calloc((size_t)nch * (size_t)S, sizeof *est);
    /* the last segment's final context per channel: the next chunk's
     * persistent context (src/dsp_plugin.c:2714-2721) */
    ora_sdm_t **last = (ora_sdm_t **)calloc((size_t)nch, sizeof(void *));
    for (int ch = 0; ch < nch; ch++) {
        pers[ch] = carry ? carry[ch] : ora_sdm_new(order, a, g, depth, cands, lat, state_limit);
        if (carry && S > 1) last[ch] = ora_sdm_new(order, a, g, depth, cands, lat, state_limit);
        for (int s = 0; s < S; s++)
            buf[ch * S + s] = (uint8_t *)malloc(size[s] + 2 * overlap + 16);
    }

    int first_par = 0;
    ora_sdm_t **snap = (ora_sdm_t **)calloc((size_t)nch, sizeof(void *));
    if (seg0_first) {
        for (int ch = 0; ch < nch; ch++) {
            cnt[ch * S] = ora_sdm_process_bits(pers[ch], fir[ch], buf[ch * S], size[0]);
            if (S > 1) {
                ora_sdm_t *t = ora_sdm_new(order, a, g, depth, cands, lat, state_limit);
                ora_sdm_copy(t, pers[ch]);
                size_t in_cnt = size[1];
                if (S > 2 && start[1] + size[1] + overlap <= count) in_cnt += overlap;
                cnt[ch * S + 1] = ora_sdm_process_bits(t, fir[ch] + start[1], buf[ch * S + 1], in_cnt);
                if (last[ch] && S == 2) ora_sdm_copy(last[ch], t);
                ora_sdm_free(t);
            }
            if (S > 2) {
                double st[ORA_MAX_ORDER];
                ora_sdm_best_state(pers[ch], st);
                size_t pos = 0;
                const size_t est_start = start[1];
                for (int s = 1; s < S; s++) {
                    size_t bnd = s >= 2 ? start[s] - est_start : 0;
                    if (bnd > pos && bnd <= count - est_start) {
                        ora_estimate_state(order, a, g, st, fir[ch] + est_start + pos, bnd - pos,
                                           state_limit, 16, st);
                        pos = bnd;
                    }
                    for (int k = 0; k < order; k++) est[ch * S + s][k] = st[k];
                }
            }
            snap[ch] = pers[ch];
        }
        first_par = 2;
    } else {
        for (int ch = 0; ch < nch; ch++) {
            snap[ch] = ora_sdm_new(order, a, g, depth, cands, lat, state_limit);
            ora_sdm_copy(snap[ch], pers[ch]);
            double st[ORA_MAX_ORDER];
            ora_sdm_best_state(pers[ch], st);
            for (int s = 1; s < S; s++)
                for (int k = 0; k < order; k++) est[ch * S + s][k] = st[k];
        }
    }

    /* the parallel phase as independent jobs on the thread pool */
    ora_seg_job_t *jobs = (ora_seg_job_t *)calloc((size_t)nch * (size_t)S, sizeof *jobs);
    int nj = 0;
    for (int ch = 0; ch < nch; ch++) {
        for (int s = first_par; s < S; s++) {
            ora_seg_job_t *j = &jobs[nj++];
            const int ext = (s < S - 1);
            if (s == 0) {
                size_t in_cnt = size[0];
                if (ext && size[0] + overlap <= count) in_cnt += overlap;
                j->in = fir[ch];
                j->count = in_cnt;
                j->discard = 0;
                j->seed = pers[ch];
                j->seed_state = NULL;
            } else {
                size_t in_start = start[s] >= overlap ? start[s] - overlap : 0;
                size_t in_cnt = start[s] + size[s] - in_start;
                if (ext && start[s] + size[s] + overlap <= count) in_cnt += overlap;
                j->in = fir[ch] + in_start;
                j->count = in_cnt;
                j->discard = start[s] >= overlap ? overlap - (size_t)lat : 0;
                j->seed = snap[ch];
                j->seed_state = est[ch * S + s];
            }
            j->bits = buf[ch * S + s];
            /* one segment: the chunk is a plain continuation of the
             * persistent context (the plugin's non-DAS path) */
            j->final_ctx = (s == S - 1) ? (S > 1 ? last[ch] : (carry ? pers[ch] : NULL)) : NULL;
        }
    }
    ora_sdm_run_jobs(order, a, g, depth, cands, lat, state_limit, jobs, nj, nthreads);
    nj = 0;
    for (int ch = 0; ch < nch; ch++)
        for (int s = first_par; s < S; s++) cnt[ch * S + s] = jobs[nj++].out_count;

    /* stitch on channel 0 */
    double qfir[255];
    pop_fir(qfir);
    if (stitch_pos) memset(stitch_pos, 0, sizeof(int) * (size_t)S);
    int *bp = (int *)calloc((size_t)S, sizeof(int));
    size_t final_count = 0;
    for (int ch = 0; ch < nch; ch++) {
        uint8_t *out = out_bits[ch];
        size_t c0 = cnt[ch * S];
        if (!seg0_first && c0 > size[0]) c0 = size[0];
        memcpy(out, buf[ch * S], c0);
        size_t wp = c0;
        for (int s = 1; s < S; s++) {
            size_t so = cnt[ch * S + s];
            if (so == 0) { if (ch == 0) bp[s] = 0; continue; }
            if (s == 1 && seg0_first) {
                memcpy(out + wp, buf[ch * S + 1], so);
                wp += so;
                continue;
            }
            size_t ps = wp >= overlap ? wp - overlap : 0;
            if (ch == 0) {
                size_t ol = wp - ps;
                if (ol > so) ol = so;
                if (ol > overlap) ol = overlap;
                bp[s] = seam_search(out + ps, buf[ch * S + s], (int)ol, lat, qfir);
            }
            size_t at = ps + (size_t)bp[s];
            memcpy(out + at, buf[ch * S + s] + bp[s], so - (size_t)bp[s]);
            wp = at + so - (size_t)bp[s];
        }
        if (ch == 0) final_count = wp;
    }
    if (stitch_pos) memcpy(stitch_pos, bp, sizeof(int) * (size_t)S);

    for (int ch = 0; ch < nch; ch++) {
        if (!seg0_first) ora_sdm_free(snap[ch]);
        if (last[ch]) {
            ora_sdm_copy(pers[ch], last[ch]);
            ora_sdm_free(last[ch]);
        }
        if (!carry) ora_sdm_free(pers[ch]);
        for (int s = 0; s < S; s++) free(buf[ch * S + s]);
    }
    free(bp); free(jobs); free(snap); free(est); free(cnt); free(buf); free(pers); free(last);
    free(start); free(size);
    return final_count;
}
