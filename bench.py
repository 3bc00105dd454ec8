#!/usr/bin/env python
"""Benchmark of the GB300 PCM -> DSD hot path on its headline workload.

Workload (one step): DSD128 stereo, 10 s of 48 kHz float32 PCM (31 log-spaced
tones at -20 dBFS plus pink noise at -30 dBFS, seeded) -> boxcar + 7-stage
half-band FIR chain to 6.144 MHz with the PCM gain and soft clip -> trellis
SDM (CLANS-7 order-7 NTF, K = 32, depth 64, lat 128) over 65,536-sample DAS
segments (overlap 8192, full-parallel seeding) -> density-aligned stitching
-> DoP framing.  The metric is output DSD samples per second over both
channels (and x realtime).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

`--impl reference` times the reference's CPU algorithm for this path (the
oracle's C port on this host's cores; the reference's own trellis.c is built
from source only where its tree is present, and never on an aarch64 GPU host)
on a bounded slice of the same workload.

Other workloads (`--workload`, one JSON line each): multistream64 (64 streams
in one batched plan), multistream64_precorr (the same streams through the
PreCorr SDM in one plan), multistream64_dsd (the same streams as DoP input,
re-encoded at their DSD rate in one plan), diff16 (the adjoint of the differentiable path),
dsd512conv6 (DSD512 5.1 with UPOLS room convolution), samerate128 (DoP DSD128
re-encode on the engine's path-table parameters), samerate128lp (the same with
the engine's 127-tap FIR lowpass instead of the boxcar), dsd2pcm128 (DSD128 ->
44.1 kHz PCM), precorr128 (PCM -> DSD128 with the PreCorr SDM) and dsd256to128
(DoP DSD256 -> DSD128 through the FP64 decimation chain and the DAS trellis) and
dsd128_seg0first (the headline's signal and trellis with the reference's own
seeding rule below DSD512, seg0-first, on 1 s chunks of one stream).  The
default run (N = 1) also runs the quick ones after the headline's timed steps
(and multistream64 at an eighth of its stream lengths), each in its own
process, and summarises them under "also" (`--also none` skips them).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "trellis SDM DSD Msamples/s & xRT at DSD128 bit-exact; batched vs plain; adjoint ms"
UNIT = "DSD Msamples/s"
WL = dict(workload="dsd128_das_stereo_10s_multitone_pink", fs_in=48000, fs_out=6144000,
          channels=2, seconds=10.0, ntf="clans-7", ntf_order=7, cands=32, depth=64, lat=128,
          das_seg_len=65536, das_overlap=64 * 128, seed_mode="full_parallel", output="dop",
          boxcar_taps=8, soft_clip=True, seed=1001,
          # engine_channel_init's PCM gain: float32(0.708) * 0.5 (src/engine.c:206-210)
          fir_gain=0.3540000021457672,
          l2="GPU arm: 512 MiB written between timed steps, outside the events; the CPU arm "
             "has no device cache to flush")
FP64_OPS_PER_CAND_SAMPLE = 5 * WL["ntf_order"] + 6   # (2N+1) mul + (3N+5) add
SDM_DRAM_BYTES_PER_SAMPLE = 9.04                      # measured, see the traffic note below
SDM_PARTS_DRAM_BYTES_PER_SAMPLE = 9.15                # the balanced launch's (parts kernel), measured


# The rows beside the headline, measured by the default run as well: the
# same-rate re-encode (boxcar and FIR lowpass), DSD256 -> DSD128, DSD -> PCM,
# PreCorr, the DSD512 5.1 UPOLS configuration and the adjoint.  The 64-stream
# batched form (about a minute per step) runs only on request.
ALSO_DEFAULT = ["samerate128", "samerate128lp", "dsd256to128", "dsd2pcm128", "precorr128",
                "dsd512conv6", "diff16", "multistream64@0.125"]


def also_command(w: str) -> list[str]:
    """The subprocess command of one `also` entry: 3 warm-up and 3 timed steps;
    name@f runs a multistream workload at f times its stream lengths."""
    name, _, scale = w.partition("@")
    return [sys.executable, os.path.abspath(__file__), "--workload", name, "--steps", "3",
            "--warmup", "3"] + (["--ms-scale", scale] if scale else [])


def run_also(names: list[str]) -> dict:
    """Each workload in its own process after the headline's timed steps; the
    headline's numbers are final by then.  Returns name -> summary."""
    out = {}
    for w in names:
        cmd = also_command(w)
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
            lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
            if r.returncode != 0 or not lines:
                out[w] = {"error": f"exit {r.returncode}: {r.stderr.strip()[-300:]}"}
                continue
            d = json.loads(lines[-1])
        except Exception as e:   # a failed side run never voids the headline line
            out[w] = {"error": repr(e)[:300]}
            continue
        rf = d.get("roofline") or {}
        cb = d.get("cpu_baseline") or {}
        out[w] = {"metric": d.get("metric"), "value": d.get("value"), "unit": d.get("unit"),
                  "higher_is_better": d.get("higher_is_better"),
                  "ms_per_step": d.get("ms_per_step"), "steps": d.get("steps"),
                  "warmup": d.get("warmup"),
                  "e2e": (d.get("e2e") or {}).get("value"),
                  "roofline_frac": rf.get("frac"), "roofline_kernel": rf.get("kernel"),
                  "cpu_baseline": {k: cb.get(k) for k in ("value", "cores", "kind", "sample")}
                  if cb else None,
                  "workload": (d.get("config") or {}).get("workload"),
                  "lengths_s": (d.get("config") or {}).get("lengths_s"),
                  "clocks": d.get("clocks"), "gpu_launches": d.get("gpu_launches")}
        for k in ("forward_ms", "exact_sdm_ms", "fd_check", "stages_ms", "parity"):
            if k in d:
                out[w][k] = d[k]
    return out


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seconds", type=float, default=WL["seconds"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--das-seg-len", type=int, default=WL["das_seg_len"],
                    help="nominal DAS segment length (profiling of small cases only)")
    ap.add_argument("--workload", default="dsd128_das",
                    choices=["dsd128_das", "multistream64", "multistream64_precorr",
                             "multistream64_dsd", "diff16",
                             "dsd512conv6",
                             "samerate128", "samerate128lp", "precorr128", "dsd2pcm128",
                             "dsd256to128", "dsd128_seg0first"],
                    help="multistream64: the batched 64-stream form; diff16: the adjoint; "
                         "samerate128 / samerate128lp / precorr128 / dsd2pcm128: the DSD "
                         "re-encode (boxcar / FIR lowpass), PreCorr and DSD -> PCM paths (each "
                         "prints its own JSON line)")
    ap.add_argument("--also", default=",".join(ALSO_DEFAULT),
                    help="dsd128_das at N=1: other workloads run after the headline, one "
                         "subprocess each (3 warm-up + 3 timed steps), summarised under "
                         "'also' in the headline's JSON line; name@f runs a multistream "
                         "workload at f times its stream lengths; 'none' skips them")
    ap.add_argument("--fd-dirs", type=int, default=32,
                    help="diff16: random unit directions of the finite-difference check")
    ap.add_argument("--ms-scale", type=float, default=1.0,
                    help="multistream64(_precorr): stream lengths scale (1.0 = 0.5-30 s)")
    ap.add_argument("--ms-lanes", type=int, default=0,
                    help="multistream64_dsd: lanes of a warp per trellis job (0 = the plan's "
                         "choice: beyond one wave of jobs the widest width that fits, here 2)")
    ap.add_argument("--ms-seg-len", type=int, default=0,
                    help="multistream64: DAS segment length (0 = autotuned)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def max_over_ranks(seconds: float) -> float:
    """The job's time: the slowest rank's timed region (all-reduce MAX).
    Works on whatever process group is initialised (NCCL on GPUs, gloo on CPU)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(seconds)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(samples_per_rank_step: int, steps: int, world: int, job_seconds: float) -> float:
    """Whole-job DSD Msamples/s: every rank converts its own stream (weak
    scaling), so the job's samples are world x the per-rank count."""
    return samples_per_rank_step * steps * world / job_seconds / 1e6


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _cpu_fir(O, pcm):
    """FP64 FIR restatement per channel, one thread per channel as the
    reference's DAS phase 1 runs it (src/dsp_plugin.c:1381-1460)."""
    import numpy as np
    from concurrent.futures import ThreadPoolExecutor
    from foo_dsd_trellis_gb300.pipeline import PCM_FIR_GAIN

    def one(c):
        return O.engine_fir(WL["fs_in"], WL["fs_out"], pcm[c], boxcar_taps=WL["boxcar_taps"],
                            g_start=PCM_FIR_GAIN, g_end=PCM_FIR_GAIN, soft_clip=True)
    with ThreadPoolExecutor(max_workers=pcm.shape[0]) as ex:
        return np.stack(list(ex.map(one, range(pcm.shape[0]))))


def _cpu_das_dop(O, f, fir, nthreads):
    """Trellis SDM port + DAS + DoP over one chunk; returns (decisions, DoP
    bytes interleaved [n/16][nch][3] as the plugin writes frames)."""
    import numpy as np
    bits, _, _ = O.das_run(f.order, np.array(f.a), np.array(f.g), WL["depth"], WL["cands"],
                           WL["lat"], 0.0, fir, seg_len=WL["das_seg_len"], seed_mode=0,
                           reposition=True, nthreads=nthreads)
    frames = [O.dop_pack_bits(bits[c], 0)[0].reshape(-1, 3) for c in range(bits.shape[0])]
    return bits, np.stack(frames, axis=1).reshape(-1)


def cpu_baseline(pcm, seconds_sample: float, nthreads: int | None = None,
                 first_frame: int = 0) -> dict:
    """The oracle's C port of the same path (FP64 FIR restatement, trellis SDM
    port bit-identical to the reference's trellis.c, DAS restatement, DoP) on
    one slice of the workload converted as its own chunk, on this host's cores."""
    from oracle import oracle as O
    from foo_dsd_trellis_gb300 import ntf
    O.build()
    f = ntf.get_filter(WL["ntf"], WL["fs_out"])
    frames = int(round(seconds_sample * WL["fs_in"]))
    x = pcm[:, first_frame:first_frame + frames]
    nthreads = nthreads or os.cpu_count() or 1
    t0 = time.perf_counter()
    fir = _cpu_fir(O, x)
    bits, _ = _cpu_das_dop(O, f, fir, nthreads)
    dt = time.perf_counter() - t0
    n_out = bits.shape[0] * bits.shape[1]
    return {"value": n_out / dt / 1e6, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{seconds_sample:g} s of the workload from frame {first_frame} "
                      f"({x.shape[0]} ch, {n_out} DSD samples) as one chunk: FP64 FIR "
                      "restatement + trellis SDM port + DAS + DoP",
            "seconds": dt}


def parity_and_cpu_baseline(pcm, gpu_dop, device: int) -> tuple[dict, dict]:
    """Outside the timed region: the oracle over the whole workload.

    The GPU FIR output (same kernel and parameters, a separate context) goes
    through the oracle's DAS (trellis SDM pinned to the reference's trellis.c)
    and DoP packer on every host core; its bytes are compared with the timed
    run's DoP output.  The same oracle run, plus the FP64 FIR restatement over
    the whole input, is the CPU baseline on the full workload."""
    import hashlib

    import numpy as np
    import torch
    from oracle import oracle as O
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.fir import FirChain
    from foo_dsd_trellis_gb300.pipeline import PCM_FIR_GAIN
    O.build()
    f = ntf.get_filter(WL["ntf"], WL["fs_out"])
    nthreads = os.cpu_count() or 1
    fc = FirChain(WL["fs_in"], WL["fs_out"], boxcar_taps=WL["boxcar_taps"], soft_clip=True,
                  num_channels=pcm.shape[0], device=device)
    gfir = fc.process(torch.from_numpy(pcm).cuda(), PCM_FIR_GAIN, PCM_FIR_GAIN).cpu().numpy()
    fc.close()
    t0 = time.perf_counter()
    bits, want = _cpu_das_dop(O, f, gfir, nthreads)
    t_das = time.perf_counter() - t0
    del gfir
    t0 = time.perf_counter()
    _cpu_fir(O, pcm)
    t_fir = time.perf_counter() - t0
    got = np.asarray(gpu_dop, np.uint8)
    same_len = len(got) == len(want)
    diff = np.nonzero(got[:len(want)] != want[:len(got)])[0]
    parity = {"bit_exact": bool(same_len and diff.size == 0), "dop_bytes": int(len(want)),
              "gpu_dop_bytes": int(len(got)), "differing_bytes": int(diff.size),
              "sha256": hashlib.sha256(want.tobytes()).hexdigest(),
              "sha256_gpu": hashlib.sha256(got.tobytes()).hexdigest(),
              "oracle": "oracle DAS (trellis SDM port pinned to the reference's trellis.c) + "
                        "DoP packer over the GPU FIR output of the whole workload, compared "
                        "with the last timed step's DoP bytes"}
    n_out = bits.shape[0] * bits.shape[1]
    cpu = {"value": n_out / (t_fir + t_das) / 1e6, "unit": UNIT, "cores": nthreads,
           "kind": "port", "seconds": t_fir + t_das, "fir_seconds": t_fir, "das_seconds": t_das,
           "sample": f"the whole workload ({pcm.shape[0]} ch, {n_out} DSD samples): FP64 FIR "
                     "restatement (one thread per channel) + trellis SDM port + DAS + DoP on "
                     f"{nthreads} threads; the DAS leg runs on the GPU's FIR output, so its "
                     "decisions are the parity check"}
    return parity, cpu


REF_SLICES = 20


def run_reference(args):
    """The CPU arm: every step converts one of REF_SLICES equal slices of the
    workload's input as its own DAS chunk (65,536-sample segments, the same
    trellis and seeding), in rotation, so REF_SLICES timed steps convert the
    whole input once."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import numpy as np
    from foo_dsd_trellis_gb300 import signals
    pcm = signals.dsd128_multitone_pink(args.seconds, WL["fs_in"], WL["channels"], WL["seed"])
    frames = pcm.shape[1]
    per = frames // REF_SLICES
    sample_s = per / WL["fs_in"]
    for i in range(args.warmup):
        cpu_baseline(pcm, sample_s, first_frame=(i % REF_SLICES) * per)
    vals, secs, outs = [], [], 0
    info = None
    for i in range(args.steps):
        info = cpu_baseline(pcm, sample_s, first_frame=(i % REF_SLICES) * per)
        secs.append(info["seconds"])
        outs += info["value"] * info["seconds"]
    v = float(outs / sum(secs))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * float(np.mean(secs)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": dict(WL, seconds=args.seconds),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": info["cores"], "kind": "port",
                             "sample": f"each step converts one {sample_s:g} s slice "
                                       f"({REF_SLICES} slices of the {args.seconds:g} s input, "
                                       "taken in rotation, so every "
                                       f"{REF_SLICES} steps convert the whole input) as one "
                                       "DAS chunk of the workload's segment length: FP64 FIR "
                                       "restatement (one thread per channel) + trellis SDM "
                                       "port + DAS + DoP"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def plain_form(f, x_dev, seg_in, overlap, lat, nseg=2):
    """The one-segment-per-launch form: the same SDM kernel, one DAS segment
    per launch, launched back to back."""
    import torch
    from foo_dsd_trellis_gb300.sdm import SegmentSpec, TrellisSdm
    g = TrellisSdm(f.order, f.a, f.g, WL["depth"], WL["cands"], lat, num_contexts=nseg + 1)
    specs = [SegmentSpec(x_dev[i * seg_in:(i + 1) * seg_in].contiguous(), channel=i,
                         discard=overlap - lat, seed_from=nseg) for i in range(nseg)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in specs:
        g.segments([s])
    dt = time.perf_counter() - t0
    g.close()
    return nseg * seg_in / dt


def run_ours(args):
    import numpy as np
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    from foo_dsd_trellis_gb300 import ntf, signals
    from foo_dsd_trellis_gb300.pipeline import OUT_DOP, PCM_FIR_GAIN, Encoder, FULL_PARALLEL

    f = ntf.get_filter(WL["ntf"], WL["fs_out"])
    # weak scaling: every rank converts its own stereo stream (own seed)
    pcm = signals.dsd128_multitone_pink(args.seconds, WL["fs_in"], WL["channels"],
                                        WL["seed"] + 2 * rank)
    nch, frames = pcm.shape
    if args.das_seg_len != WL["das_seg_len"]:
        WL["das_seg_len"] = args.das_seg_len
    enc = Encoder(WL["fs_in"], WL["fs_out"], nch, f, WL["depth"], WL["cands"], WL["lat"],
                  seg_len=WL["das_seg_len"], seed_mode=FULL_PARALLEL, reposition=True,
                  boxcar_taps=WL["boxcar_taps"], soft_clip=WL["soft_clip"],
                  output_format=OUT_DOP, device=local)
    d_pcm = torch.from_numpy(pcm).cuda()
    d_out = torch.empty(enc.out_capacity(frames) + 64, dtype=torch.uint8, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")   # > L2 (129 MB)
    lib_stream = torch.cuda.ExternalStream(enc.stream_ptr)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # every step converts the 10 s input as a new stream (plugin_flush between
    # steps, outside the timed region), so every step's output is the same and
    # the last one can be checked against the oracle
    for _ in range(args.warmup):
        enc.flush()
        enc.process(d_pcm, d_out)
    torch.cuda.synchronize()

    fp64_peak = enc.probe_fp64_gops()
    clocks = ClockSampler(local)
    launches0 = enc.launches()
    sdm0, _ = enc.sdm_work()
    step_ms, sdm_ms = [], []
    n_out = nbytes = 0
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    for _ in range(args.steps):
        enc.flush()
        flush.fill_(1)                      # evict L2 between steps (outside the events)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(lib_stream)
        n_out, nbytes = enc.process(d_pcm, d_out)
        e1.record(lib_stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        sdm_ms.append(enc.stage_ms()["sdm"])
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier()
    launches = enc.launches() - launches0
    sdm_samples = (enc.sdm_work()[0] - sdm0) / args.steps
    stages = enc.stage_ms()

    total_s = max_over_ranks(sum(step_ms) / 1000.0)
    out_samples_step = n_out * nch                 # both channels
    value = job_throughput(out_samples_step, args.steps, world, total_s)
    xrt = (n_out / WL["fs_out"]) * args.steps / total_s

    # end to end through the host-buffer C-ABI call (pinned host memory)
    h_pcm = torch.from_numpy(pcm).pin_memory().numpy()
    h_out = torch.empty(enc.out_capacity(frames) + 64, dtype=torch.uint8).pin_memory().numpy()
    enc.flush()
    enc.process_host(h_pcm, h_out)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        enc.flush()
        ns, nb = enc.process_host(h_pcm, h_out)
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_value = job_throughput(ns * nch, args.steps, world, e2e_s)

    # roofline of the dominant kernel: the persistent trellis SDM launch.  The
    # algorithmic work is the reference's K (5N + 6) FP64 operations per
    # candidate and OUTPUT sample (both channels); the DAS warm-up and overlap
    # extension of every segment are the algorithm's own redundancy and are
    # reported beside it, not counted as work.
    sdm_s = statistics.mean(sdm_ms) / 1000.0
    flops_per_sample = WL["cands"] * FP64_OPS_PER_CAND_SAMPLE
    flops = out_samples_step * flops_per_sample
    achieved = flops / sdm_s / 1e12
    issued = sdm_samples * flops_per_sample / sdm_s / 1e12
    peak = fp64_peak / 1000.0
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    sm_mhz = clk.get("sm_mhz") or 0.0
    # 2 FP64 add/mul per clock per SM (a 64-cycle warp instruction per sub-partition)
    peak_nominal = 2.0 * sms * sm_mhz * 1e6 / 1e12 if sm_mhz else None
    kernel = enc.last_sdm_kernel()
    roofline = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": None, "kernel": kernel,
                "peak_source": "DADD/DMUL issue rate measured in this run (dsdgpu_probe_fp64); "
                               "MEASURED_PEAKS.json has no FP64 entry",
                "algorithmic_flops_per_launch": flops,
                "output_samples_per_launch": out_samples_step,
                "flops_per_sample": flops_per_sample,
                "flops_definition": "output DSD samples (both channels) x K x (5N + 6)",
                "peak_nominal": peak_nominal,
                "frac_nominal": achieved / peak_nominal if peak_nominal else None,
                "peak_nominal_source": "2 FP64 add/mul per clock per SM x SMs x median SM clock "
                                       "sampled during the timed steps",
                "sdm_input_samples_per_launch": sdm_samples,
                "das_redundancy": sdm_samples / out_samples_step - 1.0,
                "issued_tflops": issued,
                "issue_frac": issued / peak}
    # DRAM bytes per launch: ncu's dram__bytes per SDM input sample of the
    # kernel that ran (one job per warp: the 4 s, 32,768-segment case; parts:
    # the 3.5 s case, profiles/sdm_parts_kernel_dsd128_das_3p5s.md), scaled by
    # the samples processed
    per = SDM_PARTS_DRAM_BYTES_PER_SAMPLE if kernel.startswith("sdm_parts") \
        else SDM_DRAM_BYTES_PER_SAMPLE
    roofline["traffic"] = per * sdm_samples if per else None
    roofline["traffic_source"] = (f"ncu dram__bytes per SDM input sample ({per} B) of a "
                                  f"{'53.7' if kernel.startswith('sdm_parts') else '73.7'} "
                                  "M-sample launch of the same kernel, scaled by SDM input samples")

    plain = None
    if not args.no_plain and rank == 0:
        seg_in = WL["das_seg_len"] + 2 * WL["das_overlap"]
        t = torch.arange(2 * seg_in, dtype=torch.float64, device="cuda")
        gen = torch.Generator(device="cuda").manual_seed(7)
        x_dev = 0.3 * torch.sin(t * 0.0013) + 0.05 * torch.rand(2 * seg_in, dtype=torch.float64,
                                                                 device="cuda", generator=gen)
        plain_sps = plain_form(f, x_dev, seg_in, WL["das_overlap"], WL["lat"])
        batched_sps = sdm_samples / sdm_s
        plain = {"msamples_per_s": plain_sps / 1e6, "batched_msamples_per_s": batched_sps / 1e6,
                 "batched_over_plain": batched_sps / plain_sps,
                 "note": "SDM input samples/s; plain = one 81,920-sample DAS segment per launch"}

    cpu = parity = None
    if rank == 0 and not args.no_cpu_baseline:
        gpu_dop = d_out[:nbytes].cpu().numpy()
        parity, cpu = parity_and_cpu_baseline(pcm, gpu_dop, local)
        one = cpu_baseline(pcm, 0.1, nthreads=1)
        cpu["single_core"] = {"value": one["value"], "cores": 1, "sample": one["sample"]}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000 * total_s / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": dict(WL, seconds=args.seconds),
                "xrt": xrt,
                "e2e": {"value": e2e_value, "unit": UNIT,
                        "h2d_bytes_per_step": int(pcm.nbytes), "d2h_bytes_per_step": int(nb)},
                "roofline": roofline, "cpu_baseline": cpu, "clocks": clk,
                "parity": parity,
                "gpu_launches": int(launches), "stages_ms": stages, "plain": plain,
                "fp64_peak_gops": fp64_peak}
        names = [w for w in args.also.split(",") if w and w != "none"]
        if world == 1 and names:
            enc.close()
            enc = None
            del d_pcm, d_out, flush
            torch.cuda.empty_cache()
            line["also"] = run_also(names)
        print(json.dumps(line), flush=True)
    if enc is not None:
        enc.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


MS_METRIC = ("trellis SDM DSD Msamples/s, batched 64-stream form (one persistent launch per "
             "NTF under a CUDA graph) vs the plain per-segment launch")


def run_multistream(args):
    """The batched workload: 64 stereo streams, lengths U(0.5, 30) s, input
    rates {44.1, 48, 88.2, 96, 176.4, 192} kHz, DSD128/DSD256 targets of the
    matching family, band-limited Gaussian noise at -12 dBFS RMS, K = 32,
    depth 64, auto NTF and latency per rate, autotuned DAS segment length,
    DoP output.  One step converts every stream once."""
    import numpy as np
    import torch
    from foo_dsd_trellis_gb300 import ntf, signals
    from foo_dsd_trellis_gb300.batch import OUT_DOP, BatchPlan, StreamSpec
    from foo_dsd_trellis_gb300.pipeline import PCM_FIR_GAIN
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    layout = signals.multistream_layout(seed=1003 + 17 * rank, scale=args.ms_scale)
    specs = [StreamSpec(e["fs_in"], e["fs_out"], e["channels"], e["frames"],
                        ntf.auto_select(e["fs_out"]), cands=32, depth=64,
                        lat=ntf.auto_latency(e["fs_in"], e["fs_out"]), gain=PCM_FIR_GAIN,
                        boxcar_taps=8, soft_clip=True, reposition=True) for e in layout]
    pcms = [signals.multistream_pcm(e) for e in layout]
    plan = BatchPlan(specs, seg_len=args.ms_seg_len, output_format=OUT_DOP, device=local,
                     max_device_bytes=int(240e9))
    info = plan.info()
    plan.load([torch.from_numpy(x).cuda() for x in pcms])
    for _ in range(args.warmup):
        plan.run()
    peak = _probe_fp64(plan)
    clocks = ClockSampler(local)
    l0 = plan.launches()
    tot_ms, sdm_ms = [], []
    clocks.start()
    for _ in range(args.steps):
        plan.run()                        # inputs (125+ GB of FIR data) are far larger than L2
        t = plan.times_ms()
        tot_ms.append(t["total"])
        sdm_ms.append(t["sdm"])
    clk = clocks.stop()
    launches = (plan.launches() - l0) // max(1, args.steps)
    total_s = max_over_ranks(sum(tot_ms) / 1000.0)
    out_samples = int(info["out_samples"])
    value = job_throughput(out_samples, args.steps, world, total_s)
    dsd_seconds = sum(plan.out_samples(i) / s.fs_out for i, s in enumerate(specs))
    # FP64 work of the SDM launches: segment input samples x K x (5N + 6)
    flops = 0.0
    for i, s in enumerate(specs):
        n = s.frames * (s.fs_out // s.fs_in)
        ov = 64 * s.lat
        S = max(1, n // info["seg_len"])
        while S > 1 and n // S < max(4 * ov, 256):
            S -= 1
        seg_in = n + (2 * ov * (S - 1) if S > 1 else 0)
        flops += seg_in * s.channels * s.cands * (5 * s.ntf.order + 6)
    sdm_s = statistics.mean(sdm_ms) / 1000.0
    achieved = flops / sdm_s / 1e12
    # the plain form: the same kernel, one segment run per launch
    pj = 2
    p_smp, p_sec = plan.time_plain(pj)
    batched_sps = info["sdm_samples"] / sdm_s
    plain_sps = p_smp / p_sec
    # end to end through the host-buffer entry point (pinned host memory)
    h_in = [torch.from_numpy(x).pin_memory().numpy() for x in pcms]
    h_out = [torch.empty(plan.out_bytes(i), dtype=torch.uint8).pin_memory().numpy()
             for i in range(len(specs))]
    t0 = time.perf_counter()
    plan.run_host(h_in, h_out)
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    if rank == 0:
        line = {"metric": MS_METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000 * total_s / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": "multistream64_dsd128_dsd256", "streams": len(specs),
                           "lengths_s": "U(0.5, 30) x %g" % args.ms_scale,
                           "rates": [44100, 48000, 88200, 96000, 176400, 192000],
                           "targets": "DSD128/DSD256 of the input's family", "cands": 32,
                           "depth": 64, "ntf": "auto per rate (CLANS-6 / CLANS-8)",
                           "lat": "auto (128)", "signal": "band-limited Gaussian noise -12 dBFS",
                           "seg_len": info["seg_len"], "seg_len_source":
                               "autotuned" if args.ms_seg_len == 0 else "fixed",
                           "blocks_per_sm": info["blocks_per_sm"], "sdm_classes": info["classes"],
                           "seed_mode": "full_parallel", "output": "dop",
                           "l2": "inputs far larger than L2 (FIR data %.0f GB)" % (
                               info["device_bytes"] / 1e9)},
                "xrt": dsd_seconds * args.steps / total_s,
                "e2e": {"value": out_samples * world / e2e_s / 1e6, "unit": UNIT,
                        "h2d_bytes_per_step": int(sum(x.nbytes for x in pcms)),
                        "d2h_bytes_per_step": int(sum(plan.out_bytes(i) for i in range(len(specs))))},
                "batched_vs_plain": {"batched_sdm_msamples_per_s": batched_sps / 1e6,
                                     "plain_sdm_msamples_per_s": plain_sps / 1e6,
                                     "ratio": batched_sps / plain_sps,
                                     "plain_sample": f"{pj} segment runs, one launch each"},
                "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak / 1000.0,
                             "unit": "TFLOP/s", "frac": achieved / (peak / 1000.0),
                             "traffic": SDM_DRAM_BYTES_PER_SAMPLE * info["sdm_samples"],
                             "kernel": "sdm_jobs_kernel<6,32>, sdm_jobs_kernel<8,32> (concurrent)"},
                "cpu_baseline": None, "clocks": clk, "gpu_launches": int(launches),
                "plan": info, "stages_ms": plan.times_ms()}
        print(json.dumps(line), flush=True)
    plan.close()


MSP_METRIC = ("PreCorr greedy SDM DSD Msamples/s, batched 64-stream form (one launch per PreCorr "
              "parameter set, one thread per channel row)")


def run_multistream_precorr(args):
    """The 64-stream layout of multistream64 in PreCorr mode (src/precorr.c:20-287):
    the same streams, lengths and signals, the PreCorr NTF per rate
    (ntf_auto_select_precorr), state limit 12, FIR chain without the soft clip,
    DoP output.  One step converts every stream once; the walk is one thread
    per channel row, so the step is as long as the longest stream's walk.  The
    CPU leg runs the oracle's PreCorr (pinned to src/precorr.c) on the eight
    shortest streams' chain outputs on every host core and checks their DoP
    bytes against the GPU's."""
    import concurrent.futures as cf

    import numpy as np
    import torch
    from foo_dsd_trellis_gb300 import ntf, signals
    from foo_dsd_trellis_gb300.batch import OUT_DOP, BatchPlan, StreamSpec
    from foo_dsd_trellis_gb300.fir import FirChain
    from foo_dsd_trellis_gb300.pipeline import PCM_FIR_GAIN
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    layout = signals.multistream_layout(seed=1003 + 17 * rank, scale=args.ms_scale)
    specs = [StreamSpec(e["fs_in"], e["fs_out"], e["channels"], e["frames"],
                        ntf.auto_select_precorr(e["fs_out"]), state_limit=12.0,
                        gain=PCM_FIR_GAIN, boxcar_taps=8, soft_clip=False, reposition=False,
                        precorr=True) for e in layout]
    pcms = [signals.multistream_pcm(e) for e in layout]
    plan = BatchPlan(specs, seg_len=0, output_format=OUT_DOP, device=local,
                     max_device_bytes=int(240e9))
    info = plan.info()
    plan.load([torch.from_numpy(x).cuda() for x in pcms])
    for _ in range(args.warmup):
        plan.run()
    clocks = ClockSampler(local)
    l0 = plan.launches()
    tot_ms = []
    clocks.start()
    for _ in range(args.steps):
        plan.run()
        tot_ms.append(plan.times_ms()["total"])
    clk = clocks.stop()
    launches = (plan.launches() - l0) // max(1, args.steps)
    total_s = max_over_ranks(sum(tot_ms) / 1000.0)
    out_samples = int(info["out_samples"])
    value = job_throughput(out_samples, args.steps, world, total_s)
    rows = sum(s.channels for s in specs)
    longest = max(s.frames * (s.fs_out // s.fs_in) for s in specs)
    h_in = [torch.from_numpy(x).pin_memory().numpy() for x in pcms]
    h_out = [torch.empty(plan.out_bytes(i), dtype=torch.uint8).pin_memory().numpy()
             for i in range(len(specs))]
    t0 = time.perf_counter()
    plan.run_host(h_in, h_out)
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle as O
        short = sorted(range(len(specs)), key=lambda i: specs[i].frames)[:8]
        firs = {}
        for i in short:
            s = specs[i]
            fc = FirChain(s.fs_in, s.fs_out, boxcar_taps=s.boxcar_taps, soft_clip=False,
                          num_channels=s.channels, device=local)
            firs[i] = fc.process(torch.from_numpy(pcms[i]).cuda(), PCM_FIR_GAIN, PCM_FIR_GAIN).cpu().numpy()
            fc.close()
        work = [(i, c) for i in short for c in range(specs[i].channels)]

        def walk(ic):
            i, c = ic
            s = specs[i]
            return O.PreCorr(s.ntf.order, np.array(s.ntf.a), np.array(s.ntf.g), 12.0).process(firs[i][c])

        nthreads = os.cpu_count() or 1
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(nthreads) as ex:
            bits = list(ex.map(walk, work))
        t_cpu = time.perf_counter() - t0
        same = True
        k = 0
        for i in short:
            s = specs[i]
            per = []
            for c in range(s.channels):
                per.append(O.dop_pack_bits(bits[k], 0)[0].reshape(-1, 3))
                k += 1
            want = np.stack(per, axis=1).reshape(-1)
            got = plan.out_view(i).cpu().numpy()
            same = same and got.shape == want.shape and bool(np.array_equal(got, want))
        n_cpu = sum(len(b) for b in bits)
        cpu = {"value": n_cpu / t_cpu / 1e6, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": f"the 8 shortest streams ({len(work)} channel rows, {n_cpu} samples): "
                         "the oracle's PreCorr on the GPU's chain output, one row per thread",
               "bit_exact_with_gpu": same}
    if rank == 0:
        line = {"metric": MSP_METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000 * total_s / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": "multistream64_precorr", "streams": len(specs),
                           "channel_rows": rows, "lengths_s": "U(0.5, 30) x %g" % args.ms_scale,
                           "rates": [44100, 48000, 88200, 96000, 176400, 192000],
                           "targets": "DSD128/DSD256 of the input's family",
                           "ntf": "auto_select_precorr per rate", "state_limit": 12.0,
                           "precorr_classes": "one per NTF", "output": "dop",
                           "l2": "inputs far larger than L2"},
                "xrt": sum(plan.out_samples(i) / s.fs_out for i, s in enumerate(specs)) *
                       args.steps / total_s,
                "e2e": {"value": out_samples * world / e2e_s / 1e6, "unit": UNIT,
                        "h2d_bytes_per_step": int(sum(x.nbytes for x in pcms)),
                        "d2h_bytes_per_step": int(sum(plan.out_bytes(i) for i in range(len(specs))))},
                "walk": {"longest_row_samples": longest,
                         "longest_row_msamples_per_s": longest * args.steps / total_s / 1e6,
                         "note": "one thread per channel row: the step lasts as long as the "
                                 "longest row's walk (the FP32 recurrence through the previous "
                                 "output)"},
                "roofline": None, "cpu_baseline": cpu, "clocks": clk,
                "gpu_launches": int(launches), "plan": info, "stages_ms": plan.times_ms()}
        print(json.dumps(line), flush=True)
    plan.close()


MSD_METRIC = ("same-rate DSD re-encode DSD Msamples/s, batched 64-stream form (DoP in -> unpack -> "
              "boxcar -> DAS trellis SDM -> DoP, one persistent launch per parameter set)")


def run_multistream_dsd(args):
    """The 64-stream layout of multistream64 with DoP input at each stream's
    DSD rate (DSD128 / DSD256): the same-rate re-encode of the engine's path
    table (CLANS-6 or the rate's NTF, K = 2, depth 4, lat 128, the rate's
    default 64-tap boxcar, path gain float32(0.708), DAS, DoP out) for every
    stream in one plan.  The DSD input is each stream's PCM encoded by this
    library's batched PCM path (set-up, untimed).  Parity: the four shortest
    streams against the single-stream pipeline on fresh contexts."""
    import numpy as np
    import torch
    from foo_dsd_trellis_gb300 import ntf, signals
    from foo_dsd_trellis_gb300.batch import OUT_BITS, OUT_DOP, BatchPlan, StreamSpec
    from foo_dsd_trellis_gb300.pipeline import FULL_PARALLEL, PCM_FIR_GAIN, Encoder
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    layout = signals.multistream_layout(seed=1003 + 17 * rank, scale=args.ms_scale)
    # the DSD sources: the PCM streams through the batched PCM path (decision bytes)
    src = BatchPlan([StreamSpec(e["fs_in"], e["fs_out"], e["channels"], e["frames"],
                                ntf.auto_select(e["fs_out"]), cands=2, depth=4,
                                lat=ntf.auto_latency(e["fs_in"], e["fs_out"]), gain=PCM_FIR_GAIN)
                     for e in layout], seg_len=65536, output_format=OUT_BITS, device=local,
                    max_device_bytes=int(240e9))
    src.load([torch.from_numpy(signals.multistream_pcm(e)).cuda() for e in layout])
    src.run()
    dops = []
    for i, e in enumerate(layout):
        b = src.out_view(i).cpu().numpy()
        n = b.shape[1] - b.shape[1] % 16
        dops.append(np.stack([signals.dop_floats(b[c, :n], 0) for c in range(e["channels"])]))
    src.close()
    gain = float(np.float32(PATH_GAIN))
    specs = [StreamSpec(e["fs_out"], e["fs_out"], e["channels"], dops[i].shape[1],
                        ntf.get_filter("clans-6", e["fs_out"]), cands=2, depth=4, lat=128,
                        gain=gain, boxcar_taps=0, soft_clip=False, reposition=True)
             for i, e in enumerate(layout)]
    plan = BatchPlan(specs, seg_len=65536, output_format=OUT_DOP, device=local,
                     max_device_bytes=int(240e9), lanes=args.ms_lanes or None)
    info = plan.info()
    plan.load([torch.from_numpy(x).cuda() for x in dops])
    for _ in range(args.warmup):
        plan.run()
    clocks = ClockSampler(local)
    l0 = plan.launches()
    tot_ms = []
    clocks.start()
    for _ in range(args.steps):
        plan.run()
        tot_ms.append(plan.times_ms()["total"])
    clk = clocks.stop()
    launches = (plan.launches() - l0) // max(1, args.steps)
    total_s = max_over_ranks(sum(tot_ms) / 1000.0)
    out_samples = int(info["out_samples"])
    value = job_throughput(out_samples, args.steps, world, total_s)
    h_in = [torch.from_numpy(x).pin_memory().numpy() for x in dops]
    h_out = [torch.empty(plan.out_bytes(i), dtype=torch.uint8).pin_memory().numpy()
             for i in range(len(specs))]
    t0 = time.perf_counter()
    plan.run_host(h_in, h_out)
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    same = True
    for i in sorted(range(len(specs)), key=lambda i: specs[i].frames)[:4]:
        s = specs[i]
        enc = Encoder(s.fs_in, s.fs_out, s.channels, s.ntf, s.depth, s.cands, s.lat,
                      seg_len=65536, seed_mode=FULL_PARALLEL, reposition=True, boxcar_taps=0,
                      soft_clip=False, output_format=OUT_DOP, device=local)
        buf = torch.empty(enc.out_capacity(s.frames) + 64, dtype=torch.uint8, device="cuda")
        _, nb = enc.process(torch.from_numpy(dops[i]).cuda(), buf, gain, gain)
        enc.close()
        same = same and bool(np.array_equal(buf[:nb].cpu().numpy(), plan.out_view(i).cpu().numpy()))
    if rank == 0:
        line = {"metric": MSD_METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000 * total_s / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": "multistream64_dsd_samerate", "streams": len(specs),
                           "lengths_s": "U(0.5, 30) x %g" % args.ms_scale,
                           "rates": "DSD128 / DSD256 (each stream's multistream64 target)",
                           "ntf": "clans-6", "cands": 2, "depth": 4, "lat": 128,
                           "lanes_per_job": args.ms_lanes or "the plan's choice",
                           "boxcar": "the rate's default (64)", "gain": "float32(0.708)",
                           "seed_mode": "full_parallel", "output": "dop",
                           "input": "DoP floats of the streams' PCM encoded by the batched PCM "
                                    "path (untimed)", "l2": "inputs larger than L2"},
                "xrt": sum(plan.out_samples(i) / s.fs_out for i, s in enumerate(specs)) *
                       args.steps / total_s,
                "e2e": {"value": out_samples * world / e2e_s / 1e6, "unit": UNIT,
                        "h2d_bytes_per_step": int(sum(x.nbytes for x in dops)),
                        "d2h_bytes_per_step": int(sum(plan.out_bytes(i) for i in range(len(specs))))},
                "parity": {"bit_exact_with_pipeline": same,
                           "sample": "the four shortest streams against the single-stream "
                                     "pipeline on fresh contexts"},
                "roofline": None, "cpu_baseline": None, "clocks": clk,
                "gpu_launches": int(launches), "plan": info, "stages_ms": plan.times_ms()}
        print(json.dumps(line), flush=True)
    plan.close()


DIFF_METRIC = ("adjoint ms: STE gradient of the in-band loss w.r.t. 127 pre-emphasis taps and "
               "the order-7 NTF, 16 clips x 2^20 DSD128 samples, checkpoints every 4096")


def run_diff(args):
    """The differentiation workload: 16 mono clips of 8192 frames at 44.1 kHz
    (31-tone multitone at -26 dBFS per tone plus pink noise at -40 dBFS,
    seeded) -> 127-tap pre-emphasis (unit impulse + N(0, 1e-3)) -> FP64 chain
    to DSD128 (2^20 samples per clip) -> exact trellis SDM (CLANS-7, K = 32,
    depth 64, lat 128) -> in-band loss (255-tap 20 kHz low-pass, decimation
    64).  One step is one backward pass (the adjoint); the forward, the exact
    SDM inside it and a surrogate evaluation are reported beside it, with a
    32-direction FP64 central-difference check (h = 1e-6) of the gradient."""
    import numpy as np
    import torch
    from foo_dsd_trellis_gb300 import ntf, signals
    from foo_dsd_trellis_gb300.diff import DiffConfig, DiffEngine
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    cfg = DiffConfig()
    f = ntf.get_filter("clans-7", cfg.fs_out)
    x = np.empty((cfg.nclips, cfg.frames), np.float32)
    for c in range(cfg.nclips):
        rng = np.random.Generator(np.random.PCG64(1004 + 31 * rank + c))
        x[c] = (signals.multitone(cfg.frames, cfg.fs_in, rng, level_db=-26.0)
                + signals.pink_noise(cfg.frames, rng, signals.db_to_amp(-40.0))).astype(np.float32)
    eng = DiffEngine(cfg, f, local)
    eng.set_input(torch.from_numpy(x).cuda())
    rng = np.random.default_rng(5)
    taps = rng.normal(0.0, 1e-3, cfg.preemph_taps)
    taps[0] += 1.0
    a, g = np.array(f.a[: f.order]), np.array(f.g[: f.order])
    loss = eng.forward(taps, a, g)
    fwd = eng.times_ms()
    for _ in range(args.warmup):
        eng.backward()
    clocks = ClockSampler(local)
    l0 = eng.launches()
    clocks.start()
    adj = []
    for _ in range(args.steps):
        gt, ga, gg = eng.backward()
        adj.append(eng.times_ms()["adjoint"])
    clk = clocks.stop()
    launches = (eng.launches() - l0) // max(1, args.steps)
    sur = eng.surrogate(taps, a, g)
    sur_ms = eng.times_ms()["surrogate"]
    # finite differences of the surrogate on random unit directions
    h = 1e-6
    worst = worst_rich = 0.0
    drng = np.random.default_rng(7)
    for _ in range(args.fd_dirs):
        # absolute for the taps, relative for the NTF coefficients
        dt = drng.standard_normal(taps.size)
        da = a * drng.standard_normal(a.size)
        dg = g * drng.standard_normal(g.size)
        ad = gt @ dt + ga @ da + gg @ dg
        fd = {}
        for hh in (h, h / 2):
            lp = eng.surrogate(taps + hh * dt, a + hh * da, g + hh * dg)
            lm = eng.surrogate(taps - hh * dt, a - hh * da, g - hh * dg)
            fd[hh] = (lp - lm) / (2 * hh)
        rich = (4 * fd[h / 2] - fd[h]) / 3
        worst = max(worst, abs(fd[h] - ad) / max(abs(fd[h]), abs(ad), 1e-300))
        worst_rich = max(worst_rich, abs(rich - ad) / max(abs(rich), abs(ad), 1e-300))
    adj_ms = statistics.mean(adj)
    max_ms = max_over_ranks(adj_ms / 1000.0) * 1000.0
    n = cfg.frames * (cfg.fs_out // cfg.fs_in)
    if rank == 0:
        line = {"metric": DIFF_METRIC, "value": max_ms, "unit": "ms", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": max_ms,
                "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic",
                "config": {"workload": "diff16_dsd128", "clips": cfg.nclips,
                           "samples_per_clip": n, "pcm": "44.1 kHz multitone + pink noise",
                           "preemph_taps": cfg.preemph_taps, "ntf": "clans-7", "cands": cfg.cands,
                           "depth": cfg.depth, "lat": cfg.lat, "checkpoint": cfg.checkpoint,
                           "loss": "255-tap 20 kHz low-pass, decimation 64, mean square",
                           "kappa": cfg.kappa, "l2": "state and adjoint data larger than L2"},
                "loss": loss, "surrogate_at_forward": sur,
                "forward_ms": fwd["forward"], "exact_sdm_ms": fwd["exact_sdm"],
                "surrogate_ms": sur_ms,
                "forward_plus_adjoint_over_adjoint": (fwd["forward"] + max_ms) / max_ms,
                "fd_check": {"directions": args.fd_dirs, "h": h, "worst_rel_err": worst,
                             "direction": "taps N(0,1); a_i N(0,1) a_i; g_i N(0,1) g_i",
                             "worst_rel_err_richardson_h_h2": worst_rich, "tolerance": 1e-4},
                "grad_norms": {"taps": float(np.linalg.norm(gt)), "a": float(np.linalg.norm(ga)),
                               "g": float(np.linalg.norm(gg))},
                "e2e": None, "roofline": None, "cpu_baseline": None, "clocks": clk,
                "gpu_launches": int(launches)}
        print(json.dumps(line), flush=True)
    eng.close()


CONV_METRIC = ("trellis SDM DSD Msamples/s & xRT at DSD512 5.1 with UPOLS room convolution "
               "(P = 4096, 65,536-tap IR), K = 16, depth 48, DAS 262,144, DoP")


def room_ir(taps: int, fs: float, seed: int, t60: float = 0.4) -> "np.ndarray":
    """Synthetic room IR: seeded Gaussian noise under an exponential decay of
    60 dB per t60 seconds, scaled so the peak of its magnitude response is 1
    (0 dB), which keeps the SDM input in range."""
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(seed))
    k = np.arange(taps)
    h = rng.standard_normal(taps) * 10.0 ** (-3.0 * k / (t60 * fs))
    peak = np.abs(np.fft.rfft(h, 4 * taps)).max()
    return (h / peak).astype(np.float32)


def run_conv(args):
    """DSD512 5.1: 6 channels of 5 s of 48 kHz pink noise at -18 dBFS (seeded)
    -> 9-stage FIR chain to 24.576 MHz (127-tap first stage, boxcar 8, engine
    gain and soft clip) -> UPOLS convolution per channel with its own 65,536-tap
    room IR (P = 4096, FP32) -> trellis SDM (auto NTF for DSD512, K = 16,
    depth 48, lat 32) over 262,144-sample DAS segments (full-parallel
    seeding, the reference's DSD512 mode) -> DoP."""
    import numpy as np
    import torch
    from foo_dsd_trellis_gb300 import ntf, signals
    from foo_dsd_trellis_gb300.pipeline import OUT_DOP, PCM_FIR_GAIN, Encoder, FULL_PARALLEL
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    fs_in, fs_out, nch, secs = 48000, 24576000, 6, args.seconds if args.seconds != WL["seconds"] else 5.0
    K, depth, lat, seg = 16, 48, ntf.auto_latency(48000, 24576000), 262144
    f = ntf.auto_select(fs_out)
    n = int(round(secs * fs_in))
    pcm = np.empty((nch, n), np.float32)
    for c in range(nch):
        rng = np.random.Generator(np.random.PCG64(1005 + 10 * rank + c))
        pcm[c] = signals.pink_noise(n, rng, signals.db_to_amp(-18.0)).astype(np.float32)
    irs = np.stack([room_ir(65536, fs_out, 2005 + 10 * rank + c) for c in range(nch)])
    enc = Encoder(fs_in, fs_out, nch, f, depth, K, lat, seg_len=seg, seed_mode=FULL_PARALLEL,
                  reposition=True, boxcar_taps=8, soft_clip=True, output_format=OUT_DOP,
                  device=local)
    enc.set_conv(irs, 4096)
    d_pcm = torch.from_numpy(pcm).cuda()
    d_out = torch.empty(enc.out_capacity(n) + 64, dtype=torch.uint8, device="cuda")
    lib_stream = torch.cuda.ExternalStream(enc.stream_ptr)
    for _ in range(args.warmup):
        enc.process(d_pcm, d_out)
    torch.cuda.synchronize()
    fp64_peak = enc.probe_fp64_gops()
    clocks = ClockSampler(local)
    l0 = enc.launches()
    w0, _ = enc.sdm_work()
    step_ms, sdm_ms = [], []
    clocks.start()
    for _ in range(args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(lib_stream)
        ns, nb = enc.process(d_pcm, d_out)       # 5 s x 6 ch of data far larger than L2
        e1.record(lib_stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        sdm_ms.append(enc.stage_ms()["sdm"])
    clk = clocks.stop()
    launches = (enc.launches() - l0) // max(1, args.steps)
    sdm_samples = (enc.sdm_work()[0] - w0) / args.steps
    total_s = max_over_ranks(sum(step_ms) / 1000.0)
    value = job_throughput(ns * nch, args.steps, world, total_s)
    h_pcm = torch.from_numpy(pcm).pin_memory().numpy()
    h_out = torch.empty(enc.out_capacity(n) + 64, dtype=torch.uint8).pin_memory().numpy()
    t0 = time.perf_counter()
    ns2, nb2 = enc.process_host(h_pcm, h_out)
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    sdm_s = statistics.mean(sdm_ms) / 1000.0
    flops = sdm_samples * K * (5 * f.order + 6)
    if rank == 0:
        st = enc.stage_ms()
        line = {"metric": CONV_METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000 * total_s / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": "dsd512_51_upols", "fs_in": fs_in, "fs_out": fs_out,
                           "channels": nch, "seconds": secs, "signal": "pink noise -18 dBFS",
                           "ir_taps": 65536, "partition": 4096, "conv_dtype": "f32",
                           "ntf": f.name, "cands": K, "depth": depth, "lat": lat,
                           "das_seg_len": seg, "seed_mode": "full_parallel", "output": "dop",
                           "l2": "working set far larger than L2"},
                "xrt": ns / fs_out * args.steps / total_s,
                "e2e": {"value": ns2 * nch / e2e_s / 1e6, "unit": UNIT,
                        "h2d_bytes_per_step": int(pcm.nbytes), "d2h_bytes_per_step": int(nb2)},
                "roofline": {"bound": "fp64", "achieved": flops / sdm_s / 1e12,
                             "peak": fp64_peak / 1000.0, "unit": "TFLOP/s",
                             "frac": flops / sdm_s / 1e12 / (fp64_peak / 1000.0),
                             "traffic": SDM_DRAM_BYTES_PER_SAMPLE * sdm_samples,
                             "traffic_source": "9.04 B per SDM input sample (ncu, sdm_jobs_kernel "
                                               "at K = 32), scaled by SDM input samples",
                             "kernel": enc.last_sdm_kernel()},
                "cpu_baseline": None, "clocks": clk, "gpu_launches": int(launches),
                "stages_ms": st}
        print(json.dumps(line), flush=True)
    enc.close()


SEG0_METRIC = ("DSD128 trellis SDM + DAS with the reference's own seeding rule below DSD512 "
               "(seg0-first), 1 s chunks of one stream, DSD Msamples/s")


def run_seg0first(args):
    """The headline's signal and trellis (DSD128 stereo, 48 kHz multitone + pink,
    CLANS-7, K = 32, depth 64, lat 128, 65,536-sample segments) under the
    reference's DSD128 seeding rule, seg0-first (src/dsp_plugin.c:2185-2283):
    seg0 serial on the channel's context, seg1 DIRECT from its end state, the
    16-level estimator walked serially over the rest of the chunk, then seg2+
    in parallel.  The input is one stream converted in 1 s chunks (the state
    carried from chunk to chunk as the plugin carries it), so each chunk has
    two serial trellis runs and one serial estimator pass on its critical
    path.  The CPU leg is the oracle's port of the same chunks on every host
    core; decisions are checked against it."""
    import numpy as np
    import torch
    from oracle import oracle as O
    from foo_dsd_trellis_gb300 import ntf, signals
    from foo_dsd_trellis_gb300.fir import FirChain
    from foo_dsd_trellis_gb300.pipeline import OUT_BITS, PCM_FIR_GAIN, SEG0_FIRST, Encoder
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    secs = args.seconds if args.seconds != WL["seconds"] else 2.0
    chunk = WL["fs_in"]                               # 1 s of input per chunk
    f = ntf.get_filter(WL["ntf"], WL["fs_out"])
    pcm = signals.dsd128_multitone_pink(secs, WL["fs_in"], WL["channels"], WL["seed"])
    nch, frames = pcm.shape
    nchunks = frames // chunk
    enc = Encoder(WL["fs_in"], WL["fs_out"], nch, f, WL["depth"], WL["cands"], WL["lat"],
                  seg_len=WL["das_seg_len"], seed_mode=SEG0_FIRST, reposition=True,
                  boxcar_taps=WL["boxcar_taps"], soft_clip=True, output_format=OUT_BITS,
                  device=local)
    d_pcm = [torch.from_numpy(np.ascontiguousarray(pcm[:, k * chunk:(k + 1) * chunk])).cuda()
             for k in range(nchunks)]
    ratio = WL["fs_out"] // WL["fs_in"]
    outs = [torch.empty((nch, chunk * ratio + 256), dtype=torch.uint8, device="cuda")
            for _ in range(nchunks)]
    lib_stream = torch.cuda.ExternalStream(enc.stream_ptr)

    def one_pass():
        enc.flush()
        counts = []
        for k in range(nchunks):
            n, _ = enc.process(d_pcm[k], outs[k])
            counts.append(n)
        return counts

    for _ in range(args.warmup):
        one_pass()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    step_ms = []
    counts = []
    for _ in range(args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(lib_stream)
        counts = one_pass()
        e1.record(lib_stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    total_s = sum(step_ms) / 1000.0
    n_out = sum(counts) * nch
    value = n_out * args.steps / total_s / 1e6
    got = [outs[k][:, :counts[k]].cpu().numpy() for k in range(nchunks)]

    # the oracle on the GPU's FIR output of the same chunks (carry across chunks)
    fc = FirChain(WL["fs_in"], WL["fs_out"], boxcar_taps=WL["boxcar_taps"], soft_clip=True,
                  num_channels=nch, device=local)
    carry = [O.sdm(f.order, np.array(f.a), np.array(f.g), WL["depth"], WL["cands"], WL["lat"])
             for _ in range(nch)]
    nthreads = os.cpu_count() or 1
    t_cpu = 0.0
    same = True
    for k in range(nchunks):
        fir = fc.process(d_pcm[k], PCM_FIR_GAIN, PCM_FIR_GAIN).cpu().numpy()
        t0 = time.perf_counter()
        want, _, _ = O.das_run(f.order, np.array(f.a), np.array(f.g), WL["depth"], WL["cands"],
                               WL["lat"], 0.0, fir, seg_len=WL["das_seg_len"], seed_mode=1,
                               reposition=True, nthreads=nthreads, carry=carry)
        t_cpu += time.perf_counter() - t0
        same = same and want.shape == got[k].shape and bool(np.array_equal(want, got[k]))
    fc.close()
    cpu_value = n_out / t_cpu / 1e6
    stages = enc.stage_ms()
    line = {"metric": SEG0_METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * total_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": dict(WL, workload="dsd128_seg0first_stereo_1s_chunks", seconds=secs,
                           seed_mode="seg0_first", chunk_frames=chunk,
                           l2="inputs stream through chunk by chunk; no flush"),
            "xrt": (sum(counts) / WL["fs_out"]) * args.steps / total_s,
            "parity": {"bit_exact": same, "oracle": "oracle DAS with the chunk carry on the "
                       "GPU's FIR output of every chunk"},
            "cpu_baseline": {"value": cpu_value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": f"the same {nchunks} chunks: trellis SDM port + DAS "
                                       "(seg0-first, carry) on the GPU's FIR output"},
            "last_chunk_stages_ms": stages, "clocks": clk}
    print(json.dumps(line), flush=True)
    enc.close()


def _probe_fp64(plan) -> float:
    import ctypes as C
    v = C.c_double()
    rc = plan.L.dsdgpu_probe_fp64(plan.h, C.byref(v))
    return v.value if rc == 0 else float("nan")


NEXT = {
    "samerate128": dict(
        metric="same-rate DSD128 re-encode (DoP in -> unpack -> 64-tap boxcar -> DAS trellis "
               "SDM -> DoP) DSD Msamples/s, bit-exact",
        workload="samerate_dsd128_stereo_10s", fs=5644800,
        path_table="DSD128 -> DSD128 row of the engine's path table (src/engine.c:61); lat 0 "
                   "there = auto = 128 at DSD128 (src/engine.c:1008-1021)",
        ntf="clans-6", cands=2, depth=4, lat=128, das_seg_len=65536, boxcar_taps=64,
        gain="float32(0.708) (path gain)"),
    "samerate128lp": dict(
        metric="same-rate DSD128 re-encode with the FIR lowpass (DoP in -> unpack -> 127-tap "
               "FP64 lowpass at 50 kHz -> DAS trellis SDM -> DoP) DSD Msamples/s, bit-exact",
        workload="samerate_lowpass_dsd128_stereo_10s", fs=5644800,
        path_table="DSD128 -> DSD128 row of the engine's path table (src/engine.c:61) with "
                   "fir_mode FIR (src/engine.c:168-181)",
        ntf="clans-6", cands=2, depth=4, lat=128, das_seg_len=65536, lowpass_taps=127,
        lowpass_cutoff_hz=50000.0, gain="float32(0.708) (path gain)"),
    "dsd256to128": dict(
        metric="DSD256 -> DSD128 re-encode through the plugin's DAS path (DoP in -> unpack -> "
               "FP64 half-band /2 -> gain, engine_process_fir_gain -> DAS trellis SDM -> DoP) "
               "DSD Msamples/s, bit-exact given the FIR stage",
        workload="dsd256_to_dsd128_stereo_10s", fs_in=11289600, fs=5644800,
        path_table="DSD256 -> DSD128 row of the engine's path table (src/engine.c:78): SDM-6, "
                   "K = 2, depth 8; lat 0 there = auto = 128 at DSD128",
        ntf="sdm-6", cands=2, depth=8, lat=128, das_seg_len=65536, boxcar_taps=0,
        soft_clip=False, gain="float32(0.708) (path gain)"),
    "precorr128": dict(
        metric="PCM 44.1 kHz -> DSD128 with the PreCorr SDM (FIR chain -> PreCorr -> DoP) "
               "DSD Msamples/s, bit-exact SDM",
        workload="precorr_dsd128_stereo_10s", fs_in=44100, fs=5644800, ntf="clans-7 (PreCorr auto)",
        state_limit=12.0, boxcar_taps=8, soft_clip=False),
    "dsd2pcm128": dict(
        metric="DSD128 -> 44.1 kHz PCM (DoP in -> unpack -> 7 half-band /2 FP64 stages -> "
               "float32) DSD input Msamples/s, float32 output within 2e-7 of the FP64 restatement",
        workload="dsd2pcm_dsd128_stereo_10s", fs=5644800, fs_out=44100, stages=7, taps=63),
}
PATH_GAIN = 0.708   # the engine's path gain (a float), include/dsd_types.h path table


def _dsd128_source(secs: float, nch: int, seed: int, rate: int = 5644800):
    """A DSD decision stream (DSD128 unless `rate` says otherwise) for the
    DSD-input workloads: the 44.1 kHz multitone + pink noise through this
    library's PCM path (set-up, untimed)."""
    import numpy as np
    import torch
    from foo_dsd_trellis_gb300 import ntf, signals
    from foo_dsd_trellis_gb300.pipeline import FULL_PARALLEL, OUT_BITS, PCM_FIR_GAIN, Encoder
    pcm = signals.dsd128_multitone_pink(secs, 44100, nch, seed)
    f = ntf.get_filter("clans-7", rate)
    src = Encoder(44100, rate, nch, f, 64, 32, 128, seg_len=65536, seed_mode=FULL_PARALLEL,
                  output_format=OUT_BITS)
    bits = torch.empty((nch, pcm.shape[1] * (rate // 44100) + 256), dtype=torch.uint8,
                       device="cuda")
    ns, _ = src.process(torch.from_numpy(pcm).cuda(), bits, PCM_FIR_GAIN, PCM_FIR_GAIN)
    src.close()
    return bits[:, : ns - ns % 16].cpu().numpy()


def _next_input(wl: str, secs: float, nch: int, seed: int):
    import numpy as np
    from foo_dsd_trellis_gb300 import signals
    if wl == "precorr128":
        return signals.dsd128_multitone_pink(secs, 44100, nch, seed), None
    bits = _dsd128_source(secs, nch, seed, NEXT[wl].get("fs_in", 5644800))
    return np.stack([signals.dop_floats(bits[c], 0) for c in range(nch)]), bits


def _next_cpu(wl: str, inp, bits, sample_s: float) -> dict:
    """The CPU leg of a DSD-path workload: the oracle's C port on a leading
    slice, one thread per channel where the path is serial per channel."""
    import numpy as np
    from concurrent.futures import ThreadPoolExecutor
    from oracle import oracle as O
    from foo_dsd_trellis_gb300 import ntf
    O.build()
    cfg = NEXT[wl]
    nch = inp.shape[0]
    fs = cfg["fs"]
    if wl in ("samerate128", "samerate128lp"):
        frames = int(sample_s * fs) // 16
        x = inp[:, :frames]
        nthreads = os.cpu_count() or 1
        f = ntf.get_filter(cfg["ntf"], fs)
        g = float(np.float32(PATH_GAIN))
        t0 = time.perf_counter()
        if wl == "samerate128":
            box = np.stack([O.Boxcar(cfg["boxcar_taps"]).process(O.dop_unpack(x[c]), g, g)
                            for c in range(nch)])
        else:
            box = np.stack([O.Lowpass(fs, cfg["lowpass_cutoff_hz"], cfg["lowpass_taps"])
                            .process(O.dop_unpack(x[c]), g, g) for c in range(nch)])
        out, _, _ = O.das_run(f.order, np.array(f.a), np.array(f.g), cfg["depth"], cfg["cands"],
                              cfg["lat"], 0.0, box, seg_len=cfg["das_seg_len"], seed_mode=0,
                              reposition=True, nthreads=nthreads)
        for c in range(nch):
            O.dop_pack_bits(out[c], 0)
        dt = time.perf_counter() - t0
        n = out.shape[0] * out.shape[1]
        what = ("DoP unpack + " + ("boxcar" if wl == "samerate128" else "FP64 lowpass restatement")
                + " + trellis SDM port + DAS + DoP")
    elif wl == "dsd256to128":
        fs_in = cfg["fs_in"]
        frames = int(sample_s * fs_in) // 16
        x = inp[:, :frames]
        nthreads = os.cpu_count() or 1
        f = ntf.get_filter(cfg["ntf"], fs)
        g = float(np.float32(PATH_GAIN))
        t0 = time.perf_counter()
        fir = np.stack([O.engine_down(O.Boxcar(max(1, cfg["boxcar_taps"])),
                                      O.Decimator(fs_in, fs), O.dop_unpack(x[c]), g, g,
                                      cfg["soft_clip"]) for c in range(nch)])
        out, _, _ = O.das_run(f.order, np.array(f.a), np.array(f.g), cfg["depth"], cfg["cands"],
                              cfg["lat"], 0.0, fir, seg_len=cfg["das_seg_len"], seed_mode=0,
                              reposition=True, nthreads=nthreads)
        for c in range(nch):
            O.dop_pack_bits(out[c], 0)
        dt = time.perf_counter() - t0
        n = out.shape[0] * out.shape[1]
        what = "DoP unpack + boxcar + FP64 decimation restatement + trellis SDM port + DAS + DoP"
    elif wl == "precorr128":
        frames = int(sample_s * 44100)
        x = inp[:, :frames]
        nthreads = nch
        f = ntf.auto_select_precorr(fs)
        from foo_dsd_trellis_gb300.pipeline import PCM_FIR_GAIN

        def one(c):
            y = O.engine_fir(44100, fs, x[c], boxcar_taps=8, g_start=PCM_FIR_GAIN,
                             g_end=PCM_FIR_GAIN, soft_clip=False)
            b = O.PreCorr(f.order, np.array(f.a), np.array(f.g), cfg["state_limit"]).process(y)
            O.dop_pack_bits(b, 0)
            return len(b)
        t0 = time.perf_counter()
        with ThreadPoolExecutor(nch) as ex:
            n = sum(ex.map(one, range(nch)))
        dt = time.perf_counter() - t0
        what = "FP64 FIR restatement + PreCorr port (bit-identical to precorr.c) + DoP"
    else:
        frames = int(sample_s * fs) // 16
        x = inp[:, :frames]
        nthreads = nch

        def one(c):
            d = O.dop_unpack(x[c])
            O.Decimator(fs, cfg["fs_out"]).process(d)
            return len(d)
        t0 = time.perf_counter()
        with ThreadPoolExecutor(nch) as ex:
            n = sum(ex.map(one, range(nch)))
        dt = time.perf_counter() - t0
        what = "DoP unpack + FP64 decimation restatement"
    return {"value": n / dt / 1e6, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"first {sample_s:g} s of the workload ({nch} ch): {what}", "seconds": dt}


def run_next(args):
    """The DSD re-encode, PreCorr and DSD -> PCM workloads: 10 s stereo at
    DSD128 through the whole-path pipeline (device buffers), the host-buffer
    entry point for e2e, and the oracle's port for the CPU leg."""
    import numpy as np
    import torch
    from foo_dsd_trellis_gb300 import _lib, ntf
    from foo_dsd_trellis_gb300.pipeline import FULL_PARALLEL, OUT_DOP, PCM_FIR_GAIN, Encoder
    wl = args.workload
    cfg = NEXT[wl]
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    nch, fs = 2, cfg["fs"]
    inp, _ = _next_input(wl, args.seconds, nch, 1101 + 2 * rank)
    if wl in ("samerate128", "samerate128lp"):
        f = ntf.get_filter(cfg["ntf"], fs)
        g = float(np.float32(PATH_GAIN))
        enc = Encoder(fs, fs, nch, f, cfg["depth"], cfg["cands"], cfg["lat"],
                      seg_len=cfg["das_seg_len"], seed_mode=FULL_PARALLEL, reposition=True,
                      boxcar_taps=0, soft_clip=False, output_format=OUT_DOP,
                      samerate_filter=_lib.SAMERATE_LOWPASS if wl == "samerate128lp"
                      else _lib.SAMERATE_BOXCAR, device=local)
    elif wl == "dsd256to128":
        f = ntf.get_filter(cfg["ntf"], fs)
        g = float(np.float32(PATH_GAIN))
        enc = Encoder(cfg["fs_in"], fs, nch, f, cfg["depth"], cfg["cands"], cfg["lat"],
                      seg_len=cfg["das_seg_len"], seed_mode=FULL_PARALLEL, reposition=True,
                      boxcar_taps=cfg["boxcar_taps"], soft_clip=cfg["soft_clip"],
                      output_format=OUT_DOP, device=local)
    elif wl == "precorr128":
        f = ntf.auto_select_precorr(fs)
        g = PCM_FIR_GAIN
        enc = Encoder(cfg["fs_in"], fs, nch, f, 64, 32, 128, state_limit=cfg["state_limit"],
                      boxcar_taps=8, soft_clip=False, output_format=OUT_DOP,
                      sdm_mode=_lib.SDM_PRECORR, device=local)
    else:
        f = ntf.get_filter("clans-7", fs)
        g = 1.0
        enc = Encoder(fs, cfg["fs_out"], nch, f, 64, 32, 128, output_format=_lib.OUT_PCM,
                      device=local)
    frames = inp.shape[1]
    d_in = torch.from_numpy(inp).cuda()
    if wl == "dsd2pcm128":
        d_out = torch.empty((nch, frames * 16 // 128 + 64), dtype=torch.float32, device="cuda")
        n_in_step = frames * 16 * nch
    else:
        d_out = torch.empty(enc.out_capacity(frames) + 64, dtype=torch.uint8, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    lib_stream = torch.cuda.ExternalStream(enc.stream_ptr)
    for _ in range(args.warmup):
        enc.process(d_in, d_out, g, g)
    torch.cuda.synchronize()
    fp64_peak = enc.probe_fp64_gops()
    clocks = ClockSampler(local)
    l0 = enc.launches()
    w0, _ = enc.sdm_work()
    step_ms, sdm_ms = [], []
    clocks.start()
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(lib_stream)
        ns, nb = enc.process(d_in, d_out, g, g)
        e1.record(lib_stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        sdm_ms.append(enc.stage_ms()["sdm"])
    torch.cuda.synchronize()
    clk = clocks.stop()
    launches = (enc.launches() - l0) // max(1, args.steps)
    sdm_samples = (enc.sdm_work()[0] - w0) / args.steps
    total_s = max_over_ranks(sum(step_ms) / 1000.0)
    units_step = n_in_step if wl == "dsd2pcm128" else ns * nch
    value = job_throughput(units_step, args.steps, world, total_s)
    # end to end: host buffers through the C-ABI call, copies inside the clock
    h_in = torch.from_numpy(inp).pin_memory().numpy()
    cap = (nch * (frames * 16 // 128 + 64) * 4) if wl == "dsd2pcm128" else enc.out_capacity(frames) + 64
    h_out = torch.empty(cap, dtype=torch.uint8).pin_memory().numpy()
    enc.process_host(h_in, h_out, g, g)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ns2, nb2 = enc.process_host(h_in, h_out, g, g)
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_units = (frames * 16 * nch) if wl == "dsd2pcm128" else ns2 * nch
    e2e = {"value": job_throughput(e2e_units, args.steps, world, e2e_s), "unit": UNIT,
           "h2d_bytes_per_step": int(inp.nbytes), "d2h_bytes_per_step": int(nb2)}
    st = enc.stage_ms()
    if wl in ("samerate128", "samerate128lp", "dsd256to128"):
        sdm_s = statistics.mean(sdm_ms) / 1000.0
        flops = sdm_samples * cfg["cands"] * (5 * f.order + 6)
        roof = {"bound": "fp64", "achieved": flops / sdm_s / 1e12, "peak": fp64_peak / 1000.0,
                "unit": "TFLOP/s", "frac": flops / sdm_s / 1e12 / (fp64_peak / 1000.0),
                "traffic": None,
                "kernel": enc.last_sdm_kernel() + " (latency-bound small trellis)",
                "algorithmic_flops_per_launch": flops, "flops_per_sample": cfg["cands"] * (5 * f.order + 6)}
    elif wl == "precorr128":
        pc_s = statistics.mean(sdm_ms) / 1000.0
        n_pc = ns * nch
        roof = {"bound": "latency", "achieved": 9.0 * n_pc / pc_s / 1e9, "peak": 6773.2,
                "unit": "GB/s", "frac": 9.0 * n_pc / pc_s / 1e9 / 6773.2, "traffic": 9.0 * n_pc,
                "kernel": "precorr_process_kernel<7,true>",
                "per_channel_msamples_per_s": ns / pc_s / 1e6,
                "note": "a serial recurrence per channel (one thread each): bound by the latency "
                        "of the output chain, so HBM (8 B in + 1 B out per sample, of measured "
                        "MEASURED_PEAKS hbm_gbs) is reported only for scale"}
    else:
        step_s = total_s / args.steps
        # FP64 instructions: stage 1 = 4 table sums + the centre tap per output,
        # stages 2-7 = 33 FMAs per output (the half-band's nonzero taps)
        outs = [frames * 16 // 2 ** (k + 1) for k in range(cfg["stages"])]
        instr = (5 * outs[0] + 33 * sum(outs[1:])) * nch
        roof = {"bound": "fp64", "achieved": instr / step_s / 1e12, "peak": fp64_peak / 1000.0,
                "unit": "T FP64 instructions/s", "frac": instr / step_s / 1e12 / (fp64_peak / 1000.0),
                "traffic": None, "kernel": "decim_bits_kernel + decim_stage_kernel (7 stages, whole step timed)",
                "algorithmic_instructions_per_launch": instr,
                "per_output": "stage 1: 4 table reads + 5 DADD; stages 2-7: 33 DFMA (an FMA "
                              "issues as one FP64 instruction; the probe's peak counts DADD/DMUL)"}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = _next_cpu(wl, inp, None, 0.5 if wl.startswith("samerate") else 1.0)
    if rank == 0:
        line = {"metric": cfg["metric"], "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000 * total_s / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32" if wl == "precorr128" else "f64", "data": "synthetic",
                "config": dict({k: v for k, v in cfg.items() if k != "metric"}, channels=nch,
                               seconds=args.seconds,
                               l2="512 MiB written between timed steps (outside the events)"),
                "xrt": (units_step / nch / fs) * args.steps / total_s,
                "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
                "gpu_launches": int(launches), "stages_ms": st, "fp64_peak_gops": fp64_peak}
        print(json.dumps(line), flush=True)
    enc.close()


def run_next_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import numpy as np
    cfg = NEXT[args.workload]
    inp, _ = _next_input(args.workload, args.seconds, 2, 1101)
    sample_s = 0.5 if args.workload.startswith("samerate") else 1.0
    for _ in range(args.warmup):
        _next_cpu(args.workload, inp, None, 0.05)
    vals, secs = [], []
    info = None
    for _ in range(args.steps):
        info = _next_cpu(args.workload, inp, None, sample_s)
        vals.append(info["value"])
        secs.append(info["seconds"])
    v = float(np.mean(vals))
    print(json.dumps({"impl": "reference", "metric": cfg["metric"], "value": v, "unit": UNIT,
                      "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1000 * float(np.mean(secs)), "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "data": "synthetic",
                      "config": dict({k: v for k, v in cfg.items() if k != "metric"},
                                     cpu_sample_seconds=sample_s),
                      "cpu_baseline": {"value": v, "unit": UNIT, "cores": info["cores"],
                                       "kind": "port", "sample": info["sample"]},
                      "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}), flush=True)


def main():
    args = parse()
    if args.impl == "reference" and args.workload in NEXT:
        run_next_reference(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload in NEXT:
        run_next(args)
    elif args.workload == "multistream64":
        run_multistream(args)
    elif args.workload == "multistream64_precorr":
        run_multistream_precorr(args)
    elif args.workload == "multistream64_dsd":
        run_multistream_dsd(args)
    elif args.workload == "diff16":
        run_diff(args)
    elif args.workload == "dsd512conv6":
        run_conv(args)
    elif args.workload == "dsd128_seg0first":
        run_seg0first(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
