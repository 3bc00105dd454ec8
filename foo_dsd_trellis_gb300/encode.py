"""Offline PCM -> DSD encoder: the counterpart of the reference's dsd_encode
tool (tools/dsd_encode.c:314-574), on the GPU.

    python -m foo_dsd_trellis_gb300.encode --input music.wav --dsd-rate 5644800 \\
        --sdm precorr --ntf auto --sdm-out out.dsf

Flags, defaults, NTF names, output formats (by extension: .dsf, .dff, .wav,
anything else raw float32) and exit codes follow the tool.  The flow is the
tool's: read the input (a WAV mixed to mono), FIR upsample to the DSD rate,
apply --gain, optionally write the FIR output (--fir-out, raw or WAV; a DSF or
DFF name is written raw with a warning), then the SDM over the whole signal
(trellis: sdm_process_block + sdm_drain, so the output has one decision per
FIR sample; PreCorr: precorr_process_block) and the output file.

Differences, all opt-in except the first:
  * the FIR output reaches the SDM as float64 (the tool hands its float32 FIR
    buffer to sdm_process_block's `const double *`, :464 and :517 — a bug);
  * --keep-channels encodes every channel of a WAV instead of a mono mix;
  * --das SEG_LEN runs the trellis segment-parallel with Density-Aligned
    Stitching (the plugin's DAS, full-parallel seeding), which is what makes
    long files fast on the GPU; the sequential trellis is one warp per
    channel.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np
import torch

from . import _lib, dsdfile, ntf

# the tool's NTF names (tools/dsd_encode.c:39-55); unknown names mean auto
NTF_NAMES = ["auto", "clans-4", "clans-5", "clans-6", "clans-7", "clans-8",
             "sdm-4", "sdm-5", "sdm-6", "sdm-7", "sdm-8"]


def _detect(path: str) -> str:
    ext = os.path.splitext(path)[1].lower()
    return {".dff": "dff", ".dsf": "dsf", ".wav": "wav"}.get(ext, "raw")


def _write_float(path: str, x: np.ndarray, rate: int, fmt: str) -> None:
    if fmt == "wav":
        dsdfile.wav_write(path, x, rate)
    else:
        # raw float32, channels one after another (one channel: the tool's file)
        np.ascontiguousarray(x, "<f4").tofile(path)


def select_filter(name: str, sdm: str, dsd_rate: int) -> ntf.NtfFilter:
    """parse_ntf_name + the tool's auto rule (tools/dsd_encode.c:479-489)."""
    name = name.lower()
    if name not in NTF_NAMES or name == "auto":
        return ntf.auto_select_precorr(dsd_rate) if sdm == "precorr" else ntf.auto_select(dsd_rate)
    return ntf.get_filter(name, dsd_rate)


def encode(args) -> int:
    quiet = args.quiet
    try:
        pcm, rate = dsdfile.read_input(args.input, args.keep_channels)
    except OSError:
        print(f"Cannot open: {args.input}", file=sys.stderr)
        return 1
    pcm_rate = args.pcm_rate if args.pcm_rate else rate
    if pcm_rate == 0:
        print("PCM rate unknown. Use --pcm-rate for raw input.", file=sys.stderr)
        return 1
    if args.samples > 0 and pcm.shape[1] > args.samples:
        pcm = pcm[:, : args.samples]
    nch, n_in = pcm.shape
    if not quiet:
        print(f"Input: {n_in} samples @ {pcm_rate} Hz ({n_in / pcm_rate:.3f} s)", file=sys.stderr)
    ratio = args.dsd_rate // pcm_rate
    if ratio < 1 or args.dsd_rate != ratio * pcm_rate:
        print(f"Invalid rate ratio: {args.dsd_rate} / {pcm_rate}", file=sys.stderr)
        return 1
    dev = torch.device(f"cuda:{args.device}")
    from .fir import FirChain
    try:
        fir = FirChain(pcm_rate, args.dsd_rate, boxcar_taps=0, soft_clip=False, num_channels=nch,
                       device=args.device)
    except _lib.DsdGpuError:
        print(f"FIR chain init failed ({pcm_rate} -> {args.dsd_rate})", file=sys.stderr)
        return 1
    y = fir.process(torch.from_numpy(pcm).to(dev), args.gain, args.gain)
    fir.close()
    n = y.shape[1]
    if not quiet:
        print(f"FIR: {n_in} -> {n} samples ({ratio}x)", file=sys.stderr)
    if args.fir_out:
        fmt = _detect(args.fir_out)
        if fmt in ("dsf", "dff"):
            print("WARNING: FIR reference is multi-bit, DFF/DSF only store 1-bit. Using raw.",
                  file=sys.stderr)
            fmt = "raw"
        _write_float(args.fir_out, y.float().cpu().numpy(), args.dsd_rate, fmt)
        if not quiet:
            print(f"FIR ref: {args.fir_out} ({n} samples)", file=sys.stderr)
    if not args.sdm_out:
        return 0
    try:
        f = select_filter(args.ntf, args.sdm, args.dsd_rate)
    except KeyError:
        print(f"NTF filter not found: {args.ntf} @ {args.dsd_rate} Hz", file=sys.stderr)
        return 1
    if args.sdm == "precorr":
        from .precorr import PreCorr
        pc = PreCorr(f.order, f.a, f.g, args.state_limit, num_channels=nch, device=args.device)
        bits = pc.process_block(y)
        pc.close()
        if not quiet:
            print(f"SDM: PreCorr, NTF={args.ntf}, order={f.order}, {n} samples", file=sys.stderr)
    elif args.das > 0:
        from .das import DasChannels
        d = DasChannels(f.order, f.a, f.g, args.depth, args.cands, args.lat,
                        state_limit=args.state_limit, num_channels=nch, device=args.device)
        bits, _ = d.process_chunk(y, seg_len=args.das)
        d.close()
        if not quiet:
            print(f"SDM: Trellis DAS, NTF={args.ntf}, depth={args.depth}, cands={args.cands}, "
                  f"lat={args.lat}, {bits.shape[1]} samples", file=sys.stderr)
    else:
        from .sdm import TrellisSdm
        s = TrellisSdm(f.order, f.a, f.g, args.depth, args.cands, args.lat, args.state_limit,
                       num_contexts=nch, device=args.device)
        head = s.process_block(y)
        tail = s.drain(n, 0, nch)
        s.close()
        bits = torch.stack([torch.cat([head[c], tail[c]])[:n] for c in range(nch)])
        if not quiet:
            print(f"SDM: Trellis, NTF={args.ntf}, depth={args.depth}, cands={args.cands}, "
                  f"lat={args.lat}, {bits.shape[1]} samples", file=sys.stderr)
    fmt = _detect(args.sdm_out)
    if fmt in ("dsf", "dff"):
        if nch > 6:
            print("DSF/DFF hold at most 6 channels", file=sys.stderr)
            return 1
        dsdfile.write_dsd_file(args.sdm_out, _lib.FILE_DSF if fmt == "dsf" else _lib.FILE_DFF,
                               bits, args.dsd_rate, args.device)
    else:
        _write_float(args.sdm_out, (bits.float() * 2.0 - 1.0).cpu().numpy(), args.dsd_rate, fmt)
    if not quiet:
        print(f"Done: {args.sdm_out}", file=sys.stderr)
    return 0


def parser() -> argparse.ArgumentParser:
    p = argparse.ArgumentParser(prog="python -m foo_dsd_trellis_gb300.encode",
                                description="DSD encoder (GPU) with the dsd_encode tool's flags")
    p.add_argument("--input", required=True, help="input PCM (WAV or raw float32 mono)")
    p.add_argument("--dsd-rate", type=int, required=True, help="target DSD rate (2822400, ...)")
    p.add_argument("--sdm", default="trellis", type=str.lower,
                   help="SDM mode: trellis or precorr (anything else: trellis)")
    p.add_argument("--ntf", default="auto", help="NTF filter: auto, clans-4..8, sdm-4..8")
    p.add_argument("--fir-out", default=None, help="FIR reference output (.raw, .wav)")
    p.add_argument("--sdm-out", default=None, help="SDM output (.raw, .dff, .dsf, .wav)")
    p.add_argument("--pcm-rate", type=int, default=0, help="PCM rate (required for raw input)")
    p.add_argument("--cands", type=int, default=8)
    p.add_argument("--lat", type=int, default=256)
    p.add_argument("--depth", type=int, default=4)
    p.add_argument("--state-limit", type=float, default=0.0)
    p.add_argument("--gain", type=float, default=1.0)
    p.add_argument("--samples", type=int, default=0, help="max input samples (0 = all)")
    p.add_argument("--quiet", action="store_true")
    p.add_argument("--keep-channels", action="store_true",
                   help="encode every WAV channel instead of a mono mix")
    p.add_argument("--das", type=int, default=0, metavar="SEG_LEN",
                   help="segment-parallel trellis with DAS, segments of SEG_LEN samples")
    p.add_argument("--device", type=int, default=0)
    return p


def main(argv=None) -> int:
    args = parser().parse_args(argv)
    if args.sdm != "precorr":
        args.sdm = "trellis"
    if not args.fir_out and not args.sdm_out:
        print("Missing required arguments.", file=sys.stderr)
        parser().print_usage(sys.stderr)
        return 1
    return encode(args)


if __name__ == "__main__":
    sys.exit(main())
