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

The input is processed in chunks (--chunk, 60 s by default) with the FIR
history and the SDM state carried, so the device holds one chunk's FIR
output plus the decisions of the whole file.

Differences, all opt-in except the first:
  * the FIR output reaches the SDM as float64 (the tool hands its float32 FIR
    buffer to sdm_process_block's `const double *`, :464 and :517 — a bug);
  * --keep-channels encodes every channel of a WAV instead of a mono mix;
  * --das SEG_LEN runs the trellis segment-parallel with Density-Aligned
    Stitching (the plugin's DAS, full-parallel seeding, chunk by chunk as the
    plugin does), which is what makes long files fast on the GPU; the
    sequential trellis is one serial walk per channel.
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
    n = n_in * ratio
    f = None
    if args.sdm_out:
        try:
            f = select_filter(args.ntf, args.sdm, args.dsd_rate)
        except KeyError:
            print(f"NTF filter not found: {args.ntf} @ {args.dsd_rate} Hz", file=sys.stderr)
            return 1
    fir_fmt = None
    fir_acc = []
    if args.fir_out:
        fir_fmt = _detect(args.fir_out)
        if fir_fmt in ("dsf", "dff"):
            print("WARNING: FIR reference is multi-bit, DFF/DSF only store 1-bit. Using raw.",
                  file=sys.stderr)
            fir_fmt = "raw"
    # the SDM runs chunk by chunk with its state carried (PreCorr, sequential
    # trellis: the same decisions as one pass; DAS: per chunk, as the plugin)
    sdm = None
    if f is not None:
        if args.sdm == "precorr":
            from .precorr import PreCorr
            sdm = PreCorr(f.order, f.a, f.g, args.state_limit, num_channels=nch, device=args.device)
        elif args.das > 0:
            from .das import DasChannels
            sdm = DasChannels(f.order, f.a, f.g, args.depth, args.cands, args.lat,
                              state_limit=args.state_limit, num_channels=nch, device=args.device)
        else:
            from .sdm import TrellisSdm
            sdm = TrellisSdm(f.order, f.a, f.g, args.depth, args.cands, args.lat, args.state_limit,
                             num_contexts=nch, device=args.device)
    bits = torch.empty((nch, n), dtype=torch.uint8, device=dev) if sdm is not None else None
    got = 0
    step = max(1, int(args.chunk * pcm_rate))
    for lo in range(0, n_in, step):
        y = fir.process(torch.from_numpy(np.ascontiguousarray(pcm[:, lo:lo + step])).to(dev),
                        args.gain, args.gain)
        if fir_fmt:
            fir_acc.append(y.float().cpu().numpy())
        if sdm is None:
            continue
        if args.sdm == "precorr":
            b = sdm.process_block(y)
        elif args.das > 0:
            b, _ = sdm.process_chunk(y, seg_len=args.das)
        else:
            parts = sdm.process_block(y)
            b = torch.stack(parts) if parts[0].numel() else None
        if b is not None and b.shape[1]:
            bits[:, got:got + b.shape[1]] = b
            got += b.shape[1]
    fir.close()
    if not quiet:
        print(f"FIR: {n_in} -> {n} samples ({ratio}x)", file=sys.stderr)
    if fir_fmt:
        _write_float(args.fir_out, np.concatenate(fir_acc, axis=1), args.dsd_rate, fir_fmt)
        if not quiet:
            print(f"FIR ref: {args.fir_out} ({n} samples)", file=sys.stderr)
    if sdm is None:
        return 0
    if args.sdm == "precorr":
        if not quiet:
            print(f"SDM: PreCorr, NTF={args.ntf}, order={f.order}, {got} samples", file=sys.stderr)
    elif args.das > 0:
        if not quiet:
            print(f"SDM: Trellis DAS, NTF={args.ntf}, depth={args.depth}, cands={args.cands}, "
                  f"lat={args.lat}, {got} samples", file=sys.stderr)
    else:
        # drain the latency (sdm_drain, tools/dsd_encode.c:519-524)
        tail = sdm.drain(n - got, 0, nch)
        if tail[0].numel():
            bits[:, got:got + tail[0].numel()] = torch.stack(tail)
            got += tail[0].numel()
        if not quiet:
            print(f"SDM: Trellis, NTF={args.ntf}, depth={args.depth}, cands={args.cands}, "
                  f"lat={args.lat}, {got} samples", file=sys.stderr)
    sdm.close()
    bits = bits[:, :got]
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
    p.add_argument("--chunk", type=float, default=60.0, metavar="SECONDS",
                   help="input processed in chunks of this length (state carried across)")
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
