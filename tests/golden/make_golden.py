"""Generate tests/golden/sdm_golden.json from the reference's own trellis SDM.

The reference's src/trellis.c (built from source by oracle/Makefile into
oracle/_ref/; the widened build for depth > 32) runs over seeded,
platform-independent inputs (tests/signals.py).  The fixture stores, per case,
the parameters, the input recipe, the decision count, the SHA-256 of the
decision bytes and the first 64 decisions; and, for the TRACES cases, the
context after each of the first 512 samples: the act list in order with each
candidate's cost (binary64 as hex), path and next bit, kept in full for the
first 4 samples and as a 16-hex-digit SHA-256 prefix per sample after that.
Run it where the reference tree is present; the JSON is committed.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from foo_dsd_trellis_gb300 import ntf  # noqa: E402
from oracle import oracle as O  # noqa: E402
from signals import multitone, sdm_input  # noqa: E402

CASES = [
    # name, ntf, rate, depth, K, lat, limit, signal, n, seed
    ("dsd64_plain_k16_d32", "clans-5", 2822400, 32, 16, 32, 0.0, "sine", 200000, 1000),
    ("dsd128_k32_d64_lat128", "clans-7", 6144000, 64, 32, 128, 0.0, "multitone", 120000, 1001),
    ("dsd128_k32_d32_lat128", "clans-6", 5644800, 32, 32, 128, 0.0, "multitone", 120000, 1002),
    ("dsd512_k16_d48_lat32", "clans-8", 22579200, 48, 16, 32, 0.0, "sine", 120000, 1004),
    ("dsd64_k2_d16_lim10", "clans-6", 2822400, 16, 2, 32, 10.0, "sine", 200000, 1005),
    ("dsd256_k8_d4_sdm8", "sdm-8", 11289600, 4, 8, 64, 0.0, "multitone", 100000, 1006),
]


TRACES = ["dsd64_plain_k16_d32", "dsd128_k32_d64_lat128", "dsd64_k2_d16_lim10"]
TRACE_SAMPLES = 512


def trace(ctx, x, nsamp=TRACE_SAMPLES):
    """Feed x one sample at a time; per sample the packed act list."""
    rows = []
    for t in range(nsamp):
        ctx.process(x[t:t + 1])
        rows.append(ctx.trace_row())
    return rows


def trace_record(rows, ctx_order_cands=4):
    import struct
    full = []
    for r in rows[:ctx_order_cands]:
        cands = [struct.unpack_from("<dQB", r, 17 * i) for i in range(len(r) // 17)]
        full.append([[float(c).hex(), "%016x" % p, nx] for c, p, nx in cands])
    return {"samples": len(rows), "full": full,
            "digests": [hashlib.sha256(r).hexdigest()[:16] for r in rows]}


def make_input(kind, n, seed):
    return sdm_input(n, seed, amp=0.45) if kind == "sine" else multitone(n, seed)


def main():
    O.build(ref=True)
    out = []
    for name, fname, rate, depth, K, lat, lim, kind, n, seed in CASES:
        f = ntf.get_filter(fname, rate)
        lib = O.ref_lib(wide=depth > 32)
        if lib is None:
            raise SystemExit("reference build missing")
        ctx = O.Sdm(lib, f.order, np.array(f.a), np.array(f.g), depth, K, lat, lim)
        x = make_input(kind, n, seed)
        y = ctx.process(x)
        bits = (y > 0).astype(np.uint8)
        out.append({"name": name, "ntf": fname, "rate": rate, "depth": depth, "cands": K,
                    "lat": lat, "state_limit": lim, "signal": kind, "n": n, "seed": seed,
                    "count": int(len(bits)),
                    "sha256": hashlib.sha256(bits.tobytes()).hexdigest(),
                    "head": "".join(str(b) for b in bits[:64]),
                    "source": "reference src/trellis.c" + (" (64-bit path build)" if depth > 32 else "")})
        if name in TRACES:
            tctx = O.Sdm(lib, f.order, np.array(f.a), np.array(f.g), depth, K, lat, lim)
            out[-1]["trace"] = trace_record(trace(tctx, x))
        print(name, len(bits), out[-1]["sha256"][:16])
    with open(os.path.join(HERE, "sdm_golden.json"), "w") as fh:
        json.dump({"cases": out}, fh, indent=1)


if __name__ == "__main__":
    main()
