"""The oracle against the committed golden digests of the reference's own
trellis.c output (tests/golden/sdm_golden.json, made by make_golden.py).  The
same fixtures are checked on the GPU path in test_sdm_golden_gpu."""
import hashlib
import json
import os

import numpy as np
import pytest

from signals import multitone, sdm_input

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "sdm_golden.json")))


def _input(c):
    return sdm_input(c["n"], c["seed"], amp=0.45) if c["signal"] == "sine" else multitone(c["n"], c["seed"])


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=[c["name"] for c in GOLDEN["cases"]])
def test_oracle_matches_golden(oracle, case):
    from foo_dsd_trellis_gb300 import ntf
    f = ntf.get_filter(case["ntf"], case["rate"])
    ctx = oracle.sdm(f.order, np.array(f.a), np.array(f.g), case["depth"], case["cands"],
                     case["lat"], case["state_limit"])
    bits = oracle.sdm_bits(ctx, _input(case))
    assert len(bits) == case["count"]
    assert "".join(str(b) for b in bits[:64]) == case["head"]
    assert hashlib.sha256(bits.tobytes()).hexdigest() == case["sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("case", GOLDEN["cases"], ids=[c["name"] for c in GOLDEN["cases"]])
def test_sdm_golden_gpu(case):
    torch = pytest.importorskip("torch")
    from foo_dsd_trellis_gb300 import ntf
    from foo_dsd_trellis_gb300.sdm import TrellisSdm
    f = ntf.get_filter(case["ntf"], case["rate"])
    g = TrellisSdm(f.order, f.a, f.g, case["depth"], case["cands"], case["lat"],
                   case["state_limit"])
    bits = g.process_block(torch.from_numpy(_input(case)).cuda())[0].cpu().numpy()
    assert len(bits) == case["count"]
    assert hashlib.sha256(bits.tobytes()).hexdigest() == case["sha256"]


@pytest.mark.parametrize("case", [c for c in GOLDEN["cases"] if "trace" in c],
                         ids=[c["name"] for c in GOLDEN["cases"] if "trace" in c])
def test_oracle_context_trace(oracle, case):
    """The oracle's context after each of the first 512 samples equals the
    reference's (act order, binary64 cost, path, next bit of every candidate)."""
    import struct
    from foo_dsd_trellis_gb300 import ntf
    f = ntf.get_filter(case["ntf"], case["rate"])
    ctx = oracle.sdm(f.order, np.array(f.a), np.array(f.g), case["depth"], case["cands"],
                     case["lat"], case["state_limit"])
    x = _input(case)
    tr = case["trace"]
    for t in range(tr["samples"]):
        ctx.process(x[t:t + 1])
        row = ctx.trace_row()
        if t < len(tr["full"]):
            cands = [struct.unpack_from("<dQB", row, 17 * i) for i in range(len(row) // 17)]
            assert [[float(c).hex(), "%016x" % p, nx] for c, p, nx in cands] == tr["full"][t], t
        assert hashlib.sha256(row).hexdigest()[:16] == tr["digests"][t], t
