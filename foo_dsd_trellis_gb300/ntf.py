"""NTF coefficient sets and their lookup rules.

The coefficients are the reference's (src/ntf.c:16-790), carried bit-exactly
in ntf_table.json (hex floats, regenerated by oracle/gen_ntf_table.py).  The lookup
functions follow the reference's: ntf_get_filter picks the first table entry
whose name matches and whose design rate is <= the DSD rate
(src/ntf.c:814-832), so 48 kHz-family rates use the 44.1 kHz table below them;
ntf_auto_select maps DSD64 -> CLANS-5, DSD128 -> CLANS-6, DSD256 and DSD512 ->
CLANS-8 (src/ntf.c:839-860).
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass

_HERE = os.path.dirname(os.path.abspath(__file__))

# ntf_filter_id_t (include/dsd_types.h:54-67)
IDS = ["clans-4", "sdm-4", "clans-5", "sdm-5", "clans-6", "sdm-6",
       "clans-7", "sdm-7", "clans-8", "sdm-8"]

DSD_RATE_64 = 2822400
DSD_RATE_128 = 5644800
DSD_RATE_256 = 11289600
DSD_RATE_512 = 22579200
DSD48_RATE_64 = 3072000
DSD48_RATE_128 = 6144000
DSD48_RATE_256 = 12288000
DSD48_RATE_512 = 24576000


@dataclass(frozen=True)
class NtfFilter:
    index: int
    name: str
    order: int
    freq: int
    a: tuple
    g: tuple


def _load():
    with open(os.path.join(_HERE, "ntf_table.json")) as f:
        doc = json.load(f)
    return [NtfFilter(e["index"], e["name"], e["order"], e["freq"],
                      tuple(float.fromhex(v) for v in e["a"]),
                      tuple(float.fromhex(v) for v in e["g"])) for e in doc["filters"]]


TABLE = _load()


def get_filter(ident, dsd_rate: int) -> NtfFilter:
    """ntf_get_filter(id, rate); `ident` is an ntf_filter_id_t int or a name."""
    name = IDS[ident] if isinstance(ident, int) else str(ident)
    for f in TABLE:
        if f.name == name and f.freq <= dsd_rate:
            return f
    raise KeyError(f"no NTF {name} for rate {dsd_rate}")


def auto_select(dsd_rate: int) -> NtfFilter:
    """ntf_auto_select(rate) (src/ntf.c:839-860)."""
    if dsd_rate >= DSD_RATE_256:
        name = "clans-8"
    elif dsd_rate >= DSD_RATE_128:
        name = "clans-6"
    else:
        name = "clans-5"
    return get_filter(name, dsd_rate)


def auto_select_precorr(dsd_rate: int) -> NtfFilter:
    """ntf_auto_select_precorr(rate) (src/ntf.c:857-873): one order above the
    trellis choice, clans-7 from DSD128 up, clans-6 below."""
    return get_filter("clans-7" if dsd_rate >= DSD_RATE_128 else "clans-6", dsd_rate)


def auto_latency(fs_in: int, fs_out: int) -> int:
    """Auto trellis latency (src/engine.c:1010-1020): 32 at DSD512 and at DSD64,
    128 from DSD128 up to below DSD512."""
    rate = max(fs_in, fs_out)
    if rate >= DSD_RATE_512:
        return 32
    if rate >= DSD_RATE_128:
        return 128
    return 32
