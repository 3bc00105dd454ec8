"""Regenerate foo_dsd_trellis_gb300/ntf_table.json from the reference's own
NTF table (src/ntf.c).

Test and build infrastructure, not product code: the package only reads the
JSON this writes.  The coefficients must be bit-identical to the reference's,
so they are not retyped: this script compiles the reference's src/ntf.c (via
oracle/Makefile, target `ref`, which reads the reference sources where they
lie) and dumps every entry with exact hex-float encodings.  Run it only where
the reference tree is present; the JSON it writes is committed.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
TABLE = os.path.join(ROOT, "foo_dsd_trellis_gb300", "ntf_table.json")
sys.path.insert(0, ROOT)


def main() -> None:
    from oracle import oracle as O
    O.build(ref=True)
    ref = O.ref_lib()
    if ref is None:
        raise SystemExit("reference sources not present; ntf_table.json left unchanged")
    L = ref.lib
    entries = []
    a = np.zeros(10)
    g = np.zeros(10)
    order = C.c_int()
    freq = C.c_uint()
    name = C.create_string_buffer(64)
    for i in range(L.ref_ntf_count()):
        L.ref_ntf_entry(i, a.ctypes.data_as(O._dp), g.ctypes.data_as(O._dp),
                        C.byref(order), C.byref(freq), name, 64)
        entries.append({
            "index": i,
            "name": name.value.decode(),
            "order": order.value,
            "freq": freq.value,
            "a": [float(v).hex() for v in a[: order.value]],
            "g": [float(v).hex() for v in g[: order.value]],
        })
    doc = {
        "source": "reference src/ntf.c, table order preserved (lookup = first entry "
                  "whose name matches and whose freq <= the DSD rate, src/ntf.c:814-832)",
        "filters": entries,
    }
    with open(TABLE, "w") as f:
        json.dump(doc, f, indent=1)
    print(f"wrote {len(entries)} filters")


if __name__ == "__main__":
    main()
