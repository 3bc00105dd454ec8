"""libdsdgpu.so loads and exports every function include/dsdgpu.h declares,
and the ctypes binding covers them (no GPU calls)."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "dsdgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dsdgpu_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from foo_dsd_trellis_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build_library()
    lib = C.CDLL(_lib.LIB_PATH)
    names = _declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    unbound = [n for n in names if n not in _lib.SIGNATURES]
    assert not unbound, unbound


def test_header_is_plain_c():
    """The boundary carries no C++ or torch types."""
    src = open(os.path.join(ROOT, "include", "dsdgpu.h")).read()
    code = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    for bad in ("torch", "std::", "template", "class ", "namespace", "cudaStream_t"):
        assert bad not in code, bad


def test_structs_match_the_c_layout(tmp_path):
    """Every parameter struct of include/dsdgpu.h has the ctypes binding's size
    and field offsets, measured by a C program compiled against the header."""
    import shutil
    import subprocess
    import pytest
    from foo_dsd_trellis_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = {
        "dsdgpu_sdm_params_t": _lib.SdmParams, "dsdgpu_segment_t": _lib.Segment,
        "dsdgpu_estimate_t": _lib.EstimateItem, "dsdgpu_fir_params_t": _lib.FirParams,
        "dsdgpu_das_params_t": _lib.DasParams, "dsdgpu_pipeline_params_t": _lib.PipelineParams,
        "dsdgpu_stream_desc_t": _lib.StreamDesc, "dsdgpu_plan_info_t": _lib.PlanInfo,
        "dsdgpu_diff_params_t": _lib.DiffParams,
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "dsdgpu.h"', "int main(void) {"]
    for cname, py in pairs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        cname, what, v = ln.split()
        got[(cname, what)] = int(v)
    for cname, py in pairs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
