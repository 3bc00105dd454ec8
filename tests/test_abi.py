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
