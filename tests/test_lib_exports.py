"""The C-ABI library builds for sm_103a, loads, and exports every entry
point include/pbd_c.h declares (no GPU needed: nothing is called)."""
import ctypes as C
import os
import re

from positionbaseddynamicsold_gb300 import build, pbd

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "pbd_c.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pbd_[a-z0-9_]+)\s*\(", src)))


def test_header_matches_binding_list():
    assert declared() == sorted(pbd.EXPORTS)


def test_library_exports_every_symbol():
    path = build.build()
    lib = C.CDLL(path)
    for name in declared():
        assert hasattr(lib, name), name


def test_sm103a_only():
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
