"""The C-ABI library builds for sm_103a and exports every entry point that
include/edxr.h declares (no GPU needed: nothing is called)."""
import ctypes
import os
import re

from edxraster_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^\s*(?:edxr_status|const char\*)\s+(edxr_\w+)\s*\(", text, re.M))
    return names


def test_library_exports_every_declared_symbol(cuda_lib):
    names = declared_symbols()
    assert "edxr_render" in names and "edxr_backward" in names
    missing = [n for n in sorted(names) if not hasattr(cuda_lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert declared_symbols() <= set(_lib.SIGNATURES)


def test_library_is_sm103a(cuda_lib):
    # the build recipe passes exactly one -gencode, for sm_103a
    from edxraster_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert os.path.getsize(build.LIB) > 0
