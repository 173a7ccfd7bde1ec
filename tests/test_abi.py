"""The C-ABI library builds for sm_103a and exports every declared entry point.

No CUDA call is made: loading libmw3gpu.so needs no GPU."""
import ctypes
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    text = open(os.path.join(ROOT, "include", "mw3gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(mw3_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_function():
    from madwave3_gb300 import build
    lib = build.build()
    syms = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (mw3_\w+)", syms))
    names = declared()
    assert len(names) >= 20
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    L = ctypes.CDLL(lib)
    for n in names:
        assert getattr(L, n) is not None


def test_binding_lists_every_declared_function():
    from madwave3_gb300 import propagator
    assert sorted(propagator.HEADER_FUNCS) == declared()


def test_sm103a_only():
    from madwave3_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
