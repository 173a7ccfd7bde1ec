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


def _c_struct_fields(text, name):
    end = re.search(r"\}\s*" + name + ";", text).start()
    body = text[text.rindex("{", 0, text.rindex("typedef struct", 0, end) + 40) + 1:end]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        decl = re.sub(r"^(const\s+)?(int32_t|double)\s*", "", decl)
        out += [re.sub(r"[*\s]|const", "", v) for v in decl.split(",")]
    return out


def _f_type_fields(text, name):
    body = re.search(r"type, bind\(c\) :: " + name + r"\n(.*?)end type", text, re.S).group(1)
    out = []
    for line in body.splitlines():
        if "::" in line:
            out += [v.strip() for v in line.split("::")[1].split(",")]
    return out


def test_fortran_module_matches_the_header():
    """include/mw3gpu.f90 (no Fortran compiler here): its bind(c) types list the
    C structs' fields in the same order, and every interface is a declared
    entry point."""
    h = open(os.path.join(ROOT, "include", "mw3gpu.h")).read()
    f = open(os.path.join(ROOT, "include", "mw3gpu.f90")).read()
    for c_name, f_name in (("mw3_grid", "mw3_grid"), ("mw3_wave", "mw3_wave"), ("mw3_prodproj", "mw3_prodproj")):
        assert [x.lower() for x in _c_struct_fields(h, c_name)] == [x.lower() for x in _f_type_fields(f, f_name)], c_name
    f_funcs = set(re.findall(r"function (mw3_\w+)\(", f))
    assert f_funcs and f_funcs <= set(declared())
