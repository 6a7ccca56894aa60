"""The C-ABI library loads and exports every entry point of include/stz_mg.h
(no compute: these run without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "stz_mg.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(stz_mg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from stzpp_gb300 import build, mg
    build.build()
    return mg.load_library()


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("stz_mg_create", "stz_mg_setup", "stz_mg_solve", "stz_mg_vcycle", "stz_mg_destroy",
                     "stz_mg_set_stencil_const", "stz_mg_set_stencil_points", "stz_mg_set_coeffs_lame"):
        assert required in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from stzpp_gb300 import mg
    assert sorted(mg.EXPORTS) == declared_functions()


def test_desc_defaults(lib):
    from stzpp_gb300.mg import Desc
    d = Desc()
    lib.stz_mg_desc_default(ctypes.byref(d))
    assert (d.precision, d.v_down, d.v_up, d.max_coarse, d.bottom, d.bottom_sweeps, d.sweep_growth) == \
        (0, 2, 2, 1024, 0, 24, 1)


def test_create_rejects_bad_arguments(lib):
    from stzpp_gb300.mg import Desc
    d = Desc()
    lib.stz_mg_desc_default(ctypes.byref(d))
    d.m, d.n, d.o = 0, 4, 5
    h = ctypes.c_void_p()
    assert lib.stz_mg_create(ctypes.byref(d), ctypes.byref(h)) == 1   # STZ_MG_ERR_ARG
    assert b"positive" in lib.stz_mg_last_error()
    assert lib.stz_mg_create(None, ctypes.byref(h)) == 1


def test_create_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from stzpp_gb300.mg import Desc
    d = Desc()
    lib.stz_mg_desc_default(ctypes.byref(d))
    d.m, d.n, d.o = 8, 8, 9
    h = ctypes.c_void_p()
    assert lib.stz_mg_create(ctypes.byref(d), ctypes.byref(h)) == 2   # STZ_MG_ERR_CUDA
    assert not h.value


def prototypes():
    """{name: [parameter kind, ...]} of the header's function declarations,
    kinds 'ptr', 'int', 'double', 'longlong'."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for m in re.finditer(r"\b(stz_mg_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", text, flags=re.S):
        name, params = m.group(1), " ".join(m.group(2).split())
        kinds = []
        if params not in ("", "void"):
            for p in params.split(","):
                p = p.strip()
                if "*" in p or p.split()[0] in ("stz_mg_handle",):
                    kinds.append("ptr")
                elif re.search(r"\blong long\b", p):
                    kinds.append("longlong")
                elif re.search(r"\bdouble\b", p):
                    kinds.append("double")
                elif re.search(r"\bint\b", p):
                    kinds.append("int")
                else:
                    kinds.append("other:" + p)
        out[name] = kinds
    return out


def _kind(t):
    if t in (ctypes.c_void_p, ctypes.c_char_p) or (isinstance(t, type) and issubclass(t, ctypes._Pointer)):
        return "ptr"
    return {ctypes.c_int: "int", ctypes.c_double: "double", ctypes.c_longlong: "longlong"}.get(t, "other")


def test_python_argtypes_match_the_header(lib):
    """Every ctypes signature the Python binding declares has the header's
    parameter count and kinds (a drifted signature would pass wrong values)."""
    protos = prototypes()
    checked = 0
    for name, kinds in protos.items():
        argtypes = getattr(lib, name).argtypes
        if argtypes is None:
            continue
        assert [_kind(t) for t in argtypes] == kinds, name
        checked += 1
    assert checked >= len(protos) - 2   # all but stz_mg_desc_default and stz_mg_last_error
