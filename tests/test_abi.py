"""The C-ABI library builds, loads and exports every declared entry point
(no compute call: this runs without a GPU)."""

import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "picca_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("pg_cf_neighbours", "pg_xcf_neighbours", "pg_cf_xi", "pg_xcf_xi",
                     "pg_plan_create", "pg_plan_destroy", "pg_plan_stats", "pg_strerror"):
        assert required in names


def test_library_exports_every_declared_symbol():
    from picca_gb300 import build_ext
    try:
        path = build_ext.build()
    except (RuntimeError, FileNotFoundError) as exc:  # no nvcc on this machine
        pytest.skip(f"cannot build: {exc}")
    import torch  # noqa: F401  (loads libcudart for the dependent library)
    lib = ctypes.CDLL(path)
    for name in declared_functions():
        assert hasattr(lib, name), name
    lib.pg_strerror.restype = ctypes.c_char_p
    assert lib.pg_strerror(-4) == b"bin index outside the histogram"
    assert lib.pg_version() == 10000


def test_no_cpu_fallback_without_gpu(monkeypatch):
    """The product path refuses to run without CUDA instead of falling back."""
    import torch
    from picca_gb300 import _native, pairs
    monkeypatch.setattr(torch.cuda, "is_available", lambda: False)
    with pytest.raises(_native.NativeError):
        pairs.require_cuda()


def _header_arity():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for name, args in re.findall(r"\b(pg_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", text):
        args = args.strip()
        out[name] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_ctypes_signatures_match_header():
    """Every argtypes list of the Python binding has the header's arity."""
    from picca_gb300 import _native, build_ext
    try:
        build_ext.build()
    except (RuntimeError, FileNotFoundError) as exc:
        pytest.skip(f"cannot build: {exc}")
    import torch  # noqa: F401
    lib = _native.lib()
    for name, arity in _header_arity().items():
        func = getattr(lib, name)
        if func.argtypes is not None:
            assert len(func.argtypes) == arity, (name, len(func.argtypes), arity)


def test_struct_layouts_match_header():
    """ctypes struct field counts equal the header's struct member counts."""
    from picca_gb300 import _native
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    for cname, pyname in (("pg_corr_params", "CorrParams"), ("pg_forest_set", "ForestSetC"),
                          ("pg_xi_rows", "XiRowsC"), ("pg_run_stats", "RunStats")):
        body = re.search(r"typedef struct " + cname + r" \{(.*?)\}", text, flags=re.S).group(1)
        members = 0
        for decl in body.split(";"):
            decl = decl.strip()
            if decl:
                members += decl.count(",") + 1
        assert len(getattr(_native, pyname)._fields_) == members, cname
