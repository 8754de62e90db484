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
    from picca_gb300 import deltaio, fast_metal, metal, wick
    lib = _native.lib()
    for binder in (deltaio._bind, fast_metal._bind, metal._bind, wick._bind):
        binder()
    for name, arity in _header_arity().items():
        func = getattr(lib, name)
        if func.argtypes is not None:
            assert len(func.argtypes) == arity, (name, len(func.argtypes), arity)


def test_struct_layouts_match_header():
    """ctypes struct field counts equal the header's struct member counts."""
    from picca_gb300 import _native
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    from picca_gb300 import deltaio, fast_metal, metal, wick
    structs = {"pg_corr_params": _native.CorrParams, "pg_forest_set": _native.ForestSetC,
               "pg_xi_rows": _native.XiRowsC, "pg_run_stats": _native.RunStats,
               "pg_dmat_params": _native.DmatParamsC, "pg_dmat_sums": _native.DmatSumsC,
               "pg_metal_pixels": metal.MetalPixelsC, "pg_wick_sums": wick.WickSumsC,
               "pg_delta_arrays": deltaio.DeltaArraysC,
               "pg_fast_metal_side": fast_metal.FastMetalSideC,
               "pg_fast_metal_params": fast_metal.FastMetalParamsC,
               "pg_fast_metal_sums": fast_metal.FastMetalSumsC}
    for cname, pystruct in structs.items():
        body = re.search(r"typedef struct " + cname + r" \{(.*?)\}", text, flags=re.S).group(1)
        members = 0
        for decl in body.split(";"):
            decl = decl.strip()
            if decl:
                members += decl.count(",") + 1
        assert len(pystruct._fields_) == members, cname


def test_host_entry_points_reject_bad_arguments():
    """Entry points check their arguments on the host and return
    PG_ERR_INVALID_ARGUMENT without touching a device."""
    import numpy as np

    from picca_gb300 import _native, deltaio, fast_metal, wick
    try:
        lib = _native.lib()
    except Exception as exc:  # pylint: disable=broad-except
        pytest.skip(f"library unavailable: {exc}")
    deltaio._bind()
    fast_metal._bind()
    wick._bind()
    bad = -1
    out = deltaio.DeltaArraysC()
    assert lib.pg_read_delta_file(None, 0, 0.0, 10.0, ctypes.byref(out)) == bad
    buf = np.zeros(2880, dtype=np.uint8)
    assert lib.pg_read_delta_file(buf.ctypes.data, -1, 0.0, 10.0, ctypes.byref(out)) == bad
    # not a FITS file: no SIMPLE / BITPIX cards
    assert lib.pg_read_delta_file(buf.ctypes.data, buf.size, 0.0, 10.0, ctypes.byref(out)) == bad
    po = np.array([0, 2], dtype=np.int64)
    x = np.zeros(2)
    order = np.array([2], dtype=np.int32)
    assert lib.pg_project_deltas(1, po.ctypes.data, x.ctypes.data, x.ctypes.data, x.ctypes.data,
                                 order.ctypes.data, 1) == bad
    assert lib.pg_fast_metal_dmat(None, None, None, None, None, None) == bad
    nbytes = ctypes.c_uint64()
    assert lib.pg_cf_wick_work_bytes(None, None, 10, 10, 1, ctypes.byref(nbytes)) == bad
    assert lib.pg_xcf_wick_factored_work_bytes(None, None, 10, 10, ctypes.byref(nbytes)) == bad
