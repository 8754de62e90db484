"""ctypes binding of ``libpicca_gb300.so`` (C ABI in ``include/picca_gb300.h``).

There is no CPU fallback: if the shared library or a CUDA device is missing,
every entry point raises :class:`NativeError`.
"""

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpicca_gb300.so")

PG_OK = 0
PG_MODE_FP64 = 0
PG_MODE_FP32_GUARD = 1
PG_DMAT_FP64 = 0
PG_DMAT_SPLIT_BF16 = 1
PG_XDMAT_MAX_OBJECTS = 256
PG_ERR_UNSUPPORTED = -6

_P = ctypes.POINTER
_c_double_p = ctypes.c_void_p  # device pointers are passed as integers


class NativeError(RuntimeError):
    """A libpicca_gb300 call failed (status code and message)."""


class CorrParams(ctypes.Structure):
    _fields_ = [
        ("r_par_min", ctypes.c_double), ("r_par_max", ctypes.c_double),
        ("r_trans_max", ctypes.c_double),
        ("num_bins_r_par", ctypes.c_int32), ("num_bins_r_trans", ctypes.c_int32),
        ("z_min_pairs", ctypes.c_double), ("z_max_pairs", ctypes.c_double),
        ("zerr_cut_deg", ctypes.c_double), ("zerr_cut_kms", ctypes.c_double),
        ("ang_max", ctypes.c_double),
        ("x_correlation", ctypes.c_int32), ("rmu_binning", ctypes.c_int32),
        ("ang_correlation", ctypes.c_int32),
        ("remove_same_half_plate_close_pairs", ctypes.c_int32),
    ]


FOREST_SET_PTR_FIELDS = (
    "pix_offset", "z", "r_comov", "dist_m", "weights", "delta", "ra", "dec", "x_cart", "y_cart",
    "z_cart", "cos_dec", "z_qso", "r_first", "r_last", "obj_r_comov", "obj_dist_m", "obj_weight",
    "thingid", "plate", "fiberid", "row")


class ForestSetC(ctypes.Structure):
    _fields_ = ([("num", ctypes.c_int64), ("num_pixels", ctypes.c_int64)]
                + [(name, ctypes.c_void_p) for name in FOREST_SET_PTR_FIELDS]
                + [("num_rows", ctypes.c_int32), ("max_pixels", ctypes.c_int32)])


class NbrGroupsC(ctypes.Structure):
    _fields_ = ([("num_groups1", ctypes.c_int32), ("num_groups2", ctypes.c_int32),
                 ("num_blocks", ctypes.c_int32), ("reserved", ctypes.c_int32)]
                + [(name, ctypes.c_void_p) for name in
                   ("start2", "cand_offsets", "cand_groups", "block_group", "block_first",
                    "block_end")])


class XiRowsC(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name in
                ("weights", "xi", "r_par", "r_trans", "z", "num_pairs")]


class DmatParamsC(ctypes.Structure):
    _fields_ = [("num_model_bins_r_par", ctypes.c_int32), ("num_model_bins_r_trans", ctypes.c_int32),
                ("redshift_evolution", ctypes.c_int32), ("row_capacity", ctypes.c_int32),
                ("product", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("z_ref", ctypes.c_double), ("alpha", ctypes.c_double), ("alpha2", ctypes.c_double)]


class DmatSumsC(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name in
                ("weights_dmat", "dmat", "r_par_eff", "r_trans_eff", "z_eff", "weight_eff")]


class RunStats(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("error_detail", ctypes.c_int32),
                ("rechecked_pairs", ctypes.c_int64), ("recheck_overflows", ctypes.c_int64),
                ("work_items", ctypes.c_int64), ("gemm_macs", ctypes.c_int64),
                ("visited_pairs", ctypes.c_int64)]


_LIB = None


def lib():
    """Load the library once; raise NativeError when it cannot be used."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise NativeError(
            f"{LIB_PATH} is missing: build it with `python -m picca_gb300.build_ext` "
            "(this package has no CPU fallback)")
    handle = ctypes.CDLL(LIB_PATH)
    handle.pg_strerror.restype = ctypes.c_char_p
    handle.pg_strerror.argtypes = [ctypes.c_int]
    handle.pg_version.restype = ctypes.c_int
    handle.pg_plan_create.argtypes = [_P(ctypes.c_void_p)]
    handle.pg_plan_destroy.argtypes = [ctypes.c_void_p]
    handle.pg_plan_stats.argtypes = [ctypes.c_void_p, _P(RunStats)]
    handle.pg_cf_neighbours.argtypes = [
        ctypes.c_void_p, _P(CorrParams), _P(ForestSetC), _P(ForestSetC), ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    handle.pg_xcf_neighbours.argtypes = handle.pg_cf_neighbours.argtypes
    handle.pg_cf_neighbours_grouped.argtypes = [
        ctypes.c_void_p, _P(CorrParams), _P(ForestSetC), _P(ForestSetC), _P(NbrGroupsC),
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    handle.pg_xcf_neighbours_grouped.argtypes = handle.pg_cf_neighbours_grouped.argtypes
    handle.pg_cf_xi.argtypes = [
        ctypes.c_void_p, _P(CorrParams), _P(ForestSetC), _P(ForestSetC), ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
        _P(XiRowsC), ctypes.c_void_p]
    handle.pg_xcf_xi.argtypes = handle.pg_cf_xi.argtypes
    handle.pg_cf_dmat_work_bytes.argtypes = [
        ctypes.c_void_p, _P(CorrParams), _P(DmatParamsC), ctypes.c_int32, ctypes.c_int32,
        ctypes.c_int64, _P(ctypes.c_uint64)]
    handle.pg_cf_dmat.argtypes = [
        ctypes.c_void_p, _P(CorrParams), _P(DmatParamsC), _P(ForestSetC), _P(ForestSetC)]
    handle.pg_cf_dmat.argtypes += [ctypes.c_void_p] * 7 + [ctypes.c_int64, ctypes.c_void_p,
                                                           ctypes.c_uint64, _P(DmatSumsC),
                                                           ctypes.c_void_p]
    handle.pg_xcf_dmat_work_bytes.argtypes = [
        ctypes.c_void_p, _P(CorrParams), _P(DmatParamsC), ctypes.c_int32, ctypes.c_int64,
        _P(ctypes.c_uint64)]
    handle.pg_xcf_dmat.argtypes = [
        ctypes.c_void_p, _P(CorrParams), _P(DmatParamsC), _P(ForestSetC), _P(ForestSetC)]
    handle.pg_xcf_dmat.argtypes += [ctypes.c_void_p] * 7 + [ctypes.c_int64, ctypes.c_void_p,
                                                            ctypes.c_uint64, _P(DmatSumsC),
                                                            ctypes.c_void_p]
    for name in ("pg_plan_create", "pg_plan_destroy", "pg_plan_stats", "pg_cf_neighbours",
                 "pg_xcf_neighbours", "pg_cf_neighbours_grouped", "pg_xcf_neighbours_grouped", "pg_cf_xi", "pg_xcf_xi", "pg_cf_dmat_work_bytes",
                 "pg_cf_dmat", "pg_xcf_dmat_work_bytes", "pg_xcf_dmat"):
        getattr(handle, name).restype = ctypes.c_int
    _LIB = handle
    return handle


def check(status, what):
    """Raise NativeError (with the status in ``.status``) for a nonzero status."""
    if status != PG_OK:
        msg = lib().pg_strerror(status).decode()
        err = NativeError(f"{what} failed: {msg} (status {status})")
        err.status = status
        raise err


class Plan:
    """Owns a pg_plan (device scratch) on the current CUDA device."""

    def __init__(self):
        self._handle = ctypes.c_void_p()
        check(lib().pg_plan_create(ctypes.byref(self._handle)), "pg_plan_create")

    @property
    def handle(self):
        return self._handle

    def stats(self):
        out = RunStats()
        check(lib().pg_plan_stats(self._handle, ctypes.byref(out)), "pg_plan_stats")
        return out

    def close(self):
        if self._handle:
            lib().pg_plan_destroy(self._handle)
            self._handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # pylint: disable=broad-except
            pass
