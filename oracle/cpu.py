"""CPU oracle for the correlation path (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this module; the library never does. It drives the FP64 C
restatement in ``pairs_oracle.c`` (see that file for the reference lines each
function follows) over :class:`picca_gb300.forests.ForestSet` inputs and
reproduces the aggregation of ``py/picca/bin/picca_cf.py:465-484`` /
``py/picca/bin/picca_xcf.py:500-518``.
"""

import ctypes
import os

import numpy as np

from . import build as _build

_LIB = None
_P = ctypes.POINTER


class OracleParams(ctypes.Structure):
    _fields_ = [
        ("r_par_min", ctypes.c_double), ("r_par_max", ctypes.c_double),
        ("r_trans_max", ctypes.c_double),
        ("num_bins_r_par", ctypes.c_int32), ("num_bins_r_trans", ctypes.c_int32),
        ("z_min_pairs", ctypes.c_double), ("z_max_pairs", ctypes.c_double),
        ("zerr_cut_deg", ctypes.c_double), ("zerr_cut_kms", ctypes.c_double),
        ("x_correlation", ctypes.c_int32), ("rmu_binning", ctypes.c_int32),
        ("ang_correlation", ctypes.c_int32),
        ("remove_same_half_plate_close_pairs", ctypes.c_int32),
    ]


class OracleSet(ctypes.Structure):
    _fields_ = [("num", ctypes.c_int64), ("pix_offset", _P(ctypes.c_int64))] + [
        (name, _P(ctypes.c_double)) for name in (
            "z", "r_comov", "dist_m", "weights", "delta", "ra", "dec", "x_cart",
            "y_cart", "z_cart", "cos_dec", "z_qso", "obj_r_comov", "obj_dist_m",
            "obj_weight")
    ] + [(name, _P(ctypes.c_int64)) for name in ("thingid", "plate", "fiberid")]


def lib():
    """Load (building if needed) the oracle shared library."""
    global _LIB
    if _LIB is None:
        path = _build.LIB
        if not os.path.exists(path):
            _build.build()
        _LIB = ctypes.CDLL(path)
        _LIB.oracle_angle.restype = ctypes.c_double
        _LIB.oracle_angle.argtypes = [ctypes.c_double] * 11
        _LIB.oracle_cf_neighbours.restype = ctypes.c_int64
        _LIB.oracle_xcf_neighbours.restype = ctypes.c_int64
    return _LIB


def _d(arr):
    return np.ascontiguousarray(arr, dtype=np.float64)


def _ptr(arr, ctype):
    return arr.ctypes.data_as(_P(ctype))


def make_params(r_par_min, r_par_max, r_trans_max, num_bins_r_par, num_bins_r_trans,
                z_min_pairs=None, z_max_pairs=None, zerr_cut_deg=None, zerr_cut_kms=None,
                x_correlation=False, rmu_binning=False, ang_correlation=False,
                remove_same_half_plate_close_pairs=False):
    nan = float("nan")
    return OracleParams(
        float(r_par_min), float(r_par_max), float(r_trans_max), int(num_bins_r_par),
        int(num_bins_r_trans),
        nan if z_min_pairs is None else float(z_min_pairs),
        nan if z_max_pairs is None else float(z_max_pairs),
        nan if zerr_cut_deg is None else float(zerr_cut_deg),
        nan if zerr_cut_kms is None else float(zerr_cut_kms),
        int(bool(x_correlation)), int(bool(rmu_binning)), int(bool(ang_correlation)),
        int(bool(remove_same_half_plate_close_pairs)))


def _as_set(fs, keep):
    """ctypes view of a ForestSet; ``keep`` holds the converted arrays alive."""
    conv = {}
    for name in ("z", "r_comov", "dist_m", "weights", "delta", "ra", "dec", "x_cart",
                 "y_cart", "z_cart", "cos_dec", "z_qso", "obj_r_comov", "obj_dist_m",
                 "obj_weight"):
        conv[name] = _d(getattr(fs, name))
    for name in ("thingid", "plate", "fiberid", "pix_offset"):
        conv[name] = np.ascontiguousarray(getattr(fs, name), dtype=np.int64)
    keep.append(conv)
    args = {"num": fs.num}
    for name, arr in conv.items():
        args[name] = _ptr(arr, ctypes.c_int64 if arr.dtype == np.int64 else ctypes.c_double)
    return OracleSet(**args)


def cf_forest_pair(params, z1, r1, m1, w1, d1, zq1, z2, r2, m2, w2, d2, zq2, ang,
                   same_half_plate, outputs):
    """Accumulate one forest pair into ``outputs`` = (we, xi, rp, rt, z, nb)."""
    arrs = [_d(a) for a in (z1, r1, m1, w1, d1, z2, r2, m2, w2, d2)]
    lib().oracle_cf_forest_pair(
        ctypes.byref(params),
        *[_ptr(a, ctypes.c_double) for a in arrs[:5]], ctypes.c_int64(len(arrs[0])),
        ctypes.c_double(zq1),
        *[_ptr(a, ctypes.c_double) for a in arrs[5:]], ctypes.c_int64(len(arrs[5])),
        ctypes.c_double(zq2), ctypes.c_double(ang), ctypes.c_int32(int(same_half_plate)),
        *[_ptr(o, ctypes.c_double) for o in outputs[:5]], _ptr(outputs[5], ctypes.c_int64))


def xcf_forest(params, z1, r1, m1, w1, d1, zq, rq, mq, wq, ang, outputs):
    """Accumulate one forest against its quasar neighbours into ``outputs``."""
    arrs = [_d(a) for a in (z1, r1, m1, w1, d1, zq, rq, mq, wq, ang)]
    lib().oracle_xcf_forest(
        ctypes.byref(params),
        *[_ptr(a, ctypes.c_double) for a in arrs[:5]], ctypes.c_int64(len(arrs[0])),
        *[_ptr(a, ctypes.c_double) for a in arrs[5:]], ctypes.c_int64(len(arrs[5])),
        *[_ptr(o, ctypes.c_double) for o in outputs[:5]], _ptr(outputs[5], ctypes.c_int64))


def neighbours(set1, set2, params, ang_max, auto_mode, f_begin=0, f_end=None, xcf=False):
    """Neighbour CSR (offsets, index) for forests [f_begin, f_end) of set1."""
    f_end = set1.num if f_end is None else f_end
    keep = []
    s1 = _as_set(set1, keep)
    s2 = _as_set(set2, keep)
    count = np.zeros(f_end - f_begin, dtype=np.int64)
    if xcf:
        lib().oracle_xcf_neighbours(ctypes.byref(s1), ctypes.byref(s2), ctypes.byref(params),
                                    ctypes.c_double(ang_max), ctypes.c_int64(f_begin),
                                    ctypes.c_int64(f_end), _ptr(count, ctypes.c_int64),
                                    None, None)
    else:
        lib().oracle_cf_neighbours(ctypes.byref(s1), ctypes.byref(s2), ctypes.c_int32(auto_mode),
                                   ctypes.c_double(ang_max), ctypes.c_int64(f_begin),
                                   ctypes.c_int64(f_end), _ptr(count, ctypes.c_int64), None, None)
    offsets = np.zeros(f_end - f_begin + 1, dtype=np.int64)
    np.cumsum(count, out=offsets[1:])
    index = np.zeros(max(int(offsets[-1]), 1), dtype=np.int64)
    if xcf:
        lib().oracle_xcf_neighbours(ctypes.byref(s1), ctypes.byref(s2), ctypes.byref(params),
                                    ctypes.c_double(ang_max), ctypes.c_int64(f_begin),
                                    ctypes.c_int64(f_end), None, _ptr(offsets, ctypes.c_int64),
                                    _ptr(index, ctypes.c_int64))
    else:
        lib().oracle_cf_neighbours(ctypes.byref(s1), ctypes.byref(s2), ctypes.c_int32(auto_mode),
                                   ctypes.c_double(ang_max), ctypes.c_int64(f_begin),
                                   ctypes.c_int64(f_end), None, _ptr(offsets, ctypes.c_int64),
                                   _ptr(index, ctypes.c_int64))
    return offsets, index[: offsets[-1]]


def rows(set1, set2, params, offsets, index, f_begin=0, f_end=None, xcf=False):
    """Per-row (healpix) raw sums (we, xi, rp, rt, z, nb), shape [nrows, nbins]."""
    f_end = set1.num if f_end is None else f_end
    num_rows = len(set1.healpix_list)
    nbins = params.num_bins_r_par * params.num_bins_r_trans
    outs = [np.zeros((num_rows, nbins)) for _ in range(5)]
    outs.append(np.zeros((num_rows, nbins), dtype=np.int64))
    keep = []
    s1 = _as_set(set1, keep)
    s2 = _as_set(set2, keep)
    row = np.ascontiguousarray(set1.row, dtype=np.int32)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    index = np.ascontiguousarray(index, dtype=np.int64)
    if index.size == 0:
        index = np.zeros(1, dtype=np.int64)
    func = lib().oracle_xcf_rows if xcf else lib().oracle_cf_rows
    func(ctypes.byref(s1), ctypes.byref(s2), ctypes.byref(params), ctypes.c_int64(f_begin),
         ctypes.c_int64(f_end), _ptr(offsets, ctypes.c_int64), _ptr(index, ctypes.c_int64),
         _ptr(row, ctypes.c_int32), ctypes.c_int32(num_rows),
         *[_ptr(o, ctypes.c_double) for o in outs[:5]], _ptr(outs[5], ctypes.c_int64))
    return outs


def normalise_rows(outs):
    """cf.compute_xi's final division by the weights (py/picca/cf.py:242-246)."""
    we, xi, rp, rt, zz, nb = [o.copy() for o in outs]
    w = we > 0
    xi[w] /= we[w]
    rp[w] /= we[w]
    rt[w] /= we[w]
    zz[w] /= we[w]
    return we, xi, rp, rt, zz, nb


def aggregate(norm_rows, healpix_list):
    """ATTRI/COR columns as in py/picca/bin/picca_cf.py:465-484."""
    we, xi, rp, rt, zz, nb = norm_rows
    sum_weights = we.sum(axis=0)
    w = sum_weights > 0
    r_par = (rp * we).sum(axis=0)
    r_par[w] /= sum_weights[w]
    r_trans = (rt * we).sum(axis=0)
    r_trans[w] /= sum_weights[w]
    z = (zz * we).sum(axis=0)
    z[w] /= sum_weights[w]
    return {"RP": r_par, "RT": r_trans, "Z": z, "NB": nb.sum(axis=0),
            "HEALPID": np.asarray(healpix_list), "WE": we, "DA": xi}


def cf_pipeline(set1, set2, params, ang_max):
    """Whole auto/cross correlation of ForestSets on the CPU oracle."""
    auto = set2 is None
    other = set1 if auto else set2
    offsets, index = neighbours(set1, other, params, ang_max, auto_mode=int(auto))
    return aggregate(normalise_rows(rows(set1, other, params, offsets, index)),
                     set1.healpix_list)


def xcf_pipeline(forests, objs, params, ang_max):
    """Whole delta x quasar correlation on the CPU oracle."""
    offsets, index = neighbours(forests, objs, params, ang_max, auto_mode=0, xcf=True)
    return aggregate(normalise_rows(rows(forests, objs, params, offsets, index, xcf=True)),
                     forests.healpix_list)
