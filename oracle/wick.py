"""CPU oracle of picca's Wick covariance of the auto-correlation (TEST
INFRASTRUCTURE ONLY).

Restates picca_wick.py (py/picca/bin/picca_wick.py:392-540) with
cf.compute_wick_terms (py/picca/cf.py:1328-1495): the 1D variance and 1D
correlation of the pixels of one forest, read from a picca_cf1d.py file and
interpolated to the nearest tabulated point (scipy interp1d, as the
reference); one random draw per forest (healpix by healpix, the generator
seeded with the first healpix of each process chunk, picca_wick.py:20-37,
cf.py:1376-1380); for every kept forest with neighbours, the weighted 1D
correlation matrices X = (w w^T) xi_1d(|dlog_lambda|) sqrt(v v^T) of the
forest and of each neighbour, and the terms T1-T3 of the pair by the C
restatement of cf.compute_wickT123_pairs (``wick_oracle.c``); then the
normalisation by WALL WALL^T and NPUSED / NPALL. Diagrams beyond the third
(T4, T5) are off by default in picca_wick.py (--max-diagram 3) and T6 is
never filled, so those columns are zero.
"""

import ctypes

import numpy as np
from scipy.interpolate import interp1d

from . import cpu

_P = ctypes.POINTER


class WickParams(ctypes.Structure):
    _fields_ = [("r_par_min", ctypes.c_double), ("r_par_max", ctypes.c_double),
                ("r_trans_max", ctypes.c_double), ("num_bins_r_par", ctypes.c_int32),
                ("num_bins_r_trans", ctypes.c_int32), ("x_correlation", ctypes.c_int32),
                ("pad", ctypes.c_int32)]


def make_params(r_par_min, r_par_max, r_trans_max, num_bins_r_par, num_bins_r_trans,
                x_correlation=False):
    return WickParams(r_par_min, r_par_max, r_trans_max, num_bins_r_par, num_bins_r_trans,
                      int(bool(x_correlation)), 0)


def _lib():
    lib = cpu.lib()
    if not getattr(lib, "_wick_bound", False):
        d = _P(ctypes.c_double)
        lib.oracle_xwick_t1234.restype = None
        lib.oracle_xwick_t1234.argtypes = (
            [_P(WickParams)] + [d] * 4 + [ctypes.c_int64] + [d] * 4 + [ctypes.c_int64, d,
                                                                     _P(ctypes.c_int64)]
            + [d] * 4)
        lib.oracle_wick_t123.restype = None
        lib.oracle_wick_t123.argtypes = (
            [_P(WickParams)] + [d] * 4 + [ctypes.c_int64] + [d] * 4 + [ctypes.c_int64,
                                                                     ctypes.c_double, d,
                                                                     _P(ctypes.c_int64)]
            + [d] * 3)
        lib._wick_bound = True
    return lib


def _dp(arr):
    return arr.ctypes.data_as(_P(ctypes.c_double))


def interpolants(cf1d):
    """(variance(log_lambda), xi_1d(|dlog_lambda|)) from a picca_cf1d.py
    table: LLMIN, DLL, v1d / nv1d, c1d / nb1d (picca_wick.py:392-421)."""
    log_lambda = cf1d["LLMIN"] + cf1d["DLL"] * np.arange(len(cf1d["v1d"]))
    variance = interp1d(log_lambda[cf1d["nv1d"] > 0], cf1d["v1d"][cf1d["nv1d"] > 0],
                        kind="nearest", fill_value="extrapolate")
    xi = interp1d((log_lambda - cf1d["LLMIN"])[cf1d["nb1d"] > 0],
                  cf1d["c1d"][cf1d["nb1d"] > 0], kind="nearest", fill_value="extrapolate")
    return variance, xi


def weighted_xi_1d(log_lambda, weights, variance, xi):
    """(w w^T) xi_1d(|dlog_lambda|) sqrt(v v^T) of one forest (cf.py:1392-1399)."""
    v = variance(log_lambda)
    return ((weights * weights[:, None]) * xi(abs(log_lambda - log_lambda[:, None]))
            * np.sqrt(v * v[:, None]))


def new_outputs(p):
    nb = p.num_bins_r_par * p.num_bins_r_trans
    return {"weights_wick": np.zeros(nb), "num_pairs_wick": np.zeros(nb, dtype=np.int64),
            "t1": np.zeros((nb, nb)), "t2": np.zeros((nb, nb)), "t3": np.zeros((nb, nb))}


def forest_pair(p, r1, w1, zw1, x1, r2, w2, zw2, x2, ang, out):
    """compute_wickT123_pairs for one forest pair, accumulated into ``out``."""
    a1 = [np.ascontiguousarray(a, dtype=np.float64) for a in (r1, w1, zw1, x1)]
    a2 = [np.ascontiguousarray(a, dtype=np.float64) for a in (r2, w2, zw2, x2)]
    _lib().oracle_wick_t123(ctypes.byref(p), *[_dp(a) for a in a1], len(a1[0]),
                            *[_dp(a) for a in a2], len(a2[0]), float(ang),
                            _dp(out["weights_wick"]),
                            out["num_pairs_wick"].ctypes.data_as(_P(ctypes.c_int64)),
                            _dp(out["t1"]), _dp(out["t2"]), _dp(out["t3"]))


def selection(fs, nproc, reject):
    """Kept forests of compute_wick_terms: healpix rows dealt to nproc
    chunks, np.random.seed(first healpix of the chunk), one rand(len(forests
    of the healpix)) draw per healpix. Returns (keep, npall, npused)."""
    chunks = {}
    for index, row in enumerate(range(len(fs.healpix_list))):
        chunks.setdefault(index % nproc, []).append(row)
    keep = np.zeros(fs.num, dtype=bool)
    rows = np.asarray(fs.row)
    npall = npused = 0
    for chunk in chunks.values():
        rng = np.random.RandomState(int(fs.healpix_list[chunk[0]]))
        for row in chunk:
            members = np.nonzero(rows == row)[0]
            draw = rng.rand(len(members)) > reject
            keep[members] = draw
            npall += len(members)
            npused += int(draw.sum())
    return keep, npall, npused


def pipeline(fs, p, ang_max, cf1d, reject, nproc=1, z_ref=2.25, alpha=2.9, alpha2=None,
             return_raw=False):
    """picca_wick.py on a ForestSet (auto-correlation, max_diagram 3)."""
    alpha2 = alpha if alpha2 is None else alpha2
    oparams = cpu.make_params(p.r_par_min, p.r_par_max, p.r_trans_max, p.num_bins_r_par,
                              p.num_bins_r_trans)
    offsets, index = cpu.neighbours(fs, fs, oparams, ang_max, auto_mode=1)
    keep, npall, npused = selection(fs, nproc, reject)
    variance, xi = interpolants(cf1d)
    po = np.asarray(fs.pix_offset)
    out = new_outputs(p)
    cache = {}

    def forest(f):
        if f not in cache:
            sl = slice(po[f], po[f + 1])
            ll, w = fs.log_lambda[sl], fs.weights[sl]
            cache[f] = (fs.r_comov[sl], w, fs.z[sl], weighted_xi_1d(ll, w, variance, xi))
        return cache[f]

    for f in np.nonzero(keep)[0]:
        r1, w1, z1, x1 = forest(f)
        zw1 = ((1 + z1) / (1 + z_ref)) ** (alpha - 1)
        for k in range(int(offsets[f]), int(offsets[f + 1])):
            g = int(index[k])
            r2, w2, z2, x2 = forest(g)
            zw2 = ((1 + z2) / (1 + z_ref)) ** (alpha2 - 1)
            ang = cpu.lib().oracle_angle(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f], fs.ra[f],
                                         fs.dec[f], fs.cos_dec[f], fs.x_cart[g], fs.y_cart[g],
                                         fs.z_cart[g], fs.ra[g], fs.dec[g])
            forest_pair(p, r1, w1, zw1, x1, r2, w2, zw2, x2, ang, out)
    res = normalise(out, npall, npused)
    if return_raw:
        res["raw"] = out
    return res


def xforest(p, r1, w1, zw1, x1, rq, wq, zwq, ang, out):
    """compute_wickT1234_pairs for one forest and its quasars."""
    a1 = [np.ascontiguousarray(a, dtype=np.float64) for a in (r1, w1, zw1, x1)]
    a2 = [np.ascontiguousarray(a, dtype=np.float64) for a in (rq, wq, zwq, ang)]
    _lib().oracle_xwick_t1234(ctypes.byref(p), *[_dp(a) for a in a1], len(a1[0]),
                              *[_dp(a) for a in a2], len(a2[0]), _dp(out["weights_wick"]),
                              out["num_pairs_wick"].ctypes.data_as(_P(ctypes.c_int64)),
                              _dp(out["t1"]), _dp(out["t2"]), _dp(out["t3"]), _dp(out["t4"]))


def xpipeline(fs, qs, p, ang_max, cf1d, reject, nproc=1, z_ref=2.25, alpha=2.9, alpha_obj=1.44,
              return_raw=False):
    """picca_xwick.py (py/picca/bin/picca_xwick.py:447-520) with
    xcf.compute_wick_terms (py/picca/xcf.py:838-1008) on a forest set and a
    quasar set, --max-diagram 4 (the default): T1-T4."""
    oparams = cpu.make_params(p.r_par_min, p.r_par_max, p.r_trans_max, p.num_bins_r_par,
                              p.num_bins_r_trans)
    offsets, index = cpu.neighbours(fs, qs, oparams, ang_max, auto_mode=0, xcf=True)
    keep, npall, npused = selection(fs, nproc, reject)
    variance, xi = interpolants(cf1d)
    po = np.asarray(fs.pix_offset)
    out = new_outputs(p)
    out["t4"] = np.zeros_like(out["t1"])
    for f in np.nonzero(keep)[0]:
        nbrs = [int(index[k]) for k in range(int(offsets[f]), int(offsets[f + 1]))]
        if not nbrs:
            continue
        sl = slice(po[f], po[f + 1])
        ll, w1, z1 = fs.log_lambda[sl], fs.weights[sl], fs.z[sl]
        x1 = weighted_xi_1d(ll, w1, variance, xi)
        zw1 = ((1 + z1) / (1 + z_ref)) ** (alpha - 1)
        ang = np.array([cpu.lib().oracle_angle(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f],
                                               fs.ra[f], fs.dec[f], fs.cos_dec[f],
                                               qs.x_cart[g], qs.y_cart[g], qs.z_cart[g],
                                               qs.ra[g], qs.dec[g]) for g in nbrs])
        zq = qs.z_qso[nbrs]
        zwq = ((1 + zq) / (1 + z_ref)) ** (alpha_obj - 1)
        xforest(p, fs.r_comov[sl], w1, zw1, x1, qs.obj_r_comov[nbrs], qs.obj_weight[nbrs], zwq,
                ang, out)
    res = normalise(out, npall, npused, terms=("t1", "t2", "t3", "t4"))
    if return_raw:
        res["raw"] = out
    return res


def normalise(out, npall, npused, terms=("t1", "t2", "t3")):
    """picca_wick.py:515-540 (picca_xwick.py:487-506 with T4)."""
    weights = out["weights_wick"] * out["weights_wick"][:, None]
    w = weights > 0.0
    res = {"WALL": out["weights_wick"].copy(), "NB": out["num_pairs_wick"].copy()}
    for key in terms:
        t = out[key].copy()
        t[w] /= weights[w]
        t *= 1.0 * npused / npall
        res[key.upper()] = t
    for key in ("T2", "T3", "T4", "T5", "T6"):
        if key not in res:
            res[key] = np.zeros_like(res["T1"])
    res["CO"] = res["T1"] + res["T2"] + res["T3"] + res["T4"] + res["T5"] + res["T6"]
    res["NPALL"], res["NPUSED"] = npall, npused
    return res
