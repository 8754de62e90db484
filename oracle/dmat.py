"""CPU oracle of picca's distortion matrices (TEST INFRASTRUCTURE ONLY).

``forest_pair`` drives the C restatement of
``cf.compute_dmat_forest_pairs_fast`` (``dmat_oracle.c``, cf.py:519-887),
``xforest`` that of ``xcf.compute_dmat_forest_pairs_fast`` (xcf.py:427-675)
and ``xpipeline`` reproduces ``picca_xdmat.py`` (xcf.compute_dmat,
py/picca/xcf.py:325-424, which skips forests without a kept neighbour
before counting NPALL);
``pipeline`` reproduces ``picca_dmat.py`` for an auto-correlation
(py/picca/bin/picca_dmat.py:21-38, :466-525 and cf.compute_dmat,
py/picca/cf.py:390-517): healpix rows dealt to ``nproc`` chunks, NumPy's
legacy generator seeded with each chunk's first healpix, one
``rand(len(neighbours)) > reject`` draw per forest in row order, neighbours
listed by healpix then position (the order of ``cf.fill_neighs`` with
``query_disc`` returning ascending pixels, which is the index order of a
healpix-sorted ForestSet), then the sums and normalisation of
picca_dmat.py:487-525.
"""

import ctypes

import numpy as np

from . import cpu

_P = ctypes.POINTER


class DmatParams(ctypes.Structure):
    _fields_ = [
        ("r_par_min", ctypes.c_double), ("r_par_max", ctypes.c_double),
        ("r_trans_max", ctypes.c_double),
        ("num_bins_r_par", ctypes.c_int32), ("num_bins_r_trans", ctypes.c_int32),
        ("num_model_bins_r_par", ctypes.c_int32), ("num_model_bins_r_trans", ctypes.c_int32),
        ("z_min_pairs", ctypes.c_double), ("z_max_pairs", ctypes.c_double),
        ("zerr_cut_deg", ctypes.c_double), ("zerr_cut_kms", ctypes.c_double),
        ("x_correlation", ctypes.c_int32), ("remove_same_half_plate_close_pairs", ctypes.c_int32),
        ("redshift_evolution", ctypes.c_int32),
        ("z_ref", ctypes.c_double), ("alpha", ctypes.c_double), ("alpha2", ctypes.c_double),
        ("rmu_binning", ctypes.c_int32), ("pad", ctypes.c_int32),
    ]


def make_params(r_par_min, r_par_max, r_trans_max, num_bins_r_par, num_bins_r_trans,
                coef_binning_model=1, z_min_pairs=None, z_max_pairs=None, zerr_cut_deg=None,
                zerr_cut_kms=None, remove_same_half_plate_close_pairs=False,
                redshift_evolution=True, z_ref=2.25, alpha=2.9, alpha2=2.9,
                rmu_binning=False, x_correlation=False):
    nan = lambda v: float("nan") if v is None else float(v)  # noqa: E731
    return DmatParams(float(r_par_min), float(r_par_max), float(r_trans_max),
                      int(num_bins_r_par), int(num_bins_r_trans),
                      int(num_bins_r_par * coef_binning_model),
                      int(num_bins_r_trans * coef_binning_model), nan(z_min_pairs),
                      nan(z_max_pairs), nan(zerr_cut_deg), nan(zerr_cut_kms),
                      int(bool(x_correlation)), int(bool(remove_same_half_plate_close_pairs)),
                      int(bool(redshift_evolution)), float(z_ref), float(alpha), float(alpha2),
                      int(bool(rmu_binning)), 0)


def _lib():
    lib = cpu.lib()
    if not getattr(lib, "_dmat_bound", False):
        d = _P(ctypes.c_double)
        lib.oracle_dmat_forest_pair.restype = None
        lib.oracle_dmat_forest_pair.argtypes = (
            [_P(DmatParams)] + [d] * 10 + [ctypes.c_int64, ctypes.c_int64, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                           ctypes.c_int32, ctypes.c_int32] + [d] * 6)
        lib.oracle_xdmat_forest.restype = None
        lib.oracle_xdmat_forest.argtypes = (
            [_P(DmatParams)] + [d] * 5 + [ctypes.c_int64] + [d] * 5 + [ctypes.c_int64,
                                                                     ctypes.c_int32] + [d] * 6)
        lib._dmat_bound = True
    return lib


def _dp(arr):
    return arr.ctypes.data_as(_P(ctypes.c_double))


def new_outputs(params):
    nb = params.num_bins_r_par * params.num_bins_r_trans
    nm = params.num_model_bins_r_par * params.num_model_bins_r_trans
    return {"weights_dmat": np.zeros(nb), "dmat": np.zeros(nb * nm),
            "r_par_eff": np.zeros(nm), "r_trans_eff": np.zeros(nm), "z_eff": np.zeros(nm),
            "weight_eff": np.zeros(nm)}


def forest_pair(params, ll1, ll2, r1, r2, m1, m2, z1, z2, w1, w2, zq1, zq2, ang,
                same_half_plate, order1, order2, outputs):
    """Adds one forest pair to ``outputs`` (dict of new_outputs arrays)."""
    arrays = [np.ascontiguousarray(a, dtype=np.float64)
              for a in (ll1, ll2, r1, r2, m1, m2, z1, z2, w1, w2)]
    _lib().oracle_dmat_forest_pair(
        ctypes.byref(params), *[_dp(a) for a in arrays], len(arrays[0]), len(arrays[1]),
        float(zq1), float(zq2), float(ang), int(bool(same_half_plate)), int(order1),
        int(order2), *[_dp(outputs[k]) for k in ("weights_dmat", "dmat", "r_par_eff",
                                                  "r_trans_eff", "z_eff", "weight_eff")])


def xforest(params, ll1, r1, m1, z1, w1, r2, m2, z2, w2, ang, order1, outputs):
    """Adds one forest and its kept objects to ``outputs``."""
    a1 = [np.ascontiguousarray(a, dtype=np.float64) for a in (ll1, r1, m1, z1, w1)]
    a2 = [np.ascontiguousarray(a, dtype=np.float64) for a in (r2, m2, z2, w2, ang)]
    _lib().oracle_xdmat_forest(
        ctypes.byref(params), *[_dp(a) for a in a1], len(a1[0]), *[_dp(a) for a in a2],
        len(a2[0]), int(order1), *[_dp(outputs[k]) for k in ("weights_dmat", "dmat",
                                                             "r_par_eff", "r_trans_eff",
                                                             "z_eff", "weight_eff")])


def selection(fs, offsets, nproc, reject):
    """Boolean mask over the neighbour list: the pairs picca_dmat.py keeps
    (rows dealt to nproc chunks, np.random.seed(first healpix of the chunk),
    one rand(len(neighbours)) draw per forest). Returns (mask, pairs, used)."""
    rows = np.arange(len(fs.healpix_list))
    chunks = {}
    for index, row in enumerate(rows):
        chunks.setdefault(index % nproc, []).append(row)
    order = sorted(chunks.values(), key=lambda c: [fs.healpix_list[r] for r in c])
    mask = np.zeros(int(offsets[-1]), dtype=bool)
    forest_rows = np.asarray(fs.row)
    for chunk in order:
        rng = np.random.RandomState(int(fs.healpix_list[chunk[0]]))
        for row in chunk:
            for f in np.nonzero(forest_rows == row)[0]:
                k0, k1 = int(offsets[f]), int(offsets[f + 1])
                mask[k0:k1] = rng.rand(k1 - k0) > reject
    return mask, int(offsets[-1]), int(mask.sum())


def pipeline(fs, params, ang_max, reject, nproc=1, order=1, fs2=None):
    """picca_dmat.py on a ForestSet (auto-correlation, or the cross with
    ``fs2``). Returns the output columns (WDM, DM, RP, RT, Z) and the pair
    counts."""
    oparams = cpu.make_params(params.r_par_min, params.r_par_max, params.r_trans_max,
                              params.num_bins_r_par, params.num_bins_r_trans)
    other = fs if fs2 is None else fs2
    offsets, index = cpu.neighbours(fs, other, oparams, ang_max, auto_mode=int(fs2 is None))
    mask, npall, npused = selection(fs, offsets, nproc, reject)
    out = new_outputs(params)
    po, po2 = np.asarray(fs.pix_offset), np.asarray(other.pix_offset)
    for f in range(fs.num):
        a0, a1 = po[f], po[f + 1]
        for k in range(int(offsets[f]), int(offsets[f + 1])):
            if not mask[k]:
                continue
            g = int(index[k])
            b0, b1 = po2[g], po2[g + 1]
            ang = cpu.lib().oracle_angle(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f], fs.ra[f],
                                         fs.dec[f], fs.cos_dec[f], other.x_cart[g],
                                         other.y_cart[g], other.z_cart[g], other.ra[g],
                                         other.dec[g])
            shp = params.remove_same_half_plate_close_pairs and (
                fs.plate[f] == other.plate[g]) and (
                (fs.fiberid[f] <= 500 and other.fiberid[g] <= 500) or
                (fs.fiberid[f] > 500 and other.fiberid[g] > 500))
            forest_pair(params, fs.log_lambda[a0:a1], other.log_lambda[b0:b1],
                        fs.r_comov[a0:a1], other.r_comov[b0:b1], fs.dist_m[a0:a1],
                        other.dist_m[b0:b1], fs.z[a0:a1], other.z[b0:b1], fs.weights[a0:a1],
                        other.weights[b0:b1], fs.z_qso[f], other.z_qso[g], ang, shp, order,
                        order, out)
    return normalise(out, params, npall, npused)


def xselection(fs, offsets, nproc, reject):
    """xcf.compute_dmat's draws (same generator use as ``selection``) and
    its counts: forests without a kept neighbour add nothing to NPALL."""
    mask, _, _ = selection(fs, offsets, nproc, reject)
    npall = npused = 0
    for f in range(fs.num):
        k0, k1 = int(offsets[f]), int(offsets[f + 1])
        used = int(mask[k0:k1].sum())
        if used:
            npall += k1 - k0
            npused += used
    return mask, npall, npused


def xpipeline(fs, qs, params, ang_max, reject, nproc=1, order=1):
    """picca_xdmat.py on a forest set and a quasar set."""
    oparams = cpu.make_params(params.r_par_min, params.r_par_max, params.r_trans_max,
                              params.num_bins_r_par, params.num_bins_r_trans)
    offsets, index = cpu.neighbours(fs, qs, oparams, ang_max, auto_mode=0, xcf=True)
    mask, npall, npused = xselection(fs, offsets, nproc, reject)
    out = new_outputs(params)
    po = np.asarray(fs.pix_offset)
    for f in range(fs.num):
        k0, k1 = int(offsets[f]), int(offsets[f + 1])
        kept = [int(index[k]) for k in range(k0, k1) if mask[k]]
        if not kept:
            continue
        ang = np.array([cpu.lib().oracle_angle(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f],
                                               fs.ra[f], fs.dec[f], fs.cos_dec[f],
                                               qs.x_cart[g], qs.y_cart[g], qs.z_cart[g],
                                               qs.ra[g], qs.dec[g]) for g in kept])
        a = slice(po[f], po[f + 1])
        xforest(params, fs.log_lambda[a], fs.r_comov[a], fs.dist_m[a], fs.z[a], fs.weights[a],
                qs.obj_r_comov[kept], qs.obj_dist_m[kept], qs.z_qso[kept],
                qs.obj_weight[kept], ang, order, out)
    return normalise(out, params, npall, npused)


def normalise(out, params, npall, npused):
    """picca_dmat.py:487-525."""
    nb = params.num_bins_r_par * params.num_bins_r_trans
    weights = out["weight_eff"].copy()
    rp, rt, zeff = out["r_par_eff"].copy(), out["r_trans_eff"].copy(), out["z_eff"].copy()
    w = weights > 0
    rp[w] /= weights[w]
    rt[w] /= weights[w]
    zeff[w] /= weights[w]
    mean_zeff = np.mean(zeff[w]) if w.any() else 0.0
    wdm = out["weights_dmat"].copy()
    dmat = out["dmat"].reshape(nb, -1).copy()
    w = wdm > 0
    dmat[w] /= wdm[w, None]
    if params.redshift_evolution:
        zeff[:] = mean_zeff
        zfac = ((1 + params.z_ref) / (1 + mean_zeff)) ** ((params.alpha - 1) +
                                                          (params.alpha2 - 1))
        dmat *= zfac
    return {"WDM": wdm, "DM": dmat, "RP": rp, "RT": rt, "Z": zeff, "NPALL": npall,
            "NPUSED": npused}
