"""Metal distortion matrices on the GPU: cf.compute_metal_dmat
(py/picca/cf.py:890-1218) with picca_metal_dmat.py
(py/picca/bin/picca_metal_dmat.py:446-520), and xcf.compute_metal_dmat
(py/picca/xcf.py:677-800) with picca_metal_xdmat.py.

Host side of ``pg_cf_metal_dmat``: the pixels of a forest set seen as an
absorber (distances from the fiducial cosmology at z_abs = 10^log_lambda /
lambda_abs - 1, redshift-evolution factor, weight kept where z_abs < z_qso,
cf.py:949-962), the list of absorber pairs, the direct and swapped passes,
and the normalisation. The forest pairs and their random rejection are the
distortion matrix's (``picca_gb300.dmat``): picca_metal_dmat.py re-seeds the
generator per chunk for every absorber pair, so each pair keeps the same
forest pairs.
"""

import ctypes

import numpy as np
import torch

from . import _native, constants
from . import dmat as _dmat
from . import pairs as _pairs
from ._native import DmatSumsC, check


class MetalPixelsC(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name in
                ("r_comov", "dist_m", "z", "zfac", "weights")]


def _bind():
    lib = _native.lib()
    if not getattr(lib, "_metal_bound", False):
        lib.pg_cf_metal_dmat.restype = ctypes.c_int
        lib.pg_cf_metal_dmat.argtypes = [
            ctypes.c_void_p, ctypes.POINTER(_native.CorrParams),
            ctypes.POINTER(_native.DmatParamsC), ctypes.c_double,
            ctypes.POINTER(_native.ForestSetC), ctypes.POINTER(_native.ForestSetC),
            ctypes.POINTER(MetalPixelsC), ctypes.POINTER(MetalPixelsC), ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(DmatSumsC),
            ctypes.c_void_p]
        lib.pg_xcf_metal_dmat.restype = ctypes.c_int
        lib.pg_xcf_metal_dmat.argtypes = lib.pg_cf_metal_dmat.argtypes
        lib._metal_bound = True
    return lib


def absorber_pixels(dev, cosmo, abs_name, alpha, z_ref=None):
    """Pixels of a DeviceForests seen as absorber ``abs_name`` (aligned with
    its compacted pixel arrays), as device tensors and their C struct.
    zfac = (1 + z_abs)^(alpha - 1), or ((1 + z_abs) / (1 + z_ref))^(alpha - 1)
    when ``z_ref`` is given (the cross's form, xcf.py:752-754)."""
    fs = dev.source
    weights = np.asarray(fs.weights, dtype=np.float64)
    keep = weights != 0
    npix = np.asarray(dev.npix)
    log_lambda = np.asarray(fs.log_lambda, dtype=np.float64)[keep]
    w = weights[keep]
    z_qso = np.repeat(np.asarray(fs.z_qso, dtype=np.float64), npix)
    z_abs = 10**log_lambda / constants.ABSORBER_IGM[abs_name] - 1
    arrays = {
        "r_comov": np.asarray(cosmo.get_r_comov(z_abs), dtype=np.float64),
        "dist_m": np.asarray(cosmo.get_dist_m(z_abs), dtype=np.float64),
        "z": z_abs,
        "zfac": ((1 + z_abs) ** (alpha - 1) if z_ref is None
                 else ((1.0 + z_abs) / (1.0 + z_ref)) ** (alpha - 1.0)),
        "weights": np.where(z_abs < z_qso, w, 0.0),
    }
    tensors = {k: torch.from_numpy(np.ascontiguousarray(v if v.size else np.zeros(1)))
               .to(dev.device) for k, v in arrays.items()}
    c = MetalPixelsC(*[tensors[k].data_ptr() for k in ("r_comov", "dist_m", "z", "zfac",
                                                        "weights")])
    return tensors, c


class MetalEngine(_dmat.DmatEngine):
    """Metal distortion-matrix passes on one CUDA device."""

    def run_pass(self, params, dparams, zevol_den, dev1, dev2, side1, side2, first, second,
                 num_pairs, sums, angles=None, cross=False):
        lib = _bind()
        entry = lib.pg_xcf_metal_dmat if cross else lib.pg_cf_metal_dmat
        out = DmatSumsC(*[sums[k].data_ptr() for k in ("weights_dmat", "dmat", "r_par_eff",
                                                         "r_trans_eff", "z_eff", "weight_eff")])
        with torch.cuda.device(self.device):
            check(entry(
                self.engine.plan.handle, ctypes.byref(params), ctypes.byref(dparams),
                float(zevol_den), ctypes.byref(dev1.c),
                ctypes.byref(dev2.c) if dev2 is not None else None, ctypes.byref(side1[1]),
                ctypes.byref(side2[1]), first.data_ptr(), second.data_ptr(),
                angles.data_ptr() if angles is not None else None, int(num_pairs),
                ctypes.byref(out), self.engine._stream()), "metal distortion matrix")
        return sums


def absorber_pairs(lambda_abs, abs_igm, lambda_abs2=None, abs_igm2=None):
    """(abs1, abs2) pairs of picca_metal_dmat.py:446-470 (without the
    fast-metals filter)."""
    first = [lambda_abs] + list(abs_igm)
    second = [lambda_abs2 or lambda_abs] + list(abs_igm2 if abs_igm2 is not None else abs_igm)
    out = []
    for i1, a1 in enumerate(first):
        i0 = i1 if (lambda_abs2 or lambda_abs) == lambda_abs else 0
        for i2, a2 in enumerate(second[i0:]):
            if i1 == 0 and i2 == 0:
                continue
            out.append((a1, a2))
    return out


def swapped_pass(abs1, abs2, x_correlation, same_tracer=False):
    """Whether cf.compute_metal_dmat adds the swapped pass (cf.py:1088-1090):
    two different absorbers in the folded auto-correlation, or an unfolded
    r_par with the same tracer on both sides (cf.lambda_abs ==
    cf.lambda_abs2, which picca only sets for two delta fields)."""
    if not x_correlation:
        return abs1 != abs2
    return bool(same_tracer)


def normalise(raw, params, dparams, npall, npused):
    """py/picca/bin/picca_metal_dmat.py:497-503 (no redshift rescaling)."""
    nb = params.num_bins_r_par * params.num_bins_r_trans
    weights = raw["weight_eff"]
    rp, rt, z = raw["r_par_eff"].copy(), raw["r_trans_eff"].copy(), raw["z_eff"].copy()
    w = weights > 0
    rp[w] /= weights[w]
    rt[w] /= weights[w]
    z[w] /= weights[w]
    wdm = raw["weights_dmat"].copy()
    dm = raw["dmat"].reshape(nb, -1).copy()
    w = wdm > 0
    dm[w, :] /= wdm[w, None]
    return {"RP": rp, "RT": rt, "Z": z, "DM": dm, "WDM": wdm, "NPALL": int(npall),
            "NPUSED": int(npused)}


def metal_distortion_matrices(fs, params, dparams, cosmo, reject, abs_igm, alpha_abs,
                              lambda_abs="LYA", z_ref=2.25, nproc=1, engine=None, mask=None,
                              only=None, fs2=None, abs_igm2=None, lambda_abs2=None):
    """picca_metal_dmat.py on a ForestSet (auto-correlation, or the cross
    with a second field ``fs2``: of the same tracer, or of a second tracer
    ``lambda_abs2`` with its absorbers ``abs_igm2``, fs2's distances being
    that tracer's): for every absorber pair (or the pairs in ``only``), the
    normalised (RP, RT, Z, DM, WDM) and the pair counts. ``alpha_abs`` maps
    absorber names to their redshift-evolution exponents."""
    eng = engine if isinstance(engine, MetalEngine) else MetalEngine(engine)
    pe = eng.engine
    dev = _pairs.DeviceForests(fs, pe.device)
    dev2 = _pairs.DeviceForests(fs2, pe.device) if fs2 is not None else None
    offsets, index, total = pe.neighbours(params, dev, dev2)
    offsets_h = offsets.cpu().numpy()
    if mask is None:
        mask = _dmat.selection_mask(fs.healpix_list, fs.row, offsets_h, nproc, reject)
    first, second, num = eng.pair_list(dev, dev2, offsets, index, mask)
    pixels = {}

    def side(which, name):
        key = (which, name)
        if key not in pixels:
            pixels[key] = absorber_pixels(dev if which == 1 or dev2 is None else dev2, cosmo,
                                          name, alpha_abs[name])
        return pixels[key]

    results = {}
    same_tracer = fs2 is not None and (lambda_abs2 is None or lambda_abs2 == lambda_abs)
    pairs_list = absorber_pairs(lambda_abs, abs_igm,
                                (lambda_abs2 or lambda_abs) if fs2 is not None else None,
                                abs_igm2)
    for abs1, abs2 in pairs_list:
        if only is not None and (abs1, abs2) not in only:
            continue
        sums = eng.alloc_sums(params, dparams)
        den = (1 + z_ref) ** (alpha_abs[abs1] + alpha_abs[abs2] - 2)
        eng.run_pass(params, dparams, den, dev, dev2, side(1, abs1), side(2, abs2), first,
                     second, num, sums)
        if swapped_pass(abs1, abs2, bool(params.x_correlation), same_tracer=same_tracer):
            den2 = (1 + z_ref) ** (alpha_abs[abs2] + alpha_abs[abs1] - 2)
            eng.run_pass(params, dparams, den2, dev, dev2, side(1, abs2), side(2, abs1), first,
                         second, num, sums)
        pe.stats()
        raw = {k: v.cpu().numpy() for k, v in sums.items()}
        results[f"{abs1}_{abs2}"] = normalise(raw, params, dparams, total, int(mask.sum()))
    return results



def quasar_pixel_set(qs):
    """The quasars of a ForestSet as one-pixel forests (the second side of
    pg_xcf_metal_dmat)."""
    from .forests import ForestSet
    n = qs.num
    return ForestSet(
        pix_offset=np.arange(n + 1, dtype=np.int64), z=np.asarray(qs.z_qso, float),
        r_comov=np.asarray(qs.obj_r_comov, float), dist_m=np.asarray(qs.obj_dist_m, float),
        weights=np.asarray(qs.obj_weight, float), delta=np.zeros(n), log_lambda=np.zeros(n),
        ra=qs.ra, dec=qs.dec, x_cart=qs.x_cart, y_cart=qs.y_cart, z_cart=qs.z_cart,
        cos_dec=qs.cos_dec, z_qso=qs.z_qso, thingid=qs.thingid, plate=qs.plate,
        fiberid=qs.fiberid, healpix=qs.healpix, healpix_list=qs.healpix_list, row=qs.row)


def quasar_side(dev_q):
    """pg_metal_pixels of the one-pixel quasar forests: their own distances,
    redshift and weight, zfac = 1."""
    fs = dev_q.source
    keep = np.asarray(fs.weights) != 0
    arrays = {"r_comov": np.asarray(fs.r_comov, float)[keep],
              "dist_m": np.asarray(fs.dist_m, float)[keep],
              "z": np.asarray(fs.z, float)[keep], "zfac": np.ones(int(keep.sum())),
              "weights": np.asarray(fs.weights, float)[keep]}
    tensors = {k: torch.from_numpy(np.ascontiguousarray(v if v.size else np.zeros(1)))
               .to(dev_q.device) for k, v in arrays.items()}
    return tensors, MetalPixelsC(*[tensors[k].data_ptr() for k in ("r_comov", "dist_m", "z",
                                                                    "zfac", "weights")])


def forests_without_pixels(fs, abs_name):
    """Forests with no pixel below their quasar redshift as ``abs_name``
    (xcf.compute_metal_dmat skips them before drawing, xcf.py:713-727)."""
    lam = constants.ABSORBER_IGM[abs_name]
    npix = np.diff(np.asarray(fs.pix_offset))
    z_abs = 10**np.asarray(fs.log_lambda, float) / lam - 1
    below = (z_abs < np.repeat(np.asarray(fs.z_qso, float), npix)).astype(np.int64)
    csum = np.concatenate([[0], np.cumsum(below)])
    off = np.asarray(fs.pix_offset)
    return (csum[off[1:]] - csum[off[:-1]]) == 0


def cross_metal_distortion_matrices(fs, qs, params, dparams, cosmo, reject, abs_igm,
                                    alpha_abs, z_ref=2.25, nproc=1, engine=None):
    """picca_metal_xdmat.py on a forest set and a quasar set: for every
    absorber, the normalised (RP, RT, Z, DM, WDM) and the pair counts."""
    eng = engine if isinstance(engine, MetalEngine) else MetalEngine(engine)
    pe = eng.engine
    dev = _pairs.DeviceForests(fs, pe.device)
    dev_objs = _pairs.DeviceForests(qs, pe.device)
    offsets, index, total = pe.neighbours(params, dev, dev_objs, xcf=True)
    offsets_h = offsets.cpu().numpy()
    qpix = quasar_pixel_set(qs)
    dev_q = _pairs.DeviceForests(qpix, pe.device)
    qside = quasar_side(dev_q)
    # quasars dropped by the compaction (zero weight) would change the
    # indices of the one-pixel set; their pairs add nothing either way
    results = {}
    for abs_name in abs_igm:
        skip = forests_without_pixels(fs, abs_name)
        mask = _dmat.selection_mask(fs.healpix_list, fs.row, offsets_h, nproc, reject,
                                    skip=skip)
        counts = offsets_h[1:] - offsets_h[:-1]
        npall = int(counts[~skip].sum())
        first, second, num = eng.pair_list(dev, dev_q, offsets, index, mask)
        side = absorber_pixels(dev, cosmo, abs_name, alpha_abs[abs_name], z_ref=z_ref)
        sums = eng.alloc_sums(params, dparams)
        eng.run_pass(params, dparams, 1.0, dev, dev_q, side, qside, first, second, num, sums,
                     cross=True)
        pe.stats()
        raw = {k: v.cpu().numpy() for k, v in sums.items()}
        results[abs_name] = normalise(raw, params, dparams, npall, int(mask.sum()))
    return results
