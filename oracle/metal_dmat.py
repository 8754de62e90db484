"""CPU oracle of picca's metal distortion matrix (TEST INFRASTRUCTURE ONLY).

NumPy restatement of cf.compute_metal_dmat (py/picca/cf.py:890-1218): for
every kept forest pair, the pixel pairs binned with the forest tracer's
distances (data bins) and with the distances the pixels would have if they
were absorber abs_igm1 / abs_igm2 (model bins), weighted by w1 w2 and by the
metals' redshift evolution, as histograms (bincount) over the bins; a second,
swapped pass (abs_igm2 on forest 1, abs_igm1 on forest 2) when the two
absorbers differ in the auto-correlation. ``pipeline`` follows
picca_metal_dmat.py (py/picca/bin/picca_metal_dmat.py:446-520): the list of
absorber pairs, one random rejection per pair of absorbers (the generator is
re-seeded per chunk for each pair, so every pair keeps the same forest pairs)
and the normalisation.
"""

import numpy as np

from . import cpu
from . import dmat as odm


class MetalParams:
    """Binning and cuts of cf.compute_metal_dmat (module globals)."""

    def __init__(self, r_par_min, r_par_max, r_trans_max, num_bins_r_par, num_bins_r_trans,
                 coef_binning_model=1, x_correlation=False,
                 remove_same_half_plate_close_pairs=False, z_ref=2.25, alpha_abs=None):
        self.r_par_min, self.r_par_max, self.r_trans_max = r_par_min, r_par_max, r_trans_max
        self.np, self.nt = int(num_bins_r_par), int(num_bins_r_trans)
        self.nmp = int(num_bins_r_par * coef_binning_model)
        self.nmt = int(num_bins_r_trans * coef_binning_model)
        self.x_correlation = bool(x_correlation)
        self.shp = bool(remove_same_half_plate_close_pairs)
        self.z_ref = z_ref
        self.alpha_abs = dict(alpha_abs or {})


def new_outputs(p):
    nb, nm = p.np * p.nt, p.nmp * p.nmt
    return {"weights_dmat": np.zeros(nb), "dmat": np.zeros(nb * nm), "r_par_eff": np.zeros(nm),
            "r_trans_eff": np.zeros(nm), "z_eff": np.zeros(nm), "weight_eff": np.zeros(nm)}


def _side(log_lambda, r_comov, dist_m, weights, z_qso, lam_abs, cosmo):
    """Pixels of one forest seen as absorber ``lam_abs``, filtered to
    z_abs < z_qso (cf.py:949-962)."""
    z_abs = 10**log_lambda / lam_abs - 1
    r_abs = cosmo.get_r_comov(z_abs)
    m_abs = cosmo.get_dist_m(z_abs)
    keep = z_abs < z_qso
    return (r_comov[keep], dist_m[keep], weights[keep], r_abs[keep], m_abs[keep], z_abs[keep])


def _pass(p, side1, side2, alpha1, alpha2, ang, same_half_plate, out):
    """One histogram pass (cf.py:995-1086)."""
    r1, m1, w1, ra1, ma1, za1 = side1
    r2, m2, w2, ra2, ma2, za2 = side2
    c, s = np.cos(ang / 2), np.sin(ang / 2)
    r_par = (r1[:, None] - r2) * c
    if not p.x_correlation:
        r_par = abs(r_par)
    r_trans = (m1[:, None] + m2) * s
    w12 = w1[:, None] * w2
    bp = np.floor((r_par - p.r_par_min) / (p.r_par_max - p.r_par_min) * p.np).astype(int)
    bt = (r_trans / p.r_trans_max * p.nt).astype(int)
    if p.shp and same_half_plate:
        w12[abs(r_par) < (p.r_par_max - p.r_par_min) / p.np] = 0.0
    bins = bt + p.nt * bp
    ok = (bp < p.np) & (bt < p.nt) & (bp >= 0)
    h = np.bincount(bins[ok], weights=w12[ok])
    out["weights_dmat"][: len(h)] += h
    rp_abs = (ra1[:, None] - ra2) * c
    if not p.x_correlation:
        rp_abs = abs(rp_abs)
    rt_abs = (ma1[:, None] + ma2) * s
    zevol = ((1 + za1[:, None]) ** (alpha1 - 1) * (1 + za2) ** (alpha2 - 1) /
             (1 + p.z_ref) ** (alpha1 + alpha2 - 2))
    mp = np.floor((rp_abs - p.r_par_min) / (p.r_par_max - p.r_par_min) * p.nmp).astype(int)
    mt = (rt_abs / p.r_trans_max * p.nmt).astype(int)
    mb = mt + p.nmt * mp
    ok &= (mp < p.nmp) & (mt < p.nmt) & (mp >= 0)
    wz = w12 * zevol
    nm = p.nmp * p.nmt
    for key, vals in (("r_par_eff", rp_abs * wz), ("r_trans_eff", rt_abs * wz),
                      ("z_eff", (za1[:, None] + za2) / 2 * wz), ("weight_eff", wz)):
        h = np.bincount(mb[ok], weights=vals[ok])
        out[key][: len(h)] += h
    h = np.bincount(mb[ok] + nm * bins[ok], weights=wz[ok])
    out["dmat"][: len(h)] += h


def forest_pair(p, cosmo, f1, f2, ang, same_half_plate, abs1, abs2, swapped, out):
    """One kept forest pair for the absorbers (abs1, abs2); f1 / f2 are
    (log_lambda, r_comov, dist_m, weights, z_qso) tuples."""
    from picca_gb300 import constants
    lam1, lam2 = constants.ABSORBER_IGM[abs1], constants.ABSORBER_IGM[abs2]
    side1 = _side(*f1[:4], f1[4], lam1, cosmo)
    side2 = _side(*f2[:4], f2[4], lam2, cosmo)
    _pass(p, side1, side2, p.alpha_abs[abs1], p.alpha_abs[abs2], ang, same_half_plate, out)
    if swapped:
        side1 = _side(*f1[:4], f1[4], lam2, cosmo)
        side2 = _side(*f2[:4], f2[4], lam1, cosmo)
        _pass(p, side1, side2, p.alpha_abs[abs2], p.alpha_abs[abs1], ang, same_half_plate,
              out)


def absorber_pairs(lambda_abs, abs_igm, lambda_abs2=None, abs_igm2=None):
    """The (abs1, abs2) list of picca_metal_dmat.py:446-470 (no fast-metals
    filter)."""
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


def pipeline(fs, cosmo, p, ang_max, reject, abs_igm, lambda_abs="LYA", nproc=1, fs2=None,
             lambda_abs2=None, abs_igm2=None):
    """picca_metal_dmat.py on a ForestSet (auto-correlation, or the cross of
    two delta fields with ``fs2``: the same tracer on both sides, or a
    second tracer ``lambda_abs2`` with its absorbers ``abs_igm2``, whose
    distances ``fs2`` already carries): per absorber pair the normalised
    (RP, RT, Z, DM, WDM) and the pair counts."""
    other = fs if fs2 is None else fs2
    oparams = cpu.make_params(p.r_par_min, p.r_par_max, p.r_trans_max, p.np, p.nt)
    offsets, index = cpu.neighbours(fs, other, oparams, ang_max, auto_mode=int(fs2 is None))
    mask, npall, npused = odm.selection(fs, offsets, nproc, reject)

    def forest(s, f):
        po = np.asarray(s.pix_offset)
        sl = slice(po[f], po[f + 1])
        return (np.asarray(s.log_lambda[sl]), np.asarray(s.r_comov[sl]),
                np.asarray(s.dist_m[sl]), np.asarray(s.weights[sl]), s.z_qso[f])

    results = {}
    same_tracer = lambda_abs2 is None or lambda_abs2 == lambda_abs
    for abs1, abs2 in absorber_pairs(lambda_abs, abs_igm, lambda_abs2,
                                     abs_igm2 if lambda_abs2 is not None else None):
        # cf.py:1088-1090: the swapped pass for two different absorbers in the
        # folded auto-correlation, or two fields of the same tracer
        swapped = (abs1 != abs2) if not p.x_correlation else (fs2 is not None and same_tracer)
        out = new_outputs(p)
        for f in range(fs.num):
            for k in range(int(offsets[f]), int(offsets[f + 1])):
                if not mask[k]:
                    continue
                g = int(index[k])
                ang = cpu.lib().oracle_angle(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f], fs.ra[f],
                                             fs.dec[f], fs.cos_dec[f], other.x_cart[g],
                                             other.y_cart[g], other.z_cart[g], other.ra[g],
                                             other.dec[g])
                shp = p.shp and fs.plate[f] == other.plate[g] and (
                    (fs.fiberid[f] <= 500) == (other.fiberid[g] <= 500))
                forest_pair(p, cosmo, forest(fs, f), forest(other, g), ang, shp, abs1, abs2,
                            swapped, out)
        results[f"{abs1}_{abs2}"] = normalise(out, p, npall, npused)
    return results


def normalise(out, p, npall, npused):
    """py/picca/bin/picca_metal_dmat.py:497-503."""
    nb = p.np * p.nt
    weights = out["weight_eff"]
    rp, rt, z = out["r_par_eff"].copy(), out["r_trans_eff"].copy(), out["z_eff"].copy()
    w = weights > 0
    rp[w] /= weights[w]
    rt[w] /= weights[w]
    z[w] /= weights[w]
    wdm = out["weights_dmat"].copy()
    dm = out["dmat"].reshape(nb, -1).copy()
    w = wdm > 0
    dm[w, :] /= wdm[w, None]
    return {"RP": rp, "RT": rt, "Z": z, "DM": dm, "WDM": wdm, "NPALL": npall, "NPUSED": npused}


def xforest(p, cosmo, f1, objs, angs, abs_name, out):
    """xcf.compute_metal_dmat for one forest and its kept quasars
    (py/picca/xcf.py:706-790); objs = (r_comov, dist_m, weights, z_qso)
    arrays. Strict range tests and truncated bins as the reference."""
    from picca_gb300 import constants
    r1, m1, w1, ra1, ma1, za1 = _side(*f1[:4], f1[4], constants.ABSORBER_IGM[abs_name], cosmo)
    if r1.size == 0:
        return
    zevol = ((1.0 + za1) / (1.0 + p.z_ref)) ** (p.alpha_abs[abs_name] - 1.0)
    nm = p.nmp * p.nmt
    for (r2, m2, w2, z2), ang in zip(zip(*objs), angs):
        c, s = np.cos(ang / 2), np.sin(ang / 2)
        r_par = (r1 - r2) * c
        r_trans = (m1 + m2) * s
        w12 = w1 * w2
        ok = (r_par > p.r_par_min) & (r_par < p.r_par_max) & (r_trans < p.r_trans_max)
        bp = ((r_par - p.r_par_min) / (p.r_par_max - p.r_par_min) * p.np).astype(int)
        bt = (r_trans / p.r_trans_max * p.nt).astype(int)
        bins = bt + p.nt * bp
        h = np.bincount(bins[ok], weights=w12[ok])
        out["weights_dmat"][: len(h)] += h
        rp_abs = (ra1 - r2) * c
        rt_abs = (ma1 + m2) * s
        mp = ((rp_abs - p.r_par_min) / (p.r_par_max - p.r_par_min) * p.nmp).astype(int)
        mt = (rt_abs / p.r_trans_max * p.nmt).astype(int)
        mb = mt + p.nmt * mp
        ok &= (rp_abs > p.r_par_min) & (rp_abs < p.r_par_max) & (rt_abs < p.r_trans_max)
        wz = w12 * zevol
        h = np.bincount(mb[ok] + nm * bins[ok], weights=wz[ok])
        out["dmat"][: len(h)] += h
        for key, vals in (("r_par_eff", rp_abs * wz), ("r_trans_eff", rt_abs * wz),
                          ("z_eff", (za1 + z2) / 2 * wz), ("weight_eff", wz)):
            h = np.bincount(mb[ok], weights=vals[ok])
            out[key][: len(h)] += h


def xselection(fs, offsets, nproc, reject, skip):
    """The draws of xcf.compute_metal_dmat: a forest without a pixel below
    its quasar redshift (``skip``) draws nothing and is not counted
    (py/picca/xcf.py:722-727)."""
    rows = np.arange(len(fs.healpix_list))
    chunks = {}
    for index, row in enumerate(rows):
        chunks.setdefault(index % nproc, []).append(row)
    mask = np.zeros(int(offsets[-1]), dtype=bool)
    forest_rows = np.asarray(fs.row)
    npall = npused = 0
    for chunk in chunks.values():
        rng = np.random.RandomState(int(fs.healpix_list[chunk[0]]))
        for row in chunk:
            for f in np.nonzero(forest_rows == row)[0]:
                if skip[f]:
                    continue
                k0, k1 = int(offsets[f]), int(offsets[f + 1])
                mask[k0:k1] = rng.rand(k1 - k0) > reject
                npall += k1 - k0
                npused += int(mask[k0:k1].sum())
    return mask, npall, npused


def xpipeline(fs, qs, cosmo, p, ang_max, reject, abs_igm, nproc=1):
    """picca_metal_xdmat.py: per absorber the normalised matrices (keys
    "QSO_" + absorber in the output file)."""
    from picca_gb300 import constants
    oparams = cpu.make_params(p.r_par_min, p.r_par_max, p.r_trans_max, p.np, p.nt)
    offsets, index = cpu.neighbours(fs, qs, oparams, ang_max, auto_mode=0, xcf=True)
    po = np.asarray(fs.pix_offset)
    results = {}
    for abs_name in abs_igm:
        lam = constants.ABSORBER_IGM[abs_name]
        skip = np.array([not np.any(10**fs.log_lambda[po[f]:po[f + 1]] / lam - 1 < fs.z_qso[f])
                         for f in range(fs.num)])
        mask, npall, npused = xselection(fs, offsets, nproc, reject, skip)
        out = new_outputs(p)
        for f in range(fs.num):
            kept = [int(index[k]) for k in range(int(offsets[f]), int(offsets[f + 1]))
                    if mask[k]]
            if not kept:
                continue
            angs = [cpu.lib().oracle_angle(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f], fs.ra[f],
                                           fs.dec[f], fs.cos_dec[f], qs.x_cart[g], qs.y_cart[g],
                                           qs.z_cart[g], qs.ra[g], qs.dec[g]) for g in kept]
            sl = slice(po[f], po[f + 1])
            xforest(p, cosmo, (fs.log_lambda[sl], fs.r_comov[sl], fs.dist_m[sl],
                               fs.weights[sl], fs.z_qso[f]),
                    (qs.obj_r_comov[kept], qs.obj_dist_m[kept], qs.obj_weight[kept],
                     qs.z_qso[kept]), angs, abs_name, out)
        results[abs_name] = normalise(out, p, npall, npused)
    return results
