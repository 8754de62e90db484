"""CPU oracle of picca's fast metal distortion matrices (TEST INFRASTRUCTURE ONLY).

NumPy restatement of calc_fast_metal_dmat of picca_fast_metal_dmat.py
(py/picca/bin/picca_fast_metal_dmat.py:30-251) and picca_fast_metal_xdmat.py
(py/picca/bin/picca_fast_metal_xdmat.py:28-215), and of the two scripts'
drivers (the list of absorber pairs, py/picca/bin/picca_fast_metal_dmat.py:
546-595; the quasar redshift histogram, py/picca/bin/picca_fast_metal_xdmat.py:
503-512). The matrix is separable: an r_par matrix from all pixel pairs of
the two pixel lists, binned with the assumed and the true absorbers'
distances, and an r_trans matrix from the histogram of the ratio of the
pairs' mean distances, spread over an oversampled r_trans grid; the full
matrix is their Kronecker product. Pinned against picca's golden
fast_metal_dmat, fast_metal_dmat_cross and fast_metal_xdmat files.
"""

import numpy as np

#: pairs whose true |r_par| is below this enter the distance-ratio histogram
NEAR_R_PAR = 20.0
#: r_trans sub-bins per bin in the bin-migration sum
OVERSAMPLE = 7


def rebin(values, factor):
    """Mean over groups of ``factor`` consecutive entries, the tail dropped
    (py/picca/bin/picca_fast_metal_dmat.py:77-99)."""
    if factor is None:
        return values
    n = values.size // factor
    return values[:n * factor].reshape(n, factor).mean(-1)


def stack_side(log_lambda, weight, lam_in, lam_out, alpha_sum, cosmo, rebin_factor=None):
    """One stack as a pixel list: true and assumed absorbers' distances,
    the true redshift and weight (1 + z_in)^(alpha_sum - 2) (:102-146)."""
    log_lambda = rebin(np.asarray(log_lambda, dtype=np.float64), rebin_factor)
    weight = rebin(np.asarray(weight, dtype=np.float64), rebin_factor)
    z_in = 10**log_lambda / lam_in - 1.0
    z_out = 10**log_lambda / lam_out - 1.0
    return {"r_in": cosmo.get_r_comov(z_in), "r_out": cosmo.get_r_comov(z_out), "z_in": z_in,
            "w": weight * (1 + z_in)**(alpha_sum - 2)}


def quasar_side(z_qso, weight_qso, cosmo):
    """The quasars' redshift histogram as a pixel list (true = assumed)."""
    r = cosmo.get_r_comov(z_qso)
    return {"r_in": r, "r_out": r, "z_in": np.asarray(z_qso, dtype=np.float64),
            "w": np.asarray(weight_qso, dtype=np.float64)}


def quasar_histogram(z_qso, weight_qso, num_bins):
    """Weighted mean redshift and summed weight of the quasars per redshift
    bin, empty bins dropped (py/picca/bin/picca_fast_metal_xdmat.py:506-512)."""
    hw, edges = np.histogram(z_qso, bins=num_bins, weights=weight_qso)
    hwz, _ = np.histogram(z_qso, bins=edges, weights=weight_qso * z_qso)
    keep = hw > 0
    return hwz[keep] / hw[keep], hw[keep]


def _pairs(side1, side2, signed):
    r_par_in = (side1["r_in"][:, None] - side2["r_in"][None, :]).ravel()
    r_par_out = (side1["r_out"][:, None] - side2["r_out"][None, :]).ravel()
    if not signed:
        r_par_in, r_par_out = np.abs(r_par_in), np.abs(r_par_out)
    dist_in = ((side1["r_in"][:, None] + side2["r_in"][None, :]) / 2).ravel()
    dist_out = ((side1["r_out"][:, None] + side2["r_out"][None, :]) / 2).ravel()
    w = (side1["w"][:, None] * side2["w"][None, :]).ravel()
    z = ((side1["z_in"][:, None] + side2["z_in"][None, :]) / 2.0).ravel()
    return r_par_in, r_par_out, dist_in, dist_out, w, z


def histograms(side1, side2, r_par_min, r_par_max, num_bins_r_par, num_bins_r_trans, signed):
    """The pair histograms (the part the GPU kernel computes): the r_par
    matrix [output bin, input bin], the distance-ratio histogram and its
    edges, and the weight sums on the output r_par bins (:148-231)."""
    r_par_in, r_par_out, dist_in, dist_out, w, z = _pairs(side1, side2, signed)
    edges = r_par_min + (r_par_max - r_par_min) / num_bins_r_par * np.arange(num_bins_r_par + 1)
    rp, _, _ = np.histogram2d(r_par_out, r_par_in, bins=(edges, edges), weights=w)
    ratio_w, ratio_edges = np.histogram(dist_out / dist_in, bins=4 * (num_bins_r_trans + 1),
                                        weights=w / dist_in**2 * (np.abs(r_par_in) < NEAR_R_PAR))
    sw, _ = np.histogram(r_par_out, bins=edges, weights=w)
    swrp, _ = np.histogram(r_par_out, bins=edges, weights=w * r_par_out)
    swz, _ = np.histogram(r_par_out, bins=edges, weights=w * z)
    return {"rp_dmat": rp, "ratio_weights": ratio_w, "ratio_edges": ratio_edges,
            "out_weight": sw, "out_weight_rp": swrp, "out_weight_z": swz}


def finish(h, r_trans_max, num_bins_r_par, num_bins_r_trans):
    """Normalised r_par and r_trans matrices, their Kronecker product and
    the effective coordinates (:157-249)."""
    nt = num_bins_r_trans
    rp = h["rp_dmat"].copy()
    col = rp.sum(axis=0)
    rp /= col + (col == 0)
    rt_edges = r_trans_max / nt * np.arange(nt + 1)
    ratios = (h["ratio_edges"][1:] + h["ratio_edges"][:-1]) / 2.0
    centres = (rt_edges[:-1] + rt_edges[1:]) / 2.0
    half = (rt_edges[1] - rt_edges[0]) / 2.0
    offsets = np.linspace(-half, half * (1 - 2.0 / OVERSAMPLE), OVERSAMPLE)[None, :]
    rt = np.zeros((nt, nt))
    for i, centre in enumerate(centres):
        rt[:, i], _ = np.histogram((ratios[:, None] * (centre + offsets)[None, :]).ravel(),
                                   bins=rt_edges,
                                   weights=(h["ratio_weights"][:, None]
                                            * (centre + offsets)[None, :]).ravel())
    col = rt.sum(axis=0)
    rt /= col + (col == 0)
    dmat = np.kron(rp, rt)
    sw = h["out_weight"]
    r_par_1d = h["out_weight_rp"] / (sw + (sw == 0))
    z_1d = h["out_weight_z"] / (sw + (sw == 0))
    lo = np.arange(nt) * r_trans_max / nt
    hi = (1 + np.arange(nt)) * r_trans_max / nt
    r_trans_1d = (2 * (hi**3 - lo**3)) / (3 * (hi**2 - lo**2))
    index = np.arange(num_bins_r_par * nt)
    return dmat, r_par_1d[index // nt], r_trans_1d[index % nt], z_1d[index // nt]


def matrix(side1, side2, r_par_min, r_par_max, r_trans_max, num_bins_r_par, num_bins_r_trans,
           signed):
    """calc_fast_metal_dmat for two pixel lists: (dmat, r_par, r_trans, z)."""
    h = histograms(side1, side2, r_par_min, r_par_max, num_bins_r_par, num_bins_r_trans, signed)
    return finish(h, r_trans_max, num_bins_r_par, num_bins_r_trans)


def absorber_pairs(lambda_abs, abs_igm, lambda_abs2=None, abs_igm2=None):
    """(abs1, abs2) pairs of picca_fast_metal_dmat.py:546-595 (without the
    relevant-metals filter)."""
    if lambda_abs2 is None:  # the script then ignores --abs-igm2 (:546-548)
        lambda_abs2, abs_igm2 = lambda_abs, abs_igm
    first = [lambda_abs] + list(abs_igm)
    second = [lambda_abs2] + list(abs_igm2 or [])
    out = []
    for i1, a1 in enumerate(first):
        i0 = i1 if lambda_abs == lambda_abs2 else 0
        for i2, a2 in enumerate(second[i0:]):
            if i1 == 0 and i2 == 0:
                continue
            out.append((a1, a2))
    return out
