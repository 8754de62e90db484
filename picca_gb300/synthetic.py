"""Seeded synthetic delta fields and quasar catalogues.

No survey data is available offline, so the benchmarks and large-scale
tests run on generated forests with the shapes of real ones:

* positions uniform on the sphere inside a RA/Dec box (a square patch, or a
  declination band of the requested area) at a given density;
* quasar redshifts uniform on [z_lo, z_hi] or distributed as (1+z)^-2
  (inverse-CDF sampling);
* pixels on a log10(lambda) grid of step 3e-4 (or a linear grid of step
  0.8 Angstrom), restricted to rest frame 1040-1200 Angstrom and observed
  lambda >= 3600 Angstrom;
* delta ~ N(0, 0.3^2), pipeline variance lognormal (median 0.1, sigma_ln
  0.5), weights ((1+z)/3.25)^1.9 / (var_pipe + 0.05^2) with z = lambda /
  1215.67 - 1, comoving distances of flat LambdaCDM (Omega_m = 0.3147), and
  the order-1 projection of ``Delta.project`` (py/picca/data.py:622-655).
"""

import numpy as np

from . import constants
from .forests import ForestSet
from .healpix import ang2pix_ring

LYA = constants.ABSORBER_IGM["LYA"]
LOG_STEP = 3e-4
LOG_START = np.log10(3600.0)


def sky_positions(rng, num, ra_range_deg, dec_range_deg):
    """Uniform positions on the sphere inside a RA/Dec box (radians)."""
    ra = np.radians(rng.uniform(ra_range_deg[0], ra_range_deg[1], num))
    s0, s1 = np.sin(np.radians(dec_range_deg[0])), np.sin(np.radians(dec_range_deg[1]))
    dec = np.arcsin(rng.uniform(s0, s1, num))
    return ra, dec


def band_for_area(area_deg2, half_height_deg, ra_start_deg=100.0):
    """RA/Dec box of a declination band of the given area."""
    solid = area_deg2 * (np.pi / 180.0) ** 2
    width = solid / (2 * np.sin(np.radians(half_height_deg)))
    return (ra_start_deg, ra_start_deg + np.degrees(width)), (-half_height_deg, half_height_deg)


def redshifts(rng, num, z_lo, z_hi, law="uniform"):
    if law == "uniform":
        return rng.uniform(z_lo, z_hi, num)
    # p(z) ~ (1+z)^-2 -> CDF ~ 1/(1+z_lo) - 1/(1+z)
    a, b = 1.0 / (1 + z_lo), 1.0 / (1 + z_hi)
    u = rng.uniform(0, 1, num)
    return 1.0 / (a - u * (a - b)) - 1.0


def make_forests(num, seed, ra_range_deg, dec_range_deg, z_lo=2.1, z_hi=3.5, z_law="uniform",
                 grid="log", max_pixels=600, cosmo=None, nside=16, project=True,
                 thingid_start=1):
    """Return a ForestSet of ``num`` synthetic projected delta forests."""
    rng = np.random.default_rng(seed)
    cosmo = cosmo or constants.Cosmo(Om=0.3147, verbose=False)
    ra, dec = sky_positions(rng, num, ra_range_deg, dec_range_deg)
    z_qso = redshifts(rng, num, z_lo, z_hi, z_law)
    lam_min = np.maximum(3600.0, 1040.0 * (1 + z_qso))
    lam_max = 1200.0 * (1 + z_qso)
    if grid == "log":
        k0 = np.ceil((np.log10(lam_min) - LOG_START) / LOG_STEP - 1e-9).astype(np.int64)
        k1 = np.floor((np.log10(lam_max) - LOG_START) / LOG_STEP + 1e-9).astype(np.int64)
    else:
        k0 = np.ceil((lam_min - 3600.0) / 0.8 - 1e-9).astype(np.int64)
        k1 = np.floor((lam_max - 3600.0) / 0.8 + 1e-9).astype(np.int64)
    npix = np.clip(k1 - k0 + 1, 0, max_pixels)
    offset = np.zeros(num + 1, dtype=np.int64)
    np.cumsum(npix, out=offset[1:])
    total = int(offset[-1])
    fid = np.repeat(np.arange(num), npix)
    k = k0[fid] + (np.arange(total) - offset[fid])
    if grid == "log":
        log_lambda = LOG_START + k * LOG_STEP
    else:
        log_lambda = np.log10(3600.0 + k * 0.8)
    z = 10**log_lambda / LYA - 1.0
    r_comov = cosmo.get_r_comov(z)
    dist_m = cosmo.get_dist_m(z)
    delta = rng.normal(0.0, 0.3, total)
    var_pipe = 0.1 * np.exp(rng.normal(0.0, 0.5, total))
    weights = ((1 + z) / 3.25) ** 1.9 / (var_pipe + 0.05**2)
    if project:
        sw = np.bincount(fid, weights=weights, minlength=num)
        safe = np.where(sw > 0, sw, 1.0)
        mean_delta = np.bincount(fid, weights=weights * delta, minlength=num) / safe
        mean_ll = np.bincount(fid, weights=weights * log_lambda, minlength=num) / safe
        mll = log_lambda - mean_ll[fid]
        num_s = np.bincount(fid, weights=weights * delta * mll, minlength=num)
        den_s = np.bincount(fid, weights=weights * mll**2, minlength=num)
        slope = np.where(den_s > 0, num_s / np.where(den_s > 0, den_s, 1.0), 0.0)
        delta = delta - (mean_delta[fid] + slope[fid] * mll)
    healpix = np.atleast_1d(ang2pix_ring(nside, np.pi / 2 - dec, ra)).astype(np.int64)
    order = np.argsort(healpix, kind="stable")
    # reorder forests by healpix (the order the correlation visits them)
    inv_pix = np.concatenate([np.arange(offset[f], offset[f + 1]) for f in order]) \
        if num < 20000 else _gather_pixels(offset, order)
    npix_o = npix[order]
    offset_o = np.zeros(num + 1, dtype=np.int64)
    np.cumsum(npix_o, out=offset_o[1:])
    thingid = np.arange(thingid_start, thingid_start + num, dtype=np.int64)
    return ForestSet(
        pix_offset=offset_o, z=z[inv_pix], r_comov=r_comov[inv_pix], dist_m=dist_m[inv_pix],
        weights=weights[inv_pix], delta=delta[inv_pix], log_lambda=log_lambda[inv_pix],
        ra=ra[order], dec=dec[order], x_cart=np.cos(ra[order]) * np.cos(dec[order]),
        y_cart=np.sin(ra[order]) * np.cos(dec[order]), z_cart=np.sin(dec[order]),
        cos_dec=np.cos(dec[order]), z_qso=z_qso[order], thingid=thingid[order],
        plate=np.zeros(num, dtype=np.int64), fiberid=np.zeros(num, dtype=np.int64),
        order=np.full(num, 1 if project else 0, dtype=np.int64), healpix=healpix[order])


def _gather_pixels(offset, order):
    """Pixel indices of the forests in ``order`` (vectorised)."""
    npix = (offset[1:] - offset[:-1])[order]
    starts = offset[:-1][order]
    out_off = np.zeros(len(order) + 1, dtype=np.int64)
    np.cumsum(npix, out=out_off[1:])
    fid = np.repeat(np.arange(len(order)), npix)
    return starts[fid] + (np.arange(out_off[-1]) - out_off[fid])


def make_quasars(num, seed, ra_range_deg, dec_range_deg, z_lo=2.1, z_hi=4.0, z_law="inv2",
                 cosmo=None, nside=16, z_ref=2.25, alpha=1.44, thingid_start=10_000_000_000):
    """Quasar catalogue ForestSet with weights ((1+z)/(1+z_ref))^(alpha-1)."""
    rng = np.random.default_rng(seed)
    cosmo = cosmo or constants.Cosmo(Om=0.3147, verbose=False)
    ra, dec = sky_positions(rng, num, ra_range_deg, dec_range_deg)
    z_qso = redshifts(rng, num, z_lo, z_hi, z_law)
    healpix = np.atleast_1d(ang2pix_ring(nside, np.pi / 2 - dec, ra)).astype(np.int64)
    order = np.argsort(healpix, kind="stable")
    ra, dec, z_qso, healpix = ra[order], dec[order], z_qso[order], healpix[order]
    return ForestSet(
        ra=ra, dec=dec, x_cart=np.cos(ra) * np.cos(dec), y_cart=np.sin(ra) * np.cos(dec),
        z_cart=np.sin(dec), cos_dec=np.cos(dec), z_qso=z_qso,
        obj_r_comov=np.asarray(cosmo.get_r_comov(z_qso)),
        obj_dist_m=np.asarray(cosmo.get_dist_m(z_qso)),
        obj_weight=((1 + z_qso) / (1 + z_ref)) ** (alpha - 1),
        thingid=np.arange(thingid_start, thingid_start + num, dtype=np.int64),
        plate=np.zeros(num, dtype=np.int64), fiberid=np.zeros(num, dtype=np.int64),
        healpix=healpix)


# The benchmark workloads ------------------------------------------------------
def patch_forests(seed=20261203):
    """1,000 forests in a 4.5 x 4.5 deg patch, z_qso ~ U(2.1, 3.5)."""
    return make_forests(1000, seed, (150.0, 154.5), (0.0, 4.5), 2.1, 3.5, "uniform")


def survey_band(num, area_deg2, seed, grid="log", half_height=None):
    """``num`` forests on a band of ``area_deg2`` with z_qso ~ (1+z)^-2 on
    [2.1, 4.0] (the benchmark surveys: 100k on 2,000 deg^2, 400k on 8,000 deg^2)."""
    if half_height is None:
        half_height = 20.0 if area_deg2 <= 4000 else 30.0
    ra_r, dec_r = band_for_area(area_deg2, half_height)
    return make_forests(num, seed, ra_r, dec_r, 2.1, 4.0, "inv2", grid=grid)


def correlation_ang_max(r_trans_max, z_min, cosmo=None):
    """compute_ang_max for a synthetic set (py/picca/utils.py:419-450)."""
    cosmo = cosmo or constants.Cosmo(Om=0.3147, verbose=False)
    r_min = cosmo.get_dist_m(z_min)
    if 2 * r_min < r_trans_max:
        return np.pi
    return float(2.0 * np.arcsin(r_trans_max / (2 * r_min)))
