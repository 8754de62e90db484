"""Seeded synthetic raw quasar spectra for the continuum fit.

Each forest is observed on picca's log-lambda grid (step 3e-4, observed
3600-5500 Angstrom, rest frame 1040-1200 Angstrom; the Dr16 defaults of
py/picca/delta_extraction/data.py:44-50) or on the linear grid of DESI
(``wave_solution="lin"``, step 0.8 Angstrom, the rest-frame step equal to
it, data.py:402-410). The flux is

    f = A * C(lambda_rf) * (1 + s * (x - 1/2)) * F + noise,

with C = (lambda_rf / 1100)^-1.5 plus Gaussian emission lines at 1033.8,
1073 and 1123 Angstrom (sigma ~ U(5, 10), amplitude ~ U(0, 0.3)), a per-quasar
amplitude A ~ U(0.5, 2) and tilt s ~ N(0, 0.2) over the normalised forest
coordinate x, and F = exp(-tau) with lognormal tau (sigma_ln 0.5) whose
mean is 0.0025 (1+z)^3.7 (mean flux ~ exp(-0.0025 (1+z)^3.7)). The noise is
Gaussian with a per-pixel signal-to-noise ratio lognormal around 2 (sigma_ln
0.5), and ivar = 1/sigma^2. Transmission corrections are 1.
"""

import numpy as np

from . import constants
from .synthetic import band_for_area, redshifts, sky_positions
from .healpix import ang2pix_ring

LYA = constants.ABSORBER_IGM["LYA"]
LINES = (1033.8, 1073.0, 1123.0)


class Grid:
    """Observed and rest-frame wavelength grids (the Forest class variables
    of Forest.set_class_variables,
    py/picca/delta_extraction/astronomical_objects/forest.py:694-748):
    evenly spaced in log10(lambda) (``wave_solution="log"``, steps in
    log10 Angstrom) or in lambda (``"lin"``, steps in Angstrom)."""

    def __init__(self, lambda_min=3600.0, lambda_max=5500.0, lambda_min_rest=1040.0,
                 lambda_max_rest=1200.0, step=3e-4, wave_solution="log", step_rest=None):
        self.step = step
        self.step_rest = step if step_rest is None else step_rest
        self.wave_solution = wave_solution
        self.lambda_min = lambda_min
        if wave_solution == "log":
            self.log_lambda_grid = np.arange(np.log10(lambda_min),
                                             np.log10(lambda_max) + step / 2, step)
            self.log_lambda_rest_frame_grid = np.arange(
                np.log10(lambda_min_rest), np.log10(lambda_max_rest) + self.step_rest / 2,
                self.step_rest)
        elif wave_solution == "lin":
            self.log_lambda_grid = np.log10(np.arange(lambda_min, lambda_max + step / 2, step))
            self.log_lambda_rest_frame_grid = np.log10(
                np.arange(lambda_min_rest, lambda_max_rest + self.step_rest / 2, self.step_rest))
        else:
            raise ValueError(f"wave_solution must be 'log' or 'lin', got {wave_solution!r}")

    @property
    def is_lin(self):
        return self.wave_solution == "lin"

    def find_bins(self, values, grid_array):
        """find_bins_log / find_bins_lin (py/picca/delta_extraction/utils.py:139-186)."""
        if self.is_lin:
            aux = 10**grid_array[0]
            step = 10**grid_array[1] - aux
            return ((10**values - aux) / step + 0.5).astype(np.int64)
        step = grid_array[1] - grid_array[0]
        return ((values - grid_array[0]) / step + 0.5).astype(np.int64)


class RawForests:
    """Flat arrays of raw forests: per pixel log_lambda, flux, ivar,
    transmission_correction; per forest z_qso, los_id, pix_offset, and the
    generating truth (amplitude, tilt) for diagnostics."""

    def __init__(self, **arrays):
        for key, val in arrays.items():
            setattr(self, key, val)
        self.num = int(len(self.z_qso))

    @property
    def npix(self):
        return np.diff(self.pix_offset)

    def forest(self, k):
        sl = slice(self.pix_offset[k], self.pix_offset[k + 1])
        return (self.log_lambda[sl], self.flux[sl], self.ivar[sl],
                self.transmission_correction[sl])


def make_raw_forests(num, seed, grid=None, z_lo=2.1, z_hi=4.0, z_law="inv2", area_deg2=8000.0,
                     nside=16, min_pixels=50):
    """Generate ``num`` raw forests (the continuum-fit inputs)."""
    grid = grid or Grid()
    rng = np.random.default_rng(seed)
    ll0 = grid.log_lambda_grid[0]

    def pixel_range(zq):
        lo = np.maximum(grid.log_lambda_grid[0],
                        grid.log_lambda_rest_frame_grid[0] + np.log10(1 + zq))
        hi = np.minimum(grid.log_lambda_grid[-1],
                        grid.log_lambda_rest_frame_grid[-1] + np.log10(1 + zq))
        if grid.is_lin:
            lam0 = grid.lambda_min
            first = np.ceil((10**lo - lam0) / grid.step - 1e-9).astype(np.int64)
            last = np.floor((10**hi - lam0) / grid.step + 1e-9).astype(np.int64)
        else:
            first = np.ceil((lo - ll0) / grid.step - 1e-9).astype(np.int64)
            last = np.floor((hi - ll0) / grid.step + 1e-9).astype(np.int64)
        return first, np.maximum(last - first + 1, 0)

    # forests shorter than the minimum are rejected as the reader does
    # ("minimum number pixels in forest", py/picca/delta_extraction/data.py:51)
    z_qso = np.zeros(0)
    while len(z_qso) < num:
        cand = redshifts(rng, 2 * num, z_lo, z_hi, z_law)
        z_qso = np.concatenate([z_qso, cand[pixel_range(cand)[1] >= min_pixels]])
    z_qso = z_qso[:num]
    k0, npix = pixel_range(z_qso)
    offset = np.zeros(num + 1, dtype=np.int64)
    np.cumsum(npix, out=offset[1:])
    total = int(offset[-1])
    fid = np.repeat(np.arange(num), npix)
    k = k0[fid] + (np.arange(total) - offset[fid])
    if grid.is_lin:
        log_lambda = np.log10(grid.lambda_min + k * grid.step)
    else:
        log_lambda = ll0 + k * grid.step
    lam = 10**log_lambda
    lam_rf = lam / (1 + z_qso[fid])
    cont = (lam_rf / 1100.0) ** -1.5
    for mu in LINES:
        amp = rng.uniform(0.0, 0.3, num)[fid]
        sig = rng.uniform(5.0, 10.0, num)[fid]
        cont = cont + amp * np.exp(-0.5 * ((lam_rf - mu) / sig) ** 2)
    amplitude = rng.uniform(0.5, 2.0, num)
    tilt = rng.normal(0.0, 0.2, num)
    x = (k - k0[fid]) / np.maximum(npix[fid] - 1, 1)
    cont = amplitude[fid] * cont * (1 + tilt[fid] * (x - 0.5))
    z_pix = lam / LYA - 1
    tau_mean = 0.0025 * (1 + z_pix) ** 3.7
    tau = tau_mean * np.exp(rng.normal(0.0, 0.5, total) - 0.125)
    transmitted = cont * np.exp(-tau)
    snr = 2.0 * np.exp(rng.normal(0.0, 0.5, total))
    sigma = cont / snr
    flux = transmitted + rng.normal(0.0, 1.0, total) * sigma
    ivar = 1.0 / sigma**2
    ra_r, dec_r = band_for_area(area_deg2, 30.0 if area_deg2 > 4000 else 20.0)
    ra, dec = sky_positions(rng, num, ra_r, dec_r)
    healpix = np.atleast_1d(ang2pix_ring(nside, np.pi / 2 - dec, ra)).astype(np.int64)
    return RawForests(
        pix_offset=offset, log_lambda=log_lambda, flux=flux, ivar=ivar,
        transmission_correction=np.ones(total), z_qso=z_qso,
        los_id=np.arange(1, num + 1, dtype=np.int64), ra=ra, dec=dec, healpix=healpix,
        true_amplitude=amplitude, true_tilt=tilt, grid=grid)
