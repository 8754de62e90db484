"""From fitted continua to the correlation input.

The hand-off between delta extraction and the correlation in picca is a set
of delta files: per forest, log lambda, delta and weight
(py/picca/delta_extraction/data.py:62-265 writes them;
py/picca/io.py:493-510 reads them back). ``forests_from_continuum`` does the
same hand-off in memory: it takes the per-pixel deltas and weights of the
Dr16 fit (``Dr16Gpu.deltas``) and applies what ``io.read_deltas`` does on
reading: z = 10^log_lambda / lambda_Lya - 1, comoving and transverse
distances from the fiducial cosmology, the redshift evolution of the weights
w * ((1 + z) / (1 + z_ref))^(alpha - 1) (py/picca/io.py:493-510) and the
projection of each forest (py/picca/data.py:622-655).
"""

import numpy as np

from . import constants
from .forests import ForestSet
from .healpix import ang2pix_ring

LYA = constants.ABSORBER_IGM["LYA"]


def forests_from_continuum(raw, delta, weights, cosmo=None, z_ref=2.25, z_evol=2.9,
                           nside=16, project=True, select=None):
    """ForestSet (sorted by healpix) of the forests of ``raw`` with the given
    per-pixel ``delta`` and ``weights`` (host arrays aligned with
    ``raw.pix_offset``). ``select`` (optional) lists the forests to keep."""
    cosmo = cosmo or constants.Cosmo(Om=0.3147, verbose=False)
    delta = np.asarray(delta, dtype=np.float64)
    weights = np.asarray(weights, dtype=np.float64)
    offsets = np.asarray(raw.pix_offset, dtype=np.int64)
    forests = np.arange(raw.num) if select is None else np.asarray(select, dtype=np.int64)
    npix = offsets[forests + 1] - offsets[forests]
    new_off = np.zeros(forests.size + 1, dtype=np.int64)
    np.cumsum(npix, out=new_off[1:])
    fid = np.repeat(np.arange(forests.size), npix)
    pix = offsets[forests][fid] + (np.arange(new_off[-1]) - new_off[fid])
    log_lambda = np.asarray(raw.log_lambda, dtype=np.float64)[pix]
    z = 10**log_lambda / LYA - 1.0
    w = weights[pix] * ((1 + z) / (1 + z_ref))**(z_evol - 1.0)
    d = delta[pix].copy()
    if project and forests.size:
        # Delta.project (order 1): remove the weighted mean and the weighted
        # linear trend in log lambda
        num = forests.size
        sw = np.bincount(fid, weights=w, minlength=num)
        safe = np.where(sw > 0, sw, 1.0)
        mean_d = np.bincount(fid, weights=w * d, minlength=num) / safe
        mean_ll = np.bincount(fid, weights=w * log_lambda, minlength=num) / safe
        mll = log_lambda - mean_ll[fid]
        num_s = np.bincount(fid, weights=w * d * mll, minlength=num)
        den_s = np.bincount(fid, weights=w * mll**2, minlength=num)
        slope = np.where(den_s > 0, num_s / np.where(den_s > 0, den_s, 1.0), 0.0)
        d = d - (mean_d[fid] + slope[fid] * mll)
    ra = np.asarray(raw.ra, dtype=np.float64)[forests]
    dec = np.asarray(raw.dec, dtype=np.float64)[forests]
    healpix = np.atleast_1d(ang2pix_ring(nside, np.pi / 2 - dec, ra)).astype(np.int64)
    fs = ForestSet(
        pix_offset=new_off, z=z, r_comov=cosmo.get_r_comov(z), dist_m=cosmo.get_dist_m(z),
        weights=w, delta=d, log_lambda=log_lambda, ra=ra, dec=dec,
        x_cart=np.cos(ra) * np.cos(dec), y_cart=np.sin(ra) * np.cos(dec), z_cart=np.sin(dec),
        cos_dec=np.cos(dec), z_qso=np.asarray(raw.z_qso, dtype=np.float64)[forests],
        thingid=np.asarray(raw.los_id, dtype=np.int64)[forests],
        plate=np.zeros(forests.size, dtype=np.int64),
        fiberid=np.zeros(forests.size, dtype=np.int64), healpix=healpix)
    return fs.take(np.argsort(healpix, kind="stable"))
