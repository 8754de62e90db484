"""Line-of-sight objects consumed by the correlation path.

Mirrors the parts of ``py/picca/data.py`` that the pair accumulation reads:
``QSO`` (position, redshift, identifiers, ``get_angle_between``) and
``Delta`` (pixel arrays, ``from_fitsio``, ``from_image``, ``project``,
``rebin``). The arithmetic of ``get_angle_between`` and ``project`` uses the
same numpy expressions as the reference so that angles and projected deltas
are bit-identical for the same input.
"""

from itertools import repeat

import numpy as np

from . import constants


class QSO:
    """Quasar: position (radians), redshift and identifiers.

    Follows ``QSO.__init__`` (py/picca/data.py:60-104)."""

    def __init__(self, los_id, ra, dec, z_qso, plate, mjd, fiberid):
        self.ra = ra
        self.dec = dec
        self.plate = plate
        self.mjd = mjd
        self.fiberid = fiberid
        self.x_cart = np.cos(ra) * np.cos(dec)
        self.y_cart = np.sin(ra) * np.cos(dec)
        self.z_cart = np.sin(dec)
        self.cos_dec = np.cos(dec)
        self.z_qso = z_qso
        self.los_id = los_id
        self.thingid = los_id
        self.weight = None
        self.weights = None
        self.r_comov = None
        self.dist_m = None
        self.log_lambda = None

    def get_angle_between(self, data):
        """Angular separation to one object or a list of objects.

        Same formula as py/picca/data.py:106-162: arccos of the clipped dot
        product of unit vectors, replaced by the flat-sky distance when both
        |dRA| and |dDec| are below 2 arcsec."""
        try:
            x_cart = np.array([d.x_cart for d in data])
            y_cart = np.array([d.y_cart for d in data])
            z_cart = np.array([d.z_cart for d in data])
            ra = np.array([d.ra for d in data])
            dec = np.array([d.dec for d in data])
            cos = x_cart * self.x_cart + y_cart * self.y_cart + z_cart * self.z_cart
            cos[cos >= 1.] = 1.
            cos[cos <= -1.] = -1.
            angl = np.arccos(cos)
            w = ((np.absolute(ra - self.ra) < constants.SMALL_ANGLE_CUT_OFF) &
                 (np.absolute(dec - self.dec) < constants.SMALL_ANGLE_CUT_OFF))
            if w.sum() != 0:
                angl[w] = np.sqrt((dec[w] - self.dec)**2 +
                                  (self.cos_dec * (ra[w] - self.ra))**2)
        except TypeError:
            cos = (data.x_cart * self.x_cart + data.y_cart * self.y_cart +
                   data.z_cart * self.z_cart)
            if cos >= 1.:
                cos = 1.
            elif cos <= -1.:
                cos = -1.
            angl = np.arccos(cos)
            if ((np.absolute(data.ra - self.ra) < constants.SMALL_ANGLE_CUT_OFF) &
                    (np.absolute(data.dec - self.dec) < constants.SMALL_ANGLE_CUT_OFF)):
                angl = np.sqrt((data.dec - self.dec)**2 +
                               (self.cos_dec * (data.ra - self.ra))**2)
        return angl


class Delta(QSO):
    """Delta field of one line of sight (py/picca/data.py:238-372)."""

    def __init__(self, los_id, ra, dec, z_qso, plate, mjd, fiberid, log_lambda,
                 weights, cont, delta, order, ivar=None, exposures_diff=None,
                 mean_snr=None, mean_reso=None, mean_z=None):
        QSO.__init__(self, los_id, ra, dec, z_qso, plate, mjd, fiberid)
        self.log_lambda = log_lambda
        self.weights = weights
        self.cont = cont
        self.delta = delta
        self.order = order
        self.ivar = ivar
        self.exposures_diff = exposures_diff
        self.mean_snr = mean_snr
        self.mean_reso = mean_reso
        self.mean_z = mean_z
        self.z = None
        self.r_comov = None
        self.dist_m = None
        self.neighbours = None
        self.fname = None

    @classmethod
    def from_fitsio(cls, hdu, order=None):
        """One BINTABLE HDU per line of sight (py/picca/data.py:376-475,
        non-Pk1D branch)."""
        header = hdu.read_header()
        blinding = header["BLINDING"] if "BLINDING" in header else "none"
        delta_name = "DELTA_BLIND" if blinding != "none" else "DELTA"
        delta = hdu[delta_name][:].astype(float)
        colnames = hdu.get_colnames()
        if "LOGLAM" in colnames:
            log_lambda = hdu["LOGLAM"][:].astype(float)
        elif "LAMBDA" in colnames:
            log_lambda = np.log10(hdu["LAMBDA"][:].astype(float))
        else:
            raise KeyError("Did not find LOGLAM or LAMBDA in delta file")
        weights = hdu["WEIGHT"][:].astype(float)
        cont = hdu["CONT"][:].astype(float)
        if "THING_ID" in header:
            los_id = header["THING_ID"]
            plate = header["PLATE"]
            mjd = header["MJD"]
            fiberid = header["FIBERID"]
        elif "LOS_ID" in header:
            los_id = header["LOS_ID"]
            plate = mjd = fiberid = los_id
        else:
            raise Exception("Could not find THING_ID or LOS_ID")
        return cls(los_id, header["RA"], header["DEC"], header["Z"], plate, mjd,
                   fiberid, log_lambda, weights, cont, delta, order)

    @classmethod
    def from_image(cls, hdul, z_min_qso=0, z_max_qso=10, order=None):
        """Image-format delta files (py/picca/data.py:520-620)."""
        meta = hdul["METADATA"]
        header = meta.read_header()
        blinding = header["BLINDING"] if "BLINDING" in header else "none"
        delta_name = "DELTA_BLIND" if blinding != "none" else "DELTA"
        delta = hdul[delta_name].read().astype(float)
        if "LOGLAM" in hdul:
            log_lambda = hdul["LOGLAM"][:].astype(float)
        elif "LAMBDA" in hdul:
            log_lambda = np.log10(hdul["LAMBDA"][:].astype(float))
        else:
            raise KeyError("Did not find LOGLAM or LAMBDA in delta file")
        weights = hdul["WEIGHT"].read().astype(float)
        w = weights > 0
        cont = hdul["CONT"].read().astype(float)
        colnames = meta.get_colnames()
        if "THING_ID" in colnames:
            los_id = meta["THING_ID"][:]
            plate = meta["PLATE"][:]
            mjd = meta["MJD"][:]
            fiberid = meta["FIBERID"][:]
        elif "LOS_ID" in colnames:
            los_id = meta["LOS_ID"][:]
            plate = mjd = fiberid = los_id
        else:
            raise Exception("Could not find THING_ID or LOS_ID")
        ra = meta["RA"][:]
        dec = meta["DEC"][:]
        z_qso = meta["Z"][:]
        deltas = []
        for (los_id_i, ra_i, dec_i, z_qso_i, plate_i, mjd_i, fiberid_i, loglam,
             weights_i, cont_i, delta_i, w_i) in zip(
                 los_id, ra, dec, z_qso, plate, mjd, fiberid, repeat(log_lambda),
                 weights, cont, delta, w):
            if z_min_qso <= z_qso_i <= z_max_qso:
                deltas.append(cls(los_id_i, ra_i, dec_i, z_qso_i, plate_i, mjd_i,
                                  fiberid_i, loglam[w_i], weights_i[w_i],
                                  cont_i[w_i], delta_i[w_i], order))
        return deltas

    def project(self):
        """Remove the weighted mean and (order 1) the weighted linear trend in
        log lambda (py/picca/data.py:622-655)."""
        if self.order is None:
            raise RuntimeError(
                "Trying to project but order is not defined for the deltas. "
                "Check previous warning to solve this issue")
        sum_weights = np.sum(self.weights)
        if sum_weights > 0.0:
            mean_delta = np.average(self.delta, weights=self.weights)
        else:
            return
        res = 0
        if (self.order == 1) and self.delta.shape[0] > 1:
            mean_log_lambda = np.average(self.log_lambda, weights=self.weights)
            meanless_log_lambda = self.log_lambda - mean_log_lambda
            mean_delta_log_lambda = (
                np.sum(self.weights * self.delta * meanless_log_lambda) /
                np.sum(self.weights * meanless_log_lambda**2))
            res = mean_delta_log_lambda * meanless_log_lambda
        elif self.order == 1:
            res = self.delta
        self.delta -= mean_delta + res

    def rebin(self, factor, dwave=0.8):
        """Rebin a linear-wavelength forest by an integer factor
        (py/picca/data.py:657-686)."""
        wave = 10**np.array(self.log_lambda)
        start = wave.min() - dwave / 2
        num_bins = np.ceil(((wave[-1] - wave[0]) / dwave + 1) / factor)
        edges = np.arange(num_bins) * dwave * factor + start
        new_indx = np.searchsorted(edges, wave)
        binned_delta = np.bincount(new_indx, weights=self.delta * self.weights,
                                   minlength=edges.size + 1)[1:-1]
        binned_weight = np.bincount(new_indx, weights=self.weights,
                                    minlength=edges.size + 1)[1:-1]
        mask = binned_weight != 0
        binned_delta[mask] /= binned_weight[mask]
        new_wave = (edges[1:] + edges[:-1]) / 2
        self.log_lambda = np.log10(new_wave[mask])
        self.delta = binned_delta[mask]
        self.weights = binned_weight[mask]
