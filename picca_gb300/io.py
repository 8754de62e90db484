"""Readers for delta files and quasar catalogues.

Mirrors the host-side input stage of the correlation path in
``py/picca/io.py``: ``read_blinding`` (:297-330), ``find_order`` (:31-112,
FITORDER lookup), ``read_delta_file`` (:333-380), ``read_deltas`` (:383-512)
and ``read_objects`` / ``read_drq`` (:515-614, :160-295, SDSS and DESI
column conventions). The per-pixel derivations (redshift, comoving distances,
redshift-evolution weights, projection) use the same expressions as the
reference so that the arrays handed to the GPU are bit-identical.

Files are read sequentially in this process; the reference's reading Pool is
a throughput detail outside the pair-accumulation path.
"""

import glob
import os
from configparser import ConfigParser

import numpy as np

from . import fitsio_lite as fitsio
from .data import Delta, QSO
from .healpix import ang2pix_ring
from .utils import userprint


def _list_delta_files(in_dir):
    in_dir = os.path.expandvars(in_dir)
    if len(in_dir) > 8 and in_dir[-8:] == ".fits.gz":
        files = glob.glob(in_dir)
    elif len(in_dir) > 5 and in_dir[-5:] == ".fits":
        files = glob.glob(in_dir)
    else:
        files = glob.glob(in_dir + "/*.fits") + glob.glob(in_dir + "/*.fits.gz")
    return sorted(files)


def read_blinding(in_dir):
    """Blinding keyword of the first delta file (py/picca/io.py:297-330)."""
    files = _list_delta_files(in_dir)
    hdul = fitsio.FITS(files[0])
    if "LAMBDA" in hdul:
        return hdul["METADATA"].read_header()["BLINDING"]
    header = hdul[1].read_header()
    return header["BLINDING"] if "BLINDING" in header else "none"


def find_order(in_dir, delta_attributes):
    """Continuum-fit polynomial order from the delta attributes file
    (py/picca/io.py:31-112): FIT_METADATA/FITORDER, then STACK_DELTAS, then
    the ``order`` key of the delta-extraction config."""
    if delta_attributes is None:
        delta_attributes = in_dir + "/../Log/delta_attributes.fits.gz"
        userprint(f"WARNING: delta_attributes file not given, setting to {delta_attributes}")
    try:
        hdul = fitsio.FITS(delta_attributes)
        for extname in ("FIT_METADATA", "STACK_DELTAS"):
            if extname in hdul and "FITORDER" in hdul[extname].read_header():
                return hdul[extname].read_header()["FITORDER"]
    except OSError:
        pass
    config = ConfigParser()
    config.read(in_dir + "/../.config.ini")
    if "expected flux" in config and "order" in config["expected flux"]:
        return config["expected flux"].getint("order")
    userprint("WARNING: `order` not found; projection will fail if requested")
    return None


def read_delta_file(filename, z_min_qso=0, z_max_qso=10, rebin_factor=None,
                    order=None):
    """All deltas of one file (py/picca/io.py:333-380)."""
    hdul = fitsio.FITS(filename)
    if "LAMBDA" in hdul:
        deltas = Delta.from_image(hdul, z_min_qso=z_min_qso, z_max_qso=z_max_qso,
                                  order=order)
    else:
        deltas = [Delta.from_fitsio(hdu, order=order) for hdu in hdul[1:]
                  if z_min_qso < hdu.read_header()["Z"] < z_max_qso]
    if rebin_factor is not None:
        card = "LAMBDA" if "LAMBDA" in hdul else 1
        if hdul[card].read_header()["WAVE_SOLUTION"] != "lin":
            raise ValueError("Delta rebinning only implemented for linear lambda bins")
        dwave = hdul[card].read_header()["DELTA_LAMBDA"]
        for delta in deltas:
            delta.rebin(rebin_factor, dwave=dwave)
    return deltas


def read_deltas(in_dir, nside, lambda_abs, alpha, z_ref, cosmo,
                max_num_spec=None, no_project=False, nproc=None,
                rebin_factor=None, z_min_qso=0, z_max_qso=10,
                delta_attributes=None, native=True):
    """Read deltas, compute z, r_comov, dist_m, evolve weights and project.

    Same contract as py/picca/io.py:383-512: returns (data, num_data, z_min,
    z_max) with ``data = {healpix: [Delta, ...]}``. ``native`` (default)
    parses, rebins and projects the deltas in the native library and
    vectorised NumPy (``picca_gb300.deltaio``, bit-identical to the
    per-object readers below).
    """
    files = _list_delta_files(in_dir)
    order = find_order(in_dir, delta_attributes)
    if native:
        from ._native import NativeError, PG_ERR_UNSUPPORTED
        try:
            return _read_deltas_native(files, in_dir, nside, lambda_abs, alpha, z_ref, cosmo,
                                       max_num_spec, no_project, nproc, z_min_qso, z_max_qso,
                                       order, rebin_factor)
        except NativeError as err:
            if getattr(err, "status", None) != PG_ERR_UNSUPPORTED:
                raise
            # a layout the native parser leaves to the per-object readers
    deltas = []
    num_data = 0
    for filename in files:
        deltas += read_delta_file(filename, z_min_qso, z_max_qso, rebin_factor, order)
        num_data = len(deltas)
        if (max_num_spec is not None) and (num_data > max_num_spec):
            break
    if max_num_spec is not None:
        deltas = deltas[:max_num_spec]
        num_data = len(deltas)

    phi = [delta.ra for delta in deltas]
    theta = [np.pi / 2. - delta.dec for delta in deltas]
    healpixs = ang2pix_ring(nside, theta, phi)
    if np.size(healpixs) == 0:
        raise AssertionError(f"ERROR: No data in {in_dir}")

    data = {}
    z_min = 10**deltas[0].log_lambda[0] / lambda_abs - 1.
    z_max = 0.
    for delta, healpix in zip(deltas, np.atleast_1d(healpixs)):
        z = 10**delta.log_lambda / lambda_abs - 1.
        z_min = min(z_min, z.min())
        z_max = max(z_max, z.max())
        delta.z = z
        if cosmo is not None:
            delta.r_comov = cosmo.get_r_comov(z)
            delta.dist_m = cosmo.get_dist_m(z)
        delta.weights *= ((1 + z) / (1 + z_ref))**(alpha - 1)
        if not no_project:
            delta.project()
        data.setdefault(int(healpix), []).append(delta)
    return data, num_data, z_min, z_max


def read_drq(drq_filename, z_min=0, z_max=10., keep_bal=False, bi_max=None,
             mode="sdss"):
    """Quasar catalogue selection (py/picca/io.py:160-295).

    Returns a dict of numpy columns (RA/DEC converted to radians)."""
    hdul = fitsio.FITS(drq_filename)
    table = hdul[1]
    cols = {name: table[name][:] for name in table.get_colnames()}
    if "desi" in mode and "TARGETID" in cols:
        obj_id_name = "TARGETID"
        if "TARGET_RA" in cols:
            cols["RA"] = cols.pop("TARGET_RA")
            cols["DEC"] = cols.pop("TARGET_DEC")
    else:
        obj_id_name = "THING_ID"
    if "Z" not in cols:
        if "Z_VI" in cols:
            cols["Z"] = cols.pop("Z_VI")
        else:
            userprint("ERROR: No valid column for redshift found in ", drq_filename)
            return None
    w = np.ones(len(cols["RA"]), dtype=bool)
    w &= cols[obj_id_name] > 0
    w &= cols["RA"] != cols["DEC"]
    w &= cols["RA"] != 0.
    w &= cols["DEC"] != 0.
    w &= cols["Z"] >= z_min
    w &= cols["Z"] < z_max
    if not keep_bal and bi_max is None and "BAL_FLAG_VI" in cols:
        w &= cols["BAL_FLAG_VI"] == 0
    if bi_max is not None:
        if "BI_CIV" not in cols:
            raise SystemExit("ERROR: --bi-max set but no BI_CIV field in HDU")
        w &= cols["BI_CIV"] <= bi_max
    out = {key: np.asarray(val)[w] for key, val in cols.items()}
    out["RA"] = np.radians(out["RA"])
    out["DEC"] = np.radians(out["DEC"])
    out["_obj_id_name"] = obj_id_name
    return out


def _read_deltas_native(files, in_dir, nside, lambda_abs, alpha, z_ref, cosmo, max_num_spec,
                        no_project, nproc, z_min_qso, z_max_qso, order, rebin_factor=None):
    """read_deltas through the native parser and projection: the per-pixel
    expressions of the per-object path, evaluated once over all pixels."""
    from . import deltaio
    arrays = deltaio.read_files(files, z_min_qso, z_max_qso, max_num_spec,
                                threads=nproc if nproc else None, rebin_factor=rebin_factor)
    num_data = len(arrays["ra"])
    ra, dec = arrays["ra"], arrays["dec"]
    healpixs = ang2pix_ring(nside, np.pi / 2. - dec, ra)
    if np.size(healpixs) == 0:
        raise AssertionError(f"ERROR: No data in {in_dir}")
    log_lambda = arrays["log_lambda"]
    threads = nproc if nproc else None
    z = deltaio.per_pixel(lambda ll: 10**ll / lambda_abs - 1., [log_lambda], threads)
    z_min = 10**log_lambda[0] / lambda_abs - 1.
    z_max = 0.
    if z.size:
        z_min = min(z_min, z.min())
        z_max = max(z_max, z.max())
    arrays["z"] = z
    if cosmo is not None:
        arrays["r_comov"] = deltaio.per_pixel(cosmo.get_r_comov, [z], threads)
        arrays["dist_m"] = deltaio.per_pixel(cosmo.get_dist_m, [z], threads)
    arrays["weights"] = deltaio.per_pixel(
        lambda w, zz: w * ((1 + zz) / (1 + z_ref))**(alpha - 1), [arrays["weights"], z], threads)
    if not no_project:
        if order is None:
            raise RuntimeError(
                "Trying to project but order is not defined for the deltas. "
                "Check previous warning to solve this issue")
        deltaio.project(arrays["pix_offset"], log_lambda, arrays["weights"], arrays["delta"],
                        np.full(num_data, int(order), dtype=np.int32))
    data = {}
    for delta, healpix in zip(deltaio.make_deltas(arrays, order), np.atleast_1d(healpixs)):
        data.setdefault(int(healpix), []).append(delta)
    return data, num_data, z_min, z_max


def read_objects(filename, nside, z_min, z_max, alpha, z_ref, cosmo,
                 mode="sdss", keep_bal=True):
    """Quasar catalogue as ``{healpix: [QSO, ...]}`` with weights and
    distances (py/picca/io.py:515-614). Returns (objs, z_min_of_catalogue)."""
    catalog = read_drq(filename, z_min=z_min, z_max=z_max, keep_bal=keep_bal,
                       mode=mode)
    phi = catalog["RA"]
    theta = np.pi / 2. - catalog["DEC"]
    healpixs = np.atleast_1d(ang2pix_ring(nside, theta, phi))
    if healpixs.size == 0:
        raise AssertionError()
    objs = {}
    if "TARGETID" in catalog and catalog["_obj_id_name"] == "TARGETID":
        if mode == "desi_mocks":
            nightcol = "TARGETID"
        elif "LAST_NIGHT" in catalog:
            nightcol = "LAST_NIGHT"
        elif "NIGHT" in catalog:
            nightcol = "NIGHT"
        else:
            nightcol = "TARGETID"
        fibercol = "FIBER" if "FIBER" in catalog else "TARGETID"
        ident = ("TARGETID", "TARGETID", nightcol, fibercol)
    else:
        ident = ("THING_ID", "PLATE", "MJD", "FIBERID")
    for healpix in np.unique(healpixs):
        sel = np.where(healpixs == healpix)[0]
        objs[int(healpix)] = [
            QSO(catalog[ident[0]][i], catalog["RA"][i], catalog["DEC"][i],
                catalog["Z"][i], catalog[ident[1]][i], catalog[ident[2]][i],
                catalog[ident[3]][i]) for i in sel
        ]
        for obj in objs[int(healpix)]:
            obj.weights = ((1. + obj.z_qso) / (1. + z_ref))**(alpha - 1.)
            if cosmo is not None:
                obj.r_comov = cosmo.get_r_comov(obj.z_qso)
                obj.dist_m = cosmo.get_dist_m(obj.z_qso)
    return objs, catalog["Z"].min()
