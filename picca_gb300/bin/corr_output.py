"""Aggregation and FITS layout shared by the correlation CLIs.

Follows ``py/picca/bin/picca_cf.py:465-580`` (identical in
``py/picca/bin/picca_xcf.py:500-615``): weight-averaged RP/RT/Z over healpix,
summed NB, header keywords of ``ATTRI``, and per-healpix ``WE``/``DA`` rows
(``DA_BLIND`` when blinded) in ``COR``.
"""

import numpy as np

from picca_gb300 import fitsio_lite


def aggregate(result):
    """ATTRI columns from the per-healpix normalised rows."""
    weights_list = result["weights"]
    sum_weights = weights_list.sum(axis=0)
    w = sum_weights > 0
    r_par = (result["r_par"] * weights_list).sum(axis=0)
    r_par[w] /= sum_weights[w]
    r_trans = (result["r_trans"] * weights_list).sum(axis=0)
    r_trans[w] /= sum_weights[w]
    z = (result["z"] * weights_list).sum(axis=0)
    z[w] /= sum_weights[w]
    num_pairs = result["num_pairs"].astype(np.int64).sum(axis=0)
    return r_par, r_trans, z, num_pairs


def write(path, result, module, args, blinding):
    """Write the ATTRI and COR HDUs."""
    r_par, r_trans, z, num_pairs = aggregate(result)
    header = [
        {"name": "RPMIN", "value": module.r_par_min, "comment": "Minimum r-parallel [h^-1 Mpc]"},
        {"name": "RPMAX", "value": module.r_par_max, "comment": "Maximum r-parallel [h^-1 Mpc]"},
        {"name": "RTMAX", "value": module.r_trans_max,
         "comment": "Maximum r-transverse [h^-1 Mpc]"},
        {"name": "NP", "value": module.num_bins_r_par, "comment": "Number of bins in r-parallel"},
        {"name": "NT", "value": module.num_bins_r_trans,
         "comment": "Number of bins in r-transverse"},
        {"name": "ZMIN", "value": module.z_min_pairs, "comment": "Minimum redshift of pairs"},
        {"name": "ZMAX", "value": module.z_max_pairs, "comment": "Maximum redshift of pairs"},
        {"name": "NSIDE", "value": module.nside, "comment": "Healpix nside"},
        {"name": "OMEGAM", "value": args.fid_Om,
         "comment": "Omega_matter(z=0) of fiducial LambdaCDM cosmology"},
        {"name": "OMEGAR", "value": args.fid_Or,
         "comment": "Omega_radiation(z=0) of fiducial LambdaCDM cosmology"},
        {"name": "OMEGAK", "value": args.fid_Ok,
         "comment": "Omega_k(z=0) of fiducial LambdaCDM cosmology"},
        {"name": "WL", "value": args.fid_wl,
         "comment": "Equation of state of dark energy of fiducial LambdaCDM cosmology"},
        {"name": "BLINDING", "value": blinding,
         "comment": "String specifying the blinding strategy"},
        {"name": "RMU_BIN", "value": module.rmu_binning, "comment": "True if binned in r, mu"},
    ]
    attri = {
        "columns": [r_par, r_trans, z, num_pairs],
        "names": ["RP", "RT", "Z", "NB"],
        "comments": ["R-parallel" if not module.rmu_binning else "Mu",
                     "R-transverse" if not module.rmu_binning else "Radial separation",
                     "Redshift", "Number of pairs"],
        "units": ["h^-1 Mpc" if not module.rmu_binning else "", "h^-1 Mpc", "", ""],
        "header": header,
        "extname": "ATTRI",
    }
    da_name = "DA" if blinding == "none" else "DA_BLIND"
    cor = {
        "columns": [np.asarray(result["healpix_list"], dtype=np.int64), result["weights"],
                    result["xi"]],
        "names": ["HEALPID", "WE", da_name],
        "comments": ["Healpix index", "Sum of weight", "Correlation"],
        "header": [{"name": "HLPXSCHM", "value": "RING", "comment": "Healpix scheme"}],
        "extname": "COR",
    }
    fitsio_lite.write_fits(path, [attri, cor])
