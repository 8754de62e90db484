#!/usr/bin/env python3
"""Metal distortion matrices of the delta x quasar cross-correlation on the GPU.

Drop-in for ``py/picca/bin/picca_metal_xdmat.py``: the same flags, module
globals (alpha_abs of the tracer and the metals), readers, one matrix per
absorber of ``--abs-igm`` with the random rejection per process chunk (a
forest without a pixel below its quasar redshift draws nothing,
py/picca/xcf.py:713-727), normalisation and FITS layout (HDU ``ATTRI`` with
NPALL / NPUSED / ABS_IGM and the header keywords, HDU ``MDMAT`` with
RP_QSO_ / RT_QSO_ / Z_QSO_ / DM_QSO_ / WDM_QSO_ columns per absorber).
"""

import argparse
import sys
import time
from multiprocessing import cpu_count

import numpy as np

from picca_gb300 import constants, fitsio_lite, io, metal, pairs, utils, xcf
from picca_gb300.forests import ForestSet
from picca_gb300.utils import userprint


def parse_args(cmdargs=None):
    parser = argparse.ArgumentParser(
        formatter_class=argparse.ArgumentDefaultsHelpFormatter,
        description="Compute the metal distortion matrices of the cross-correlation delta x "
                    "object")
    parser.add_argument("--out", type=str, default=None, required=True, help="Output file name")
    parser.add_argument("--in-dir", type=str, default=None, required=True,
                        help="Directory to delta files")
    parser.add_argument("--drq", type=str, default=None, required=True,
                        help="Catalog of objects in format selected by mode")
    parser.add_argument("--mode", type=str, default="sdss",
                        choices=["sdss", "desi", "desi_mocks", "desi_healpix"],
                        help="Mode for reading the catalog")
    parser.add_argument("--rp-min", type=float, default=-200.0,
                        help="Min r-parallel [h^-1 Mpc]")
    parser.add_argument("--rp-max", type=float, default=200.0, help="Max r-parallel [h^-1 Mpc]")
    parser.add_argument("--rt-max", type=float, default=200.0, help="Max r-transverse [h^-1 Mpc]")
    parser.add_argument("--np", type=int, default=100, help="Number of r-parallel bins")
    parser.add_argument("--nt", type=int, default=50, help="Number of r-transverse bins")
    parser.add_argument("--coef-binning-model", type=int, default=1,
                        help="Coefficient multiplying np and nt to get finner binning for the "
                             "model")
    parser.add_argument("--z-min-obj", type=float, default=0, help="Min redshift for object field")
    parser.add_argument("--z-max-obj", type=float, default=10,
                        help="Max redshift for object field")
    parser.add_argument("--z-min-sources", type=float, default=0.0,
                        help="Limit the minimum redshift of the quasars used as sources")
    parser.add_argument("--z-max-sources", type=float, default=10.0,
                        help="Limit the maximum redshift of the quasars used as sources")
    parser.add_argument("--lambda-abs", type=str, default="LYA",
                        help="Name of the absorption in picca.constants")
    parser.add_argument("--abs-igm", type=str, default=[], nargs="*",
                        help="List of names of metal absorption in picca.constants")
    parser.add_argument("--z-ref", type=float, default=2.25, help="Reference redshift")
    parser.add_argument("--z-evol-del", type=float, default=2.9,
                        help="Exponent of the redshift evolution of the delta field")
    parser.add_argument("--z-evol-obj", type=float, default=1.44,
                        help="Exponent of the redshift evolution of the object field")
    parser.add_argument("--metal-alpha", type=float, default=1.0,
                        help="Exponent of the redshift evolution of the metal delta field")
    parser.add_argument("--fid-Om", type=float, default=0.315, help="Omega_matter(z=0)")
    parser.add_argument("--fid-Or", type=float, default=0.0, help="Omega_radiation(z=0)")
    parser.add_argument("--fid-Ok", type=float, default=0.0, help="Omega_k(z=0)")
    parser.add_argument("--fid-wl", type=float, default=-1.0,
                        help="Equation of state of dark energy")
    parser.add_argument("--rej", type=float, default=1.0,
                        help="Fraction of rejected object-forests pairs: -1=no rejection, "
                             "1=all rejection")
    parser.add_argument("--nside", type=int, default=16, help="Healpix nside")
    parser.add_argument("--nproc", type=int, default=None,
                        help="Number of processes of the reference run to reproduce (sets the "
                             "chunking of the random rejection)")
    parser.add_argument("--nspec", type=int, default=None,
                        help="Maximum number of spectra to read")
    parser.add_argument("--rebin-factor", type=int, default=None,
                        help="Rebin factor for deltas")
    parser.add_argument("--in-attributes", type=str, default=None,
                        help="Delta attributes file (continuum-fit order for the projection)")
    return parser.parse_args(cmdargs)


def header_cards(args, blinding):
    """ATTRI keywords of picca_metal_xdmat.py."""
    return [
        {"name": "RPMIN", "value": xcf.r_par_min, "comment": "Minimum r-parallel [h^-1 Mpc]"},
        {"name": "RPMAX", "value": xcf.r_par_max, "comment": "Maximum r-parallel [h^-1 Mpc]"},
        {"name": "RTMAX", "value": xcf.r_trans_max,
         "comment": "Maximum r-transverse [h^-1 Mpc]"},
        {"name": "NP", "value": xcf.num_bins_r_par, "comment": "Number of bins in r-parallel"},
        {"name": "NT", "value": xcf.num_bins_r_trans,
         "comment": "Number of bins in r-transverse"},
        {"name": "COEFMOD", "value": args.coef_binning_model,
         "comment": "Coefficient for model binning"},
        {"name": "REJ", "value": xcf.reject, "comment": "Rejection factor"},
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
    ]


def write(path, results, args, blinding):
    names = list(results)
    attri = {
        "columns": [np.array([results[n]["NPALL"] for n in names], dtype=np.int64),
                    np.array([results[n]["NPUSED"] for n in names], dtype=np.int64),
                    np.array(names, dtype="S" + str(max(len(n) for n in names)))],
        "names": ["NPALL", "NPUSED", "ABS_IGM"],
        "comments": ["Number of pairs", "Number of used pairs", "Absorption name"],
        "header": header_cards(args, blinding),
        "extname": "ATTRI",
    }
    dm_prefix = "DM_" if blinding == "none" else "DM_BLIND_"
    cols, col_names, comments, units = [], [], [], []
    for name in names:
        r = results[name]
        for key, prefix, comment, unit in (("RP", "RP_", "R-parallel", "h^-1 Mpc"),
                                           ("RT", "RT_", "R-transverse", "h^-1 Mpc"),
                                           ("Z", "Z_", "Redshift", ""),
                                           ("DM", dm_prefix, "Distortion matrix", ""),
                                           ("WDM", "WDM_", "Sum of weight", "")):
            cols.append(r[key])
            col_names.append(prefix + "QSO_" + name)
            comments.append(comment)
            units.append(unit)
    fitsio_lite.write_fits(path, [attri, {"columns": cols, "names": col_names,
                                          "comments": comments, "units": units,
                                          "extname": "MDMAT"}])


def main(cmdargs=None):
    """Compute the metal distortion matrices of the cross-correlation"""
    args = parse_args(cmdargs)
    if args.nproc is None:
        args.nproc = max(cpu_count() // 2, 1)
    xcf.r_par_max, xcf.r_par_min, xcf.r_trans_max = args.rp_max, args.rp_min, args.rt_max
    xcf.num_bins_r_par, xcf.num_bins_r_trans = args.np, args.nt
    xcf.num_model_bins_r_par = args.np * args.coef_binning_model
    xcf.num_model_bins_r_trans = args.nt * args.coef_binning_model
    xcf.nside = args.nside
    xcf.z_ref = args.z_ref
    xcf.alpha = args.z_evol_del
    xcf.alpha_obj = args.z_evol_obj
    xcf.reject = args.rej
    xcf.lambda_abs = constants.ABSORBER_IGM[args.lambda_abs]
    xcf.alpha_abs = {args.lambda_abs: args.z_evol_del}
    for name in args.abs_igm:
        xcf.alpha_abs[name] = args.metal_alpha
    blinding = io.read_blinding(args.in_dir)
    xcf.cosmo = constants.Cosmo(Om=args.fid_Om, Or=args.fid_Or, Ok=args.fid_Ok,
                                wl=args.fid_wl, verbose=False)
    t0 = time.time()
    data, num_data, z_min, _ = io.read_deltas(
        args.in_dir, args.nside, xcf.lambda_abs, args.z_evol_del, xcf.z_ref, cosmo=xcf.cosmo,
        max_num_spec=args.nspec, rebin_factor=args.rebin_factor,
        z_min_qso=args.z_min_sources, z_max_qso=args.z_max_sources,
        delta_attributes=args.in_attributes)
    xcf.data = data
    xcf.num_data = num_data
    objs, z_min2 = io.read_objects(args.drq, args.nside, args.z_min_obj, args.z_max_obj,
                                   args.z_evol_obj, xcf.z_ref, xcf.cosmo, mode=args.mode)
    xcf.objs = objs
    xcf.ang_max = utils.compute_ang_max(xcf.cosmo, xcf.r_trans_max, z_min, z_min2)
    userprint(f"done, npix = {len(data)}")
    t1 = time.time()
    fs, qs = ForestSet.from_deltas(data), ForestSet.from_objects(objs)
    params = pairs.make_params(xcf.r_par_min, xcf.r_par_max, xcf.r_trans_max,
                               xcf.num_bins_r_par, xcf.num_bins_r_trans, xcf.ang_max,
                               x_correlation=True)
    dparams = metal._dmat.make_dmat_params(xcf.num_bins_r_par, xcf.num_bins_r_trans,
                                           coef_binning_model=args.coef_binning_model)
    results = metal.cross_metal_distortion_matrices(fs, qs, params, dparams, xcf.cosmo,
                                                    xcf.reject, args.abs_igm, xcf.alpha_abs,
                                                    z_ref=xcf.z_ref, nproc=args.nproc)
    userprint(f"picca_metal_xdmat.py - Time computing all metal matrix: "
              f"{(time.time() - t1) / 60:.3f} minutes")
    write(args.out, results, args, blinding)
    userprint(f"picca_metal_xdmat.py - Time total : {(time.time() - t0) / 60:.3f} minutes")
    return results


if __name__ == "__main__":
    main(sys.argv[1:])
