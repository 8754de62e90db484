#!/usr/bin/env python3
"""Fast metal distortion matrices of the auto-correlation on the GPU.

Drop-in for ``py/picca/bin/picca_fast_metal_dmat.py``: the same flags, the
matrices computed from the STACK_DELTAS table of one or two delta-attributes
files (one matrix per absorber pair of ``--lambda-abs`` / ``--abs-igm`` and
``--lambda-abs2`` / ``--abs-igm2``), and the same FITS layout (HDU ``ATTRI``
with ABS_IGM and the header keywords, HDU ``MDMAT`` with RP_ / RT_ / Z_ /
DM_ (DM_BLIND_ when blinded) columns per pair). r_par is folded (the
reference sets x_correlation False whatever --unfold-cf says).
"""

import argparse
import os
import sys
import time

import numpy as np

from picca_gb300 import constants, fast_metal, fitsio_lite, io
from picca_gb300.utils import userprint


def parse_args(cmdargs=None):
    parser = argparse.ArgumentParser(
        formatter_class=argparse.ArgumentDefaultsHelpFormatter,
        description="Compute the fast metal distortion matrices of the auto-correlation from "
                    "the stacked deltas")
    parser.add_argument("--out", type=str, default=None, required=True, help="Output file name")
    parser.add_argument("-i", "--in-attributes", type=str, default=None, required=True,
                        help="Path to delta_attributes.fits.gz file with hdu STACK_DELTAS "
                             'containing table with at least rows "LOGLAM" and "WEIGHT"')
    parser.add_argument("--in-attributes2", type=str, default=None,
                        help="Path to 2nd delta_attributes.fits.gz file")
    parser.add_argument("--delta-dir", type=str, default=None,
                        help="Path to directory with delta*.gz to get the blinding info "
                             "(default is trying to guess from attributes file)")
    parser.add_argument("--rp-min", type=float, default=0.0, help="Min r-parallel [h^-1 Mpc]")
    parser.add_argument("--rp-max", type=float, default=200.0, help="Max r-parallel [h^-1 Mpc]")
    parser.add_argument("--rt-max", type=float, default=200.0, help="Max r-transverse [h^-1 Mpc]")
    parser.add_argument("--np", type=int, default=50, help="Number of r-parallel bins")
    parser.add_argument("--nt", type=int, default=50, help="Number of r-transverse bins")
    parser.add_argument("--coef-binning-model", type=int, default=1,
                        help="Coefficient multiplying np and nt to get finner binning for the "
                             "model")
    parser.add_argument("--z-min-sources", type=float, default=0.0,
                        help="Limit the minimum redshift of the quasars used as sources")
    parser.add_argument("--z-max-sources", type=float, default=10.0,
                        help="Limit the maximum redshift of the quasars used as sources")
    parser.add_argument("--lambda-abs", type=str, default="LYA",
                        help="Name of the absorption in picca.constants defining the redshift "
                             "of the delta")
    parser.add_argument("--lambda-abs2", type=str, default=None,
                        help="Name of the absorption in picca.constants defining the redshift "
                             "of the 2nd delta")
    parser.add_argument("--abs-igm", type=str, default=[], required=True, nargs="*",
                        help="List of names of metal absorption in picca.constants present in "
                             "forest")
    parser.add_argument("--abs-igm2", type=str, default=[], nargs="*",
                        help="List of names of metal absorption in picca.constants present in "
                             "2nd forest")
    parser.add_argument("--z-ref", type=float, default=2.25, help="Reference redshift")
    parser.add_argument("--z-evol", type=float, default=2.9,
                        help="Exponent of the redshift evolution of the delta field")
    parser.add_argument("--z-evol2", type=float, default=2.9,
                        help="Exponent of the redshift evolution of the 2nd delta field")
    parser.add_argument("--metal-alpha", type=float, default=1.0,
                        help="Exponent of the redshift evolution of the metal delta field")
    parser.add_argument("--fid-Om", type=float, default=0.315,
                        help="Omega_matter(z=0) of fiducial LambdaCDM cosmology")
    parser.add_argument("--fid-Or", type=float, default=0.0,
                        help="Omega_radiation(z=0) of fiducial LambdaCDM cosmology")
    parser.add_argument("--fid-Ok", type=float, default=0.0,
                        help="Omega_k(z=0) of fiducial LambdaCDM cosmology")
    parser.add_argument("--fid-wl", type=float, default=-1.0,
                        help="Equation of state of dark energy of fiducial LambdaCDM cosmology")
    parser.add_argument("--unfold-cf", action="store_true",
                        help="rp can be positive or negative depending on the relative "
                             "position between absorber1 and absorber2")
    parser.add_argument("--rebin-factor", type=int, default=None,
                        help="Rebin factor for deltas. If not None, deltas will be rebinned by "
                             "that factor")
    parser.add_argument("--relevant-metals", action="store_true",
                        help="compute only the metal correlations used by Vega i.e. 4 LyaxSi "
                             "matrices and CIVxCIV")
    return parser.parse_args(cmdargs)


def read_stack(path):
    """STACK_DELTAS table of a delta-attributes file."""
    hdu = fitsio_lite.FITS(path)["STACK_DELTAS"]
    return {"LOGLAM": np.asarray(hdu["LOGLAM"][:], dtype=np.float64),
            "WEIGHT": np.asarray(hdu["WEIGHT"][:], dtype=np.float64)}


def guess_delta_dir(args):
    if args.delta_dir is None:
        args.delta_dir = os.path.dirname(args.in_attributes) + "/../Delta/"
        if not os.path.isdir(args.delta_dir):
            userprint("Tried to guess the delta directory (containing the delta*.gz files) "
                      f"but '{args.delta_dir}' is not valid")
            userprint("Please specify the directory with option --delta-dir")
            sys.exit(1)
    return args.delta_dir


def header_cards(args, num_bins_r_par, num_bins_r_trans, blinding, cross=False):
    """ATTRI keywords of picca_fast_metal_dmat.py / picca_fast_metal_xdmat.py."""
    cards = [
        {"name": "RPMIN", "value": args.rp_min, "comment": "Minimum r-parallel [h^-1 Mpc]"},
        {"name": "RPMAX", "value": args.rp_max, "comment": "Maximum r-parallel [h^-1 Mpc]"},
        {"name": "RTMAX", "value": args.rt_max, "comment": "Maximum r-transverse [h^-1 Mpc]"},
        {"name": "NP", "value": num_bins_r_par, "comment": "Number of bins in r-parallel"},
        {"name": "NT", "value": num_bins_r_trans, "comment": " Number of bins in r-transverse"},
        {"name": "COEFMOD", "value": args.coef_binning_model,
         "comment": "Coefficient for model binning"},
    ]
    if not cross:
        cards += [{"name": "REJ", "value": None, "comment": "Rejection factor"},
                  {"name": "ALPHAMET", "value": args.metal_alpha,
                   "comment": "Evolution of metal bias"}]
    cards += [
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
    return cards


def write(path, names, results, header, blinding, prefix=""):
    """ATTRI (ABS_IGM) and MDMAT (RP_ / RT_ / Z_ / DM_ per name)."""
    attri = {"columns": [np.array(names, dtype="S" + str(max(len(n) for n in names)))],
             "names": ["ABS_IGM"], "comments": ["Absorption name"], "header": header,
             "extname": "ATTRI"}
    dm_prefix = "DM_" if blinding == "none" else "DM_BLIND_"
    cols, col_names, comments, units = [], [], [], []
    for name, (dmat, r_par, r_trans, z) in zip(names, results):
        for value, key, comment, unit in ((r_par, "RP_", "R-parallel", "h^-1 Mpc"),
                                          (r_trans, "RT_", "R-transverse", "h^-1 Mpc"),
                                          (z, "Z_", "Redshift", ""),
                                          (dmat, dm_prefix, "Distortion matrix", "")):
            cols.append(value)
            col_names.append(key + prefix + name)
            comments.append(comment)
            units.append(unit)
    fitsio_lite.write_fits(path, [attri, {"columns": cols, "names": col_names,
                                          "comments": comments, "units": units,
                                          "extname": "MDMAT"}])


def main(cmdargs=None):
    """Compute the fast metal distortion matrices of the auto-correlation"""
    args = parse_args(cmdargs)
    num_bins_r_par = args.np * args.coef_binning_model
    num_bins_r_trans = args.nt * args.coef_binning_model
    alpha_abs = {args.lambda_abs: args.z_evol}
    for name in args.abs_igm:
        alpha_abs[name] = args.metal_alpha
    blinding = io.read_blinding(guess_delta_dir(args))
    cosmo = constants.Cosmo(Om=args.fid_Om, Or=args.fid_Or, Ok=args.fid_Ok, wl=args.fid_wl,
                            verbose=False)
    t0 = time.time()
    stack1 = read_stack(args.in_attributes)
    stack2 = read_stack(args.in_attributes2) if args.in_attributes2 is not None else stack1
    t1 = time.time()
    userprint(f"picca_fast_metal_dmat.py - Time reading data: {(t1 - t0) / 60:.3f} minutes")
    if args.lambda_abs2 is None:
        args.lambda_abs2 = args.lambda_abs
        args.abs_igm2 = args.abs_igm
    lam_out1 = constants.ABSORBER_IGM[args.lambda_abs]
    lam_out2 = constants.ABSORBER_IGM[args.lambda_abs2]
    engine = fast_metal.FastMetalEngine()
    names, results = [], []
    for abs1, abs2 in fast_metal.absorber_pairs(args.lambda_abs, args.abs_igm, args.lambda_abs2,
                                                args.abs_igm2, relevant=args.relevant_metals):
        userprint("Computing", abs1, abs2)
        side1 = fast_metal.stack_side(stack1["LOGLAM"], stack1["WEIGHT"],
                                      constants.ABSORBER_IGM[abs1], lam_out1,
                                      alpha_abs[abs1] + args.z_evol, cosmo, args.rebin_factor)
        side2 = fast_metal.stack_side(stack2["LOGLAM"], stack2["WEIGHT"],
                                      constants.ABSORBER_IGM[abs2], lam_out2,
                                      alpha_abs[abs2] + args.z_evol2, cosmo, args.rebin_factor)
        results.append(fast_metal.fast_metal_matrix(
            side1, side2, args.rp_min, args.rp_max, args.rt_max, num_bins_r_par,
            num_bins_r_trans, signed=False, engine=engine))
        names.append(abs1 + "_" + abs2)
    t2 = time.time()
    userprint(f"picca_fast_metal_dmat.py - Time computing all metal matrices : "
              f"{(t2 - t1) / 60:.3f} minutes")
    write(args.out, names, results,
          header_cards(args, num_bins_r_par, num_bins_r_trans, blinding), blinding)
    userprint(f"picca_fast_metal_dmat.py - Time total : {(time.time() - t0) / 60:.3f} minutes")
    return dict(zip(names, results))


if __name__ == "__main__":
    main(sys.argv[1:])
