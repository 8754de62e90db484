#!/usr/bin/env python3
"""Metal distortion matrices of the auto-correlation on the GPU.

Drop-in for ``py/picca/bin/picca_metal_dmat.py`` (auto-correlation of one
delta field): the same flags (:60-334), module globals (:336-352), reader,
list of absorber pairs (:446-470, including ``--fast-metals``), random
rejection per process chunk (the generator re-seeded per chunk for every
absorber pair, so all pairs keep the same forest pairs), normalisation
(:497-503) and FITS layout (HDU ``ATTRI`` with NPALL / NPUSED / ABS_IGM and
the header keywords, HDU ``MDMAT`` with RP_ / RT_ / Z_ / DM_ / WDM_ columns per
absorber pair). A second delta field (``--in-dir2``) and a second tracer
(``--lambda-abs2``, with its absorbers ``--abs-igm2``) are read as the
reference does (py/picca/bin/picca_metal_dmat.py:389-421).
"""

import argparse
import sys
import time
from multiprocessing import cpu_count

import numpy as np

from picca_gb300 import cf, constants, fitsio_lite, io, metal, pairs, utils
from picca_gb300.utils import userprint

DEFAULT_SI_METALS = ["SiIII(1207)", "SiII(1190)", "SiII(1193)", "SiII(1260)"]


def parse_args(cmdargs=None):
    parser = argparse.ArgumentParser(
        formatter_class=argparse.ArgumentDefaultsHelpFormatter,
        description="Compute the metal distortion matrices of the auto-correlation")
    parser.add_argument("--out", type=str, default=None, required=True, help="Output file name")
    parser.add_argument("--in-dir", type=str, default=None, required=True,
                        help="Directory to delta files")
    parser.add_argument("--in-dir2", type=str, default=None, help="Directory to 2nd delta files")
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
                        help="Name of the absorption in picca.constants")
    parser.add_argument("--lambda-abs2", type=str, default=None,
                        help="Name of the absorption of the 2nd delta")
    parser.add_argument("--abs-igm", type=str, default=[], nargs="*",
                        help="List of names of metal absorption in picca.constants")
    parser.add_argument("--abs-igm2", type=str, default=[], nargs="*",
                        help="List of names of metal absorption of the 2nd delta")
    parser.add_argument("--z-ref", type=float, default=2.25, help="Reference redshift")
    parser.add_argument("--z-evol", type=float, default=2.9,
                        help="Exponent of the redshift evolution of the delta field")
    parser.add_argument("--z-evol2", type=float, default=2.9,
                        help="Exponent of the redshift evolution of the 2nd delta field")
    parser.add_argument("--metal-alpha", type=float, default=1.0,
                        help="Exponent of the redshift evolution of the metal delta field")
    parser.add_argument("--fid-Om", type=float, default=0.315, help="Omega_matter(z=0)")
    parser.add_argument("--fid-Or", type=float, default=0.0, help="Omega_radiation(z=0)")
    parser.add_argument("--fid-Ok", type=float, default=0.0, help="Omega_k(z=0)")
    parser.add_argument("--fid-wl", type=float, default=-1.0,
                        help="Equation of state of dark energy")
    parser.add_argument("--remove-same-half-plate-close-pairs", action="store_true",
                        help="Reject pairs in the first bin in r-parallel from same half plate")
    parser.add_argument("--rej", type=float, default=1.0,
                        help="Fraction of rejected forest-forest pairs: -1=no rejection, "
                             "1=all rejection")
    parser.add_argument("--nside", type=int, default=16, help="Healpix nside")
    parser.add_argument("--nproc", type=int, default=None,
                        help="Number of processes of the reference run to reproduce (sets the "
                             "chunking of the random rejection)")
    parser.add_argument("--nspec", type=int, default=None,
                        help="Maximum number of spectra to read")
    parser.add_argument("--unfold-cf", action="store_true",
                        help="rp can be positive or negative depending on the relative position")
    parser.add_argument("--rebin-factor", type=int, default=None,
                        help="Rebin factor for deltas")
    parser.add_argument("--fast-metals", action="store_true",
                        help="Compute only the LYA x Si and CIV(eff) x CIV(eff) matrices")
    parser.add_argument("--in-attributes", type=str, default=None,
                        help="Delta attributes file (continuum-fit order for the projection)")
    return parser.parse_args(cmdargs)


def header_cards(args, blinding):
    """ATTRI keywords (py/picca/bin/picca_metal_dmat.py:522-583)."""
    return [
        {"name": "RPMIN", "value": cf.r_par_min, "comment": "Minimum r-parallel [h^-1 Mpc]"},
        {"name": "RPMAX", "value": cf.r_par_max, "comment": "Maximum r-parallel [h^-1 Mpc]"},
        {"name": "RTMAX", "value": cf.r_trans_max, "comment": "Maximum r-transverse [h^-1 Mpc]"},
        {"name": "NP", "value": cf.num_bins_r_par, "comment": "Number of bins in r-parallel"},
        {"name": "NT", "value": cf.num_bins_r_trans, "comment": " Number of bins in r-transverse"},
        {"name": "COEFMOD", "value": args.coef_binning_model,
         "comment": "Coefficient for model binning"},
        {"name": "REJ", "value": cf.reject, "comment": "Rejection factor"},
        {"name": "ALPHAMET", "value": args.metal_alpha, "comment": "Evolution of metal bias"},
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
            col_names.append(prefix + name)
            comments.append(comment)
            units.append(unit)
    mdmat = {"columns": cols, "names": col_names, "comments": comments, "units": units,
             "extname": "MDMAT"}
    fitsio_lite.write_fits(path, [attri, mdmat])


def main(cmdargs=None):
    """Compute the metal distortion matrices"""
    args = parse_args(cmdargs)
    if args.nproc is None:
        args.nproc = max(cpu_count() // 2, 1)
    cf.r_par_max, cf.r_par_min, cf.r_trans_max = args.rp_max, args.rp_min, args.rt_max
    cf.num_bins_r_par, cf.num_bins_r_trans = args.np, args.nt
    cf.num_model_bins_r_par = args.np * args.coef_binning_model
    cf.num_model_bins_r_trans = args.nt * args.coef_binning_model
    cf.nside = args.nside
    cf.z_ref = args.z_ref
    cf.alpha = args.z_evol
    cf.reject = args.rej
    cf.lambda_abs = constants.ABSORBER_IGM[args.lambda_abs]
    cf.remove_same_half_plate_close_pairs = args.remove_same_half_plate_close_pairs
    # picca sets x_correlation only for a second field or tracer
    # (py/picca/bin/picca_metal_dmat.py:389-401)
    two_fields = bool(args.in_dir2 or args.lambda_abs2)
    cf.x_correlation = bool(two_fields and (args.lambda_abs2 or args.unfold_cf))
    cf.alpha_abs = {args.lambda_abs: cf.alpha}
    for name in args.abs_igm:
        cf.alpha_abs[name] = args.metal_alpha
    if two_fields:
        cf.alpha2 = args.z_evol2
        if args.in_dir2 is None:
            args.in_dir2 = args.in_dir
        cf.lambda_abs2 = (constants.ABSORBER_IGM[args.lambda_abs2] if args.lambda_abs2
                          else cf.lambda_abs)
        # without --lambda-abs2 picca stores alpha2 under the key None, so the
        # tracer keeps alpha (py/picca/bin/picca_metal_dmat.py:399)
        cf.alpha_abs[args.lambda_abs2] = cf.alpha2
        for name in args.abs_igm2:
            cf.alpha_abs[name] = args.metal_alpha
    blinding = io.read_blinding(args.in_dir)
    cf.cosmo = constants.Cosmo(Om=args.fid_Om, Or=args.fid_Or, Ok=args.fid_Ok, wl=args.fid_wl,
                               verbose=False)
    t0 = time.time()
    data, num_data, z_min, _ = io.read_deltas(
        args.in_dir, cf.nside, cf.lambda_abs, cf.alpha, cf.z_ref, cf.cosmo,
        max_num_spec=args.nspec, rebin_factor=args.rebin_factor,
        z_min_qso=args.z_min_sources, z_max_qso=args.z_max_sources,
        delta_attributes=args.in_attributes)
    cf.data = data
    cf.num_data = num_data
    cf.ang_max = utils.compute_ang_max(cf.cosmo, cf.r_trans_max, z_min)
    userprint(f"done, npix = {len(data)}")
    from picca_gb300.forests import ForestSet
    fs2 = None
    if args.in_dir2:
        data2, num_data2, z_min2, _ = io.read_deltas(
            args.in_dir2, cf.nside, cf.lambda_abs2, cf.alpha2, cf.z_ref, cf.cosmo,
            max_num_spec=args.nspec, rebin_factor=args.rebin_factor,
            z_min_qso=args.z_min_sources, z_max_qso=args.z_max_sources,
            delta_attributes=args.in_attributes)
        cf.data2 = data2
        cf.num_data2 = num_data2
        cf.ang_max = utils.compute_ang_max(cf.cosmo, cf.r_trans_max, z_min, z_min2)
        fs2 = ForestSet.from_deltas(data2)
    lambda_abs2 = args.lambda_abs2
    if args.lambda_abs2 is None:
        # the second list is then the first one (py/picca/bin/picca_metal_dmat.py:449-451)
        args.lambda_abs2 = args.lambda_abs
        args.abs_igm2 = args.abs_igm
    t1 = time.time()
    fs = ForestSet.from_deltas(data)
    params = pairs.make_params(cf.r_par_min, cf.r_par_max, cf.r_trans_max, cf.num_bins_r_par,
                               cf.num_bins_r_trans, cf.ang_max,
                               x_correlation=cf.x_correlation,
                               remove_same_half_plate_close_pairs=(
                                   cf.remove_same_half_plate_close_pairs))
    dparams = metal._dmat.make_dmat_params(cf.num_bins_r_par, cf.num_bins_r_trans,
                                           coef_binning_model=args.coef_binning_model)
    only = None
    if args.fast_metals:
        only = [(a1, a2) for a1, a2 in metal.absorber_pairs(args.lambda_abs, args.abs_igm,
                                                            args.lambda_abs2, args.abs_igm2)
                if (a1 == "LYA" and a2 in DEFAULT_SI_METALS) or (a1 == "CIV(eff)" and a1 == a2)]
    results = metal.metal_distortion_matrices(
        fs, params, dparams, cf.cosmo, cf.reject, args.abs_igm, cf.alpha_abs,
        lambda_abs=args.lambda_abs, z_ref=cf.z_ref, nproc=args.nproc, only=only, fs2=fs2,
        abs_igm2=args.abs_igm2 if fs2 is not None else None, lambda_abs2=lambda_abs2)
    userprint(f"picca_metal_dmat.py - Time computing all metal matrices : "
              f"{(time.time() - t1) / 60:.3f} minutes")
    write(args.out, results, args, blinding)
    userprint(f"picca_metal_dmat.py - Time total : {(time.time() - t0) / 60:.3f} minutes")
    return results


if __name__ == "__main__":
    main(sys.argv[1:])
