#!/usr/bin/env python3
"""Distortion matrix of the auto-correlation on the GPU.

Drop-in for ``py/picca/bin/picca_dmat.py``: the same flags (:41-345), module
globals (:347-398), readers (:410-465), random rejection per process chunk
(:466-485 with ``calc_dmat`` :21-38: healpix dealt by index % nproc, NumPy's
generator seeded with each chunk's first healpix), normalisation (:487-525)
and FITS layout (:527-640: HDU ``DMAT`` with WDM/DM and the header keywords,
HDU ``ATTRI`` with RP/RT/Z). ``--nproc`` only sets the chunking of the random
draws (the default, as in the reference, is half the host's cores); every
selected forest pair runs in one GPU launch.
"""

import argparse
import sys
import time
from multiprocessing import cpu_count

from picca_gb300 import cf, constants, fitsio_lite, io, utils
from picca_gb300.utils import userprint


def parse_args(cmdargs=None):
    parser = argparse.ArgumentParser(
        formatter_class=argparse.ArgumentDefaultsHelpFormatter,
        description="Compute the distortion matrix between two delta fields")
    parser.add_argument("--out", type=str, default=None, required=True, help="Output file name")
    parser.add_argument("--in-dir", type=str, default=None, required=True,
                        help="Directory to delta files")
    parser.add_argument("--in-dir2", type=str, default=None, required=False,
                        help="Directory to 2nd delta files")
    parser.add_argument("--rp-min", type=float, default=0.0, help="Min r-parallel [h^-1 Mpc]")
    parser.add_argument("--rp-max", type=float, default=200.0, help="Max r-parallel [h^-1 Mpc]")
    parser.add_argument("--rt-max", type=float, default=200.0, help="Max r-transverse [h^-1 Mpc]")
    parser.add_argument("--np", type=int, default=50, help="Number of r-parallel bins")
    parser.add_argument("--nt", type=int, default=50, help="Number of r-transverse bins")
    parser.add_argument("--rmu-binning", action="store_true",
                        help="Estimate in r,mu binning. np becomes mu bins. nt becomes r bins. "
                             "rp min max is always 0, 1")
    parser.add_argument("--coef-binning-model", type=int, default=1,
                        help="Coefficient multiplying np and nt to get finner binning for the "
                             "model")
    parser.add_argument("--zerr-cut-deg", type=float, default=None,
                        help="Angular cut (deg) between a pixel and the other background quasar")
    parser.add_argument("--zerr-cut-kms", type=float, default=None,
                        help="Velocity cut (km/s) between a pixel and the other background quasar")
    parser.add_argument("--z-min-sources", type=float, default=0.0,
                        help="Limit the minimum redshift of the quasars used as sources")
    parser.add_argument("--z-max-sources", type=float, default=10.0,
                        help="Limit the maximum redshift of the quasars used as sources")
    parser.add_argument("--z-min-pairs", type=float, default=None,
                        help="Limit the minimum redshift of the absorber pairs")
    parser.add_argument("--z-max-pairs", type=float, default=None,
                        help="Limit the maximum redshift of the absorber pairs")
    parser.add_argument("--lambda-abs", type=str, default="LYA",
                        help="Name of the absorption in picca.constants")
    parser.add_argument("--lambda-abs2", type=str, default=None,
                        help="Name of the absorption of the 2nd delta")
    parser.add_argument("--z-evol", type=float, default=2.9,
                        help="Exponent of the redshift evolution of the delta field")
    parser.add_argument("--z-evol2", type=float, default=2.9,
                        help="Exponent of the redshift evolution of the 2nd delta field")
    parser.add_argument("--fid-Om", type=float, default=0.315, help="Omega_matter(z=0)")
    parser.add_argument("--fid-Or", type=float, default=0.0, help="Omega_radiation(z=0)")
    parser.add_argument("--fid-Ok", type=float, default=0.0, help="Omega_k(z=0)")
    parser.add_argument("--fid-wl", type=float, default=-1.0,
                        help="Equation of state of dark energy")
    parser.add_argument("--distance-template", type=str, required=False,
                        help="Template cosmology (CAMB; not supported here)")
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
    parser.add_argument("--in-attributes", type=str, default=None,
                        help="Delta attributes file (continuum-fit order for the projection)")
    parser.add_argument("--no-redshift-evolution", action="store_true",
                        help="Ignore redshift evolution when computing distortion matrix")
    return parser.parse_args(cmdargs)


def header_cards(args, num_pairs, num_pairs_used, blinding, module=cf):
    """Keywords of the DMAT HDU (py/picca/bin/picca_dmat.py:527-610 and
    py/picca/bin/picca_xdmat.py, from the module globals of ``module``; the
    references list NPUSED, OMEGAM and OMEGAR twice, one card each)."""
    return [
        {"name": "RPMIN", "value": module.r_par_min, "comment": "Minimum r-parallel [h^-1 Mpc]"},
        {"name": "RPMAX", "value": module.r_par_max, "comment": "Maximum r-parallel [h^-1 Mpc]"},
        {"name": "RTMAX", "value": module.r_trans_max, "comment": "Maximum r-transverse [h^-1 Mpc]"},
        {"name": "NP", "value": module.num_bins_r_par, "comment": "Number of bins in r-parallel"},
        {"name": "NT", "value": module.num_bins_r_trans, "comment": "Number of bins in r-transverse"},
        {"name": "COEFMOD", "value": args.coef_binning_model,
         "comment": "Coefficient for model binning"},
        {"name": "ZMIN", "value": module.z_min_pairs, "comment": "Minimum redshift of pairs"},
        {"name": "ZMAX", "value": module.z_max_pairs, "comment": "Maximum redshift of pairs"},
        {"name": "REJ", "value": module.reject, "comment": "Rejection factor"},
        {"name": "NPALL", "value": int(num_pairs), "comment": "Number of pairs"},
        {"name": "NPUSED", "value": int(num_pairs_used), "comment": "Number of used pairs"},
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


def write(path, result, args, blinding, module=cf):
    """The DMAT and ATTRI HDUs of picca_dmat.py / picca_xdmat.py."""
    dmat_name = "DM" if blinding == "none" else "DM_BLIND"
    dmat_hdu = {
        "columns": [result["WDM"], result["DM"]],
        "names": ["WDM", dmat_name],
        "comments": ["Sum of weight", "Distortion matrix"],
        "units": ["", ""],
        "header": header_cards(args, result["NPALL"], result["NPUSED"], blinding, module),
        "extname": "DMAT",
    }
    attri = {
        "columns": [result["RP"], result["RT"], result["Z"]],
        "names": ["RP", "RT", "Z"],
        "comments": ["R-parallel", "R-transverse", "Redshift"],
        "units": ["h^-1 Mpc", "h^-1 Mpc", ""],
        "extname": "ATTRI",
    }
    fitsio_lite.write_fits(path, [dmat_hdu, attri])


def main(cmdargs=None):
    """Compute the distortion matrix"""
    args = parse_args(cmdargs)
    if args.nproc is None:
        args.nproc = max(cpu_count() // 2, 1)
    userprint("nproc", args.nproc)
    cf.rmu_binning = args.rmu_binning
    if cf.rmu_binning:
        args.rp_min = 0
        args.rp_max = 1
    cf.r_par_max = args.rp_max
    cf.r_par_min = args.rp_min
    cf.r_trans_max = args.rt_max
    cf.z_min_pairs = args.z_min_pairs
    cf.z_max_pairs = args.z_max_pairs
    cf.num_bins_r_par = args.np
    cf.num_bins_r_trans = args.nt
    cf.num_model_bins_r_par = args.np * args.coef_binning_model
    cf.num_model_bins_r_trans = args.nt * args.coef_binning_model
    cf.nside = args.nside
    cf.redshift_evolution_in_distortion_matrix = not args.no_redshift_evolution
    if args.no_redshift_evolution:
        userprint("ignore redshift evolution in the distortion matrix")
    cf.z_ref = 2.25
    cf.alpha = args.z_evol
    cf.alpha2 = args.z_evol
    cf.reject = args.rej
    cf.lambda_abs = constants.ABSORBER_IGM[args.lambda_abs]
    cf.remove_same_half_plate_close_pairs = args.remove_same_half_plate_close_pairs
    cf.x_correlation = False
    cf.ang_correlation = False
    if (args.zerr_cut_deg is None) != (args.zerr_cut_kms is None):
        raise ValueError("Options --zerr-cut-deg and --zerr-cut-kms must be specified together")
    cf.zerr_cut_deg = args.zerr_cut_deg
    cf.zerr_cut_kms = args.zerr_cut_kms

    blinding = io.read_blinding(args.in_dir)
    cosmo = constants.Cosmo(Om=args.fid_Om, Or=args.fid_Or, Ok=args.fid_Ok, wl=args.fid_wl,
                            blinding=blinding, template=args.distance_template)
    t0 = time.time()
    data, num_data, z_min, _ = io.read_deltas(
        args.in_dir, cf.nside, cf.lambda_abs, cf.alpha, cf.z_ref, cosmo,
        max_num_spec=args.nspec, rebin_factor=args.rebin_factor,
        z_min_qso=args.z_min_sources, z_max_qso=args.z_max_sources,
        delta_attributes=args.in_attributes)
    cf.data = data
    cf.data2 = None
    cf.num_data = num_data
    cf.ang_max = utils.compute_ang_max(cosmo, cf.r_trans_max, z_min)
    userprint(f"done, npix = {len(data)}")

    if args.in_dir2 or args.lambda_abs2:
        if args.lambda_abs2 or args.unfold_cf:
            cf.x_correlation = True
        cf.alpha2 = args.z_evol2
        if args.in_dir2 is None:
            args.in_dir2 = args.in_dir
        cf.lambda_abs2 = (constants.ABSORBER_IGM[args.lambda_abs2] if args.lambda_abs2
                          else cf.lambda_abs)
        data2, num_data2, z_min2, _ = io.read_deltas(
            args.in_dir2, cf.nside, cf.lambda_abs2, cf.alpha2, cf.z_ref, cosmo,
            max_num_spec=args.nspec, rebin_factor=args.rebin_factor,
            z_min_qso=args.z_min_sources, z_max_qso=args.z_max_sources,
            delta_attributes=args.in_attributes)
        cf.data2 = data2
        cf.num_data2 = num_data2
        cf.ang_max = utils.compute_ang_max(cosmo, cf.r_trans_max, z_min, z_min2)
        userprint(f"done, npix = {len(data2)}")

    t1 = time.time()
    userprint(f"picca_dmat.py - Time reading data: {(t1 - t0) / 60:.3f} minutes")
    result = cf.compute_dmat_all(args.nproc)
    t2 = time.time()
    userprint(f"picca_dmat.py - Time computing distortion matrix: {(t2 - t1) / 60:.3f} minutes")
    write(args.out, result, args, blinding)
    userprint(f"picca_dmat.py - Time total : {(time.time() - t0) / 60:.3f} minutes")
    return result


if __name__ == "__main__":
    main(sys.argv[1:])
