#!/usr/bin/env python3
"""Auto- and cross-correlation of delta fields on the GPU.

Drop-in for ``py/picca/bin/picca_cf.py``: the same flags (:42-338), the same
module-global setup (:340-368), readers (:383-447), aggregation (:465-484)
and FITS layout (:486-580: HDU ``ATTRI`` with RP/RT/Z/NB and the binning
header, HDU ``COR`` with HEALPID/WE/DA). The pair loop runs on the GPU in one
launch over every healpix instead of a fork Pool; ``--nproc`` is accepted
and ignored. ``--precision`` selects the GPU arithmetic.
"""

import argparse
import sys
import time

from picca_gb300 import cf, constants, io, utils
from picca_gb300.bin import corr_output
from picca_gb300.utils import userprint


def parse_args(cmdargs=None):
    parser = argparse.ArgumentParser(
        formatter_class=argparse.ArgumentDefaultsHelpFormatter,
        description="Compute the auto and cross-correlation of delta fields")
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
                        help="Estimate in r,mu binning. np becomes mu bins. nt becomes r bins.")
    parser.add_argument("--zerr-cut-deg", type=float, default=None,
                        help="Angular cut (deg) between a pixel and the other background quasar")
    parser.add_argument("--zerr-cut-kms", type=float, default=None,
                        help="Velocity cut (km/s) between a pixel and the other background quasar")
    parser.add_argument("--z-min-sources", type=float, default=0.0,
                        help="Limit the minimum redshift of the quasars used as sources")
    parser.add_argument("--z-max-sources", type=float, default=10.0,
                        help="Limit the maximum redshift of the quasars used as sources")
    parser.add_argument("--z-min-pairs", type=float, default=None,
                        help="Minimum redshift of the absorber pairs")
    parser.add_argument("--z-max-pairs", type=float, default=None,
                        help="Maximum redshift of the absorber pairs")
    parser.add_argument("--lambda-abs", type=str, default="LYA",
                        help="Name of the absorption in picca.constants")
    parser.add_argument("--lambda-abs2", type=str, default=None,
                        help="Name of the absorption of the 2nd delta")
    parser.add_argument("--z-ref", type=float, default=2.25, help="Reference redshift")
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
    parser.add_argument("--no-project", action="store_true",
                        help="Do not project out continuum fitting modes")
    parser.add_argument("--remove-same-half-plate-close-pairs", action="store_true",
                        help="Reject pairs in the first bin in r-parallel from same half plate")
    parser.add_argument("--nside", type=int, default=16, help="Healpix nside")
    parser.add_argument("--nproc", type=int, default=None, help="Accepted for compatibility")
    parser.add_argument("--nspec", type=int, default=None,
                        help="Maximum number of spectra to read")
    parser.add_argument("--unfold-cf", action="store_true",
                        help="rp can be positive or negative depending on the relative position")
    parser.add_argument("--shuffle-distrib-forest-seed", type=int, default=None,
                        help="Shuffle the distribution of forests on the sky with this seed")
    parser.add_argument("--rebin-factor", type=int, default=None,
                        help="Rebin factor for deltas")
    parser.add_argument("--in-attributes", type=str, default=None,
                        help="Delta attributes file (continuum-fit order for the projection)")
    parser.add_argument("--precision", choices=["fp64", "fp32_guard"], default="fp32_guard",
                        help="GPU arithmetic: plain FP64, or FP32 geometry with FP64 "
                             "bin-edge re-decision (bins and counts identical to FP64)")
    return parser.parse_args(cmdargs)


def main(cmdargs=None):
    """Compute the auto and cross-correlation of delta fields"""
    args = parse_args(cmdargs)
    cf.rmu_binning = args.rmu_binning
    if cf.rmu_binning:
        args.rp_min = 0
        args.rp_max = 1
    cf.r_par_max = args.rp_max
    cf.r_trans_max = args.rt_max
    cf.r_par_min = args.rp_min
    cf.z_min_pairs = args.z_min_pairs
    cf.z_max_pairs = args.z_max_pairs
    cf.num_bins_r_par = args.np
    cf.num_bins_r_trans = args.nt
    cf.nside = args.nside
    cf.z_ref = args.z_ref
    cf.alpha = args.z_evol
    cf.lambda_abs = constants.ABSORBER_IGM[args.lambda_abs]
    cf.remove_same_half_plate_close_pairs = args.remove_same_half_plate_close_pairs
    cf.precision = args.precision
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
        max_num_spec=args.nspec, no_project=args.no_project, rebin_factor=args.rebin_factor,
        z_min_qso=args.z_min_sources, z_max_qso=args.z_max_sources,
        delta_attributes=args.in_attributes)
    cf.data = data
    cf.data2 = None
    cf.num_data = num_data
    cf.x_correlation = False
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
            max_num_spec=args.nspec, no_project=args.no_project,
            rebin_factor=args.rebin_factor, z_min_qso=args.z_min_sources,
            z_max_qso=args.z_max_sources, delta_attributes=args.in_attributes)
        cf.data2 = data2
        cf.num_data2 = num_data2
        cf.ang_max = utils.compute_ang_max(cosmo, cf.r_trans_max, z_min, z_min2)
        userprint(f"done, npix = {len(data2)}")

    if args.shuffle_distrib_forest_seed is not None:
        cf.data = utils.shuffle_distrib_forests(cf.data, args.shuffle_distrib_forest_seed)

    t1 = time.time()
    userprint(f"picca_cf.py - Time reading data: {(t1 - t0) / 60:.3f} minutes")
    result = cf.compute_xi_all()
    t2 = time.time()
    userprint(f"picca_cf.py - Time computing correlation function: {(t2 - t1) / 60:.3f} minutes")

    corr_output.write(args.out, result, cf, args, blinding)
    userprint(f"picca_cf.py - Time total : {(time.time() - t0) / 60:.3f} minutes")
    return result


if __name__ == "__main__":
    main(sys.argv[1:])
