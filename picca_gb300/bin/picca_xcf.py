#!/usr/bin/env python3
"""Delta x quasar cross-correlation on the GPU.

Drop-in for ``py/picca/bin/picca_xcf.py``: same flags, module-global setup
(:351-373), object and delta readers (:390-434), removal of the mean delta
versus observed wavelength (:435-468), aggregation and FITS layout
(:500-615). The pair loop runs on the GPU in one launch.
"""

import argparse
import sys
import time

from picca_gb300 import constants, io, prep_del, utils, xcf
from picca_gb300.bin import corr_output
from picca_gb300.utils import userprint


def parse_args(cmdargs=None):
    parser = argparse.ArgumentParser(
        formatter_class=argparse.ArgumentDefaultsHelpFormatter,
        description="Compute the cross-correlation between a catalog of objects and a delta field.")
    parser.add_argument("--out", type=str, default=None, required=True, help="Output file name")
    parser.add_argument("--in-dir", type=str, default=None, required=True,
                        help="Directory to delta files")
    parser.add_argument("--drq", type=str, default=None, required=True,
                        help="Catalog of objects in format selected by mode")
    parser.add_argument("--mode", type=str, choices=["desi", "desi_healpix", "desi_mocks", "sdss"],
                        default="sdss", help="Mode for reading the catalog")
    parser.add_argument("--rp-min", type=float, default=-200.0, help="Min r-parallel [h^-1 Mpc]")
    parser.add_argument("--rp-max", type=float, default=200.0, help="Max r-parallel [h^-1 Mpc]")
    parser.add_argument("--rt-max", type=float, default=200.0, help="Max r-transverse [h^-1 Mpc]")
    parser.add_argument("--np", type=int, default=100, help="Number of r-parallel bins")
    parser.add_argument("--nt", type=int, default=50, help="Number of r-transverse bins")
    parser.add_argument("--rmu-binning", action="store_true", help="Estimate in r,mu binning")
    parser.add_argument("--z-min-obj", type=float, default=0, help="Min redshift for object field")
    parser.add_argument("--z-max-obj", type=float, default=10, help="Max redshift for object field")
    parser.add_argument("--zerr-cut-deg", type=float, default=None,
                        help="Angular cut (deg) of the quasar-pair redshift-error veto")
    parser.add_argument("--zerr-cut-kms", type=float, default=None,
                        help="Velocity cut (km/s) of the quasar-pair redshift-error veto")
    parser.add_argument("--z-min-sources", type=float, default=0.0,
                        help="Limit the minimum redshift of the quasars used as sources")
    parser.add_argument("--z-max-sources", type=float, default=10.0,
                        help="Limit the maximum redshift of the quasars used as sources")
    parser.add_argument("--z-min-pairs", type=float, default=None,
                        help="Minimum redshift of the pairs")
    parser.add_argument("--z-max-pairs", type=float, default=None,
                        help="Maximum redshift of the pairs")
    parser.add_argument("--lambda-abs", type=str, default="LYA",
                        help="Name of the absorption in picca.constants")
    parser.add_argument("--z-ref", type=float, default=2.25, help="Reference redshift")
    parser.add_argument("--z-evol-del", type=float, default=2.9,
                        help="Exponent of the redshift evolution of the delta field")
    parser.add_argument("--z-evol-obj", type=float, default=1.44,
                        help="Exponent of the redshift evolution of the object field")
    parser.add_argument("--fid-Om", type=float, default=0.315, help="Omega_matter(z=0)")
    parser.add_argument("--fid-Or", type=float, default=0.0, help="Omega_radiation(z=0)")
    parser.add_argument("--fid-Ok", type=float, default=0.0, help="Omega_k(z=0)")
    parser.add_argument("--fid-wl", type=float, default=-1.0,
                        help="Equation of state of dark energy")
    parser.add_argument("--distance-template", type=str, required=False,
                        help="Template cosmology (CAMB; not supported here)")
    parser.add_argument("--no-project", action="store_true",
                        help="Do not project out continuum fitting modes")
    parser.add_argument("--no-remove-mean-lambda-obs", action="store_true",
                        help="Do not remove mean delta versus lambda_obs")
    parser.add_argument("--nside", type=int, default=16, help="Healpix nside")
    parser.add_argument("--nproc", type=int, default=None, help="Accepted for compatibility")
    parser.add_argument("--nspec", type=int, default=None, help="Maximum number of spectra")
    parser.add_argument("--shuffle-distrib-obj-seed", type=int, default=None,
                        help="Shuffle the distribution of objects on the sky with this seed")
    parser.add_argument("--shuffle-distrib-forest-seed", type=int, default=None,
                        help="Shuffle the distribution of forests on the sky with this seed")
    parser.add_argument("--rebin-factor", type=int, default=None, help="Rebin factor for deltas")
    parser.add_argument("--in-attributes", type=str, default=None,
                        help="Delta attributes file (continuum-fit order for the projection)")
    parser.add_argument("--precision", choices=["fp64", "fp32_guard"], default="fp32_guard",
                        help="GPU arithmetic (see picca_cf.py)")
    return parser.parse_args(cmdargs)


def main(cmdargs=None):
    """Compute the cross-correlation between a catalog of objects and a delta field."""
    args = parse_args(cmdargs)
    xcf.rmu_binning = args.rmu_binning
    if xcf.rmu_binning:
        args.rp_min = -1
        args.rp_max = 1
    xcf.r_par_max = args.rp_max
    xcf.r_par_min = args.rp_min
    xcf.z_min_pairs = args.z_min_pairs
    xcf.z_max_pairs = args.z_max_pairs
    xcf.r_trans_max = args.rt_max
    xcf.num_bins_r_par = args.np
    xcf.num_bins_r_trans = args.nt
    xcf.nside = args.nside
    xcf.lambda_abs = constants.ABSORBER_IGM[args.lambda_abs]
    xcf.precision = args.precision
    if (args.zerr_cut_deg is None) != (args.zerr_cut_kms is None):
        raise ValueError("Options --zerr-cut-deg and --zerr-cut-kms must be specified together")
    xcf.zerr_cut_deg = args.zerr_cut_deg
    xcf.zerr_cut_kms = args.zerr_cut_kms

    blinding = io.read_blinding(args.in_dir)
    cosmo = constants.Cosmo(Om=args.fid_Om, Or=args.fid_Or, Ok=args.fid_Ok, wl=args.fid_wl,
                            blinding=blinding, template=args.distance_template)
    t0 = time.time()
    if args.z_min_obj is None or args.z_max_obj is None:
        raise ValueError("--z-min-obj / --z-max-obj must be numbers")
    objs, z_min2 = io.read_objects(args.drq, args.nside, args.z_min_obj, args.z_max_obj,
                                   args.z_evol_obj, args.z_ref, cosmo, mode=args.mode)
    xcf.objs = objs
    data, num_data, z_min, z_max = io.read_deltas(
        args.in_dir, args.nside, xcf.lambda_abs, args.z_evol_del, args.z_ref, cosmo=cosmo,
        max_num_spec=args.nspec, no_project=args.no_project, rebin_factor=args.rebin_factor,
        z_min_qso=args.z_min_sources, z_max_qso=args.z_max_sources,
        delta_attributes=args.in_attributes)
    xcf.data = data
    xcf.num_data = num_data
    userprint(f"done, npix = {len(data)}")
    if not args.no_remove_mean_lambda_obs:
        prep_del.remove_mean_lambda_obs(xcf.data, z_min, z_max, xcf.lambda_abs)
    if args.shuffle_distrib_obj_seed is not None:
        xcf.objs = utils.shuffle_distrib_forests(objs, args.shuffle_distrib_obj_seed)
    if args.shuffle_distrib_forest_seed is not None:
        xcf.data = utils.shuffle_distrib_forests(xcf.data, args.shuffle_distrib_forest_seed)
    xcf.ang_max = utils.compute_ang_max(cosmo, xcf.r_trans_max, z_min, z_min2)
    t1 = time.time()
    userprint(f"picca_xcf.py - Time reading data: {(t1 - t0) / 60:.3f} minutes")
    result = xcf.compute_xi_all()
    t2 = time.time()
    userprint(f"picca_xcf.py - Time computing cross-correlation function: "
              f"{(t2 - t1) / 60:.3f} minutes")
    corr_output.write(args.out, result, xcf, args, blinding)
    userprint(f"picca_xcf.py - Time total: {(time.time() - t0) / 60:.3f} minutes")
    return result


if __name__ == "__main__":
    main(sys.argv[1:])
