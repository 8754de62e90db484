#!/usr/bin/env python3
"""Distortion matrix of the delta x quasar cross-correlation on the GPU.

Drop-in for ``py/picca/bin/picca_xdmat.py``: the same flags (:45-340),
module globals (:342-392), readers (:404-460), random rejection per process
chunk (healpix dealt by index % nproc, NumPy's generator seeded with each
chunk's first healpix; forests without a kept quasar are not counted,
py/picca/xcf.py:382-386), normalisation and FITS layout (HDU ``DMAT`` with
WDM/DM and the header keywords, HDU ``ATTRI`` with RP/RT/Z). ``--nproc``
only sets the chunking of the random draws; every kept pair runs in one GPU
launch.
"""

import argparse
import sys
import time
from multiprocessing import cpu_count

from picca_gb300 import constants, io, utils, xcf
from picca_gb300.bin import picca_dmat
from picca_gb300.utils import userprint


def parse_args(cmdargs=None):
    parser = argparse.ArgumentParser(
        formatter_class=argparse.ArgumentDefaultsHelpFormatter,
        description="Compute the distortion matrix of the cross-correlation delta x object")
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
    parser.add_argument("--rmu-binning", action="store_true",
                        help="Estimate in r,mu binning. np becomes mu bins. nt becomes r bins. "
                             "rp min max is always -1, 1")
    parser.add_argument("--coef-binning-model", type=int, default=1,
                        help="Coefficient multiplying np and nt to get finner binning for the "
                             "model")
    parser.add_argument("--z-min-obj", type=float, default=0, help="Min redshift for object field")
    parser.add_argument("--z-max-obj", type=float, default=10,
                        help="Max redshift for object field")
    parser.add_argument("--zerr-cut-deg", type=float, default=None,
                        help="Angular cut (deg) between a pixel and the background quasar")
    parser.add_argument("--zerr-cut-kms", type=float, default=None,
                        help="Velocity cut (km/s) between a pixel and the background quasar")
    parser.add_argument("--z-min-sources", type=float, default=0.0,
                        help="Limit the minimum redshift of the quasars used as sources")
    parser.add_argument("--z-max-sources", type=float, default=10.0,
                        help="Limit the maximum redshift of the quasars used as sources")
    parser.add_argument("--z-min-pairs", type=float, default=None,
                        help="Limit the minimum redshift of the absorber-object pairs")
    parser.add_argument("--z-max-pairs", type=float, default=None,
                        help="Limit the maximum redshift of the absorber-object pairs")
    parser.add_argument("--lambda-abs", type=str, default="LYA",
                        help="Name of the absorption in picca.constants")
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
    parser.add_argument("--no-redshift-evolution", action="store_true",
                        help="Ignore redshift evolution when computing distortion matrix")
    return parser.parse_args(cmdargs)


def main(cmdargs=None):
    """Compute the distortion matrix of the cross-correlation delta x object"""
    args = parse_args(cmdargs)
    if args.nproc is None:
        args.nproc = max(cpu_count() // 2, 1)
    userprint("nproc", args.nproc)
    xcf.rmu_binning = args.rmu_binning
    if xcf.rmu_binning:
        args.rp_min = -1
        args.rp_max = 1
    xcf.r_par_max = args.rp_max
    xcf.r_par_min = args.rp_min
    xcf.r_trans_max = args.rt_max
    xcf.z_min_pairs = args.z_min_pairs
    xcf.z_max_pairs = args.z_max_pairs
    xcf.num_bins_r_par = args.np
    xcf.num_bins_r_trans = args.nt
    xcf.num_model_bins_r_par = args.np * args.coef_binning_model
    xcf.num_model_bins_r_trans = args.nt * args.coef_binning_model
    xcf.nside = args.nside
    xcf.redshift_evolution_in_distortion_matrix = not args.no_redshift_evolution
    if args.no_redshift_evolution:
        userprint("ignore redshift evolution in the distortion matrix")
    xcf.z_ref = 2.25
    xcf.alpha = args.z_evol_del
    xcf.alpha_obj = args.z_evol_obj
    xcf.lambda_abs = constants.ABSORBER_IGM[args.lambda_abs]
    xcf.reject = args.rej
    xcf.ang_correlation = False
    if (args.zerr_cut_deg is None) != (args.zerr_cut_kms is None):
        raise ValueError("Options --zerr-cut-deg and --zerr-cut-kms must be specified together")
    xcf.zerr_cut_deg = args.zerr_cut_deg
    xcf.zerr_cut_kms = args.zerr_cut_kms

    blinding = io.read_blinding(args.in_dir)
    cosmo = constants.Cosmo(Om=args.fid_Om, Or=args.fid_Or, Ok=args.fid_Ok, wl=args.fid_wl,
                            blinding=blinding, template=args.distance_template)
    t0 = time.time()
    data, num_data, z_min, z_max = io.read_deltas(
        args.in_dir, args.nside, xcf.lambda_abs, args.z_evol_del, xcf.z_ref, cosmo=cosmo,
        max_num_spec=args.nspec, rebin_factor=args.rebin_factor,
        z_min_qso=args.z_min_sources, z_max_qso=args.z_max_sources,
        delta_attributes=args.in_attributes)
    xcf.data = data
    xcf.num_data = num_data
    userprint(f"done, npix = {len(data)}")
    if args.z_min_obj is None or args.z_max_obj is None:
        raise ValueError("--z-min-obj / --z-max-obj must be numbers")
    objs, z_min2 = io.read_objects(args.drq, args.nside, args.z_min_obj, args.z_max_obj,
                                   args.z_evol_obj, xcf.z_ref, cosmo, mode=args.mode)
    xcf.objs = objs
    xcf.ang_max = utils.compute_ang_max(cosmo, xcf.r_trans_max, z_min, z_min2)
    t1 = time.time()
    userprint(f"picca_xdmat.py - Time reading data: {(t1 - t0) / 60:.3f} minutes")
    result = xcf.compute_dmat_all(args.nproc)
    t2 = time.time()
    userprint(f"picca_xdmat.py - Time computing distortion matrix: {(t2 - t1) / 60:.3f} minutes")
    picca_dmat.write(args.out, result, args, blinding, module=xcf)
    userprint(f"picca_xdmat.py - Time total : {(time.time() - t0) / 60:.3f} minutes")
    return result


if __name__ == "__main__":
    main(sys.argv[1:])
