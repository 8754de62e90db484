#!/usr/bin/env python3
"""Wick covariance of the delta x quasar cross-correlation on the GPU.

Drop-in for ``py/picca/bin/picca_xwick.py`` (covariance as explained in
Delubac et al. 2015): the same flags, readers, random draw per forest
(healpix dealt to ``--nproc`` chunks, the generator seeded with each chunk's
first healpix), 1D variance and correlation from the ``--cf1d`` file,
normalisation and FITS layout (HDU ``COV`` with CO / WALL / NB / T1-T6 and
the header keywords). ``--nproc`` only sets the chunking of the random
draws; the terms run on the GPU. ``--max-diagram`` 4 (the default): T1-T4,
with T5 = T6 = 0; the reference's diagrams 5-6 read a neighbour list
(``dneighs``) that nothing fills, so ``--max-diagram`` above 4 is refused.
"""

import argparse
import sys
import time
from multiprocessing import cpu_count

from picca_gb300 import constants, fitsio_lite, io, pairs, utils, wick
from picca_gb300.forests import ForestSet
from picca_gb300.utils import userprint


def parse_args(cmdargs=None):
    parser = argparse.ArgumentParser(
        formatter_class=argparse.ArgumentDefaultsHelpFormatter,
        description="Compute the wick covariance for the cross-correlation of object x forests")
    parser.add_argument("--out", type=str, default=None, required=True, help="Output file name")
    parser.add_argument("--in-dir", type=str, default=None, required=True,
                        help="Directory to delta files")
    parser.add_argument("--drq", type=str, default=None, required=True,
                        help="Catalog of objects in DRQ format")
    parser.add_argument("--mode", type=str, default="sdss",
                        choices=["sdss", "desi", "desi_mocks", "desi_healpix"],
                        help="type of catalog supplied, default sdss")
    parser.add_argument("--rp-min", type=float, default=-200.0,
                        help="Min r-parallel [h^-1 Mpc]")
    parser.add_argument("--rp-max", type=float, default=200.0, help="Max r-parallel [h^-1 Mpc]")
    parser.add_argument("--rt-max", type=float, default=200.0, help="Max r-transverse [h^-1 Mpc]")
    parser.add_argument("--np", type=int, default=100, help="Number of r-parallel bins")
    parser.add_argument("--nt", type=int, default=50, help="Number of r-transverse bins")
    parser.add_argument("--z-min-obj", type=float, default=0, help="Min redshift for object field")
    parser.add_argument("--z-max-obj", type=float, default=10,
                        help="Max redshift for object field")
    parser.add_argument("--z-min-sources", type=float, default=0.0,
                        help="Limit the minimum redshift of the quasars used as sources for "
                             "spectra")
    parser.add_argument("--z-max-sources", type=float, default=10.0,
                        help="Limit the maximum redshift of the quasars used as sources for "
                             "spectra")
    parser.add_argument("--lambda-abs", type=str, default="LYA",
                        help="Name of the absorption in picca.constants defining the redshift "
                             "of the delta")
    parser.add_argument("--z-ref", type=float, default=2.25, help="Reference redshift")
    parser.add_argument("--z-evol-del", type=float, default=2.9,
                        help="Exponent of the redshift evolution of the delta field")
    parser.add_argument("--z-evol-obj", type=float, default=1.44,
                        help="Exponent of the redshift evolution of the object field")
    parser.add_argument("--fid-Om", type=float, default=0.315,
                        help="Omega_matter(z=0) of fiducial LambdaCDM cosmology")
    parser.add_argument("--fid-Or", type=float, default=0.0,
                        help="Omega_radiation(z=0) of fiducial LambdaCDM cosmology")
    parser.add_argument("--fid-Ok", type=float, default=0.0,
                        help="Omega_k(z=0) of fiducial LambdaCDM cosmology")
    parser.add_argument("--fid-wl", type=float, default=-1.0,
                        help="Equation of state of dark energy of fiducial LambdaCDM cosmology")
    parser.add_argument("--max-diagram", type=int, default=4, help="Maximum diagram to compute")
    parser.add_argument("--cf1d", type=str, required=True,
                        help="1D auto-correlation of pixels from the same forest file: "
                             "picca_cf1d.py")
    parser.add_argument("--cf", type=str, default=None,
                        help="3D auto-correlation of pixels from different forests: "
                             "picca_cf.py")
    parser.add_argument("--rej", type=float, default=1.0,
                        help="Fraction of rejected object-forests pairs: -1=no rejection, "
                             "1=all rejection")
    parser.add_argument("--nside", type=int, default=16, help="Healpix nside")
    parser.add_argument("--nproc", type=int, default=None, help="Number of processors")
    parser.add_argument("--nspec", type=int, default=None,
                        help="Maximum number of spectra to read")
    parser.add_argument("--rebin-factor", type=int, default=None,
                        help="Rebin factor for deltas. If not None, deltas will be rebinned by "
                             "that factor")
    parser.add_argument("--in-attributes", type=str, default=None,
                        help="Filename for the delta attributes file (continuum-fit order for "
                             "the projection)")
    return parser.parse_args(cmdargs)


def main(cmdargs=None):
    """Compute the wick covariance for the cross-correlation of object x forests"""
    args = parse_args(cmdargs)
    if args.nproc is None:
        args.nproc = cpu_count() // 2
    if args.max_diagram > 4:
        sys.exit("picca_gb300: --max-diagram above 4 (T5, T6) is not provided; the reference's "
                 "diagrams 5-6 read a neighbour list that is never filled")
    if (args.fid_Or != 0.0) or (args.fid_Ok != 0.0) or (args.fid_wl != -1.0):
        userprint("ERROR: Cosmology with other than Omega_m set are not yet implemented")
        sys.exit()
    blinding = io.read_blinding(args.in_dir)
    cosmo = constants.Cosmo(Om=args.fid_Om, Or=args.fid_Or, Ok=args.fid_Ok, wl=args.fid_wl,
                            verbose=False)
    t0 = time.time()
    data, num_data, z_min, z_max = io.read_deltas(
        args.in_dir, args.nside, constants.ABSORBER_IGM[args.lambda_abs], args.z_evol_del,
        args.z_ref, cosmo, max_num_spec=args.nspec, nproc=args.nproc,
        rebin_factor=args.rebin_factor, z_min_qso=args.z_min_sources,
        z_max_qso=args.z_max_sources, delta_attributes=args.in_attributes)
    userprint(f"done, npix = {len(data)}, ndels = {num_data}")
    if args.z_min_obj is None:
        r_min = max(0.0, cosmo.get_r_comov(z_min) + args.rp_min)
        args.z_min_obj = cosmo.distance_to_redshift(r_min)
    if args.z_max_obj is None:
        r_max = max(0.0, cosmo.get_r_comov(z_max) + args.rp_max)
        args.z_max_obj = cosmo.distance_to_redshift(r_max)
    objs, z_min2 = io.read_objects(args.drq, args.nside, args.z_min_obj, args.z_max_obj,
                                   args.z_evol_obj, args.z_ref, cosmo, mode=args.mode)
    userprint(f"done, npix = {len(objs)}")
    ang_max = utils.compute_ang_max(cosmo, args.rt_max, z_min, z_min2)
    cf1d = wick.read_cf1d(args.cf1d)
    fs, qs = ForestSet.from_deltas(data), ForestSet.from_objects(objs)
    params = pairs.make_params(args.rp_min, args.rp_max, args.rt_max, args.np, args.nt, ang_max,
                               x_correlation=True)
    t1 = time.time()
    result = wick.cross_wick_covariance(fs, qs, params, cf1d, args.rej, nproc=args.nproc,
                                        z_ref=args.z_ref, alpha=args.z_evol_del,
                                        alpha_obj=args.z_evol_obj)
    userprint(f"picca_xwick.py - Time computing the Wick terms: {(time.time() - t1) / 60:.3f} "
              "minutes")
    from picca_gb300.bin.picca_wick import write
    write(args.out, result, args, blinding)
    userprint(f"picca_xwick.py - Time total : {(time.time() - t0) / 60:.3f} minutes")
    return result


if __name__ == "__main__":
    main(sys.argv[1:])
