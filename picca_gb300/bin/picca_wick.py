#!/usr/bin/env python3
"""Wick covariance of the Lyman-alpha auto-correlation on the GPU.

Drop-in for ``py/picca/bin/picca_wick.py`` (covariance as explained in
Delubac et al. 2015): the same flags, readers, random draw per forest
(healpix dealt to ``--nproc`` chunks, the generator seeded with each chunk's
first healpix), 1D variance and correlation from the ``--cf1d`` file,
normalisation and FITS layout (HDU ``COV`` with CO / WALL / NB / T1-T6 and
the header keywords). ``--nproc`` only sets the chunking of the random
draws; the terms run on the GPU. One delta field and ``--max-diagram`` 3
(the default), where T4-T6 are zero; the reference's code for diagrams 4-5
and for a second field does not run, so those options are refused.
"""

import argparse
import sys
import time
from multiprocessing import cpu_count

import numpy as np

from picca_gb300 import constants, fitsio_lite, io, pairs, utils, wick
from picca_gb300.forests import ForestSet
from picca_gb300.utils import userprint


def parse_args(cmdargs=None):
    parser = argparse.ArgumentParser(
        formatter_class=argparse.ArgumentDefaultsHelpFormatter,
        description="Compute the wick covariance for the auto-correlation of forests")
    parser.add_argument("--out", type=str, default=None, required=True, help="Output file name")
    parser.add_argument("--in-dir", type=str, default=None, required=True,
                        help="Directory to delta files")
    parser.add_argument("--in-dir2", type=str, default=None,
                        help="Directory to 2nd delta files")
    parser.add_argument("--rp-min", type=float, default=0.0, help="Min r-parallel [h^-1 Mpc]")
    parser.add_argument("--rp-max", type=float, default=200.0, help="Max r-parallel [h^-1 Mpc]")
    parser.add_argument("--rt-max", type=float, default=200.0, help="Max r-transverse [h^-1 Mpc]")
    parser.add_argument("--np", type=int, default=50, help="Number of r-parallel bins")
    parser.add_argument("--nt", type=int, default=50, help="Number of r-transverse bins")
    parser.add_argument("--z-min-sources", type=float, default=0.0,
                        help="Limit the minimum redshift of the quasars used as sources for "
                             "spectra")
    parser.add_argument("--z-max-sources", type=float, default=10.0,
                        help="Limit the maximum redshift of the quasars used as sources for "
                             "spectra")
    parser.add_argument("--lambda-abs", type=str, default="LYA",
                        help="Name of the absorption in picca.constants defining the redshift "
                             "of the delta")
    parser.add_argument("--lambda-abs2", type=str, default=None,
                        help="Name of the absorption in picca.constants defining the redshift "
                             "of the 2nd delta")
    parser.add_argument("--z-ref", type=float, default=2.25, help="Reference redshift")
    parser.add_argument("--z-evol", type=float, default=2.9,
                        help="Exponent of the redshift evolution of the delta field")
    parser.add_argument("--z-evol2", type=float, default=2.9,
                        help="Exponent of the redshift evolution of the 2nd delta field")
    parser.add_argument("--fid-Om", type=float, default=0.315,
                        help="Omega_matter(z=0) of fiducial LambdaCDM cosmology")
    parser.add_argument("--fid-Or", type=float, default=0.0,
                        help="Omega_radiation(z=0) of fiducial LambdaCDM cosmology")
    parser.add_argument("--fid-Ok", type=float, default=0.0,
                        help="Omega_k(z=0) of fiducial LambdaCDM cosmology")
    parser.add_argument("--fid-wl", type=float, default=-1.0,
                        help="Equation of state of dark energy of fiducial LambdaCDM cosmology")
    parser.add_argument("--no-project", action="store_true",
                        help="Do not project out continuum fitting modes")
    parser.add_argument("--max-diagram", type=int, default=3, help="Maximum diagram to compute")
    parser.add_argument("--cf1d", type=str, required=True,
                        help="1D auto-correlation of pixels from the same forest file: "
                             "picca_cf1d.py")
    parser.add_argument("--cf1d2", type=str, default=None,
                        help="1D auto-correlation of pixels from the same forest file of the "
                             "2nd delta field: picca_cf1d.py")
    parser.add_argument("--cf", type=str, default=None,
                        help="3D auto-correlation of pixels from different forests: "
                             "picca_cf.py")
    parser.add_argument("--cf2", type=str, default=None,
                        help="3D auto-correlation of pixels from different forests for 2nd "
                             "catalog: picca_cf.py")
    parser.add_argument("--cf12", type=str, default=None,
                        help="3D auto-correlation of pixels from different forests for cross "
                             "1st and 2nd catalog: picca_cf.py")
    parser.add_argument("--unfold-cf", action="store_true",
                        help="rp can be positive or negative depending on the relative "
                             "position between absorber1 and absorber2")
    parser.add_argument("--rej", type=float, default=1.0,
                        help="Fraction of rejected pairs: -1=no rejection, 1=all rejection")
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


def header_cards(args, npall, npused, blinding):
    """COV keywords of picca_wick.py:548-598."""
    return [
        {"name": "RPMIN", "value": args.rp_min, "comment": "Minimum r-parallel [h^-1 Mpc]"},
        {"name": "RPMAX", "value": args.rp_max, "comment": "Maximum r-parallel [h^-1 Mpc]"},
        {"name": "RTMAX", "value": args.rt_max, "comment": "Maximum r-transverse [h^-1 Mpc]"},
        {"name": "NP", "value": args.np, "comment": "Number of bins in r-parallel"},
        {"name": "NT", "value": args.nt, "comment": "Number of bins in r-transverse"},
        {"name": "REJ", "value": args.rej, "comment": "Rejection factor"},
        {"name": "NPALL", "value": npall, "comment": "Number of pairs"},
        {"name": "NPUSED", "value": npused, "comment": "Number of used pairs"},
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


def write(path, result, args, blinding):
    names = ["CO", "WALL", "NB", "T1", "T2", "T3", "T4", "T5", "T6"]
    comments = ["Sum of weight", "Covariance", "Nomber of pairs", "T1", "T2", "T3", "T4", "T5",
                "T6"]
    fitsio_lite.write_fits(path, [{
        "columns": [result[n] for n in names], "names": names, "comments": comments,
        "header": header_cards(args, result["NPALL"], result["NPUSED"], blinding),
        "extname": "COV"}])


def main(cmdargs=None):
    """Compute the wick covariance for the auto-correlation of forests"""
    args = parse_args(cmdargs)
    if args.nproc is None:
        args.nproc = cpu_count() // 2
    userprint("nproc", args.nproc)
    if args.max_diagram > 3:
        sys.exit("picca_gb300: --max-diagram above 3 (T4, T5) is not provided; the reference's "
                 "compute_wickT45_pairs does not run")
    if args.in_dir2 or args.lambda_abs2:
        sys.exit("picca_gb300: the Wick covariance of two delta fields is not provided; the "
                 "reference's two-field branch relabels the first field")
    if (args.fid_Or != 0.0) or (args.fid_Ok != 0.0) or (args.fid_wl != -1.0):
        userprint("ERROR: Cosmology with other than Omega_m set are not yet implemented")
        sys.exit()
    blinding = io.read_blinding(args.in_dir)
    cosmo = constants.Cosmo(Om=args.fid_Om, Or=args.fid_Or, Ok=args.fid_Ok, wl=args.fid_wl,
                            verbose=False)
    t0 = time.time()
    data, num_data, z_min, _ = io.read_deltas(
        args.in_dir, args.nside, constants.ABSORBER_IGM[args.lambda_abs], args.z_evol,
        args.z_ref, cosmo, max_num_spec=args.nspec, nproc=args.nproc,
        rebin_factor=args.rebin_factor, z_min_qso=args.z_min_sources,
        z_max_qso=args.z_max_sources, delta_attributes=args.in_attributes)
    ang_max = utils.compute_ang_max(cosmo, args.rt_max, z_min)
    userprint(f"done, npix = {len(data)}")
    cf1d = wick.read_cf1d(args.cf1d)
    fs = ForestSet.from_deltas(data)
    params = pairs.make_params(args.rp_min, args.rp_max, args.rt_max, args.np, args.nt, ang_max)
    t1 = time.time()
    result = wick.wick_covariance(fs, params, cf1d, args.rej, nproc=args.nproc,
                                  z_ref=args.z_ref, alpha=args.z_evol, alpha2=args.z_evol)
    userprint(f"picca_wick.py - Time computing the Wick terms: {(time.time() - t1) / 60:.3f} "
              f"minutes ({num_data} forests)")
    write(args.out, result, args, blinding)
    userprint(f"picca_wick.py - Time total : {(time.time() - t0) / 60:.3f} minutes")
    return result


if __name__ == "__main__":
    main(sys.argv[1:])
