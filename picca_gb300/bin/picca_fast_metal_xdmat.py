#!/usr/bin/env python3
"""Fast metal distortion matrices of the delta x quasar cross-correlation on
the GPU.

Drop-in for ``py/picca/bin/picca_fast_metal_xdmat.py``: the same flags, the
matrices computed from the STACK_DELTAS table of a delta-attributes file
against the quasars of the catalogue compressed to a redshift histogram of
``--qso-z-bins`` bins (one matrix per absorber of ``--abs-igm``, signed
r_par = forest - quasar), and the same FITS layout (HDU ``ATTRI`` with
ABS_IGM and the header keywords, HDU ``MDMAT`` with RP_QSO_ / RT_QSO_ /
Z_QSO_ / DM_QSO_ columns per absorber).
"""

import argparse
import sys
import time

import numpy as np

from picca_gb300 import constants, fast_metal, io
from picca_gb300.bin.picca_fast_metal_dmat import (guess_delta_dir, header_cards, read_stack,
                                                   write)
from picca_gb300.utils import userprint


def parse_args(cmdargs=None):
    parser = argparse.ArgumentParser(
        formatter_class=argparse.ArgumentDefaultsHelpFormatter,
        description="Compute the fast metal distortion matrices of the cross-correlation "
                    "delta x object from the stacked deltas")
    parser.add_argument("--out", type=str, default=None, required=True, help="Output file name")
    parser.add_argument("-i", "--in-attributes", type=str, default=None, required=True,
                        help="Path to delta_attributes.fits.gz file with hdu STACK_DELTAS "
                             'containing table with at least rows "LOGLAM" and "WEIGHT"')
    parser.add_argument("--delta-dir", type=str, default=None,
                        help="Path to directory with delta*.gz to get the blinding info "
                             "(default is trying to guess from attributes file)")
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
    parser.add_argument("--coef-binning-model", type=int, default=1,
                        help="Coefficient multiplying np and nt to get finner binning for the "
                             "model")
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
    parser.add_argument("--obj-name", type=str, default="QSO", help="Name of the object tracer")
    parser.add_argument("--abs-igm", type=str, default=None, nargs="*",
                        help="List of names of metal absorption in picca.constants")
    parser.add_argument("--z-ref", type=float, default=2.25, help="Reference redshift")
    parser.add_argument("--z-evol-del", type=float, default=2.9,
                        help="Exponent of the redshift evolution of the delta field")
    parser.add_argument("--z-evol-obj", type=float, default=1.44,
                        help="Exponent of the redshift evolution of the object field")
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
    parser.add_argument("--rebin-factor", type=int, default=None,
                        help="Rebin factor for deltas. If not None, deltas will be rebinned by "
                             "that factor")
    parser.add_argument("--qso-z-bins", type=int, default=1000,
                        help="Bins for the distribution of QSO redshifts")
    return parser.parse_args(cmdargs)


def main(cmdargs=None):
    """Compute the fast metal distortion matrices of the cross-correlation"""
    args = parse_args(cmdargs)
    num_bins_r_par = args.np * args.coef_binning_model
    num_bins_r_trans = args.nt * args.coef_binning_model
    alpha_abs = {args.lambda_abs: args.z_evol_del}
    for name in args.abs_igm:
        alpha_abs[name] = args.metal_alpha
    blinding = io.read_blinding(guess_delta_dir(args))
    cosmo = constants.Cosmo(Om=args.fid_Om, Or=args.fid_Or, Ok=args.fid_Ok, wl=args.fid_wl,
                            verbose=False)
    t0 = time.time()
    stack = read_stack(args.in_attributes)
    catalog = io.read_drq(args.drq, z_min=args.z_min_obj, z_max=args.z_max_obj, keep_bal=True,
                          mode=args.mode)
    z_qso = np.asarray(catalog["Z"], dtype=np.float64)
    weight_qso = ((1.0 + z_qso) / (1.0 + args.z_ref)) ** (args.z_evol_obj - 1.0)
    userprint(f"Use histogram of QSO redshifts with {args.qso_z_bins} bins")
    z_hist, w_hist = fast_metal.quasar_histogram(z_qso, weight_qso, args.qso_z_bins)
    quasars = fast_metal.quasar_side(z_hist, w_hist, cosmo)
    t1 = time.time()
    userprint(f"picca_metal_xdmat.py - Time reading data: {(t1 - t0) / 60:.3f} minutes")
    lam_out = constants.ABSORBER_IGM[args.lambda_abs]
    engine = fast_metal.FastMetalEngine()
    dev_quasars = engine.upload(quasars)
    names, results = [], []
    for name in args.abs_igm:
        userprint("Computing", name)
        side = fast_metal.stack_side(stack["LOGLAM"], stack["WEIGHT"],
                                     constants.ABSORBER_IGM[name], lam_out,
                                     alpha_abs[name] + alpha_abs[args.lambda_abs], cosmo,
                                     args.rebin_factor)
        sums = engine.histograms_device(engine.upload(side), dev_quasars, args.rp_min,
                                        args.rp_max, num_bins_r_par, num_bins_r_trans,
                                        signed=True)
        h = {k: v.cpu().numpy() for k, v in sums.items()}
        results.append(fast_metal.finish(h, args.rt_max, num_bins_r_par, num_bins_r_trans))
        names.append(name)
    t2 = time.time()
    userprint(f"picca_metal_xdmat.py - Time computing all metal matrix: "
              f"{(t2 - t1) / 60:.3f} minutes")
    write(args.out, names, results,
          header_cards(args, num_bins_r_par, num_bins_r_trans, blinding, cross=True), blinding,
          prefix=args.obj_name + "_")
    userprint(f"picca_metal_xdmat.py - Time total : {(time.time() - t0) / 60:.3f} minutes")
    return dict(zip(names, results))


if __name__ == "__main__":
    main(sys.argv[1:])
