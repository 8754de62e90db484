"""The golden correlation cases of picca's own test-suite
(py/picca/tests/test_3_cor.py:229-316 including the rebinned image case, :458-488, :636-664, :791-1002), as
(command-line arguments, host-side preparation) pairs shared by the oracle
and GPU parity tests."""

import os

from picca_gb300 import constants, io, prep_del, utils
from picca_gb300.forests import ForestSet

CASES = {
    "cf": dict(kind="cf", in_dir="Delta_LYA", args=[
        "--rp-min", "0.0", "--rp-max", "60.0", "--rt-max", "60.0", "--np", "15", "--nt", "15",
        "--remove-same-half-plate-close-pairs"]),
    "cf_zcuts": dict(kind="cf", in_dir="Delta_LYA", args=[
        "--rp-min", "0.0", "--rp-max", "60.0", "--rt-max", "60.0", "--np", "15", "--nt", "15",
        "--remove-same-half-plate-close-pairs", "--z-min-pairs", "2.25", "--z-max-pairs", "2.3",
        "--z-min-sources", "2.3", "--z-max-sources", "2.5"]),
    "cf_cross": dict(kind="cf", in_dir="Delta_LYA", in_dir2="Delta_LYA", args=[
        "--rp-min", "-60.0", "--rp-max", "60.0", "--rt-max", "60.0", "--np", "30", "--nt", "15",
        "--remove-same-half-plate-close-pairs", "--unfold-cf"]),
    "cf_cross_zcuts": dict(kind="cf", in_dir="Delta_LYA", in_dir2="Delta_LYA", args=[
        "--rp-min", "-60.0", "--rp-max", "60.0", "--rt-max", "60.0", "--np", "30", "--nt", "15",
        "--remove-same-half-plate-close-pairs", "--unfold-cf", "--z-min-pairs", "2.25",
        "--z-max-pairs", "2.3", "--z-min-sources", "2.3", "--z-max-sources", "2.5"]),
    "cf_image": dict(kind="cf", in_dir="Delta_LYA_image", args=[
        "--rp-min", "0.0", "--rp-max", "60.0", "--rt-max", "60.0", "--np", "15", "--nt", "15"]),
    "cf_image_rebinned": dict(kind="cf", in_dir="Delta_LYA_image", args=[
        "--rp-min", "0.0", "--rp-max", "60.0", "--rt-max", "60.0", "--np", "15", "--nt", "15",
        "--rebin-factor", "3"]),
    "cf_image_zcuts": dict(kind="cf", in_dir="Delta_LYA_image", args=[
        "--rp-min", "0.0", "--rp-max", "60.0", "--rt-max", "60.0", "--np", "15", "--nt", "15",
        "--z-min-pairs", "2.25", "--z-max-pairs", "2.3", "--z-min-sources", "2.3",
        "--z-max-sources", "2.5"]),
    "xcf": dict(kind="xcf", in_dir="Delta_LYA", args=[
        "--rp-min", "-60.0", "--rp-max", "60.0", "--rt-max", "60.0", "--np", "30", "--nt", "15",
        "--z-evol-obj", "1."]),
    "xcf_zcuts": dict(kind="xcf", in_dir="Delta_LYA", args=[
        "--rp-min", "-60.0", "--rp-max", "60.0", "--rt-max", "60.0", "--np", "30", "--nt", "15",
        "--z-evol-obj", "1.", "--z-min-pairs", "2.25", "--z-max-pairs", "2.3",
        "--z-min-sources", "2.3", "--z-max-sources", "2.5"]),
}


# picca's golden distortion matrices (py/picca/tests/test_3_cor.py:318-347,
# :489-520, :666-697, :858-1039): the correlation case whose flags they share,
# plus the random rejection and no redshift evolution.
DMAT_CASES = {"dmat": "cf", "dmat_zcuts": "cf_zcuts", "dmat_cross": "cf_cross",
              "dmat_cross_zcuts": "cf_cross_zcuts", "xdmat": "xcf", "xdmat_zcuts": "xcf_zcuts"}
DMAT_ARGS = ["--rej", "0.99", "--no-redshift-evolution"]


def dmat_cli_args(case, base, out):
    """Full command line of the picca_dmat / picca_xdmat drop-in."""
    return cli_args(DMAT_CASES[case], base, out) + DMAT_ARGS


def cli_args(case, base, out):
    """Full command line for the drop-in CLI."""
    spec = CASES[case]
    args = ["--in-dir", os.path.join(base, spec["in_dir"]) + "/", "--out", out,
            "--nproc", "1", "--in-attributes", os.path.join(base, "delta_attributes.fits.gz")]
    if "in_dir2" in spec:
        args += ["--in-dir2", os.path.join(base, spec["in_dir2"]) + "/"]
    if spec["kind"] == "xcf":
        args += ["--drq", os.path.join(base, "cat.fits")]
    return args + spec["args"]


def _opt(args, name, default, cast=float):
    return cast(args[args.index(name) + 1]) if name in args else default


def prepare(case, base):
    """Host-side preparation identical to the CLIs: returns (set1, set2 or
    None, params dict, ang_max, kind)."""
    spec = CASES[case]
    args = spec["args"]
    attributes = os.path.join(base, "delta_attributes.fits.gz")
    cosmo = constants.Cosmo(Om=0.315, verbose=False)
    z_min_src = _opt(args, "--z-min-sources", 0.0)
    z_max_src = _opt(args, "--z-max-sources", 10.0)
    params = dict(
        r_par_min=_opt(args, "--rp-min", 0.0), r_par_max=_opt(args, "--rp-max", 200.0),
        r_trans_max=_opt(args, "--rt-max", 200.0), num_bins_r_par=_opt(args, "--np", 50, int),
        num_bins_r_trans=_opt(args, "--nt", 50, int),
        z_min_pairs=_opt(args, "--z-min-pairs", None), z_max_pairs=_opt(args, "--z-max-pairs", None),
        x_correlation="--unfold-cf" in args,
        remove_same_half_plate_close_pairs="--remove-same-half-plate-close-pairs" in args)
    data, _, z_min, z_max = io.read_deltas(
        os.path.join(base, spec["in_dir"]) + "/", 16, constants.ABSORBER_IGM["LYA"], 2.9, 2.25,
        cosmo, z_min_qso=z_min_src, z_max_qso=z_max_src, delta_attributes=attributes,
        rebin_factor=_opt(args, "--rebin-factor", None, int))
    if spec["kind"] == "cf":
        ang_max = utils.compute_ang_max(cosmo, params["r_trans_max"], z_min)
        set2 = None
        if "in_dir2" in spec:
            data2, _, z_min2, _ = io.read_deltas(
                os.path.join(base, spec["in_dir2"]) + "/", 16, constants.ABSORBER_IGM["LYA"],
                2.9, 2.25, cosmo, z_min_qso=z_min_src, z_max_qso=z_max_src,
                delta_attributes=attributes)
            ang_max = utils.compute_ang_max(cosmo, params["r_trans_max"], z_min, z_min2)
            set2 = ForestSet.from_deltas(data2)
        return ForestSet.from_deltas(data), set2, params, ang_max, "cf"
    objs, z_min2 = io.read_objects(os.path.join(base, "cat.fits"), 16, 0, 10,
                                   _opt(args, "--z-evol-obj", 1.44), 2.25, cosmo)
    prep_del.remove_mean_lambda_obs(data, z_min, z_max, constants.ABSORBER_IGM["LYA"])
    ang_max = utils.compute_ang_max(cosmo, params["r_trans_max"], z_min, z_min2)
    return ForestSet.from_deltas(data), ForestSet.from_objects(objs), params, ang_max, "xcf"
