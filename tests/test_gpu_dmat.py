"""GPU parity of the distortion matrix (pg_cf_dmat through the C ABI).

* Function level: the 22-argument ``cf.compute_dmat_forest_pairs_fast``
  drop-in against picca's own function on the golden forest-pair cases
  (same-half-plate veto, redshift evolution, model binning twice as fine,
  order 0, z and velocity cuts).
* CLI level: the ``picca_dmat.py`` and ``picca_xdmat.py`` drop-ins against
  picca's six golden distortion matrices (auto, z cuts, the cross of two
  delta sets with and without z cuts, delta x quasar with and without z
  cuts; reference rule rtol 1e-5 / atol 1e-8; NPALL and NPUSED exact).
* The 17-argument ``xcf.compute_dmat_forest_pairs_fast`` drop-in against
  picca's own function on the golden xcf cases.
* Oracle level: synthetic forests with several process chunks, random
  plates (same-half-plate vetoes), z cuts, redshift evolution, r-mu binning
  and a forced split of each forest pair's bins into chunks.

Both arithmetic forms of the eta products are checked: FP64 on the CUDA
cores, and the tensor-core form (rows scaled by powers of two, 48-bit fixed
point split into six 8-bit digits, exact digit products, error below 2^-46
of the largest row x column product). Tolerance: the kernel regroups the
reference's sums (the eta projections become a product of per-bin and
per-pixel partial sums, added with atomics), so results differ from the
oracle by rounding only: |got - want| <= 1e-9 |want| + 1e-11 max|want| per
array.
"""

import os

import numpy as np
import pytest

from conftest import golden
from corr_cases import DMAT_CASES, dmat_cli_args
from oracle import cpu
from oracle import dmat as odm
from test_oracle_golden import compare_like_reference

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return torch


def close(got, want, rtol=1e-9, scale_tol=1e-11):
    got, want = np.asarray(got), np.asarray(want)
    assert got.shape == want.shape
    scale = float(np.max(np.abs(want))) if want.size else 0.0
    err = np.abs(got - want)
    bound = rtol * np.abs(want) + scale_tol * scale
    return bool(np.all(err <= bound)), float(np.max(err) if err.size else 0.0)


@pytest.mark.parametrize("product", ["split_bf16", "fp64"])
def test_forest_pair_cases_match_reference(cuda, product):
    from picca_gb300 import cf
    cf.dmat_product = product
    f = golden("dmat_cases.npz")
    for k in range(int(f["num_cases"])):
        pre = f"dm{k}_"
        p = f[pre + "params"]
        nan_none = lambda v: None if np.isnan(v) else float(v)  # noqa: E731
        cf.r_par_min, cf.r_par_max, cf.r_trans_max = 0., 60., 60.
        cf.num_bins_r_par, cf.num_bins_r_trans = int(p[0]), int(p[1])
        cf.num_model_bins_r_par = int(p[0]) * int(p[2])
        cf.num_model_bins_r_trans = int(p[1]) * int(p[2])
        cf.remove_same_half_plate_close_pairs = bool(p[3])
        cf.redshift_evolution_in_distortion_matrix = bool(p[4])
        cf.z_min_pairs, cf.z_max_pairs = nan_none(p[7]), nan_none(p[8])
        cf.zerr_cut_deg, cf.zerr_cut_kms = nan_none(p[9]), nan_none(p[10])
        cf.x_correlation = False
        cf.rmu_binning = False
        cf.z_ref, cf.alpha, cf.alpha2 = 2.25, 2.9, 2.9
        nb = cf.num_bins_r_par * cf.num_bins_r_trans
        nm = cf.num_model_bins_r_par * cf.num_model_bins_r_trans
        out = {"weights_dmat": np.zeros(nb), "dmat": np.zeros(nb * nm), "r_par_eff": np.zeros(nm),
               "r_trans_eff": np.zeros(nm), "z_eff": np.zeros(nm), "weight_eff": np.zeros(nm)}
        zq1, zq2, ang, shp = f[pre + "scalars"]
        cf.compute_dmat_forest_pairs_fast(
            f[pre + "ll1"], f[pre + "ll2"], f[pre + "r1"], f[pre + "r2"], f[pre + "m1"],
            f[pre + "m2"], f[pre + "z1"], f[pre + "z2"], f[pre + "w1"], f[pre + "w2"], zq1, zq2,
            ang, out["weights_dmat"], out["dmat"], out["r_par_eff"], out["r_trans_eff"],
            out["z_eff"], out["weight_eff"], bool(shp), int(p[5]), int(p[6]))
        for key, got in out.items():
            ok, err = close(got, f[pre + "out_" + key])
            assert ok, (product, k, key, err)
    cf.dmat_product = "split_bf16"


@pytest.mark.parametrize("case", sorted(DMAT_CASES))
def test_cli_matches_golden_dmat(cuda, case, picca_inputs, tmp_path):
    from picca_gb300 import fitsio_lite
    from picca_gb300.bin import picca_dmat, picca_xdmat
    out = str(tmp_path / f"{case}.fits.gz")
    cli = picca_xdmat if DMAT_CASES[case].startswith("xcf") else picca_dmat
    cli.main(dmat_cli_args(case, picca_inputs, out))
    with fitsio_lite.FITS(out) as h:
        dm = h["DMAT"]
        hdr = dm.read_header()
        got = {"WDM": dm["WDM"][:], "DM": dm["DM"][:], "RP": h["ATTRI"]["RP"][:],
               "RT": h["ATTRI"]["RT"][:], "Z": h["ATTRI"]["Z"][:]}
    want = golden(f"cor_{case}.npz")
    assert int(hdr["NPALL"]) == int(want["hdr_NPALL"])
    assert int(hdr["NPUSED"]) == int(want["hdr_NPUSED"])
    compare_like_reference(got, want, names=("WDM", "DM", "RP", "RT", "Z"))


@pytest.mark.parametrize("product", ["split_bf16", "fp64"])
def test_xcf_forest_cases_match_reference(cuda, product):
    from picca_gb300 import xcf
    xcf.dmat_product = product
    f = golden("xdmat_cases.npz")
    for k in range(int(f["num_cases"])):
        pre = f"xd{k}_"
        p = f[pre + "params"]
        nan_none = lambda v: None if np.isnan(v) else float(v)  # noqa: E731
        xcf.r_par_min, xcf.r_par_max, xcf.r_trans_max = -60., 60., 60.
        xcf.num_bins_r_par, xcf.num_bins_r_trans = int(p[0]), int(p[1])
        xcf.num_model_bins_r_par = int(p[0]) * int(p[2])
        xcf.num_model_bins_r_trans = int(p[1]) * int(p[2])
        xcf.redshift_evolution_in_distortion_matrix = bool(p[3])
        xcf.z_min_pairs, xcf.z_max_pairs = nan_none(p[5]), nan_none(p[6])
        xcf.rmu_binning = False
        xcf.z_ref, xcf.alpha, xcf.alpha_obj = 2.25, 2.9, 1.44
        nb = xcf.num_bins_r_par * xcf.num_bins_r_trans
        nm = xcf.num_model_bins_r_par * xcf.num_model_bins_r_trans
        out = {"weights_dmat": np.zeros(nb), "dmat": np.zeros(nb * nm), "r_par_eff": np.zeros(nm),
               "r_trans_eff": np.zeros(nm), "z_eff": np.zeros(nm), "weight_eff": np.zeros(nm)}
        xcf.compute_dmat_forest_pairs_fast(
            f[pre + "ll1"], f[pre + "r1"], f[pre + "m1"], f[pre + "z1"], f[pre + "w1"],
            f[pre + "r2"], f[pre + "m2"], f[pre + "z2"], f[pre + "w2"], f[pre + "ang"],
            out["weights_dmat"], out["dmat"], out["r_par_eff"], out["r_trans_eff"],
            out["z_eff"], out["weight_eff"], int(p[4]))
        for key, got in out.items():
            ok, err = close(got, f[pre + "out_" + key])
            assert ok, (product, k, key, err)
    xcf.dmat_product = "split_bf16"


def _synthetic(seed=7, num=160):
    from picca_gb300 import synthetic
    fs = synthetic.make_forests(num, seed, (150.0, 152.5), (0.0, 2.5), max_pixels=400)
    rng = np.random.default_rng(seed)
    fs.plate = rng.integers(0, 3, fs.num).astype(np.int64)
    fs.fiberid = rng.integers(1, 1000, fs.num).astype(np.int64)
    fs.order = rng.integers(0, 2, fs.num).astype(np.int64)
    return fs


CASES = {
    "plain": dict(np=10, nt=10, coef=1, zevol=True, shp=False, rmu=False, zcut=None, nproc=1,
                  reject=0.9),
    "coef2_chunks": dict(np=10, nt=8, coef=2, zevol=True, shp=True, rmu=False,
                         zcut=(2.3, 2.9), nproc=3, reject=0.85),
    "rmu": dict(np=10, nt=12, coef=1, zevol=False, shp=True, rmu=True, zcut=None, nproc=2,
                reject=0.9),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_synthetic_matches_oracle(cuda, case):
    from picca_gb300 import dmat, pairs
    c = CASES[case]
    fs = _synthetic()
    rp_min, rp_max, rt_max = (0., 1., 60.) if c["rmu"] else (0., 60., 60.)
    zmin, zmax = c["zcut"] if c["zcut"] else (None, None)
    oparams = odm.make_params(rp_min, rp_max, rt_max, c["np"], c["nt"],
                              coef_binning_model=c["coef"], z_min_pairs=zmin, z_max_pairs=zmax,
                              remove_same_half_plate_close_pairs=c["shp"],
                              redshift_evolution=c["zevol"], rmu_binning=c["rmu"])
    ang_max = 0.02
    # the oracle pipeline with per-forest orders
    nbr_params = cpu.make_params(rp_min, rp_max, rt_max, c["np"], c["nt"])
    offsets, index = cpu.neighbours(fs, fs, nbr_params, ang_max, auto_mode=1)
    mask, npall, npused = odm.selection(fs, offsets, c["nproc"], c["reject"])
    out = odm.new_outputs(oparams)
    po = np.asarray(fs.pix_offset)
    for f in range(fs.num):
        for k in range(int(offsets[f]), int(offsets[f + 1])):
            if not mask[k]:
                continue
            g = int(index[k])
            ang = cpu.lib().oracle_angle(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f], fs.ra[f],
                                         fs.dec[f], fs.cos_dec[f], fs.x_cart[g], fs.y_cart[g],
                                         fs.z_cart[g], fs.ra[g], fs.dec[g])
            shp = c["shp"] and fs.plate[f] == fs.plate[g] and (
                (fs.fiberid[f] <= 500) == (fs.fiberid[g] <= 500))
            a = slice(po[f], po[f + 1])
            b = slice(po[g], po[g + 1])
            odm.forest_pair(oparams, fs.log_lambda[a], fs.log_lambda[b], fs.r_comov[a],
                            fs.r_comov[b], fs.dist_m[a], fs.dist_m[b], fs.z[a], fs.z[b],
                            fs.weights[a], fs.weights[b], fs.z_qso[f], fs.z_qso[g], ang, shp,
                            int(fs.order[f]), int(fs.order[g]), out)
    assert npused > 50
    params = pairs.make_params(rp_min, rp_max, rt_max, c["np"], c["nt"], ang_max,
                               z_min_pairs=zmin, z_max_pairs=zmax, rmu_binning=c["rmu"],
                               remove_same_half_plate_close_pairs=c["shp"])
    for capacity, product in ((0, "split_bf16"), (24, "split_bf16"), (0, "fp64")):
        dparams = dmat.make_dmat_params(c["np"], c["nt"], coef_binning_model=c["coef"],
                                        redshift_evolution=c["zevol"], row_capacity=capacity,
                                        product=product)
        res = dmat.distortion_matrix(fs, None, params, dparams, c["reject"], nproc=c["nproc"])
        assert res["NPALL"] == npall and res["NPUSED"] == npused
        assert res["forest_pairs_used"] == npused
        for key in out:
            ok, err = close(res["raw"][key], out[key])
            assert ok, (case, capacity, product, key, err)


XCASES = {
    "plain": dict(np=12, nt=10, coef=1, zevol=True, rmu=False, zcut=None, nproc=1, reject=0.6),
    "coef2_zcut": dict(np=10, nt=8, coef=2, zevol=True, rmu=False, zcut=(2.2, 2.9), nproc=3,
                       reject=0.3),
    "rmu": dict(np=10, nt=12, coef=1, zevol=False, rmu=True, zcut=None, nproc=2, reject=0.8),
}


@pytest.mark.parametrize("case", sorted(XCASES))
def test_synthetic_xcf_matches_oracle(cuda, case):
    """Forests with up to several hundred kept quasars (items split at
    PG_XDMAT_MAX_OBJECTS), random orders, both products."""
    from picca_gb300 import dmat, pairs, synthetic
    c = XCASES[case]
    fs = _synthetic(seed=11, num=60)
    qs = synthetic.make_quasars(1500, 12, (150.0, 152.5), (0.0, 2.5), z_lo=2.0, z_hi=3.6)
    rp_min, rp_max, rt_max = (-1., 1., 60.) if c["rmu"] else (-60., 60., 60.)
    zmin, zmax = c["zcut"] if c["zcut"] else (None, None)
    ang_max = 0.03
    oparams = odm.make_params(rp_min, rp_max, rt_max, c["np"], c["nt"],
                              coef_binning_model=c["coef"], z_min_pairs=zmin, z_max_pairs=zmax,
                              redshift_evolution=c["zevol"], rmu_binning=c["rmu"], alpha=2.9,
                              alpha2=1.44, x_correlation=True)
    # the xcf neighbour pre-cut scales r_par by r_trans_max in r-mu binning
    nbr_params = cpu.make_params(rp_min, rp_max, rt_max, c["np"], c["nt"],
                                 rmu_binning=c["rmu"])
    offsets, index = cpu.neighbours(fs, qs, nbr_params, ang_max, auto_mode=0, xcf=True)
    mask, npall, npused = odm.xselection(fs, offsets, c["nproc"], c["reject"])
    out = odm.new_outputs(oparams)
    po = np.asarray(fs.pix_offset)
    for f in range(fs.num):
        kept = [int(index[k]) for k in range(int(offsets[f]), int(offsets[f + 1])) if mask[k]]
        if not kept:
            continue
        ang = np.array([cpu.lib().oracle_angle(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f],
                                               fs.ra[f], fs.dec[f], fs.cos_dec[f],
                                               qs.x_cart[g], qs.y_cart[g], qs.z_cart[g],
                                               qs.ra[g], qs.dec[g]) for g in kept])
        a = slice(po[f], po[f + 1])
        odm.xforest(oparams, fs.log_lambda[a], fs.r_comov[a], fs.dist_m[a], fs.z[a],
                    fs.weights[a], qs.obj_r_comov[kept], qs.obj_dist_m[kept], qs.z_qso[kept],
                    qs.obj_weight[kept], ang, int(fs.order[f]), out)
    params = pairs.make_params(rp_min, rp_max, rt_max, c["np"], c["nt"], ang_max,
                               z_min_pairs=zmin, z_max_pairs=zmax, rmu_binning=c["rmu"],
                               x_correlation=True)
    for product in ("split_bf16", "fp64"):
        dparams = dmat.make_dmat_params(c["np"], c["nt"], coef_binning_model=c["coef"],
                                        redshift_evolution=c["zevol"], alpha=2.9, alpha2=1.44,
                                        product=product)
        res = dmat.cross_distortion_matrix(fs, qs, params, dparams, c["reject"],
                                           nproc=c["nproc"])
        assert res["NPALL"] == npall and res["NPUSED"] == npused
        if case != "rmu":
            assert res["items"] > int((np.diff(offsets) > 0).sum())  # some forests split
        for key in out:
            ok, err = close(res["raw"][key], out[key])
            assert ok, (case, product, key, err)
