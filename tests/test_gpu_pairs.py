"""GPU parity of the pair accumulation (through the C ABI).

* Function level: the 20/16-argument ``compute_xi_forest_pairs_fast`` drop-ins
  against picca's own functions (golden pair cases), both arithmetic modes.
* CLI level: ``picca_cf.py`` / ``picca_xcf.py`` drop-ins against picca's
  golden correlation files (reference rule rtol 1e-5 / atol 1e-8; exact NB).
* Oracle level: neighbour lists identical to the CPU oracle's, per-healpix
  pair counts identical, sums within 1e-12 (FP64 mode) and within the
  precision-form tolerance (FP32 geometry + FP64 guard) on synthetic forests.

Tolerances: FP64 mode sums differ from the oracle only by summation order
(rtol 1e-12). FP32_GUARD mode: pair counts and bin decisions bit-exact; the
weight, r_par, r_trans and z sums within rtol 2e-6 per healpix row and bin;
xi (delta*w carried as an FP32 hi/lo pair, products and run sums
error-compensated) within 1e-6 relative of the oracle's xi in every bin with
pairs, and within 1e-10 of the bin's sum of |delta1 w1 delta2 w2| (the
oracle on |delta|). The golden CLI comparison in FP32_GUARD mode uses the
reference rule.
"""

import importlib
import os

import numpy as np
import pytest

from conftest import golden
from corr_cases import CASES, cli_args, prepare
from test_oracle_golden import compare_like_reference

pytestmark = pytest.mark.gpu

MODES = ("fp64", "fp32_guard")


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from picca_gb300 import build_ext
    build_ext.build()
    return torch


def _set_cf_globals(cf, p):
    cf.r_par_min, cf.r_par_max, cf.r_trans_max = p[0], p[1], p[2]
    cf.num_bins_r_par, cf.num_bins_r_trans = int(p[3]), int(p[4])
    cf.z_min_pairs = None if np.isnan(p[5]) else float(p[5])
    cf.z_max_pairs = None if np.isnan(p[6]) else float(p[6])
    cf.zerr_cut_deg = None if np.isnan(p[7]) else float(p[7])
    cf.zerr_cut_kms = None if np.isnan(p[8]) else float(p[8])
    cf.x_correlation = bool(p[9])
    cf.rmu_binning = bool(p[10])
    cf.ang_correlation = bool(p[11])
    cf.remove_same_half_plate_close_pairs = bool(p[12])


def _cf_abs_sum(f, pre):
    """Per-bin sum of |delta1 w1 delta2 w2| of a golden case (oracle on |delta|)."""
    from oracle import cpu as oracle
    from test_oracle_golden import _cf_case_params
    params = _cf_case_params(f[pre + "params"])
    nbins = params.num_bins_r_par * params.num_bins_r_trans
    outs = [np.zeros(nbins) for _ in range(5)] + [np.zeros(nbins, dtype=np.int64)]
    zq1, zq2, ang, shp = f[pre + "scalars"]
    oracle.cf_forest_pair(params, f[pre + "z1"], f[pre + "r1"], f[pre + "m1"], f[pre + "w1"],
                          np.abs(f[pre + "d1"]), zq1, f[pre + "z2"], f[pre + "r2"], f[pre + "m2"],
                          f[pre + "w2"], np.abs(f[pre + "d2"]), zq2, ang, bool(shp), outs)
    return np.abs(outs[1])


@pytest.mark.parametrize("precision", MODES)
def test_cf_pair_function_gpu(cuda, precision):
    from picca_gb300 import cf
    f = golden("pair_cases.npz")
    cf.precision = precision
    for k in range(int(f["num_cf_cases"])):
        pre = f"cf{k}_"
        _set_cf_globals(cf, f[pre + "params"])
        nbins = cf.num_bins_r_par * cf.num_bins_r_trans
        outs = [np.zeros(nbins) for _ in range(5)] + [np.zeros(nbins, dtype=np.int64)]
        zq1, zq2, ang, shp = f[pre + "scalars"]
        cf.compute_xi_forest_pairs_fast(
            f[pre + "z1"], f[pre + "r1"], f[pre + "m1"], f[pre + "w1"], f[pre + "d1"], zq1,
            f[pre + "z2"], f[pre + "r2"], f[pre + "m2"], f[pre + "w2"], f[pre + "d2"], zq2,
            ang, bool(shp), *outs)
        name = str(f[pre + "name"])
        assert np.array_equal(outs[5], f[pre + "out_nb"]), (k, name, precision)
        rtol = 1e-12 if precision == "fp64" else 2e-6
        for key, got in zip(("we", "rp", "rt", "z"), (outs[0], outs[2], outs[3], outs[4])):
            want = f[pre + "out_" + key]
            assert np.allclose(got, want, rtol=rtol, atol=0), (k, name, key)
        want_xi = f[pre + "out_xi"]
        abs_sum = _cf_abs_sum(f, pre)
        err = np.abs(outs[1] - want_xi)
        has = f[pre + "out_nb"] > 0
        if precision != "fp64":  # FP64: same terms summed in another order (bound below)
            assert np.all(err[has] <= 1e-6 * np.abs(want_xi[has])), (k, name, "xi")
        xtol = 1e-12 if precision == "fp64" else 1e-10
        assert np.all(err <= xtol * abs_sum + 1e-300), (k, name, "xi")


@pytest.mark.parametrize("precision", MODES)
def test_xcf_pair_function_gpu(cuda, precision):
    from picca_gb300 import xcf
    f = golden("pair_cases.npz")
    xcf.precision = precision
    for k in range(int(f["num_xcf_cases"])):
        pre = f"xcf{k}_"
        p = f[pre + "params"]
        xcf.r_par_min, xcf.r_par_max, xcf.r_trans_max = p[0], p[1], p[2]
        xcf.num_bins_r_par, xcf.num_bins_r_trans = int(p[3]), int(p[4])
        xcf.z_min_pairs = None if np.isnan(p[5]) else float(p[5])
        xcf.z_max_pairs = None if np.isnan(p[6]) else float(p[6])
        xcf.rmu_binning = bool(p[7])
        xcf.ang_correlation = False
        xcf.zerr_cut_deg = xcf.zerr_cut_kms = None
        nbins = xcf.num_bins_r_par * xcf.num_bins_r_trans
        outs = [np.zeros(nbins) for _ in range(5)] + [np.zeros(nbins, dtype=np.int64)]
        xcf.compute_xi_forest_pairs_fast(
            f[pre + "z1"], f[pre + "r1"], f[pre + "m1"], f[pre + "w1"], f[pre + "d1"],
            f[pre + "zq"], f[pre + "rq"], f[pre + "mq"], f[pre + "wq"], f[pre + "ang"], *outs)
        name = str(f[pre + "name"])
        assert np.array_equal(outs[5], f[pre + "out_nb"]), (k, name, precision)
        rtol = 1e-12 if precision == "fp64" else 2e-6
        for key, idx in (("we", 0), ("rp", 2), ("rt", 3), ("z", 4)):
            want = f[pre + "out_" + key]
            assert np.allclose(outs[idx], want, rtol=rtol, atol=1e-9 if key == "rp" else 0), (
                k, name, key)
        has = f[pre + "out_nb"] > 0
        want_xi = f[pre + "out_xi"]
        xrel = 1e-9 if precision == "fp64" else 1e-6
        assert np.all(np.abs(outs[1] - want_xi)[has] <= xrel * np.abs(want_xi[has]) + 1e-300), (
            k, name, "xi")


@pytest.mark.parametrize("precision", MODES)
@pytest.mark.parametrize("case", sorted(CASES))
def test_cli_matches_golden(cuda, picca_inputs, tmp_path, case, precision):
    from picca_gb300 import fitsio_lite
    from picca_gb300.bin import picca_cf, picca_xcf
    import picca_gb300.cf
    import picca_gb300.xcf
    importlib.reload(picca_gb300.cf)
    importlib.reload(picca_gb300.xcf)
    out = os.path.join(tmp_path, f"{case}.fits.gz")
    args = cli_args(case, picca_inputs, out) + ["--precision", precision]
    if CASES[case]["kind"] == "cf":
        picca_cf.main(args)
    else:
        picca_xcf.main(args)
    hdul = fitsio_lite.FITS(out)
    got = {c: hdul["ATTRI"][c][:] for c in ("RP", "RT", "Z", "NB")}
    got.update({c: hdul["COR"][c][:] for c in ("HEALPID", "WE", "DA")})
    want = golden(f"cor_{case}.npz")
    compare_like_reference(got, want)


def _synthetic_sets(seed=7, num=600, xcf=False, grid="log"):
    from picca_gb300 import synthetic
    fs = synthetic.make_forests(num, seed, (150.0, 156.0), (0.0, 6.0), 2.1, 3.5, "uniform",
                                grid=grid)
    if xcf:
        qs = synthetic.make_quasars(int(num * 1.5), seed + 1, (150.0, 156.0), (0.0, 6.0))
        return fs, qs
    return fs, None


@pytest.mark.parametrize("precision", MODES)
@pytest.mark.parametrize("variant", ["auto", "cross", "auto_cuts", "auto_lin", "auto_rmu",
                                     "cross_rmu"])
def test_cf_gpu_matches_oracle_synthetic(cuda, precision, variant):
    """``auto_lin``: forests on the DESI-like linear grid (0.8 Angstrom,
    150-600 pixels), which the pair kernel stages in several chunks.
    ``*_rmu``: r-mu bins (--rmu-binning; mu in [0, 1] for the auto, [-1, 1]
    for two fields), which the precision form computes per pair from the
    staged coordinates."""
    from oracle import cpu as oracle
    from picca_gb300 import pairs, synthetic
    fs, _ = _synthetic_sets(grid="lin" if variant == "auto_lin" else "log",
                            num=300 if variant == "auto_lin" else 600)
    if variant == "auto_lin":
        npix = np.diff(fs.pix_offset)
        assert npix.max() > 400 and npix.min() >= 150
    fs2 = None
    kwargs = dict(r_par_min=0.0, r_par_max=200.0, r_trans_max=200.0, num_bins_r_par=50,
                  num_bins_r_trans=50)
    if variant in ("cross", "cross_rmu"):
        fs2 = synthetic.make_forests(500, 99, (150.0, 156.0), (0.0, 6.0), 2.1, 3.5, "uniform",
                                     thingid_start=5000)
        kwargs.update(r_par_min=-200.0, num_bins_r_par=100, x_correlation=True)
    if variant == "auto_rmu":
        kwargs.update(r_par_min=0.0, r_par_max=1.0, rmu_binning=True)
    if variant == "cross_rmu":
        kwargs.update(r_par_min=-1.0, r_par_max=1.0, rmu_binning=True)
    if variant == "auto_cuts":
        fs.plate[:] = np.arange(fs.num) % 3
        fs.fiberid[:] = (np.arange(fs.num) * 37) % 1000
        kwargs.update(z_min_pairs=2.2, z_max_pairs=2.6, zerr_cut_deg=3.0, zerr_cut_kms=1500.0,
                      remove_same_half_plate_close_pairs=True)
    ang_max = synthetic.correlation_ang_max(200.0, float(fs.z.min()))
    p_or = oracle.make_params(**kwargs)
    offsets, index = oracle.neighbours(fs, fs2 if fs2 is not None else fs, p_or, ang_max,
                                       auto_mode=int(fs2 is None))
    ref = oracle.rows(fs, fs2 if fs2 is not None else fs, p_or, offsets, index)
    ref_abs = oracle.rows(_abs_delta(fs), _abs_delta(fs2 if fs2 is not None else fs), p_or,
                          offsets, index)
    mode = pairs.MODE_FP64 if precision == "fp64" else pairs.MODE_FP32_GUARD
    res = pairs.correlate(fs, fs2, pairs.make_params(ang_max=ang_max, **kwargs), mode=mode)
    # neighbour lists identical
    assert np.array_equal(res["offsets"].cpu().numpy(), offsets)
    assert np.array_equal(res["index"].cpu().numpy()[: res["num_pairs_forest"]], index)
    _compare_rows(res["raw"], ref, ref_abs[1], precision)


@pytest.mark.parametrize("precision", MODES)
@pytest.mark.parametrize("grid", ["log", "lin"])
def test_xcf_gpu_matches_oracle_synthetic(cuda, precision, grid):
    from oracle import cpu as oracle
    from picca_gb300 import pairs, synthetic
    fs, qs = _synthetic_sets(xcf=True, grid=grid, num=600 if grid == "log" else 300)
    kwargs = dict(r_par_min=-200.0, r_par_max=200.0, r_trans_max=200.0, num_bins_r_par=100,
                  num_bins_r_trans=50)
    ang_max = synthetic.correlation_ang_max(200.0, float(fs.z.min()))
    p_or = oracle.make_params(**kwargs)
    offsets, index = oracle.neighbours(fs, qs, p_or, ang_max, auto_mode=0, xcf=True)
    ref = oracle.rows(fs, qs, p_or, offsets, index, xcf=True)
    ref_abs = oracle.rows(_abs_delta(fs), qs, p_or, offsets, index, xcf=True)
    mode = pairs.MODE_FP64 if precision == "fp64" else pairs.MODE_FP32_GUARD
    res = pairs.correlate(fs, qs, pairs.make_params(ang_max=ang_max, x_correlation=True,
                                                    **kwargs), mode=mode, xcf=True)
    assert np.array_equal(res["offsets"].cpu().numpy(), offsets)
    assert np.array_equal(res["index"].cpu().numpy()[: res["num_pairs_forest"]], index)
    _compare_rows(res["raw"], ref, ref_abs[1], precision)


def _abs_delta(fs):
    import copy
    out = copy.copy(fs)
    out.delta = np.abs(fs.delta)
    return out


def _compare_rows(got, ref, abs_sum, precision):
    we, xi, rp, rt, zz, nb = got
    r_we, r_xi, r_rp, r_rt, r_zz, r_nb = ref
    assert np.array_equal(nb, r_nb), "pair counts differ"
    rtol = 1e-12 if precision == "fp64" else 2e-6
    for name, a, b in (("we", we, r_we), ("rp", rp, r_rp), ("rt", rt, r_rt), ("z", zz, r_zz)):
        assert np.allclose(a, b, rtol=rtol, atol=1e-300), (name, np.max(np.abs(a - b)))
    # xi: per bin relative to the oracle's xi, and against the sum of |terms|
    err = np.abs(xi - r_xi)
    has = r_nb > 0
    if precision != "fp64":  # FP64: same terms summed in another order (bound below)
        assert np.all(err[has] <= 1e-6 * np.abs(r_xi[has])), \
            np.max(err[has] / np.maximum(np.abs(r_xi[has]), 1e-300))
    xtol = 1e-12 if precision == "fp64" else 1e-10
    assert np.all(err <= xtol * np.abs(abs_sum) + 1e-300), np.max(err / (np.abs(abs_sum) + 1e-300))
