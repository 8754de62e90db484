"""GPU parity of the fast metal distortion matrices (pg_fast_metal_dmat
through the C ABI): the picca_fast_metal_dmat.py / picca_fast_metal_xdmat.py
drop-ins against picca's golden fast_metal_dmat, fast_metal_dmat_cross and
fast_metal_xdmat files (the reference's tolerance, rtol 1e-5 / atol 1e-8),
and the pair histograms against the NumPy oracle on synthetic stacks: every
pair must land in numpy's bin, so the histograms agree to FP64 summation
order (|got - want| <= 1e-10 |want| + 1e-12 max|want|) and the ratio edges
exactly. Cases: folded and signed r_par, rebinning, a second stack, a
constant distance ratio (numpy widens the range by 1/2 each way), an empty
side, and an r_par matrix too large for shared memory."""

import os

import numpy as np
import pytest

from conftest import golden, write_catalogue, write_delta_dir, write_stack_attributes
from oracle import fast_metal as ofm
from test_oracle_golden import compare_like_reference

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return torch


@pytest.fixture(scope="module")
def inputs(tmp_path_factory):
    base = str(tmp_path_factory.mktemp("fast_metal"))
    os.makedirs(os.path.join(base, "Log"))
    write_stack_attributes(os.path.join(base, "Log", "delta_attributes.fits.gz"))
    write_delta_dir(os.path.join(base, "Delta"))
    write_catalogue(os.path.join(base, "cat.fits"))
    return base


def read_mdmat(path):
    from picca_gb300 import fitsio_lite
    with fitsio_lite.FITS(path) as h:
        names = [x.decode() if isinstance(x, bytes) else str(x) for x in h["ATTRI"]["ABS_IGM"][:]]
        cols = {c: h["MDMAT"][c][:] for c in h["MDMAT"].get_colnames()}
    return names, cols


@pytest.mark.parametrize("case,extra", [
    ("cor_fast_metal_dmat", ["--rp-min", "+0.0", "--np", "15"]),
    ("cor_fast_metal_dmat_cross", ["--rp-min", "-60.0", "--np", "30", "--unfold-cf",
                                   "--abs-igm2", "SiIII(1207)"]),
])
def test_cli_matches_golden_auto(cuda, inputs, tmp_path, case, extra):
    from picca_gb300.bin import picca_fast_metal_dmat
    out = str(tmp_path / "fast_metal_dmat.fits.gz")
    attributes = os.path.join(inputs, "Log", "delta_attributes.fits.gz")
    args = ["--in-attributes", attributes, "--out", out, "--abs-igm", "SiIII(1207)",
            "--rp-max", "+60.0", "--rt-max", "+60.0", "--nt", "15"] + extra
    if case.endswith("cross"):
        args += ["--in-attributes2", attributes]
    picca_fast_metal_dmat.main(args)
    want = golden(case + ".npz")
    names, cols = read_mdmat(out)
    assert names == [str(x) for x in want["ABS_IGM"]]
    assert sorted(cols) == sorted(k for k in want if k != "ABS_IGM")
    compare_like_reference(cols, want, names=tuple(cols))


def test_cli_matches_golden_cross(cuda, inputs, tmp_path):
    from picca_gb300.bin import picca_fast_metal_xdmat
    out = str(tmp_path / "fast_metal_xdmat.fits.gz")
    picca_fast_metal_xdmat.main([
        "--in-attributes", os.path.join(inputs, "Log", "delta_attributes.fits.gz"),
        "--drq", os.path.join(inputs, "cat.fits"), "--out", out, "--abs-igm", "SiIII(1207)",
        "--rp-min", "-60.0", "--rp-max", "+60.0", "--rt-max", "+60.0", "--np", "30",
        "--nt", "15", "--z-evol-obj", "1."])
    want = golden("cor_fast_metal_xdmat.npz")
    names, cols = read_mdmat(out)
    assert names == ["SiIII(1207)"]
    assert sorted(cols) == sorted(k for k in want if k != "ABS_IGM")
    compare_like_reference(cols, want, names=tuple(cols))


def close(got, want, rtol=1e-10, scale_tol=1e-12):
    got, want = np.asarray(got, dtype=np.float64), np.asarray(want, dtype=np.float64)
    assert got.shape == want.shape
    scale = float(np.max(np.abs(want))) if want.size else 0.0
    err = np.abs(got - want)
    assert np.all(err <= rtol * np.abs(want) + scale_tol * scale), float(err.max())


def synthetic_stack(seed, n, lo=3.56, step=3e-4):
    rng = np.random.default_rng(seed)
    log_lambda = lo + step * np.arange(n)
    weight = rng.uniform(20.0, 90.0, n)
    weight[rng.random(n) < 0.2] = 0.0
    return log_lambda, weight


def compare_histograms(engine, s1, s2, rp_min, rp_max, np_, nt, signed):
    want = ofm.histograms(s1, s2, rp_min, rp_max, np_, nt, signed)
    got = engine.histograms(s1, s2, rp_min, rp_max, np_, nt, signed)
    assert np.array_equal(got["ratio_edges"], want["ratio_edges"])
    for key in ("rp_dmat", "ratio_weights", "out_weight", "out_weight_rp", "out_weight_z"):
        close(got[key], want[key])
    from picca_gb300 import fast_metal
    for g, w in zip(fast_metal.finish(got, 80.0, np_, nt), ofm.finish(want, 80.0, np_, nt)):
        close(g, w, rtol=1e-9, scale_tol=1e-11)


@pytest.mark.parametrize("signed,rebin,rp_min,np_,nt", [
    (False, None, 0.0, 20, 16),
    (False, 3, -40.0, 40, 20),
    (True, None, -80.0, 32, 16),
    (True, 2, -80.0, 170, 12),  # r_par matrix in global memory
])
def test_histograms_match_oracle(cuda, signed, rebin, rp_min, np_, nt):
    from picca_gb300 import constants, fast_metal
    c = constants.Cosmo(Om=0.3147, verbose=False)
    A = constants.ABSORBER_IGM
    engine = fast_metal.FastMetalEngine()
    ll1, w1 = synthetic_stack(3, 1700)
    ll2, w2 = synthetic_stack(4, 1300, lo=3.57)
    s1 = fast_metal.stack_side(ll1, w1, A["SiII(1260)"], A["LYA"], 3.9, c, rebin)
    s2 = fast_metal.stack_side(ll2, w2, A["LYA"], A["LYA"], 5.8, c, rebin)
    compare_histograms(engine, s1, s2, rp_min, 80.0, np_, nt, signed)
    # the product and the oracle prepare the sides the same way
    o1 = ofm.stack_side(ll1, w1, A["SiII(1260)"], A["LYA"], 3.9, c, rebin)
    for key in ("r_in", "r_out", "z_in", "w"):
        assert np.array_equal(o1[key], s1[key])


def test_quasar_side_and_edge_cases(cuda):
    from picca_gb300 import constants, fast_metal
    c = constants.Cosmo(Om=0.3147, verbose=False)
    A = constants.ABSORBER_IGM
    engine = fast_metal.FastMetalEngine()
    rng = np.random.default_rng(9)
    z_qso = rng.uniform(2.0, 3.6, 5000)
    zh, wh = fast_metal.quasar_histogram(z_qso, ((1 + z_qso) / 3.25)**0.44, 700)
    q = fast_metal.quasar_side(zh, wh, c)
    ll, w = synthetic_stack(5, 900)
    s = fast_metal.stack_side(ll, w, A["SiIII(1207)"], A["LYA"], 3.9, c)
    compare_histograms(engine, s, q, -60.0, 60.0, 30, 15, True)
    # one pixel per side: a single distance ratio, range widened to +-1/2
    one = {k: v[:1] for k, v in s.items()}
    compare_histograms(engine, one, {k: v[:1] for k, v in q.items()}, -60.0, 60.0, 30, 15, True)
    # an empty side: numpy's empty-range edges (0, 1) and zero sums
    empty = {k: v[:0] for k, v in s.items()}
    got = engine.histograms(empty, q, -60.0, 60.0, 30, 15, True)
    assert np.array_equal(got["ratio_edges"], np.linspace(0, 1, 4 * 16 + 1))
    assert not np.any(got["rp_dmat"]) and not np.any(got["out_weight"])
