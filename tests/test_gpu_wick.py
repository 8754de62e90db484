"""GPU parity of the Wick covariance (pg_wick_xi_matrices and pg_cf_wick
through the C ABI): the picca_wick.py drop-in against picca's golden
wick.fits.gz (the reference's tolerance, NB / NPALL / NPUSED exact); the
weighted 1D correlation matrices bit for bit against the oracle's NumPy
expression; and the raw sums against the C oracle on synthetic forests,
folded and signed r_par, 15 x 15 and 50 x 50 bins. The GPU sums the same
FP64 products in another order and with fused multiply-adds:
|got - want| <= 1e-9 |want| + 1e-12 max|want| (NB exact)."""

import os

import numpy as np
import pytest

from conftest import golden, write_attributes, write_delta_dir
from oracle import wick as ow
from test_oracle_golden import compare_like_reference

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    return torch


def close(got, want, rtol=1e-9, scale_tol=1e-12):
    got, want = np.asarray(got, dtype=np.float64), np.asarray(want, dtype=np.float64)
    assert got.shape == want.shape
    scale = float(np.max(np.abs(want))) if want.size else 0.0
    err = np.abs(got - want)
    assert np.all(err <= rtol * np.abs(want) + scale_tol * scale), float(err.max())


def test_cli_matches_golden_wick(cuda, tmp_path):
    from picca_gb300 import fitsio_lite
    from picca_gb300.bin import picca_wick
    base = str(tmp_path)
    write_delta_dir(os.path.join(base, "Delta_LYA"))
    write_attributes(os.path.join(base, "attributes.fits.gz"))
    cf1d = golden("cf1d.npz")
    fitsio_lite.write_fits(os.path.join(base, "cf1d.fits.gz"), [{
        "columns": [cf1d[k] for k in ("v1d", "wv1d", "nv1d", "c1d", "nc1d", "nb1d")],
        "names": ["v1d", "wv1d", "nv1d", "c1d", "nc1d", "nb1d"], "extname": "1DCOR",
        "header": [{"name": "LLMIN", "value": float(cf1d["LLMIN"])},
                   {"name": "DLL", "value": float(cf1d["DLL"])}]}])
    out = os.path.join(base, "wick.fits.gz")
    picca_wick.main(["--in-dir", os.path.join(base, "Delta_LYA") + "/", "--out", out,
                     "--cf1d", os.path.join(base, "cf1d.fits.gz"), "--rp-min", "+0.0",
                     "--rp-max", "+60.0", "--rt-max", "+60.0", "--np", "15", "--nt", "15",
                     "--rej", "0.99", "--nproc", "1",
                     "--in-attributes", os.path.join(base, "attributes.fits.gz")])
    want = golden("cor_wick.npz")
    with fitsio_lite.FITS(out) as h:
        cov = h["COV"]
        header = cov.read_header()
        got = {c: cov[c][:] for c in cov.get_colnames()}
    assert int(header["NPALL"]) == int(want["hdr_NPALL"])
    assert int(header["NPUSED"]) == int(want["hdr_NPUSED"])
    assert list(got) == ["CO", "WALL", "NB", "T1", "T2", "T3", "T4", "T5", "T6"]
    compare_like_reference(got, want, names=tuple(got))


def synthetic(n, seed, max_pixels):
    from picca_gb300 import synthetic as syn
    return syn.make_forests(n, seed, (150.0, 152.0), (0.0, 2.0), max_pixels=max_pixels)


def test_xi_matrices_bitwise(cuda):
    from picca_gb300 import pairs, wick
    fs = synthetic(30, 4, 180)
    cf1d = golden("cf1d.npz")
    tables = wick.OneDTables(cf1d)
    variance, xi = ow.interpolants(cf1d)
    engine = wick.WickEngine()
    dev = pairs.DeviceForests(fs, engine.device, compact=False)
    forests = np.arange(0, fs.num, 2)
    arena, offsets, _ = engine.xi_matrices(dev, tables, forests)
    arena = arena.cpu().numpy()
    off = offsets.cpu().numpy()
    po = np.asarray(fs.pix_offset)
    for f in forests:
        sl = slice(po[f], po[f + 1])
        want = ow.weighted_xi_1d(fs.log_lambda[sl], fs.weights[sl], variance, xi)
        np.fill_diagonal(want, 0.0)
        n = po[f + 1] - po[f]
        got = arena[off[f]:off[f] + n * n].reshape(n, n)
        assert np.array_equal(got, want)


@pytest.mark.parametrize("unfold,rp_min,rp_max,np_,nt,reject,target", [
    (False, 0.0, 60.0, 15, 15, 0.6, None),
    (True, -60.0, 60.0, 30, 15, 0.6, None),
    (False, 0.0, 200.0, 50, 50, 0.9, None),
    (False, 0.0, 200.0, 50, 50, 0.9, 1e5),  # every pair cut into many slices
])
def test_synthetic_matches_oracle(cuda, monkeypatch, unfold, rp_min, rp_max, np_, nt, reject,
                                  target):
    from picca_gb300 import constants, pairs, utils, wick
    if target is not None:
        monkeypatch.setattr(wick, "SLICE_TARGET", target)
    fs = synthetic(70, 13, 220)
    cf1d = golden("cf1d.npz")
    cosmo = constants.Cosmo(Om=0.3147, verbose=False)
    ang_max = utils.compute_ang_max(cosmo, rp_max, 2.0)
    p = ow.make_params(rp_min, rp_max, rp_max, np_, nt, x_correlation=unfold)
    want = ow.pipeline(fs, p, ang_max, cf1d, reject, nproc=2, return_raw=True)
    params = pairs.make_params(rp_min, rp_max, rp_max, np_, nt, ang_max, x_correlation=unfold)
    got = wick.wick_covariance(fs, params, cf1d, reject, nproc=2, return_raw=True)
    assert (got["NPALL"], got["NPUSED"]) == (want["NPALL"], want["NPUSED"])
    assert want["NB"].sum() > 0
    assert np.array_equal(got["NB"], want["NB"])
    raw_g, raw_w = got["raw"], want["raw"]
    close(raw_g["weights_wick"], raw_w["weights_wick"])
    nb = np_ * nt
    for key in ("t1", "t2", "t3"):
        close(raw_g[key].reshape(nb, nb), raw_w[key])
    for key in ("CO", "T1", "T2", "T3"):
        close(got[key], want[key])


def write_cf1d(path):
    from picca_gb300 import fitsio_lite
    cf1d = golden("cf1d.npz")
    fitsio_lite.write_fits(path, [{
        "columns": [cf1d[k] for k in ("v1d", "wv1d", "nv1d", "c1d", "nc1d", "nb1d")],
        "names": ["v1d", "wv1d", "nv1d", "c1d", "nc1d", "nb1d"], "extname": "1DCOR",
        "header": [{"name": "LLMIN", "value": float(cf1d["LLMIN"])},
                   {"name": "DLL", "value": float(cf1d["DLL"])}]}])
    return path


def test_cli_matches_golden_xwick(cuda, tmp_path):
    from conftest import write_catalogue
    from picca_gb300 import fitsio_lite
    from picca_gb300.bin import picca_xwick
    base = str(tmp_path)
    write_delta_dir(os.path.join(base, "Delta_LYA"))
    write_attributes(os.path.join(base, "attributes.fits.gz"))
    write_catalogue(os.path.join(base, "cat.fits"))
    out = os.path.join(base, "xwick.fits.gz")
    picca_xwick.main(["--in-dir", os.path.join(base, "Delta_LYA") + "/",
                      "--drq", os.path.join(base, "cat.fits"), "--out", out,
                      "--cf1d", write_cf1d(os.path.join(base, "cf1d.fits.gz")),
                      "--rp-min", "-60.0", "--rp-max", "+60.0", "--rt-max", "+60.0",
                      "--np", "30", "--nt", "15", "--rej", "0.99", "--nproc", "1",
                      "--z-evol-obj", "1.",
                      "--in-attributes", os.path.join(base, "attributes.fits.gz")])
    want = golden("cor_xwick.npz")
    with fitsio_lite.FITS(out) as h:
        cov = h["COV"]
        header = cov.read_header()
        got = {c: cov[c][:] for c in cov.get_colnames()}
    assert int(header["NPALL"]) == int(want["hdr_NPALL"])
    assert int(header["NPUSED"]) == int(want["hdr_NPUSED"])
    compare_like_reference(got, want, names=tuple(got))


@pytest.mark.parametrize("np_,nt,rp,reject,target,method", [
    (30, 15, 60.0, 0.5, None, "sweep"), (100, 50, 200.0, 0.9, None, "sweep"),
    (100, 50, 200.0, 0.9, 1e5, "sweep"), (30, 15, 60.0, 0.5, None, "factored"),
    (100, 50, 200.0, 0.9, None, "factored")])
def test_synthetic_cross_matches_oracle(cuda, monkeypatch, np_, nt, rp, reject, target, method):
    from picca_gb300 import constants, pairs, synthetic as syn, utils, wick
    if target is not None:
        monkeypatch.setattr(wick, "SLICE_TARGET", target)
    fs = synthetic(60, 17, 200)
    qs = syn.make_quasars(900, 18, (150.0, 152.0), (0.0, 2.0), z_lo=2.0, z_hi=3.6)
    cf1d = golden("cf1d.npz")
    cosmo = constants.Cosmo(Om=0.3147, verbose=False)
    ang_max = utils.compute_ang_max(cosmo, rp, 2.0, 2.0)
    p = ow.make_params(-rp, rp, rp, np_, nt, x_correlation=True)
    want = ow.xpipeline(fs, qs, p, ang_max, cf1d, reject, nproc=2, alpha_obj=1.44,
                        return_raw=True)
    params = pairs.make_params(-rp, rp, rp, np_, nt, ang_max, x_correlation=True)
    got = wick.cross_wick_covariance(fs, qs, params, cf1d, reject, nproc=2, alpha_obj=1.44,
                                     return_raw=True, method=method)
    assert (got["NPALL"], got["NPUSED"]) == (want["NPALL"], want["NPUSED"])
    assert want["NB"].sum() > 0
    assert np.array_equal(got["NB"], want["NB"])
    nb = np_ * nt
    close(got["raw"]["weights_wick"], want["raw"]["weights_wick"])
    for key in ("t1", "t2", "t3", "t4"):
        close(got["raw"][key].reshape(nb, nb), want["raw"][key])
    for key in ("CO", "T1", "T2", "T3", "T4"):
        close(got[key], want[key])
