"""GPU parity of the metal distortion matrix (pg_cf_metal_dmat through the
C ABI): the picca_metal_dmat.py drop-in against picca's golden
metal_dmat.fits.gz (reference rule, NPALL / NPUSED exact), and the host
driver against the NumPy oracle on synthetic forests with several metals,
model bins twice as fine, same-half-plate vetoes and a folded and an
unfolded r_par. Tolerance: FP64 sums in another order than numpy's
bincounts: |got - want| <= 1e-9 |want| + 1e-11 max|want|."""

import os

import numpy as np
import pytest

from conftest import golden
from oracle import metal_dmat as omd
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
    scale = float(np.max(np.abs(want))) if want.size else 0.0
    err = np.abs(got - want)
    return bool(np.all(err <= rtol * np.abs(want) + scale_tol * scale)), float(err.max())


def test_cli_matches_golden_metal_dmat(cuda, picca_inputs, tmp_path):
    from picca_gb300 import fitsio_lite
    from picca_gb300.bin import picca_metal_dmat
    out = str(tmp_path / "metal_dmat.fits.gz")
    picca_metal_dmat.main([
        "--in-dir", os.path.join(picca_inputs, "Delta_LYA") + "/", "--out", out,
        "--abs-igm", "SiIII(1207)", "--rp-min", "+0.0", "--rp-max", "+60.0", "--rt-max", "+60.0",
        "--np", "15", "--nt", "15", "--rej", "0.99", "--nproc", "1",
        "--in-attributes", os.path.join(picca_inputs, "delta_attributes.fits.gz")])
    want = golden("cor_metal_dmat.npz")
    with fitsio_lite.FITS(out) as h:
        attri, mdmat = h["ATTRI"], h["MDMAT"]
        names = [x.decode() if isinstance(x, bytes) else str(x) for x in attri["ABS_IGM"][:]]
        assert names == [str(x) for x in want["ABS_IGM"]]
        assert np.array_equal(attri["NPALL"][:], want["NPALL"])
        assert np.array_equal(attri["NPUSED"][:], want["NPUSED"])
        for name in names:
            got = {k: mdmat[f"{k}_{name}"][:] for k in ("RP", "RT", "Z", "DM", "WDM")}
            ref = {k: want[f"{k}_{name}"] for k in ("RP", "RT", "Z", "DM", "WDM")}
            compare_like_reference(got, ref, names=("RP", "RT", "Z", "DM", "WDM"))


@pytest.mark.parametrize("unfold", [False, True])
def test_synthetic_matches_oracle(cuda, unfold):
    from picca_gb300 import constants, dmat, metal, pairs, synthetic
    fs = synthetic.make_forests(80, 21, (150.0, 152.5), (0.0, 2.5), max_pixels=400)
    rng = np.random.default_rng(21)
    fs.plate = rng.integers(0, 3, fs.num).astype(np.int64)
    fs.fiberid = rng.integers(1, 1000, fs.num).astype(np.int64)
    cosmo = constants.Cosmo(Om=0.3147, verbose=False)
    metals = ["SiIII(1207)", "SiII(1260)"]
    alpha = {"LYA": 2.9, "SiIII(1207)": 1.0, "SiII(1260)": 1.2}
    rp_min = -60. if unfold else 0.
    p = omd.MetalParams(rp_min, 60., 60., 12, 10, coef_binning_model=2, x_correlation=unfold,
                        remove_same_half_plate_close_pairs=True, z_ref=2.25, alpha_abs=alpha)
    want = omd.pipeline(fs, cosmo, p, 0.02, reject=0.8, abs_igm=metals, nproc=2) \
        if not unfold else None
    params = pairs.make_params(rp_min, 60., 60., 12, 10, 0.02, x_correlation=unfold,
                               remove_same_half_plate_close_pairs=True)
    dparams = dmat.make_dmat_params(12, 10, coef_binning_model=2)
    got = metal.metal_distortion_matrices(fs, params, dparams, cosmo, 0.8, metals, alpha,
                                          z_ref=2.25, nproc=2)
    if unfold:
        # the oracle's pipeline is the auto-correlation with folded r_par; with
        # r_par unfolded compare one absorber pair forest pair by forest pair
        from oracle import cpu
        from oracle import dmat as odm
        oparams = cpu.make_params(rp_min, 60., 60., 12, 10)
        offsets, index = cpu.neighbours(fs, fs, oparams, 0.02, auto_mode=1)
        mask, npall, npused = odm.selection(fs, offsets, 2, 0.8)
        want = {}
        po = np.asarray(fs.pix_offset)
        for abs1, abs2 in omd.absorber_pairs("LYA", metals):
            out = omd.new_outputs(p)
            for f in range(fs.num):
                for k in range(int(offsets[f]), int(offsets[f + 1])):
                    if not mask[k]:
                        continue
                    g = int(index[k])
                    ang = cpu.lib().oracle_angle(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f],
                                                 fs.ra[f], fs.dec[f], fs.cos_dec[f],
                                                 fs.x_cart[g], fs.y_cart[g], fs.z_cart[g],
                                                 fs.ra[g], fs.dec[g])
                    shp = fs.plate[f] == fs.plate[g] and (
                        (fs.fiberid[f] <= 500) == (fs.fiberid[g] <= 500))
                    sl = lambda h: (fs.log_lambda[po[h]:po[h + 1]],  # noqa: E731
                                    fs.r_comov[po[h]:po[h + 1]], fs.dist_m[po[h]:po[h + 1]],
                                    fs.weights[po[h]:po[h + 1]], fs.z_qso[h])
                    omd.forest_pair(p, cosmo, sl(f), sl(g), ang, shp, abs1, abs2, False, out)
            want[f"{abs1}_{abs2}"] = omd.normalise(out, p, npall, npused)
    assert list(got) == list(want)
    for name in want:
        assert got[name]["NPALL"] == want[name]["NPALL"]
        assert got[name]["NPUSED"] == want[name]["NPUSED"]
        for key in ("RP", "RT", "Z", "DM", "WDM"):
            ok, err = close(got[name][key], want[name][key])
            assert ok, (unfold, name, key, err)


def test_cli_matches_golden_metal_xdmat(cuda, picca_inputs, tmp_path):
    from picca_gb300 import fitsio_lite
    from picca_gb300.bin import picca_metal_xdmat
    out = str(tmp_path / "metal_xdmat.fits.gz")
    picca_metal_xdmat.main([
        "--in-dir", os.path.join(picca_inputs, "Delta_LYA") + "/",
        "--drq", os.path.join(picca_inputs, "cat.fits"), "--out", out,
        "--abs-igm", "SiIII(1207)", "--rp-min", "-60.0", "--rp-max", "+60.0",
        "--rt-max", "+60.0", "--np", "30", "--nt", "15", "--rej", "0.99", "--nproc", "1",
        "--z-evol-obj", "1.",
        "--in-attributes", os.path.join(picca_inputs, "delta_attributes.fits.gz")])
    want = golden("cor_metal_xdmat.npz")
    with fitsio_lite.FITS(out) as h:
        attri, mdmat = h["ATTRI"], h["MDMAT"]
        assert np.array_equal(attri["NPALL"][:], want["NPALL"])
        assert np.array_equal(attri["NPUSED"][:], want["NPUSED"])
        name = "QSO_SiIII(1207)"
        got = {k: mdmat[f"{k}_{name}"][:] for k in ("RP", "RT", "Z", "DM", "WDM")}
        ref = {k: want[f"{k}_{name}"] for k in ("RP", "RT", "Z", "DM", "WDM")}
        compare_like_reference(got, ref, names=("RP", "RT", "Z", "DM", "WDM"))


def test_synthetic_xcf_matches_oracle(cuda):
    from picca_gb300 import constants, dmat, metal, pairs, synthetic
    fs = synthetic.make_forests(60, 31, (150.0, 152.5), (0.0, 2.5), max_pixels=400)
    qs = synthetic.make_quasars(800, 32, (150.0, 152.5), (0.0, 2.5), z_lo=2.0, z_hi=3.6)
    cosmo = constants.Cosmo(Om=0.3147, verbose=False)
    metals = ["SiIII(1207)", "SiII(1527)"]
    alpha = {"LYA": 2.9, "SiIII(1207)": 1.0, "SiII(1527)": 1.3}
    p = omd.MetalParams(-60., 60., 60., 12, 10, coef_binning_model=2, x_correlation=True,
                        z_ref=2.25, alpha_abs=alpha)
    want = omd.xpipeline(fs, qs, cosmo, p, 0.03, reject=0.7, abs_igm=metals, nproc=3)
    params = pairs.make_params(-60., 60., 60., 12, 10, 0.03, x_correlation=True)
    dparams = dmat.make_dmat_params(12, 10, coef_binning_model=2)
    got = metal.cross_metal_distortion_matrices(fs, qs, params, dparams, cosmo, 0.7, metals,
                                                alpha, z_ref=2.25, nproc=3)
    assert list(got) == list(want)
    for name in want:
        assert got[name]["NPALL"] == want[name]["NPALL"]
        assert got[name]["NPUSED"] == want[name]["NPUSED"]
        for key in ("RP", "RT", "Z", "DM", "WDM"):
            ok, err = close(got[name][key], want[name][key])
            assert ok, (name, key, err)


def test_cli_matches_golden_metal_dmat_cross(cuda, picca_inputs, tmp_path):
    """py/picca/tests/test_3_cor.py:526-557."""
    from picca_gb300 import fitsio_lite
    from picca_gb300.bin import picca_metal_dmat
    out = str(tmp_path / "metal_dmat_cross.fits.gz")
    delta_dir = os.path.join(picca_inputs, "Delta_LYA") + "/"
    picca_metal_dmat.main([
        "--in-dir", delta_dir, "--in-dir2", delta_dir, "--out", out,
        "--abs-igm", "SiIII(1207)", "--abs-igm2", "SiIII(1207)", "--rp-min", "-60.0",
        "--rp-max", "+60.0", "--rt-max", "+60.0", "--np", "30", "--nt", "15", "--rej", "0.99",
        "--nproc", "1", "--remove-same-half-plate-close-pairs", "--unfold-cf",
        "--in-attributes", os.path.join(picca_inputs, "delta_attributes.fits.gz")])
    want = golden("cor_metal_dmat_cross.npz")
    with fitsio_lite.FITS(out) as h:
        attri, mdmat = h["ATTRI"], h["MDMAT"]
        assert np.array_equal(attri["NPALL"][:], want["NPALL"])
        assert np.array_equal(attri["NPUSED"][:], want["NPUSED"])
        for name in (str(x) for x in want["ABS_IGM"]):
            got = {k: mdmat[f"{k}_{name}"][:] for k in ("RP", "RT", "Z", "DM", "WDM")}
            ref = {k: want[f"{k}_{name}"] for k in ("RP", "RT", "Z", "DM", "WDM")}
            compare_like_reference(got, ref, names=("RP", "RT", "Z", "DM", "WDM"))


def test_second_tracer_matches_oracle(cuda):
    """picca_metal_dmat.py with --lambda-abs2: the second field's distances are
    those of its own tracer (here LYB), every absorber of the first list is
    paired with every one of the second, r_par is unfolded and no swapped
    pass is made (py/picca/bin/picca_metal_dmat.py:389-470,
    py/picca/cf.py:1088-1090)."""
    from picca_gb300 import constants, dmat, metal, pairs, synthetic
    cosmo = constants.Cosmo(Om=0.3147, verbose=False)
    # the first field: LYA forests of quasars at z 3.5-4; the second: forests
    # moved to 0.85 of their wavelengths (rest frame 884-1020 A, below LYB)
    # of quasars at z 3.8-4.6, so that both overlap in observed wavelength
    fs = synthetic.make_forests(60, 31, (150.0, 152.5), (0.0, 2.5), z_lo=3.5, z_hi=4.0,
                                max_pixels=400)
    fs2 = synthetic.make_forests(60, 32, (150.0, 152.5), (0.0, 2.5), z_lo=3.8, z_hi=4.6,
                                 max_pixels=400, thingid_start=10_000)
    fs2.log_lambda = np.asarray(fs2.log_lambda) + np.log10(0.85)
    # the second field as LYB forests: z and distances of that tracer
    lam2 = constants.ABSORBER_IGM["LYB"]
    z2 = 10**np.asarray(fs2.log_lambda) / lam2 - 1.0
    fs2.z = z2
    fs2.r_comov = cosmo.get_r_comov(z2)
    fs2.dist_m = cosmo.get_dist_m(z2)
    alpha = {"LYA": 2.9, "LYB": 2.9, "SiIII(1207)": 1.0, "SiII(1260)": 1.0}
    p = omd.MetalParams(-60.0, 60.0, 60.0, 12, 10, coef_binning_model=1, x_correlation=True,
                        z_ref=2.25, alpha_abs=alpha)
    ang_max = 0.03
    want = omd.pipeline(fs, cosmo, p, ang_max, 0.7, ["SiIII(1207)"], nproc=2, fs2=fs2,
                        lambda_abs2="LYB", abs_igm2=["SiII(1260)"])
    params = pairs.make_params(-60.0, 60.0, 60.0, 12, 10, ang_max, x_correlation=True)
    dparams = dmat.make_dmat_params(12, 10)
    got = metal.metal_distortion_matrices(fs, params, dparams, cosmo, 0.7, ["SiIII(1207)"],
                                          alpha, z_ref=2.25, nproc=2, fs2=fs2,
                                          abs_igm2=["SiII(1260)"], lambda_abs2="LYB")
    # the tracer pair itself (LYA_LYB) is the correlation, not a metal matrix
    assert sorted(got) == sorted(want) == sorted(
        ["LYA_SiII(1260)", "SiIII(1207)_LYB", "SiIII(1207)_SiII(1260)"])
    assert np.abs(want["SiIII(1207)_LYB"]["DM"]).sum() > 0
    for name in want:
        assert got[name]["NPALL"] == want[name]["NPALL"]
        assert got[name]["NPUSED"] == want[name]["NPUSED"]
        assert want[name]["WDM"].sum() > 0
        for key in ("WDM", "DM", "RP", "RT", "Z"):
            ok, err = close(got[name][key], want[name][key])
            assert ok, (name, key, err)
