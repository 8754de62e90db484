"""The fast metal distortion-matrix oracle against picca's golden files:
fast_metal_dmat.fits.gz (auto, r_par 0-60, 15 x 15 bins), fast_metal_dmat_cross
.fits.gz (the same stack twice, r_par -60-60 folded, 30 x 15) and
fast_metal_xdmat.fits.gz (stack x quasar-redshift histogram, signed r_par),
commands at py/picca/tests/test_3_cor.py:384-409, :562-589, :731-757. The
reference's own tolerance (rtol 1e-5, atol 1e-8, py/picca/tests/
test_helpers.py:45-108) is used."""

import os

import numpy as np

from conftest import golden, write_catalogue
from oracle import fast_metal as ofm
from picca_gb300 import constants, io

A = constants.ABSORBER_IGM
ALPHA = {"LYA": 2.9, "SiIII(1207)": 1.0}


def cosmo():
    return constants.Cosmo(Om=0.315, Or=0.0, Ok=0.0, wl=-1.0, verbose=False)


def check(got, want):
    assert got.shape == want.shape
    assert np.allclose(want, got, rtol=1e-5, atol=1e-8)


def test_absorber_pairs():
    assert ofm.absorber_pairs("LYA", ["SiIII(1207)"]) == [("LYA", "SiIII(1207)"),
                                                          ("SiIII(1207)", "SiIII(1207)")]
    # without --lambda-abs2 the script ignores --abs-igm2
    assert ofm.absorber_pairs("LYA", ["SiIII(1207)"], None, ["CIV(eff)"]) == \
        ofm.absorber_pairs("LYA", ["SiIII(1207)"])
    assert ofm.absorber_pairs("LYA", ["SiII(1260)"], "CIV(eff)", ["SiIII(1207)"]) == [
        ("LYA", "SiIII(1207)"), ("SiII(1260)", "CIV(eff)"), ("SiII(1260)", "SiIII(1207)")]


def test_auto_matches_golden():
    st = golden("stack_lya_nodla.npz")
    c = cosmo()
    for case, rp_min, np_ in (("cor_fast_metal_dmat", 0.0, 15),
                              ("cor_fast_metal_dmat_cross", -60.0, 30)):
        want = golden(case + ".npz")
        pairs = ofm.absorber_pairs("LYA", ["SiIII(1207)"])
        assert [f"{a}_{b}" for a, b in pairs] == [str(x) for x in want["ABS_IGM"]]
        for a1, a2 in pairs:
            s1 = ofm.stack_side(st["LOGLAM"], st["WEIGHT"], A[a1], A["LYA"], ALPHA[a1] + 2.9, c)
            s2 = ofm.stack_side(st["LOGLAM"], st["WEIGHT"], A[a2], A["LYA"], ALPHA[a2] + 2.9, c)
            dm, rp, rt, z = ofm.matrix(s1, s2, rp_min, 60.0, 60.0, np_, 15, signed=False)
            name = f"{a1}_{a2}"
            for key, value in (("DM", dm), ("RP", rp), ("RT", rt), ("Z", z)):
                check(value, want[f"{key}_{name}"])


def test_cross_matches_golden(tmp_path):
    st = golden("stack_lya_nodla.npz")
    c = cosmo()
    path = os.path.join(tmp_path, "cat.fits")
    write_catalogue(path)
    cat = io.read_drq(path, z_min=0, z_max=10, keep_bal=True, mode="sdss")
    z_qso = np.asarray(cat["Z"], dtype=np.float64)
    w_qso = ((1.0 + z_qso) / (1.0 + 2.25)) ** (1.0 - 1.0)
    z_hist, w_hist = ofm.quasar_histogram(z_qso, w_qso, 1000)
    assert np.isclose(w_hist.sum(), w_qso.sum())
    want = golden("cor_fast_metal_xdmat.npz")
    s1 = ofm.stack_side(st["LOGLAM"], st["WEIGHT"], A["SiIII(1207)"], A["LYA"], 1.0 + 2.9, c)
    dm, rp, rt, z = ofm.matrix(s1, ofm.quasar_side(z_hist, w_hist, c), -60.0, 60.0, 60.0, 30,
                               15, signed=True)
    for key, value in (("DM", dm), ("RP", rp), ("RT", rt), ("Z", z)):
        check(value, want[f"{key}_QSO_SiIII(1207)"])


def test_rebin():
    x = np.arange(10, dtype=np.float64)
    assert np.array_equal(ofm.rebin(x, 3), np.array([1.0, 4.0, 7.0]))
    assert ofm.rebin(x, None) is x
