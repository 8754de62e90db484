"""The distortion-matrix oracle against picca: its forest-pair functions
against picca's own cf.compute_dmat_forest_pairs_fast and
xcf.compute_dmat_forest_pairs_fast (fixtures made by
tests/golden/make_golden.py), and the whole picca_dmat.py / picca_xdmat.py
restatements against picca's six golden distortion matrices
(py/picca/tests/test_3_cor.py: auto, z cuts, the cross of two delta sets
with and without z cuts, delta x quasar with and without z cuts; rejection
0.99, one process, no redshift evolution)."""

import os

import numpy as np

import pytest

from conftest import golden
from corr_cases import DMAT_CASES, prepare
from oracle import dmat as odm
from test_oracle_golden import compare_like_reference


def _case_params(p):
    nan_none = lambda v: None if np.isnan(v) else float(v)  # noqa: E731
    return odm.make_params(0., 60., 60., int(p[0]), int(p[1]), coef_binning_model=int(p[2]),
                           remove_same_half_plate_close_pairs=bool(p[3]),
                           redshift_evolution=bool(p[4]), z_min_pairs=nan_none(p[7]),
                           z_max_pairs=nan_none(p[8]), zerr_cut_deg=nan_none(p[9]),
                           zerr_cut_kms=nan_none(p[10]))


def test_forest_pair_matches_reference():
    f = golden("dmat_cases.npz")
    assert int(f["num_cases"]) >= 8
    for k in range(int(f["num_cases"])):
        pre = f"dm{k}_"
        p = f[pre + "params"]
        params = _case_params(p)
        out = odm.new_outputs(params)
        zq1, zq2, ang, shp = f[pre + "scalars"]
        odm.forest_pair(params, f[pre + "ll1"], f[pre + "ll2"], f[pre + "r1"], f[pre + "r2"],
                        f[pre + "m1"], f[pre + "m2"], f[pre + "z1"], f[pre + "z2"],
                        f[pre + "w1"], f[pre + "w2"], zq1, zq2, ang, bool(shp), int(p[5]),
                        int(p[6]), out)
        for key, got in out.items():
            want = f[pre + "out_" + key]
            # picca's sums of the fixtures ran through NumPy (pairwise); the
            # oracle sums left to right as numba does
            scale = np.max(np.abs(want)) if want.size else 0.0
            assert np.allclose(got, want, rtol=1e-12, atol=1e-12 * scale), (k, key)


def test_xforest_matches_reference():
    f = golden("xdmat_cases.npz")
    assert int(f["num_cases"]) >= 8
    for k in range(int(f["num_cases"])):
        pre = f"xd{k}_"
        p = f[pre + "params"]
        nan_none = lambda v: None if np.isnan(v) else float(v)  # noqa: E731
        params = odm.make_params(-60., 60., 60., int(p[0]), int(p[1]),
                                 coef_binning_model=int(p[2]), redshift_evolution=bool(p[3]),
                                 z_min_pairs=nan_none(p[5]), z_max_pairs=nan_none(p[6]),
                                 alpha=2.9, alpha2=1.44, x_correlation=True)
        out = odm.new_outputs(params)
        odm.xforest(params, f[pre + "ll1"], f[pre + "r1"], f[pre + "m1"], f[pre + "z1"],
                    f[pre + "w1"], f[pre + "r2"], f[pre + "m2"], f[pre + "z2"], f[pre + "w2"],
                    f[pre + "ang"], int(p[4]), out)
        for key, got in out.items():
            want = f[pre + "out_" + key]
            scale = np.max(np.abs(want)) if want.size else 0.0
            assert np.allclose(got, want, rtol=1e-12, atol=1e-12 * scale), (k, key)


def oracle_dmat(case, base):
    """picca_dmat.py / picca_xdmat.py restated on the CPU for a golden case."""
    set1, set2, params, ang_max, kind = prepare(DMAT_CASES[case], base)
    p = odm.make_params(params["r_par_min"], params["r_par_max"], params["r_trans_max"],
                        params["num_bins_r_par"], params["num_bins_r_trans"],
                        z_min_pairs=params["z_min_pairs"], z_max_pairs=params["z_max_pairs"],
                        remove_same_half_plate_close_pairs=params[
                            "remove_same_half_plate_close_pairs"],
                        redshift_evolution=False,
                        x_correlation=params["x_correlation"] or kind == "xcf")
    if kind == "xcf":
        return odm.xpipeline(set1, set2, p, ang_max, reject=0.99, nproc=1, order=1)
    return odm.pipeline(set1, p, ang_max, reject=0.99, nproc=1, order=1, fs2=set2)


@pytest.mark.parametrize("case", sorted(DMAT_CASES))
def test_pipeline_matches_golden_dmat(case, picca_inputs):
    got = oracle_dmat(case, picca_inputs)
    want = golden(f"cor_{case}.npz")
    assert got["NPALL"] == int(want["hdr_NPALL"])
    assert got["NPUSED"] == int(want["hdr_NPUSED"])
    compare_like_reference(got, want, names=("WDM", "DM", "RP", "RT", "Z"))
