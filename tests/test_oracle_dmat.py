"""The distortion-matrix oracle against picca: its forest-pair function
against picca's own cf.compute_dmat_forest_pairs_fast (fixtures made by
tests/golden/make_golden.py), and the whole picca_dmat.py restatement
against picca's golden dmat.fits.gz (py/picca/tests/test_3_cor.py:318-347:
rp 0-60, rt 60, 15x15 bins, rejection 0.99, one process, same-half-plate
veto, no redshift evolution)."""

import os

import numpy as np

from conftest import golden
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


def test_pipeline_matches_golden_dmat(picca_inputs):
    from picca_gb300 import constants, io, utils
    from picca_gb300.forests import ForestSet
    cosmo = constants.Cosmo(Om=0.315, verbose=False)
    data, _, z_min, _ = io.read_deltas(
        os.path.join(picca_inputs, "Delta_LYA") + "/", 16, constants.ABSORBER_IGM["LYA"], 2.9,
        2.25, cosmo, delta_attributes=os.path.join(picca_inputs, "delta_attributes.fits.gz"))
    fs = ForestSet.from_deltas(data)
    params = odm.make_params(0., 60., 60., 15, 15, remove_same_half_plate_close_pairs=True,
                             redshift_evolution=False)
    ang_max = utils.compute_ang_max(cosmo, 60., z_min)
    got = odm.pipeline(fs, params, ang_max, reject=0.99, nproc=1, order=1)
    want = golden("cor_dmat.npz")
    assert got["NPALL"] == int(want["hdr_NPALL"])
    assert got["NPUSED"] == int(want["hdr_NPUSED"])
    compare_like_reference(got, want, names=("WDM", "DM", "RP", "RT", "Z"))
