"""Host logic of the distortion matrix (no GPU): the random rejection of
picca_dmat.py reproduced by picca_gb300.dmat.selection_mask against the
oracle's forest-by-forest restatement, for one and several process chunks,
and the normalisation against the oracle's."""

import numpy as np
import pytest

from oracle import cpu
from oracle import dmat as odm
from picca_gb300 import dmat, synthetic


@pytest.fixture(scope="module")
def forests():
    fs = synthetic.make_forests(300, 11, (150.0, 153.0), (0.0, 3.0))
    params = cpu.make_params(0., 60., 60., 15, 15)
    offsets, _ = cpu.neighbours(fs, fs, params, 0.02, auto_mode=1)
    return fs, offsets


@pytest.mark.parametrize("nproc", [1, 3, 64])
@pytest.mark.parametrize("reject", [0.99, 0.5, -1.0])
def test_selection_matches_oracle(forests, nproc, reject):
    fs, offsets = forests
    want, npall, npused = odm.selection(fs, offsets, nproc, reject)
    got = dmat.selection_mask(fs.healpix_list, fs.row, offsets, nproc, reject)
    assert np.array_equal(got, want)
    assert npall == int(offsets[-1]) and npused == int(got.sum())


def test_selection_needs_grouped_forests():
    with pytest.raises(ValueError):
        dmat.selection_mask(np.array([1, 2]), np.array([1, 0]), np.array([0, 1, 2]), 1, 0.5)


def test_normalise_matches_oracle():
    rng = np.random.default_rng(3)
    params = odm.make_params(0., 60., 60., 4, 3, coef_binning_model=2)
    raw = odm.new_outputs(params)
    for key in raw:
        raw[key][:] = rng.uniform(0.0, 2.0, raw[key].size)
    raw["weight_eff"][::5] = 0.0
    raw["weights_dmat"][::4] = 0.0
    for evolution in (False, True):
        params.redshift_evolution = int(evolution)
        want = odm.normalise(raw, params, 10, 3)
        pc = dmat.make_dmat_params(4, 3, coef_binning_model=2, redshift_evolution=evolution)
        got = dmat.normalise(raw, params, pc, 10, 3)
        for key in ("WDM", "DM", "RP", "RT", "Z"):
            assert np.array_equal(got[key], want[key]), key
        assert got["NPALL"] == 10 and got["NPUSED"] == 3
