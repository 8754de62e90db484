"""The Wick covariance oracle against picca's golden wick.fits.gz (command at
py/picca/tests/test_3_cor.py:412-441: r 0-60 Mpc/h, 15 x 15 bins, rejection
0.99, one process), with the reference's tolerance (rtol 1e-5, atol 1e-8;
NB, NPALL and NPUSED exact), and the host parts of the GPU path (the
nearest-point 1D tables, the random draw per forest) against scipy and the
oracle."""

import os

import numpy as np
import pytest

from conftest import golden, write_attributes, write_delta_dir
from oracle import wick as ow
from picca_gb300 import constants, io, utils
from picca_gb300 import wick as pw
from picca_gb300.forests import ForestSet
from test_oracle_golden import compare_like_reference


@pytest.fixture(scope="module")
def test_forests(tmp_path_factory):
    base = str(tmp_path_factory.mktemp("wick"))
    write_delta_dir(os.path.join(base, "Delta_LYA"))
    write_attributes(os.path.join(base, "attributes.fits.gz"))
    cosmo = constants.Cosmo(Om=0.315, verbose=False)
    data, _, z_min, _ = io.read_deltas(os.path.join(base, "Delta_LYA") + "/", 16,
                                       constants.ABSORBER_IGM["LYA"], 2.9, 2.25, cosmo,
                                       delta_attributes=os.path.join(base, "attributes.fits.gz"))
    return ForestSet.from_deltas(data), utils.compute_ang_max(cosmo, 60.0, z_min)


def test_oracle_matches_golden_wick(test_forests):
    fs, ang_max = test_forests
    got = ow.pipeline(fs, ow.make_params(0.0, 60.0, 60.0, 15, 15), ang_max, golden("cf1d.npz"),
                      0.99, nproc=1)
    want = golden("cor_wick.npz")
    assert got["NPALL"] == int(want["hdr_NPALL"])
    assert got["NPUSED"] == int(want["hdr_NPUSED"])
    compare_like_reference(got, want, names=("CO", "WALL", "NB", "T1", "T2", "T3", "T4", "T5",
                                             "T6"))


def test_selection_matches_oracle(test_forests):
    fs, _ = test_forests
    for nproc, reject in ((1, 0.99), (3, 0.9), (2, 0.5)):
        a = pw.selection(fs, nproc, reject)
        b = ow.selection(fs, nproc, reject)
        assert np.array_equal(a[0], b[0]) and a[1:] == b[1:]


def test_one_d_tables_match_scipy():
    cf1d = golden("cf1d.npz")
    variance, xi = ow.interpolants(cf1d)
    tables = pw.OneDTables(cf1d)
    rng = np.random.default_rng(2)
    ll = cf1d["LLMIN"] + rng.uniform(-0.01, 0.3, 5000)
    # grid points and cell bounds themselves (ties go to the lower point)
    grid = cf1d["LLMIN"] + cf1d["DLL"] * np.arange(len(cf1d["v1d"]))
    ll = np.concatenate([ll, grid, tables.var_bounds])
    assert np.array_equal(tables.variance(ll), variance(ll))
    d = np.abs(rng.uniform(-0.2, 0.2, 5000))
    d = np.concatenate([d, tables.xi_bounds, tables.xi_x])
    idx = np.clip(np.searchsorted(tables.xi_bounds, d, side="left"), 0, tables.xi_y.size - 1)
    assert np.array_equal(tables.xi_y[idx], xi(d))


def test_oracle_matches_golden_xwick(test_forests, tmp_path):
    from conftest import write_catalogue
    fs, _ = test_forests
    path = os.path.join(tmp_path, "cat.fits")
    write_catalogue(path)
    cosmo = constants.Cosmo(Om=0.315, verbose=False)
    objs, z_min2 = io.read_objects(path, 16, 0, 10, 1.0, 2.25, cosmo)
    qs = ForestSet.from_objects(objs)
    z_min = float(np.min(fs.z))
    ang_max = utils.compute_ang_max(cosmo, 60.0, z_min, z_min2)
    got = ow.xpipeline(fs, qs, ow.make_params(-60.0, 60.0, 60.0, 30, 15, x_correlation=True),
                       ang_max, golden("cf1d.npz"), 0.99, nproc=1, alpha_obj=1.0)
    want = golden("cor_xwick.npz")
    assert got["NPALL"] == int(want["hdr_NPALL"])
    assert got["NPUSED"] == int(want["hdr_NPUSED"])
    compare_like_reference(got, want, names=("CO", "WALL", "NB", "T1", "T2", "T3", "T4", "T5",
                                             "T6"))
