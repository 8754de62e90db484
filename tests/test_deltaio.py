"""The native delta reader and projection (pg_read_delta_file,
pg_project_deltas; host code in the CUDA library) against the per-object
readers, which follow py/picca/io.py:333-512 and py/picca/data.py:376-655:
picca's test delta files in both layouts (one table per line of sight, and
the image layout), redshift cuts, max_num_spec, no projection and order 0,
all bit for bit."""

import os

import numpy as np
import pytest

from conftest import write_attributes, write_delta_dir, write_image_dir
from picca_gb300 import constants, io
from picca_gb300.forests import ForestSet


@pytest.fixture(scope="module")
def dirs(tmp_path_factory):
    base = str(tmp_path_factory.mktemp("deltaio"))
    write_delta_dir(os.path.join(base, "Delta_LYA"))
    write_image_dir(os.path.join(base, "Delta_LYA_image"))
    write_attributes(os.path.join(base, "attr1.fits.gz"), order=1)
    write_attributes(os.path.join(base, "attr0.fits.gz"), order=0)
    return base


def same_sets(a, b):
    for key in ("pix_offset", "z", "r_comov", "dist_m", "weights", "delta", "log_lambda", "ra",
                "dec", "x_cart", "y_cart", "z_cart", "cos_dec", "z_qso", "thingid", "plate",
                "fiberid", "order", "healpix", "healpix_list"):
        assert np.array_equal(np.asarray(getattr(a, key)), np.asarray(getattr(b, key))), key


@pytest.mark.parametrize("layout", ["Delta_LYA", "Delta_LYA_image"])
@pytest.mark.parametrize("kwargs", [
    {},
    {"z_min_qso": 2.3, "z_max_qso": 2.9},
    {"max_num_spec": 300},
    {"no_project": True},
    {"attr": "attr0.fits.gz"},
])
def test_native_matches_per_object(dirs, layout, kwargs):
    kwargs = dict(kwargs)
    attr = os.path.join(dirs, kwargs.pop("attr", "attr1.fits.gz"))
    cosmo = constants.Cosmo(Om=0.315, verbose=False)
    args = (os.path.join(dirs, layout) + "/", 16, constants.ABSORBER_IGM["LYA"], 2.9, 2.25, cosmo)
    got = io.read_deltas(*args, delta_attributes=attr, native=True, **kwargs)
    want = io.read_deltas(*args, delta_attributes=attr, native=False, **kwargs)
    assert got[1] == want[1] and got[2] == want[2] and got[3] == want[3]
    assert sorted(got[0]) == sorted(want[0])
    same_sets(ForestSet.from_deltas(got[0]), ForestSet.from_deltas(want[0]))
    for hp in want[0]:
        for a, b in zip(got[0][hp], want[0][hp]):
            assert np.array_equal(a.cont, b.cont)
            assert (a.los_id, a.plate, a.mjd, a.fiberid) == (b.los_id, b.plate, b.mjd, b.fiberid)


def test_projection_orders_and_sizes():
    from picca_gb300 import deltaio
    from picca_gb300.data import Delta
    rng = np.random.default_rng(4)
    sizes = [1, 2, 7, 8, 9, 63, 128, 129, 300, 1000]
    po = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    n = int(po[-1])
    ll = 3.56 + 3e-4 * np.arange(n) + rng.normal(0, 1e-5, n)
    w = rng.uniform(0.1, 5.0, n)
    d = rng.normal(0, 0.3, n)
    for order in (0, 1):
        got = d.copy()
        deltaio.project(po, ll, w, got, np.full(len(sizes), order, dtype=np.int32))
        for f in range(len(sizes)):
            sl = slice(po[f], po[f + 1])
            obj = Delta(1, 0.1, 0.2, 2.5, 1, 1, 1, ll[sl].copy(), w[sl].copy(), None,
                        d[sl].copy(), order)
            obj.project()
            assert np.array_equal(got[sl], obj.delta), (order, sizes[f])
