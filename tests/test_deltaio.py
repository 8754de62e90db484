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


@pytest.mark.parametrize("save_format,wave", [("ImageHDU", "log"), ("ImageHDU", "lin"),
                                              ("BinTableHDU", "log"), ("BinTableHDU", "lin")])
def test_writer_round_trip(tmp_path, save_format, wave):
    """delta_extraction's delta files (py/picca/delta_extraction/data.py:62-265)
    written by deltaio.write_deltas and read back by both readers: every
    forest, pixel and value recovered."""
    from picca_gb300 import deltaio
    rng = np.random.default_rng(7)
    grid = (3.5563 + 3e-4 * np.arange(900)) if wave == "log" else \
        np.log10(3600.0 + 0.8 * np.arange(900))
    nf = 40
    starts = rng.integers(0, 500, nf)
    lengths = rng.integers(30, 380, nf)
    index = np.concatenate([np.arange(s, s + n) for s, n in zip(starts, lengths)])
    po = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    n = int(po[-1])
    arrays = {"los_id": np.arange(100, 100 + nf), "ra": rng.uniform(0, 0.1, nf),
              "dec": rng.uniform(0, 0.1, nf), "z_qso": rng.uniform(2.2, 3.4, nf),
              "healpix": rng.integers(0, 3, nf), "pix_offset": po,
              "delta": rng.normal(0, 0.3, n), "weights": rng.uniform(0.5, 3.0, n),
              "cont": rng.uniform(1.0, 2.0, n)}
    deltaio.write_deltas(str(tmp_path), arrays, grid, index, save_format=save_format,
                         wave_solution=wave)
    files = sorted(str(p) for p in (tmp_path / "Delta").iterdir())
    # the pixel step as picca writes it: unrounded in the table layout
    # (Forest.get_header, delta_extraction/astronomical_objects/forest.py:580-601),
    # rounded to two decimals in the image layout (delta_extraction/data.py:97-108)
    from picca_gb300 import fitsio_lite
    exact = (grid[1] - grid[0]) if wave == "log" else (10**grid[1] - 10**grid[0])
    key = "DELTA_LOG_LAMBDA" if wave == "log" else "DELTA_LAMBDA"
    headers = fitsio_lite.hdu_headers(deltaio.file_bytes(files[0]))
    step_header = headers[1]
    if save_format == "ImageHDU":
        step_header = next(h for h in headers if str(h.get("EXTNAME", "")).strip() == "LAMBDA")
    assert step_header[key] == (round(exact, 2) if save_format == "ImageHDU" else exact)
    assert step_header["WAVE_SOLUTION"] == wave
    got = deltaio.read_files(files)
    # forests come back grouped by healpix file, in file order
    order = np.concatenate([np.nonzero(arrays["healpix"] == hp)[0]
                            for hp in sorted(np.unique(arrays["healpix"]),
                                             key=lambda h: f"delta-{h}.fits.gz")])
    assert np.array_equal(got["los_id"], arrays["los_id"][order])
    for key in ("ra", "dec", "z_qso"):
        assert np.array_equal(got[key], arrays[key][order])
    want_ll = np.concatenate([grid[index[po[f]:po[f + 1]]] for f in order])
    if wave == "lin":  # stored as wavelength, read back as log10 of it
        want_ll = np.log10(10**want_ll)
    assert np.array_equal(got["log_lambda"], want_ll)
    for key in ("delta", "weights", "cont"):
        want = np.concatenate([arrays[key][po[f]:po[f + 1]] for f in order])
        assert np.array_equal(got[key], want)
    # the per-object readers see the same files
    per_object = [d for path in files for d in io.read_delta_file(path)]
    assert [d.los_id for d in per_object] == list(got["los_id"])
    assert np.array_equal(np.concatenate([d.delta for d in per_object]), got["delta"])
    # rebinning reads WAVE_SOLUTION / DELTA_LAMBDA (HIERARCH cards) back
    if wave == "lin":
        rebinned = deltaio.read_files(files, rebin_factor=3)
        per_object = [d for path in files for d in io.read_delta_file(path, rebin_factor=3)]
        for key in ("log_lambda", "delta", "weights"):
            assert np.array_equal(np.concatenate([getattr(d, key) for d in per_object]),
                                  rebinned[key]), key
        assert rebinned["log_lambda"].size < got["log_lambda"].size
    else:
        with pytest.raises(ValueError):
            deltaio.read_files(files, rebin_factor=3)


def test_text_identifiers_use_per_object_reader(tmp_path):
    """Image files whose METADATA keeps coadded SDSS identifiers as text
    (PLATE '3655-3657', py/picca/delta_extraction/astronomical_objects/
    sdss_forest.py:144-161) are left to the per-object readers."""
    from picca_gb300 import _native, deltaio, fitsio_lite
    rng = np.random.default_rng(3)
    grid = 3.5563 + 3e-4 * np.arange(200)
    nf = 5
    inside = rng.random((nf, 200)) < 0.7
    img = {k: np.where(inside, rng.uniform(0.5, 1.5, (nf, 200)), np.nan)
           for k in ("DELTA", "WEIGHT", "CONT")}
    meta = {"columns": [np.arange(nf, dtype=np.int64) + 7, rng.uniform(0, 0.1, nf),
                        rng.uniform(0, 0.1, nf), rng.uniform(2.2, 3.0, nf),
                        np.array([b"3655-3657"] * nf), np.array([b"55240-55244"] * nf),
                        np.array([b"0012-0300"] * nf)],
            "names": ["THING_ID", "RA", "DEC", "Z", "PLATE", "MJD", "FIBERID"],
            "header": [{"name": "BLINDING", "value": "none"}], "extname": "METADATA"}
    os.makedirs(tmp_path / "Delta")
    path = str(tmp_path / "Delta" / "delta-1.fits.gz")
    fitsio_lite.write_hdus(path, [("image", "LAMBDA", 10**grid, []), ("table", meta)]
                           + [("image", k, v, []) for k, v in img.items()])
    with pytest.raises(_native.NativeError) as info:
        deltaio.read_file(path)
    assert info.value.status == _native.PG_ERR_UNSUPPORTED
    cosmo = constants.Cosmo(Om=0.315, verbose=False)
    args = (str(tmp_path / "Delta") + "/", 16, constants.ABSORBER_IGM["LYA"], 2.9, 2.25, cosmo)
    got = io.read_deltas(*args, no_project=True, native=True)
    want = io.read_deltas(*args, no_project=True, native=False)
    assert got[1] == want[1] == nf
    for hp in want[0]:
        for a, b in zip(got[0][hp], want[0][hp]):
            assert np.array_equal(a.delta, b.delta) and a.plate == b.plate


@pytest.mark.parametrize("kwargs", [{"rebin_factor": 3}, {"rebin_factor": 2, "max_num_spec": 300},
                                    {"rebin_factor": 5, "no_project": True}])
def test_native_rebinning_matches_per_object(dirs, kwargs):
    """--rebin-factor on the image layout (linear wavelength grid)."""
    attr = os.path.join(dirs, "attr1.fits.gz")
    cosmo = constants.Cosmo(Om=0.315, verbose=False)
    args = (os.path.join(dirs, "Delta_LYA_image") + "/", 16, constants.ABSORBER_IGM["LYA"], 2.9,
            2.25, cosmo)
    got = io.read_deltas(*args, delta_attributes=attr, native=True, **kwargs)
    want = io.read_deltas(*args, delta_attributes=attr, native=False, **kwargs)
    assert got[1] == want[1] and got[2] == want[2] and got[3] == want[3]
    same_sets(ForestSet.from_deltas(got[0]), ForestSet.from_deltas(want[0]))
    for hp in want[0]:
        for a, b in zip(got[0][hp], want[0][hp]):
            assert np.array_equal(a.cont, b.cont)


def test_rebin_arrays_matches_delta_rebin():
    from picca_gb300 import deltaio
    from picca_gb300.data import Delta
    rng = np.random.default_rng(12)
    sizes = [1, 2, 3, 7, 40, 333, 600]
    lls, ws, ds = [], [], []
    for n in sizes:
        start = 3600.0 + 0.8 * rng.integers(0, 500)
        pix = np.sort(rng.choice(np.arange(3 * n), n, replace=False))  # gaps
        lls.append(np.log10(start + 0.8 * pix))
        w = rng.uniform(0.1, 3.0, n)
        w[rng.random(n) < 0.2] = 0.0  # bins whose pixels all have no weight
        ws.append(w)
        ds.append(rng.normal(0, 0.3, n))
    po = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    for factor in (1, 2, 3, 4):
        new_po, ll, d, w = deltaio.rebin_arrays(po, np.concatenate(lls), np.concatenate(ds),
                                                np.concatenate(ws), factor, 0.8)
        for f in range(len(sizes)):
            obj = Delta(1, 0.1, 0.2, 2.5, 1, 1, 1, lls[f].copy(), ws[f].copy(), None,
                        ds[f].copy(), 1)
            obj.rebin(factor, dwave=0.8)
            sl = slice(new_po[f], new_po[f + 1])
            assert np.array_equal(ll[sl], obj.log_lambda), (factor, sizes[f])
            assert np.array_equal(d[sl], obj.delta) and np.array_equal(w[sl], obj.weights)


def test_rebin_arrays_jittered_wavelengths():
    """Pixels off the nominal grid (up to half a pixel), so that many fall
    next to a bin edge: the bin search must agree with searchsorted."""
    from picca_gb300 import deltaio
    from picca_gb300.data import Delta
    rng = np.random.default_rng(21)
    sizes = rng.integers(1, 300, 60)
    lls, ws, ds = [], [], []
    for n in sizes:
        wave = 3700.0 + 0.8 * np.arange(n) + rng.uniform(-0.45, 0.45, n) * 0.8
        lls.append(np.log10(np.sort(wave)))
        ws.append(rng.uniform(0.1, 3.0, n))
        ds.append(rng.normal(0, 0.3, n))
    po = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    for factor in (1, 2, 7):
        new_po, ll, d, w = deltaio.rebin_arrays(po, np.concatenate(lls), np.concatenate(ds),
                                                np.concatenate(ws), factor, 0.8)
        for f in range(len(sizes)):
            obj = Delta(1, 0.1, 0.2, 2.5, 1, 1, 1, lls[f].copy(), ws[f].copy(), None,
                        ds[f].copy(), 1)
            obj.rebin(factor, dwave=0.8)
            sl = slice(new_po[f], new_po[f + 1])
            assert np.array_equal(ll[sl], obj.log_lambda), (factor, f)
            assert np.array_equal(d[sl], obj.delta) and np.array_equal(w[sl], obj.weights)


def test_hierarch_cards():
    """Keywords longer than eight characters are written as HIERARCH cards:
    the comment is kept when the card has room for it, and a card that
    cannot hold its value is refused instead of being cut."""
    from picca_gb300 import fitsio_lite
    card = fitsio_lite._card("DELTA_LAMBDA", 0.7999999999997272, "pixel step")
    assert len(card) == 80
    assert card.rstrip().endswith("/ pixel step")
    header, _ = fitsio_lite._parse_header(fitsio_lite._header_bytes([card]), 0)
    assert header["DELTA_LAMBDA"] == 0.7999999999997272
    long_text = "x" * 60
    with pytest.raises(ValueError):
        fitsio_lite._card("A_VERY_LONG_KEYWORD", long_text)
    # a comment that does not fit is dropped, the value is kept whole
    card = fitsio_lite._card("WAVE_SOLUTION", "lin", "c" * 70)
    assert "'lin" in card and "/" not in card
