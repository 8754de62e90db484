"""Shared fixtures: the ``gpu`` marker and writers that rebuild picca's test
inputs (delta files, quasar catalogue, delta attributes) from the committed
``tests/golden/*.npz`` fixtures, so the same tests run on machines without
the picca sources."""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from picca_gb300 import fitsio_lite  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden(name):
    """Fixture arrays as a plain dict (an NpzFile re-reads on each access)."""
    with np.load(os.path.join(GOLDEN, name), allow_pickle=False) as f:
        out = {k: f[k] for k in f.files}
    return out


def write_delta_dir(out_dir):
    """Rebuild py/picca/tests/data/test_delta/Delta_LYA as FITS files."""
    src = golden("delta_lya.npz")
    os.makedirs(out_dir, exist_ok=True)
    offsets = np.concatenate([[0], np.cumsum(src["npix"])])
    names = src["file_names"]
    for file_index, name in enumerate(names):
        tables = []
        for k in np.where(src["file_index"] == file_index)[0]:
            sl = slice(offsets[k], offsets[k + 1])
            tables.append({
                "columns": [src["LOGLAM"][sl], src["DELTA"][sl], src["WEIGHT"][sl],
                            src["CONT"][sl]],
                "names": ["LOGLAM", "DELTA", "WEIGHT", "CONT"],
                "extname": str(src["los_id"][k]),
                "header": [
                    {"name": "RA", "value": float(src["ra"][k])},
                    {"name": "DEC", "value": float(src["dec"][k])},
                    {"name": "Z", "value": float(src["z"][k])},
                    {"name": "THING_ID", "value": int(src["los_id"][k])},
                    {"name": "PLATE", "value": int(src["plate"][k])},
                    {"name": "MJD", "value": int(src["mjd"][k])},
                    {"name": "FIBERID", "value": int(src["fiberid"][k])},
                    {"name": "ORDER", "value": 1},
                ],
            })
        fitsio_lite.write_fits(os.path.join(out_dir, str(name)), tables)
    return out_dir


def write_image_dir(out_dir):
    """Rebuild py/picca/tests/data/test_delta/Delta_LYA_image as FITS files."""
    src = golden("delta_lya_image.npz")
    os.makedirs(out_dir, exist_ok=True)
    for index, name in enumerate(src["file_names"]):
        meta_cols = [k for k in src if k.startswith(f"f{index}_META_")]
        path = os.path.join(out_dir, str(name))
        # image HDUs then a METADATA table: write both with the lite writers
        lam_cards = [{"name": k.split("_HDR_", 1)[1], "value": src[k].item()}
                     for k in src if k.startswith(f"f{index}_HDR_")]
        images = [("LAMBDA", src[f"f{index}_LAMBDA"], lam_cards)]
        for key in ("DELTA", "WEIGHT", "CONT"):
            images.append((key, src[f"f{index}_{key}"], []))
        tmp_img = path + ".img"
        fitsio_lite.write_image_hdus(tmp_img, images)
        tmp_tab = path + ".tab"
        fitsio_lite.write_fits(tmp_tab, [{
            "columns": [src[k] for k in meta_cols],
            "names": [k.split("_META_", 1)[1] for k in meta_cols],
            "extname": "METADATA",
            "header": [{"name": "BLINDING", "value": str(src[f"f{index}_BLINDING"])}],
        }])
        with open(tmp_img, "rb") as a, open(tmp_tab, "rb") as b:
            raw_img = a.read()
            raw_tab = b.read()
        # drop the table file's primary HDU (first 2880-byte block)
        with open(path, "wb") as out:
            out.write(raw_img + raw_tab[2880:])
        os.remove(tmp_img)
        os.remove(tmp_tab)
    return out_dir


def write_attributes(path, order=1):
    """Minimal delta-attributes file carrying FIT_METADATA/FITORDER."""
    fitsio_lite.write_fits(path, [{
        "columns": [np.zeros(1, dtype=np.int64)], "names": ["LOS_ID"],
        "extname": "FIT_METADATA",
        "header": [{"name": "FITORDER", "value": order}],
    }])
    return path


def write_stack_attributes(path):
    """Rebuild the STACK_DELTAS table of py/picca/tests/data/test_cor/
    input_from_delta_extraction_lya_nodla/Log/delta_attributes.fits.gz."""
    src = golden("stack_lya_nodla.npz")
    cols = list(src)
    fitsio_lite.write_fits(path, [{"columns": [src[c] for c in cols], "names": cols,
                                   "extname": "STACK_DELTAS"}])
    return path


def write_catalogue(path):
    """Rebuild py/picca/tests/data/test_delta/cat.fits."""
    src = golden("cat.npz")
    cols = list(src)
    fitsio_lite.write_fits(path, [{"columns": [src[c] for c in cols], "names": cols,
                                   "extname": "CAT"}])
    return path


@pytest.fixture(scope="session")
def picca_inputs(tmp_path_factory):
    """Directory with Delta_LYA/, Delta_LYA_image/, cat.fits and attributes."""
    base = tmp_path_factory.mktemp("picca_inputs")
    write_delta_dir(os.path.join(base, "Delta_LYA"))
    write_image_dir(os.path.join(base, "Delta_LYA_image"))
    write_catalogue(os.path.join(base, "cat.fits"))
    write_attributes(os.path.join(base, "delta_attributes.fits.gz"))
    return str(base)
