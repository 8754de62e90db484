"""The Dr16ExpectedFlux drop-in (picca's expected-flux plugin interface)
against the oracle's Dr16 loop, and its iteration files.

Same tolerances as the GPU continuum tests: fit parameters within 1e-7 of
the oracle's (FP64 mode), weights within 1e-6 relative, deltas within 1e-6
absolute, and the same accepted/rejected forests with the same reasons.
"""

import types

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CONFIG = {"iter out prefix": "delta_attributes", "num bins variance": "20",
          "num processors": "1", "var lss mod": "1.0", "num iterations": "3",
          "min num qso in fit": "5", "order": "1"}


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from picca_gb300 import build_ext
    build_ext.build()
    return torch


def _forests(raw):
    out = []
    for k in range(raw.num):
        ll, fl, iv, tc = raw.forest(k)
        out.append(types.SimpleNamespace(los_id=int(raw.los_id[k]), z=float(raw.z_qso[k]),
                                         log_lambda=ll.copy(), flux=fl.copy(), ivar=iv.copy(),
                                         transmission_correction=tc.copy()))
    return out


def test_plugin_matches_oracle(cuda, tmp_path):
    from oracle import continuum as oc
    from picca_gb300 import fitsio_lite, synthetic_spectra
    from picca_gb300.delta_extraction.expected_fluxes.dr16_expected_flux import (
        Dr16ExpectedFlux)
    raw = synthetic_spectra.make_raw_forests(300, 41)
    config = dict(CONFIG, **{"out dir": str(tmp_path) + "/"})
    (tmp_path / "Log").mkdir()
    flux = Dr16ExpectedFlux(config, grid=raw.grid)
    forests = _forests(raw)
    flux.compute_expected_flux(forests)

    orc = oc.Dr16Oracle(raw.grid, num_iterations=3, min_num_qso_in_fit=5)
    conts, params = orc.run(raw)
    ref_delta, ref_weights = orc.deltas(raw, conts)
    for k, forest in enumerate(forests):
        (a, b, chi2, ndata), reason = params[k]
        assert forest.bad_continuum_reason == reason
        got = flux.continuum_fit_parameters[forest.los_id]
        assert got[3] == ndata
        if reason is None:
            scale = max(1.0, abs(a), abs(b))
            assert abs(got[0] - a) <= 1e-7 * scale and abs(got[1] - b) <= 1e-7 * scale
            flux.extract_deltas(forest)
            sl = slice(raw.pix_offset[k], raw.pix_offset[k + 1])
            assert np.allclose(forest.weights, ref_weights[sl], rtol=1e-6, atol=0)
            w = ref_weights[sl] > 0
            assert np.allclose(forest.deltas[w], ref_delta[sl][w], rtol=0, atol=1e-6)
            # host weights of the interface equal the device weights
            host_w = flux.compute_forest_weights(forest, flux.los_ids[forest.los_id][
                "mean expected flux"])
            assert np.allclose(host_w, forest.weights, rtol=1e-12, atol=0)
        else:
            assert forest.los_id not in flux.los_ids
    # iteration files with the reference's HDUs
    for name in ("delta_attributes_iteration1.fits.gz", "delta_attributes_iteration2.fits.gz",
                 "delta_attributes.fits.gz"):
        hdul = fitsio_lite.FITS(str(tmp_path / "Log" / name))
        for ext in ("STACK_DELTAS", "VAR_FUNC", "CONT", "FIT_METADATA"):
            assert hdul[ext].get_nrows() > 0
    meta = fitsio_lite.FITS(str(tmp_path / "Log" / "delta_attributes.fits.gz"))["FIT_METADATA"]
    assert meta.get_nrows() == raw.num
    assert meta.read_header()["FITORDER"] == 1


def test_compute_continuum_function(cuda):
    from oracle import continuum as oc
    from picca_gb300 import synthetic_spectra
    from picca_gb300.delta_extraction.expected_fluxes.dr16_expected_flux import (
        compute_continuum)
    raw = synthetic_spectra.make_raw_forests(20, 43)
    orc = oc.Dr16Oracle(raw.grid)
    rest = raw.grid.log_lambda_rest_frame_grid
    for k, forest in enumerate(_forests(raw)[:5]):
        cont, reason, (a, b, chi2, ndata) = compute_continuum(
            forest, orc.get_mean_cont, orc.get_eta, orc.get_var_lss, orc.get_fudge, False, 1,
            grid=raw.grid)
        ll, fl, iv, tc = raw.forest(k)
        ref_cont, ref_reason, ref_fit, _ = oc.fit_forest(
            ll, fl, iv, raw.z_qso[k], orc.get_mean_cont, orc.get_eta, orc.get_var_lss,
            orc.get_fudge, rest[0], rest[-1], transmission_correction=tc, order=1)
        assert reason == ref_reason
        assert ndata == ref_fit[3]
        if reason is None:
            assert np.allclose(cont, ref_cont, rtol=1e-7, atol=0)
