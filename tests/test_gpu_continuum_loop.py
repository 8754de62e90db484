"""The GPU Dr16 loop (continuum.Dr16Gpu) against picca's own loop functions.

The fixtures ``continuum_loop_<grid>.npz`` are written by
tests/golden/make_golden.py, which runs picca's
Dr16ExpectedFlux.compute_expected_flux
(py/picca/delta_extraction/expected_fluxes/dr16_expected_flux.py:380-464)
as plain Python on synthetic raw forests, with a SciPy minimiser standing in
for iminuit (not installed), and records every iteration. Here the GPU loop
runs on the same forests; at every iteration the reference's fitted
(zero point, slope) are injected (the fit kernels evaluate the model at a
given start with max_iter = 0), so that everything downstream of the
minimiser is compared exactly:

* chi2 and ndata at those parameters (least_squares_cont_model.py:65-95);
* the mean continuum (_compute_mean_cont, expected_flux.py:256-308);
* the variance statistics (LeastsSquaresVarStats.initialize_delta_arrays,
  least_squares_var_stats.py:134-184) and the fitted eta / var_lss / fudge;
* the delta stack (compute_delta_stack, expected_flux.py:190-236);
* the final expected flux and weights (populate_los_ids,
  dr16_expected_flux.py:706-740, compute_forest_weights :466-488) and the
  deltas (extract_deltas, expected_flux.py:328-349).

The GPU's own Newton fit is then compared with the reference's minimum at
the reference's model state (find_bins is pinned on the CPU,
tests/test_oracle_continuum.py). Tolerances: sums that differ only by summation
order within 1e-9 relative; counts exact; the variance functions (bounded
least squares here, a general minimiser in the fixture) within 2e-5.
"""

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from picca_gb300 import build_ext
    build_ext.build()
    return torch


def _setup(f):
    from picca_gb300 import continuum, synthetic_spectra
    wave = str(f["wave_solution"])
    step = 3e-4 if wave == "log" else 0.8
    grid = synthetic_spectra.Grid(step=step, wave_solution=wave)
    # the linear grid is log10 of the wavelengths, which libm may round one
    # ulp apart on another machine: the fixture's own grids are used
    for key in ("log_lambda_grid", "log_lambda_rest_frame_grid"):
        assert np.allclose(getattr(grid, key), f[key], rtol=0, atol=1e-14)
        setattr(grid, key, f[key].copy())
    raw = synthetic_spectra.RawForests(
        pix_offset=f["pix_offset"], log_lambda=f["log_lambda"], flux=f["flux"],
        ivar=f["ivar"], transmission_correction=f["transmission_correction"],
        z_qso=f["z_qso"], los_id=f["los_id"], grid=grid)
    eng = continuum.Dr16Gpu(grid, num_iterations=int(f["num_iterations"]),
                            min_num_qso_in_fit=int(f["min_num_qso_in_fit"]),
                            fit_mode=continuum.FIT_FP64)
    assert np.allclose(eng.log_lambda_var_func_grid, f["log_lambda_var_func_grid"],
                       rtol=0, atol=1e-14)
    return eng, raw, continuum.DeviceSpectra(raw, eng.device)


def _inject(eng, spectra, f, it):
    """The fit of iteration ``it`` at the reference's parameters: good
    forests evaluated at (zero point, slope), the others marked bad."""
    import torch
    pre = f"it{it}_"
    good = ~f[pre + "bad"]
    n = spectra.num
    dev = eng.device
    out = {"zero_point": torch.full((n,), float("nan"), dtype=torch.float64, device=dev),
           "slope": torch.full((n,), float("nan"), dtype=torch.float64, device=dev),
           "chi2": torch.full((n,), float("nan"), dtype=torch.float64, device=dev),
           "ndata": torch.zeros(n, dtype=torch.int32, device=dev),
           "status": torch.ones(n, dtype=torch.int32, device=dev),
           "iterations": torch.zeros(n, dtype=torch.int32, device=dev),
           "continuum": torch.zeros(max(spectra.num_pixels, 1), dtype=torch.float64,
                                    device=dev)}
    start = np.stack([np.nan_to_num(f[pre + "zero_point"]), np.nan_to_num(f[pre + "slope"])], 1)
    index = np.nonzero(good)[0].astype(np.int32)
    return eng.fit(spectra, start=start, max_iter=0, index=index, out=out), good


def _set_state(eng, f, it):
    """Continue from the reference's model state after iteration ``it``."""
    from scipy.interpolate import interp1d  # noqa: F401
    pre = f"it{it}_"
    eng.mean_cont_x = f[pre + "mean_cont_x"].copy()
    eng.mean_cont_y = f[pre + "mean_cont_y"].copy()
    nodes = np.isin(f["log_lambda_var_func_grid"], f[pre + "var_x"])
    eng.var_x = f[pre + "var_x"].copy()
    eng.eta = f[pre + "eta"][nodes].copy()
    eng.var_lss = f[pre + "var_lss"][nodes].copy()
    eng.fudge = f[pre + "fudge"][nodes].copy()


@pytest.mark.parametrize("wave", ["log", "lin"])
def test_dr16_loop_matches_reference_functions(cuda, wave):
    from picca_gb300 import continuum
    f = golden(f"continuum_loop_{wave}.npz")
    eng, raw, spectra = _setup(f)
    iters = int(f["num_iterations"])
    fit = None
    for it in range(iters):
        pre = f"it{it}_"
        fit, good = _inject(eng, spectra, f, it)
        host = continuum.fit_results_to_host(fit)
        assert np.array_equal(host["status"] == 0, good), it
        assert np.allclose(host["chi2"][good], f[pre + "chi2"][good], rtol=1e-10, atol=1e-10), it
        assert np.array_equal(host["ndata"][good], f[pre + "ndata"][good].astype(int)), it
        last = it == iters - 1
        if not last:
            sums = eng._stacks(spectra, fit, mean_cont=True, var_stats=True, delta_stack=False)
            # variance statistics before the fits
            stats = continuum.normalise_var_stats(sums)
            np.testing.assert_array_equal(stats["num_pixels"], f[pre + "num_pixels"])
            np.testing.assert_array_equal(stats["num_qso"], f[pre + "num_qso"])
            for key in ("var_delta", "var2_delta"):
                np.testing.assert_allclose(stats[key], f[pre + key], rtol=1e-9, atol=1e-14,
                                           err_msg=f"{key} iteration {it}")
            eng.update_mean_cont(sums)
            np.testing.assert_array_equal(eng.mean_cont_x, f[pre + "mean_cont_x"])
            np.testing.assert_allclose(eng.mean_cont_y, f[pre + "mean_cont_y"], rtol=1e-9)
            np.testing.assert_allclose(eng.mean_cont_weight, f[pre + "mean_cont_weight"],
                                       rtol=1e-9)
            eng.update_var_functions(sums)
            np.testing.assert_array_equal(eng.var_x, f[pre + "var_x"])
            nodes = np.isin(f["log_lambda_var_func_grid"], f[pre + "var_x"])
            np.testing.assert_allclose(eng.eta, f[pre + "eta"][nodes], rtol=0, atol=2e-5)
            np.testing.assert_allclose(eng.var_lss, f[pre + "var_lss"][nodes], rtol=0, atol=2e-5)
            fudge_ref = f[pre + "fudge"][nodes] / continuum.FUDGE_REF
            assert np.all(np.abs(eng.fudge / continuum.FUDGE_REF - fudge_ref) <=
                          2e-5 * np.maximum(1.0, np.abs(fudge_ref))), it
            _set_state(eng, f, it)
        # the delta stack, with the variance functions of this iteration's end
        sums = eng._stacks(spectra, fit, mean_cont=False, var_stats=False, delta_stack=True)
        eng.update_stack(sums)
        np.testing.assert_array_equal(eng.stack_x, f[pre + "stack_x"])
        np.testing.assert_allclose(eng.stack_y, f[pre + "stack_y"], rtol=1e-9)
        eng.stack_y = f[pre + "stack_y"].copy()
    # final deltas and weights
    delta, weights = eng.deltas(spectra, fit)
    delta, weights = delta.cpu().numpy(), weights.cpu().numpy()
    good = np.isin(f["los_id"], f["los_good"])
    po = f["pix_offset"]
    sel = np.concatenate([np.arange(po[k], po[k + 1]) for k in np.nonzero(good)[0]])
    np.testing.assert_allclose(weights[sel], f["los_weights"], rtol=1e-10, atol=0)
    w = f["los_weights"] > 0
    want = f["flux"][sel][w] / f["los_mean_expected_flux"][w] - 1
    np.testing.assert_allclose(delta[sel][w], want, rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("wave", ["log", "lin"])
@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_newton_fit_matches_reference_minimum(cuda, wave, mode):
    """The GPU Newton fit from picca's starting point at the reference's
    model state reaches the minimum that the fixture's minimiser found on
    picca's own chi2: (a, b) within 1e-4 of max(1, |a|, |b|) and the chi2 at
    least as low (within 1e-6 of max(|chi2|, ndata))."""
    from picca_gb300 import continuum
    f = golden(f"continuum_loop_{wave}.npz")
    eng, raw, spectra = _setup(f)
    eng.fit_mode = continuum.FIT_FP64 if mode == "fp64" else continuum.FIT_MIXED
    for it in range(int(f["num_iterations"])):
        pre = f"it{it}_"
        fit = continuum.fit_results_to_host(eng.fit(spectra))
        good = ~f[pre + "bad"] & (fit["status"] == 0)
        assert good.mean() > 0.9
        a, b = f[pre + "zero_point"][good], f[pre + "slope"][good]
        scale = np.maximum(1.0, np.maximum(np.abs(a), np.abs(b)))
        assert np.max(np.abs(fit["zero_point"][good] - a) / scale) < 1e-4, it
        assert np.max(np.abs(fit["slope"][good] - b) / scale) < 1e-4, it
        chi_scale = np.maximum(np.abs(f[pre + "chi2"][good]), f[pre + "ndata"][good])
        excess = (fit["chi2"][good] - f[pre + "chi2"][good]) / chi_scale
        k = int(np.argmax(excess))
        assert excess[k] <= 1e-6, (it, k, fit["chi2"][good][k], f[pre + "chi2"][good][k],
                                   fit["zero_point"][good][k], a[k], fit["slope"][good][k], b[k],
                                   fit["iterations"][good][k])
        if it + 1 < int(f["num_iterations"]):
            _set_state(eng, f, it)
        eng.stack_x, eng.stack_y = f[pre + "stack_x"], f[pre + "stack_y"]
