"""GPU parity of the Dr16 continuum fit (through the C ABI).

Tolerances: the GPU and the oracle minimise the same chi2 to the same
optimum (|step| < 1e-10 relative); FP64 mode: (a, b) within 1e-7 relative,
chi2 within 1e-10 relative; mixed mode (FP32 per-pixel terms and sums, FP64
2x2 solve; the FP32 rounding of the gradient and of the model leaves about
1e-7 on the optimum, and forests where it is estimated above 2e-6 are finished
in FP64): (a, b) within 3e-6, chi2 within 1e-6, the FP32 continuum within
3e-6 relative. chi2 = sum (f - C)^2 / D + sum log D is a sum
of terms of either sign that can cancel, so its tolerance is relative to
max(|chi2|, ndata), the scale of the sum of |terms| (each (f - C)^2 / D is
about one). Histogram sums of positive terms agree to 1e-8 relative (only
the summation order and the fit's stopping point differ); the signed sum of
deltas per variance bin to 1e-7 of its sum of |delta|, bounded above by
sqrt(count * sum delta^2). After three iterations of the full loop the mean
continuum, the variance functions and the weights agree to 1e-6 relative
and the deltas to 1e-6 absolute.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("GPU tests need a CUDA device")
    from picca_gb300 import build_ext
    build_ext.build()
    return torch


@pytest.fixture(scope="module")
def raw():
    from picca_gb300 import synthetic_spectra
    return synthetic_spectra.make_raw_forests(400, 31)


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_fit_matches_oracle(cuda, raw, mode):
    from oracle import continuum as oc
    from picca_gb300 import continuum
    fit_mode = continuum.FIT_FP64 if mode == "fp64" else continuum.FIT_MIXED
    gpu = continuum.Dr16Gpu(raw.grid, num_iterations=1, fit_mode=fit_mode)
    spectra = continuum.DeviceSpectra(raw, gpu.device)
    res = continuum.fit_results_to_host(gpu.fit(spectra))
    orc = oc.Dr16Oracle(raw.grid)
    conts, params = orc.fit_all(raw)
    tol_ab, tol_chi2 = (1e-7, 1e-10) if mode == "fp64" else (3e-6, 1e-6)
    for k in range(raw.num):
        (a, b, chi2, ndata), reason = params[k]
        status = res["status"][k]
        assert continuum.STATUS_REASONS[int(status)] == reason, (k, status, reason)
        assert res["ndata"][k] == ndata
        if reason is None:
            scale = max(1.0, abs(a), abs(b))
            assert abs(res["zero_point"][k] - a) <= tol_ab * scale, k
            assert abs(res["slope"][k] - b) <= tol_ab * scale, k
            assert abs(res["chi2"][k] - chi2) <= tol_chi2 * max(abs(chi2), ndata), k
            sl = slice(raw.pix_offset[k], raw.pix_offset[k + 1])
            assert np.allclose(res["continuum"][sl], conts[k], rtol=tol_ab, atol=0)


def test_stacks_match_oracle(cuda, raw):
    from oracle import continuum as oc
    from picca_gb300 import continuum
    gpu = continuum.Dr16Gpu(raw.grid, num_iterations=1)
    spectra = continuum.DeviceSpectra(raw, gpu.device)
    fit = gpu.fit(spectra)
    sums = gpu._stacks(spectra, fit)
    orc = oc.Dr16Oracle(raw.grid)
    conts, _ = orc.fit_all(raw)
    ref = orc.stacks(raw, conts)
    for key in ref:
        if key == "v_mean":
            abs_scale = np.sqrt(ref["v_np"] * ref["v_d2"])
            assert np.all(np.abs(sums[key] - ref[key]) <= 1e-7 * abs_scale + 1e-12), key
        else:
            assert np.allclose(sums[key], ref[key], rtol=1e-8, atol=1e-8), key


def test_dr16_loop_matches_oracle(cuda, raw):
    from oracle import continuum as oc
    from picca_gb300 import continuum
    gpu = continuum.Dr16Gpu(raw.grid, num_iterations=3, min_num_qso_in_fit=5)
    spectra = continuum.DeviceSpectra(raw, gpu.device)
    fit = gpu.run(spectra)
    delta, weights = gpu.deltas(spectra, fit)
    orc = oc.Dr16Oracle(raw.grid, num_iterations=3, min_num_qso_in_fit=5)
    conts, params = orc.run(raw)
    ref_delta, ref_weights = orc.deltas(raw, conts)
    grid = orc.var_grid
    assert np.allclose(orc.get_eta(grid), continuum.interp1d(
        gpu.var_x, gpu.eta, kind="cubic", fill_value="extrapolate")(grid), rtol=1e-6, atol=1e-9)
    assert np.allclose(orc.get_mean_cont(raw.grid.log_lambda_rest_frame_grid),
                       continuum.interp1d(gpu.mean_cont_x, gpu.mean_cont_y,
                                          fill_value="extrapolate")(
                           raw.grid.log_lambda_rest_frame_grid), rtol=1e-6)
    status = fit["status"].cpu().numpy()
    assert np.array_equal(status == 0, np.array([p[1] is None for p in params]))
    w = ref_weights > 0
    assert np.array_equal(weights.cpu().numpy() > 0, w)
    assert np.allclose(weights.cpu().numpy(), ref_weights, rtol=1e-6)
    assert np.allclose(delta.cpu().numpy()[w], ref_delta[w], rtol=0, atol=1e-6)


def test_fit_select_matches_full_fit(cuda, raw):
    """pg_cont_fit_select fits only the listed forests, writes them in
    place, and gives the results of the full fit."""
    import torch
    from picca_gb300 import continuum
    gpu = continuum.Dr16Gpu(raw.grid, num_iterations=1, fit_mode=continuum.FIT_MIXED)
    spectra = continuum.DeviceSpectra(raw, gpu.device)
    full = continuum.fit_results_to_host(gpu.fit(spectra))
    out = gpu.fit(spectra)
    for key in ("zero_point", "slope", "chi2"):
        out[key].fill_(-7.0)
    index = torch.arange(1, raw.num, 3, dtype=torch.int32, device=gpu.device)
    gpu.fit(spectra, index=index, out=out)
    got = continuum.fit_results_to_host(out)
    sel = np.zeros(raw.num, bool)
    sel[index.cpu().numpy()] = True
    ok = sel & (full["status"] == 0)
    for key in ("zero_point", "slope", "chi2"):
        assert np.array_equal(got[key][ok], full[key][ok]), key
        assert np.all(got[key][~sel] == -7.0), key
    assert np.array_equal(got["status"][sel], full["status"][sel])
