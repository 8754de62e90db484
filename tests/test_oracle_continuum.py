"""Pin the continuum-fit oracle.

* ``oracle.continuum.chi2`` is bit-identical to picca's own
  ``LeastsSquaresContModel.__call__`` (least_squares_cont_model.py:65-95) and
  its ndata, on the fixtures made by tests/golden/make_golden.py.
* The reference minimises with iminuit's MIGRAD (absent here); the oracle's
  damped Newton minimiser is checked to reach the minimum: no lower chi2 is
  found by scipy's Nelder-Mead from the same start, and the gradient is
  zero at the solution.
* The (eta, var_lss, fudge) solver minimises the reference objective
  (least_squares_var_stats.py:104-132) within its box limits.
"""

import numpy as np
import pytest
from scipy.optimize import minimize

from conftest import golden
from oracle import continuum as oc


def _case(f, k):
    pre = f"c{k}_"
    return {key: f[pre + key] for key in ("ll", "flux", "ivar", "mean_cont", "eta", "var_lss",
                                          "fudge", "scalars", "points", "chi2", "ndata")}


def test_chi2_matches_reference_bit_for_bit():
    f = golden("continuum_cases.npz")
    for k in range(int(f["num_cases"])):
        c = _case(f, k)
        _, ll_min, ll_max = c["scalars"]
        for (a, b), want in zip(c["points"], c["chi2"]):
            got, ndata = oc.chi2(a, b, c["ll"], c["flux"], c["ivar"], c["mean_cont"], c["eta"],
                                 c["var_lss"], c["fudge"], ll_min, ll_max)
            assert got == want, (k, a, b, got, want)
        assert ndata == int(c["ndata"])


def test_newton_reaches_the_minimum():
    f = golden("continuum_cases.npz")
    for k in range(int(f["num_cases"])):
        c = _case(f, k)
        _, ll_min, ll_max = c["scalars"]
        w = c["ivar"] > 0
        x = (c["ll"] - ll_min) / (ll_max - ll_min)
        a0 = (c["flux"] * c["ivar"]).sum() / c["ivar"].sum()
        a, b, iters, ok = oc.newton_fit(a0, 0.0, x[w], c["flux"][w], c["ivar"][w],
                                        c["mean_cont"][w], c["eta"][w], c["var_lss"][w],
                                        c["fudge"][w])
        assert ok and iters < 50

        def fun(p):
            return oc.chi2(p[0], p[1], c["ll"], c["flux"], c["ivar"], c["mean_cont"], c["eta"],
                           c["var_lss"], c["fudge"], ll_min, ll_max)[0]

        best = fun([a, b])
        res = minimize(fun, [a0, 0.0], method="Nelder-Mead",
                       options={"xatol": 1e-12, "fatol": 1e-12, "maxiter": 20000})
        assert best <= res.fun + 1e-9 * abs(res.fun)
        _, grad, _ = oc._chi2_derivatives(a, b, x[w], c["flux"][w], c["ivar"][w],
                                          c["mean_cont"][w], c["eta"][w], c["var_lss"][w],
                                          c["fudge"][w])
        assert np.abs(grad).max() < 1e-6 * max(1.0, abs(best))


def test_var_stats_solver_minimises_reference_objective():
    rng = np.random.default_rng(3)
    var_pipe = 10**(oc.VAR_PIPE_MIN + ((np.arange(oc.NUM_VAR_BINS) + .5) *
                                       (oc.VAR_PIPE_MAX - oc.VAR_PIPE_MIN) / oc.NUM_VAR_BINS))
    for _ in range(5):
        eta, vlss, fudge = rng.uniform(0.6, 1.4), rng.uniform(0.01, 0.25), rng.uniform(0, 2)
        var_delta = eta * var_pipe + vlss + fudge * oc.FUDGE_REF / var_pipe
        var_delta *= 1 + 0.05 * rng.normal(size=var_pipe.size)
        var2 = (0.1 * var_delta)**2 + 1e-6
        nqso = rng.integers(50, 500, var_pipe.size).astype(float)

        def objective(p):
            model = p[0] * var_pipe + p[1] + p[2] * oc.FUDGE_REF / var_pipe
            sel = nqso > 100
            return np.sum((var_delta - model)[sel]**2 / var2[sel])

        sol = oc.var_stats_fit(var_delta, var2, nqso, var_pipe, 100, (0.5, 1.5), (0., 0.3),
                               start=[1.0, 0.1, 0.0])
        best = objective([sol[0], sol[1], sol[2] / oc.FUDGE_REF])
        res = minimize(objective, [1.0, 0.1, 0.0], method="L-BFGS-B",
                       bounds=[(0.5, 1.5), (0., 0.3), (0, None)],
                       options={"ftol": 1e-15, "gtol": 1e-12, "maxiter": 10000})
        assert best <= res.fun * (1 + 1e-9) + 1e-12


@pytest.mark.parametrize("wave", ["log", "lin"])
def test_find_bins_match_reference(wave):
    """find_bins_log / find_bins_lin of the host code on the fixture's pixels
    (observed, rest-frame and variance grids) equal picca's."""
    from picca_gb300 import synthetic_spectra
    f = golden(f"continuum_loop_{wave}.npz")
    grid = synthetic_spectra.Grid(step=3e-4 if wave == "log" else 0.8, wave_solution=wave)
    zpix = np.repeat(f["z_qso"], np.diff(f["pix_offset"]))
    ll = f["log_lambda"]
    np.testing.assert_array_equal(grid.find_bins(ll, grid.log_lambda_grid), f["bins_obs"])
    np.testing.assert_array_equal(
        grid.find_bins(ll - np.log10(1 + zpix), grid.log_lambda_rest_frame_grid), f["bins_rest"])
    np.testing.assert_array_equal(grid.find_bins(ll, f["log_lambda_var_func_grid"]),
                                  f["bins_var"])


def test_box_lsq3_matches_bounded_least_squares():
    """The exact face-enumeration solver of the (eta, var_lss, fudge) fits
    (continuum.box_lsq3) equals scipy's bounded least squares (BVLS) on
    random problems with and without active bounds."""
    from scipy.optimize import lsq_linear
    from picca_gb300 import continuum
    rng = np.random.default_rng(3)
    var_pipe = 10**rng.uniform(-5, 0.3, 40)
    for trial in range(200):
        n = int(rng.integers(3, 40))
        v = var_pipe[:n]
        mat = np.stack([v, np.ones(n), 1e-7 / v], axis=1) * rng.uniform(0.5, 2, n)[:, None]
        truth = np.array([rng.uniform(0.2, 1.8), rng.uniform(-0.1, 0.4), rng.uniform(-1, 3)])
        rhs = mat @ truth + rng.normal(0, 0.05, n) * np.abs(mat @ truth).mean()
        got = continuum.box_lsq3(mat, rhs, (0.5, 1.5), (0.0, 0.3))
        want = lsq_linear(mat, rhs, bounds=([0.5, 0.0, 0.0], [1.5, 0.3, np.inf]),
                          method="bvls", tol=1e-14).x
        if got is None:
            continue
        f_got = np.sum((mat @ got - rhs) ** 2)
        f_want = np.sum((mat @ want - rhs) ** 2)
        assert f_got <= f_want * (1 + 1e-10) + 1e-300, trial
        np.testing.assert_allclose(got, want, rtol=1e-6, atol=1e-9)
