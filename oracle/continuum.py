"""CPU oracle for the Dr16 continuum fit (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this module. It restates in FP64 numpy:

* ``LeastsSquaresContModel.__call__`` / ``get_continuum_model`` /
  ``get_continuum_weights`` (py/picca/delta_extraction/least_squares/
  least_squares_cont_model.py:65-197) as :func:`chi2`;
* ``compute_continuum`` (py/picca/delta_extraction/expected_fluxes/
  utils.py:12-136) as :func:`fit_forest`. The reference minimises with
  iminuit's MIGRAD (a third-party package absent here, iminuit>=2.26.0 per
  requirements.txt:3), which stops at an estimated distance to minimum of
  2e-4. This oracle minimises the same chi2 with a damped Newton iteration
  on (zero_point, slope) to |step| < 1e-12, i.e. it returns the optimum MIGRAD
  approaches; parity is therefore stated on chi2 and on (a, b) at the
  optimum;
* the Dr16 outer loop (py/picca/delta_extraction/expected_fluxes/
  dr16_expected_flux.py:380-464): mean-continuum update (expected_flux.py:
  256-308), variance statistics and (eta, var_lss, fudge) fit
  (dr16_expected_flux.py:516-617, least_squares_var_stats.py:83-214; the fit
  is a box-constrained linear least-squares problem, solved exactly with
  scipy.optimize.lsq_linear) and the delta stack (expected_flux.py:190-236).
"""

import numpy as np
from scipy.interpolate import interp1d
from scipy.optimize import lsq_linear

VAR_PIPE_MIN = np.log10(1e-5)
VAR_PIPE_MAX = np.log10(2.)
NUM_VAR_BINS = 100
FUDGE_REF = 1e-7


def continuum_model(log_lambda, zero_point, slope, mean_cont, ll_min, ll_max):
    """C = (b (L - Lmin)/(Lmax - Lmin) + a) * mean_cont (cont_model.py:97-144)."""
    line = slope * (log_lambda - ll_min) / (ll_max - ll_min) + zero_point
    return line * mean_cont


def continuum_weights(ivar, cont, eta, var_lss, fudge, use_constant_weight=False):
    """Weights of cont_model.py:146-197."""
    w = ivar > 0
    weights = np.empty_like(ivar)
    weights[~w] = 0
    if use_constant_weight:
        weights[w] = 1
        return weights
    var_pipe = 1. / ivar[w] / cont[w]**2
    variance = eta[w] * var_pipe + var_lss[w] + fudge[w] / var_pipe
    weights[w] = 1.0 / cont[w]**2 / variance
    return weights


def chi2(zero_point, slope, log_lambda, flux, ivar, mean_cont, eta, var_lss, fudge, ll_min,
         ll_max, use_constant_weight=False):
    """chi2 of cont_model.py:65-95 and the number of data points."""
    cont = continuum_model(log_lambda, zero_point, slope, mean_cont, ll_min, ll_max)
    weights = continuum_weights(ivar, cont, eta, var_lss, fudge, use_constant_weight)
    w = weights > 0
    contrib = (flux - cont)**2 * weights
    return contrib.sum() - np.log(weights[w]).sum(), int(flux[w].size)


def _chi2_derivatives(a, b, x, flux, ivar, mc, eta, vlss, fudge):
    """Analytic chi2, gradient and Hessian in (a, b) for ivar > 0 pixels.

    With C = (a + b x) mc and D = eta/ivar + vlss C^2 + fudge ivar C^4,
    chi2 = sum (f - C)^2 / D + sum log D."""
    c = (b * x + a) * mc
    c2 = c * c
    d = eta / ivar + vlss * c2 + fudge * ivar * c2 * c2
    dd = 2 * vlss * c + 4 * fudge * ivar * c2 * c          # dD/dC
    d2d = 2 * vlss + 12 * fudge * ivar * c2                 # d2D/dC2
    r = flux - c
    g = -2 * r / d - r * r * dd / (d * d) + dd / d          # dchi2/dC
    h = (2 / d + 4 * r * dd / (d * d) + 2 * r * r * dd * dd / d**3 - r * r * d2d / (d * d)
         + d2d / d - dd * dd / (d * d))                     # d2chi2/dC2
    val = (r * r / d).sum() + np.log(d).sum()
    ja, jb = mc, x * mc
    grad = np.array([(g * ja).sum(), (g * jb).sum()])
    hess = np.array([[(h * ja * ja).sum(), (h * ja * jb).sum()],
                     [(h * ja * jb).sum(), (h * jb * jb).sum()]])
    return val, grad, hess


def newton_fit(a0, b0, x, flux, ivar, mc, eta, vlss, fudge, fix_slope=False, max_iter=100,
               tol=1e-12):
    """Damped Newton minimisation of chi2(a, b); returns (a, b, iterations, ok)."""
    a, b = float(a0), float(b0)
    val, grad, hess = _chi2_derivatives(a, b, x, flux, ivar, mc, eta, vlss, fudge)
    for it in range(max_iter):
        if fix_slope:
            step = np.array([-grad[0] / hess[0, 0] if hess[0, 0] > 0 else -grad[0], 0.0])
        else:
            try:
                step = -np.linalg.solve(hess, grad)
                if step @ grad >= 0:  # not a descent direction: gradient step
                    step = -grad / max(np.abs(np.diag(hess)).max(), 1e-300)
            except np.linalg.LinAlgError:
                step = -grad / max(np.abs(np.diag(hess)).max(), 1e-300)
        t = 1.0
        while True:
            na, nb = a + t * step[0], b + t * step[1]
            nval, ngrad, nhess = _chi2_derivatives(na, nb, x, flux, ivar, mc, eta, vlss, fudge)
            if np.isfinite(nval) and nval <= val + 1e-4 * t * (step @ grad):
                break
            t *= 0.5
            if t < 1e-10:
                return a, b, it, bool(np.abs(grad).max() < 1e-6 * max(1.0, abs(val)))
        a, b, val, grad, hess = na, nb, nval, ngrad, nhess
        if np.abs(t * step).max() < tol * max(1.0, abs(a), abs(b)):
            return a, b, it + 1, True
    return a, b, max_iter, False


def fit_forest(log_lambda, flux, ivar, z_qso, get_mean_cont, get_eta, get_var_lss, get_fudge,
               ll_rest_min, ll_rest_max, transmission_correction=None, order=1,
               use_constant_weight=False):
    """compute_continuum (utils.py:12-136) with the Newton minimiser.

    Returns (cont or None, bad_continuum_reason, (a, b, chi2, ndata), start)."""
    mean_cont = get_mean_cont(log_lambda - np.log10(1 + z_qso))
    if transmission_correction is not None:
        mean_cont = mean_cont * transmission_correction
    ll_max = ll_rest_max + np.log10(1 + z_qso)
    ll_min = ll_rest_min + np.log10(1 + z_qso)
    eta, var_lss, fudge = get_eta(log_lambda), get_var_lss(log_lambda), get_fudge(log_lambda)
    zero_point = (flux * ivar).sum() / ivar.sum()
    w = ivar > 0
    x = (log_lambda - ll_min) / (ll_max - ll_min)
    if use_constant_weight:
        # unit weights: chi2 = sum (f - C)^2 is linear least squares in (a, b)
        ja, jb = mean_cont[w], x[w] * mean_cont[w]
        if order == 0:
            a, b = float((ja * flux[w]).sum() / (ja * ja).sum()), 0.0
        else:
            mat = np.array([[(ja * ja).sum(), (ja * jb).sum()], [(ja * jb).sum(), (jb * jb).sum()]])
            a, b = np.linalg.solve(mat, [(ja * flux[w]).sum(), (jb * flux[w]).sum()])
        ok = True
    else:
        a, b, _, ok = newton_fit(zero_point, 0.0, x[w], flux[w], ivar[w], mean_cont[w], eta[w],
                                 var_lss[w], fudge[w], fix_slope=(order == 0))
    cont = continuum_model(log_lambda, a, b, mean_cont, ll_min, ll_max)
    reason = None
    if not ok:
        reason = "minuit didn't converge"
    if np.any(cont < 0):
        reason = "negative continuum"
    if np.all(cont == 0):
        reason = "zero continuum"
    value, ndata = chi2(a, b, log_lambda, flux, ivar, mean_cont, eta, var_lss, fudge, ll_min,
                        ll_max, use_constant_weight)
    if reason is None:
        return cont, None, (a, b, value, ndata), zero_point
    return None, reason, (np.nan, np.nan, np.nan, ndata), zero_point


def var_stats_fit(var_delta, var2_delta, num_qso, var_pipe_values, min_num_qso, limit_eta,
                  limit_var_lss, fit_eta=True, fit_var_lss=True, fit_fudge=True, start=None):
    """(eta, var_lss, fudge) of one wavelength bin: the chi2 of
    least_squares_var_stats.py:104-132 is linear least squares in (eta,
    var_lss, fudge/FUDGE_REF) with box limits; solved exactly."""
    sel = (num_qso > min_num_qso) & (var2_delta > 0)
    if sel.sum() == 0:
        return None
    wgt = 1.0 / np.sqrt(var2_delta[sel])
    cols = [var_pipe_values[sel], np.ones(sel.sum()), FUDGE_REF / var_pipe_values[sel]]
    lo = [limit_eta[0], limit_var_lss[0], 0.0]
    hi = [limit_eta[1], limit_var_lss[1], np.inf]
    fixed = [not fit_eta, not fit_var_lss, not fit_fudge]
    target = var_delta[sel].copy()
    keep = []
    for k in range(3):
        if fixed[k]:
            target -= cols[k] * start[k]
        else:
            keep.append(k)
    mat = np.stack([cols[k] * wgt for k in keep], axis=1)
    res = lsq_linear(mat, target * wgt, bounds=([lo[k] for k in keep], [hi[k] for k in keep]),
                     method="bvls", tol=1e-14)
    out = list(start) if start is not None else [1.0, 0.1, 0.0]
    for k, v in zip(keep, res.x):
        out[k] = v
    return out[0], out[1], out[2] * FUDGE_REF
