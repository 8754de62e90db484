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


def find_bins_log(values, grid):
    """find_bins_log (py/picca/delta_extraction/utils.py:163-186)."""
    step = grid[1] - grid[0]
    return ((values - grid[0]) / step + 0.5).astype(np.int64)


def forest_weights(log_lambda, ivar, continuum, get_eta, get_var_lss, get_fudge, var_lss_mod=1.0):
    """Dr16ExpectedFlux.compute_forest_weights (dr16_expected_flux.py:466-488)."""
    w = ivar > 0
    weights = np.empty_like(log_lambda)
    weights[~w] = 0.0
    var_pipe = 1. / ivar[w] / continuum[w]**2
    weights[w] = 1.0 / (get_eta(log_lambda[w]) * var_pipe +
                        var_lss_mod * get_var_lss(log_lambda[w]) +
                        get_fudge(log_lambda[w]) / var_pipe)
    return weights


class Dr16Oracle:
    """Dr16ExpectedFlux.compute_expected_flux restated per forest in numpy
    (dr16_expected_flux.py:380-464 with the helpers cited above)."""

    def __init__(self, grid, num_iterations=5, order=1, limit_eta=(0.5, 1.5),
                 limit_var_lss=(0., 0.3), min_num_qso_in_fit=100, num_bins_variance=20,
                 var_lss_mod=1.0):
        self.grid = grid
        self.num_iterations = num_iterations
        self.order = order
        self.limit_eta = limit_eta
        self.limit_var_lss = limit_var_lss
        self.min_num_qso_in_fit = min_num_qso_in_fit
        self.var_lss_mod = var_lss_mod
        rest = grid.log_lambda_rest_frame_grid
        self.var_grid = np.linspace(grid.log_lambda_grid[0], grid.log_lambda_grid[-1],
                                    num_bins_variance)
        self.get_mean_cont = interp1d(rest, np.ones_like(rest), fill_value="extrapolate")
        nvb = num_bins_variance
        self.get_eta = interp1d(self.var_grid, np.ones(nvb), fill_value="extrapolate",
                                kind="cubic")
        self.get_var_lss = interp1d(self.var_grid, np.full(nvb, 0.1), fill_value="extrapolate",
                                    kind="cubic")
        self.get_fudge = interp1d(self.var_grid, np.zeros(nvb), fill_value="extrapolate",
                                  kind="cubic")
        self.get_stack_delta = None

    def fit_all(self, raw):
        rest = self.grid.log_lambda_rest_frame_grid
        conts, params = [], []
        for k in range(raw.num):
            ll, fl, iv, tc = raw.forest(k)
            cont, reason, fit, _ = fit_forest(ll, fl, iv, raw.z_qso[k], self.get_mean_cont,
                                              self.get_eta, self.get_var_lss, self.get_fudge,
                                              rest[0], rest[-1], transmission_correction=tc,
                                              order=self.order)
            conts.append(cont)
            params.append((fit, reason))
        return conts, params

    def stacks(self, raw, conts):
        grid = self.grid
        rest, obs = grid.log_lambda_rest_frame_grid, grid.log_lambda_grid
        out = {"mc_num": np.zeros_like(rest), "mc_w": np.zeros_like(rest),
               "s_num": np.zeros_like(obs), "s_w": np.zeros_like(obs)}
        nvar = len(self.var_grid) * NUM_VAR_BINS
        for key in ("v_mean", "v_d2", "v_d4", "v_np", "v_nq"):
            out[key] = np.zeros(nvar)
        for k in range(raw.num):
            cont = conts[k]
            if cont is None:
                continue
            ll, fl, iv, _ = raw.forest(k)
            weights = forest_weights(ll, iv, cont, self.get_eta, self.get_var_lss,
                                     self.get_fudge, self.var_lss_mod)
            bins = find_bins_log(ll - np.log10(1 + raw.z_qso[k]), rest)
            out["mc_num"] += np.bincount(bins, weights=fl / (cont + 1e-16) * weights,
                                         minlength=len(rest))
            out["mc_w"] += np.bincount(bins, weights=weights, minlength=len(rest))
            delta = np.zeros_like(ll)
            w = iv > 0
            delta[w] = fl[w] / cont[w]
            bins = find_bins_log(ll, obs)
            out["s_num"] += np.bincount(bins, weights=delta * weights, minlength=len(obs))
            out["s_w"] += np.bincount(bins, weights=weights, minlength=len(obs))
            var_pipe = np.empty_like(ll)
            var_pipe[w] = 1 / iv[w] / cont[w]**2
            var_pipe[~w] = np.inf
            w &= (np.log10(var_pipe) > VAR_PIPE_MIN) & (np.log10(var_pipe) < VAR_PIPE_MAX)
            vbins = ((np.log10(var_pipe[w]) - VAR_PIPE_MIN) /
                     (VAR_PIPE_MAX - VAR_PIPE_MIN) * NUM_VAR_BINS).astype(int)
            lbins = find_bins_log(ll[w], self.var_grid)
            bins = vbins + NUM_VAR_BINS * lbins
            d = fl[w] / cont[w] - 1
            out["v_mean"] += np.bincount(bins, weights=d, minlength=nvar)
            out["v_d2"] += np.bincount(bins, weights=d**2, minlength=nvar)
            out["v_d4"] += np.bincount(bins, weights=d**4, minlength=nvar)
            out["v_np"] += np.bincount(bins, minlength=nvar)
            out["v_nq"][np.unique(bins)] += 1
        return out

    def update(self, sums, last):
        """Mean continuum (expected_flux.py:291-308), variance functions
        (least_squares_var_stats.py:183-198, dr16_expected_flux.py:531-617)
        and the delta stack (expected_flux.py:226-236) from the bin sums."""
        grid = self.grid
        if not last:
            mean_cont = sums["mc_num"].copy()
            w = sums["mc_w"] > 0
            mean_cont[w] /= sums["mc_w"][w]
            mean_cont /= mean_cont[w].mean()
            rest = grid.log_lambda_rest_frame_grid[w]
            new_cont = self.get_mean_cont(rest) * mean_cont[w]
            self.get_mean_cont = interp1d(rest, new_cont, fill_value="extrapolate")
            var_delta = sums["v_d2"].copy()
            mean_delta = sums["v_mean"].copy()
            var2 = sums["v_d4"].copy()
            npix = sums["v_np"]
            w = npix > 0
            var_delta[w] /= npix[w]
            mean_delta[w] /= npix[w]
            var_delta -= mean_delta**2
            var2[w] /= npix[w]
            var2 -= var_delta**2
            var2[w] /= npix[w]
            var_pipe = 10**(VAR_PIPE_MIN + ((np.arange(NUM_VAR_BINS) + .5) *
                                            (VAR_PIPE_MAX - VAR_PIPE_MIN) / NUM_VAR_BINS))
            eta = self.get_eta(self.var_grid)
            vlss = self.get_var_lss(self.var_grid)
            fudge = self.get_fudge(self.var_grid)
            npix_bin = np.zeros(len(self.var_grid))
            for index in range(len(self.var_grid)):
                sl = slice(index * NUM_VAR_BINS, (index + 1) * NUM_VAR_BINS)
                npix_bin[index] = npix[sl].sum()
                sel = (sums["v_nq"][sl] > self.min_num_qso_in_fit) & (var2[sl] > 0)
                if sel.sum() == 0:
                    continue
                sol = var_stats_fit(var_delta[sl], var2[sl], sums["v_nq"][sl], var_pipe,
                                    self.min_num_qso_in_fit, self.limit_eta, self.limit_var_lss,
                                    start=[eta[index], vlss[index], fudge[index] / FUDGE_REF])
                eta[index], vlss[index], fudge[index] = sol
            w = npix_bin > 0
            self.get_eta = interp1d(self.var_grid[w], eta[w], fill_value="extrapolate",
                                    kind="cubic")
            self.get_var_lss = interp1d(self.var_grid[w], vlss[w], fill_value="extrapolate",
                                        kind="cubic")
            self.get_fudge = interp1d(self.var_grid[w], fudge[w], fill_value="extrapolate",
                                      kind="cubic")
        self.update_stack(sums)

    def update_stack(self, sums):
        """compute_delta_stack's normalisation (expected_flux.py:226-236)."""
        grid = self.grid
        stack = sums["s_num"].copy()
        w = sums["s_w"] > 0
        stack[w] /= sums["s_w"][w]
        self.get_stack_delta = interp1d(grid.log_lambda_grid[w], stack[w], kind="nearest",
                                        fill_value="extrapolate")

    def run(self, raw):
        """All iterations; returns the last (continua, fit parameters). As in
        compute_expected_flux (dr16_expected_flux.py:426-449) the delta stack
        is computed after the variance functions are updated, so its weights
        use the new ones."""
        conts = params = None
        for iteration in range(self.num_iterations):
            conts, params = self.fit_all(raw)
            last = iteration == self.num_iterations - 1
            self.update(self.stacks(raw, conts), last)
            if not last:
                self.update_stack(self.stacks(raw, conts))
        return conts, params

    def deltas(self, raw, conts):
        """populate_los_ids + extract_deltas (dr16_expected_flux.py:706-740,
        expected_flux.py:328-349): per-pixel deltas and weights."""
        delta = np.zeros(raw.pix_offset[-1])
        weights = np.zeros(raw.pix_offset[-1])
        for k in range(raw.num):
            if conts[k] is None:
                continue
            ll, fl, iv, _ = raw.forest(k)
            expected = conts[k] * self.get_stack_delta(ll)
            w = forest_weights(ll, iv, expected, self.get_eta, self.get_var_lss, self.get_fudge,
                               self.var_lss_mod)
            sl = slice(raw.pix_offset[k], raw.pix_offset[k + 1])
            d = np.zeros_like(fl)
            d[w > 0] = fl[w > 0] / expected[w > 0] - 1
            delta[sl] = d
            weights[sl] = w
        return delta, weights
