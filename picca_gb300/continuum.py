"""GPU Dr16 continuum fitting (host driver of the ``pg_cont_*`` C ABI).

Mirrors ``Dr16ExpectedFlux.compute_expected_flux``
(py/picca/delta_extraction/expected_fluxes/dr16_expected_flux.py:380-464):
for ``num_iterations`` iterations, fit every forest's continuum
(``compute_continuum``, expected_fluxes/utils.py:12-136) on the GPU, then,
except after the last iteration, update the mean continuum
(expected_flux.py:256-308) and the variance functions eta, var_lss and
fudge (dr16_expected_flux.py:516-617), and stack the deltas
(expected_flux.py:190-236). The bin sums run on the GPU; the normalisations,
interpolators and the twenty (eta, var_lss, fudge) fits (a box-constrained
linear least-squares problem per wavelength bin, solved exactly) run on the
host. ``deltas()`` returns the final deltas and weights
(populate_los_ids + extract_deltas, dr16_expected_flux.py:706-740,
expected_flux.py:328-349).
"""

import ctypes
import hashlib

import numpy as np
import torch
from scipy.interpolate import PPoly, interp1d, make_interp_spline
from scipy.optimize import lsq_linear

from . import _native
from ._native import check

VAR_PIPE_MIN = np.log10(1e-5)
VAR_PIPE_MAX = np.log10(2.)
NUM_VAR_BINS = 100
FUDGE_REF = 1e-7
ETA_DEFAULT, VAR_LSS_DEFAULT, FUDGE_DEFAULT = 1.0, 0.1, 0.0
FIT_FP64 = 0
FIT_MIXED = 1
STATUS_REASONS = {0: None, 1: "minuit didn't converge", 2: "negative continuum",
                  3: "zero continuum"}

_P = ctypes.POINTER


class SpectraC(ctypes.Structure):
    _fields_ = [("num", ctypes.c_int64), ("num_pixels", ctypes.c_int64)] + [
        (n, ctypes.c_void_p) for n in ("pix_offset", "log_lambda", "flux", "ivar",
                                       "transmission_correction", "z_qso")]


class ContModelC(ctypes.Structure):
    _fields_ = [
        ("num_mean_cont", ctypes.c_int32), ("mean_cont_x", ctypes.c_void_p),
        ("mean_cont_y", ctypes.c_void_p), ("num_var_intervals", ctypes.c_int32),
        ("var_breaks", ctypes.c_void_p), ("eta_coef", ctypes.c_void_p),
        ("var_lss_coef", ctypes.c_void_p), ("fudge_coef", ctypes.c_void_p),
        ("num_stack", ctypes.c_int32), ("stack_x", ctypes.c_void_p), ("stack_y", ctypes.c_void_p),
        ("log_lambda_rest_min", ctypes.c_double), ("log_lambda_rest_max", ctypes.c_double),
        ("var_lss_mod", ctypes.c_double), ("order", ctypes.c_int32),
        ("use_constant_weight", ctypes.c_int32)]


class ContFitC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("zero_point", "slope", "chi2", "ndata", "status",
                                               "iterations", "continuum")]


class ContStacksC(ctypes.Structure):
    _fields_ = [
        ("rest_bins", ctypes.c_int32), ("rest_grid0", ctypes.c_double),
        ("rest_step", ctypes.c_double), ("mean_cont_num", ctypes.c_void_p),
        ("mean_cont_weight", ctypes.c_void_p), ("var_lambda_bins", ctypes.c_int32),
        ("var_grid0", ctypes.c_double), ("var_step", ctypes.c_double),
        ("var_mean", ctypes.c_void_p), ("var_delta2", ctypes.c_void_p),
        ("var_delta4", ctypes.c_void_p), ("var_npix", ctypes.c_void_p),
        ("var_nqso", ctypes.c_void_p), ("obs_bins", ctypes.c_int32),
        ("obs_grid0", ctypes.c_double), ("obs_step", ctypes.c_double),
        ("stack_num", ctypes.c_void_p), ("stack_weight", ctypes.c_void_p),
        ("wave_lin", ctypes.c_int32)]


def _bind():
    lib = _native.lib()
    if getattr(lib, "_cont_bound", False):
        return lib
    lib.pg_cont_fit_batch.argtypes = [ctypes.c_void_p, _P(SpectraC), _P(ContModelC),
                                      ctypes.c_void_p, ctypes.c_int32, ctypes.c_double,
                                      ctypes.c_int32, _P(ContFitC), ctypes.c_void_p]
    lib.pg_cont_fit_select.argtypes = [ctypes.c_void_p, _P(SpectraC), _P(ContModelC),
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                       ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
                                       _P(ContFitC), ctypes.c_void_p]
    lib.pg_cont_stacks_accumulate.argtypes = [ctypes.c_void_p, _P(SpectraC), _P(ContModelC),
                                              _P(ContFitC), _P(ContStacksC), ctypes.c_void_p]
    lib.pg_cont_deltas.argtypes = [ctypes.c_void_p, _P(SpectraC), _P(ContModelC), _P(ContFitC),
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.pg_cont_fit_warm.argtypes = [ctypes.c_void_p, _P(SpectraC), _P(ContModelC),
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                     ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                     _P(ContFitC), ctypes.c_void_p]
    for name in ("pg_cont_fit_batch", "pg_cont_fit_select", "pg_cont_fit_warm",
                 "pg_cont_stacks_accumulate", "pg_cont_deltas"):
        getattr(lib, name).restype = ctypes.c_int
    lib._cont_bound = True
    return lib


def cubic_ppoly(x, y):
    """Breakpoints and (4, m) coefficients of scipy's interp1d(kind='cubic')
    (a not-a-knot cubic B-spline) in piecewise-polynomial form."""
    spl = make_interp_spline(np.asarray(x, float), np.asarray(y, float), k=3)
    pp = PPoly.from_spline(spl)
    keep = np.diff(pp.x) > 0
    breaks = np.concatenate([pp.x[:-1][keep], [pp.x[1:][keep][-1]]])
    return breaks, np.ascontiguousarray(pp.c[:, keep])


def find_bins_log(values, grid):
    """find_bins_log (py/picca/delta_extraction/utils.py:163-186)."""
    step = grid[1] - grid[0]
    return ((values - grid[0]) / step + 0.5).astype(np.int64)


class DeviceSpectra:
    """Raw forests resident on the device."""

    def __init__(self, raw, device):
        arrays = {"pix_offset": np.asarray(raw.pix_offset, np.int64),
                  "log_lambda": raw.log_lambda, "flux": raw.flux, "ivar": raw.ivar,
                  "transmission_correction": raw.transmission_correction,
                  "z_qso": raw.z_qso}
        self.tensors = {k: torch.as_tensor(np.ascontiguousarray(v)).to(device)
                        for k, v in arrays.items()}
        self.num = int(raw.num)
        self.num_pixels = int(raw.pix_offset[-1])
        self.c = SpectraC(self.num, self.num_pixels,
                          *[self.tensors[k].data_ptr() for k in
                            ("pix_offset", "log_lambda", "flux", "ivar",
                             "transmission_correction", "z_qso")])
        self.h2d_bytes = sum(int(t.numel() * t.element_size()) for t in self.tensors.values())


class Dr16Gpu:
    """The Dr16 iteration on the GPU for a set of raw forests."""

    def __init__(self, grid, num_iterations=5, order=1, limit_eta=(0.5, 1.5),
                 limit_var_lss=(0., 0.3), min_num_qso_in_fit=100, num_bins_variance=20,
                 var_lss_mod=1.0, use_constant_weight=False, use_ivar_as_weight=False,
                 force_stack_delta_to_zero=True, fit_mode=FIT_FP64, max_iter=100, tol=1e-10,
                 device=None):
        from .pairs import require_cuda
        require_cuda()
        self.device = torch.device(device or "cuda")
        self.grid = grid
        self.num_iterations = num_iterations
        self.order = order
        self.limit_eta = limit_eta
        self.limit_var_lss = limit_var_lss
        self.min_num_qso_in_fit = min_num_qso_in_fit
        self.num_bins_variance = num_bins_variance
        self.var_lss_mod = var_lss_mod
        self.use_constant_weight = use_constant_weight
        self.use_ivar_as_weight = use_ivar_as_weight
        self.force_stack_delta_to_zero = force_stack_delta_to_zero
        self.fit_mode = fit_mode
        self.max_iter = max_iter
        self.tol = tol
        with torch.cuda.device(self.device):
            self.plan = _native.Plan()
        _bind()
        rest = grid.log_lambda_rest_frame_grid
        # _initialize_variance_wavelength_array (expected_flux.py:122-142)
        if getattr(grid, "wave_solution", "log") == "lin":
            self.log_lambda_var_func_grid = np.log10(np.linspace(
                10**grid.log_lambda_grid[0], 10**grid.log_lambda_grid[-1], num_bins_variance))
        else:
            self.log_lambda_var_func_grid = np.linspace(
                grid.log_lambda_grid[0], grid.log_lambda_grid[-1], num_bins_variance)
        # initial interpolators (dr16_expected_flux.py:198-286, expected_flux.py:95-113)
        self.mean_cont_x = rest.copy()
        self.mean_cont_y = np.ones_like(rest)
        self.mean_cont_weight = np.zeros_like(rest)
        nvb = num_bins_variance
        if use_ivar_as_weight:
            eta, vlss = np.ones(nvb), np.zeros(nvb)
        elif use_constant_weight:
            eta, vlss = np.zeros(nvb), np.ones(nvb)
        else:
            eta, vlss = np.full(nvb, ETA_DEFAULT), np.full(nvb, VAR_LSS_DEFAULT)
        self.fit_functions = not (use_ivar_as_weight or use_constant_weight)
        self.var_x = self.log_lambda_var_func_grid.copy()
        self.eta = eta
        self.var_lss = vlss
        self.fudge = np.full(nvb, FUDGE_DEFAULT)
        self.num_pixels_var = np.zeros(nvb)
        self.valid_fit = np.ones(nvb, bool) if not self.fit_functions else np.zeros(nvb, bool)
        self.stack_x = None
        self.stack_y = None
        self.stack_weight = None
        self.history = []
        self.refined = []  # forests finished in two-float per counted mixed fit
        self._model_cache = {}

    # -- model -------------------------------------------------------------
    def _model_key(self, with_stack):
        parts = [self.mean_cont_x, self.mean_cont_y, self.var_x, self.eta, self.var_lss,
                 self.fudge]
        if with_stack:
            parts += [self.stack_x, self.stack_y]
        h = hashlib.blake2b(digest_size=16)
        for a in parts:
            h.update(b"-" if a is None else np.ascontiguousarray(a, dtype=np.float64).tobytes())
            h.update(b"|")
        return (with_stack, self.var_lss_mod, self.order, bool(self.use_constant_weight),
                h.digest())

    def _model(self, with_stack=False):
        """The device model of the current state, rebuilt only when the state
        (mean continuum, variance functions, stack) changed."""
        key = self._model_key(with_stack)
        cached = self._model_cache.get(with_stack)
        if cached is not None and cached[0] == key:
            return cached[1], cached[2]
        model, keep = self._build_model(with_stack)
        self._model_cache[with_stack] = (key, model, keep)
        return model, keep

    def _build_model(self, with_stack=False):
        dev = self.device
        keep = {}
        keep["mcx"] = torch.as_tensor(self.mean_cont_x, dtype=torch.float64).to(dev)
        keep["mcy"] = torch.as_tensor(self.mean_cont_y, dtype=torch.float64).to(dev)
        coefs = []
        for vals in (self.eta, self.var_lss, self.fudge):
            breaks, coef = cubic_ppoly(self.var_x, vals)
            coefs.append(coef)
        keep["brk"] = torch.as_tensor(breaks).to(dev)
        keep["eta"] = torch.as_tensor(coefs[0]).to(dev)
        keep["vlss"] = torch.as_tensor(coefs[1]).to(dev)
        keep["fudge"] = torch.as_tensor(coefs[2]).to(dev)
        rest = self.grid.log_lambda_rest_frame_grid
        model = ContModelC()
        model.num_mean_cont = len(self.mean_cont_x)
        model.mean_cont_x = keep["mcx"].data_ptr()
        model.mean_cont_y = keep["mcy"].data_ptr()
        model.num_var_intervals = coefs[0].shape[1]
        model.var_breaks = keep["brk"].data_ptr()
        model.eta_coef = keep["eta"].data_ptr()
        model.var_lss_coef = keep["vlss"].data_ptr()
        model.fudge_coef = keep["fudge"].data_ptr()
        if with_stack and self.stack_x is not None:
            keep["sx"] = torch.as_tensor(self.stack_x).to(dev)
            keep["sy"] = torch.as_tensor(self.stack_y).to(dev)
            model.num_stack = len(self.stack_x)
            model.stack_x = keep["sx"].data_ptr()
            model.stack_y = keep["sy"].data_ptr()
        model.log_lambda_rest_min = float(rest[0])
        model.log_lambda_rest_max = float(rest[-1])
        model.var_lss_mod = float(self.var_lss_mod)
        model.order = int(self.order)
        model.use_constant_weight = int(bool(self.use_constant_weight))
        return model, keep

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    # -- steps -------------------------------------------------------------
    def fit(self, spectra, start=None, mode=None, max_iter=None, index=None, out=None,
            count_refined=False):
        """Continuum fit of every forest (or of the forests listed in the
        int32 device tensor ``index``, written into an existing result dict
        ``out``); returns a dict of device tensors."""
        lib = _bind()
        dev = self.device
        n = spectra.num
        if out is None:
            out = self._new_fit(spectra)
        fit_c = ContFitC(*[out[k].data_ptr() for k in ("zero_point", "slope", "chi2", "ndata",
                                                        "status", "iterations", "continuum")])
        model, keep = self._model()
        start_ptr = None
        if start is not None:
            start = torch.as_tensor(start, dtype=torch.float64, device=dev).contiguous()
            start_ptr = start.data_ptr()
        if index is not None:
            index = torch.as_tensor(index, dtype=torch.int32, device=dev).contiguous()
        mode = int(self.fit_mode if mode is None else mode)
        with torch.cuda.device(dev):
            check(lib.pg_cont_fit_select(
                self.plan.handle, ctypes.byref(spectra.c), ctypes.byref(model), start_ptr,
                None if index is None else index.data_ptr(),
                n if index is None else int(index.numel()),
                int(self.max_iter if max_iter is None else max_iter), float(self.tol), mode,
                ctypes.byref(fit_c), self._stream()), "continuum fit")
            if count_refined and mode == FIT_MIXED:
                # forests the mixed fit finished in two-float (synchronises)
                self.refined.append(int(self.plan.stats().work_items))
        out["_keep"] = (keep, start, fit_c, index)
        return out

    def _new_fit(self, spectra):
        n = spectra.num
        dev = self.device
        return {"zero_point": torch.empty(n, dtype=torch.float64, device=dev),
                "slope": torch.empty(n, dtype=torch.float64, device=dev),
                "chi2": torch.empty(n, dtype=torch.float64, device=dev),
                "ndata": torch.empty(n, dtype=torch.int32, device=dev),
                "status": torch.empty(n, dtype=torch.int32, device=dev),
                "iterations": torch.empty(n, dtype=torch.int32, device=dev),
                "continuum": torch.empty(max(spectra.num_pixels, 1), dtype=torch.float64,
                                         device=dev)}

    def fit_warm(self, spectra, start, max_iter=3, chi2_tol=1e-7, ab_tol=1e-5):
        """Certified Newton fits from the warm start ``start`` (FP64 [num, 2],
        device): a forest gets status 0 only when its point is certified
        against its own chi2 (remaining Newton step at most ab_tol of
        max(1, |a|, |b|), chi2 excess over the quadratic model's minimum at
        most chi2_tol of max(|chi2|, ndata)); the others get status 1 and are
        left for the plain fit."""
        lib = _bind()
        out = self._new_fit(spectra)
        fit_c = ContFitC(*[out[k].data_ptr() for k in ("zero_point", "slope", "chi2", "ndata",
                                                        "status", "iterations", "continuum")])
        model, keep = self._model()
        start = torch.as_tensor(start, dtype=torch.float64, device=self.device).contiguous()
        with torch.cuda.device(self.device):
            check(lib.pg_cont_fit_warm(
                self.plan.handle, ctypes.byref(spectra.c), ctypes.byref(model),
                start.data_ptr(), None, spectra.num, int(max_iter), float(chi2_tol),
                float(ab_tol), ctypes.byref(fit_c), self._stream()), "warm continuum fit")
        out["_keep"] = (keep, start, fit_c, None)
        return out

    def _stacks(self, spectra, fit, mean_cont=True, var_stats=True, delta_stack=True):
        lib = _bind()
        dev = self.device
        grid = self.grid
        rest, obs = grid.log_lambda_rest_frame_grid, grid.log_lambda_grid
        nvar = self.num_bins_variance * NUM_VAR_BINS
        bufs = {k: torch.zeros(n, dtype=torch.float64, device=dev) for k, n in (
            ("mc_num", len(rest)), ("mc_w", len(rest)), ("v_mean", nvar), ("v_d2", nvar),
            ("v_d4", nvar), ("v_np", nvar), ("v_nq", nvar), ("s_num", len(obs)),
            ("s_w", len(obs)))}
        st = ContStacksC()
        lin = getattr(grid, "wave_solution", "log") == "lin"
        st.wave_lin = int(lin)

        def origin_step(g):
            # find_bins_lin works on lambda, find_bins_log on log10(lambda)
            if lin:
                return float(10**g[0]), float(10**g[1] - 10**g[0])
            return float(g[0]), float(g[1] - g[0])

        st.rest_bins = len(rest)
        st.rest_grid0, st.rest_step = origin_step(rest)
        if mean_cont:
            st.mean_cont_num = bufs["mc_num"].data_ptr()
            st.mean_cont_weight = bufs["mc_w"].data_ptr()
        st.var_lambda_bins = self.num_bins_variance
        st.var_grid0, st.var_step = origin_step(self.log_lambda_var_func_grid)
        if var_stats:
            st.var_mean = bufs["v_mean"].data_ptr()
            st.var_delta2 = bufs["v_d2"].data_ptr()
            st.var_delta4 = bufs["v_d4"].data_ptr()
            st.var_npix = bufs["v_np"].data_ptr()
            st.var_nqso = bufs["v_nq"].data_ptr()
        st.obs_bins = len(obs)
        st.obs_grid0, st.obs_step = origin_step(obs)
        if delta_stack:
            st.stack_num = bufs["s_num"].data_ptr()
            st.stack_weight = bufs["s_w"].data_ptr()
        model, keep = self._model()
        fit_c = fit["_keep"][2]
        with torch.cuda.device(dev):
            check(lib.pg_cont_stacks_accumulate(self.plan.handle, ctypes.byref(spectra.c),
                                                ctypes.byref(model), ctypes.byref(fit_c),
                                                ctypes.byref(st), self._stream()), "stacks")
        stats = self.plan.stats()
        if stats.status != 0:
            raise _native.NativeError(f"stack accumulation: device status {stats.status}")
        del keep
        return {k: v.cpu().numpy() for k, v in bufs.items()}

    def update_mean_cont(self, sums):
        """_compute_mean_cont normalisation (expected_flux.py:291-308)."""
        mean_cont = sums["mc_num"].copy()
        weight = sums["mc_w"]
        w = weight > 0
        mean_cont[w] /= weight[w]
        mean_cont /= mean_cont[w].mean()
        rest = self.grid.log_lambda_rest_frame_grid[w]
        old = interp1d(self.mean_cont_x, self.mean_cont_y, fill_value="extrapolate")
        self.mean_cont_y = old(rest) * mean_cont[w]
        self.mean_cont_x = rest
        self.mean_cont_weight = weight[w]

    def update_var_functions(self, sums):
        """Variance statistics and the (eta, var_lss, fudge) fits
        (least_squares_var_stats.py:183-198, dr16_expected_flux.py:531-617)."""
        nvb = self.num_bins_variance
        stats = normalise_var_stats(sums)
        var_delta, var2_delta = stats["var_delta"], stats["var2_delta"]
        num_pixels, num_qso = stats["num_pixels"], stats["num_qso"]
        var_pipe_values = 10**(VAR_PIPE_MIN + ((np.arange(NUM_VAR_BINS) + .5) *
                                               (VAR_PIPE_MAX - VAR_PIPE_MIN) / NUM_VAR_BINS))
        eta = interp1d(self.var_x, self.eta, kind="cubic", fill_value="extrapolate")(
            self.log_lambda_var_func_grid)
        vlss = interp1d(self.var_x, self.var_lss, kind="cubic", fill_value="extrapolate")(
            self.log_lambda_var_func_grid)
        fudge = interp1d(self.var_x, self.fudge, kind="cubic", fill_value="extrapolate")(
            self.log_lambda_var_func_grid)
        shape = (nvb, NUM_VAR_BINS)
        npix_bin = num_pixels.reshape(shape).sum(axis=1)
        sols, failed = fit_var_bins(
            var_delta.reshape(shape), var2_delta.reshape(shape), num_qso.reshape(shape),
            var_pipe_values, self.min_num_qso_in_fit, self.limit_eta, self.limit_var_lss,
            np.stack([eta, vlss, fudge / FUDGE_REF], axis=1))
        eta, vlss, fudge = sols[:, 0].copy(), sols[:, 1].copy(), sols[:, 2].copy()
        eta[failed], vlss[failed], fudge[failed] = ETA_DEFAULT, VAR_LSS_DEFAULT, FUDGE_DEFAULT
        valid = ~failed
        w = npix_bin > 0
        self.var_x = self.log_lambda_var_func_grid[w]
        self.eta, self.var_lss, self.fudge = eta[w], vlss[w], fudge[w]
        self.num_pixels_var = npix_bin[w]
        self.valid_fit = valid[w]

    def update_stack(self, sums):
        """compute_delta_stack normalisation and interpolator (expected_flux.py:226-236)."""
        stack = sums["s_num"].copy()
        weight = sums["s_w"]
        w = weight > 0
        stack[w] /= weight[w]
        self.stack_x = self.grid.log_lambda_grid[w]
        self.stack_y = stack[w]
        self.stack_weight = weight[w]

    def update_model(self, spectra, fit, last):
        """The updates of one iteration after the fits, in the reference's
        order (dr16_expected_flux.py:426-449): mean continuum and variance
        statistics from the weights of the current variance functions, then
        (except after the last iteration) the new mean continuum and variance
        functions, then the delta stack with the weights of the NEW variance
        functions (compute_delta_stack runs after compute_var_stats)."""
        refit = (not last) and self.fit_functions
        sums = self._stacks(spectra, fit, mean_cont=not last, var_stats=refit,
                            delta_stack=not refit)
        if not last:
            self.update_mean_cont(sums)
            if self.fit_functions:
                self.update_var_functions(sums)
                sums = self._stacks(spectra, fit, mean_cont=False, var_stats=False,
                                    delta_stack=True)
        self.update_stack(sums)

    def run(self, spectra, start=None, mode=None, on_iteration=None):
        """The Dr16 outer loop. ``start`` optionally warm-starts every
        iteration's fit (e.g. with learned (a, b)); ``on_iteration(iteration,
        fit)`` is called after each iteration's updates (picca saves its
        iteration files there). Returns the last fit."""
        fit = None
        for iteration in range(self.num_iterations):
            fit = self.fit(spectra, start=start, mode=mode)
            self.update_model(spectra, fit, iteration == self.num_iterations - 1)
            self.history.append({"iteration": iteration,
                                 "iterations_mean": float(fit["iterations"].float().mean()),
                                 "accepted": int((fit["status"] == 0).sum())})
            if on_iteration is not None:
                on_iteration(iteration, fit)
        return fit

    def deltas(self, spectra, fit):
        """Final deltas and weights per pixel (device tensors)."""
        lib = _bind()
        dev = self.device
        delta = torch.empty(max(spectra.num_pixels, 1), dtype=torch.float64, device=dev)
        weights = torch.empty_like(delta)
        model, keep = self._model(with_stack=self.force_stack_delta_to_zero)
        fit_c = fit["_keep"][2]
        with torch.cuda.device(dev):
            check(lib.pg_cont_deltas(self.plan.handle, ctypes.byref(spectra.c),
                                     ctypes.byref(model), ctypes.byref(fit_c), delta.data_ptr(),
                                     weights.data_ptr(), self._stream()), "deltas")
        torch.cuda.synchronize(dev)
        del keep
        return delta, weights


def normalise_var_stats(sums):
    """The normalisation of the variance statistics
    (LeastsSquaresVarStats.initialize_delta_arrays,
    least_squares_var_stats.py:176-184) applied to the bin sums."""
    var_delta = sums["v_d2"].copy()
    mean_delta = sums["v_mean"].copy()
    var2_delta = sums["v_d4"].copy()
    num_pixels = sums["v_np"]
    w = num_pixels > 0
    var_delta[w] /= num_pixels[w]
    mean_delta[w] /= num_pixels[w]
    var_delta -= mean_delta**2
    var2_delta[w] /= num_pixels[w]
    var2_delta -= var_delta**2
    var2_delta[w] /= num_pixels[w]
    return {"var_delta": var_delta, "var2_delta": var2_delta, "mean_delta": mean_delta,
            "num_pixels": num_pixels, "num_qso": sums["v_nq"]}


def _faces(limit_eta, limit_var_lss):
    """Every face of the box eta x var_lss x fudge' (fudge' >= 0): for each
    variable None (free) or the bound it is held at."""
    out = []
    for e in (None, limit_eta[0], limit_eta[1]):
        for v in (None, limit_var_lss[0], limit_var_lss[1]):
            for f in (None, 0.0):
                out.append((e, v, f))
    return out


def box_lsq3_gram(gram, mty, limit_eta, limit_var_lss):
    """Exact minimisers of x' G x - 2 x' m (the least squares ||A x - y||^2
    through its Gram matrix G = A'A and m = A'y) over eta in limit_eta,
    var_lss in limit_var_lss, fudge' >= 0, for a batch of problems
    (gram [B, 3, 3], mty [B, 3]). The objective is convex, so its minimum over
    the box is the solution of one face (the free variables solved with the
    others held at their bounds) that lies in the box; every face is solved
    for every problem at once and the best feasible one kept. Returns (x
    [B, 3], ok [B]); ok is False where a face's system is rank deficient (the
    caller then uses an iterative bounded solver)."""
    gram = np.asarray(gram, dtype=np.float64)
    mty = np.asarray(mty, dtype=np.float64)
    nb = gram.shape[0]
    lo = np.array([limit_eta[0], limit_var_lss[0], 0.0])
    hi = np.array([limit_eta[1], limit_var_lss[1], np.inf])
    best = np.zeros((nb, 3))
    best_val = np.full(nb, np.inf)
    ok = np.ones(nb, bool)
    for face in _faces(limit_eta, limit_var_lss):
        x = np.tile(np.array([0.0 if b is None else b for b in face]), (nb, 1))
        free = [k for k in range(3) if face[k] is None]
        feasible = np.ones(nb, bool)
        if free:
            fixed = [k for k in range(3) if face[k] is not None]
            sub = gram[:, free][:, :, free]
            eig = np.linalg.eigvalsh(sub)
            # numpy.linalg.matrix_rank's tolerance on the (symmetric) Gram block
            rank = (eig > eig.max(axis=1, keepdims=True) * len(free) *
                    np.finfo(np.float64).eps).sum(axis=1)
            ok &= rank == len(free)
            r = mty[:, free]
            if fixed:
                r = r - np.einsum("bij,j->bi", gram[:, free][:, :, fixed], x[0, fixed])
            safe = np.where((rank == len(free))[:, None, None], sub, np.eye(len(free)))
            x[:, free] = np.linalg.solve(safe, r[..., None])[..., 0]
            feasible = (np.all(x[:, free] >= lo[free] - 1e-15, axis=1) &
                        np.all(x[:, free] <= hi[free] + 1e-15, axis=1))
        val = np.einsum("bi,bij,bj->b", x, gram, x) - 2 * np.einsum("bi,bi->b", x, mty)
        take = feasible & (val < best_val)
        best[take] = x[take]
        best_val[take] = val[take]
    return best, ok


def box_lsq3(mat, rhs, limit_eta, limit_var_lss):
    """box_lsq3_gram for one problem given as (A, y); None when a face's
    system is rank deficient."""
    x, ok = box_lsq3_gram((mat.T @ mat)[None], (mat.T @ rhs)[None], limit_eta, limit_var_lss)
    return x[0] if ok[0] else None


def fit_var_bins(var_delta, var2_delta, num_qso, var_pipe_values, min_num_qso, limit_eta,
                 limit_var_lss, start):
    """(eta, var_lss, fudge) of every wavelength bin at once (arrays
    [bins, NUM_VAR_BINS]; start [bins, 3] with fudge / FUDGE_REF): the
    batched form of fit_var_bin. Returns [bins, 3] (fudge in its own units)
    and a mask of the bins whose fit failed."""
    sel = (num_qso > min_num_qso) & (var2_delta > 0)
    wsq = np.where(sel, 1.0 / np.where(sel, var2_delta, 1.0), 0.0)  # wgt^2
    cols = np.stack([var_pipe_values, np.ones_like(var_pipe_values),
                     FUDGE_REF / var_pipe_values], axis=1)
    gram = np.einsum("bi,ij,ik->bjk", wsq, cols, cols)
    mty = np.einsum("bi,ij->bj", wsq * np.where(sel, var_delta, 0.0), cols)
    x, ok = box_lsq3_gram(gram, mty, limit_eta, limit_var_lss)
    out = np.array(x)
    failed = np.zeros(len(out), bool)
    for b in range(len(out)):
        if not sel[b].any():
            # flat chi2: the minimiser stays at its starting point
            out[b] = start[b]
        elif not ok[b]:
            sol = fit_var_bin(var_delta[b], var2_delta[b], num_qso[b], var_pipe_values,
                              min_num_qso, limit_eta, limit_var_lss, start[b])
            if sol is None:
                failed[b] = True
            else:
                out[b] = (sol[0], sol[1], sol[2] / FUDGE_REF)
    out[:, 2] *= FUDGE_REF
    return out, failed


def fit_var_bin(var_delta, var2_delta, num_qso, var_pipe_values, min_num_qso, limit_eta,
                limit_var_lss, start):
    """(eta, var_lss, fudge) of one wavelength bin. The chi2 of
    least_squares_var_stats.py:104-132 is linear in (eta, var_lss,
    fudge / FUDGE_REF) with box limits (dr16_expected_flux.py:549-563), so
    its minimum is found exactly by bounded least squares."""
    sel = (num_qso > min_num_qso) & (var2_delta > 0)
    if sel.sum() == 0:
        # flat chi2: the minimiser stays at its starting point
        return float(start[0]), float(start[1]), float(start[2]) * FUDGE_REF
    wgt = 1.0 / np.sqrt(var2_delta[sel])
    mat = np.stack([var_pipe_values[sel], np.ones(sel.sum()),
                    FUDGE_REF / var_pipe_values[sel]], axis=1) * wgt[:, None]
    exact = box_lsq3(mat, var_delta[sel] * wgt, limit_eta, limit_var_lss)
    if exact is not None:
        return float(exact[0]), float(exact[1]), float(exact[2]) * FUDGE_REF
    res = lsq_linear(mat, var_delta[sel] * wgt,
                     bounds=([limit_eta[0], limit_var_lss[0], 0.0],
                             [limit_eta[1], limit_var_lss[1], np.inf]),
                     method="bvls", tol=1e-14)
    if not res.success:
        return None
    return float(res.x[0]), float(res.x[1]), float(res.x[2]) * FUDGE_REF


def fit_results_to_host(fit):
    return {k: v.cpu().numpy() for k, v in fit.items() if not k.startswith("_")}
