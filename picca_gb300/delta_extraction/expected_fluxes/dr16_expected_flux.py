"""GPU drop-in for picca's ``Dr16ExpectedFlux`` expected-flux plugin.

Selected in a picca delta-extraction configuration with::

    [expected flux]
    type = Dr16ExpectedFlux
    module name = picca_gb300.delta_extraction.expected_fluxes.dr16_expected_flux

It keeps the interface of
py/picca/delta_extraction/expected_fluxes/dr16_expected_flux.py:
``__init__(config)`` with the same accepted options and defaults (:20-36 and
py/picca/delta_extraction/expected_flux.py:14-26), ``compute_expected_flux
(forests)`` (:380-464), ``compute_forest_weights(forest, continuum)``
(:466-488), ``populate_los_ids(forests)`` (:706-740), ``extract_deltas
(forest)`` (expected_flux.py:328-349), the ``los_ids`` and
``continuum_fit_parameters`` dictionaries, the ``get_*`` interpolators and
``save_iteration_step`` with its STACK_DELTAS, VAR_FUNC, CONT and
FIT_METADATA HDUs (expected_flux.py:351-430, dr16_expected_flux.py:618-704).
The whole iteration runs on the GPU through :class:`picca_gb300.continuum.
Dr16Gpu`; ``num processors`` is accepted and ignored.

Forests are any objects with picca's ``Forest`` attributes ``los_id``,
``z`` (quasar redshift), ``log_lambda``, ``flux``, ``ivar`` and
``transmission_correction``; the method sets ``forest.continuum`` and
``forest.bad_continuum_reason`` as the reference does. The wavelength grids
(picca's ``Forest`` class variables) come from the ``grid`` argument or, when
picca itself is importable, from ``Forest``. Differences from the
reference: the continuum minimiser is a damped Newton method on the same
chi2 (the reference uses iminuit's MIGRAD), the variance functions are
fitted by exact bounded linear least squares (the same chi2), only a
one-dimensional mean continuum is supported, and Pk1d forests' ``ivar``
entry is not produced. Both wavelength solutions are supported: on the
linear grid the bins follow find_bins_lin and the variance functions' grid
is linear in lambda (expected_flux.py:122-142); forests longer than 224
pixels are fitted with FP64 per-pixel terms held in shared memory.
"""

import logging
import os

import numpy as np
from scipy.interpolate import interp1d

from ... import continuum as gpu_continuum
from ... import fitsio_lite

try:  # subclass picca's base class when picca is importable
    from picca.delta_extraction.expected_flux import ExpectedFlux as _Base  # noqa: F401
except Exception:  # noqa: BLE001 - picca or one of its dependencies is missing
    _Base = object

# py/picca/delta_extraction/expected_flux.py:14-26 and
# py/picca/delta_extraction/expected_fluxes/dr16_expected_flux.py:20-36
accepted_options = sorted([
    "iter out prefix", "num bins variance", "num processors", "out dir", "var lss mod",
    "force stack delta to zero", "limit eta", "limit var lss", "min num qso in fit",
    "num iterations", "order", "use constant weight", "use ivar as weight",
])
defaults = {
    "iter out prefix": "delta_attributes",
    "num bins variance": 20,
    "num processors": 0,
    "var lss mod": 1.0,
    "force stack delta to zero": True,
    "limit eta": (0.5, 1.5),
    "limit var lss": (0., 0.3),
    "num iterations": 5,
    "min num qso in fit": 100,
    "order": 1,
    "use constant weight": False,
    "use ivar as weight": False,
}


class ExpectedFluxError(Exception):
    """Invalid configuration or input (picca's ExpectedFluxError)."""


class _Grid:
    def __init__(self, log_lambda_grid, log_lambda_rest_frame_grid, wave_solution="log"):
        self.log_lambda_grid = np.asarray(log_lambda_grid, dtype=np.float64)
        self.log_lambda_rest_frame_grid = np.asarray(log_lambda_rest_frame_grid,
                                                     dtype=np.float64)
        self.wave_solution = wave_solution


def _forest_class_grid():
    try:
        from picca.delta_extraction.astronomical_objects.forest import Forest
    except Exception as error:  # noqa: BLE001
        raise ExpectedFluxError(
            "no wavelength grid: pass grid= or make picca's Forest class importable") from error
    return _Grid(Forest.log_lambda_grid, Forest.log_lambda_rest_frame_grid,
                 Forest.wave_solution)


def _option(config, name, kind):
    """Read an option like configparser's get/getint/getfloat/getboolean,
    falling back to the defaults above."""
    value = config.get(name) if hasattr(config, "get") else None
    if value is None:
        return defaults.get(name)
    if isinstance(value, str):
        text = value.strip()
        if kind is int:
            return int(text)
        if kind is float:
            return float(text)
        if kind is bool:
            if text.lower() in ("1", "yes", "true", "on"):
                return True
            if text.lower() in ("0", "no", "false", "off"):
                return False
            raise ExpectedFluxError(f"option '{name}': not a boolean: {value}")
        if kind is tuple:
            parts = text.strip("()[] ").split(",")
            return tuple(float(v) for v in parts)
        return text
    return value


class Dr16ExpectedFlux(_Base):
    """Dr16 expected flux (du Mas des Bourboux et al. 2020) on the GPU."""

    def __init__(self, config, grid=None, fit_mode=gpu_continuum.FIT_FP64, device=None):
        self.logger = logging.getLogger(__name__)
        for key in (config.keys() if hasattr(config, "keys") else []):
            if key not in accepted_options:
                raise ExpectedFluxError(f"unrecognised option in [expected flux]: {key}")
        self.iter_out_prefix = _option(config, "iter out prefix", str)
        if self.iter_out_prefix is None or "/" in self.iter_out_prefix:
            raise ExpectedFluxError("'iter out prefix' must be a file prefix without folders")
        self.num_bins_variance = _option(config, "num bins variance", int)
        self.num_processors = _option(config, "num processors", int)
        out_dir = _option(config, "out dir", str)
        self.out_dir = None if out_dir is None else out_dir + "Log/"
        self.var_lss_mod = _option(config, "var lss mod", float)
        self.force_stack_delta_to_zero = _option(config, "force stack delta to zero", bool)
        self.limit_eta = tuple(_option(config, "limit eta", tuple))
        self.limit_var_lss = tuple(_option(config, "limit var lss", tuple))
        self.min_num_qso_in_fit = _option(config, "min num qso in fit", int)
        self.num_iterations = _option(config, "num iterations", int)
        self.order = _option(config, "order", int)
        self.use_constant_weight = _option(config, "use constant weight", bool)
        self.use_ivar_as_weight = _option(config, "use ivar as weight", bool)
        if self.order not in (0, 1):
            raise ExpectedFluxError("'order' must be 0 or 1")
        if self.use_constant_weight and self.use_ivar_as_weight:
            raise ExpectedFluxError("'use constant weight' and 'use ivar as weight' "
                                    "are mutually exclusive")
        self.grid = grid if grid is not None else _forest_class_grid()
        if getattr(self.grid, "wave_solution", "log") not in ("log", "lin"):
            raise ExpectedFluxError("Forest.wave_solution must be 'lin' or 'log'")
        self.gpu = gpu_continuum.Dr16Gpu(
            self.grid, num_iterations=self.num_iterations, order=self.order,
            limit_eta=self.limit_eta, limit_var_lss=self.limit_var_lss,
            min_num_qso_in_fit=self.min_num_qso_in_fit,
            num_bins_variance=self.num_bins_variance, var_lss_mod=self.var_lss_mod,
            use_constant_weight=self.use_constant_weight,
            use_ivar_as_weight=self.use_ivar_as_weight,
            force_stack_delta_to_zero=self.force_stack_delta_to_zero, fit_mode=fit_mode,
            device=device)
        self.log_lambda_var_func_grid = self.gpu.log_lambda_var_func_grid
        self.los_ids = {}
        self.continuum_fit_parameters = None
        self._refresh_interpolators()

    # -- interpolators (expected_flux.py:95-113, dr16_expected_flux.py:198-286)
    def _refresh_interpolators(self):
        g = self.gpu
        self.get_mean_cont = interp1d(g.mean_cont_x, g.mean_cont_y, fill_value="extrapolate")
        self.get_mean_cont_weight = interp1d(g.mean_cont_x, g.mean_cont_weight,
                                             fill_value="extrapolate")
        self.get_eta = interp1d(g.var_x, g.eta, kind="cubic", fill_value="extrapolate")
        self.get_var_lss = interp1d(g.var_x, g.var_lss, kind="cubic", fill_value="extrapolate")
        self.get_fudge = interp1d(g.var_x, g.fudge, kind="cubic", fill_value="extrapolate")
        npix = g.num_pixels_var if len(g.num_pixels_var) == len(g.var_x) else np.zeros(
            len(g.var_x))
        self.get_num_pixels = interp1d(g.var_x, npix, kind="nearest", fill_value="extrapolate")
        self.get_valid_fit = interp1d(g.var_x, np.asarray(g.valid_fit, dtype=float),
                                      kind="nearest", fill_value="extrapolate")
        if g.stack_x is not None:
            self.get_stack_delta = interp1d(g.stack_x, g.stack_y, kind="nearest",
                                            fill_value="extrapolate")
            self.get_stack_delta_weights = interp1d(g.stack_x, g.stack_weight, kind="nearest",
                                                    fill_value=0.0, bounds_error=False)
        else:
            self.get_stack_delta = None
            self.get_stack_delta_weights = None

    # -- the iteration (dr16_expected_flux.py:380-464) ----------------------
    def compute_expected_flux(self, forests):
        forests = list(forests)
        raw = _pack(forests)
        spectra = gpu_continuum.DeviceSpectra(raw, self.gpu.device)

        def on_iteration(iteration, fit):
            self._refresh_interpolators()
            self._set_fit_parameters(forests, fit)
            if self.out_dir is not None and os.path.isdir(self.out_dir):
                last = iteration == self.num_iterations - 1
                self.save_iteration_step(-1 if last else iteration)

        fit = self.gpu.run(spectra, on_iteration=on_iteration)
        host = gpu_continuum.fit_results_to_host(fit)
        for k, forest in enumerate(forests):
            reason = gpu_continuum.STATUS_REASONS[int(host["status"][k])]
            forest.bad_continuum_reason = reason
            sl = slice(raw.pix_offset[k], raw.pix_offset[k + 1])
            forest.continuum = None if reason is not None else host["continuum"][sl].copy()
        delta, weights = self.gpu.deltas(spectra, fit)
        self._populate(forests, raw, host, weights.cpu().numpy())

    def _set_fit_parameters(self, forests, fit):
        host = {k: fit[k].cpu().numpy() for k in ("zero_point", "slope", "chi2", "ndata",
                                                   "status")}
        params = {}
        for k, forest in enumerate(forests):
            if host["status"][k] == 0:
                params[forest.los_id] = (host["zero_point"][k], host["slope"][k],
                                         host["chi2"][k], int(host["ndata"][k]))
            else:
                params[forest.los_id] = (np.nan, np.nan, np.nan, int(host["ndata"][k]))
        self.continuum_fit_parameters = params

    def _populate(self, forests, raw, host, weights):
        """populate_los_ids (dr16_expected_flux.py:706-740) from the device
        weights: mean expected flux = continuum * stack(lambda)."""
        self.los_ids = {}
        expected = np.array(host["continuum"][:len(raw.log_lambda)], dtype=np.float64)
        if self.force_stack_delta_to_zero and len(expected):
            expected = expected * self.get_stack_delta(raw.log_lambda)
        for k, forest in enumerate(forests):
            if forest.bad_continuum_reason is not None:
                continue
            sl = slice(raw.pix_offset[k], raw.pix_offset[k + 1])
            self.los_ids[forest.los_id] = {"mean expected flux": expected[sl].copy(),
                                           "weights": weights[sl].copy(),
                                           "continuum": forest.continuum}

    def populate_los_ids(self, forests):
        """Host version of populate_los_ids for forests whose continuum is set."""
        self.los_ids = {}
        for forest in forests:
            if forest.bad_continuum_reason is not None:
                continue
            mean_expected_flux = np.copy(forest.continuum)
            if self.force_stack_delta_to_zero:
                mean_expected_flux *= self.get_stack_delta(forest.log_lambda)
            self.los_ids[forest.los_id] = {
                "mean expected flux": mean_expected_flux,
                "weights": self.compute_forest_weights(forest, mean_expected_flux),
                "continuum": forest.continuum}

    def compute_forest_weights(self, forest, continuum):
        """dr16_expected_flux.py:466-488."""
        w = forest.ivar > 0
        weights = np.empty_like(forest.log_lambda)
        weights[~w] = 0.0
        var_pipe = 1. / forest.ivar[w] / continuum[w]**2
        var_lss = self.get_var_lss(forest.log_lambda[w])
        eta = self.get_eta(forest.log_lambda[w])
        fudge = self.get_fudge(forest.log_lambda[w])
        weights[w] = 1.0 / (eta * var_pipe + self.var_lss_mod * var_lss + fudge / var_pipe)
        return weights

    def extract_deltas(self, forest):
        """expected_flux.py:328-349."""
        info = self.los_ids.get(forest.los_id)
        if info is None:
            return
        w = info["weights"] > 0
        expected_flux = info["mean expected flux"]
        forest.deltas = np.zeros_like(forest.flux)
        forest.deltas[w] = forest.flux[w] / expected_flux[w] - 1
        forest.weights = info["weights"]
        forest.continuum = info["continuum"]

    # -- iteration files (expected_flux.py:351-430, dr16_expected_flux.py:618-704)
    def save_iteration_step(self, iteration):
        if iteration == -1:
            name = self.iter_out_prefix + ".fits.gz"
        else:
            name = self.iter_out_prefix + f"_iteration{iteration + 1}.fits.gz"
        grid = self.grid
        tables = []
        if self.get_stack_delta is not None:
            tables.append({
                "columns": [grid.log_lambda_grid, self.get_stack_delta(grid.log_lambda_grid),
                            self.get_stack_delta_weights(grid.log_lambda_grid)],
                "names": ["LOGLAM", "STACK", "WEIGHT"], "units": ["log(Angstrom)", "", ""],
                "extname": "STACK_DELTAS"})
        vg = self.log_lambda_var_func_grid
        tables.append({
            "columns": [vg, self.get_eta(vg), self.get_var_lss(vg), self.get_fudge(vg),
                        self.get_num_pixels(vg).astype(np.int32),
                        self.get_valid_fit(vg).astype(bool)],
            "names": ["LOGLAM", "ETA", "VAR_LSS", "FUDGE", "NUM_PIXELS", "VALID_FIT"],
            "units": ["log(Angstrom)", "", "", "", "", ""], "extname": "VAR_FUNC"})
        rest = grid.log_lambda_rest_frame_grid
        tables.append({
            "columns": [rest, self.get_mean_cont(rest), self.get_mean_cont_weight(rest)],
            "names": ["LOGLAM_REST", "MEAN_CONT", "WEIGHT"],
            "units": ["log(Angstrom)", "", ""], "extname": "CONT"})
        if self.continuum_fit_parameters is not None:
            los = sorted(self.continuum_fit_parameters)
            vals = [self.continuum_fit_parameters[key] for key in los]
            tables.append({
                "columns": [np.array(los), np.array([v[0] for v in vals]),
                            np.array([v[1] for v in vals]), np.array([v[2] for v in vals]),
                            np.array([v[3] for v in vals], dtype=np.int64),
                            np.array([not np.any(np.isnan(v)) for v in vals])],
                "names": ["LOS_ID", "ZERO_POINT", "SLOPE", "CHI2", "NUM_DATAPOINTS",
                          "ACCEPTED_FIT"],
                "header": [{"name": "FITORDER", "value": self.order,
                            "comment": "order of the polynomial used for continuum fitting"}],
                "extname": "FIT_METADATA"})
        fitsio_lite.write_fits(os.path.join(self.out_dir, name), tables)


def _pack(forests):
    """Concatenate picca-style forests into the flat arrays of the GPU fit."""
    from ...synthetic_spectra import RawForests
    npix = np.array([len(f.log_lambda) for f in forests], dtype=np.int64)
    offsets = np.zeros(len(forests) + 1, dtype=np.int64)
    np.cumsum(npix, out=offsets[1:])

    def cat(attr):
        if not forests:
            return np.zeros(0)
        return np.concatenate([np.asarray(getattr(f, attr), dtype=np.float64) for f in forests])

    return RawForests(log_lambda=cat("log_lambda"), flux=cat("flux"), ivar=cat("ivar"),
                      transmission_correction=cat("transmission_correction"),
                      z_qso=np.array([f.z for f in forests], dtype=np.float64),
                      los_id=np.array([f.los_id for f in forests]), pix_offset=offsets)


def compute_continuum(forest, get_mean_cont, get_eta, get_var_lss, get_fudge,
                      use_constant_weight, order, grid=None):
    """One forest's continuum fit on the GPU, with the signature and results
    of py/picca/delta_extraction/expected_fluxes/utils.py:12-136:
    (continuum or None, bad-continuum reason or None, (a, b, chi2, ndata))."""
    if grid is None:
        grid = _forest_class_grid()
    gpu = gpu_continuum.Dr16Gpu(grid, num_iterations=1, order=order,
                                use_constant_weight=use_constant_weight)
    gpu.mean_cont_x = np.asarray(get_mean_cont.x, dtype=np.float64)
    gpu.mean_cont_y = np.asarray(get_mean_cont.y, dtype=np.float64)
    gpu.var_x = np.asarray(get_eta.x, dtype=np.float64)
    gpu.eta = np.asarray(get_eta.y, dtype=np.float64)
    gpu.var_lss = np.asarray(get_var_lss(gpu.var_x), dtype=np.float64)
    gpu.fudge = np.asarray(get_fudge(gpu.var_x), dtype=np.float64)
    raw = _pack([forest])
    res = gpu_continuum.fit_results_to_host(
        gpu.fit(gpu_continuum.DeviceSpectra(raw, gpu.device)))
    reason = gpu_continuum.STATUS_REASONS[int(res["status"][0])]
    ndata = int(res["ndata"][0])
    if reason is not None:
        return None, reason, (np.nan, np.nan, np.nan, ndata)
    return (res["continuum"][:len(forest.log_lambda)].copy(), None,
            (res["zero_point"][0], res["slope"][0], res["chi2"][0], ndata))
