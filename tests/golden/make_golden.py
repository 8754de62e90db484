"""Generate the golden fixtures used by the parity tests.

Run once in a checkout that has the picca sources next to it
(``python tests/golden/make_golden.py /path/to/picca``). It writes:

* ``delta_lya.npz`` / ``delta_lya_image.npz`` / ``cat.npz``: the inputs of
  picca's correlation tests (``py/picca/tests/data/test_delta``) converted to
  compact numpy arrays, so tests can rebuild the FITS files anywhere;
* ``cor_<case>.npz``: every column and the ATTRI header of picca's golden
  correlation outputs (``py/picca/tests/data/test_cor/*.fits.gz``), produced by
  the commands at ``py/picca/tests/test_3_cor.py:229-316, :458-488,
  :636-664, :791-1002``;
* ``cor_dmat.npz``: picca's golden distortion matrix (``test_cor/dmat.fits.gz``,
  command at ``py/picca/tests/test_3_cor.py:318-347``);
* ``dmat_cases.npz``: inputs and outputs of picca's own
  ``cf.compute_dmat_forest_pairs_fast`` on forest pairs of the test data;
* ``cor_dmat_zcuts.npz``, ``cor_dmat_cross.npz``, ``cor_dmat_cross_zcuts.npz``,
  ``cor_xdmat.npz``, ``cor_xdmat_zcuts.npz``: picca's other golden distortion
  matrices (``test_cor/*.fits.gz``, commands in py/picca/tests/test_3_cor.py);
* ``cor_metal_dmat.npz``, ``cor_metal_dmat_cross.npz``,
  ``cor_metal_xdmat.npz``: picca's golden metal distortion matrices
  (``test_cor/metal_dmat.fits.gz``, ``metal_dmat_cross.fits.gz``,
  ``metal_xdmat.fits.gz``);
* ``cor_fast_metal_dmat.npz``, ``cor_fast_metal_dmat_cross.npz``,
  ``cor_fast_metal_xdmat.npz``: picca's golden fast metal distortion
  matrices, and ``stack_lya_nodla.npz`` their input (the STACK_DELTAS table
  of ``test_cor/input_from_delta_extraction_lya_nodla/Log/
  delta_attributes.fits.gz``);
* ``cor_wick.npz``, ``cor_xwick.npz`` and ``cf1d.npz``: picca's golden Wick
  covariances (``test_cor/wick.fits.gz``, ``xwick.fits.gz``) and their
  1D-correlation input
  (``test_cor/cf1d.fits.gz``);
* ``xdmat_cases.npz``: inputs and outputs of picca's own
  ``xcf.compute_dmat_forest_pairs_fast`` on forests of the test data and the
  quasars around them;
* ``pair_cases.npz``: inputs and outputs of picca's own
  ``cf.compute_xi_forest_pairs_fast`` and ``xcf.compute_xi_forest_pairs_fast``
  run here as plain Python (numba, healpy, fitsio, camb and iminuit replaced by
  import stand-ins, the functions themselves unmodified) on forest pairs from
  the test data, for every option branch of the kernels.
"""

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from picca_gb300 import fitsio_lite  # noqa: E402
from picca_gb300 import constants as gb_constants  # noqa: E402
from picca_gb300 import io as gb_io  # noqa: E402
from picca_gb300.healpix import ang2pix_ring  # noqa: E402


def _convert_delta_dir(src_dir, out_path):
    files = sorted(f for f in os.listdir(src_dir) if f.endswith(".fits.gz"))
    rec = {k: [] for k in ("file_index", "los_id", "ra", "dec", "z", "plate", "mjd",
                           "fiberid", "npix")}
    pix = {k: [] for k in ("LOGLAM", "DELTA", "WEIGHT", "CONT")}
    for index, name in enumerate(files):
        hdul = fitsio_lite.FITS(os.path.join(src_dir, name))
        for hdu in hdul[1:]:
            header = hdu.read_header()
            rec["file_index"].append(index)
            rec["los_id"].append(header["THING_ID"])
            rec["ra"].append(header["RA"])
            rec["dec"].append(header["DEC"])
            rec["z"].append(header["Z"])
            rec["plate"].append(header["PLATE"])
            rec["mjd"].append(header["MJD"])
            rec["fiberid"].append(header["FIBERID"])
            rec["npix"].append(hdu.get_nrows())
            for key in pix:
                pix[key].append(hdu[key][:])
    out = {k: np.asarray(v) for k, v in rec.items()}
    out.update({k: np.concatenate(v) for k, v in pix.items()})
    out["file_names"] = np.asarray(files)
    np.savez_compressed(out_path, **out)


def _convert_image_dir(src_dir, out_path):
    files = sorted(f for f in os.listdir(src_dir) if f.endswith(".fits.gz"))
    out = {"file_names": np.asarray(files)}
    for index, name in enumerate(files):
        hdul = fitsio_lite.FITS(os.path.join(src_dir, name))
        meta = hdul["METADATA"]
        out[f"f{index}_LAMBDA"] = hdul["LAMBDA"][:]
        lam_header = hdul["LAMBDA"].read_header()
        for key in ("WAVE_SOLUTION", "DELTA_LAMBDA", "DELTA_LOG_LAMBDA"):
            if key in lam_header:
                out[f"f{index}_HDR_{key}"] = np.asarray(lam_header[key])
        for key in ("DELTA", "WEIGHT", "CONT"):
            out[f"f{index}_{key}"] = np.asarray(hdul[key].read(), dtype=float)
        for col in meta.get_colnames():
            out[f"f{index}_META_{col}"] = meta[col][:]
        out[f"f{index}_BLINDING"] = np.asarray(meta.read_header().get("BLINDING", "none"))
    np.savez_compressed(out_path, **out)


def _convert_cat(src, out_path):
    table = fitsio_lite.FITS(src)[1]
    np.savez_compressed(out_path, **{c: table[c][:] for c in table.get_colnames()})


def _convert_cor(src, out_path):
    hdul = fitsio_lite.FITS(src)
    attri = hdul["ATTRI"]
    cor = hdul["COR"]
    out = {c: attri[c][:] for c in attri.get_colnames()}
    out.update({c: cor[c][:] for c in cor.get_colnames()})
    header = attri.read_header()
    for key in ("RPMIN", "RPMAX", "RTMAX", "NP", "NT", "NSIDE"):
        out["hdr_" + key] = np.asarray(header[key])
    np.savez_compressed(out_path, **out)


class _LimitDict(dict):
    def __missing__(self, key):
        return None


class _MinuitStandIn:
    """Stand-in for iminuit.Minuit in the fixture runs (iminuit is not
    installed; no iminuit code is involved): ``migrad`` minimises the
    reference's own cost function with SciPy, the parameters scaled by the
    step sizes iminuit is given (``errors``), limits as bounds, fixed
    parameters held. The continuum fit (zero point, slope) uses local
    searches from the start only (L-BFGS-B and a small Nelder-Mead simplex,
    each polished from the better result): picca's continuum chi2 is
    unbounded below where a pixel's noise model crosses zero (picca drops
    log w for w <= 0), away from the start. The variance fit (eta, var_lss,
    fudge) is a convex quadratic whose fudge column is scaled very
    differently from the others; Powell's method is added there. ``valid``
    reports SciPy's success and a cost of normal size: a chi2 of order 1e8
    or more means the search ended on that singular region, where MIGRAD's
    outcome is undefined, and the fit is reported as not converged;
    ``fval`` is the cost at the result."""

    def __init__(self, fcn, *args, name=None, **start):
        import inspect
        self.fcn = fcn
        if name is None:
            name = [p for p in inspect.signature(fcn).parameters]
        self.names = list(name)
        self.values = {n: float(start[n]) for n in self.names}
        self.errors = {}
        self.limits = _LimitDict()
        self.fixed = {}
        self.errordef = 1.0
        self.print_level = 0
        self.valid = False
        self.fval = None

    def _cost(self, free, x):
        vals = dict(self.values)
        vals.update(zip(free, x))
        return float(self.fcn(*[vals[n] for n in self.names]))

    def migrad(self):
        from scipy.optimize import minimize
        free = [n for n in self.names if not self.fixed.get(n, False)]
        x0 = np.array([self.values[n] for n in free])
        bounds = []
        for n in free:
            lim = self.limits[n]
            lo, hi = (None, None) if lim is None else lim
            bounds.append((-np.inf if lo is None else lo, np.inf if hi is None else hi))
        x0 = np.clip(x0, [b[0] for b in bounds], [b[1] for b in bounds])
        step = np.array([abs(self.errors.get(n, 0.0)) or max(abs(v), 1.0)
                         for n, v in zip(free, x0)])
        sb = [(lo / sc if np.isfinite(lo) else -np.inf, hi / sc if np.isfinite(hi) else np.inf)
              for (lo, hi), sc in zip(bounds, step)]
        cost = lambda y: self._cost(free, y * step)  # noqa: E731
        y0 = x0 / step
        local = "fudge" not in self.names
        methods = [("L-BFGS-B", {"ftol": 1e-15, "gtol": 1e-12, "maxiter": 5000}),
                   ("Nelder-Mead", {"xatol": 1e-13, "fatol": 1e-13, "maxiter": 20000,
                                    "maxfev": 40000})]
        if not local:
            methods.append(("Powell", {"xtol": 1e-13, "ftol": 1e-15, "maxiter": 20000}))

        def run(method, opts, y):
            if method == "Nelder-Mead":
                opts = dict(opts, initial_simplex=np.vstack([y, y + 0.05 * np.eye(len(y))]))
            return minimize(cost, y, method=method, bounds=sb, options=opts)

        def value(r):
            return r.fun if np.isfinite(r.fun) else np.inf

        with np.errstate(all="ignore"):
            results = [run(m, o, y0) for m, o in methods]
            best = min(results, key=value)
            for _ in range(3):  # polish from the best point
                for method, opts in methods:
                    if method == "Nelder-Mead":
                        opts = dict(opts, initial_simplex=np.vstack(
                            [best.x, best.x + 1e-3 * np.eye(len(best.x))]))
                        res = minimize(cost, best.x, method=method, bounds=sb, options=opts)
                    else:
                        res = run(method, opts, best.x)
                    if value(res) < value(best):
                        best = res
        for n, v in zip(free, best.x * step):
            self.values[n] = float(v)
        self.fval = self._cost(free, best.x * step)
        self.valid = bool(np.isfinite(self.fval) and abs(self.fval) < 1e8 and
                          any(r.success for r in results))

    def hesse(self):
        return None


def _install_stand_ins():
    """Stand-ins for the reference's third-party imports (no code of those
    projects is involved; the pair functions need none of them)."""
    numba = types.ModuleType("numba")

    def njit(*args, **kwargs):
        if args and callable(args[0]):
            return args[0]
        return lambda func: func

    numba.njit = njit
    numba.jit = njit
    numba.int32 = np.int32
    numba.prange = range
    numba_types = types.ModuleType("numba.types")
    numba_types.bool_ = np.bool_
    numba.types = numba_types
    healpy = types.ModuleType("healpy")
    healpy.query_disc = lambda nside, vec, radius, inclusive=True: np.arange(12 * nside * nside)
    healpy.ang2pix = lambda nside, theta, phi: ang2pix_ring(nside, theta, phi)
    fitsio = types.ModuleType("fitsio")
    fitsio.FITS = fitsio_lite.FITS
    camb = types.ModuleType("camb")
    iminuit = types.ModuleType("iminuit")
    iminuit.util = types.SimpleNamespace(IMinuitWarning=Warning)
    iminuit.Minuit = _MinuitStandIn
    for name, mod in (("numba", numba), ("numba.types", numba_types), ("healpy", healpy),
                      ("fitsio", fitsio), ("camb", camb), ("iminuit", iminuit)):
        sys.modules[name] = mod


def _pair_cases(reference_py, delta_dir, attributes):
    sys.dont_write_bytecode = True
    _install_stand_ins()
    sys.path.insert(0, reference_py)
    import picca.cf as ref_cf  # pylint: disable=import-outside-toplevel
    import picca.xcf as ref_xcf  # pylint: disable=import-outside-toplevel

    cosmo = gb_constants.Cosmo(Om=0.315, verbose=False)
    data, _, _, _ = gb_io.read_deltas(delta_dir, 16, 1215.67, 2.9, 2.25, cosmo,
                                      delta_attributes=attributes)
    deltas = [d for hp in sorted(data) for d in data[hp]]
    rng = np.random.default_rng(20261203)
    # pick close pairs so that many pixel pairs land inside the grid
    pairs = []
    for _ in range(4000):
        a, b = rng.integers(0, len(deltas), 2)
        if a == b:
            continue
        ang = deltas[a].get_angle_between(deltas[b])
        if ang < 0.01 and abs(deltas[a].z_qso - deltas[b].z_qso) < 0.4:
            pairs.append((a, b, ang))
        if len(pairs) >= 6:
            break
    # one same-plate pair for the half-plate veto
    for a in range(len(deltas)):
        for b in range(a + 1, len(deltas)):
            if deltas[a].plate == deltas[b].plate and (
                    (deltas[a].fiberid <= 500) == (deltas[b].fiberid <= 500)) and (
                        abs(deltas[a].z_qso - deltas[b].z_qso) < 0.5):
                ang = deltas[a].get_angle_between(deltas[b])
                if ang < 0.016:
                    pairs.append((a, b, ang))
                    break
        if len(pairs) >= 7:
            break

    cf_variants = [
        dict(name="auto", r_par_min=0., r_par_max=60., r_trans_max=60., np=15, nt=15,
             x_correlation=False, remove_shp=True),
        dict(name="auto_zcut", r_par_min=0., r_par_max=60., r_trans_max=60., np=15, nt=15,
             z_min_pairs=2.25, z_max_pairs=2.3, remove_shp=True),
        dict(name="cross", r_par_min=-60., r_par_max=60., r_trans_max=60., np=30, nt=15,
             x_correlation=True, remove_shp=True),
        dict(name="zerr", r_par_min=0., r_par_max=200., r_trans_max=200., np=50, nt=50,
             zerr_cut_deg=2.0, zerr_cut_kms=30000.),
        dict(name="rmu", r_par_min=0., r_par_max=1., r_trans_max=60., np=10, nt=15,
             rmu_binning=True),
        dict(name="angl", r_par_min=1., r_par_max=1.02, r_trans_max=0.01, np=10, nt=10,
             ang_correlation=True),
        dict(name="auto_fine", r_par_min=0., r_par_max=200., r_trans_max=200., np=50, nt=50),
    ]
    out = {}
    case_index = 0
    for variant in cf_variants:
        for (a, b, _) in pairs:
            d1, d2 = deltas[a], deltas[b]
            ref_cf.r_par_min = variant["r_par_min"]
            ref_cf.r_par_max = variant["r_par_max"]
            ref_cf.r_trans_max = variant["r_trans_max"]
            ref_cf.num_bins_r_par = variant["np"]
            ref_cf.num_bins_r_trans = variant["nt"]
            ref_cf.z_min_pairs = variant.get("z_min_pairs")
            ref_cf.z_max_pairs = variant.get("z_max_pairs")
            ref_cf.zerr_cut_deg = variant.get("zerr_cut_deg")
            ref_cf.zerr_cut_kms = variant.get("zerr_cut_kms")
            ref_cf.x_correlation = variant.get("x_correlation", False)
            ref_cf.rmu_binning = variant.get("rmu_binning", False)
            ref_cf.ang_correlation = variant.get("ang_correlation", False)
            ref_cf.remove_same_half_plate_close_pairs = variant.get("remove_shp", False)
            nbins = variant["np"] * variant["nt"]
            arrays = [np.zeros(nbins) for _ in range(5)] + [np.zeros(nbins, dtype=np.int64)]
            ang = d1.get_angle_between(d2)
            same_half_plate = (d1.plate == d2.plate) and (
                (d1.fiberid <= 500 and d2.fiberid <= 500) or
                (d1.fiberid > 500 and d2.fiberid > 500))
            if ref_cf.ang_correlation:
                r1, m1 = 10.0**d1.log_lambda, 10.0**d1.log_lambda
                r2, m2 = 10.0**d2.log_lambda, 10.0**d2.log_lambda
            else:
                r1, m1, r2, m2 = d1.r_comov, d1.dist_m, d2.r_comov, d2.dist_m
            ref_cf.compute_xi_forest_pairs_fast(
                d1.z, r1, m1, d1.weights, d1.delta, d1.z_qso,
                d2.z, r2, m2, d2.weights, d2.delta, d2.z_qso,
                ang, same_half_plate, *arrays)
            prefix = f"cf{case_index}_"
            out[prefix + "params"] = np.array([
                variant["r_par_min"], variant["r_par_max"], variant["r_trans_max"],
                variant["np"], variant["nt"],
                np.nan if variant.get("z_min_pairs") is None else variant["z_min_pairs"],
                np.nan if variant.get("z_max_pairs") is None else variant["z_max_pairs"],
                np.nan if variant.get("zerr_cut_deg") is None else variant["zerr_cut_deg"],
                np.nan if variant.get("zerr_cut_kms") is None else variant["zerr_cut_kms"],
                float(ref_cf.x_correlation), float(ref_cf.rmu_binning),
                float(ref_cf.ang_correlation),
                float(ref_cf.remove_same_half_plate_close_pairs)])
            out[prefix + "scalars"] = np.array([d1.z_qso, d2.z_qso, ang, float(same_half_plate)])
            for key, val in (("z1", d1.z), ("r1", r1), ("m1", m1), ("w1", d1.weights),
                             ("d1", d1.delta), ("z2", d2.z), ("r2", r2), ("m2", m2),
                             ("w2", d2.weights), ("d2", d2.delta)):
                out[prefix + key] = np.asarray(val, dtype=float)
            for key, val in zip(("we", "xi", "rp", "rt", "z", "nb"), arrays):
                out[prefix + "out_" + key] = val
            out[prefix + "name"] = np.asarray(variant["name"])
            case_index += 1
    out["num_cf_cases"] = np.asarray(case_index)

    # xcf: one forest against many quasars (the other forests' quasars)
    xcf_variants = [
        dict(name="xcf", r_par_min=-60., r_par_max=60., r_trans_max=60., np=30, nt=15),
        dict(name="xcf_zcut", r_par_min=-60., r_par_max=60., r_trans_max=60., np=30, nt=15,
             z_min_pairs=2.25, z_max_pairs=2.3),
        dict(name="xcf_rmu", r_par_min=-1., r_par_max=1., r_trans_max=60., np=20, nt=15,
             rmu_binning=True),
        dict(name="xcf_wide", r_par_min=-200., r_par_max=200., r_trans_max=200., np=100, nt=50),
    ]
    xcase = 0
    qso_ids = rng.permutation(len(deltas))
    for variant in xcf_variants:
        for forest_index in (int(pairs[0][0]), int(pairs[1][0]), int(pairs[2][1])):
            d1 = deltas[forest_index]
            cands = [deltas[i] for i in qso_ids[:400] if i != forest_index]
            ang = d1.get_angle_between(cands)
            keep = ang < 0.03
            objs = [c for c, k in zip(cands, keep) if k]
            ang = ang[keep]
            z_qso = np.array([o.z_qso for o in objs])
            r_qso = np.asarray(cosmo.get_r_comov(z_qso), dtype=float)
            m_qso = np.asarray(cosmo.get_dist_m(z_qso), dtype=float)
            w_qso = ((1. + z_qso) / (1. + 2.25))**(1.44 - 1.)
            ref_xcf.r_par_min = variant["r_par_min"]
            ref_xcf.r_par_max = variant["r_par_max"]
            ref_xcf.r_trans_max = variant["r_trans_max"]
            ref_xcf.num_bins_r_par = variant["np"]
            ref_xcf.num_bins_r_trans = variant["nt"]
            ref_xcf.z_min_pairs = variant.get("z_min_pairs")
            ref_xcf.z_max_pairs = variant.get("z_max_pairs")
            ref_xcf.rmu_binning = variant.get("rmu_binning", False)
            ref_xcf.ang_correlation = False
            nbins = variant["np"] * variant["nt"]
            arrays = [np.zeros(nbins) for _ in range(5)] + [np.zeros(nbins, dtype=np.int64)]
            ref_xcf.compute_xi_forest_pairs_fast(
                d1.z, d1.r_comov, d1.dist_m, d1.weights, d1.delta,
                z_qso, r_qso, m_qso, w_qso, ang, *arrays)
            prefix = f"xcf{xcase}_"
            out[prefix + "params"] = np.array([
                variant["r_par_min"], variant["r_par_max"], variant["r_trans_max"],
                variant["np"], variant["nt"],
                np.nan if variant.get("z_min_pairs") is None else variant["z_min_pairs"],
                np.nan if variant.get("z_max_pairs") is None else variant["z_max_pairs"],
                float(ref_xcf.rmu_binning)])
            for key, val in (("z1", d1.z), ("r1", d1.r_comov), ("m1", d1.dist_m),
                             ("w1", d1.weights), ("d1", d1.delta), ("zq", z_qso),
                             ("rq", r_qso), ("mq", m_qso), ("wq", w_qso), ("ang", ang)):
                out[prefix + key] = np.asarray(val, dtype=float)
            for key, val in zip(("we", "xi", "rp", "rt", "z", "nb"), arrays):
                out[prefix + "out_" + key] = val
            out[prefix + "name"] = np.asarray(variant["name"])
            xcase += 1
    out["num_xcf_cases"] = np.asarray(xcase)
    np.savez_compressed(os.path.join(HERE, "pair_cases.npz"), **out)
    return case_index, xcase


def _convert_dmat(src, out_path):
    hdul = fitsio_lite.FITS(src)
    dm = hdul["DMAT"]
    attri = hdul["ATTRI"]
    out = {c: dm[c][:] for c in dm.get_colnames()}
    out.update({c: attri[c][:] for c in attri.get_colnames()})
    header = dm.read_header()
    for key in ("RPMIN", "RPMAX", "RTMAX", "NP", "NT", "COEFMOD", "REJ", "NPALL", "NPUSED"):
        out["hdr_" + key] = np.asarray(header[key])
    np.savez_compressed(out_path, **out)


def _dmat_cases(reference_py, delta_dir, attributes):
    """Inputs and outputs of picca's own cf.compute_dmat_forest_pairs_fast
    (run as plain Python) on forest pairs of the test data."""
    sys.dont_write_bytecode = True
    _install_stand_ins()
    sys.path.insert(0, reference_py)
    import picca.cf as ref_cf  # pylint: disable=import-outside-toplevel

    cosmo = gb_constants.Cosmo(Om=0.315, verbose=False)
    data, _, _, _ = gb_io.read_deltas(delta_dir, 16, 1215.67, 2.9, 2.25, cosmo,
                                      delta_attributes=attributes)
    deltas = [d for hp in sorted(data) for d in data[hp]]
    rng = np.random.default_rng(20261204)
    pairs = []
    for _ in range(4000):
        a, b = rng.integers(0, len(deltas), 2)
        if a == b:
            continue
        ang = deltas[a].get_angle_between(deltas[b])
        if ang < 0.01 and abs(deltas[a].z_qso - deltas[b].z_qso) < 0.4:
            pairs.append((a, b))
        if len(pairs) >= 3:
            break
    for a in range(len(deltas)):
        for b in range(a + 1, len(deltas)):
            if deltas[a].plate == deltas[b].plate and (
                    (deltas[a].fiberid <= 500) == (deltas[b].fiberid <= 500)) and (
                        abs(deltas[a].z_qso - deltas[b].z_qso) < 0.5):
                if deltas[a].get_angle_between(deltas[b]) < 0.016:
                    pairs.append((a, b))
                    break
        if len(pairs) >= 4:
            break
    variants = [
        dict(name="auto", np=15, nt=15, coef=1, shp=True, zevol=False, order=(1, 1)),
        dict(name="auto_zevol", np=15, nt=15, coef=1, shp=False, zevol=True, order=(1, 1)),
        dict(name="auto_coef2_order0", np=10, nt=10, coef=2, shp=False, zevol=True,
             order=(0, 1)),
        dict(name="auto_zcut_zerr", np=15, nt=15, coef=1, shp=True, zevol=True, order=(1, 0),
             z_min_pairs=2.2, z_max_pairs=2.4, zerr_cut_deg=2.0, zerr_cut_kms=30000.),
    ]
    out = {}
    case = 0
    for variant in variants:
        for (a, b) in pairs:
            d1, d2 = deltas[a], deltas[b]
            ref_cf.r_par_min, ref_cf.r_par_max, ref_cf.r_trans_max = 0., 60., 60.
            ref_cf.num_bins_r_par, ref_cf.num_bins_r_trans = variant["np"], variant["nt"]
            ref_cf.num_model_bins_r_par = variant["np"] * variant["coef"]
            ref_cf.num_model_bins_r_trans = variant["nt"] * variant["coef"]
            ref_cf.z_min_pairs = variant.get("z_min_pairs")
            ref_cf.z_max_pairs = variant.get("z_max_pairs")
            ref_cf.zerr_cut_deg = variant.get("zerr_cut_deg")
            ref_cf.zerr_cut_kms = variant.get("zerr_cut_kms")
            ref_cf.x_correlation = False
            ref_cf.rmu_binning = False
            ref_cf.remove_same_half_plate_close_pairs = variant["shp"]
            ref_cf.redshift_evolution_in_distortion_matrix = variant["zevol"]
            ref_cf.z_ref, ref_cf.alpha, ref_cf.alpha2 = 2.25, 2.9, 2.9
            nb = variant["np"] * variant["nt"]
            nm = nb * variant["coef"] ** 2
            arrays = dict(weights_dmat=np.zeros(nb), dmat=np.zeros(nb * nm),
                          r_par_eff=np.zeros(nm), r_trans_eff=np.zeros(nm), z_eff=np.zeros(nm),
                          weight_eff=np.zeros(nm))
            ang = d1.get_angle_between(d2)
            shp = (d1.plate == d2.plate) and (
                (d1.fiberid <= 500 and d2.fiberid <= 500) or
                (d1.fiberid > 500 and d2.fiberid > 500))
            try:
                ref_cf.compute_dmat_forest_pairs_fast(
                    d1.log_lambda, d2.log_lambda, d1.r_comov, d2.r_comov, d1.dist_m,
                    d2.dist_m, d1.z, d2.z, d1.weights, d2.weights, d1.z_qso, d2.z_qso, ang,
                    arrays["weights_dmat"], arrays["dmat"], arrays["r_par_eff"],
                    arrays["r_trans_eff"], arrays["z_eff"], arrays["weight_eff"], shp,
                    variant["order"][0], variant["order"][1])
            except IndexError:
                # cf.py:544-568 counts the pairs without those vetoed as same
                # half-plate, while cf.py:702 stores every pair in range: with a
                # vetoed pair the reference writes past its array (silently
                # under numba). Such a pair cannot serve as a fixture.
                continue
            prefix = f"dm{case}_"
            out[prefix + "params"] = np.array([
                variant["np"], variant["nt"], variant["coef"], float(variant["shp"]),
                float(variant["zevol"]), variant["order"][0], variant["order"][1],
                np.nan if variant.get("z_min_pairs") is None else variant["z_min_pairs"],
                np.nan if variant.get("z_max_pairs") is None else variant["z_max_pairs"],
                np.nan if variant.get("zerr_cut_deg") is None else variant["zerr_cut_deg"],
                np.nan if variant.get("zerr_cut_kms") is None else variant["zerr_cut_kms"]])
            out[prefix + "scalars"] = np.array([d1.z_qso, d2.z_qso, ang, float(shp)])
            for key, val in (("ll1", d1.log_lambda), ("ll2", d2.log_lambda), ("r1", d1.r_comov),
                             ("r2", d2.r_comov), ("m1", d1.dist_m), ("m2", d2.dist_m),
                             ("z1", d1.z), ("z2", d2.z), ("w1", d1.weights),
                             ("w2", d2.weights)):
                out[prefix + key] = np.asarray(val, dtype=float)
            for key, val in arrays.items():
                out[prefix + "out_" + key] = val
            out[prefix + "name"] = np.asarray(variant["name"])
            case += 1
    out["num_cases"] = np.asarray(case)
    np.savez_compressed(os.path.join(HERE, "dmat_cases.npz"), **out)
    return case


def _xdmat_cases(reference_py, delta_dir, attributes, catalogue):
    """Inputs and outputs of picca's own xcf.compute_dmat_forest_pairs_fast
    (run as plain Python) on forests of the test data with the quasars
    around them."""
    sys.dont_write_bytecode = True
    _install_stand_ins()
    if reference_py not in sys.path:
        sys.path.insert(0, reference_py)
    import picca.xcf as ref_xcf  # pylint: disable=import-outside-toplevel

    cosmo = gb_constants.Cosmo(Om=0.315, verbose=False)
    data, _, _, _ = gb_io.read_deltas(delta_dir, 16, 1215.67, 2.9, 2.25, cosmo,
                                      delta_attributes=attributes)
    objs, _ = gb_io.read_objects(catalogue, 16, 0, 10, 1.44, 2.25, cosmo)
    deltas = [d for hp in sorted(data) for d in data[hp]]
    quasars = [o for hp in sorted(objs) for o in objs[hp]]
    rng = np.random.default_rng(20261205)
    picks = []
    for a in rng.permutation(len(deltas)):
        d = deltas[a]
        near = [o for o in quasars if o.thingid != d.thingid and
                d.get_angle_between(o) < 0.02]
        if len(near) >= 3:
            picks.append((d, near[:12]))
        if len(picks) >= 3:
            break
    variants = [
        dict(name="xcf", np=30, nt=15, coef=1, zevol=False, order=1),
        dict(name="xcf_zevol", np=30, nt=15, coef=1, zevol=True, order=1),
        dict(name="xcf_coef2_order0", np=10, nt=8, coef=2, zevol=True, order=0),
        dict(name="xcf_zcut", np=30, nt=15, coef=1, zevol=True, order=1, z_min_pairs=2.25,
             z_max_pairs=2.6),
    ]
    out = {}
    case = 0
    for variant in variants:
        for d, near in picks:
            ref_xcf.r_par_min, ref_xcf.r_par_max, ref_xcf.r_trans_max = -60., 60., 60.
            ref_xcf.num_bins_r_par, ref_xcf.num_bins_r_trans = variant["np"], variant["nt"]
            ref_xcf.num_model_bins_r_par = variant["np"] * variant["coef"]
            ref_xcf.num_model_bins_r_trans = variant["nt"] * variant["coef"]
            ref_xcf.z_min_pairs = variant.get("z_min_pairs")
            ref_xcf.z_max_pairs = variant.get("z_max_pairs")
            ref_xcf.rmu_binning = False
            ref_xcf.redshift_evolution_in_distortion_matrix = variant["zevol"]
            ref_xcf.z_ref, ref_xcf.alpha, ref_xcf.alpha_obj = 2.25, 2.9, 1.44
            nb = variant["np"] * variant["nt"]
            nm = nb * variant["coef"] ** 2
            arrays = dict(weights_dmat=np.zeros(nb), dmat=np.zeros(nb * nm),
                          r_par_eff=np.zeros(nm), r_trans_eff=np.zeros(nm), z_eff=np.zeros(nm),
                          weight_eff=np.zeros(nm))
            ang = np.array([d.get_angle_between(o) for o in near])
            r2 = np.array([o.r_comov for o in near])
            m2 = np.array([o.dist_m for o in near])
            w2 = np.array([o.weights for o in near])
            z2 = np.array([o.z_qso for o in near])
            ref_xcf.compute_dmat_forest_pairs_fast(
                d.log_lambda, d.r_comov, d.dist_m, d.z, d.weights, r2, m2, z2, w2, ang,
                arrays["weights_dmat"], arrays["dmat"], arrays["r_par_eff"],
                arrays["r_trans_eff"], arrays["z_eff"], arrays["weight_eff"], variant["order"])
            prefix = f"xd{case}_"
            out[prefix + "params"] = np.array([
                variant["np"], variant["nt"], variant["coef"], float(variant["zevol"]),
                variant["order"],
                np.nan if variant.get("z_min_pairs") is None else variant["z_min_pairs"],
                np.nan if variant.get("z_max_pairs") is None else variant["z_max_pairs"]])
            for key, val in (("ll1", d.log_lambda), ("r1", d.r_comov), ("m1", d.dist_m),
                             ("z1", d.z), ("w1", d.weights), ("r2", r2), ("m2", m2),
                             ("z2", z2), ("w2", w2), ("ang", ang)):
                out[prefix + key] = np.asarray(val, dtype=float)
            for key, val in arrays.items():
                out[prefix + "out_" + key] = val
            out[prefix + "name"] = np.asarray(variant["name"])
            case += 1
    out["num_cases"] = np.asarray(case)
    np.savez_compressed(os.path.join(HERE, "xdmat_cases.npz"), **out)
    return case


def _continuum_cases(reference_py):
    """chi2 of picca's own LeastsSquaresContModel (least_squares_cont_model.py:
    65-197) on synthetic forests at several (zero_point, slope) points."""
    sys.dont_write_bytecode = True
    if reference_py not in sys.path:
        sys.path.insert(0, reference_py)
    from picca.delta_extraction.least_squares.least_squares_cont_model import (  # noqa: E501 pylint: disable=import-outside-toplevel
        LeastsSquaresContModel)
    from picca_gb300 import synthetic_spectra
    raw = synthetic_spectra.make_raw_forests(12, 424242)
    rng = np.random.default_rng(77)
    grid = raw.grid
    out = {"num_cases": np.asarray(raw.num)}
    for k in range(raw.num):
        ll, fl, iv, _ = raw.forest(k)
        iv = iv.copy()
        iv[rng.random(len(iv)) < 0.05] = 0.0  # some masked pixels
        zq = raw.z_qso[k]
        mean_cont = 1.0 + 0.2 * np.sin(ll * 40.0)
        eta = 0.8 + 0.4 * rng.random(len(ll))
        var_lss = 0.05 + 0.1 * rng.random(len(ll))
        fudge = 1e-3 * rng.random(len(ll))
        ll_min = grid.log_lambda_rest_frame_grid[0] + np.log10(1 + zq)
        ll_max = grid.log_lambda_rest_frame_grid[-1] + np.log10(1 + zq)
        forest = types.SimpleNamespace(log_lambda=ll, flux=fl, ivar=iv)
        model = LeastsSquaresContModel(
            forest=forest,
            mean_cont_kwargs={"mean_cont": mean_cont, "log_lambda_max": ll_max,
                              "log_lambda_min": ll_min},
            weights_kwargs={"use_constant_weight": False, "eta": eta, "var_lss": var_lss,
                            "fudge": fudge})
        a0 = (fl * iv).sum() / iv.sum()
        points = [(a0, 0.0), (1.1 * a0, 0.3 * a0), (0.8 * a0, -0.2 * a0), (a0, 0.05)]
        values = [model(a, b) for a, b in points]
        pre = f"c{k}_"
        for key, val in (("ll", ll), ("flux", fl), ("ivar", iv), ("mean_cont", mean_cont),
                         ("eta", eta), ("var_lss", var_lss), ("fudge", fudge)):
            out[pre + key] = np.asarray(val, dtype=float)
        out[pre + "scalars"] = np.array([zq, ll_min, ll_max])
        out[pre + "points"] = np.array(points)
        out[pre + "chi2"] = np.array(values)
        out[pre + "ndata"] = np.asarray(model.get_ndata())
    np.savez_compressed(os.path.join(HERE, "continuum_cases.npz"), **out)
    return raw.num


def _continuum_loop_cases(reference_py, wave_solution, num, seed, iterations=3):
    """picca's own Dr16 continuum loop on synthetic raw forests:
    Dr16ExpectedFlux.compute_expected_flux (dr16_expected_flux.py:380-464)
    run as plain Python, with iminuit replaced by _MinuitStandIn, recording
    at every iteration (where the reference saves its iteration files) the
    fit of every forest (zero point, slope, chi2, ndata, reason), the mean
    continuum (_compute_mean_cont, expected_flux.py:256-308), the variance
    statistics of LeastsSquaresVarStats (least_squares_var_stats.py:134-198)
    with the fitted eta / var_lss / fudge, and the delta stack
    (compute_delta_stack, expected_flux.py:190-236); then populate_los_ids
    (dr16_expected_flux.py:706-740) and compute_forest_weights (:466-488),
    and find_bins_log / find_bins_lin (delta_extraction/utils.py:139-186) on
    the pixels. Written to continuum_loop_<wave_solution>.npz."""
    sys.dont_write_bytecode = True
    _install_stand_ins()
    if reference_py not in sys.path:
        sys.path.insert(0, reference_py)
    import logging  # pylint: disable=import-outside-toplevel
    from scipy.interpolate import interp1d  # pylint: disable=import-outside-toplevel
    from picca.delta_extraction.astronomical_objects.forest import Forest  # noqa: E501 pylint: disable=import-outside-toplevel
    import picca.delta_extraction.expected_fluxes.dr16_expected_flux as ref_dr16  # noqa: E501 pylint: disable=import-outside-toplevel
    from picca.delta_extraction import utils as ref_utils  # noqa: E501 pylint: disable=import-outside-toplevel
    from picca_gb300 import synthetic_spectra

    step = 3e-4 if wave_solution == "log" else 0.8
    grid = synthetic_spectra.Grid(step=step, wave_solution=wave_solution)
    Forest.set_class_variables(3600.0, 5500.0, 1040.0, 1200.0, step, step, wave_solution,
                               "10**-17 erg/(s cm2 Angstrom)")
    assert np.array_equal(Forest.log_lambda_grid, grid.log_lambda_grid)
    assert np.array_equal(Forest.log_lambda_rest_frame_grid, grid.log_lambda_rest_frame_grid)
    raw = synthetic_spectra.make_raw_forests(num, seed, grid=grid)
    rng = np.random.default_rng(seed + 1)
    forests = []
    for k in range(raw.num):
        ll, fl, iv, tc = raw.forest(k)
        iv = iv.copy()
        iv[rng.random(len(iv)) < 0.03] = 0.0  # masked pixels
        forests.append(types.SimpleNamespace(
            log_lambda=ll.copy(), flux=fl.copy(), ivar=iv, transmission_correction=tc.copy(),
            z=float(raw.z_qso[k]), los_id=int(raw.los_id[k]), continuum=None,
            bad_continuum_reason=None))

    class _Log:
        def __getattr__(self, name):
            return lambda *a, **k: None

    flux = ref_dr16.Dr16ExpectedFlux.__new__(ref_dr16.Dr16ExpectedFlux)
    flux.logger = _Log()
    flux.los_ids = {}
    flux.num_bins_variance = 20
    flux.num_processors = 1
    flux.num_iterations = iterations
    flux.order = 1
    flux.use_constant_weight = False
    flux.use_ivar_as_weight = False
    flux.force_stack_delta_to_zero = True
    flux.var_lss_mod = 1.0
    flux.limit_eta = (0.5, 1.5)
    flux.limit_var_lss = (0.0, 0.3)
    flux.min_num_qso_in_fit = 5
    flux.continuum_fit_parameters = None
    flux.fit_variance_functions = []
    flux.out_dir = None
    flux._initialize_variance_wavelength_array()
    flux._initialize_mean_continuum_arrays()
    flux._initialize_variance_functions()
    out = {"wave_solution": np.asarray(wave_solution), "num_iterations": np.asarray(iterations),
           "min_num_qso_in_fit": np.asarray(5),
           "pix_offset": np.concatenate([[0], np.cumsum([len(f.flux) for f in forests])]),
           "log_lambda": np.concatenate([f.log_lambda for f in forests]),
           "flux": np.concatenate([f.flux for f in forests]),
           "ivar": np.concatenate([f.ivar for f in forests]),
           "transmission_correction": np.concatenate([f.transmission_correction
                                                      for f in forests]),
           "z_qso": np.array([f.z for f in forests]),
           "los_id": np.array([f.los_id for f in forests]),
           "log_lambda_var_func_grid": flux.log_lambda_var_func_grid.copy(),
           "log_lambda_grid": grid.log_lambda_grid,
           "log_lambda_rest_frame_grid": grid.log_lambda_rest_frame_grid}
    var_stats = []
    original = ref_dr16.LeastsSquaresVarStats

    def recording_var_stats(*args, **kwargs):
        obj = original(*args, **kwargs)
        var_stats.append(obj)
        return obj

    ref_dr16.LeastsSquaresVarStats = recording_var_stats
    snapshots = []

    def save_iteration_step(iteration):
        it = len(snapshots)
        pre = f"it{it}_"
        params = np.array([flux.continuum_fit_parameters[f.los_id] for f in forests])
        snap = {pre + "zero_point": params[:, 0], pre + "slope": params[:, 1],
                pre + "chi2": params[:, 2], pre + "ndata": params[:, 3],
                pre + "bad": np.array([f.bad_continuum_reason is not None for f in forests]),
                pre + "stack_x": np.asarray(flux.get_stack_delta.x),
                pre + "stack_y": np.asarray(flux.get_stack_delta.y)}
        if it < iterations - 1:
            snap[pre + "mean_cont_x"] = np.asarray(flux.get_mean_cont.x)
            snap[pre + "mean_cont_y"] = np.asarray(flux.get_mean_cont.y)
            snap[pre + "mean_cont_weight"] = np.asarray(flux.get_mean_cont_weight.y)
            vs = var_stats[-1]
            snap[pre + "var_delta"] = vs.var_delta
            snap[pre + "var2_delta"] = vs.var2_delta
            snap[pre + "num_pixels"] = vs.num_pixels
            snap[pre + "num_qso"] = vs.num_qso
            snap[pre + "eta"] = flux.get_eta(flux.log_lambda_var_func_grid)
            snap[pre + "var_lss"] = flux.get_var_lss(flux.log_lambda_var_func_grid)
            snap[pre + "fudge"] = flux.get_fudge(flux.log_lambda_var_func_grid)
            snap[pre + "var_x"] = np.asarray(flux.get_eta.x)
        snapshots.append(snap)

    flux.save_iteration_step = save_iteration_step
    logging.disable(logging.CRITICAL)
    flux.compute_expected_flux(forests)
    ref_dr16.LeastsSquaresVarStats = original
    for snap in snapshots:
        out.update(snap)
    good = [f for f in forests if f.bad_continuum_reason is None]
    out["los_good"] = np.array([f.los_id for f in good])
    out["los_mean_expected_flux"] = np.concatenate(
        [flux.los_ids[f.los_id]["mean expected flux"] for f in good])
    out["los_weights"] = np.concatenate([flux.los_ids[f.los_id]["weights"] for f in good])
    out["los_continuum"] = np.concatenate([flux.los_ids[f.los_id]["continuum"] for f in good])
    # the weights of the last iteration's continua (compute_forest_weights)
    out["forest_weights"] = np.concatenate([flux.compute_forest_weights(f, f.continuum)
                                            for f in good])
    # find_bins on the observed and rest-frame grids
    finder = ref_utils.find_bins_log if wave_solution == "log" else ref_utils.find_bins_lin
    out["bins_obs"] = finder(out["log_lambda"], grid.log_lambda_grid)
    zpix = np.repeat(out["z_qso"], np.diff(out["pix_offset"]))
    out["bins_rest"] = finder(out["log_lambda"] - np.log10(1 + zpix),
                              grid.log_lambda_rest_frame_grid)
    out["bins_var"] = finder(out["log_lambda"], flux.log_lambda_var_func_grid)
    np.savez_compressed(os.path.join(HERE, f"continuum_loop_{wave_solution}.npz"), **out)
    return len(good)


def main(picca_root):
    tests = os.path.join(picca_root, "py", "picca", "tests", "data")
    _convert_delta_dir(os.path.join(tests, "test_delta", "Delta_LYA"),
                       os.path.join(HERE, "delta_lya.npz"))
    _convert_image_dir(os.path.join(tests, "test_delta", "Delta_LYA_image"),
                       os.path.join(HERE, "delta_lya_image.npz"))
    _convert_cat(os.path.join(tests, "test_delta", "cat.fits"), os.path.join(HERE, "cat.npz"))
    for case in ("cf", "cf_zcuts", "cf_cross", "cf_cross_zcuts", "cf_image",
                 "cf_image_rebinned", "cf_image_zcuts", "xcf", "xcf_zcuts"):
        _convert_cor(os.path.join(tests, "test_cor", case + ".fits.gz"),
                     os.path.join(HERE, f"cor_{case}.npz"))
    ncf, nxcf = _pair_cases(os.path.join(picca_root, "py"),
                            os.path.join(tests, "test_delta", "Delta_LYA") + "/",
                            os.path.join(tests, "test_delta", "delta_attributes.fits.gz"))
    ncont = _continuum_cases(os.path.join(picca_root, "py"))
    for wave, num, seed in (("log", 240, 606), ("lin", 80, 707)):
        _continuum_loop_cases(os.path.join(picca_root, "py"), wave, num, seed)
    _convert_dmat(os.path.join(tests, "test_cor", "dmat.fits.gz"),
                  os.path.join(HERE, "cor_dmat.npz"))
    ndm = _dmat_cases(os.path.join(picca_root, "py"),
                      os.path.join(tests, "test_delta", "Delta_LYA") + "/",
                      os.path.join(tests, "test_delta", "delta_attributes.fits.gz"))
    extra_dmat(picca_root)
    extra_metal(picca_root)
    extra_fast_metal(picca_root)
    extra_wick(picca_root)
    print(f"wrote fixtures: {ncf} cf pair cases, {nxcf} xcf cases, {ncont} continuum cases, "
          f"{ndm} distortion-matrix cases")


def _convert_metal_dmat(src, out_path):
    hdul = fitsio_lite.FITS(src)
    attri = hdul["ATTRI"]
    mdmat = hdul["MDMAT"]
    out = {c: mdmat[c][:] for c in mdmat.get_colnames()}
    out["NPALL"] = attri["NPALL"][:]
    out["NPUSED"] = attri["NPUSED"][:]
    out["ABS_IGM"] = np.asarray([str(x) for x in attri["ABS_IGM"][:]])
    header = attri.read_header()
    for key in ("RPMIN", "RPMAX", "RTMAX", "NP", "NT", "COEFMOD", "REJ", "ALPHAMET"):
        if key in header:
            out["hdr_" + key] = np.asarray(header[key])
    np.savez_compressed(out_path, **out)


def extra_metal(picca_root):
    """picca's golden metal distortion matrices (test_cor/metal_dmat.fits.gz
    and metal_xdmat.fits.gz, commands at py/picca/tests/test_3_cor.py:351-382
    and :700-729)."""
    tests = os.path.join(picca_root, "py", "picca", "tests", "data")
    _convert_metal_dmat(os.path.join(tests, "test_cor", "metal_dmat.fits.gz"),
                        os.path.join(HERE, "cor_metal_dmat.npz"))
    _convert_metal_dmat(os.path.join(tests, "test_cor", "metal_xdmat.fits.gz"),
                        os.path.join(HERE, "cor_metal_xdmat.npz"))
    _convert_metal_dmat(os.path.join(tests, "test_cor", "metal_dmat_cross.fits.gz"),
                        os.path.join(HERE, "cor_metal_dmat_cross.npz"))


def _convert_fast_metal(src, out_path):
    hdul = fitsio_lite.FITS(src)
    attri = hdul["ATTRI"]
    mdmat = hdul["MDMAT"]
    out = {c: mdmat[c][:] for c in mdmat.get_colnames()}
    out["ABS_IGM"] = np.asarray([str(x) for x in attri["ABS_IGM"][:]])
    np.savez_compressed(out_path, **out)


def extra_fast_metal(picca_root):
    """picca's golden fast metal distortion matrices (test_cor/
    fast_metal_dmat.fits.gz, fast_metal_dmat_cross.fits.gz,
    fast_metal_xdmat.fits.gz; commands at py/picca/tests/test_3_cor.py:384-409,
    :562-589 and :731-757) and their input, the STACK_DELTAS table of
    test_cor/input_from_delta_extraction_lya_nodla/Log/delta_attributes.fits.gz."""
    tests = os.path.join(picca_root, "py", "picca", "tests", "data")
    for case in ("fast_metal_dmat", "fast_metal_dmat_cross", "fast_metal_xdmat"):
        _convert_fast_metal(os.path.join(tests, "test_cor", case + ".fits.gz"),
                            os.path.join(HERE, f"cor_{case}.npz"))
    stack = fitsio_lite.FITS(os.path.join(
        tests, "test_cor", "input_from_delta_extraction_lya_nodla", "Log",
        "delta_attributes.fits.gz"))["STACK_DELTAS"]
    np.savez_compressed(os.path.join(HERE, "stack_lya_nodla.npz"),
                        **{c: stack[c][:] for c in stack.get_colnames()})


def extra_wick(picca_root):
    """picca's golden Wick covariances (test_cor/wick.fits.gz and
    xwick.fits.gz, commands at py/picca/tests/test_3_cor.py:412-441 and
    :759-791) and their 1D-correlation input (test_cor/cf1d.fits.gz, HDU
    1DCOR)."""
    tests = os.path.join(picca_root, "py", "picca", "tests", "data", "test_cor")
    hdu = fitsio_lite.FITS(os.path.join(tests, "cf1d.fits.gz"))[1]
    header = hdu.read_header()
    out = {c: hdu[c][:] for c in hdu.get_colnames()}
    out["LLMIN"], out["DLL"] = np.asarray(header["LLMIN"]), np.asarray(header["DLL"])
    np.savez_compressed(os.path.join(HERE, "cf1d.npz"), **out)
    for case in ("wick", "xwick"):
        cov = fitsio_lite.FITS(os.path.join(tests, case + ".fits.gz"))["COV"]
        header = cov.read_header()
        out = {c: cov[c][:] for c in cov.get_colnames()}
        for key in ("NPALL", "NPUSED"):
            out["hdr_" + key] = np.asarray(header[key])
        np.savez_compressed(os.path.join(HERE, f"cor_{case}.npz"), **out)


def extra_rebin(picca_root):
    """The image-layout inputs with their LAMBDA header cards (WAVE_SOLUTION,
    DELTA_LAMBDA: HIERARCH keywords), and picca's rebinned image-layout
    correlation (py/picca/tests/test_3_cor.py:288-316)."""
    tests = os.path.join(picca_root, "py", "picca", "tests", "data")
    _convert_image_dir(os.path.join(tests, "test_delta", "Delta_LYA_image"),
                       os.path.join(HERE, "delta_lya_image.npz"))
    _convert_cor(os.path.join(tests, "test_cor", "cf_image_rebinned.fits.gz"),
                 os.path.join(HERE, "cor_cf_image_rebinned.npz"))


def extra_dmat(picca_root):
    """The other golden distortion matrices (cf z cuts, the cross of two
    delta sets, delta x quasar) and the xcf forest cases."""
    tests = os.path.join(picca_root, "py", "picca", "tests", "data")
    for case in ("dmat_zcuts", "dmat_cross", "dmat_cross_zcuts", "xdmat", "xdmat_zcuts"):
        _convert_dmat(os.path.join(tests, "test_cor", case + ".fits.gz"),
                      os.path.join(HERE, f"cor_{case}.npz"))
    return _xdmat_cases(os.path.join(picca_root, "py"),
                        os.path.join(tests, "test_delta", "Delta_LYA") + "/",
                        os.path.join(tests, "test_delta", "delta_attributes.fits.gz"),
                        os.path.join(tests, "test_delta", "cat.fits"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/picca")
    main(sys.argv[1])
