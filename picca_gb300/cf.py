"""Drop-in replacement for the correlation part of ``picca.cf``.

Same module globals (py/picca/cf.py:28-79) and the same functions:

* ``fill_neighs(healpixs)`` sets ``delta.neighbours`` (py/picca/cf.py:82-135);
* ``compute_xi(healpixs)`` returns ``(weights, xi, r_par, r_trans, z,
  num_pairs)`` for those healpix (py/picca/cf.py:138-247);
* ``compute_xi_forest_pairs_fast(...)`` keeps the 20-argument signature and
  accumulates one forest pair in place (py/picca/cf.py:250-387).

All pair arithmetic runs on the GPU through ``libpicca_gb300``. The first
``fill_neighs`` / ``compute_xi`` call computes the neighbour lists and the
per-healpix sums of *every* healpix in one launch (``compute_xi_all``) and
later calls are served from that result, which replaces the reference's
one-process-per-healpix Pool. ``precision`` selects the arithmetic:
``"fp64"`` (plain form) or ``"fp32_guard"`` (FP32 geometry with FP64 bin-edge
re-decision; bin indices and pair counts identical to FP64).
"""

import numpy as np

from . import pairs as _pairs
from .forests import ForestSet

num_bins_r_par = None
num_bins_r_trans = None
num_model_bins_r_trans = None
num_model_bins_r_par = None
r_par_max = None
r_par_min = None
z_min_pairs = None
z_max_pairs = None
r_trans_max = None
ang_max = None
nside = None

zerr_cut_deg = None
zerr_cut_kms = None

counter = None
num_data = None
num_data2 = None

z_ref = None
alpha = None
alpha2 = None
alpha_abs = None
lambda_abs = None
lambda_abs2 = None

data = None
data2 = None

cosmo = None

reject = None
lock = None
x_correlation = False
rmu_binning = False
ang_correlation = False
remove_same_half_plate_close_pairs = False

# arithmetic of the GPU pair kernel: "fp64" or "fp32_guard"
precision = "fp32_guard"

_cache = {"key": None, "result": None, "engine": None}


def _mode():
    if precision == "fp64":
        return _pairs.MODE_FP64
    if precision == "fp32_guard":
        return _pairs.MODE_FP32_GUARD
    raise ValueError(f"unknown precision {precision!r}")


def _params():
    if num_bins_r_par is None or num_bins_r_trans is None or ang_max is None:
        raise ValueError("cf module globals (num_bins_r_par, num_bins_r_trans, ang_max, ...) "
                         "must be set before computing correlations")
    return _pairs.make_params(
        r_par_min, r_par_max, r_trans_max, num_bins_r_par, num_bins_r_trans, ang_max,
        z_min_pairs=z_min_pairs, z_max_pairs=z_max_pairs, zerr_cut_deg=zerr_cut_deg,
        zerr_cut_kms=zerr_cut_kms, x_correlation=x_correlation, rmu_binning=rmu_binning,
        ang_correlation=ang_correlation,
        remove_same_half_plate_close_pairs=remove_same_half_plate_close_pairs)


def _state_key():
    return (id(data), id(data2), num_bins_r_par, num_bins_r_trans, r_par_min, r_par_max,
            r_trans_max, z_min_pairs, z_max_pairs, zerr_cut_deg, zerr_cut_kms, ang_max,
            x_correlation, rmu_binning, ang_correlation, remove_same_half_plate_close_pairs,
            precision)


def _engine():
    if _cache["engine"] is None:
        _cache["engine"] = _pairs.PairEngine()
    return _cache["engine"]


def _check_fiberids(fs):
    if remove_same_half_plate_close_pairs and getattr(fs, "fiberid_is_str", False):
        raise RuntimeError("Trying to figure out if two spectra come from the same half plate "
                           "but combined reobservations were given")


def compute_xi_all():
    """Neighbours and pair sums of every healpix of ``data`` in one GPU pass.

    Returns a dict with ``healpix_list``, normalised per-healpix arrays
    ``weights, xi, r_par, r_trans, z, num_pairs`` ([num_healpix, nbins]) and
    run statistics. Results are cached until a global or ``data`` changes."""
    key = _state_key()
    if _cache["key"] == key and _cache["result"] is not None:
        return _cache["result"]
    if data is None:
        raise ValueError("cf.data is not set")
    fs1 = ForestSet.from_deltas(data, ang_correlation=ang_correlation)
    fs2 = ForestSet.from_deltas(data2, ang_correlation=ang_correlation) if data2 is not None else None
    _check_fiberids(fs1)
    if fs2 is not None:
        _check_fiberids(fs2)
    res = _pairs.correlate(fs1, fs2, _params(), mode=_mode(), engine=_engine())
    we, xi, rp, rt, zz, nb = res["raw"]
    xi_n, rp_n, rt_n, zz_n = _pairs.normalise(we, xi, rp, rt, zz)
    index = res["index"].cpu().numpy()[: res["num_pairs_forest"]]
    offsets = res["offsets"].cpu().numpy()
    result = {
        "healpix_list": fs1.healpix_list, "weights": we, "xi": xi_n, "r_par": rp_n,
        "r_trans": rt_n, "z": zz_n, "num_pairs": nb, "raw": res["raw"],
        "candidate_pairs": res["candidate_pairs"], "rechecked_pairs": res["rechecked_pairs"],
        "forest_pairs": res["num_pairs_forest"], "nbr_offsets": offsets, "nbr_index": index,
        "set1": fs1, "set2": fs2,
    }
    _cache["key"] = key
    _cache["result"] = result
    return result


def _deltas_in_order(dataset, healpix_list):
    return [d for hp in healpix_list for d in dataset[hp]]


def fill_neighs(healpixs):
    """Set ``delta.neighbours`` for every delta of ``healpixs``.

    Neighbours are the deltas of ``data2`` (or ``data``) within ``ang_max``
    with a different thingid, and, for the auto-correlation, smaller RA."""
    result = compute_xi_all()
    fs1, fs2 = result["set1"], result["set2"]
    others = _deltas_in_order(data2 if fs2 is not None else data,
                              (fs2 if fs2 is not None else fs1).healpix_list)
    firsts = np.searchsorted(fs1.row, np.arange(len(fs1.healpix_list)))
    offsets, index = result["nbr_offsets"], result["nbr_index"]
    for healpix in healpixs:
        row = int(np.searchsorted(fs1.healpix_list, healpix))
        for k, delta in enumerate(data[healpix]):
            f = firsts[row] + k
            delta.neighbours = [others[g] for g in index[offsets[f]:offsets[f + 1]]]


def compute_xi(healpixs):
    """Correlation function of the given healpixs (sums over them), same
    return tuple as the reference."""
    result = compute_xi_all()
    rows = np.searchsorted(result["healpix_list"], np.asarray(list(healpixs)))
    we, xi, rp, rt, zz, nb = result["raw"]
    weights = we[rows].sum(axis=0)
    xi_s = xi[rows].sum(axis=0)
    rp_s = rp[rows].sum(axis=0)
    rt_s = rt[rows].sum(axis=0)
    z_s = zz[rows].sum(axis=0)
    num_pairs = nb[rows].sum(axis=0).astype(np.int64)
    for healpix in healpixs:
        for delta in data[healpix]:
            delta.neighbours = None
    xi_n, rp_n, rt_n, z_n = _pairs.normalise(weights, xi_s, rp_s, rt_s, z_s)
    return weights, xi_n, rp_n, rt_n, z_n, num_pairs


def compute_xi_forest_pairs_fast(z1, r_comov1, dist_m1, weights1, delta1, z_qso_1, z2, r_comov2,
                                 dist_m2, weights2, delta2, z_qso_2, ang, same_half_plate,
                                 rebin_weight, rebin_xi, rebin_r_par, rebin_r_trans, rebin_z,
                                 rebin_num_pairs):
    """One forest pair on the GPU, accumulated in place into the six arrays
    (py/picca/cf.py:250-387 signature)."""
    import torch  # pylint: disable=import-outside-toplevel

    def one(z, r, m, w, d, zq, plate, fiber):
        n = len(z)
        return ForestSet(
            pix_offset=np.array([0, n], dtype=np.int64), z=np.asarray(z, float),
            r_comov=np.asarray(r, float), dist_m=np.asarray(m, float),
            weights=np.asarray(w, float), delta=np.asarray(d, float),
            log_lambda=np.zeros(n), ra=np.zeros(1), dec=np.zeros(1), x_cart=np.ones(1),
            y_cart=np.zeros(1), z_cart=np.zeros(1), cos_dec=np.ones(1),
            z_qso=np.array([float(zq)]), thingid=np.array([plate]), plate=np.array([plate]),
            fiberid=np.array([fiber]), healpix=np.zeros(1, dtype=np.int64))

    fs1 = one(z1, r_comov1, dist_m1, weights1, delta1, z_qso_1, 0, 1)
    fs2 = one(z2, r_comov2, dist_m2, weights2, delta2, z_qso_2, 0 if same_half_plate else 1, 1)
    engine = _engine()
    dev1 = _pairs.DeviceForests(fs1, engine.device)
    dev2 = _pairs.DeviceForests(fs2, engine.device)
    params = _pairs.make_params(
        r_par_min, r_par_max, r_trans_max, num_bins_r_par, num_bins_r_trans, np.pi,
        z_min_pairs=z_min_pairs, z_max_pairs=z_max_pairs, zerr_cut_deg=zerr_cut_deg,
        zerr_cut_kms=zerr_cut_kms, x_correlation=x_correlation, rmu_binning=rmu_binning,
        ang_correlation=ang_correlation,
        remove_same_half_plate_close_pairs=remove_same_half_plate_close_pairs)
    dev = engine.device
    offsets = torch.tensor([0, 1], dtype=torch.int64, device=dev)
    index = torch.zeros(1, dtype=torch.int32, device=dev)
    angles = torch.tensor([float(ang)], dtype=torch.float64, device=dev)
    order = torch.zeros(1, dtype=torch.int32, device=dev)
    nbins = len(rebin_weight)
    rows = engine.alloc_rows(1, nbins)
    engine.accumulate(params, dev1, dev2, offsets, index, order, 1, rows, _mode(),
                      angles=angles)
    engine.stats()
    we, xi, rp, rt, zz, nb = [r.cpu().numpy() for r in rows]
    rebin_weight += we
    rebin_xi += xi
    rebin_r_par += rp
    rebin_r_trans += rt
    rebin_z += zz
    rebin_num_pairs += nb
