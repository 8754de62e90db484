"""Drop-in replacement for the correlation part of ``picca.cf``.

Same module globals (py/picca/cf.py:28-79) and the same functions:

* ``fill_neighs(healpixs)`` sets ``delta.neighbours`` (py/picca/cf.py:82-135);
* ``compute_xi(healpixs)`` returns ``(weights, xi, r_par, r_trans, z,
  num_pairs)`` for those healpix (py/picca/cf.py:138-247);
* ``compute_xi_forest_pairs_fast(...)`` keeps the 20-argument signature and
  accumulates one forest pair in place (py/picca/cf.py:250-387);
* ``compute_dmat(healpixs)`` returns the raw distortion-matrix sums of those
  healpix with the reference's random rejection (py/picca/cf.py:390-517),
  and ``compute_dmat_forest_pairs_fast(...)`` keeps the 22-argument signature
  (py/picca/cf.py:519-887);
* ``compute_metal_dmat(healpixs, abs_igm1, abs_igm2)`` returns the raw metal
  distortion-matrix sums (py/picca/cf.py:890-1218).

All pair arithmetic runs on the GPU through ``libpicca_gb300``. The first
``fill_neighs`` / ``compute_xi`` call computes the neighbour lists and the
per-healpix sums of *every* healpix in one launch (``compute_xi_all``) and
later calls are served from that result, which replaces the reference's
one-process-per-healpix Pool. ``precision`` selects the arithmetic:
``"fp64"`` (plain form) or ``"fp32_guard"`` (FP32 geometry with FP64 bin-edge
re-decision; bin indices and pair counts identical to FP64).
"""

import numpy as np

from . import dmat as _dmat
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

# variables for distortion matrix
redshift_evolution_in_distortion_matrix = True
# arithmetic of the distortion-matrix eta products: "split_bf16" (tensor
# cores, exact 8-bit digit products) or "fp64"
dmat_product = "split_bf16"

# arithmetic of the GPU pair kernel: "fp64" or "fp32_guard"
precision = "fp32_guard"

_cache = {"key": None, "result": None, "engine": None, "dmat_engine": None,
          "nbr_key": None, "nbr": None}


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
    res = _pairs.correlate(fs1, fs2, _params(), mode=_mode(), engine=_engine(), pinned=True)
    we, xi, rp, rt, zz, nb = res["raw"]
    xi_n, rp_n, rt_n, zz_n = _pairs.normalise(we, xi, rp, rt, zz)
    index = res["index"].cpu().numpy()[: res["num_pairs_forest"]]
    offsets = res["offsets"].cpu().numpy()
    result = {
        "healpix_list": fs1.healpix_list, "weights": we, "xi": xi_n, "r_par": rp_n,
        "r_trans": rt_n, "z": zz_n, "num_pairs": nb, "raw": res["raw"],
        "candidate_pairs": res["candidate_pairs"], "rechecked_pairs": res["rechecked_pairs"],
        "forest_pairs": res["num_pairs_forest"], "nbr_offsets": offsets, "nbr_index": index,
        "set1": fs1, "set2": fs2, "h2d_bytes": res["h2d_bytes"],
        "d2h_bytes": sum(int(a.nbytes) for a in res["raw"]) + int(offsets.nbytes) + int(index.nbytes),
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


def _single_forest(z, r, m, w, d, zq, plate, fiber, log_lambda=None, order=-1):
    """A one-forest ForestSet (the per-pair drop-ins). Same-half-plate pairs
    are expressed through the plate number with fiber ids on one half."""
    n = len(z)
    return ForestSet(
        pix_offset=np.array([0, n], dtype=np.int64), z=np.asarray(z, float),
        r_comov=np.asarray(r, float), dist_m=np.asarray(m, float),
        weights=np.asarray(w, float), delta=np.asarray(d, float),
        log_lambda=np.zeros(n) if log_lambda is None else np.asarray(log_lambda, float),
        ra=np.zeros(1), dec=np.zeros(1), x_cart=np.ones(1), y_cart=np.zeros(1),
        z_cart=np.zeros(1), cos_dec=np.ones(1), z_qso=np.array([float(zq)]),
        thingid=np.array([plate]), plate=np.array([plate]), fiberid=np.array([fiber]),
        order=np.array([order], dtype=np.int64), healpix=np.zeros(1, dtype=np.int64))


def compute_xi_forest_pairs_fast(z1, r_comov1, dist_m1, weights1, delta1, z_qso_1, z2, r_comov2,
                                 dist_m2, weights2, delta2, z_qso_2, ang, same_half_plate,
                                 rebin_weight, rebin_xi, rebin_r_par, rebin_r_trans, rebin_z,
                                 rebin_num_pairs):
    """One forest pair on the GPU, accumulated in place into the six arrays
    (py/picca/cf.py:250-387 signature)."""
    import torch  # pylint: disable=import-outside-toplevel

    fs1 = _single_forest(z1, r_comov1, dist_m1, weights1, delta1, z_qso_1, 0, 1)
    fs2 = _single_forest(z2, r_comov2, dist_m2, weights2, delta2, z_qso_2,
                         0 if same_half_plate else 1, 1)
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


def _dmat_params():
    if num_model_bins_r_par is None or num_model_bins_r_trans is None:
        raise ValueError("cf.num_model_bins_r_par / num_model_bins_r_trans must be set "
                         "before computing a distortion matrix")
    return _dmat.make_dmat_params(
        num_bins_r_par, num_bins_r_trans,
        redshift_evolution=redshift_evolution_in_distortion_matrix,
        z_ref=2.25 if z_ref is None else z_ref, alpha=2.9 if alpha is None else alpha,
        alpha2=(alpha if alpha2 is None else alpha2) if alpha is not None else 2.9,
        num_model_bins_r_par=num_model_bins_r_par,
        num_model_bins_r_trans=num_model_bins_r_trans, product=dmat_product)


def _dmat_engine():
    if _cache["dmat_engine"] is None:
        _cache["dmat_engine"] = _dmat.DmatEngine(_engine())
    return _cache["dmat_engine"]


def _neighbour_state():
    """Device forests and neighbour CSR of ``data`` (and ``data2``), cached
    like compute_xi_all."""
    key = _state_key()
    if _cache["nbr_key"] == key and _cache["nbr"] is not None:
        return _cache["nbr"]
    if data is None:
        raise ValueError("cf.data is not set")
    if ang_correlation:
        raise ValueError("the distortion matrix has no angular form")
    engine = _engine()
    fs1 = ForestSet.from_deltas(data)
    fs2 = ForestSet.from_deltas(data2) if data2 is not None else None
    _check_fiberids(fs1)
    if fs2 is not None:
        _check_fiberids(fs2)
    dev1 = _pairs.DeviceForests(fs1, engine.device)
    dev2 = _pairs.DeviceForests(fs2, engine.device) if fs2 is not None else None
    offsets, index, total = engine.neighbours(_params(), dev1, dev2)
    state = {"set1": fs1, "set2": fs2, "dev1": dev1, "dev2": dev2, "offsets": offsets,
             "index": index, "total": total, "offsets_host": offsets.cpu().numpy()}
    _cache["nbr_key"] = key
    _cache["nbr"] = state
    return state


def _dmat_sums(state, mask):
    """GPU sums of the pairs selected by ``mask`` (a bool array over the
    neighbour CSR); returns host arrays."""
    engine = _dmat_engine()
    fs1, fs2 = state["set1"], state["set2"]
    dev1, dev2 = state["dev1"], state["dev2"]
    first, second, num_sel = engine.pair_list(dev1, dev2, state["offsets"], state["index"], mask)
    if num_sel:
        _dmat.check_orders(fs2 if fs2 is not None else fs1, np.unique(second.cpu().numpy()))
    params, dparams = _params(), _dmat_params()
    side1 = _dmat.DmatEngine.side_arrays(dev1, engine.device)
    side2 = _dmat.DmatEngine.side_arrays(dev2, engine.device) if dev2 is not None else None
    sums = engine.alloc_sums(params, dparams)
    engine.accumulate(params, dparams, dev1, dev2, side1, side2, first, second, num_sel, sums)
    engine.engine.stats()
    return {k: v.cpu().numpy() for k, v in sums.items()}


def compute_dmat(healpixs):
    """Raw distortion-matrix sums of ``healpixs`` (py/picca/cf.py:390-517).

    The random rejection draws ``np.random.rand(len(neighbours)) > reject``
    from NumPy's global generator for every delta of the healpixs, in order,
    as the reference does; the selected forest pairs run on the GPU. Returns
    ``(weights_dmat, dmat [nb, nm], r_par_eff, r_trans_eff, z_eff,
    weight_eff, num_pairs, num_pairs_used)``."""
    state = _neighbour_state()
    fs1 = state["set1"]
    offsets = state["offsets_host"]
    firsts = np.searchsorted(fs1.row, np.arange(len(fs1.healpix_list)))
    mask = np.zeros(int(state["total"]), dtype=bool)
    num_pairs = 0
    num_pairs_used = 0
    visited = []
    for healpix in healpixs:
        row = int(np.searchsorted(fs1.healpix_list, healpix))
        for k, delta in enumerate(data[healpix]):
            f = firsts[row] + k
            visited.append(f)
            if getattr(delta, "order", None) is None:
                raise RuntimeError("Trying to compute the distortion matrix but order is not "
                                   "defined for the deltas. Check previous warning to solve "
                                   "this issue")
            start, end = int(offsets[f]), int(offsets[f + 1])
            w = np.random.rand(end - start) > reject
            num_pairs += end - start
            num_pairs_used += int(w.sum())
            mask[start:end] = w
    raw = _dmat_sums(state, mask)
    for healpix in healpixs:
        for delta in data[healpix]:
            if hasattr(delta, "neighbours"):
                delta.neighbours = None
    nb = num_bins_r_par * num_bins_r_trans
    return (raw["weights_dmat"], raw["dmat"].reshape(nb, -1), raw["r_par_eff"],
            raw["r_trans_eff"], raw["z_eff"], raw["weight_eff"], num_pairs, num_pairs_used)


def compute_dmat_all(nproc):
    """The whole picca_dmat.py computation for ``nproc`` processes: the
    random rejection of every chunk (healpix index % nproc, generator seeded
    with the chunk's first healpix) and one GPU pass over all selected forest
    pairs. Returns the normalised columns (WDM, DM, RP, RT, Z) and NPALL /
    NPUSED."""
    state = _neighbour_state()
    fs1 = state["set1"]
    _dmat.check_orders(fs1, np.arange(fs1.num))
    mask = _dmat.selection_mask(fs1.healpix_list, fs1.row, state["offsets_host"], nproc, reject)
    raw = _dmat_sums(state, mask)
    result = _dmat.normalise(raw, _params(), _dmat_params(), state["total"], int(mask.sum()))
    result["raw"] = raw
    return result


def compute_dmat_forest_pairs_fast(log_lambda1, log_lambda2, r_comov1, r_comov2, dist_m1,
                                   dist_m2, z1, z2, weights1, weights2, z_qso_1, z_qso_2, ang,
                                   weights_dmat, dmat, r_par_eff, r_trans_eff, z_eff,
                                   weight_eff, same_half_plate, order1, order2):
    """One forest pair on the GPU, accumulated in place into the six arrays
    (py/picca/cf.py:519-545 signature)."""
    import torch  # pylint: disable=import-outside-toplevel

    zeros1, zeros2 = np.zeros(len(z1)), np.zeros(len(z2))
    fs1 = _single_forest(z1, r_comov1, dist_m1, weights1, zeros1, z_qso_1, 0, 1,
                         log_lambda=log_lambda1, order=int(order1))
    fs2 = _single_forest(z2, r_comov2, dist_m2, weights2, zeros2, z_qso_2,
                         0 if same_half_plate else 1, 1, log_lambda=log_lambda2,
                         order=int(order2))
    engine = _dmat_engine()
    dev = engine.device
    dev1 = _pairs.DeviceForests(fs1, dev)
    dev2 = _pairs.DeviceForests(fs2, dev)
    params = _pairs.make_params(
        r_par_min, r_par_max, r_trans_max, num_bins_r_par, num_bins_r_trans, np.pi,
        z_min_pairs=z_min_pairs, z_max_pairs=z_max_pairs, zerr_cut_deg=zerr_cut_deg,
        zerr_cut_kms=zerr_cut_kms, x_correlation=x_correlation, rmu_binning=rmu_binning,
        remove_same_half_plate_close_pairs=remove_same_half_plate_close_pairs)
    dparams = _dmat_params()
    side1 = _dmat.DmatEngine.side_arrays(dev1, dev)
    side2 = _dmat.DmatEngine.side_arrays(dev2, dev)
    pair = torch.zeros(1, dtype=torch.int32, device=dev)
    angles = torch.tensor([float(ang)], dtype=torch.float64, device=dev)
    sums = engine.alloc_sums(params, dparams)
    engine.accumulate(params, dparams, dev1, dev2, side1, side2, pair, pair, 1, sums,
                      angles=angles)
    engine.engine.stats()
    weights_dmat += sums["weights_dmat"].cpu().numpy()
    dmat += sums["dmat"].cpu().numpy().reshape(np.shape(dmat))
    r_par_eff += sums["r_par_eff"].cpu().numpy()
    r_trans_eff += sums["r_trans_eff"].cpu().numpy()
    z_eff += sums["z_eff"].cpu().numpy()
    weight_eff += sums["weight_eff"].cpu().numpy()


def compute_metal_dmat(healpixs, abs_igm1="LYA", abs_igm2="SiIII(1207)"):
    """Raw metal distortion-matrix sums of ``healpixs`` for the absorbers
    (abs_igm1, abs_igm2) (py/picca/cf.py:890-1218): the random rejection
    from NumPy's global generator as picca draws it, the direct and (for two
    different absorbers) swapped passes on the GPU; module globals
    ``cosmo``, ``alpha_abs`` and ``z_ref`` as picca_metal_dmat.py sets them.
    Returns ``(weights_dmat, dmat [nb, nm], r_par_eff, r_trans_eff, z_eff,
    weight_eff, num_pairs, num_pairs_used)``."""
    from . import metal as _metal  # pylint: disable=import-outside-toplevel

    if cosmo is None or alpha_abs is None:
        raise ValueError("cf.cosmo and cf.alpha_abs must be set for the metal distortion "
                         "matrix")
    state = _neighbour_state()
    fs1 = state["set1"]
    if state["set2"] is not None:
        raise NotImplementedError("the metal distortion matrix of two delta fields is not "
                                  "supported")
    offsets = state["offsets_host"]
    firsts = np.searchsorted(fs1.row, np.arange(len(fs1.healpix_list)))
    mask = np.zeros(int(state["total"]), dtype=bool)
    num_pairs = num_pairs_used = 0
    for healpix in healpixs:
        row = int(np.searchsorted(fs1.healpix_list, healpix))
        for k, _ in enumerate(data[healpix]):
            f = firsts[row] + k
            start, end = int(offsets[f]), int(offsets[f + 1])
            w = np.random.rand(end - start) > reject
            num_pairs += end - start
            num_pairs_used += int(w.sum())
            mask[start:end] = w
    if _cache.get("metal_engine") is None:
        _cache["metal_engine"] = _metal.MetalEngine(_engine())
    engine = _cache["metal_engine"]
    dev = state["dev1"]
    first, second, num = engine.pair_list(dev, None, state["offsets"], state["index"], mask)
    params = _params()
    dparams = _dmat.make_dmat_params(num_bins_r_par, num_bins_r_trans,
                                     num_model_bins_r_par=num_model_bins_r_par,
                                     num_model_bins_r_trans=num_model_bins_r_trans)
    zr = 2.25 if z_ref is None else z_ref
    side1 = _metal.absorber_pixels(dev, cosmo, abs_igm1, alpha_abs[abs_igm1])
    side2 = _metal.absorber_pixels(dev, cosmo, abs_igm2, alpha_abs[abs_igm2])
    sums = engine.alloc_sums(params, dparams)
    den = (1 + zr) ** (alpha_abs[abs_igm1] + alpha_abs[abs_igm2] - 2)
    engine.run_pass(params, dparams, den, dev, None, side1, side2, first, second, num, sums)
    if _metal.swapped_pass(abs_igm1, abs_igm2, x_correlation,
                           lambda_abs2 is not None and lambda_abs == lambda_abs2):
        engine.run_pass(params, dparams, den, dev, None, side2, side1, first, second, num,
                        sums)
    engine.engine.stats()
    raw = {k: v.cpu().numpy() for k, v in sums.items()}
    for healpix in healpixs:
        for delta in data[healpix]:
            if hasattr(delta, "neighbours"):
                delta.neighbours = None
    nb = num_bins_r_par * num_bins_r_trans
    return (raw["weights_dmat"], raw["dmat"].reshape(nb, -1), raw["r_par_eff"],
            raw["r_trans_eff"], raw["z_eff"], raw["weight_eff"], num_pairs, num_pairs_used)
