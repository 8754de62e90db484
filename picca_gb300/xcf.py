"""Drop-in replacement for the correlation part of ``picca.xcf``.

Same module globals (py/picca/xcf.py:27-68) and functions ``fill_neighs``
(:71-123), ``compute_xi`` (:126-220), the 16-argument
``compute_xi_forest_pairs_fast`` (:223-322), ``compute_dmat`` (:325-424), the
17-argument ``compute_dmat_forest_pairs_fast`` (:427-675) and
``compute_metal_dmat`` (:677-800), computed on the GPU. As in ``picca_gb300.cf``, the first call runs every healpix in one
launch (``compute_xi_all``) and later calls are served from that result.
"""

import numpy as np

from . import dmat as _dmat
from . import pairs as _pairs
from .forests import ForestSet

num_bins_r_par = None
num_bins_r_trans = None
num_model_bins_r_par = None
num_model_bins_r_trans = None
r_par_max = None
r_par_min = None
r_trans_max = None
z_min_pairs = None
z_max_pairs = None
ang_max = None
nside = None

zerr_cut_deg = None
zerr_cut_kms = None

counter = None
num_data = None

z_ref = None
alpha = None
alpha_obj = None
lambda_abs = None
alpha_abs = None

data = None
objs = None

reject = None
lock = None

cosmo = None
rmu_binning = False
ang_correlation = False

# variables for distortion matrix
redshift_evolution_in_distortion_matrix = True
# arithmetic of the distortion-matrix eta products: "split_bf16" or "fp64"
dmat_product = "split_bf16"

precision = "fp32_guard"

_cache = {"key": None, "result": None, "engine": None, "dmat_engine": None, "nbr_key": None,
          "nbr": None}


def _mode():
    if precision == "fp64":
        return _pairs.MODE_FP64
    if precision == "fp32_guard":
        return _pairs.MODE_FP32_GUARD
    raise ValueError(f"unknown precision {precision!r}")


def _params(angle_max=None):
    return _pairs.make_params(
        r_par_min, r_par_max, r_trans_max, num_bins_r_par, num_bins_r_trans,
        ang_max if angle_max is None else angle_max, z_min_pairs=z_min_pairs,
        z_max_pairs=z_max_pairs, zerr_cut_deg=zerr_cut_deg, zerr_cut_kms=zerr_cut_kms,
        x_correlation=True, rmu_binning=rmu_binning, ang_correlation=ang_correlation)


def _engine():
    if _cache["engine"] is None:
        _cache["engine"] = _pairs.PairEngine()
    return _cache["engine"]


def _state_key():
    return (id(data), id(objs), num_bins_r_par, num_bins_r_trans, r_par_min, r_par_max,
            r_trans_max, z_min_pairs, z_max_pairs, zerr_cut_deg, zerr_cut_kms, ang_max,
            rmu_binning, ang_correlation, precision)


def compute_xi_all():
    """Quasar neighbours and pair sums of every healpix in one GPU pass."""
    key = _state_key()
    if _cache["key"] == key and _cache["result"] is not None:
        return _cache["result"]
    if data is None or objs is None:
        raise ValueError("xcf.data and xcf.objs must be set")
    if ang_max is None or num_bins_r_par is None:
        raise ValueError("xcf module globals must be set before computing correlations")
    fs = ForestSet.from_deltas(data, ang_correlation=ang_correlation)
    qs = ForestSet.from_objects(objs, ang_correlation=ang_correlation)
    res = _pairs.correlate(fs, qs, _params(), mode=_mode(), xcf=True, engine=_engine())
    we, xi, rp, rt, zz, nb = res["raw"]
    xi_n, rp_n, rt_n, zz_n = _pairs.normalise(we, xi, rp, rt, zz)
    result = {
        "healpix_list": fs.healpix_list, "weights": we, "xi": xi_n, "r_par": rp_n,
        "r_trans": rt_n, "z": zz_n, "num_pairs": nb, "raw": res["raw"],
        "candidate_pairs": res["candidate_pairs"], "rechecked_pairs": res["rechecked_pairs"],
        "forest_pairs": res["num_pairs_forest"],
        "nbr_offsets": res["offsets"].cpu().numpy(),
        "nbr_index": res["index"].cpu().numpy()[: res["num_pairs_forest"]],
        "set1": fs, "set2": qs,
    }
    _cache["key"] = key
    _cache["result"] = result
    return result


def fill_neighs(healpixs):
    """Set ``delta.neighbours`` (array of QSO) for every delta of healpixs."""
    result = compute_xi_all()
    fs, qs = result["set1"], result["set2"]
    quasars = [o for hp in qs.healpix_list for o in objs[hp]]
    firsts = np.searchsorted(fs.row, np.arange(len(fs.healpix_list)))
    offsets, index = result["nbr_offsets"], result["nbr_index"]
    for healpix in healpixs:
        row = int(np.searchsorted(fs.healpix_list, healpix))
        for k, delta in enumerate(data[healpix]):
            f = firsts[row] + k
            delta.neighbours = np.array([quasars[g] for g in index[offsets[f]:offsets[f + 1]]])


def compute_xi(healpixs):
    """(weights, xi, r_par, r_trans, z, num_pairs) summed over healpixs."""
    result = compute_xi_all()
    rows = np.searchsorted(result["healpix_list"], np.asarray(list(healpixs)))
    we, xi, rp, rt, zz, nb = result["raw"]
    weights = we[rows].sum(axis=0)
    sums = [a[rows].sum(axis=0) for a in (xi, rp, rt, zz)]
    num_pairs = nb[rows].sum(axis=0).astype(np.int64)
    for healpix in healpixs:
        for delta in data[healpix]:
            delta.neighbours = None
    xi_n, rp_n, rt_n, z_n = _pairs.normalise(weights, *sums)
    return weights, xi_n, rp_n, rt_n, z_n, num_pairs


def compute_xi_forest_pairs_fast(z1, r_comov1, dist_m1, weights1, delta1, z2, r_comov2, dist_m2,
                                 weights2, ang, rebin_weight, rebin_xi, rebin_r_par,
                                 rebin_r_trans, rebin_z, rebin_num_pairs):
    """One forest against quasar arrays (z2, r_comov2, dist_m2, weights2,
    ang), accumulated in place (py/picca/xcf.py:223-322 signature)."""
    import torch  # pylint: disable=import-outside-toplevel

    n = len(z1)
    m = len(z2)
    fs = ForestSet(
        pix_offset=np.array([0, n], dtype=np.int64), z=np.asarray(z1, float),
        r_comov=np.asarray(r_comov1, float), dist_m=np.asarray(dist_m1, float),
        weights=np.asarray(weights1, float), delta=np.asarray(delta1, float),
        log_lambda=np.zeros(n), ra=np.zeros(1), dec=np.zeros(1), x_cart=np.ones(1),
        y_cart=np.zeros(1), z_cart=np.zeros(1), cos_dec=np.ones(1), z_qso=np.zeros(1),
        thingid=np.array([-1]), healpix=np.zeros(1, dtype=np.int64))
    qs = ForestSet(
        ra=np.zeros(m), dec=np.zeros(m), x_cart=np.ones(m), y_cart=np.zeros(m),
        z_cart=np.zeros(m), cos_dec=np.ones(m), z_qso=np.asarray(z2, float),
        obj_r_comov=np.asarray(r_comov2, float), obj_dist_m=np.asarray(dist_m2, float),
        obj_weight=np.asarray(weights2, float), thingid=np.arange(m, dtype=np.int64),
        healpix=np.zeros(m, dtype=np.int64))
    engine = _engine()
    dev1 = _pairs.DeviceForests(fs, engine.device)
    dev2 = _pairs.DeviceForests(qs, engine.device)
    dev = engine.device
    offsets = torch.tensor([0, m], dtype=torch.int64, device=dev)
    index = torch.arange(max(m, 1), dtype=torch.int32, device=dev)
    angles = torch.tensor(np.asarray(ang, dtype=float).reshape(-1) if m else [0.0],
                          dtype=torch.float64, device=dev)
    order = torch.zeros(1, dtype=torch.int32, device=dev)
    nbins = len(rebin_weight)
    rows = engine.alloc_rows(1, nbins)
    if m:
        engine.accumulate(_params(np.pi), dev1, dev2, offsets, index, order, 1, rows, _mode(),
                          xcf=True, angles=angles)
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
        raise ValueError("xcf.num_model_bins_r_par / num_model_bins_r_trans must be set "
                         "before computing a distortion matrix")
    return _dmat.make_dmat_params(
        num_bins_r_par, num_bins_r_trans,
        redshift_evolution=redshift_evolution_in_distortion_matrix,
        z_ref=2.25 if z_ref is None else z_ref, alpha=2.9 if alpha is None else alpha,
        alpha2=1.44 if alpha_obj is None else alpha_obj,
        num_model_bins_r_par=num_model_bins_r_par,
        num_model_bins_r_trans=num_model_bins_r_trans, product=dmat_product)


def _dmat_engine():
    if _cache["dmat_engine"] is None:
        _cache["dmat_engine"] = _dmat.XDmatEngine(_engine())
    return _cache["dmat_engine"]


def _neighbour_state():
    """Device forests, quasars and the quasar-neighbour CSR, cached."""
    key = _state_key()
    if _cache["nbr_key"] == key and _cache["nbr"] is not None:
        return _cache["nbr"]
    if data is None or objs is None:
        raise ValueError("xcf.data and xcf.objs must be set")
    if ang_correlation:
        raise ValueError("the distortion matrix has no angular form")
    engine = _engine()
    fs = ForestSet.from_deltas(data)
    qs = ForestSet.from_objects(objs)
    dev1 = _pairs.DeviceForests(fs, engine.device)
    dev2 = _pairs.DeviceForests(qs, engine.device)
    offsets, index, total = engine.neighbours(_params(), dev1, dev2, xcf=True)
    state = {"set1": fs, "set2": qs, "dev1": dev1, "dev2": dev2,
             "offsets": offsets.cpu().numpy(), "index": index.cpu().numpy()[:total],
             "total": total}
    _cache["nbr_key"] = key
    _cache["nbr"] = state
    return state


def _dmat_sums(state, mask):
    engine = _dmat_engine()
    items = _dmat.xcf_items(state["offsets"], state["index"], mask, state["dev1"].npix)
    if len(items[0]):
        _dmat.check_orders(state["set1"], np.unique(items[0]))
    ditems = engine.device_items(*items)
    side = _dmat.DmatEngine.side_arrays(state["dev1"], engine.device)
    params, dparams = _params(), _dmat_params()
    sums = engine.alloc_sums(params, dparams)
    engine.xaccumulate(params, dparams, state["dev1"], state["dev2"], side, ditems, sums)
    engine.engine.stats()
    return {k: v.cpu().numpy() for k, v in sums.items()}


def compute_dmat(healpixs):
    """Raw cross distortion-matrix sums of ``healpixs``
    (py/picca/xcf.py:325-424): ``np.random.rand(len(neighbours)) > reject``
    from NumPy's global generator for every delta, forests without a kept
    quasar skipped before counting; the kept pairs run on the GPU. Returns
    ``(weights_dmat, dmat [nb, nm], r_par_eff, r_trans_eff, z_eff,
    weight_eff, num_pairs, num_pairs_used)``."""
    state = _neighbour_state()
    fs = state["set1"]
    offsets = state["offsets"]
    firsts = np.searchsorted(fs.row, np.arange(len(fs.healpix_list)))
    mask = np.zeros(int(state["total"]), dtype=bool)
    num_pairs = 0
    num_pairs_used = 0
    for healpix in healpixs:
        row = int(np.searchsorted(fs.healpix_list, healpix))
        for k, delta in enumerate(data[healpix]):
            if getattr(delta, "order", None) is None:
                raise RuntimeError("Trying to compute the distortion matrix but order is not "
                                   "defined for the deltas. Check previous warning to solve "
                                   "this issue")
            f = firsts[row] + k
            start, end = int(offsets[f]), int(offsets[f + 1])
            w = np.random.rand(end - start) > reject
            if w.sum() == 0:
                continue
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
    """The whole picca_xdmat.py computation for ``nproc`` processes (random
    rejection per chunk of healpix) in one GPU pass; normalised columns
    (WDM, DM, RP, RT, Z) and NPALL / NPUSED."""
    state = _neighbour_state()
    fs = state["set1"]
    _dmat.check_orders(fs, np.arange(fs.num))
    mask = _dmat.selection_mask(fs.healpix_list, fs.row, state["offsets"], nproc, reject)
    npall, npused = _dmat.xcf_counts(state["offsets"], mask)
    raw = _dmat_sums(state, mask)
    result = _dmat.normalise(raw, _params(), _dmat_params(), npall, npused)
    result["raw"] = raw
    return result


def compute_dmat_forest_pairs_fast(log_lambda1, r_comov1, dist_m1, z1, weights1, r_comov2,
                                   dist_m2, z2, weights2, ang, weights_dmat, dmat, r_par_eff,
                                   r_trans_eff, z_eff, weight_eff, order1):
    """One forest against quasar arrays, accumulated in place
    (py/picca/xcf.py:427-445 signature)."""
    import torch  # pylint: disable=import-outside-toplevel

    n = len(z1)
    m = len(z2)
    if m == 0:
        return
    fs = ForestSet(
        pix_offset=np.array([0, n], dtype=np.int64), z=np.asarray(z1, float),
        r_comov=np.asarray(r_comov1, float), dist_m=np.asarray(dist_m1, float),
        weights=np.asarray(weights1, float), delta=np.zeros(n),
        log_lambda=np.asarray(log_lambda1, float), ra=np.zeros(1), dec=np.zeros(1),
        x_cart=np.ones(1), y_cart=np.zeros(1), z_cart=np.zeros(1), cos_dec=np.ones(1),
        z_qso=np.zeros(1), thingid=np.array([-1]), order=np.array([int(order1)]),
        healpix=np.zeros(1, dtype=np.int64))
    qs = ForestSet(
        ra=np.zeros(m), dec=np.zeros(m), x_cart=np.ones(m), y_cart=np.zeros(m),
        z_cart=np.zeros(m), cos_dec=np.ones(m), z_qso=np.asarray(z2, float),
        obj_r_comov=np.asarray(r_comov2, float), obj_dist_m=np.asarray(dist_m2, float),
        obj_weight=np.asarray(weights2, float), thingid=np.arange(m, dtype=np.int64),
        healpix=np.zeros(m, dtype=np.int64))
    engine = _dmat_engine()
    dev = engine.device
    dev1 = _pairs.DeviceForests(fs, dev)
    dev2 = _pairs.DeviceForests(qs, dev)
    params, dparams = _params(np.pi), _dmat_params()
    side = _dmat.DmatEngine.side_arrays(dev1, dev)
    nitem = (m + _dmat._native.PG_XDMAT_MAX_OBJECTS - 1) // _dmat._native.PG_XDMAT_MAX_OBJECTS
    starts = np.arange(nitem) * _dmat._native.PG_XDMAT_MAX_OBJECTS
    counts = np.minimum(m - starts, _dmat._native.PG_XDMAT_MAX_OBJECTS)
    ditems = engine.device_items(np.zeros(nitem), starts, counts, np.arange(m))
    angles = torch.tensor(np.asarray(ang, dtype=float).reshape(-1), dtype=torch.float64,
                          device=dev)
    sums = engine.alloc_sums(params, dparams)
    engine.xaccumulate(params, dparams, dev1, dev2, side, ditems, sums, angles=angles)
    engine.engine.stats()
    weights_dmat += sums["weights_dmat"].cpu().numpy()
    dmat += sums["dmat"].cpu().numpy().reshape(np.shape(dmat))
    r_par_eff += sums["r_par_eff"].cpu().numpy()
    r_trans_eff += sums["r_trans_eff"].cpu().numpy()
    z_eff += sums["z_eff"].cpu().numpy()
    weight_eff += sums["weight_eff"].cpu().numpy()


def compute_metal_dmat(healpixs, abs_igm="SiII(1526)"):
    """Raw delta x quasar metal distortion-matrix sums of ``healpixs``
    (py/picca/xcf.py:677-800): a forest without a pixel below its quasar
    redshift as ``abs_igm`` is skipped before its draw; the others draw
    ``np.random.rand(len(neighbours)) > reject`` from NumPy's global
    generator; the kept pairs run on the GPU. Module globals ``cosmo``,
    ``alpha_abs`` and ``z_ref`` as picca_metal_xdmat.py sets them."""
    import torch  # pylint: disable=import-outside-toplevel

    from . import metal as _metal  # pylint: disable=import-outside-toplevel
    if cosmo is None or alpha_abs is None:
        raise ValueError("xcf.cosmo and xcf.alpha_abs must be set for the metal distortion "
                         "matrix")
    state = _neighbour_state()
    fs, qs = state["set1"], state["set2"]
    offsets = state["offsets"]
    skip = _metal.forests_without_pixels(fs, abs_igm)
    firsts = np.searchsorted(fs.row, np.arange(len(fs.healpix_list)))
    mask = np.zeros(int(state["total"]), dtype=bool)
    num_pairs = num_pairs_used = 0
    for healpix in healpixs:
        row = int(np.searchsorted(fs.healpix_list, healpix))
        for k, _ in enumerate(data[healpix]):
            f = firsts[row] + k
            if skip[f]:
                continue
            start, end = int(offsets[f]), int(offsets[f + 1])
            w = np.random.rand(end - start) > reject
            num_pairs += end - start
            num_pairs_used += int(w.sum())
            mask[start:end] = w
    if _cache.get("metal_engine") is None:
        _cache["metal_engine"] = _metal.MetalEngine(_engine())
    engine = _cache["metal_engine"]
    dev = state["dev1"]
    dev_q = _pairs.DeviceForests(_metal.quasar_pixel_set(qs), engine.device)
    off_d = torch.from_numpy(offsets).to(engine.device)
    idx_d = torch.from_numpy(np.asarray(state["index"], dtype=np.int32)
                             if state["total"] else np.zeros(1, np.int32)).to(engine.device)
    first, second, num = engine.pair_list(dev, dev_q, off_d, idx_d, mask)
    params = _params()
    dparams = _dmat.make_dmat_params(num_bins_r_par, num_bins_r_trans,
                                     num_model_bins_r_par=num_model_bins_r_par,
                                     num_model_bins_r_trans=num_model_bins_r_trans)
    zr = 2.25 if z_ref is None else z_ref
    side = _metal.absorber_pixels(dev, cosmo, abs_igm, alpha_abs[abs_igm], z_ref=zr)
    sums = engine.alloc_sums(params, dparams)
    engine.run_pass(params, dparams, 1.0, dev, dev_q, side, _metal.quasar_side(dev_q), first,
                    second, num, sums, cross=True)
    engine.engine.stats()
    raw = {k: v.cpu().numpy() for k, v in sums.items()}
    for healpix in healpixs:
        for delta in data[healpix]:
            if hasattr(delta, "neighbours"):
                delta.neighbours = None
    nb = num_bins_r_par * num_bins_r_trans
    return (raw["weights_dmat"], raw["dmat"].reshape(nb, -1), raw["r_par_eff"],
            raw["r_trans_eff"], raw["z_eff"], raw["weight_eff"], num_pairs, num_pairs_used)
