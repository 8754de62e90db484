"""Distortion matrix of the auto-correlation on the GPU.

Host side of ``pg_cf_dmat``: the random rejection of forest pairs
(``cf.compute_dmat``, py/picca/cf.py:390-517, driven by ``calc_dmat`` of
py/picca/bin/picca_dmat.py:21-38 and :466-485), the list of selected forest
pairs ordered by cost, the device buffers of the raw sums and the
normalisation of py/picca/bin/picca_dmat.py:487-525.

Selection. picca_dmat.py deals the sorted healpix to ``nproc`` chunks
(index % nproc), seeds NumPy's legacy generator with the first healpix of
each chunk and draws ``rand(len(neighbours)) > reject`` for every forest of
the chunk, healpix by healpix, in the order of ``data[healpix]``. Neighbour
lists are in the order of ``cf.fill_neighs`` (healpix ascending, then read
order), which is the index order of a ForestSet. Because consecutive
``rand(n)`` calls of one generator return the same stream as one call for
the total, the draws of a chunk are made in large blocks and scattered over
the neighbour lists of its forests.
"""

import ctypes

import numpy as np
import torch

from . import _native
from ._native import DmatParamsC, DmatSumsC, check
from . import pairs as _pairs

_DRAW_BLOCK = 1 << 24


def make_dmat_params(num_bins_r_par, num_bins_r_trans, coef_binning_model=1,
                     redshift_evolution=True, z_ref=2.25, alpha=2.9, alpha2=2.9,
                     num_model_bins_r_par=None, num_model_bins_r_trans=None, row_capacity=0,
                     product="split_bf16"):
    """pg_dmat_params. The model bins default to coef_binning_model times the
    data bins (py/picca/bin/picca_dmat.py:366-369); row_capacity 0 keeps the
    library's default chunking of a forest pair's bins; ``product`` selects
    the arithmetic of the eta products: "split_bf16" (tensor cores, exact
    digit products) or "fp64"."""
    products = {"fp64": _native.PG_DMAT_FP64, "split_bf16": _native.PG_DMAT_SPLIT_BF16}
    if product not in products:
        raise ValueError(f"unknown product {product!r}")
    nmp = num_model_bins_r_par or int(num_bins_r_par * coef_binning_model)
    nmt = num_model_bins_r_trans or int(num_bins_r_trans * coef_binning_model)
    return DmatParamsC(int(nmp), int(nmt), int(bool(redshift_evolution)), int(row_capacity),
                       products[product], 0, float(z_ref), float(alpha), float(alpha2))


def _ranges(starts, ends):
    """Concatenation of [starts[k], ends[k]) as one int64 index array."""
    lengths = ends - starts
    total = int(lengths.sum())
    if total == 0:
        return np.zeros(0, dtype=np.int64)
    first = np.repeat(starts - np.concatenate([[0], np.cumsum(lengths)[:-1]]), lengths)
    return first + np.arange(total, dtype=np.int64)


def chunk_rows(num_rows, nproc):
    """Rows (ranks of the sorted healpix) of each process chunk, in the order
    picca_dmat.py maps them (py/picca/bin/picca_dmat.py:472-485)."""
    return [np.arange(p, num_rows, nproc) for p in range(min(nproc, num_rows))]


def selection_mask(healpix_list, forest_rows, nbr_offsets, nproc, reject, skip=None):
    """Boolean mask over the neighbour CSR of the pairs picca_dmat.py keeps
    when run with ``nproc`` processes. ``forest_rows`` must be
    non-decreasing (forests grouped by healpix, as ForestSet stores them).
    Forests flagged in ``skip`` draw nothing (xcf.compute_metal_dmat skips
    forests without a usable pixel before drawing)."""
    forest_rows = np.asarray(forest_rows)
    offsets = np.asarray(nbr_offsets, dtype=np.int64)
    if forest_rows.size and np.any(np.diff(forest_rows) < 0):
        raise ValueError("forests must be grouped by healpix in ascending order")
    num_rows = len(healpix_list)
    row_ids = np.arange(num_rows)
    first = np.searchsorted(forest_rows, row_ids, side="left")
    last = np.searchsorted(forest_rows, row_ids, side="right")
    mask = np.zeros(int(offsets[-1]) if offsets.size else 0, dtype=bool)
    for rows in chunk_rows(num_rows, max(int(nproc), 1)):
        rng = np.random.RandomState(int(healpix_list[rows[0]]))
        if skip is None:
            positions = _ranges(offsets[first[rows]], offsets[last[rows]])
        else:
            forests = np.concatenate([np.arange(first[r], last[r]) for r in rows])
            forests = forests[~np.asarray(skip)[forests]]
            positions = _ranges(offsets[forests], offsets[forests + 1])
        for k in range(0, len(positions), _DRAW_BLOCK):
            part = positions[k:k + _DRAW_BLOCK]
            mask[part] = rng.rand(len(part)) > reject
    return mask


class DmatEngine:
    """Distortion-matrix sums on one CUDA device (a PairEngine's plan)."""

    def __init__(self, engine=None, device=None):
        self.engine = engine or _pairs.PairEngine(device)
        self.device = self.engine.device
        self._work = None

    def work_buffer(self, params, dparams, max_pixels1, max_pixels2, num_pairs=0):
        """Device work buffer for the kernel (grown, never shrunk); at most
        one slice per forest pair."""
        nbytes = ctypes.c_uint64()
        with torch.cuda.device(self.device):
            check(_native.lib().pg_cf_dmat_work_bytes(
                self.engine.plan.handle, ctypes.byref(params), ctypes.byref(dparams),
                int(max_pixels1), int(max_pixels2), int(num_pairs), ctypes.byref(nbytes)),
                "dmat work size")
        need = int(nbytes.value)
        if self._work is None or self._work.numel() < need:
            self._work = torch.empty(max(need, 16), dtype=torch.uint8, device=self.device)
        return self._work

    def alloc_sums(self, params, dparams):
        nb = params.num_bins_r_par * params.num_bins_r_trans
        nm = dparams.num_model_bins_r_par * dparams.num_model_bins_r_trans
        dev = self.device
        return {"weights_dmat": torch.zeros(nb, dtype=torch.float64, device=dev),
                "dmat": torch.zeros(nb * nm, dtype=torch.float64, device=dev),
                "r_par_eff": torch.zeros(nm, dtype=torch.float64, device=dev),
                "r_trans_eff": torch.zeros(nm, dtype=torch.float64, device=dev),
                "z_eff": torch.zeros(nm, dtype=torch.float64, device=dev),
                "weight_eff": torch.zeros(nm, dtype=torch.float64, device=dev)}

    @staticmethod
    def side_arrays(dev_forests, device):
        """Device log_lambda (compacted like the set) and per-forest order."""
        fs = dev_forests.source
        ll = np.asarray(fs.log_lambda, dtype=np.float64)
        if fs.num_pixels:
            ll = ll[np.asarray(fs.weights) != 0]
        if ll.size == 0:
            ll = np.zeros(1)
        order = np.asarray(fs.order, dtype=np.int32)
        if order.size == 0:
            order = np.zeros(1, dtype=np.int32)
        return (torch.from_numpy(np.ascontiguousarray(ll)).to(device),
                torch.from_numpy(np.ascontiguousarray(order)).to(device))

    def pair_list(self, dev1, dev2, offsets, index, mask):
        """Selected (first, second) forest pairs on the device, longest first."""
        dev = self.device
        total = int(mask.size)
        if total == 0 or not mask.any():
            z = torch.zeros(1, dtype=torch.int32, device=dev)
            return z, z, 0
        mask_d = torch.from_numpy(mask).to(dev)
        k = torch.nonzero(mask_d[:total]).flatten()
        first = torch.searchsorted(offsets, k, right=True) - 1
        second = index[:total][k].long()
        other = dev2 if dev2 is not None else dev1
        npix1 = torch.from_numpy(dev1.npix).to(dev)
        npix2 = torch.from_numpy(other.npix).to(dev)
        cost = npix1[first] * npix2[second]
        order = torch.argsort(cost, descending=True, stable=True)
        return (first[order].to(torch.int32).contiguous(),
                second[order].to(torch.int32).contiguous(), int(k.numel()))

    def accumulate(self, params, dparams, dev1, dev2, side1, side2, first, second, num_pairs,
                   sums, angles=None):
        """Launch pg_cf_dmat (asynchronous on the current stream)."""
        other = dev2 if dev2 is not None else dev1
        work = self.work_buffer(params, dparams, dev1.max_pixels, other.max_pixels,
                                max(int(num_pairs), 1))
        out = DmatSumsC(*[sums[k].data_ptr() for k in ("weights_dmat", "dmat", "r_par_eff",
                                                         "r_trans_eff", "z_eff", "weight_eff")])
        s2 = ctypes.byref(dev2.c) if dev2 is not None else None
        ll2 = side2[0].data_ptr() if side2 is not None else None
        or2 = side2[1].data_ptr() if side2 is not None else None
        with torch.cuda.device(self.device):
            check(_native.lib().pg_cf_dmat(
                self.engine.plan.handle, ctypes.byref(params), ctypes.byref(dparams),
                ctypes.byref(dev1.c), s2, side1[0].data_ptr(), ll2, side1[1].data_ptr(), or2,
                first.data_ptr(), second.data_ptr(),
                angles.data_ptr() if angles is not None else None, int(num_pairs),
                work.data_ptr(), int(work.numel()), ctypes.byref(out),
                self.engine._stream()), "distortion matrix")
        return sums


def normalise(raw, params, dparams, num_pairs, num_pairs_used):
    """py/picca/bin/picca_dmat.py:487-525 on host arrays. Returns a dict of
    the FITS columns (WDM, DM, RP, RT, Z) and the pair counts."""
    nb = params.num_bins_r_par * params.num_bins_r_trans
    weights = raw["weight_eff"].copy()
    r_par, r_trans, zeff = raw["r_par_eff"].copy(), raw["r_trans_eff"].copy(), raw["z_eff"].copy()
    w = weights > 0.0
    r_par[w] /= weights[w]
    r_trans[w] /= weights[w]
    zeff[w] /= weights[w]
    mean_zeff = np.mean(zeff[w]) if w.any() else float("nan")
    weights_dmat = raw["weights_dmat"].copy()
    dmat = raw["dmat"].reshape(nb, -1).copy()
    w = weights_dmat > 0
    dmat[w] /= weights_dmat[w, None]
    if dparams.redshift_evolution:
        zeff[:] = mean_zeff
        zfac = ((1 + dparams.z_ref) / (1 + mean_zeff)) ** ((dparams.alpha - 1) +
                                                            (dparams.alpha2 - 1))
        dmat *= zfac
    return {"WDM": weights_dmat, "DM": dmat, "RP": r_par, "RT": r_trans, "Z": zeff,
            "NPALL": int(num_pairs), "NPUSED": int(num_pairs_used)}


def check_orders(fs, forests):
    """cf.compute_dmat refuses deltas without a polynomial order
    (py/picca/cf.py:430-436 and :467-472)."""
    if len(forests) and np.any(np.asarray(fs.order)[forests] < 0):
        raise RuntimeError("Trying to compute the distortion matrix but order is not defined "
                           "for the deltas. Check previous warning to solve this issue")


def distortion_matrix(fs1, fs2, params, dparams, reject, nproc=1, engine=None, mask=None):
    """picca_dmat.py on ForestSets: neighbours, the selection of ``nproc``
    chunks (or a given mask over the neighbour CSR), the GPU sums and the
    normalisation. Returns the normalised columns, the raw sums (host) and
    run statistics."""
    dm = engine if isinstance(engine, DmatEngine) else DmatEngine(engine)
    pe = dm.engine
    dev1 = _pairs.DeviceForests(fs1, pe.device)
    dev2 = _pairs.DeviceForests(fs2, pe.device) if fs2 is not None else None
    offsets, index, total = pe.neighbours(params, dev1, dev2)
    offsets_h = offsets.cpu().numpy()
    if mask is None:
        mask = selection_mask(fs1.healpix_list, fs1.row, offsets_h, nproc, reject)
    first, second, num_sel = dm.pair_list(dev1, dev2, offsets, index, mask)
    if num_sel:
        used = np.unique(first.cpu().numpy())
        check_orders(fs1, used)
        check_orders(fs2 if fs2 is not None else fs1, np.unique(second.cpu().numpy()))
    side1 = DmatEngine.side_arrays(dev1, pe.device)
    side2 = DmatEngine.side_arrays(dev2, pe.device) if dev2 is not None else None
    sums = dm.alloc_sums(params, dparams)
    dm.accumulate(params, dparams, dev1, dev2, side1, side2, first, second, num_sel, sums)
    stats = pe.stats()
    raw = {k: v.cpu().numpy() for k, v in sums.items()}
    result = normalise(raw, params, dparams, total, int(mask.sum()))
    result["raw"] = raw
    result["forest_pairs_used"] = num_sel
    result["work_items"] = int(stats.work_items)
    return result


# ---------------------------------------------------------------------------
# Delta x quasar distortion matrix: xcf.compute_dmat (py/picca/xcf.py:325-424)
# and picca_xdmat.py (py/picca/bin/picca_xdmat.py).

def xcf_counts(nbr_offsets, mask):
    """NPALL and NPUSED as xcf.compute_dmat counts them: a forest without a
    kept quasar is skipped before its neighbours are counted
    (py/picca/xcf.py:382-386)."""
    offsets = np.asarray(nbr_offsets, dtype=np.int64)
    csum = np.concatenate([[0], np.cumsum(mask, dtype=np.int64)])
    kept = csum[offsets[1:]] - csum[offsets[:-1]]
    counts = offsets[1:] - offsets[:-1]
    return int(counts[kept > 0].sum()), int(kept.sum())


def xcf_items(nbr_offsets, nbr_index, mask, npix, max_objects=_native.PG_XDMAT_MAX_OBJECTS):
    """Work items of pg_xcf_dmat from the kept neighbours: (item_forest,
    item_start, item_count, obj_index) with each forest's kept quasars in
    chunks of at most max_objects, the costliest items first."""
    offsets = np.asarray(nbr_offsets, dtype=np.int64)
    kept = np.nonzero(mask)[0]
    obj_index = np.asarray(nbr_index, dtype=np.int32)[kept]
    forest = np.searchsorted(offsets, kept, side="right") - 1
    if kept.size == 0:
        z = np.zeros(0, dtype=np.int32)
        return z, z, z, obj_index
    starts = np.flatnonzero(np.r_[True, forest[1:] != forest[:-1]])
    ends = np.r_[starts[1:], kept.size]
    item_forest, item_start, item_count = [], [], []
    for s0, s1 in zip(starts, ends):
        for a in range(s0, s1, max_objects):
            item_forest.append(forest[s0])
            item_start.append(a)
            item_count.append(min(max_objects, s1 - a))
    item_forest = np.asarray(item_forest, dtype=np.int32)
    item_start = np.asarray(item_start, dtype=np.int32)
    item_count = np.asarray(item_count, dtype=np.int32)
    cost = np.asarray(npix)[item_forest] * item_count
    order = np.argsort(-cost, kind="stable")
    return item_forest[order], item_start[order], item_count[order], obj_index


class XDmatEngine(DmatEngine):
    """Cross (delta x quasar) distortion-matrix sums on one CUDA device."""

    def xwork_buffer(self, params, dparams, max_pixels, num_items):
        nbytes = ctypes.c_uint64()
        with torch.cuda.device(self.device):
            check(_native.lib().pg_xcf_dmat_work_bytes(
                self.engine.plan.handle, ctypes.byref(params), ctypes.byref(dparams),
                int(max_pixels), int(num_items), ctypes.byref(nbytes)), "xdmat work size")
        need = int(nbytes.value)
        if self._work is None or self._work.numel() < need:
            self._work = torch.empty(max(need, 16), dtype=torch.uint8, device=self.device)
        return self._work

    def xaccumulate(self, params, dparams, dev_forests, dev_objs, side, items, sums,
                    angles=None):
        """Launch pg_xcf_dmat; items = device int32 tensors (forest, start,
        count, obj_index) and their number."""
        item_forest, item_start, item_count, obj_index, num_items = items
        work = self.xwork_buffer(params, dparams, dev_forests.max_pixels, max(num_items, 1))
        out = DmatSumsC(*[sums[k].data_ptr() for k in ("weights_dmat", "dmat", "r_par_eff",
                                                         "r_trans_eff", "z_eff", "weight_eff")])
        with torch.cuda.device(self.device):
            check(_native.lib().pg_xcf_dmat(
                self.engine.plan.handle, ctypes.byref(params), ctypes.byref(dparams),
                ctypes.byref(dev_forests.c), ctypes.byref(dev_objs.c), side[0].data_ptr(),
                side[1].data_ptr(), item_forest.data_ptr(), item_start.data_ptr(),
                item_count.data_ptr(), obj_index.data_ptr(),
                angles.data_ptr() if angles is not None else None, int(num_items),
                work.data_ptr(), int(work.numel()), ctypes.byref(out),
                self.engine._stream()), "cross distortion matrix")
        return sums

    def device_items(self, item_forest, item_start, item_count, obj_index):
        dev = self.device

        def up(a):
            a = np.asarray(a, dtype=np.int32)
            return torch.from_numpy(a if a.size else np.zeros(1, dtype=np.int32)).to(dev)
        return (up(item_forest), up(item_start), up(item_count), up(obj_index),
                int(len(item_forest)))


def cross_distortion_matrix(fs, qs, params, dparams, reject, nproc=1, engine=None, mask=None):
    """picca_xdmat.py on a forest set and a quasar set: neighbours, the
    random rejection of ``nproc`` chunks, the GPU sums and the
    normalisation. Returns the normalised columns, the raw sums (host) and
    run statistics."""
    dm = engine if isinstance(engine, XDmatEngine) else XDmatEngine(engine)
    pe = dm.engine
    dev1 = _pairs.DeviceForests(fs, pe.device)
    dev2 = _pairs.DeviceForests(qs, pe.device)
    offsets, index, total = pe.neighbours(params, dev1, dev2, xcf=True)
    offsets_h = offsets.cpu().numpy()
    index_h = index.cpu().numpy()[:total]
    if mask is None:
        mask = selection_mask(fs.healpix_list, fs.row, offsets_h, nproc, reject)
    npall, npused = xcf_counts(offsets_h, mask)
    items = xcf_items(offsets_h, index_h, mask, dev1.npix)
    if len(items[0]):
        check_orders(fs, np.unique(items[0]))
    ditems = dm.device_items(*items)
    side = DmatEngine.side_arrays(dev1, pe.device)
    sums = dm.alloc_sums(params, dparams)
    dm.xaccumulate(params, dparams, dev1, dev2, side, ditems, sums)
    stats = pe.stats()
    raw = {k: v.cpu().numpy() for k, v in sums.items()}
    result = normalise(raw, params, dparams, npall, npused)
    result["raw"] = raw
    result["work_items"] = int(stats.work_items)
    result["items"] = int(ditems[4])
    result["pixel_object_pairs"] = float(np.sum(dev1.npix[items[0]].astype(np.float64) *
                                                items[2]))
    return result
