"""Wick covariance of the auto-correlation on the GPU: cf.compute_wick_terms
with cf.compute_wickT123_pairs (py/picca/cf.py:1328-1626) and picca_wick.py
(py/picca/bin/picca_wick.py:392-540).

Host side of ``pg_wick_xi_matrices`` / ``pg_cf_wick``: the 1D variance and
1D correlation of the pixels of one forest from a picca_cf1d.py table
(nearest tabulated point, as scipy's interp1d in the reference), the random
draw per forest, the forest pairs (every neighbour of a kept forest), the
per-pixel redshift-evolution factors, and the normalisation. The weighted 1D
correlation matrix of each forest in a pair is built once on the device; the
O(K^2) sum over pairs of pixel pairs runs in ``csrc/pg_wick.cu``.

Diagrams 4 and 5 (picca_wick.py --max-diagram > 3) and the two-field form
(--in-dir2 / --lambda-abs2) are not provided: the reference's own code for
them does not run (compute_wickT45_pairs indexes the 1-3 pixel pairs with
the 1-2 bins, and the second field's relabelling loop renames the first
field), and picca_wick.py's default is --max-diagram 3, where T4-T6 are 0.
"""

import ctypes

import numpy as np
import torch

from . import _native
from . import pairs as _pairs
from ._native import check

_P = ctypes.POINTER


SUM_KEYS = ("weights_wick", "num_pairs_wick", "t1", "t2", "t3", "t4")


class WickSumsC(ctypes.Structure):
    _fields_ = [(k, ctypes.c_void_p) for k in SUM_KEYS]


def _bind():
    lib = _native.lib()
    if not getattr(lib, "_wick_bound", False):
        vp, i64, i32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32
        lib.pg_wick_xi_matrices.restype = ctypes.c_int
        lib.pg_wick_xi_matrices.argtypes = [vp, _P(_native.ForestSetC), vp, vp, vp, vp, i32, vp,
                                            i64, vp, vp, vp]
        lib.pg_cf_wick_work_bytes.restype = ctypes.c_int
        lib.pg_cf_wick_work_bytes.argtypes = [vp, _P(_native.CorrParams), i32, i32, i64,
                                              _P(ctypes.c_uint64)]
        lib.pg_cf_wick.restype = ctypes.c_int
        lib.pg_cf_wick.argtypes = [vp, _P(_native.CorrParams), _P(_native.ForestSetC),
                                   _P(_native.ForestSetC), vp, vp, vp, vp, vp, vp, vp, vp, vp,
                                   vp, vp, i64, vp, ctypes.c_uint64, _P(WickSumsC), vp]
        lib.pg_xcf_wick_work_bytes.restype = ctypes.c_int
        lib.pg_xcf_wick_work_bytes.argtypes = lib.pg_cf_wick_work_bytes.argtypes
        lib.pg_xcf_wick.restype = ctypes.c_int
        lib.pg_xcf_wick.argtypes = [vp, _P(_native.CorrParams), _P(_native.ForestSetC),
                                    _P(_native.ForestSetC), vp, vp, vp, vp, vp, vp, vp, vp, vp,
                                    vp, vp, i64, i32, vp, ctypes.c_uint64, _P(WickSumsC), vp]
        lib.pg_xcf_wick_factored_work_bytes.restype = ctypes.c_int
        lib.pg_xcf_wick_factored_work_bytes.argtypes = [vp, _P(_native.CorrParams), i32, i32,
                                                        _P(ctypes.c_uint64)]
        lib.pg_xcf_wick_factored.restype = ctypes.c_int
        lib.pg_xcf_wick_factored.argtypes = [vp, _P(_native.CorrParams), _P(_native.ForestSetC),
                                             _P(_native.ForestSetC), vp, vp, vp, vp, vp, vp, vp,
                                             vp, vp, i64, i32, vp, ctypes.c_uint64,
                                             _P(WickSumsC), vp]
        lib._wick_bound = True
    return lib


def read_cf1d(path):
    """HDU 1 of a picca_cf1d.py file: LLMIN, DLL and the v1d / nv1d / c1d /
    nb1d columns (py/picca/bin/picca_wick.py:392-421)."""
    from . import fitsio_lite
    hdu = fitsio_lite.FITS(path)[1]
    header = hdu.read_header()
    out = {k: np.asarray(hdu[k][:]) for k in ("v1d", "nv1d", "c1d", "nb1d")}
    out["LLMIN"], out["DLL"] = float(header["LLMIN"]), float(header["DLL"])
    return out


class OneDTables:
    """The reference's nearest-point interpolants of a picca_cf1d.py table:
    the variance at a pixel's log_lambda (evaluated here on the host), and
    the 1D correlation at |dlog_lambda| as cell bounds and values for the
    device (scipy interp1d kind="nearest": the value of the point whose
    cell, bounded by the midpoints x[k] / 2 + x[k + 1] / 2, holds the
    argument; ties go to the lower point; beyond the ends, the end points)."""

    def __init__(self, cf1d):
        log_lambda = cf1d["LLMIN"] + cf1d["DLL"] * np.arange(len(cf1d["v1d"]))
        kv = np.asarray(cf1d["nv1d"]) > 0
        self.var_x = log_lambda[kv]
        self.var_y = np.asarray(cf1d["v1d"], dtype=np.float64)[kv]
        kx = np.asarray(cf1d["nb1d"]) > 0
        self.xi_x = (log_lambda - cf1d["LLMIN"])[kx]
        self.xi_y = np.ascontiguousarray(np.asarray(cf1d["c1d"], dtype=np.float64)[kx])
        if self.var_x.size == 0 or self.xi_x.size == 0:
            raise ValueError("empty 1D correlation table")
        self.xi_bounds = np.ascontiguousarray(self._bounds(self.xi_x))
        self.var_bounds = self._bounds(self.var_x)

    @staticmethod
    def _bounds(x):
        half = x / 2.0
        return half[1:] + half[:-1]

    def variance(self, log_lambda):
        idx = np.searchsorted(self.var_bounds, log_lambda, side="left")
        return self.var_y[np.clip(idx, 0, self.var_y.size - 1)]


def selection(fs, nproc, reject):
    """Kept forests of cf.compute_wick_terms (py/picca/cf.py:1376-1380 with
    picca_wick.py:20-37, 498-512): healpix rows dealt to nproc chunks, the
    generator seeded with the chunk's first healpix, one rand(len(forests))
    draw per healpix. Returns (keep, npall, npused)."""
    keep = np.zeros(fs.num, dtype=bool)
    rows = np.asarray(fs.row)
    members = {}
    for f, row in enumerate(rows):
        members.setdefault(int(row), []).append(f)
    chunks = {}
    for index in range(len(fs.healpix_list)):
        chunks.setdefault(index % nproc, []).append(index)
    npall = npused = 0
    for chunk in chunks.values():
        rng = np.random.RandomState(int(fs.healpix_list[chunk[0]]))
        for row in chunk:
            forests = members.get(row, [])
            draw = rng.rand(len(forests)) > reject
            keep[forests] = draw
            npall += len(forests)
            npused += int(draw.sum())
    return keep, npall, npused


class WickEngine:
    """Wick terms T1-T3 on one CUDA device."""

    def __init__(self, engine=None, device=None):
        self.engine = engine or _pairs.PairEngine(device)
        self.device = self.engine.device
        self._work = None

    def _stream(self):
        return self.engine._stream()

    def xi_matrices(self, dev, tables, forests):
        """Arena of the weighted 1D correlation matrices of ``forests``
        (indices into dev's set) and the per-forest offsets into it."""
        lib = _bind()
        fs = dev.source
        npix = np.asarray(dev.npix, dtype=np.int64)
        offsets = np.zeros(max(fs.num, 1), dtype=np.int64)
        forests = np.unique(np.asarray(forests, dtype=np.int64))
        sizes = npix[forests] ** 2
        offsets[forests] = np.concatenate([[0], np.cumsum(sizes)[:-1]]) if forests.size else []
        total = int(sizes.sum()) if forests.size else 0
        ll = np.asarray(fs.log_lambda, dtype=np.float64)
        var = tables.variance(ll) if ll.size else np.zeros(1)
        dvc = self.device
        t = {"ll": torch.from_numpy(np.ascontiguousarray(ll if ll.size else np.zeros(1))).to(dvc),
             "var": torch.from_numpy(np.ascontiguousarray(var)).to(dvc),
             "bounds": torch.from_numpy(tables.xi_bounds if tables.xi_bounds.size
                                        else np.zeros(1)).to(dvc),
             "values": torch.from_numpy(tables.xi_y).to(dvc),
             "forests": torch.from_numpy(forests.astype(np.int32) if forests.size
                                         else np.zeros(1, dtype=np.int32)).to(dvc),
             "offsets": torch.from_numpy(offsets).to(dvc)}
        arena = torch.empty(max(total, 1), dtype=torch.float64, device=dvc)
        with torch.cuda.device(dvc):
            check(lib.pg_wick_xi_matrices(
                self.engine.plan.handle, ctypes.byref(dev.c), t["ll"].data_ptr(),
                t["var"].data_ptr(), t["bounds"].data_ptr(), t["values"].data_ptr(),
                int(tables.xi_y.size), t["forests"].data_ptr(), int(forests.size),
                t["offsets"].data_ptr(), arena.data_ptr(), self._stream()), "Wick xi matrices")
        return arena, t["offsets"], t

    def alloc_sums(self, nb, cross=False):
        dvc = self.device
        out = {"weights_wick": torch.zeros(nb, dtype=torch.float64, device=dvc),
               "num_pairs_wick": torch.zeros(nb, dtype=torch.int64, device=dvc)}
        for key in ("t1", "t2", "t3") + (("t4",) if cross else ()):
            out[key] = torch.zeros(nb * nb, dtype=torch.float64, device=dvc)
        return out

    @staticmethod
    def _sums_struct(sums):
        return WickSumsC(*[sums[k].data_ptr() if k in sums else None for k in SUM_KEYS])

    def work_buffer(self, params, max_pixels1, max_pixels2, num_pairs):
        lib = _bind()
        nbytes = ctypes.c_uint64()
        with torch.cuda.device(self.device):
            check(lib.pg_cf_wick_work_bytes(self.engine.plan.handle, ctypes.byref(params),
                                            int(max_pixels1), int(max_pixels2), int(num_pairs),
                                            ctypes.byref(nbytes)), "Wick work size")
        need = int(nbytes.value)
        if self._work is None or self._work.numel() < need:
            self._work = torch.empty(max(need, 16), dtype=torch.uint8, device=self.device)
        return self._work

    def plan_pairs(self, dev, first, second, num_pairs, angles=None):
        """Work units of pg_cf_wick: the forest pairs, costly ones cut into
        slices (``slice_units``), as device arrays."""
        npix = torch.from_numpy(np.asarray(dev.npix, dtype=np.int64)).to(self.device)
        num_pairs = int(num_pairs)
        cost = (npix[first[:num_pairs].long()] * npix[second[:num_pairs].long()]).cpu().numpy()
        unit, sl, sls = slice_units(cost)
        u = torch.from_numpy(unit).to(self.device)
        return {"first": first[u].contiguous(), "second": second[u].contiguous(),
                "angles": angles[u].contiguous() if angles is not None else None,
                "slice": torch.from_numpy(sl).to(self.device),
                "slices": torch.from_numpy(sls).to(self.device), "num": int(unit.size)}

    def launch_pairs(self, params, dev, zw1, zw2, xo, xa, units, sums):
        """Launch pg_cf_wick on planned units (asynchronous, current stream)."""
        lib = _bind()
        work = self.work_buffer(params, dev.max_pixels, dev.max_pixels, max(units["num"], 1))
        angles = units["angles"]
        with torch.cuda.device(self.device):
            check(lib.pg_cf_wick(
                self.engine.plan.handle, ctypes.byref(params), ctypes.byref(dev.c), None,
                zw1.data_ptr(), zw2.data_ptr(), xo.data_ptr(), xa.data_ptr(), xo.data_ptr(),
                xa.data_ptr(), units["first"].data_ptr(), units["second"].data_ptr(),
                angles.data_ptr() if angles is not None else None, units["slice"].data_ptr(),
                units["slices"].data_ptr(), units["num"], work.data_ptr(), int(work.numel()),
                ctypes.byref(self._sums_struct(sums)), self._stream()), "Wick terms")
        return sums

    def accumulate(self, params, dev, zw1, zw2, xo, xa, first, second, num_pairs, sums,
                   angles=None):
        """Plan and launch pg_cf_wick for the forest pairs."""
        units = self.plan_pairs(dev, first, second, num_pairs, angles)
        return self.launch_pairs(params, dev, zw1, zw2, xo, xa, units, sums)

    def plan_items(self, dev, items):
        """Work units of pg_xcf_wick (forest, first neighbour, neighbour
        count), costly items cut into slices, as device arrays."""
        item_forest, item_start, item_count, obj_index, num_items, max_quasars = items
        npix = torch.from_numpy(np.asarray(dev.npix, dtype=np.int64)).to(self.device)
        cost = (npix[item_forest[:num_items].long()] * item_count[:num_items].long()).cpu().numpy()
        unit, sl, sls = slice_units(cost)
        u = torch.from_numpy(unit).to(self.device)
        return {"forest": item_forest[u].contiguous(), "start": item_start[u].contiguous(),
                "count": item_count[u].contiguous(), "index": obj_index,
                "slice": torch.from_numpy(sl).to(self.device),
                "slices": torch.from_numpy(sls).to(self.device), "num": int(unit.size),
                "max_quasars": int(max_quasars)}

    def launch_items(self, params, dev, qdev, zw1, zw_obj, xo, xa, units, sums):
        """Launch pg_xcf_wick on planned units (asynchronous, current stream)."""
        lib = _bind()
        nbytes = ctypes.c_uint64()
        with torch.cuda.device(self.device):
            check(lib.pg_xcf_wick_work_bytes(self.engine.plan.handle, ctypes.byref(params),
                                             int(dev.max_pixels), units["max_quasars"],
                                             max(units["num"], 1), ctypes.byref(nbytes)),
                  "cross Wick work size")
            need = int(nbytes.value)
            if self._work is None or self._work.numel() < need:
                self._work = torch.empty(max(need, 16), dtype=torch.uint8, device=self.device)
            check(lib.pg_xcf_wick(
                self.engine.plan.handle, ctypes.byref(params), ctypes.byref(dev.c),
                ctypes.byref(qdev.c), zw1.data_ptr(), zw_obj.data_ptr(), xo.data_ptr(),
                xa.data_ptr(), units["forest"].data_ptr(), units["start"].data_ptr(),
                units["count"].data_ptr(), units["index"].data_ptr(), None,
                units["slice"].data_ptr(), units["slices"].data_ptr(), units["num"],
                units["max_quasars"], self._work.data_ptr(), int(self._work.numel()),
                ctypes.byref(self._sums_struct(sums)), self._stream()), "cross Wick terms")
        return sums

    def launch_items_factored(self, params, dev, qdev, zw1, zw_obj, xo, xa, items, sums):
        """pg_xcf_wick_factored on work items (forest, first neighbour,
        neighbour count): T2 + T4 and T3 as FP64 GEMMs over each forest's
        nonempty bins (the call waits for each item's bin count)."""
        lib = _bind()
        item_forest, item_start, item_count, obj_index, num_items, max_quasars = items
        nbytes = ctypes.c_uint64()
        with torch.cuda.device(self.device):
            check(lib.pg_xcf_wick_factored_work_bytes(
                self.engine.plan.handle, ctypes.byref(params), int(dev.max_pixels),
                int(max_quasars), ctypes.byref(nbytes)), "cross Wick work size")
            need = int(nbytes.value)
            if self._work is None or self._work.numel() < need:
                self._work = torch.empty(max(need, 16), dtype=torch.uint8, device=self.device)
            check(lib.pg_xcf_wick_factored(
                self.engine.plan.handle, ctypes.byref(params), ctypes.byref(dev.c),
                ctypes.byref(qdev.c), zw1.data_ptr(), zw_obj.data_ptr(), xo.data_ptr(),
                xa.data_ptr(), item_forest.data_ptr(), item_start.data_ptr(),
                item_count.data_ptr(), obj_index.data_ptr(), None, int(num_items),
                int(max_quasars), self._work.data_ptr(), int(self._work.numel()),
                ctypes.byref(self._sums_struct(sums)), self._stream()), "cross Wick terms")
        return sums

    def accumulate_cross(self, params, dev, qdev, zw1, zw_obj, xo, xa, items, sums):
        """Plan and launch pg_xcf_wick for work items (forest, first
        neighbour, neighbour count) of the neighbour index."""
        units = self.plan_items(dev, items)
        return self.launch_items(params, dev, qdev, zw1, zw_obj, xo, xa, units, sums)

    def stats(self):
        return self.engine.stats()


#: pairs of listed pixel pairs per slice the host aims at when it cuts a
#: costly work unit (the sweep of one unit is one CTA's)
SLICE_TARGET = 2.0e9
MAX_SLICES = 128


def slice_units(cost):
    """Cut work units into slices by their bound on the sweep, (pixel pairs
    of the unit)^2: returns (unit index, slice, slices) per entry, costliest
    slices first."""
    cost = np.asarray(cost, dtype=np.float64)
    slices = np.clip(np.ceil(cost * cost / SLICE_TARGET), 1, MAX_SLICES).astype(np.int64)
    unit = np.repeat(np.arange(cost.size, dtype=np.int64), slices)
    start = np.concatenate([[0], np.cumsum(slices)[:-1]]) if cost.size else np.zeros(0, np.int64)
    sl = np.arange(unit.size, dtype=np.int64) - np.repeat(start, slices)
    per = (cost * cost / slices)[unit]
    order = np.argsort(-per, kind="stable")
    return (unit[order], sl[order].astype(np.int32), slices[unit][order].astype(np.int32))


def forest_pairs(dev, offsets, index, mask):
    """(first, second) device lists of the neighbour entries in ``mask``,
    longest pixel grids first (a better balance of the persistent CTAs)."""
    total = int(mask.size)
    device = dev.device
    if total == 0 or not mask.any():
        z = torch.zeros(1, dtype=torch.int32, device=device)
        return z, z, 0
    k = torch.nonzero(torch.from_numpy(mask).to(device)).flatten()
    first = torch.searchsorted(offsets, k, right=True) - 1
    second = index[:total][k].long()
    npix = torch.from_numpy(np.asarray(dev.npix, dtype=np.int64)).to(device)
    order = torch.argsort(npix[first] * npix[second], descending=True, stable=True)
    return (first[order].to(torch.int32).contiguous(),
            second[order].to(torch.int32).contiguous(), int(k.numel()))


def evolution(z, z_ref, alpha):
    """((1 + z) / (1 + z_ref))^(alpha - 1) per pixel (cf.py:1545-1546)."""
    return ((1 + np.asarray(z, dtype=np.float64)) / (1 + z_ref)) ** (alpha - 1)


def normalise(raw, npall, npused):
    """py/picca/bin/picca_wick.py:515-540 (picca_xwick.py:487-506): every
    term divided by WALL WALL^T where positive and scaled by NPUSED / NPALL;
    the terms not computed are 0."""
    nb = raw["weights_wick"].size
    weights = raw["weights_wick"] * raw["weights_wick"][:, None]
    w = weights > 0.0
    out = {"WALL": raw["weights_wick"].copy(), "NB": raw["num_pairs_wick"].copy()}
    for key in ("t1", "t2", "t3", "t4"):
        if key not in raw:
            continue
        t = raw[key].reshape(nb, nb).copy()
        t[w] /= weights[w]
        t *= 1.0 * npused / npall
        out[key.upper()] = t
    for key in ("T4", "T5", "T6"):
        if key not in out:
            out[key] = np.zeros((nb, nb))
    out["CO"] = out["T1"] + out["T2"] + out["T3"] + out["T4"] + out["T5"] + out["T6"]
    out["NPALL"], out["NPUSED"] = int(npall), int(npused)
    return out


def wick_covariance(fs, params, cf1d, reject, nproc=1, z_ref=2.25, alpha=2.9, alpha2=None,
                    engine=None, return_raw=False):
    """picca_wick.py for one delta field (auto-correlation, --max-diagram 3)
    on a ForestSet: the normalised COV columns (CO, WALL, NB, T1-T6) and
    NPALL / NPUSED."""
    alpha2 = alpha if alpha2 is None else alpha2
    engine = engine or WickEngine()
    pe = engine.engine
    tables = OneDTables(cf1d)
    dev = _pairs.DeviceForests(fs, pe.device, compact=False)
    offsets, index, _ = pe.neighbours(params, dev)
    keep, npall, npused = selection(fs, nproc, reject)
    off_h = offsets.cpu().numpy()
    mask = np.repeat(keep, np.diff(off_h))
    first, second, num = forest_pairs(dev, offsets, index, mask)
    nb = params.num_bins_r_par * params.num_bins_r_trans
    sums = engine.alloc_sums(nb)
    if num:
        used = np.unique(np.concatenate([first[:num].cpu().numpy(),
                                         second[:num].cpu().numpy()]))
        xa, xo, _keep_alive = engine.xi_matrices(dev, tables, used)
        z = np.asarray(fs.z, dtype=np.float64)
        zw1 = torch.from_numpy(np.ascontiguousarray(evolution(z, z_ref, alpha)
                                                    if z.size else np.zeros(1))).to(pe.device)
        zw2 = torch.from_numpy(np.ascontiguousarray(evolution(z, z_ref, alpha2)
                                                    if z.size else np.zeros(1))).to(pe.device)
        engine.accumulate(params, dev, zw1, zw2, xo, xa, first, second, num, sums)
        stats = engine.stats()
        if stats.status != 0:
            raise _native.NativeError(f"Wick kernel reported status {stats.status}")
    raw = {k: v.cpu().numpy() for k, v in sums.items()}
    out = normalise(raw, npall, npused)
    if return_raw:
        out["raw"] = raw
    return out


def cross_wick_covariance(fs, qs, params, cf1d, reject, nproc=1, z_ref=2.25, alpha=2.9,
                          alpha_obj=1.44, engine=None, return_raw=False, method="factored"):
    """picca_xwick.py (py/picca/bin/picca_xwick.py:447-520, --max-diagram 4,
    the default) on a forest set and a quasar set: the normalised COV
    columns (CO, WALL, NB, T1-T6, T5 = T6 = 0) and NPALL / NPUSED. Every
    neighbouring quasar of a kept forest enters (no per-pair draw).
    ``method``: "factored" (GEMMs over each forest's bins,
    pg_xcf_wick_factored) or "sweep" (all pairs of listed pairs,
    pg_xcf_wick)."""
    engine = engine or WickEngine()
    pe = engine.engine
    tables = OneDTables(cf1d)
    dev = _pairs.DeviceForests(fs, pe.device, compact=False)
    qdev = _pairs.DeviceForests(qs, pe.device)
    offsets, index, total = pe.neighbours(params, dev, qdev, xcf=True)
    keep, npall, npused = selection(fs, nproc, reject)
    off_h = offsets.cpu().numpy()
    counts = np.diff(off_h)
    forests = np.nonzero(keep & (counts > 0))[0]
    nb = params.num_bins_r_par * params.num_bins_r_trans
    sums = engine.alloc_sums(nb, cross=True)
    if forests.size:
        if total >= 2**31 or counts[forests].max() > 65535:
            raise _native.NativeError("too many forest-quasar neighbours for the cross Wick "
                                      "kernel")
        order = np.argsort(-(np.asarray(dev.npix)[forests] * counts[forests]), kind="stable")
        forests = forests[order]
        dvc = pe.device
        items = (torch.from_numpy(forests.astype(np.int32)).to(dvc),
                 torch.from_numpy(off_h[forests].astype(np.int32)).to(dvc),
                 torch.from_numpy(counts[forests].astype(np.int32)).to(dvc),
                 index, int(forests.size), int(counts[forests].max()))
        xa, xo, _keep_alive = engine.xi_matrices(dev, tables, forests)
        z = np.asarray(fs.z, dtype=np.float64)
        zw1 = torch.from_numpy(np.ascontiguousarray(evolution(z, z_ref, alpha)
                                                    if z.size else np.zeros(1))).to(dvc)
        zq = np.asarray(qs.z_qso, dtype=np.float64)
        zw_obj = torch.from_numpy(np.ascontiguousarray(evolution(zq, z_ref, alpha_obj)
                                                       if zq.size else np.zeros(1))).to(dvc)
        if method == "factored":
            engine.launch_items_factored(params, dev, qdev, zw1, zw_obj, xo, xa, items, sums)
        elif method == "sweep":
            engine.accumulate_cross(params, dev, qdev, zw1, zw_obj, xo, xa, items, sums)
        else:
            raise ValueError(f"unknown method {method}")
        stats = engine.stats()
        if stats.status != 0:
            raise _native.NativeError(f"cross Wick kernel reported status {stats.status}")
    raw = {k: v.cpu().numpy() for k, v in sums.items()}
    out = normalise(raw, npall, npused)
    if return_raw:
        out["raw"] = raw
    return out
