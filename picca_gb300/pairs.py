"""Device orchestration of the pair accumulation.

Host-side driver of the C ABI: uploads :class:`~picca_gb300.forests.ForestSet`
arrays to the GPU (PyTorch tensors are used only as device allocations),
builds neighbour lists with the two-pass ``pg_*_neighbours`` protocol, orders
work items by cost (longest first, for the persistent kernels' dynamic
queue), and accumulates per-healpix rows with ``pg_cf_xi`` / ``pg_xcf_xi``.
This replaces the fork-Pool loop of ``py/picca/bin/picca_cf.py:452-458``
(``corr_func`` -> ``cf.fill_neighs`` + ``cf.compute_xi``) by one launch over
every healpix.
"""

import ctypes
import math

import numpy as np
import torch

from . import _native
from ._native import CorrParams, ForestSetC, NbrGroupsC, XiRowsC, check

MODE_FP64 = _native.PG_MODE_FP64
MODE_FP32_GUARD = _native.PG_MODE_FP32_GUARD


def _nan(value):
    return float("nan") if value is None else float(value)


def make_params(r_par_min, r_par_max, r_trans_max, num_bins_r_par, num_bins_r_trans, ang_max,
                z_min_pairs=None, z_max_pairs=None, zerr_cut_deg=None, zerr_cut_kms=None,
                x_correlation=False, rmu_binning=False, ang_correlation=False,
                remove_same_half_plate_close_pairs=False):
    """pg_corr_params from picca's module-global values (None disables a cut)."""
    return CorrParams(
        float(r_par_min), float(r_par_max), float(r_trans_max), int(num_bins_r_par),
        int(num_bins_r_trans), _nan(z_min_pairs), _nan(z_max_pairs), _nan(zerr_cut_deg),
        _nan(zerr_cut_kms), float(ang_max), int(bool(x_correlation)), int(bool(rmu_binning)),
        int(bool(ang_correlation)), int(bool(remove_same_half_plate_close_pairs)))


def require_cuda():
    """The product path runs on a CUDA device only; fail loudly otherwise."""
    if not torch.cuda.is_available():
        raise _native.NativeError("picca_gb300 needs a CUDA device (no CPU fallback)")
    _native.lib()


class DeviceForests:
    """A ForestSet resident in device memory.

    Zero-weight pixels are dropped (the reference skips them,
    py/picca/cf.py:317-319 and :331-332); ``r_first`` / ``r_last`` keep the
    first and last comoving distance of the full forest for the xcf pre-cut.
    """

    def __init__(self, fs, device=None, compact=True, pinned=False, packed=None):
        require_cuda()
        self.device = torch.device(device or "cuda")
        self.source = fs
        self.num = fs.num
        self.num_rows = len(fs.healpix_list)
        if packed is None:
            packed = pack_host(fs, compact=compact, pinned=pinned)
        self.host = {k: (v.numpy() if isinstance(v, torch.Tensor) else v)
                     for k, v in packed.items()}
        self.tensors = {k: torch.as_tensor(v).to(self.device, non_blocking=True)
                        for k, v in packed.items()}
        self.h2d_bytes = sum(int(t.numel() * t.element_size()) for t in self.tensors.values())
        npix = np.diff(self.host["pix_offset"]) if self.num else np.zeros(0, dtype=np.int64)
        self.npix = npix
        self.max_pixels = int(npix.max()) if npix.size and npix.max() > 0 else 1
        self.num_pixels = int(self.host["pix_offset"][-1]) if self.num else 0
        self.c = self._struct()

    @staticmethod
    def _host_arrays(fs, compact):
        out = {}
        offset = np.asarray(fs.pix_offset, dtype=np.int64)
        has_pixels = fs.num_pixels > 0
        if has_pixels:
            first = offset[:-1]
            last = np.maximum(offset[1:] - 1, first)
            nonempty = offset[1:] > offset[:-1]
            r = np.asarray(fs.r_comov, dtype=np.float64)
            out["r_first"] = np.where(nonempty, r[np.minimum(first, max(len(r) - 1, 0))], 0.0)
            out["r_last"] = np.where(nonempty, r[np.minimum(last, max(len(r) - 1, 0))], 0.0)
        else:
            out["r_first"] = np.zeros(fs.num)
            out["r_last"] = np.zeros(fs.num)
        if has_pixels and compact:
            keep = np.asarray(fs.weights) != 0
            kept = np.zeros(len(keep) + 1, dtype=np.int64)
            np.cumsum(keep, out=kept[1:])
            new_offset = kept[offset]
            out["pix_offset"] = new_offset
            for key in ("z", "r_comov", "dist_m", "weights", "delta"):
                out[key] = np.ascontiguousarray(np.asarray(getattr(fs, key), dtype=np.float64)[keep])
        else:
            out["pix_offset"] = offset.copy()
            for key in ("z", "r_comov", "dist_m", "weights", "delta"):
                out[key] = np.ascontiguousarray(getattr(fs, key), dtype=np.float64)
        for key in ("ra", "dec", "x_cart", "y_cart", "z_cart", "cos_dec", "z_qso",
                    "obj_r_comov", "obj_dist_m", "obj_weight"):
            out[key] = np.ascontiguousarray(getattr(fs, key), dtype=np.float64)
        for key in ("thingid", "plate", "fiberid"):
            out[key] = np.ascontiguousarray(getattr(fs, key), dtype=np.int64)
        out["row"] = np.ascontiguousarray(fs.row, dtype=np.int32)
        # keep every array non-empty so device pointers are valid
        for key, val in out.items():
            if val.size == 0:
                out[key] = np.zeros(1, dtype=val.dtype)
        return out

    def _struct(self):
        c = ForestSetC()
        c.num = self.num
        c.num_pixels = self.num_pixels
        for name in _native.FOREST_SET_PTR_FIELDS:
            setattr(c, name, self.tensors[name].data_ptr())
        c.num_rows = max(self.num_rows, 1)
        c.max_pixels = self.max_pixels
        return c


def pack_host(fs, compact=True, pinned=False):
    """Host arrays in the device layout (optionally in pinned memory, for
    asynchronous uploads)."""
    host = DeviceForests._host_arrays(fs, compact)
    if pinned:
        return {k: torch.from_numpy(v).pin_memory() for k, v in host.items()}
    return host


def _group_bounds(row):
    """Start offsets of the runs of equal values of a non-decreasing array
    (None when it is not sorted)."""
    row = np.asarray(row)
    if row.size == 0:
        return np.zeros(1, dtype=np.int64)
    if np.any(np.diff(row) < 0):
        return None
    change = np.nonzero(np.diff(row))[0] + 1
    return np.concatenate([[0], change, [row.size]]).astype(np.int64)


def _caps(host, bounds):
    """Bounding cap of every group: centre (normalised sum of the members'
    unit vectors) and radius (largest angle from the centre to a member)."""
    x, y, z = (np.asarray(host[k], dtype=np.float64) for k in ("x_cart", "y_cart", "z_cart"))
    starts = bounds[:-1]
    sx, sy, sz = (np.add.reduceat(v, starts) for v in (x, y, z))
    norm = np.sqrt(sx * sx + sy * sy + sz * sz)
    safe = np.where(norm > 0, norm, 1.0)
    cx, cy, cz = sx / safe, sy / safe, sz / safe
    gid = np.repeat(np.arange(starts.size), np.diff(bounds))
    ang = np.arccos(np.clip(x * cx[gid] + y * cy[gid] + z * cz[gid], -1.0, 1.0))
    radius = np.maximum.reduceat(ang, starts)
    radius = np.where(norm > 0, radius, np.pi)
    return np.stack([cx, cy, cz], axis=1), radius


def neighbour_groups(host1, host2, num1, num2, ang_max, block=256):
    """Groups for pg_*_neighbours_grouped: the healpix rows of both sets
    (objects are stored sorted by healpix) with, per row of the query set,
    every row of the other set whose bounding cap comes within ang_max of
    the row's cap (triangle inequality: a superset of the rows that can hold
    a neighbour, the role of healpy.query_disc in cf.fill_neighs,
    py/picca/cf.py:105-122). Returns host arrays, or None when a set is not
    sorted by row (the brute-force search is then used)."""
    if num1 == 0 or num2 == 0:
        return None
    b1 = _group_bounds(np.asarray(host1["row"])[:num1])
    b2 = _group_bounds(np.asarray(host2["row"])[:num2])
    if b1 is None or b2 is None:
        return None
    c1, r1 = _caps({k: np.asarray(host1[k])[:num1] for k in ("x_cart", "y_cart", "z_cart")}, b1)
    c2, r2 = _caps({k: np.asarray(host2[k])[:num2] for k in ("x_cart", "y_cart", "z_cart")}, b2)
    sep = np.arccos(np.clip(c1 @ c2.T, -1.0, 1.0))
    reach = float(ang_max) + r1[:, None] + r2[None, :] + 1e-6
    cand = sep <= reach
    cand_offsets = np.zeros(b1.size, dtype=np.int32)
    np.cumsum(cand.sum(axis=1), out=cand_offsets[1:])
    cand_groups = np.nonzero(cand)[1].astype(np.int32)  # row-major: ascending per group
    sizes = np.diff(b1)
    nblk = (sizes + block - 1) // block
    block_group = np.repeat(np.arange(b1.size - 1, dtype=np.int32), nblk)
    first_of_group = np.repeat(b1[:-1], nblk)
    k = np.arange(block_group.size) - np.repeat(np.concatenate([[0], np.cumsum(nblk)[:-1]]), nblk)
    block_first = (first_of_group + k * block).astype(np.int64)
    block_end = np.minimum(block_first + block, np.repeat(b1[1:], nblk)).astype(np.int64)
    return {"start2": b2, "cand_offsets": cand_offsets,
            "cand_groups": cand_groups if cand_groups.size else np.zeros(1, dtype=np.int32),
            "block_group": block_group, "block_first": block_first, "block_end": block_end,
            "num_groups1": b1.size - 1, "num_groups2": b2.size - 1}


class PairEngine:
    """Neighbour search + pair accumulation on one CUDA device."""

    def __init__(self, device=None):
        require_cuda()
        self.device = torch.device(device or "cuda")
        with torch.cuda.device(self.device):
            self.plan = _native.Plan()
        self.last_stats = None

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def groups(self, params, dev1, dev2=None):
        """Device copy of the grouped-search structure of (dev1, dev2), cached
        per pair of sets and ang_max; None when a set is not sorted by row."""
        other = dev2 if dev2 is not None else dev1
        key = (id(dev1), id(other), float(params.ang_max))
        cache = getattr(self, "_groups_cache", None)
        if cache is not None and cache[0] == key:
            return cache[1]
        host = neighbour_groups(dev1.host, other.host, dev1.num, other.num, params.ang_max)
        if host is None:
            out = None
        else:
            tensors = {k: torch.from_numpy(np.ascontiguousarray(v)).to(self.device)
                       for k, v in host.items() if isinstance(v, np.ndarray)}
            c = NbrGroupsC(int(host["num_groups1"]), int(host["num_groups2"]),
                           int(host["block_group"].size), 0,
                           *[tensors[k].data_ptr() for k in
                             ("start2", "cand_offsets", "cand_groups", "block_group",
                              "block_first", "block_end")])
            out = (c, tensors, (dev1, other))  # keeps the sets alive with the key
        self._groups_cache = (key, out)
        return out

    def neighbours(self, params, dev1, dev2=None, xcf=False, grouped=True):
        """Neighbour CSR (offsets int64 [n1+1], index int32) on the device.
        With ``grouped`` (the default) only candidate healpix rows are
        scanned (``neighbour_groups``); the lists are the same."""
        lib = _native.lib()
        n1 = dev1.num
        counts = torch.zeros(max(n1, 1), dtype=torch.int64, device=self.device)
        s2 = ctypes.byref(dev2.c) if dev2 is not None else None
        groups = self.groups(params, dev1, dev2) if grouped else None
        if groups is not None:
            gfunc = lib.pg_xcf_neighbours_grouped if xcf else lib.pg_cf_neighbours_grouped
            gref = ctypes.byref(groups[0])

            def func(plan, par, d1, d2, cnt, off, idx, stream):
                return gfunc(plan, par, d1, d2, gref, cnt, off, idx, stream)
        else:
            func = lib.pg_xcf_neighbours if xcf else lib.pg_cf_neighbours
        with torch.cuda.device(self.device):
            check(func(self.plan.handle, ctypes.byref(params), ctypes.byref(dev1.c), s2,
                       counts.data_ptr(), None, None, self._stream()), "neighbour count")
            offsets = torch.zeros(n1 + 1, dtype=torch.int64, device=self.device)
            if n1:
                torch.cumsum(counts[:n1], 0, out=offsets[1:])
            total = int(offsets[-1].item())
            index = torch.zeros(max(total, 1), dtype=torch.int32, device=self.device)
            if n1:
                check(func(self.plan.handle, ctypes.byref(params), ctypes.byref(dev1.c), s2,
                           None, offsets.data_ptr(), index.data_ptr(), self._stream()),
                      "neighbour fill")
        return offsets, index, total

    def work_order(self, dev1, dev2, offsets, index, total, xcf=False):
        """Forests with work, longest first. Returns (order int32, num_work,
        candidate pixel pairs)."""
        n1 = dev1.num
        if n1 == 0 or total == 0:
            return torch.zeros(1, dtype=torch.int32, device=self.device), 0, 0
        npix1 = torch.from_numpy(dev1.npix).to(self.device)
        if xcf:
            per_forest = offsets[1:] - offsets[:-1]
        else:
            other = dev2 if dev2 is not None else dev1
            npix2 = torch.from_numpy(other.npix).to(self.device)
            per_nbr = npix2[index[:total].long()]
            csum = torch.zeros(total + 1, dtype=torch.int64, device=self.device)
            torch.cumsum(per_nbr, 0, out=csum[1:])
            per_forest = csum[offsets[1:]] - csum[offsets[:-1]]
        cost = npix1 * per_forest
        self.last_cost = cost  # candidate pixel pairs per forest of set 1
        order = torch.argsort(cost, descending=True, stable=True)
        num_work = int((cost > 0).sum().item())
        candidates = int(cost.sum().item())
        return order.to(torch.int32).contiguous(), num_work, candidates

    def alloc_rows(self, num_rows, nbins):
        rows = [torch.zeros(num_rows * nbins, dtype=torch.float64, device=self.device)
                for _ in range(5)]
        rows.append(torch.zeros(num_rows * nbins, dtype=torch.int64, device=self.device))
        return rows

    def accumulate(self, params, dev1, dev2, offsets, index, order, num_work, rows, mode,
                   xcf=False, angles=None):
        """Launch the pair kernel (asynchronous on the current stream)."""
        lib = _native.lib()
        out = XiRowsC(*[r.data_ptr() for r in rows])
        s2 = ctypes.byref(dev2.c) if dev2 is not None else None
        func = lib.pg_xcf_xi if xcf else lib.pg_cf_xi
        ang_ptr = angles.data_ptr() if angles is not None else None
        with torch.cuda.device(self.device):
            check(func(self.plan.handle, ctypes.byref(params), ctypes.byref(dev1.c), s2,
                       offsets.data_ptr(), index.data_ptr(), ang_ptr, order.data_ptr(),
                       int(num_work), int(mode), ctypes.byref(out), self._stream()),
                  "pair accumulation")
        return rows

    def stats(self):
        self.last_stats = self.plan.stats()
        if self.last_stats.status != 0:
            raise _native.NativeError(
                f"device-side error {self.last_stats.status} "
                f"({_native.lib().pg_strerror(self.last_stats.status).decode()}), "
                f"detail {self.last_stats.error_detail}")
        return self.last_stats


class GraphStep:
    """One accumulation step (rows zeroed, then the pair kernel with its
    scratch reset and constants) captured once in a CUDA graph and replayed
    with a single graph launch. The neighbour lists, work order and rows are
    the captured buffers: refill them in place between replays (same sizes)
    to run another step of the same shape. Replays are asynchronous on the
    current stream."""

    def __init__(self, engine, params, dev1, dev2, offsets, index, order, num_work, rows, mode,
                 xcf=False):
        self.engine = engine
        self._keep = (params, dev1, dev2, offsets, index, order, rows)
        dev = engine.device

        def step():
            for r in rows:
                r.zero_()
            engine.accumulate(params, dev1, dev2, offsets, index, order, num_work, rows, mode,
                              xcf=xcf)

        # one eager step first: kernel modules loaded and attributes set
        # outside the capture
        step()
        torch.cuda.synchronize(dev)
        engine.stats()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.device(dev), torch.cuda.graph(self.graph):
            step()
        torch.cuda.synchronize(dev)

    def replay(self):
        self.graph.replay()


def rows_to_numpy(rows, num_rows, nbins):
    """Device rows -> numpy (we, xi, rp, rt, z, nb), each [num_rows, nbins]."""
    return [r.view(num_rows, nbins).cpu().numpy() for r in rows]


def normalise(we, xi, rp, rt, zz):
    """cf.compute_xi's division by the weights (py/picca/cf.py:242-246)."""
    xi, rp, rt, zz = xi.copy(), rp.copy(), rt.copy(), zz.copy()
    w = we > 0
    xi[w] /= we[w]
    rp[w] /= we[w]
    rt[w] /= we[w]
    zz[w] /= we[w]
    return xi, rp, rt, zz


def correlate(fs1, fs2, params, mode=MODE_FP64, xcf=False, engine=None, device=None,
              pinned=False):
    """Whole correlation of ForestSets: returns a dict with per-row raw
    sums, normalised rows and run statistics (host numpy arrays). With
    ``pinned`` the host arrays are staged in page-locked memory and uploaded
    asynchronously."""
    engine = engine or PairEngine(device)
    dev1 = DeviceForests(fs1, engine.device, pinned=pinned)
    dev2 = DeviceForests(fs2, engine.device, pinned=pinned) if fs2 is not None else None
    nbins = params.num_bins_r_par * params.num_bins_r_trans
    num_rows = len(fs1.healpix_list)
    offsets, index, total = engine.neighbours(params, dev1, dev2, xcf=xcf)
    order, num_work, candidates = engine.work_order(dev1, dev2, offsets, index, total, xcf=xcf)
    rows = engine.alloc_rows(max(num_rows, 1), nbins)
    engine.accumulate(params, dev1, dev2, offsets, index, order, num_work, rows, mode, xcf=xcf)
    stats = engine.stats()
    we, xi, rp, rt, zz, nb = rows_to_numpy(rows, max(num_rows, 1), nbins)
    h2d = dev1.h2d_bytes + (dev2.h2d_bytes if dev2 is not None else 0)
    return {"raw": (we, xi, rp, rt, zz, nb), "num_rows": num_rows, "nbins": nbins, "h2d_bytes": h2d,
            "num_pairs_forest": total, "candidate_pairs": candidates,
            "rechecked_pairs": int(stats.rechecked_pairs), "work_items": int(stats.work_items),
            "visited_pairs": int(stats.visited_pairs),
            "offsets": offsets, "index": index}


def ang_max_ok(value):
    return value is not None and math.isfinite(value) and value > 0
