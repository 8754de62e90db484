"""Launch-shape autotuner for the precision-form pair kernels (no counterpart
in picca).

The kernels' launch shape is a runtime choice of the plan (pg_plan_set_tuning):
warps per CTA (the CTA size) and CTAs per SM (each CTA keeps its own
shared-memory histogram, so this is the number of histogram replicas per SM).
``tune_pairs`` times every candidate shape on a fixed random sample of the
workload's work items with CUDA events, keeps the fastest, and caches the
choice per (device, kernel, bins, wavelength grid, precision mode) in a JSON
file, so later runs of the same kind of workload reuse it without timing.
The pair counts do not depend on the shape (tests/test_gpu_autotune.py).
"""

import ctypes
import json
import os

import numpy as np
import torch

from . import _native
from ._native import check


class TuningC(ctypes.Structure):
    _fields_ = [("cf_warps", ctypes.c_int32), ("cf_blocks_per_sm", ctypes.c_int32),
                ("xcf_warps", ctypes.c_int32), ("xcf_blocks_per_sm", ctypes.c_int32)]


# (warps per CTA, CTAs per SM); 0 = the default (most warps / as many as fit)
CF_CANDIDATES = [(0, 0), (16, 0), (12, 0), (8, 0), (8, 1), (4, 0)]
XCF_CANDIDATES = [(0, 0), (12, 0), (8, 0), (8, 1), (4, 0)]


def _bind():
    lib = _native.lib()
    if not getattr(lib, "_tune_bound", False):
        lib.pg_plan_set_tuning.argtypes = [ctypes.c_void_p, ctypes.POINTER(TuningC)]
        lib.pg_plan_get_tuning.argtypes = [ctypes.c_void_p, ctypes.POINTER(TuningC)]
        lib.pg_plan_set_tuning.restype = ctypes.c_int
        lib.pg_plan_get_tuning.restype = ctypes.c_int
        lib._tune_bound = True
    return lib


def set_tuning(plan, cf=(0, 0), xcf=(0, 0)):
    t = TuningC(int(cf[0]), int(cf[1]), int(xcf[0]), int(xcf[1]))
    check(_bind().pg_plan_set_tuning(plan.handle, ctypes.byref(t)), "set tuning")


def get_tuning(plan):
    t = TuningC()
    check(_bind().pg_plan_get_tuning(plan.handle, ctypes.byref(t)), "get tuning")
    return (t.cf_warps, t.cf_blocks_per_sm), (t.xcf_warps, t.xcf_blocks_per_sm)


def default_cache_path():
    base = os.environ.get("PICCA_GB300_TUNE_CACHE")
    if base:
        return base
    return os.path.join(os.path.expanduser("~"), ".cache", "picca_gb300", "pair_tuning.json")


def _load(path):
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _save(path, table):
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "w") as fh:
        json.dump(table, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def cache_key(device, xcf, nbins, grid, mode):
    name = torch.cuda.get_device_name(device).replace(" ", "_")
    return f"{name}|{'xcf' if xcf else 'cf'}|bins={nbins}|grid={grid}|mode={int(mode)}"


def tune_pairs(engine, params, dev1, dev2, offsets, index, order, num_work, num_rows, mode,
               xcf=False, grid="log", sample_items=2000, reps=2, cache_path=None, retune=False,
               seed=1):
    """Choose and apply the launch shape of the pair kernel for this kind of
    workload. ``num_rows`` is the number of output rows (healpix pixels) of
    the workload. Returns {"key", "choice", "cached", "alternatives":
    [{"warps", "ctas_per_sm", "ms"}], "sample_items"}; the plan of ``engine``
    keeps the choice."""
    cache_path = cache_path or default_cache_path()
    nbins = int(params.num_bins_r_par) * int(params.num_bins_r_trans)
    key = cache_key(engine.device, xcf, nbins, grid, mode)
    table = _load(cache_path)
    cf_now, xcf_now = get_tuning(engine.plan)
    if not retune and key in table:
        choice = tuple(table[key]["choice"])
        set_tuning(engine.plan, cf=choice if not xcf else cf_now, xcf=choice if xcf else xcf_now)
        return {"key": key, "choice": list(choice), "cached": True,
                "alternatives": table[key].get("alternatives", []),
                "sample_items": table[key].get("sample_items")}
    n = min(int(sample_items), int(num_work))
    gen = torch.Generator(device=order.device).manual_seed(seed)
    sub = order[:num_work][torch.randperm(num_work, device=order.device, generator=gen)[:n]]
    sub = sub.contiguous()
    rows = engine.alloc_rows(max(int(num_rows), 1), nbins)
    results = []
    for cand in (XCF_CANDIDATES if xcf else CF_CANDIDATES):
        set_tuning(engine.plan, cf=cand if not xcf else cf_now, xcf=cand if xcf else xcf_now)
        times = []
        for rep in range(reps + 1):
            for r in rows:
                r.zero_()
            start = torch.cuda.Event(enable_timing=True)
            end = torch.cuda.Event(enable_timing=True)
            start.record()
            engine.accumulate(params, dev1, dev2, offsets, index, sub, n, rows, mode, xcf=xcf)
            end.record()
            torch.cuda.synchronize(engine.device)
            if rep:
                times.append(start.elapsed_time(end))
        engine.stats()
        results.append({"warps": cand[0], "ctas_per_sm": cand[1], "ms": float(np.min(times))})
    best = min(results, key=lambda r: r["ms"])
    choice = (best["warps"], best["ctas_per_sm"])
    set_tuning(engine.plan, cf=choice if not xcf else cf_now, xcf=choice if xcf else xcf_now)
    table[key] = {"choice": list(choice), "alternatives": results, "sample_items": n}
    try:
        _save(cache_path, table)
    except OSError:
        pass
    return {"key": key, "choice": list(choice), "cached": False, "alternatives": results,
            "sample_items": n}
