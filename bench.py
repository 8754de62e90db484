"""Benchmark of the GPU correlation path (one JSON line on stdout).

A step is one pass of the hot path over the whole synthetic survey: neighbour
lists of every forest + pair accumulation into per-healpix rows (the work of
``cf.fill_neighs`` + ``cf.compute_xi`` over every healpix,
py/picca/bin/picca_cf.py:452-458). ``value`` is candidate pixel pairs per
second with inputs resident in HBM; ``e2e`` is the same through the public
drop-in ``cf.compute_xi_all`` from host ``Delta`` objects (packing, pinned
upload, neighbours, pairs, rows and neighbour lists back), every e2e step.

Default workload: the 400k-forest auto-correlation on 8,000 deg^2 (50 x 50
bins, r_par and r_trans 0-200 Mpc/h, precision form), with the
cross-correlation of the same forests against 600k quasars (100 x 50 bins,
r_par -200 to 200) as the ``xcf`` object and the Dr16 continuum fit (plain
and learned warm start, 400k raw forests) as the ``continuum`` object.
``--config 1`` / ``1lin`` run the 100k-forest survey (log or 0.8 A linear
grid), ``--config 0`` the 1,000-forest patch. ``--impl reference`` times the
CPU oracle (FP64 C restatement of picca's numba kernel, OpenMP over all host
cores) on a bounded sample of the same workload.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

CONFIGS = {
    # name: (num forests, area deg^2, grid, description)
    "0": (1000, None, "log", "1,000 forests in a 4.5x4.5 deg patch"),
    "1": (100_000, 2000.0, "log", "100k forests on 2,000 deg^2"),
    "1lin": (100_000, 2000.0, "lin", "100k forests on 2,000 deg^2, 0.8 A grid"),
    "2": (400_000, 8000.0, "log", "400k forests on 8,000 deg^2"),
}
METRIC = "cf pixel-pairs/s at stated FP64-oracle error; continuum fits/s plain vs learned"
# DRAM bytes (read + write) of the pair kernel per candidate pixel pair, from
# an ncu capture of the kernel on a sample of work items (profiles/); the
# roofline entry scales it to the launch by the candidate pairs processed.
# Captured on 200 random work items of the 400k-forest survey: 1.249 GB for
# 5.405e9 candidate pixel pairs.
PAIR_DRAM_BYTES_PER_CANDIDATE = 0.2311
PAIR_TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of cf_xi_diag_kernel "
                       "on 200 random work items of this survey, scaled by candidate pairs "
                       "(profiles/cf_xi_diag_kernel_400k_survey_sample.md)")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--config", default="2", choices=sorted(CONFIGS))
    p.add_argument("--precision", choices=["fp32_guard", "fp64"], default="fp32_guard")
    p.add_argument("--check-fraction", type=float, default=0.01,
                   help="fraction of work items re-run in FP64 for the error report")
    p.add_argument("--cpu-seconds", type=float, default=15.0,
                   help="target CPU time of the oracle sample")
    p.add_argument("--continuum-forests", type=int, default=400_000,
                   help="raw forests of the continuum-fit leg; 0 skips it")
    p.add_argument("--continuum-train", type=int, default=200_000,
                   help="raw forests (separate seed) the warm-start network is trained on")
    p.add_argument("--continuum-iterations", type=int, default=5)
    p.add_argument("--profile-items", type=int, default=0,
                   help="profiling aid: run the pair kernel once on this many randomly chosen "
                        "work items of the workload and exit (no timing, no JSON line)")
    p.add_argument("--tune-items", type=int, default=2000,
                   help="work items the launch-shape tuner and the graph comparison time "
                        "(0: default launch shape, no graph comparison)")
    p.add_argument("--legs", default="xcf,continuum",
                   help="comma-separated extra legs: xcf, continuum, dmat, wick, delta_io "
                        "(dmat and wick also run alone with --dmat-only / --wick-only)")
    p.add_argument("--e2e-steps", type=int, default=2,
                   help="steps of the end-to-end leg through cf.compute_xi_all")
    p.add_argument("--dmat-reject", type=float, default=0.99,
                   help="random rejection of the distortion-matrix leg (picca_dmat.py --rej); "
                        "a value >= 1 skips the leg")
    p.add_argument("--dmat-only", action="store_true",
                   help="run only the distortion-matrix leg on --config (prints its JSON)")
    p.add_argument("--dmat-product", choices=["split_bf16", "fp64"], default="split_bf16",
                   help="arithmetic of the eta products in the distortion-matrix leg")
    p.add_argument("--wick-reject", type=float, default=0.99995,
                   help="forest rejection of the Wick covariance legs")
    p.add_argument("--wick-only", action="store_true",
                   help="run only the Wick covariance legs (one JSON line)")
    p.add_argument("--continuum-only", action="store_true",
                   help="run only the continuum leg (plain and learned fits; one JSON line)")
    p.add_argument("--continuum-correlation", type=int, default=50_000,
                   help="forests whose plain- and learned-fit deltas are correlated (0 skips)")
    return p.parse_args()


def make_workload(cfg):
    from picca_gb300 import synthetic
    num, area, grid, _ = CONFIGS[cfg]
    if area is None:
        fs = synthetic.patch_forests()
    else:
        fs = synthetic.survey_band(num, area, seed=20261203, grid=grid)
    params = dict(r_par_min=0.0, r_par_max=200.0, r_trans_max=200.0, num_bins_r_par=50,
                  num_bins_r_trans=50)
    ang_max = synthetic.correlation_ang_max(200.0, float(fs.z.min()))
    return fs, params, ang_max


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        with open(path) as handle:
            return json.load(handle), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def cpu_sample(fs, params, ang_max, seconds, cfg):
    """Time the CPU oracle on a bounded sample of the workload, parallel over
    healpix rows as the reference's Pool is: 2 x cores healpix, a few forests
    (with all their neighbours) in each. Returns (pixel pairs/s, sample
    description, threads)."""
    from oracle import cpu as oracle
    p = oracle.make_params(**params)
    rng = np.random.default_rng(5)
    cores = os.cpu_count() or 1
    rows = rng.choice(len(fs.healpix_list), size=min(len(fs.healpix_list), 2 * cores),
                      replace=False)
    npix = np.diff(fs.pix_offset)
    per_forest = float(np.mean(npix)) ** 2 * 900.0  # ~pairs of one forest with its neighbours
    per_row = max(1, int(seconds * 1.5e8 * cores / (per_forest * len(rows))))
    picks = []
    for r in rows:
        members = np.where(fs.row == r)[0]
        picks.append(rng.choice(members, size=min(len(members), per_row), replace=False))
    sample = np.sort(np.concatenate(picks))
    sub = fs.take(sample)
    t0 = time.perf_counter()
    offsets, index = oracle.neighbours(sub, fs, p, ang_max, auto_mode=1)
    oracle.rows(sub, fs, p, offsets, index)
    elapsed = time.perf_counter() - t0
    csum = np.concatenate([[0], np.cumsum(npix[index])])
    cand = int((npix[sample] * (csum[offsets[1:]] - csum[offsets[:-1]])).sum())
    return cand / elapsed, (f"{len(sample)} forests with all their neighbours, from "
                            f"{len(rows)} healpix of config {cfg}; {elapsed:.1f} s"), cores


def fp64_peak_tflops():
    """FP64 throughput of this GPU measured live: cuBLAS DGEMM 4096^3, best
    of 3 (CUDA events)."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = float("inf")
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return 2.0 * n ** 3 / best / 1e12


def dmat_cpu_sample(fs, params, dparams, pairs_host, seconds):
    """The oracle's forest-pair restatement of
    cf.compute_dmat_forest_pairs_fast on a bounded sample of the selected
    forest pairs, on every host core (threads: the ctypes call releases the
    GIL). Returns (forest pairs/s, pixel pairs/s, sample description,
    threads)."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import cpu as ocpu
    from oracle import dmat as odm
    cores = os.cpu_count() or 1
    op = odm.make_params(params["r_par_min"], params["r_par_max"], params["r_trans_max"],
                         params["num_bins_r_par"], params["num_bins_r_trans"],
                         redshift_evolution=bool(dparams.redshift_evolution))
    po = np.asarray(fs.pix_offset)
    first, second = pairs_host
    rng = np.random.default_rng(9)

    def work(chunk):
        out = odm.new_outputs(op)
        npp = 0
        for f, g in chunk:
            a = slice(po[f], po[f + 1])
            b = slice(po[g], po[g + 1])
            ang = ocpu.lib().oracle_angle(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f], fs.ra[f],
                                          fs.dec[f], fs.cos_dec[f], fs.x_cart[g], fs.y_cart[g],
                                          fs.z_cart[g], fs.ra[g], fs.dec[g])
            odm.forest_pair(op, fs.log_lambda[a], fs.log_lambda[b], fs.r_comov[a],
                            fs.r_comov[b], fs.dist_m[a], fs.dist_m[b], fs.z[a], fs.z[b],
                            fs.weights[a], fs.weights[b], fs.z_qso[f], fs.z_qso[g], ang, False,
                            int(fs.order[f]), int(fs.order[g]), out)
            npp += (po[f + 1] - po[f]) * (po[g + 1] - po[g])
        return npp

    order = rng.permutation(len(first))
    n = npp = 0
    elapsed = 0.0
    with ThreadPoolExecutor(cores) as ex:
        while elapsed < seconds and n < len(order):
            pick = order[n:n + 8 * cores]
            chunks = [list(zip(first[pick[k::cores]], second[pick[k::cores]]))
                      for k in range(cores)]
            t0 = time.perf_counter()
            npp += sum(ex.map(work, chunks))
            elapsed += time.perf_counter() - t0
            n += len(pick)
    return (n / elapsed, npp / elapsed,
            f"{n} selected forest pairs of the same workload (random), {elapsed:.1f} s", cores)


def dmat_leg(args, fs, params, ang_max, cpu_seconds):
    """Distortion matrix (picca_dmat.py defaults: 50 x 50 bins, r 0-200 Mpc/h,
    model bins = data bins, redshift evolution) of the same forests with
    --rej args.dmat_reject: one warm-up and one timed kernel launch over
    every selected forest pair (CUDA events on the launching stream), the
    whole host-to-host call (upload, neighbours, random rejection, kernel,
    download, normalisation) timed by the wall clock, and the oracle on a
    sample of the selected pairs."""
    import torch

    from picca_gb300 import dmat, pairs
    if args.dmat_reject >= 1.0:
        return None
    cparams = pairs.make_params(ang_max=ang_max, **params)
    dparams = dmat.make_dmat_params(params["num_bins_r_par"], params["num_bins_r_trans"],
                                    product=args.dmat_product)
    engine = dmat.DmatEngine()
    pe = engine.engine
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = dmat.distortion_matrix(fs, None, cparams, dparams, args.dmat_reject, nproc=1,
                                 engine=engine)
    torch.cuda.synchronize()
    e2e_first = time.perf_counter() - t0
    t0 = time.perf_counter()
    res = dmat.distortion_matrix(fs, None, cparams, dparams, args.dmat_reject, nproc=1,
                                 engine=engine)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    # kernel alone
    dev = pairs.DeviceForests(fs, pe.device)
    offsets, index, total = pe.neighbours(cparams, dev)
    mask = dmat.selection_mask(fs.healpix_list, fs.row, offsets.cpu().numpy(), 1,
                               args.dmat_reject)
    first, second, nsel = engine.pair_list(dev, None, offsets, index, mask)
    side = dmat.DmatEngine.side_arrays(dev, pe.device)
    stream = torch.cuda.current_stream()
    times = []
    for _ in range(2):
        sums = engine.alloc_sums(cparams, dparams)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        engine.accumulate(cparams, dparams, dev, None, side, None, first, second, nsel, sums)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
        stats = pe.stats()
    kernel_s = times[-1]
    f_h, g_h = first.cpu().numpy()[:nsel], second.cpu().numpy()[:nsel]
    npix = dev.npix
    pixel_pairs = float(np.sum(npix[f_h].astype(np.float64) * npix[g_h]))
    macs = float(stats.gemm_macs)
    peak = fp64_peak_tflops()
    achieved = 2.0 * macs / kernel_s / 1e12
    del dev, sums, side, first, second, offsets, index
    torch.cuda.empty_cache()
    cpu_pairs, cpu_pix, cpu_desc, cores = dmat_cpu_sample(fs, params, dparams, (f_h, g_h),
                                                          cpu_seconds)
    cross = xdmat_leg(args, fs, params, ang_max, engine)
    metals = metal_leg(args, fs, params, ang_max, engine, mask)
    return {
        "metric": "distortion-matrix forest pairs per second",
        "value": nsel / kernel_s, "unit": "forest-pairs/s",
        "pixel_pairs_per_s": pixel_pairs / kernel_s, "kernel_ms": kernel_s * 1e3,
        "dtype": "f32 geometry + f64 sums" + (", bf16 digit products" if
                                               args.dmat_product == "split_bf16" else
                                               ", f64 products"),
        "config": {"workload": "same forests, 50x50 data bins = model bins, r 0-200 Mpc/h, "
                   "redshift evolution, random rejection %.2f (one chunk)" % args.dmat_reject,
                   "neighbour_pairs": int(res["NPALL"]), "selected_forest_pairs": int(nsel),
                   "pixel_pairs": pixel_pairs},
        "e2e": {"value": nsel / e2e_s, "unit": "forest-pairs/s", "seconds": e2e_s,
                "first_call_seconds": e2e_first},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "gemm_macs": macs,
                     "peak_source": "cuBLAS DGEMM 4096^3 measured in this run",
                     "achieved_counts": "2 x multiply-adds of the per-pair U E^T products",
                     "note": "the products are FP64-accurate (exact 8-bit digit products on "
                             "the BF16 tensor cores unless --dmat-product fp64): frac above 1 "
                             "is their rate over the native FP64 rate; the FP64 pipe (run "
                             "sums) is the busiest unit in the ncu capture"},
        "cpu_baseline": {"value": cpu_pairs, "unit": "forest-pairs/s",
                         "pixel_pairs_per_s": cpu_pix, "cores": cores, "kind": "port",
                         "sample": cpu_desc},
        "cross": cross,
        "metal": metals,
        "fast_metal": fast_metal_leg(args),
    }


def fast_metal_leg(args):
    """picca_fast_metal_dmat.py on a DESI-like stack (0.8 A pixels over
    3600-5772 A, 2,716 pixels, synthetic weights), LYA and the four silicon
    lines (14 absorber pairs), 50 x 50 bins, r 0-200 Mpc/h: the pair
    histograms of all pairs timed with CUDA events, the whole computation
    (side preparation, uploads, histograms, host epilogue) with the host
    clock, and the NumPy oracle on one core for one pair."""
    import torch

    from oracle import fast_metal as ofm
    from picca_gb300 import constants, fast_metal
    cosmo = constants.Cosmo(Om=0.3147, verbose=False)
    lam = 3600.0 + 0.8 * np.arange(2716)
    log_lambda = np.log10(lam)
    rng = np.random.default_rng(11)
    weight = rng.uniform(10.0, 90.0, lam.size)
    metals = ["SiII(1190)", "SiII(1193)", "SiIII(1207)", "SiII(1260)"]
    alpha = {"LYA": 2.9, **{m: 1.0 for m in metals}}
    A = constants.ABSORBER_IGM
    pairs_ = fast_metal.absorber_pairs("LYA", metals)
    engine = fast_metal.FastMetalEngine()

    def sides(a1, a2, mod):
        return (mod.stack_side(log_lambda, weight, A[a1], A["LYA"], alpha[a1] + 2.9, cosmo),
                mod.stack_side(log_lambda, weight, A[a2], A["LYA"], alpha[a2] + 2.9, cosmo))

    def run_all():
        out = []
        for a1, a2 in pairs_:
            s1, s2 = sides(a1, a2, fast_metal)
            out.append(fast_metal.fast_metal_matrix(s1, s2, 0.0, 200.0, 200.0, 50, 50, False,
                                                    engine=engine))
        return out

    run_all()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run_all()
    e2e_s = time.perf_counter() - t0
    devs = [tuple(engine.upload(s) for s in sides(a1, a2, fast_metal)) for a1, a2 in pairs_]
    stream = torch.cuda.current_stream()
    times = []
    for _ in range(3):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for d1, d2 in devs:
            engine.histograms_device(d1, d2, 0.0, 200.0, 50, 50, False)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    kernel_s = min(times)
    pix_pairs = float(len(pairs_)) * lam.size * lam.size
    t0 = time.perf_counter()
    s1, s2 = sides(*pairs_[0], ofm)
    ofm.matrix(s1, s2, 0.0, 200.0, 200.0, 50, 50, False)
    cpu_s = time.perf_counter() - t0
    return {"metric": "fast metal distortion matrices: stack pixel pairs per second",
            "value": pix_pairs / kernel_s, "unit": "pixel-pairs/s",
            "kernel_ms": kernel_s * 1e3, "matrices": len(pairs_), "dtype": "f64",
            "config": {"workload": "stack of 2,716 pixels (0.8 A, 3600-5772 A), LYA + 4 Si "
                                   "lines = 14 absorber pairs, 50 x 50 bins, r 0-200 Mpc/h"},
            "e2e": {"value": pix_pairs / e2e_s, "unit": "pixel-pairs/s", "seconds": e2e_s},
            "cpu_baseline": {"value": lam.size * lam.size / cpu_s, "unit": "pixel-pairs/s",
                             "cores": 1, "kind": "port",
                             "sample": f"one absorber pair, NumPy restatement, {cpu_s:.2f} s"}}


def metal_leg(args, fs, params, ang_max, engine, mask):
    """Metal distortion matrix LYA x SiIII(1207) (picca_metal_dmat.py:
    direct and swapped passes) over the same kept forest pairs: one warm-up
    and one timed run of both passes (CUDA events), and the oracle (NumPy,
    one core) on a sample of the kept pairs."""
    import torch

    from oracle import cpu as ocpu
    from oracle import metal_dmat as omd
    from picca_gb300 import constants, dmat, metal, pairs
    cosmo = constants.Cosmo(Om=0.3147, verbose=False)
    alpha = {"LYA": 2.9, "SiIII(1207)": 1.0}
    cparams = pairs.make_params(ang_max=ang_max, **params)
    dparams = dmat.make_dmat_params(params["num_bins_r_par"], params["num_bins_r_trans"])
    meng = metal.MetalEngine(engine.engine)
    pe = meng.engine
    dev = pairs.DeviceForests(fs, pe.device)
    offsets, index, _ = pe.neighbours(cparams, dev)
    first, second, num = meng.pair_list(dev, None, offsets, index, mask)
    side_l = metal.absorber_pixels(dev, cosmo, "LYA", alpha["LYA"])
    side_s = metal.absorber_pixels(dev, cosmo, "SiIII(1207)", alpha["SiIII(1207)"])
    den = (1 + 2.25) ** (alpha["LYA"] + alpha["SiIII(1207)"] - 2)
    stream = torch.cuda.current_stream()
    times = []
    for _ in range(2):
        sums = meng.alloc_sums(cparams, dparams)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        meng.run_pass(cparams, dparams, den, dev, None, side_l, side_s, first, second, num, sums)
        meng.run_pass(cparams, dparams, den, dev, None, side_s, side_l, first, second, num, sums)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
        pe.stats()
    f_h, g_h = first.cpu().numpy()[:num], second.cpu().numpy()[:num]
    npix = np.diff(fs.pix_offset)
    pix_pairs = 2.0 * float(np.sum(npix[f_h].astype(np.float64) * npix[g_h]))
    del dev, sums, side_l, side_s, first, second
    torch.cuda.empty_cache()
    # oracle sample
    p = omd.MetalParams(params["r_par_min"], params["r_par_max"], params["r_trans_max"],
                        params["num_bins_r_par"], params["num_bins_r_trans"], z_ref=2.25,
                        alpha_abs=alpha)
    out = omd.new_outputs(p)
    po = np.asarray(fs.pix_offset)
    rng = np.random.default_rng(3)
    pick = rng.permutation(len(f_h))
    n = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < min(args.cpu_seconds, 10.0) and n < len(pick):
        f, g = int(f_h[pick[n]]), int(g_h[pick[n]])
        ang = ocpu.lib().oracle_angle(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f], fs.ra[f],
                                      fs.dec[f], fs.cos_dec[f], fs.x_cart[g], fs.y_cart[g],
                                      fs.z_cart[g], fs.ra[g], fs.dec[g])
        side = lambda h: (fs.log_lambda[po[h]:po[h + 1]], fs.r_comov[po[h]:po[h + 1]],  # noqa
                          fs.dist_m[po[h]:po[h + 1]], fs.weights[po[h]:po[h + 1]], fs.z_qso[h])
        omd.forest_pair(p, cosmo, side(f), side(g), ang, False, "LYA", "SiIII(1207)", True, out)
        n += 1
    cpu_s = time.perf_counter() - t0
    return {"metric": "metal distortion-matrix kept forest pairs per second (LYA x SiIII(1207), "
                      "direct and swapped passes)",
            "value": num / times[-1], "unit": "forest-pairs/s", "kernel_ms": times[-1] * 1e3,
            "pixel_pairs_per_s": pix_pairs / times[-1], "dtype": "f64",
            "cpu_baseline": {"value": n / cpu_s, "unit": "forest-pairs/s", "cores": 1,
                             "kind": "port", "sample": f"{n} kept forest pairs, NumPy "
                                                       f"restatement, {cpu_s:.1f} s"}}


def delta_io_leg(fs, num=20_000, per_file=1_000):
    """Delta-file reading (io.read_deltas: parse, z, distances, weights,
    projection) of the first ``num`` bench forests written as picca delta
    files (one BINTABLE per line of sight, gzip, ``per_file`` per file):
    the native parser and projection against the per-object readers, wall
    clock, all host threads for the native path."""
    import shutil
    import tempfile

    from picca_gb300 import constants, fitsio_lite, io
    num = min(num, fs.num)
    base = tempfile.mkdtemp(prefix="deltas_")
    po = np.asarray(fs.pix_offset)
    os.makedirs(os.path.join(base, "Delta"))
    try:
        for k in range(0, num, per_file):
            tables = []
            for f in range(k, min(k + per_file, num)):
                sl = slice(po[f], po[f + 1])
                tables.append({
                    "columns": [fs.log_lambda[sl], fs.delta[sl], fs.weights[sl],
                                np.ones(po[f + 1] - po[f])],
                    "names": ["LOGLAM", "DELTA", "WEIGHT", "CONT"], "extname": str(f),
                    "header": [{"name": "RA", "value": float(fs.ra[f])},
                               {"name": "DEC", "value": float(fs.dec[f])},
                               {"name": "Z", "value": float(fs.z_qso[f])},
                               {"name": "THING_ID", "value": int(f)},
                               {"name": "PLATE", "value": 1}, {"name": "MJD", "value": 1},
                               {"name": "FIBERID", "value": f % 1000 + 1}]})
            fitsio_lite.write_fits(os.path.join(base, "Delta", f"delta-{k // per_file}.fits.gz"),
                                   tables)
        attr = os.path.join(base, "attributes.fits.gz")
        fitsio_lite.write_fits(attr, [{"columns": [np.zeros(1, dtype=np.int64)],
                                       "names": ["LOS_ID"], "extname": "FIT_METADATA",
                                       "header": [{"name": "FITORDER", "value": 1}]}])
        cosmo = constants.Cosmo(Om=0.3147, verbose=False)
        times = {}
        for native in (True, False):
            t0 = time.perf_counter()
            _, n, _, _ = io.read_deltas(os.path.join(base, "Delta") + "/", 16,
                                        constants.ABSORBER_IGM["LYA"], 2.9, 2.25, cosmo,
                                        delta_attributes=attr, native=native)
            times[native] = time.perf_counter() - t0
    finally:
        shutil.rmtree(base, ignore_errors=True)
    return {"metric": "delta files read per second (parse, z, distances, weights, projection)",
            "value": n / times[True], "unit": "forests/s", "forests": n,
            "files": (n + per_file - 1) // per_file, "threads": os.cpu_count(),
            "cpu_baseline": {"value": n / times[False], "unit": "forests/s", "cores": 1,
                             "kind": "port", "sample": "the same files through the "
                             "per-object readers (io.read_deltas(native=False))"}}


def synthetic_cf1d():
    """A picca_cf1d.py table for the Wick legs: 1,000 offsets of 3e-4 in
    log10(lambda) from 3600 A, unit correlation at zero offset and a small
    anticorrelation decaying with the offset, variance 0.05-0.15."""
    k = np.arange(1000)
    c1d = np.where(k == 0, 1.0, -0.015 * np.exp(-k / 40.0))
    v1d = 0.1 + 0.05 * np.sin(k / 60.0)
    ones = np.ones(k.size, dtype=np.int64)
    return {"LLMIN": float(np.log10(3600.0)), "DLL": 3e-4, "v1d": v1d, "nv1d": ones,
            "c1d": c1d, "nb1d": ones}


def wick_cpu_sample(fs, qs, cparams, pairs_or_items, cf1d, seconds, cross=False):
    """The oracle's C restatement of compute_wickT123_pairs (auto) or
    compute_wickT1234_pairs (cross) on a bounded sample of the same work, on
    every host core (threads: the ctypes call releases the GIL). Returns
    (work units/s, sample description, threads)."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import cpu as ocpu
    from oracle import wick as ow
    cores = os.cpu_count() or 1
    p = ow.make_params(cparams.r_par_min, cparams.r_par_max, cparams.r_trans_max,
                       cparams.num_bins_r_par, cparams.num_bins_r_trans,
                       x_correlation=bool(cparams.x_correlation))
    variance, xi = ow.interpolants(cf1d)
    po = np.asarray(fs.pix_offset)
    zw = ((1 + np.asarray(fs.z)) / 3.25) ** 1.9

    def xmat(f):
        sl = slice(po[f], po[f + 1])
        return ow.weighted_xi_1d(fs.log_lambda[sl], fs.weights[sl], variance, xi)

    def angle(f, g, other):
        return ocpu.lib().oracle_angle(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f], fs.ra[f],
                                       fs.dec[f], fs.cos_dec[f], other.x_cart[g],
                                       other.y_cart[g], other.z_cart[g], other.ra[g],
                                       other.dec[g])

    def work(unit):
        out = ow.new_outputs(p)
        out["t4"] = np.zeros_like(out["t1"])
        if cross:
            f, nbrs = unit
            sl = slice(po[f], po[f + 1])
            zq = qs.z_qso[nbrs]
            ow.xforest(p, fs.r_comov[sl], fs.weights[sl], zw[sl], xmat(f), qs.obj_r_comov[nbrs],
                       qs.obj_weight[nbrs], ((1 + zq) / 3.25) ** 0.44,
                       np.array([angle(f, g, qs) for g in nbrs]), out)
        else:
            f, g = unit
            a, b = slice(po[f], po[f + 1]), slice(po[g], po[g + 1])
            ow.forest_pair(p, fs.r_comov[a], fs.weights[a], zw[a], xmat(f), fs.r_comov[b],
                           fs.weights[b], zw[b], xmat(g), angle(f, g, fs), out)
        return int(out["num_pairs_wick"].sum())

    rng = np.random.default_rng(5)
    units = list(pairs_or_items)
    order = rng.permutation(len(units))
    n = 0
    listed = []
    t0 = time.perf_counter()
    with ThreadPoolExecutor(cores) as ex:
        while time.perf_counter() - t0 < seconds and n < len(order):
            pick = [units[i] for i in order[n:n + cores]]
            listed += list(ex.map(work, pick))
            n += len(pick)
    elapsed = time.perf_counter() - t0
    pairs2 = float(np.sum(np.square(np.asarray(listed, dtype=np.float64))))
    what = "forests with their quasars" if cross else "forest pairs"
    return (n / elapsed, pairs2 / elapsed,
            f"{n} {what} of the same selection (random), C restatement, {elapsed:.1f} s",
            cores)


def wick_leg(args, fs, params, ang_max):
    """Wick covariance (picca_wick.py T1-T3, picca_xwick.py T1-T4) of the
    bench forests, forests kept with probability 1 - args.wick_reject: the
    drop-in call timed end to end (host clock), the Wick kernel alone
    (CUDA events), its FP64 rate against the measured DGEMM peak (one FMA
    per pair of listed pixel pairs), and the C oracle on the host cores."""
    import torch

    from picca_gb300 import pairs, synthetic, wick
    cf1d = synthetic_cf1d()
    out = {"reject": args.wick_reject, "cf1d": "synthetic (1,000 offsets of 3e-4)"}
    peak = fp64_peak_tflops()
    for name in ("auto", "cross"):
        if name == "cross":
            num, area, _, _ = CONFIGS[args.config]
            if area is None:  # the patch of the CPU-runnable case
                ra_r = tuple(np.degrees([np.min(fs.ra), np.max(fs.ra)]))
                dec_r = tuple(np.degrees([np.min(fs.dec), np.max(fs.dec)]))
            else:
                ra_r, dec_r = synthetic.band_for_area(area, 20.0 if area <= 4000 else 30.0)
            qs = synthetic.make_quasars(int(1.5 * fs.num), 20261207, ra_r, dec_r)
            cparams = pairs.make_params(ang_max=ang_max, x_correlation=True,
                                        **dict(params, r_par_min=-200.0, num_bins_r_par=100))
        else:
            qs = None
            cparams = pairs.make_params(ang_max=ang_max, **params)
        engine = wick.WickEngine()
        run = (lambda: wick.cross_wick_covariance(fs, qs, cparams, cf1d, args.wick_reject,
                                                  engine=engine)) if qs is not None else \
            (lambda: wick.wick_covariance(fs, cparams, cf1d, args.wick_reject, engine=engine))
        run()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = run()
        e2e_s = time.perf_counter() - t0
        # the kernel alone, on the same work
        pe = engine.engine
        tables = wick.OneDTables(cf1d)
        dev = pairs.DeviceForests(fs, pe.device, compact=False)
        keep, _, _ = wick.selection(fs, 1, args.wick_reject)
        stream = torch.cuda.current_stream()
        nb = cparams.num_bins_r_par * cparams.num_bins_r_trans
        z = np.asarray(fs.z, dtype=np.float64)
        zw1 = torch.from_numpy(wick.evolution(z, 2.25, 2.9)).to(pe.device)
        if qs is None:
            offsets, index, _ = pe.neighbours(cparams, dev)
            mask = np.repeat(keep, np.diff(offsets.cpu().numpy()))
            first, second, num = wick.forest_pairs(dev, offsets, index, mask)
            if num == 0:
                out[name] = None
                continue
            used = np.unique(np.concatenate([first[:num].cpu().numpy(),
                                             second[:num].cpu().numpy()]))
            xa, xo, _alive = engine.xi_matrices(dev, tables, used)
            plan = engine.plan_pairs(dev, first, second, num)
            launch = lambda sums: engine.launch_pairs(cparams, dev, zw1, zw1, xo, xa, plan,  # noqa
                                                      sums)
            units = list(zip(first[:num].cpu().numpy(), second[:num].cpu().numpy()))
            work_units = num
        else:
            qdev = pairs.DeviceForests(qs, pe.device)
            offsets, index, total = pe.neighbours(cparams, dev, qdev, xcf=True)
            off_h = offsets.cpu().numpy()
            counts = np.diff(off_h)
            forests = np.nonzero(keep & (counts > 0))[0]
            if forests.size == 0:
                out[name] = None
                continue
            items = (torch.from_numpy(forests.astype(np.int32)).to(pe.device),
                     torch.from_numpy(off_h[forests].astype(np.int32)).to(pe.device),
                     torch.from_numpy(counts[forests].astype(np.int32)).to(pe.device),
                     index, int(forests.size), int(counts[forests].max()))
            xa, xo, _alive = engine.xi_matrices(dev, tables, forests)
            zq = torch.from_numpy(wick.evolution(qs.z_qso, 2.25, 1.44)).to(pe.device)
            launch = lambda sums: engine.launch_items_factored(  # noqa
                cparams, dev, qdev, zw1, zq, xo, xa, items, sums)
            idx_h = index.cpu().numpy()
            units = [(int(f), idx_h[off_h[f]:off_h[f + 1]]) for f in forests]
            work_units = int(forests.size)
        times = []
        for _ in range(2):
            sums = engine.alloc_sums(nb, cross=qs is not None)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            launch(sums)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
            stats = engine.stats()
        kernel_s = times[-1]
        pairs2 = float(stats.visited_pairs)
        # the sweep (auto): one FMA per pair of listed pairs; the factored
        # cross: its GEMM multiply-adds
        flops = 2.0 * (pairs2 if qs is None else float(stats.gemm_macs))
        achieved = flops / kernel_s / 1e12
        cpu_units, cpu_pairs2, desc, cores = wick_cpu_sample(
            fs, qs, cparams, units, cf1d, min(args.cpu_seconds, 15.0), cross=qs is not None)
        unit = "forests/s" if qs is not None else "forest-pairs/s"
        out[name] = {
            "metric": ("cross " if qs is not None else "") + "Wick covariance work per second",
            "value": work_units / kernel_s, "unit": unit,
            "pairs_of_pixel_pairs_per_s": pairs2 / kernel_s, "kernel_ms": kernel_s * 1e3,
            "work": {"units": work_units, "pairs_of_pixel_pairs": pairs2,
                     "bins": f"{cparams.num_bins_r_par} x {cparams.num_bins_r_trans}",
                     "npused": res["NPUSED"], "npall": res["NPALL"]},
            "e2e": {"value": work_units / e2e_s, "unit": unit, "seconds": e2e_s},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak,
                         "peak_source": "cuBLAS DGEMM 4096^3 measured in this run",
                         "achieved_counts": "2 flops (one FMA) per pair of listed pixel pairs"
                         if qs is None else "2 flops per GEMM multiply-add (U^T X U, W^T cW; "
                         "the direct same-quasar sums and the scatter not counted)"},
            "cpu_baseline": {"value": cpu_units, "unit": unit,
                             "pairs_of_pixel_pairs_per_s": cpu_pairs2, "cores": cores,
                             "kind": "port", "sample": desc}}
        del engine, dev
        torch.cuda.empty_cache()
    return out


def xdmat_leg(args, fs, params, ang_max, engine):
    """Delta x quasar distortion matrix (picca_xdmat.py defaults: r_par -200
    to 200, 100 x 50 bins, redshift evolution) of the same forests against
    1.5 quasars per forest on the same area, random rejection
    args.dmat_reject: one warm-up and one timed kernel launch."""
    import torch

    from picca_gb300 import dmat, pairs, synthetic
    if args.config not in ("1", "2"):
        return None
    num, area, _, _ = CONFIGS[args.config]
    half = 20.0 if area <= 4000 else 30.0
    ra_r, dec_r = synthetic.band_for_area(area, half)
    qs = synthetic.make_quasars(int(1.5 * num), 20261207, ra_r, dec_r)
    xparams = dict(params, r_par_min=-200.0, num_bins_r_par=100)
    cparams = pairs.make_params(ang_max=ang_max, x_correlation=True, **xparams)
    dparams = dmat.make_dmat_params(100, 50, alpha2=1.44, product=args.dmat_product)
    xeng = dmat.XDmatEngine(engine.engine)
    pe = xeng.engine
    dev1 = pairs.DeviceForests(fs, pe.device)
    dev2 = pairs.DeviceForests(qs, pe.device)
    offsets, index, total = pe.neighbours(cparams, dev1, dev2, xcf=True)
    offsets_h = offsets.cpu().numpy()
    mask = dmat.selection_mask(fs.healpix_list, fs.row, offsets_h, 1, args.dmat_reject)
    items = dmat.xcf_items(offsets_h, index.cpu().numpy()[:total], mask, dev1.npix)
    ditems = xeng.device_items(*items)
    side = dmat.DmatEngine.side_arrays(dev1, pe.device)
    stream = torch.cuda.current_stream()
    times = []
    for _ in range(2):
        sums = xeng.alloc_sums(cparams, dparams)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        xeng.xaccumulate(cparams, dparams, dev1, dev2, side, ditems, sums)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
        pe.stats()
    kept = int(mask.sum())
    pix_obj = float(np.sum(dev1.npix[items[0]].astype(np.float64) * items[2]))
    del dev1, dev2, sums, side, ditems
    torch.cuda.empty_cache()
    return {"metric": "cross distortion-matrix kept forest-quasar pairs per second",
            "value": kept / times[-1], "unit": "forest-quasar-pairs/s",
            "pixel_quasar_pairs_per_s": pix_obj / times[-1], "kernel_ms": times[-1] * 1e3,
            "config": {"quasars": qs.num, "neighbour_pairs": int(total), "kept_pairs": kept,
                       "work_items": int(len(items[0])),
                       "bins": "100 x 50, r_par -200 to 200 Mpc/h"}}



def continuum_leg(args, cpu_seconds):
    """The plain batched Dr16 fit and the learned warm start.

    A fit is one forest in one outer iteration. Both legs run the same
    number of iterations of the whole Dr16 loop (fits, GPU histograms, host
    updates) on the same forests; the warm-start network is trained first
    on plain fits of a separate set (training time reported separately)."""
    import torch

    from picca_gb300 import continuum, learned, synthetic_spectra
    if args.continuum_forests <= 0:
        return None
    iters = args.continuum_iterations
    eval_raw = synthetic_spectra.make_raw_forests(args.continuum_forests, 20261204)
    train_raw = synthetic_spectra.make_raw_forests(args.continuum_train, 20261205)

    def timed_loop(run):
        torch.cuda.synchronize()
        start = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        start.record()
        out = run()
        end.record()
        torch.cuda.synchronize()
        return out, start.elapsed_time(end) / 1e3

    mixed = continuum.FIT_MIXED
    # warm-up on a small set (module loading, first launches)
    small = synthetic_spectra.make_raw_forests(2000, 7)
    for mode in (mixed, continuum.FIT_FP64):
        eng = continuum.Dr16Gpu(small.grid, num_iterations=2, fit_mode=mode)
        eng.run(continuum.DeviceSpectra(small, eng.device))

    # plain leg: FP32 per-pixel terms, FP64 2x2 Newton solve;
    # fit kernel time measured separately
    eng_p = continuum.Dr16Gpu(eval_raw.grid, num_iterations=iters, fit_mode=mixed)
    spectra = continuum.DeviceSpectra(eval_raw, eng_p.device)
    fit_events = []
    orig_fit = eng_p.fit

    def fit_timed(sp, **kw):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        out = orig_fit(sp, **kw)
        e1.record()
        fit_events.append((e0, e1))
        return out

    eng_p.fit = fit_timed
    plain_fit, plain_s = timed_loop(lambda: eng_p.run(spectra))
    fit_ms = [a.elapsed_time(b) for a, b in fit_events]
    plain = continuum.fit_results_to_host(plain_fit)
    # forests the mixed fit finishes in two-float, on the last model state
    eng_p.fit = orig_fit
    eng_p.fit(spectra, count_refined=True)

    # the same first-iteration fit with every per-pixel term in FP64
    eng_64 = continuum.Dr16Gpu(eval_raw.grid, num_iterations=1)
    eng_32 = continuum.Dr16Gpu(eval_raw.grid, num_iterations=1, fit_mode=mixed)
    f32, _ = timed_loop(lambda: eng_32.fit(spectra))
    f64, fp64_s = timed_loop(lambda: eng_64.fit(spectra))
    f32, f64 = continuum.fit_results_to_host(f32), continuum.fit_results_to_host(f64)
    both = (f32["status"] == 0) & (f64["status"] == 0)
    sc64 = np.maximum(1.0, np.maximum(np.abs(f64["zero_point"]), np.abs(f64["slope"])))
    d_mixed = (np.maximum(np.abs(f32["zero_point"] - f64["zero_point"]),
                          np.abs(f32["slope"] - f64["slope"]))[both] / sc64[both])
    chi_scale = np.maximum(np.abs(f64["chi2"]), f64["ndata"])
    dchi_mixed = (np.abs(f32["chi2"] - f64["chi2"]) / chi_scale)[both]
    del eng_64, eng_32

    # training (separate seed) on plain fits
    eng_t = continuum.Dr16Gpu(train_raw.grid, num_iterations=iters, fit_mode=mixed)
    train = continuum.DeviceSpectra(train_raw, eng_t.device)
    (feats, targs, _), collect_s = timed_loop(lambda: learned.collect_training(eng_t, train))
    net = learned.WarmStartMLP(seed=0)
    hist, train_s = timed_loop(lambda: net.train(feats, targs, epochs=16, batch=4096, lr=2e-3))
    num_samples = int(feats.shape[0])
    del feats, targs, train

    # learned leg on the same evaluation forests
    eng_w = continuum.Dr16Gpu(eval_raw.grid, num_iterations=iters, fit_mode=mixed)
    (warm_fit, stats), warm_s = timed_loop(lambda: learned.run_warm(eng_w, spectra, net))
    warm = continuum.fit_results_to_host(warm_fit)
    ok = (plain["status"] == 0) & (warm["status"] == 0)
    scale = np.maximum(1.0, np.maximum(np.abs(plain["zero_point"]), np.abs(plain["slope"])))
    dab = np.maximum(np.abs(warm["zero_point"] - plain["zero_point"]),
                     np.abs(warm["slope"] - plain["slope"]))[ok] / scale[ok]
    # chi2 sums terms of both signs: relative to max(|chi2|, ndata)
    dchi = (np.abs(warm["chi2"] - plain["chi2"]) /
            np.maximum(np.abs(plain["chi2"]), plain["ndata"]))[ok]
    # learned warm start end to end: the deltas of both fits feed the auto-correlation
    # (50k forests of a contiguous stretch of the survey band)
    e2e_corr = None
    if args.continuum_correlation > 0:
        from picca_gb300 import pairs, pipeline
        from picca_gb300.synthetic import correlation_ang_max
        sel = np.argsort(eval_raw.ra, kind="stable")[:min(args.continuum_correlation,
                                                          eval_raw.num)]
        sel.sort()
        xis = []
        for eng, fit in ((eng_p, plain_fit), (eng_w, warm_fit)):
            delta, weights = eng.deltas(spectra, fit)
            fs = pipeline.forests_from_continuum(eval_raw, delta.cpu().numpy(),
                                                 weights.cpu().numpy(), select=sel)
            ang_max = correlation_ang_max(200.0, float(fs.z.min()))
            params = pairs.make_params(0.0, 200.0, 200.0, 50, 50, ang_max)
            res = pairs.correlate(fs, None, params, mode=pairs.MODE_FP32_GUARD)
            we, xi = res["raw"][0].sum(axis=0), res["raw"][1].sum(axis=0)
            xis.append(np.where(we > 0, xi / np.where(we > 0, we, 1.0), 0.0))
        scale = np.max(np.abs(xis[0]))
        e2e_corr = {"forests": int(sel.size), "bins": int(xis[0].size),
                    "xi_max_abs_diff_over_max_xi": float(np.max(np.abs(xis[1] - xis[0])) / scale),
                    "xi_rms_diff_over_rms_xi": float(np.sqrt(np.mean((xis[1] - xis[0])**2)) /
                                                     np.sqrt(np.mean(xis[0]**2)))}

    # the fit stage alone, plain vs learned, on the same model state at every
    # iteration (the loop advances with the plain fit): each stage is timed
    # with CUDA events, best of three, and the learned stage includes the
    # features, the network, the certified fit and the plain re-fit of the
    # forests that were not certified
    eng_c = continuum.Dr16Gpu(eval_raw.grid, num_iterations=iters, fit_mode=mixed)
    per_iter = []
    for iteration in range(iters):
        best_p, best_w = np.inf, np.inf
        for _ in range(3):
            fp, tp = timed_loop(lambda: eng_c.fit(spectra))
            (fw, _, fb), tw = timed_loop(lambda: learned.warm_fit(eng_c, spectra, net))
            best_p, best_w = min(best_p, tp), min(best_w, tw)
        hp, hw = continuum.fit_results_to_host(fp), continuum.fit_results_to_host(fw)
        both = (hp["status"] == 0) & (hw["status"] == 0)
        sc = np.maximum(1.0, np.maximum(np.abs(hp["zero_point"]), np.abs(hp["slope"])))
        d = np.maximum(np.abs(hw["zero_point"] - hp["zero_point"]),
                       np.abs(hw["slope"] - hp["slope"]))[both] / sc[both]
        dc = ((hw["chi2"] - hp["chi2"]) / np.maximum(np.abs(hp["chi2"]), hp["ndata"]))[both]
        per_iter.append({"plain_ms": best_p * 1e3, "learned_ms": best_w * 1e3,
                         "speedup": best_p / best_w,
                         "fallback_fraction": float(fb.float().mean().item()),
                         "ab_max_rel": float(d.max()) if d.size else None,
                         "chi2_excess_max_rel": float(dc.max()) if dc.size else None,
                         "chi2_abs_max_rel": float(np.abs(dc).max()) if dc.size else None,
                         "status_agree": float(np.mean((hp["status"] == 0) ==
                                                       (hw["status"] == 0)))})
        eng_c.update_model(spectra, fp, iteration == iters - 1)
        del fp, fw
    # the learned stage's parts on the final model state: features, and the
    # network by the fused tcgen05 kernel and by the layer-by-layer GEMMs
    model_c, keep_c = eng_c._model()
    (feat, _), feat_s = timed_loop(lambda: learned.features(eng_c, spectra, model_c))
    net.forward_fused(feat)
    y_fused, fused_s = timed_loop(lambda: net.forward_fused(feat))
    y_gemm, gemm_s = timed_loop(lambda: net.forward(feat))
    _, both_s = timed_loop(lambda: net.warm_start(eng_c, spectra, model_c))
    parts = {"features_and_network_one_kernel_ms": both_s * 1e3,
             "features_ms": feat_s * 1e3, "network_fused_tcgen05_ms": fused_s * 1e3,
             "network_layer_gemms_ms": gemm_s * 1e3,
             "network_fused_vs_gemms_rel_norm": float((y_fused - y_gemm).norm() /
                                                      y_gemm.norm())}
    del feat, y_fused, y_gemm, keep_c
    loop_plain = sum(r["plain_ms"] for r in per_iter)
    loop_learned = sum(r["learned_ms"] for r in per_iter)
    same_state = {"per_iteration": per_iter,
                  "plain_fits_per_s": eval_raw.num * iters / (loop_plain / 1e3),
                  "learned_fits_per_s": eval_raw.num * iters / (loop_learned / 1e3),
                  "learned_over_plain": loop_plain / loop_learned,
                  "ab_max_rel": max(r["ab_max_rel"] or 0.0 for r in per_iter),
                  "chi2_excess_max_rel": max(r["chi2_excess_max_rel"] or 0.0 for r in per_iter),
                  "certificate": {"chi2_tol": learned.CHI2_TOL, "ab_tol": learned.AB_TOL},
                  "learned_stage_parts": parts}
    del eng_c

    nfits = eval_raw.num * iters
    # bytes per forest-fit: 40 n + 32 (n pixels; four FP64 inputs, continuum out)
    npix = float(eval_raw.pix_offset[-1])
    fit_bytes = 40.0 * npix + 32.0 * eval_raw.num
    pk, source = peaks()
    achieved = fit_bytes / (np.mean(fit_ms) / 1e3) / 1e9
    return {
        "forests": eval_raw.num, "iterations": iters,
        "solver": ("damped Newton, warp per forest; FP32 per-pixel terms, exact-product FP32 "
                   "2x2 solve, two-float finish of the forests FP32 rounding could move"),
        "fp64_terms_fit_s": fp64_s, "mixed_vs_fp64_ab_max_rel": float(d_mixed.max()),
        "two_float_finish_fraction": float(eng_p.refined[-1] / eval_raw.num),
        "mixed_vs_fp64_chi2_max_rel": float(dchi_mixed.max()),
        "plain_fits_per_s": nfits / plain_s, "learned_fits_per_s": nfits / warm_s,
        "learned_over_plain": plain_s / warm_s,
        "fallback_rate": float(np.mean([st["fallback"] for st in stats]) / eval_raw.num),
        "newton_iterations_plain_last": float(plain["iterations"].mean()),
        "newton_iterations_learned_last": float(warm["iterations"].mean()),
        "ab_max_rel_diff": float(dab.max()) if dab.size else None,
        "chi2_max_rel_diff": float(dchi.max()) if dchi.size else None,
        "accepted_fraction": float(ok.mean()),
        "fit_kernel_ms_mean": float(np.mean(fit_ms)),
        "fit_roofline": {"bound": "hbm", "achieved": achieved, "peak": pk.get("hbm_gbs"),
                         "unit": "GB/s", "frac": achieved / pk.get("hbm_gbs", 6800.0),
                         "bytes_per_launch": fit_bytes, "peak_source": source},
        "fit_stage_same_model_state": same_state,
        "deltas_to_xi_plain_vs_learned": e2e_corr,
        "training": {"forests": args.continuum_train, "samples": num_samples, "epochs": len(hist),
                     "collect_s": collect_s, "train_s": train_s, "loss_first": hist[0],
                     "loss_last": hist[-1]},
    }


def graph_saving(engine, cparams, dev, offsets, index, order, num_work, num_rows, nbins, mode,
                 sample_items, reps=5):
    """Per-step time of the accumulation on a sample of work items launched
    eagerly (rows zeroed, scratch reset, constants, the kernel) and replayed
    from a CUDA graph (pairs.GraphStep), CUDA events on the current stream."""
    import torch

    from picca_gb300 import pairs
    gen = torch.Generator(device=order.device).manual_seed(2)
    n = min(int(sample_items), int(num_work))
    sub = order[:num_work][torch.randperm(num_work, device=order.device,
                                          generator=gen)[:n]].contiguous()
    rows = engine.alloc_rows(num_rows, nbins)

    def timed(fn):
        out = []
        for _ in range(reps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            out.append(a.elapsed_time(b))
        return float(np.median(out))

    def eager():
        for r in rows:
            r.zero_()
        engine.accumulate(cparams, dev, None, offsets, index, sub, n, rows, mode)

    eager()
    eager_ms = timed(eager)
    g = pairs.GraphStep(engine, cparams, dev, None, offsets, index, sub, n, rows, mode)
    graph_ms = timed(g.replay)
    engine.stats()
    return {"sample_items": n, "eager_ms": eager_ms, "graph_ms": graph_ms,
            "saving_ms_per_step": eager_ms - graph_ms,
            "note": "a full step is one long kernel: the launch overhead a graph removes is "
                    "this saving per step"}


def survey_quasars(cfg, fs):
    """Quasar catalogue of a workload: 600k on the 8,000 deg^2 band (75 per
    deg^2, the forests' z law), 1.5 per forest otherwise, same area."""
    from picca_gb300 import synthetic
    num, area, _, _ = CONFIGS[cfg]
    if area is None:  # the patch of the CPU-runnable case
        ra_r = tuple(np.degrees([np.min(fs.ra), np.max(fs.ra)]))
        dec_r = tuple(np.degrees([np.min(fs.dec), np.max(fs.dec)]))
    else:
        ra_r, dec_r = synthetic.band_for_area(area, 20.0 if area <= 4000 else 30.0)
    return synthetic.make_quasars(int(1.5 * num), 20261207, ra_r, dec_r)


def xcf_cpu_sample(fs, qs, p_or, ang_max, seconds):
    """The CPU oracle's xcf (neighbours + pixel-quasar pairs) on a bounded
    random sample of forests with all their quasars, on every host core.
    Returns (candidate pixel-quasar pairs/s, description, threads)."""
    from oracle import cpu as oracle
    rng = np.random.default_rng(11)
    cores = os.cpu_count() or 1
    npix = np.diff(fs.pix_offset)
    per_forest = float(np.mean(npix)) * 2500.0
    n = int(max(cores, min(fs.num, seconds * 1.5e8 * cores / per_forest)))
    sample = np.sort(rng.choice(fs.num, size=min(n, fs.num), replace=False))
    sub = fs.take(sample)
    t0 = time.perf_counter()
    offsets, index = oracle.neighbours(sub, qs, p_or, ang_max, auto_mode=0, xcf=True)
    oracle.rows(sub, qs, p_or, offsets, index, xcf=True)
    elapsed = time.perf_counter() - t0
    cand = int((npix[sample] * np.diff(offsets)).sum())
    return cand / elapsed, (f"{len(sample)} random forests with all their quasars, C "
                            f"restatement of xcf.compute_xi_forest_pairs_fast; {elapsed:.1f} s"), cores


def xcf_leg(args, fs, ang_max, steps, warmup):
    """The delta x quasar cross-correlation of the same forests (picca_xcf.py:
    r_par -200 to 200 in 100 bins x r_trans 0-200 in 50), precision form: a
    step is quasar neighbours + pixel-quasar pairs of the whole survey. Per
    bin error against the plain FP64 kernel on 1% of the forests, FP32
    roofline of the pair kernel, and the CPU oracle on a sample."""
    import torch

    from oracle import cpu as oracle
    from picca_gb300 import pairs
    qs = survey_quasars(args.config, fs)
    kw = dict(r_par_min=-200.0, r_par_max=200.0, r_trans_max=200.0, num_bins_r_par=100,
              num_bins_r_trans=50)
    params = pairs.make_params(ang_max=ang_max, x_correlation=True, **kw)
    engine = pairs.PairEngine()
    d1 = pairs.DeviceForests(fs, engine.device)
    d2 = pairs.DeviceForests(qs, engine.device)
    nrows, nbins = len(fs.healpix_list), 5000
    stream = torch.cuda.current_stream()

    def step(kern=None):
        offsets, index, total = engine.neighbours(params, d1, d2, xcf=True)
        order, num_work, cand = engine.work_order(d1, d2, offsets, index, total, xcf=True)
        rows = engine.alloc_rows(nrows, nbins)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        engine.accumulate(params, d1, d2, offsets, index, order, num_work, rows,
                          pairs.MODE_FP32_GUARD, xcf=True)
        e1.record(stream)
        if kern is not None:
            kern.append((e0, e1))
        return rows, cand, (offsets, index, order, num_work)

    tuning = None
    if args.tune_items > 0:
        from picca_gb300 import autotune
        offsets_t, index_t, total_t = engine.neighbours(params, d1, d2, xcf=True)
        order_t, num_work_t, _ = engine.work_order(d1, d2, offsets_t, index_t, total_t,
                                                   xcf=True)
        tuning = autotune.tune_pairs(engine, params, d1, d2, offsets_t, index_t, order_t,
                                     num_work_t, nrows, pairs.MODE_FP32_GUARD, xcf=True,
                                     grid=CONFIGS[args.config][2],
                                     sample_items=4 * args.tune_items)
        del offsets_t, index_t, order_t
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    kern = []
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(steps):
        rows, cand, work = step(kern)
    t1.record(stream)
    torch.cuda.synchronize()
    elapsed = t0.elapsed_time(t1) / 1e3
    kmean = float(np.mean([a.elapsed_time(b) / 1e3 for a, b in kern]))
    accepted = int(rows[5].sum().item())
    check = precision_check(engine, params, d1, d2, work, nrows, nbins, args.check_fraction,
                            xcf=True)
    pk, source = peaks()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    fp32_peak = sms * 128 * 2 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    flops = 10.0 * cand + 9.0 * accepted
    p_or = oracle.make_params(**kw, x_correlation=True)
    cpu_val, cpu_desc, cores = xcf_cpu_sample(fs, qs, p_or, ang_max, min(args.cpu_seconds, 10.0))
    out = {
        "metric": "xcf candidate pixel-quasar pairs per second (precision form)",
        "value": cand * steps / elapsed, "unit": "pixel-quasar-pairs/s",
        "steps": steps, "warmup": warmup, "ms_per_step": elapsed / steps * 1e3,
        "config": {"workload": f"{fs.num} forests x {qs.num} quasars, r_par -200 to 200 "
                               "(100 bins) x r_trans 0-200 (50 bins) Mpc/h",
                   "candidate_pixel_quasar_pairs_per_step": int(cand),
                   "accepted_pairs_per_step": accepted},
        "roofline": {"bound": "fp32", "achieved": flops / kmean / 1e12, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": flops / kmean / 1e12 / fp32_peak,
                     "traffic": None, "kernel_ms": kmean * 1e3,
                     "peak_source": f"SMs x 128 FP32 lanes x 2 x sm_max_mhz ({source} peaks file)"},
        "precision_check_vs_fp64_kernel": check,
        "tuning": tuning,
        "cpu_baseline": {"value": cpu_val, "unit": "pixel-quasar-pairs/s", "cores": cores,
                         "kind": "port", "sample": cpu_desc},
    }
    del engine, d1, d2
    torch.cuda.empty_cache()
    return out


def precision_check(engine, params, d1, d2, work, nrows, nbins, fraction, xcf=False):
    """The precision form against the plain all-FP64 kernel on a random
    `fraction` of the work items: pair counts, per-bin relative errors of
    xi, the weights and the r_par / r_trans / z sums (bins with pairs), and
    both kernels' rates on the sample."""
    import torch

    from picca_gb300 import pairs
    offsets, index, order, num_work = work
    n_check = max(1, int(num_work * fraction))
    gen = torch.Generator(device=order.device).manual_seed(3)
    sub = order[:num_work][torch.randperm(num_work, device=order.device,
                                          generator=gen)[:n_check]].contiguous()
    sample_cand = int(engine.last_cost[sub.long()].sum().item())
    stream = torch.cuda.current_stream()
    r32 = engine.alloc_rows(nrows, nbins)
    r64 = engine.alloc_rows(nrows, nbins)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record(stream)
    engine.accumulate(params, d1, d2, offsets, index, sub, n_check, r32, pairs.MODE_FP32_GUARD,
                      xcf=xcf)
    ev[1].record(stream)
    ev[2].record(stream)
    engine.accumulate(params, d1, d2, offsets, index, sub, n_check, r64, pairs.MODE_FP64, xcf=xcf)
    ev[3].record(stream)
    torch.cuda.synchronize()
    fast_s = ev[0].elapsed_time(ev[1]) / 1e3
    fp64_s = ev[2].elapsed_time(ev[3]) / 1e3
    a = [r.cpu().numpy() for r in r32]
    b = [r.cpu().numpy() for r in r64]
    has = b[5] > 0

    def rel(k):
        return np.abs(a[k][has] - b[k][has]) / np.maximum(np.abs(b[k][has]), 1e-300)

    def norm_abs(k):  # the normalised mean (sum / weights): r_par, r_trans in Mpc/h, z
        return np.abs(a[k][has] / a[0][has] - b[k][has] / b[0][has])

    xi = rel(1)
    xi_n = np.abs(a[1][has] / a[0][has] - b[1][has] / b[0][has]) / np.maximum(
        np.abs(b[1][has] / b[0][has]), 1e-300)
    return {
        "work_items_checked": int(n_check), "bins_with_pairs": int(has.sum()),
        "nb_identical": bool(np.array_equal(a[5], b[5])),
        "xi_max_rel": float(xi.max()), "xi_p99_rel": float(np.percentile(xi, 99)),
        "xi_median_rel": float(np.median(xi)),
        "xi_normalised_max_rel": float(xi_n.max()),
        "we_max_rel": float(rel(0).max()), "we_p99_rel": float(np.percentile(rel(0), 99)),
        "r_par_max_abs_mpc": float(norm_abs(2).max()),
        "r_trans_max_abs_mpc": float(norm_abs(3).max()), "z_max_abs": float(norm_abs(4).max()),
        "sample_candidate_pixel_pairs": sample_cand,
        "precision_form_pairs_per_s_on_sample": sample_cand / fast_s,
        "plain_fp64_kernel_pairs_per_s_on_sample": sample_cand / fp64_s,
        "precision_form_over_fp64_kernel": fp64_s / fast_s,
    }


def delta_dict(fs):
    """{healpix: [Delta]} of a ForestSet (what picca_cf.py holds after
    reading the delta files): objects whose pixel arrays are views into the
    set's arrays, in the set's order."""
    from picca_gb300 import deltaio
    arrays = {"pix_offset": np.asarray(fs.pix_offset), "ra": fs.ra, "dec": fs.dec,
              "z_qso": fs.z_qso, "plate": fs.plate, "mjd": np.zeros(fs.num, dtype=np.int64),
              "fiberid": fs.fiberid, "los_id": fs.thingid, "z": fs.z, "r_comov": fs.r_comov,
              "dist_m": fs.dist_m, "weights": fs.weights, "log_lambda": fs.log_lambda,
              "delta": fs.delta, "cont": np.ones(fs.num_pixels)}
    deltas = deltaio.make_deltas(arrays, 1)
    out = {}
    for hp, d in zip(np.asarray(fs.healpix).tolist(), deltas):
        out.setdefault(hp, []).append(d)
    return out


def reference_step_seconds(args):
    """CPU time of one reference step: the whole --steps/--warmup run stays
    within a few minutes."""
    return float(min(args.cpu_seconds, max(2.0, 150.0 / max(args.steps, 1))))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    fs, params, ang_max = make_workload(args.config)
    seconds = reference_step_seconds(args)
    vals = []
    for _ in range(args.warmup):
        cpu_sample(fs, params, ang_max, min(2.0, seconds), args.config)
    desc, cores = "", 1
    step_ms = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        v, desc, cores = cpu_sample(fs, params, ang_max, seconds, args.config)
        step_ms.append((time.perf_counter() - t0) * 1e3)
        vals.append(v)
    value = float(np.median(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "pixel-pairs/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        # a step is one bounded sample of the workload (``sample`` below)
        "ms_per_step": float(np.median(step_ms)), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(args.config), "bins": "50x50",
                   "r_par": "0-200", "r_trans": "0-200"},
        "cpu_baseline": {"value": value, "unit": "pixel-pairs/s", "cores": cores,
                         "kind": "port", "sample": desc + " (median over steps)"},
        "e2e": {"value": value, "unit": "pixel-pairs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_name(cfg):
    return (CONFIGS[cfg][3] + ", auto-correlation 50x50 bins, r_par 0-200, r_trans 0-200 "
            "Mpc/h")


def run_ours(args):
    import torch
    import torch.distributed as dist

    from picca_gb300 import pairs

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    if args.continuum_only:
        if rank == 0:
            print(json.dumps(continuum_leg(args, args.cpu_seconds)), flush=True)
        return
    fs, params, ang_max = make_workload(args.config)
    if args.wick_only:
        if rank == 0:
            print(json.dumps(wick_leg(args, fs, params, ang_max)), flush=True)
        return
    if args.dmat_only:
        if rank == 0:
            print(json.dumps(dmat_leg(args, fs, params, ang_max, args.cpu_seconds)), flush=True)
        return
    legs = set(x for x in args.legs.split(",") if x)
    mode = pairs.MODE_FP32_GUARD if args.precision == "fp32_guard" else pairs.MODE_FP64
    cparams = pairs.make_params(ang_max=ang_max, **params)
    engine = pairs.PairEngine()
    packed = pairs.pack_host(fs, pinned=True)
    dev = pairs.DeviceForests(fs, engine.device, packed=packed)
    nbins = params["num_bins_r_par"] * params["num_bins_r_trans"]
    num_rows = len(fs.healpix_list)
    stream = torch.cuda.current_stream()

    def step(timings=None, device_forests=dev):
        offsets, index, total = engine.neighbours(cparams, device_forests)
        order, num_work, cand = engine.work_order(device_forests, None, offsets, index, total)
        rows = engine.alloc_rows(num_rows, nbins)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        engine.accumulate(cparams, device_forests, None, offsets, index, order, num_work, rows,
                          mode)
        ev1.record(stream)
        if timings is not None:
            timings.append((ev0, ev1))
        return rows, cand, total, (offsets, index, order, num_work)

    if args.profile_items > 0:
        offsets, index, total = engine.neighbours(cparams, dev)
        order, num_work, _ = engine.work_order(dev, None, offsets, index, total)
        gen = torch.Generator(device=order.device).manual_seed(1)
        n = min(args.profile_items, num_work)
        sub = order[:num_work][torch.randperm(num_work, device=order.device,
                                              generator=gen)[:n]].contiguous()
        cand = int(engine.last_cost[sub.long()].sum().item())
        rows = engine.alloc_rows(num_rows, nbins)
        engine.accumulate(cparams, dev, None, offsets, index, sub, n, rows, mode)
        torch.cuda.synchronize()
        print(json.dumps({"profile_items": n, "candidate_pixel_pairs": cand,
                          "workload": CONFIGS[args.config][3]}), flush=True)
        return

    # launch shape of the pair kernel, tuned on a sample of the work items
    # (cached per device, bins, grid and mode), and the CUDA-graph replay of
    # a step on the same sample against its eager launches
    tuning, graph_info = None, None
    if mode != pairs.MODE_FP64 and args.tune_items > 0:
        from picca_gb300 import autotune
        offsets_t, index_t, total_t = engine.neighbours(cparams, dev)
        order_t, num_work_t, _ = engine.work_order(dev, None, offsets_t, index_t, total_t)
        tuning = autotune.tune_pairs(engine, cparams, dev, None, offsets_t, index_t, order_t,
                                     num_work_t, num_rows, mode, grid=CONFIGS[args.config][2],
                                     sample_items=args.tune_items)
        graph_info = graph_saving(engine, cparams, dev, offsets_t, index_t, order_t, num_work_t,
                                  num_rows, nbins, mode, args.tune_items)
        del offsets_t, index_t, order_t

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # device-resident timed region
    kern = []
    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    cands = []
    for _ in range(args.steps):
        rows, cand, total, work = step(kern)
        cands.append(cand)
    t_end.record(stream)
    barrier()
    clocks = sampler.stop()
    elapsed = t_start.elapsed_time(t_end) / 1e3
    kernel_s = [a.elapsed_time(b) / 1e3 for a, b in kern]
    stats = engine.stats()
    if world > 1:
        t = torch.tensor([elapsed], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    pairs_per_step = cands[0]
    value = pairs_per_step * args.steps * world / elapsed
    accepted = int(rows[5].sum().item())

    # FP64 error report on a sample of work items (plain FP64 kernel vs ours)
    check = {}
    if mode != pairs.MODE_FP64 and args.check_fraction > 0:
        check = precision_check(engine, cparams, dev, None, work, num_rows, nbins,
                                args.check_fraction)
    offsets_w = index_w = order_w = None
    del work, rows, offsets_w, index_w, order_w
    num_pixels, resident_bytes = int(dev.num_pixels), int(dev.h2d_bytes)
    del dev, packed
    torch.cuda.empty_cache()

    # end to end through the drop-in cf module: {healpix: [Delta]} on the
    # host -> packing, pinned upload, neighbours, pairs, rows and neighbour
    # lists back, every step
    from picca_gb300 import cf as cfmod
    data = delta_dict(fs)
    cfmod.data, cfmod.data2 = data, None
    cfmod.r_par_min, cfmod.r_par_max = params["r_par_min"], params["r_par_max"]
    cfmod.r_trans_max = params["r_trans_max"]
    cfmod.num_bins_r_par, cfmod.num_bins_r_trans = params["num_bins_r_par"], params["num_bins_r_trans"]
    cfmod.z_min_pairs = cfmod.z_max_pairs = cfmod.zerr_cut_deg = cfmod.zerr_cut_kms = None
    cfmod.ang_max, cfmod.nside = ang_max, 16
    cfmod.x_correlation = cfmod.rmu_binning = cfmod.ang_correlation = False
    cfmod.remove_same_half_plate_close_pairs = False
    cfmod.precision = args.precision
    barrier()
    e2e_steps = max(1, args.e2e_steps)
    h2d = d2h = 0
    e2e_t0 = time.perf_counter()
    for _ in range(e2e_steps):
        cfmod._cache["key"] = None
        cfmod._cache["result"] = None
        res_e = cfmod.compute_xi_all()
        h2d, d2h = res_e["h2d_bytes"], res_e["d2h_bytes"]
    torch.cuda.synchronize()
    e2e_elapsed = time.perf_counter() - e2e_t0
    e2e_cand = res_e["candidate_pairs"]
    e2e_nb_same = None
    del res_e
    cfmod._cache["result"] = None
    cfmod.data = None
    del data
    if world > 1:
        t = torch.tensor([e2e_elapsed], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_elapsed = float(t.item())
    e2e_value = e2e_cand * e2e_steps * world / e2e_elapsed

    # roofline of the pair kernel (FP32 CUDA-core bound)
    pk, source = peaks()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    flops = 10.0 * pairs_per_step + 9.0 * accepted
    kmean = float(np.mean(kernel_s))
    achieved = flops / kmean / 1e12
    fp32_peak = sms * 128 * 2 * pk.get("sm_max_mhz", 2070.0) * 1e6 / 1e12
    launches_per_step = 2 + (5 if mode != pairs.MODE_FP64 else 1)

    if rank != 0:
        return
    cpu_val, cpu_desc, cores = cpu_sample(fs, params, ang_max, args.cpu_seconds, args.config)
    del engine
    torch.cuda.empty_cache()
    extra = {}
    if "xcf" in legs:
        extra["xcf"] = xcf_leg(args, fs, ang_max, min(args.steps, 5), min(args.warmup, 2))
        print("xcf leg: " + json.dumps(extra["xcf"]), file=sys.stderr, flush=True)
    if "dmat" in legs:
        extra["dmat"] = dmat_leg(args, fs, params, ang_max, args.cpu_seconds)
        print("dmat leg: " + json.dumps(extra["dmat"]), file=sys.stderr, flush=True)
    if "wick" in legs:
        extra["wick"] = wick_leg(args, fs, params, ang_max)
        print("wick leg: " + json.dumps(extra["wick"]), file=sys.stderr, flush=True)
    if "delta_io" in legs:
        extra["delta_io"] = delta_io_leg(fs)
        print("delta io leg: " + json.dumps(extra["delta_io"]), file=sys.stderr, flush=True)
    if "continuum" in legs:
        extra["continuum"] = continuum_leg(args, args.cpu_seconds)
        print("continuum leg: " + json.dumps(extra["continuum"]), file=sys.stderr, flush=True)
    line = {
        "metric": METRIC, "value": value, "unit": "pixel-pairs/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64guard"
        if mode != pairs.MODE_FP64 else "f64", "data": "synthetic",
        "config": {"workload": workload_name(args.config), "forests": fs.num,
                   "pixels": num_pixels, "forest_pairs": int(total),
                   "candidate_pixel_pairs_per_step": int(pairs_per_step),
                   "accepted_pixel_pairs_per_step": accepted, "precision": args.precision,
                   "l2": "inputs larger than L2 (%.1f GB resident)" % (resident_bytes / 1e9),
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_value, "unit": "pixel-pairs/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                "path": "cf.compute_xi_all from {healpix: [Delta]} host objects (packing, "
                        "pinned upload, neighbours, pairs, rows and neighbour lists back)"},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                     "traffic": PAIR_DRAM_BYTES_PER_CANDIDATE * pairs_per_step
                     if PAIR_DRAM_BYTES_PER_CANDIDATE else None,
                     "traffic_source": PAIR_TRAFFIC_SOURCE,
                     "kernel_ms": kmean * 1e3,
                     "peak_source": f"SMs x 128 FP32 lanes x 2 x sm_max_mhz ({source} peaks file)",
                     "flops_per_launch": flops},
        "precision_check_vs_fp64_kernel": check,
        "tuning": tuning,
        "graph": graph_info,
        "rechecked_pairs_last_step": int(stats.rechecked_pairs),
        "evaluated_pixel_pairs_last_step": int(stats.visited_pairs),
        "clocks": clocks,
        "cpu_baseline": {"value": cpu_val, "unit": "pixel-pairs/s", "cores": cores,
                         "kind": "port", "sample": cpu_desc},
    }
    line.update(extra)
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
