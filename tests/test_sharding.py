"""Healpix sharding of the pair accumulation over two processes (gloo on
CPU): the union of the ranks' rows equals the unsharded rows bit for bit.
The per-rank accumulation uses the CPU oracle, so this checks the host
logic of the multi-process path (assignment, work selection, gather)."""

import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _workload():
    from picca_gb300 import synthetic
    from oracle import cpu as oracle
    fs = synthetic.make_forests(240, 5, (150.0, 154.0), (0.0, 4.0), 2.1, 3.5, "uniform")
    ang_max = synthetic.correlation_ang_max(200.0, float(fs.z.min()))
    params = oracle.make_params(0.0, 200.0, 200.0, 20, 20)
    offsets, index = oracle.neighbours(fs, fs, params, ang_max, auto_mode=1)
    return fs, params, offsets, index


def _rank_rows(rank, world, port, out_path):
    import torch.distributed as dist
    from oracle import cpu as oracle
    from picca_gb300 import sharding
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    fs, params, offsets, index = _workload()
    num_rows = len(fs.healpix_list)
    npix = np.diff(fs.pix_offset)
    cost = np.array([npix[f] * npix[index[offsets[f]:offsets[f + 1]]].sum()
                     for f in range(fs.num)], dtype=float)
    owned = sharding.assign_rows(sharding.row_costs(num_rows, fs.row, cost), world)
    mine = sharding.shard_forests(fs.row, owned[rank])
    nbins = 400
    acc = [np.zeros((num_rows, nbins)) for _ in range(5)] + [
        np.zeros((num_rows, nbins), dtype=np.int64)]
    # forests are sorted by healpix row: each owned row is one forest range,
    # accumulated in the same order as the single-process run
    for r in owned[rank]:
        forests = mine[np.asarray(fs.row)[mine] == r]
        if forests.size == 0:
            continue
        f0, f1 = int(forests[0]), int(forests[-1]) + 1
        assert f1 - f0 == forests.size
        # the oracle indexes offsets from f_begin
        part = oracle.rows(fs, fs, params, offsets[f0:], index, f_begin=f0, f_end=f1)
        for a, p in zip(acc, part):
            a += p
    full = sharding.gather_rows(acc, owned[rank], num_rows)
    if rank == 0:
        np.savez(out_path, *full)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gather_equals_single_process(tmp_path):
    import socket
    import torch.multiprocessing as mp
    from oracle import cpu as oracle
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "rows.npz")
    mp.start_processes(_rank_rows, args=(2, port, out), nprocs=2, start_method="spawn")
    fs, params, offsets, index = _workload()
    ref = oracle.rows(fs, fs, params, offsets, index)
    got = np.load(out)
    for k, r in enumerate(ref):
        assert np.array_equal(got[f"arr_{k}"], r), k


def test_assignment_covers_every_row_once():
    from picca_gb300 import sharding
    cost = np.array([5.0, 1.0, 3.0, 3.0, 0.0, 8.0])
    owned = sharding.assign_rows(cost, 3)
    rows = np.sort(np.concatenate(owned))
    assert np.array_equal(rows, np.arange(6))
    loads = [cost[o].sum() for o in owned]
    assert max(loads) - min(loads) <= cost.max()


def _wick_workload():
    from picca_gb300 import synthetic
    from oracle import wick as ow
    fs = synthetic.make_forests(120, 9, (150.0, 152.0), (0.0, 2.0), 2.1, 3.5, "uniform",
                                max_pixels=160)
    ang_max = synthetic.correlation_ang_max(60.0, float(fs.z.min()))
    return fs, ow.make_params(0.0, 60.0, 60.0, 15, 15), ang_max


def _wick_partial(fs, p, ang_max, forests_subset):
    """The oracle's raw Wick sums over the kept forests in ``forests_subset``
    (the per-forest draws made exactly as a single process makes them)."""
    from conftest import golden
    from oracle import cpu
    from oracle import wick as ow
    offsets, index = cpu.neighbours(fs, fs, cpu.make_params(0.0, 60.0, 60.0, 15, 15), ang_max,
                                    auto_mode=1)
    keep, npall, npused = ow.selection(fs, 2, 0.6)
    variance, xi = ow.interpolants(golden("cf1d.npz"))
    po = np.asarray(fs.pix_offset)
    out = ow.new_outputs(p)

    def forest(f):
        sl = slice(po[f], po[f + 1])
        return (fs.r_comov[sl], fs.weights[sl], ((1 + fs.z[sl]) / 3.25) ** 1.9,
                ow.weighted_xi_1d(fs.log_lambda[sl], fs.weights[sl], variance, xi))

    for f in np.nonzero(keep)[0]:
        if f not in forests_subset:
            continue
        r1, w1, zw1, x1 = forest(f)
        for k in range(int(offsets[f]), int(offsets[f + 1])):
            g = int(index[k])
            r2, w2, zw2, x2 = forest(g)
            ang = cpu.lib().oracle_angle(fs.x_cart[f], fs.y_cart[f], fs.z_cart[f], fs.ra[f],
                                         fs.dec[f], fs.cos_dec[f], fs.x_cart[g], fs.y_cart[g],
                                         fs.z_cart[g], fs.ra[g], fs.dec[g])
            ow.forest_pair(p, r1, w1, zw1, x1, r2, w2, zw2, x2, ang, out)
    return out, npall, npused


def _rank_wick(rank, world, port, out_path):
    import sys
    import torch.distributed as dist
    from picca_gb300 import sharding
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    fs, p, ang_max = _wick_workload()
    owned = sharding.assign_rows(sharding.row_costs(len(fs.healpix_list), fs.row,
                                                    np.diff(fs.pix_offset)), world)
    mine = set(int(f) for f in sharding.shard_forests(fs.row, owned[rank]))
    raw, _, _ = _wick_partial(fs, p, ang_max, mine)
    keys = ("weights_wick", "num_pairs_wick", "t1", "t2", "t3")
    total = sharding.reduce_sums([raw[k] for k in keys])
    if rank == 0:
        np.savez(out_path, **dict(zip(keys, total)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_wick_sums_equal_single_process(tmp_path):
    """Kept forests split by healpix over two gloo ranks, partial Wick sums
    reduced: the single-process sums (NB exact, FP64 sums to rounding)."""
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "wick.npz")
    mp.start_processes(_rank_wick, args=(2, port, out), nprocs=2, start_method="spawn")
    fs, p, ang_max = _wick_workload()
    ref, _, _ = _wick_partial(fs, p, ang_max, set(range(fs.num)))
    got = np.load(out)
    assert ref["num_pairs_wick"].sum() > 0
    assert np.array_equal(got["num_pairs_wick"], ref["num_pairs_wick"])
    for key in ("weights_wick", "t1", "t2", "t3"):
        scale = np.abs(ref[key]).max()
        assert np.all(np.abs(got[key] - ref[key]) <= 1e-12 * np.abs(ref[key]) + 1e-14 * scale)
