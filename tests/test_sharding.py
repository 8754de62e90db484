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
