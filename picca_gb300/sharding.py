"""Splitting a correlation over processes (one per GPU) by healpix.

A forest pair contributes only to the row of the first forest's healpix
(py/picca/cf.py:161-240; rows per healpix, py/picca/bin/picca_cf.py:454-473),
so a partition of the healpix rows gives independent shards: a rank
accumulates the rows of its healpix, reading the other forests only as
neighbours, and the full result is the union of disjoint rows. Nothing is
reduced; :func:`gather_rows` only assembles the rows for the output file.

Rows are dealt out longest-first to the least-loaded rank (LPT), with the
number of candidate pixel pairs of a row as its cost. The distortion, metal
and Wick matrices are sums over kept forest pairs instead of rows: the same
split of the kept forests by healpix applies, and :func:`reduce_sums` adds
the ranks' un-normalised sums once at the end.
"""

import numpy as np


def row_costs(num_rows, forest_rows, forest_cost):
    """Cost of each healpix row: the sum of its forests' costs."""
    cost = np.zeros(num_rows, dtype=np.float64)
    np.add.at(cost, np.asarray(forest_rows, dtype=np.int64), np.asarray(forest_cost, float))
    return cost


def assign_rows(cost, world):
    """LPT assignment of rows to ``world`` ranks; returns a list of sorted
    row-index arrays (every row exactly once)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = np.argsort(-np.asarray(cost, dtype=np.float64), kind="stable")
    load = np.zeros(world)
    owned = [[] for _ in range(world)]
    for row in order:
        rank = int(np.argmin(load))
        owned[rank].append(int(row))
        load[rank] += cost[row]
    return [np.array(sorted(rows), dtype=np.int64) for rows in owned]


def shard_forests(forest_rows, rows):
    """Indices of the forests (work items) whose row belongs to ``rows``."""
    mask = np.isin(np.asarray(forest_rows, dtype=np.int64), rows)
    return np.nonzero(mask)[0].astype(np.int32)


def gather_rows(arrays, rows, num_rows, group=None):
    """Assemble disjoint per-rank rows into full [num_rows, nbins] arrays on
    every rank (torch.distributed; any backend). ``arrays`` are this rank's
    full-size row arrays, zero outside ``rows``. Because the shards are
    disjoint, adding the ranks' arrays places each row unchanged (x + 0 =
    x exactly)."""
    import torch
    import torch.distributed as dist
    out = []
    for arr in arrays:
        t = torch.as_tensor(np.ascontiguousarray(arr))
        if t.dtype not in (torch.float64, torch.int64):
            raise TypeError("rows are float64 or int64")
        mask = np.zeros(num_rows, dtype=bool)
        mask[rows] = True
        t = t.clone()
        t[torch.as_tensor(~mask)] = 0
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        out.append(t.numpy())
    return out


def reduce_sums(arrays, group=None):
    """Total of per-rank partial sums on every rank (torch.distributed
    all_reduce, SUM; any backend). The distortion matrices, the metal
    matrices and the Wick terms are sums over kept forest pairs rather than
    per-healpix rows (py/picca/bin/picca_dmat.py:487-494,
    py/picca/bin/picca_wick.py:515-530 add the process chunks' tuples), so
    splitting the kept forests over ranks needs one reduction of the
    un-normalised sums at the end; the random draws are made identically on
    every rank before the split, so the kept pairs are the single-process
    ones."""
    import torch
    import torch.distributed as dist
    out = []
    for arr in arrays:
        t = torch.as_tensor(np.ascontiguousarray(arr)).clone()
        if t.dtype not in (torch.float64, torch.int64):
            raise TypeError("sums are float64 or int64")
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        out.append(t.numpy())
    return out
