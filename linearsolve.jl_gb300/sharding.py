"""Multi-GPU sharding of independent work (batched systems, serving keys).

Batched systems and served requests are independent, so N GPUs take disjoint
shards with no exchange on the data path; only the host gathers results.
Systems are assigned greedily, largest first, to the rank with the least LU
work so far (work ~ n^3), which balances uneven sizes; serving keys are
assigned the same way by their size (affinity: a key's factorization lives
on one GPU).
"""
from __future__ import annotations

import numpy as np


def shard_systems(sizes, world: int):
    """Return a list of index arrays, one per rank, covering every system once."""
    sizes = np.asarray(sizes, dtype=np.int64)
    order = np.argsort(-sizes, kind="stable")
    load = np.zeros(world, dtype=np.float64)
    parts = [[] for _ in range(world)]
    for i in order:
        r = int(np.argmin(load))
        parts[r].append(int(i))
        load[r] += float(sizes[i]) ** 3
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def pack(sizes, A, b, idx):
    """Sub-batch (sizes, A_packed, b_packed) of the systems in idx."""
    sizes = np.asarray(sizes, dtype=np.int64)
    a_off = np.zeros(len(sizes), dtype=np.int64)
    b_off = np.zeros(len(sizes), dtype=np.int64)
    if len(sizes) > 1:
        a_off[1:] = np.cumsum(sizes[:-1] ** 2)
        b_off[1:] = np.cumsum(sizes[:-1])
    sub_sizes = sizes[idx]
    A_sub = np.concatenate([A[a_off[i]:a_off[i] + sizes[i] ** 2] for i in idx]) if len(idx) else np.zeros(0)
    b_sub = np.concatenate([b[b_off[i]:b_off[i] + sizes[i]] for i in idx]) if len(idx) else np.zeros(0)
    return sub_sizes, A_sub, b_sub


def gpu_solve_fn(ctx, precision: str = "fp64"):
    """solve_fn for solve_distributed: the shard through the batched kernels
    of this rank's GPU (one graph launch)."""
    from .device import Batch

    def solve(ss, As, bs):
        bt = Batch(ctx, ss, precision)
        try:
            x = bt.solve(As, bs)
            if (bt.info != 0).any():
                raise RuntimeError("singular system in the shard")
            return x
        finally:
            bt.close()
    return solve


def shard_keys(key_sizes, world: int):
    """Serving affinity: key -> rank, balancing sum n^3 over the ranks
    (largest keys first), so each key's factorization lives on one GPU."""
    order = sorted(range(len(key_sizes)), key=lambda k: -int(key_sizes[k]))
    load = [0.0] * world
    owner = [0] * len(key_sizes)
    for k in order:
        r = min(range(world), key=lambda i: load[i])
        owner[k] = r
        load[r] += float(key_sizes[k]) ** 3
    return owner


def solve_distributed(sizes, A, b, rank: int, world: int, solve_fn, group=None):
    """Each rank solves its shard with solve_fn(sub_sizes, A_sub, b_sub) -> x_sub;
    the shards are gathered on every rank (torch.distributed all_gather_object)
    and reassembled in the original order."""
    import torch.distributed as dist
    parts = shard_systems(sizes, world)
    idx = parts[rank]
    ss, As, bs = pack(sizes, A, b, idx)
    x_sub = solve_fn(ss, As, bs) if len(idx) else np.zeros(0)
    gathered = [None] * world
    dist.all_gather_object(gathered, (idx, np.asarray(x_sub)), group=group)
    sizes = np.asarray(sizes, dtype=np.int64)
    b_off = np.zeros(len(sizes), dtype=np.int64)
    if len(sizes) > 1:
        b_off[1:] = np.cumsum(sizes[:-1])
    x = np.empty(int(sizes.sum()), dtype=np.float64)
    for ridx, rx in gathered:
        pos = 0
        for i in ridx:
            n = int(sizes[i])
            x[b_off[i]:b_off[i] + n] = rx[pos:pos + n]
            pos += n
    return x
