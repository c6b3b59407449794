"""Sharding an ensemble across processes (one per GPU).

Realizations are independent and every random number is keyed by the
realization id, so a shard [offset, offset + count) of an ensemble draws
exactly the streams it would draw in one call.  Each rank runs its range
with no exchange on the data path; the only exchange is one all-gather of
(count, mean, stddev) per tracked species and grid point at the end, merged
with tl_merge_moments (Chan, Golub, LeVeque pairwise update).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _ffi as F


def shard_range(total: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous split of `total` realizations: (offset, count) of `rank`."""
    base, rem = divmod(total, world)
    count = base + (1 if rank < rem else 0)
    offset = rank * base + min(rank, rem)
    return offset, count


def merge_moments(counts, means, stddevs):
    """Merge per-shard (count, mean, sample stddev) arrays of equal shape."""
    counts = np.ascontiguousarray(counts, np.int64)
    means = np.ascontiguousarray(means, np.float64)
    stddevs = np.ascontiguousarray(stddevs, np.float64)
    shape = means.shape[1:]
    L = int(np.prod(shape)) if shape else 1
    mo = np.zeros(L)
    so = np.zeros(L)
    n = C.c_int64()
    P = C.POINTER
    F.check(F.lib().tl_merge_moments(len(counts), L, counts.ctypes.data_as(P(C.c_int64)),
                                     means.ctypes.data_as(P(C.c_double)), stddevs.ctypes.data_as(P(C.c_double)),
                                     C.byref(n), mo.ctypes.data_as(P(C.c_double)), so.ctypes.data_as(P(C.c_double))),
            "tl_merge_moments")
    return n.value, mo.reshape(shape), so.reshape(shape)


def simulate_sharded(run_shard, total: int, group=None):
    """Run this rank's share of `total` realizations and merge the moments
    over the process group.

    run_shard(offset, count) -> (mean, stddev) numpy arrays of one shape
    (e.g. Model.simulate with realization_offset=offset, n=count).
    Returns (count, mean, stddev) of the whole ensemble on every rank.
    """
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    off, cnt = shard_range(total, world, rank)
    mean, sd = run_shard(off, cnt)
    if world == 1:
        return merge_moments([cnt], mean[None], sd[None])
    payload = torch.from_numpy(np.concatenate([[float(cnt)], np.ravel(mean), np.ravel(sd)]))
    if dist.get_backend(group) == "nccl":
        payload = payload.cuda()
    parts = [torch.zeros_like(payload) for _ in range(world)]
    dist.all_gather(parts, payload, group=group)
    L = mean.size
    arr = np.stack([p.cpu().numpy() for p in parts])
    counts = arr[:, 0].astype(np.int64)
    means = arr[:, 1:1 + L].reshape((world,) + mean.shape)
    sds = arr[:, 1 + L:].reshape((world,) + mean.shape)
    return merge_moments(counts, means, sds)
