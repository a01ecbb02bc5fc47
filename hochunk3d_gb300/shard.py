"""Packet-id sharding of one iteration over processes (newtts.F90:185-188
splits np over MPI ranks; newdisktherm.F90:472-486 sums the tallies with
MPI_ALLREDUCE).

Every rank holds the whole grid and runs the packet range
``shard_range(np_total, rank, world)`` of the iteration: the counter-based
streams are keyed by the global packet id and every shard tallies at the
scales of the whole iteration, so the int64 tallies of the shards sum to
those of one process bit for bit.  The sum is one ``SUM`` all-reduce of the
int64 arrays over a ``torch.distributed`` group (NCCL on GPUs, gloo on
CPUs).  With the summed absorbed-path tally set back into each rank's
context (``Context.set_lucy_tally``), ``hc3d_lucy_update`` solves the same
temperatures on every rank: no broadcast is needed.
"""
from __future__ import annotations

from typing import Callable

import numpy as np

from . import hc3d

# the int64 tallies an iteration sums (the counters too)
SUM_KEYS = ("si", "sq", "su", "sv", "si2", "sq2", "su2", "sv2", "nums", "ti", "tq", "tu", "tv", "ti2", "tq2",
            "tu2", "tv2", "numt", "image_i", "image_q", "image_u", "image_v", "nabs", "dtauabs", "jmean", "killed",
            "dbig", "dsg", "jsg", "counters")


def shard_range(np_total: int, rank: int, world: int) -> tuple[int, int]:
    """[lo, hi): the packet ids of rank `rank` of `world`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    return np_total * rank // world, np_total * (rank + 1) // world


def shard_params(model: hc3d.Model, np_total: int, rank: int, world: int, **over) -> hc3d.RunParams:
    """The run parameters of this rank's shard of an iteration of np_total packets."""
    lo, hi = shard_range(np_total, rank, world)
    return model.run_params(np_total=np_total, np=hi - lo, packet_offset=lo, **over)


def allreduce_tallies(tallies: dict, group=None) -> dict:
    """Sum the int64 (and int32 count) tallies of every rank in place: one
    SUM all-reduce per array, over torch.distributed's default group or
    `group`."""
    import torch
    import torch.distributed as dist

    for k in SUM_KEYS:
        a = tallies.get(k)
        if a is None or not isinstance(a, np.ndarray) or a.size == 0:
            continue
        t = torch.from_numpy(np.ascontiguousarray(a.ravel(order="F")).astype(np.int64))
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        tallies[k] = t.numpy().astype(a.dtype).reshape(a.shape, order="F")
    return tallies


def run_shard(ctx: hc3d.Context, params: hc3d.RunParams, np_total: int) -> dict:
    """One rank's shard on its GPU: the packets of params, tallied at the
    scales of the whole iteration of np_total packets."""
    ctx.zero()
    ctx.run_chunk(params, np_total, final=True)
    return ctx.tallies(params)


def sharded_iteration(run: Callable[[hc3d.RunParams], dict], model: hc3d.Model, np_total: int, rank: int,
                      world: int, group=None, **over) -> dict:
    """Run this rank's shard with `run` (params -> tallies) and return the
    tallies of the whole iteration, summed over the ranks."""
    t = run(shard_params(model, np_total, rank, world, **over))
    return allreduce_tallies(t, group)
