"""Multi-process packet sharding on CPU (gloo, world_size 2), through the
library's sharding module (hochunk3d_gb300/shard.py).

The packet loop shards by packet id (the reference splits np over MPI ranks,
newtts.F90:185-188).  Tallies are int64 fixed point, so the all-reduce of the
shards equals the single-process run exactly.  The ranks run the oracle on
CPU as their shard's runner; on GPUs each rank runs shard.run_shard with the
library on its own device (tests/test_gpu_shard.py checks that runner and
the temperature update of the summed tallies on one GPU).
"""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from tests.helpers import make_model

KEYS = ("si", "sq", "nums", "ti", "tv", "numt", "image_i", "nabs", "dtauabs", "jmean")


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, directory, n, q, name):
    import torch.distributed as dist

    import oracle.oracle as O
    from hochunk3d_gb300 import hc3d, shard

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    try:
        # each rank writes its own copy of the model files: two ranks writing
        # one directory at once could read each other's half-written files
        m = make_model(directory / f"rank{rank}", name)
    except Exception as e:  # report instead of leaving the parent waiting
        q.put(e)
        raise
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r = shard.sharded_iteration(lambda p: O.run(m, p, scales=hc3d.tally_scales(n)), m, n, rank, world, iter=2,
                                ipeel=1)
    out = {k: np.ascontiguousarray(r[k]).astype(np.int64) for k in KEYS + ("counters",)}
    if rank == 0:
        q.put(out)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("name", ["tiny3d", "tiny_isrf"])
def test_two_rank_shards_sum_to_the_single_run(tmp_path, built, name):
    """With external illumination the shards split stellar and external
    packets by the iteration's global stellar share (np_total)."""
    import oracle.oracle as O
    from hochunk3d_gb300 import hc3d

    n = 1500
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, tmp_path / "m", n, q, name)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=300)
    if isinstance(got, Exception):
        raise got
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    m = make_model(tmp_path / "single", name)
    ref = O.run(m, m.run_params(np=n, iter=2, ipeel=1), scales=hc3d.tally_scales(n))
    for k in KEYS + ("counters",):
        np.testing.assert_array_equal(got[k], np.ascontiguousarray(ref[k]).astype(np.int64), err_msg=k)


def test_shard_ranges_cover_the_iteration():
    from hochunk3d_gb300 import shard

    for n, world in ((1500, 2), (7, 3), (1, 4), (10**8, 8)):
        spans = [shard.shard_range(n, r, world) for r in range(world)]
        assert spans[0][0] == 0 and spans[-1][1] == n
        assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
    with pytest.raises(ValueError):
        shard.shard_range(10, 2, 2)


def _reduce_rank(rank, world, port, q):
    import torch.distributed as dist

    from hochunk3d_gb300 import shard

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = {"nabs": np.full((3, 4, 2, 4), rank + 1, dtype=np.int64, order="F"),
         "killed": np.full((3, 4, 2), 10 * (rank + 1), dtype=np.int32, order="F"),
         "counters": np.arange(16, dtype=np.int64) * (rank + 1), "path_scale": 2.0 ** 20}
    t["nabs"][1, 2, 0, 3] = 1 << 40
    r = shard.allreduce_tallies(t)
    if rank == 0:
        q.put({k: v for k, v in r.items()})
    dist.barrier()
    dist.destroy_process_group()


def test_allreduce_keeps_shapes_and_types():
    """The int64 sums are exact (2^40 + 2^40 = 2^41), int32 counts stay int32 in
    their Fortran shape, scalars are left alone."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_reduce_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got["nabs"].dtype == np.int64 and got["nabs"].shape == (3, 4, 2, 4)
    assert got["nabs"][0, 0, 0, 0] == 3 and got["nabs"][1, 2, 0, 3] == 2 << 40
    assert got["killed"].dtype == np.int32 and np.all(got["killed"] == 30)
    np.testing.assert_array_equal(got["counters"], np.arange(16) * 3)
    assert got["path_scale"] == 2.0 ** 20
