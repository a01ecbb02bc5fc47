"""The library's sharding path on one GPU (hochunk3d_gb300/shard.py): the
shards of an iteration, each run by shard.run_shard in its own context (as
each rank would on its own GPU), sum to the tallies of one context running
the whole iteration, bit for bit in both forms; the summed absorbed-path
tally set back into a context (hc3d_set_lucy_tally) gives the temperatures
of the whole iteration.  The sum is taken here on the host; across
processes it is shard.allreduce_tallies (tests/test_dist.py, gloo)."""
from __future__ import annotations

import numpy as np
import pytest

from hochunk3d_gb300 import hc3d, shard

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [hc3d.PREC_MIXED, hc3d.PREC_FP64])
@pytest.mark.parametrize("ipeel", [0, 1])
def test_three_shards_sum_to_one_run(model_factory, prec, ipeel):
    m = model_factory("tiny3d")
    n, world = 9000, 3
    whole = m.run_params(np=n, iter=2, ipeel=ipeel)
    ctx = hc3d.Context(prec).load(m)
    want = shard.run_shard(ctx, whole, n)
    td_want, _, _ = ctx.lucy_update(m.info.ltot, n)
    ctx.close()
    parts = []
    for r in range(world):
        c = hc3d.Context(prec).load(m)
        parts.append(shard.run_shard(c, shard.shard_params(m, n, r, world, iter=2, ipeel=ipeel), n))
        c.close()
    keys = [k for k in shard.SUM_KEYS if k in want and isinstance(want[k], np.ndarray) and want[k].size]
    for k in keys:
        got = sum(p[k].astype(np.int64) for p in parts)
        np.testing.assert_array_equal(got, want[k].astype(np.int64), err_msg=k)
    # the temperatures of the summed tally, solved in a shard's context
    c = hc3d.Context(prec).load(m)
    shard.run_shard(c, shard.shard_params(m, n, 0, world, iter=2, ipeel=ipeel), n)
    c.set_lucy_tally(sum(p["dtauabs"].astype(np.int64) for p in parts))
    td, _, _ = c.lucy_update(m.info.ltot, n)
    c.close()
    np.testing.assert_array_equal(td, td_want)
