"""Limb darkening on the GPU (CLIMB=YES): the sm_103a kernels against the
oracle through the C-ABI."""
from __future__ import annotations

import numpy as np
import pytest

from hochunk3d_gb300 import hc3d
from tests.helpers import splitmix_uniforms, trace_key

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def O(built):
    import oracle.oracle as orc

    return orc


def test_trace_fp64_limb_darkened_packets_match_oracle(model_factory, O):
    m = model_factory("tiny3d", CLIMB="YES")
    ctx = hc3d.Context(hc3d.PREC_FP64).load(m)
    n = 32
    p = m.run_params(np=n, iter=3, ipeel=1)
    assert p.limb == 1
    U = splitmix_uniforms(n, 4096, seed=5150)
    traces = ctx.trace(p, U, max_rec=2048)
    same = 0
    for k in range(n):
        want, exhausted, _ = O.trace(m, p, pid=k, uniforms=U[k], max_rec=2048)
        assert not exhausted
        got = traces[k]
        if got.shape == want.shape and np.array_equal(trace_key(got), trace_key(want)):
            same += 1
            np.testing.assert_allclose(got["tsum"], want["tsum"], rtol=1e-5, atol=1e-12)
            np.testing.assert_allclose(got["x"], want["x"], rtol=1e-9, atol=1e-9)
    assert same >= n - 1, same


@pytest.mark.parametrize("prec", [hc3d.PREC_FP64, hc3d.PREC_MIXED])
def test_stream_run_limb_darkened_matches_oracle(model_factory, O, prec):
    """2000 peeled packets: counters and SED counts as the oracle's; the FP64
    form also matches most peeled-SED bins exactly (the 12/5 (mu + mu^2)
    weight of the stellar peel-off)."""
    m = model_factory("tiny3d", CLIMB="YES")
    ctx = hc3d.Context(prec).load(m)
    n = 2000
    p = m.run_params(np=n, iter=3, ipeel=1)
    ctx.zero()
    ctx.run(p)
    t = ctx.tallies(p)
    r = O.run(m, p)
    ended = t["counters"][hc3d.CNT["escaped"]] + t["counters"][hc3d.CNT["aflux"]] + t["counters"][hc3d.CNT["abflux"]]
    assert ended + t["counters"][hc3d.CNT["stuck"]] == n
    if prec == hc3d.PREC_FP64:
        for k in (0, 4, 5, 6, 9, 12, 13, 14):
            assert abs(int(t["counters"][k]) - int(r["counters"][k])) <= 2 + 0.002 * abs(int(r["counters"][k])), k
        assert np.mean(t["ti"] == r["ti"]) > 0.97
    else:
        a = t["ti"][..., 0].sum() / t["stokes_scale"]
        b = r["ti"][..., 0].sum() / r["stokes_scale"]
        assert abs(a - b) <= 0.05 * b
