"""A peeled iteration run in chunks (hc3d_run_chunk): the packets still in
flight at the end of a chunk continue in the next one, and the tallies equal
those of one hc3d_run_iteration of the whole range, bit for bit in both
forms (a packet's history does not depend on the chunk or wave it runs in).
While a chunked iteration is open, the calls that would lose its packets
refuse; hc3d_zero_tallies discards it."""
from __future__ import annotations

import numpy as np
import pytest

from hochunk3d_gb300 import hc3d

pytestmark = pytest.mark.gpu
KEYS = ("si", "sq", "su", "nums", "ti", "tq", "tu", "numt", "image_i", "image_q", "nabs", "dtauabs", "jmean",
        "killed", "counters")


@pytest.mark.parametrize("prec", [hc3d.PREC_MIXED, hc3d.PREC_FP64])
@pytest.mark.parametrize("name", ["tiny3d", "tiny_acc"])
def test_chunks_equal_one_run(model_factory, prec, name):
    m = model_factory(name)
    n = 12000
    whole = m.run_params(np=n, iter=3, ipeel=1)
    ctx = hc3d.Context(prec).load(m)
    ctx.zero()
    ctx.run(whole)
    want = ctx.tallies(whole)
    ctx.zero()
    cuts = [0, 3000, 3100, 9000, n]
    for k in range(len(cuts) - 1):
        q = m.run_params(np_total=n, np=cuts[k + 1] - cuts[k], iter=3, ipeel=1, packet_offset=cuts[k])
        ctx.run_chunk(q, n, final=k == len(cuts) - 2)
    got = ctx.tallies(whole)
    for key in KEYS:
        np.testing.assert_array_equal(got[key], want[key], err_msg=key)
    ctx.close()


def test_open_chunk_guards(model_factory):
    m = model_factory("tiny3d")
    ctx = hc3d.Context(hc3d.PREC_MIXED).load(m)
    # a short queue: few events per lane and wave, so that packets are in flight when the chunk returns
    ctx.set_wave_options(queue_records=1 << 20)
    ctx.zero()
    n = 800000
    q = m.run_params(np_total=n, np=400000, iter=3, ipeel=1)
    ctx.run_chunk(q, n, final=False)
    for call in (lambda: ctx.run(m.run_params(np=100, iter=4, ipeel=1)),
                 lambda: ctx.set_wave_options(regen=4),
                 lambda: ctx.run_chunk(m.run_params(np_total=n, np=100, iter=5, ipeel=1, packet_offset=400000), n,
                                       final=True)):
        with pytest.raises(hc3d.Hc3dError) as e:
            call()
        assert e.value.code in (-4,)
    ctx.zero()  # discards the open iteration
    p = m.run_params(np=2000, iter=4, ipeel=1)
    ctx.run(p)
    c = ctx.tallies(p)["counters"]
    assert c[hc3d.CNT["escaped"]] + c[hc3d.CNT["aflux"]] + c[hc3d.CNT["abflux"]] == 2000
    ctx.close()
