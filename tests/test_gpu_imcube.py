"""GPU parity of the per-frequency peel-off image cube (IMCUBE,
peeloff_3d.f90:271-282) through the C-ABI: the FP64 form's cube against the
oracle's (identical int64 bins), and in both forms the cube summed over
frequency equals the broadband image exactly, with the origin and interaction
components of I adding up to the total."""
from __future__ import annotations

import numpy as np
import pytest

from hochunk3d_gb300 import compare as K
from hochunk3d_gb300 import hc3d

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def O(built):
    import oracle.oracle as orc

    return orc


@pytest.mark.parametrize("prec", [hc3d.PREC_FP64, hc3d.PREC_MIXED])
def test_cube(model_factory, O, prec):
    m = model_factory("tiny3d", IMCUBE="YES")
    p = m.run_params(np=3000, iter=3, ipeel=1)
    assert p.imcube == 1
    ctx = hc3d.Context(prec).load(m)
    ctx.zero()
    ctx.run(p)
    t = ctx.tallies(p)
    ctx.close()
    cube = t["image_m_i"]
    np.testing.assert_array_equal(cube[..., 0].sum(axis=3), t["image_i"])
    for c in "quv":
        np.testing.assert_array_equal(t["image_m_" + c].sum(axis=3), t["image_" + c])
    np.testing.assert_array_equal(cube[..., 1:5].sum(axis=4), cube[..., 0])
    np.testing.assert_array_equal(cube[..., 5:8].sum(axis=4), cube[..., 0])
    if prec == hc3d.PREC_FP64:
        r = O.run(m, p, nthreads=8)
        fr = {k: K.same_fraction(t[k], r[k]) for k in ("image_m_i", "image_m_q", "image_m_u", "image_m_v")}
        print("\nimage cube identical-bin fractions " + " ".join(f"{k}={v:.4f}" for k, v in fr.items()))
        assert min(fr.values()) >= 0.95, fr


def test_cube_in_unpeeled_and_imageless_runs(model_factory):
    """An unpeeled run (a Lucy iteration) has no cube to tally and runs; a
    peeled run without images cannot bin the cube and is refused."""
    m = model_factory("tiny3d", IMCUBE="YES")
    ctx = hc3d.Context(hc3d.PREC_MIXED).load(m)
    p = m.run_params(np=100, iter=3, ipeel=0)
    assert p.imcube == 1
    ctx.zero()
    ctx.run(p)
    q = m.run_params(np=100, iter=3, ipeel=1, image=0)
    ctx.zero()
    with pytest.raises(hc3d.Hc3dError) as e:
        ctx.run(q)
    assert e.value.code == -1 and "imcube" in str(e.value)
    ctx.close()
