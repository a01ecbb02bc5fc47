"""Known answers of the physics on the GPU, through the C-ABI."""
from __future__ import annotations

import numpy as np
import pytest

from hochunk3d_gb300 import hc3d
from tests.helpers import dilution_temperature, make_gray_model

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [hc3d.PREC_MIXED, hc3d.PREC_FP64])
def test_optically_thin_lucy_temperature_is_radiative_equilibrium(tmp_path, built, prec):
    """Gray, purely absorbing dust in an optically thin envelope: one Lucy
    iteration of 2e5 packets (packet loop and tfinal on the device) gives
    T = T* W(r)^(1/4) to 1 % in the median cell and 3 % in every cell with
    dust."""
    m = make_gray_model(tmp_path)
    n = 200000
    ctx = hc3d.Context(prec).load(m)
    p = m.run_params(np=n, iter=1, ipeel=0)
    ctx.zero()
    ctx.run(p)
    c = ctx.tallies(p)["counters"]
    td, _, _ = ctx.lucy_update(m.info.ltot, n)
    ctx.close()
    assert c[hc3d.CNT["tot"]] < 1e-3 * n  # optically thin
    sel = m.densarr[:-1, ..., 2] > 0
    want = np.broadcast_to(dilution_temperature(m)[:, None, None], sel.shape)[sel]
    got = td[:-1, ..., 2][sel] * 11605.0
    rel = np.abs(got - want) / want
    assert sel.sum() > 500
    assert np.median(rel) < 0.01 and rel.max() < 0.03, (np.median(rel), rel.max())
