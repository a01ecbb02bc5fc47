"""The densities of gridset built on the GPU (hc3d_model_densities_gpu)
against the host build of the same model: densities, (rho V)^(1/4), cell
volumes and grid masses agree to rounding, and the cells without dust are
the same cells."""
from __future__ import annotations

import numpy as np
import pytest

from hochunk3d_gb300 import hc3d
from tests.helpers import make_model


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tiny", "tiny3d", "plain", "full3d"])
def test_device_densities_match_host(tmp_path, built, name):
    m = make_model(tmp_path / name, name, warm=False)
    dens, mass, vol = m.densarr.copy(), m.massarr.copy(), m.vcell.copy()
    mdisk, menv = m.info.massdisk, m.info.massenv
    ms = m.densities_gpu(0)
    assert ms > 0.0
    np.testing.assert_array_equal(m.densarr == 0.0, dens == 0.0)
    np.testing.assert_allclose(m.densarr, dens, rtol=1e-12, atol=0.0)
    np.testing.assert_allclose(m.massarr, mass, rtol=1e-12, atol=0.0)
    np.testing.assert_allclose(m.vcell, vol, rtol=1e-13, atol=0.0)
    assert m.info.massdisk == pytest.approx(mdisk, rel=1e-12)
    assert m.info.massenv == pytest.approx(menv, rel=1e-12)
    # a second build repeats the first bit for bit
    d1 = m.densarr.copy()
    m.densities_gpu(0)
    np.testing.assert_array_equal(m.densarr, d1)
