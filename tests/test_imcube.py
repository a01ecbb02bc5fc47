"""The per-frequency peel-off image cube (IMCUBE, peeloff_3d.f90:271-282) in
the CPU oracle: I binned by the three SED components of the ray (all,
origin, interaction), Q, U, V by frequency; summed over frequency it is the
broadband image, and the origin and interaction components each add up to
the total.  CPU only."""
from __future__ import annotations

import numpy as np
import pytest

from hochunk3d_gb300 import configs, hc3d


@pytest.fixture(scope="module")
def O(built):
    import oracle.oracle as orc

    return orc


def test_imcube_key_and_oracle_cube_sums(tmp_path, built, O):
    m = hc3d.Model(configs.write_par(tmp_path, "tiny3d", IMCUBE="YES"))
    p = m.run_params(np=1500, iter=3, ipeel=1)
    assert p.imcube == 1
    assert hc3d.Model(configs.write_par(tmp_path / "b", "tiny3d")).run_params().imcube == 0
    r = O.run(m, p)
    cube = r["image_m_i"]
    assert cube.shape == (p.npeel, p.nxhst, p.nxhst, p.nfreq, hc3d.NO)
    np.testing.assert_array_equal(cube[..., 0].sum(axis=3), r["image_i"])
    for c in "quv":
        np.testing.assert_array_equal(r["image_m_" + c].sum(axis=3), r["image_" + c])
    np.testing.assert_array_equal(cube[..., 1:5].sum(axis=4), cube[..., 0])
    np.testing.assert_array_equal(cube[..., 5:8].sum(axis=4), cube[..., 0])
    assert np.count_nonzero(cube[..., 0].sum(axis=(0, 1, 2))) > 5  # several frequency planes are lit
