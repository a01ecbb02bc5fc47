"""The model set-up built on the GPU against the host build of the same
model: the densities of gridset (hc3d_model_densities_gpu) -- densities,
(rho V)^(1/4), cell volumes and grid masses agree to rounding and the cells
without dust are the same cells -- and the setemiss tables
(hc3d_model_tables_gpu)."""
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


STRUCTURED = {
    "gap": {"CGAPD": "YES", "RGAPD1": 3.0, "RGAPD2": 5.0, "RHOSCALE_GAP(1)": 0.1, "RHOSCALE_GAP(2)": 0.1},
    "gap_puff_curve": {"CGAPD": "YES", "RGAPD1": 3.0, "RGAPD2": 5.0, "CGAPPUFF": "YES", "GAPHEIGHT": 0.5,
                       "GAPLENGTH": 2.0, "CGAPCURVE": "YES", "GAPCURVEHEIGHT": 0.3, "GAPCURVELENGTH": 3.0,
                       "GAPCURVEEXP": 1.2},
    "rim": {"CRIMPUFF": "YES", "RIMHEIGHT": 1.0, "RIMLENGTH": 0.5, "CRIMCURVE": "YES", "RIMCURVEHEIGHT": 0.3,
            "RIMCURVELENGTH": 0.8, "RIMCURVEEXP": 1.0},
    "cutoff": {"CRADEXP": "YES", "RADEXP": 20.0},
    "spiral": {"NPG": 17, "CSPIRAL": "YES", "PITCH": 15.0, "SN": 4, "SW": 0.5, "RSPIRAL1": 2.0, "RSPIRAL2": 50.0},
    "warp": {"NPG": 9, "CDISKWARP": "YES", "WARPHEIGHT": 1.0, "WEXP": 41.0, "WARPLENGTH": 5.0},
    "envelope_gap": {"RATE": 5e-6, "CGAPE": "YES", "RGAPE1": 20.0, "RGAPE2": 60.0, "CGAPEDENS": "SCALE",
                     "FRACTE": 0.01},
}


@pytest.mark.gpu
@pytest.mark.parametrize("option", sorted(STRUCTURED))
def test_device_densities_of_structured_disks_match_host(tmp_path, built, option):
    """The disk structure of densdiskg (gap with its own density law, puffed
    and curved rim and gap wall, radial cutoff, spiral arms, warp) and the
    envelope gap on the GPU: the host build of the same model to 1e-12."""
    over = {"NRG": 60, "NTG": 41, "NPG": 2, "MASSD": 0.01, "RATE": 1e-9}
    over.update(STRUCTURED[option])
    m = make_model(tmp_path / option, "tiny", warm=False, **over)
    dens, mass = m.densarr.copy(), m.massarr.copy()
    mdisk, menv = m.info.massdisk, m.info.massenv
    m.densities_gpu(0)
    np.testing.assert_array_equal(m.densarr == 0.0, dens == 0.0)
    np.testing.assert_allclose(m.densarr, dens, rtol=1e-12, atol=0.0)
    np.testing.assert_allclose(m.massarr, mass, rtol=1e-12, atol=0.0)
    assert m.info.massdisk == pytest.approx(mdisk, rel=1e-12)
    assert m.info.massenv == pytest.approx(menv, rel=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tiny", "plain"])
def test_device_tables_match_host(tmp_path, built, name):
    """setemiss on the GPU (hc3d_model_tables_gpu): the cumulative emissivity
    rows and the Planck-mean factors of the host build, to rounding."""
    m = make_model(tmp_path / name, name, warm=False)
    kb, kp = m.kapBint.copy(), m.kappap.copy()
    ms = m.tables_gpu(0)
    assert ms > 0.0
    assert np.all(np.isfinite(m.kapBint)) and np.all(m.kappap > 0.0)
    np.testing.assert_allclose(m.kappap, kp, rtol=1e-11, atol=0.0)
    np.testing.assert_allclose(m.kapBint, kb, rtol=1e-11, atol=1e-300)
    rows = m.kapBint.reshape(m.nT, m.nnu, -1, order="F")
    assert np.all(rows[:, -1, :] == 1.0)
    assert np.all(np.diff(rows, axis=1) >= 0.0)
