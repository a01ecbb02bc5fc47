"""Disk structure of densdiskg (densdiskg.f90:25-155): gap, radial cutoff,
spiral arms, warp and puffed rim, built by the host gridset.  CPU only."""
from __future__ import annotations

import numpy as np
import pytest

from hochunk3d_gb300 import configs, hc3d

GRID = {"NRG": 60, "NTG": 41, "NPG": 2, "MASSD": 0.01, "RATE": 1e-9, "NP": 1000, "NPMIN": 1000}


def _model(tmp_path, name, **over):
    cfg = dict(GRID)
    cfg.update(over)
    return hc3d.Model(configs.write_par(tmp_path / name, "tiny", **cfg))


def _midplane(m, slot=0):
    """Disk density of the midplane cells (the two cells beside theta = 90 deg) against the cell radius."""
    it = (m.shape4[1] - 1) // 2 - 1
    rave = np.sqrt(m.rarr[:-1] * m.rarr[1:])
    return rave, m.densarr[:-1, it, 0, slot]


def test_plain_disk_unchanged_and_mass_normalised(tmp_path, built):
    m = _model(tmp_path, "plain")
    assert m.info.massdisk == pytest.approx(0.01, rel=1e-9)


def test_gap_empties_the_gap(tmp_path, built):
    m = _model(tmp_path, "gap", CGAPD="YES", RGAPD1=3.0, RGAPD2=5.0, **{"RHOSCALE_GAP(1)": 0.0,
                                                                         "RHOSCALE_GAP(2)": 0.0})
    r, d = _midplane(m)
    au = m.info.autors
    inside = (r > 3.2 * au) & (r < 4.8 * au)
    outside = (r > 5.5 * au) & (r < 50 * au)
    assert inside.sum() >= 2 and outside.sum() >= 2
    assert np.all(d[inside] == 0.0) and np.all(d[outside] > 0.0)
    assert m.info.massdisk == pytest.approx(0.01, rel=1e-9)
    # a gap scaled by 0.1 of the outside surface density is neither empty nor the full disk
    g = _model(tmp_path, "gap01", CGAPD="YES", RGAPD1=3.0, RGAPD2=5.0,
               **{"RHOSCALE_GAP(1)": 0.1, "RHOSCALE_GAP(2)": 0.1})
    _, dg = _midplane(g)
    assert np.all(dg[inside] > 0.0)
    p = _model(tmp_path, "nogap")
    _, dp = _midplane(p)
    assert np.all(dg[inside] < dp[inside])


def test_radial_cutoff_is_exponential(tmp_path, built):
    p = _model(tmp_path, "base")
    e = _model(tmp_path, "exp", CRADEXP="YES", RADEXP=20.0)
    r, dp = _midplane(p)
    _, de = _midplane(e)
    ok = (dp > 0) & (de > 0) & (r < 200 * p.info.autors)
    slope = np.polyfit(r[ok], np.log(de[ok] / dp[ok]), 1)[0]
    # rcoord = r sin(theta) of the cells beside the midplane: within 1e-5 of r
    assert slope == pytest.approx(-1.0 / (20.0 * p.info.autors), rel=1e-4)
    assert e.info.massdisk == pytest.approx(0.01, rel=1e-9)


def test_spiral_arms_vary_with_azimuth_inside_their_radii(tmp_path, built):
    m = _model(tmp_path, "spiral", NPG=17, CSPIRAL="YES", PITCH=15.0, SN=4, SW=0.5, RSPIRAL1=2.0, RSPIRAL2=50.0)
    it = (m.shape4[1] - 1) // 2 - 1
    rave = np.sqrt(m.rarr[:-1] * m.rarr[1:])
    d = m.densarr[:-1, it, :-1, 0]
    au = m.info.autors
    arms = (rave > 3 * au) & (rave < 40 * au) & (d.min(axis=1) > 0)
    plain = (rave > 60 * au) & (d.min(axis=1) > 0)
    assert arms.sum() >= 3 and plain.sum() >= 1
    contrast = d[arms].max(axis=1) / d[arms].min(axis=1)
    assert np.all(contrast > 1.5)
    np.testing.assert_allclose(d[plain].max(axis=1), d[plain].min(axis=1), rtol=1e-12)
    assert m.info.massdisk == pytest.approx(0.01, rel=1e-9)


def test_warp_lifts_one_side(tmp_path, built):
    """The warp (cos(phi/2)^WEXP, falling off from the rim) reshapes the disk
    near phi = 0 and leaves it alone near phi = 180 deg, where only the mass
    renormalisation scales it."""
    m = _model(tmp_path, "warp", NPG=9, CDISKWARP="YES", WARPHEIGHT=1.0, WEXP=41.0, WARPLENGTH=5.0)
    flat = _model(tmp_path, "flat", NPG=9)
    w, f = m.densarr[:-1, :-1, :-1, 0], flat.densarr[:-1, :-1, :-1, 0]
    both = (w > 0) & (f > 0)
    near0 = (w[:, :, 0] / np.where(both[:, :, 0], f[:, :, 0], 1.0))[both[:, :, 0]]  # phi = 22.5 deg
    far = (w[:, :, 3] / np.where(both[:, :, 3], f[:, :, 3], 1.0))[both[:, :, 3]]  # phi = 157.5 deg
    assert near0.max() / near0.min() > 1.5
    np.testing.assert_allclose(far, far[0], rtol=1e-9)
    assert m.info.massdisk == pytest.approx(0.01, rel=1e-9)


def test_puffed_rim_thickens_the_inner_disk(tmp_path, built):
    p = _model(tmp_path, "nopuff")
    q = _model(tmp_path, "puff", CRIMPUFF="YES", RIMHEIGHT=1.0, RIMLENGTH=0.5)
    ntg = p.shape4[1]
    ir = int(np.argmax(p.densarr[:-1, (ntg - 1) // 2 - 1, 0, 0] > 0))  # innermost disk cell
    col_p = p.densarr[ir + 1, :-1, 0, 0]
    col_q = q.densarr[ir + 1, :-1, 0, 0]
    # more of the column's density sits away from the midplane
    w = np.abs(np.arange(ntg - 1) - (ntg - 2) / 2.0)
    assert (col_q * w).sum() / col_q.sum() > (col_p * w).sum() / col_p.sum()


@pytest.mark.parametrize("mode", ["CONST", "SCALE"])
def test_envelope_gap(tmp_path, built, mode):
    """CGAPE (densenv.f90:52-58,114-119): the envelope between RGAPE1 and
    RGAPE2 takes RHOGAPE (CONST) or FRACTE times its density (SCALE)."""
    over = {"RATE": 5e-6, "MASSD": 0.0001, "CGAPE": "YES", "RGAPE1": 20.0, "RGAPE2": 60.0, "CGAPEDENS": mode,
            "FRACTE": 0.01, "RHOGAPE": 3e-21}
    g = _model(tmp_path, "egap" + mode, **over)
    p = _model(tmp_path, "enogap" + mode, RATE=5e-6, MASSD=0.0001)
    au = g.info.autors
    rave = np.sqrt(g.rarr[:-1] * g.rarr[1:])
    it = 5  # a polar-angle cell off the disk, outside the cavity
    e_g, e_p = g.densarr[:-1, it, 0, 2], p.densarr[:-1, it, 0, 2]
    gap = (rave > 21 * au) & (rave < 59 * au) & (e_p > 0)
    away = ((rave < 19 * au) | (rave > 61 * au)) & (e_p > 0)
    assert gap.sum() >= 2 and away.sum() >= 2
    if mode == "CONST":
        np.testing.assert_allclose(e_g[gap], 3e-21, rtol=1e-12)
    else:
        np.testing.assert_allclose(e_g[gap], 0.01 * e_p[gap], rtol=1e-12)
    np.testing.assert_array_equal(e_g[away], e_p[away])
