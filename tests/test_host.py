"""CPU tests of the boundary and the host-side model set-up (no GPU calls)."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from hochunk3d_gb300 import configs, hc3d

ROOT = Path(__file__).resolve().parents[1]


def header_functions() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(hc3d_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_header_symbol(built):
    L = hc3d.lib()
    names = header_functions()
    assert len(names) >= 18
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(hc3d.SIGNATURES) >= names
    assert "sm_103a" in hc3d.version()


def test_missing_key_is_an_error(tmp_path, built):
    par = configs.write_par(tmp_path, "tiny")
    text = "\n".join(l for l in par.read_text().splitlines() if "= NRG =" not in l.replace("  ", " ") and "NRG" not in l)
    par.write_text(text)
    with pytest.raises(hc3d.Hc3dError) as e:
        hc3d.Model(par)
    assert "NRG" in str(e.value)


@pytest.mark.parametrize("key", ["DIFFUSION", "CHSEQ"])
def test_unsupported_options_are_rejected(tmp_path, built, key):
    par = configs.write_par(tmp_path, "tiny", **{key: "YES"})
    with pytest.raises(hc3d.Hc3dError) as e:
        hc3d.Model(par)
    assert e.value.code == -7


def test_spots_without_accretion_are_rejected(tmp_path, built):
    """Hot spots take their temperature from the accretion shock: CSPOT=YES
    without CDISKACC=YES would emit the spots' packets at T = 0."""
    par = configs.write_par(tmp_path, "tiny", CSPOT="YES")
    with pytest.raises(hc3d.Hc3dError) as e:
        hc3d.Model(par)
    assert e.value.code == -1 and "CDISKACC" in str(e.value)
    m = hc3d.Model(configs.write_par(tmp_path, "tiny", CDISKACC="YES"))
    assert m.info.accfrac > 0 and m.sources.ispot == 0


def test_external_illumination_needs_its_field(tmp_path, built):
    par = configs.write_par(tmp_path, "tiny", COUTILLUM="YES")
    with pytest.raises(hc3d.Hc3dError) as e:
        hc3d.Model(par)
    assert e.value.code == -1 and "ISRF_FILE" in str(e.value)


def test_grid_walls(model_factory):
    m = model_factory("plain", warm=False)
    nrg, ntg, npg, ndg = m.shape4
    mid = ntg // 2
    assert m.tan2arr[mid] == -1.0 and m.tan2arr[0] == 0.0 and m.tan2arr[-1] == 0.0
    assert m.thetarr[0] == 0.0 and m.thetarr[-1] == np.pi and m.thetarr[mid] == np.pi / 2
    np.testing.assert_allclose(m.thetarr + m.thetarr[::-1], np.pi, rtol=0, atol=1e-14)
    # power-law spacing, pexp = 2 (gridset.f90:544-548)
    k = np.arange(1, mid + 1)
    np.testing.assert_allclose(m.thetarr[mid + 1:] - np.pi / 2, np.pi / 2 / mid**2 * k**2, rtol=1e-12, atol=1e-15)
    # log radial grid from the sublimation radius to rmax (gridset.f90:438-446)
    r = m.rarr[1:]
    np.testing.assert_allclose(np.diff(np.log(r)), np.log(r[1] / r[0]), rtol=1e-9)
    assert m.rarr[0] == 1.0 and r[0] == pytest.approx(m.info.rminsub)
    assert r[-1] == pytest.approx(5000.0 * m.info.autors)


def test_disk_mass_is_normalised(model_factory):
    m = model_factory("plain", warm=False)
    msun = 1.989e33
    mdisk = (m.densarr[..., 0] * m.vcell).sum() / msun
    assert mdisk == pytest.approx(0.01, rel=1e-12)
    # cavity density inside 20 degrees of the pole, envelope outside it
    nrg, ntg = m.shape4[:2]
    th = 0.5 * (m.thetarr[:-1] + m.thetarr[1:])
    pole = th < np.radians(15)
    assert (m.densarr[5:-1, :-1, 0, 3][:, pole] > 0).all() and (m.densarr[5:-1, :-1, 0, 2][:, pole] == 0).all()


def test_setemiss_tables(model_factory):
    m = model_factory("tiny", warm=False)
    kb = m.kapBint.reshape(m.ndg_tab, m.nnu, m.nT)  # (nT,nnu,ndg) Fortran -> C order reversed
    assert np.all(np.diff(kb, axis=1) >= -1e-12)
    np.testing.assert_allclose(kb[:, -1, :], 1.0)
    kp = m.kappap.reshape(m.ndg_tab, m.nT)
    assert np.all(kp > 0) and np.all(np.diff(kp[0][100:]) > 0)


def test_fractal_field_conserves_cell_average(model_factory):
    m = model_factory("tiny3d", warm=False)
    m0 = model_factory("tiny3d", warm=False, CFRACTAL="NO")
    env = m.densarr[:-1, :-1, :-1, 2]
    env0 = m0.densarr[:-1, :-1, :-1, 2]
    sel = env0 > 0
    ratio = env[sel] / env0[sel]
    assert ratio.max() / ratio.min() > 20  # clumps with contrast ~100
    assert ratio.mean() == pytest.approx(1.0, rel=0.15)


def test_tally_scales_formula():
    ss, sq, ps = hc3d.tally_scales(10**6)
    assert (ss, sq, ps) == (2.0**34, 2.0**26, 2.0**28)
    ss, sq, ps = hc3d.tally_scales(10**8)
    assert ss == 2.0**27 and ps == 2.0**21


def test_model_footprint_counts_grid_and_images(tmp_path, built):
    """The server's admission size grows with the cells and the peel-off images."""
    a = hc3d.Model(configs.write_par(tmp_path / "a", "tiny"))
    b = hc3d.Model(configs.write_par(tmp_path / "b", "tiny", NPG=9))
    c = hc3d.Model(configs.write_par(tmp_path / "c", "tiny", NPEEL=1, THETE="45.0", PHIE="0.0"))
    fa, fb, fc = (int(hc3d.lib().hc3d_model_footprint(m._h)) for m in (a, b, c))
    assert 0 < fc < fa < fb
    assert fb - fa >= (b.info.ncells - a.info.ncells) * 200


def test_new_entry_points_reject_bad_arguments(built):
    """The batch, graph, autotune, reset and server entry points check their
    arguments before they touch a device (no GPU needed)."""
    L = hc3d.lib()
    assert L.hc3d_reset(None) == -1
    assert L.hc3d_run_batch(None, None, 1) == -1
    assert L.hc3d_lucy_iterations(None, None, 3, 1.0, None, None) == -1
    assert L.hc3d_autotune(None, None, None) == -1
    h = C.c_void_p()
    assert L.hc3d_server_create(C.byref(h), C.byref(hc3d.ServerOpts(0, 0, 0, 0))) == -1  # no slots
    assert L.hc3d_server_create(C.byref(h), C.byref(hc3d.ServerOpts(0, 0, 65, 0))) == -1  # too many
    assert L.hc3d_server_submit(None, None, None) == -1
    r = hc3d.Result()
    assert L.hc3d_server_wait(None, 1, C.byref(r)) == -1
    assert L.hc3d_model_footprint(None) == -1
    L.hc3d_result_free(None)
    L.hc3d_server_destroy(None)
    # the small-grain entry points
    assert L.hc3d_set_species(None, None) == -1
    assert L.hc3d_load_sg_tables(None, None) == -1
    assert L.hc3d_get_imean(None, None, None) == -1
    assert L.hc3d_set_imean(None, None, None) == -1
    assert L.hc3d_model_load(None, None) == -1
    assert hc3d.host_lib().hc3d_model_sg_tables(None, None) == -1
    assert L.hc3d_set_lucy_tally(None, None) == -1
