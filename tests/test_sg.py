"""Very small grains and PAHs (FSG > 0) on the host and in the oracle, CPU
only: the species of the model (reapar.f90:239-268, gridset.f90:950-1075),
the four device slots chosen from them, the emission spectra
(draine_cdf.f90), the ISRF integral (isrf_cdf.f90:191-214), and the oracle's
rep_draine (rep_draine.f90), int_mean (int_mean.f90:19-94) and small-grain
branch (emit_common.f90:31-53) against the independent restatement of
tests/golden/ref_routines.py."""
from __future__ import annotations

import os

import numpy as np
import pytest

from hochunk3d_gb300 import configs, hc3d
from tests.golden import ref_routines as R
from tests.test_isrf import C_UM, NISRF


@pytest.fixture(scope="module")
def O(built):
    import oracle.oracle as orc

    return orc


def _fixture_dir(model_factory, name="tiny_sg"):
    """The model and the directory of its .par file and fixtures (PARDIR)."""
    m = model_factory(name)
    return m, os.path.dirname(m.par_path)


def test_species_and_slots(model_factory):
    m = model_factory("tiny_sg")
    assert m.shape4[3] == 8 and m.sg
    # disk 1, disk 2, the envelope and disk 1's small grains; no cavity
    assert list(m.slot_species) == [1, 2, 3, 5]
    assert m.sg_slot == 4 and m.sg_species == 4
    d = m.densarr
    filled = [bool((d[..., s] > 0).any()) for s in range(8)]
    assert filled == [True, False, True, False, True, False, False, False]
    # the small grains follow disk 1's shape with FSG / (1 - FSG) of its mass
    sel = d[..., 0] > 0
    np.testing.assert_array_equal(sel, d[..., 4] > 0)
    np.testing.assert_allclose(d[..., 4][sel] / d[..., 0][sel], 0.2 / 0.8, rtol=1e-12)
    # without small grains the host arrays keep the four species
    t = model_factory("tiny")
    assert t.shape4[3] == 4 and not t.sg and list(t.slot_species) == [1, 2, 3, 4]


def test_too_many_species_rejected(tmp_path):
    par = configs.write_par(tmp_path, "tiny_sg", **{"FSG(3)": 0.1, "CHOLE": "YES"})
    with pytest.raises(hc3d.Hc3dError) as e:
        hc3d.Model(par)
    assert "four species" in str(e.value)


def test_fsg_needs_isrf_file(tmp_path):
    cfg = dict(configs.CONFIGS["tiny_sg"])
    cfg.pop("ISRF_FILE")
    configs.CONFIGS["_tmp_sg"] = cfg
    try:
        par = configs.write_par(tmp_path, "_tmp_sg")
        with pytest.raises(hc3d.Hc3dError) as e:
            hc3d.Model(par)
        assert "ISRF_FILE" in str(e.value)
    finally:
        del configs.CONFIGS["_tmp_sg"]


def test_spectra_match_restatement(model_factory):
    m, d = _fixture_dir(model_factory)
    cdf, logcdf, logfreq, uratio = R.draine_cdf(d)
    np.testing.assert_array_equal(m.sg_uratio, uratio)
    np.testing.assert_allclose(m.sg_cdf, cdf, rtol=1e-13, atol=0)
    np.testing.assert_allclose(m.sg_logcdf, logcdf, rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(m.sg_logfreq, logfreq, rtol=1e-13, atol=0)
    # the spectra differ from row to row; the hottest continuum (U = 1e7)
    # has a higher mean frequency than U = 1e3's
    nu = 10.0 ** logfreq[1:]
    mean_nu = [np.sum(np.diff(cdf[j]) * nu) for j in range(18)]
    assert all(a != b for a, b in zip(mean_nu, mean_nu[1:])) and mean_nu[17] > mean_nu[9]


def test_isrf_integral_matches_restatement(model_factory):
    m, d = _fixture_dir(model_factory)
    lnu, nufnu = np.loadtxt(f"{d}/{configs.ISRF_FILE}", comments="#", unpack=True)
    freqin = 10.0 ** lnu
    logfreqin = np.log10(freqin)
    logpdfin = np.log10(10.0 ** nufnu / freqin)
    lmin = max(C_UM / (freqin[-1] * 0.99999999), 0.05)
    lmax = min(C_UM / (freqin[0] * 1.0000001), 5000.0)
    lam = lmin * (lmax / lmin) ** (np.arange(1, NISRF + 1) / NISRF)
    freq = (C_UM / lam)[::-1].copy()
    j = np.clip(np.searchsorted(freqin, freq, side="left"), 1, len(freqin) - 1)
    lp = logpdfin[j - 1] + (np.log10(freq) - logfreqin[j - 1]) / (logfreqin[j] - logfreqin[j - 1]) * (
        logpdfin[j] - logpdfin[j - 1])
    pdf = 10.0 ** lp
    sp = m.sg_species
    L = m.nlammax
    tabs = [a.reshape((L, -1), order="F") for a in (m.nudust, m.gdust, m.pldust, m.kappad, m.adust)]

    def kappa_of(nu):
        g, pl, kap, alb = R.opacset(nu, tabs[0][:, sp:sp + 1], m.nlambda[sp:sp + 1], tabs[1][:, sp:sp + 1],
                                    tabs[2][:, sp:sp + 1], tabs[3][:, sp:sp + 1], tabs[4][:, sp:sp + 1])[0]
        return kap, alb

    want = R.isrf_sg_integral(freq, pdf, kappa_of, float(m.kappav[sp]))
    assert m.isrfkap_int == pytest.approx(want, rel=1e-11)


def test_rep_draine_matches_restatement(O, model_factory):
    m, d = _fixture_dir(model_factory)
    cdf, logcdf, logfreq, _ = R.draine_cdf(d)
    rng = np.random.default_rng(7)
    for _ in range(400):
        jm = int(rng.integers(1, 19))
        jmf = float(rng.uniform(-0.9, 1.0))
        x = float(rng.uniform(1e-9, 1.0 - 1e-12))
        got = O.rep_draine(m, jm, jmf, x)[0]
        want = R.rep_draine(cdf, logcdf, logfreq, jm, jmf, x)
        assert got == pytest.approx(want, rel=1e-12), (jm, jmf, x)


def test_int_mean_matches_restatement(O, model_factory):
    """Random path tallies through the oracle's int_mean and the restatement:
    identical rows, fractions to 1e-12; ratios spanning the 18 spectra."""
    m = model_factory("tiny_sg")
    nrg, ntg, npg = m.shape3
    rng = np.random.default_rng(11)
    ps = 2.0 ** 20
    jsg = np.zeros(m.shape3, dtype=np.int64, order="F")
    jsg[:-1, :-1, :-1] = (10.0 ** rng.uniform(-3, 9, size=(nrg - 1, ntg - 1, npg - 1)) * ps).astype(np.int64)
    jsg[3, 4, 0] = 0
    ltot, nphot, rcm = m.info.ltot, 20000.0, m.params.rstar_cm
    im, fr = O.int_mean(m, jsg, ps, ltot, nphot, rcm)
    kv = float(m.kappav[m.sg_species])
    rows = set()
    for ir in range(nrg - 1):
        for it in range(ntg - 1):
            for ip in range(npg - 1):
                jm = float(jsg[ir, it, ip]) / ps * m.rarr[ir + 1] * (1.0 / (1.0 / (rcm * kv)) / (4.0 * R.PI))
                w_im, w_f = R.int_mean_cell(jm, m.vcell[ir, it, ip], nphot, ltot, m.isrfkap_int, m.sg_uratio)
                assert im[ir, it, ip] == w_im
                assert fr[ir, it, ip] == pytest.approx(w_f, rel=1e-12, abs=1e-13)
                rows.add(w_im)
    assert im[3, 4, 0] == 1 and fr[3, 4, 0] == 0.0
    assert rows == set(range(1, 19))


def test_oracle_small_grain_branch(O, model_factory):
    """A Lucy iteration of the oracle: small-grain absorptions are counted in
    dsg (and nabs of species 5), the path tally jsg covers the cells the
    packets cross, int_mean spreads the cells over the spectra; the second
    iteration needs its result and re-emits by it."""
    m = model_factory("tiny_sg")
    q = m.run_params(np=20000, iter=1, ipeel=0)
    r = O.run(m, q, nthreads=8)
    assert r["errors"] == 0
    nabs = r["nabs"].sum(axis=(0, 1, 2))
    assert r["dsg"].sum() == nabs[4] > 0 and r["dbig"].sum() == nabs[0] + nabs[2]
    assert nabs[1] == nabs[3] == 0 and nabs[5:].sum() == 0
    assert (r["jsg"] > 0).sum() > 0.5 * (m.densarr.sum(axis=3) > 0).sum()
    im, fr = O.int_mean(m, r["jsg"], r["path_scale"], m.info.ltot, q.np, q.rstar_cm)
    sel = m.densarr[..., 4] > 0
    assert len(set(im[sel].tolist())) > 10
    q2 = m.run_params(np=4000, iter=2, ipeel=1)
    with pytest.raises(ValueError):
        O.run(m, q2)
    r2 = O.run(m, q2, nthreads=8, imean=im, imfract=fr)
    assert r2["errors"] == 0 and r2["dsg"].sum() > 0
    c = r2["counters"]
    assert c[hc3d.CNT["escaped"]] + c[hc3d.CNT["aflux"]] + c[hc3d.CNT["abflux"]] == 4000
