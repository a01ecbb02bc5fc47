"""External illumination (COUTILLUM=YES): the field's tables (isrf_cdf), the
stellar/external packet split (newdisktherm.F90:143-175), rep_isrf, and the
external packets of the oracle.  CPU only."""
from __future__ import annotations

import numpy as np
import pytest

from hochunk3d_gb300 import configs, hc3d

C_UM = 2.99792458e14
NISRF = 200


@pytest.fixture(scope="module")
def O(built):
    import oracle.oracle as orc

    return orc


def isrf_tables(path):
    """isrf_cdf.f90:28-243 restated in numpy (ISRF_AV = 0)."""
    lnu, nufnu = np.loadtxt(path, comments="#", unpack=True)
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
    cdf = np.zeros(NISRF)
    for i in range(1, NISRF):
        cdf[i] = cdf[i - 1] + 0.5 * (pdf[i] + pdf[i - 1]) * (freq[i] - freq[i - 1])
    total = cdf[-1]
    cdf = cdf / total
    logcdf = np.full(NISRF, -99.0)
    logcdf[1:] = np.log10(cdf[1:])
    logfreq = np.zeros(NISRF)
    logfreq[1:] = np.log10(freq[1:] * 1.2398 / C_UM)
    return total, cdf, logcdf, logfreq


def star_packets(frac, n):
    """newdisktherm.F90:143-175 without accretion, restated."""
    npout = int(frac * float(n))
    if frac * float(n) - npout > 0.5:
        npout += 1
    ns = int(float(n) * (1.0 - frac))
    rn = float(np.float32(n)) * (1.0 - frac)
    if rn - ns > 0.5:
        ns += 1
    if ns + npout != n:
        ns += n - (ns + npout)
    return ns


def test_isrf_tables_and_luminosity(tmp_path, built):
    par = configs.write_par(tmp_path, "tiny_isrf")
    m = hc3d.Model(par)
    total, cdf, logcdf, logfreq = isrf_tables(tmp_path / configs.ISRF_FILE)
    assert m.nisrf == NISRF
    np.testing.assert_allclose(m.isrf_cdf, cdf, rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(m.isrf_logcdf, logcdf, rtol=1e-12)
    np.testing.assert_allclose(m.isrf_logfreq, logfreq, rtol=1e-12, atol=1e-14)
    assert m.isrf_cdf[0] == 0.0 and m.isrf_cdf[-1] == 1.0 and np.all(np.diff(m.isrf_cdf) >= 0)
    # newtts.F90:207 and gridset.f90:206-209
    rmax_cm = m.rarr[-1] * 6.9598e10 * m.info.rstar_rsun
    l_isrf = total * 4.0 * np.pi * rmax_cm ** 2 / 4.0 * 10.0
    assert m.info.l_isrf == pytest.approx(l_isrf, rel=1e-6)
    assert m.info.ltot == pytest.approx(m.info.lstar + m.info.l_isrf, rel=1e-15)
    assert m.info.isrf_frac == pytest.approx(m.info.l_isrf / m.info.ltot, rel=1e-15)
    assert 0.2 < m.info.isrf_frac < 0.8
    p = m.run_params(np=4000)
    assert p.ext_illum == 1 and p.n_star == star_packets(m.info.isrf_frac, 4000)
    # without external illumination every packet is stellar
    q = hc3d.Model(configs.write_par(tmp_path / "plain", "tiny")).run_params(np=4000)
    assert q.ext_illum == 0 and q.n_star == 4000


@pytest.mark.parametrize("frac", [0.0, 1e-9, 0.25, 0.5, 0.5430346503563943, 0.9999, 1.0])
def test_star_packet_split(built, frac):
    for n in (0, 1, 2, 3, 7, 10, 999, 1000, 65537, 999999, 16777217, 100000000):
        got = hc3d.star_packets(frac, n)
        assert got == star_packets(frac, n), (frac, n)
        assert 0 <= got <= n


def test_rep_isrf_against_restatement_and_distribution(O, model_factory):
    m = model_factory("tiny_isrf", warm=False)
    rng = np.random.default_rng(5)
    xi = np.concatenate([rng.random(3000), [1e-12, 1e-9, 0.5, 1.0 - 1e-12]])
    got = O.rep_isrf(m, xi)
    cdf, lc, lf = m.isrf_cdf, m.isrf_logcdf, m.isrf_logfreq
    i = np.searchsorted(cdf, xi, side="left")  # nr.f locate: cdf(i) < xi <= cdf(i+1)
    i = np.where(i >= NISRF, NISRF - 1, i)
    i = np.where(i == 0, 1, i)
    want = 10.0 ** (lf[i - 1] + (np.log10(xi) - lc[i - 1]) / (lc[i] - lc[i - 1]) * (lf[i] - lf[i - 1]))
    np.testing.assert_allclose(got, want, rtol=1e-13)
    # the sampled frequencies follow the field's cumulative distribution
    u = got[:3000]
    freq = 10.0 ** lf
    for k in (20, 60, 100, 140, 180):
        frac = np.mean(u <= freq[k])
        assert abs(frac - cdf[k]) < 4.0 * np.sqrt(cdf[k] * (1 - cdf[k]) / 3000) + 1e-3, (k, frac, cdf[k])


def test_external_packets_of_the_oracle(O, model_factory):
    """External packets start just inside rmax heading inwards; every packet
    ends once; the unscattered external packets are left out of sumsub."""
    m = model_factory("tiny_isrf")
    n = 3000
    p = m.run_params(np=n, iter=2, ipeel=1)
    ns = p.n_star
    assert 0 < ns < n
    r = O.run(m, p)
    c = r["counters"]
    assert c[hc3d.CNT["escaped"]] + c[hc3d.CNT["aflux"]] + c[hc3d.CNT["abflux"]] + r["errors"] == n
    unscat = (c[hc3d.CNT["sumall"]] - c[hc3d.CNT["sumsub"]]) / r["stokes_scale"]
    assert unscat == int(unscat) and 0 < unscat <= n - ns
    # the origin slot of external packets (i_orig = 4, propagate.f90 indx 1+i_orig) holds scattered ones only
    assert r["nums"][..., 4].sum() > 0
    # trace of an external packet: first record on the sphere of 0.999999 rmax, in the outermost shell
    recs, _, _ = O.trace(m, p, pid=n - 1)
    x0 = np.array([recs["x"][0], recs["y"][0], recs["z"][0]])
    assert recs["ir"][0] == m.shape4[0] - 1
    assert np.linalg.norm(x0) == pytest.approx(0.999999 * p.rmax, rel=1e-12)
    # a stellar packet starts on the star
    recs, _, _ = O.trace(m, p, pid=0)
    assert recs["ir"][0] == 1
    assert np.linalg.norm([recs["x"][0], recs["y"][0], recs["z"][0]]) == pytest.approx(1.0, rel=1e-12)


def test_thin_model_external_packets_cross_unscattered(O, model_factory):
    """With almost no dust nearly every external packet crosses the grid
    without interacting, so sumall - sumsub counts the external packets."""
    m = model_factory("tiny_isrf", warm=False, MASSD=1e-14, RATE=1e-16, RHOCONST1=1e-30, RHOCONST2=1e-30)
    n = 2000
    p = m.run_params(np=n, iter=2, ipeel=0)
    r = O.run(m, p)
    c = r["counters"]
    unscat = (c[hc3d.CNT["sumall"]] - c[hc3d.CNT["sumsub"]]) / r["stokes_scale"]
    assert unscat >= 0.99 * (n - p.n_star)
    assert c[hc3d.CNT["escaped"]] + c[hc3d.CNT["aflux"]] == n


def test_sharded_external_runs_sum_to_one_run(O, model_factory):
    """Two packet ranges of one iteration (packet_offset) split the stellar
    and external packets by the iteration's global n_star, so their tallies
    add up exactly to the single run's."""
    m = model_factory("tiny_isrf")
    n = 2400
    whole = m.run_params(np=n, iter=2, ipeel=1)
    a = O.run(m, whole)
    k = 1100
    first = m.run_params(np=k, iter=2, ipeel=1, n_star=whole.n_star)
    second = m.run_params(np=n - k, iter=2, ipeel=1, packet_offset=k, n_star=whole.n_star)
    sc = hc3d.tally_scales(n)  # the fixed-point scales of the whole iteration on both ranges
    a = O.run(m, whole, scales=sc)
    b, c = O.run(m, first, scales=sc), O.run(m, second, scales=sc)
    assert 0 < whole.n_star < n
    for key in ("si", "nums", "ti", "numt", "nabs", "dtauabs", "jmean"):
        np.testing.assert_array_equal(a[key], b[key] + c[key], err_msg=key)
