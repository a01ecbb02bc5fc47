"""Disk accretion and stellar hot spots on the host and in the CPU oracle
(CPU only):

* the luminosities, accretion rate, shock temperature, spot size and the
  sublimation radius of gridset.f90:72-264, and the packet shares of
  newdisktherm.F90:143-175,209,256,258, against the independent Python
  restatement of tests/golden/ref_routines.py;
* known answers of the samplers: bbfreq draws the Planck function (mean
  4 zeta(5)/zeta(4) T, and its CDF); accretion packets start at radii drawn
  from the accretion luminosity profile, at uniform azimuth and Gaussian
  heights of the disk scale height; hot-spot packets start inside a spot and
  stellar packets fall in a spot as often as the spots cover the star;
* inputs the reference cannot run are rejected with a message.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from hochunk3d_gb300 import configs, hc3d
from tests.golden import ref_routines as R

ZETA4 = math.pi ** 4 / 90.0
ZETA5 = 1.0369277551433699


@pytest.fixture(scope="module")
def acc(tmp_path_factory, built):
    return hc3d.Model(configs.write_par(tmp_path_factory.mktemp("acc"), "tiny_acc"))


@pytest.fixture(scope="module")
def O(built):
    import oracle.oracle as orc

    return orc


def _close(a, b, rtol=1e-12):
    return abs(a - b) <= rtol * max(abs(a), abs(b))


@pytest.mark.parametrize("over", [{}, {"CALPHA": "YES", "ALPHA/MDOT": 0.01, "FMASSD1": 0.7, "ZSCALE(2)": 0.02},
                                  {"CTEMP": "YES", "TSPOT/FSPOT": 9000.0, "NSPOT": 1},
                                  {"CSPOT": "NO", "CRMIN": "AU", "RMIND(1)": 0.2, "RMIND(2)": 0.2}])
def test_luminosities_match_restatement(tmp_path, built, over):
    cfg = dict(configs.BASE)
    cfg.update(configs.CONFIGS["tiny_acc"])
    cfg.update(over)
    m = hc3d.Model(configs.write_par(tmp_path, "tiny_acc", **over))
    i = m.info
    tstar, rstar, massc, massd = 4000.0, 2.0, 0.5, cfg["MASSD"]
    autors = 1.49598e13 / R.RSOL / rstar
    rminsub0 = (1600.0 / tstar) ** (-2.1)  # setup.f90:67
    if cfg["CRMIN"] == "RSUB":
        rmind = [rminsub0 * cfg["RMIND(1)"], rminsub0 * cfg["RMIND(2)"]]
    else:
        rmind = [cfg["RMIND(1)"] * autors, cfg["RMIND(2)"] * autors]
    fm = [cfg["FMASSD1"], 1.0 - cfg["FMASSD1"]]
    z1 = [cfg["ZSCALE(1)"], cfg["ZSCALE(2)"]]  # CZMIN=RSTAR: scale heights at R*
    rmaxd = [cfg["RMAXD(1)"] * autors, cfg["RMAXD(2)"] * autors]
    rmincgs = rstar * R.RSOL
    rho0 = [R.rho0_disk(massd, fm[k], rmaxd[k], rmind[k], cfg[f"A({k + 1})"], cfg[f"B({k + 1})"], z1[k], rmincgs)
            for k in range(2)]
    ialpha = 1 if cfg["CALPHA"] == "YES" else 0
    itemp = 1 if cfg["CTEMP"] == "YES" else 0
    fspot = 1.0 if cfg["CSPOT"] == "NO" else (cfg["TSPOT/FSPOT"] if not itemp else 0.0)
    want = R.accretion_luminosity(tstar, rstar, massc, massd, min(rmind), cfg["RTRUNC"], rho0, z1, ialpha,
                                  cfg["ALPHA/MDOT"], cfg["ALPHA/MDOT"], 0.0, itemp, fspot, cfg["TSPOT/FSPOT"],
                                  cfg["NSPOT"])
    for k in ("lstar", "lacc", "lacc2", "ltot", "accfrac", "accfrac2", "mdot_msun_yr", "tshock_k", "thspot_deg",
              "fspot", "tave_k", "rminsub"):
        assert _close(getattr(i, k), want[k]), (k, getattr(i, k), want[k])
    assert i.accfrac > 0.0 and i.accfrac2 > 0.0
    S = m.sources
    if cfg["CSPOT"] == "YES":
        s1, s2, csprad = R.spot_geometry(cfg["SPOTLAT"], want["thspot_deg"])
        assert S.ispot == 1 and S.nspot == cfg["NSPOT"]
        np.testing.assert_allclose(list(S.spot1), s1, rtol=0, atol=1e-15)
        np.testing.assert_allclose(list(S.spot2), s2, rtol=0, atol=1e-15)
        assert _close(S.csprad, csprad)
    else:
        assert S.ispot == 0
    assert _close(S.tshock, want["tshock_k"] / 11605.0)
    # the new sublimation radius sets the inner disk radius (CRMIN=RSUB) and the accretion radii
    if cfg["CRMIN"] == "RSUB":
        assert _close(S.rddustmin, want["rminsub"] * min(cfg["RMIND(1)"], cfg["RMIND(2)"]))


def test_packet_shares_match_restatement(built):
    rng = np.random.default_rng(11)
    cases = [(1000, 0.0577, 0.632, 0.0), (1000, 0.0, 0.0, 0.0), (997, 0.1, 0.0, 0.3), (20000, 0.0577, 0.632, 0.0),
             (1, 0.5, 0.4, 0.0), (3, 0.34, 0.33, 0.2)]
    for _ in range(200):
        a, b = rng.uniform(0, 0.5, 2)
        cases.append((int(rng.integers(1, 5000)), float(a), float(b), float(rng.uniform(0, 0.5 - a / 2))))
    for n, a, b, f in cases:
        want = R.packet_shares(n, a, b, f)
        n_acc, n_spot, n_star = hc3d.packet_split(a, b, f, n)
        got = {"acc": n_acc, "spot": n_spot - n_acc, "star": n_star - n_spot, "ext": n - n_star}
        assert got == want, (n, a, b, f)
        if b == 0.0 and a == 0.0:
            assert n_star == hc3d.star_packets(f, n)


def test_bbfreq_is_the_planck_function(O):
    """bbfreq at T: x = nu/T has the density 15/pi^4 x^3/(e^x - 1) (energy
    per unit frequency of a blackbody), mean 4 zeta(5)/zeta(4) = 3.8322; the
    oracle's draws for given uniforms equal the restatement's."""
    T = 0.7
    x = O.sample_bbfreq(T, 5, 200000) / T
    assert abs(x.mean() - 4 * ZETA5 / ZETA4) < 4 * x.std() / math.sqrt(len(x))
    # CDF of the Planck energy spectrum: 1 - 15/pi^4 sum_k e^{-kx} (x^3/k + 3x^2/k^2 + 6x/k^3 + 6/k^4)
    xs = np.sort(x)
    k = np.arange(1, 200)[:, None]
    cdf = 1.0 - 15 / math.pi ** 4 * np.sum(np.exp(-k * xs) * (xs ** 3 / k + 3 * xs ** 2 / k ** 2 + 6 * xs / k ** 3
                                                                + 6 / k ** 4), axis=0)
    ks = np.max(np.abs(cdf - (np.arange(1, len(xs) + 1) - 0.5) / len(xs)))
    assert ks < 1.63 / math.sqrt(len(xs)) + 1e-3, ks
    zeta = R.inczeta()
    assert abs(zeta[-1] - ZETA4) < 1e-6
    u = O.stream(5, 1, 17, 5)
    assert x[17] * T == R.bbfreq(T, list(u), zeta)


def test_accretion_points(acc, O):
    m = acc
    S = m.sources
    p = m.run_params(np=40000)
    e = O.sample_emission(m, p, 0, p.n_acc)
    assert np.all(e["kind"] == 1)
    x, y, z = e["x"], e["y"], e["z"]
    r = np.hypot(x, y)
    assert np.all((r > S.rddustmin) & (r < S.rmaxdmax))
    # w = 1/r has the density (1 - sqrt(w)) on (1/rmaxdmax, 1/rddustmin)
    w = np.sort(1.0 / r)
    F = lambda v: v - 2.0 / 3.0 * v ** 1.5
    lo, hi = 1.0 / S.rmaxdmax, 1.0 / S.rddustmin
    cdf = (F(w) - F(lo)) / (F(hi) - F(lo))
    n = len(w)
    assert np.max(np.abs(cdf - (np.arange(1, n + 1) - 0.5) / n)) < 1.63 / math.sqrt(n) + 1e-3
    # uniform azimuth; heights Gaussian in units of sum(fmass z1 r^b)
    phi = np.sort(np.mod(np.arctan2(y, x), 2 * np.pi) / (2 * np.pi))
    assert np.max(np.abs(phi - (np.arange(1, n + 1) - 0.5) / n)) < 1.63 / math.sqrt(n) + 1e-3
    h = S.zfac[0] * r ** S.zexp[0] + S.zfac[1] * r ** S.zexp[1]
    g = z / h
    assert abs(g.mean()) < 4 / math.sqrt(n) and abs(g.std() - 1.0) < 0.05
    # the cell of the start point holds it
    ir, it = e["ir"].astype(int), e["it"].astype(int)
    rr = np.sqrt(x * x + y * y + z * z)
    assert np.all((m.rarr[ir - 1] <= rr) & (rr <= m.rarr[ir]))
    cb = z / rr
    assert np.all((m.costarr[it - 1] >= cb) & (cb >= m.costarr[it]))
    # the gap's cells (no disk dust) emit from the gas, the others from disk slot 1
    has = (m.densarr[ir - 1, it - 1, 0, 0] + m.densarr[ir - 1, it - 1, 0, 1]) > 0
    assert np.all(e["extra"][~has] == -1) and np.all(e["extra"][has] == 0)
    assert 0.02 < np.mean(~has) < 0.8
    # gas packets radiate at the Pringle temperature: nu/T is a Planck draw
    rt = rr[~has]
    t0 = S.gas_num / (S.gas_den * (rt * S.rstar * S.rsun) ** 3)
    T = (t0 * (1 - np.sqrt(1 / rt))) ** 0.25 / 11605.0
    xg = e["nu"][~has] / T
    assert abs(xg.mean() - 4 * ZETA5 / ZETA4) < 5 * xg.std() / math.sqrt(len(xg))


def test_spot_packets(acc, O):
    m = acc
    S = m.sources
    p = m.run_params(np=40000)
    e = O.sample_emission(m, p, p.n_acc, p.n_spot - p.n_acc)
    assert np.all(e["kind"] == 2) and np.all(e["extra"] == 1)
    x, y, z = e["x"], e["y"], e["z"]
    d1 = S.spot1[0] * x + S.spot1[1] * y + S.spot1[2] * z
    d2 = S.spot2[0] * x + S.spot2[1] * y + S.spot2[2] * z
    assert np.all((d1 >= S.csprad - 1e-12) | (d2 >= S.csprad - 1e-12))
    # half of them are X-rays (0.015-0.06 um), the others a Planck draw at the shock temperature
    xr = (e["nu"] >= 1.2398 / 0.06) & (e["nu"] <= 1.2398 / 0.015)
    assert abs(xr.mean() - 0.5) < 5 * math.sqrt(0.25 / len(xr)) + 0.01
    s = e[p.n_spot - p.n_acc - 4000:]
    st = O.sample_emission(m, p, p.n_spot, p.n_star - p.n_spot)
    assert np.all(st["kind"] == 3)
    # stellar packets fall in a spot as often as the spots cover the star: nspot (1 - csprad) / 2
    cover = S.nspot * (1.0 - S.csprad) / 2.0
    f = st["extra"].mean()
    assert abs(f - cover) < 5 * math.sqrt(cover * (1 - cover) / len(st)), (f, cover)
    assert len(s) > 0


@pytest.mark.parametrize("over,msg", [({"CDISKACC": "NO"}, "CDISKACC"), ({"NSPOT": 3}, "NSPOT"),
                                      ({"MASSD": 0.0}, "MASSD"),
                                      ({"CTEMP": "YES", "TSPOT/FSPOT": 3000.0}, "spot")])
def test_unrunnable_inputs_are_rejected(tmp_path, built, over, msg):
    with pytest.raises(hc3d.Hc3dError) as e:
        hc3d.Model(configs.write_par(tmp_path, "tiny_acc", **over))
    assert msg.lower() in str(e.value).lower()


def test_models_without_sources_are_unchanged(tmp_path, built):
    m = hc3d.Model(configs.write_par(tmp_path, "tiny"))
    p = m.run_params(np=1000)
    assert m.sources is None and p.n_acc == 0 and p.n_spot == 0 and p.n_star == 1000
    assert m.info.lacc == 0 and m.info.accfrac == 0 and m.info.tave_k == 4000.0
