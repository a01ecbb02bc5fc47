"""GPU parity tests: the sm_103a kernels, called through the C-ABI, against
the CPU oracle and the committed golden traces."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from hochunk3d_gb300 import hc3d
from tests.helpers import splitmix_uniforms, trace_key

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def O(built):
    import oracle.oracle as orc

    return orc


def _ctx(model, precision):
    return hc3d.Context(precision).load(model)


@pytest.mark.parametrize("name", ["tiny", "tiny3d"])
def test_trace_fp64_reproduces_golden_cell_sequence(model_factory, name):
    """Single-packet traces fed identical uniforms: the (kind, ir, it, ip,
    iface) sequence is bit-exact and tau agrees to 1e-5 relative."""
    g = np.load(GOLDEN / f"trace_{name}.npz")
    m = model_factory(name)
    ctx = _ctx(m, hc3d.PREC_FP64)
    p = m.run_params(np=32, iter=3, ipeel=1)
    U = splitmix_uniforms(len(g["nrec"]), int(g["nu"]), seed=int(g["seed"]))
    traces = ctx.trace(p, U, max_rec=2048)
    off = 0
    for k, n in enumerate(g["nrec"]):
        want = np.stack([g[f][off:off + n] for f in ("kind", "ir", "it", "ip", "iface")], axis=1)
        np.testing.assert_array_equal(trace_key(traces[k]), want, err_msg=f"packet {k}")
        np.testing.assert_allclose(traces[k]["tsum"], g["tsum"][off:off + n], rtol=1e-5, atol=1e-12)
        np.testing.assert_allclose(traces[k]["x"], g["x"][off:off + n], rtol=1e-9, atol=1e-9)
        off += n


@pytest.mark.parametrize("name", ["tiny", "tiny3d"])
def test_trace_mixed_follows_fp64(model_factory, name):
    """The FP32 walk reproduces the FP64 cell sequence for most packets."""
    g = np.load(GOLDEN / f"trace_{name}.npz")
    m = model_factory(name)
    ctx = _ctx(m, hc3d.PREC_MIXED)
    p = m.run_params(np=32, iter=3, ipeel=1)
    U = splitmix_uniforms(len(g["nrec"]), int(g["nu"]), seed=int(g["seed"]))
    traces = ctx.trace(p, U, max_rec=2048)
    same = 0
    off = 0
    for k, n in enumerate(g["nrec"]):
        want = np.stack([g[f][off:off + n] for f in ("kind", "ir", "it", "ip", "iface")], axis=1)
        got = trace_key(traces[k])
        same += int(got.shape == want.shape and np.array_equal(got, want))
        off += n
    assert same >= 0.75 * len(g["nrec"]), same


@pytest.mark.parametrize("name", ["tiny", "tiny3d"])
def test_stream_run_fp64_matches_oracle(model_factory, O, name):
    """2000 packets on the Philox streams: the FP64 kernel and the oracle
    agree packet for packet (counts equal up to rare last-ulp branch flips of
    the device transcendentals)."""
    g = np.load(GOLDEN / f"trace_{name}.npz")
    m = model_factory(name)
    ctx = _ctx(m, hc3d.PREC_FP64)
    n = int(g["run_np"])
    p = m.run_params(np=n, iter=3, ipeel=1)
    ctx.zero()
    ctx.run(p)
    t = ctx.tallies(p)
    r = O.run(m, p)
    for k in (0, 4, 5, 6, 9, 12, 13, 14):
        assert abs(int(t["counters"][k]) - int(r["counters"][k])) <= 2 + 0.002 * abs(int(r["counters"][k])), k
    np.testing.assert_allclose(t["nums"].sum(axis=(1, 2, 3)), r["nums"].sum(axis=(1, 2, 3)), rtol=0.01, atol=3)
    np.testing.assert_allclose(t["numt"].sum(axis=(1, 2)), r["numt"].sum(axis=(1, 2)), rtol=0.01, atol=3)
    # most bins agree exactly
    eq = np.mean(t["ti"] == r["ti"])
    assert eq > 0.97, eq
    # and the golden run counts
    np.testing.assert_allclose(t["nums"].sum(axis=(1, 2, 3)), g["run_nums"], rtol=0.01, atol=3)


def test_lucy_update_matches_oracle_tfinal(model_factory, O):
    m = model_factory("tiny")
    for prec in (hc3d.PREC_FP64, hc3d.PREC_MIXED):
        ctx = _ctx(m, prec)
        n = 20000
        p = m.run_params(np=n, iter=2, ipeel=0)
        ctx.zero()
        ctx.run(p)
        t = ctx.tallies(p)
        na = t["dtauabs"] / t["path_scale"]
        want = O.tfinal(m, na, m.info.ltot, n)
        td, rel, conv = ctx.lucy_update(m.info.ltot, n)
        sel = m.densarr > 0
        np.testing.assert_allclose(td[sel], want[sel], rtol=1e-9)


def _chi2(a, b, mask_min=20):
    """chi^2/dof of two Stokes-I bin sums; the variance of a sum of Poisson-many
    weights w is the sum of w^2."""
    ia, ib = a["si_sum"], b["si_sum"]
    va = a["si2_sum"]
    vb = b["si2_sum"]
    ok = (a["n"] >= mask_min) & (b["n"] >= mask_min)
    d = (ia - ib)[ok] ** 2 / np.maximum(va + vb, 1e-300)[ok]
    return d.sum() / max(ok.sum(), 1), int(ok.sum())


def _sed(t, key="si", sq="si2", n="nums"):
    return {"si_sum": t[key][..., 0] / t["stokes_scale"], "si2_sum": t[sq][..., 0] / t["square_scale"],
            "n": t[n][..., 0]}


def test_mixed_vs_fp64_sed_chi2(model_factory):
    """Mixed-precision SEDs and peeled SEDs against the all-FP64 form:
    chi^2/dof <= 1.2 per bin."""
    m = model_factory("tiny3d")
    n = 200000
    res = {}
    for prec in (hc3d.PREC_FP64, hc3d.PREC_MIXED):
        ctx = _ctx(m, prec)
        p = m.run_params(np=n, iter=4, ipeel=1)
        ctx.zero()
        ctx.run(p)
        res[prec] = ctx.tallies(p)
    c2, dof = _chi2(_sed(res[0]), _sed(res[1]))
    assert dof > 20 and c2 <= 1.2, (c2, dof)
    c2, dof = _chi2(_sed(res[0], "ti", "ti2", "numt"), _sed(res[1], "ti", "ti2", "numt"))
    assert dof > 20 and c2 <= 1.2, (c2, dof)


def test_lucy_temperatures_mixed_vs_fp64(model_factory):
    """Three Lucy iterations in each precision: temperatures agree within 1%
    in the cells whose absorbed-path estimator is well sampled."""
    out = {}
    for prec in (hc3d.PREC_FP64, hc3d.PREC_MIXED):
        m = model_factory("tiny", warm=False, NP=40000)
        mm = m
        ctx = _ctx(mm, prec)
        td0 = mm.tdust.copy(order="F")
        n = 60000
        for it in (1, 2, 3):
            p = mm.run_params(np=n, iter=it, ipeel=0)
            ctx.zero()
            ctx.run(p)
            t = ctx.tallies(p)
            td, rel, conv = ctx.lucy_update(mm.info.ltot, n)
        out[prec] = (td, t["dtauabs"] / t["path_scale"])
        mm.set_tdust(td0)
    (ta, na), (tb, _) = out[0], out[1]
    sel = (na > 50) & (ta > 1.0 / 11605)
    rel = np.abs(tb[sel] - ta[sel]) / ta[sel]
    assert sel.sum() > 20
    assert np.median(rel) < 0.01 and np.mean(rel) < 0.01, (np.median(rel), np.mean(rel))


def test_reproducible_and_shardable(model_factory):
    """Same seed -> bit-identical tallies; two shards by packet_offset sum to
    the single call exactly (int64 fixed point, order independent)."""
    m = model_factory("tiny3d")
    ctx = _ctx(m, hc3d.PREC_MIXED)
    n = 30000
    p = m.run_params(np=n, iter=2, ipeel=1)
    ctx.zero(); ctx.run(p); a = ctx.tallies(p)
    ctx.zero(); ctx.run(p); b = ctx.tallies(p)
    ctx.zero()
    ctx.run(m.run_params(np=n // 3, iter=2, ipeel=1))
    ctx.run(m.run_params(np=n - n // 3, packet_offset=n // 3, iter=2, ipeel=1))
    c = ctx.tallies(p)
    for k in ("si", "sq", "nums", "ti", "tq", "numt", "image_i", "image_u", "nabs", "dtauabs", "jmean", "killed"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
        np.testing.assert_array_equal(a[k], c[k], err_msg=k)


def test_full_size_plain_model_properties(model_factory):
    """The plain model at full size (200x199x1 grid, 1e6 packets, 10 peel
    directions, 149^2 images): size-independent properties hold."""
    m = model_factory("plain")
    ctx = _ctx(m, hc3d.PREC_MIXED)
    n = m.info.np
    p = m.run_params(np=n, iter=6, ipeel=1)
    ctx.zero()
    ctx.run(p)
    t = ctx.tallies(p)
    c = t["counters"]
    nf, faults = ctx.fault_log()
    ended = c[hc3d.CNT["escaped"]] + c[hc3d.CNT["aflux"]] + c[hc3d.CNT["abflux"]] + c[hc3d.CNT["stuck"]]
    assert ended == n
    assert c[hc3d.CNT["stuck"]] <= n * 1e-5, (c[hc3d.CNT["stuck"]], faults[:8])
    assert c[hc3d.CNT["sumsub"]] == c[hc3d.CNT["sumall"]]
    # Stokes I of escaping packets is exactly 1 (stokes.f90 normalises by a)
    assert t["si"][..., 0].sum() == t["nums"][..., 0].sum() * int(t["stokes_scale"])
    # polarisation never exceeds intensity in any peeled bin
    ok = t["numt"][..., 0] > 0
    pol = np.hypot(t["tq"][..., 0], t["tu"][..., 0])[ok]
    assert np.all(pol <= t["ti"][..., 0][ok] * (1 + 1e-6) + 8)
    # the broadband image holds the peeled flux that lands inside the image
    assert t["image_i"].sum() <= t["ti"][..., 0].sum() + 8 * t["numt"][..., 0].sum()


def test_invalid_arguments_are_rejected(model_factory):
    m = model_factory("tiny")
    ctx = _ctx(m, hc3d.PREC_MIXED)
    with pytest.raises(hc3d.Hc3dError) as e:
        ctx.run(m.run_params(np=-5))
    assert e.value.code == -1
    with pytest.raises(hc3d.Hc3dError) as e:
        ctx.run(m.run_params(np=10, ipeel=1, npeel=1000))
    assert e.value.code == -1
    # limb darkening needs the table that a CLIMB=YES model loads
    with pytest.raises(hc3d.Hc3dError) as e:
        ctx.run(m.run_params(np=10, limb=1))
    assert e.value.code == -1 and "limb" in str(e.value)
    with pytest.raises(hc3d.Hc3dError) as e:
        ctx.run(m.run_params(np=10, limb=2))
    assert e.value.code == -1


def test_tts_writes_reference_outputs(fixtures_dir, built):
    from hochunk3d_gb300 import configs

    par = configs.write_par(fixtures_dir / "tts", "tiny")
    out = fixtures_dir / "tts_out"
    st = hc3d.tts(par, out)
    assert st.iterations == 3
    flux = (out / "flux.dat").read_text().splitlines()
    assert "nfreq,nph,nmu,nap" in flux[0] and flux[1].startswith("# Lambda")
    assert len(flux) == 2 + 50 * 10
    row = flux[2].split()
    assert len(row) == 9
    peel = sorted(out.glob("peel_flux*.dat"))
    assert len(peel) == 10 * 8  # 10 directions x 8 components
    assert len(list(out.glob("e_ALL_*_I_img.dat"))) == 10
    tm = (out / "tmidplane1.dat").read_text().splitlines()
    assert len(tm) == 2 + 39
    # the .unf grid files of gridset and of each iteration (output.F90:38-150)
    for name in ("marr", "darr", "darrtot", "tarr", "darr_000", "diffus", "diffdir"):
        assert (out / f"{name}.unf").stat().st_size > 0, name
    for it in (1, 2, 3):
        for name in ("diffus", "diffdir", "killed"):
            assert (out / f"{name}_{it:03d}.unf").exists(), (name, it)


@pytest.mark.parametrize("prec", [hc3d.PREC_MIXED, hc3d.PREC_FP64])
def test_lucy_graph_equals_the_step_by_step_loop(model_factory, prec):
    """Three Lucy iterations as one CUDA graph give the temperatures, the
    convergence maxima and the last iteration's tallies of three rounds of
    zero + run + update, bit for bit."""
    m = model_factory("tiny3d", warm=False)
    n = 20000
    td0 = m.tdust.copy(order="F")
    ctx = _ctx(m, prec)
    rels = []
    for it in (1, 2, 3):
        p = m.run_params(np=n, iter=it, ipeel=0)
        ctx.zero()
        ctx.run(p)
        td_a, rel, _ = ctx.lucy_update(m.info.ltot, n)
        rels.append(rel)
    ta = ctx.tallies(m.run_params(np=n, iter=3, ipeel=0))
    ctx.close()
    m.set_tdust(td0)
    ctx = _ctx(m, prec)
    td_b, rel_b = ctx.lucy_iterations(m.run_params(np=n, iter=1, ipeel=0), 3, m.info.ltot)
    tb = ctx.tallies(m.run_params(np=n, iter=3, ipeel=0))
    ctx.close()
    np.testing.assert_array_equal(td_a, td_b)
    np.testing.assert_array_equal(np.array(rels), rel_b)
    for k in ("nabs", "dtauabs", "jmean", "si", "nums", "counters"):
        np.testing.assert_array_equal(ta[k], tb[k], err_msg=k)


@pytest.mark.parametrize("ipeel", [1, 0])
def test_autotune_keeps_results(model_factory, ipeel):
    """The autotuner times every candidate and keeps the fastest; the tallies
    of a batch are the same before and after, and under every setting by hand
    (queue depth, regeneration threshold, queue-slot chunk and block size do
    not change any packet's history)."""
    m = model_factory("tiny3d")
    ctx = _ctx(m, hc3d.PREC_MIXED)
    p = m.run_params(np=30000, iter=2, ipeel=ipeel)
    ctx.zero(); ctx.run(p); a = ctx.tallies(p)
    res = ctx.autotune(m.run_params(np=20000, iter=7, ipeel=ipeel))
    # peeled: 4 queue depths, the 3 other regeneration thresholds, the other peel-off block shape
    assert len(res["candidates"]) == (8 if ipeel else 3) and all(c["ms"] > 0 for c in res["candidates"])
    if ipeel:
        assert {c["regen"] for c in res["candidates"]} == {1, 4, 8, 16}
        assert {c["peel_threads"] for c in res["candidates"]} == {128, 192}
    keys = ("si", "nums", "nabs", "dtauabs", "jmean", "counters") + (("ti", "numt", "image_i") if ipeel else ())
    settings = [{}] + ([{"queue_records": 1 << 20, "regen": 16, "qchunk": 1, "peel_shape": 2},
                        {"queue_records": 1 << 21, "regen": 4, "qchunk": 32, "peel_shape": 1},
                        {"peel_shape": 2}] if ipeel else [])
    for opt in settings:
        if opt:
            ctx.set_wave_options(**opt)
        ctx.zero(); ctx.run(p); b = ctx.tallies(p)
        for k in keys:
            np.testing.assert_array_equal(a[k], b[k], err_msg=f"{k} {opt}")
