"""The model-run server on the GPU (hc3d_server_*): results are the same
alone and in the mix, and admission follows the device-footprint budget."""
from __future__ import annotations

import numpy as np
import pytest

from hochunk3d_gb300 import configs, hc3d

pytestmark = pytest.mark.gpu

KEYS = ("si", "nums", "ti", "numt")


@pytest.fixture(scope="module")
def pars(tmp_path_factory, built):
    d = tmp_path_factory.mktemp("serve")
    out = [configs.write_par(d / "a", "tiny", NP=6000, NPMIN=3000),
           configs.write_par(d / "b", "tiny3d", NP=6000, NPMIN=3000),
           configs.write_par(d / "c", "tiny_isrf", NP=6000, NPMIN=3000),
           configs.write_par(d / "d", "tiny", NP=6000, NPMIN=3000, MASSD=0.001, TSTAR=6000.0, I1=-77)]
    return out


def _run(server, pars, **kw):
    tickets = [server.submit(p, n_lucy=2, **kw) for p in pars]
    return [server.wait(t) for t in tickets]


def test_results_same_alone_and_in_the_mix(pars):
    """Each request alone on a one-slot server, then all four together on a
    four-slot server (their runs overlap on the device): every SED and peeled
    SED is bit-identical."""
    alone = []
    s1 = hc3d.Server(slots=1)
    for p in pars:
        alone += _run(s1, [p])
    s1.close()
    s4 = hc3d.Server(slots=4)
    mixed = _run(s4, pars + pars)  # each model twice, eight requests in flight
    st = s4.stats()
    s4.close()
    assert st["completed"] == 8 and st["peak_running"] >= 2
    for k, r in enumerate(mixed):
        a = alone[k % 4]
        assert r["packets"] == a["packets"] and r["iterations"] == 3
        for key in KEYS:
            np.testing.assert_array_equal(r[key], a[key], err_msg=f"request {k} {key}")
    # the four models really differ
    assert not np.array_equal(alone[0]["si"], alone[3]["si"])


def test_requested_peel_directions_and_packets(pars):
    s = hc3d.Server(slots=2)
    th = np.radians([30.0, 60.0, 85.0])
    t = s.submit(pars[0], n_lucy=1, np_lucy=4000, np_=5000, thete=th)
    r = s.wait(t)
    with pytest.raises(hc3d.Hc3dError):
        s.wait(t)  # a ticket is waited for once
    s.close()
    assert r["ti"].shape[1] == 3 and r["numt"].sum() > 0
    assert r["packets"] == 4000 + 5000 and r["iterations"] == 2


def test_admission_by_device_footprint(pars):
    """With a budget that holds one model at a time, requests run one by one
    (although four slots are free) and still give the same results; a model
    larger than the budget is refused."""
    m = hc3d.Model(pars[0])
    fp = int(hc3d.lib().hc3d_model_footprint(m._h))
    assert fp > 0
    ref = hc3d.Server(slots=1)
    want = _run(ref, pars[:1])[0]
    ref.close()
    s = hc3d.Server(slots=4, hbm_budget=int(1.5 * fp))
    got = _run(s, [pars[0]] * 4)
    st = s.stats()
    assert st["peak_running"] == 1 and st["peak_in_use_bytes"] <= int(1.5 * fp)
    for r in got:
        for key in KEYS:
            np.testing.assert_array_equal(r[key], want[key])
        assert r["footprint_bytes"] == fp
    big_par = configs.write_par(pars[0].parent.parent / "big", "tiny", NRG=100, NTG=99, NPG=17)
    assert int(hc3d.lib().hc3d_model_footprint(hc3d.Model(big_par)._h)) > int(1.5 * fp)
    big = s.submit(big_par, n_lucy=1)
    with pytest.raises(hc3d.Hc3dError) as e:
        s.wait(big)
    assert e.value.code == -3
    s.close()


@pytest.mark.parametrize("prec", [hc3d.PREC_MIXED, hc3d.PREC_FP64])
def test_batched_launch_equals_separate_runs(pars, prec):
    """The unpeeled packet loops of four models in one persistent launch
    (hc3d_run_batch) give each model the tallies of its own run: bit for bit
    in the FP64 form (built without contracted multiply-adds).  The mixed
    form's two kernels (k_transport, k_transport_batch) are compiled
    separately and the compiler may fuse an FP32 multiply and add in one and
    not the other, so a packet can take a different branch after a last-bit
    difference (a diverged long history touches many cells): its tallies
    agree to 1e-3 of each array's total; the counts (si, nums, nabs, killed)
    are identical in 90 % of the bins, and the FP32 path-length sums (jmean,
    dtauabs), whose every crossing may round differently, agree to 1e-4 of the
    bin in 90 % of the bins."""
    models = [hc3d.Model(p) for p in pars]
    params = [m.run_params(np=6000 + 1000 * k, iter=2, ipeel=0) for k, m in enumerate(models)]
    want = []
    for m, p in zip(models, params):
        ctx = hc3d.Context(prec).load(m)
        ctx.zero(); ctx.run(p)
        want.append(ctx.tallies(p))
        ctx.close()
    ctxs = [hc3d.Context(prec).load(m) for m in models]
    for c in ctxs:
        c.zero()
    hc3d.run_batch(ctxs, params)
    for k, (c, p) in enumerate(zip(ctxs, params)):
        got = c.tallies(p)
        for key in ("si", "nums", "nabs", "dtauabs", "jmean", "killed", "counters"):
            if prec == hc3d.PREC_FP64:
                np.testing.assert_array_equal(got[key], want[k][key], err_msg=f"model {k} {key}")
                continue
            a, b = got[key].astype(np.float64), want[k][key].astype(np.float64)
            assert np.abs(a - b).sum() <= 1e-3 * np.abs(b).sum() + 2, (k, key)
            if key in ("jmean", "dtauabs"):
                nz = (a != 0) | (b != 0)
                close = np.abs(a - b) <= 1e-4 * np.maximum(np.abs(a), np.abs(b))
                assert np.mean(close[nz]) >= 0.9, (k, key, float(np.mean(close[nz])))
            elif key != "counters":
                assert np.mean(got[key] == want[k][key]) >= 0.9, (k, key)
        c.close()


@pytest.mark.parametrize("prec", [hc3d.PREC_MIXED, hc3d.PREC_FP64])
def test_batched_peeled_launch_equals_separate_runs(pars, prec):
    """The peeled iterations of four models in one persistent launch
    (hc3d_run_batch, peel-off rays walked by the thread of each event) give
    each model the SED, peeled SED and images of its own wavefront run: bit
    for bit in the FP64 form, and in the mixed form to 1e-3 of each array's
    total (the two paths are separately compiled FP32 code)."""
    models = [hc3d.Model(p) for p in pars]
    params = [m.run_params(np=4000 + 500 * k, iter=3, ipeel=1) for k, m in enumerate(models)]
    want = []
    for m, p in zip(models, params):
        ctx = hc3d.Context(prec).load(m)
        ctx.zero(); ctx.run(p)
        want.append(ctx.tallies(p))
        ctx.close()
    ctxs = [hc3d.Context(prec).load(m) for m in models]
    for c in ctxs:
        c.zero()
    hc3d.run_batch(ctxs, params)
    for k, (c, p) in enumerate(zip(ctxs, params)):
        got = c.tallies(p)
        for key in ("si", "sq", "nums", "ti", "tq", "tu", "numt", "image_i", "image_q", "nabs", "dtauabs"):
            if prec == hc3d.PREC_FP64:
                np.testing.assert_array_equal(got[key], want[k][key], err_msg=f"model {k} {key}")
                continue
            a, b = got[key].astype(np.float64), want[k][key].astype(np.float64)
            assert np.abs(a - b).sum() <= 1e-3 * np.abs(b).sum() + 16, (k, key)
        c.close()
