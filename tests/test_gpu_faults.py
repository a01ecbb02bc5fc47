"""Host-side fault injection on the GPU path (no GPU fault is raised).

Each failure is made on the host -- bad values in the arrays a caller passes,
an empty dust table, a request that is cancelled or cannot be built -- and
the test checks that the C-ABI returns its error code with a message, that
no kernel hangs, and that the context or server stays usable afterwards.
The reference stops the process in these cases (select_dust.f90:24-31,
dust.f90:182, closest_wall.f90:65)."""
from __future__ import annotations

import time

import numpy as np
import pytest

from hochunk3d_gb300 import configs, hc3d
from tests.helpers import make_model

pytestmark = pytest.mark.gpu


@pytest.fixture()
def fresh(tmp_path, built):
    """A tiny model of its own (the tests write into its arrays)."""
    return make_model(tmp_path / "m", "tiny")


@pytest.mark.parametrize("bad", [np.nan, -1e-18, np.inf])
def test_load_grid_rejects_bad_densities(fresh, bad):
    m = fresh
    cell = (5, 7, 0, 0)
    keep = m.densarr[cell]
    m.densarr[cell] = bad
    ctx = hc3d.Context(hc3d.PREC_MIXED)
    with pytest.raises(hc3d.Hc3dError) as e:
        ctx.load(m)
    assert e.value.code == -1 and "densarr" in str(e.value)
    ctx.close()
    m.densarr[cell] = keep
    ctx = hc3d.Context(hc3d.PREC_MIXED).load(m)  # the restored grid loads and runs
    p = m.run_params(np=2000, iter=2, ipeel=1)
    ctx.zero()
    ctx.run(p)
    c = ctx.tallies(p)["counters"]
    assert c[hc3d.CNT["escaped"]] + c[hc3d.CNT["aflux"]] + c[hc3d.CNT["abflux"]] == 2000
    ctx.close()


def test_load_tables_rejects_an_empty_dust_table(fresh):
    m = fresh
    keep = m.nlambda.copy()
    m.nlambda[:] = 0
    ctx = hc3d.Context(hc3d.PREC_MIXED)
    with pytest.raises(hc3d.Hc3dError) as e:
        ctx.load(m)
    assert e.value.code == -1 and "nlambda" in str(e.value)
    ctx.close()
    m.nlambda[:] = keep
    hc3d.Context(hc3d.PREC_MIXED).load(m).close()


@pytest.mark.parametrize("prec", [hc3d.PREC_MIXED, hc3d.PREC_FP64])
def test_zero_opacity_shell_is_crossed(fresh, prec, built):
    """A shell of cells with no dust: packets cross it without an interaction,
    no walk stops (stuck counters and the fault log stay empty), every packet
    is accounted for, and the FP64 form agrees with the oracle."""
    import oracle.oracle as O

    m = fresh
    m.densarr[10:14, :, :, :] = 0.0
    m.massarr[10:14, :, :, :] = 0.0
    ctx = hc3d.Context(prec).load(m)
    n = 20000
    p = m.run_params(np=n, iter=2, ipeel=1)
    ctx.zero()
    ctx.run(p)
    t = ctx.tallies(p)
    c = t["counters"]
    nf, _ = ctx.fault_log()
    ctx.close()
    assert c[hc3d.CNT["stuck"]] == 0 and c[hc3d.CNT["peel_stuck"]] == 0 and nf == 0
    assert c[hc3d.CNT["escaped"]] + c[hc3d.CNT["aflux"]] + c[hc3d.CNT["abflux"]] == n
    assert t["nabs"][10:14].sum() == 0 and t["dtauabs"][10:14].sum() == 0
    assert t["jmean"][10:14].sum() > 0  # the shell is crossed
    if prec == hc3d.PREC_FP64:
        r = O.run(m, p, nthreads=4)
        np.testing.assert_allclose(t["nums"].sum(), r["nums"].sum(), rtol=0.002)
        assert np.mean(t["ti"] == r["ti"]) > 0.97


def test_server_request_errors_and_cancellation(tmp_path, built):
    """A request whose .par file does not exist returns HC3D_ERR_IO; a queued
    request that is cancelled returns HC3D_ERR_CANCELLED without running; a
    running request that is cancelled stops at its next iteration; the
    server goes on serving, and the next request's result is unchanged."""
    par = configs.write_par(tmp_path / "a", "tiny", NP=6000, NPMIN=3000)
    ref = hc3d.Server(slots=1)
    want = ref.wait(ref.submit(par, n_lucy=2))
    ref.close()
    s = hc3d.Server(slots=1)
    missing = s.submit(tmp_path / "nowhere.par", n_lucy=1)
    # one long request on the only slot, then one that waits in the queue
    long_par = configs.write_par(tmp_path / "b", "tiny", NP=3000000, NPMIN=3000000)
    running = s.submit(long_par, n_lucy=50, np_lucy=3000000)
    queued = s.submit(par, n_lucy=2)
    with pytest.raises(hc3d.Hc3dError) as e:
        s.wait(missing)
    assert e.value.code == -6
    assert s.cancel(queued) == 0
    with pytest.raises(hc3d.Hc3dError) as e:
        s.wait(queued)
    assert e.value.code == -9
    t0 = time.perf_counter()
    while s.stats()["running"] == 0 and time.perf_counter() - t0 < 60:
        time.sleep(0.05)
    assert s.cancel(running) == 0
    with pytest.raises(hc3d.Hc3dError) as e:
        s.wait(running)
    assert e.value.code == -9
    assert s.cancel(running) == -1  # waited for already
    got = s.wait(s.submit(par, n_lucy=2))
    st = s.stats()
    s.close()
    assert st["running"] == 0 and st["in_use_bytes"] == 0
    for k in ("si", "nums", "ti", "numt"):
        np.testing.assert_array_equal(got[k], want[k], err_msg=k)
