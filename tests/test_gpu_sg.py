"""GPU parity of the very small grains and PAHs (FSG > 0; emit_common.f90:
31-53, rep_draine.f90, emit_sg.f90, int_mean.f90) against the CPU oracle,
through the C-ABI, on the tiny_sg model: the device slots carry species 1,
2, 3 and 5 (disk 1's small grains).

* Traces fed identical uniforms: the FP64 kernel's (kind, ir, it, ip, iface)
  sequence equals the oracle's, in the first iteration (spectrum row 2) and
  in a later one with the oracle's int_mean result set on the device.
* Counter-based runs: FP64 counts (SEDs, absorptions of both grain kinds)
  and the small grains' path tally identical to the oracle's in >= 95 % of
  the bins; the peeled SED and image sums, which weigh every re-emission by
  exp(-tau) at its frequency, to 1e-9 relative in every bin: a small
  grain's frequency is 10**logfreq, and CUDA's pow and the C library's may
  differ in the last bit, so the peel-off optical depths of those packets do.
* hc3d_lucy_update's int_mean on the device equals the oracle's int_mean of
  the device's own path tally: the same spectrum row in every cell, the
  fraction to 1e-12.
* The mixed form's escape and peeled SEDs are within chi^2/dof <= 1.2 of
  the oracle on the same streams; the Lucy graph equals the step-by-step
  loop; the device density build equals the host build for eight species.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from hochunk3d_gb300 import compare as K
from hochunk3d_gb300 import hc3d
from tests.helpers import splitmix_uniforms, trace_key

pytestmark = pytest.mark.gpu
THREADS = max(1, min(16, os.cpu_count() or 1))


@pytest.fixture(scope="module")
def O(built):
    import oracle.oracle as orc

    return orc


def _iteration1(m, O, n=20000):
    """The oracle's first Lucy iteration and its int_mean result."""
    q = m.run_params(np=n, iter=1, ipeel=0)
    r = O.run(m, q, nthreads=THREADS)
    im, fr = O.int_mean(m, r["jsg"], r["path_scale"], m.info.ltot, q.np, q.rstar_cm)
    return im, fr


@pytest.mark.parametrize("it", [1, 2])
def test_fp64_traces_match_oracle(model_factory, O, it):
    m = model_factory("tiny_sg")
    im = fr = None
    if it > 1:
        im, fr = _iteration1(m, O)
    p = m.run_params(np=32, iter=it, ipeel=1)
    U = splitmix_uniforms(32, 4000, seed=91 + it)
    ctx = hc3d.Context(hc3d.PREC_FP64).load(m)
    if it > 1:
        ctx.set_imean(im, fr)
    traces = ctx.trace(p, U, max_rec=4096)
    ctx.close()
    absorptions = 0
    for k in range(32):
        want, _, _ = O.trace(m, p, k, U[k], max_rec=4096, imean=im, imfract=fr)
        np.testing.assert_array_equal(trace_key(traces[k]), trace_key(want), err_msg=f"packet {k}")
        np.testing.assert_allclose(traces[k]["x"], want["x"], rtol=1e-9, atol=1e-9)
        absorptions += int(np.sum(want["kind"] == 6))
    assert absorptions > 0


def test_fp64_run_matches_oracle(model_factory, O):
    m = model_factory("tiny_sg")
    im, fr = _iteration1(m, O)
    p = m.run_params(np=4000, iter=2, ipeel=1)
    ctx = hc3d.Context(hc3d.PREC_FP64).load(m)
    ctx.set_imean(im, fr)
    ctx.zero()
    ctx.run(p)
    t = ctx.tallies(p)
    nf, _ = ctx.fault_log()
    ctx.close()
    r = O.run(m, p, nthreads=THREADS, imean=im, imfract=fr)
    assert nf == 0 and r["errors"] == 0
    keys = ("si", "sq", "su", "nums", "tq", "tu", "numt", "nabs", "dbig", "dsg", "jsg")
    frac = {k: K.same_fraction(t[k], r[k]) for k in keys + ("ti", "image_i")}
    print("\ntiny_sg identical-bin fractions " + " ".join(f"{k}={v:.4f}" for k, v in frac.items()))
    low = {k: frac[k] for k in keys if frac[k] < 0.95}
    assert not low, low
    for k in ("ti", "image_i"):
        # fixed-point units (x stokes_scale): 1e-9 relative plus 64 units of rounding
        a, b = t[k].astype(np.float64), r[k].astype(np.float64)
        worst = np.max(np.abs(a - b) - 1e-9 * np.abs(b))
        print(f"{k}: largest difference beyond 1e-9 relative: {worst:.3g} units")
        assert worst <= 64.0, (k, worst)
    assert r["dsg"].sum() > 0 and abs(int(t["dsg"].sum()) - int(r["dsg"].sum())) <= 2 + 0.002 * r["dsg"].sum()


def test_device_int_mean_matches_oracle(model_factory, O):
    """An unpeeled first iteration in either form, then hc3d_lucy_update: the
    device's imean and imfract equal the oracle's int_mean of the same jsg."""
    m = model_factory("tiny_sg")
    n = 20000
    p = m.run_params(np=n, iter=1, ipeel=0)
    for prec in (hc3d.PREC_FP64, hc3d.PREC_MIXED):
        ctx = hc3d.Context(prec).load(m)
        ctx.zero()
        ctx.run(p)
        t = ctx.tallies(p)
        ctx.lucy_update(m.info.ltot, n)
        im, fr = ctx.get_imean()
        ctx.close()
        w_im, w_fr = O.int_mean(m, t["jsg"], t["path_scale"], m.info.ltot, n, p.rstar_cm)
        cells = (slice(0, -1), slice(0, -1), slice(0, -1))
        np.testing.assert_array_equal(im[cells], w_im[cells])
        np.testing.assert_allclose(fr[cells], w_fr[cells], rtol=1e-12, atol=1e-13)
        sel = m.densarr[..., 4][cells] > 0
        assert len(set(im[cells][sel].tolist())) > 8


def test_mixed_run_chi2_vs_oracle(model_factory, O):
    m = model_factory("tiny_sg")
    im, fr = _iteration1(m, O)
    p = m.run_params(np=100000, iter=2, ipeel=1)
    ctx = hc3d.Context(hc3d.PREC_MIXED).load(m)
    ctx.set_imean(im, fr)
    ctx.zero()
    ctx.run(p)
    t = ctx.tallies(p)
    nf, _ = ctx.fault_log()
    ctx.close()
    r = O.run(m, p, nthreads=THREADS, imean=im, imfract=fr)
    assert nf == 0
    rep = K.sed_report(r, t)
    print("\ntiny_sg mixed vs oracle: " + " ".join(f"{k}={v:.3g}" for k, v in rep.items()))
    for tag in ("sed", "peeled_sed"):
        for c in "iqu":
            c2, dof = rep[f"{tag}_chi2_{c}"], rep[f"{tag}_dof_{c}"]
            assert dof >= 20 and c2 <= 1.2, (tag, c, c2, dof)
    # the small grains take the oracle's share of the absorptions (the totals
    # themselves scatter by the packets trapped in the disk midplane, each
    # absorbed thousands of times)
    share_t = float(t["dsg"].sum()) / float(t["dsg"].sum() + t["dbig"].sum())
    share_r = float(r["dsg"].sum()) / float(r["dsg"].sum() + r["dbig"].sum())
    print(f"small-grain share of absorptions: mixed {share_t:.5f} oracle {share_r:.5f}")
    assert abs(share_t - share_r) <= 0.02 * share_r


def test_lucy_graph_equals_step_loop(model_factory):
    """Three Lucy iterations with small grains as one CUDA graph: the graph's
    int_mean of each iteration feeds the next, as in the step-by-step loop."""
    m = model_factory("tiny_sg")
    n = 8000
    p = m.run_params(np=n, iter=1, ipeel=0)
    ctx = hc3d.Context(hc3d.PREC_FP64).load(m)
    td_g, _ = ctx.lucy_iterations(p, 3, m.info.ltot)
    im_g, fr_g = ctx.get_imean()
    t_g = ctx.tallies(p)
    ctx.close()
    ctx = hc3d.Context(hc3d.PREC_FP64).load(m)
    for k in range(3):
        q = m.run_params(np=n, iter=1 + k, ipeel=0)
        ctx.zero()
        ctx.run(q)
        td, _, _ = ctx.lucy_update(m.info.ltot, n)
    im_s, fr_s = ctx.get_imean()
    t_s = ctx.tallies(p)
    ctx.close()
    np.testing.assert_array_equal(td_g, td)
    np.testing.assert_array_equal(im_g, im_s)
    np.testing.assert_array_equal(fr_g, fr_s)
    for key in ("nabs", "dsg", "jsg"):
        np.testing.assert_array_equal(t_g[key], t_s[key], err_msg=key)


def test_device_densities_eight_species(tmp_path, built):
    from tests.helpers import make_model

    m = make_model(tmp_path / "sg", "tiny_sg", warm=False)
    host, mass = m.densarr.copy(), m.massarr.copy()
    assert m.densities_gpu(0) > 0.0
    np.testing.assert_array_equal(m.densarr == 0.0, host == 0.0)
    np.testing.assert_allclose(m.densarr, host, rtol=1e-12, atol=0.0)
    np.testing.assert_allclose(m.massarr, mass, rtol=1e-12, atol=0.0)
    assert (m.densarr[..., 4] > 0).sum() > 0
