"""The Lucy update that allocates nothing (hc3d_lucy_update_noalloc).

Its results are compared with hc3d_lucy_update() of a context on the same
tallies, on two calls in a row: the second call reuses the library's fixed
scratch array that the first call left behind.  Device buffers are torch
tensors owned by the test, as a caller without cudaMalloc would own its own.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from hochunk3d_gb300 import hc3d

RTOL = 1e-9  # the tolerance of the Lucy parity tests


def _buffers(m, dev, dtauabs, path_scale, tdust_in, tdust_out, n, keep):
    """hc3d_lucy_buffers over device tensors (kept alive in `keep`)."""
    import torch

    def d(a, dtype):
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=dtype).ravel(order="F"))).to(dev)
        keep.append(t)
        return t

    nrg, ntg, npg, ndg = m.shape4
    assert m.ndg_tab >= ndg
    b = hc3d.LucyBuffers()
    b.device = dev.index or 0
    b.stream = torch.cuda.current_stream(dev).cuda_stream
    b.nrg, b.ntg, b.npg, b.ndg = nrg, ntg, npg, ndg
    b.dtauabs = d(dtauabs, np.int64).data_ptr()
    b.path_scale = path_scale
    b.densarr = d(m.densarr, np.float64).data_ptr()
    b.massarr = d(m.massarr, np.float64).data_ptr()
    b.tdust_in = tdust_in.data_ptr()
    b.tdust_out = tdust_out.data_ptr()
    b.nT = m.nT
    b.lTint = d(m.lTint, np.float64).data_ptr()
    b.kappap = d(m.kappap[: m.nT * ndg], np.float64).data_ptr()
    for s in range(ndg):
        b.kappav[s] = m.kappav[s]
    b.ltot = m.info.ltot
    b.np = n
    return b


def _call(b):
    rel, conv = C.c_double(-1.0), C.c_int(-1)
    rc = hc3d.lib().hc3d_lucy_update_noalloc(C.byref(b), C.byref(rel), C.byref(conv))
    assert rc == 0, rc
    return rel.value, bool(conv.value)


@pytest.mark.gpu
def test_noalloc_lucy_matches_context_update_twice(model_factory):
    import torch

    dev = torch.device("cuda", 0)
    m = model_factory("tiny")
    t0 = m.tdust.copy(order="F")
    ctx = hc3d.Context(hc3d.PREC_MIXED).load(m)
    nrg, ntg, npg, ndg = m.shape4
    nslots = min(m.ndg_tab, 4, ndg)
    keep = []
    cur = torch.from_numpy(t0.ravel(order="F").copy()).to(dev)
    n = 40000
    rels = []
    for it in (1, 2):
        p = m.run_params(np=n, iter=it, ipeel=0)
        ctx.zero()
        ctx.run(p)
        tal = ctx.tallies(p)
        want, want_rel, want_conv = ctx.lucy_update(m.info.ltot, n)
        # first call: separate output buffer; second call: in place
        out = torch.empty_like(cur) if it == 1 else cur
        b = _buffers(m, dev, tal["dtauabs"], tal["path_scale"], cur, out, n, keep)
        rel, conv = _call(b)
        got = out.cpu().numpy().reshape(m.shape4, order="F")
        cells = (slice(0, nrg - 1), slice(0, ntg - 1), slice(0, npg - 1), slice(0, nslots))
        np.testing.assert_allclose(got[cells], want[cells], rtol=RTOL, err_msg=f"call {it}")
        assert want_rel > 0.0
        np.testing.assert_allclose(rel, want_rel, rtol=RTOL, err_msg=f"call {it}")
        assert conv == want_conv
        rels.append(rel)
        cur = out
    assert rels[0] != rels[1]
    m.set_tdust(t0)
    ctx.close()


def test_noalloc_rejects_grids_beyond_the_limit(built):
    """Returns HC3D_ERR_INVALID before touching the device (no GPU needed)."""
    b = hc3d.LucyBuffers()
    fake = 256  # never dereferenced: the size check comes first
    for f in ("dtauabs", "densarr", "massarr", "tdust_in", "tdust_out", "lTint", "kappap"):
        setattr(b, f, fake)
    b.nrg, b.ntg, b.npg, b.ndg = 1024, 1024, 129, 1   # 135,266,304 > 2^27
    b.nT, b.np, b.ltot, b.path_scale = 1000, 1, 1.0, 1.0
    rel, conv = C.c_double(0), C.c_int(0)
    assert hc3d.lib().hc3d_lucy_update_noalloc(C.byref(b), C.byref(rel), C.byref(conv)) == -1
    assert hc3d.lib().hc3d_lucy_update_noalloc(None, C.byref(rel), C.byref(conv)) == -1
