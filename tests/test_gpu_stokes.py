"""GPU parity of the polarised outputs: every Stokes array of the escape SED
(si..sv, propagate.f90:206-319), the peeled SED (ti..tv, peeloff_3d.f90:
249-267) and the broadband images (image_i..image_v, peeloff_3d.f90:
173-177), called through the C-ABI, against the CPU oracle.

* The all-FP64 form follows the oracle packet for packet on the Philox
  streams, so most int64 bins are identical; the test reports the fraction of
  identical bins of every array and bounds it from below.
* The mixed form is compared per bin by chi^2/dof of I, Q and U on the same
  packets (the same Philox streams).  The variance of a bin's difference is
  taken as the sum of both sides' sums of squared weights, as for two
  independent runs.  Two independent oracle runs of the same size give
  chi^2/dof between 0.8 and 1.3 with that estimate (heavy-tailed weights), so
  the bound of 1.2 is asserted on the same streams, where a systematic error
  larger than the Poisson error of a bin still shows; the independent-stream
  values are printed beside it.
* A sign or quadrant error of the Q/U rotation (findangle3, stokespeel) that
  leaves I intact changes the Q and U bins and fails both tests.
"""
from __future__ import annotations

import os
from pathlib import Path

import numpy as np
import pytest

from hochunk3d_gb300 import compare as K
from hochunk3d_gb300 import hc3d
from tests.helpers import splitmix_uniforms, trace_key

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
SED_KEYS = ("si", "sq", "su", "sv", "si2", "sq2", "su2", "sv2", "nums")
PSED_KEYS = ("ti", "tq", "tu", "tv", "ti2", "tq2", "tu2", "tv2", "numt")
IMG_KEYS = ("image_i", "image_q", "image_u", "image_v")
THREADS = max(1, min(16, os.cpu_count() or 1))


@pytest.fixture(scope="module")
def O(built):
    import oracle.oracle as orc

    return orc


def _run(m, prec, p):
    ctx = hc3d.Context(prec).load(m)
    ctx.zero()
    ctx.run(p)
    t = ctx.tallies(p)
    ctx.close()
    return t


@pytest.mark.parametrize("name", ["tiny", "tiny3d"])
def test_fp64_every_stokes_array_matches_oracle(model_factory, O, name):
    """2000 packets on the Philox streams: for every Stokes array of the SED,
    the peeled SED and the images, the fraction of identical int64 bins (over
    bins non-zero on either side) is at least 0.95, and the Q, U sums of every
    peel direction agree with the oracle's to 1 % of that direction's I."""
    g = np.load(GOLDEN / f"trace_{name}.npz")
    m = model_factory(name)
    n = int(g["run_np"])
    p = m.run_params(np=n, iter=3, ipeel=1)
    t = _run(m, hc3d.PREC_FP64, p)
    r = O.run(m, p)
    fr = {k: K.same_fraction(t[k], r[k]) for k in SED_KEYS + PSED_KEYS + IMG_KEYS}
    print(f"\n{name}: identical-bin fractions " + " ".join(f"{k}={v:.4f}" for k, v in fr.items()))
    low = {k: v for k, v in fr.items() if v < 0.95}
    assert not low, low
    for c in ("q", "u", "v"):
        a = t["t" + c][..., 0].sum(axis=(0, 2)).astype(np.float64)
        b = r["t" + c][..., 0].sum(axis=(0, 2)).astype(np.float64)
        i = r["ti"][..., 0].sum(axis=(0, 2)).astype(np.float64)
        np.testing.assert_array_less(np.abs(a - b), 0.01 * i + 8, err_msg=c)
        a = t["image_" + c].sum(axis=(1, 2)).astype(np.float64)
        b = r["image_" + c].sum(axis=(1, 2)).astype(np.float64)
        i = r["image_i"].sum(axis=(1, 2)).astype(np.float64)
        np.testing.assert_array_less(np.abs(a - b), 0.01 * i + 8, err_msg="image_" + c)


def _image_stats(t, r, comp, j, b):
    """Binned image sums of the library (t) and the oracle (r) with the
    oracle's per-pixel ray counts and sums of squared weights; the library
    keeps no per-pixel squares, so the variance of the difference is twice
    the oracle's (both sides sample the same distribution under test)."""
    ss_t, ss_r = t["stokes_scale"], r["stokes_scale"]
    m2 = r["image_m2_d"]
    cnt = K.binned_image(m2[..., 0], b)
    a = (K.binned_image(t["image_" + comp] / ss_t, b), None, cnt)
    o = (K.binned_image(r["image_" + comp] / ss_r, b), K.binned_image(m2[..., 1 + j], b), cnt)
    return K.chi2(o, a, var_b="a")


@pytest.mark.parametrize("name,n,block", [("tiny3d", 200000, 3), ("plain", 100000, 10)])
def test_mixed_stokes_chi2_vs_oracle(model_factory, O, name, n, block):
    """The mixed form against the oracle on the same packets: chi^2/dof <= 1.2
    of Stokes I, Q and U per bin of the escape SED, the peeled SED and the
    images summed over block x block pixels (bins with >= 20 packets)."""
    m = model_factory(name)
    p = m.run_params(np=n, iter=4, ipeel=1)
    t = _run(m, hc3d.PREC_MIXED, p)
    r = O.run(m, p, nthreads=THREADS)
    rep = K.sed_report(r, t)
    for j, c in enumerate("iqu"):
        rep[f"image_chi2_{c}"], rep[f"image_dof_{c}"] = _image_stats(t, r, c, j, block)
    # the same comparison on independent streams, for information
    q = m.run_params(np=n, iter=5, ipeel=1)
    ti = _run(m, hc3d.PREC_MIXED, q)
    ind = K.sed_report(r, ti)
    print(f"\n{name} same streams: " + " ".join(f"{k}={v:.3g}" for k, v in rep.items()))
    print(f"{name} independent streams: " + " ".join(f"{k}={v:.3g}" for k, v in ind.items() if "chi2" in k))
    for tag in ("sed", "peeled_sed", "image"):
        for c in "iqu":
            c2, dof = rep[f"{tag}_chi2_{c}"], rep[f"{tag}_dof_{c}"]
            assert dof >= 20 and c2 <= 1.2, (tag, c, c2, dof)


EPS32 = 2.0 ** -24


def _wall_normal(iface: int, p: np.ndarray) -> np.ndarray:
    """Unit normal at p of the wall family of iface: a sphere (1, 2), a cone
    through p about the z axis (3, 4; the midplane when z = 0), or a plane
    through the z axis (5, 6)."""
    x, y, z = p
    if iface in (1, 2):
        n = p.copy()
    elif iface in (3, 4):
        rho2 = x * x + y * y
        n = np.array([0.0, 0.0, 1.0]) if z == 0.0 else np.array([x, y, -rho2 / z])
    else:
        n = np.array([-y, x, 0.0])
    return n / max(np.linalg.norm(n), 1e-300)


DIR32 = 2.0 ** -11  # direction error of an FP32 scattering: acosf near +-1 loses half the bits


def _first_divergence(want: np.ndarray, got: np.ndarray, wrec, grec):
    """The first differing record j of two traces, its cause and the size of
    the gap relative to its bound.

    Both forms left the common record j-1 along (nearly) the same straight
    segment and stopped at different points of it (a different wall, or a
    wall against an interaction).  The mixed form's stopping point differs
    from the FP64 one by the FP32 rounding of the coordinates (|p| 2^-24 per
    coordinate) and by the FP32 direction of the last scattering or
    emission, whose azimuth comes from acosf and is good to about 2^-11 rad
    near +-1, times the path L travelled since that event.  Either moves the
    crossing of a wall by that amount over |n.u|, n the wall's normal and u
    the direction (a grazing crossing is ill-conditioned).  The divergence is
    a 'tie' when the two stopping points differ by at most 4 times that
    bound for the wall crossed, otherwise a 'walk' error."""
    n = min(len(want), len(got))
    diff = np.nonzero(np.any(want[:n] != got[:n], axis=1))[0]
    j = int(diff[0]) if len(diff) else n
    j = min(j, len(wrec) - 1, len(grec) - 1)
    pos = lambda r, k: np.array([r["x"][k], r["y"][k], r["z"][k]])
    po, pm = pos(wrec, j), pos(grec, j)
    if j == 0:
        return j, "walk", float("inf")
    p0 = pos(wrec, j - 1)
    seg = po - p0 if np.linalg.norm(po - p0) > np.linalg.norm(pm - p0) else pm - p0
    u = seg / max(np.linalg.norm(seg), 1e-300)
    gap = abs(float(np.dot(pm - p0, u)) - float(np.dot(po - p0, u)))
    iface = int(got[j][4]) if got[j][4] > 0 else int(want[j][4])
    where = pm if got[j][4] > 0 else po
    ev = max([i for i in range(j) if want[i][0] != 1] or [0])  # the last emission or interaction
    path = float(np.sum(np.linalg.norm(np.diff(np.stack([pos(wrec, i) for i in range(ev, j)] + [where]), axis=0),
                                       axis=1)))
    cos_nu = abs(float(np.dot(_wall_normal(iface, where), u)))
    bound = 4.0 * (EPS32 * np.linalg.norm(where) * np.sqrt(3.0) + DIR32 * path) / max(cos_nu, 1e-12)
    ratio = gap / bound
    return j, ("tie" if ratio <= 1.0 else "walk"), ratio


@pytest.mark.parametrize("name", ["tiny", "tiny3d"])
def test_mixed_trace_divergences_are_near_wall_ties(model_factory, O, name):
    """Where the FP32 walk's cell sequence leaves the FP64 oracle's (same
    injected uniforms), the first differing record is a tie within the FP32
    precision of the position and direction at the wall crossed (see
    _first_divergence); no divergence is a walk error.  At most a quarter of
    the traces diverge."""
    g = np.load(GOLDEN / f"trace_{name}.npz")
    m = model_factory(name)
    ctx = hc3d.Context(hc3d.PREC_MIXED).load(m)
    p = m.run_params(np=32, iter=3, ipeel=1)
    U = splitmix_uniforms(len(g["nrec"]), int(g["nu"]), seed=int(g["seed"]))
    traces = ctx.trace(p, U, max_rec=2048)
    ctx.close()
    report = []
    for k in range(len(g["nrec"])):
        wrec, ex, _ = O.trace(m, p, k, U[k], max_rec=2048)
        want, got = trace_key(wrec), trace_key(traces[k])
        if want.shape == got.shape and np.array_equal(want, got):
            continue
        j, cause, ratio = _first_divergence(want, got, wrec, traces[k])
        report.append((k, j, len(want), cause, ratio, tuple(int(v) for v in want[j]) if j < len(want) else None,
                       tuple(int(v) for v in got[j]) if j < len(got) else None))
    print(f"\n{name}: {len(report)} of {len(g['nrec'])} mixed traces differ from the FP64 oracle")
    for k, j, nw, cause, ratio, a, b in report:
        print(f"  packet {k}: first divergence at record {j} of {nw} ({cause}; gap / FP32 bound = {ratio:.3g}): "
              f"oracle (kind, ir, it, ip, iface) {a}, mixed {b}")
    assert len(report) <= 0.25 * len(g["nrec"])
    walks = [x for x in report if x[3] == "walk"]
    assert not walks, walks
