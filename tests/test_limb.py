"""Limb darkening of the stellar emission (CLIMB=YES): the table and the
sampling of samptabl.f90 (tabl_mod, not shipped, restated with ntab = 100)
and the peel-off weight of newdisktherm.F90:349-355.  CPU only."""
from __future__ import annotations

import numpy as np
import pytest

from hochunk3d_gb300 import configs, hc3d


@pytest.fixture(scope="module")
def O(built):
    import oracle.oracle as orc

    return orc


def test_table_and_sampling(O, model_factory):
    m = model_factory("tiny", warm=False, CLIMB="YES")
    ntab = m.ntab
    assert ntab == 100
    d = 1.0 / ntab
    x = np.concatenate([[0.0], d * np.arange(2, ntab + 1)])
    prob = np.concatenate([[0.0], 0.5 * (x[1:] ** 3 + x[1:] ** 2)])
    np.testing.assert_allclose(m.limb_xmu, x, rtol=0, atol=1e-15)
    np.testing.assert_allclose(m.limb_prob, prob, rtol=1e-15, atol=0)
    assert m.limb_prob[-1] == pytest.approx(1.0, abs=1e-15)
    rng = np.random.default_rng(11)
    xi = np.concatenate([rng.random(4000), [1e-12, 0.5, 1 - 1e-12]])
    got = O.darkening(m, xi)
    # darkening: n = locate(prob, xi); mu = xmu(n+1) - (prob(n+1) - xi) / (prob(n+1) - prob(n)) * delmu
    n = np.clip(np.searchsorted(prob, xi, side="left"), 1, ntab - 1)
    want = x[n] - (prob[n] - xi) / (prob[n] - prob[n - 1]) * d
    np.testing.assert_allclose(got, want, rtol=1e-14, atol=1e-15)
    assert np.all((got > 0) & (got <= 1.0))
    # above the first interval the sampled cosines follow the cumulative (mu^3 + mu^2)/2
    mu = got[:4000]
    for t in (0.2, 0.4, 0.6, 0.8):
        f = 0.5 * (t ** 3 + t ** 2)
        assert abs(np.mean(mu <= t) - f) < 4 * np.sqrt(f * (1 - f) / 4000) + 1e-3


def test_limb_darkened_star_in_the_oracle(O, model_factory):
    """Every packet ends once; limb darkening changes the peeled stellar flux
    (weight 12/5 (mu + mu^2) against 4 mu) and leaves the packet count alone."""
    out = {}
    for climb in ("NO", "YES"):
        m = model_factory("tiny", warm=True, CLIMB=climb)
        n = 2000
        p = m.run_params(np=n, iter=2, ipeel=1)
        assert p.limb == (1 if climb == "YES" else 0)
        r = O.run(m, p)
        c = r["counters"]
        assert c[hc3d.CNT["escaped"]] + c[hc3d.CNT["aflux"]] + c[hc3d.CNT["abflux"]] + r["errors"] == n
        out[climb] = r
    assert not np.array_equal(out["NO"]["ti"], out["YES"]["ti"])
    # the direct stellar peel-off of both: total weight per direction ~ the same (both normalised to 2)
    a = out["NO"]["ti"][..., 1].sum() / out["NO"]["stokes_scale"]
    b = out["YES"]["ti"][..., 1].sum() / out["YES"]["stokes_scale"]
    assert abs(a - b) < 0.1 * a
