"""Statistics that compare two photon-loop results bin by bin.

Every result of the mixed-precision form states its error against the
all-FP64 form (or the CPU oracle) with these measures:

* ``chi2``: chi^2 per degree of freedom of two Stokes sums per bin.  A bin's
  sum is a sum of packet weights w, so its variance is estimated by the sum
  of w^2 (the ``si2``/``ti2`` tallies of propagate.f90:206-319 and
  peeloff_3d.f90:249-267).  Bins with fewer than ``min_count`` packets on
  either side are left out.
* ``max_rel_err``: the largest |a - b| / |b| of Stokes I over bins with at
  least ``min_count`` packets on both sides.
* ``precise_rel_err``: the largest |a - b| / |b| of Stokes I over the bins
  that b measures to better than a given Monte Carlo error
  (sqrt(sum w^2) / sum w), so that a 1 % bound is tested only where the
  bins resolve 1 %.
* ``binned_image``: images summed over b x b pixel blocks, so that the
  per-pixel counts of a small run reach the chi^2 threshold.

Tallies are the dictionaries of ``Context.tallies`` (int64 fixed point with
their scales), or of the CPU oracle, which has the same keys.
"""
from __future__ import annotations

import numpy as np

STOKES = ("i", "q", "u", "v")


def _f(t: dict, key: str, square: bool = False) -> np.ndarray:
    scale = t["square_scale"] if square else t["stokes_scale"]
    return np.asarray(t[key], dtype=np.float64) / scale


def sed_arrays(t: dict, peeled: bool, comp: str, origin: int = 0):
    """(sum, sum of squares, count) of one Stokes component of the escape SED
    (peeled=False: s*, nums) or the peeled SED (peeled=True: t*, numt), for
    the origin component ``origin`` (0: all packets)."""
    p = "t" if peeled else "s"
    n = "numt" if peeled else "nums"
    return (_f(t, p + comp)[..., origin], _f(t, p + comp + "2", True)[..., origin],
            np.asarray(t[n], dtype=np.float64)[..., origin])


def chi2(a, b, min_count: int = 20, var_b=None):
    """chi^2/dof and dof of two binned sums a = (sum, sumsq, count) and b.

    The variance of a - b is the sum of the two sums of squares, or, when
    ``var_b`` is "a", twice a's sum of squares (for a result that has no
    second moments: under the hypothesis that both sides sample the same
    distribution, their variances are equal)."""
    sa, va, na = a
    sb, vb, nb = b
    if var_b == "a":
        vb = va
    ok = (na >= min_count) & (nb >= min_count) & ((va + vb) > 0)
    if not ok.any():
        return float("nan"), 0
    d = (sa - sb)[ok] ** 2 / (va + vb)[ok]
    return float(d.sum() / ok.sum()), int(ok.sum())


def max_rel_err(a, b, min_count: int = 100) -> float:
    """Largest |a - b| / |b| of two binned Stokes-I sums over bins with at
    least min_count packets on both sides."""
    sa, _, na = a
    sb, _, nb = b
    ok = (na >= min_count) & (nb >= min_count) & (sb != 0)
    if not ok.any():
        return float("nan")
    return float(np.max(np.abs(sa[ok] - sb[ok]) / np.abs(sb[ok])))


def precise_rel_err(a, b, mc_max: float = 0.005):
    """(largest |a - b| / |b|, bins) of Stokes I over the bins whose Monte Carlo
    error in b, sqrt(sum w^2) / sum w, is at most mc_max."""
    sa, _, _ = a
    sb, vb, nb = b
    with np.errstate(divide="ignore", invalid="ignore"):
        mc = np.sqrt(vb) / np.abs(sb)
    ok = (nb > 1) & (sb != 0) & (mc <= mc_max)
    if not ok.any():
        return float("nan"), 0
    return float(np.max(np.abs(sa[ok] - sb[ok]) / np.abs(sb[ok]))), int(ok.sum())


def quantiles(x: np.ndarray, qs=(50, 90, 99, 100)) -> dict:
    x = np.asarray(x, dtype=np.float64)
    if x.size == 0:
        return {("max" if q == 100 else f"p{q}"): None for q in qs}
    return {("max" if q == 100 else f"p{q}"): float(np.percentile(x, q)) for q in qs}


def binned_image(img: np.ndarray, b: int) -> np.ndarray:
    """Sum (npeel, nx, nx) images over b x b pixel blocks (edge blocks that do
    not fill b x b are dropped)."""
    k, nx, ny = img.shape
    mx, my = nx // b, ny // b
    return img[:, :mx * b, :my * b].reshape(k, mx, b, my, b).sum(axis=(2, 4))


def same_fraction(a: np.ndarray, b: np.ndarray) -> float:
    """Fraction of bins, among those non-zero on either side, whose int64
    values are identical."""
    nz = (a != 0) | (b != 0)
    if not nz.any():
        return 1.0
    return float(np.mean(a[nz] == b[nz]))


def sed_report(a: dict, b: dict, min_count: int = 20, rel_min_count: int = 100, peeled: bool = True) -> dict:
    """chi^2/dof of I, Q, U (and V) of the escape SED and, when both carry it,
    the peeled SED, and the largest relative Stokes-I error."""
    out = {}
    for tag, pe in (("sed", False), ("peeled_sed", True)):
        if pe and (not peeled or "ti" not in a or "ti" not in b or np.asarray(a["ti"]).size == 0):
            continue
        for c in STOKES:
            out[f"{tag}_chi2_{c}"], out[f"{tag}_dof_{c}"] = chi2(sed_arrays(a, pe, c), sed_arrays(b, pe, c),
                                                               min_count)
        out[f"{tag}_max_rel_err_i"] = max_rel_err(sed_arrays(a, pe, "i"), sed_arrays(b, pe, "i"), rel_min_count)
    return out
