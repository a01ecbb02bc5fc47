"""Shared set-up of the parity tests: small models with a warm dust profile."""
from __future__ import annotations

from pathlib import Path

import numpy as np

from hochunk3d_gb300 import configs, hc3d


def warm_tdust(model: hc3d.Model) -> np.ndarray:
    """A deterministic warm temperature field, T = 1600 K (r/Rsub)^-0.45,
    floored at 10 K, in units of K/11605: it exercises absorption,
    re-emission at infrared wavelengths and the sublimation mask."""
    nrg, ntg, npg, ndg = model.shape4
    rave = np.sqrt(model.rarr[:-1] * model.rarr[1:])
    T = 1600.0 * (rave / model.info.rminsub) ** -0.45
    T = np.clip(T, 10.0, 1600.0) / 11605.0
    td = np.full(model.shape4, 0.1 / 11605.0, order="F")
    td[:-1, :, :, :] = T[:, None, None, None]
    return np.asfortranarray(td)


def make_model(directory: Path, name: str, warm: bool = True, **over) -> hc3d.Model:
    par = configs.write_par(directory, name, **over)
    m = hc3d.Model(par)
    if warm:
        m.set_tdust(warm_tdust(m))
    return m


def seeded_uniforms(npkt: int, nu: int, seed: int = 20261203) -> np.ndarray:
    """Uniform draws in (0,1) for the trace harness, independent of Philox."""
    rng = np.random.default_rng(seed)
    u = rng.random((npkt, nu))
    return np.clip(u, 1e-12, 1.0 - 1e-12)


def trace_key(recs) -> np.ndarray:
    """The integer part of a trace: (kind, ir, it, ip, iface) per record."""
    return np.stack([recs["kind"], recs["ir"], recs["it"], recs["ip"], recs["iface"]], axis=1)


def splitmix_uniforms(npkt: int, nu: int, seed: int = 20261203) -> np.ndarray:
    """Uniform draws in (0,1) for the trace harness from splitmix64: exact and
    portable (no dependence on a library's generator)."""
    n = npkt * nu
    idx = np.arange(1, n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    u = ((z >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)
    return u.reshape(npkt, nu)
