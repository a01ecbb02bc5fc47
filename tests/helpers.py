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


def make_gray_model(directory: Path, rate: float = 1e-11, np_: int = 100000) -> hc3d.Model:
    """An optically thin Ulrich envelope (no disk, no cavity) of gray,
    purely absorbing dust around the 4000 K star of the tiny grid: its Lucy
    temperatures must be those of radiative equilibrium with the diluted
    stellar field, T = T* W(r)^(1/4)."""
    d = Path(directory)
    configs.write_fixtures(d)
    lam = 10.0 ** np.linspace(-2.0, 4.0, 241)
    with open(d / "gray_dust.par", "w") as f:
        for l in lam:  # lambda, C_ext, C_sca, kappa, g, p_max, (unused): kappa = 100 cm^2/g at every lambda
            f.write(f" {l:.6e} {1e-20:.6e} {0.0:.6e} {100.0:.6e} {0.0:.6e} {0.0:.6e} {0.0:.6e}\n")
    over = {f"DUSTNAME({k})": "gray_dust.par" for k in range(1, 9)}
    over.update({"MASSD": 0.0, "RATE": rate, "CHOLE": "NO", "NP": np_, "NPMIN": np_})
    return hc3d.Model(configs.write_par(d, "tiny", **over))


def dilution_temperature(model: hc3d.Model) -> np.ndarray:
    """T* <W>^(1/4) per radial cell, <W> the volume mean over the shell of the
    geometric dilution factor W(r) = (1 - sqrt(1 - (R*/r)^2)) / 2 (r in R*)."""
    out = []
    for a, b in zip(model.rarr[:-1], model.rarr[1:]):
        rr = np.linspace(a, b, 2001)
        w = 0.5 * (1.0 - np.sqrt(np.clip(1.0 - 1.0 / rr ** 2, 0.0, 1.0)))
        f, g = w * rr ** 2, rr ** 2  # trapezoid rule on a uniform grid
        out.append((f.sum() - 0.5 * (f[0] + f[-1])) / (g.sum() - 0.5 * (g[0] + g[-1])))
    return model.info.tstar_k * np.array(out) ** 0.25
