"""Benchmark of the GB300 photon-packet Monte Carlo loop.

Workload: the full-3D precision model (grid 400 x 199 x 64 with a seeded
3-level fractal envelope, 80 peel-off directions = 20 inclinations x 4
azimuths, 301^2 broadband Stokes I,Q,U,V images, 50 wavelength bins), on a
Lucy temperature field (two GPU Lucy iterations, averaged over azimuth and
committed; the CPU reference arm uses the same field).  The steps are chunks
of one final, peeled iteration (hc3d_run_chunk): each starts its batch of
packets, the packets in flight carry over to the next step, and the last
timed step runs them all to their end and solves tfinal, so the timed steps
pay for every history of their packets.

  value  packets/s with the model resident in HBM (CUDA events on the
         library's stream around each step; L2 flushed between steps)
  e2e    the same through the C-ABI with host buffers, as a second chunked
         iteration: run parameters in, every tally back to host each step
  roofline  the dominant kernel (transport k_wave or peel-off k_peel_mixed):
         algorithmic bytes per launch (propagation crossings x (4S+16) B, or
         peel crossings x 4S B; S = 3 active species) over its event-timed
         duration, against the measured HBM peak; traffic = DRAM bytes per
         launch from the ncu capture in profiles/traffic_<workload>.txt,
         scaled by crossings
  cpu_baseline  the CPU oracle (C restatement, FP64) on the host cores, on
         a bounded sample of the same workload
  model_grid  models/hr of 12 seeded models of the model-grid distribution
         (photon counts scaled down to 5e4..5e5 per iteration) on the
         model-run server, four concurrent runs against one at a time
  serving  Poisson arrivals at 20 requests/s (SED + 3 inclinations each):
         p50/p99 latency and packets/s against the same requests as an
         offline batch, with the results of both compared

``--impl reference`` times the CPU oracle alone (the reference cannot be
built here: no Fortran compiler and 14 modules missing).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "packets/s mixed vs FP64 on 1 GB300 at ≤1% SED err; models/hr; serving p99 latency"
WORKLOAD = "full3d"
S_ACTIVE = 3
B_PROP = 4 * S_ACTIVE + 16
B_PEEL = 4 * S_ACTIVE


def profiled_traffic(workload: str) -> dict:
    """Per kernel, (DRAM bytes, device ns) per cell crossing from the ncu
    capture summarised in profiles/traffic_<workload>.txt (lines "kernel
    bytes ns"); ns is None for a line without it."""
    p = ROOT / "profiles" / f"traffic_{workload}.txt"
    out = {}
    if p.exists():
        for line in p.read_text().splitlines():
            parts = line.split()
            if len(parts) in (2, 3) and not line.startswith("#"):
                try:
                    out[parts[0]] = (float(parts[1]), float(parts[2]) if len(parts) == 3 else None)
                except ValueError:
                    pass
    return out


def env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def __enter__(self):
        cmd = ["nvidia-smi", f"--id={self.device}",
               "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
               "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
               "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"]
        try:
            self._proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def build_model(tmp: Path, name: str):
    from hochunk3d_gb300 import configs, hc3d

    par = configs.write_par(tmp, name)
    return hc3d.Model(par)


def warm_up_temperatures(model, ctx, n_lucy: int, iters: int = 2):
    """Untimed set-up: Lucy iterations (no peel-off) to a realistic dust field."""
    td = None
    for it in range(1, iters + 1):
        p = model.run_params(np=n_lucy, iter=it, ipeel=0)
        ctx.zero()
        ctx.run(p)
        td, rel, conv = ctx.lucy_update(model.info.ltot, n_lucy)
    model.set_tdust(td)
    return td


def run_cpu_oracle(model, np_, threads, iter_=9, seed_offset=0):
    import oracle.oracle as O

    p = model.run_params(np=np_, iter=iter_, ipeel=1, packet_offset=seed_offset)
    t0 = time.perf_counter()
    r = O.run(model, p, nthreads=threads)
    return time.perf_counter() - t0, r


def cpu_baseline(model, workload, budget_s: float = 15.0):
    """The oracle (FP64 C restatement) on all host cores, on a time-boxed
    sample of the workload: the threads claim consecutive packet ids one at
    a time for budget_s seconds, then finish the packets they hold; the rate
    is the packets run over the whole time.  Crossings/s is reported beside
    packets/s: it depends less on how many long histories the sample holds."""
    import oracle.oracle as O

    threads = os.cpu_count() or 1
    p = model.run_params(np=1 << 30, iter=9, ipeel=1, packet_offset=1 << 40)
    t0 = time.perf_counter()
    done, r = O.run_timed(model, p, threads, budget_s)
    dt = time.perf_counter() - t0
    cross = int(r["counters"][10] + r["counters"][11])
    return {"value": done / dt, "unit": "packets/s", "cores": threads, "kind": "port",
            "crossings_per_s": cross / dt,
            "sample": f"{done} packets of the {workload} peeled iteration claimed for {budget_s:.0f} s (oracle C "
                      f"restatement, FP64, {threads} threads, {dt:.1f} s with the packets in hand)"}


GRID_SHAPES = [(100, 99, 2), (200, 199, 2), (200, 199, 33)]  # NRG, NTG, NPG (NPG = azimuthal cells + 1)


def model_grid_pars(tmp: Path, n: int, np_lo: float, np_hi: float, seed: int):
    """Seeded models of the model-grid distribution: log-uniform disk mass
    1e-4..0.1 Msun and infall rate 1e-7..1e-4 Msun/yr, cavity angle 5..45 deg,
    stellar temperature 3000..10000 K, a grid of GRID_SHAPES, photon counts
    log-uniform in [np_lo, np_hi]; two Lucy iterations and the peeled one."""
    from hochunk3d_gb300 import configs

    rng = np.random.default_rng(seed)
    pars = []
    for k in range(n):
        g = GRID_SHAPES[int(rng.integers(len(GRID_SHAPES)))]
        npk = int(10 ** rng.uniform(math.log10(np_lo), math.log10(np_hi)))
        cav = float(rng.uniform(5.0, 45.0))
        over = {"NRG": g[0], "NTG": g[1], "NPG": g[2], "MASSD": float(10 ** rng.uniform(-4, -1)),
                "RATE": float(10 ** rng.uniform(-7, -4)), "THET1": cav, "THET2": cav,
                "TSTAR": float(rng.uniform(3000.0, 10000.0)), "NP": npk, "NPMIN": min(npk, 10000),
                "NIMIN": 2, "NIMAX": 2, "I1": -(1000 + k)}
        pars.append(configs.write_par(tmp / f"model{k:03d}", "plain", **over))
    return pars


def model_grid_throughput(tmp: Path, device: int, n: int = 12, slots: int = 4, np_lo: float = 5e4,
                          np_hi: float = 5e5, one_at_a_time: bool = True):
    """Models per hour of a seeded model grid on the server, with `slots`
    concurrent runs and with one run at a time."""
    from hochunk3d_gb300 import hc3d

    pars = model_grid_pars(tmp / "grid", n, np_lo, np_hi, seed=4)
    out = {"models": n, "packets_per_model": f"log-uniform {np_lo:.0e}..{np_hi:.0e} per iteration",
           "iterations": "2 Lucy + 1 peeled", "grids": [list(g) for g in GRID_SHAPES]}
    # the Lucy iterations of the grid: one batched launch per iteration for all
    # models (hc3d_run_batch) against one launch per model
    models = [hc3d.Model(p) for p in pars]
    ctxs = [hc3d.Context(hc3d.PREC_MIXED, device=device).load(m) for m in models]
    lucy = {}
    for mode in ("batched", "one_by_one"):
        for c, m in zip(ctxs, models):
            c.reset().load(m)
        t0 = time.perf_counter()
        pk = 0
        for it in (1, 2):
            ps = [m.run_params(np=int(m.info.np_lucy), iter=it, ipeel=0) for m in models]
            for c in ctxs:
                c.zero()
            if mode == "batched":
                hc3d.run_batch(ctxs, ps)
            else:
                for c, p in zip(ctxs, ps):
                    c.run(p)
            for c, m, p in zip(ctxs, models, ps):
                c.lucy_update(m.info.ltot, p.np, want_tdust=False)
            pk += sum(p.np for p in ps)
        dt = time.perf_counter() - t0
        lucy[mode] = {"seconds": dt, "packets_per_s": pk / dt}
    for c in ctxs:
        c.close()
    out["lucy_iterations"] = lucy
    # the whole grid with its Lucy iterations batched: the models built on the
    # host, both Lucy iterations of all models as one launch each, then the
    # peeled iterations of the models on `slots` host threads, one context each
    from concurrent.futures import ThreadPoolExecutor

    t0 = time.perf_counter()
    models = [hc3d.Model(p) for p in pars]
    ctxs = [hc3d.Context(hc3d.PREC_MIXED, device=device).load(m) for m in models]
    pk = 0
    for it in (1, 2):
        ps = [m.run_params(np=int(m.info.np_lucy), iter=it, ipeel=0) for m in models]
        for c in ctxs:
            c.zero()
        hc3d.run_batch(ctxs, ps)
        for c, m, p in zip(ctxs, models, ps):
            c.lucy_update(m.info.ltot, p.np, want_tdust=False)
        pk += sum(p.np for p in ps)

    def peeled(cm):
        c, m = cm
        p = m.run_params(np=int(m.info.np), iter=3, ipeel=1)
        c.zero()
        c.run(p)
        c.tallies(p, grid=False)
        return p.np

    with ThreadPoolExecutor(slots) as ex:
        pk += sum(ex.map(peeled, zip(ctxs, models)))
    dt = time.perf_counter() - t0
    for c in ctxs:
        c.close()
    out["batched_lucy_pipeline"] = {"seconds": dt, "models_per_hr": n / dt * 3600.0, "packets_per_s": pk / dt,
                                    "peel_threads": slots}
    # the whole grid as one launch per iteration: both Lucy iterations and
    # the peeled iteration of every model batched (hc3d_run_batch)
    t0 = time.perf_counter()
    models = [hc3d.Model(p) for p in pars]
    ctxs = [hc3d.Context(hc3d.PREC_MIXED, device=device).load(m) for m in models]
    pk = 0
    for it in (1, 2, 3):
        peel = it == 3
        ps = [m.run_params(np=int(m.info.np if peel else m.info.np_lucy), iter=it, ipeel=1 if peel else 0)
              for m in models]
        for c in ctxs:
            c.zero()
        hc3d.run_batch(ctxs, ps)
        for c, m, p in zip(ctxs, models, ps):
            if peel:
                c.tallies(p, grid=False)
            else:
                c.lucy_update(m.info.ltot, p.np, want_tdust=False)
        pk += sum(p.np for p in ps)
    dt = time.perf_counter() - t0
    for c in ctxs:
        c.close()
    out["batched_pipeline"] = {"seconds": dt, "models_per_hr": n / dt * 3600.0, "packets_per_s": pk / dt,
                               "launches": 3}
    for k in ((slots, 1) if one_at_a_time else (slots,)):
        srv = hc3d.Server(slots=k, device=device)
        t0 = time.perf_counter()
        res = [srv.wait(t) for t in [srv.submit(p) for p in pars]]
        dt = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        pk = sum(r["packets"] for r in res)
        key = "concurrent" if k > 1 else "one_at_a_time"
        out[key] = {"slots": k, "seconds": dt, "models_per_hr": n / dt * 3600.0, "packets_per_s": pk / dt,
                    "peak_running": st["peak_running"]}
    return out


def lucy_scale(tmp: Path, device: int, n_iter: int, np_: int) -> dict:
    """The Lucy-scale workload (400 x 399 x 128 cells, 100 frequencies): n_iter
    unpeeled Lucy iterations of np_ packets from the reference's starting
    temperatures (0.1 K), as one CUDA graph (hc3d_lucy_iterations), with the
    convergence maximum max dT/T of each iteration."""
    import torch

    from hochunk3d_gb300 import hc3d

    model = build_model(tmp, "lucy")
    ctx = hc3d.Context(hc3d.PREC_MIXED, device=device).load(model)
    warm = model.run_params(np=20000, iter=900, ipeel=0)  # loads the kernels; untimed
    ctx.zero()
    ctx.run(warm)
    ctx.set_tdust(model.tdust)
    p = model.run_params(np=np_, iter=1, ipeel=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, rel = ctx.lucy_iterations(p, n_iter, model.info.ltot, want_tdust=False)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    ctx.close()
    return {"workload": "lucy", "grid": [int(v) for v in model.shape4[:3]], "cells": int(model.info.ncells),
            "iterations": n_iter, "packets_per_iteration": np_, "seconds": dt,
            "packets_per_s": n_iter * np_ / dt, "max_rel_change_per_iteration": [float(v) for v in rel],
            "note": "one CUDA graph of n iterations (tally reset, packet loop, tfinal); temperatures from 0.1 K"}


def serving_latency(tmp: Path, device: int, n: int = 60, rate: float = 20.0, slots: int = 8, np_req: int = 20000):
    """Requests of models of the model-grid distribution, each asking for its
    SED and three peel-off inclinations (one Lucy iteration of np_req
    packets, a peeled iteration of np_req packets).  The same requests are
    first run as one offline batch, which gives the server's capacity in
    requests/s; then Poisson arrivals at 0.8 of that capacity (a sustainable
    load) and at `rate` requests/s give p50/p99 latency from submission to
    result.  Above capacity the queue grows for as long as requests arrive,
    so the latency there is mostly waiting."""
    from hochunk3d_gb300 import hc3d

    pars = model_grid_pars(tmp / "serve", n, np_req, np_req, seed=5)
    th = np.radians([30.0, 60.0, 85.0])
    req = {"n_lucy": 1, "np_lucy": np_req, "np_": np_req, "thete": th, "phie": np.zeros(3)}
    srv = hc3d.Server(slots=slots, device=device)
    srv.wait(srv.submit(pars[0], **req))  # slot warm-up: pools, queues, kernels
    t1 = time.perf_counter()
    off = [srv.wait(t) for t in [srv.submit(p, **req) for p in pars]]
    off_dt = time.perf_counter() - t1
    capacity = n / off_dt

    def poisson(r, seed):
        gaps = np.random.default_rng(seed).exponential(1.0 / r, n)
        t0 = time.perf_counter()
        tickets, due = [], 0.0
        for k in range(n):
            due += gaps[k]
            wait = t0 + due - time.perf_counter()
            if wait > 0:
                time.sleep(wait)
            tickets.append(srv.submit(pars[k], **req))
        res = [srv.wait(t) for t in tickets]
        span = time.perf_counter() - t0
        lat = np.array([x["t_done"] - x["t_submit"] for x in res]) * 1000.0
        svc = np.array([x["t_done"] - x["t_admit"] for x in res]) * 1000.0
        same = all(np.array_equal(a["si"], b["si"]) and np.array_equal(a["ti"], b["ti"]) for a, b in zip(res, off))
        return {"rate_per_s": r, "utilisation": r / capacity, "p50_ms": float(np.percentile(lat, 50)),
                "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max()),
                "run_p50_ms": float(np.percentile(svc, 50)), "run_p99_ms": float(np.percentile(svc, 99)),
                "packets_per_s": sum(x["packets"] for x in res) / span, "results_equal_to_offline_batch": bool(same)}

    sustainable = poisson(0.8 * capacity, 7)
    at_rate = poisson(rate, 6)
    srv.close()
    return {"requests": n, "slots": slots,
            "request": f"1 Lucy x {np_req:.0e} + peeled {np_req:.0e} packets, SED + 3 inclinations",
            "capacity_requests_per_s": capacity,
            "offline_batch_packets_per_s": sum(r["packets"] for r in off) / off_dt,
            "sustainable": sustainable, "at_rate": at_rate,
            # the keys of a single arrival rate, at the stated rate
            "rate_per_s": rate, "p50_ms": at_rate["p50_ms"], "p99_ms": at_rate["p99_ms"],
            "results_equal_to_offline_batch": sustainable["results_equal_to_offline_batch"] and
            at_rate["results_equal_to_offline_batch"]}


def shared_field(model, workload: str):
    """The temperature field both arms run their timed packets on, and its
    description: for the full-3D workload the committed azimuthal average of
    the GPU's two Lucy set-up iterations (tests/golden/make_lucy_field.py),
    otherwise the analytic warm profile of the tests."""
    from tests.helpers import warm_tdust

    if workload == "full3d":
        try:
            from tests.golden.make_lucy_field import LUCY_PACKETS, field

            return field(model), (f"Lucy field of two set-up iterations x {LUCY_PACKETS} packets, azimuthal average "
                                  "(tests/golden/full3d_tdust_phiavg.npz)")
        except (OSError, ValueError):
            pass
    return warm_tdust(model), "analytic warm profile, T = 1600 K (r/Rsub)^-0.45"


def concurrent_batches(model, prec, device: int, n_total: int, k: int, it: int, ipeel: int, seed_shift: int = 0):
    """One iteration of n_total packets as k concurrent runs of n_total / k
    packets (packet ranges of the same streams, each on its own context and
    stream, driven by its own host thread).  The per-batch tallies give
    batch-means error bars; their sum equals one run's tallies exactly (int64
    fixed point, packets keyed by their global id).  Returns (wall seconds,
    list of per-batch tallies)."""
    import threading

    import torch

    from hochunk3d_gb300 import hc3d

    nb = n_total // k
    ctxs = [hc3d.Context(prec, device=device).load(model) for _ in range(k)]
    for c in ctxs:  # loads the kernels; untimed
        c.zero()
        c.run(model.run_params(np=1000, iter=500, ipeel=ipeel))
        c.zero()
    params = []
    for b in range(k):
        q = model.run_params(np_total=n_total, np=nb, iter=it, ipeel=ipeel, packet_offset=b * nb)
        q.seed = q.seed + seed_shift
        params.append(q)
    errs = []

    def work(c, q):
        try:
            c.run(q)
        except Exception as e:  # noqa: BLE001 - reported below
            errs.append(e)

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    th = [threading.Thread(target=work, args=(c, q)) for c, q in zip(ctxs, params)]
    for t_ in th:
        t_.start()
    for t_ in th:
        t_.join()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    if errs:
        raise errs[0]
    tal = [c.tallies(q, grid=ipeel == 0) for c, q in zip(ctxs, params)]
    for c in ctxs:
        c.close()
    return dt, tal


def batch_stats(parts: list, total_key) -> tuple[np.ndarray, np.ndarray]:
    """(sum, batch-means standard error of the sum) over the batches of a
    quantity total_key(tallies) -> array."""
    x = np.stack([total_key(t) for t in parts]).astype(np.float64)
    k = x.shape[0]
    return x.sum(axis=0), np.sqrt(k * x.var(axis=0, ddof=1))


def fp64_comparison(model, td_init, td_lucy, td_sed, device: int, n_sed: int, n_lucy: int, k: int = 8) -> dict:
    """The mixed form against the all-FP64 form on the same inputs and the
    same packet streams, with each error set beside the Monte Carlo error of
    the statistic it is measured on.

    The Monte Carlo error of a bin comes from batch means: the peeled batch
    runs as k concurrent runs of n_sed / k packets (concurrent_batches), and
    the spread of the k partial sums gives the error of the total.  (The sum
    of squared weights of a bin underestimates it: one packet's long random
    walk puts many correlated peel-off rays in the same bin.)  Bins the FP64
    run measures to <= 0.5 % are "precise"; the <= 1 % criterion is tested on
    them, at the resolution of the SED bins and of their sums over frequency
    (per inclination or peel-off direction) and over inclination (per
    frequency).  Both forms are timed alike (the k runs' wall time).

    Lucy: both forms run the two set-up iterations on the same streams from
    the same starting field td_init (td_lucy is the mixed form's result).  The
    temperatures are compared in the cells whose absorbed-energy tally of the
    second iteration has a batch-means error <= 1 % (about 0.25 % in T, which
    goes as the fourth root), from k concurrent batches of the mixed form's
    second iteration."""
    import torch

    from hochunk3d_gb300 import hc3d

    out = {}

    def lucy(prec):
        model.set_tdust(td_init)
        c = hc3d.Context(prec, device=device).load(model)
        t0 = time.perf_counter()
        for it in (1, 2):
            p = model.run_params(np=n_lucy, iter=it, ipeel=0)
            c.zero()
            c.run(p)
            td, _, _ = c.lucy_update(model.info.ltot, n_lucy)
            if it == 1:
                td1 = td
        dt = time.perf_counter() - t0
        c.close()
        return td, td1, dt

    td64, _, lucy_s = lucy(hc3d.PREC_FP64)
    _, td1_mixed, _ = lucy(hc3d.PREC_MIXED)
    # the error of the second iteration's tally, by batch means, on the mixed form's first-iteration field
    model.set_tdust(td1_mixed)
    _, parts = concurrent_batches(model, hc3d.PREC_MIXED, device, n_lucy, k, 2, 0)
    e_sum, e_err = batch_stats(parts, lambda t: t["dtauabs"])
    with np.errstate(divide="ignore", invalid="ignore"):
        e_rel = np.where(e_sum > 0, e_err / e_sum, np.inf)
    levels = {}
    holds = True
    for lim in (0.01, 0.04):
        sel = (e_rel <= lim) & (td64 > 1.0 / 11605.0) & (model.densarr > 0)
        rel = np.abs(td_lucy[sel] - td64[sel]) / td64[sel]
        levels[f"tally_err_le_{lim:g}"] = {"cells": int(sel.sum()), "tdust_rel": K_quantiles(rel),
                                           "max_rel": float(rel.max()) if rel.size else None}
        # <= 1 % in every cell measured to 0.25 %; at the 1 % level, in 99 % of the cells (the
        # differences there are of the size of the Monte Carlo error itself)
        if rel.size:
            holds = holds and (rel.max() if lim == 0.01 else np.percentile(rel, 99)) <= 0.01
    out["lucy"] = {"iterations": 2, "packets_per_iteration": n_lucy,
                   "cells_with_dust": int((model.densarr > 0).sum()),
                   "criterion": "cells whose second-iteration absorbed-energy tally has a batch-means error "
                                f"<= 1 % or <= 4 % ({k} batches; about 0.25 % or 1 % in T, its fourth root): "
                                "every cell of the first set, and 99 % of the second, within 1 %",
                   "levels": levels, "tdust_err_le_1pct": bool(holds), "fp64_seconds": lucy_s}
    # the speed of both forms, measured as the timed steps are: a chunk in
    # the steady state of an iteration (after a chunk that fills the pool)
    model.set_tdust(td_sed)

    def chunk_rate(prec, n_chunk):
        c = hc3d.Context(prec, device=device).load(model)
        c.zero()
        np_it = 3 * n_chunk
        c.run_chunk(model.run_params(np_total=np_it, np=n_chunk, iter=502, ipeel=1), np_it, False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c.run_chunk(model.run_params(np_total=np_it, np=n_chunk, iter=502, ipeel=1, packet_offset=n_chunk),
                    np_it, False)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        c.zero()
        c.close()
        return n_chunk / dt

    n_chunk = max(20000, n_sed // 5)
    r64 = chunk_rate(hc3d.PREC_FP64, n_chunk)
    r32 = chunk_rate(hc3d.PREC_MIXED, n_chunk)
    # the error: the peeled batch in both forms, as k concurrent batches
    t64, pa = concurrent_batches(model, hc3d.PREC_FP64, device, n_sed, k, 501, 1)
    t32, pb = concurrent_batches(model, hc3d.PREC_MIXED, device, n_sed, k, 501, 1)
    sed = {}
    ok = True
    views = {
        "sed": (lambda t: t["si"][..., 0].astype(np.float64) / t["stokes_scale"]),
        "peeled_sed": (lambda t: t["ti"][..., 0].astype(np.float64) / t["stokes_scale"]),
    }
    for tag, f in views.items():
        a, ea = batch_stats(pa, f)
        b, _ = batch_stats(pb, f)
        res = {}
        # bins; sums over frequency (per inclination / direction); sums over angle (per frequency)
        for lvl, red in (("bins", lambda x: x), ("per_angle", lambda x: x.sum(axis=0)),
                         ("per_frequency", lambda x: x.reshape(x.shape[0], -1).sum(axis=1))):
            av, bv = red(a), red(b)
            ev = np.sqrt(red(ea ** 2)) if lvl == "bins" else None
            if ev is None:  # the error of a sum of bins: batch means of the summed quantity
                ev = batch_stats(pa, lambda t, f=f, red=red: red(f(t)))[1]
            with np.errstate(divide="ignore", invalid="ignore"):
                mc = np.where(av != 0, ev / np.abs(av), np.inf)
                err = np.where(av != 0, np.abs(bv - av) / np.abs(av), np.inf)
            pr = mc <= 0.005
            res[lvl] = {"precise": int(pr.sum()), "of": int((av != 0).sum()),
                        "max_rel_err": float(err[pr].max()) if pr.any() else None,
                        "median_mc_err_of_precise": float(np.median(mc[pr])) if pr.any() else None}
            if pr.any():
                ok = ok and err[pr].max() <= 0.01
        tot_a, tot_b = float(a.sum()), float(b.sum())
        res["flux_rel_err"] = abs(tot_b - tot_a) / abs(tot_a) if tot_a else None
        sed[tag] = res
    ia = sum(t["image_i"].astype(np.float64).sum() for t in pa)
    ib = sum(t["image_i"].astype(np.float64).sum() for t in pb)
    out.update({"value": r64, "unit": "packets/s", "packets_per_step": n_chunk,
                "step": "a chunk in the steady state of a peeled iteration, as the timed steps",
                "mixed_same_step": r32, "speedup_mixed_over_fp64": r32 / r64,
                "error_batches": {"packets": n_sed, "batches": k, "fp64_seconds": t64, "mixed_seconds": t32,
                                  "note": "k concurrent runs of n / k packets that drain (error bars only)"},
                "sed_vs_fp64": sed, "image_flux_rel_err": abs(ib - ia) / abs(ia) if ia else None,
                "sed_err_le_1pct": bool(ok),
                "criterion": "Stokes I of every bin (and sum of bins) the FP64 run measures to <= 0.5 % "
                             "Monte Carlo error (batch means) is within 1 % in the mixed form",
                "same_streams": True})
    return out


def K_quantiles(x):
    from hochunk3d_gb300 import compare as K

    return K.quantiles(x)


def reference_arm(args):
    """The reference's method on the host cores: the oracle (FP64 C
    restatement) with all threads, on the workload and temperature field of
    the GPU arm's default steps (shared_field).  A step is a time-boxed
    sample: the threads claim the step's packets one at a time for about
    3 s, then finish those they hold.  Only the host model set-up
    (libhc3d_host.so) and the oracle are loaded."""
    rank, world, _ = env_rank()
    if rank != 0:
        return
    with tempfile.TemporaryDirectory() as td:
        from hochunk3d_gb300.build import build_host_library, build_oracle

        build_host_library()
        build_oracle()
        model = build_model(Path(td), args.workload)
        td_field, field_desc = shared_field(model, args.workload)
        model.set_tdust(td_field)
        import oracle.oracle as O

        threads = os.cpu_count() or 1
        step_s = 3.0
        times, cross, done_total = [], 0, 0
        for s in range(args.warmup + args.steps):
            p = model.run_params(np=1 << 30, iter=9, ipeel=1, packet_offset=(s + 1) << 32)
            t0 = time.perf_counter()
            done, r = O.run_timed(model, p, threads, step_s)
            dt = time.perf_counter() - t0
            if s >= args.warmup:
                times.append(dt)
                done_total += done
                cross += int(r["counters"][10] + r["counters"][11])
        v = done_total / sum(times)
        n = done_total // max(len(times), 1)
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "packets/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / len(times),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic",
                "config": {"workload": args.workload, "packets_per_step": n,
                           "temperatures": field_desc + " (the GPU arm's timed steps)"},
                "cpu_baseline": {"value": v, "unit": "packets/s", "cores": threads, "kind": "port",
                                 "crossings_per_s": cross / sum(times),
                                 "sample": f"about {n} packets per step (claimed for {step_s:.0f} s, then "
                                           f"finished), oracle C restatement with {threads} threads"},
                "e2e": {"value": v, "unit": "packets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--step-seconds", type=float, default=2.0)
    ap.add_argument("--packets", type=int, default=1_000_000, help="packets per step (0 = calibrate)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lucy-packets", type=int, default=2_000_000)
    ap.add_argument("--workload", default=WORKLOAD, help="model of configs.CONFIGS (full3d, plain, ...)")
    ap.add_argument("--temps", default="shared", choices=["shared", "warm", "lucy"],
                    help="temperature field of the timed steps: the field the reference arm also uses (default; "
                         "see shared_field), the analytic warm profile, or this run's two Lucy set-up iterations")
    ap.add_argument("--other-temps", action="store_true",
                    help="also time two whole runs on another temperature field (the analytic warm profile)")
    ap.add_argument("--full-iteration", type=int, default=0,
                    help="packets of the one full peeled iteration timed after the steps (the published run's "
                         "batch: its last long histories are charged once per this many packets); 0 = skip")
    ap.add_argument("--no-fp64", action="store_true", help="skip the all-FP64 comparison run")
    ap.add_argument("--fp64-packets", type=int, default=1_000_000,
                    help="packets of the peeled batch that both forms run for the speed-up and the error")
    ap.add_argument("--no-serving", action="store_true", help="skip the model-grid and serving measurements")
    ap.add_argument("--grid-models", type=int, default=12, help="models of the model-grid measurement")
    ap.add_argument("--grid-packets", default="5e4,5e5",
                    help="photon-count range per iteration of the model-grid measurement (the model-grid "
                         "distribution is 1e6,1e8; the default is scaled down to keep the benchmark to minutes)")
    ap.add_argument("--grid-only", action="store_true",
                    help="run only the model-grid measurement (one-off runs at the distribution's photon counts)")
    ap.add_argument("--lucy-scale", type=int, default=0,
                    help="run only the Lucy-scale measurement: this many Lucy iterations of --lucy-scale-packets "
                         "as one CUDA graph (the configuration's 10 x 1e8)")
    ap.add_argument("--lucy-scale-packets", type=int, default=100_000_000)
    ap.add_argument("--serve-only", action="store_true",
                    help="run only the serving measurement (one-off runs at larger requests)")
    ap.add_argument("--serve-requests", type=int, default=60, help="requests of the serving measurement")
    ap.add_argument("--serve-packets", type=int, default=20000,
                    help="packets of each request's Lucy and peeled iterations (the model-grid distribution is "
                         "1e6..1e8; the default is scaled down to keep the benchmark to minutes)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default peel-off queue depth")
    ap.add_argument("--profile-chunks", type=int, default=0,
                    help="run this many untimed chunks of one peeled iteration after the set-up (no drain) and "
                         "print their crossing and launch counts (the command of the steady-state ncu captures)")
    ap.add_argument("--profile-step", action="store_true",
                    help="run one untimed peeled step after the Lucy set-up and print its crossing and launch "
                         "counts (the command a DRAM-traffic capture of k_wave / k_peel_mixed runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        reference_arm(args)
        return

    import torch

    rank, world, local = env_rank()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from hochunk3d_gb300 import hc3d
    from hochunk3d_gb300.build import build_library, build_oracle

    if rank == 0:
        build_library()
        build_oracle()
    if world > 1:
        torch.distributed.barrier()

    if args.lucy_scale > 0:
        with tempfile.TemporaryDirectory() as td:
            res = lucy_scale(Path(td), local, args.lucy_scale, args.lucy_scale_packets)
        if rank == 0:
            print(json.dumps({"lucy_scale": res}))
        return

    if args.serve_only:
        with tempfile.TemporaryDirectory() as td:
            res = serving_latency(Path(td), local, n=args.serve_requests, np_req=args.serve_packets)
        if rank == 0:
            print(json.dumps({"serving": res}))
        return

    if args.grid_only:
        with tempfile.TemporaryDirectory() as td:
            lo, hi = (float(v) for v in args.grid_packets.split(","))
            res = model_grid_throughput(Path(td), local, n=args.grid_models, np_lo=lo, np_hi=hi,
                                        one_at_a_time=hi <= 1e6)
        if rank == 0:
            print(json.dumps({"model_grid": res}))
        return

    with tempfile.TemporaryDirectory() as td:
        model = build_model(Path(td), args.workload)
        from tests.helpers import warm_tdust

        ctx = hc3d.Context(hc3d.PREC_MIXED, device=local).load(model)
        td_init = model.tdust.copy(order="F")
        td_lucy = warm_up_temperatures(model, ctx, args.lucy_packets)
        td_shared, shared_desc = shared_field(model, args.workload)
        td_steps = {"shared": td_shared, "warm": warm_tdust(model), "lucy": td_lucy}[args.temps]
        steps_desc = {"shared": shared_desc + "; the reference arm's field",
                      "warm": "analytic warm profile, T = 1600 K (r/Rsub)^-0.45",
                      "lucy": f"this run's two Lucy set-up iterations x {args.lucy_packets} packets"}[args.temps]
        model.set_tdust(td_steps)
        ctx.set_tdust(td_steps)
        # the wavefront settings, chosen by timing a sample chunk of the timed
        # steps' size (untimed set-up): a smaller sample favours a shallower
        # peel-off queue than the steps want
        tune_np = args.packets if args.packets > 0 else 200000
        tune = ctx.autotune(model.run_params(np=tune_np, iter=900, ipeel=1)) if not args.no_autotune else None
        stream = torch.cuda.ExternalStream(ctx.stream)
        flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")

        def restore():
            """Untimed: every step starts from the same temperature field (a
            step's tfinal moves the field on)."""
            ctx.set_tdust(td_steps)

        def step(np_, it, off, e2e=False, T=None):
            p = model.run_params(np=np_, iter=it, ipeel=1, packet_offset=off)
            ctx.zero()
            ctx.run(p)
            if e2e:
                T = ctx.tallies(p)
                td_, rel, conv = ctx.lucy_update(model.info.ltot, np_, want_tdust=True)
                return T, td_
            ctx.lucy_update(model.info.ltot, np_, want_tdust=False)
            return None

        if args.profile_chunks > 0:
            # the steady state of a chunked iteration: K chunks of --packets,
            # no drain (the packets in flight are discarded)
            n = args.packets
            np_it = n * (args.profile_chunks + 1)
            ctx.zero()
            launches = 0
            for s_ in range(args.profile_chunks):
                ctx.run_chunk(model.run_params(np_total=np_it, np=n, iter=310, ipeel=1, packet_offset=s_ * n),
                              np_it, False)
                launches += ctx.last_launch_stats()[0]
            c = ctx.tallies(model.run_params(np=n, ipeel=1), grid=False)["counters"]
            ctx.zero()
            print(json.dumps({"workload": args.workload, "packets_per_chunk": n, "chunks": args.profile_chunks,
                              "crossings": {"prop": int(c[hc3d.CNT["cross_prop"]]),
                                            "peel": int(c[hc3d.CNT["cross_peel"]])},
                              "launches": {"k_wave<float>": launches // 2, "k_peel_mixed<float>": launches // 2}}))
            ctx.close()
            return

        if args.profile_step:
            n = args.packets
            step(n, 300, 0)
            c = ctx.tallies(model.run_params(np=n, ipeel=1), grid=False)["counters"]
            waves = ctx.last_launch_stats()[0] // 2
            print(json.dumps({"workload": args.workload, "packets": n,
                              "crossings": {"prop": int(c[hc3d.CNT["cross_prop"]]),
                                            "peel": int(c[hc3d.CNT["cross_peel"]])},
                              "launches": {"k_wave<float>": waves, "k_peel_mixed<float>": waves}}))
            ctx.close()
            return

        # The steps are chunks of one peeled iteration (hc3d_run_chunk): step s
        # starts packets [s n, (s+1) n) and returns once all of them have
        # started; the packets still in flight (the long random walks in the
        # disk) continue in the next step.  The last timed step ends the
        # iteration: it runs every packet still in flight -- those of the
        # warm-up steps too -- to its end and solves tfinal.  So the timed
        # steps carry the whole cost of their packets, the longest histories
        # included, once per iteration as in the published run's 1e8-packet
        # iteration, instead of once per step.
        n = args.packets
        it_no = 300

        def chunk(np_it, s_, final=False, n_=None, it_=it_no):
            q = model.run_params(np_total=np_it, np=n if n_ is None else n_, iter=it_, ipeel=1,
                                 packet_offset=(s_ * world + rank) * n)
            ctx.run_chunk(q, np_it, final)
            return q

        np_it = n * world * (args.warmup + args.steps)
        ctx.zero()
        for w in range(args.warmup):
            chunk(np_it, w)
        ev = []
        kern_ms = []
        c_prev = ctx.tallies(model.run_params(np=n, ipeel=1), grid=False)["counters"]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            for s in range(args.steps):
                last = s == args.steps - 1
                flush.zero_()
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                chunk(np_it, args.warmup + s, final=last)
                if last:
                    ctx.lucy_update(model.info.ltot, np_it, want_tdust=False)
                e1.record(stream)
                e1.synchronize()
                ev.append(e0.elapsed_time(e1))
                kern_ms.append(ctx.last_launch_stats())
        torch.cuda.synchronize()
        c_now = ctx.tallies(model.run_params(np=n, ipeel=1), grid=False)["counters"]
        cross_prop = int(c_now[hc3d.CNT["cross_prop"]] - c_prev[hc3d.CNT["cross_prop"]])
        cross_peel = int(c_now[hc3d.CNT["cross_peel"]] - c_prev[hc3d.CNT["cross_peel"]])
        step_ms = sum(ev) / len(ev)
        if world > 1:
            t = torch.tensor([step_ms], device=f"cuda:{local}")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            step_ms = float(t.item())
        value = n * world / (step_ms / 1000.0)
        steps_detail = {"first_steps_ms": [round(v, 1) for v in ev[:3]], "last_step_ms": round(ev[-1], 1),
                        "note": "the last step runs the iteration's packets in flight to their end and tfinal"}
        restore()

        # end to end through the C-ABI with host buffers: a second chunked
        # iteration of max(2, steps/2) steps, each with the step's run
        # parameters in (peel-off directions, apertures) and the tallies out,
        # its last step ending the iteration
        e2e_times = []
        h2d = d2h = 0
        k2 = max(2, args.steps // 2)
        np_it2 = n * world * k2
        ctx.zero()
        for s in range(k2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            q = chunk(np_it2, s, final=s == k2 - 1, it_=it_no + 1)
            T = ctx.tallies(q, grid=False)
            if s == k2 - 1:
                ctx.lucy_update(model.info.ltot, np_it2, want_tdust=False)
            torch.cuda.synchronize()
            e2e_times.append(time.perf_counter() - t0)
            d2h = sum(v.nbytes for k, v in T.items() if isinstance(v, np.ndarray))
            h2d = 8 * 4 * model.npeel + 8 * len(model.aperture2)
        e2e = n * world / (sum(e2e_times) / len(e2e_times))
        iteration = {"packets": np_it, "timed_steps_packets": n * world * args.steps,
                     "warmup_steps_packets": n * world * args.warmup}
        restore()

        # the published run's whole peeled iteration in one call (full-3D: 1e8
        # packets), timed with CUDA events
        full_it = None
        if args.full_iteration > 0:
            restore()
            ctx.zero()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(args.full_iteration, 470, 1 << 38)
            e1.record(stream)
            e1.synchronize()
            fms = e0.elapsed_time(e1)
            fst = ctx.last_launch_stats()
            full_it = {"packets": args.full_iteration, "seconds": fms / 1000.0,
                       "packets_per_s": args.full_iteration / (fms / 1000.0), "waves": fst[0] // 2,
                       "transport_ms": fst[1], "peel_ms": fst[2],
                       "note": "one disk() call: zero, packet loop, tfinal; the temperatures of the timed steps"}

        # another temperature field, for comparison (--other-temps): steps on
        # the analytic warm profile (hot disk interior: long histories), or on
        # the shared field when the steps ran on another
        other = None
        if args.other_temps:
            td_other = warm_tdust(model) if args.temps != "warm" else td_shared
            ot = []
            for s_ in range(2):
                ctx.set_tdust(td_other)
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                step(n, 450 + s_, (1 << 37) + s_ * n)
                e1.record(stream)
                e1.synchronize()
                ot.append(e0.elapsed_time(e1))
            other = {"temperatures": "analytic warm profile" if args.temps != "warm" else shared_desc,
                     "steps": 2, "ms_per_step": sum(ot) / 2, "packets_per_s": n / (sum(ot) / 2 / 1000.0),
                     "note": "whole runs of n packets (each run drains)"}
            restore()

        fp64 = None
        if not args.no_fp64:
            fp64 = fp64_comparison(model, td_init, td_lucy, td_steps, local, args.fp64_packets, args.lucy_packets)

        launches = sum(k[0] for k in kern_ms)
        tms = sum(k[1] for k in kern_ms) / len(kern_ms)
        pms = sum(k[2] for k in kern_ms) / len(kern_ms)
        waves = launches / 2 / args.steps  # one k_wave and one k_peel launch per wave
        peak, peak_kind = measured_peaks()
        # The dominant kernel.  The two kernels of a wave run on two streams
        # and share the SMs, so each one's event-timed span includes time it
        # waited for the other's blocks; the device time of each alone comes
        # from the ncu launch list (ns per crossing, profiles/traffic_*.txt)
        # scaled by this run's crossings, and the larger one is dominant.
        prof = profiled_traffic(args.workload)
        dev_ms = {}
        for kn, cr in (("k_peel_mixed<float>", cross_peel), ("k_wave<float>", cross_prop)):
            ns = prof.get(kn, (None, None))[1]
            if ns is not None:
                dev_ms[kn] = ns * cr / args.steps / 1e6
        if dev_ms:
            peel_dominant = dev_ms.get("k_peel_mixed<float>", 0.0) >= dev_ms.get("k_wave<float>", 0.0)
        else:
            peel_dominant = pms >= tms
        if peel_dominant:
            kname, kms, kcross, kb = "k_peel_mixed<float>", pms, cross_peel / args.steps, B_PEEL
        else:
            kname, kms, kcross, kb = "k_wave<float>", tms, cross_prop / args.steps, B_PROP
        kbytes = kcross * kb
        achieved = kbytes / (kms / 1000.0) / 1e9
        per_cross = prof.get(kname, (None, None))[0]
        traffic = per_cross * kcross / waves if per_cross is not None else None
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_kind, "traffic": traffic, "kernel": kname,
                "algorithmic_bytes_per_launch": kbytes / waves, "launches_per_step": waves,
                "kernel_ms_per_step": kms, "transport_ms_per_step": tms, "peel_ms_per_step": pms,
                "device_ms_per_step_from_ncu": dev_ms or None,
                "crossings_per_step": {"prop": cross_prop // args.steps, "peel": cross_peel // args.steps}}
        cpu = None
        if rank == 0 and not args.no_cpu_baseline:
            cpu = cpu_baseline(model, args.workload)
        # the density build of gridset on the device against the host build of
        # the same arrays (after the timed region; the loaded grid is unchanged)
        host_dens_ms = model.info.density_host_ms
        model.densities_gpu(local)
        t0 = time.perf_counter()
        dev_ms = model.densities_gpu(local)
        call_ms = (time.perf_counter() - t0) * 1000.0
        grid_build = {"cells": int(model.info.ncells), "host_ms": host_dens_ms, "device_kernel_ms": dev_ms,
                      "device_call_ms": call_ms, "cells_per_s": model.info.ncells / (dev_ms / 1000.0)}
        host_tab_ms = model.info.tables_host_ms
        model.tables_gpu(local)
        t0 = time.perf_counter()
        tab_ms = model.tables_gpu(local)
        tab_call_ms = (time.perf_counter() - t0) * 1000.0
        table_build = {"rows": int(model.nT), "intervals": int(model.nnu), "host_ms": host_tab_ms,
                       "host_threads": min(16, os.cpu_count() or 1), "device_kernel_ms": tab_ms,
                       "device_call_ms": tab_call_ms}
        grid_runs = serving = None
        if rank == 0 and not args.no_serving:
            lo, hi = (float(v) for v in args.grid_packets.split(","))
            grid_runs = model_grid_throughput(Path(td), local, n=args.grid_models, np_lo=lo, np_hi=hi,
                                              one_at_a_time=hi <= 1e6)
            serving = serving_latency(Path(td), local, n=args.serve_requests, np_req=args.serve_packets)
        if rank == 0:
            line = {"metric": METRIC, "value": value, "unit": "packets/s", "n_gpus": world, "steps": args.steps,
                    "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
                    "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
                    "config": {"workload": args.workload,
                               "grid": [model.shape4[0], model.shape4[1], model.shape4[2] - 1],
                               "peel_directions": int(model.npeel), "image": [int(model._p.nxhst)] * 2 + [4],
                               "nfreq": int(model._p.nfreq), "packets_per_step": n,
                               "step": f"a chunk of one peeled iteration of {np_it} packets: {n} packets start "
                                       "in the step, packets in flight at its end continue in the next step, and "
                                       "the last step runs them all to their end and solves tfinal",
                               "steps_detail": steps_detail,
                               "l2": "256 MiB buffer written between timed steps",
                               "temperatures": steps_desc + " (constant over the iteration; tfinal after it)",
                               "autotune": tune},
                    "iteration": iteration, "other_temperatures": other, "full_iteration": full_it,
                    "e2e": {"value": e2e, "unit": "packets/s", "h2d_bytes_per_step": int(h2d),
                            "d2h_bytes_per_step": int(d2h)},
                    "fp64": fp64, "grid_build": grid_build, "table_build": table_build,
                    "model_grid": grid_runs, "serving": serving,
                    "roofline": roof, "cpu_baseline": cpu, "clocks": clk.summary(),
                    "gpu_launches": launches}
            print(json.dumps(line))
        ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
