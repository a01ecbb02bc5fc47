"""ctypes binding of the CPU oracle (oracle/hc3d_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check of
__graft_entry__.py and by the cpu_baseline / reference legs of bench.py.  The
product (hochunk3d_gb300/) never imports it.

Parity status: unpinned at the reference-test level (the reference ships no
tests, golden outputs or runnable build); see the header of hc3d_oracle.c.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from hochunk3d_gb300 import hc3d
from hochunk3d_gb300.hc3d import NO, P, DustTables, Grid, RunParams, SgTables, Tallies, TraceRec, TRACE_DTYPE

ROOT = Path(__file__).resolve().parent
LIB_PATH = ROOT / "_build" / "libhc3d_oracle.so"


class OrcTallies(C.Structure):
    _fields_ = [("fx", Tallies), ("si_d", P(C.c_double)), ("ti_d", P(C.c_double)), ("image_i_d", P(C.c_double)),
                ("dtauabs_d", P(C.c_double)), ("errors", C.c_int64), ("image_m2_d", P(C.c_double))]


_LIB = None


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            from hochunk3d_gb300.build import build_oracle

            build_oracle()
        L = C.CDLL(str(LIB_PATH))
        dp = P(C.c_double)
        L.orc_run_range.argtypes = [P(DustTables), P(Grid), P(RunParams), P(OrcTallies), C.c_int64, C.c_int64]
        L.orc_run_mt.argtypes = [P(DustTables), P(Grid), P(RunParams), P(OrcTallies), C.c_int]
        L.orc_run_mt_timed.argtypes = [P(DustTables), P(Grid), P(RunParams), P(OrcTallies), C.c_int, C.c_double,
                                       P(C.c_int64)]
        L.orc_trace_packet.argtypes = [P(DustTables), P(Grid), P(RunParams), P(OrcTallies), C.c_int64, dp, C.c_int,
                                       P(TraceRec), C.c_int, P(C.c_int)]
        L.orc_stream.argtypes = [C.c_uint64, C.c_int, C.c_int64, C.c_int, dp]
        L.orc_philox.argtypes = [P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]
        L.orc_radface_roots.argtypes = [C.c_double] * 8 + [dp, P(C.c_int)]
        L.orc_next_wall.argtypes = [P(DustTables), P(Grid)] + [C.c_double] * 6 + [C.c_int] * 4 + [dp, P(C.c_int)]
        L.orc_locate_c.argtypes = [dp, C.c_int, C.c_double]
        L.orc_findangle3_c.argtypes = [C.c_double] * 10 + [dp]
        L.orc_sample_stokes.argtypes = [P(DustTables), P(Grid), C.c_double, C.c_uint64, C.c_int, dp, dp]
        L.orc_lucydustfreq_c.argtypes = [P(DustTables), P(Grid), C.c_double, C.c_int, C.c_double]
        L.orc_lucydustfreq_c.restype = C.c_double
        L.orc_rep_isrf_c.argtypes = [P(DustTables), P(Grid), C.c_double]
        L.orc_rep_isrf_c.restype = C.c_double
        L.orc_darkening_c.argtypes = [P(DustTables), P(Grid), C.c_double]
        L.orc_darkening_c.restype = C.c_double
        L.orc_dusttemp.argtypes = [P(DustTables)] + [C.c_double] * 4 + [C.c_int, C.c_double]
        L.orc_dusttemp.restype = C.c_double
        L.orc_tfinal.argtypes = [P(DustTables), P(Grid), dp, C.c_double, C.c_double, dp]
        L.orc_sample_emission.argtypes = [P(DustTables), P(Grid), P(RunParams), C.c_int64, C.c_int64, dp]
        L.orc_sample_bbfreq.argtypes = [C.c_double, C.c_uint64, C.c_int64, dp]
        ip = P(C.c_int)
        L.orc_closest_wall_c.argtypes = [C.c_int, dp, ip, C.c_int, dp, ip, dp]
        L.orc_phiface_roots.argtypes = [C.c_double] * 8 + [dp, ip]
        L.orc_dustmat_c.argtypes = [C.c_double] * 4 + [dp]
        L.orc_stokespeel_c.argtypes = [C.c_double, C.c_double, dp] + [C.c_double] * 6
        L.orc_stokes_c.argtypes = [C.c_double, C.c_double, dp, dp, C.c_int]
        L.orc_opacset_c.argtypes = [P(DustTables), P(Grid), C.c_double, dp]
        L.orc_select_dust_c.argtypes = [C.c_int, dp, dp, C.c_double]
        i32 = P(C.c_int32)
        L.orc_set_sg.argtypes = [P(SgTables), C.c_int, i32, dp]
        L.orc_set_sg.restype = None
        L.orc_rep_draine_c.argtypes = [P(SgTables), C.c_int, C.c_double, C.c_double]
        L.orc_rep_draine_c.restype = C.c_double
        L.orc_int_mean.argtypes = [P(Grid), P(SgTables), P(C.c_int64), C.c_double, C.c_double, C.c_double,
                                   C.c_double, C.c_double, i32, dp]
        L.orc_int_mean.restype = None
        _LIB = L
    return _LIB


class OracleTallies:
    """Host tally buffers of one oracle run, shaped like the GPU tallies."""

    def __init__(self, model: hc3d.Model, params: RunParams, scales=None):
        nrg, ntg, npg, ndg = model.shape4
        npeel = params.npeel if params.ipeel else 0
        self.sed_shape = (params.nfreq, params.nmu, params.nph, params.nap, NO)
        self.psed_shape = (params.nfreq, max(npeel, 1), params.nap, NO)
        self.img_shape = (max(npeel, 1), params.nxhst, params.nxhst)
        self.g4 = (nrg, ntg, npg, ndg)
        self.g3 = (nrg, ntg, npg)
        self.a = {}
        T = OrcTallies()
        for n in ("si", "sq", "su", "sv", "si2", "sq2", "su2", "sv2", "nums"):
            self._add(T.fx, n, self.sed_shape)
        for n in ("ti", "tq", "tu", "tv", "ti2", "tq2", "tu2", "tv2", "numt"):
            self._add(T.fx, n, self.psed_shape)
        for n in ("image_i", "image_q", "image_u", "image_v"):
            self._add(T.fx, n, self.img_shape)
        if params.imcube:
            self._add(T.fx, "image_m_i", self.img_shape + (params.nfreq, NO))
            for n in ("image_m_q", "image_m_u", "image_m_v"):
                self._add(T.fx, n, self.img_shape + (params.nfreq,))
        self._add(T.fx, "nabs", self.g4)
        self._add(T.fx, "dtauabs", self.g4)
        self._add(T.fx, "jmean", self.g3)
        self._add(T.fx, "killed", self.g3, np.int32, C.c_int32)
        self._add(T.fx, "dbig", self.g3, np.int32, C.c_int32)
        self._add(T.fx, "dsg", self.g3, np.int32, C.c_int32)
        self._add(T.fx, "jsg", self.g3)
        for n, shape in (("si_d", self.sed_shape), ("ti_d", self.psed_shape), ("image_i_d", self.img_shape),
                         ("dtauabs_d", self.g4), ("image_m2_d", self.img_shape + (4,))):
            arr = np.zeros(shape, dtype=np.float64, order="F")
            self.a[n] = arr
            setattr(T, n, arr.ctypes.data_as(P(C.c_double)))
        ss, sq, ps = scales if scales is not None else hc3d.tally_scales(params.np)
        T.fx.stokes_scale, T.fx.square_scale, T.fx.path_scale = ss, sq, ps
        self.T = T

    def _add(self, fx, name, shape, dtype=np.int64, ctype=C.c_int64):
        arr = np.zeros(shape, dtype=dtype, order="F")
        self.a[name] = arr
        setattr(fx, name, arr.ctypes.data_as(P(ctype)))

    def result(self) -> dict:
        r = dict(self.a)
        r["counters"] = np.array(self.T.fx.counters[:], dtype=np.int64)
        r["errors"] = int(self.T.errors)
        r["stokes_scale"] = self.T.fx.stokes_scale
        r["square_scale"] = self.T.fx.square_scale
        r["path_scale"] = self.T.fx.path_scale
        return r


# the small-grain inputs of the oracle's runs (module state of hc3d_oracle.c),
# kept alive here while they are set
_SG_KEEP: list = []


def set_sg(model: hc3d.Model, imean=None, imfract=None) -> None:
    """Point the oracle's runs at the model's small grains (spectra, the
    species weighting the jsg tally) and the cells' spectrum rows and
    fractions (None before the first int_mean), or clear them."""
    L = lib()
    _SG_KEEP.clear()
    if not model.sg:
        L.orc_set_sg(None, -1, None, None)
        return
    s = model.sg_tables
    im = None if imean is None else np.asfortranarray(imean, dtype=np.int32)
    fr = None if imfract is None else np.asfortranarray(imfract, dtype=np.float64)
    _SG_KEEP.extend([s, im, fr, model])
    L.orc_set_sg(C.byref(s), model.sg_species, None if im is None else im.ctypes.data_as(P(C.c_int32)),
                 None if fr is None else fr.ctypes.data_as(P(C.c_double)))


def _sg_for(model: hc3d.Model, params: RunParams, imean, imfract) -> None:
    if model.sg and params.iter != 1 and imean is None:
        raise ValueError("small grains after the first iteration need imean and imfract (int_mean)")
    set_sg(model, imean, imfract)


def int_mean(model: hc3d.Model, jsg: np.ndarray, path_scale: float, ltot: float, nphot: float,
             rstar_cm: float) -> tuple[np.ndarray, np.ndarray]:
    """int_mean (int_mean.f90:19-94) of the jsg tally: (imean, imfract), (nrg,ntg,npg)."""
    g, s = model.grid, model.sg_tables
    j = np.asfortranarray(jsg, dtype=np.int64)
    im = np.zeros(model.shape3, dtype=np.int32, order="F")
    fr = np.zeros(model.shape3, dtype=np.float64, order="F")
    kv = float(model.kappav[model.sg_species])
    lib().orc_int_mean(C.byref(g), C.byref(s), j.ctypes.data_as(P(C.c_int64)), float(path_scale), float(rstar_cm),
                       kv, float(ltot), float(nphot), im.ctypes.data_as(P(C.c_int32)),
                       fr.ctypes.data_as(P(C.c_double)))
    return im, fr


def rep_draine(model: hc3d.Model, jm: int, jmf: float, xran) -> np.ndarray:
    """Small-grain re-emission frequencies of spectrum row jm mixed by jmf, for the uniforms xran."""
    s = model.sg_tables
    return np.array([lib().orc_rep_draine_c(C.byref(s), int(jm), float(jmf), float(x)) for x in np.atleast_1d(xran)])


def run(model: hc3d.Model, params: RunParams, nthreads: int = 1, scales=None, imean=None, imfract=None) -> dict:
    """Run params.np packets of params on the CPU; int64 tallies summed over threads.
    A model with small grains past the first iteration takes int_mean's
    imean and imfract."""
    L = lib()
    _sg_for(model, params, imean, imfract)
    t, g = model.tables, model.grid
    if nthreads <= 1:
        ot = OracleTallies(model, params, scales)
        L.orc_run_range(C.byref(t), C.byref(g), C.byref(params), C.byref(ot.T), 0, params.np)
        return ot.result()
    parts = [OracleTallies(model, params, scales) for _ in range(nthreads)]
    arr = (OrcTallies * nthreads)(*[p.T for p in parts])
    L.orc_run_mt(C.byref(t), C.byref(g), C.byref(params), arr, nthreads)
    # the structs were copied into arr; the buffers they point to are shared
    res = parts[0].result()
    res["counters"] = np.zeros(16, dtype=np.int64)
    res["errors"] = 0
    for k in range(nthreads):
        r = parts[k].result()
        res["counters"] += np.array(arr[k].fx.counters[:], dtype=np.int64)
        res["errors"] += int(arr[k].errors)
        if k:
            for n, v in r.items():
                if isinstance(v, np.ndarray) and n != "counters":
                    res[n] = res[n] + v
    return res


def run_timed(model: hc3d.Model, params: RunParams, nthreads: int, seconds: float) -> tuple[int, dict]:
    """Packets of params (ids from 0, params.np at most) claimed by nthreads
    threads for `seconds` seconds, each thread then finishing its packet:
    (packets run, their tallies' counters)."""
    L = lib()
    _sg_for(model, params, None, None)
    t, g = model.tables, model.grid
    parts = [OracleTallies(model, params) for _ in range(nthreads)]
    arr = (OrcTallies * nthreads)(*[p.T for p in parts])
    done = C.c_int64(0)
    L.orc_run_mt_timed(C.byref(t), C.byref(g), C.byref(params), arr, nthreads, float(seconds), C.byref(done))
    counters = np.zeros(16, dtype=np.int64)
    for k in range(nthreads):
        counters += np.array(arr[k].fx.counters[:], dtype=np.int64)
    return int(done.value), {"counters": counters}


def trace(model: hc3d.Model, params: RunParams, pid: int, uniforms=None, max_rec: int = 4096, imean=None,
          imfract=None):
    L = lib()
    _sg_for(model, params, imean, imfract)
    t, g = model.tables, model.grid
    ot = OracleTallies(model, params)
    recs = np.zeros(max_rec, dtype=TRACE_DTYPE)
    ex = C.c_int(0)
    if uniforms is None:
        n = L.orc_trace_packet(C.byref(t), C.byref(g), C.byref(params), C.byref(ot.T), pid, None, 0,
                               recs.ctypes.data_as(P(TraceRec)), max_rec, C.byref(ex))
    else:
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        n = L.orc_trace_packet(C.byref(t), C.byref(g), C.byref(params), C.byref(ot.T), pid,
                               u.ctypes.data_as(P(C.c_double)), len(u), recs.ctypes.data_as(P(TraceRec)), max_rec,
                               C.byref(ex))
    return recs[:n], bool(ex.value), ot.result()


def rep_isrf(model: hc3d.Model, xi) -> np.ndarray:
    """Frequencies of external packets for the uniforms xi (rep_isrf)."""
    L = lib()
    t, g = model.tables, model.grid
    return np.array([L.orc_rep_isrf_c(C.byref(t), C.byref(g), float(x)) for x in np.atleast_1d(xi)])


def darkening(model: hc3d.Model, xi) -> np.ndarray:
    """Emission cosines of the limb-darkening table for the uniforms xi (darkening)."""
    L = lib()
    t, g = model.tables, model.grid
    return np.array([L.orc_darkening_c(C.byref(t), C.byref(g), float(x)) for x in np.atleast_1d(xi)])


def stream(seed: int, it: int, pid: int, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.float64)
    lib().orc_stream(seed, it, pid, n, out.ctypes.data_as(P(C.c_double)))
    return out


def philox(ctr, key) -> list[int]:
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox(c, k, o)
    return list(o)


def tfinal(model: hc3d.Model, na: np.ndarray, ltot: float, nphot: float) -> np.ndarray:
    """Lucy temperatures from the absorbed-path tally na (nrg,ntg,npg,ndg)."""
    t, g = model.tables, model.grid
    na = np.asfortranarray(na, dtype=np.float64)
    out = np.zeros(model.shape4, dtype=np.float64, order="F")
    lib().orc_tfinal(C.byref(t), C.byref(g), na.ctypes.data_as(P(C.c_double)), ltot, nphot,
                     out.ctypes.data_as(P(C.c_double)))
    return out


EMISSION_DTYPE = np.dtype([("kind", "<f8"), ("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("nu", "<f8"),
                           ("ir", "<f8"), ("it", "<f8"), ("ip", "<f8"), ("extra", "<f8")])


def sample_emission(model: hc3d.Model, params: RunParams, pid0: int, n: int) -> np.ndarray:
    """The emission of packets [pid0, pid0 + n) without transport: a record
    array of kind (1 accretion, 2 hot spot, 3 star, 4 external, -1 dropped),
    position, frequency, cell and extra (accretion: the emitting disk slot,
    -1 the gas; star and hot spot: 1 when radiating at the shock temperature)."""
    t, g = model.tables, model.grid
    out = np.zeros(9 * n, dtype=np.float64)
    lib().orc_sample_emission(C.byref(t), C.byref(g), C.byref(params), int(pid0), int(n),
                              out.ctypes.data_as(P(C.c_double)))
    return out.view(EMISSION_DTYPE)


def sample_bbfreq(teff: float, seed: int, n: int) -> np.ndarray:
    """n frequencies of the blackbody sampler bbfreq at temperature teff (K/11605)."""
    out = np.zeros(n, dtype=np.float64)
    lib().orc_sample_bbfreq(float(teff), int(seed), int(n), out.ctypes.data_as(P(C.c_double)))
    return out
