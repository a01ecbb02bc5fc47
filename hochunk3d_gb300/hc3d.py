"""ctypes binding of the GB300 photon-packet Monte Carlo library (libhc3d.so).

The Python host mirrors the Fortran caller of ``disk()``:

* :class:`Model` -- setup/reapar/dustinit/atmosinit/gridset of a ``.par``
  file (newtts.F90:141-290), built by the library's C++ host code;
* :class:`Context` -- one GPU context holding tables, grid and tallies;
  :meth:`Context.disk` is one call of ``disk(converge, iter, i1)``
  (newdisktherm.F90:1): the packet loop on the GPU followed by the Lucy
  temperature update (``tfinal``, newdisktherm.F90:557);
* :func:`tts` -- the whole program ``tts`` (newtts.F90) in the library.

There is no CPU fallback: every function that computes needs ``libhc3d.so``
and a CUDA device, and raises :class:`Hc3dError` otherwise.  Building a
model from its .par file needs only ``libhc3d_host.so`` (host code, no
CUDA), which ``libhc3d.so`` links against.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libhc3d.so"
HOST_LIB_PATH = PKG / "libhc3d_host.so"

NDG = 8
NO = 8
PREC_MIXED = 0
PREC_FP64 = 1

ERRORS = {
    -1: "HC3D_ERR_INVALID", -2: "HC3D_ERR_CUDA", -3: "HC3D_ERR_NOMEM", -4: "HC3D_ERR_STATE",
    -5: "HC3D_ERR_DEVICE", -6: "HC3D_ERR_IO", -7: "HC3D_ERR_UNSUPPORTED", -8: "HC3D_ERR_TIMEOUT",
    -9: "HC3D_ERR_CANCELLED",
}

CNT = {
    "flux": 0, "sflux": 1, "nscat": 2, "scount": 3, "tot": 4, "abflux": 5, "aflux": 6, "sumsub": 7,
    "sumall": 8, "escaped": 9, "cross_prop": 10, "cross_peel": 11, "events": 12, "peels": 13, "stuck": 14,
    "peel_stuck": 15,
}

P = C.POINTER
dp = P(C.c_double)
ip_ = P(C.c_int)
i64p = P(C.c_int64)
i32p = P(C.c_int32)


class Hc3dError(RuntimeError):
    def __init__(self, code: int, msg: str = ""):
        self.code = code
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")


class DeviceOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("block_size", C.c_int), ("grid_blocks", C.c_int)]


class DustTables(C.Structure):
    _fields_ = [
        ("ndg", C.c_int), ("nlammax", C.c_int), ("nlambda", ip_),
        ("nudust", dp), ("kappad", dp), ("adust", dp), ("gdust", dp), ("pldust", dp), ("kappav", dp),
        ("nT", C.c_int), ("nnu", C.c_int), ("lTint", dp), ("nuint", dp), ("kapBint", dp), ("kappap", dp),
        ("tsub", C.c_double), ("nhnu", C.c_int), ("hnuint", dp), ("atmosnu", dp), ("lognu", dp), ("loghnu", dp),
        ("nisrf", C.c_int), ("isrf_cdf", dp), ("isrf_logcdf", dp), ("isrf_logfreq", dp),
        ("ntab", C.c_int), ("limb_xmu", dp), ("limb_prob", dp),
    ]


class Grid(C.Structure):
    _fields_ = [
        ("nrg", C.c_int), ("ntg", C.c_int), ("npg", C.c_int), ("ndg", C.c_int),
        ("rarr", dp), ("r2arr", dp), ("thetarr", dp), ("costarr", dp), ("tan2arr", dp),
        ("phiarr", dp), ("aarr", dp), ("barr", dp),
        ("densarr", dp), ("massarr", dp), ("vcell", dp), ("tdust", dp),
    ]


class Sources(C.Structure):
    """hc3d_sources: constants of the disk-accretion and hot-spot packets."""
    _fields_ = [
        ("rddustmin", C.c_double), ("rmaxdmax", C.c_double), ("rmax", C.c_double),
        ("zfac", C.c_double * 2), ("zexp", C.c_double * 2), ("kapv", C.c_double * 2),
        ("gas_num", C.c_double), ("gas_den", C.c_double), ("rstar", C.c_double), ("rsun", C.c_double),
        ("ispot", C.c_int), ("nspot", C.c_int), ("spot1", C.c_double * 4), ("spot2", C.c_double * 4),
        ("csprad", C.c_double), ("fspot", C.c_double), ("tshock", C.c_double),
    ]


class RunParams(C.Structure):
    _fields_ = [
        ("np", C.c_int64), ("packet_offset", C.c_int64), ("seed", C.c_uint64), ("iter", C.c_int),
        ("ipeel", C.c_int), ("npeel", C.c_int), ("thete", dp), ("phie", dp),
        ("nfreq", C.c_int), ("nmu", C.c_int), ("nph", C.c_int), ("nap", C.c_int), ("nxhst", C.c_int),
        ("rmaxi", C.c_double), ("aperture2", dp), ("numin", C.c_double), ("numax", C.c_double),
        ("rstar_cm", C.c_double), ("tstar", C.c_double), ("limb", C.c_int), ("iintmax", C.c_int),
        ("max_interactions", C.c_int64), ("image", C.c_int),
        ("ext_illum", C.c_int), ("n_star", C.c_int64), ("rmax", C.c_double),
        ("n_acc", C.c_int64), ("n_spot", C.c_int64), ("sources", C.POINTER(Sources)), ("imcube", C.c_int),
    ]


class Tallies(C.Structure):
    _fields_ = [(n, i64p) for n in ("si", "sq", "su", "sv", "si2", "sq2", "su2", "sv2", "nums",
                                     "ti", "tq", "tu", "tv", "ti2", "tq2", "tu2", "tv2", "numt",
                                     "image_i", "image_q", "image_u", "image_v",
                                     "nabs", "dtauabs", "jmean")] + [
        ("killed", i32p), ("dbig", i32p), ("counters", C.c_int64 * 16),
        ("stokes_scale", C.c_double), ("square_scale", C.c_double), ("path_scale", C.c_double),
        ("image_m_i", i64p), ("image_m_q", i64p), ("image_m_u", i64p), ("image_m_v", i64p),
        ("dsg", i32p), ("jsg", i64p),
    ]


class SgTables(C.Structure):
    """hc3d_sg_tables: the small grains' emission spectra (draine_cdf.f90) and ISRF integral."""
    _fields_ = [("nemit", C.c_int), ("ndraine", C.c_int), ("cdf", dp), ("logcdf", dp), ("logfreq", dp),
                ("uratio", dp), ("isrfkap_int", C.c_double), ("sg_slot", C.c_int)]


class LucyBuffers(C.Structure):
    """hc3d_lucy_buffers: caller-owned device buffers of hc3d_lucy_update_noalloc."""
    _fields_ = [
        ("device", C.c_int), ("stream", C.c_void_p),
        ("nrg", C.c_int), ("ntg", C.c_int), ("npg", C.c_int), ("ndg", C.c_int),
        ("dtauabs", C.c_void_p), ("path_scale", C.c_double),
        ("densarr", C.c_void_p), ("massarr", C.c_void_p), ("tdust_in", C.c_void_p), ("tdust_out", C.c_void_p),
        ("nT", C.c_int), ("lTint", C.c_void_p), ("kappap", C.c_void_p),
        ("kappav", C.c_double * 8), ("ltot", C.c_double), ("np", C.c_int64),
    ]


class TraceRec(C.Structure):
    _fields_ = [("kind", C.c_int32), ("ir", C.c_int32), ("it", C.c_int32), ("ip", C.c_int32),
                ("iface", C.c_int32), ("pad", C.c_int32), ("tsum", C.c_double),
                ("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


TRACE_DTYPE = np.dtype([("kind", "<i4"), ("ir", "<i4"), ("it", "<i4"), ("ip", "<i4"), ("iface", "<i4"),
                        ("pad", "<i4"), ("tsum", "<f8"), ("x", "<f8"), ("y", "<f8"), ("z", "<f8")])


class ModelInfo(C.Structure):
    _fields_ = [
        ("np", C.c_int64), ("npmin", C.c_int64), ("np_lucy", C.c_int64), ("nimin", C.c_int), ("nimax", C.c_int),
        ("ipeel", C.c_int), ("ilucy", C.c_int), ("ndg_active", C.c_int), ("ltot", C.c_double),
        ("tstar_k", C.c_double), ("rstar_rsun", C.c_double), ("autors", C.c_double), ("rminsub", C.c_double),
        ("massdisk", C.c_double), ("massenv", C.c_double), ("ncells", C.c_int64),
        ("density_host_ms", C.c_double), ("tables_host_ms", C.c_double),
        ("lstar", C.c_double), ("l_isrf", C.c_double), ("isrf_frac", C.c_double),
        ("lacc", C.c_double), ("lacc2", C.c_double), ("accfrac", C.c_double), ("accfrac2", C.c_double),
        ("mdot_msun_yr", C.c_double), ("tshock_k", C.c_double), ("fspot", C.c_double),
        ("thspot_deg", C.c_double), ("tave_k", C.c_double),
        ("slot_species", C.c_int32 * 4), ("has_sg", C.c_int), ("ndg", C.c_int),
    ]


class TtsStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("max_rel_change", C.c_double),
                ("seconds_lucy", C.c_double), ("seconds_final", C.c_double), ("packets_total", C.c_int64),
                ("counters", C.c_int64 * 16)]


class TuneResult(C.Structure):
    _fields_ = [("n", C.c_int), ("best", C.c_int), ("queue_records", C.c_int64 * 12), ("block_size", C.c_int * 12),
                ("regen", C.c_int * 12), ("peel_shape", C.c_int * 12), ("peel_threads", C.c_int * 12),
                ("ms", C.c_double * 12)]


class ServerOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("slots", C.c_int), ("hbm_budget", C.c_int64)]


class Request(C.Structure):
    _fields_ = [("par_path", C.c_char_p), ("par_dir", C.c_char_p), ("n_lucy", C.c_int), ("np_lucy", C.c_int64),
                ("np", C.c_int64), ("npeel", C.c_int), ("thete", dp), ("phie", dp)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int), ("err", C.c_char * 256), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double), ("footprint_bytes", C.c_int64), ("packets", C.c_int64),
                ("iterations", C.c_int), ("max_rel_change", C.c_double), ("nfreq", C.c_int), ("nmu", C.c_int),
                ("nph", C.c_int), ("nap", C.c_int), ("npeel", C.c_int), ("si", i64p), ("nums", i64p),
                ("ti", i64p), ("numt", i64p), ("stokes_scale", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("budget_bytes", C.c_int64), ("in_use_bytes", C.c_int64), ("peak_in_use_bytes", C.c_int64),
                ("running", C.c_int), ("peak_running", C.c_int), ("queued", C.c_int64), ("completed", C.c_int64)]


# every symbol the public headers declare, with its ctypes signature
SIGNATURES = {
    "hc3d_create": (C.c_int, [P(C.c_void_p), P(DeviceOpts)]),
    "hc3d_destroy": (None, [C.c_void_p]),
    "hc3d_reset": (C.c_int, [C.c_void_p]),
    "hc3d_get_error": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    "hc3d_version": (C.c_char_p, []),
    "hc3d_set_species": (C.c_int, [C.c_void_p, i32p]),
    "hc3d_load_tables": (C.c_int, [C.c_void_p, P(DustTables)]),
    "hc3d_load_sg_tables": (C.c_int, [C.c_void_p, P(SgTables)]),
    "hc3d_get_imean": (C.c_int, [C.c_void_p, i32p, dp]),
    "hc3d_set_imean": (C.c_int, [C.c_void_p, i32p, dp]),
    "hc3d_load_grid": (C.c_int, [C.c_void_p, P(Grid)]),
    "hc3d_zero_tallies": (C.c_int, [C.c_void_p]),
    "hc3d_set_tdust": (C.c_int, [C.c_void_p, dp]),
    "hc3d_set_wave_options": (C.c_int, [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_int]),
    "hc3d_run_chunk": (C.c_int, [C.c_void_p, P(RunParams), C.c_int64, C.c_int]),
    "hc3d_run_iteration": (C.c_int, [C.c_void_p, P(RunParams)]),
    "hc3d_get_tallies": (C.c_int, [C.c_void_p, P(RunParams), P(Tallies)]),
    "hc3d_lucy_update": (C.c_int, [C.c_void_p, C.c_double, C.c_int64, dp, dp, ip_]),
    "hc3d_lucy_update_noalloc": (C.c_int, [P(LucyBuffers), dp, ip_]),
    "hc3d_set_lucy_tally": (C.c_int, [C.c_void_p, P(C.c_int64)]),
    "hc3d_lucy_iterations": (C.c_int, [C.c_void_p, P(RunParams), C.c_int, C.c_double, dp, dp]),
    "hc3d_autotune": (C.c_int, [C.c_void_p, P(RunParams), P(TuneResult)]),
    "hc3d_run_batch": (C.c_int, [P(C.c_void_p), P(RunParams), C.c_int]),
    "hc3d_get_stream": (C.c_void_p, [C.c_void_p]),
    "hc3d_last_kernel_ms": (C.c_int, [C.c_void_p, P(C.c_double)]),
    "hc3d_last_launch_stats": (C.c_int, [C.c_void_p, ip_, P(C.c_double), P(C.c_double)]),
    "hc3d_get_fault_log": (C.c_int, [C.c_void_p, P(C.c_uint64), C.c_int, ip_]),
    "hc3d_get_wave_log": (C.c_int, [C.c_void_p, dp, C.c_int, ip_]),
    "hc3d_trace_packets": (C.c_int, [C.c_void_p, P(RunParams), C.c_int, dp, C.c_int, P(TraceRec), C.c_int, i32p]),
    "hc3d_model_create": (C.c_int, [P(C.c_void_p), C.c_char_p, C.c_char_p, C.c_char_p, C.c_size_t]),
    "hc3d_model_destroy": (None, [C.c_void_p]),
    "hc3d_model_views": (C.c_int, [C.c_void_p, P(DustTables), P(Grid), P(RunParams), P(ModelInfo)]),
    "hc3d_model_set_tdust": (C.c_int, [C.c_void_p, dp]),
    "hc3d_model_sg_tables": (C.c_int, [C.c_void_p, P(SgTables)]),
    "hc3d_model_load": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hc3d_model_densities_gpu": (C.c_int, [C.c_void_p, C.c_int, P(C.c_double), C.c_char_p, C.c_size_t]),
    "hc3d_model_tables_gpu": (C.c_int, [C.c_void_p, C.c_int, P(C.c_double), C.c_char_p, C.c_size_t]),
    "hc3d_tts": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, P(DeviceOpts), P(TtsStats), C.c_char_p, C.c_size_t]),
    "hc3d_write_synthetic_dust": (C.c_int, [C.c_char_p]),
    "hc3d_write_wavelength_grid": (C.c_int, [C.c_char_p, C.c_double]),
    "hc3d_write_synthetic_isrf": (C.c_int, [C.c_char_p]),
    "hc3d_write_synthetic_draine": (C.c_int, [C.c_char_p]),
    "hc3d_write_outputs": (C.c_int, [C.c_void_p, P(RunParams), P(Tallies), dp, dp, C.c_char_p]),
    "hc3d_write_grid_unf": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, dp, i32p]),
    "hc3d_star_packets": (C.c_int64, [C.c_double, C.c_int64]),
    "hc3d_packet_split": (C.c_int, [C.c_double, C.c_double, C.c_double, C.c_int64, P(C.c_int64), P(C.c_int64),
                                    P(C.c_int64)]),
    "hc3d_server_create": (C.c_int, [P(C.c_void_p), P(ServerOpts)]),
    "hc3d_server_submit": (C.c_int, [C.c_void_p, P(Request), P(C.c_int64)]),
    "hc3d_server_wait": (C.c_int, [C.c_void_p, C.c_int64, P(Result)]),
    "hc3d_result_free": (None, [P(Result)]),
    "hc3d_server_cancel": (C.c_int, [C.c_void_p, C.c_int64]),
    "hc3d_server_get_stats": (C.c_int, [C.c_void_p, P(ServerStats)]),
    "hc3d_server_destroy": (None, [C.c_void_p]),
    "hc3d_model_footprint": (C.c_int64, [C.c_void_p]),
}

# entry points of libhc3d_host.so (the model set-up, no CUDA)
HOST_SYMBOLS = ("hc3d_model_create", "hc3d_model_destroy", "hc3d_model_views", "hc3d_model_set_tdust",
                "hc3d_model_sg_tables", "hc3d_star_packets", "hc3d_packet_split", "hc3d_write_synthetic_dust",
                "hc3d_write_wavelength_grid", "hc3d_write_synthetic_isrf", "hc3d_write_synthetic_draine")

_LIB = None
_HOST = None


def _bind(L: C.CDLL, names) -> C.CDLL:
    for name in names:
        res, args = SIGNATURES[name]
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


def host_lib() -> C.CDLL:
    """Load libhc3d_host.so, the host-only model set-up; fail loudly if absent."""
    global _HOST
    if _HOST is None:
        if not HOST_LIB_PATH.exists():
            raise Hc3dError(-4, f"{HOST_LIB_PATH} is not built; run hochunk3d_gb300.build.build_host_library()")
        _HOST = _bind(C.CDLL(str(HOST_LIB_PATH)), HOST_SYMBOLS)
    return _HOST


def lib() -> C.CDLL:
    """Load libhc3d.so (built by ``__graft_entry__.build()``); fail loudly if absent."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise Hc3dError(-4, f"{LIB_PATH} is not built; run hochunk3d_gb300.build.build_library()")
        host_lib()  # the same instance serves libhc3d.so's dependency on it
        _LIB = _bind(C.CDLL(str(LIB_PATH)), SIGNATURES)
    return _LIB


def _ptr(a: np.ndarray, t=C.c_double):
    return a.ctypes.data_as(P(t))


def _arr(ptr, n: int, dtype=np.float64) -> np.ndarray:
    if not ptr or n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def tally_scales(np_: int) -> tuple[float, float, float]:
    """Fixed-point scales the library picks for an epoch whose first call runs np_ packets."""
    budget = max(int(np_), 1 << 20) * 16.0
    L = 0
    while float(1 << L) < budget and L < 62:
        L += 1
    sb = max(16, min(40, 58 - L))
    pb = max(12, min(32, 52 - L))
    return math.ldexp(1.0, sb), math.ldexp(1.0, sb - 8), math.ldexp(1.0, pb)


def star_packets(isrf_frac: float, np_: int) -> int:
    """Stellar packets of an iteration of np_ packets (hc3d_star_packets)."""
    return int(host_lib().hc3d_star_packets(float(isrf_frac), int(np_)))


def packet_split(accfrac: float, accfrac2: float, isrf_frac: float, np_: int) -> tuple[int, int, int]:
    """(n_acc, n_spot, n_star) of an iteration of np_ packets (hc3d_packet_split)."""
    a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
    rc = host_lib().hc3d_packet_split(float(accfrac), float(accfrac2), float(isrf_frac), int(np_), C.byref(a),
                                      C.byref(b), C.byref(c))
    if rc != 0:
        raise Hc3dError(rc, "hc3d_packet_split")
    return a.value, b.value, c.value


# ---------------------------------------------------------------------------
class Model:
    """A model built from a .par file by the library's host setup code.

    The numpy attributes are copies of the library's arrays in the reference's
    Fortran (column-major) layout; ``tables``/``grid``/``params`` are ctypes
    views that point into arrays this object keeps alive.
    """

    def __init__(self, par_path: str | os.PathLike, par_dir: str | os.PathLike | None = None):
        L = host_lib()
        h = C.c_void_p()
        err = C.create_string_buffer(1024)
        rc = L.hc3d_model_create(C.byref(h), str(par_path).encode(),
                                 None if par_dir is None else str(par_dir).encode(), err, 1024)
        if rc != 0:
            raise Hc3dError(rc, err.value.decode())
        self._h = h
        self.par_path = os.fspath(par_path)
        t, g, p, info = DustTables(), Grid(), RunParams(), ModelInfo()
        L.hc3d_model_views(h, C.byref(t), C.byref(g), C.byref(p), C.byref(info))
        self.info = info
        nrg, ntg, npg, ndg = g.nrg, g.ntg, g.npg, g.ndg
        n4 = nrg * ntg * npg
        self.shape4 = (nrg, ntg, npg, ndg)
        self.shape3 = (nrg, ntg, npg)
        # grid arrays (copies, Fortran order)
        self.rarr = _arr(g.rarr, nrg); self.r2arr = _arr(g.r2arr, nrg)
        self.thetarr = _arr(g.thetarr, ntg); self.costarr = _arr(g.costarr, ntg); self.tan2arr = _arr(g.tan2arr, ntg)
        self.phiarr = _arr(g.phiarr, npg); self.aarr = _arr(g.aarr, npg); self.barr = _arr(g.barr, npg)
        self.densarr = _arr(g.densarr, n4 * ndg).reshape(self.shape4, order="F")
        self.massarr = _arr(g.massarr, n4 * ndg).reshape(self.shape4, order="F")
        self.vcell = _arr(g.vcell, n4).reshape(self.shape3, order="F")
        self.tdust = _arr(g.tdust, n4 * ndg).reshape(self.shape4, order="F")
        # dust tables
        self.ndg_tab, self.nlammax, self.nT, self.nnu, self.nhnu = t.ndg, t.nlammax, t.nT, t.nnu, t.nhnu
        nl = t.nlammax * t.ndg
        self.nlambda = _arr(t.nlambda, t.ndg, np.int32)
        self.nudust = _arr(t.nudust, nl); self.kappad = _arr(t.kappad, nl); self.adust = _arr(t.adust, nl)
        self.gdust = _arr(t.gdust, nl); self.pldust = _arr(t.pldust, nl); self.kappav = _arr(t.kappav, t.ndg)
        self.lTint = _arr(t.lTint, t.nT); self.nuint = _arr(t.nuint, t.nnu)
        self.kapBint = _arr(t.kapBint, t.nT * t.nnu * t.ndg); self.kappap = _arr(t.kappap, t.nT * t.ndg)
        self.tsub = t.tsub
        self.hnuint = _arr(t.hnuint, t.nhnu); self.atmosnu = _arr(t.atmosnu, t.nhnu)
        self.lognu = _arr(t.lognu, t.nhnu); self.loghnu = _arr(t.loghnu, t.nhnu)
        self.nisrf = t.nisrf
        self.isrf_cdf = _arr(t.isrf_cdf, t.nisrf); self.isrf_logcdf = _arr(t.isrf_logcdf, t.nisrf)
        self.isrf_logfreq = _arr(t.isrf_logfreq, t.nisrf)
        self.ntab = t.ntab
        self.limb_xmu = _arr(t.limb_xmu, t.ntab); self.limb_prob = _arr(t.limb_prob, t.ntab)
        # run parameters
        # small grains: the species of the four device slots and the emission spectra
        self.slot_species = np.array(info.slot_species[:], dtype=np.int32)
        self.sg = None
        if info.has_sg:
            sg = SgTables()
            rc = L.hc3d_model_sg_tables(h, C.byref(sg))
            if rc != 0:
                raise Hc3dError(rc, "hc3d_model_sg_tables")
            ne, nd = sg.nemit, sg.ndraine
            self.sg_cdf = _arr(sg.cdf, ne * nd).reshape((ne, nd), order="F")
            self.sg_logcdf = _arr(sg.logcdf, ne * nd).reshape((ne, nd), order="F")
            self.sg_logfreq = _arr(sg.logfreq, nd)
            self.sg_uratio = _arr(sg.uratio, ne)
            self.isrfkap_int = sg.isrfkap_int
            self.sg_slot = sg.sg_slot
            self.sg = True
        self.npeel = p.npeel
        self.thete = _arr(p.thete, p.npeel); self.phie = _arr(p.phie, p.npeel)
        self.aperture2 = _arr(p.aperture2, p.nap)
        self._p = p
        self.params = self.run_params()

    # ctypes views over this object's numpy copies
    @property
    def tables(self) -> DustTables:
        t = DustTables()
        t.ndg, t.nlammax, t.nT, t.nnu, t.nhnu, t.tsub = self.ndg_tab, self.nlammax, self.nT, self.nnu, self.nhnu, self.tsub
        t.nlambda = _ptr(self.nlambda, C.c_int)
        for n in ("nudust", "kappad", "adust", "gdust", "pldust", "kappav", "lTint", "nuint", "kapBint", "kappap",
                  "hnuint", "atmosnu", "lognu", "loghnu"):
            setattr(t, n, _ptr(getattr(self, n)))
        t.nisrf = self.nisrf
        if self.nisrf:
            for n in ("isrf_cdf", "isrf_logcdf", "isrf_logfreq"):
                setattr(t, n, _ptr(getattr(self, n)))
        t.ntab = self.ntab
        if self.ntab:
            t.limb_xmu, t.limb_prob = _ptr(self.limb_xmu), _ptr(self.limb_prob)
        return t

    @property
    def grid(self) -> Grid:
        g = Grid()
        g.nrg, g.ntg, g.npg, g.ndg = self.shape4
        for n in ("rarr", "r2arr", "thetarr", "costarr", "tan2arr", "phiarr", "aarr", "barr"):
            setattr(g, n, _ptr(getattr(self, n)))
        for n in ("densarr", "massarr", "vcell", "tdust"):
            a = getattr(self, n)
            assert a.flags.f_contiguous
            setattr(g, n, a.ctypes.data_as(dp))
        return g

    @property
    def sg_tables(self) -> SgTables | None:
        """hc3d_sg_tables view of the small grains' spectra, or None without small grains."""
        if not self.sg:
            return None
        s = SgTables()
        s.nemit, s.ndraine = self.sg_cdf.shape
        for n, a in (("cdf", self.sg_cdf), ("logcdf", self.sg_logcdf)):
            assert a.flags.f_contiguous
            setattr(s, n, a.ctypes.data_as(dp))
        s.logfreq, s.uratio = _ptr(self.sg_logfreq), _ptr(self.sg_uratio)
        s.isrfkap_int, s.sg_slot = self.isrfkap_int, self.sg_slot
        return s

    @property
    def sg_species(self) -> int:
        """0-based species whose opacity weights the small grains' path tally (-1 without them)."""
        return int(self.slot_species[self.sg_slot - 1]) - 1 if self.sg else -1

    def run_params(self, np_total: int | None = None, **over) -> RunParams:
        """The model's run parameters with fields of RunParams overridden.

        The shares of the iteration (n_acc, n_spot, n_star: accretion,
        hot-spot, stellar and external packets) follow np unless n_star is
        given.  A shard of an iteration (packet_offset > 0, or np below the
        whole) passes np_total, the packets of the whole iteration, so that
        every shard splits the sources as one run would."""
        q = RunParams()
        for f, _ in RunParams._fields_:
            setattr(q, f, getattr(self._p, f))
        q.thete = _ptr(self.thete)
        q.phie = _ptr(self.phie)
        q.aperture2 = _ptr(self.aperture2)
        for k, v in over.items():
            if not hasattr(q, k):
                raise AttributeError(f"RunParams has no field {k}")
            setattr(q, k, v)
        if "n_star" not in over and (np_total is not None or "np" in over):
            # the shares of the iteration's packets (newdisktherm.F90:143-175)
            i = self.info
            n_acc, n_spot, n_star = packet_split(i.accfrac, i.accfrac2, i.isrf_frac,
                                                 q.np if np_total is None else np_total)
            q.n_star = n_star
            if "n_acc" not in over:
                q.n_acc = n_acc
            if "n_spot" not in over:
                q.n_spot = n_spot
        return q

    @property
    def sources(self) -> Sources | None:
        """The accretion and hot-spot constants of the model (None without either)."""
        return self._p.sources.contents if self._p.sources else None

    def set_tdust(self, tdust: np.ndarray) -> None:
        self.tdust = np.asfortranarray(tdust, dtype=np.float64).copy(order="F")

    def densities_gpu(self, device: int = 0) -> float:
        """Recompute the densities of gridset on the GPU (hc3d_model_densities_gpu)
        and refresh densarr, massarr, vcell and info; returns the device time in ms."""
        L = lib()
        ms = C.c_double(0.0)
        err = C.create_string_buffer(1024)
        rc = L.hc3d_model_densities_gpu(self._h, device, C.byref(ms), err, 1024)
        if rc != 0:
            raise Hc3dError(rc, err.value.decode())
        t, g, p, info = DustTables(), Grid(), RunParams(), ModelInfo()
        host_lib().hc3d_model_views(self._h, C.byref(t), C.byref(g), C.byref(p), C.byref(info))
        n4 = g.nrg * g.ntg * g.npg
        self.densarr = _arr(g.densarr, n4 * g.ndg).reshape(self.shape4, order="F")
        self.massarr = _arr(g.massarr, n4 * g.ndg).reshape(self.shape4, order="F")
        self.vcell = _arr(g.vcell, n4).reshape(self.shape3, order="F")
        self.info = info
        return ms.value

    def tables_gpu(self, device: int = 0) -> float:
        """Recompute the setemiss tables kapBint and kappap on the GPU
        (hc3d_model_tables_gpu) and refresh them; returns the device time in ms."""
        L = lib()
        ms = C.c_double(0.0)
        err = C.create_string_buffer(1024)
        rc = L.hc3d_model_tables_gpu(self._h, device, C.byref(ms), err, 1024)
        if rc != 0:
            raise Hc3dError(rc, err.value.decode())
        t, g, p, info = DustTables(), Grid(), RunParams(), ModelInfo()
        host_lib().hc3d_model_views(self._h, C.byref(t), C.byref(g), C.byref(p), C.byref(info))
        self.kapBint = _arr(t.kapBint, t.nT * t.nnu * t.ndg)
        self.kappap = _arr(t.kappap, t.nT * t.ndg)
        return ms.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            host_lib().hc3d_model_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
class Context:
    """One GPU context: device tables, grid and tallies of the photon loop."""

    def __init__(self, precision: int = PREC_MIXED, device: int = 0, block_size: int = 0, grid_blocks: int = 0):
        L = lib()
        h = C.c_void_p()
        o = DeviceOpts(device, precision, block_size, grid_blocks)
        rc = L.hc3d_create(C.byref(h), C.byref(o))
        if rc != 0:
            raise Hc3dError(rc, "hc3d_create failed (is a CUDA device visible?)")
        self._h = h
        self.precision = precision
        self.model: Model | None = None

    def _check(self, rc: int) -> None:
        if rc != 0:
            buf = C.create_string_buffer(1024)
            lib().hc3d_get_error(self._h, buf, 1024)
            raise Hc3dError(rc, buf.value.decode())

    def load(self, model: Model) -> "Context":
        t, g = model.tables, model.grid
        sp = np.ascontiguousarray(model.slot_species, dtype=np.int32)
        self._check(lib().hc3d_set_species(self._h, _ptr(sp, C.c_int32)))
        self._check(lib().hc3d_load_tables(self._h, C.byref(t)))
        self._check(lib().hc3d_load_grid(self._h, C.byref(g)))
        if model.sg:
            s = model.sg_tables
            self._check(lib().hc3d_load_sg_tables(self._h, C.byref(s)))
        self.model = model
        return self

    def get_imean(self) -> tuple[np.ndarray, np.ndarray]:
        """(imean, imfract), (nrg,ntg,npg): int_mean's spectrum rows and fractions (hc3d_get_imean)."""
        shape = self.model.shape3
        im = np.zeros(shape, dtype=np.int32, order="F")
        fr = np.zeros(shape, dtype=np.float64, order="F")
        self._check(lib().hc3d_get_imean(self._h, _ptr(im, C.c_int32), _ptr(fr)))
        return im, fr

    def set_imean(self, imean: np.ndarray, imfract: np.ndarray) -> None:
        """Set the cells' spectrum rows and fractions (hc3d_set_imean), (nrg,ntg,npg)."""
        im = np.asfortranarray(imean, dtype=np.int32)
        fr = np.asfortranarray(imfract, dtype=np.float64)
        self._check(lib().hc3d_set_imean(self._h, _ptr(im, C.c_int32), _ptr(fr)))

    def reset(self) -> "Context":
        """Drop the loaded model, keeping the stream, packet pool and queue (hc3d_reset)."""
        self._check(lib().hc3d_reset(self._h))
        self.model = None
        return self

    def set_tdust(self, tdust: np.ndarray) -> None:
        """Replace the device temperature field (hc3d_set_tdust); (nrg,ntg,npg,ndg), K/11605."""
        td = np.asfortranarray(tdust, dtype=np.float64)
        if td.shape != self.model.shape4:
            raise Hc3dError(-1, f"tdust shape {td.shape} != {self.model.shape4}")
        self._check(lib().hc3d_set_tdust(self._h, td.ctypes.data_as(dp)))

    def zero(self) -> None:
        self._check(lib().hc3d_zero_tallies(self._h))

    def run(self, params: RunParams) -> None:
        self._check(lib().hc3d_run_iteration(self._h, C.byref(params)))

    def tallies(self, params: RunParams, grid: bool = True) -> dict:
        m = self.model
        nrg, ntg, npg, ndg = m.shape4
        npeel = params.npeel if params.ipeel else 0
        sed_shape = (params.nfreq, params.nmu, params.nph, params.nap, NO)
        psed_shape = (params.nfreq, npeel, params.nap, NO)
        img_shape = (npeel, params.nxhst, params.nxhst)
        out = {}
        T = Tallies()
        keep = []

        def buf(name, shape, dtype=np.int64, ctype=C.c_int64):
            a = np.zeros(int(np.prod(shape)) if len(shape) else 0, dtype=dtype)
            keep.append(a)
            out[name] = (a, shape)
            setattr(T, name, a.ctypes.data_as(P(ctype)))

        for n in ("si", "sq", "su", "sv", "si2", "sq2", "su2", "sv2", "nums"):
            buf(n, sed_shape)
        if npeel:
            for n in ("ti", "tq", "tu", "tv", "ti2", "tq2", "tu2", "tv2", "numt"):
                buf(n, psed_shape)
            if params.image:
                for n in ("image_i", "image_q", "image_u", "image_v"):
                    buf(n, img_shape)
                if params.imcube:  # (npeel, nx, nx, nfreq, no) and (npeel, nx, nx, nfreq)
                    buf("image_m_i", img_shape + (params.nfreq, NO))
                    for n in ("image_m_q", "image_m_u", "image_m_v"):
                        buf(n, img_shape + (params.nfreq,))
        if grid:
            buf("nabs", (nrg, ntg, npg, ndg))
            buf("dtauabs", (nrg, ntg, npg, ndg))
            buf("jmean", (nrg, ntg, npg))
            buf("killed", (nrg, ntg, npg), np.int32, C.c_int32)
            buf("dbig", (nrg, ntg, npg), np.int32, C.c_int32)
            buf("dsg", (nrg, ntg, npg), np.int32, C.c_int32)
            buf("jsg", (nrg, ntg, npg))
        self._check(lib().hc3d_get_tallies(self._h, C.byref(params), C.byref(T)))
        res = {k: a.reshape(s, order="F") for k, (a, s) in out.items()}
        res["counters"] = np.array(T.counters[:], dtype=np.int64)
        res["stokes_scale"], res["square_scale"], res["path_scale"] = T.stokes_scale, T.square_scale, T.path_scale
        return res

    @property
    def stream(self) -> int:
        """cudaStream_t (as an int) of this context's kernels."""
        return lib().hc3d_get_stream(self._h) or 0

    def last_kernel_ms(self) -> float:
        v = C.c_double(0)
        self._check(lib().hc3d_last_kernel_ms(self._h, C.byref(v)))
        return v.value

    def fault_log(self) -> tuple[int, list[tuple[int, int]]]:
        """(count, [(packet id, fault code), ...]) of packets stopped by a fault."""
        buf = np.zeros(256, dtype=np.uint64)
        n = C.c_int(0)
        self._check(lib().hc3d_get_fault_log(self._h, buf.ctypes.data_as(P(C.c_uint64)), 256, C.byref(n)))
        k = min(n.value, 256)
        return n.value, [(int(v) & ((1 << 56) - 1), int(v) >> 56) for v in buf[:k]]

    def wave_log(self) -> np.ndarray:
        """Per wave of the last peeled run: E, active, alive, transport ms, peel ms, interactions."""
        n = C.c_int(0)
        lib().hc3d_get_wave_log(self._h, None, 0, C.byref(n))
        out = np.zeros((max(n.value, 1), 6))
        self._check(lib().hc3d_get_wave_log(self._h, _ptr(out), n.value, C.byref(n)))
        return out[: n.value]

    def last_launch_stats(self) -> tuple[int, float, float]:
        """(launches, transport ms, peel-off ms) of the last run."""
        n, a, b = C.c_int(0), C.c_double(0), C.c_double(0)
        self._check(lib().hc3d_last_launch_stats(self._h, C.byref(n), C.byref(a), C.byref(b)))
        return n.value, a.value, b.value

    def lucy_update(self, ltot: float, np_: int, want_tdust: bool = True):
        m = self.model
        td = np.zeros(m.shape4, dtype=np.float64, order="F") if want_tdust else None
        rel = C.c_double(0)
        conv = C.c_int(0)
        self._check(lib().hc3d_lucy_update(self._h, ltot, int(np_), None if td is None else td.ctypes.data_as(dp),
                                           C.byref(rel), C.byref(conv)))
        return td, rel.value, bool(conv.value)

    def set_lucy_tally(self, dtauabs: np.ndarray) -> None:
        """Replace the absorbed-path tally (hc3d_set_lucy_tally): (nrg,ntg,npg,ndg) int64 at this
        context's path_scale, e.g. the sum of the shards of an iteration."""
        a = np.asfortranarray(dtauabs, dtype=np.int64)
        self._check(lib().hc3d_set_lucy_tally(self._h, a.ctypes.data_as(P(C.c_int64))))

    def run_chunk(self, params: RunParams, np_iteration: int, final: bool) -> None:
        """One chunk of a peeled iteration of np_iteration packets (hc3d_run_chunk):
        with final False the packets still in flight continue in the next chunk."""
        self._check(lib().hc3d_run_chunk(self._h, C.byref(params), int(np_iteration), 1 if final else 0))

    def set_wave_options(self, queue_records: int = 0, regen: int = 0, qchunk: int = 0, peel_shape: int = 0) -> None:
        """Queue depth, regeneration threshold, queue-slot chunk and peel-off
        block shape (1, 2) of the wavefront form (hc3d_set_wave_options; 0
        keeps a setting)."""
        self._check(lib().hc3d_set_wave_options(self._h, int(queue_records), int(regen), int(qchunk),
                                                int(peel_shape)))

    def autotune(self, sample: RunParams) -> dict:
        """Time the sample batch under each candidate setting and keep the fastest (hc3d_autotune)."""
        r = TuneResult()
        self._check(lib().hc3d_autotune(self._h, C.byref(sample), C.byref(r)))
        return {"candidates": [{"queue_records": int(r.queue_records[k]), "block_size": int(r.block_size[k]),
                                "regen": int(r.regen[k]), "peel_shape": int(r.peel_shape[k]),
                                "peel_threads": int(r.peel_threads[k]), "ms": float(r.ms[k])} for k in range(r.n)],
                "best": int(r.best)}

    def lucy_iterations(self, params: RunParams, n_iter: int, ltot: float, want_tdust: bool = True):
        """n_iter Lucy iterations as one CUDA graph (hc3d_lucy_iterations):
        returns (tdust, max_rel_change per iteration)."""
        m = self.model
        td = np.zeros(m.shape4, dtype=np.float64, order="F") if want_tdust else None
        rel = np.zeros(n_iter, dtype=np.float64)
        self._check(lib().hc3d_lucy_iterations(self._h, C.byref(params), int(n_iter), float(ltot), _ptr(rel),
                                               None if td is None else td.ctypes.data_as(dp)))
        return td, rel

    def trace(self, params: RunParams, uniforms: np.ndarray, max_rec: int = 4096):
        u = np.ascontiguousarray(uniforms, dtype=np.float64)
        if u.ndim == 1:
            u = u[None, :]
        npkt, nu = u.shape
        recs = np.zeros(npkt * max_rec, dtype=TRACE_DTYPE)
        nrec = np.zeros(npkt, dtype=np.int32)
        self._check(lib().hc3d_trace_packets(self._h, C.byref(params), npkt, _ptr(u), nu,
                                             recs.ctypes.data_as(P(TraceRec)), max_rec, _ptr(nrec, C.c_int32)))
        return [recs[k * max_rec: k * max_rec + nrec[k]] for k in range(npkt)]

    def disk(self, converge: str, iter_: int, np_: int | None = None, ipeel: int | None = None,
             packet_offset: int = 0):
        """One call of disk(converge, iter, i1) (newdisktherm.F90:1): zero the
        tallies (initarr(.false.)), run the packet loop, read the tallies and
        solve the Lucy temperatures (tfinal).  Returns (tallies, converge,
        max_rel_change, tdust)."""
        m = self.model
        n = m.info.np if np_ is None else np_
        pe = (m.info.ipeel if converge == "yes" else 0) if ipeel is None else ipeel
        params = m.run_params(np=n, iter=iter_, ipeel=pe, packet_offset=packet_offset)
        self.zero()
        self.run(params)
        tal = self.tallies(params)
        td, rel, conv = self.lucy_update(m.info.ltot, n)
        m.set_tdust(td)
        new = "yes" if (converge == "yes" or conv) else "no"
        return tal, new, rel, td

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().hc3d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tts(par_path, out_dir, par_dir=None, precision: int = PREC_MIXED, device: int = 0) -> TtsStats:
    """Run program tts (newtts.F90) on the GPU and write its ASCII outputs."""
    st = TtsStats()
    err = C.create_string_buffer(1024)
    o = DeviceOpts(device, precision, 0, 0)
    Path(out_dir).mkdir(parents=True, exist_ok=True)
    rc = lib().hc3d_tts(str(par_path).encode(), None if par_dir is None else str(par_dir).encode(),
                        str(out_dir).encode(), C.byref(o), C.byref(st), err, 1024)
    if rc != 0:
        raise Hc3dError(rc, err.value.decode())
    return st


def run_batch(contexts, params) -> None:
    """The packet loops of several loaded contexts in one persistent launch
    (hc3d_run_batch), unpeeled or peeled; each context's tallies equal a run
    of its own (bit for bit in the FP64 form)."""
    n = len(contexts)
    hs = (C.c_void_p * n)(*[c._h.value for c in contexts])
    ps = (RunParams * n)(*params)
    rc = lib().hc3d_run_batch(hs, ps, n)
    if rc != 0:
        buf = C.create_string_buffer(1024)
        lib().hc3d_get_error(contexts[0]._h, buf, 1024)
        raise Hc3dError(rc, buf.value.decode())


class Server:
    """A model-run server on one GPU (hc3d_server_*): requests are queued,
    admitted by device footprint against an HBM budget and run on `slots`
    concurrent contexts."""

    def __init__(self, slots: int = 4, precision: int = PREC_MIXED, device: int = 0, hbm_budget: int = 0):
        h = C.c_void_p()
        rc = lib().hc3d_server_create(C.byref(h), C.byref(ServerOpts(device, precision, slots, hbm_budget)))
        if rc != 0:
            raise Hc3dError(rc, "hc3d_server_create failed")
        self._h = h

    def submit(self, par_path, par_dir=None, n_lucy: int = -1, np_lucy: int = 0, np_: int = 0,
               thete=None, phie=None) -> int:
        """Queue a model run; thete/phie (radians) override the model's peel-off directions."""
        q = Request(str(par_path).encode(), None if par_dir is None else str(par_dir).encode(), n_lucy, np_lucy,
                    np_, 0, None, None)
        keep = []
        if thete is not None:
            th = np.ascontiguousarray(thete, dtype=np.float64)
            ph = np.ascontiguousarray(phie if phie is not None else np.zeros_like(th), dtype=np.float64)
            keep = [th, ph]
            q.npeel, q.thete, q.phie = len(th), _ptr(th), _ptr(ph)
        t = C.c_int64(0)
        rc = lib().hc3d_server_submit(self._h, C.byref(q), C.byref(t))
        del keep
        if rc != 0:
            raise Hc3dError(rc, "hc3d_server_submit failed")
        return t.value

    def wait(self, ticket: int) -> dict:
        """Block until the request is done; its SEDs and timings as a dict."""
        r = Result()
        rc = lib().hc3d_server_wait(self._h, ticket, C.byref(r))
        if rc != 0:
            raise Hc3dError(rc, r.err.decode())
        sed = (r.nfreq, r.nmu, r.nph, r.nap, NO)
        psed = (r.nfreq, r.npeel, r.nap, NO)
        nsed, npsed = int(np.prod(sed)), int(np.prod(psed))
        out = {k: getattr(r, k) for k in ("t_submit", "t_admit", "t_done", "footprint_bytes", "packets",
                                          "iterations", "max_rel_change", "stokes_scale")}
        out["si"] = np.ctypeslib.as_array(r.si, shape=(nsed,)).copy().reshape(sed, order="F")
        out["nums"] = np.ctypeslib.as_array(r.nums, shape=(nsed,)).copy().reshape(sed, order="F")
        if npsed:
            out["ti"] = np.ctypeslib.as_array(r.ti, shape=(npsed,)).copy().reshape(psed, order="F")
            out["numt"] = np.ctypeslib.as_array(r.numt, shape=(npsed,)).copy().reshape(psed, order="F")
        else:
            out["ti"] = np.zeros(psed, dtype=np.int64)
            out["numt"] = np.zeros(psed, dtype=np.int64)
        lib().hc3d_result_free(C.byref(r))
        return out

    def cancel(self, ticket: int) -> int:
        """Cancel a request (hc3d_server_cancel): a queued one is dropped, a
        running one stops before its next iteration; its wait then raises
        Hc3dError with code HC3D_ERR_CANCELLED.  Returns the call's code."""
        return int(lib().hc3d_server_cancel(self._h, ticket))

    def stats(self) -> dict:
        st = ServerStats()
        lib().hc3d_server_get_stats(self._h, C.byref(st))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().hc3d_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def version() -> str:
    return lib().hc3d_version().decode()
