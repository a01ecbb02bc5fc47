"""Benchmark models as complete .par files (reapar.f90 keys) plus their fixtures.

The reference's shipped ``mctherm.par`` lacks keys that ``reapar`` requires
(NXIMG, RMAXD(1..2), RMIND(1..2), CDISKCURV, ...), so the models here are
written out in full.  Dust and stellar-spectrum inputs are synthetic fixtures
written by the library (``hc3d_write_synthetic_dust``,
``hc3d_write_wavelength_grid`` and ``hc3d_write_synthetic_isrf``): the dust
files the reference names are not shipped.

Models:
  plain   -- the plain small model: star 4000 K, 2 Rsun; flared disk
             0.01 Msun, Rsub..300 AU, rho ~ r^-2.25, h ~ r^1.25, h = 0.01 R* at
             R*; Ulrich envelope Mdot 5e-6 Msun/yr, Rc 100 AU, 5000 AU;
             conical cavity 20 deg at 1e-20 g/cc; grid 200 x 199 x 1;
             1e6 packets, 5 Lucy iterations, 10 inclinations, 149^2 images,
             50 wavelength bins over 0.1-3000 um.
  full3d  -- the same model with a seeded 3-level fractal envelope (clump
             fraction 0.5, contrast 100), grid 400 x 199 x 64, 1e8 packets,
             20 inclinations x 4 azimuths, 301^2 Stokes images.
  lucy    -- grid 400 x 399 x 128, 100 wavelength bins, 10 Lucy iterations of
             1e8 packets.
  tiny    -- a small grid of the plain model for CPU parity tests.
  tiny3d  -- a small 3-D grid (with azimuthal walls) for CPU parity tests.
  tiny_isrf -- tiny with external illumination (COUTILLUM=YES, a synthetic
             field of three diluted blackbodies, ISRF_SCL 10).
  tiny_acc -- tiny with disk accretion (CDISKACC=YES, Mdot 3e-7 Msun/yr,
             magnetospheric truncation at 5 R*), two hot spots at latitude
             60 deg covering 5 % of the star, and a gap between 0.1 and
             0.2 AU where the accretion packets are emitted by the gas.
  tiny_sg -- tiny with very small grains and PAHs: 20 % of the mass of disk
             1 in small grains (species 5), which re-emit from 18 synthetic
             emission spectra by the cells' mean intensity; no cavity, so
             the device slots carry species 1, 2, 3 and 5.
"""
from __future__ import annotations

import math
from pathlib import Path

DUST_FILE = "synth_dust.par"
WAVE_FILE = "synth_wavegrid.ascii"
ISRF_FILE = "synth_isrf.dat"


def _inclinations(n: int) -> list[float]:
    mus = [1.0 - (k + 0.5) / n for k in range(n)]
    return [round(math.degrees(math.acos(m)), 2) + 0.013 for m in mus]


BASE = {
    # preliminaries
    "NP": 1000000, "NPMIN": 10000, "NIMIN": 5, "NIMAX": 5, "CPEEL": "YES", "CLUCY": "YES", "I1": -2211,
    "IWRITE": 100000, "CWARN": "NO", "PARDIR": "'.'", "DENSINPUT": "NO",
    # central source
    "CLIMB": "NO", "CPLANCKST": "YES", "ATNAME": WAVE_FILE, "RSTAR": 2.0, "TSTAR": 4000.0, "MASSC": 0.5,
    "CSPOT": "NO", "SPOTLAT": 45.0, "NSPOT": 1, "CTEMP": "NO", "TSPOT/FSPOT": 0.01,
    # outside illumination
    "COUTILLUM": "NO", "ISRF_SCL": 1.0, "ISRF_AV": 0.0,
    # disk
    "MASSD": 0.01, "RMAXD(1)": 300.0, "RMAXD(2)": 300.0, "CRMIN": "RSUB", "RMIND(1)": 1.0, "RMIND(2)": 1.0,
    "CZMIN": "RSTAR", "FMASSD1": 1.0, "CHSEQ": "NO", "ITER_HSEQ": 3, "DISK_HSEQ": 1, "CDISKCURV": "CYL",
    "CGAPD": "NO", "RGAPD1": 3.0, "RGAPD2": 5.0, "CSPIRAL": "NO", "PITCH": 30.0, "SN": 10, "SW": 0.5,
    "RSPIRAL1": 1.0, "RSPIRAL2": 100.0, "CDISKWARP": "NO", "WARPHEIGHT": 1.0, "WEXP": 41, "WARPLENGTH": 5.0,
    "CRIMPUFF": "NO", "RIMHEIGHT": 1.0, "RIMLENGTH": 0.01, "CGAPPUFF": "NO", "GAPHEIGHT": 1.0, "GAPLENGTH": 1.0,
    "CRIMCURVE": "NO", "RIMCURVEHEIGHT": 1.0, "RIMCURVELENGTH": 1.0, "RIMCURVEEXP": 1.0,
    "CGAPCURVE": "NO", "GAPCURVEHEIGHT": 1.0, "GAPCURVELENGTH": 1.0, "GAPCURVEEXP": 1.0,
    "CMISALIGN": "NO", "RADMISALIGN": 1.0, "INCMISALIGN": 0.0,
    "DUSTNAME(1)": DUST_FILE, "DUSTNAME(5)": DUST_FILE, "FSG(1)": 0.0, "ZSCALE(1)": 0.01, "A(1)": 2.25,
    "B(1)": 1.25, "ZSCALE_GAP(1)": 0.01, "A_GAP(1)": 2.25, "B_GAP(1)": 1.25, "RHOSCALE_GAP(1)": 0.0,
    "DUSTNAME(2)": DUST_FILE, "DUSTNAME(6)": DUST_FILE, "FSG(2)": 0.0, "ZSCALE(2)": 0.01, "A(2)": 2.25,
    "B(2)": 1.25, "ZSCALE_GAP(2)": 0.01, "A_GAP(2)": 2.25, "B_GAP(2)": 1.25, "RHOSCALE_GAP(2)": 0.0,
    "CRADEXP": "NO", "RADEXP": 50.0,
    "CDISKACC": "NO", "CALPHA": "NO", "ALPHA/MDOT": 1e-8, "RTRUNC": 5.0,
    # envelope
    "DUSTNAME(3)": DUST_FILE, "DUSTNAME(7)": DUST_FILE, "FSG(3)": 0.0, "RMAX": 5000.0, "RMINE": 1.0,
    "ENVTYPE": "ULRICH", "RATE": 5.0e-6, "RC": 100.0, "RHODENS1": 1e-14, "ENVEXP": 1.5, "RHOAMB": 0.0,
    "CFRACTAL": "NO", "DENSRATIO": 0.5, "FRACTMASK": "0,0,1,0", "IFSEED": -3144,
    "CGAPE": "NO", "RGAPE1": 3.0, "RGAPE2": 5.0, "CGAPEDENS": "SCALE", "FRACTE": 0.001, "RHOGAPE": 1e-15,
    # cavity
    "DUSTNAME(4)": DUST_FILE, "DUSTNAME(8)": DUST_FILE, "FSG(4)": 0.0, "CHOLE": "YES", "CSHAPE": "POLYN",
    "RCHOLE": 300.0, "THET1": 20.0, "EX1": 1.0, "Z01": 0.0, "THET2": 20.0, "EX2": 1.0, "Z02": 0.0, "EXF": 0.0,
    "RHOCONST1": 1e-20, "RHOCONST2": 1e-20, "RMIN_SG": 1.0,
    # output
    "IMFILT": "NO", "IMCUBE": "NO", "IMSPARSE": "NO", "NPEEL": 10, "NAP": 1, "RMAXI": 1000.0,
    "APMIN": 100000.0, "APMAX": 100000.0, "THETE": ",".join(f"{t:.3f}" for t in _inclinations(10)),
    "PHIE": ",".join(["0.0"] * 10), "NMU": 10, "NPH": 1, "NFREQ": 50,
    "PARTIALPEEL": "NO", "SPARSEF": 3, "SPARSED": 96, "SPARSERMIN": 10.0, "SPARSERMAX": 1200.0, "DIFFUSION": "NO",
    # grid
    "NRG": 200, "NTG": 199, "NPG": 2, "NXIMG": 149,
    # extensions
    "SEDLMIN": 0.1, "SEDLMAX": 3000.0, "IMAGE": "YES", "MAXINT": 1000000,
}


def _full3d() -> dict:
    th = _inclinations(20)
    phis = [0.0, 90.0, 180.0, 270.0]
    thete = [t for t in th for _ in phis]
    phie = [p for _ in th for p in phis]
    return {
        "NP": 100000000, "NRG": 400, "NTG": 199, "NPG": 65, "NPEEL": 80, "NXIMG": 301,
        "THETE": ",".join(f"{t:.3f}" for t in thete), "PHIE": ",".join(f"{p:.1f}" for p in phie),
        "CFRACTAL": "YES", "DENSRATIO": 0.5, "FRACTMASK": "0,0,1,0", "IFSEED": -3144, "FRACTLEV": 3,
        "FRACTN": 32, "FRACTCONTRAST": 100.0,
    }


CONFIGS = {
    "plain": {},
    "full3d": _full3d(),
    "lucy": {"NP": 100000000, "NRG": 400, "NTG": 399, "NPG": 129, "NFREQ": 100, "NIMIN": 10, "NIMAX": 10,
             "CPEEL": "NO", "NPMIN": 100000000},
    "tiny": {"NP": 4000, "NPMIN": 2000, "NIMIN": 2, "NIMAX": 2, "NRG": 40, "NTG": 31, "NPG": 2, "NXIMG": 31,
             "MASSD": 0.0001, "RATE": 5e-7},
    # tiny with external illumination: ISRF_SCL 10 gives the outside field
    # about 40 % of the luminosity
    "tiny_isrf": {"NP": 4000, "NPMIN": 2000, "NIMIN": 2, "NIMAX": 2, "NRG": 40, "NTG": 31, "NPG": 2, "NXIMG": 31,
                  "MASSD": 0.0001, "RATE": 5e-7, "COUTILLUM": "YES", "ISRF_SCL": 10.0, "ISRF_FILE": ISRF_FILE},
    "tiny_acc": {"NP": 4000, "NPMIN": 2000, "NIMIN": 2, "NIMAX": 2, "NRG": 40, "NTG": 31, "NPG": 2, "NXIMG": 31,
                 "MASSD": 0.001, "RATE": 5e-7, "CDISKACC": "YES", "CALPHA": "NO", "ALPHA/MDOT": 3e-7, "RTRUNC": 5.0,
                 "CSPOT": "YES", "SPOTLAT": 60.0, "NSPOT": 2, "CTEMP": "NO", "TSPOT/FSPOT": 0.05,
                 "CGAPD": "YES", "RGAPD1": 0.1, "RGAPD2": 0.2, "RHOSCALE_GAP(1)": 0.0, "RHOSCALE_GAP(2)": 0.0},
    "tiny_sg": {"NP": 4000, "NPMIN": 2000, "NIMIN": 2, "NIMAX": 2, "NRG": 40, "NTG": 31, "NPG": 2, "NXIMG": 31,
                "MASSD": 0.001, "RATE": 5e-7, "FSG(1)": 0.2, "CHOLE": "NO", "ISRF_FILE": ISRF_FILE},
    "tiny3d": {"NP": 4000, "NPMIN": 2000, "NIMIN": 2, "NIMAX": 2, "NRG": 40, "NTG": 31, "NPG": 9, "NXIMG": 31,
               "MASSD": 0.0001, "RATE": 5e-7, "NPEEL": 4, "THETE": "30.013,60.013,80.013,120.013",
               "PHIE": "0.0,90.0,180.0,270.0", "CFRACTAL": "YES", "FRACTLEV": 2, "FRACTN": 8},
}


def par_text(cfg: dict) -> str:
    lines = ["' =================== Parameter file (GB300 photon loop benchmark model) ==================='", ""]
    for k, v in cfg.items():
        lines.append(f"{v!s:>24} = {k:>12} = ")
    return "\n".join(lines) + "\n"


def write_fixtures(directory: str | Path) -> Path:
    """Write the synthetic dust file and stellar wavelength grid (host only, no GPU)."""
    from . import hc3d

    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    L = hc3d.host_lib()
    rc = L.hc3d_write_synthetic_dust(str(d / DUST_FILE).encode())
    if rc != 0:
        raise hc3d.Hc3dError(rc, "cannot write dust fixture")
    rc = L.hc3d_write_wavelength_grid(str(d / WAVE_FILE).encode(), 4000.0)
    if rc != 0:
        raise hc3d.Hc3dError(rc, "cannot write wavelength fixture")
    rc = L.hc3d_write_synthetic_isrf(str(d / ISRF_FILE).encode())
    if rc != 0:
        raise hc3d.Hc3dError(rc, "cannot write external-field fixture")
    rc = L.hc3d_write_synthetic_draine(str(d).encode())
    if rc != 0:
        raise hc3d.Hc3dError(rc, "cannot write small-grain spectra fixtures")
    return d


def write_par(directory: str | Path, name: str = "plain", **over) -> Path:
    """Write fixtures and <name>.par into directory; keyword overrides replace keys."""
    d = write_fixtures(directory)
    cfg = dict(BASE)
    cfg.update(CONFIGS[name])
    cfg.update(over)
    cfg["PARDIR"] = f"'{d}'"
    path = d / f"{name}.par"
    path.write_text(par_text(cfg))
    return path
