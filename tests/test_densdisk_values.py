"""The disk densities of the host gridset against an independent Python
restatement of densdiskg.f90:25-155 (tests/golden/ref_routines.py), cell by
cell, for models with every structure option: gap with its own density law,
puffed and curved gap wall, puffed and curved rim, radial cutoff; warp of two
spots and spiral arms.  The disk-mass normalisation and the density scales
rho0 / rhogap0 are constants per region, so each cell's density divided by
the restatement's (with unit density scales) is one constant outside the
gap and one inside it, to rounding; the empty cells agree exactly.  CPU only."""
from __future__ import annotations

import math

import numpy as np
import pytest

from hochunk3d_gb300 import configs, hc3d
from tests.golden import ref_routines as R

GRID = {"NRG": 60, "NTG": 41, "MASSD": 0.01, "RATE": 1e-9, "NP": 1000, "NPMIN": 1000}
CASES = {
    "gap_rim_cutoff": {"NPG": 2, "CGAPD": "YES", "RGAPD1": 3.0, "RGAPD2": 8.0, "RHOSCALE_GAP(1)": 0.3,
                       "A_GAP(1)": 1.5, "B_GAP(1)": 1.1, "ZSCALE_GAP(1)": 0.02, "CGAPPUFF": "YES", "GAPHEIGHT": 0.5,
                       "GAPLENGTH": 4.0, "CGAPCURVE": "YES", "GAPCURVEHEIGHT": 0.2, "GAPCURVELENGTH": 6.0,
                       "GAPCURVEEXP": 1.3, "CRIMPUFF": "YES", "RIMHEIGHT": 0.7, "RIMLENGTH": 0.2,
                       "CRIMCURVE": "YES", "RIMCURVEHEIGHT": 0.3, "RIMCURVELENGTH": 0.5, "RIMCURVEEXP": 0.8,
                       "CRADEXP": "YES", "RADEXP": 40.0},
    "warp_spiral": {"NPG": 17, "CDISKWARP": "YES", "WARPHEIGHT": 0.8, "WEXP": 3.0, "WARPLENGTH": 4.0, "NSPOT": 2,
                    "CSPIRAL": "YES", "PITCH": 15.0, "SN": 6, "SW": 0.4, "RSPIRAL1": 1.0, "RSPIRAL2": 60.0},
}


def _params(cfg: dict) -> dict:
    rstar, tstar = cfg["RSTAR"], cfg["TSTAR"]
    autors = 1.49598e13 / 6.9598e10 / rstar
    rminsub = (1600.0 / tstar) ** (-2.1)  # CRMIN=RSUB, no accretion: tave = tstar
    on = lambda k: 1 if cfg.get(k, "NO") == "YES" else 0
    P = {"idiskcurve": 1 if cfg["CDISKCURV"] == "SPH" else 0, "a": cfg["A(1)"], "b": cfg["B(1)"],
         "z1": cfg["ZSCALE(1)"], "rho0": 1.0, "rddust": rminsub * cfg["RMIND(1)"], "rmaxd": cfg["RMAXD(1)"] * autors,
         "igapd": on("CGAPD"), "rgapd1": max(cfg["RGAPD1"] * autors, 1.0), "rgapd2": cfg["RGAPD2"] * autors,
         "agap": cfg["A_GAP(1)"], "bgap": cfg["B_GAP(1)"], "z1gap": cfg["ZSCALE_GAP(1)"],
         "rhogap0": 1.0 if cfg["RHOSCALE_GAP(1)"] != 0.0 else 0.0,
         "idiskwarp": on("CDISKWARP"), "warpheight": cfg["WARPHEIGHT"], "wexp": float(cfg["WEXP"]),
         "warplength": cfg["WARPLENGTH"] * autors, "nspot": int(cfg["NSPOT"]),
         "irimcurve": on("CRIMCURVE"), "rimcurveheight": cfg["RIMCURVEHEIGHT"],
         "rimcurvelength": cfg["RIMCURVELENGTH"] * autors, "rimcurveexp": cfg["RIMCURVEEXP"],
         "irimpuff": on("CRIMPUFF"), "rimheight": cfg["RIMHEIGHT"], "rimlength": cfg["RIMLENGTH"] * autors,
         "igappuff": on("CGAPPUFF"), "gapheight": cfg["GAPHEIGHT"], "gaplength": cfg["GAPLENGTH"] * autors,
         "igapcurve": on("CGAPCURVE"), "gapcurveheight": cfg["GAPCURVEHEIGHT"],
         "gapcurvelength": cfg["GAPCURVELENGTH"] * autors, "gapcurveexp": cfg["GAPCURVEEXP"],
         "ispiral": on("CSPIRAL"), "pitch": cfg["PITCH"] * math.pi / 180.0, "sn": int(cfg["SN"]), "sw": cfg["SW"],
         "rspiral1": cfg["RSPIRAL1"] * autors, "rspiral2": cfg["RSPIRAL2"] * autors,
         "iradexp": on("CRADEXP"), "radexp": cfg["RADEXP"] * autors}
    return P


@pytest.mark.parametrize("case", sorted(CASES))
def test_disk_densities_match_restatement(tmp_path, built, case):
    over = dict(GRID)
    over.update(CASES[case])
    m = hc3d.Model(configs.write_par(tmp_path, "tiny", **over))
    cfg = dict(configs.BASE)
    cfg.update(configs.CONFIGS["tiny"])
    cfg.update(over)
    P = _params(cfg)
    nrg, ntg, npg, _ = m.shape4
    ratios = {}
    nonzero = 0
    for ir in range(nrg - 1):
        rad = 10.0 ** (0.5 * (math.log10(m.rarr[ir]) + math.log10(m.rarr[ir + 1])))  # gridset.f90:493-498
        for it in range(ntg - 1):
            t1, t2 = m.thetarr[it] * m.thetarr[it], m.thetarr[it + 1] * m.thetarr[it + 1]
            thet = (0.5 * (t1 + t2)) ** 0.5  # gridset.f90:615-618, pexp = 2
            cost, sint = math.cos(thet), math.sin(thet)
            for ip in range(npg - 1):
                phi = 0.5 * (m.phiarr[ip] + m.phiarr[ip + 1])
                region = []
                want = R.densdiskg(rad, sint, cost, phi, P, region)
                got = m.densarr[ir, it, ip, 0]
                assert (want == 0.0) == (got == 0.0), (ir, it, ip, got, want)
                if want != 0.0:
                    nonzero += 1
                    ratios.setdefault(region[0], []).append(got / want)
    assert nonzero > 500
    for reg, v in ratios.items():
        v = np.array(v)
        np.testing.assert_allclose(v, v[0], rtol=1e-11, err_msg=f"{case} region {reg}")
    if P["igapd"]:
        assert len(ratios) == 2  # both the gap's law and the disk's were exercised
