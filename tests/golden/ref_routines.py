"""A second, independent restatement of the reference's self-contained
routines in plain Python, written from the Fortran bodies without reference
to the C oracle (oracle/hc3d_oracle.c).  tests/test_ref_routines.py checks
the oracle's C functions against it on random inputs, so that a
transcription error in either restatement shows as a disagreement.

TEST INFRASTRUCTURE ONLY.  Each function cites the reference lines it
follows.  Scalars are Python floats (IEEE doubles, like the Fortran real*8);
arithmetic is written in the Fortran's order so that results agree to the
last bit where no transcendental function is involved (a Fortran power with
an integral exponent, x**2 or x**2.d0, is a product, so it is written x * x).
"""
from __future__ import annotations

import math

import numpy as np

PI = 3.1415926535897932384626433
R2P = 2.0 * PI
HUGE = 1.7976931348623157e308
SIGT = 5.670400e-5  # constants.f90:20


# ---- closest_wall.f90:13-66 ----------------------------------------------------
class ClosestWall:
    """The module's state: the largest negative root and the two smallest
    non-negative roots, with their wall ids."""

    def __init__(self):
        self.tn1, self.tp1, self.tp2 = -HUGE, HUGE, HUGE
        self.in1 = self.ip1 = self.ip2 = 0

    def insert(self, t: float, i: int) -> None:
        if t < 0.0:
            if t > self.tn1:
                self.tn1, self.in1 = t, i
        elif t < self.tp1:
            self.tp2, self.ip2 = self.tp1, self.ip1
            self.tp1, self.ip1 = t, i
        elif t < self.tp2:
            self.tp2, self.ip2 = t, i

    def next_wall(self, on_wall: bool):
        """(t, id), or None where the Fortran stops ("no valid solution").
        On a wall, the root nearest zero is the wall itself: when the
        negative root is closer to zero than the first positive one, the
        first positive root is the next wall, else the second."""
        if on_wall:
            t, i = (self.tp1, self.ip1) if abs(self.tn1) < abs(self.tp1) else (self.tp2, self.ip2)
        else:
            t, i = self.tp1, self.ip1
        return None if t == HUGE else (t, i)


# ---- radface.f90:44-62 ----------------------------------------------------------
def radface(cw: ClosestWall, ux, uy, uz, x1, y1, z1, r2_1, r2_2) -> None:
    bb = 2.0 * (x1 * ux + y1 * uy + uz * z1)
    rr = x1 * x1 + y1 * y1 + z1 * z1
    for r2, wall in ((r2_1, 1), (r2_2, 2)):
        cc = rr - r2
        d = bb * bb - 4.0 * cc
        if d > 0.0:
            d = math.sqrt(d)
            cw.insert((-bb + d) * 0.5, wall)
            cw.insert((-bb - d) * 0.5, wall)


# ---- phiface.f90:48-56 ------------------------------------------------------------
def phiface(cw: ClosestWall, a1, b1, c1, d1, a2, b2, c2, d2, ux, uy, uz, x1, y1, z1) -> None:
    for a, b, c, d, wall in ((a1, b1, c1, d1, 5), (a2, b2, c2, d2, 6)):
        den = a * ux + b * uy + c * uz
        if den != 0.0:
            cw.insert(-(a * x1 + b * y1 + c * z1 + d) / den, wall)


def check(x: float) -> float:
    """check.f90: clamp a cosine to [-1, 1]."""
    return 1.0 if x > 1.0 else (-1.0 if x < -1.0 else x)


# ---- findangle3.f90:31-67 ------------------------------------------------------------
def findangle3(cost1, sint1, phi1, cosp1, sinp1, cost2, sint2, phi2, cosp2, sinp2):
    """(costnew, sintnew, ri1, phinew) for the incident direction 1 and the
    outgoing direction 2; ri1 is None where the Fortran leaves it unset."""
    costnew = check(cost1 * cost2 + (sint1 * sint2 * (cosp1 * cosp2 + sinp1 * sinp2)))
    sintnew = math.sqrt(1.0 - costnew * costnew)
    ri1 = None
    if sint1 > 1.0e-8:
        if sintnew > 1.0e-8:
            cosx = check((cost2 - (cost1 * costnew)) / (sint1 * sintnew))
            x = math.acos(cosx)
            if phi2 > phi1:
                if phi2 - phi1 > PI:
                    ri1, phinew = x, PI + x
                else:
                    ri1, phinew = R2P - x, PI - x
            else:
                if phi1 - phi2 > PI:
                    ri1, phinew = R2P - x, PI - x
                else:
                    ri1, phinew = x, PI + x
        else:
            phinew = 0.0
    else:
        phinew = phi2
    return costnew, sintnew, ri1, phinew


# ---- dust.f90:70-74 and dustmat.f90:40-65 --------------------------------------------------
def phase_terms(g: float):
    g2 = g * g
    return g2, g2 + 1.0, 1.0 - g2, 2.0 * g


def dustmat(cost, cost2, g, pl):
    """(p1, p2, p3, p4) of the modified Cornette & Shanks phase matrix at the
    scattering cosine cost (cost2 = cost^2); p4 = 0 (circular polarisation
    off in the reference)."""
    g2, g2p1, onemg2, twog = phase_terms(g)
    temp = g2p1 - twog * cost
    p1 = 1.5 * onemg2 / (2.0 + g2) * (1.0 + cost2) / (temp * math.sqrt(temp))
    p2 = -pl * p1 * (1.0 - cost2) / (1.0 + cost2)
    p3 = p1 * 2.0 * cost / (1.0 + cost2)
    return p1, p2, p3, 0.0


def peak_of(g):
    """The rejection envelope of stokes.f90:49-57 (times 1.01)."""
    g2, g2p1, onemg2, twog = phase_terms(g)
    temp = g2p1 - twog if g > 0.0 else g2p1 + twog
    return 1.5 * onemg2 / (2.0 + g2) * 2.0 / temp / math.sqrt(temp) * 1.01


def _rotation(upper, p1, p2, p3, p4, s2a, c2a, sini2, cosi2):
    """The Mueller matrix rows of stokes.f90:230-240 (upper: ri1 > pi, the
    angle ri3 = 2 pi - ri1) and :359-369 (otherwise); s2a, c2a are the
    double-angle sine and cosine of ri3 or ri1."""
    sin2i2 = 2.0 * sini2 * cosi2
    cos2i2 = 2.0 * cosi2 * cosi2 - 1.0
    sin2 = sin2i2 * s2a
    cos2 = cos2i2 * c2a
    sin2cos1 = sin2i2 * c2a
    cos2sin1 = cos2i2 * s2a
    a21 = p2 * cos2i2
    a22 = p1 * cos2 - p3 * sin2
    if upper:
        a11, a12, a13 = p1, p2 * c2a, p2 * s2a
        a23 = p1 * cos2sin1 + p3 * sin2cos1
        a24 = -p4 * sin2i2
        a31 = -p2 * sin2i2
        a32 = -p1 * sin2cos1 - p3 * cos2sin1
        a42 = -p4 * s2a
    else:
        a11, a12, a13 = p1, p2 * c2a, -p2 * s2a
        a23 = -p1 * cos2sin1 - p3 * sin2cos1
        a24 = p4 * sin2i2
        a31 = p2 * sin2i2
        a32 = p1 * sin2cos1 + p3 * cos2sin1
        a42 = p4 * s2a
    a33 = -p1 * sin2 + p3 * cos2
    a34 = -p4 * cos2i2
    a43 = p4 * c2a
    a44 = p3
    return (a11, a12, a13), (a21, a22, a23, a24), (a31, a32, a33, a34), (a42, a43, a44)


def _apply(rows, s):
    (a11, a12, a13), (a21, a22, a23, a24), (a31, a32, a33, a34), (a42, a43, a44) = rows
    i, q, u, v = s
    return (a11 * i + a12 * q + a13 * u, a21 * i + a22 * q + a23 * u + a24 * v,
            a31 * i + a32 * q + a33 * u + a34 * v, a42 * q + a43 * u + a44 * v)


def _cosi2(cost, sint, sini, bmu, sinbt, costp, sintp):
    """sini2, cosi2 of stokes.f90:147-178 / stokespeel.f90:150-185 (cost,
    sint: the outgoing direction; costp, sintp: the incident one)."""
    if abs(cost) < 1.0:
        sini2 = sini * sintp / sint
        bott = sint * sinbt
        cosi2 = costp / bott - cost * bmu / bott
        if cosi2 >= 1.0:
            cosi2, sini2 = 1.0, 0.0
        if cosi2 <= -1.0:
            cosi2, sini2 = -1.0, 0.0
        return sini2, cosi2
    cosi2 = 0.0
    if cost >= 1.0:
        cosi2 = -1.0
    if cost <= -1.0:
        cosi2 = 1.0
    return 0.0, cosi2


# ---- stokespeel.f90:49-376 --------------------------------------------------------------
def stokespeel(s, cost, sint, ri1, bmu, costp, sintp, g, pl):
    """The Stokes vector s = (i, q, u, v) scattered by the angle bmu = cos(Theta)
    and rotated by ri1 into the peel-off direction (cost, sint); the incident
    direction is (costp, sintp).  Not divided by the accepted a: the result
    carries the phase-function weight."""
    cosb2 = bmu * bmu
    p1, p2, p3, p4 = dustmat(bmu, cosb2, g, pl)
    if abs(bmu) > 1.0:
        bmu = 1.0 if bmu > 1.0 else -1.0
        cosb2 = 1.0
    sinbt = math.sqrt(1.0 - cosb2)
    upper = ri1 > PI
    ang = R2P - ri1 if upper else ri1
    ci, si = math.cos(ang), math.sin(ang)
    s2a = 2.0 * si * ci
    c2a = 2.0 * ci * ci - 1.0
    if bmu == 1.0:
        return tuple(s)
    if bmu == -1.0:
        sini2, cosi2 = 1.0, 0.0
    else:
        sini2, cosi2 = _cosi2(cost, sint, si, bmu, sinbt, costp, sintp)
    return _apply(_rotation(upper, p1, p2, p3, p4, s2a, c2a, sini2, cosi2), s)


# ---- stokes.f90:46-388 (the dust branch, idust != 0) --------------------------------------
def stokes(state, g, pl, uniforms):
    """One scattering: state = (sip, sqp, sup, svp, cost, sint, phi, cosp,
    sinp); the uniforms are drawn in the Fortran order (bmu, ri1, the
    rejection test, repeated).  Returns (new state, number of uniforms used),
    or None when the uniforms run out."""
    sip, sqp, sup, svp, cost, sint, phi, cosp, sinp = state
    costp, sintp, phip = cost, sint, phi
    peak = peak_of(g)
    it = iter(uniforms)
    used = 0
    while True:
        try:
            bmu = 1.0 - 2.0 * next(it)
            cosb2 = bmu * bmu
            p1, p2, p3, p4 = dustmat(bmu, cosb2, g, pl)
            if abs(bmu) > 1.0:
                bmu = 1.0 if bmu > 1.0 else -1.0
                cosb2 = 1.0
            sinbt = math.sqrt(1.0 - cosb2)
            ri1 = R2P * next(it)
            upper = ri1 > PI
            ang = R2P - ri1 if upper else ri1
            ci, si = math.cos(ang), math.sin(ang)
            s2a = 2.0 * si * ci
            c2a = 2.0 * ci * ci - 1.0
            rprob = (p1 * sip + p2 * c2a * sqp + (p2 * s2a if upper else -p2 * s2a) * sup) / sip
            if rprob > peak:
                peak = rprob
            xran = next(it)
            used += 3
        except StopIteration:
            return None
        if not (peak * xran > rprob):
            break
    a = rprob
    if bmu == 1.0:
        return (sip, sqp, sup, svp, cost, sint, phi, cosp, sinp), used
    if bmu == -1.0:
        si, sini2, ci, cosi2 = 1.0, 1.0, 0.0, 0.0
        cost, sint = -costp, sintp
    else:
        cost = costp * bmu + sintp * sinbt * ci
        if abs(cost) < 1.0:
            sint = abs(math.sqrt(1.0 - cost * cost))
        else:
            cost = 1.0 if cost >= 1.0 else -1.0
            sint = 0.0
        sini2, cosi2 = _cosi2(cost, sint, si, bmu, sinbt, costp, sintp)
    cosdph = -cosi2 * ci + sini2 * si * bmu if upper else -ci * cosi2 + si * sini2 * bmu
    if abs(cosdph) > 1.0:
        cosdph = 1.0 if cosdph > 1.0 else -1.0
    phi = phip + math.acos(cosdph) if upper else phip - math.acos(cosdph)
    if phi > R2P:
        phi -= R2P
    if phi < 0.0:
        phi += R2P
    i, q, u, v = _apply(_rotation(upper, p1, p2, p3, p4, s2a, c2a, sini2, cosi2), (sip, sqp, sup, svp))
    return (i / a, q / a, u / a, v / a, cost, sint, phi, math.cos(phi), math.sin(phi)), used


# ---- opacset, dust.f90:9-80 -----------------------------------------------------------------
def opacset(nu, nudust, nlambda, gdust, pldust, kappad, adust):
    """(g, pl, kappa, albedo) of every species at frequency nu.  The tables
    are (nlammax, ndg) arrays (Fortran order: column id), nudust decreasing
    down a column (frequency falls as the wavelength grows)."""
    out = []
    for k in range(len(nlambda)):
        n = int(nlambda[k])
        nd = nudust[:, k]
        if nu >= nd[0]:
            j0 = j1 = 0
            f = 1.0
        elif nu <= nd[n - 1]:
            j0 = j1 = n - 1
            f = 1.0
        else:
            i0, i1 = 1, n
            while i1 - i0 > 1:
                i = (i1 + i0) // 2
                if nu <= nd[i - 1]:
                    i0 = i
                else:
                    i1 = i
            j0, j1 = i0 - 1, i1 - 1
            f = (nu - nd[j1]) / (nd[j0] - nd[j1])
        if j0 == j1:
            out.append((gdust[j0, k], pldust[j0, k], kappad[j0, k], adust[j0, k]))
            continue
        fm1 = 1.0 - f
        out.append(tuple(fm1 * t[j1, k] + f * t[j0, k] for t in (gdust, pldust, kappad, adust)))
    return out


# ---- select_dust.f90:16-42 ------------------------------------------------------------------
def select_dust(xran, kapd, dens):
    """0-based species chosen by its share of the opacity, or -1 where the
    Fortran stops (no opacity, or no species reached)."""
    opac = 0.0
    for k, d in zip(kapd, dens):
        opac = opac + k * d
    if opac == 0:
        return -1
    frac = 0.0
    tol = float(np.float32(1.0e-10))  # the Fortran literal 1.e-10 is default (single) precision
    for idx, (k, d) in enumerate(zip(kapd, dens)):
        frac = frac + k * d / opac
        if xran <= frac + tol:
            return idx
    return -1


# ---- KapP, dust.f90:114-141, and dusttemp.f90:30-50 ---------------------------------------
def kapp(T, lTint, kappap_row):
    nT = len(lTint)
    lT = math.log(T)
    k = int(float(nT - 1) * (lT - lTint[0]) / (lTint[nT - 1] - lTint[0])) + 1
    if k < 1 or k > nT - 1:
        return kappap_row[0] if k < 1 else kappap_row[nT - 1]
    f = (lT - lTint[k - 1]) / (lTint[k] - lTint[k - 1])
    return (1.0 - f) * kappap_row[k - 1] + f * kappap_row[k]


def dusttemp(na, T0, ltot, nphot, kappav, massarr, lTint, kappap_row, max_iter: int = 1000):
    """The fixed point Td = ((na ltot) / (4 sigma nphot kappav KapP(Td)))^(1/4)
    / 11605 / massarr, clamped to [0.1, 1600] K (in units of 11605 K)."""
    eps = 1.0e-5
    Td = T0 if T0 != 0.0 else 0.1 / 11605.0
    Told = 0.5 * Td
    n = 0
    while abs(Td - Told) > eps * Td and n < max_iter:
        n += 1
        Told = Td
        Td = ((na * ltot) / (4.0 * SIGT * nphot * kappav * kapp(Td, lTint, kappap_row))) ** 0.25 / 11605.0
        Td = Td / massarr if massarr > 0.0 else 0.1 / 11605.0
        if Td > 1600.0 / 11605.0:
            Td = 1600.0 / 11605.0
        Td = max(Td, 0.1 / 11605.0)
    return Td


# ---- lucydustfreq.f90:44-147 ---------------------------------------------------------------
def lucydustfreq(T0, xi, lTint, nuint, kapB):
    """Re-emission frequency for the uniform xi at temperature T0 from the
    cumulative table kapB(j, i) (nT x nnu, 0-based), log-interpolated
    between the bracketing frequencies.  The reference's branches for a
    table that is not monotone are kept, including its reset of i1 to 1."""
    nT, nnu = len(lTint), len(nuint)
    lT0 = math.log(T0)
    j = int(float(nT - 1) * (lT0 - lTint[0]) / (lTint[nT - 1] - lTint[0])) + 1
    f = (lT0 - lTint[j - 1]) / (lTint[j] - lTint[j - 1])
    f = min(max(f, 0.0), 1.0)

    def P(i):
        return (1.0 - f) * kapB[j - 1, i - 1] + f * kapB[j, i - 1]

    i0, i1 = 1, nnu
    P0 = P(i0)
    if xi < P0:
        return T0 * xi * nuint[0] / P0 if P0 > 0.0 else T0 * nuint[0]
    P1 = min(P(i1), 1.0)
    if xi >= P1:
        if P1 < 1.0 and xi < 1.0:
            return T0 * nuint[nnu - 1] * (1.0 - P1) / (1.0 - xi)
        return T0 * nuint[nnu - 1]
    while i1 - i0 > 1:
        i = (i0 + i1) // 2
        p = P(i)
        if p > 1.0:
            p = 1.0
        if p < P0:
            P0, i0 = p, i
        if p > P1:
            P1, i1 = p, 1
        if p > xi:
            i1, P1 = i, p
        else:
            i0, P0 = i, p
    if xi < P0:
        g = 0.0
    elif xi > P1:
        g = 1.0
    elif P0 <= 0.0:
        g = 0.5
    elif P1 <= 0.0 or xi <= 0.0:
        g = f  # the Fortran leaves f as it was
    else:
        g = math.log(xi / P0) / math.log(P1 / P0)
    return T0 * nuint[i0 - 1] * (nuint[i1 - 1] / nuint[i0 - 1]) ** g


# ---- diskflux, flux.f90:23-60: the escape SED columns --------------------------------------
def diskflux_sed(si, sq, su, sv, si2, sq2, su2, sv2, nums, np_, nmu, nph, ltot_lsun):
    """The normalised SED and its error columns as flux.f90 forms them:
    I / rnorm with rnorm = np / nmu / nph / (L/Lsun); the relative error of I
    sqrt((si2 - si^2/n) / (n - 1) n) / si + 1/n, and for Q, U, V the same
    without the 1/n term, in bins with more than one packet."""
    import numpy as np

    rnorm = float(np_) / float(nmu) / float(nph) / ltot_lsun
    out = {}
    n = nums.astype(np.float64)
    ok = n > 1.0
    with np.errstate(divide="ignore", invalid="ignore"):
        for key, s, s2 in (("i", si, si2), ("q", sq, sq2), ("u", su, su2), ("v", sv, sv2)):
            e = np.sqrt((s2 - s * s / n) / (n - 1.0) * n) / si
            if key == "i":
                e = e + 1.0 / n
            out[key + "_err"] = np.where(ok, e, 0.0)
    for key, s in (("i", si), ("q", sq), ("u", su), ("v", sv)):
        out[key] = s / rnorm
    return out


# ---- disk accretion and hot spots ------------------------------------------------
GN = 6.67428e-8   # constants.f90:19
MSOL = 1.989e33   # constants.f90:13
RSOL = 6.9598e10  # constants.f90:11
DEG2RAD = PI / 180.0
RAD2DEG = 180.0 / PI


def rho0_disk(massd, fmass, rmaxd, rmind, a, b, z1, rmincgs):
    """setup_wave.f90:60-92: the disk density scale of one species slot."""
    z1cgs = rmincgs * z1
    p = b - a
    if not (rmaxd > 0.0 and fmass > 0.0):
        return 0.0
    const = R2P ** 1.5 * rmincgs ** 2 * z1cgs
    if p != -2.0 and p != -1.5:
        den = 1.0 / (p + 2.0) * (rmaxd ** (p + 2.0) - rmind ** (p + 2.0)) - \
              1.0 / (p + 1.5) * (rmaxd ** (p + 1.5) - rmind ** (p + 1.5))
    elif p == -2.0:
        den = math.log(rmaxd / rmind) - 1.0 / (p + 1.5) * (rmaxd ** (p + 1.5) - rmind ** (p + 1.5))
    else:
        den = 1.0 / (p + 2.0) * (rmaxd ** (p + 2.0) - rmind ** (p + 2.0)) - math.log(rmaxd / rmind)
    return massd * MSOL / const / den * fmass


def accretion_luminosity(tstar, rstar, massc, massd, rddustmin, rtrunc, rho0, z1, ialpha, alphad, mdotdisk,
                         l_isrf, itemp, fspot, tspot, nspot, tsub=1600.0):
    """gridset.f90:72-264 with CDISKACC=YES: the accretion rates of the two
    disk slots, lacc, lacc2, the luminosity fractions, the shock temperature,
    the spot size and the mean stellar temperature with its sublimation
    radius.  Returns a dict."""
    rmincgs = rstar * RSOL
    yr = 3600.0 * 24.0 * 365.25
    lstar = 4.0 * PI * SIGT * tstar ** 4 * rmincgs ** 2
    vc = math.sqrt(GN * MSOL * massc / rmincgs)
    mdotcgs = [0.0, 0.0]
    if ialpha == 1:
        for i in range(2):
            mdotcgs[i] = math.sqrt(18.0 * PI ** 3.0) * alphad * vc * rho0[i] * (z1[i] * rmincgs) ** 3.0 / rmincgs
    else:
        tot = mdotdisk / (yr / MSOL)
        ratio = (rho0[0] * (z1[0] * z1[0] * z1[0]) / rho0[1] / (z1[1] * z1[1] * z1[1])) if rho0[1] != 0.0 else math.inf
        mdotcgs[1] = tot / (1.0 + ratio)
        mdotcgs[0] = tot - mdotcgs[1]
    mdot = mdotcgs[0] + mdotcgs[1]
    lacc = GN * (MSOL * massc) * mdot / 2.0 / (rddustmin * rmincgs)
    lacc2 = GN * (MSOL * massc) * mdot * (1.0 / rmincgs - 1.0 / (rmincgs * rtrunc)) if massd > 0.0 else 0.0
    if massd <= 0.0:
        lacc = 0.0
    ltot = lacc + lacc2 + lstar + l_isrf
    out = {"lstar": lstar, "lacc": lacc, "lacc2": lacc2, "ltot": ltot, "accfrac": lacc / ltot,
           "accfrac2": lacc2 / ltot, "mdot_msun_yr": mdot * yr / MSOL, "tshock_k": 0.0, "thspot_deg": 0.0,
           "fspot": fspot}
    if lacc2 > 0.0:
        if itemp == 0:
            tshock = tstar * (1.0 + 0.5 * lacc2 / lstar / fspot) ** 0.25
        else:
            tshock = tspot
            fspot = 0.5 * lacc2 / lstar / ((tshock / tstar) ** 4 - 1.0)
        th = math.acos(1.0 - 2.0 * fspot) if nspot == 1 else math.acos(1.0 - fspot)
        out.update(tshock_k=tshock, thspot_deg=th * RAD2DEG, fspot=fspot)
    tave = tstar * (1.0 + 0.5 * lacc2 / lstar) ** 0.25
    out["tave_k"] = tave
    out["rminsub"] = (tsub / tave) ** (-2.1)
    return out


def packet_shares(np_, accfrac, accfrac2, isrf_frac):
    """newdisktherm.F90:143-175 and the loop tests of 209, 256, 258: the
    number of accretion, hot-spot, stellar and external packets of an
    iteration of np_ packets (iphot = 1..np_)."""
    npout = int(isrf_frac * np_)
    if isrf_frac * np_ - npout > 0.5:
        npout += 1
    ns = int(np_ * (1.0 - accfrac - isrf_frac))
    rn = float(np.float32(np_)) * (1.0 - accfrac - isrf_frac)  # real(np): single precision
    if rn - ns > 0.5:
        ns += 1
    npacc = int(np_ * accfrac)
    npaccstar = int(accfrac2 * np_)
    if int(ns * accfrac2) - npaccstar > 0.5:
        npaccstar += 1
    if ns + npacc + npout != np_:
        ns = ns + np_ - (ns + npacc + npout)
    counts = {"acc": 0, "spot": 0, "star": 0, "ext": 0}
    for iphot in range(1, np_ + 1):
        if iphot < npacc:
            counts["acc"] += 1
        elif iphot <= npacc + ns:
            counts["spot" if iphot < npacc + npaccstar else "star"] += 1
        else:
            counts["ext"] += 1
    return counts


def inczeta(izmax=145):
    """zetainit, random.f90:79-97."""
    z = [0.0] * izmax
    for j in range(izmax, 0, -1):
        term = 1.0 / float(j * j * j * j)
        for i in range(izmax, j - 1, -1):
            z[i - 1] = z[i - 1] + term
    return z


def bbfreq(teff, u, zeta=None):
    """random.f90:49-77 with the five uniforms u."""
    zeta = zeta or inczeta()
    z0 = zeta[-1] * u[0]
    i = 1
    while z0 > zeta[i - 1]:
        i += 1
    return -math.log(u[1] * u[2] * u[3] * u[4]) * teff / float(i)


def spot_geometry(spotlat, thspot_deg):
    """spotset.f90:187-206: (scspot, ssspot, cspot, sspot) of both spots and csprad."""
    th1 = (90.0 - spotlat) * DEG2RAD
    ph1 = 0.0 * DEG2RAD
    th2, ph2 = PI - th1, ph1 + PI
    s1 = (math.sin(th1) * math.cos(ph1), math.sin(th1) * math.sin(ph1), math.cos(th1), math.sin(th1))
    s2 = (math.sin(th2) * math.cos(ph2), math.sin(th2) * math.sin(ph2), math.cos(th2), math.sin(th2))
    return s1, s2, math.cos(thspot_deg * DEG2RAD)


def _rpow(x, y):
    """x**y for a real exponent as C and Fortran form it: NaN for x < 0 and y
    not an integer (Python would return a complex number)."""
    if x < 0.0 and y != int(y):
        return float("nan")
    return x ** y


def _powi(x, n):
    """x**n for an integer n, as the Fortran runtime forms it (squaring)."""
    r, u = 1.0, abs(n)
    while u:
        if u & 1:
            r *= x
        u >>= 1
        if u:
            x *= x
    return 1.0 / r if n < 0 else r


def densdiskg(rad, sint, cost, phi, P, region_out=None):
    """densdiskg.f90:25-155 for one disk slot.  P holds the slot's scaled
    parameters (lengths in stellar radii, angles in radians): a, b, z1, rho0,
    rddust, rmaxd; the gap's agap, bgap, z1gap, rhogap0, rgapd1, rgapd2; and
    the switches and parameters of the warp, rim and gap puffs and curves,
    spiral arms and radial cutoff (keys as the Fortran names).  region_out,
    when given, receives "gap" or "disk": which density law applied."""
    rp = rad * sint
    zp = rad * cost
    rcoord = rad if P["idiskcurve"] == 1 else rp
    rmin = 1.0
    ingap = P["igapd"] == 1 and P["rgapd1"] < rcoord < P["rgapd2"]
    if ingap:
        adens, bdens, rhodens, zscale = P["agap"], P["bgap"], P["rhogap0"], P["z1gap"]
    else:
        adens, bdens, rhodens, zscale = P["a"], P["b"], P["rho0"], P["z1"]
    if region_out is not None:
        region_out.append("gap" if ingap else "disk")
    warp = warp2 = 0.0
    if P["idiskwarp"] == 1:
        q = (rcoord - P["rddust"]) / P["warplength"]
        fall = math.exp(-(q * q))
        warp = P["warpheight"] * _rpow(math.cos(phi / 2.0), P["wexp"]) * fall
        if phi >= PI:
            warp = -warp
        if P["nspot"] == 2:
            warp2 = P["warpheight"] * _rpow(math.cos(phi / 2.0 - PI / 2.0), P["wexp"]) * fall
    rimcurve = 0.0
    if P["irimcurve"] == 1:
        rimcurve = P["rimcurveheight"] * math.exp(-_rpow((rcoord - P["rddust"]) / P["rimcurvelength"], P["rimcurveexp"]))
    rimpuff = 0.0
    if P["irimpuff"] == 1:
        q = (rcoord - P["rddust"]) / P["rimlength"]
        rimpuff = P["rimheight"] * math.exp(-(q * q))
    if rcoord < P["rddust"]:
        rimpuff = 0.0
    gappuff = 0.0
    if P["igappuff"] == 1 and P["igapd"] == 1:
        q = (rcoord - P["rgapd2"]) / P["gaplength"]
        gappuff = P["gapheight"] * math.exp(-(q * q))
    if rcoord < P["rgapd2"]:
        gappuff = 0.0
    gapcurve = 0.0
    if P["igapcurve"] == 1 and P["igapd"] == 1:
        gapcurve = P["gapcurveheight"] * math.exp(-_rpow((rcoord - P["rgapd2"]) / P["gapcurvelength"], P["gapcurveexp"]))
    if rcoord < P["rgapd2"]:
        gapcurve = 0.0
    spiral = 1.0
    if P["ispiral"] == 1:
        sfact = 1.0
        for i in range(2, P["sn"] + 1, 2):
            sfact = sfact * float(np.float32(i) / (np.float32(i) - np.float32(1)))
        s = math.sin(math.log(rcoord) / math.tan(P["pitch"]) - phi + float(np.float32(0.7854)))
        spiral = 1.0 - P["sw"] + sfact * P["sw"] * _powi(s, P["sn"])
        if rcoord < P["rspiral1"] or rcoord > P["rspiral2"]:
            spiral = 1.0
    zmr = zscale * (rcoord / rmin) ** bdens
    if phi < PI / 2.0 or phi > 3.0 * PI / 2.0:
        if zp > 0.0:
            zmr = zmr * (1.0 + warp)
        densfact1 = 1.0 / (1.0 + warp)
    else:
        if zp < 0.0:
            zmr = zmr * (1.0 + warp2)
        densfact1 = 1.0 / (1.0 + warp2)
    puff = 1.0 + rimpuff + gappuff - rimcurve - gapcurve
    densfact = 1.0 / puff * densfact1
    zmr = zmr * puff
    if rcoord > P["rmaxd"] or rhodens == 0.0 or rcoord < P["rddust"] or zmr < 1.0e-10:
        return 0.0
    gexp = (zp / zmr) * (zp / zmr)
    if gexp > 1.0e-15:
        if gexp < 120.0:
            dens = densfact * spiral * rhodens * (rcoord / rmin) ** (-adens) * math.exp(-0.5 * gexp)
        else:
            dens = 0.0
    else:
        dens = densfact * spiral * rhodens * (rcoord / rmin) ** (-adens)
    if P["iradexp"] == 1:
        dens = dens * math.exp(-rcoord / P["radexp"])
    return dens


# ---- very small grains and PAHs ---------------------------------------------------
U_NAMES = ("0.50", "1.00", "2.00", "5.00", "10.0", "20.0", "30.0", "1e2", "3e2", "1e3", "3e3", "1e4", "3e4",
           "1e5", "3e5", "1e6", "3e6", "1e7")


def draine_cdf(directory, ndraine: int = 1000):
    """draine_cdf.f90:1-79: (cdf, logcdf) (nemit, ndraine), logfreq (ndraine),
    uratio (nemit) from the emit_draine_<U>.dat files of directory."""
    nemit = len(U_NAMES)
    pdf = np.zeros((nemit, ndraine))
    freq = np.zeros(ndraine)
    for j, name in enumerate(U_NAMES):
        rows = np.loadtxt(f"{directory}/emit_draine_{name}.dat")[:ndraine]
        for i in range(ndraine):
            lam, p = rows[i]
            pdf[j, ndraine - 1 - i] = p
            freq[ndraine - 1 - i] = 1.2398 / lam
    cdf = np.zeros((nemit, ndraine))
    logcdf = np.zeros((nemit, ndraine))
    logfreq = np.zeros(ndraine)
    for j in range(nemit):
        for i in range(1, ndraine):
            cdf[j, i] = cdf[j, i - 1] + 0.5 * (pdf[j, i] + pdf[j, i - 1]) * (freq[i] - freq[i - 1])
        total = cdf[j, ndraine - 1]
        logcdf[j, 0] = -10.0
        for i in range(1, ndraine):
            cdf[j, i] = cdf[j, i] / total
            logcdf[j, i] = math.log10(cdf[j, i])
            logfreq[i] = math.log10(freq[i])
    uratio = np.array([float(np.float32(v)) for v in (0.5, 1.0, 2.0, 5.0, 10.0, 20.0, 30.0, 1e2, 3e2, 1e3, 3e3, 1e4,
                                                        3e4, 1e5, 3e5, 1e6, 3e6, 1e7)])
    return cdf, logcdf, logfreq, uratio


def locate(xx, x) -> int:
    """nr.f:131-150 (1-based result, with the fix-up at the first element)."""
    n = len(xx)
    jl, ju = 0, n + 1
    asc = xx[n - 1] > xx[0]
    while ju - jl > 1:
        jm = (ju + jl) // 2
        if asc == (x > xx[jm - 1]):
            jl = jm
        else:
            ju = jm
    if jl == 0 and x == xx[0]:
        jl = 1
    return jl


def locate3(row, x) -> int:
    """locate3.f90:1-24 on one row of the table (no fix-up at the first element)."""
    n = len(row)
    jl, ju = 0, n + 1
    asc = row[n - 1] > row[0]
    while ju - jl > 1:
        jm = (ju + jl) // 2
        if asc == (x > row[jm - 1]):
            jl = jm
        else:
            ju = jm
    return jl


def rep_draine(cdf, logcdf, logfreq, jmean: int, jmf: float, xran: float) -> float:
    """rep_draine.f90:1-65 (jmean 1-based)."""
    nemit, ndraine = cdf.shape

    def logf(j):
        ifreq = locate3(cdf[j - 1], xran)
        if ifreq == ndraine:
            ifreq = ndraine - 1
        if ifreq == 0:
            ifreq = 1
        return (math.log10(xran) - logcdf[j - 1, ifreq - 1]) / (logcdf[j - 1, ifreq] - logcdf[j - 1, ifreq - 1]) * \
            (logfreq[ifreq] - logfreq[ifreq - 1]) + logfreq[ifreq - 1]

    lf1 = logf(jmean)
    lf = lf1 + jmf * (logf(jmean + 1) - lf1) if jmean + 1 <= nemit else lf1
    return 10.0 ** lf


def int_mean_cell(jmean_cell: float, vcell: float, nphot: float, ltot: float, isrfkap_int: float, uratio):
    """int_mean.f90:30,64-94 for one cell: (imean 1-based, imfract) of the
    mean intensity jmean_cell (the reference's jmean before its normalisation)."""
    nemit = len(uratio)
    jm = jmean_cell / vcell / nphot * ltot
    jratio = jm / isrfkap_int
    im = locate(uratio, jratio)
    if im > nemit:
        im = nemit
    if im < 1:
        im = 1
    if jratio == 0.0:
        f = 0.0
    elif im == nemit:
        f = 1.0
    else:
        jr1, jr2 = math.log10(uratio[im - 1]), math.log10(uratio[im])
        f = (math.log10(jratio) - jr1) / (jr2 - jr1)
    return im, f


def isrf_sg_integral(freq_hz, pdf, kappa_of, kappav: float) -> float:
    """isrf_cdf.f90:191-209: the ISRF pdf weighted by the absorption opacity
    kappa(nu) kappav (1 - albedo(nu)) of the small grains, trapezoid rule;
    kappa_of(nu) returns (kappa, albedo) at nu in units of 1.2398/lambda[um]."""
    s = 0.0
    for i in range(1, len(freq_hz)):
        testnu = 1.2398 / (2.9979e14 / freq_hz[i])
        kap, alb = kappa_of(testnu)
        s = s + 0.5 * (pdf[i] + pdf[i - 1]) * (freq_hz[i] - freq_hz[i - 1]) * kap * kappav * (1.0 - alb)
    return s
