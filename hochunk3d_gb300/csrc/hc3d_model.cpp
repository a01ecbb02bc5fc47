// hc3d_model.cpp -- the Fortran host's setup work, restated in C++:
// reapar/setup (input and units), dustinit/setemiss (opacity and Planck
// tables), atmosinit (stellar spectrum CDF), setup_wave (disk rho0) and
// gridset (walls, cell volumes, densities).  Each function cites the
// reference lines it follows.
#include "hc3d_model.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <thread>

namespace hc3d {

// ---------------------------------------------------------------------------
// configuration.f90:28-56 -- value = NAME = comment; the value is the text
// before the first '=', the name the trimmed text between the first two.
// ---------------------------------------------------------------------------
static std::string trim(const std::string& s) {
  size_t b = s.find_first_not_of(" \t\r\n");
  if (b == std::string::npos) return "";
  size_t e = s.find_last_not_of(" \t\r\n");
  return s.substr(b, e - b + 1);
}

bool ParFile::load(const std::string& path, std::string* err) {
  std::ifstream f(path);
  if (!f) {
    *err = "cannot open parameter file " + path;
    return false;
  }
  std::string line;
  while (std::getline(f, line)) {
    size_t p1 = line.find('=');
    if (p1 == std::string::npos) continue;
    size_t p2 = line.find('=', p1 + 1);
    if (p2 == std::string::npos) continue;
    std::string value = trim(line.substr(0, p1));
    std::string name = trim(line.substr(p1 + 1, p2 - p1 - 1));
    kv_[name] = value;  // later duplicates win, like the Fortran key() scan order
  }
  return true;
}

// Fortran list-directed read of the first item: quotes stripped, stops at
// blank or comma.
static std::string first_item(const std::string& v) {
  std::string s = trim(v);
  if (!s.empty() && (s[0] == '\'' || s[0] == '"')) {
    char q = s[0];
    size_t e = s.find(q, 1);
    return e == std::string::npos ? s.substr(1) : s.substr(1, e - 1);
  }
  size_t e = s.find_first_of(" \t,");
  return e == std::string::npos ? s : s.substr(0, e);
}

static bool parse_real(const std::string& tok, double* out) {
  std::string t = tok;
  for (auto& ch : t)
    if (ch == 'd' || ch == 'D') ch = 'e';
  char* end = nullptr;
  errno = 0;
  double v = std::strtod(t.c_str(), &end);
  if (end == t.c_str() || errno != 0) return false;
  *out = v;
  return true;
}

bool ParFile::str(const std::string& key, std::string* out, std::string* err) const {
  auto it = kv_.find(key);
  if (it == kv_.end()) {
    *err = "ERROR: parameter " + key + " not found";
    return false;
  }
  *out = first_item(it->second);
  return true;
}

bool ParFile::real(const std::string& key, double* out, std::string* err) const {
  std::string s;
  if (!str(key, &s, err)) return false;
  if (!parse_real(s, out)) {
    *err = "Parameter " + key + " is not a real";
    return false;
  }
  return true;
}

bool ParFile::integer(const std::string& key, int64_t* out, std::string* err) const {
  std::string s;
  if (!str(key, &s, err)) return false;
  if (s == "YES") { *out = 1; return true; }
  if (s == "NO") { *out = 0; return true; }
  double v;
  if (!parse_real(s, &v)) {
    *err = "Parameter " + key + " is not an integer";
    return false;
  }
  *out = (int64_t)v;
  return true;
}

bool ParFile::reals(const std::string& key, std::vector<double>* out, std::string* err) const {
  auto it = kv_.find(key);
  if (it == kv_.end()) {
    *err = "ERROR: parameter " + key + " not found";
    return false;
  }
  out->clear();
  std::string s = it->second;
  for (auto& ch : s)
    if (ch == ',') ch = ' ';
  std::istringstream is(s);
  std::string tok;
  while (is >> tok) {
    double v;
    if (!parse_real(tok, &v)) {
      *err = "Parameter " + key + " is not a list of reals";
      return false;
    }
    out->push_back(v);
  }
  return true;
}

bool ParFile::ints(const std::string& key, std::vector<int64_t>* out, std::string* err) const {
  std::vector<double> v;
  if (!reals(key, &v, err)) return false;
  out->clear();
  for (double x : v) out->push_back((int64_t)x);
  return true;
}

// ---------------------------------------------------------------------------
// mathsubs.f90: expm1 (Abramowitz & Stegun 4.2.45 polynomial) and the
// normalised Planck function Bnu.
// ---------------------------------------------------------------------------
static double expm1_as(double x) {
  static const double coef[7] = {0.9999999995, 0.4999999206, 0.1666653019, 0.0416573475,
                                 0.0083013598, 0.0013298820, 0.0001413161};
  if (std::fabs(x) > 0.6931472) return std::exp(x) - 1.0;
  double sum = 0.0;
  for (int i = 6; i >= 0; --i) sum = x * (coef[i] + sum);
  return sum;
}

static double Bnu(double nu, double T) {
  const double norm = 0.1539897;  // 15/pi^4
  double x = nu / T;
  if (x == 0.0) return 0.0;
  return norm * x * x * x / expm1_as(x);
}

// ---------------------------------------------------------------------------
// opacset for one species (dust.f90:9-80), host copy used by setemiss.
// ---------------------------------------------------------------------------
static void opacset1(const Model& m, int id, double nu, double* kappa, double* albedo) {
  const int nl = m.nlambda[id];
  const double* nud = &m.nudust[(size_t)id * m.nlammax];
  const double* kap = &m.kappad[(size_t)id * m.nlammax];
  const double* alb = &m.adust[(size_t)id * m.nlammax];
  if (nu >= nud[0]) {
    *kappa = kap[0];
    *albedo = alb[0];
  } else if (nu <= nud[nl - 1]) {
    *kappa = kap[nl - 1];
    *albedo = alb[nl - 1];
  } else {
    int i0 = 1, i1 = nl;
    while (i1 - i0 > 1) {
      int i = (i1 + i0) / 2;
      if (nu <= nud[i - 1]) i0 = i; else i1 = i;
    }
    double f = (nu - nud[i1 - 1]) / (nud[i0 - 1] - nud[i1 - 1]);
    double fm1 = 1.0 - f;
    *kappa = fm1 * kap[i1 - 1] + f * kap[i0 - 1];
    *albedo = fm1 * alb[i1 - 1] + f * alb[i0 - 1];
  }
}

// nr.f qsimp/trapzd (nr.f:183-225); returns the last estimate instead of
// stopping when JMAX is reached.
template <class F>
static double qsimp(F func, double a, double b) {
  const double EPS = 1.e-5;
  const int JMAX = 20;
  double ost = -1.e30, os = -1.e30, st = 0.0, s = 0.0;
  for (int j = 1; j <= JMAX; ++j) {
    if (j == 1) {
      st = 0.5 * (b - a) * (func(a) + func(b));
    } else {
      int it = 1 << (j - 2);
      double tnm = (double)it, del = (b - a) / tnm, x = a + 0.5 * del, sum = 0.0;
      for (int k = 0; k < it; ++k) {
        sum += func(x);
        x += del;
      }
      st = 0.5 * (st + (b - a) * sum / tnm);
    }
    s = (4.0 * st - ost) / 3.0;
    if (std::fabs(s - os) < EPS * std::fabs(os)) return s;
    os = s;
    ost = st;
  }
  return s;
}

// setemiss, dust.f90:394-474: cumulative kappa*B_nu integrals over the
// nuint grid (scaled by T) for every temperature; kapBint normalised to 1 at
// nnu and kappap = the unnormalised total (Planck-mean kappa / kappa_V).
void setemiss_species(const Model& m, int id, double* kapB, double* kapp) {
  const int nT = m.nT, nnu = m.nnu;
  auto rows = [&](int i_begin, int i_end) {
    for (int i = i_begin; i < i_end; ++i) {
      const double Teff = std::exp(m.lTint[i]);
      double nu1 = 0.0, kappa, albedo;
      opacset1(m, id, nu1, &kappa, &albedo);
      double kappa1 = (1.0 - albedo) * kappa;
      double acc = 0.0;
      for (int j = 0; j < nnu; ++j) {
        double nu0 = nu1;
        nu1 = m.nuint[j] * Teff;
        double dnu = nu1 - nu0;
        double dx = dnu / Teff;
        double kappa0 = kappa1;
        opacset1(m, id, nu1, &kappa, &albedo);
        kappa1 = (1.0 - albedo) * kappa;
        double v = 0.0;
        if (nu0 / Teff < 50.0) {
          v = qsimp([&](double f) { return ((1.0 - f) * kappa0 + f * kappa1) * Bnu(nu0 + f * dnu, Teff); }, 0.0,
                    1.0);
        }
        acc = (j == 0) ? dx * v : dx * v + acc;
        kapB[(size_t)i + (size_t)nT * j] = acc;
      }
      kapp[i] = kapB[(size_t)i + (size_t)nT * (nnu - 1)];
      for (int j = 0; j < nnu - 1; ++j) kapB[(size_t)i + (size_t)nT * j] /= kapp[i];
      kapB[(size_t)i + (size_t)nT * (nnu - 1)] = 1.0;
    }
  };
  unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (unsigned k = 0; k < nth; ++k) th.emplace_back(rows, (int)(nT * k / nth), (int)(nT * (k + 1) / nth));
  for (auto& t : th) t.join();
}

// ---------------------------------------------------------------------------
// dustinit, dust.f90:314-391: 7-column file lam(um) cext csca kap g pmax thet
// ---------------------------------------------------------------------------
static bool read_dust(Model* m, int id, const std::string& path, std::string* err) {
  std::ifstream f(path);
  if (!f) {
    *err = "cannot open dust file " + path;
    return false;
  }
  int i = 0, iv = 0;
  std::string line;
  const size_t o = (size_t)id * m->nlammax;
  while (std::getline(f, line)) {
    std::istringstream is(line);
    double lam, cext, csca, kap, hgg, pmax, thet;
    if (!(is >> lam >> cext >> csca >> kap >> hgg >> pmax >> thet)) {
      if (trim(line).empty()) continue;
      break;
    }
    if (i >= m->nlammax) {
      *err = "error, too many wavelengths in dust opacity file";
      return false;
    }
    if (lam <= 0.55) iv = i + 1;
    m->lamdust[o + i] = 10000.0 * lam;
    m->nudust[o + i] = 12398.0 / m->lamdust[o + i];
    m->kappad[o + i] = kap;
    m->adust[o + i] = csca / cext;
    m->gdust[o + i] = hgg;
    m->pldust[o + i] = pmax;
    if (i == 0) m->kappad[o + i] = 0.00001 * m->kappad[o + i];
    ++i;
  }
  if (i < 2 || iv < 1 || iv >= i) {
    *err = "dust file " + path + " has too few rows or no row at 0.55um";
    return false;
  }
  m->nlambda[id] = i;
  double f5 = (5500.0 - m->lamdust[o + iv - 1]) / (m->lamdust[o + iv] - m->lamdust[o + iv - 1]);
  m->kappav[id] = (1.0 - f5) * m->kappad[o + iv - 1] + f5 * m->kappad[o + iv];
  for (int k = 0; k < i; ++k) m->kappad[o + k] /= m->kappav[id];
  return true;
}

// atmosinit, starbarb.f90:3-110 (the parts the photon loop reads).
static bool atmosinit(Model* m, const std::string& path, std::string* err) {
  std::ifstream f(path);
  if (!f) {
    *err = "cannot open atmosphere file " + path;
    return false;
  }
  std::string line;
  std::getline(f, line);  // header
  std::vector<double> w, fl;
  while (std::getline(f, line)) {
    std::istringstream is(line);
    double wtmp, ftmp;
    if (!(is >> wtmp >> ftmp)) break;
    if (m->iplanckst == 1) ftmp = Bnu(1.2398 / wtmp, m->tstar_k / 11605.0);
    w.push_back(wtmp);
    fl.push_back(ftmp);
  }
  const int nh = (int)w.size();
  if (nh < 3) {
    *err = "atmosphere file has fewer than 3 samples";
    return false;
  }
  std::vector<double> winv(nh), ff(nh);
  for (int i = 0; i < nh; ++i) {
    winv[nh - 1 - i] = 1.0 / w[i];
    ff[nh - 1 - i] = fl[i];
  }
  m->hnuint.assign(nh, 0.0);
  m->atmosnu.assign(nh, 0.0);
  m->lognu.assign(nh, 0.0);
  m->loghnu.assign(nh, 0.0);
  for (int i = 0; i < nh; ++i) {
    m->atmosnu[i] = 1.2398 * winv[i];
    m->lognu[i] = std::log10(m->atmosnu[i]);
    m->hnuint[i] = i == 0 ? 0.0 : m->hnuint[i - 1] + 0.5 * (ff[i] + ff[i - 1]) * (winv[i] - winv[i - 1]);
  }
  double fbol = m->hnuint[nh - 1];
  if (fbol == 0.0) {
    *err = "error, atmosphere file is all zeros";
    return false;
  }
  for (int i = 0; i < nh; ++i) {
    m->hnuint[i] /= fbol;
    if (i > 0) m->loghnu[i] = std::log10(m->hnuint[i]);
  }
  return true;
}

// ---------------------------------------------------------------------------
// zerod (module not shipped): root mu0 in [mu,1] of the Ulrich streamline
// equation mu0^3 + (r/Rc - 1) mu0 - (r/Rc) mu = 0 (Ulrich 1976), by the
// closed form of the depressed cubic, polished by Newton steps.
// ---------------------------------------------------------------------------
double zerod(double mu, double rx) {
  const double p = rx - 1.0, q = -rx * mu;
  double x;
  double disc = 0.25 * q * q + p * p * p / 27.0;
  if (disc > 0.0) {
    double sd = std::sqrt(disc);
    x = std::cbrt(-0.5 * q + sd) + std::cbrt(-0.5 * q - sd);
  } else if (p < 0.0) {
    double r = std::sqrt(-p / 3.0);
    double arg = std::max(-1.0, std::min(1.0, (3.0 * q) / (2.0 * p) * std::sqrt(-3.0 / p)));
    x = 2.0 * r * std::cos(std::acos(arg) / 3.0);  // the largest real root
  } else {
    x = 0.0;
  }
  for (int k = 0; k < 3; ++k) {
    double fx = x * x * x + p * x + q, d = 3.0 * x * x + p;
    if (d != 0.0) x -= fx / d;
  }
  return std::max(0.0, std::min(1.0, x));
}

// densdisk, densdiskg.f90:1-155: the flared disk with its gap, spiral arms,
// warp, rim and gap puffs and curves and radial cutoff, at azimuth phi.
// x**n for an integer n as the Fortran runtime forms it: a product by
// repeated squaring (the reciprocal for n < 0)
static double powi(double x, int n) {
  double r = 1.0;
  unsigned u = n < 0 ? (unsigned)(-n) : (unsigned)n;
  while (u) {
    if (u & 1u) r *= x;
    u >>= 1;
    if (u) x *= x;
  }
  return n < 0 ? 1.0 / r : r;
}

double densdisk(const Model& m, double rad, double sint, double cost, double phi, int id) {
  const double rp = rad * sint, zp = rad * cost;
  const double rcoord = m.idiskcurve == 1 ? rad : rp;
  const double rmin = 1.0;
  // inside the gap the gap's density law (densdiskg.f90:34-44)
  const bool ingap = m.igapd == 1 && rcoord < m.rgapd2 && rcoord > m.rgapd1;
  const double adens = ingap ? m.agap[id] : m.a[id], bdens = ingap ? m.bgap[id] : m.b[id];
  const double rhodens = ingap ? m.rhogap0[id] : m.rho0[id], zscale = ingap ? m.z1gap[id] : m.z1[id];
  // warp of spot longitudes 0 and 180 deg (densdiskg.f90:46-68)
  double warp = 0.0, warp2 = 0.0;
  if (m.idiskwarp == 1) {
    const double fall = std::exp(-std::pow((rcoord - m.rddust[id]) / m.warplength, 2.0));
    warp = (phi < kPi ? 1.0 : -1.0) * m.warpheight * std::pow(std::cos(phi / 2.0), m.wexp) * fall;
    if (m.nspot == 2) warp2 = m.warpheight * std::pow(std::cos(phi / 2.0 - kPi / 2.0), m.wexp) * fall;
  }
  double rimcurve = 0.0, rimpuff = 0.0, gappuff = 0.0, gapcurve = 0.0;
  if (m.irimcurve == 1)
    rimcurve = m.rimcurveheight * std::exp(-std::pow((rcoord - m.rddust[id]) / m.rimcurvelength, m.rimcurveexp));
  if (m.irimpuff == 1) rimpuff = m.rimheight * std::exp(-std::pow((rcoord - m.rddust[id]) / m.rimlength, 2.0));
  if (rcoord < m.rddust[id]) rimpuff = 0.0;
  if (m.igappuff == 1 && m.igapd == 1) gappuff = m.gapheight * std::exp(-std::pow((rcoord - m.rgapd2) / m.gaplength, 2.0));
  if (rcoord < m.rgapd2) gappuff = 0.0;
  if (m.igapcurve == 1 && m.igapd == 1)
    gapcurve = m.gapcurveheight * std::exp(-std::pow((rcoord - m.rgapd2) / m.gapcurvelength, m.gapcurveexp));
  if (rcoord < m.rgapd2) gapcurve = 0.0;
  // spiral arms (densdiskg.f90:101-112): SN-th power of a logarithmic spiral,
  // normalised by the product of is/(is-1) over even is
  double spiral = 1.0;
  if (m.ispiral == 1) {
    // the factors real(is)/(real(is)-1) and the phase 0.7854 are default
    // (single precision) reals in the Fortran; the integer power is a
    // product by squaring, as the Fortran runtime forms x**n
    double sfact = 1.0;
    for (int is = 2; is <= m.sn; is += 2) sfact = sfact * (double)((float)is / ((float)is - 1.0f));
    spiral = 1.0 - m.sw +
             sfact * m.sw * powi(std::sin(std::log(rcoord) / std::tan(m.pitch) - phi + (double)0.7854f), m.sn);
    if (rcoord < m.rspiral1 || rcoord > m.rspiral2) spiral = 1.0;
  }
  double zmr = zscale * std::pow(rcoord / rmin, bdens);
  double densfact1 = 1.0;
  if (phi < kPi / 2.0 || phi > 3.0 * kPi / 2.0) {
    if (zp > 0.0) zmr = zmr * (1.0 + warp);  // the warp lifts the +z side of spot 1 only
    densfact1 = 1.0 / (1.0 + warp);
  } else {
    if (zp < 0.0) zmr = zmr * (1.0 + warp2);
    densfact1 = 1.0 / (1.0 + warp2);
  }
  const double puff = 1.0 + rimpuff + gappuff - rimcurve - gapcurve;
  const double densfact = 1.0 / puff * densfact1;
  zmr = zmr * puff;
  if (rcoord > m.rmaxd[id] || rhodens == 0.0 || rcoord < m.rddust[id] || zmr < 1.e-10) return 0.0;
  const double gexp = (zp / zmr) * (zp / zmr);
  double dens;
  if (gexp > 1.e-15) {
    if (gexp < 120.0) dens = densfact * spiral * rhodens * std::pow(rcoord / rmin, -adens) * std::exp(-0.5 * gexp);
    else dens = 0.0;
  } else {
    dens = densfact * spiral * rhodens * std::pow(rcoord / rmin, -adens);
  }
  if (m.iradexp == 1) dens = dens * std::exp(-rcoord / m.radexp);
  return dens;
}

// densenv, densenv.f90:1-128: Ulrich envelope (or power law) with a
// polynomial bipolar cavity and an optional gap; species id is the envelope
// (slot 3) or cavity (slot 4).
double densenv(const Model& m, double rad, double thetin, double costin, double sina, int id) {
  const bool is_env = (id == 2 || id == 6), is_cav = (id == 3 || id == 7);
  int inhole = 0;
  double thet = thetin;
  double cosa = std::fabs(costin);
  if (thet > kPiHalf) thet = kPi - thet;
  (void)thet;
  const double rp = rad * sina, zp = rad * cosa;
  const double zup = m.c1e * std::pow(rp, m.ex1) + m.z01;
  const double xmu = zp / rad;
  double dens;
  if (rad > m.rmine) {
    if (m.ienvtype == 1) {
      double rx = rad / m.rc;
      double xmu0 = zerod(xmu, rx);
      double ratio = xmu0 > 0.0 ? xmu / xmu0 : 1.0;
      double factor = 1.0 / (ratio + 2.0 * (xmu0 * xmu0) / rx);
      dens = m.rhoe0 * std::pow(rx, -1.5) * factor / std::sqrt(1.0 + ratio);
    } else {
      dens = m.rhodens1 * std::pow(rad, -m.envexp);  // densenvpw.f90
    }
  } else {
    dens = 0.0;
  }
  // constant density in the envelope gap, before the ambient floor and the cavity
  const bool ingape = m.igape == 1 && rad < m.rgape2 && rad > m.rgape1;
  if (ingape && m.igapedens == 0) dens = m.rhogape;
  if (rad > m.rmine && dens < m.rhoamb) dens = m.rhoamb;
  if (m.ihole == 1 && m.ipoly == 1) {
    double zlo = m.c2e * std::pow(rp, m.ex2) + m.z02;
    if (zp > zlo) {
      inhole = 1;
      dens = m.rhoconst2 * std::pow(rad, -m.exf);
    }
    if (zp > zup) {
      inhole = 1;
      dens = m.rhoconst1 * std::pow(rad, -m.exf);
    }
  }
  if (ingape && m.igapedens == 1) dens = dens * m.fracte;  // scaled density in the gap
  if (rad >= m.rmax) dens = 0.0;
  if (rad <= m.rmine) dens = 0.0;
  if (is_cav && inhole == 0) dens = 0.0;
  if (is_env && inhole == 1) dens = 0.0;
  return dens;
}


// ---------------------------------------------------------------------------
// reapar + setup: read the keys the photon loop depends on and convert units
// (reapar.f90:32-535, setup.f90:26-231).
// ---------------------------------------------------------------------------
#define REQ(call) \
  do {            \
    if (!(call)) return false; \
  } while (0)

// isrf_cdf (isrf_cdf.f90:1-243): the external radiation field on 200
// log-spaced wavelengths inside the table's range (clamped to 0.05-5000 um),
// log-log interpolated, reddened by ISRF_AV magnitudes of the extinction law
// r400_ice095.par (read only when ISRF_AV is not zero), integrated by the
// trapezoid rule in frequency, normalised, and the frequencies converted to
// units of 1.2398/lambda[um].  Row 1 keeps its frequency in Hz with
// logcdf = -99 and logfreq = 0, as the Fortran leaves them.
static bool isrf_cdf(Model* m, std::string* err) {
  const double c = 2.99792458e14;  // um Hz
  std::vector<double> lnu, nufnu;
  {
    FILE* f = std::fopen(m->isrf_file.c_str(), "r");
    if (!f) { *err = "cannot open ISRF_FILE " + m->isrf_file; return false; }
    char line[512];
    while (std::fgets(line, sizeof line, f)) {
      double a, b;
      if (line[0] == '#') continue;
      if (std::sscanf(line, "%lf %lf", &a, &b) == 2) { lnu.push_back(a); nufnu.push_back(b); }
    }
    std::fclose(f);
  }
  const int nin = (int)lnu.size();
  if (nin < 2) { *err = "ISRF_FILE " + m->isrf_file + " has fewer than two rows"; return false; }
  for (int i = 1; i < nin; ++i)
    if (!(lnu[i] > lnu[i - 1])) { *err = "ISRF_FILE frequencies must increase"; return false; }
  std::vector<double> freqin(nin), logfreqin(nin), logpdfin(nin);
  for (int i = 0; i < nin; ++i) {
    freqin[i] = std::pow(10.0, lnu[i]);
    const double pdf = std::pow(10.0, nufnu[i]) / freqin[i];
    logfreqin[i] = std::log10(freqin[i]);
    logpdfin[i] = std::log10(pdf);
  }
  double lmin = c / (freqin[nin - 1] * 0.99999999), lmax = c / (freqin[0] * 1.0000001);
  if (lmin < 0.05) lmin = 0.05;
  if (lmax > 5000.0) lmax = 5000.0;
  const int n = kNisrf;
  std::vector<double> freq(n), pdf(n), cdf(n), logcdf(n), logfreq(n);
  for (int i = 1; i <= n; ++i) {
    const double lam = lmin * std::pow(lmax / lmin, (double)i / (double)n);
    freq[n - i] = c / lam;
  }
  // extinction law: columns lam, -, -, kappa (isrf_cdf.f90:120-134)
  std::vector<double> fext, kext;
  double kapvext = 1.0;
  if (m->isrf_av != 0.0) {
    const std::string path = m->pardir + "/r400_ice095.par";
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) { *err = "ISRF_AV is not zero and the extinction law " + path + " cannot be opened"; return false; }
    char line[512];
    while (std::fgets(line, sizeof line, f)) {
      double lam, j1, j2, kap;
      if (std::sscanf(line, "%lf %lf %lf %lf", &lam, &j1, &j2, &kap) == 4) { fext.push_back(c / lam); kext.push_back(kap); }
    }
    std::fclose(f);
    if (fext.size() < 2) { *err = "extinction law " + path + " has fewer than two rows"; return false; }
    std::reverse(fext.begin(), fext.end());
    std::reverse(kext.begin(), kext.end());
  }
  auto locate = [](const std::vector<double>& xx, int nn, double x) {  // nr.f locate2 on xx[0..nn)
    int jl = 0, ju = nn + 1;
    const bool asc = xx[nn - 1] > xx[0];
    while (ju - jl > 1) {
      const int jm = (ju + jl) / 2;
      if (asc == (x > xx[jm - 1])) jl = jm; else ju = jm;
    }
    return jl;
  };
  const int next = (int)fext.size();
  if (next >= 2) {
    const double fv = c / 0.55;
    const int j = locate(fext, next, fv);
    if (j < 1 || j >= next) { *err = "extinction law does not cover 0.55 um"; return false; }
    kapvext = kext[j - 1] + (fv - fext[j - 1]) / (fext[j] - fext[j - 1]) * (kext[j] - kext[j - 1]);
  }
  for (int i = 0; i < n; ++i) {
    const double fq = freq[i];
    double ext = 1.0;
    if (next >= 2) {
      int j = locate(fext, next, fq);
      if (j == 0 && fq == fext[0]) j = 1;
      double kt;
      if (j == next) kt = kext[next - 1];
      else if (j == 0) kt = kext[0];
      else kt = kext[j - 1] + (fq - fext[j - 1]) / (fext[j] - fext[j - 1]) * (kext[j] - kext[j - 1]);
      ext = std::exp(-kt / kapvext / 1.086 * m->isrf_av);
    }
    int j = locate(freqin, nin, fq);
    if (j < 1) j = 1;
    if (j > nin - 1) j = nin - 1;
    const double lp = logpdfin[j - 1] + (std::log10(fq) - logfreqin[j - 1]) / (logfreqin[j] - logfreqin[j - 1]) *
                                            (logpdfin[j] - logpdfin[j - 1]);
    pdf[i] = std::pow(10.0, lp) * ext;
  }
  cdf[0] = 0.0;
  for (int i = 1; i < n; ++i) cdf[i] = cdf[i - 1] + 0.5 * (pdf[i] + pdf[i - 1]) * (freq[i] - freq[i - 1]);
  m->isrf_pdf = pdf;
  m->isrf_fhz = freq;
  m->isrf_int = cdf[n - 1];
  if (!(m->isrf_int > 0.0)) { *err = "ISRF_FILE integrates to zero"; return false; }
  cdf[0] = 0.0;
  logcdf[0] = -99.0;
  logfreq[0] = 0.0;
  for (int i = 1; i < n; ++i) {
    cdf[i] = cdf[i] / cdf[n - 1];
    logcdf[i] = std::log10(cdf[i]);
    freq[i] = freq[i] * 1.2398 / c;
    logfreq[i] = std::log10(freq[i]);
  }
  m->isrf_cdfv = cdf;
  m->isrf_logcdf = logcdf;
  m->isrf_logfreq = logfreq;
  return true;
}

// The ISRF weighted by the absorption opacity of the small grains, the unit
// of the mean-intensity ratio of int_mean (isrf_cdf.f90:199-209): the
// trapezoid sum of pdf(nu) kappa(nu) kappa_V (1 - albedo(nu)) over the
// field's rows, the opacity at 1.2398 / (2.9979e14 / nu).  The reference
// takes species 5's dust; here it is the small-grain species of the first
// device slot that holds one (sg_slot), whose opacity also weights the
// device's path tally, so that the ratio is formed from one dust file.  The
// two agree whenever that species reads species 5's file.
static void sg_isrf_weight(Model* m) {
  m->sg_slot = -1;
  for (int s = 0; s < 4 && m->sg_slot < 0; ++s)
    if (m->slot_species[s] >= 5) m->sg_slot = s;
  m->isrfkap_int = 0.0;
  if (m->sg_slot < 0) return;
  const int id = m->slot_species[m->sg_slot] - 1;
  const std::vector<double>& pdf = m->isrf_pdf;
  const std::vector<double>& freq = m->isrf_fhz;
  for (size_t i = 1; i < freq.size(); ++i) {
    const double testnu = 1.2398 / (2.9979e14 / freq[i]);
    double kappa, albedo;
    opacset1(*m, id, testnu, &kappa, &albedo);
    m->isrfkap_int += 0.5 * (pdf[i] + pdf[i - 1]) * (freq[i] - freq[i - 1]) * kappa * m->kappav[id] * (1.0 - albedo);
  }
}

// draine_cdf (draine_cdf.f90:1-79): the small grains' emission spectra for
// 18 ratios U of the mean intensity to the ISRF's, each 1000 rows
// (lambda [um], j_nu) read from emit_draine_<U>.dat in PARDIR, reordered to
// increasing frequency 1.2398/lambda, integrated by the trapezoid rule and
// normalised; row 1 keeps logcdf = -10 and logfreq = 0, as the Fortran sets
// them.
static bool draine_cdf(Model* m, std::string* err) {
  static const char* const names[kNemit] = {"0.50", "1.00", "2.00", "5.00", "10.0", "20.0", "30.0", "1e2", "3e2",
                                            "1e3",  "3e3",  "1e4",  "3e4",  "1e5",  "3e5",  "1e6",  "3e6", "1e7"};
  static const float uratio[kNemit] = {0.5f, 1.0f,  2.0f,  5.0f,  10.0f, 20.0f, 30.0f, 1.e2f, 3.e2f,
                                       1.e3f, 3.e3f, 1.e4f, 3.e4f, 1.e5f, 3.e5f, 1.e6f, 3.e6f, 1.e7f};
  const int nd = kNdraine;
  std::vector<double> pdf((size_t)kNemit * nd), freq(nd);
  for (int j = 0; j < kNemit; ++j) {
    const std::string path = m->pardir + "/emit_draine_" + names[j] + ".dat";
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) { *err = "FSG > 0: cannot open the small-grain emission spectrum " + path; return false; }
    for (int i = 0; i < nd; ++i) {
      double lam, p;
      if (std::fscanf(f, "%lf %lf", &lam, &p) != 2 || !(lam > 0.0)) {
        std::fclose(f);
        *err = path + " holds fewer than 1000 rows of lambda [um] and j_nu";
        return false;
      }
      pdf[(size_t)j * nd + (nd - 1 - i)] = p;
      freq[nd - 1 - i] = 1.2398 / lam;
    }
    std::fclose(f);
  }
  for (int i = 1; i < nd; ++i)
    if (!(freq[i] > freq[i - 1])) { *err = "emit_draine_*.dat: wavelengths must increase down the file"; return false; }
  m->sg_logcdf.assign((size_t)kNemit * nd, 0.0);
  m->sg_cdf.assign((size_t)kNemit * nd, 0.0);
  m->sg_logfreq.assign(nd, 0.0);
  m->sg_uratio.assign(kNemit, 0.0);
  std::vector<double> cdf(nd);
  for (int j = 0; j < kNemit; ++j) {
    const double* pj = &pdf[(size_t)j * nd];
    cdf[0] = 0.0;
    for (int i = 1; i < nd; ++i) cdf[i] = cdf[i - 1] + 0.5 * (pj[i] + pj[i - 1]) * (freq[i] - freq[i - 1]);
    if (!(cdf[nd - 1] > 0.0)) { *err = std::string("emit_draine_") + names[j] + ".dat integrates to zero"; return false; }
    // cdf_d and logcdf_d (nemit, ndraine), Fortran order: spectrum j, frequency i at j + nemit i
    m->sg_logcdf[(size_t)j] = -10.0;
    m->sg_cdf[(size_t)j] = 0.0;
    for (int i = 1; i < nd; ++i) {
      const double v = cdf[i] / cdf[nd - 1];
      m->sg_cdf[(size_t)j + (size_t)kNemit * i] = v;
      m->sg_logcdf[(size_t)j + (size_t)kNemit * i] = std::log10(v);
    }
    m->sg_uratio[j] = (double)uratio[j];
  }
  m->sg_logfreq[0] = 0.0;
  for (int i = 1; i < nd; ++i) m->sg_logfreq[i] = std::log10(freq[i]);
  return true;
}

static bool read_par(Model* m, const ParFile& P, const std::string* par_dir, std::string* err) {
  int64_t iv;
  std::string sv;
  REQ(P.integer("NP", &m->np, err));
  REQ(P.integer("NPMIN", &m->npmin, err));
  REQ(P.integer("NIMIN", &iv, err)); m->nimin = (int)iv;
  REQ(P.integer("NIMAX", &iv, err)); m->nimax = (int)iv;
  REQ(P.integer("CPEEL", &iv, err)); m->ipeel = (int)iv;
  REQ(P.integer("CLUCY", &iv, err)); m->ilucy = (int)iv;
  if (m->ilucy != 1) { *err = "CLUCY=NO (Bjorkman & Wood temperatures) is not supported; use CLUCY=YES"; return false; }
  if (P.has("SEED")) { REQ(P.integer("SEED", &iv, err)); m->seed = (uint64_t)iv; }
  else { REQ(P.integer("I1", &iv, err)); m->seed = (uint64_t)(iv < 0 ? -iv : iv); }
  REQ(P.str("PARDIR", &m->pardir, err));
  if (par_dir) m->pardir = *par_dir;
  REQ(P.integer("COUTILLUM", &iv, err)); m->iout = (int)iv;
  if (m->iout) {
    REQ(P.real("ISRF_SCL", &m->isrf_scl, err));
    REQ(P.real("ISRF_AV", &m->isrf_av, err));
    if (!P.has("ISRF_FILE")) {
      *err = "COUTILLUM=YES needs ISRF_FILE (the external radiation field, log10 nu and log10 nu*F_nu per line)";
      return false;
    }
    REQ(P.str("ISRF_FILE", &sv, err)); m->isrf_file = m->pardir + "/" + sv;
  }
  REQ(P.integer("CLIMB", &iv, err)); m->limb = (int)iv;
  if (m->limb) {
    // table (samptabl.f90:1-23): xmu(1) = 0, xmu(i) = i/ntab, prob(i) = 0.5 (mu^3 + mu^2), prob(1) = 0
    const double delmu = 1.0 / (double)kNtab;
    m->limb_xmu.assign(kNtab, 0.0);
    m->limb_prob.assign(kNtab, 0.0);
    for (int i = 2; i <= kNtab; ++i) {
      const double x = delmu * (double)i;
      m->limb_xmu[i - 1] = x;
      m->limb_prob[i - 1] = 0.5 * (std::pow(x, 3.0) + std::pow(x, 2.0));
    }
  }
  REQ(P.integer("CPLANCKST", &iv, err)); m->iplanckst = (int)iv;
  REQ(P.str("ATNAME", &sv, err)); m->atname = m->pardir + "/" + sv;
  REQ(P.real("RSTAR", &m->rstar, err));
  REQ(P.real("TSTAR", &m->tstar_k, err));
  REQ(P.real("MASSC", &m->massc, err));
  // hot spots (reapar.f90:288-305); the spot radius and temperature follow from the accretion shock in gridset
  // (reapar reads these keys whether or not CSPOT is set; the shock of CDISKACC uses NSPOT, CTEMP and
  // TSPOT/FSPOT without spots too)
  REQ(P.integer("CSPOT", &iv, err)); m->ispot = (int)iv;
  if (P.has("SPOTLAT")) REQ(P.real("SPOTLAT", &m->spotlat, err));
  if (P.has("NSPOT")) { REQ(P.integer("NSPOT", &iv, err)); m->nspot = (int)iv; }
  if (P.has("CTEMP")) { REQ(P.integer("CTEMP", &iv, err)); m->itemp = (int)iv; }
  if (P.has("TSPOT/FSPOT")) REQ(P.real("TSPOT/FSPOT", m->itemp ? &m->tspot : &m->fspot, err));
  if (!m->ispot) m->fspot = 1.0;  // reapar.f90:302-305
  REQ(P.real("MASSD", &m->massd, err));
  REQ(P.str("CRMIN", &sv, err));
  const int irminsub = sv == "RSTAR" ? 0 : sv == "RSUB" ? 1 : sv == "AU" ? 2 : -1;
  if (irminsub < 0) { *err = "CRMIN should be one of RSTAR/RSUB/AU"; return false; }
  m->irminsub = irminsub;
  std::string czmin;
  REQ(P.str("CZMIN", &czmin, err));
  double fmassd1;
  REQ(P.real("FMASSD1", &fmassd1, err));
  if (P.has("CDISKCURV")) { REQ(P.str("CDISKCURV", &sv, err)); m->idiskcurve = sv == "SPH" ? 1 : 0; }
  // disk accretion (reapar.f90:275-284); RTRUNC is read whether or not it is used
  if (P.has("CDISKACC")) { REQ(P.integer("CDISKACC", &iv, err)); m->idiskacc = (int)iv; }
  if (m->idiskacc) {
    REQ(P.integer("CALPHA", &iv, err)); m->ialpha = (int)iv;
    REQ(P.real("ALPHA/MDOT", m->ialpha ? &m->alphad : &m->mdotdisk, err));
  }
  if (P.has("RTRUNC")) REQ(P.real("RTRUNC", &m->rtrunc, err));
  if (m->ispot && !m->idiskacc) {
    // the spot temperature exists only through the accretion shock luminosity (gridset.f90:169-178):
    // the reference would emit the spot's packets at T = 0
    *err = "CSPOT=YES needs CDISKACC=YES: the hot-spot temperature comes from the accretion shock";
    return false;
  }
  if (m->idiskacc && m->nspot != 1 && m->nspot != 2) { *err = "NSPOT must be 1 or 2"; return false; }
  if (m->idiskacc && m->itemp == 0 && m->fspot == 0.0) {
    *err = "ERROR: fspot=0 and CDISKACC=yes - 0 area hotspot is a singularity";  // reapar.f90:307-311
    return false;
  }
  const char* off_keys[] = {"CHSEQ", "CMISALIGN", "DIFFUSION", "DENSINPUT"};
  for (const char* k : off_keys) {
    if (P.has(k)) {
      REQ(P.integer(k, &iv, err));
      if (iv != 0) { *err = std::string(k) + "=YES is not supported by this build"; return false; }
    }
  }
  // disk structure (reapar.f90:155-271)
  auto flag = [&](const char* k, int* out) {
    *out = 0;
    if (!P.has(k)) return true;
    int64_t v;
    if (!P.integer(k, &v, err)) return false;
    *out = (int)v;
    return true;
  };
  REQ(flag("CGAPD", &m->igapd));
  REQ(flag("CSPIRAL", &m->ispiral));
  REQ(flag("CDISKWARP", &m->idiskwarp));
  REQ(flag("CRIMPUFF", &m->irimpuff));
  REQ(flag("CGAPPUFF", &m->igappuff));
  REQ(flag("CRIMCURVE", &m->irimcurve));
  REQ(flag("CGAPCURVE", &m->igapcurve));
  REQ(flag("CRADEXP", &m->iradexp));
  if (m->igapd) {
    REQ(P.real("RGAPD1", &m->rgapd1, err));
    REQ(P.real("RGAPD2", &m->rgapd2, err));
    for (int d = 1; d <= 2; ++d) {
      char key[64];
      snprintf(key, sizeof key, "ZSCALE_GAP(%d)", d); REQ(P.real(key, &m->z1gap[d - 1], err));
      snprintf(key, sizeof key, "A_GAP(%d)", d); REQ(P.real(key, &m->agap[d - 1], err));
      snprintf(key, sizeof key, "B_GAP(%d)", d); REQ(P.real(key, &m->bgap[d - 1], err));
      snprintf(key, sizeof key, "RHOSCALE_GAP(%d)", d); REQ(P.real(key, &m->rhoscale_gap[d - 1], err));
    }
  }
  if (m->ispiral) {
    REQ(P.real("PITCH", &m->pitch, err));
    REQ(P.integer("SN", &iv, err)); m->sn = (int)iv;
    REQ(P.real("SW", &m->sw, err));
    REQ(P.real("RSPIRAL1", &m->rspiral1, err));
    REQ(P.real("RSPIRAL2", &m->rspiral2, err));
  }
  if (m->idiskwarp) {
    REQ(P.real("WARPHEIGHT", &m->warpheight, err));
    REQ(P.real("WEXP", &m->wexp, err));
    REQ(P.real("WARPLENGTH", &m->warplength, err));
  }
  if (m->irimpuff) { REQ(P.real("RIMHEIGHT", &m->rimheight, err)); REQ(P.real("RIMLENGTH", &m->rimlength, err)); }
  if (m->igappuff) { REQ(P.real("GAPHEIGHT", &m->gapheight, err)); REQ(P.real("GAPLENGTH", &m->gaplength, err)); }
  if (m->irimcurve) {
    REQ(P.real("RIMCURVEHEIGHT", &m->rimcurveheight, err));
    REQ(P.real("RIMCURVELENGTH", &m->rimcurvelength, err));
    REQ(P.real("RIMCURVEEXP", &m->rimcurveexp, err));
  }
  if (m->igapcurve) {
    REQ(P.real("GAPCURVEHEIGHT", &m->gapcurveheight, err));
    REQ(P.real("GAPCURVELENGTH", &m->gapcurvelength, err));
    REQ(P.real("GAPCURVEEXP", &m->gapcurveexp, err));
  }
  if (m->iradexp) REQ(P.real("RADEXP", &m->radexp, err));
  // envelope gap (reapar.f90:369-391)
  REQ(flag("CGAPE", &m->igape));
  if (m->igape) {
    REQ(P.real("RGAPE1", &m->rgape1, err));
    REQ(P.real("RGAPE2", &m->rgape2, err));
    REQ(P.str("CGAPEDENS", &sv, err));
    if (sv == "SCALE") m->igapedens = 1;
    else if (sv == "CONST") m->igapedens = 0;
    else { *err = "CGAPEDENS should be set to SCALE or CONST"; return false; }
    REQ(P.real("FRACTE", &m->fracte, err));
    REQ(P.real("RHOGAPE", &m->rhogape, err));
  }
  double rmind_in[HC3D_NDG] = {0}, fsg[4] = {0};
  for (int d = 1; d <= 2; ++d) {
    char key[64];
    snprintf(key, sizeof key, "DUSTNAME(%d)", d);
    REQ(P.str(key, &sv, err)); m->dustname[d - 1] = sv;
    snprintf(key, sizeof key, "FSG(%d)", d); REQ(P.real(key, &fsg[d - 1], err));
    snprintf(key, sizeof key, "ZSCALE(%d)", d); REQ(P.real(key, &m->z1[d - 1], err));
    snprintf(key, sizeof key, "RMIND(%d)", d); REQ(P.real(key, &rmind_in[d - 1], err));
    snprintf(key, sizeof key, "RMAXD(%d)", d); REQ(P.real(key, &m->rmaxd[d - 1], err));
    snprintf(key, sizeof key, "A(%d)", d); REQ(P.real(key, &m->a[d - 1], err));
    snprintf(key, sizeof key, "B(%d)", d); REQ(P.real(key, &m->b[d - 1], err));
  }
  REQ(P.str("DUSTNAME(3)", &sv, err)); m->dustname[2] = sv;
  REQ(P.str("DUSTNAME(4)", &sv, err)); m->dustname[3] = sv;
  REQ(P.real("FSG(3)", &fsg[2], err));
  REQ(P.real("FSG(4)", &fsg[3], err));
  for (int k = 0; k < 4; ++k) {
    if (!(fsg[k] >= 0.0 && fsg[k] <= 1.0)) { *err = "FSG(1..4) must lie in [0, 1]"; return false; }
    m->fsg[k] = fsg[k];
  }
  // the small-grain species 5-8 take the FSG share of their parent's mass
  // (reapar.f90:259-262,338-339,419-420); their dust files are read when
  // any FSG is above zero (species 5's opacity weights the ISRF integral)
  if (m->has_sg()) {
    for (int d = 5; d <= 8; ++d) {
      char key[64];
      snprintf(key, sizeof key, "DUSTNAME(%d)", d);
      REQ(P.str(key, &sv, err)); m->dustname[d - 1] = sv;
    }
    if (m->isrf_file.empty()) {
      if (!P.has("ISRF_FILE")) {
        *err = "FSG > 0 needs ISRF_FILE: the small grains' emission spectrum is chosen by the mean intensity "
               "in units of the ISRF absorbed by them";
        return false;
      }
      REQ(P.str("ISRF_FILE", &sv, err)); m->isrf_file = m->pardir + "/" + sv;
    }
  }
  m->fmass[0] = fmassd1 * (1.0 - fsg[0]); m->fmass[4] = fmassd1 * fsg[0];
  m->fmass[1] = (1.0 - fmassd1) * (1.0 - fsg[1]); m->fmass[5] = (1.0 - fmassd1) * fsg[1];
  m->fmass[2] = 1.0 - fsg[2]; m->fmass[6] = fsg[2];
  m->fmass[3] = 1.0 - fsg[3]; m->fmass[7] = fsg[3];
  for (int d = 0; d < 2; ++d) m->rddust[d] = m->rmind_in[d] = rmind_in[d];
  REQ(P.real("RMAX", &m->rmax, err));
  double rmine_in;
  REQ(P.real("RMINE", &rmine_in, err));
  m->rmine_in = rmine_in;
  REQ(P.str("ENVTYPE", &sv, err));
  m->ienvtype = sv == "ULRICH" ? 1 : sv == "POWLAW" ? 0 : -1;
  if (m->ienvtype < 0) { *err = "ERROR: ENVTYPE should be set to ULRICH or POWLAW"; return false; }
  REQ(P.real("RATE", &m->rate, err));
  REQ(P.real("RC", &m->rc, err));
  if (m->ienvtype == 0) { REQ(P.real("RHODENS1", &m->rhodens1, err)); REQ(P.real("ENVEXP", &m->envexp, err)); }
  REQ(P.real("RHOAMB", &m->rhoamb, err));
  REQ(P.integer("CFRACTAL", &iv, err)); m->ifractal = (int)iv;
  if (m->ifractal) {
    std::vector<int64_t> fm;
    REQ(P.real("DENSRATIO", &m->densratio, err));
    REQ(P.ints("FRACTMASK", &fm, err));
    REQ(P.integer("IFSEED", &m->ifseed, err));
    for (size_t k = 0; k < 4 && k < fm.size(); ++k) m->fractmask[k] = m->fractmask[k + 4] = (int)fm[k];
    if (P.has("FRACTLEV")) { REQ(P.integer("FRACTLEV", &iv, err)); m->fractlev = (int)iv; }
    if (P.has("FRACTN")) { REQ(P.integer("FRACTN", &iv, err)); m->fractn = (int)iv; }
    if (P.has("FRACTCONTRAST")) REQ(P.real("FRACTCONTRAST", &m->fractcontrast, err));
  }
  REQ(P.integer("CHOLE", &iv, err)); m->ihole = (int)iv;
  if (m->ihole) {
    REQ(P.str("CSHAPE", &sv, err));
    if (sv == "STREAM") { *err = "CSHAPE=STREAM is not supported; use POLYN"; return false; }
    m->ipoly = 1;
    REQ(P.real("EX1", &m->ex1, err)); REQ(P.real("EX2", &m->ex2, err));
    REQ(P.real("THET1", &m->thet1, err)); REQ(P.real("Z01", &m->z01, err));
    REQ(P.real("THET2", &m->thet2, err)); REQ(P.real("Z02", &m->z02, err));
    REQ(P.real("EXF", &m->exf, err));
    REQ(P.real("RHOCONST1", &m->rhoconst1, err)); REQ(P.real("RHOCONST2", &m->rhoconst2, err));
  }
  REQ(P.integer("NPEEL", &iv, err)); m->npeel = (int)iv;
  REQ(P.integer("NAP", &iv, err)); m->nap = (int)iv;
  REQ(P.integer("NXIMG", &iv, err)); m->nxhst = (int)iv;
  REQ(P.real("RMAXI", &m->rmaxi, err));
  double apmin, apmax;
  REQ(P.real("APMIN", &apmin, err)); REQ(P.real("APMAX", &apmax, err));
  REQ(P.reals("THETE", &m->thete, err)); REQ(P.reals("PHIE", &m->phie, err));
  if ((int)m->thete.size() < m->npeel || (int)m->phie.size() < m->npeel) {
    *err = "THETE/PHIE list shorter than NPEEL"; return false;
  }
  m->thete.resize(m->npeel); m->phie.resize(m->npeel);
  for (double t : m->thete)
    if (t == 0.0) { *err = "ERROR: THETE has to be <> 0"; return false; }
  REQ(P.integer("NRG", &iv, err)); m->nrg = (int)iv;
  REQ(P.integer("NTG", &iv, err)); m->ntg = (int)iv;
  REQ(P.integer("NPG", &iv, err)); m->npg = (int)iv;
  REQ(P.integer("NMU", &iv, err)); m->nmu = (int)iv;
  REQ(P.integer("NPH", &iv, err)); m->nph = (int)iv;
  REQ(P.integer("NFREQ", &iv, err)); m->nfreq = (int)iv;
  if (m->nrg < 3 || m->ntg < 3 || m->npg < 2 || m->ntg % 2 == 0) {
    *err = "grid needs NRG>=3, NPG>=2 and an odd NTG>=3"; return false;
  }
  if ((double)m->nrg * m->ntg * m->npg > 1e9) { *err = "Number of grid cells requested is too large"; return false; }
  double lmin = 0.01, lmax = 5000.0;
  if (P.has("SEDLMIN")) REQ(P.real("SEDLMIN", &lmin, err));
  if (P.has("SEDLMAX")) REQ(P.real("SEDLMAX", &lmax, err));
  if (P.has("IMAGE")) { REQ(P.integer("IMAGE", &iv, err)); m->image = (int)iv; }
  if (P.has("IMCUBE")) { REQ(P.integer("IMCUBE", &iv, err)); m->imcube = (int)iv; }  // reapar.f90:472
  if (P.has("MAXINT")) REQ(P.integer("MAXINT", &m->maxint, err));

  // ---- setup.f90:26-231 ----
  m->numin = 1.2398 / lmax;
  m->numax = 1.2398 / lmin;
  m->autors = kAu / kRsun / m->rstar;
  m->tsub_k = 1600.0;
  m->rminsub = std::pow(m->tsub_k / m->tstar_k, -2.10);
  if (irminsub == 1) {
    m->rmine = m->rminsub * rmine_in;
    for (int d = 0; d < 2; ++d) m->rddust[d] = m->rminsub * rmind_in[d];
  } else if (irminsub == 2) {
    m->rmine = rmine_in * m->autors;
    for (int d = 0; d < 2; ++d) m->rddust[d] = rmind_in[d] * m->autors;
  } else {
    m->rmine = rmine_in;
  }
  m->rspiral1 *= m->autors;
  m->rspiral2 *= m->autors;
  if (czmin == "RSUB") {
    const double muc = 2.3, rcgs = m->rminsub * m->rstar * kRsun, mcgs = m->massc * kMsun;
    const double honr = std::sqrt(kBoltz * m->tsub_k / kGn / mcgs * rcgs / muc / kMH);
    for (int d = 0; d < 2; ++d) {
      m->z1[d] = m->z1[d] * honr * m->rminsub / std::pow(m->rminsub, m->b[d]);
      m->z1gap[d] = m->z1gap[d] * honr * m->rminsub / std::pow(m->rminsub, m->bgap[d]);
    }
  } else if (czmin == "R100") {
    for (int d = 0; d < 2; ++d) {
      m->z1[d] = m->z1[d] * m->autors / std::pow(100.0 * m->autors, m->b[d]);
      m->z1gap[d] = m->z1gap[d] * m->autors / std::pow(100.0 * m->autors, m->bgap[d]);
    }
  }
  m->rgapd1 *= m->autors;
  if (m->rgapd1 < 1.0) m->rgapd1 = 1.0;
  m->rgapd2 *= m->autors;
  m->rgape1 *= m->autors;
  m->rgape2 *= m->autors;
  m->warplength *= m->autors;
  m->gaplength *= m->autors;
  m->rimlength *= m->autors;
  m->rimcurvelength *= m->autors;
  m->gapcurvelength *= m->autors;
  m->radexp *= m->autors;
  m->pitch = m->pitch * kPi / 180.0;
  if (m->massd == 0.0) {  // reapar.f90:315-326
    // Switches off the disk's structure options.  The reference does this
    // before its setup; here it follows the unit scaling above, which reads
    // none of these flags, so the order gives the same model.  (The other
    // massd == 0 reset of the reference, the inner radius and the radial
    // grid of a disk-less model, is the radial grid of gridset below.)
    m->idiskwarp = 0; m->igapd = 0; m->ispiral = 0; m->igappuff = 0; m->irimpuff = 0;
    m->idiskacc = 0;
    if (m->ispot) {
      *err = "CSPOT=YES needs a disk (MASSD > 0) with CDISKACC=YES: the hot-spot temperature comes from the "
             "accretion shock";
      return false;
    }
  }
  m->rmax *= m->autors;
  for (int d = 0; d < 2; ++d) m->rmaxd[d] *= m->autors;
  m->rmaxi *= m->autors;
  m->rc *= m->autors;
  m->z01 *= m->autors;
  m->z02 *= m->autors;
  m->aperture2.resize(m->nap);
  for (int i = 0; i < m->nap; ++i) {
    double ap = m->nap == 1 ? apmin
                            : std::pow(10.0, (double)i / (double)(m->nap - 1) * (std::log10(apmax) - std::log10(apmin)) +
                                                 std::log10(apmin));
    ap *= m->autors;
    m->aperture2[i] = ap * ap;
  }
  for (int d = 0; d < 2; ++d) {
    if (m->rddust[d] > m->rmaxd[d] && m->fmass[d] > 0.0) { *err = "ERROR, rddust > rmaxd"; return false; }
    if (m->rmaxd[d] > m->rmax) m->rmax = m->rmaxd[d] * 1.001;
  }
  m->rddustmin = std::min(m->rddust[0], m->rddust[1]);
  for (int k = 0; k < m->npeel; ++k) {
    m->thete[k] *= kR2p / 360.0;
    m->phie[k] *= kR2p / 360.0;
  }
  return true;
}

// envset, envset.f90:18-80
static void envset(Model* m) {
  const double rdcgs = m->rc * m->rstar * kRsun;
  const double cst = 1.0 / 3.15576e7 * std::sqrt(kMsun) / (4.0 * kPi) / std::sqrt(kGn);
  m->rhoe0 = cst * m->rate / std::sqrt(m->massc) / std::pow(rdcgs, 1.5);
  const double z1max = m->rmax;
  if (m->thet1 < 89.999) {
    double r1max = z1max * std::tan(m->thet1 * kPi / 180.0);
    m->c1e = (z1max - m->z01) / std::pow(r1max, m->ex1);
    double r2max = z1max * std::tan(m->thet2 * kPi / 180.0);
    m->c2e = (z1max - m->z02) / std::pow(r2max, m->ex2);
  } else {
    m->c1e = 0.0;
    m->c2e = 0.0;
  }
}

// The small-grain disk species 5 and 6 share the geometry of disk species 1
// and 2 (reapar.f90:239-268: scale heights, exponents, radii, gap law; the
// fractal mask of species 5-8 is that of 1-4).  Called after each step that
// moves the parents' geometry.
static void sg_geometry(Model* m) {
  for (int d = 0; d < 2; ++d) {
    m->z1[d + 4] = m->z1[d]; m->a[d + 4] = m->a[d]; m->b[d + 4] = m->b[d];
    m->rmaxd[d + 4] = m->rmaxd[d]; m->rddust[d + 4] = m->rddust[d];
    m->z1gap[d + 4] = m->z1gap[d]; m->agap[d + 4] = m->agap[d]; m->bgap[d + 4] = m->bgap[d];
    m->rhoscale_gap[d + 4] = m->rhoscale_gap[d];
  }
}

// setup_wave, setup_wave.f90:46-80: disk rho0 before gridset rescales it.
static void setup_rho0(Model* m) {
  const double rmincgs = m->rstar * kRsun;
  for (int id : {0, 1, 4, 5}) {
    const double z1cgs = rmincgs * m->z1[id];
    const double p = m->b[id] - m->a[id];
    const double rmind = m->rddust[id];
    if (m->rmaxd[id] > 0.0 && m->fmass[id] > 0.0) {
      const double cst = std::pow(kR2p, 1.5) * rmincgs * rmincgs * z1cgs;
      double denom;
      if (p != -2.0 && p != -1.5)
        denom = 1.0 / (p + 2.0) * (std::pow(m->rmaxd[id], p + 2.0) - std::pow(rmind, p + 2.0)) -
                1.0 / (p + 1.5) * (std::pow(m->rmaxd[id], p + 1.5) - std::pow(rmind, p + 1.5));
      else if (p == -2.0)
        denom = std::log(m->rmaxd[id] / rmind) -
                1.0 / (p + 1.5) * (std::pow(m->rmaxd[id], p + 1.5) - std::pow(rmind, p + 1.5));
      else
        denom = 1.0 / (p + 2.0) * (std::pow(m->rmaxd[id], p + 2.0) - std::pow(rmind, p + 2.0)) -
                std::log(m->rmaxd[id] / rmind);
      m->rho0[id] = m->massd * kMsun / cst / denom * m->fmass[id];
    } else {
      m->rho0[id] = 0.0;
    }
  }
}

// The luminosities of gridset.f90:72-290: the star, the external field
// (newtts.F90:207, rmax in stellar radii) and, with CDISKACC, the accretion
// luminosity of the disk (lacc) and of the shock on the star (lacc2), the
// hot-spot size and temperature, the mean stellar temperature tave and the
// sublimation radius it sets, and the constants of the accretion and spot
// sources (spotset.f90:179-206).  Runs after setup_rho0 (the accretion rate
// of CALPHA=YES scales with the disk's rho0) and before the grid walls, which
// the new sublimation radius moves.
static bool luminosities(Model* m, std::string* err) {
  const double rmincgs = m->rstar * kRsun;
  const double yr = 3600.0 * 24.0 * 365.25;
  const double deg2rad = kPi / 180.0, rad2deg = 180.0 / kPi;
  m->lstar = 4.0 * kPi * kSigt * std::pow(m->tstar_k, 4.0) * rmincgs * rmincgs;
  m->l_isrf = m->iout ? m->isrf_int * 4.0 * kPi * std::pow(m->rmax * kRsun * m->rstar, 2.0) / 4.0 * m->isrf_scl : 0.0;
  m->mdotcgs[0] = m->mdotcgs[1] = 0.0;
  m->lacc = m->lacc2 = 0.0;
  m->tshock_k = 0.0;
  m->thspot_deg = 0.0;
  if (m->idiskacc) {
    const double vc = std::sqrt(kGn * kMsun * m->massc / rmincgs);
    if (m->ialpha) {
      // eqs. 5 and 6 of Whitney et al. 2003 (ApJ 591, 1049) for each disk slot
      double mdot = 0.0;
      for (int id = 0; id < 2; ++id) {
        m->mdotcgs[id] = std::sqrt(18.0 * std::pow(kPi, 3.0)) * m->alphad * vc * m->rho0[id] *
                         std::pow(m->z1[id] * rmincgs, 3.0) / rmincgs;
        mdot += m->mdotcgs[id];
      }
      m->mdotdisk = mdot * yr / kMsun;
    } else {
      // the total rate split between the slots as rho0 z1^3 (IEEE: all to slot 1 when slot 2 is empty)
      const double mdottot = m->mdotdisk / (yr / kMsun);
      const double z1a = m->z1[0] * m->z1[0] * m->z1[0], z1b = m->z1[1] * m->z1[1] * m->z1[1];
      const double ratio = m->rho0[0] * z1a / m->rho0[1] / z1b;
      m->mdotcgs[1] = mdottot / (1.0 + ratio);
      m->mdotcgs[0] = mdottot - m->mdotcgs[1];
    }
    m->mdot_cgs = m->mdotcgs[0] + m->mdotcgs[1];
    m->mdotdisk = m->mdot_cgs * yr / kMsun;
    m->lacc = kGn * (kMsun * m->massc) * m->mdot_cgs / 2.0 / (m->rddustmin * rmincgs);
    if (m->massd > 0.0) m->lacc2 = kGn * (kMsun * m->massc) * m->mdot_cgs * (1.0 / rmincgs - 1.0 / (rmincgs * m->rtrunc));
    else m->lacc = 0.0;
  }
  m->ltot = m->lacc + m->lacc2 + m->lstar + m->l_isrf;
  m->accfrac = m->lacc / m->ltot;
  m->accfrac2 = m->lacc2 / m->ltot;
  m->isrf_frac = m->l_isrf / m->ltot;
  if (m->idiskacc && m->lacc2 > 0.0) {
    double fluxratio;
    if (m->itemp == 0) {
      fluxratio = 0.5 * m->lacc2 / m->lstar / m->fspot;
      m->tshock_k = m->tstar_k * std::pow(1.0 + fluxratio, 0.25);
      m->tspot = m->tshock_k;
    } else {
      m->tshock_k = m->tspot;
      fluxratio = std::pow(m->tshock_k / m->tstar_k, 4.0) - 1.0;
      m->fspot = 0.5 * m->lacc2 / m->lstar / fluxratio;
    }
    if (m->nspot == 1) m->thspot_deg = std::acos(1.0 - 2.0 * m->fspot) * rad2deg;
    else if (m->nspot == 2) m->thspot_deg = std::acos(1.0 - m->fspot) * rad2deg;
    else { *err = "error!  nspot not set (NSPOT must be 1 or 2)"; return false; }
    if (!(m->tshock_k > 0.0) || !std::isfinite(m->tshock_k) || !(m->fspot > 0.0) || !std::isfinite(m->thspot_deg)) {
      *err = "the hot spots have no valid temperature or size (CTEMP=YES needs TSPOT > TSTAR; the spots "
             "cannot cover more than the star)";
      return false;
    }
  }
  // mean stellar temperature including the shock, and the sublimation radius it sets
  m->tave_k = m->tstar_k * std::pow(1.0 + 0.5 * m->lacc2 / m->lstar, 0.25);
  m->rminsub = std::pow(m->tsub_k / m->tave_k, -2.1);
  if ((m->rminsub > m->rmaxd[0] || m->rminsub > m->rmaxd[1]) && m->massd > 0.0) {
    *err = "ERROR.  dust sublimation radius larger than RMAXD; increase RMAXD";
    return false;
  }
  if (m->irminsub == 1) {
    m->rmine = m->rminsub * m->rmine_in;
    for (int d = 0; d < 2; ++d) m->rddust[d] = m->rminsub * m->rmind_in[d];
  }
  for (int d = 0; d < 2; ++d)
    if (m->rddust[d] > m->rmaxd[d] && m->fmass[d] > 0.0) { *err = "ERROR, rddust > rmaxd"; return false; }
  m->rddustmin = std::min(m->rddust[0], m->rddust[1]);
  m->rmaxdmax = std::max(m->rmaxd[0], m->rmaxd[1]);
  // the source constants
  hc3d_sources& s = m->src;
  s = hc3d_sources{};
  s.rddustmin = m->rddustmin;
  s.rmaxdmax = m->rmaxdmax;
  s.rmax = m->rmax;
  for (int d = 0; d < 2; ++d) {
    s.zfac[d] = m->fmass[d] * m->z1[d];
    s.zexp[d] = m->b[d];
    s.kapv[d] = 0.0;  // set with the dust tables (build_model)
  }
  // The reference sets the gas temperature's accretion rate only for CALPHA=YES; for CALPHA=NO it
  // leaves it unset.  Both use the total rate here (what its FITS writer uses for the same formula).
  s.gas_num = 3.0 * kGn * (kMsun * m->massc) * m->mdot_cgs;
  s.gas_den = 8.0 * kPi * kSigt;
  s.rstar = m->rstar;
  s.rsun = kRsun;
  s.ispot = m->ispot;
  s.nspot = m->nspot;
  if (m->ispot) {
    const double thspot = m->thspot_deg * deg2rad;
    const double th1 = (90.0 - m->spotlat) * deg2rad, ph1 = 0.0 * deg2rad;  // spotlon = 0 (reapar.f90:291)
    const double th2 = kPi - th1, ph2 = ph1 + kPi;
    s.spot1[0] = std::sin(th1) * std::cos(ph1); s.spot1[1] = std::sin(th1) * std::sin(ph1);
    s.spot1[2] = std::cos(th1); s.spot1[3] = std::sin(th1);
    s.spot2[0] = std::sin(th2) * std::cos(ph2); s.spot2[1] = std::sin(th2) * std::sin(ph2);
    s.spot2[2] = std::cos(th2); s.spot2[3] = std::sin(th2);
    s.csprad = std::cos(thspot);
  }
  s.fspot = m->fspot;
  s.tshock = m->tshock_k / 11605.0;
  if (m->idiskacc && !(m->rddustmin < m->rmaxdmax)) {
    *err = "CDISKACC=YES needs the disk's inner radius below its outer radius (no radius to emit from)";
    return false;
  }
  return true;
}

// gridset walls and densities, gridset.f90:411-664 and 954-1098
static bool gridset(Model* m, std::string* err) {
  const int nrg = m->nrg, ntg = m->ntg, npg = m->npg;
  const double rmin = 1.0, rmincgs = m->rstar * kRsun;
  m->rarr.assign(nrg, 0.0);
  m->r2arr.assign(nrg, 0.0);
  m->ravearr.assign(nrg - 1, 0.0);
  // radial walls (gridset.f90:423-455)
  m->rarr[0] = rmin;
  if (m->massd == 0.0) {
    const double rexpnew = 3.0;  // grid_mod rexp
    const double dr = (m->rmax - m->rmine) / std::pow((double)(nrg - 1), rexpnew);
    for (int ir = 2; ir <= nrg; ++ir) m->rarr[ir - 1] = m->rmine + dr * std::pow((double)(ir - 1), rexpnew);
  } else {
    const double rdduste = std::min(std::min(m->rddust[0], m->rddust[1]), m->rmine);
    const double rfac = std::pow(m->rmax / rdduste, 1.0 / (double)(nrg - 2));
    for (int ir = 2; ir <= nrg; ++ir) m->rarr[ir - 1] = rdduste * std::pow(rfac, ir - 2);
  }
  auto locate = [](const std::vector<double>& xx, double x) {
    int n = (int)xx.size(), jl = 0, ju = n + 1;
    bool asc = xx[n - 1] > xx[0];
    while (ju - jl > 1) {
      int jm = (ju + jl) / 2;
      if (asc == (x > xx[jm - 1])) jl = jm; else ju = jm;
    }
    if (jl == 0 && x == xx[0]) jl = 1;
    return jl;
  };
  if (m->rddustmin < m->rmine) {
    int ir = locate(m->rarr, m->rmine);
    if (ir >= 1 && ir < nrg) m->rarr[ir] = m->rmine;
  }
  if (m->rmine < m->rddustmin) {
    int ir = locate(m->rarr, m->rddustmin);
    if (ir >= 1 && ir < nrg) m->rarr[ir] = m->rddustmin;
  }
  for (int ir = 0; ir < nrg; ++ir) m->r2arr[ir] = std::pow(m->rarr[ir], 2.0);
  for (int ir = 0; ir < nrg - 1; ++ir) {
    double r1 = std::log10(m->rarr[ir]), r2 = std::log10(m->rarr[ir + 1]);
    m->ravearr[ir] = std::pow(10.0, 0.5 * (r1 + r2));
  }
  for (int ir = 1; ir < nrg; ++ir)
    if (!(m->rarr[ir] > m->rarr[ir - 1])) { *err = "radial walls are not increasing"; return false; }
  // polar walls, power law pexp=2 (gridset.f90:529-604)
  const int nttmp = ntg / 2;
  const int pexp = 2;
  m->thetarr.assign(ntg, 0.0);
  std::vector<double> tmpth(nttmp + 1);
  const double mm = kPi / 2.0 / std::pow((double)nttmp, pexp);
  for (int it = 1; it <= nttmp; ++it) tmpth[it] = mm * std::pow((double)it, pexp);
  for (int it = 1; it <= nttmp; ++it) m->thetarr[nttmp + 1 + it - 1] = tmpth[it] + kPiHalf;
  m->thetarr[nttmp] = kPiHalf;
  for (int it = 1; it <= nttmp; ++it) m->thetarr[it - 1] = kPi - m->thetarr[ntg - it];
  for (double te : m->thete)
    for (double tw : m->thetarr)
      if (te == tw) { *err = "ERROR: peeloff angle is exactly the same as one of the wall angles"; return false; }
  m->costarr.assign(ntg, 0.0);
  m->sintarr.assign(ntg, 0.0);
  m->tan2arr.assign(ntg, 0.0);
  for (int it = 1; it <= ntg; ++it) {
    double& th = m->thetarr[it - 1];
    if (it == 1) {
      th = 0.0; m->costarr[0] = 1.0; m->sintarr[0] = 0.0; m->tan2arr[0] = 0.0;
    } else if (it == ntg) {
      th = kPi; m->costarr[it - 1] = -1.0; m->sintarr[it - 1] = 0.0; m->tan2arr[it - 1] = 0.0;
    } else if (it == nttmp + 1) {
      th = kPiHalf; m->costarr[it - 1] = 0.0; m->sintarr[it - 1] = 1.0; m->tan2arr[it - 1] = -1.0;
    } else {
      m->costarr[it - 1] = std::cos(th);
      m->sintarr[it - 1] = std::sin(th);
      m->tan2arr[it - 1] = std::pow(std::tan(th), 2.0);
    }
  }
  m->thetavearr.assign(ntg - 1, 0.0);
  for (int it = 0; it < ntg - 1; ++it) {
    if (m->thetarr[it + 1] < m->thetarr[it]) { *err = "Error - thetarr is not monotonically increasing"; return false; }
    double th1 = std::pow(m->thetarr[it], pexp), th2 = std::pow(m->thetarr[it + 1], pexp);
    m->thetavearr[it] = std::pow(0.5 * (th1 + th2), 1.0 / pexp);
  }
  // azimuthal walls (gridset.f90:642-650)
  m->phiarr.assign(npg, 0.0);
  m->aarr.assign(npg, 0.0);
  m->barr.assign(npg, 0.0);
  const double dp = kR2p / (double)(npg - 1);
  for (int ip = 0; ip < npg; ++ip) {
    m->phiarr[ip] = dp * (double)ip;
    m->aarr[ip] = std::sin(m->phiarr[ip]);
    m->barr[ip] = -std::cos(m->phiarr[ip]);
  }
  // ---- densities (gridset.f90:954-1098), the fractal factor first ----
  const auto t_dens = std::chrono::steady_clock::now();
  if (m->ifractal) fractal_field(m);
  // species: disk 1, disk 2, envelope, cavity, and with FSG > 0 their
  // small-grain shares 5-8 (grid_mod.f90:13-20)
  m->ndg = m->has_sg() ? 8 : 4;
  std::vector<int> disk_ids = {0, 1}, env_ids = {2, 3};
  if (m->ndg == 8) { disk_ids = {0, 1, 4, 5}; env_ids = {2, 3, 6, 7}; }
  const int64_t n4 = m->n4();
  m->densarr.assign(n4 * m->ndg, 0.0);
  m->massarr.assign(n4 * m->ndg, 0.0);
  m->vcell.assign(n4, 0.0);
  auto cell = [&](int ir, int it, int ip) { return (int64_t)ir + (int64_t)nrg * (it + (int64_t)ntg * ip); };
  const bool phidep = m->disk_depends_on_phi();
  auto phic = [&](int ip) { return 0.5 * (m->phiarr[ip] + m->phiarr[ip + 1]); };
  // the gap's density scale: rho0 times RHOSCALE_GAP times the ratio of the
  // surface densities just outside and just inside the gap's outer wall,
  // integrated over theta and phi with rhogap0 = rho0 (gridset.f90:906-942)
  for (int id : disk_ids) m->rhogap0[id] = m->rho0[id];
  if (m->igapd) {
    double rhogap[2];
    for (int id = 0; id < 2; ++id) {
      double sig[2] = {0.0, 0.0};
      for (int i = 0; i < 2; ++i) {
        const double rad = m->rgapd2 * (i == 0 ? 0.9 : 1.1);
        for (int it = 0; it < ntg - 1; ++it) {
          const double thet = m->thetavearr[it], cost = std::cos(thet), sint = std::sin(thet);
          const double dcost = m->costarr[it] - m->costarr[it + 1];
          for (int ip = 0; ip < npg - 1; ++ip)
            sig[i] += std::fabs(densdisk(*m, rad, sint, cost, phic(ip), id) * rad * dcost * rmincgs) / (double)(npg - 1);
        }
      }
      // The reference divides by the surface density just inside the gap's
      // outer wall; a disk with none there (sig[0] = 0 while the slot holds
      // a disk) leaves the gap's density scale undefined: reject the model.
      if (!(sig[0] > 0.0)) {
        if (m->rho0[id] != 0.0 && m->rhoscale_gap[id] != 0.0) {
          *err = "CGAPD=YES: the disk has no density just inside the gap's outer wall (0.9 RGAPD2), so the "
                 "gap's density scale rho0 RHOSCALE_GAP sigma(1.1 RGAPD2) / sigma(0.9 RGAPD2) is undefined";
          return false;
        }
        rhogap[id] = 0.0;
        continue;
      }
      rhogap[id] = m->rho0[id] * m->rhoscale_gap[id] * sig[1] / sig[0];
    }
    for (int id = 0; id < 2; ++id) m->rhogap0[id] = rhogap[id];
    // the small grains' gap scale follows their parent's (gridset.f90:950-951)
    for (int id = 4; id < 6; ++id)
      m->rhogap0[id] = m->fmass[id - 4] > 0.0 ? m->fmass[id] / m->fmass[id - 4] * m->rhogap0[id - 4] : 0.0;
  }
  // disk mass normalisation: diskscl = massd*fmass / mass on the grid
  double diskscl[HC3D_NDG] = {1, 1, 1, 1, 1, 1, 1, 1};
  if (m->massd > 0.0) {
    double tmpmass[HC3D_NDG] = {0};
    for (int id : disk_ids) {
      if (m->rho0[id] == 0.0) continue;
      for (int ir = 0; ir < nrg - 1; ++ir) {
        const double rad = m->ravearr[ir];
        const double dr3 = std::pow(m->rarr[ir + 1], 3.0) - std::pow(m->rarr[ir], 3.0);
        for (int it = 0; it < ntg - 1; ++it) {
          const double thet = m->thetavearr[it], cost = std::cos(thet), sint = std::sin(thet);
          const double dcost = std::cos(m->thetarr[it + 1]) - std::cos(m->thetarr[it]);
          const double dd0 = phidep ? 0.0 : densdisk(*m, rad, sint, cost, 0.0, id);
          if (!phidep && dd0 == 0.0) continue;
          for (int ip = 0; ip < npg - 1; ++ip) {
            const double dd = phidep ? densdisk(*m, rad, sint, cost, phic(ip), id) : dd0;
            const double dpp = m->phiarr[ip + 1] - m->phiarr[ip];
            const double vol = -dr3 * dcost * dpp / 3.0 * std::pow(rmincgs, 3.0);
            tmpmass[id] += dd * vol;
          }
        }
      }
      tmpmass[id] /= kMsun;
      if (tmpmass[id] > 0.0) diskscl[id] = m->massd * m->fmass[id] / tmpmass[id];
    }
  }
  m->massdisk = 0.0;
  m->massenv = 0.0;
  const double r3 = std::pow(rmincgs, 3.0);
  for (int ir = 0; ir < nrg - 1; ++ir) {
    const double rad = m->ravearr[ir];
    const double dr3 = std::pow(m->rarr[ir + 1], 3.0) - std::pow(m->rarr[ir], 3.0);
    for (int it = 0; it < ntg - 1; ++it) {
      const double thet = m->thetavearr[it], cost = std::cos(thet), sint = std::sin(thet);
      const double dcost = std::cos(m->thetarr[it + 1]) - std::cos(m->thetarr[it]);
      double dens_r[HC3D_NDG];
      for (int id : disk_ids) dens_r[id] = densdisk(*m, rad, sint, cost, 0.0, id) * diskscl[id];
      for (int id : env_ids) dens_r[id] = densenv(*m, rad, thet, cost, sint, id) * m->fmass[id];
      for (int ip = 0; ip < npg - 1; ++ip) {
        if (phidep)
          for (int id : disk_ids) dens_r[id] = densdisk(*m, rad, sint, cost, phic(ip), id) * diskscl[id];
        const double dpp = m->phiarr[ip + 1] - m->phiarr[ip];
        const double vol = -dr3 * dcost * dpp / 3.0 * r3;
        const int64_t c = cell(ir, it, ip);
        m->vcell[c] = vol;
        for (int id = 0; id < m->ndg; ++id) {
          double d = dens_r[id];
          if (m->ifractal && m->fractmask[id] == 1)
            d *= m->densvar[ir + (int64_t)(nrg - 1) * (it + (int64_t)(ntg - 1) * ip)];
          m->densarr[c + n4 * id] = d;
          m->massarr[c + n4 * id] = std::pow(d * vol, 0.25);
          if (id % 4 < 2) m->massdisk += d * vol; else m->massenv += d * vol;
        }
      }
    }
  }
  m->massdisk /= kMsun;
  m->massenv /= kMsun;
  m->ndg_active = 0;
  bool filled[HC3D_NDG] = {false};
  for (int id = 0; id < m->ndg; ++id) {
    bool any = false;
    for (int64_t k = 0; k < n4 && !any; ++k) any = m->densarr[k + n4 * id] > 0.0;
    filled[id] = any;
    if (any) m->ndg_active++;
  }
  // The device carries four species slots: disk 1 and disk 2 in slots 1-2
  // (the accretion source draws among them), and two more.  Without small
  // grains those are the envelope and the cavity; with them, the species
  // among 3-8 that hold density, in their order.
  m->slot_species[0] = 1; m->slot_species[1] = 2; m->slot_species[2] = 3; m->slot_species[3] = 4;
  if (m->ndg == 8) {
    std::vector<int> more;
    for (int id = 2; id < 8; ++id)
      if (filled[id]) more.push_back(id + 1);
    if (more.size() > 2) {
      *err = "FSG > 0: more than four species hold density (disk 1, disk 2 and " + std::to_string(more.size()) +
             " of envelope, cavity and the small grains); the device carries four species";
      return false;
    }
    for (int cand : {3, 4, 5, 6, 7, 8}) {
      if (more.size() >= 2) break;
      if (std::find(more.begin(), more.end(), cand) == more.end()) more.push_back(cand);
    }
    std::sort(more.begin(), more.end());
    m->slot_species[2] = more[0]; m->slot_species[3] = more[1];
    sg_isrf_weight(m);
  }
  m->density_host_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_dens).count();
  // initarr(.true.): tdust2 = 0.1 K, tdust = tdust2 (initarr.f90:50,78-84)
  m->tdust.assign(n4 * m->ndg, 0.1 / 11605.0);
  // Lucy packets per iteration (newtts.F90:159-182)
  const int64_t ncells = m->ncells();
  int64_t npl = (ntg < 10 && npg < 10) ? 100 * ncells : (int64_t)(3.0 * (double)ncells);
  if (npl > m->np) npl = m->np;
  if (npl < m->npmin) npl = m->npmin;
  m->np_lucy = npl;
  return true;
}

bool build_model(Model* m, const std::string& par_path, const std::string* par_dir, std::string* err) {
  ParFile P;
  if (!P.load(par_path, err)) return false;
  if (!read_par(m, P, par_dir, err)) return false;
  envset(m);
  // dustinit: one table per species; identical files are read and integrated once
  m->ndg = m->has_sg() ? 8 : 4;
  m->nlambda.assign(m->ndg, 0);
  const size_t nl = (size_t)m->nlammax * m->ndg;
  m->nudust.assign(nl, 0); m->kappad.assign(nl, 0); m->adust.assign(nl, 0);
  m->gdust.assign(nl, 0); m->pldust.assign(nl, 0); m->lamdust.assign(nl, 0);
  m->kappav.assign(m->ndg, 0);
  for (int id = 0; id < m->ndg; ++id)
    if (!read_dust(m, id, m->pardir + "/" + m->dustname[id], err)) return false;
  const double Tmin = 0.1, Tmax = 2100.0;
  m->lTint.resize(m->nT);
  for (int i = 0; i < m->nT; ++i)
    m->lTint[i] = std::log(Tmin / 11605.0) + (double)i * std::log(Tmax / Tmin) / (double)(m->nT - 1);
  const double numax = 32.0, numin = numax / 1024.0;
  m->nuint.resize(m->nnu);
  for (int i = 0; i < m->nnu; ++i) m->nuint[i] = numin + (double)i * (numax - numin) / (double)(m->nnu - 1);
  const auto t_tab = std::chrono::steady_clock::now();
  m->kapBint.assign((size_t)m->nT * m->nnu * m->ndg, 0.0);
  m->kappap.assign((size_t)m->nT * m->ndg, 0.0);
  for (int id = 0; id < m->ndg; ++id) {
    int same = -1;
    for (int j = 0; j < id; ++j)
      if (m->dustname[j] == m->dustname[id]) { same = j; break; }
    double* kb = &m->kapBint[(size_t)id * m->nT * m->nnu];
    double* kp = &m->kappap[(size_t)id * m->nT];
    if (same >= 0) {
      std::copy(&m->kapBint[(size_t)same * m->nT * m->nnu], &m->kapBint[(size_t)(same + 1) * m->nT * m->nnu], kb);
      std::copy(&m->kappap[(size_t)same * m->nT], &m->kappap[(size_t)(same + 1) * m->nT], kp);
    } else {
      setemiss_species(*m, id, kb, kp);
    }
  }
  m->tables_host_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_tab).count();
  if (!atmosinit(m, m->atname, err)) return false;
  if ((m->iout || m->has_sg()) && !isrf_cdf(m, err)) return false;
  if (m->has_sg() && !draine_cdf(m, err)) return false;
  sg_geometry(m);
  setup_rho0(m);
  for (int d = 0; d < 2; ++d) m->src.kapv[d] = 0.0;
  if (!luminosities(m, err)) return false;
  for (int d = 0; d < 2; ++d) m->src.kapv[d] = m->kappav[d] * (m->rstar * kRsun);
  sg_geometry(m);
  if (!gridset(m, err)) return false;
  return true;
}

hc3d_dust_tables Model::tables_view() const {
  hc3d_dust_tables t;
  std::memset(&t, 0, sizeof t);
  t.ndg = ndg; t.nlammax = nlammax; t.nlambda = nlambda.data();
  t.nudust = nudust.data(); t.kappad = kappad.data(); t.adust = adust.data();
  t.gdust = gdust.data(); t.pldust = pldust.data(); t.kappav = kappav.data();
  t.nT = nT; t.nnu = nnu; t.lTint = lTint.data(); t.nuint = nuint.data();
  t.kapBint = kapBint.data(); t.kappap = kappap.data(); t.tsub = tsub_k;
  t.nhnu = (int)hnuint.size(); t.hnuint = hnuint.data(); t.atmosnu = atmosnu.data();
  t.lognu = lognu.data(); t.loghnu = loghnu.data();
  if (iout) {
    t.nisrf = (int)isrf_cdfv.size(); t.isrf_cdf = isrf_cdfv.data(); t.isrf_logcdf = isrf_logcdf.data();
    t.isrf_logfreq = isrf_logfreq.data();
  }
  if (limb) {
    t.ntab = (int)limb_xmu.size(); t.limb_xmu = limb_xmu.data(); t.limb_prob = limb_prob.data();
  }
  return t;
}

hc3d_grid Model::grid_view() const {
  hc3d_grid g;
  std::memset(&g, 0, sizeof g);
  g.nrg = nrg; g.ntg = ntg; g.npg = npg; g.ndg = ndg;
  g.rarr = rarr.data(); g.r2arr = r2arr.data(); g.thetarr = thetarr.data(); g.costarr = costarr.data();
  g.tan2arr = tan2arr.data(); g.phiarr = phiarr.data(); g.aarr = aarr.data(); g.barr = barr.data();
  g.densarr = densarr.data(); g.massarr = massarr.data(); g.vcell = vcell.data(); g.tdust = tdust.data();
  return g;
}

hc3d_run_params Model::params_view() const {
  hc3d_run_params p;
  std::memset(&p, 0, sizeof p);
  p.np = np; p.packet_offset = 0; p.seed = seed; p.iter = 1; p.ipeel = ipeel; p.npeel = npeel;
  p.thete = thete.data(); p.phie = phie.data(); p.nfreq = nfreq; p.nmu = nmu; p.nph = nph; p.nap = nap;
  p.nxhst = nxhst; p.rmaxi = rmaxi; p.aperture2 = aperture2.data(); p.numin = numin; p.numax = numax;
  p.rstar_cm = rstar * kRsun; p.tstar = tstar_k / 11605.0; p.limb = limb; p.iintmax = 10000;
  p.max_interactions = maxint; p.image = image; p.imcube = imcube && ipeel && image ? 1 : 0;
  p.ext_illum = iout; p.rmax = rmax;
  set_shares(&p, np);
  return p;
}

hc3d_model_info Model::info() const {
  hc3d_model_info i;
  std::memset(&i, 0, sizeof i);
  i.np = np; i.npmin = npmin; i.np_lucy = np_lucy; i.nimin = nimin; i.nimax = nimax; i.ipeel = ipeel;
  i.ilucy = ilucy; i.ndg_active = ndg_active; i.ltot = ltot; i.tstar_k = tstar_k; i.rstar_rsun = rstar;
  i.autors = autors; i.rminsub = rminsub; i.massdisk = massdisk; i.massenv = massenv; i.ncells = ncells();
  i.density_host_ms = density_host_ms;
  i.tables_host_ms = tables_host_ms;
  i.lstar = lstar; i.l_isrf = l_isrf; i.isrf_frac = isrf_frac;
  i.lacc = lacc; i.lacc2 = lacc2; i.accfrac = accfrac; i.accfrac2 = accfrac2; i.mdot_msun_yr = mdotdisk;
  i.tshock_k = tshock_k; i.fspot = fspot; i.thspot_deg = thspot_deg; i.tave_k = tave_k;
  for (int s = 0; s < 4; ++s) i.slot_species[s] = slot_species[s];
  i.has_sg = sg_slot >= 0 ? 1 : 0;
  i.ndg = ndg;
  return i;
}

}  // namespace hc3d

// ---------------------------------------------------------------------------
// C entry points of hc3d_host.h (model part)
// ---------------------------------------------------------------------------

static void put_err(char* err, size_t len, const std::string& s) {
  if (err && len) {
    std::snprintf(err, len, "%s", s.c_str());
  }
}

extern "C" int hc3d_model_create(hc3d_model** out, const char* par_path, const char* par_dir, char* err,
                                 size_t errlen) {
  if (!out || !par_path) return HC3D_ERR_INVALID;
  *out = nullptr;
  hc3d_model* m = new (std::nothrow) hc3d_model();
  if (!m) return HC3D_ERR_NOMEM;
  std::string e;
  std::string pd = par_dir ? par_dir : "";
  try {
    if (!hc3d::build_model(&m->m, par_path, par_dir ? &pd : nullptr, &e)) {
      put_err(err, errlen, e);
      delete m;
      bool unsup = e.find("not supported") != std::string::npos;
      bool io = e.find("cannot open") != std::string::npos;
      return unsup ? HC3D_ERR_UNSUPPORTED : io ? HC3D_ERR_IO : HC3D_ERR_INVALID;
    }
  } catch (const std::bad_alloc&) {
    put_err(err, errlen, "host allocation failed");
    delete m;
    return HC3D_ERR_NOMEM;
  }
  *out = m;
  return HC3D_OK;
}

extern "C" void hc3d_model_destroy(hc3d_model* m) { delete m; }

extern "C" int hc3d_model_views(hc3d_model* m, hc3d_dust_tables* t, hc3d_grid* g, hc3d_run_params* p,
                                hc3d_model_info* info) {
  if (!m) return HC3D_ERR_INVALID;
  if (t) *t = m->m.tables_view();
  if (g) *g = m->m.grid_view();
  if (p) *p = m->m.params_view();
  if (info) *info = m->m.info();
  return HC3D_OK;
}

extern "C" int hc3d_model_sg_tables(hc3d_model* m, hc3d_sg_tables* sg) {
  if (!m || !sg) return HC3D_ERR_INVALID;
  const hc3d::Model& M = m->m;
  if (M.sg_slot < 0) return HC3D_ERR_STATE;
  std::memset(sg, 0, sizeof *sg);
  sg->nemit = hc3d::kNemit;
  sg->ndraine = hc3d::kNdraine;
  sg->cdf = M.sg_cdf.data();
  sg->logcdf = M.sg_logcdf.data();
  sg->logfreq = M.sg_logfreq.data();
  sg->uratio = M.sg_uratio.data();
  sg->isrfkap_int = M.isrfkap_int;
  sg->sg_slot = M.sg_slot + 1;
  return HC3D_OK;
}

extern "C" int hc3d_model_set_tdust(hc3d_model* m, const double* tdust) {
  if (!m || !tdust) return HC3D_ERR_INVALID;
  std::copy(tdust, tdust + m->m.tdust.size(), m->m.tdust.begin());
  return HC3D_OK;
}

extern "C" int64_t hc3d_star_packets(double isrf_frac, int64_t np) {
  // newdisktherm.F90:143-175 with accfrac = 0: npout and ns rounded to the
  // nearest packet (ns from the single-precision real(np)), then ns takes up
  // the difference
  int64_t npout = (int64_t)(isrf_frac * (double)np);
  double rn = isrf_frac * (double)np;
  if (rn - (double)npout > 0.5) npout += 1;
  int64_t ns = (int64_t)((double)np * (1.0 - isrf_frac));
  rn = (double)(float)np * (1.0 - isrf_frac);
  if (rn - (double)ns > 0.5) ns += 1;
  const int64_t nsum = ns + npout;
  if (nsum != np) ns = ns + np - nsum;
  return ns;
}

extern "C" int hc3d_packet_split(double accfrac, double accfrac2, double isrf_frac, int64_t np, int64_t* n_acc,
                                 int64_t* n_spot, int64_t* n_star) {
  if (np < 0 || !n_acc || !n_spot || !n_star) return HC3D_ERR_INVALID;
  // newdisktherm.F90:143-175: shares rounded as the reference rounds them (the
  // accretion and hot-spot shares are truncated), ns takes up the difference
  int64_t npout = (int64_t)(isrf_frac * (double)np);
  double rn = isrf_frac * (double)np;
  if (rn - (double)npout > 0.5) npout += 1;
  int64_t ns = (int64_t)((double)np * (1.0 - accfrac - isrf_frac));
  rn = (double)(float)np * (1.0 - accfrac - isrf_frac);
  if (rn - (double)ns > 0.5) ns += 1;
  const int64_t npacc = (int64_t)((double)np * accfrac);
  int64_t npaccstar = (int64_t)(accfrac2 * (double)np);
  rn = (double)(int64_t)((double)ns * accfrac2);
  if (rn - (double)npaccstar > 0.5) npaccstar += 1;
  const int64_t nsum = ns + npacc + npout;
  if (nsum != np) ns = ns + np - nsum;
  // the packet loop runs iphot = 1..np: iphot < npacc accretion, iphot <
  // npacc + npaccstar hot spot, iphot <= npacc + ns star, the rest external
  // (newdisktherm.F90:209,256,258); global ids here are iphot - 1
  *n_star = std::max<int64_t>(0, std::min<int64_t>(np, npacc + ns));
  *n_acc = std::max<int64_t>(0, std::min<int64_t>(*n_star, npacc - 1));
  *n_spot = std::max<int64_t>(*n_acc, std::min<int64_t>(*n_star, npacc + npaccstar - 1));
  return HC3D_OK;
}

void hc3d::Model::set_shares(hc3d_run_params* p, int64_t np_total) const {
  p->sources = has_sources() ? &src : nullptr;
  hc3d_packet_split(accfrac, accfrac2, isrf_frac, np_total, &p->n_acc, &p->n_spot, &p->n_star);
}

// Fixture writers ------------------------------------------------------------
extern "C" int hc3d_write_synthetic_dust(const char* path) {
  // kappa: kV*(0.55/lam) below 100 um, continued as lam^-1.7 beyond, flat
  // below 0.1 um; albedo 0.5 -> 0 and g 0.6 -> 0 linear in log(lam) over
  // 0.1-10 um; pmax = 0.5.
  FILE* f = std::fopen(path, "w");
  if (!f) return HC3D_ERR_IO;
  const int n = 241;
  const double kV = 100.0;
  for (int i = 0; i < n; ++i) {
    double lam = std::pow(10.0, -2.0 + 6.0 * i / (double)(n - 1));  // 0.01 .. 10000 um
    double l = std::max(lam, 0.1);
    double kap = l <= 100.0 ? kV * (0.55 / l) : kV * (0.55 / 100.0) * std::pow(l / 100.0, -1.7);
    double x = (std::log10(lam) - std::log10(0.1)) / 2.0;
    x = std::max(0.0, std::min(1.0, x));
    double alb = 0.5 * (1.0 - x), g = 0.6 * (1.0 - x);
    double cext = kap * 1.0e-22;
    std::fprintf(f, " %.6e %.6e %.6e %.6e %.6e %.6e %.6e\n", lam, cext, alb * cext, kap, g, 0.5, 0.0);
  }
  std::fclose(f);
  return HC3D_OK;
}

extern "C" int hc3d_write_synthetic_isrf(const char* path) {
  // three diluted blackbodies of the Mathis, Mezger & Panagia (1983) form,
  // nu F_nu = sum W_i 4 pi nu B_nu(T_i), (T_i, W_i) = (7500 K, 1e-14),
  // (4000 K, 1.65e-13), (3000 K, 4e-13); 44 frequencies, log-spaced over
  // 10^11.45 .. 10^15.55 Hz
  FILE* f = std::fopen(path, "w");
  if (!f) return HC3D_ERR_IO;
  const double h = 6.62607015e-27, k = 1.380649e-16, c = 2.99792458e10;
  const double T[3] = {7500.0, 4000.0, 3000.0}, W[3] = {1.0e-14, 1.65e-13, 4.0e-13};
  std::fprintf(f, "# synthetic external radiation field: log10 nu[Hz]  log10 nu*F_nu[erg/s/cm^2]\n");
  const int n = 44;
  for (int i = 0; i < n; ++i) {
    const double lnu = 11.45 + (15.55 - 11.45) * i / (double)(n - 1), nu = std::pow(10.0, lnu);
    double s = 0.0;
    for (int q = 0; q < 3; ++q) {
      const double x = h * nu / (k * T[q]);
      if (x < 700.0) s += W[q] * 4.0 * hc3d::kPi * nu * (2.0 * h * nu * nu * nu / (c * c)) / std::expm1(x);
    }
    std::fprintf(f, " %.4f  %.4f\n", lnu, std::log10(std::max(s, 1.0e-300)));
  }
  std::fclose(f);
  return HC3D_OK;
}

extern "C" int hc3d_write_synthetic_draine(const char* dir) {
  // j_nu of grains heated by U times the ISRF: PAH bands (Gaussians in
  // lambda at 3.3, 6.2, 7.7, 8.6, 11.3, 12.7 um) plus a modified blackbody
  // nu^(3+2) / (exp(h nu / k T) - 1) at T = 18 K U^(1/6), both scaling with
  // U; 1000 rows, lambda log-spaced over 1-1000 um.
  if (!dir) return HC3D_ERR_INVALID;
  static const char* const names[hc3d::kNemit] = {"0.50", "1.00", "2.00", "5.00", "10.0", "20.0",
                                                 "30.0", "1e2",  "3e2",  "1e3",  "3e3",  "1e4",
                                                 "3e4",  "1e5",  "3e5",  "1e6",  "3e6",  "1e7"};
  static const double U[hc3d::kNemit] = {0.5, 1, 2, 5, 10, 20, 30, 1e2, 3e2, 1e3, 3e3, 1e4, 3e4, 1e5, 3e5, 1e6, 3e6, 1e7};
  const double band[6] = {3.3, 6.2, 7.7, 8.6, 11.3, 12.7}, width[6] = {0.04, 0.1, 0.3, 0.15, 0.2, 0.3},
               amp[6] = {0.5, 1.0, 2.0, 0.6, 1.2, 0.5};
  const double h = 6.62607015e-27, k = 1.380649e-16, c = 2.99792458e14;  // c in um/s
  for (int j = 0; j < hc3d::kNemit; ++j) {
    const std::string path = std::string(dir) + "/emit_draine_" + names[j] + ".dat";
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) return HC3D_ERR_IO;
    const double T = 18.0 * std::pow(U[j], 1.0 / 6.0);
    // the continuum's peak nu^5/(e^x - 1) sits near x = 4.97: normalise it to 1 there
    const double xpk = 4.965, nupk = xpk * k * T / h;
    const double cpk = std::pow(nupk, 5.0) / std::expm1(xpk);
    for (int i = 0; i < hc3d::kNdraine; ++i) {
      const double lam = std::pow(10.0, 3.0 * i / (double)(hc3d::kNdraine - 1));
      const double nu = c / lam, x = h * nu / (k * T);
      double cont = x < 700.0 ? std::pow(nu, 5.0) / std::expm1(x) / cpk : 0.0;
      double pah = 0.0;
      for (int b = 0; b < 6; ++b) pah += amp[b] * std::exp(-0.5 * std::pow((lam - band[b]) / width[b], 2.0));
      const double jnu = U[j] * (0.3 * pah + cont) * 1.0e-18 + 1.0e-40;
      std::fprintf(f, " %12.5f  %12.5e\n", lam, jnu);
    }
    std::fclose(f);
  }
  return HC3D_OK;
}

extern "C" int hc3d_write_wavelength_grid(const char* path, double tstar_k) {
  // 1321 log-spaced wavelengths over 0.0091-1e6 um (the span of the shipped
  // Kurucz tables); the flux column is the Planck function at tstar_k.
  FILE* f = std::fopen(path, "w");
  if (!f) return HC3D_ERR_IO;
  std::fprintf(f, "# synthetic wavelength grid, Planck Teff = %.1f K\n", tstar_k);
  const int n = 1321;
  for (int i = 0; i < n; ++i) {
    double lam = std::pow(10.0, std::log10(0.0091) + (std::log10(1.0e6) - std::log10(0.0091)) * i / (double)(n - 1));
    double x = 1.2398 / lam / (tstar_k / 11605.0);
    double b = x < 700.0 ? x * x * x / std::expm1(x) : 0.0;
    std::fprintf(f, " %14.4f  %.4e\n", lam, b);
  }
  std::fclose(f);
  return HC3D_OK;
}
