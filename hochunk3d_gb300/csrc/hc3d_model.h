// hc3d_model.h -- host model: the data newtts.F90 builds before calling disk().
#pragma once

#include <cmath>
#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "../../include/hc3d.h"
#include "../../include/hc3d_host.h"

namespace hc3d {

// physical constants, constants.f90:11-26
constexpr double kPi = 3.1415926535897932384626433;
constexpr double kR2p = 2.0 * kPi;
constexpr double kPiHalf = 0.5 * kPi;
constexpr double kRsun = 6.9598e10;
constexpr double kMsun = 1.989e33;
constexpr double kLsun = 3.839e33;
constexpr double kGn = 6.67428e-8;
constexpr double kSigt = 5.670400e-5;
constexpr double kBoltz = 1.3806503e-16;
constexpr double kMH = 1.67262158e-24;
constexpr double kC = 2.99792458e10;
constexpr double kAu = 1.49598e13;
constexpr double kPc = 3.0857e18;

// ".par" file: value = KEY = comment (configuration.f90:28-56)
class ParFile {
 public:
  bool load(const std::string& path, std::string* err);
  bool has(const std::string& key) const { return kv_.count(key) != 0; }
  bool str(const std::string& key, std::string* out, std::string* err) const;
  bool real(const std::string& key, double* out, std::string* err) const;
  bool integer(const std::string& key, int64_t* out, std::string* err) const;  // YES/NO -> 1/0
  bool reals(const std::string& key, std::vector<double>* out, std::string* err) const;
  bool ints(const std::string& key, std::vector<int64_t>* out, std::string* err) const;

 private:
  std::map<std::string, std::string> kv_;
};

constexpr int kNisrf = 200;  // isrf_mod nisrf
constexpr int kNemit = 18;     // draine_mod nemit: mean-intensity ratios of the small-grain spectra
constexpr int kNdraine = 1000; // draine_mod ndraine: frequencies of each spectrum
constexpr int kNtab = 100;   // tabl_mod ntab (module not shipped; restated)

struct Model {
  // ---- reapar/setup scalars (units after setup.f90) ----
  int64_t np = 0, npmin = 0, np_lucy = 0;
  int nimin = 0, nimax = 0, ipeel = 0, ilucy = 1, limb = 0, iplanckst = 1;
  double rstar = 1, tstar_k = 4000, massc = 0.5, massd = 0;
  double rmax = 0, rmaxi = 0, rc = 0, rate = 0, rhoamb = 0;
  double rmine = 0, rminsub = 0, autors = 1, rddustmin = 0;
  double rmaxd[HC3D_NDG] = {0}, rddust[HC3D_NDG] = {0};
  double z1[HC3D_NDG] = {0}, a[HC3D_NDG] = {0}, b[HC3D_NDG] = {0}, fmass[HC3D_NDG] = {0}, rho0[HC3D_NDG] = {0};
  int ihole = 0, ipoly = 1, istream = 0, ienvtype = 1;
  double thet1 = 0, thet2 = 0, ex1 = 1, ex2 = 1, z01 = 0, z02 = 0, exf = 0, rhoconst1 = 0, rhoconst2 = 0;
  double c1e = 0, c2e = 0, rhoe0 = 0, rhodens1 = 0, envexp = 0;
  int idiskcurve = 0;
  int ifractal = 0, fractlev = 3, fractn = 32;
  double densratio = 0.5, fractcontrast = 100.0;
  int fractmask[HC3D_NDG] = {0};
  int64_t ifseed = 0;
  int nfreq = 0, nmu = 0, nph = 0, nap = 0, npeel = 0, nxhst = 0;
  std::vector<double> thete, phie, aperture2;
  double numin = 0, numax = 0;
  double ltot = 0;
  double massdisk = 0, massenv = 0;
  double density_host_ms = 0;  // wall time of the host density build, the fractal factor included
  double tables_host_ms = 0;   // wall time of the host setemiss tables
  // external illumination (COUTILLUM, ISRF_SCL, ISRF_AV; isrf_mod)
  int iout = 0;
  double isrf_scl = 1.0, isrf_av = 0.0, isrf_int = 0.0;
  double lstar = 0, l_isrf = 0, isrf_frac = 0;
  std::string isrf_file;
  std::vector<double> isrf_cdfv, isrf_logcdf, isrf_logfreq;
  // disk structure of densdiskg (densdiskg.f90:25-155): gap, spiral arms,
  // warp, puffed and curved inner rim and outer gap wall, radial cutoff
  int igapd = 0, ispiral = 0, idiskwarp = 0, irimpuff = 0, igappuff = 0, irimcurve = 0, igapcurve = 0, iradexp = 0;
  double rgapd1 = 0, rgapd2 = 0;
  double z1gap[HC3D_NDG] = {0}, agap[HC3D_NDG] = {0}, bgap[HC3D_NDG] = {0}, rhoscale_gap[HC3D_NDG] = {0},
         rhogap0[HC3D_NDG] = {0};
  double pitch = 0, sw = 0, rspiral1 = 0, rspiral2 = 0;
  int sn = 0, nspot = 1;
  double warpheight = 0, wexp = 0, warplength = 1;
  double rimheight = 0, rimlength = 1, gapheight = 0, gaplength = 1;
  double rimcurveheight = 0, rimcurvelength = 1, rimcurveexp = 1;
  double gapcurveheight = 0, gapcurvelength = 1, gapcurveexp = 1;
  double radexp = 1;
  // envelope gap (CGAPE, densenv.f90:52-58,114-119): constant density rhogape,
  // or the envelope density scaled by fracte, between rgape1 and rgape2
  int igape = 0, igapedens = 0;
  double rgape1 = 0, rgape2 = 0, fracte = 1, rhogape = 0;
  bool disk_depends_on_phi() const { return idiskwarp || ispiral; }
  // disk accretion and stellar hot spots (reapar.f90:275-312, gridset.f90:72-270, spotset.f90:179-206)
  int idiskacc = 0, ialpha = 0, ispot = 0, itemp = 0, irminsub = 0;
  double alphad = 0, mdotdisk = 0, rtrunc = 5, spotlat = 0, tspot = 0, fspot = 1;
  double rmine_in = 0, rmind_in[2] = {0, 0};
  double mdotcgs[2] = {0, 0}, mdot_cgs = 0, lacc = 0, lacc2 = 0, accfrac = 0, accfrac2 = 0;
  double tshock_k = 0, thspot_deg = 0, tave_k = 0, rmaxdmax = 0;
  hc3d_sources src{};
  bool has_sources() const { return idiskacc || ispot; }
  // very small grains and PAHs (FSG(1..4) > 0): species 5-8 of the reference
  // numbering (grid_mod.f90:13-20) hold the small-grain share of disk 1,
  // disk 2, envelope and cavity; they re-emit from the emission spectra of
  // draine_cdf.f90 (18 mean-intensity ratios x 1000 frequencies) instead of
  // at a temperature.  isrfkap_int is the ISRF weighted by the small grains'
  // absorption opacity (isrf_cdf.f90:191-214), the unit of int_mean's ratio.
  double fsg[4] = {0, 0, 0, 0};
  bool has_sg() const { return fsg[0] > 0.0 || fsg[1] > 0.0 || fsg[2] > 0.0 || fsg[3] > 0.0; }
  int slot_species[4] = {1, 2, 3, 4};  // the species (1..8) each device slot holds
  std::vector<double> sg_cdf, sg_logcdf;  // (nemit,ndraine) Fortran order
  std::vector<double> sg_logfreq, sg_uratio;  // (ndraine), (nemit)
  double isrfkap_int = 0.0;
  int sg_slot = -1;  // the first device slot holding small grains; -1 = none
  std::vector<double> isrf_pdf, isrf_fhz;  // the ISRF's pdf on its 200 frequencies in Hz
  // limb-darkening table (tabl_mod) for CLIMB=YES
  std::vector<double> limb_xmu, limb_prob;
  int image = 1;
  int imcube = 0;  // IMCUBE: the per-frequency image cube of the peeled packets
  int64_t maxint = 1000000;
  uint64_t seed = 0;
  std::string atname, pardir;
  std::string dustname[HC3D_NDG];

  // ---- dust_mod ----
  int ndg = 0;  // slots carried across the boundary
  int nlammax = 1001;
  std::vector<int> nlambda;
  std::vector<double> nudust, kappad, adust, gdust, pldust, lamdust, kappav;
  int nT = 1000, nnu = 1025;
  std::vector<double> lTint, nuint, kapBint, kappap;
  double tsub_k = 1600.0;
  std::vector<double> hnuint, atmosnu, lognu, loghnu;

  // ---- grid_mod ----
  int nrg = 0, ntg = 0, npg = 0;
  std::vector<double> rarr, r2arr, ravearr, thetarr, costarr, sintarr, tan2arr, thetavearr, phiarr, aarr, barr;
  std::vector<double> densarr, massarr, vcell, tdust;
  std::vector<double> densvar;
  int ndg_active = 0;

  hc3d_dust_tables tables_view() const;
  hc3d_grid grid_view() const;
  hc3d_run_params params_view() const;  // pointers into this model
  // n_acc, n_spot, n_star and sources of p for an iteration of np_total packets
  void set_shares(hc3d_run_params* p, int64_t np_total) const;
  hc3d_model_info info() const;
  int64_t ncells() const { return (int64_t)(nrg - 1) * (ntg - 1) * (npg - 1); }
  int64_t n4() const { return (int64_t)nrg * ntg * npg; }
};

// The project fractal generator (CFRACTAL=YES): clump centres, the cell box
// of one clump, its inside test, the bisection's target volume fraction and
// the density factors (shared by the host build and hc3d_gridbuild.cu).
struct FractalBox {
  double cr, ct, cp;       // clump radius in cells along r, theta, phi
  int r0, r1, t0, t1, p0, p1;  // cell range (r, theta clamped; phi wraps)
};
std::vector<double> fractal_points(const Model& m);
void fractal_field(Model* m);  // densvar of the host build
double fractal_target(const Model& m);
void fractal_factors(const Model& m, double fv, double* a, double* b);
#ifdef __CUDACC__
#define HC3D_HD __host__ __device__
#else
#define HC3D_HD
#endif
// double arithmetic rounded operation by operation on host and device (the
// device would otherwise contract a * b + c into one rounding)
HC3D_HD inline double fr_add(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
HC3D_HD inline double fr_mul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
// splitmix64 and a uniform in (0, 1) from its top 53 bits
HC3D_HD inline uint64_t fractal_splitmix(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
HC3D_HD inline double fractal_u01(uint64_t* s) {
  return fr_mul((double)(fractal_splitmix(s) >> 11) + 0.5, 1.0 / 9007199254740992.0);
}
// centres of every level, level by level: fractn at level 1, fractn/8+1
// children per centre at each next level, spread 0.25 of the index ranges
// shrinking by 0.35 per level; returns the number of centres written to
// buf (3 doubles each); the last level's are the final
// fractn * (fractn/8+1)^(fractlev-1)
HC3D_HD inline int fractal_generate(int nr, int nt, int np, int fractn, int fractlev, int64_t ifseed, double* buf) {
  uint64_t s = (uint64_t)ifseed * 0x2545F4914F6CDD1Dull + 12345;
  int n = 0;
  for (int k = 0; k < fractn; ++k, ++n) {
    buf[3 * n] = fr_mul(fractal_u01(&s), nr);
    buf[3 * n + 1] = fr_mul(fractal_u01(&s), nt);
    buf[3 * n + 2] = fr_mul(fractal_u01(&s), np);
  }
  int beg = 0, cnt = fractn;
  double spread = 0.25;
  for (int lev = 2; lev <= fractlev; ++lev) {
    const int nb = n;
    for (int c = beg; c < beg + cnt; ++c)
      for (int k = 0; k < fractn / 8 + 1; ++k, ++n) {
        const double ds = fr_mul(2.0, spread);
        buf[3 * n] = fr_add(buf[3 * c], fr_mul(fr_mul(fr_add(fractal_u01(&s), -0.5), ds), nr));
        buf[3 * n + 1] = fr_add(buf[3 * c + 1], fr_mul(fr_mul(fr_add(fractal_u01(&s), -0.5), ds), nt));
        buf[3 * n + 2] = fr_add(buf[3 * c + 2], fr_mul(fr_mul(fr_add(fractal_u01(&s), -0.5), ds), np));
      }
    beg = nb;
    cnt = n - nb;
    spread *= 0.35;
  }
  return n;
}
// centres of all levels of fractal_generate: fractn (1 + m + m^2 + ...), m = fractn/8+1
HC3D_HD inline int fractal_total(int fractn, int fractlev) {
  int n = fractn, lvl = fractn;
  for (int lev = 2; lev <= fractlev; ++lev) { lvl *= fractn / 8 + 1; n += lvl; }
  return n;
}
// The cells of clump radius rad (a fraction of each index range) around
// centre (r, t, p): the box the radius spans (at least half a cell).
HC3D_HD inline FractalBox fractal_box(int nr, int nt, int np, double rad, double r, double t, double p) {
  FractalBox b;
  b.cr = fmax(0.5, fr_mul(rad, nr)); b.ct = fmax(0.5, fr_mul(rad, nt)); b.cp = fmax(0.5, fr_mul(rad, np));
  const int r0 = (int)floor(r - b.cr), r1 = (int)ceil(r + b.cr), t0 = (int)floor(t - b.ct), t1 = (int)ceil(t + b.ct);
  b.r0 = r0 > 0 ? r0 : 0; b.r1 = r1 < nr - 1 ? r1 : nr - 1;
  b.t0 = t0 > 0 ? t0 : 0; b.t1 = t1 < nt - 1 ? t1 : nt - 1;
  b.p0 = (int)floor(p - b.cp); b.p1 = (int)ceil(p + b.cp);
  return b;
}

// the inside test of cell (ir, it, ipp) for the clump of box B and centre
// (r, t, p): dr^2 + dt^2 + dp^2 <= 1 on the cell centre, each product and
// sum rounded on its own
HC3D_HD inline bool fractal_inside(const FractalBox& B, int ir, int it, int ipp, double r, double t, double p) {
#ifdef __CUDA_ARCH__
  const double dr = __ddiv_rn(__dsub_rn(__dadd_rn((double)ir, 0.5), r), B.cr);
  const double dt = __ddiv_rn(__dsub_rn(__dadd_rn((double)it, 0.5), t), B.ct);
  const double dp = __ddiv_rn(__dsub_rn(__dadd_rn((double)ipp, 0.5), p), B.cp);
  return __dadd_rn(__dadd_rn(__dmul_rn(dr, dr), __dmul_rn(dt, dt)), __dmul_rn(dp, dp)) <= 1.0;
#else
  const double dr = ((double)ir + 0.5 - r) / B.cr, dt = ((double)it + 0.5 - t) / B.ct,
               dp = ((double)ipp + 0.5 - p) / B.cp;
  const double x = dr * dr, y = dt * dt, z = dp * dp;
  return (x + y) + z <= 1.0;
#endif
}

// setup.f90 + reapar.f90 + dustinit + atmosinit + setup_wave + gridset
bool build_model(Model* m, const std::string& par_path, const std::string* par_dir, std::string* err);

// setemiss (dust.f90:394-474) for one species table, kapBint and kappap only
void setemiss_species(const Model& m, int id, double* kapB /*(nT,nnu)*/, double* kapp /*(nT)*/);

// densdisk (densdiskg.f90:1-155) and densenv (densenv.f90:1-128) for the
// options the benchmark models use
double densdisk(const Model& m, double rad, double sint, double cost, double phi, int id);
double densenv(const Model& m, double rad, double thetin, double costin, double sina, int id);
// zerod: the Ulrich streamline root mu0 (module not shipped; restated)
double zerod(double mu, double rx);

}  // namespace hc3d

// opaque handle of hc3d_host.h
struct hc3d_model {
  hc3d::Model m;
};
