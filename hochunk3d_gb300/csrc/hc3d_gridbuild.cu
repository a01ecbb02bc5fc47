// hc3d_gridbuild.cu -- the densities of gridset (gridset.f90:954-1098) on
// the GPU: disk mass normalisation, per-cell species densities, cell volumes
// and (rho V)^(1/4), for a model whose walls, parameters, gap scale
// (rhogap0, gridset.f90:906-942) and fractal field the host set up.  Every
// disk structure option of densdiskg and the envelope gap are evaluated;
// a warped or spiral disk per azimuthal cell.  One thread per (r, theta) column of cells walks the
// azimuthal cells of that column, as the host loop does; the two mass sums
// are reduced per column and then over columns in a fixed order, so a run
// repeats bit for bit.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cuda_runtime.h>

#include "hc3d_model.h"

namespace hc3d {
namespace {

// the density parameters of a Model, copied by value into the kernels
struct DensParams {
  int nrg, ntg, npg;
  int idiskcurve, ienvtype, ihole, ipoly, ifractal;
  // species: 4, or 8 with the small grains; the disk species' ids (0, 1 and 4, 5)
  int ndg, ndisk, disk_id[4];
  int fractmask[HC3D_NDG];
  double rho0[HC3D_NDG], z1[HC3D_NDG], a[HC3D_NDG], b[HC3D_NDG], rmaxd[HC3D_NDG], rddust[HC3D_NDG];
  double fmass[HC3D_NDG];
  double rc, rhoe0, rmine, rmax, envexp, rhodens1, rhoamb;
  double c1e, ex1, z01, c2e, ex2, z02, rhoconst1, rhoconst2, exf;
  double r3;  // rmincgs^3
  // disk structure (densdiskg.f90:25-155) and the envelope gap (densenv.f90:52-58,114-119)
  int igapd, idiskwarp, nspot, irimcurve, irimpuff, igappuff, igapcurve, ispiral, sn, iradexp;
  double rgapd1, rgapd2, agap[HC3D_NDG], bgap[HC3D_NDG], rhogap0[HC3D_NDG], z1gap[HC3D_NDG];
  double warpheight, wexp, warplength, rimcurveheight, rimcurvelength, rimcurveexp, rimheight, rimlength;
  double gapheight, gaplength, gapcurveheight, gapcurvelength, gapcurveexp;
  double sw, pitch, rspiral1, rspiral2, radexp;
  int igape, igapedens;
  double rgape1, rgape2, rhogape, fracte;
};

// zerod: the Ulrich cubic mu0^3 + (r/Rc - 1) mu0 - (r/Rc) mu = 0, closed form
// then three Newton steps, the root clamped to [0, 1] (as the host restatement)
__device__ double zerod_dev(double mu, double rx) {
  const double p = rx - 1.0, q = -rx * mu;
  double x;
  const double disc = 0.25 * q * q + p * p * p / 27.0;
  if (disc > 0.0) {
    const double sd = sqrt(disc);
    x = cbrt(-0.5 * q + sd) + cbrt(-0.5 * q - sd);
  } else if (p < 0.0) {
    const double r = sqrt(-p / 3.0);
    const double arg = fmax(-1.0, fmin(1.0, (3.0 * q) / (2.0 * p) * sqrt(-3.0 / p)));
    x = 2.0 * r * cos(acos(arg) / 3.0);
  } else {
    x = 0.0;
  }
  for (int k = 0; k < 3; ++k) {
    const double fx = x * x * x + p * x + q, d = 3.0 * x * x + p;
    if (d != 0.0) x -= fx / d;
  }
  return fmax(0.0, fmin(1.0, x));
}

// densdiskg.f90:1-155 at azimuth phi (species 0, 1): the flared disk with
// its gap and the gap's density law, warp, spiral arms, puffed and curved
// rim and gap wall, and radial cutoff -- the algebra of the host build
// (hc3d_model.cpp densdisk) term by term
__device__ double densdisk_dev(const DensParams& P, double rad, double sint, double cost, double phi, int id) {
  const double pi = 3.14159265358979323846;
  const double rp = rad * sint, zp = rad * cost;
  const double rcoord = P.idiskcurve == 1 ? rad : rp;
  const bool ingap = P.igapd == 1 && rcoord < P.rgapd2 && rcoord > P.rgapd1;
  const double adens = ingap ? P.agap[id] : P.a[id], bdens = ingap ? P.bgap[id] : P.b[id];
  const double rhodens = ingap ? P.rhogap0[id] : P.rho0[id], zscale = ingap ? P.z1gap[id] : P.z1[id];
  double warp = 0.0, warp2 = 0.0;
  if (P.idiskwarp == 1) {
    const double fall = exp(-pow((rcoord - P.rddust[id]) / P.warplength, 2.0));
    warp = (phi < pi ? 1.0 : -1.0) * P.warpheight * pow(cos(phi / 2.0), P.wexp) * fall;
    if (P.nspot == 2) warp2 = P.warpheight * pow(cos(phi / 2.0 - pi / 2.0), P.wexp) * fall;
  }
  double rimcurve = 0.0, rimpuff = 0.0, gappuff = 0.0, gapcurve = 0.0;
  if (P.irimcurve == 1)
    rimcurve = P.rimcurveheight * exp(-pow((rcoord - P.rddust[id]) / P.rimcurvelength, P.rimcurveexp));
  if (P.irimpuff == 1) rimpuff = P.rimheight * exp(-pow((rcoord - P.rddust[id]) / P.rimlength, 2.0));
  if (rcoord < P.rddust[id]) rimpuff = 0.0;
  if (P.igappuff == 1 && P.igapd == 1) gappuff = P.gapheight * exp(-pow((rcoord - P.rgapd2) / P.gaplength, 2.0));
  if (rcoord < P.rgapd2) gappuff = 0.0;
  if (P.igapcurve == 1 && P.igapd == 1)
    gapcurve = P.gapcurveheight * exp(-pow((rcoord - P.rgapd2) / P.gapcurvelength, P.gapcurveexp));
  if (rcoord < P.rgapd2) gapcurve = 0.0;
  double spiral = 1.0;
  if (P.ispiral == 1) {
    // single-precision factors and phase, integer power by squaring (as the host build)
    double sfact = 1.0;
    for (int is = 2; is <= P.sn; is += 2) sfact = sfact * (double)((float)is / ((float)is - 1.0f));
    const double sx = sin(log(rcoord) / tan(P.pitch) - phi + (double)0.7854f);
    double sp = 1.0, xx = sx;
    for (unsigned u = (unsigned)P.sn; u;) {
      if (u & 1u) sp *= xx;
      u >>= 1;
      if (u) xx *= xx;
    }
    spiral = 1.0 - P.sw + sfact * P.sw * sp;
    if (rcoord < P.rspiral1 || rcoord > P.rspiral2) spiral = 1.0;
  }
  double zmr = zscale * pow(rcoord, bdens);
  double densfact1 = 1.0;
  if (phi < pi / 2.0 || phi > 3.0 * pi / 2.0) {
    if (zp > 0.0) zmr = zmr * (1.0 + warp);
    densfact1 = 1.0 / (1.0 + warp);
  } else {
    if (zp < 0.0) zmr = zmr * (1.0 + warp2);
    densfact1 = 1.0 / (1.0 + warp2);
  }
  const double puff = 1.0 + rimpuff + gappuff - rimcurve - gapcurve;
  const double densfact = 1.0 / puff * densfact1;
  zmr = zmr * puff;
  if (rcoord > P.rmaxd[id] || rhodens == 0.0 || rcoord < P.rddust[id] || zmr < 1.e-10) return 0.0;
  const double gexp = (zp / zmr) * (zp / zmr);
  double dens;
  if (gexp > 1.e-15) {
    if (gexp < 120.0) dens = densfact * spiral * rhodens * pow(rcoord, -adens) * exp(-0.5 * gexp);
    else dens = 0.0;
  } else {
    dens = densfact * spiral * rhodens * pow(rcoord, -adens);
  }
  if (P.iradexp == 1) dens = dens * exp(-rcoord / P.radexp);
  return dens;
}

// densenv.f90:1-128: Ulrich envelope or power law with a polynomial bipolar
// cavity; id 2 is the envelope, 3 the cavity
__device__ double densenv_dev(const DensParams& P, double rad, double costin, double sina, int id) {
  const double cosa = fabs(costin);
  const double rp = rad * sina, zp = rad * cosa;
  const double zup = P.c1e * pow(rp, P.ex1) + P.z01;
  const double xmu = zp / rad;
  double dens = 0.0;
  int inhole = 0;
  if (rad > P.rmine) {
    if (P.ienvtype == 1) {
      const double rx = rad / P.rc;
      const double xmu0 = zerod_dev(xmu, rx);
      const double ratio = xmu0 > 0.0 ? xmu / xmu0 : 1.0;
      const double factor = 1.0 / (ratio + 2.0 * (xmu0 * xmu0) / rx);
      dens = P.rhoe0 * pow(rx, -1.5) * factor / sqrt(1.0 + ratio);
    } else {
      dens = P.rhodens1 * pow(rad, -P.envexp);
    }
  }
  // constant density in the envelope gap, before the ambient floor and the cavity
  const bool ingape = P.igape == 1 && rad < P.rgape2 && rad > P.rgape1;
  if (ingape && P.igapedens == 0) dens = P.rhogape;
  if (rad > P.rmine && dens < P.rhoamb) dens = P.rhoamb;
  if (P.ihole == 1 && P.ipoly == 1) {
    const double zlo = P.c2e * pow(rp, P.ex2) + P.z02;
    if (zp > zlo) {
      inhole = 1;
      dens = P.rhoconst2 * pow(rad, -P.exf);
    }
    if (zp > zup) {
      inhole = 1;
      dens = P.rhoconst1 * pow(rad, -P.exf);
    }
  }
  if (ingape && P.igapedens == 1) dens = dens * P.fracte;  // scaled density in the gap
  if (rad >= P.rmax) dens = 0.0;
  if (rad <= P.rmine) dens = 0.0;
  if (id % 4 == 3 && inhole == 0) dens = 0.0;
  if (id % 4 == 2 && inhole == 1) dens = 0.0;
  return dens;
}

struct Walls {
  const double *rarr, *ravearr, *thetarr, *thetavearr, *phiarr, *densvar;
};

// unnormalised disk mass of each column (every disk species), for diskscl
__global__ void k_disk_colmass(DensParams P, Walls w, double* colmass) {
  const int ncol = (P.nrg - 1) * (P.ntg - 1);
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const int ir = col % (P.nrg - 1), it = col / (P.nrg - 1);
  const double rad = w.ravearr[ir];
  const double dr3 = pow(w.rarr[ir + 1], 3.0) - pow(w.rarr[ir], 3.0);
  const double thet = w.thetavearr[it], cost = cos(thet), sint = sin(thet);
  const double dcost = cos(w.thetarr[it + 1]) - cos(w.thetarr[it]);
  const bool phidep = P.idiskwarp || P.ispiral;
  for (int k = 0; k < P.ndisk; ++k) {
    const int id = P.disk_id[k];
    double m = 0.0;
    if (P.rho0[id] != 0.0) {
      const double dd0 = phidep ? 0.0 : densdisk_dev(P, rad, sint, cost, 0.0, id);
      if (phidep || dd0 != 0.0)
        for (int ip = 0; ip < P.npg - 1; ++ip) {
          const double dd = phidep ? densdisk_dev(P, rad, sint, cost, 0.5 * (w.phiarr[ip] + w.phiarr[ip + 1]), id) : dd0;
          m += dd * (-dr3 * dcost * (w.phiarr[ip + 1] - w.phiarr[ip]) / 3.0 * P.r3);
        }
    }
    colmass[(size_t)k * ncol + col] = m;
  }
}

// sums[k] = sum over columns of v[k * n + col], one block, fixed order
__global__ void k_sum_columns(const double* v, int n, int nsum, double* sums) {
  __shared__ double part[256];
  for (int k = 0; k < nsum; ++k) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += v[(size_t)k * n + i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
      if ((int)threadIdx.x < h) part[threadIdx.x] += part[threadIdx.x + h];
      __syncthreads();
    }
    if (threadIdx.x == 0) sums[k] = part[0];
    __syncthreads();
  }
}

// densities, volumes and (rho V)^(1/4) of every cell of a column; per-column
// disk and envelope masses into colmass[0..1][col]
__global__ void k_density(DensParams P, Walls w, const double* diskscl, double* densarr, double* massarr,
                          double* vcell, double* colmass) {
  const int ncol = (P.nrg - 1) * (P.ntg - 1);
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const int ir = col % (P.nrg - 1), it = col / (P.nrg - 1);
  const int64_t n4 = (int64_t)P.nrg * P.ntg * P.npg;
  const double rad = w.ravearr[ir];
  const double dr3 = pow(w.rarr[ir + 1], 3.0) - pow(w.rarr[ir], 3.0);
  const double thet = w.thetavearr[it], cost = cos(thet), sint = sin(thet);
  const double dcost = cos(w.thetarr[it + 1]) - cos(w.thetarr[it]);
  double dens_r[HC3D_NDG];
  const bool phidep = P.idiskwarp || P.ispiral;
  for (int id = 0; id < P.ndg; ++id)
    dens_r[id] = id % 4 < 2 ? densdisk_dev(P, rad, sint, cost, 0.0, id) * diskscl[id]
                            : densenv_dev(P, rad, cost, sint, id) * P.fmass[id];
  double mdisk = 0.0, menv = 0.0;
  for (int ip = 0; ip < P.npg - 1; ++ip) {
    if (phidep)
      for (int k = 0; k < P.ndisk; ++k) {
        const int id = P.disk_id[k];
        dens_r[id] = densdisk_dev(P, rad, sint, cost, 0.5 * (w.phiarr[ip] + w.phiarr[ip + 1]), id) * diskscl[id];
      }
    const double vol = -dr3 * dcost * (w.phiarr[ip + 1] - w.phiarr[ip]) / 3.0 * P.r3;
    const int64_t c = (int64_t)ir + (int64_t)P.nrg * (it + (int64_t)P.ntg * ip);
    vcell[c] = vol;
    for (int id = 0; id < P.ndg; ++id) {
      double d = dens_r[id];
      if (P.ifractal && P.fractmask[id] == 1)
        d *= w.densvar[ir + (int64_t)(P.nrg - 1) * (it + (int64_t)(P.ntg - 1) * ip)];
      densarr[c + n4 * id] = d;
      massarr[c + n4 * id] = pow(d * vol, 0.25);
      if (id % 4 < 2) mdisk += d * vol;
      else menv += d * vol;
    }
  }
  colmass[col] = mdisk;
  colmass[(size_t)ncol + col] = menv;
}

// ---- the fractal factor (CFRACTAL=YES) --------------------------------------
// the clump centres of every level, drawn in their one sequence by one thread
__global__ void k_fractal_points(int nr, int nt, int np, int fractn, int fractlev, int64_t ifseed, double* buf) {
  if (blockIdx.x == 0 && threadIdx.x == 0) fractal_generate(nr, nt, np, fractn, fractlev, ifseed, buf);
}

// one block per clump centre: the cells of its box inside the clump set
// their bit of the cell set; count receives the number of bits newly set
__global__ void k_fractal_mark(const double* pts, int npts, int nr, int nt, int np, double rad, unsigned* bits,
                               unsigned long long* count) {
  const int c = blockIdx.x;
  if (c >= npts) return;
  const double r = pts[3 * c], t = pts[3 * c + 1], p = pts[3 * c + 2];
  const FractalBox B = fractal_box(nr, nt, np, rad, r, t, p);
  const int64_t nbr = B.r1 - B.r0 + 1, nbt = B.t1 - B.t0 + 1, nbp = B.p1 - B.p0 + 1;
  const int64_t nbox = nbr > 0 && nbt > 0 && nbp > 0 ? nbr * nbt * nbp : 0;
  for (int64_t q0 = 0; q0 < nbox; q0 += blockDim.x) {
    const int64_t q = q0 + threadIdx.x;
    bool fresh = false;
    if (q < nbox) {
      const int ir = B.r0 + (int)(q % nbr);
      const int it = B.t0 + (int)((q / nbr) % nbt);
      const int ipp = B.p0 + (int)(q / (nbr * nbt));
      if (fractal_inside(B, ir, it, ipp, r, t, p)) {
        const int ip = ((ipp % np) + np) % np;
        const int64_t k = ir + (int64_t)nr * (it + (int64_t)nt * ip);
        const unsigned bit = 1u << (k & 31);
        fresh = (atomicOr(bits + (k >> 5), bit) & bit) == 0u;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, fresh);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, (unsigned long long)__popc(m));
  }
}

// densvar: a in the marked cells, b elsewhere
__global__ void k_fractal_fill(const unsigned* bits, int64_t nc, double a, double b, double* densvar) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nc; k += (int64_t)gridDim.x * blockDim.x)
    densvar[k] = ((bits[k >> 5] >> (k & 31)) & 1u) ? a : b;
}

struct DevBufs {
  std::vector<void*> p;
  ~DevBufs() {
    for (void* q : p) cudaFree(q);
  }
  template <class T>
  T* alloc(size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, n * sizeof(T) + 16) != cudaSuccess) return nullptr;
    p.push_back(q);
    return static_cast<T*>(q);
  }
};

}  // namespace

// The densities of gridset on device `device`; replaces m.densarr, massarr,
// vcell, massdisk, massenv and ndg_active.  ms receives the device time.
int densities_gpu(Model& m, int device, double* ms, std::string* err) {
  if (cudaSetDevice(device) != cudaSuccess) { *err = "no CUDA device"; return HC3D_ERR_CUDA; }
  const int nrg = m.nrg, ntg = m.ntg, npg = m.npg;
  const int ncol = (nrg - 1) * (ntg - 1);
  const int64_t n4 = m.n4();
  if ((m.ndg != 4 && m.ndg != 8) || ncol <= 0 || m.densarr.size() != (size_t)n4 * m.ndg) {
    *err = "model grid not built";
    return HC3D_ERR_STATE;
  }
  const int ndg = m.ndg;
  DensParams P;
  std::memset(&P, 0, sizeof P);
  P.nrg = nrg; P.ntg = ntg; P.npg = npg;
  P.idiskcurve = m.idiskcurve; P.ienvtype = m.ienvtype; P.ihole = m.ihole; P.ipoly = m.ipoly;
  P.ifractal = m.ifractal;
  P.ndg = ndg;
  P.ndisk = ndg == 8 ? 4 : 2;
  P.disk_id[0] = 0; P.disk_id[1] = 1; P.disk_id[2] = 4; P.disk_id[3] = 5;
  for (int id = 0; id < HC3D_NDG; ++id) {
    P.fractmask[id] = m.fractmask[id]; P.fmass[id] = m.fmass[id];
    P.rho0[id] = m.rho0[id]; P.z1[id] = m.z1[id]; P.a[id] = m.a[id]; P.b[id] = m.b[id];
    P.rmaxd[id] = m.rmaxd[id]; P.rddust[id] = m.rddust[id];
    P.agap[id] = m.agap[id]; P.bgap[id] = m.bgap[id]; P.rhogap0[id] = m.rhogap0[id]; P.z1gap[id] = m.z1gap[id];
  }
  P.rc = m.rc; P.rhoe0 = m.rhoe0; P.rmine = m.rmine; P.rmax = m.rmax; P.envexp = m.envexp;
  P.rhodens1 = m.rhodens1; P.rhoamb = m.rhoamb;
  P.c1e = m.c1e; P.ex1 = m.ex1; P.z01 = m.z01; P.c2e = m.c2e; P.ex2 = m.ex2; P.z02 = m.z02;
  P.rhoconst1 = m.rhoconst1; P.rhoconst2 = m.rhoconst2; P.exf = m.exf;
  P.igapd = m.igapd; P.idiskwarp = m.idiskwarp; P.nspot = m.nspot; P.irimcurve = m.irimcurve;
  P.irimpuff = m.irimpuff; P.igappuff = m.igappuff; P.igapcurve = m.igapcurve; P.ispiral = m.ispiral;
  P.sn = m.sn; P.iradexp = m.iradexp;
  P.rgapd1 = m.rgapd1; P.rgapd2 = m.rgapd2;
  P.warpheight = m.warpheight; P.wexp = m.wexp; P.warplength = m.warplength;
  P.rimcurveheight = m.rimcurveheight; P.rimcurvelength = m.rimcurvelength; P.rimcurveexp = m.rimcurveexp;
  P.rimheight = m.rimheight; P.rimlength = m.rimlength; P.gapheight = m.gapheight; P.gaplength = m.gaplength;
  P.gapcurveheight = m.gapcurveheight; P.gapcurvelength = m.gapcurvelength; P.gapcurveexp = m.gapcurveexp;
  P.sw = m.sw; P.pitch = m.pitch; P.rspiral1 = m.rspiral1; P.rspiral2 = m.rspiral2; P.radexp = m.radexp;
  P.igape = m.igape; P.igapedens = m.igapedens; P.rgape1 = m.rgape1; P.rgape2 = m.rgape2;
  P.rhogape = m.rhogape; P.fracte = m.fracte;
  const double rmincgs = m.rstar * kRsun;
  P.r3 = std::pow(rmincgs, 3.0);
  DevBufs B;
  double *d_r = B.alloc<double>(nrg), *d_ra = B.alloc<double>(nrg), *d_t = B.alloc<double>(ntg),
         *d_ta = B.alloc<double>(ntg), *d_p = B.alloc<double>(npg);
  const int nr1 = nrg - 1, nt1 = ntg - 1, np1 = npg - 1;
  const int64_t nc = (int64_t)nr1 * nt1 * np1;
  const size_t nvar = m.ifractal ? (size_t)nc : 1;
  double* d_var = B.alloc<double>(nvar);
  // the fractal factor's clump centres (all levels) and cell set
  const int fr_total = m.ifractal ? fractal_total(m.fractn, m.fractlev) : 1;
  int fr_last = m.fractn;
  for (int lev = 2; lev <= m.fractlev; ++lev) fr_last *= m.fractn / 8 + 1;
  double* d_pts = B.alloc<double>(3 * (size_t)fr_total);
  unsigned* d_bits = B.alloc<unsigned>(m.ifractal ? (size_t)(nc + 31) / 32 : 1);
  unsigned long long* d_cnt = B.alloc<unsigned long long>(1);
  if (!d_pts || !d_bits || !d_cnt) {
    *err = "device allocation failed";
    return HC3D_ERR_NOMEM;
  }
  // d_s: the column sums [0, 8), then diskscl [8, 16)
  double *d_dens = B.alloc<double>((size_t)n4 * ndg), *d_mass = B.alloc<double>((size_t)n4 * ndg),
         *d_vol = B.alloc<double>((size_t)n4), *d_col = B.alloc<double>((size_t)4 * ncol), *d_s = B.alloc<double>(16);
  if (!d_r || !d_ra || !d_t || !d_ta || !d_p || !d_var || !d_dens || !d_mass || !d_vol || !d_col || !d_s) {
    *err = "device allocation failed";
    return HC3D_ERR_NOMEM;
  }
  auto up = [](double* d, const std::vector<double>& h, size_t n) {
    return cudaMemcpy(d, h.data(), sizeof(double) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  };
  if (!up(d_r, m.rarr, nrg) || !up(d_ra, m.ravearr, nrg - 1) || !up(d_t, m.thetarr, ntg) ||
      !up(d_ta, m.thetavearr, ntg - 1) || !up(d_p, m.phiarr, npg)) {
    *err = "upload failed";
    return HC3D_ERR_CUDA;
  }
  // zero the wall-index entries (ir = nrg, it = ntg, ip = npg) as the host arrays have them
  cudaMemset(d_dens, 0, sizeof(double) * n4 * ndg);
  cudaMemset(d_mass, 0, sizeof(double) * n4 * ndg);
  cudaMemset(d_vol, 0, sizeof(double) * n4);
  Walls w{d_r, d_ra, d_t, d_ta, d_p, d_var};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int threads = 128, blocks = (ncol + threads - 1) / threads;
  cudaEventRecord(e0);
  // The fractal factor: the clump centres, then the clump radius by
  // bisection to the volume fraction of the factors (each step marks the
  // cells inside the clumps and counts them), then the factor of each cell.
  // The same steps as the host build, so the same cells are marked.
  if (m.ifractal) {
    k_fractal_points<<<1, 32>>>(nr1, nt1, np1, m.fractn, m.fractlev, m.ifseed, d_pts);
    const double* pts = d_pts + 3 * (size_t)(fr_total - fr_last);
    bool ok = true;
    auto mark = [&](double rad) -> int64_t {
      unsigned long long n = 0;
      ok = ok && cudaMemset(d_bits, 0, sizeof(unsigned) * (size_t)((nc + 31) / 32)) == cudaSuccess &&
           cudaMemset(d_cnt, 0, sizeof(unsigned long long)) == cudaSuccess;
      k_fractal_mark<<<fr_last, 256>>>(pts, fr_last, nr1, nt1, np1, rad, d_bits, d_cnt);
      ok = ok && cudaMemcpy(&n, d_cnt, sizeof n, cudaMemcpyDeviceToHost) == cudaSuccess;
      return (int64_t)n;
    };
    const double fv_target = fractal_target(m);
    double lo = 0.0, hi = 0.5;
    for (int k = 0; k < 30; ++k) {
      const double mid = 0.5 * (lo + hi);
      if ((double)mark(mid) / (double)nc < fv_target) lo = mid; else hi = mid;
    }
    const double fv = std::max((double)mark(hi) / (double)nc, 1.0 / (double)nc);
    double fa, fb;
    fractal_factors(m, fv, &fa, &fb);
    k_fractal_fill<<<(int)std::min<int64_t>((nc + 255) / 256, 4096), 256>>>(d_bits, nc, fa, fb, d_var);
    if (!ok || cudaGetLastError() != cudaSuccess) {
      *err = "fractal factor kernels failed";
      return HC3D_ERR_CUDA;
    }
  }
  // disk mass normalisation: diskscl = massd * fmass / mass on the grid
  double diskscl[HC3D_NDG] = {1, 1, 1, 1, 1, 1, 1, 1};
  if (m.massd > 0.0) {
    k_disk_colmass<<<blocks, threads>>>(P, w, d_col);
    k_sum_columns<<<1, 256>>>(d_col, ncol, P.ndisk, d_s);
    double tm[4];
    if (cudaMemcpy(tm, d_s, sizeof(double) * P.ndisk, cudaMemcpyDeviceToHost) != cudaSuccess) {
      *err = "disk mass reduction failed";
      return HC3D_ERR_CUDA;
    }
    for (int k = 0; k < P.ndisk; ++k) {
      const int id = P.disk_id[k];
      if (m.rho0[id] == 0.0) continue;
      const double tmp = tm[k] / kMsun;
      if (tmp > 0.0) diskscl[id] = m.massd * m.fmass[id] / tmp;
    }
  }
  cudaMemcpy(d_s + 8, diskscl, sizeof(diskscl), cudaMemcpyHostToDevice);
  k_density<<<blocks, threads>>>(P, w, d_s + 8, d_dens, d_mass, d_vol, d_col);
  k_sum_columns<<<1, 256>>>(d_col, ncol, 2, d_s);
  cudaEventRecord(e1);
  if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    *err = "density kernels failed";
    return HC3D_ERR_CUDA;
  }
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ms) *ms = t;
  double sums[2];
  if (m.ifractal) {
    m.densvar.resize((size_t)nc);
    if (cudaMemcpy(m.densvar.data(), d_var, sizeof(double) * nc, cudaMemcpyDeviceToHost) != cudaSuccess) {
      *err = "download failed";
      return HC3D_ERR_CUDA;
    }
  }
  m.densarr.resize((size_t)n4 * ndg);
  m.massarr.resize((size_t)n4 * ndg);
  m.vcell.resize((size_t)n4);
  if (cudaMemcpy(m.densarr.data(), d_dens, sizeof(double) * n4 * ndg, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(m.massarr.data(), d_mass, sizeof(double) * n4 * ndg, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(m.vcell.data(), d_vol, sizeof(double) * n4, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(sums, d_s, sizeof(sums), cudaMemcpyDeviceToHost) != cudaSuccess) {
    *err = "download failed";
    return HC3D_ERR_CUDA;
  }
  m.massdisk = sums[0] / kMsun;
  m.massenv = sums[1] / kMsun;
  m.ndg_active = 0;
  for (int id = 0; id < m.ndg; ++id) {
    bool any = false;
    for (int64_t k = 0; k < n4 && !any; ++k) any = m.densarr[k + n4 * id] > 0.0;
    if (any) m.ndg_active++;
  }
  return HC3D_OK;
}

}  // namespace hc3d

extern "C" int hc3d_model_densities_gpu(hc3d_model* mdl, int device, double* ms, char* err, size_t errlen) {
  if (!mdl) return HC3D_ERR_INVALID;
  std::string e;
  const int r = hc3d::densities_gpu(mdl->m, device, ms, &e);
  if (r && err && errlen) std::snprintf(err, errlen, "%s", e.c_str());
  return r;
}
