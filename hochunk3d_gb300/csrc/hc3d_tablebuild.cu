// hc3d_tablebuild.cu -- setemiss (dust.f90:394-474) on the GPU: the
// cumulative emissivity tables kapBint(nT, nnu) and the Planck-mean factors
// kappap(nT) of every distinct dust table of a model.
//
// Layout of the work: one thread per (temperature, frequency interval)
// evaluates the Simpson integral of kappa_abs(nu) B_nu(T) over its interval
// (the integrand is the linear interpolation of kappa_abs between the two
// interval ends times the Planck function, as the host restatement); one
// thread per temperature row then forms the running sum over the intervals
// in the host's order and normalises the row.  The unit is compiled with
// separately rounded multiplies and adds, so the only differences from the
// host build are those of exp() between the two math libraries.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cuda_runtime.h>

#include "hc3d_model.h"

namespace hc3d {
namespace {

struct DustRow {
  const double *nud, *kap, *alb;  // nudust, kappad, adust of one table (descending nu)
  int nl;
};

// opacset for one table (dust.f90:9-80): kappa and albedo at nu by bisection
// and linear interpolation; clamped to the end values outside the table
__device__ void opac1(const DustRow& d, double nu, double* kappa, double* albedo) {
  if (nu >= d.nud[0]) {
    *kappa = d.kap[0];
    *albedo = d.alb[0];
  } else if (nu <= d.nud[d.nl - 1]) {
    *kappa = d.kap[d.nl - 1];
    *albedo = d.alb[d.nl - 1];
  } else {
    int i0 = 1, i1 = d.nl;
    while (i1 - i0 > 1) {
      const int i = (i1 + i0) / 2;
      if (nu <= d.nud[i - 1]) i0 = i;
      else i1 = i;
    }
    const double f = (nu - d.nud[i1 - 1]) / (d.nud[i0 - 1] - d.nud[i1 - 1]);
    const double fm1 = 1.0 - f;
    *kappa = fm1 * d.kap[i1 - 1] + f * d.kap[i0 - 1];
    *albedo = fm1 * d.alb[i1 - 1] + f * d.alb[i0 - 1];
  }
}

// exp(x) - 1 as the reference's Planck routine forms it: a degree-7
// polynomial for |x| <= ln 2, exp(x) - 1 beyond (the same coefficients as
// the host restatement)
__device__ double expm1_poly(double x) {
  const double c[7] = {0.9999999995, 0.4999999206, 0.1666653019, 0.0416573475,
                       0.0083013598, 0.0013298820, 0.0001413161};
  if (fabs(x) > 0.6931472) return exp(x) - 1.0;
  double s = 0.0;
#pragma unroll
  for (int i = 6; i >= 0; --i) s = x * (c[i] + s);
  return s;
}

// normalised Planck function in x = nu / T, 15/pi^4 x^3 / (e^x - 1)
__device__ double planck(double nu, double T) {
  const double x = nu / T;
  if (x == 0.0) return 0.0;
  return 0.1539897 * x * x * x / expm1_poly(x);
}

struct Segment {
  double k0, k1, nu0, dnu, T;
  __device__ double operator()(double f) const { return ((1.0 - f) * k0 + f * k1) * planck(nu0 + f * dnu, T); }
};

// qsimp/trapzd (nr.f:183-225) on [0, 1]: relative tolerance 1e-5, at most 20
// refinements, the last estimate when the tolerance is not met
__device__ double simpson01(const Segment& g) {
  const double EPS = 1.e-5;
  double ost = -1.e30, os = -1.e30, st = 0.0, s = 0.0;
  for (int j = 1; j <= 20; ++j) {
    if (j == 1) {
      st = 0.5 * (g(0.0) + g(1.0));
    } else {
      const int it = 1 << (j - 2);
      const double tnm = (double)it, del = 1.0 / tnm;
      double x = 0.5 * del, sum = 0.0;
      for (int k = 0; k < it; ++k) {
        sum += g(x);
        x += del;
      }
      st = 0.5 * (st + sum / tnm);
    }
    s = (4.0 * st - ost) / 3.0;
    if (fabs(s - os) < EPS * fabs(os)) return s;
    os = s;
    ost = st;
  }
  return s;
}

// one thread per (temperature i, interval j): dx * integral, into kapB[i + nT j]
__global__ void k_emiss_intervals(DustRow d, const double* lTint, const double* nuint, int nT, int nnu,
                                  double* kapB) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)nT * nnu) return;
  const int i = (int)(t % nT), j = (int)(t / nT);
  const double Teff = exp(lTint[i]);
  const double nu0 = j == 0 ? 0.0 : nuint[j - 1] * Teff;
  const double nu1 = nuint[j] * Teff;
  const double dnu = nu1 - nu0, dx = dnu / Teff;
  double kappa, albedo;
  opac1(d, nu0, &kappa, &albedo);
  const double k0 = (1.0 - albedo) * kappa;
  opac1(d, nu1, &kappa, &albedo);
  const double k1 = (1.0 - albedo) * kappa;
  double v = 0.0;
  if (nu0 / Teff < 50.0) v = simpson01(Segment{k0, k1, nu0, dnu, Teff});
  kapB[t] = dx * v;
}

// one thread per temperature row: running sum in interval order, kappap =
// the total, the row normalised to end at 1
__global__ void k_emiss_rows(int nT, int nnu, double* kapB, double* kapp) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nT) return;
  double acc = 0.0;
  for (int j = 0; j < nnu; ++j) {
    const size_t k = (size_t)i + (size_t)nT * j;
    acc = j == 0 ? kapB[k] : kapB[k] + acc;
    kapB[k] = acc;
  }
  kapp[i] = acc;
  for (int j = 0; j < nnu - 1; ++j) kapB[(size_t)i + (size_t)nT * j] /= acc;
  kapB[(size_t)i + (size_t)nT * (nnu - 1)] = 1.0;
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

struct Events {
  cudaEvent_t a = nullptr, b = nullptr;
  Events() {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  ~Events() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

}  // namespace

// setemiss of every distinct dust table of m on device `device`; slots that
// name the same file as an earlier slot copy its rows, as the host build
// does.  Replaces m.kapBint and m.kappap; ms receives the device time.
int tables_gpu(Model& m, int device, double* ms, std::string* err) {
  if (cudaSetDevice(device) != cudaSuccess) {
    *err = "no CUDA device";
    return HC3D_ERR_CUDA;
  }
  const int nT = m.nT, nnu = m.nnu, ndg = m.ndg;
  if (ndg <= 0 || nT < 2 || nnu < 2 || (int)m.lTint.size() != nT || (int)m.nuint.size() != nnu) {
    *err = "model dust tables not set up";
    return HC3D_ERR_STATE;
  }
  const size_t row = (size_t)nT * nnu, nl = (size_t)m.nlammax * ndg;
  DevBufs B;
  double *d_lT = B.alloc<double>(nT), *d_nu = B.alloc<double>(nnu), *d_nud = B.alloc<double>(nl),
         *d_kap = B.alloc<double>(nl), *d_alb = B.alloc<double>(nl), *d_kb = B.alloc<double>(row * ndg),
         *d_kp = B.alloc<double>((size_t)nT * ndg);
  if (!d_lT || !d_nu || !d_nud || !d_kap || !d_alb || !d_kb || !d_kp) {
    *err = "device allocation failed";
    return HC3D_ERR_NOMEM;
  }
  auto up = [](double* d, const std::vector<double>& h) {
    return cudaMemcpy(d, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice) == cudaSuccess;
  };
  if (!up(d_lT, m.lTint) || !up(d_nu, m.nuint) || !up(d_nud, m.nudust) || !up(d_kap, m.kappad) ||
      !up(d_alb, m.adust)) {
    *err = "upload failed";
    return HC3D_ERR_CUDA;
  }
  int same[HC3D_NDG];
  for (int id = 0; id < ndg; ++id) {
    same[id] = -1;
    for (int j = 0; j < id; ++j)
      if (m.dustname[j] == m.dustname[id]) {
        same[id] = j;
        break;
      }
  }
  Events ev;
  cudaEventRecord(ev.a);
  for (int id = 0; id < ndg; ++id) {
    if (same[id] >= 0) continue;
    const size_t off = (size_t)id * m.nlammax;
    DustRow d{d_nud + off, d_kap + off, d_alb + off, m.nlambda[id]};
    if (d.nl < 2) {
      *err = "dust table with fewer than two wavelengths";
      return HC3D_ERR_INVALID;
    }
    const int threads = 128;
    k_emiss_intervals<<<(unsigned)((row + threads - 1) / threads), threads>>>(d, d_lT, d_nu, nT, nnu,
                                                                               d_kb + row * id);
    k_emiss_rows<<<(nT + threads - 1) / threads, threads>>>(nT, nnu, d_kb + row * id, d_kp + (size_t)nT * id);
  }
  cudaEventRecord(ev.b);
  if (cudaEventSynchronize(ev.b) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    *err = "table kernels failed";
    return HC3D_ERR_CUDA;
  }
  float t = 0.f;
  cudaEventElapsedTime(&t, ev.a, ev.b);
  if (ms) *ms = t;
  m.kapBint.resize(row * ndg);
  m.kappap.resize((size_t)nT * ndg);
  for (int id = 0; id < ndg; ++id) {
    const int src = same[id] >= 0 ? same[id] : id;
    if (cudaMemcpy(&m.kapBint[row * id], d_kb + row * src, sizeof(double) * row, cudaMemcpyDeviceToHost) !=
            cudaSuccess ||
        cudaMemcpy(&m.kappap[(size_t)nT * id], d_kp + (size_t)nT * src, sizeof(double) * nT,
                   cudaMemcpyDeviceToHost) != cudaSuccess) {
      *err = "download failed";
      return HC3D_ERR_CUDA;
    }
  }
  return HC3D_OK;
}

}  // namespace hc3d

extern "C" int hc3d_model_tables_gpu(hc3d_model* mdl, int device, double* ms, char* err, size_t errlen) {
  if (!mdl) return HC3D_ERR_INVALID;
  std::string e;
  const int r = hc3d::tables_gpu(mdl->m, device, ms, &e);
  if (r && err && errlen) std::snprintf(err, errlen, "%s", e.c_str());
  return r;
}
