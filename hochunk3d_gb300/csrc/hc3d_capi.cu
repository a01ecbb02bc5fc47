// hc3d_capi.cu -- the C-ABI of include/hc3d.h: context, device layouts,
// the Lucy temperature solve and tally read-back.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/hc3d.h"
#include "hc3d_device.h"
#include "hc3d_lucy.cuh"

using namespace hc3d;

struct hc3d_ctx {
  int device = 0, precision = HC3D_PREC_MIXED, block_size = 128, grid_blocks = 0;
  int sm_count = 0;
  std::string err;
  cudaStream_t stream = nullptr;
  bool tables = false, grid = false;
  // model
  DevModel dm{};
  std::vector<void*> core_allocs;   // counters, fault log, run arguments: the context's lifetime
  std::vector<void*> model_allocs;  // dust tables: until hc3d_reset
  std::vector<void*> grid_allocs;
  double tsub = 1600.0;
  double kappav[kSlots] = {0, 0, 0, 0};
  double* d_kappap = nullptr;  // (nT, kSlots)
  double* d_massarr = nullptr; // (ncell*4)
  double* d_tdust = nullptr;   // (ncell*4), also dm.tdust
  float* d_tdustf = nullptr;   // (ncell*4) FP32 copy, also dm.tdustf
  unsigned char* d_peelmask = nullptr;
  float4* d_rho4p = nullptr;  // (ncell) peel-masked FP32 densities, also dm.rho4p
  int ndg_in = 0;
  // species (1..8, reference numbering) of the four device slots (hc3d_set_species)
  int species[kSlots] = {1, 2, 3, 4};
  // small grains: emission spectra (hc3d_load_sg_tables) and the int_mean result of the last Lucy update
  bool sg_tables = false;
  double isrfkap_int = 0.0;
  std::vector<double> sg_uratio;
  int* d_imean = nullptr;
  double* d_imfract = nullptr;
  double* d_vcell = nullptr;   // (ncell) cell volumes, cm^3 (int_mean)
  double* d_uratio = nullptr;  // (nemit)
  bool imean_set = false;
  // tallies
  DevTallies dt{};
  TallyDims dims{};
  bool run_tallies = false;
  std::vector<void*> run_allocs;
  bool scales_set = false;
  int64_t epoch_np = 0, epoch_budget = 0;
  int status_seen = 0;
  unsigned long long* d_work = nullptr;
  int* d_status = nullptr;
  double* d_peeldir = nullptr;
  double* d_ap2 = nullptr;
  unsigned long long* d_maxrel = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaStream_t pstream = nullptr;   // the peel-off kernels of the wavefront loop
  std::vector<cudaEvent_t> wev;     // 4 per wave: k_wave start/end (stream), k_peel start/end (pstream)
  cudaEvent_t join = nullptr;       // end of the last k_peel of a run, waited for on stream
  double last_ms = 0.0, last_transport_ms = 0.0, last_peel_ms = 0.0;
  int last_launches = 0;
  std::vector<double> wave_log;  // per wave: E, active, alive after, transport ms, peel ms, events
  // wavefront form
  std::vector<void*> wave_allocs;
  WaveBufs wave{};
  int64_t pool_threads = 0, qcap = 0;
  int wave_blocks = 0, peel_blocks = 0;
  int peel_variant = 0;                   // block shape of the mixed-form peel-off kernel
  int peel_blocks_v[kPeelVariants] = {};  // its persistent grid per shape
  int64_t queue_records = 1 << 22;  // peel-off events held per wave
  int regen = 1;                    // k_wave regeneration threshold (lanes of a warp)
  // a peeled iteration run in chunks (hc3d_run_chunk): packets in flight stay in the pool
  bool chunk_open = false;
  int64_t carry_alive = 0;
  uint32_t chunk_key0 = 0, chunk_key1 = 0;
  int qchunk = 8;                   // k_wave queue slots reserved per atomic
  bool use_waves = true;            // peeled runs use the wavefront form
};

namespace {

int fail(hc3d_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

// the species index (0-based, in the ndg species of the host arrays) device
// slot s reads; -1 when the host arrays do not describe that species
int slot_src(const hc3d_ctx* c, int s, int ndg) {
  const int id = c->species[s] - 1;
  return id < ndg ? id : -1;
}

bool has_sg_slots(const hc3d_ctx* c) {
  for (int s = 0; s < kSlots; ++s)
    if (c->species[s] >= 5) return true;
  return false;
}

// the slot masks of the species map (grid_mod.f90:13-20: species 1, 2, 5, 6
// are disk species, 5-8 small grains)
void apply_species(hc3d_ctx* c) {
  c->dm.disk_mask = c->dm.sg_mask = 0u;
  for (int s = 0; s < kSlots; ++s) {
    const int sp = c->species[s];
    if (sp == 1 || sp == 2 || sp == 5 || sp == 6) c->dm.disk_mask |= 1u << s;
    if (sp >= 5) c->dm.sg_mask |= 1u << s;
  }
  c->dm.sg_on = (c->dm.sg_mask && c->sg_tables) ? 1 : 0;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(c, HC3D_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Device memory of a context is stream-ordered on the context's stream
// (cudaMallocAsync / cudaFreeAsync): loading, resetting or destroying one
// context never waits for the kernels of another context on the device.
template <class T>
int dalloc(hc3d_ctx* c, std::vector<void*>& owner, T** p, size_t n) {
  void* q = nullptr;
  cudaError_t e = cudaMallocAsync(&q, std::max<size_t>(n, 1) * sizeof(T), c->stream);
  if (e != cudaSuccess) return fail(c, HC3D_ERR_NOMEM, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
  owner.push_back(q);
  *p = (T*)q;
  return HC3D_OK;
}

template <class T>
int dupload(hc3d_ctx* c, std::vector<void*>& owner, T** p, const T* src, size_t n) {
  int r = dalloc(c, owner, p, n);
  if (r) return r;
  if (n) {
    // from pageable memory the call returns once src has been staged
    cudaError_t e = cudaMemcpyAsync(*p, src, n * sizeof(T), cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return fail(c, HC3D_ERR_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
  }
  return HC3D_OK;
}

// device -> host on the context's stream, complete on return
int d2h(hc3d_ctx* c, void* dst, const void* src, size_t bytes) {
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(c, HC3D_ERR_CUDA, std::string("device to host copy: ") + cudaGetErrorString(e));
  return HC3D_OK;
}

void free_all(hc3d_ctx* c, std::vector<void*>& v) {
  for (void* p : v) cudaFreeAsync(p, c->stream);
  v.clear();
}

int ceil_log2(double x) {
  int k = 0;
  while ((double)(1ull << k) < x && k < 62) ++k;
  return k;
}

// ---- Lucy temperature (tfinal restated; dusttemp.f90:30-50 fixed point) ----
struct LucyArgs {
  int64_t ncell;
  int nT;
  const double* lTint;
  const double* kappap;  // (nT, kSlots)
  double kappav[kSlots];
  double ltot, nphot, path_scale, tsub, na_min;
  int nslots;
};

__device__ double dusttemp_dev(const LucyArgs& a, double na, double T0, int s, double massarr) {
  return lucy_dusttemp(a.lTint, a.nT, a.kappap + (size_t)s * a.nT, a.kappav[s], a.ltot, a.nphot, na, T0, massarr);
}

// The peel-off walk of the mixed form reads one row per cell with the peel
// mask applied (a species hotter than Tsub contributes no opacity,
// peeloff_3d.f90:105-110): rho4p = rho4f with the masked slots zeroed.
__device__ __forceinline__ float4 masked_rho(float4 r, unsigned mask) {
  return make_float4((mask & 1u) ? r.x : 0.f, (mask & 2u) ? r.y : 0.f, (mask & 4u) ? r.z : 0.f,
                     (mask & 8u) ? r.w : 0.f);
}

__global__ void k_lucy(LucyArgs a, const unsigned long long* dtauabs, const double* rho4d, const double* massarr,
                       double* tdust, float* tdustf, unsigned char* peelmask, unsigned long long* maxrel,
                       const float4* rho4f, float4* rho4p) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.ncell; c += (int64_t)gridDim.x * blockDim.x) {
    unsigned mask = 0;
    for (int s = 0; s < kSlots; ++s) {
      double T = tdust[4 * c + s];
      if (s < a.nslots && rho4d[4 * c + s] > 0.0) {
        const double na = (double)(long long)dtauabs[(int64_t)s * a.ncell + c] / a.path_scale;
        const double Td = dusttemp_dev(a, na, T, s, massarr[4 * c + s]);
        if (na >= a.na_min) {
          const double rel = fabs(Td - T) / Td;
          atomicMax(maxrel, (unsigned long long)__double_as_longlong(rel));
        }
        T = Td;
        tdust[4 * c + s] = Td;
        tdustf[4 * c + s] = (float)Td;
      }
      if (T < a.tsub / 11605.0) mask |= 1u << s;
    }
    peelmask[c] = (unsigned char)mask;
    rho4p[c] = masked_rho(rho4f[c], mask);
  }
}

__global__ void k_peelmask(int64_t ncell, const double* tdust, double tsub, unsigned char* peelmask,
                           const float4* rho4f, float4* rho4p) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncell; c += (int64_t)gridDim.x * blockDim.x) {
    unsigned mask = 0;
    for (int s = 0; s < kSlots; ++s)
      if (tdust[4 * c + s] < tsub / 11605.0) mask |= 1u << s;
    peelmask[c] = (unsigned char)mask;
    rho4p[c] = masked_rho(rho4f[c], mask);
  }
}

// ---- int_mean.f90:19-94 -------------------------------------------------------
// The mean intensity of each cell in units of the ISRF absorbed by the small
// grains: the path tally jsg (ds kappa/kappa_V (1 - albedo) over the cell's
// outer radius, x path_scale) times the outer radius, rstar_cm kappa_V /
// (4 pi), over vcell and the packets, times ltot, over isrfkap_int.  The
// spectrum row is where the ratio falls in uratio (nr locate, clamped to
// 1..nemit), imfract the fraction of the way to the next row in log10 (0
// where the ratio is 0, 1 on the last row).
struct IntMeanArgs {
  int64_t ncell;
  int nr1;                 // nrg - 1
  double path_scale, jconst, nphot, ltot, isrfkap_int;
  int nemit;
  const double* rarr;      // (nrg)
  const double* vcell;     // (ncell)
  const double* uratio;    // (nemit)
};

__device__ __forceinline__ void int_mean_cell(const IntMeanArgs& a, int64_t c, const unsigned long long* jsg, int* imean,
                                              double* imfract) {
  const int ir = (int)(c % a.nr1) + 1;
  double jm = (double)(long long)jsg[c] / a.path_scale;
  jm = jm * a.rarr[ir];
  jm = jm * a.jconst;
  jm = jm / a.vcell[c] / a.nphot * a.ltot;
  const double jratio = jm / a.isrfkap_int;
  int jl = 0, ju = a.nemit + 1;
  while (ju - jl > 1) {
    const int jmid = (ju + jl) / 2;
    if (jratio > a.uratio[jmid - 1]) jl = jmid; else ju = jmid;
  }
  if (jl == 0 && jratio == a.uratio[0]) jl = 1;
  int im = jl;
  if (im > a.nemit) im = a.nemit;
  if (im < 1) im = 1;
  double f;
  if (jratio == 0.0) f = 0.0;
  else if (im == a.nemit) f = 1.0;
  else {
    const double jr1 = log10(a.uratio[im - 1]), jr2 = log10(a.uratio[im]);
    f = (log10(jratio) - jr1) / (jr2 - jr1);
  }
  imean[c] = im;
  imfract[c] = f;
}

__global__ void k_intmean(IntMeanArgs a, const unsigned long long* jsg, int* imean, double* imfract) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.ncell; c += (int64_t)gridDim.x * blockDim.x)
    int_mean_cell(a, c, jsg, imean, imfract);
}

int grid_blocks_for(hc3d_ctx* c, int64_t n) {
  int64_t b = (n + 255) / 256;
  int64_t cap = (int64_t)c->sm_count * 8;
  return (int)std::max<int64_t>(1, std::min(b, cap));
}

int alloc_run_tallies(hc3d_ctx* c, const TallyDims& d) {
  free_all(c, c->run_allocs);
  c->run_tallies = false;
  int r;
  if ((r = dalloc(c, c->run_allocs, &c->dt.sed, (size_t)9 * d.nsed))) return r;
  if ((r = dalloc(c, c->run_allocs, &c->dt.psed, (size_t)9 * std::max<int64_t>(d.npsed, 1)))) return r;
  if ((r = dalloc(c, c->run_allocs, &c->dt.img, (size_t)4 * std::max<int64_t>(d.nimg, 1)))) return r;
  c->dt.cube = nullptr;
  if (d.ncube > 0) {
    if ((r = dalloc(c, c->run_allocs, &c->dt.cube, (size_t)(kNo + 3) * d.ncube))) return r;
    CK(cudaMemsetAsync(c->dt.cube, 0, sizeof(unsigned long long) * (kNo + 3) * d.ncube, c->stream));
  }
  CK(cudaMemsetAsync(c->dt.sed, 0, sizeof(unsigned long long) * 9 * d.nsed, c->stream));
  CK(cudaMemsetAsync(c->dt.psed, 0, sizeof(unsigned long long) * 9 * std::max<int64_t>(d.npsed, 1), c->stream));
  CK(cudaMemsetAsync(c->dt.img, 0, sizeof(unsigned long long) * 4 * std::max<int64_t>(d.nimg, 1), c->stream));
  c->dims = d;
  c->run_tallies = true;
  return HC3D_OK;
}

bool same_dims(const TallyDims& a, const TallyDims& b) {
  return a.nfreq == b.nfreq && a.nmu == b.nmu && a.nph == b.nph && a.nap == b.nap && a.npeel == b.npeel &&
         a.nx == b.nx && a.ncube == b.ncube;
}

TallyDims dims_of(const hc3d_run_params* p) {
  TallyDims d;
  d.nfreq = p->nfreq; d.nmu = p->nmu; d.nph = p->nph; d.nap = p->nap;
  d.npeel = p->ipeel ? p->npeel : 0;
  d.nx = p->nxhst;
  d.nsed = (int64_t)p->nfreq * p->nmu * p->nph * p->nap * kNo;
  d.npsed = (int64_t)p->nfreq * d.npeel * p->nap * kNo;
  d.nimg = (int64_t)d.npeel * p->nxhst * p->nxhst;
  d.ncube = (p->imcube && p->ipeel && p->image) ? d.nimg * p->nfreq : 0;
  return d;
}

int check_params(hc3d_ctx* c, const hc3d_run_params* p) {
  if (!p) return fail(c, HC3D_ERR_INVALID, "params is NULL");
  if (p->np < 0 || p->packet_offset < 0) return fail(c, HC3D_ERR_INVALID, "np and packet_offset must be >= 0");
  if (p->nfreq < 1 || p->nmu < 1 || p->nph < 1 || p->nap < 1)
    return fail(c, HC3D_ERR_INVALID, "nfreq, nmu, nph and nap must be >= 1");
  if (!p->aperture2) return fail(c, HC3D_ERR_INVALID, "aperture2 is NULL");
  if (p->ipeel) {
    if (p->npeel < 1 || p->npeel > kMaxPeel) return fail(c, HC3D_ERR_INVALID, "npeel must be in 1..256");
    if (!p->thete || !p->phie) return fail(c, HC3D_ERR_INVALID, "thete/phie are NULL");
    if (p->nxhst < 1) return fail(c, HC3D_ERR_INVALID, "nxhst must be >= 1");
  }
  if (p->limb != 0 && p->limb != 1) return fail(c, HC3D_ERR_INVALID, "limb must be 0 or 1");
  if (p->imcube && p->ipeel && !p->image)
    return fail(c, HC3D_ERR_INVALID, "imcube needs image = 1 (the cube is binned by image pixel)");
  if (p->limb == 1 && c->tables && c->dm.nlimb < 2)
    return fail(c, HC3D_ERR_INVALID, "limb = 1 needs the limb-darkening table (ntab) of hc3d_load_tables");
  if (!(p->numin > 0.0) || !(p->numax > p->numin)) return fail(c, HC3D_ERR_INVALID, "need 0 < numin < numax");
  if (!(p->rstar_cm > 0.0) || !(p->rmaxi > 0.0 || !p->ipeel)) return fail(c, HC3D_ERR_INVALID, "bad rstar_cm/rmaxi");
  return HC3D_OK;
}

int set_scales(hc3d_ctx* c, int64_t np) {
  const double budget = (double)std::max<int64_t>(np, 1 << 20) * 16.0;
  const int L = ceil_log2(budget);
  const int sb = std::max(16, std::min(40, 58 - L));
  const int qb = sb - 8;
  const int pb = std::max(12, std::min(32, 52 - L));
  c->dt.stokes_scale = std::ldexp(1.0, sb);
  c->dt.square_scale = std::ldexp(1.0, qb);
  c->dt.path_scale = std::ldexp(1.0, pb);
  c->epoch_budget = (int64_t)budget;
  c->scales_set = true;
  return HC3D_OK;
}

int prepare_run(hc3d_ctx* c, const hc3d_run_params* p, RunArgs* a) {
  int r = check_params(c, p);
  if (r) return r;
  if (!c->tables || !c->grid) return fail(c, HC3D_ERR_STATE, "load tables and grid before running");
  TallyDims d = dims_of(p);
  if (!c->run_tallies || !same_dims(d, c->dims)) {
    if (c->scales_set && c->epoch_np > 0 && c->run_tallies)
      return fail(c, HC3D_ERR_STATE, "tally shape changed without hc3d_zero_tallies()");
    if ((r = alloc_run_tallies(c, d))) return r;
  }
  if (!c->scales_set) set_scales(c, p->np);
  if (c->epoch_np + p->np > c->epoch_budget)
    return fail(c, HC3D_ERR_INVALID, "fixed-point tally budget exceeded: call hc3d_zero_tallies() first");
  std::vector<double> pdir(4 * (size_t)std::max(1, d.npeel));
  for (int k = 0; k < d.npeel; ++k) {
    pdir[4 * k + 0] = std::cos(p->thete[k]);
    pdir[4 * k + 1] = std::sin(p->thete[k]);
    pdir[4 * k + 2] = std::cos(p->phie[k]);
    pdir[4 * k + 3] = std::sin(p->phie[k]);
  }
  CK(cudaMemcpyAsync(c->d_peeldir, pdir.data(), sizeof(double) * pdir.size(), cudaMemcpyHostToDevice, c->stream));
  if (p->nap > 64) return fail(c, HC3D_ERR_INVALID, "nap must be <= 64");
  CK(cudaMemcpyAsync(c->d_ap2, p->aperture2, sizeof(double) * p->nap, cudaMemcpyHostToDevice, c->stream));
  std::memset(a, 0, sizeof(*a));
  a->np = p->np;
  a->packet_offset = p->packet_offset;
  a->key0 = (uint32_t)p->seed ^ ((uint32_t)p->iter * 0x9E3779B9u);
  a->key1 = (uint32_t)(p->seed >> 32);
  a->ipeel = p->ipeel ? 1 : 0;
  a->npeel = d.npeel;
  a->image = p->ipeel && p->image ? 1 : 0;
  a->nfreq = p->nfreq; a->nmu = p->nmu; a->nph = p->nph; a->nap = p->nap; a->nx = p->nxhst;
  a->rmaxi = p->rmaxi;
  a->fractxh = p->nxhst > 0 ? 2.0 * p->rmaxi / (double)p->nxhst : 1.0;
  a->numin = p->numin;
  a->lnurat = std::log(p->numax / p->numin);
  a->rstar_cm = p->rstar_cm;
  for (int s = 0; s < kSlots; ++s) a->kapfac[s] = (float)(p->rstar_cm * c->kappav[s]);
  a->iintmax = p->iintmax > 0 ? p->iintmax : 10000;
  a->max_interactions = p->max_interactions;
  if (p->ext_illum) {
    if (c->dm.nisrf < 2)
      return fail(c, HC3D_ERR_INVALID, "ext_illum needs the external-illumination tables (nisrf) of hc3d_load_tables");
    if (!(p->rmax > 1.0)) return fail(c, HC3D_ERR_INVALID, "ext_illum needs rmax > 1 (stellar radii)");
    if (p->n_star < 0) return fail(c, HC3D_ERR_INVALID, "n_star < 0");
  }
  a->limb = p->limb;
  a->regen = c->regen;
  a->imcube = d.ncube > 0 ? 1 : 0;
  a->iter1 = p->iter == 1 ? 1 : 0;
  if (c->dm.sg_on) {
    c->dm.sg_jfacd = 1.0 / (p->rstar_cm * c->kappav[c->dm.sg_slot]);
    c->dm.sg_jfac = (float)c->dm.sg_jfacd;
  }
  if (c->dm.sg_mask) {
    if (!c->dm.sg_on) return fail(c, HC3D_ERR_STATE, "a slot holds small grains: load their spectra (hc3d_load_sg_tables)");
    if (p->iter != 1 && !c->imean_set)
      return fail(c, HC3D_ERR_STATE,
                  "small grains after the first iteration re-emit by the mean intensity of the last: run "
                  "hc3d_lucy_update after an iteration or set it with hc3d_set_imean");
  }
  a->qchunk = c->qchunk;
  // disk accretion and hot-spot packets
  a->n_acc = 0;
  a->n_spot = 0;
  a->src_on = 0;
  if (p->sources) {
    const hc3d_sources& S = *p->sources;
    if (p->n_acc < 0 || p->n_spot < p->n_acc) return fail(c, HC3D_ERR_INVALID, "need 0 <= n_acc <= n_spot");
    if (p->n_acc > 0 && !(S.rddustmin > 0.0 && S.rddustmin < S.rmaxdmax && S.rmax > 0.0 && S.gas_den > 0.0 &&
                          S.rstar > 0.0 && S.rsun > 0.0))
      return fail(c, HC3D_ERR_INVALID, "accretion packets need 0 < rddustmin < rmaxdmax, rmax, gas_den, rstar, rsun > 0");
    if (p->n_spot > p->n_acc && !(S.tshock > 0.0))
      return fail(c, HC3D_ERR_INVALID, "hot-spot packets need tshock > 0");
    if (S.ispot && ((S.nspot != 1 && S.nspot != 2) || !(S.csprad >= -1.0 && S.csprad <= 1.0)))
      return fail(c, HC3D_ERR_INVALID, "spots need nspot 1 or 2 and -1 <= csprad <= 1");
    if (S.ispot && S.fspot < 1.0 && S.csprad < 1.0 && !(S.tshock > 0.0))
      return fail(c, HC3D_ERR_INVALID, "stellar packets that fall in a spot need tshock > 0");
    a->src = S;
    a->src_on = 1;
    a->n_acc = p->n_acc;
    a->n_spot = p->n_spot;
  } else if (p->n_acc || p->n_spot) {
    return fail(c, HC3D_ERR_INVALID, "n_acc and n_spot need sources");
  }
  a->ext_illum = p->ext_illum ? 1 : 0;
  a->n_star = p->n_star;
  a->rmax = p->rmax;
  a->peeldir = c->d_peeldir;
  a->aperture2 = c->d_ap2;
  a->work = c->d_work;
  a->status = c->d_status;
  return HC3D_OK;
}

// Release the wavefront buffers (after both streams are idle).
void drop_wave(hc3d_ctx* c) {
  c->chunk_open = false;  // packets in flight are lost with the pool
  c->carry_alive = 0;
  if (!c->wave.pool) return;
  cudaStreamSynchronize(c->pstream);
  cudaStreamSynchronize(c->stream);
  free_all(c, c->wave_allocs);
  c->wave = WaveBufs{};
}

// Allocate the packet pool and the two event queues of the wavefront form once per context.
int ensure_wave(hc3d_ctx* c) {
  const bool f64 = c->precision == HC3D_PREC_FP64;
  int per_sm = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f64 ? wave_fn_fp64() : wave_fn_mixed(), 128, c->dm.dust_smem));
  if (per_sm < 1) per_sm = 1;
  if (c->wave.pool) {
    // kept across hc3d_reset while the dust tables of the new model allow the same residency
    if (c->sm_count * per_sm == c->wave_blocks) return HC3D_OK;
    drop_wave(c);
  }
  c->wave_blocks = c->sm_count * per_sm;
  c->pool_threads = (int64_t)c->wave_blocks * 128;
  int per_sm_p = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_p, f64 ? peel_fn_fp64() : peel_fn_mixed(0), 256, 0));
  c->peel_blocks = c->sm_count * std::max(1, per_sm_p);
  for (int v = 0; v < kPeelVariants; ++v) {
    int k = 0;
    if (!f64) CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, peel_fn_mixed(v), peel_threads_mixed(v), 0));
    c->peel_blocks_v[v] = c->sm_count * std::max(1, k);
  }
  // room for every thread's qchunk reserved slots on top of one record each (see run_waves' E)
  c->qcap = std::max<int64_t>(c->queue_records, c->pool_threads * (int64_t)(c->qchunk + 1));
  const size_t slot = f64 ? slot_bytes_fp64() : slot_bytes_mixed();
  const size_t rec = f64 ? rec_bytes_fp64() : rec_bytes_mixed();
  int r;
  unsigned char *pool, *q0, *q1;
  if ((r = dalloc(c, c->wave_allocs, &pool, slot * (size_t)c->pool_threads)) ||
      (r = dalloc(c, c->wave_allocs, &q0, rec * (size_t)c->qcap)) ||
      (r = dalloc(c, c->wave_allocs, &q1, rec * (size_t)c->qcap)) ||
      (r = dalloc(c, c->wave_allocs, &c->wave.qcount[0], 1)) || (r = dalloc(c, c->wave_allocs, &c->wave.qcount[1], 1)) ||
      (r = dalloc(c, c->wave_allocs, &c->wave.alive, 1)) ||
      (r = dalloc(c, c->wave_allocs, &c->wave.next_ray[0], 1)) || (r = dalloc(c, c->wave_allocs, &c->wave.next_ray[1], 1)))
    return r;
  c->wave.pool = pool;
  c->wave.queue[0] = q0;
  c->wave.queue[1] = q1;
  return HC3D_OK;
}

// the events of wave w (created on first use, kept with the context)
int wave_events(hc3d_ctx* c, int w) {
  while ((int)c->wev.size() < 4 * (w + 1)) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    c->wev.push_back(e);
  }
  return HC3D_OK;
}

// The wavefront loop of one peeled run: waves until the batch is exhausted
// and no packet is alive.  The per-wave event budget E keeps a queue within
// its capacity: at most min(pool, alive + unstarted) threads append, each at
// most E records.  Wave w's k_wave fills queue w % 2 on the context's stream;
// its k_peel walks that queue on the second stream, while k_wave of wave w + 1
// fills the other queue on the first.  So the peel-off work of one wave runs
// beside the transport of the next -- in particular beside the long packet
// histories that leave most of the device idle at the end of a batch.  Before
// k_wave reuses a queue it waits for the k_peel that read it.
//
// drain = false (a chunk of an iteration, hc3d_run_chunk): the loop stops
// once every packet of the call has been started; the packets still in
// flight stay in the pool and continue in the next chunk of the iteration.
int run_waves(hc3d_ctx* c, const hc3d_run_params* p, const RunArgs& a, bool drain = true) {
  int r;
  if ((r = ensure_wave(c))) return r;
  const bool f64 = c->precision == HC3D_PREC_FP64;
  const size_t slot = f64 ? slot_bytes_fp64() : slot_bytes_mixed();
  int64_t alive_prev = 0;
  if (c->chunk_open) alive_prev = c->carry_alive;
  else CK(cudaMemsetAsync(c->wave.pool, 0, slot * (size_t)c->pool_threads, c->stream));
  LaunchCfg wc{c->wave_blocks, 128, c->stream}, pc{c->peel_blocks, 256, c->pstream};
  if (!f64) {
    pc.variant = c->peel_variant;
    pc.threads = peel_threads_mixed(c->peel_variant);
    pc.blocks = c->peel_blocks_v[c->peel_variant];
  }
  unsigned long long work = 0, events_prev = 0;
  CK(cudaMemcpyAsync(&events_prev, c->dt.counters + HC3D_CNT_EVENTS, sizeof(events_prev), cudaMemcpyDeviceToHost,
                     c->stream));
  c->last_transport_ms = c->last_peel_ms = 0.0;
  c->last_launches = 0;
  c->wave_log.clear();
  int nwave = 0;
  int prev_peel_end[2] = {-1, -1};  // index in wev of the k_peel end that last read each queue
  for (int wave = 0;; ++wave) {
    const int64_t remaining = p->np - (int64_t)std::min<unsigned long long>(work, (unsigned long long)p->np);
    const int64_t active = std::min<int64_t>(c->pool_threads, alive_prev + remaining);
    if (active <= 0) break;
    // each appending lane takes at most E records and leaves fewer than qchunk reserved slots unused
    const int E = (int)std::max<int64_t>(1, std::min<int64_t>(c->qcap / active - c->qchunk, 1 << 20));
    const int q = wave & 1;
    if ((r = wave_events(c, wave))) return r;
    const int ev = 4 * wave;
    if (prev_peel_end[q] >= 0) CK(cudaStreamWaitEvent(c->stream, c->wev[prev_peel_end[q]], 0));  // queue q read
    CK(cudaMemsetAsync(c->wave.qcount[q], 0, sizeof(unsigned long long), c->stream));
    CK(cudaMemsetAsync(c->wave.alive, 0, sizeof(unsigned int), c->stream));
    CK(cudaEventRecord(c->wev[ev], c->stream));
    cudaError_t e = f64 ? launch_wave_transport_fp64(c->dm, c->dt, c->dims, a, c->wave, q, E, wc)
                        : launch_wave_transport_mixed(c->dm, c->dt, c->dims, a, c->wave, q, E, wc);
    if (e != cudaSuccess) return fail(c, HC3D_ERR_CUDA, std::string("wave launch: ") + cudaGetErrorString(e));
    CK(cudaEventRecord(c->wev[ev + 1], c->stream));
    // the peel-off rays of this wave, on the second stream
    CK(cudaStreamWaitEvent(c->pstream, c->wev[ev + 1], 0));
    CK(cudaMemsetAsync(c->wave.next_ray[q], 0, sizeof(unsigned long long), c->pstream));
    CK(cudaEventRecord(c->wev[ev + 2], c->pstream));
    e = f64 ? launch_wave_peel_fp64(c->dm, c->dt, c->dims, a, c->wave, q, pc)
            : launch_wave_peel_mixed(c->dm, c->dt, c->dims, a, c->wave, q, pc);
    if (e != cudaSuccess) return fail(c, HC3D_ERR_CUDA, std::string("peel-off launch: ") + cudaGetErrorString(e));
    CK(cudaEventRecord(c->wev[ev + 3], c->pstream));
    prev_peel_end[q] = ev + 3;
    // whether another wave is needed: the counters after this k_wave (the
    // copies wait for it on the first stream, not for the k_peel)
    unsigned int alive = 0;
    unsigned long long events = 0;
    CK(cudaMemcpyAsync(&alive, c->wave.alive, sizeof(alive), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&work, c->d_work, sizeof(work), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&events, c->dt.counters + HC3D_CNT_EVENTS, sizeof(events), cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->wave_log.insert(c->wave_log.end(),
                       {(double)E, (double)active, (double)alive, 0.0, 0.0, (double)(events - events_prev)});
    events_prev = events;
    alive_prev = alive;
    ++nwave;
    if (work >= (unsigned long long)p->np && (alive == 0 || !drain)) break;
  }
  c->chunk_open = !drain && alive_prev > 0;
  c->carry_alive = c->chunk_open ? alive_prev : 0;
  c->chunk_key0 = a.key0;
  c->chunk_key1 = a.key1;
  // the first stream waits for the last k_peel, so that what follows on it
  // (tallies, temperatures) sees every ray
  CK(cudaEventRecord(c->join, c->pstream));
  CK(cudaStreamWaitEvent(c->stream, c->join, 0));
  CK(cudaEventSynchronize(c->join));
  for (int w = 0; w < nwave; ++w) {
    float t0 = 0.f, t1 = 0.f;
    CK(cudaEventElapsedTime(&t0, c->wev[4 * w], c->wev[4 * w + 1]));
    CK(cudaEventElapsedTime(&t1, c->wev[4 * w + 2], c->wev[4 * w + 3]));
    c->last_transport_ms += t0;
    c->last_peel_ms += t1;
    c->wave_log[6 * w + 3] = t0;
    c->wave_log[6 * w + 4] = t1;
  }
  c->last_launches = 2 * nwave;
  // the span of the loop: first k_wave start to last k_peel end (the kernels overlap)
  float span = 0.f;
  if (nwave) CK(cudaEventElapsedTime(&span, c->wev[0], c->join));
  c->last_ms = span;
  return HC3D_OK;
}

int finish_run(hc3d_ctx* c) {
  CK(cudaStreamSynchronize(c->stream));
  int st = 0;
  if (int r_ = d2h(c, &st, c->d_status, sizeof(int))) return r_;
  if (st && !c->status_seen) c->status_seen = st;
  return HC3D_OK;
}

}  // namespace

extern "C" const char* hc3d_version(void) { return "hc3d 0.1 sm_103a"; }

extern "C" int hc3d_create(hc3d_ctx** out, const hc3d_device_opts* opts) {
  if (!out) return HC3D_ERR_INVALID;
  *out = nullptr;
  hc3d_ctx* c = new (std::nothrow) hc3d_ctx();
  if (!c) return HC3D_ERR_NOMEM;
  if (opts) {
    c->device = opts->device;
    c->precision = opts->precision;
    if (opts->block_size > 0) c->block_size = opts->block_size;
    c->grid_blocks = opts->grid_blocks;
  }
  if (c->precision != HC3D_PREC_MIXED && c->precision != HC3D_PREC_FP64) {
    delete c;
    return HC3D_ERR_INVALID;
  }
  if (c->block_size % 32 != 0 || c->block_size > 128) {
    delete c;
    return HC3D_ERR_INVALID;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || c->device < 0 || c->device >= ndev) {
    delete c;
    return HC3D_ERR_CUDA;
  }
  if (cudaSetDevice(c->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return HC3D_ERR_CUDA;
  }
  if (cudaStreamCreateWithFlags(&c->pstream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->join) != cudaSuccess) {
    if (c->pstream) cudaStreamDestroy(c->pstream);
    cudaStreamDestroy(c->stream);
    delete c;
    return HC3D_ERR_CUDA;
  }
  {
    // keep freed stream-ordered memory in this process's pool for the next
    // model instead of returning it to the driver at every synchronisation
    cudaMemPool_t mp;
    if (cudaDeviceGetDefaultMemPool(&mp, c->device) == cudaSuccess) {
      uint64_t keep = ~0ull;
      cudaMemPoolSetAttribute(mp, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  std::vector<void*>& own = c->core_allocs;
  if (dalloc(c, own, &c->d_work, 1) || dalloc(c, own, &c->d_status, 1) ||
      dalloc(c, own, &c->d_peeldir, 4 * kMaxPeel) || dalloc(c, own, &c->d_ap2, 64) ||
      dalloc(c, own, &c->d_maxrel, 1) || dalloc(c, own, &c->dt.counters, 16) ||
      dalloc(c, own, &c->dt.fault_log, kFaultLog) || dalloc(c, own, &c->dt.fault_count, 1)) {
    free_all(c, own);
    cudaStreamDestroy(c->stream);
    delete c;
    return HC3D_ERR_NOMEM;
  }
  cudaMemsetAsync(c->dt.counters, 0, 16 * sizeof(unsigned long long), c->stream);
  cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream);
  cudaStreamSynchronize(c->stream);
  if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
    free_all(c, own);
    cudaStreamDestroy(c->stream);
    delete c;
    return HC3D_ERR_CUDA;
  }
  apply_species(c);
  *out = c;
  return HC3D_OK;
}

extern "C" int hc3d_set_species(hc3d_ctx* c, const int32_t* species) {
  if (!c || !species) return HC3D_ERR_INVALID;
  if (c->tables || c->grid) return fail(c, HC3D_ERR_STATE, "set the species before hc3d_load_tables and hc3d_load_grid");
  if (species[0] != 1 || species[1] != 2)
    return fail(c, HC3D_ERR_INVALID, "slots 1 and 2 hold the thermal disk species 1 and 2");
  if (!(species[2] >= 3 && species[2] <= 8 && species[3] > species[2] && species[3] <= 8))
    return fail(c, HC3D_ERR_INVALID, "slots 3 and 4 hold two species of 3..8 in increasing order");
  for (int s = 0; s < kSlots; ++s) c->species[s] = species[s];
  apply_species(c);
  return HC3D_OK;
}

extern "C" int hc3d_load_sg_tables(hc3d_ctx* c, const hc3d_sg_tables* t) {
  if (!c || !t) return HC3D_ERR_INVALID;
  if (!has_sg_slots(c)) return fail(c, HC3D_ERR_STATE, "no slot holds small grains (hc3d_set_species)");
  if (!c->tables) return fail(c, HC3D_ERR_STATE, "load the dust tables first");
  if (c->sg_tables) return fail(c, HC3D_ERR_STATE, "small-grain spectra already loaded in this context");
  if (t->nemit < 2 || t->nemit > 64 || t->ndraine < 3 || !t->cdf || !t->logcdf || !t->logfreq || !t->uratio)
    return fail(c, HC3D_ERR_INVALID, "small-grain spectra: bad dimensions or a NULL pointer");
  if (t->sg_slot < 1 || t->sg_slot > kSlots || c->species[t->sg_slot - 1] < 5)
    return fail(c, HC3D_ERR_INVALID, "sg_slot must name a slot that holds small grains");
  if (!(t->isrfkap_int > 0.0) || std::isinf(t->isrfkap_int))
    return fail(c, HC3D_ERR_INVALID, "isrfkap_int must be positive and finite");
  for (int j = 1; j < t->nemit; ++j)
    if (!(t->uratio[j] > t->uratio[j - 1]) || !(t->uratio[0] > 0.0))
      return fail(c, HC3D_ERR_INVALID, "uratio must be positive and increase");
  CK(cudaSetDevice(c->device));
  // rows of one spectrum contiguous on the device: [j * ndraine + i] from the Fortran (nemit, ndraine)
  const int ne = t->nemit, nd = t->ndraine;
  std::vector<double> cdf((size_t)ne * nd), lc((size_t)ne * nd);
  for (int i = 0; i < nd; ++i)
    for (int j = 0; j < ne; ++j) {
      cdf[(size_t)j * nd + i] = t->cdf[(size_t)j + (size_t)ne * i];
      lc[(size_t)j * nd + i] = t->logcdf[(size_t)j + (size_t)ne * i];
    }
  std::vector<void*>& own = c->model_allocs;
  double *d_cdf, *d_lc, *d_lf, *d_ur;
  int r;
  if ((r = dupload(c, own, &d_cdf, cdf.data(), cdf.size())) || (r = dupload(c, own, &d_lc, lc.data(), lc.size())) ||
      (r = dupload(c, own, &d_lf, t->logfreq, (size_t)nd)) || (r = dupload(c, own, &d_ur, t->uratio, (size_t)ne)))
    return r;
  CK(cudaStreamSynchronize(c->stream));
  c->dm.sg_nemit = ne; c->dm.sg_nd = nd;
  c->dm.sg_cdf = d_cdf; c->dm.sg_logcdf = d_lc; c->dm.sg_logfreq = d_lf;
  c->d_uratio = d_ur;
  c->dm.sg_slot = t->sg_slot - 1;
  c->isrfkap_int = t->isrfkap_int;
  c->sg_uratio.assign(t->uratio, t->uratio + ne);
  c->sg_tables = true;
  apply_species(c);
  return HC3D_OK;
}

extern "C" int hc3d_get_imean(hc3d_ctx* c, int32_t* imean, double* imfract) {
  if (!c || (!imean && !imfract)) return HC3D_ERR_INVALID;
  if (!c->grid || !c->d_imean) return fail(c, HC3D_ERR_STATE, "no slot of the loaded grid holds small grains");
  if (!c->imean_set) return fail(c, HC3D_ERR_STATE, "int_mean has not run (hc3d_lucy_update) nor been set");
  CK(cudaSetDevice(c->device));
  const DevModel& m = c->dm;
  const int64_t n = m.ncell, n4 = (int64_t)m.nrg * m.ntg * m.npg;
  std::vector<int> im((size_t)n);
  std::vector<double> fr((size_t)n);
  if (int r_ = d2h(c, im.data(), c->d_imean, sizeof(int) * n)) return r_;
  if (int r_ = d2h(c, fr.data(), c->d_imfract, sizeof(double) * n)) return r_;
  if (imean) std::fill(imean, imean + n4, 0);
  if (imfract) std::fill(imfract, imfract + n4, 0.0);
  for (int ip = 1; ip < m.npg; ++ip)
    for (int it = 1; it < m.ntg; ++it)
      for (int ir = 1; ir < m.nrg; ++ir) {
        const int64_t c4 = (int64_t)(ir - 1) + (int64_t)m.nrg * ((it - 1) + (int64_t)m.ntg * (ip - 1));
        const int64_t cc = (int64_t)(ir - 1) + (int64_t)(m.nrg - 1) * ((it - 1) + (int64_t)(m.ntg - 1) * (ip - 1));
        if (imean) imean[c4] = im[cc];
        if (imfract) imfract[c4] = fr[cc];
      }
  return HC3D_OK;
}

extern "C" int hc3d_set_imean(hc3d_ctx* c, const int32_t* imean, const double* imfract) {
  if (!c || !imean || !imfract) return HC3D_ERR_INVALID;
  if (!c->grid || !c->d_imean) return fail(c, HC3D_ERR_STATE, "no slot of the loaded grid holds small grains");
  if (!c->sg_tables) return fail(c, HC3D_ERR_STATE, "load the small-grain spectra first");
  CK(cudaSetDevice(c->device));
  const DevModel& m = c->dm;
  const int64_t n = m.ncell;
  std::vector<int> im((size_t)n);
  std::vector<double> fr((size_t)n);
  for (int ip = 1; ip < m.npg; ++ip)
    for (int it = 1; it < m.ntg; ++it)
      for (int ir = 1; ir < m.nrg; ++ir) {
        const int64_t c4 = (int64_t)(ir - 1) + (int64_t)m.nrg * ((it - 1) + (int64_t)m.ntg * (ip - 1));
        const int64_t cc = (int64_t)(ir - 1) + (int64_t)(m.nrg - 1) * ((it - 1) + (int64_t)(m.ntg - 1) * (ip - 1));
        if (imean[c4] < 1 || imean[c4] > m.sg_nemit || !std::isfinite(imfract[c4]))
          return fail(c, HC3D_ERR_INVALID, "imean must lie in 1..nemit and imfract be finite");
        im[cc] = imean[c4];
        fr[cc] = imfract[c4];
      }
  CK(cudaMemcpyAsync(c->d_imean, im.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d_imfract, fr.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->imean_set = true;
  return HC3D_OK;
}

extern "C" void hc3d_destroy(hc3d_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_all(c, c->run_allocs);
  free_all(c, c->grid_allocs);
  free_all(c, c->model_allocs);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->pstream) cudaStreamSynchronize(c->pstream);
  for (cudaEvent_t e : c->wev) cudaEventDestroy(e);
  c->wev.clear();
  if (c->join) cudaEventDestroy(c->join);
  free_all(c, c->wave_allocs);
  free_all(c, c->core_allocs);
  if (c->pstream) cudaStreamDestroy(c->pstream);
  if (c->stream) {
    cudaStreamSynchronize(c->stream);
    cudaStreamDestroy(c->stream);
  }
  delete c;
}

extern "C" int hc3d_reset(hc3d_ctx* c) {
  if (!c) return HC3D_ERR_INVALID;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  free_all(c, c->run_allocs);
  free_all(c, c->grid_allocs);
  free_all(c, c->model_allocs);
  c->tables = c->grid = c->run_tallies = false;
  c->scales_set = false;
  c->epoch_np = c->epoch_budget = 0;
  c->dm = DevModel{};
  c->dims = TallyDims{};
  c->d_kappap = c->d_massarr = c->d_tdust = nullptr;
  c->d_tdustf = nullptr;
  c->d_peelmask = nullptr;
  c->d_rho4p = nullptr;
  c->ndg_in = 0;
  for (int s = 0; s < kSlots; ++s) c->species[s] = s + 1;
  c->sg_tables = false;
  c->imean_set = false;
  c->d_imean = nullptr; c->d_imfract = nullptr; c->d_vcell = nullptr; c->d_uratio = nullptr;
  apply_species(c);
  // the run tallies go; the counters and the fault log stay with the context
  DevTallies keep{};
  keep.counters = c->dt.counters;
  keep.fault_log = c->dt.fault_log;
  keep.fault_count = c->dt.fault_count;
  c->dt = keep;
  CK(cudaMemsetAsync(c->dt.counters, 0, 16 * sizeof(unsigned long long), c->stream));
  CK(cudaMemsetAsync(c->dt.fault_count, 0, sizeof(unsigned long long), c->stream));
  CK(cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream));
  c->status_seen = 0;
  c->wave_log.clear();
  CK(cudaStreamSynchronize(c->stream));
  return HC3D_OK;
}

extern "C" void* hc3d_get_stream(hc3d_ctx* c) { return c ? (void*)c->stream : nullptr; }

extern "C" int hc3d_last_kernel_ms(hc3d_ctx* c, double* ms) {
  if (!c || !ms) return HC3D_ERR_INVALID;
  *ms = c->last_ms;
  return HC3D_OK;
}

extern "C" int hc3d_get_error(const hc3d_ctx* c, char* buf, size_t len) {
  if (!c || !buf || !len) return HC3D_ERR_INVALID;
  std::snprintf(buf, len, "%s", c->err.c_str());
  return HC3D_OK;
}

extern "C" int hc3d_load_tables(hc3d_ctx* c, const hc3d_dust_tables* t) {
  if (!c || !t) return HC3D_ERR_INVALID;
  if (t->ndg < 1 || t->ndg > HC3D_NDG || t->nlammax < 2 || t->nT < 2 || t->nnu < 2 || t->nhnu < 3)
    return fail(c, HC3D_ERR_INVALID, "bad table dimensions");
  if (!t->nlambda || !t->nudust || !t->kappad || !t->adust || !t->gdust || !t->pldust || !t->kappav || !t->lTint ||
      !t->nuint || !t->kapBint || !t->kappap || !t->hnuint || !t->atmosnu || !t->lognu || !t->loghnu)
    return fail(c, HC3D_ERR_INVALID, "a table pointer is NULL");
  CK(cudaSetDevice(c->device));
  if (c->tables) {
    // tables own their allocations at the front of model_allocs; rebuild the context tables
    return fail(c, HC3D_ERR_STATE, "tables already loaded in this context");
  }
  std::vector<double> nud((size_t)t->nlammax * kSlots), kap(nud.size()), alb(nud.size()), gg(nud.size()),
      pl(nud.size());
  std::vector<double> kB((size_t)t->nT * t->nnu * kSlots), kp((size_t)t->nT * kSlots);
  for (int s = 0; s < kSlots; ++s) {
    // a slot whose species the tables do not describe repeats slot 1's table (it holds no density)
    const int src = slot_src(c, s, t->ndg) >= 0 ? slot_src(c, s, t->ndg) : 0;
    const int nl = t->nlambda[src];
    if (nl < 2 || nl > t->nlammax) return fail(c, HC3D_ERR_INVALID, "nlambda out of range");
    c->dm.nlambda[s] = nl;
    for (int i = 0; i < t->nlammax; ++i) {
      const size_t o = (size_t)src * t->nlammax + i, q = (size_t)s * t->nlammax + i;
      nud[q] = t->nudust[o]; kap[q] = t->kappad[o]; alb[q] = t->adust[o]; gg[q] = t->gdust[o]; pl[q] = t->pldust[o];
    }
    std::memcpy(&kB[(size_t)s * t->nT * t->nnu], t->kapBint + (size_t)src * t->nT * t->nnu,
                sizeof(double) * t->nT * t->nnu);
    std::memcpy(&kp[(size_t)s * t->nT], t->kappap + (size_t)src * t->nT, sizeof(double) * t->nT);
    c->dm.kappav[s] = t->kappav[src];
    c->kappav[s] = t->kappav[src];
  }
  // unique dust tables: slots whose rows are identical share one table
  {
    const size_t L = (size_t)t->nlammax;
    std::vector<double> un(L * kSlots), uk(un.size()), ua(un.size()), ug(un.size()), up(un.size());
    int ntab = 0;
    size_t smem = 0;
    for (int s = 0; s < kSlots; ++s) {
      const int nl = c->dm.nlambda[s];
      int found = -1;
      for (int u = 0; u < ntab && found < 0; ++u) {
        if (c->dm.tab_nl[u] != nl) continue;
        const size_t so = (size_t)s * L, uo = (size_t)u * L, b = sizeof(double) * nl;
        if (!std::memcmp(&nud[so], &un[uo], b) && !std::memcmp(&kap[so], &uk[uo], b) &&
            !std::memcmp(&alb[so], &ua[uo], b) && !std::memcmp(&gg[so], &ug[uo], b) && !std::memcmp(&pl[so], &up[uo], b))
          found = u;
      }
      if (found < 0) {
        found = ntab++;
        const size_t so = (size_t)s * L, uo = (size_t)found * L;
        std::copy(&nud[so], &nud[so] + L, &un[uo]); std::copy(&kap[so], &kap[so] + L, &uk[uo]);
        std::copy(&alb[so], &alb[so] + L, &ua[uo]); std::copy(&gg[so], &gg[so] + L, &ug[uo]);
        std::copy(&pl[so], &pl[so] + L, &up[uo]);
        c->dm.tab_nl[found] = nl;
        smem += 5 * sizeof(double) * (size_t)nl;
      }
      c->dm.table_of[s] = found;
    }
    c->dm.ntab = ntab;
    c->dm.dust_smem = smem <= 48 * 1024 ? (int)smem : 0;
    un.resize(L * ntab); uk.resize(un.size()); ua.resize(un.size()); ug.resize(un.size()); up.resize(un.size());
    nud.swap(un); kap.swap(uk); alb.swap(ua); gg.swap(ug); pl.swap(up);
  }
  std::vector<void*>& own = c->model_allocs;
  int r;
  double *d_nud, *d_kap, *d_alb, *d_g, *d_pl, *d_lT, *d_nuint, *d_kB, *d_hn, *d_an, *d_ln, *d_lh;
  if ((r = dupload(c, own, &d_nud, nud.data(), nud.size())) || (r = dupload(c, own, &d_kap, kap.data(), kap.size())) ||
      (r = dupload(c, own, &d_alb, alb.data(), alb.size())) || (r = dupload(c, own, &d_g, gg.data(), gg.size())) ||
      (r = dupload(c, own, &d_pl, pl.data(), pl.size())) || (r = dupload(c, own, &d_lT, t->lTint, (size_t)t->nT)) ||
      (r = dupload(c, own, &d_nuint, t->nuint, (size_t)t->nnu)) || (r = dupload(c, own, &d_kB, kB.data(), kB.size())) ||
      (r = dupload(c, own, &c->d_kappap, kp.data(), kp.size())) ||
      (r = dupload(c, own, &d_hn, t->hnuint, (size_t)t->nhnu)) ||
      (r = dupload(c, own, &d_an, t->atmosnu, (size_t)t->nhnu)) ||
      (r = dupload(c, own, &d_ln, t->lognu, (size_t)t->nhnu)) ||
      (r = dupload(c, own, &d_lh, t->loghnu, (size_t)t->nhnu)))
    return r;
  c->dm.nlammax = t->nlammax;
  c->dm.nudust = d_nud; c->dm.kappad = d_kap; c->dm.adust = d_alb; c->dm.gdust = d_g; c->dm.pldust = d_pl;
  c->dm.nT = t->nT; c->dm.nnu = t->nnu; c->dm.lTint = d_lT; c->dm.nuint = d_nuint; c->dm.kapBint = d_kB;
  c->dm.nhnu = t->nhnu; c->dm.hnuint = d_hn; c->dm.atmosnu = d_an; c->dm.lognu = d_ln; c->dm.loghnu = d_lh;
  // external radiation field (isrf_mod), FP64 in both forms: one draw per external packet
  c->dm.nisrf = 0;
  if (t->nisrf > 0) {
    if (t->nisrf < 2 || !t->isrf_cdf || !t->isrf_logcdf || !t->isrf_logfreq)
      return fail(c, HC3D_ERR_INVALID, "external-illumination tables: nisrf < 2 or a NULL pointer");
    double *d_ic, *d_il, *d_if;
    if ((r = dupload(c, own, &d_ic, t->isrf_cdf, (size_t)t->nisrf)) ||
        (r = dupload(c, own, &d_il, t->isrf_logcdf, (size_t)t->nisrf)) ||
        (r = dupload(c, own, &d_if, t->isrf_logfreq, (size_t)t->nisrf)))
      return r;
    c->dm.nisrf = t->nisrf; c->dm.isrf_cdf = d_ic; c->dm.isrf_logcdf = d_il; c->dm.isrf_logfreq = d_if;
  }
  // partial sums of the blackbody sampler (zetainit, random.f90:79-97): inczeta(i) = sum_{j<=i} 1/j^4,
  // accumulated from j = izmax down to 1 as the reference does
  {
    std::vector<double> z(kIzmax, 0.0);
    for (int j = kIzmax; j >= 1; --j) {
      const double term = 1.0 / (double)(j * j * j * j);
      for (int i = kIzmax; i >= j; --i) z[i - 1] = z[i - 1] + term;
    }
    double* d_z;
    if ((r = dupload(c, own, &d_z, z.data(), z.size()))) return r;
    c->dm.inczeta = d_z;
  }
  // limb-darkening table (tabl_mod)
  c->dm.nlimb = 0;
  if (t->ntab > 0) {
    if (t->ntab < 2 || !t->limb_xmu || !t->limb_prob)
      return fail(c, HC3D_ERR_INVALID, "limb-darkening table: ntab < 2 or a NULL pointer");
    double *d_x, *d_p;
    if ((r = dupload(c, own, &d_x, t->limb_xmu, (size_t)t->ntab)) ||
        (r = dupload(c, own, &d_p, t->limb_prob, (size_t)t->ntab)))
      return r;
    c->dm.nlimb = t->ntab; c->dm.limb_xmu = d_x; c->dm.limb_prob = d_p;
  }
  // FP32 copies for the mixed form
  {
    auto f32 = [](const double* p, size_t n) { return std::vector<float>(p, p + n); };
    const float* fp[12] = {};
    const std::vector<float> h[12] = {
        f32(nud.data(), nud.size()), f32(kap.data(), kap.size()), f32(alb.data(), alb.size()),
        f32(gg.data(), gg.size()),   f32(pl.data(), pl.size()),   f32(t->lTint, (size_t)t->nT),
        f32(t->nuint, (size_t)t->nnu), f32(kB.data(), kB.size()), f32(t->hnuint, (size_t)t->nhnu),
        f32(t->atmosnu, (size_t)t->nhnu), f32(t->lognu, (size_t)t->nhnu), f32(t->loghnu, (size_t)t->nhnu)};
    for (int k = 0; k < 12; ++k) {
      float* d = nullptr;
      if ((r = dupload(c, own, &d, h[k].data(), h[k].size()))) return r;
      fp[k] = d;
    }
    c->dm.nudustf = fp[0]; c->dm.kappadf = fp[1]; c->dm.adustf = fp[2]; c->dm.gdustf = fp[3]; c->dm.pldustf = fp[4];
    c->dm.lTintf = fp[5]; c->dm.nuintf = fp[6]; c->dm.kapBintf = fp[7]; c->dm.hnuintf = fp[8];
    c->dm.atmosnuf = fp[9]; c->dm.lognuf = fp[10]; c->dm.loghnuf = fp[11];
  }
  // dust-table guide of the mixed form (see DevModel), on the FP32 tables
  {
    const size_t L = (size_t)t->nlammax;
    std::vector<short2> dg((size_t)kSlots * kDustGuide, make_short2(1, 1));
    for (int u = 0; u < c->dm.ntab; ++u) {
      const int nl = c->dm.tab_nl[u];
      std::vector<float> f(nl);
      for (int i = 0; i < nl; ++i) f[i] = (float)nud[(size_t)u * L + i];
      // i0(nu): the last row (1-based) with f[i-1] >= nu, for f[nl-1] < nu < f[0]
      auto i0 = [&](double nu) {
        int k = 1;
        while (k < nl - 1 && (double)f[k] >= nu) ++k;
        return k;
      };
      const double lo = std::log((double)f[nl - 1]), hi = std::log((double)f[0]);
      const double w = (hi - lo) / kDustGuide;
      for (int b = 0; b < kDustGuide; ++b) {
        const int a = i0(std::exp(lo + (b + 1) * w)), z = i0(std::exp(lo + b * w));
        dg[(size_t)u * kDustGuide + b] = make_short2((short)std::max(1, a - 1), (short)std::min(nl - 1, z + 1));
      }
      c->dm.dlnlo[u] = (float)lo;
      c->dm.dginv[u] = (float)(kDustGuide / (hi - lo));
    }
    short2* d_dg = nullptr;
    if ((r = dupload(c, own, &d_dg, dg.data(), dg.size()))) return r;
    c->dm.dguide = d_dg;
  }
  // Lucy CDF of the mixed form: row pairs interleaved per frequency, and the
  // guide of index brackets per probability level (see DevModel)
  {
    const int nT = t->nT, nnu = t->nnu;
    if (nnu > 32767) return fail(c, HC3D_ERR_INVALID, "nnu too large for the CDF guide");
    std::vector<float2> pair((size_t)kSlots * (nT - 1) * nnu);
    std::vector<short2> guide((size_t)kSlots * (nT - 1) * kGuide);
    std::vector<int> last((size_t)nT * (kGuide + 1));
    for (int s = 0; s < kSlots; ++s) {
      const double* K = kB.data() + (size_t)s * nT * nnu;
      auto kf = [&](int j, int i) { return (float)K[(size_t)(j - 1) + (size_t)nT * (i - 1)]; };
      // last[j][b]: the last index i with K(j,i) <= b/kGuide (0 if none), for a non-decreasing row
      for (int j = 1; j <= nT; ++j) {
        int i = 0;
        for (int b = 0; b <= kGuide; ++b) {
          const float lev = (float)b / (float)kGuide;
          while (i < nnu && kf(j, i + 1) <= lev) ++i;
          last[(size_t)(j - 1) * (kGuide + 1) + b] = i;
        }
      }
      for (int j = 1; j < nT; ++j) {
        float2* row = &pair[((size_t)s * (nT - 1) + (j - 1)) * nnu];
        for (int i = 1; i <= nnu; ++i) row[i - 1] = make_float2(kf(j, i), kf(j + 1, i));
        const int* a = &last[(size_t)(j - 1) * (kGuide + 1)];
        const int* b2 = &last[(size_t)j * (kGuide + 1)];
        short2* g = &guide[((size_t)s * (nT - 1) + (j - 1)) * kGuide];
        for (int b = 0; b < kGuide; ++b) {
          const int lo = std::max(1, std::min(a[b], b2[b]));
          const int hi = std::min(nnu, std::max(a[b + 1], b2[b + 1]) + 1);
          g[b] = make_short2((short)lo, (short)hi);
        }
      }
    }
    float2* d_pair = nullptr;
    short2* d_guide = nullptr;
    if ((r = dupload(c, own, &d_pair, pair.data(), pair.size())) ||
        (r = dupload(c, own, &d_guide, guide.data(), guide.size())))
      return r;
    c->dm.kpairf = d_pair;
    c->dm.kguide = d_guide;
  }
  c->tsub = t->tsub > 0.0 ? t->tsub : 1600.0;
  c->tables = true;
  if (c->grid) {
    k_peelmask<<<grid_blocks_for(c, c->dm.ncell), 256, 0, c->stream>>>(c->dm.ncell, c->d_tdust, c->tsub, c->d_peelmask,
                                                                       c->dm.rho4f, c->d_rho4p);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
  }
  return HC3D_OK;
}

extern "C" int hc3d_load_grid(hc3d_ctx* c, const hc3d_grid* g) {
  if (!c || !g) return HC3D_ERR_INVALID;
  if (g->nrg < 3 || g->ntg < 3 || g->npg < 2 || g->ndg < 1 || g->ndg > HC3D_NDG)
    return fail(c, HC3D_ERR_INVALID, "bad grid dimensions");
  if (!g->rarr || !g->r2arr || !g->thetarr || !g->costarr || !g->tan2arr || !g->phiarr || !g->aarr || !g->barr ||
      !g->densarr || !g->massarr || !g->tdust)
    return fail(c, HC3D_ERR_INVALID, "a grid pointer is NULL");
  CK(cudaSetDevice(c->device));
  const int nrg = g->nrg, ntg = g->ntg, npg = g->npg;
  const int64_t n4 = (int64_t)nrg * ntg * npg;
  const int64_t ncell = (int64_t)(nrg - 1) * (ntg - 1) * (npg - 1);
  // the kernels index cells with 32-bit arithmetic
  if (ncell >= ((int64_t)1 << 31) || 4 * ncell >= ((int64_t)1 << 31))
    return fail(c, HC3D_ERR_INVALID, "grid has 2^29 or more cells");
  // the species outside the four device slots must be empty
  for (int id = 0; id < g->ndg; ++id) {
    bool mapped = false;
    for (int s = 0; s < kSlots; ++s) mapped = mapped || c->species[s] == id + 1;
    if (mapped) continue;
    for (int64_t k = 0; k < n4; ++k)
      if (g->densarr[k + n4 * id] != 0.0)
        return fail(c, HC3D_ERR_UNSUPPORTED,
                    "species " + std::to_string(id + 1) + " holds density but no device slot carries it "
                    "(hc3d_set_species names the four species the device carries)");
  }
  for (int64_t k = 0; k < n4 * g->ndg; ++k)
    if (!(g->densarr[k] >= 0.0) || std::isinf(g->densarr[k]))
      return fail(c, HC3D_ERR_INVALID, "densarr holds a negative, NaN or infinite value");
  for (int i = 1; i < nrg; ++i)
    if (!(g->rarr[i] > g->rarr[i - 1])) return fail(c, HC3D_ERR_INVALID, "rarr must increase");
  free_all(c, c->grid_allocs);
  c->grid = false;
  std::vector<float> tan2f(ntg), hemi(ntg), af(npg), bf(npg);
  for (int i = 0; i < ntg; ++i) {
    tan2f[i] = (float)g->tan2arr[i];
    hemi[i] = g->costarr[i] > 0.0 ? 1.0f : -1.0f;
  }
  for (int i = 0; i < npg; ++i) {
    af[i] = (float)g->aarr[i];
    bf[i] = (float)g->barr[i];
  }
  int src_of[kSlots];
  for (int s = 0; s < kSlots; ++s) src_of[s] = slot_src(c, s, g->ndg);
  std::vector<float4> rf(ncell);
  std::vector<double> rd(4 * ncell, 0.0), td(4 * ncell, 0.1 / 11605.0), ma(4 * ncell, 0.0);
  for (int ip = 1; ip < npg; ++ip)
    for (int it = 1; it < ntg; ++it)
      for (int ir = 1; ir < nrg; ++ir) {
        const int64_t c4 = (int64_t)(ir - 1) + (int64_t)nrg * ((it - 1) + (int64_t)ntg * (ip - 1));
        const int64_t cc = (int64_t)(ir - 1) + (int64_t)(nrg - 1) * ((it - 1) + (int64_t)(ntg - 1) * (ip - 1));
        float v[4] = {0, 0, 0, 0};
        for (int s = 0; s < kSlots; ++s) {
          const int id = src_of[s];
          if (id < 0) continue;
          const double d = g->densarr[c4 + n4 * id];
          v[s] = (float)d;
          rd[4 * cc + s] = d;
          td[4 * cc + s] = g->tdust[c4 + n4 * id];
          ma[4 * cc + s] = g->massarr[c4 + n4 * id];
        }
        rf[cc] = make_float4(v[0], v[1], v[2], v[3]);
      }
  std::vector<void*>& own = c->grid_allocs;
  int r;
  double *d_r, *d_r2, *d_th, *d_ct, *d_ph, *d_t2, *d_a, *d_b, *d_rd;
  float *d_t2f, *d_hemi, *d_af, *d_bf;
  float4* d_rf;
  if ((r = dupload(c, own, &d_r, g->rarr, (size_t)nrg)) || (r = dupload(c, own, &d_r2, g->r2arr, (size_t)nrg)) ||
      (r = dupload(c, own, &d_th, g->thetarr, (size_t)ntg)) || (r = dupload(c, own, &d_ct, g->costarr, (size_t)ntg)) ||
      (r = dupload(c, own, &d_ph, g->phiarr, (size_t)npg)) ||
      (r = dupload(c, own, &d_t2, g->tan2arr, (size_t)ntg)) || (r = dupload(c, own, &d_a, g->aarr, (size_t)npg)) ||
      (r = dupload(c, own, &d_b, g->barr, (size_t)npg)) || (r = dupload(c, own, &d_t2f, tan2f.data(), tan2f.size())) ||
      (r = dupload(c, own, &d_hemi, hemi.data(), hemi.size())) || (r = dupload(c, own, &d_af, af.data(), af.size())) ||
      (r = dupload(c, own, &d_bf, bf.data(), bf.size())) || (r = dupload(c, own, &d_rf, rf.data(), rf.size())) ||
      (r = dupload(c, own, &d_rd, rd.data(), rd.size())) || (r = dupload(c, own, &c->d_tdust, td.data(), td.size())) ||
      (r = dupload(c, own, &c->d_massarr, ma.data(), ma.size())) || (r = dalloc(c, own, &c->d_peelmask, (size_t)ncell)) ||
      (r = dalloc(c, own, &c->d_rho4p, (size_t)ncell)))
    return r;
  {
    const std::vector<float> tdf(td.begin(), td.end());
    if ((r = dupload(c, own, &c->d_tdustf, tdf.data(), tdf.size()))) return r;
  }
  DevTallies& t = c->dt;
  if ((r = dalloc(c, own, &t.nabs, (size_t)kSlots * ncell)) || (r = dalloc(c, own, &t.dtauabs, (size_t)kSlots * ncell)) ||
      (r = dalloc(c, own, &t.jmean, (size_t)ncell)) || (r = dalloc(c, own, &t.killed, (size_t)ncell)) ||
      (r = dalloc(c, own, &t.dbig, (size_t)ncell)))
    return r;
  // small-grain tallies and the int_mean result, when a slot holds small grains
  t.dsg = nullptr; t.jsg = nullptr;
  c->d_imean = nullptr; c->d_imfract = nullptr;
  c->imean_set = false;
  c->d_vcell = nullptr;
  if (has_sg_slots(c)) {
    std::vector<double> vc((size_t)ncell);
    for (int ip = 1; ip < npg; ++ip)
      for (int it = 1; it < ntg; ++it)
        for (int ir = 1; ir < nrg; ++ir) {
          const int64_t c4 = (int64_t)(ir - 1) + (int64_t)nrg * ((it - 1) + (int64_t)ntg * (ip - 1));
          const int64_t cc = (int64_t)(ir - 1) + (int64_t)(nrg - 1) * ((it - 1) + (int64_t)(ntg - 1) * (ip - 1));
          vc[cc] = g->vcell[c4];
          if (!(vc[cc] > 0.0)) return fail(c, HC3D_ERR_INVALID, "vcell must be positive (int_mean divides by it)");
        }
    if ((r = dalloc(c, own, &t.dsg, (size_t)ncell)) || (r = dalloc(c, own, &t.jsg, (size_t)ncell)) ||
        (r = dalloc(c, own, &c->d_imean, (size_t)ncell)) || (r = dalloc(c, own, &c->d_imfract, (size_t)ncell)) ||
        (r = dupload(c, own, &c->d_vcell, vc.data(), vc.size())))
      return r;
    CK(cudaMemsetAsync(t.dsg, 0, sizeof(unsigned int) * ncell, c->stream));
    CK(cudaMemsetAsync(t.jsg, 0, sizeof(unsigned long long) * ncell, c->stream));
  }
  DevModel& m = c->dm;
  m.nrg = nrg; m.ntg = ntg; m.npg = npg; m.ncell = ncell;
  m.rarr = d_r; m.r2arr = d_r2; m.thetarr = d_th; m.costarr = d_ct; m.phiarr = d_ph; m.tan2d = d_t2; m.tan2f = d_t2f; m.hemi = d_hemi;
  {
    std::vector<float> rf32(g->rarr, g->rarr + nrg), r2f32(g->r2arr, g->r2arr + nrg);
    float *d_rarrf = nullptr, *d_r2arrf = nullptr;
    if ((r = dupload(c, own, &d_rarrf, rf32.data(), rf32.size())) ||
        (r = dupload(c, own, &d_r2arrf, r2f32.data(), r2f32.size())))
      return r;
    m.rarrf = d_rarrf;
    m.r2arrf = d_r2arrf;
    std::vector<float2> cs(ntg);
    for (int i = 0; i < ntg; ++i) cs[i] = make_float2((float)std::cos(g->thetarr[i]), (float)std::sin(g->thetarr[i]));
    float2* d_cs = nullptr;
    if ((r = dupload(c, own, &d_cs, cs.data(), cs.size()))) return r;
    m.thcs = d_cs;
    std::vector<float2> r2p(nrg - 1), cf(ntg), pf(npg), cc(ntg);
    for (int i = 0; i < nrg - 1; ++i) r2p[i] = make_float2(r2f32[i], r2f32[i + 1]);
    for (int i = 0; i < ntg; ++i) cf[i] = make_float2(tan2f[i], hemi[i]);
    for (int i = 0; i < ntg; ++i) {
      // cos^2 theta of the wall; the midplane (tan2arr = -1) and the poles (tan2arr = 0) are marked
      const double cth = std::cos(g->thetarr[i]);
      if (g->tan2arr[i] < 0.0) cc[i] = make_float2(-1.f, 0.f);
      else if (g->tan2arr[i] == 0.0) cc[i] = make_float2(1.f, 0.f);
      else cc[i] = make_float2((float)(cth * cth), hemi[i]);
    }
    for (int i = 0; i < npg; ++i) pf[i] = make_float2(af[i], bf[i]);
    float2 *d_r2p = nullptr, *d_cf = nullptr, *d_pf = nullptr, *d_cc = nullptr;
    if ((r = dupload(c, own, &d_r2p, r2p.data(), r2p.size())) || (r = dupload(c, own, &d_cf, cf.data(), cf.size())) ||
        (r = dupload(c, own, &d_pf, pf.data(), pf.size())) || (r = dupload(c, own, &d_cc, cc.data(), cc.size())))
      return r;
    m.r2pair = d_r2p;
    m.conef = d_cf;
    m.conec = d_cc;
    m.planef = d_pf;
  }
  m.aarrd = d_a; m.barrd = d_b; m.aarrf = d_af; m.barrf = d_bf; m.rho4f = d_rf; m.rho4d = d_rd;
  m.peelmask = c->d_peelmask; m.rho4p = c->d_rho4p; m.tdust = c->d_tdust; m.tdustf = c->d_tdustf;
  m.imean = c->d_imean; m.imfract = c->d_imfract;
  c->ndg_in = g->ndg;
  k_peelmask<<<grid_blocks_for(c, ncell), 256, 0, c->stream>>>(ncell, c->d_tdust, c->tsub, c->d_peelmask, d_rf,
                                                                c->d_rho4p);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->stream));
  c->grid = true;
  return hc3d_zero_tallies(c);
}

extern "C" int hc3d_set_wave_options(hc3d_ctx* c, int64_t queue_records, int regen, int qchunk, int peel_shape) {
  if (!c || queue_records < 0 || regen < 0 || regen > 32 || qchunk < 0 || qchunk > 64 || peel_shape < 0 ||
      peel_shape > kPeelVariants)
    return HC3D_ERR_INVALID;
  if (c->chunk_open) return fail(c, HC3D_ERR_STATE, "a chunked iteration has packets in flight");
  if (queue_records > 0 && queue_records < 1024) return fail(c, HC3D_ERR_INVALID, "queue_records < 1024");
  if ((queue_records && queue_records != c->queue_records) || (qchunk && qchunk != c->qchunk)) {
    drop_wave(c);  // reallocated at the next peeled run
    if (queue_records) c->queue_records = queue_records;
    if (qchunk) c->qchunk = qchunk;
  }
  if (regen) c->regen = regen;
  if (peel_shape) c->peel_variant = peel_shape - 1;
  return HC3D_OK;
}

extern "C" int hc3d_set_tdust(hc3d_ctx* c, const double* tdust) {
  if (!c || !tdust) return HC3D_ERR_INVALID;
  if (!c->grid) return fail(c, HC3D_ERR_STATE, "load the grid first");
  CK(cudaSetDevice(c->device));
  const int nrg = c->dm.nrg, ntg = c->dm.ntg, npg = c->dm.npg;
  const int64_t n4 = (int64_t)nrg * ntg * npg, ncell = c->dm.ncell;
  // the device layout of hc3d_load_grid: 4 slots per compact cell; empty slots keep the floor value
  std::vector<double> td(4 * ncell, 0.1 / 11605.0);
  for (int ip = 1; ip < npg; ++ip)
    for (int it = 1; it < ntg; ++it)
      for (int ir = 1; ir < nrg; ++ir) {
        const int64_t c4 = (int64_t)(ir - 1) + (int64_t)nrg * ((it - 1) + (int64_t)ntg * (ip - 1));
        const int64_t cc = (int64_t)(ir - 1) + (int64_t)(nrg - 1) * ((it - 1) + (int64_t)(ntg - 1) * (ip - 1));
        for (int s = 0; s < kSlots; ++s) {
          const int id = slot_src(c, s, c->ndg_in);
          if (id < 0) continue;
          const double v = tdust[c4 + n4 * id];
          if (!(v >= 0.0) || std::isinf(v)) return fail(c, HC3D_ERR_INVALID, "tdust holds a negative, NaN or infinite value");
          td[4 * cc + s] = v > 0.0 ? v : 0.1 / 11605.0;  // 0: the 0.1 K floor of the starting field
        }
      }
  const std::vector<float> tdf(td.begin(), td.end());
  CK(cudaMemcpyAsync(c->d_tdust, td.data(), td.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->d_tdustf, tdf.data(), tdf.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
  k_peelmask<<<grid_blocks_for(c, ncell), 256, 0, c->stream>>>(ncell, c->d_tdust, c->tsub, c->d_peelmask, c->dm.rho4f,
                                                                c->d_rho4p);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->stream));
  return HC3D_OK;
}

extern "C" int hc3d_zero_tallies(hc3d_ctx* c) {
  if (!c) return HC3D_ERR_INVALID;
  CK(cudaSetDevice(c->device));
  if (c->grid) {
    const int64_t n = c->dm.ncell;
    CK(cudaMemsetAsync(c->dt.nabs, 0, sizeof(unsigned long long) * kSlots * n, c->stream));
    CK(cudaMemsetAsync(c->dt.dtauabs, 0, sizeof(unsigned long long) * kSlots * n, c->stream));
    CK(cudaMemsetAsync(c->dt.jmean, 0, sizeof(unsigned long long) * n, c->stream));
    CK(cudaMemsetAsync(c->dt.killed, 0, sizeof(unsigned int) * n, c->stream));
    CK(cudaMemsetAsync(c->dt.dbig, 0, sizeof(unsigned int) * n, c->stream));
    if (c->dt.dsg) CK(cudaMemsetAsync(c->dt.dsg, 0, sizeof(unsigned int) * n, c->stream));
    if (c->dt.jsg) CK(cudaMemsetAsync(c->dt.jsg, 0, sizeof(unsigned long long) * n, c->stream));
  }
  if (c->run_tallies) {
    CK(cudaMemsetAsync(c->dt.sed, 0, sizeof(unsigned long long) * 9 * c->dims.nsed, c->stream));
    CK(cudaMemsetAsync(c->dt.psed, 0, sizeof(unsigned long long) * 9 * std::max<int64_t>(c->dims.npsed, 1), c->stream));
    CK(cudaMemsetAsync(c->dt.img, 0, sizeof(unsigned long long) * 4 * std::max<int64_t>(c->dims.nimg, 1), c->stream));
    if (c->dims.ncube > 0)
      CK(cudaMemsetAsync(c->dt.cube, 0, sizeof(unsigned long long) * (kNo + 3) * c->dims.ncube, c->stream));
  }
  CK(cudaMemsetAsync(c->dt.counters, 0, sizeof(unsigned long long) * 16, c->stream));
  CK(cudaMemsetAsync(c->dt.fault_count, 0, sizeof(unsigned long long), c->stream));
  CK(cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->scales_set = false;
  c->epoch_np = 0;
  c->status_seen = 0;
  c->chunk_open = false;  // packets of an unfinished chunked iteration are discarded
  c->carry_alive = 0;
  return HC3D_OK;
}

// Launch shape of the per-thread transport kernel: a persistent grid of the
// resident blocks, or fewer blocks when the batch is small.
LaunchCfg transport_cfg(hc3d_ctx* c, int64_t np) {
  LaunchCfg cfg;
  cfg.threads = c->block_size;
  cfg.stream = c->stream;
  if (c->grid_blocks > 0) {
    cfg.blocks = c->grid_blocks;
    return cfg;
  }
  int per_sm = 0;
  cudaError_t e;
  if (c->precision == HC3D_PREC_FP64) {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, transport_fn_fp64(), cfg.threads, c->dm.dust_smem);
  } else {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, transport_fn_mixed(), cfg.threads, c->dm.dust_smem);
  }
  if (e != cudaSuccess || per_sm < 1) per_sm = 1;
  cfg.blocks = c->sm_count * per_sm;
  const int64_t need = (np + cfg.threads - 1) / cfg.threads;
  if (need < cfg.blocks) cfg.blocks = (int)std::max<int64_t>(1, need);
  return cfg;
}

extern "C" int hc3d_run_iteration(hc3d_ctx* c, const hc3d_run_params* p) {
  if (!c) return HC3D_ERR_INVALID;
  if (c->chunk_open)
    return fail(c, HC3D_ERR_STATE, "a chunked iteration has packets in flight: end it with hc3d_run_chunk(final = 1) "
                                   "or discard it with hc3d_zero_tallies()");
  CK(cudaSetDevice(c->device));
  RunArgs a;
  int r = prepare_run(c, p, &a);
  if (r) return r;
  if (p->np == 0) return HC3D_OK;
  CK(cudaMemsetAsync(c->d_work, 0, sizeof(unsigned long long), c->stream));
  if (p->ipeel && c->use_waves) {
    if ((r = run_waves(c, p, a))) return r;
    if ((r = finish_run(c))) return r;
    c->epoch_np += p->np;
    return HC3D_OK;
  }
  const LaunchCfg cfg = transport_cfg(c, p->np);
  CK(cudaEventRecord(c->ev0, c->stream));
  cudaError_t e = c->precision == HC3D_PREC_FP64 ? launch_transport_fp64(c->dm, c->dt, c->dims, a, cfg)
                                                 : launch_transport_mixed(c->dm, c->dt, c->dims, a, cfg);
  if (e != cudaSuccess) return fail(c, HC3D_ERR_CUDA, std::string("transport launch: ") + cudaGetErrorString(e));
  CK(cudaEventRecord(c->ev1, c->stream));
  if ((r = finish_run(c))) return r;
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->last_ms = ms;
  c->last_transport_ms = ms;
  c->last_peel_ms = 0.0;
  c->last_launches = 1;
  c->epoch_np += p->np;
  return HC3D_OK;
}

extern "C" int hc3d_run_chunk(hc3d_ctx* c, const hc3d_run_params* p, int64_t np_iteration, int final) {
  if (!c || !p) return HC3D_ERR_INVALID;
  if (!p->ipeel || !c->use_waves) {
    // the per-thread form finishes every packet it starts: a chunk is a run
    if (np_iteration < p->np) return fail(c, HC3D_ERR_INVALID, "np_iteration < np");
    if (!c->scales_set && c->grid && c->tables) set_scales(c, np_iteration);
    return hc3d_run_iteration(c, p);
  }
  if (np_iteration < p->np) return fail(c, HC3D_ERR_INVALID, "np_iteration < np");
  CK(cudaSetDevice(c->device));
  if (!c->scales_set && !c->chunk_open && c->grid && c->tables) {
    // the fixed-point scales of the whole iteration (prepare_run keeps them)
    const TallyDims d = dims_of(p);
    if (!c->run_tallies || !same_dims(d, c->dims)) {
      int r = check_params(c, p);
      if (r) return r;
      if ((r = alloc_run_tallies(c, d))) return r;
    }
    set_scales(c, np_iteration);
  }
  RunArgs a;
  int r = prepare_run(c, p, &a);
  if (r) return r;
  if (c->chunk_open && (a.key0 != c->chunk_key0 || a.key1 != c->chunk_key1))
    return fail(c, HC3D_ERR_STATE, "the chunks of an iteration must share its seed and iteration number");
  CK(cudaMemsetAsync(c->d_work, 0, sizeof(unsigned long long), c->stream));
  if ((r = run_waves(c, p, a, final != 0))) return r;
  if ((r = finish_run(c))) return r;
  c->epoch_np += p->np;
  return HC3D_OK;
}

// Several models' packets in one persistent launch (k_transport_batch): the
// Lucy iterations of a model grid run as one launch per iteration, the
// small models' long-history tails beside the bulk of the others.  Each
// context keeps its own tallies, which equal those of hc3d_run_iteration.
extern "C" int hc3d_run_batch(hc3d_ctx* const* ctxs, const hc3d_run_params* params, int n) {
  if (!ctxs || !params || n < 1 || n > kMaxBatch) return HC3D_ERR_INVALID;
  hc3d_ctx* c = ctxs[0];
  if (!c) return HC3D_ERR_INVALID;
  for (int j = 0; j < n; ++j) {
    if (!ctxs[j]) return HC3D_ERR_INVALID;
    if (ctxs[j]->device != c->device || ctxs[j]->precision != c->precision)
      return fail(c, HC3D_ERR_INVALID, "batched contexts must share the device and the precision");
    for (int i = 0; i < j; ++i)
      if (ctxs[i] == ctxs[j]) return fail(c, HC3D_ERR_INVALID, "a context appears twice in the batch");
  }
  CK(cudaSetDevice(c->device));
  std::vector<BatchItem> items((size_t)n);
  std::vector<int64_t> first((size_t)n + 1, 0);
  for (int j = 0; j < n; ++j) {
    hc3d_ctx* cj = ctxs[j];
    const int r = prepare_run(cj, &params[j], &items[(size_t)j].a);
    if (r) {
      if (cj != c) c->err = "model " + std::to_string(j) + ": " + cj->err;
      return r;
    }
    if (cudaStreamSynchronize(cj->stream) != cudaSuccess) return fail(c, HC3D_ERR_CUDA, "batch: stream sync");
    items[(size_t)j].m = cj->dm;
    items[(size_t)j].m.dust_smem = 0;
    items[(size_t)j].t = cj->dt;
    items[(size_t)j].d = cj->dims;
    first[(size_t)j + 1] = first[(size_t)j] + params[j].np;
  }
  const int64_t total = first[(size_t)n];
  if (total == 0) return HC3D_OK;
  std::vector<void*> tmp;
  BatchItem* d_items = nullptr;
  int64_t* d_first = nullptr;
  unsigned long long* d_work = nullptr;
  int r;
  if ((r = dupload(c, tmp, &d_items, items.data(), items.size())) ||
      (r = dupload(c, tmp, &d_first, first.data(), first.size())) || (r = dalloc(c, tmp, &d_work, 1))) {
    free_all(c, tmp);
    return r;
  }
  CK(cudaMemsetAsync(d_work, 0, sizeof(unsigned long long), c->stream));
  int per_sm = 0;
  const bool f64 = c->precision == HC3D_PREC_FP64;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f64 ? transport_batch_fn_fp64() : transport_batch_fn_mixed(),
                                                    128, 0) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  LaunchCfg cfg;
  cfg.threads = 128;
  cfg.blocks = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)c->sm_count * per_sm, (total + 127) / 128));
  cfg.stream = c->stream;
  CK(cudaEventRecord(c->ev0, c->stream));
  cudaError_t e = f64 ? launch_transport_batch_fp64(d_items, d_first, n, d_work, total, cfg)
                      : launch_transport_batch_mixed(d_items, d_first, n, d_work, total, cfg);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev1, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  free_all(c, tmp);
  if (e != cudaSuccess) return fail(c, HC3D_ERR_CUDA, std::string("batched transport: ") + cudaGetErrorString(e));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  for (int j = 0; j < n; ++j) {
    hc3d_ctx* cj = ctxs[j];
    if ((r = finish_run(cj))) return r;
    cj->epoch_np += params[j].np;
    cj->last_ms = cj->last_transport_ms = ms;
    cj->last_peel_ms = 0.0;
    cj->last_launches = 1;
  }
  return HC3D_OK;
}

// The autotuner: times one sample batch under each candidate launch setting
// and keeps the fastest.  Peeled runs (the wavefront form) tune the depth of
// the peel-off queue, which sets the events per packet in a wave and so the
// number of waves; runs without peel-off tune the block size of the
// per-thread transport kernel.  Every candidate runs the same packets (the
// streams are keyed by packet id), so the timings differ by the setting
// alone.  The tallies are zeroed afterwards.
extern "C" int hc3d_autotune(hc3d_ctx* c, const hc3d_run_params* sample, hc3d_tune_result* out) {
  if (!c || !sample || !out || sample->np <= 0) return HC3D_ERR_INVALID;
  if (!c->tables || !c->grid) return fail(c, HC3D_ERR_STATE, "load tables and grid first");
  if (c->chunk_open) return fail(c, HC3D_ERR_STATE, "a chunked iteration has packets in flight");
  std::memset(out, 0, sizeof *out);
  const bool waves = sample->ipeel && c->use_waves;
  const int64_t q0 = c->queue_records;
  const int b0 = c->block_size, g0 = c->regen, v0 = c->peel_variant;
  // time the sample under the context's current settings as candidate k.
  // Peeled runs time it as the middle chunk of an iteration (after a chunk
  // of the same size that fills the pool; the packets in flight are then
  // discarded), so that the longest histories' tail does not decide the
  // choice; other runs time the whole sample.
  auto time_one = [&](int k) -> int {
    int r = hc3d_zero_tallies(c);
    double ms = 0.0;
    if (!r && waves) {
      hc3d_run_params q = *sample;
      q.packet_offset = sample->packet_offset + sample->np;
      r = hc3d_run_chunk(c, sample, 2 * sample->np, 0);
      const auto t0 = std::chrono::steady_clock::now();
      if (!r) r = hc3d_run_chunk(c, &q, 2 * sample->np, 0);
      ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      if (!r) r = hc3d_zero_tallies(c);
    } else if (!r) {
      const auto t0 = std::chrono::steady_clock::now();
      r = hc3d_run_iteration(c, sample);
      ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    if (r) {
      c->chunk_open = false;
      c->carry_alive = 0;
      if (c->queue_records != q0) drop_wave(c);
      c->queue_records = q0;
      c->block_size = b0;
      c->regen = g0;
      c->peel_variant = v0;
      return r;
    }
    out->queue_records[k] = c->queue_records;
    out->block_size[k] = c->block_size;
    out->regen[k] = c->regen;
    out->peel_shape[k] = c->peel_variant;
    out->peel_threads[k] = c->precision == HC3D_PREC_MIXED ? peel_threads_mixed(c->peel_variant) : 256;
    out->ms[k] = ms;
    if (k == 0 || ms < out->ms[out->best]) out->best = k;
    return HC3D_OK;
  };
  int n = 0, r;
  if (waves) {
    // the queue depth at the current threshold, then the threshold at the best depth
    const int64_t queues[4] = {1 << 20, 1 << 21, 1 << 22, 1 << 23};
    for (int k = 0; k < 4; ++k, ++n) {
      if (c->queue_records != queues[k]) {
        drop_wave(c);  // reallocated by the next run at the new depth
        c->queue_records = queues[k];
      }
      if ((r = time_one(n))) return r;
    }
    const int64_t qbest = out->queue_records[out->best];
    if (c->queue_records != qbest) drop_wave(c);
    c->queue_records = qbest;
    const int regens[4] = {1, 4, 8, 16};
    for (int k = 0; k < 4; ++k) {
      if (regens[k] == out->regen[out->best]) continue;  // timed above
      c->regen = regens[k];
      if ((r = time_one(n++))) return r;
    }
    c->regen = out->regen[out->best];
    if (c->precision == HC3D_PREC_MIXED) {
      // the peel-off kernel's block shape at the best depth and threshold
      for (int v = 0; v < kPeelVariants; ++v) {
        if (v == out->peel_shape[out->best]) continue;
        c->peel_variant = v;
        if ((r = time_one(n++))) return r;
      }
      c->peel_variant = out->peel_shape[out->best];
    }
  } else {
    const int blocks[3] = {64, 96, 128};
    for (int k = 0; k < 3; ++k, ++n) {
      c->block_size = blocks[k];
      if ((r = time_one(n))) return r;
    }
    c->block_size = out->block_size[out->best];
  }
  out->n = n;
  return hc3d_zero_tallies(c);
}

extern "C" int hc3d_get_fault_log(hc3d_ctx* c, uint64_t* entries, int max, int* n) {
  if (!c || !n) return HC3D_ERR_INVALID;
  unsigned long long cnt = 0;
  if (int r_ = d2h(c, &cnt, c->dt.fault_count, sizeof(cnt))) return r_;
  *n = (int)std::min<unsigned long long>(cnt, (unsigned long long)kFaultLog);
  if (entries && max > 0) {
    const int k = std::min(*n, max);
    if (k) if (int r_ = d2h(c, entries, c->dt.fault_log, sizeof(uint64_t) * k)) return r_;
  }
  *n = (int)std::min<unsigned long long>(cnt, (unsigned long long)0x7fffffff);
  return HC3D_OK;
}

extern "C" int hc3d_get_wave_log(hc3d_ctx* c, double* out, int max_waves, int* n) {
  if (!c || !n) return HC3D_ERR_INVALID;
  *n = (int)(c->wave_log.size() / 6);
  if (out)
    std::copy(c->wave_log.begin(), c->wave_log.begin() + 6 * std::min(*n, std::max(max_waves, 0)), out);
  return HC3D_OK;
}

extern "C" int hc3d_last_launch_stats(hc3d_ctx* c, int* launches, double* transport_ms, double* peel_ms) {
  if (!c) return HC3D_ERR_INVALID;
  if (launches) *launches = c->last_launches;
  if (transport_ms) *transport_ms = c->last_transport_ms;
  if (peel_ms) *peel_ms = c->last_peel_ms;
  return HC3D_OK;
}

extern "C" int hc3d_get_tallies(hc3d_ctx* c, const hc3d_run_params* p, hc3d_tallies* out) {
  if (!c || !out) return HC3D_ERR_INVALID;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  if (!c->grid) return fail(c, HC3D_ERR_STATE, "no grid loaded");
  if (p && c->run_tallies && !same_dims(dims_of(p), c->dims))
    return fail(c, HC3D_ERR_INVALID, "params do not match the tally shape of the runs");
  out->stokes_scale = c->dt.stokes_scale;
  out->square_scale = c->dt.square_scale;
  out->path_scale = c->dt.path_scale;
  if (c->run_tallies) {
    int64_t* sed[9] = {out->si, out->sq, out->su, out->sv, out->si2, out->sq2, out->su2, out->sv2, out->nums};
    for (int k = 0; k < 9; ++k)
      if (sed[k]) if (int r_ = d2h(c, sed[k], c->dt.sed + k * c->dims.nsed, sizeof(int64_t) * c->dims.nsed)) return r_;
    int64_t* ps[9] = {out->ti, out->tq, out->tu, out->tv, out->ti2, out->tq2, out->tu2, out->tv2, out->numt};
    if (c->dims.npsed > 0)
      for (int k = 0; k < 9; ++k)
        if (ps[k]) if (int r_ = d2h(c, ps[k], c->dt.psed + k * c->dims.npsed, sizeof(int64_t) * c->dims.npsed)) return r_;
    int64_t* im[4] = {out->image_i, out->image_q, out->image_u, out->image_v};
    if (c->dims.nimg > 0)
      for (int k = 0; k < 4; ++k)
        if (im[k]) if (int r_ = d2h(c, im[k], c->dt.img + k * c->dims.nimg, sizeof(int64_t) * c->dims.nimg)) return r_;
    const int64_t nc = c->dims.ncube;
    if (nc > 0) {
      if (out->image_m_i)
        if (int r_ = d2h(c, out->image_m_i, c->dt.cube, sizeof(int64_t) * kNo * nc)) return r_;
      int64_t* qv[3] = {out->image_m_q, out->image_m_u, out->image_m_v};
      for (int k = 0; k < 3; ++k)
        if (qv[k]) if (int r_ = d2h(c, qv[k], c->dt.cube + (kNo + k) * nc, sizeof(int64_t) * nc)) return r_;
    }
  }
  const DevModel& m = c->dm;
  const int64_t n = m.ncell, n4 = (int64_t)m.nrg * m.ntg * m.npg;
  const int ndg = c->ndg_in;
  // device slot s goes to the species it holds in the (nrg,ntg,npg,ndg) layout; slots = 1 for a per-cell tally
  auto scatter = [&](const std::vector<unsigned long long>& src, int slots, int64_t* dst) {
    std::fill(dst, dst + n4 * slots, 0);
    for (int s = 0; s < std::min(slots, kSlots); ++s) {
      const int id = slots == 1 ? 0 : slot_src(c, s, slots);
      if (id < 0) continue;
      for (int ip = 1; ip < m.npg; ++ip)
        for (int it = 1; it < m.ntg; ++it)
          for (int ir = 1; ir < m.nrg; ++ir) {
            const int64_t c4 = (int64_t)(ir - 1) + (int64_t)m.nrg * ((it - 1) + (int64_t)m.ntg * (ip - 1));
            const int64_t cc = (int64_t)(ir - 1) + (int64_t)(m.nrg - 1) * ((it - 1) + (int64_t)(m.ntg - 1) * (ip - 1));
            dst[c4 + n4 * id] = (int64_t)src[(size_t)s * n + cc];
          }
    }
  };
  std::vector<unsigned long long> buf;
  if (out->nabs) {
    buf.resize((size_t)kSlots * n);
    if (int r_ = d2h(c, buf.data(), c->dt.nabs, sizeof(unsigned long long) * buf.size())) return r_;
    scatter(buf, ndg, out->nabs);
  }
  if (out->dtauabs) {
    buf.resize((size_t)kSlots * n);
    if (int r_ = d2h(c, buf.data(), c->dt.dtauabs, sizeof(unsigned long long) * buf.size())) return r_;
    scatter(buf, ndg, out->dtauabs);
  }
  if (out->jmean) {
    buf.resize((size_t)n);
    if (int r_ = d2h(c, buf.data(), c->dt.jmean, sizeof(unsigned long long) * n)) return r_;
    scatter(buf, 1, out->jmean);
  }
  auto scatter32 = [&](const unsigned int* dsrc, int32_t* dst) -> int {
    std::vector<unsigned int> b32((size_t)n);
    if (int r_ = d2h(c, b32.data(), dsrc, sizeof(unsigned int) * n)) return r_;
    std::fill(dst, dst + n4, 0);
    for (int ip = 1; ip < m.npg; ++ip)
      for (int it = 1; it < m.ntg; ++it)
        for (int ir = 1; ir < m.nrg; ++ir) {
          const int64_t c4 = (int64_t)(ir - 1) + (int64_t)m.nrg * ((it - 1) + (int64_t)m.ntg * (ip - 1));
          const int64_t cc = (int64_t)(ir - 1) + (int64_t)(m.nrg - 1) * ((it - 1) + (int64_t)(m.ntg - 1) * (ip - 1));
          dst[c4] = (int32_t)b32[cc];
        }
    return HC3D_OK;
  };
  int r;
  if (out->killed && (r = scatter32(c->dt.killed, out->killed))) return r;
  if (out->dbig && (r = scatter32(c->dt.dbig, out->dbig))) return r;
  if (out->dsg) {
    if (c->dt.dsg) {
      if ((r = scatter32(c->dt.dsg, out->dsg))) return r;
    } else {
      std::fill(out->dsg, out->dsg + n4, 0);
    }
  }
  if (out->jsg) {
    if (c->dt.jsg) {
      buf.resize((size_t)n);
      if (int r_ = d2h(c, buf.data(), c->dt.jsg, sizeof(unsigned long long) * n)) return r_;
      scatter(buf, 1, out->jsg);
    } else {
      std::fill(out->jsg, out->jsg + n4, 0);
    }
  }
  unsigned long long cnt[16];
  if (int r_ = d2h(c, cnt, c->dt.counters, sizeof(cnt))) return r_;
  for (int k = 0; k < 16; ++k) out->counters[k] = (int64_t)cnt[k];
  return HC3D_OK;
}

LucyArgs lucy_args(hc3d_ctx* c, double ltot, int64_t np) {
  LucyArgs a;
  a.ncell = c->dm.ncell;
  a.nT = c->dm.nT;
  a.lTint = c->dm.lTint;
  a.kappap = c->d_kappap;
  for (int s = 0; s < kSlots; ++s) a.kappav[s] = c->kappav[s];
  a.ltot = ltot;
  a.nphot = (double)np;
  a.path_scale = c->dt.path_scale;
  a.tsub = c->tsub;
  a.na_min = 1.0e4;
  a.nslots = 0;  // the slots the host arrays describe (a prefix: the species ascend)
  for (int s = 0; s < kSlots; ++s)
    if (slot_src(c, s, c->ndg_in) >= 0) a.nslots = s + 1;
  return a;
}

IntMeanArgs intmean_args(hc3d_ctx* c, double ltot, int64_t np) {
  IntMeanArgs a{};
  a.ncell = c->dm.ncell;
  a.nr1 = c->dm.nrg - 1;
  a.path_scale = c->dt.path_scale;
  a.jconst = 1.0 / c->dm.sg_jfacd / (4.0 * 3.1415926535897932384626433);
  a.nphot = (double)np;
  a.ltot = ltot;
  a.isrfkap_int = c->isrfkap_int;
  a.nemit = c->dm.sg_nemit;
  a.rarr = c->dm.rarr;
  a.vcell = c->d_vcell;
  a.uratio = c->d_uratio;
  return a;
}

// the device temperatures into the reference's (nrg,ntg,npg,ndg) layout; the
// species no slot carries keep the 0.1 K floor of the starting field
int tdust_to_host(hc3d_ctx* c, double* tdust_out) {
  const DevModel& m = c->dm;
  const int64_t n = m.ncell, n4 = (int64_t)m.nrg * m.ntg * m.npg;
  std::vector<double> td((size_t)4 * n);
  if (int r_ = d2h(c, td.data(), c->d_tdust, sizeof(double) * td.size())) return r_;
  std::fill(tdust_out, tdust_out + n4 * c->ndg_in, 0.1 / 11605.0);
  for (int s = 0; s < kSlots; ++s) {
    const int id = slot_src(c, s, c->ndg_in);
    if (id < 0) continue;
    for (int ip = 1; ip < m.npg; ++ip)
      for (int it = 1; it < m.ntg; ++it)
        for (int ir = 1; ir < m.nrg; ++ir) {
          const int64_t c4 = (int64_t)(ir - 1) + (int64_t)m.nrg * ((it - 1) + (int64_t)m.ntg * (ip - 1));
          const int64_t cc = (int64_t)(ir - 1) + (int64_t)(m.nrg - 1) * ((it - 1) + (int64_t)(m.ntg - 1) * (ip - 1));
          tdust_out[c4 + n4 * id] = td[4 * cc + s];
        }
  }
  return HC3D_OK;
}

extern "C" int hc3d_set_lucy_tally(hc3d_ctx* c, const int64_t* dtauabs) {
  if (!c || !dtauabs) return HC3D_ERR_INVALID;
  if (!c->grid) return fail(c, HC3D_ERR_STATE, "load the grid first");
  if (!c->scales_set) return fail(c, HC3D_ERR_STATE, "no packets were run since the last hc3d_zero_tallies()");
  CK(cudaSetDevice(c->device));
  const DevModel& m = c->dm;
  const int64_t n = m.ncell, n4 = (int64_t)m.nrg * m.ntg * m.npg;
  std::vector<unsigned long long> buf((size_t)kSlots * n, 0ull);
  for (int s = 0; s < kSlots; ++s) {
    const int id = slot_src(c, s, c->ndg_in);
    if (id < 0) continue;
    for (int ip = 1; ip < m.npg; ++ip)
      for (int it = 1; it < m.ntg; ++it)
        for (int ir = 1; ir < m.nrg; ++ir) {
          const int64_t c4 = (int64_t)(ir - 1) + (int64_t)m.nrg * ((it - 1) + (int64_t)m.ntg * (ip - 1));
          const int64_t cc = (int64_t)(ir - 1) + (int64_t)(m.nrg - 1) * ((it - 1) + (int64_t)(m.ntg - 1) * (ip - 1));
          buf[(size_t)s * n + cc] = (unsigned long long)dtauabs[c4 + n4 * id];
        }
  }
  CK(cudaMemcpyAsync(c->dt.dtauabs, buf.data(), sizeof(unsigned long long) * buf.size(), cudaMemcpyHostToDevice,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return HC3D_OK;
}

extern "C" int hc3d_lucy_update(hc3d_ctx* c, double ltot, int64_t np, double* tdust_out, double* max_rel_change,
                                int* converged) {
  if (!c) return HC3D_ERR_INVALID;
  if (!c->tables || !c->grid) return fail(c, HC3D_ERR_STATE, "load tables and grid first");
  if (!(ltot > 0.0) || np <= 0) return fail(c, HC3D_ERR_INVALID, "need ltot > 0 and np > 0");
  if (!c->scales_set) return fail(c, HC3D_ERR_STATE, "no packets were run since the last hc3d_zero_tallies()");
  CK(cudaSetDevice(c->device));
  const LucyArgs a = lucy_args(c, ltot, np);
  CK(cudaMemsetAsync(c->d_maxrel, 0, sizeof(unsigned long long), c->stream));
  k_lucy<<<grid_blocks_for(c, a.ncell), 256, 0, c->stream>>>(a, c->dt.dtauabs, c->dm.rho4d, c->d_massarr, c->d_tdust, c->d_tdustf,
                                                           c->d_peelmask, c->d_maxrel, c->dm.rho4f, c->d_rho4p);
  CK(cudaGetLastError());
  if (c->dm.sg_on) {
    const IntMeanArgs ia = intmean_args(c, ltot, np);
    k_intmean<<<grid_blocks_for(c, ia.ncell), 256, 0, c->stream>>>(ia, c->dt.jsg, c->d_imean, c->d_imfract);
    CK(cudaGetLastError());
    c->imean_set = true;
  }
  unsigned long long bits = 0;
  CK(cudaMemcpyAsync(&bits, c->d_maxrel, sizeof(bits), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  double rel;
  std::memcpy(&rel, &bits, sizeof(rel));
  if (max_rel_change) *max_rel_change = rel;
  if (converged) *converged = rel < 0.01 ? 1 : 0;
  if (tdust_out) return tdust_to_host(c, tdust_out);
  return HC3D_OK;
}

// The Lucy iterations of newtts.F90:294-330 with a fixed count, captured as
// one CUDA graph: per iteration, the tally reset of initarr(.false.), the
// packet loop without peel-off and the temperature update (tfinal).  The
// graph's kernels read their arguments from the capture, so iteration k runs
// with iter = p->iter + k exactly as hc3d_zero_tallies + hc3d_run_iteration
// + hc3d_lucy_update would; no host step sits between the iterations.
extern "C" int hc3d_lucy_iterations(hc3d_ctx* c, const hc3d_run_params* p, int n_iter, double ltot,
                                    double* max_rel_change, double* tdust_out) {
  if (!c || !p || !max_rel_change || n_iter < 1 || n_iter > 1000) return HC3D_ERR_INVALID;
  if (p->ipeel) return fail(c, HC3D_ERR_INVALID, "the Lucy iterations run without peel-off (ipeel = 0)");
  if (!(ltot > 0.0) || p->np <= 0) return fail(c, HC3D_ERR_INVALID, "need ltot > 0 and np > 0");
  if (!c->tables || !c->grid) return fail(c, HC3D_ERR_STATE, "load tables and grid first");
  CK(cudaSetDevice(c->device));
  std::vector<RunArgs> args((size_t)n_iter);
  for (int k = 0; k < n_iter; ++k) {
    hc3d_run_params q = *p;
    q.iter = p->iter + k;
    c->scales_set = false;  // each iteration starts from zeroed tallies
    c->epoch_np = 0;
    const int r = prepare_run(c, &q, &args[(size_t)k]);
    if (r) return r;
    if (c->dm.sg_on) c->imean_set = true;  // the graph's int_mean of iteration k feeds iteration k + 1
  }
  const IntMeanArgs ia = intmean_args(c, ltot, p->np);
  std::vector<void*> tmp;
  unsigned long long* d_rel = nullptr;
  int r = dalloc(c, tmp, &d_rel, (size_t)n_iter);
  if (r) return r;
  const LaunchCfg cfg = transport_cfg(c, p->np);
  const LucyArgs la = lucy_args(c, ltot, p->np);
  const int64_t n = c->dm.ncell;
  CK(cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream));
  CK(cudaMemsetAsync(c->dt.fault_count, 0, sizeof(unsigned long long), c->stream));
  CK(cudaMemsetAsync(d_rel, 0, sizeof(unsigned long long) * n_iter, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  cudaGraph_t graph = nullptr;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < n_iter && e == cudaSuccess; ++k) {
    const cudaStream_t st = c->stream;
    if (e == cudaSuccess) e = cudaMemsetAsync(c->dt.nabs, 0, sizeof(unsigned long long) * kSlots * n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->dt.dtauabs, 0, sizeof(unsigned long long) * kSlots * n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->dt.jmean, 0, sizeof(unsigned long long) * n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->dt.killed, 0, sizeof(unsigned int) * n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->dt.dbig, 0, sizeof(unsigned int) * n, st);
    if (e == cudaSuccess && c->dt.dsg) e = cudaMemsetAsync(c->dt.dsg, 0, sizeof(unsigned int) * n, st);
    if (e == cudaSuccess && c->dt.jsg) e = cudaMemsetAsync(c->dt.jsg, 0, sizeof(unsigned long long) * n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->dt.sed, 0, sizeof(unsigned long long) * 9 * c->dims.nsed, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->dt.counters, 0, sizeof(unsigned long long) * 16, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_work, 0, sizeof(unsigned long long), st);
    if (e == cudaSuccess)
      e = c->precision == HC3D_PREC_FP64 ? launch_transport_fp64(c->dm, c->dt, c->dims, args[(size_t)k], cfg)
                                         : launch_transport_mixed(c->dm, c->dt, c->dims, args[(size_t)k], cfg);
    if (e == cudaSuccess) {
      k_lucy<<<grid_blocks_for(c, la.ncell), 256, 0, st>>>(la, c->dt.dtauabs, c->dm.rho4d, c->d_massarr, c->d_tdust,
                                                           c->d_tdustf, c->d_peelmask, d_rel + k, c->dm.rho4f,
                                                           c->d_rho4p);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess && c->dm.sg_on) {
      k_intmean<<<grid_blocks_for(c, ia.ncell), 256, 0, st>>>(ia, c->dt.jsg, c->d_imean, c->d_imfract);
      e = cudaGetLastError();
    }
  }
  const cudaError_t ec = cudaStreamEndCapture(c->stream, &graph);
  if (e == cudaSuccess) e = ec;
  cudaGraphExec_t exec = nullptr;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev0, c->stream);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev1, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    free_all(c, tmp);
    return fail(c, HC3D_ERR_CUDA, std::string("Lucy graph: ") + cudaGetErrorString(e));
  }
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->last_ms = ms;
  c->last_transport_ms = ms;
  c->last_peel_ms = 0.0;
  c->last_launches = 2 * n_iter;
  std::vector<unsigned long long> bits((size_t)n_iter);
  r = d2h(c, bits.data(), d_rel, sizeof(unsigned long long) * n_iter);
  free_all(c, tmp);
  if (r) return r;
  for (int k = 0; k < n_iter; ++k) std::memcpy(&max_rel_change[k], &bits[(size_t)k], sizeof(double));
  if ((r = finish_run(c))) return r;
  // the tallies now hold the last iteration, as after the step-by-step loop
  c->scales_set = true;
  c->epoch_np = p->np;
  if (tdust_out) return tdust_to_host(c, tdust_out);
  return HC3D_OK;
}

extern "C" int hc3d_trace_packets(hc3d_ctx* c, const hc3d_run_params* p, int npkt, const double* uniforms, int nu,
                                  hc3d_trace_rec* recs, int max_rec, int32_t* nrec) {
  if (!c || !uniforms || !recs || !nrec || npkt < 1 || nu < 1 || max_rec < 1) return HC3D_ERR_INVALID;
  if ((int64_t)npkt * nu > (int64_t)1 << 28 || (int64_t)npkt * max_rec > (int64_t)1 << 26)
    return fail(c, HC3D_ERR_INVALID, "trace request too large");
  CK(cudaSetDevice(c->device));
  hc3d_run_params q = *p;
  q.np = npkt;
  RunArgs a;
  int r = prepare_run(c, &q, &a);
  if (r) return r;
  std::vector<void*> tmp;
  double* d_u;
  hc3d_trace_rec* d_rec;
  int* d_n;
  if ((r = dupload(c, tmp, &d_u, uniforms, (size_t)npkt * nu)) || (r = dalloc(c, tmp, &d_rec, (size_t)npkt * max_rec)) ||
      (r = dalloc(c, tmp, &d_n, (size_t)npkt))) {
    free_all(c, tmp);
    return r;
  }
  a.inj = d_u;
  a.ninj = nu;
  a.trace = d_rec;
  a.max_rec = max_rec;
  a.nrec = d_n;
  LaunchCfg cfg;
  cfg.threads = 128;
  cfg.blocks = (npkt + 127) / 128;
  cfg.stream = c->stream;
  cudaError_t e = c->precision == HC3D_PREC_FP64 ? launch_transport_fp64(c->dm, c->dt, c->dims, a, cfg)
                                                 : launch_transport_mixed(c->dm, c->dt, c->dims, a, cfg);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(recs, d_rec, sizeof(hc3d_trace_rec) * (size_t)npkt * max_rec, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(nrec, d_n, sizeof(int32_t) * npkt, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  free_all(c, tmp);
  if (e != cudaSuccess) return fail(c, HC3D_ERR_CUDA, std::string("trace: ") + cudaGetErrorString(e));
  c->epoch_np += npkt;
  return HC3D_OK;
}
