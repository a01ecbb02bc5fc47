// hc3d_device.h -- device-side data layout shared by the transport kernels
// and the C-ABI layer.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/hc3d.h"

namespace hc3d {

constexpr int kSlots = 4;   // species slots carried on the device (disk1, disk2, and two of species 3-8)
constexpr int kNo = 8;      // SED components (output.F90:232-239)
constexpr int kMaxPeel = 256;
constexpr int kFaultLog = 256;
constexpr int kGuide = 64;      // probability levels of the Lucy-CDF guide table
constexpr int kDustGuide = 64;  // ln(nu) buckets of the dust-table guide
constexpr int kIzmax = 145;     // terms of the blackbody sampler's mixture (random.f90:17)

// Fortran-layout sizes of the tally arrays of one run configuration.
struct TallyDims {
  int nfreq, nmu, nph, nap, npeel, nx;
  int64_t nsed;    // nfreq*nmu*nph*nap*no
  int64_t npsed;   // nfreq*npeel*nap*no
  int64_t nimg;    // npeel*nx*nx
  int64_t ncube;   // npeel*nx*nx*nfreq with the image cube, else 0
};

// Device tallies (int64 fixed point).  Grid tallies use the compact cell
// index c = (ir-1) + (nrg-1)*((it-1) + (ntg-1)*(ip-1)).
struct DevTallies {
  unsigned long long* sed;    // [9][nsed]: si sq su sv si2 sq2 su2 sv2 nums
  unsigned long long* psed;   // [9][npsed]: ti .. numt
  unsigned long long* img;    // [4][nimg]: I Q U V
  unsigned long long* cube;   // [kNo + 3][ncube]: I of the kNo SED components, then Q U V (image cube)
  unsigned long long* nabs;   // [kSlots][ncell]
  unsigned long long* dtauabs;// [kSlots][ncell]
  unsigned long long* jmean;  // [ncell]
  unsigned int* killed;       // [ncell]
  unsigned int* dbig;         // [ncell]
  unsigned int* dsg;          // [ncell] small-grain absorptions (models with small-grain slots)
  unsigned long long* jsg;    // [ncell] small-grain absorption path, the input of int_mean (same)
  unsigned long long* counters; // [16]
  double stokes_scale, square_scale, path_scale;
  unsigned long long* fault_log;   // [kFaultLog]: packet id | code << 56
  unsigned long long* fault_count;
};

// Read-only model data on the device.
struct DevModel {
  // grid
  int nrg, ntg, npg;
  int64_t ncell;
  const double* rarr;     // (nrg)
  const float* rarrf;     // (nrg)
  const float* r2arrf;    // (nrg) squares of rarr rounded to FP32
  const double* r2arr;    // (nrg)
  const double* thetarr;  // (ntg)
  const double* costarr;  // (ntg) cos of the polar walls (accretion packets locate their cell by it)
  const double* phiarr;   // (npg)
  const double* tan2d;    // (ntg)
  const float* tan2f;     // (ntg)
  const float* hemi;      // (ntg) +1 upper, -1 lower (cone nappe)
  const float2* thcs;     // (ntg) cos, sin of the polar walls (mixed-form safe distance)
  // interleaved FP32 wall data of the mixed-form wall search (one load per family)
  const float2* r2pair;   // (nrg-1) squared inner and outer radius of radial cell ir (index ir-1)
  const float2* conef;    // (ntg) tan^2 and hemisphere sign of polar wall it (index it-1)
  const float2* conec;    // (ntg) cos^2 theta and hemisphere sign of polar wall it: C < 0 marks the
                          // midplane, a hemisphere sign of 0 a pole (mixed-form peel-off walk)
  const float2* planef;   // (npg) A = sin(phi), B = -cos(phi) of azimuthal wall ip (index ip-1)
  const double* aarrd; const double* barrd;  // (npg)
  const float* aarrf; const float* barrf;    // (npg)
  const float4* rho4f;    // (ncell) species slots x,y,z,w  (mixed form)
  const double* rho4d;    // (ncell*4)                     (FP64 form)
  const unsigned char* peelmask;  // (ncell) bit s: tdust(s) < Tsub
  const float4* rho4p;    // (ncell) rho4f with the slots outside the peel mask zeroed (mixed-form peel-off)
  const double* tdust;    // (ncell*4) K/11605
  const float* tdustf;    // (ncell*4) FP32 copy (mixed form)
  // dust tables
  int nlammax;
  int nlambda[kSlots];
  int ntab;               // unique dust tables (species slots reading the same file share one)
  int table_of[kSlots];   // slot -> table
  int tab_nl[kSlots];     // rows of each table
  int dust_smem;          // bytes of dynamic shared memory staging the tables; 0 = global memory
  const double* nudust; const double* kappad; const double* adust; const double* gdust; const double* pldust;  // (nlammax, ntab)
  double kappav[kSlots];
  int nT, nnu;
  const double* lTint; const double* nuint; const double* kapBint;  // kapBint (nT,nnu,kSlots)
  int nhnu;
  const double* hnuint; const double* atmosnu; const double* lognu; const double* loghnu;
  int nisrf;  // external radiation field (isrf_mod): cdf_i, logcdf_i, logfreq_i; 0 = none
  const double* isrf_cdf; const double* isrf_logcdf; const double* isrf_logfreq;
  const double* inczeta;   // (kIzmax) partial sums of 1/i^4 of bbfreq (random.f90:79-97)
  int nlimb;  // rows of the limb-darkening table (tabl_mod ntab), CLIMB=YES; 0 = none
  const double* limb_xmu; const double* limb_prob;
  // FP32 copies of the per-event tables, read by the mixed form
  const float* nudustf; const float* kappadf; const float* adustf; const float* gdustf; const float* pldustf;
  const float* lTintf; const float* nuintf; const float* kapBintf;
  const float* hnuintf; const float* atmosnuf; const float* lognuf; const float* loghnuf;
  // Lucy CDF of the mixed form: kpairf[(slot*(nT-1) + j-1)*nnu + i-1] = (K(j,i), K(j+1,i)) of the
  // FP32 kapBint rows j and j+1; kguide[(slot*(nT-1) + j-1)*kGuide + b] = (lo, hi) brackets the
  // frequency index where the interpolated CDF of rows j, j+1 crosses a level in [b, b+1)/kGuide
  const float2* kpairf;
  const short2* kguide;
  // dust-table guide of the mixed form: dguide[u*kDustGuide + b] = (lo, hi) brackets the row i0 of
  // table u (nud(i0) >= nu > nud(i0+1)) for ln(nu) in bucket b of [dlnlo[u], dlnlo[u] + kDustGuide/dginv[u])
  const short2* dguide;
  float dlnlo[kSlots], dginv[kSlots];
  // species of the slots (grid_mod.f90:13-20): bit s of disk_mask = slot s holds a disk species
  // (absorbed packets take origin 2, propagate.f90:114-119), of sg_mask = small grains
  unsigned disk_mask, sg_mask;
  // very small grains and PAHs (emit_common.f90:31-53, rep_draine.f90, draine_cdf.f90)
  int sg_on;              // 1: sg_mask != 0 and the emission spectra are loaded
  int sg_slot;            // the slot whose opacity weights the jsg path tally
  float sg_jfac;          // 1 / (rstar_cm kappa_V) of sg_slot: kapd -> kappa/kappa_V
  double sg_jfacd;
  int sg_nemit, sg_nd;    // 18 spectra x 1000 frequencies
  const double* sg_cdf;   // [j * sg_nd + i]: cdf_d(j+1, i+1)
  const double* sg_logcdf;// [j * sg_nd + i]: logcdf_d(j+1, i+1)
  const double* sg_logfreq; // (sg_nd)
  const int* imean;       // (ncell) spectrum row 1..nemit of each cell (int_mean.f90:64-94)
  const double* imfract;  // (ncell) its interpolation fraction
};

// One call of the packet loop.
struct RunArgs {
  int64_t np, packet_offset;
  uint32_t key0, key1;
  int ipeel, npeel, image;
  int nfreq, nmu, nph, nap, nx;
  double rmaxi, fractxh;
  double numin, lnurat;
  double rstar_cm;
  float kapfac[kSlots];      // rstar_cm * kappa_V of each slot, FP32 (mixed-form opacities)
  int iintmax;
  int64_t max_interactions;
  int limb;                  // 1: Eddington limb darkening of the stellar emission
  int ext_illum;             // packets with global id >= n_star enter from the outer sphere
  int64_t n_star;
  double rmax;               // outer radius, R*
  int64_t n_acc, n_spot;     // ids < n_acc: disk accretion; [n_acc, n_spot): hot spot
  int src_on;                // 1: src holds the accretion and spot constants
  int regen;                 // k_wave regeneration threshold: waiting lanes of a warp before they take new packets
  int qchunk;                // k_wave: peel-off queue slots a lane reserves at a time
  int imcube;                // 1: tally the per-frequency image cube
  int iter1;                 // 1: the first Lucy iteration (small grains emit from spectrum row 2)
  hc3d_sources src;
  const double* peeldir;     // [npeel][4]: coste sinte cospe sinpe
  const double* aperture2;   // [nap]
  unsigned long long* work;  // packet counter
  int* status;               // first fault code
  // trace harness
  const double* inj; int ninj;
  void* trace; int max_rec; int* nrec;
};

struct LaunchCfg {
  int blocks, threads;
  cudaStream_t stream;
  int variant = 0;  // block shape of the mixed-form peel-off kernel (see peel_threads_mixed)
};

constexpr int kPeelVariants = 2;  // block shapes of the mixed-form peel-off kernel

// entry points of the two instantiations
cudaError_t launch_transport_mixed(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                   const LaunchCfg& cfg);
cudaError_t launch_transport_fp64(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                  const LaunchCfg& cfg);
// Buffers of the wavefront form: the packet pool (one slot per thread of
// k_wave) and two peel-off event queues, so that the peel-off rays of one
// wave are walked while k_wave fills the other queue with the next wave.
struct WaveBufs {
  void* pool;
  void* queue[2];
  unsigned long long* qcount[2];
  unsigned int* alive;
  unsigned long long* next_ray[2];  // ray counters of k_peel
};

// k_wave: advance every live packet by up to E events, appending peel-off
// records to queue q; k_peel: walk the peel-off rays of queue q.
cudaError_t launch_wave_transport_mixed(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                        const WaveBufs& w, int q, int E, const LaunchCfg& cfg);
cudaError_t launch_wave_peel_mixed(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                   const WaveBufs& w, int q, const LaunchCfg& cfg);
cudaError_t launch_wave_transport_fp64(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                       const WaveBufs& w, int q, int E, const LaunchCfg& cfg);
cudaError_t launch_wave_peel_fp64(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                  const WaveBufs& w, int q, const LaunchCfg& cfg);
size_t slot_bytes_mixed();
size_t slot_bytes_fp64();
size_t rec_bytes_mixed();
size_t rec_bytes_fp64();
const void* wave_fn_mixed();
const void* wave_fn_fp64();
const void* peel_fn_mixed(int variant);
int peel_threads_mixed(int variant);
const void* peel_fn_fp64();

// One model of a batched launch: its device model (dust tables read from
// global memory), tallies, tally shape and run arguments.
struct BatchItem {
  DevModel m;
  DevTallies t;
  TallyDims d;
  RunArgs a;
};
constexpr int kMaxBatch = 256;
// k_transport over the packets of several models at once: packet g of the
// launch belongs to model j with first[j] <= g < first[j+1]
cudaError_t launch_transport_batch_mixed(const BatchItem* items, const int64_t* first, int n, unsigned long long* work,
                                         int64_t total, const LaunchCfg& cfg);
cudaError_t launch_transport_batch_fp64(const BatchItem* items, const int64_t* first, int n, unsigned long long* work,
                                        int64_t total, const LaunchCfg& cfg);
const void* transport_batch_fn_mixed();
const void* transport_batch_fn_fp64();

int transport_regs_mixed();
int transport_regs_fp64();
const void* transport_fn_mixed();
const void* transport_fn_fp64();

}  // namespace hc3d
