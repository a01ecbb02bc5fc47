// hc3d_noalloc.cu -- the Lucy temperature update without any allocation.
//
// hc3d_lucy_update() works on the device buffers of a context, which
// hc3d_create()/hc3d_load_grid() obtain with cudaMalloc.  Some callers cannot
// allocate device memory at the point where they need the update: a Fortran
// host whose arrays already live in managed or pre-registered memory and that
// runs under a memory pool it does not own, an in-situ coupling inside
// another code's CUDA graph, or a service that has reserved all of its device
// memory up front.  hc3d_lucy_update_noalloc() serves them: the caller passes
// every input and output as a device pointer, and the only working memory --
// the per-block maxima of the convergence test and a completion counter -- is
// a file-scope __device__ array of fixed size in this translation unit.
//
// The array exists once per device that loads the library and lives until
// the process exits.  Every call shares it: it keeps the last call's contents,
// the counter is cleared at the start of each call, and two calls that
// overlap on the GPU (different streams, or different host threads without
// ordering) race on it.
#include <algorithm>
#include <cstdio>
#include <cstring>

#include "../../include/hc3d.h"
#include "hc3d_lucy.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kPerThread = 4;
constexpr long long kMaxBlocks = HC3D_NOALLOC_MAX_ELEMENTS / (kThreads * kPerThread);

// [0, kMaxBlocks): per-block maxima of |T_new - T_old| / T_new (as ordered
// bits of non-negative doubles); [kMaxBlocks]: blocks finished;
// [kMaxBlocks + 1]: the maximum over all blocks.
static __device__ __align__(256) unsigned long long g_lucy_scratch[kMaxBlocks + 2];

struct Args {
  int nrg, ntg, npg, ndg;
  long long n;  // nrg*ntg*npg*ndg
  const long long* dtauabs;
  double path_scale;
  const double *densarr, *massarr, *tdust_in;
  double* tdust_out;
  int nT;
  const double *lTint, *kappap;
  double kappav[HC3D_NDG];
  double ltot, nphot, na_min;
};

__global__ void __launch_bounds__(kThreads) k_lucy_noalloc(Args a, unsigned long long* scratch) {
  __shared__ unsigned long long smax[kThreads / 32];
  __shared__ bool last;
  unsigned long long mx = 0;
  const long long n4 = (long long)a.nrg * a.ntg * a.npg;
  const long long base = (long long)blockIdx.x * kThreads * kPerThread;
#pragma unroll
  for (int j = 0; j < kPerThread; ++j) {
    const long long k = base + (long long)j * kThreads + threadIdx.x;
    if (k >= a.n) break;
    const int s = (int)(k / n4);
    const long long c4 = k - (long long)s * n4;
    const int ir = (int)(c4 % a.nrg);
    const int it = (int)((c4 / a.nrg) % a.ntg);
    const int ip = (int)(c4 / ((long long)a.nrg * a.ntg));
    const double T0 = a.tdust_in[k];
    double T = T0;
    if (ir < a.nrg - 1 && it < a.ntg - 1 && ip < a.npg - 1 && a.densarr[k] > 0.0) {
      const double na = (double)a.dtauabs[k] / a.path_scale;
      T = hc3d::lucy_dusttemp(a.lTint, a.nT, a.kappap + (size_t)s * a.nT, a.kappav[s], a.ltot, a.nphot, na, T0,
                              a.massarr[k]);
      if (na >= a.na_min) {
        const unsigned long long bits = (unsigned long long)__double_as_longlong(fabs(T - T0) / T);
        mx = bits > mx ? bits : mx;
      }
    }
    a.tdust_out[k] = T;
  }
  // block maximum, then the last block to finish reduces the block maxima
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long v = __shfl_down_sync(0xffffffffu, mx, o);
    mx = v > mx ? v : mx;
  }
  if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long b = 0;
    for (int w = 0; w < kThreads / 32; ++w) b = smax[w] > b ? smax[w] : b;
    scratch[blockIdx.x] = b;
    __threadfence();
    last = atomicAdd(&scratch[kMaxBlocks], 1ull) == (unsigned long long)gridDim.x - 1;
  }
  __syncthreads();
  if (last) {
    unsigned long long b = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += kThreads) {
      const unsigned long long v = ((volatile unsigned long long*)scratch)[i];
      b = v > b ? v : b;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long v = __shfl_down_sync(0xffffffffu, b, o);
      b = v > b ? v : b;
    }
    if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long r = 0;
      for (int w = 0; w < kThreads / 32; ++w) r = smax[w] > r ? smax[w] : r;
      scratch[kMaxBlocks + 1] = r;
    }
  }
}

}  // namespace

extern "C" int hc3d_lucy_update_noalloc(const hc3d_lucy_buffers* b, double* max_rel_change, int* converged) {
  if (!b || !b->dtauabs || !b->densarr || !b->massarr || !b->tdust_in || !b->tdust_out || !b->lTint || !b->kappap)
    return HC3D_ERR_INVALID;
  if (b->nrg < 2 || b->ntg < 2 || b->npg < 2 || b->ndg < 1 || b->ndg > HC3D_NDG || b->nT < 2 || b->np <= 0 ||
      !(b->ltot > 0.0) || !(b->path_scale > 0.0))
    return HC3D_ERR_INVALID;
  const long long n = (long long)b->nrg * b->ntg * b->npg * b->ndg;
  if (n > HC3D_NOALLOC_MAX_ELEMENTS) {
    std::fprintf(stderr,
                 "hc3d_lucy_update_noalloc: %lld grid elements (nrg*ntg*npg*ndg) exceed the maximum of %lld; "
                 "use hc3d_lucy_update\n",
                 n, (long long)HC3D_NOALLOC_MAX_ELEMENTS);
    return HC3D_ERR_INVALID;
  }
  if (b->device < 0 || b->device >= 64) return HC3D_ERR_INVALID;
  if (cudaSetDevice(b->device) != cudaSuccess) return HC3D_ERR_CUDA;
  // the scratch array's address on this device, looked up on every call (it
  // allocates nothing), so that a context the host recreated finds it anew
  void* addr = nullptr;
  if (cudaGetSymbolAddress(&addr, g_lucy_scratch) != cudaSuccess || !addr) return HC3D_ERR_CUDA;
  unsigned long long* scratch = static_cast<unsigned long long*>(addr);
  cudaStream_t st = static_cast<cudaStream_t>(b->stream);
  if (cudaMemsetAsync(scratch + kMaxBlocks, 0, 2 * sizeof(unsigned long long), st) != cudaSuccess)
    return HC3D_ERR_CUDA;
  Args a;
  std::memset(&a, 0, sizeof a);
  a.nrg = b->nrg; a.ntg = b->ntg; a.npg = b->npg; a.ndg = b->ndg; a.n = n;
  a.dtauabs = reinterpret_cast<const long long*>(b->dtauabs);
  a.path_scale = b->path_scale;
  a.densarr = b->densarr; a.massarr = b->massarr; a.tdust_in = b->tdust_in; a.tdust_out = b->tdust_out;
  a.nT = b->nT; a.lTint = b->lTint; a.kappap = b->kappap;
  for (int s = 0; s < b->ndg; ++s) a.kappav[s] = b->kappav[s];
  a.ltot = b->ltot;
  a.nphot = (double)b->np;
  a.na_min = 1.0e4;
  const long long blocks = (n + (long long)kThreads * kPerThread - 1) / ((long long)kThreads * kPerThread);
  k_lucy_noalloc<<<(unsigned)blocks, kThreads, 0, st>>>(a, scratch);
  if (cudaGetLastError() != cudaSuccess) return HC3D_ERR_CUDA;
  unsigned long long bits = 0;
  if (cudaMemcpyAsync(&bits, scratch + kMaxBlocks + 1, sizeof(bits), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return HC3D_ERR_CUDA;
  double rel;
  std::memcpy(&rel, &bits, sizeof rel);
  if (max_rel_change) *max_rel_change = rel;
  if (converged) *converged = rel < 0.01 ? 1 : 0;
  return HC3D_OK;
}
