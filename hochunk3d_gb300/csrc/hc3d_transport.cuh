// hc3d_transport.cuh -- the photon-packet loop as sm_103a device code.
//
// One templated implementation, instantiated twice:
//   R = double : the all-FP64 form.  Its translation unit is compiled with
//                --fmad=false so that it rounds like the CPU restatement of
//                the reference and can be compared with it packet by packet.
//   R = float  : the mixed form.  Directions, Stokes vectors, angles, cone and
//                plane roots, opacities and the propagation tau integral are
//                FP32.  FP64 is kept for the position, the radial-face
//                quadratic (cancellation-free form), the cumulative peel-off
//                escape tau and the per-event table lookups (opacset,
//                lucydustfreq, atmosfreq).
//
// The routine-by-routine structure follows the reference: disk() packet loop
// (newdisktherm.F90:256-377), propagate (propagate.f90:27-319), the cell walk
// (radface.f90:44-62, phiface.f90:48-56, closest_wall.f90:13-66, thetaface and
// tauint restated from their call sites peeloff_3d.f90:88-154), scattering
// (stokes.f90:46-388, dustmat.f90:40-65, select_dust.f90:16-42), re-emission
// (reemit.f90:17-34, lucydustfreq.f90:19-157) and peel-off (peeloff_3d.f90:
// 52-286, findangle3.f90:31-67, stokespeel.f90:49-376).  Random draws are
// taken in the same order as the Fortran; the stream is counter-based
// Philox4x32-10 keyed by (seed, iteration, packet id).
//
// Execution: a persistent grid; every thread takes the next packet id from a
// global counter when its packet ends (regeneration), so the cost of long
// packet histories is balanced across the device.  All tallies are int64
// fixed-point atomics: sums do not depend on the order packets finish in.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "hc3d_device.h"

namespace hc3d {
namespace dev {

constexpr double kPi = 3.1415926535897932384626433;
constexpr double kR2p = 2.0 * kPi;
constexpr double kTauMax = 25.0;  // peeloff_3d.f90:40

// ---- math overloads ---------------------------------------------------------
__device__ __forceinline__ float xsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double xsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float xcos(float x) { return cosf(x); }
__device__ __forceinline__ double xcos(double x) { return cos(x); }
__device__ __forceinline__ float xsin(float x) { return sinf(x); }
__device__ __forceinline__ double xsin(double x) { return sin(x); }
__device__ __forceinline__ float xacos(float x) { return acosf(x); }
__device__ __forceinline__ double xacos(double x) { return acos(x); }
__device__ __forceinline__ float xlog(float x) { return logf(x); }
__device__ __forceinline__ double xlog(double x) { return log(x); }
__device__ __forceinline__ float xabs(float x) { return fabsf(x); }
__device__ __forceinline__ double xabs(double x) { return fabs(x); }
template <class R> __device__ __forceinline__ R rhuge();
template <> __device__ __forceinline__ float rhuge<float>() { return 3.402823466e38f; }
template <> __device__ __forceinline__ double rhuge<double>() { return 1.7976931348623157e308; }

// ---- Philox4x32-10 (Salmon et al., SC'11) -------------------------------------
struct Rng {
  uint32_t k0, k1, c0, c2, c3;
  uint32_t b[4];
  int left;
  const double* inj;
  int ninj, pos;
};

__device__ __forceinline__ void philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                       uint32_t k1, uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

__device__ __forceinline__ void rng_init(Rng& r, uint32_t key0, uint32_t key1, uint64_t pid) {
  r.k0 = key0; r.k1 = key1; r.c0 = 0;
  r.c2 = (uint32_t)pid; r.c3 = (uint32_t)(pid >> 32);
  r.left = 0; r.inj = nullptr; r.ninj = 0; r.pos = 0;
}

// a[i] of a four-element array by selects, so that the array stays in
// registers (a runtime index would place it in local memory)
template <class T>
__device__ __forceinline__ T pick4(const T (&a)[4], int i) {
  return i == 0 ? a[0] : (i == 1 ? a[1] : (i == 2 ? a[2] : a[3]));
}

__device__ __forceinline__ uint32_t next_u32(Rng& r) {
  if (r.left == 0) {
    philox(r.c0, 0u, r.c2, r.c3, r.k0, r.k1, r.b);
    r.c0++;
    r.left = 4;
  }
  uint32_t u = pick4(r.b, 4 - r.left);
  r.left--;
  return u;
}

// The trace harness draws from an injected list.  Past its end the draws
// continue as the equidistributed sequence frac(0.5 + k (sqrt(5) - 1) / 2),
// k = 0, 1, ..., so that a rejection loop (stokes) still ends when a caller
// passes too few uniforms; the CPU restatement continues the same way.
__device__ __forceinline__ double inj_next(Rng& r) {
  if (r.pos < r.ninj) return r.inj[r.pos++];
  const double v = 0.5 + (double)(r.pos++ - r.ninj) * 0.6180339887498949;
  return v - floor(v);
}

template <class R> __device__ __forceinline__ R ran(Rng& r);
template <> __device__ __forceinline__ double ran<double>(Rng& r) {
  if (r.inj) return inj_next(r);
  return ((double)next_u32(r) + 0.5) * (1.0 / 4294967296.0);
}
template <> __device__ __forceinline__ float ran<float>(Rng& r) {
  if (r.inj) return (float)inj_next(r);
  return ((float)(next_u32(r) >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

// ---- packet state: the tts_mod/stokesvar_mod globals of one packet ------------
// Positions: FP64 in the FP64 form.  The mixed form carries each coordinate
// as an unevaluated FP32 pair hi + lo (about 44 significant bits), advanced
// with error-free FP32 transformations, so no FP64 instruction -- 64 cycles
// of latency each on this GPU -- sits on the per-event critical path.
struct Pos2 {
  float hi, lo;
};
template <class R> struct PosOf { using T = double; };
template <> struct PosOf<float> { using T = Pos2; };
__device__ __forceinline__ double dval(double v) { return v; }
__device__ __forceinline__ double dval(const Pos2& v) { return (double)v.hi + (double)v.lo; }
__device__ __forceinline__ void set_pos(double& d, double v) { d = v; }
__device__ __forceinline__ void set_pos(Pos2& d, double v) {
  d.hi = (float)v;
  d.lo = (float)(v - (double)d.hi);
}

// Lucy CDF rows of one cell and species slot (mixed form, lucy_freq_mixed)
struct LucyRow {
  int key;  // 4 * cell + slot; -1 = empty
  int pr;   // row pair: slot * (nT - 1) + j - 1
  float T0, f, P0, P1;
};

template <class R>
struct Pkt {
  typename PosOf<R>::T x, y, z;
  R ux, uy, uz;
  R cost, sint, cosp, sinp, phi;
  R sip, sqp, sup, svp;
  R nub;
  R cosb, sinb, lp;
  int ir, it, ip;
  int on_wall;
  int i_orig;
  R kapd[kSlots], albedo[kSlots], g[kSlots], pl[kSlots];
  float safe;  // mixed form: a step shorter than this from here stays in the cell (0 = unknown)
  LucyRow lrow;  // mixed form: cached Lucy CDF rows of the current cell
};

// Event counters (HC3D_CNT_*) of a thread and its last fault code.  The
// counters live in the block's shared memory, so they take no registers on
// the packet's chain of events; local_init() clears them, flush() adds them
// to the device counters once per block.  The peel-off walks count in
// registers instead (PeelCount): their crossings would make every lane hit
// the same shared counter.
struct Local {
  unsigned long long* sc;  // the block's 16 counters
  int fault;
  __device__ __forceinline__ void add(int k, unsigned long long v = 1ull) const { atomicAdd(sc + k, v); }
};

__device__ __forceinline__ void local_init(Local& L, unsigned long long* sc) {
  if (threadIdx.x < 16) sc[threadIdx.x] = 0ull;
  __syncthreads();
  L.sc = sc;
  L.fault = 0;
}

struct PeelCount {
  unsigned peels, cross, stuck;
};

// trace record (hc3d_trace_rec of hc3d.h)
struct TraceRec {
  int32_t kind, ir, it, ip, iface, pad;
  double tsum, x, y, z;
};
struct Tracer {
  TraceRec* recs;
  int max_rec;
  int n;
  __device__ __forceinline__ void add(int kind, int ir, int it, int ip, int iface, double tsum, double x, double y,
                                      double z) {
    if (recs && n < max_rec) {
      TraceRec& r = recs[n++];
      r.kind = kind; r.ir = ir; r.it = it; r.ip = ip; r.iface = iface; r.pad = 0;
      r.tsum = tsum; r.x = x; r.y = y; r.z = z;
    }
  }
};

// ---- closest_wall.f90:13-66 ----------------------------------------------------
template <class R>
struct Walls {
  R tn1, tp1, tp2;
  int in1, ip1, ip2;
  __device__ __forceinline__ void reset() {
    tn1 = -rhuge<R>(); tp1 = rhuge<R>(); tp2 = rhuge<R>();
    in1 = 0; ip1 = 0; ip2 = 0;
  }
  __device__ __forceinline__ void insert(R t, int i) {
    if (t < R(0)) {
      if (t > tn1) { tn1 = t; in1 = i; }
    } else {
      if (t < tp1) { tp2 = tp1; ip2 = ip1; tp1 = t; ip1 = i; }
      else if (t < tp2) { tp2 = t; ip2 = i; }
    }
  }
  __device__ __forceinline__ bool next(int on_wall, R& t, int& i) const {
    if (on_wall) {
      if (xabs(tn1) < xabs(tp1)) { t = tp1; i = ip1; }
      else { t = tp2; i = ip2; }
    } else {
      t = tp1; i = ip1;
    }
    return t != rhuge<R>();
  }
};

// radface.f90:44-62: both roots (-b +- sqrt(D))/2 of each sphere (FP64 form)
__device__ __forceinline__ void radface(Walls<double>& w, double ux, double uy, double uz, double x, double y,
                                        double z, double R2_1, double R2_2) {
  const double bb = 2.0 * (x * ux + y * uy + uz * z);
  const double rr = x * x + y * y + z * z;
  double cc = rr - R2_1;
  double descr = bb * bb - 4.0 * cc;
  if (descr > 0.0) {
    descr = sqrt(descr);
    w.insert((-bb + descr) * 0.5, 1);
    w.insert((-bb - descr) * 0.5, 1);
  }
  cc = rr - R2_2;
  descr = bb * bb - 4.0 * cc;
  if (descr > 0.0) {
    descr = sqrt(descr);
    w.insert((-bb + descr) * 0.5, 2);
    w.insert((-bb - descr) * 0.5, 2);
  }
}

// thetaface (module not shipped; restated): one cone wall on the nappe of its
// hemisphere; tan2 < 0 is the midplane plane z = 0; tan2 == 0 is a pole.
__device__ __forceinline__ void cone_roots(Walls<double>& w, double ux, double uy, double uz, double x, double y,
                                           double z, double tan2, double hemi, int id) {
  if (tan2 == 0.0) return;
  if (tan2 < 0.0) {
    if (uz != 0.0) w.insert(-z / uz, id);
    return;
  }
  const double a = ux * ux + uy * uy - tan2 * uz * uz;
  const double b = 2.0 * (x * ux + y * uy - tan2 * z * uz);
  const double cq = x * x + y * y - tan2 * z * z;
  if (a == 0.0) {
    if (b != 0.0) {
      const double t = -cq / b;
      if ((z + t * uz) * hemi > 0.0) w.insert(t, id);
    }
    return;
  }
  double descr = b * b - 4.0 * a * cq;
  if (descr > 0.0) {
    descr = sqrt(descr);
    const double t1 = (-b + descr) / (2.0 * a);
    const double t2 = (-b - descr) / (2.0 * a);
    if ((z + t1 * uz) * hemi > 0.0) w.insert(t1, id);
    if ((z + t2 * uz) * hemi > 0.0) w.insert(t2, id);
  }
}

// The wall a packet stands on after crossing wall iface of its old cell, as a
// wall id of the new cell (1<->2, 3<->4, 5<->6).
__device__ __forceinline__ int own_after(int iface) { return ((iface - 1) ^ 1) + 1; }

// The wall machinery of one step (peeloff_3d.f90:92-115), FP64 form.
// on_wall is the reference's on_wall flag (nonzero on a wall).
template <class R>
__device__ __forceinline__ bool next_wall(const DevModel& m, R ux, R uy, R uz, double x, double y, double z, int ir,
                                          int it, int ip, int on_wall, R& dt, int& iface) {
  static_assert(sizeof(R) == 8, "next_wall is the FP64 form");
  Walls<R> w;
  w.reset();
  radface(w, ux, uy, uz, x, y, z, __ldg(m.r2arr + ir - 1), __ldg(m.r2arr + ir));
  if (m.ntg > 2) {
    cone_roots(w, ux, uy, uz, x, y, z, __ldg(m.tan2d + it - 1), (double)__ldg(m.hemi + it - 1), 3);
    cone_roots(w, ux, uy, uz, x, y, z, __ldg(m.tan2d + it), (double)__ldg(m.hemi + it), 4);
    if (m.npg > 2) {
      // phiface.f90:48-56 with C = D = 0
      const double A1 = __ldg(m.aarrd + ip - 1), B1 = __ldg(m.barrd + ip - 1);
      const double A2 = __ldg(m.aarrd + ip), B2 = __ldg(m.barrd + ip);
      const double d1 = A1 * ux + B1 * uy;
      if (d1 != 0.0) w.insert(-(A1 * x + B1 * y) / d1, 5);
      const double d2 = A2 * ux + B2 * uy;
      if (d2 != 0.0) w.insert(-(A2 * x + B2 * y) / d2, 6);
    }
  }
  return w.next(on_wall != 0, dt, iface);
}

// A straight ray of the mixed form, parametrised by its path length S from
// the start point.  S is an unevaluated FP32 pair (hi + lo) advanced by an
// error-free FP32 sum, so the FP32 position x0 + S u carries no error that
// grows along the ray.  The FP64 radial terms |x|^2 and x.u are formed from
// the FP64 start point only when a sphere root needs them (first use).
struct PathLen {
  float hi, lo;
};

__device__ __forceinline__ void path_add(PathLen& s, float d) {
  const float t = s.hi + d;
  const float bp = t - s.hi;
  s.lo += (s.hi - (t - bp)) + (d - bp);
  s.hi = t;
}

__device__ __forceinline__ double path_f64(const PathLen& s) { return (double)s.hi + (double)s.lo; }

struct Ray {
  float x0, y0, z0, ux, uy, uz;  // FP32 start point and direction
  float urho2, uz2;              // ux^2 + uy^2, uz^2
  Pos2 xs, ys, zs;               // the start point as pairs
  double rr0, hb0, u2;           // FP64 |x0|^2, x0.u, |u|^2 once `dbl` is set
  bool dbl;
};

__device__ __forceinline__ void ray_init(Ray& r, const Pos2& x, const Pos2& y, const Pos2& z, float ux, float uy,
                                         float uz) {
  r.x0 = x.hi; r.y0 = y.hi; r.z0 = z.hi;
  r.ux = ux; r.uy = uy; r.uz = uz;
  r.urho2 = ux * ux + uy * uy;
  r.uz2 = uz * uz;
  r.xs = x; r.ys = y; r.zs = z;
  r.dbl = false;
}

__device__ __forceinline__ void ray_f64(Ray& r) {
  if (r.dbl) return;
  const double uxd = r.ux, uyd = r.uy, uzd = r.uz;
  const double x = dval(r.xs), y = dval(r.ys), z = dval(r.zs);
  r.rr0 = x * x + y * y + z * z;
  r.hb0 = x * uxd + y * uyd + z * uzd;
  r.u2 = uxd * uxd + uyd * uyd + uzd * uzd;
  r.dbl = true;
}

// FP64 point of the ray at path length S
__device__ __forceinline__ void ray_at(const Ray& r, const PathLen& S, double& x, double& y, double& z) {
  const double s = path_f64(S);
  x = fma(s, (double)r.ux, dval(r.xs));
  y = fma(s, (double)r.uy, dval(r.ys));
  z = fma(s, (double)r.uz, dval(r.zs));
}

// x + S u as a pair: x a pair, S a pair, u FP32 (error-free product and sum)
__device__ __forceinline__ Pos2 pos_step(const Pos2& x, const PathLen& S, float u) {
  const float pr = S.hi * u;
  const float pe = fmaf(S.hi, u, -pr) + S.lo * u;
  const float sm = x.hi + pr;
  const float bp = sm - x.hi;
  const float e = ((x.hi - (sm - bp)) + (pr - bp)) + (x.lo + pe);
  const float hi = sm + e;
  return Pos2{hi, e - (hi - sm)};
}

// the point of the ray at path length S, as pairs
__device__ __forceinline__ void ray_pos(const Ray& r, const PathLen& S, Pos2& x, Pos2& y, Pos2& z) {
  x = pos_step(r.xs, S, r.ux);
  y = pos_step(r.ys, S, r.uy);
  z = pos_step(r.zs, S, r.uz);
}

// A sphere root from FP32 |x|^2 - R^2 is exact enough unless the point lies
// within 2^-12 R^2 of the sphere (|x|^2 - R^2 cancels) or the ray grazes it
// (hb^2 - c within 2^-10 R^2 of zero); those cases are redone in FP64.  The
// inner sphere counts only for a ray moving inwards, the one case whose root
// is used.
constexpr float kNearSphere = 1.0f / 4096.0f;
constexpr float kGrazeSphere = 1.0f / 1024.0f;

// square root of a positive FP32 value by the reciprocal square root (the
// wall searches take it of discriminants already tested > 0)
__device__ __forceinline__ float fsqrt_pos(float x) { return x * rsqrtf(x); }

// The mixed-form wall search on a Ray at path length S.  The reference keeps
// the roots of every wall in closest_wall and skips the root of the wall it
// stands on by the on_wall rule; here the walls in `own` (bit id) contribute
// only their far root, and the next wall is the smallest non-negative root
// of the rest, a minimum over at most six candidates.  FP32, except the
// near-sphere and grazing sphere roots (FP64).
// kCache: keep the FP64 terms of the start point in the Ray once formed (the
// transport walk, where one event's steps repeat the refinement); the
// peel-off walk forms them afresh each time and keeps its registers.
template <bool kCache>
__device__ __forceinline__ bool next_wall_ray(const DevModel& m, Ray& r, const PathLen& S, int ir, int it, int ip,
                                              int own, float& dt, int& iface) {
  float best = 3.402823466e38f;
  int bi = 0;
  auto cand = [&](float t, int id) {
    if (t >= 0.f && t < best) {
      best = t;
      bi = id;
    }
  };
  const float ux = r.ux, uy = r.uy, uz = r.uz;
  const float xr = fmaf(S.hi, ux, fmaf(S.lo, ux, r.x0));
  const float yr = fmaf(S.hi, uy, fmaf(S.lo, uy, r.y0));
  const float zr = fmaf(S.hi, uz, fmaf(S.lo, uz, r.z0));
  // terms shared by the spheres and the cones
  const float pxy = xr * ux + yr * uy, pz = zr * uz;
  const float rho2 = xr * xr + yr * yr, z2 = zr * zr;
  // spheres: t^2 + 2 hb t + c = 0 with hb = x.u, c = |x|^2 - R^2, disc = hb^2 - c
  const bool in_own = (own & 2) != 0, out_own = (own & 4) != 0;
  float hb = pxy + pz;
  const float rr = rho2 + z2;
  const float2 r2io = __ldg(m.r2pair + ir - 1);
  const float r2i = r2io.x, r2o = r2io.y;
  float ci = rr - r2i, co = rr - r2o;
  float di = hb * hb - ci, dq = hb * hb - co;
  const bool fix = (!in_own && hb < 0.f && (fabsf(ci) < kNearSphere * r2i || fabsf(di) < kGrazeSphere * r2i)) ||
                   (!out_own && (fabsf(co) < kNearSphere * r2o || fabsf(dq) < kGrazeSphere * r2o));
  if (fix) {
    double rr0, hb0, u2;
    if constexpr (kCache) {
      ray_f64(r);
      rr0 = r.rr0; hb0 = r.hb0; u2 = r.u2;
    } else {
      const double uxd = ux, uyd = uy, uzd = uz;
      const double x = dval(r.xs), y = dval(r.ys), z = dval(r.zs);
      rr0 = x * x + y * y + z * z;
      hb0 = x * uxd + y * uyd + z * uzd;
      u2 = uxd * uxd + uyd * uyd + uzd * uzd;
    }
    const double s = path_f64(S);
    const double hbd = fma(s, u2, hb0);
    const double rrd = fma(s, fma(s, u2, hb0 + hb0), rr0);
    const double cid = rrd - __ldg(m.r2arr + ir - 1), cod = rrd - __ldg(m.r2arr + ir);
    hb = (float)hbd;
    ci = (float)cid; co = (float)cod;
    di = (float)(hbd * hbd - cid); dq = (float)(hbd * hbd - cod);
  }
  if (in_own) {
    if (hb < 0.f) cand(-2.f * hb, 1);
  } else if (hb < 0.f && di > 0.f) {  // inner sphere: reached only moving inwards
    cand(__fdividef(fmaxf(ci, 0.f), fsqrt_pos(di) - hb), 1);
  }
  if (out_own) {
    if (hb < 0.f) cand(-2.f * hb, 2);
  } else if (dq > 0.f) {  // outer sphere: the exit root
    const float sq = fsqrt_pos(dq);
    cand(hb > 0.f ? __fdividef(fmaxf(-co, 0.f), hb + sq) : sq - hb, 2);
  }
  if (m.ntg > 2) {
    // cones x^2 + y^2 = tan2 z^2: a t^2 + b t + cq = 0
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int id = 3 + k;
      const float2 cw = __ldg(m.conef + it - 1 + k);
      const float tan2 = cw.x, hemi = cw.y;
      if (tan2 == 0.f) continue;
      const bool mine = (own >> id) & 1;
      if (tan2 < 0.f) {
        if (!mine && uz != 0.f) cand(__fdividef(-zr, uz), id);
        continue;
      }
      const float a = fmaf(-tan2, r.uz2, r.urho2);
      const float b = 2.f * fmaf(-tan2, pz, pxy);
      if (mine) {
        if (a != 0.f) {
          const float t = __fdividef(-b, a);
          if ((zr + t * uz) * hemi > 0.f) cand(t, id);
        }
        continue;
      }
      const float cq = fmaf(-tan2, z2, rho2);
      if (a == 0.f) {
        if (b != 0.f) {
          const float t = __fdividef(-cq, b);
          if ((zr + t * uz) * hemi > 0.f) cand(t, id);
        }
        continue;
      }
      const float disc = b * b - 4.f * a * cq;
      if (disc > 0.f) {
        const float sq = fsqrt_pos(disc), inv = __fdividef(0.5f, a);
        const float t1 = (-b + sq) * inv, t2 = (-b - sq) * inv;
        if ((zr + t1 * uz) * hemi > 0.f) cand(t1, id);
        if ((zr + t2 * uz) * hemi > 0.f) cand(t2, id);
      }
    }
    if (m.npg > 2) {
      // The azimuth of a straight line changes monotonically (by less than
      // pi), so only the plane on the side it turns towards can be met:
      // phi(ip) (id 6) when (x cross u)_z > 0, phi(ip-1) (id 5) otherwise.
      const int k = xr * uy - yr * ux > 0.f ? 1 : 0;
      const int id = 5 + k;
      if (!((own >> id) & 1)) {
        const float2 ab = __ldg(m.planef + ip - 1 + k);
        const float A = ab.x, B = ab.y;
        const float d = A * ux + B * uy;
        if (d != 0.f) cand(__fdividef(-(A * xr + B * yr), d), id);
      }
    }
  }
  dt = best;
  iface = bi;
  return bi != 0;
}

// wall -> index step, peeloff_3d.f90:120-139
__device__ __forceinline__ void step_index(int npg, int iface, int& ir, int& it, int& ip) {
  ir += (int)(iface == 2) - (int)(iface == 1);
  it += (int)(iface == 4) - (int)(iface == 3);
  ip += (int)(iface == 6) - (int)(iface == 5);
  ip = ip == 0 ? npg - 1 : (ip == npg ? 1 : ip);
}

// compact cell index; hc3d_load_grid keeps the cell count below 2^31
__device__ __forceinline__ int64_t cidx(const DevModel& m, int ir, int it, int ip) {
  return (int64_t)((ir - 1) + (m.nrg - 1) * ((it - 1) + (m.ntg - 1) * (ip - 1)));
}

template <class R> struct Rho { R v[kSlots]; };
template <class R> __device__ __forceinline__ Rho<R> load_rho(const DevModel& m, int64_t c);
template <> __device__ __forceinline__ Rho<float> load_rho<float>(const DevModel& m, int64_t c) {
  float4 q = __ldg(m.rho4f + c);
  Rho<float> r;
  r.v[0] = q.x; r.v[1] = q.y; r.v[2] = q.z; r.v[3] = q.w;
  return r;
}
template <> __device__ __forceinline__ Rho<double> load_rho<double>(const DevModel& m, int64_t c) {
  const double2* p = reinterpret_cast<const double2*>(m.rho4d + 4 * c);
  double2 a = __ldg(p), b = __ldg(p + 1);
  Rho<double> r;
  r.v[0] = a.x; r.v[1] = a.y; r.v[2] = b.x; r.v[3] = b.y;
  return r;
}

__device__ __forceinline__ unsigned long long fx(double v, double scale) {
  return (unsigned long long)llround(v * scale);
}

// ---- dust tables: unique per-species tables, staged in shared memory ---------------
// R-typed: the FP64 form reads the FP64 tables, the mixed form their FP32 copies.
template <class R>
struct DustView {
  const R* nud[kSlots];
  const R* kap[kSlots];
  const R* alb[kSlots];
  const R* g[kSlots];
  const R* pl[kSlots];
};

template <class R> __device__ __forceinline__ const R* tab(const double* d, const float* f);
template <> __device__ __forceinline__ const double* tab<double>(const double* d, const float*) { return d; }
template <> __device__ __forceinline__ const float* tab<float>(const double*, const float* f) { return f; }

// Copy the unique dust tables into the block's dynamic shared memory (when
// the host sized it, DevModel::dust_smem > 0) and point the view at them;
// otherwise read them from global memory.  Called by every thread of the
// block before any divergence.
template <class R>
__device__ __forceinline__ void dust_view(const DevModel& m, R* smem, DustView<R>& v) {
  const R* nud = tab<R>(m.nudust, m.nudustf);
  const R* kap = tab<R>(m.kappad, m.kappadf);
  const R* alb = tab<R>(m.adust, m.adustf);
  const R* gg = tab<R>(m.gdust, m.gdustf);
  const R* pl = tab<R>(m.pldust, m.pldustf);
  size_t off = 0;
#pragma unroll
  for (int u = 0; u < kSlots; ++u) {  // unrolled: the view's pointers stay in registers
    v.nud[u] = v.kap[u] = v.alb[u] = v.g[u] = v.pl[u] = nullptr;
    if (u >= m.ntab) continue;
    const int nl = m.tab_nl[u];
    const size_t go = (size_t)u * m.nlammax;
    if (m.dust_smem > 0) {
      R* base = smem + off;
      for (int i = threadIdx.x; i < nl; i += blockDim.x) {
        base[i] = nud[go + i];
        base[nl + i] = kap[go + i];
        base[2 * nl + i] = alb[go + i];
        base[3 * nl + i] = gg[go + i];
        base[4 * nl + i] = pl[go + i];
      }
      v.nud[u] = base; v.kap[u] = base + nl; v.alb[u] = base + 2 * nl; v.g[u] = base + 3 * nl; v.pl[u] = base + 4 * nl;
      off += 5 * (size_t)nl;
    } else {
      v.nud[u] = nud + go; v.kap[u] = kap + go; v.alb[u] = alb + go; v.g[u] = gg + go; v.pl[u] = pl + go;
    }
  }
  if (m.dust_smem > 0) __syncthreads();
}

// ---- opacset, dust.f90:9-80 ---------------------------------------------------------
// Computed once per unique table; species slots sharing a dust file share
// the result (only kappa_V differs), which is what the per-slot loop of the
// reference computes for them.
template <class R>
__device__ __forceinline__ void opacset(const DevModel& m, const DustView<R>& v, Pkt<R>& p, R nu, const RunArgs& a) {
  if constexpr (sizeof(R) == 4) {
    // mixed form: the same bracket from the ln(nu) guide of each table, then
    // a short bisection inside it; values kept in registers
    const float lnu = logf(nu);
    float gt[kSlots], plt[kSlots], kt[kSlots], at[kSlots];
#pragma unroll
    for (int u = 0; u < kSlots; ++u) {
      gt[u] = plt[u] = kt[u] = at[u] = 0.f;
      if (u >= m.ntab) continue;
      const int nl = m.tab_nl[u];
      const float* nud = v.nud[u];
      int i0 = 1, i1 = nl;
      if (nu >= nud[0]) {
        i0 = i1 = 1;
      } else if (nu <= nud[nl - 1]) {
        i0 = i1 = nl;
      } else {
        const int b = min(max((int)((lnu - m.dlnlo[u]) * m.dginv[u]), 0), kDustGuide - 1);
        const short2 gb = __ldg(m.dguide + u * kDustGuide + b);
        if (nud[gb.x - 1] >= nu && nu > nud[gb.y]) { i0 = gb.x; i1 = gb.y + 1; }
        while (i1 - i0 > 1) {
          const int i = (i1 + i0) / 2;
          if (nu <= nud[i - 1]) i0 = i; else i1 = i;
        }
      }
      if (i0 == i1) {
        gt[u] = v.g[u][i0 - 1]; plt[u] = v.pl[u][i0 - 1]; kt[u] = v.kap[u][i0 - 1]; at[u] = v.alb[u][i0 - 1];
      } else {
        const float n1 = nud[i1 - 1], n0 = nud[i0 - 1];
        const float f = (nu - n1) / (n0 - n1), fm1 = 1.f - f;
        gt[u] = fm1 * v.g[u][i1 - 1] + f * v.g[u][i0 - 1];
        plt[u] = fm1 * v.pl[u][i1 - 1] + f * v.pl[u][i0 - 1];
        kt[u] = fm1 * v.kap[u][i1 - 1] + f * v.kap[u][i0 - 1];
        at[u] = fm1 * v.alb[u][i1 - 1] + f * v.alb[u][i0 - 1];
      }
    }
#pragma unroll
    for (int id = 0; id < kSlots; ++id) {
      const int u = m.table_of[id];
      float g_ = gt[0], pl_ = plt[0], k_ = kt[0], a_ = at[0];
#pragma unroll
      for (int q = 1; q < kSlots; ++q)
        if (u == q) { g_ = gt[q]; pl_ = plt[q]; k_ = kt[q]; a_ = at[q]; }
      p.g[id] = g_; p.pl[id] = pl_; p.albedo[id] = a_;
      p.kapd[id] = k_ * a.kapfac[id];
    }
    return;
  }
  R gt[kSlots], plt[kSlots], kt[kSlots], at[kSlots];
  for (int u = 0; u < m.ntab; ++u) {
    const int nl = m.tab_nl[u];
    const R* nud = v.nud[u];
    if (nu >= nud[0]) {
      gt[u] = v.g[u][0]; plt[u] = v.pl[u][0]; kt[u] = v.kap[u][0]; at[u] = v.alb[u][0];
    } else if (nu <= nud[nl - 1]) {
      gt[u] = v.g[u][nl - 1]; plt[u] = v.pl[u][nl - 1]; kt[u] = v.kap[u][nl - 1]; at[u] = v.alb[u][nl - 1];
    } else {
      int i0 = 1, i1 = nl;
      while (i1 - i0 > 1) {
        const int i = (i1 + i0) / 2;
        if (nu <= nud[i - 1]) i0 = i; else i1 = i;
      }
      const R n1 = nud[i1 - 1], n0 = nud[i0 - 1];
      const R f = (nu - n1) / (n0 - n1), fm1 = R(1) - f;
      gt[u] = fm1 * v.g[u][i1 - 1] + f * v.g[u][i0 - 1];
      plt[u] = fm1 * v.pl[u][i1 - 1] + f * v.pl[u][i0 - 1];
      kt[u] = fm1 * v.kap[u][i1 - 1] + f * v.kap[u][i0 - 1];
      at[u] = fm1 * v.alb[u][i1 - 1] + f * v.alb[u][i0 - 1];
    }
  }
#pragma unroll
  for (int id = 0; id < kSlots; ++id) {
    const int u = m.table_of[id];
    p.g[id] = gt[u]; p.pl[id] = plt[u]; p.albedo[id] = at[u];
    p.kapd[id] = (R)((double)kt[u] * a.rstar_cm * m.kappav[id]);
  }
}

// ---- tauint (restated; module not shipped) -------------------------------------
enum { TI_INTERACT = 0, TI_ESCAPE = 1, TI_STAR = 2, TI_FAULT = 3 };
// fault codes of the fault log: walk left the index range, found no wall,
// exceeded the crossing cap; species selection found no opacity
enum { F_RANGE = 1, F_NOWALL = 2, F_CAP = 3, F_SELECT = 4 };

// Re-derive the cell of a position from the walls: the consistency check
// testgrid (called at peeloff_3d.f90:90; the module is not shipped).  The
// FP32 walk uses it when it finds no wall or keeps crossing walls at zero
// distance.  Returns 0 inside the grid, 1 beyond rmax, 2 inside the star.
static __device__ __noinline__ int relocate(const DevModel& m, double x, double y, double z, int& ir, int& it,
                                            int& ip) {
  const double rr = x * x + y * y + z * z;
  if (rr >= __ldg(m.r2arr + m.nrg - 1)) return 1;
  if (rr <= __ldg(m.r2arr)) return 2;
  auto loc = [](const double* xx, int n, double v) {
    int jl = 0, ju = n + 1;
    while (ju - jl > 1) {
      const int jm = (ju + jl) / 2;
      if (v > __ldg(xx + jm - 1)) jl = jm; else ju = jm;
    }
    return jl;
  };
  ir = min(max(loc(m.r2arr, m.nrg, rr), 1), m.nrg - 1);
  const double th = acos(fmin(1.0, fmax(-1.0, z / sqrt(rr))));
  it = min(max(loc(m.thetarr, m.ntg, th), 1), m.ntg - 1);
  double ph = atan2(y, x);
  if (ph < 0.0) ph += kR2p;
  ip = min(max(loc(m.phiarr, m.npg, ph), 1), m.npg - 1);
  return 0;
}

// FP32 walk: a crossing shorter than this (relative to |x|) is at zero distance
__device__ __forceinline__ bool tiny_step(const DevModel& m, float dt, int ir) {
  return dt <= 1.0e-6f * __ldg(m.rarrf + min(ir, m.nrg - 1));
}

// Round a float to the nearest int64 (halves away from zero) with integer
// operations only: the fixed-point conversion of the mixed form.  |v| must be
// below 2^63; the tally scales keep it far below.
__device__ __forceinline__ long long f2ll(float v) {
  const unsigned b = __float_as_uint(v);
  const int ex = (int)((b >> 23) & 0xffu);
  const unsigned mant = (b & 0x7fffffu) | 0x800000u;
  const int e = ex - 150;  // |v| = mant * 2^e
  long long r;
  if (ex == 0 || e < -24) r = 0;
  else if (e >= 0) r = e > 39 ? 0x7fffffffffffffffll : (long long)mant << e;
  else r = (long long)((mant + (1u << (-e - 1))) >> (-e));
  return (b >> 31) ? -r : r;
}

// scale is a power of two, so v * scale is exact
__device__ __forceinline__ unsigned long long fxf(float v, float scale) {
  return (unsigned long long)f2ll(v * scale);
}

// The small grains' absorption path of a step ds in cell c (models with
// small-grain slots): ds kappa(nu)/kappa_V (1 - albedo(nu)) of slot sg_slot,
// over the cell's outer radius like jmean.  int_mean turns it into the mean
// intensity in units of the ISRF absorbed by the same grains (the tally of
// the reference's tauint is restated; its source is absent).
template <class R>
__device__ __forceinline__ void tally_jsg(const DevModel& m, const DevTallies& t, const Pkt<R>& p, int64_t c, R ds,
                                          R rout) {
  if (!m.sg_on) return;
  if constexpr (sizeof(R) == 4) {
    const float w = pick4(p.kapd, m.sg_slot) * (1.f - pick4(p.albedo, m.sg_slot)) * m.sg_jfac;
    atomicAdd(t.jsg + c, fxf(ds * w / rout, (float)t.path_scale));
  } else {
    const double w = pick4(p.kapd, m.sg_slot) * (1.0 - pick4(p.albedo, m.sg_slot)) * m.sg_jfacd;
    atomicAdd(t.jsg + c, fx((double)ds * w / (double)rout, t.path_scale));
  }
}

// A lower bound on the distance from a point inside cell (ir, it, ip) to
// every wall of the cell: the spheres |r - R|, the cones r|sin(theta - theta_w)|
// = |rho cos(theta_w) - z sin(theta_w)| (rho the cylindrical radius; the
// midplane gives |z|, a pole is no wall) and the planes |A x + B y|, less a
// margin for FP32 rounding of the point and of the walls.
__device__ __forceinline__ float safe_dist(const DevModel& m, float x, float y, float z, int ir, int it, int ip) {
  const float rc2 = x * x + y * y;
  const float r = sqrtf(rc2 + z * z), rc = sqrtf(rc2);
  float d = fminf(r - __ldg(m.rarrf + ir - 1), __ldg(m.rarrf + ir) - r);
  if (m.ntg > 2) {
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      if (__ldg(m.tan2f + it - 1 + k) == 0.f) continue;
      const float2 cs = __ldg(m.thcs + it - 1 + k);
      d = fminf(d, fabsf(rc * cs.x - z * cs.y));
    }
    if (m.npg > 2) {
#pragma unroll
      for (int k = 0; k < 2; ++k)
        d = fminf(d, fabsf(__ldg(m.aarrf + ip - 1 + k) * x + __ldg(m.barrf + ip - 1 + k) * y));
    }
  }
  return d - 1.0e-6f * r;
}

// Mixed form of tauint: the step of one event is a Ray from the event point;
// the walk, the tau integral and the Lucy tallies are FP32, the FP64 point
// where the walk stops is formed once, at the end.
static __device__ __forceinline__ int tauint_mixed(const DevModel& m, const DevTallies& t, Pkt<float>& p, float tau, Local& L,
                                   Tracer& tr) {
  float tsum = 0.f;
  const int cap = 4 * (m.nrg + m.ntg + m.npg) + 64;
  int nreloc = 0, ntiny = 0;
  Ray ray;
  ray_init(ray, p.x, p.y, p.z, p.ux, p.uy, p.uz);
  PathLen S{0.f, 0.f};
  const float ps = (float)t.path_scale;
  if (p.on_wall == 0 && p.ir >= 1 && p.ir <= m.nrg - 1 && p.it >= 1 && p.it <= m.ntg - 1) {
    // From a point inside the cell, a step shorter than the safe distance
    // ends in the cell: the interaction the walk would find, without the
    // wall search.  The safe distance holds for a ball around the point
    // where it was formed; each such step uses up its length.
    const int64_t c = cidx(m, p.ir, p.it, p.ip);
    const Rho<float> rho = load_rho<float>(m, c);
    float opac = 0.f;
#pragma unroll
    for (int s = 0; s < kSlots; ++s) opac += p.kapd[s] * rho.v[s];
    const float ds = tau / opac;
    if (opac > 0.f && !(ds < p.safe)) p.safe = safe_dist(m, p.x.hi, p.y.hi, p.z.hi, p.ir, p.it, p.ip);
    if (opac > 0.f && ds < p.safe) {
      p.safe -= ds;
      L.add(HC3D_CNT_CROSS_PROP);
#pragma unroll
      for (int s = 0; s < kSlots; ++s)
        if (rho.v[s] > 0.f)
          atomicAdd(t.dtauabs + (int64_t)s * m.ncell + c, fxf(p.kapd[s] * (1.f - p.albedo[s]) * rho.v[s] * ds, ps));
      atomicAdd(t.jmean + c, fxf(ds / __ldg(m.rarrf + p.ir), ps));
      tally_jsg<float>(m, t, p, c, ds, __ldg(m.rarrf + p.ir));
      path_add(S, ds);
      ray_pos(ray, S, p.x, p.y, p.z);
      tr.add(2, p.ir, p.it, p.ip, 0, (double)tau, dval(p.x), dval(p.y), dval(p.z));
      return TI_INTERACT;
    }
  }
  p.safe = 0.f;
  auto at = [&]() { ray_pos(ray, S, p.x, p.y, p.z); };
  auto reloc = [&]() {
    double x, y, z;
    ray_at(ray, S, x, y, z);
    int jr = p.ir, jt = p.it, jp = p.ip;
    const int where = relocate(m, x, y, z, jr, jt, jp);
    p.ir = jr; p.it = jt; p.ip = jp;
    return where;
  };
  for (int n = 0;; ++n) {
    if (n > cap || p.it < 1 || p.it > m.ntg - 1 || p.ir < 1 || p.ir > m.nrg - 1) {
      L.fault = n > cap ? F_CAP : F_RANGE;
      at();
      return TI_FAULT;
    }
    // the cell's density, loaded before the wall search (latency overlap)
    const int64_t c = cidx(m, p.ir, p.it, p.ip);
    const Rho<float> rho = load_rho<float>(m, c);
    float dt;
    int iface;
    if (!next_wall_ray<true>(m, ray, S, p.ir, p.it, p.ip, p.on_wall, dt, iface)) {
      at();
      if (nreloc < 4) {
        ++nreloc;
        const int where = reloc();
        if (where == 1) { p.ir = m.nrg; return TI_ESCAPE; }
        if (where == 2) { p.ir = 0; return TI_STAR; }
        p.on_wall = 0;
        continue;
      }
      L.fault = F_NOWALL;
      return TI_FAULT;
    }
    float opac = 0.f;
#pragma unroll
    for (int s = 0; s < kSlots; ++s) opac += p.kapd[s] * rho.v[s];
    const float dtau = opac * dt;
    const float rout = __ldg(m.rarrf + p.ir);
    L.add(HC3D_CNT_CROSS_PROP);
    const bool stop = tsum + dtau > tau;
    const float ds = stop ? (tau - tsum) / opac : dt;
#pragma unroll
    for (int s = 0; s < kSlots; ++s)
      if (rho.v[s] > 0.f)
        atomicAdd(t.dtauabs + (int64_t)s * m.ncell + c, fxf(p.kapd[s] * (1.f - p.albedo[s]) * rho.v[s] * ds, ps));
    atomicAdd(t.jmean + c, fxf(ds / rout, ps));
    tally_jsg<float>(m, t, p, c, ds, rout);
    if (stop) {
      path_add(S, ds);
      at();
      p.on_wall = 0;
      tr.add(2, p.ir, p.it, p.ip, 0, (double)tau, dval(p.x), dval(p.y), dval(p.z));
      return TI_INTERACT;
    }
    tsum += dtau;
    step_index(m.npg, iface, p.ir, p.it, p.ip);
    path_add(S, dt);
    p.on_wall = 1 << own_after(iface);
    if (tr.recs) {
      at();
      tr.add(1, p.ir, p.it, p.ip, iface, (double)tsum, dval(p.x), dval(p.y), dval(p.z));
    }
    if (p.ir == m.nrg) { at(); return TI_ESCAPE; }
    if (p.ir == 0) { at(); return TI_STAR; }
    if (!tiny_step(m, dt, p.ir)) {
      ntiny = 0;
    } else if (++ntiny > 6 && nreloc < 4) {
      ++nreloc;
      ntiny = 0;
      at();
      const int where = reloc();
      if (where == 1) { p.ir = m.nrg; return TI_ESCAPE; }
      if (where == 2) { p.ir = 0; return TI_STAR; }
      p.on_wall = 0;
    }
  }
}

// tauint in either form: the FP64 form walks with the reference's wall
// machinery (closest_wall rule), the mixed form with tauint_mixed.
template <class R>
__device__ __forceinline__ int tauint(const DevModel& m, const DevTallies& t, Pkt<R>& p, R tau, Local& L, Tracer& tr) {
  if constexpr (sizeof(R) == 4) {
    return tauint_mixed(m, t, p, tau, L, tr);
  } else {
    R tsum = R(0);
    const int cap = 4 * (m.nrg + m.ntg + m.npg) + 64;
    const double uxd = (double)p.ux, uyd = (double)p.uy, uzd = (double)p.uz;
    for (int n = 0;; ++n) {
      if (n > cap || p.it < 1 || p.it > m.ntg - 1 || p.ir < 1 || p.ir > m.nrg - 1) {
        L.fault = n > cap ? F_CAP : F_RANGE;
        return TI_FAULT;
      }
      R dt;
      int iface;
      if (!next_wall<R>(m, p.ux, p.uy, p.uz, p.x, p.y, p.z, p.ir, p.it, p.ip, p.on_wall, dt, iface)) {
        L.fault = F_NOWALL;
        return TI_FAULT;
      }
      const int64_t c = cidx(m, p.ir, p.it, p.ip);
      const Rho<R> rho = load_rho<R>(m, c);
      R opac = R(0);
#pragma unroll
      for (int s = 0; s < kSlots; ++s) opac += p.kapd[s] * rho.v[s];
      const R dtau = opac * dt;
      const double rout = __ldg(m.rarr + p.ir);
      L.add(HC3D_CNT_CROSS_PROP);
      if (tsum + dtau > tau) {
        const R ds = (tau - tsum) / opac;
        p.x += (double)ds * uxd;
        p.y += (double)ds * uyd;
        p.z += (double)ds * uzd;
        p.on_wall = 0;
#pragma unroll
        for (int s = 0; s < kSlots; ++s)
          if (rho.v[s] > R(0)) {
            const R v = p.kapd[s] * (R(1) - p.albedo[s]) * rho.v[s] * ds;
            atomicAdd(t.dtauabs + (int64_t)s * m.ncell + c, fx((double)v, t.path_scale));
          }
        atomicAdd(t.jmean + c, fx((double)ds / rout, t.path_scale));
        tally_jsg<R>(m, t, p, c, ds, (R)rout);
        tr.add(2, p.ir, p.it, p.ip, 0, (double)tau, p.x, p.y, p.z);
        return TI_INTERACT;
      }
#pragma unroll
      for (int s = 0; s < kSlots; ++s)
        if (rho.v[s] > R(0)) {
          const R v = p.kapd[s] * (R(1) - p.albedo[s]) * rho.v[s] * dt;
          atomicAdd(t.dtauabs + (int64_t)s * m.ncell + c, fx((double)v, t.path_scale));
        }
      atomicAdd(t.jmean + c, fx((double)dt / rout, t.path_scale));
      tally_jsg<R>(m, t, p, c, dt, (R)rout);
      tsum += dtau;
      step_index(m.npg, iface, p.ir, p.it, p.ip);
      p.x += (double)dt * uxd;
      p.y += (double)dt * uyd;
      p.z += (double)dt * uzd;
      p.on_wall = 1 << own_after(iface);
      tr.add(1, p.ir, p.it, p.ip, iface, (double)tsum, p.x, p.y, p.z);
      if (p.ir == m.nrg) return TI_ESCAPE;
      if (p.ir == 0) return TI_STAR;
    }
  }
}

// ---- select_dust.f90:16-42 ---------------------------------------------------
template <class R>
__device__ __forceinline__ int select_dust(const DevModel& m, const Pkt<R>& p, Rng& rng) {
  const R xran = ran<R>(rng);
  const Rho<R> rho = load_rho<R>(m, cidx(m, p.ir, p.it, p.ip));
  R opac = R(0), frac = R(0);
#pragma unroll
  for (int s = 0; s < kSlots; ++s) opac += p.kapd[s] * rho.v[s];
  if (opac == R(0)) return -1;
  int last = -1;
  const R inv = R(1) / opac;  // mixed form: one division
#pragma unroll
  for (int s = 0; s < kSlots; ++s) {
    if constexpr (sizeof(R) == 4) frac += p.kapd[s] * rho.v[s] * inv;
    else frac += p.kapd[s] * rho.v[s] / opac;
    if (p.kapd[s] * rho.v[s] > R(0)) last = s;
    if (xran <= frac + (R)(double)1.e-10f) return s;
  }
  // FP32 fractions can sum to just below 1; the draw then belongs to the
  // last species with opacity (the FP64 form keeps the reference's stop)
  return sizeof(R) == 4 ? last : -1;
}

// ---- dustmat.f90:40-65 -----------------------------------------------------------
template <class R>
__device__ __forceinline__ void dustmat(R g, R pl, R cost, R cost2, R& p1, R& p2, R& p3) {
  const R g2 = g * g;
  const R temp = (g2 + R(1)) - (R(2) * g) * cost;
  p1 = R(1.5) * (R(1) - g2) / (R(2) + g2) * (R(1) + cost2) / (temp * xsqrt(temp));
  p2 = -pl * p1 * (R(1) - cost2) / (R(1) + cost2);
  p3 = p1 * R(2) * cost / (R(1) + cost2);
}

template <class R>
__device__ __forceinline__ R peak_of(R g) {
  const R g2 = g * g;
  R temp;
  if (g > R(0)) temp = (g2 + R(1)) - R(2) * g;
  else temp = (g2 + R(1)) + R(2) * g;
  const R peak = R(1.5) * (R(1) - g2) / (R(2) + g2) * R(2) / temp / xsqrt(temp);
  return peak * R(1.01);
}

// Mueller rotation of a Stokes vector (the a21..a44 blocks of stokes.f90 and
// stokespeel.f90); s2x/c2x: double angle of i1 (or i3), sin2i2/cos2i2 of i2.
template <class R>
__device__ __forceinline__ void mueller(bool upper, R p1, R p2, R p3, R s2x, R c2x, R sini2, R cosi2, R& si, R& sq,
                                        R& su, R& sv) {
  const R sin2i2 = R(2) * sini2 * cosi2, cos2i2 = R(2) * cosi2 * cosi2 - R(1);
  const R sin2 = sin2i2 * s2x, cos2 = cos2i2 * c2x;
  const R sin2cos1 = sin2i2 * c2x, cos2sin1 = cos2i2 * s2x;
  R a11, a12, a13, a21, a22, a23, a31, a32, a33, a44;
  if (upper) {
    a11 = p1; a12 = p2 * c2x; a13 = p2 * s2x;
    a21 = p2 * cos2i2; a22 = p1 * cos2 - p3 * sin2; a23 = p1 * cos2sin1 + p3 * sin2cos1;
    a31 = -p2 * sin2i2; a32 = -p1 * sin2cos1 - p3 * cos2sin1; a33 = -p1 * sin2 + p3 * cos2;
    a44 = p3;
  } else {
    a11 = p1; a12 = p2 * c2x; a13 = -p2 * s2x;
    a21 = p2 * cos2i2; a22 = p1 * cos2 - p3 * sin2; a23 = -p1 * cos2sin1 - p3 * sin2cos1;
    a31 = p2 * sin2i2; a32 = p1 * sin2cos1 + p3 * cos2sin1; a33 = -p1 * sin2 + p3 * cos2;
    a44 = p3;
  }
  // p4 = 0 (dustmat.f90:65): a24 = a34 = a42 = a43 = 0
  const R i = a11 * si + a12 * sq + a13 * su;
  const R q = a21 * si + a22 * sq + a23 * su + R(0) * sv;
  const R u = a31 * si + a32 * sq + a33 * su + R(0) * sv;
  const R v = R(0) * sq + R(0) * su + a44 * sv;
  si = i; sq = q; su = u; sv = v;
}

// ---- stokes.f90:46-388 --------------------------------------------------------------
template <class R>
__device__ __forceinline__ void stokes(Pkt<R>& p, int id, Rng& rng) {
  const R costp = p.cost, sintp = p.sint, phip = p.phi;
  const R g = pick4(p.g, id), pl = pick4(p.pl, id);
  R peak = peak_of<R>(g);
  R bmu, cosb2, sinbt, p1, p2, p3, rprob, ci, si_;
  bool upper;
  for (;;) {
    bmu = R(1) - R(2) * ran<R>(rng);
    cosb2 = bmu * bmu;
    dustmat<R>(g, pl, bmu, cosb2, p1, p2, p3);
    if (xabs(bmu) > R(1)) { bmu = bmu > R(1) ? R(1) : R(-1); cosb2 = R(1); }
    sinbt = xsqrt(R(1) - cosb2);
    const R ri1 = (R)kR2p * ran<R>(rng);
    upper = ri1 > (R)kPi;
    const R ang = upper ? (R)kR2p - ri1 : ri1;
    ci = xcos(ang);
    si_ = xsin(ang);
    const R s2 = R(2) * si_ * ci, c2 = R(2) * ci * ci - R(1);
    const R a12 = p2 * c2, a13 = upper ? p2 * s2 : -p2 * s2;
    rprob = (p1 * p.sip + a12 * p.sqp + a13 * p.sup) / p.sip;
    if (rprob > peak) peak = rprob;
    const R xran = ran<R>(rng);
    if (!(peak * xran > rprob)) break;
  }
  const R a = rprob;
  if (bmu == R(1)) return;
  const R s2x = R(2) * si_ * ci, c2x = R(2) * ci * ci - R(1);
  R cosi2 = R(0), sini2 = R(0);
  if (bmu == R(-1)) {
    si_ = R(1); sini2 = R(1); ci = R(0); cosi2 = R(0);
    p.cost = -costp; p.sint = sintp;
  } else {
    p.cost = costp * bmu + sintp * sinbt * ci;
    if (xabs(p.cost) < R(1)) {
      p.sint = xabs(xsqrt(R(1) - p.cost * p.cost));
      sini2 = si_ * sintp / p.sint;
      const R bott = p.sint * sinbt;
      cosi2 = costp / bott - p.cost * bmu / bott;
      if (cosi2 >= R(1)) { cosi2 = R(1); sini2 = R(0); }
      if (cosi2 <= R(-1)) { cosi2 = R(-1); sini2 = R(0); }
    } else {
      if (p.cost >= R(1)) { p.cost = R(1); cosi2 = R(-1); }
      if (p.cost <= R(-1)) { p.cost = R(-1); cosi2 = R(1); }
      p.sint = R(0); sini2 = R(0);
    }
  }
  R cosdph = upper ? -cosi2 * ci + sini2 * si_ * bmu : -ci * cosi2 + si_ * sini2 * bmu;
  if (xabs(cosdph) > R(1)) cosdph = cosdph > R(1) ? R(1) : R(-1);
  p.phi = upper ? phip + xacos(cosdph) : phip - xacos(cosdph);
  if (p.phi > (R)kR2p) p.phi -= (R)kR2p;
  if (p.phi < R(0)) p.phi += (R)kR2p;
  R si = p.sip, sq = p.sqp, su = p.sup, sv = p.svp;
  mueller<R>(upper, p1, p2, p3, s2x, c2x, sini2, cosi2, si, sq, su, sv);
  p.sip = si / a; p.sqp = sq / a; p.sup = su / a; p.svp = sv / a;
  p.cosp = xcos(p.phi);
  p.sinp = xsin(p.phi);
}

__device__ __forceinline__ float xcheck(float x) { return x > 1.f ? 1.f : (x < -1.f ? -1.f : x); }
__device__ __forceinline__ double xcheck(double x) { return x > 1.0 ? 1.0 : (x < -1.0 ? -1.0 : x); }

// ---- findangle3.f90:31-67 (phi2 = the module phie = 0, as the reference calls it)
template <class R>
__device__ __forceinline__ void findangle3(R cost1, R sint1, R phi1, R cosp1, R sinp1, R cost2, R sint2, R phi2,
                                           R cosp2, R sinp2, R& costnew, R& ri1) {
  costnew = xcheck(cost1 * cost2 + (sint1 * sint2 * (cosp1 * cosp2 + sinp1 * sinp2)));
  const R sintnew = xsqrt(R(1) - costnew * costnew);
  ri1 = R(0);
  if (sint1 > R(1.e-8) && sintnew > R(1.e-8)) {
    const R cosx = xcheck((cost2 - (cost1 * costnew)) / (sint1 * sintnew));
    const R x = xacos(cosx);
    if (phi2 > phi1) ri1 = (phi2 - phi1) > (R)kPi ? x : (R)kR2p - x;
    else ri1 = (phi1 - phi2) > (R)kPi ? (R)kR2p - x : x;
  }
}

// ---- stokespeel.f90:49-376 -----------------------------------------------------------
template <class R>
__device__ __forceinline__ void stokespeel(R g, R pl, R& sip, R& sqp, R& sup, R& svp, R cost, R sint, R ri1, R bmu,
                                           R costp, R sintp) {
  R cosb2 = bmu * bmu;
  R p1, p2, p3;
  dustmat<R>(g, pl, bmu, cosb2, p1, p2, p3);
  if (xabs(bmu) > R(1)) { bmu = bmu > R(1) ? R(1) : R(-1); cosb2 = R(1); }
  const R sinbt = xsqrt(R(1) - cosb2);
  const bool upper = ri1 > (R)kPi;
  const R ang = upper ? (R)kR2p - ri1 : ri1;
  R ci = xcos(ang), si_ = xsin(ang);
  if (bmu == R(1)) return;
  const R s2x = R(2) * si_ * ci, c2x = R(2) * ci * ci - R(1);
  R cosi2 = R(0), sini2 = R(0);
  if (bmu == R(-1)) {
    si_ = R(1); sini2 = R(1); ci = R(0); cosi2 = R(0);
  } else if (xabs(cost) < R(1)) {
    sini2 = si_ * sintp / sint;
    const R bott = sint * sinbt;
    cosi2 = costp / bott - cost * bmu / bott;
    if (cosi2 >= R(1)) { cosi2 = R(1); sini2 = R(0); }
    if (cosi2 <= R(-1)) { cosi2 = R(-1); sini2 = R(0); }
  } else {
    if (cost >= R(1)) cosi2 = R(-1);
    if (cost <= R(-1)) cosi2 = R(1);
    sini2 = R(0);
  }
  mueller<R>(upper, p1, p2, p3, s2x, c2x, sini2, cosi2, sip, sqp, sup, svp);
}

// ---- peel-off events -------------------------------------------------------------------
// Everything a peel-off ray needs from the event that spawns it: the packet
// state at a scattering (before stokes), at a re-emission (after reemit) or at
// its emission from the stellar surface.  Peel-off rays draw no random numbers,
// so they can run after the event, in any order and on any thread.
constexpr int kRecNoPeel = 1 << 15;  // PeelRec flag: the event has no peel-off rays

template <class R>
struct PeelRec {
  typename PosOf<R>::T x, y, z;
  int ir, it, ip;
  int flags;  // bit0 on_wall, bit1 scattered, bits2-4 i_orig, bits5-6 idust2, bit7 stellar-surface emission,
              // bits8-14 walls the event sits on, bit15 no peel-off (kRecNoPeel)
  int inub;
  R sip, sqp, sup, svp;
  R d0, d1, d2, d3, d4;  // scattered: cost, sint, phi, cosp, sinp of the incident packet; stellar: cosb, sinb, coslp, sinlp
  R g, pl;               // phase-matrix parameters of the scattering species
  R kapd[kSlots];
};

template <class R>
__device__ __forceinline__ int nu_bin(const RunArgs& a, R nub) {
  int inub;
  if constexpr (sizeof(R) == 4)
    inub = (int)((float)a.nfreq * logf(nub / (float)a.numin) / (float)a.lnurat) + 1;
  else
    inub = (int)((double)a.nfreq * log(nub / a.numin) / a.lnurat) + 1;
  return inub < 1 ? 1 : (inub > a.nfreq ? a.nfreq : inub);
}

template <class R>
__device__ __forceinline__ void make_rec(PeelRec<R>& e, const Pkt<R>& p, const RunArgs& a, int iflag, int idust2,
                                         int extra = 0) {
  e.x = p.x; e.y = p.y; e.z = p.z;
  e.ir = p.ir; e.it = p.it; e.ip = p.ip;
  e.flags = (p.on_wall ? 1 : 0) | (iflag << 1) | (p.i_orig << 2) | (idust2 << 5) | (p.on_wall << 8) | extra;
  e.inub = nu_bin<R>(a, p.nub);
  e.sip = p.sip; e.sqp = p.sqp; e.sup = p.sup; e.svp = p.svp;
  e.d0 = p.cost; e.d1 = p.sint; e.d2 = p.phi; e.d3 = p.cosp; e.d4 = p.sinp;
  e.g = pick4(p.g, idust2); e.pl = pick4(p.pl, idust2);
#pragma unroll
  for (int s = 0; s < kSlots; ++s) e.kapd[s] = p.kapd[s];
}

__device__ __forceinline__ void add9(unsigned long long* base, int64_t stride, int64_t b, double i, double q, double u,
                                     double v, double ss, double sq) {
  atomicAdd(base + b, fx(i, ss));
  atomicAdd(base + stride + b, fx(q, ss));
  atomicAdd(base + 2 * stride + b, fx(u, ss));
  atomicAdd(base + 3 * stride + b, fx(v, ss));
  atomicAdd(base + 4 * stride + b, fx(i * i, sq));
  atomicAdd(base + 5 * stride + b, fx(q * q, sq));
  atomicAdd(base + 6 * stride + b, fx(u * u, sq));
  atomicAdd(base + 7 * stride + b, fx(v * v, sq));
  atomicAdd(base + 8 * stride + b, 1ull);
}


// ---- peeloff_3d.f90:52-286: one observer direction k of one event (FP64 form) ----------
// The mixed form walks its peel-off rays in k_peel_mixed.
template <class R>
__device__ void peel_ray(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a,
                         const PeelRec<R>& e, int k, Local& L) {
  static_assert(sizeof(R) == 8, "peel_ray is the FP64 form");
  const double* pd = a.peeldir + 4 * k;
  const R coste = (R)__ldg(pd), sinte = (R)__ldg(pd + 1), cospe = (R)__ldg(pd + 2), sinpe = (R)__ldg(pd + 3);
  const int flags = e.flags;
  const int iflag = (flags >> 1) & 1;
  const int i_orig = (flags >> 2) & 7;
  if (flags & kRecNoPeel) return;
  R sip = e.sip, sqp = e.sqp, sup = e.sup, svp = e.svp;
  if (flags & 128) {
    // newdisktherm.F90:342-360: weight of a stellar-surface packet, uniform
    // disk (limb = 0) or Eddington limb darkening (limb = 1)
    const R cosnorm = e.d0 * coste + (e.d1 * sinte * (cospe * e.d2 + sinpe * e.d3));
    if (!(cosnorm > R(0))) return;
    sip = a.limb ? R(12.0 / 5.0) * e.sip * (cosnorm + cosnorm * cosnorm) : R(4) * e.sip * cosnorm;
  }
  double xp1 = e.x, yp1 = e.y, zp1 = e.z;
  int ir = e.ir, it = e.it, ip = e.ip;
  int on_wall = (flags >> 8) & 127;
  const R ux1 = sinte * cospe, uy1 = sinte * sinpe, uz1 = coste;
  L.add(HC3D_CNT_PEELS);
  if (on_wall) {
    const double rsq1 = xp1 * xp1 + yp1 * yp1 + zp1 * zp1;
    const bool outwards = (double)ux1 * xp1 + (double)uy1 * yp1 + (double)uz1 * zp1 > 0.0;
    const bool inner_wall = fabs(rsq1 - __ldg(m.r2arr + ir - 1)) < fabs(rsq1 - __ldg(m.r2arr + ir));
    if (inner_wall && !outwards) {
      if (ir == 1) return;
      ir = ir - 1;
      on_wall = 1 << 2;
    }
    if (!inner_wall && outwards) {
      ir = ir + 1;
      on_wall = 1 << 1;
    }
  }
  double tsum = 0.0;
  const int cap = 4 * (m.nrg + m.ntg + m.npg) + 64;
  const double uxd = (double)ux1, uyd = (double)uy1, uzd = (double)uz1;
  for (int n = 0;; ++n) {
    if (n > cap || it < 1 || it > m.ntg - 1 || ir < 1 || ir > m.nrg - 1) {
      L.add(HC3D_CNT_PEEL_STUCK);
      return;
    }
    R dt;
    int iface;
    if (!next_wall<R>(m, ux1, uy1, uz1, xp1, yp1, zp1, ir, it, ip, on_wall, dt, iface)) {
      L.add(HC3D_CNT_PEEL_STUCK);
      return;
    }
    const int64_t c = cidx(m, ir, it, ip);
    const Rho<R> rho = load_rho<R>(m, c);
    const unsigned mask = __ldg(m.peelmask + c);
    R opac = R(0);
#pragma unroll
    for (int s = 0; s < kSlots; ++s)
      if (mask & (1u << s)) opac += e.kapd[s] * rho.v[s];
    tsum += (double)(opac * dt);
    L.add(HC3D_CNT_CROSS_PEEL);
    if (tsum > kTauMax) return;
    step_index(m.npg, iface, ir, it, ip);
    xp1 += (double)dt * uxd;
    yp1 += (double)dt * uyd;
    zp1 += (double)dt * uzd;
    on_wall = 1 << own_after(iface);
    if (ir == m.nrg) break;
    if (ir == 0) return;
  }
  const R factor = (R)exp(-tsum);
  sip *= factor; sqp *= factor; sup *= factor; svp *= factor;
  if (iflag == 1) {
    R bmu, ri1;
    findangle3<R>(e.d0, e.d1, e.d2, e.d3, e.d4, coste, sinte, R(0), cospe, sinpe, bmu, ri1);
    stokespeel<R>(e.g, e.pl, sip, sqp, sup, svp, coste, sinte, ri1, bmu, e.d0, e.d1);
  }
  const double cte = (double)coste, ste = (double)sinte, cpe = (double)cospe, spe = (double)sinpe;
  const double yimage = zp1 * ste - yp1 * cte * spe - xp1 * cte * cpe;
  const double ximage = yp1 * cpe - xp1 * spe;
  const int ix = (int)((ximage + a.rmaxi) / a.fractxh) + 1;
  const int iy = (int)((yimage + a.rmaxi) / a.fractxh) + 1;
  const double rho2 = ximage * ximage + yimage * yimage;
  const int inub = e.inub;
  const int i_inter = iflag == 1 ? 2 : (i_orig == 1 ? 1 : 3);
  const int indx[3] = {1, 1 + i_orig, 5 + i_inter};
  const double dsip = (double)sip, dsqp = (double)sqp, dsup = (double)sup, dsvp = (double)svp;
  for (int ia = 1; ia <= a.nap; ++ia) {
    if (rho2 < __ldg(a.aperture2 + ia - 1)) {
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int64_t b = (int64_t)(inub - 1) + (int64_t)a.nfreq * (k + (int64_t)a.npeel * ((ia - 1) + (int64_t)a.nap * (indx[q] - 1)));
        add9(t.psed, d.npsed, b, dsip, dsqp, dsup, dsvp, t.stokes_scale, t.square_scale);
      }
    }
  }
  if (a.image && ix <= a.nx && iy <= a.nx && ix > 0 && iy > 0) {
    const int64_t b = (int64_t)k + (int64_t)a.npeel * ((ix - 1) + (int64_t)a.nx * (iy - 1));
    atomicAdd(t.img + b, fx(dsip, t.stokes_scale));
    atomicAdd(t.img + d.nimg + b, fx(dsqp, t.stokes_scale));
    atomicAdd(t.img + 2 * d.nimg + b, fx(dsup, t.stokes_scale));
    atomicAdd(t.img + 3 * d.nimg + b, fx(dsvp, t.stokes_scale));
    if (a.imcube) {  // peeloff_3d.f90:271-282: I by the three SED components, Q U V
      const int64_t bc = b + d.nimg * (int64_t)(inub - 1);
#pragma unroll
      for (int q = 0; q < 3; ++q) atomicAdd(t.cube + (int64_t)(indx[q] - 1) * d.ncube + bc, fx(dsip, t.stokes_scale));
      atomicAdd(t.cube + (int64_t)kNo * d.ncube + bc, fx(dsqp, t.stokes_scale));
      atomicAdd(t.cube + (int64_t)(kNo + 1) * d.ncube + bc, fx(dsup, t.stokes_scale));
      atomicAdd(t.cube + (int64_t)(kNo + 2) * d.ncube + bc, fx(dsvp, t.stokes_scale));
    }
  }
}

// ---- peel-off rays of the mixed form: a warp-synchronous ray pool --------------
// Each lane of a warp holds one (event, direction) ray.  A loop iteration
// refills the lanes whose ray ended (one atomic per warp), advances every
// live ray by one cell crossing, and parks the rays that left the grid in a
// per-warp buffer; the buffer is tallied 32 rays at a time, so the long
// tally code (peeloff_3d.f90:155-282) runs with every lane busy instead of
// one lane at a time.
struct PeelDir {
  float ux, uy, uz, coste, sinte, cospe, sinpe;
};

struct PeelEsc {
  unsigned long long e;
  float tsum, xf, yf, zf;
  int k;
};

constexpr int kPeelThreads = 256;
constexpr int kPeelBuf = 64;
constexpr int kPeelChunk = 256;  // rays a warp reserves per atomic, at most
constexpr int kPeelStage = 4;    // records a warp stages in shared memory
constexpr int kPeelSub = 16;     // crossings per lane between refills of the ray pool

// peeloff_3d.f90:155-282 for one ray of the mixed form that reached the grid
// edge: attenuation, the Stokes rotation of a scattered packet, image pixel
// and aperture binning
__device__ __forceinline__ void peel_tally_mixed(const DevTallies& t, const TallyDims& d, const RunArgs& a,
                                                 const PeelRec<float>& e, const PeelDir& dd, int k, float tsum,
                                                 float xf, float yf, float zf) {
  const int flags = e.flags;
  const int iflag = (flags >> 1) & 1;
  const int i_orig = (flags >> 2) & 7;
  const float coste = dd.coste, sinte = dd.sinte, cospe = dd.cospe, sinpe = dd.sinpe;
  float sip = e.sip, sqp = e.sqp, sup = e.sup, svp = e.svp;
  if (flags & 128) {  // newdisktherm.F90:342-360, limb = 0 or 1
    const float cosnorm = e.d0 * coste + (e.d1 * sinte * (cospe * e.d2 + sinpe * e.d3));
    sip = a.limb ? (float)(12.0 / 5.0) * e.sip * (cosnorm + cosnorm * cosnorm) : 4.f * e.sip * cosnorm;
  }
  const float factor = expf(-tsum);
  sip *= factor; sqp *= factor; sup *= factor; svp *= factor;
  if (iflag == 1) {
    float bmu, ri1;
    findangle3<float>(e.d0, e.d1, e.d2, e.d3, e.d4, coste, sinte, 0.f, cospe, sinpe, bmu, ri1);
    stokespeel<float>(e.g, e.pl, sip, sqp, sup, svp, coste, sinte, ri1, bmu, e.d0, e.d1);
  }
  const float yimage = zf * sinte - yf * coste * sinpe - xf * coste * cospe;
  const float ximage = yf * cospe - xf * sinpe;
  const float rmaxi = (float)a.rmaxi, fractxh = (float)a.fractxh;
  const int ix = (int)((ximage + rmaxi) / fractxh) + 1;
  const int iy = (int)((yimage + rmaxi) / fractxh) + 1;
  const float rho2 = ximage * ximage + yimage * yimage;
  const int i_inter = iflag == 1 ? 2 : (i_orig == 1 ? 1 : 3);
  const int indx[3] = {1, 1 + i_orig, 5 + i_inter};
  // the fixed-point values, converted once for all the bins they go to
  const float ss = (float)t.stokes_scale, sq = (float)t.square_scale;
  const unsigned long long v[9] = {fxf(sip, ss), fxf(sqp, ss), fxf(sup, ss), fxf(svp, ss),
                                   fxf(sip * sip, sq), fxf(sqp * sqp, sq), fxf(sup * sup, sq), fxf(svp * svp, sq), 1ull};
  for (int ia = 1; ia <= a.nap; ++ia) {
    if (rho2 < (float)__ldg(a.aperture2 + ia - 1)) {
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int64_t b = (int64_t)(e.inub - 1) +
                          (int64_t)a.nfreq * (k + (int64_t)a.npeel * ((ia - 1) + (int64_t)a.nap * (indx[q] - 1)));
#pragma unroll
        for (int j = 0; j < 9; ++j) atomicAdd(t.psed + j * d.npsed + b, v[j]);
      }
    }
  }
  if (a.image && ix <= a.nx && iy <= a.nx && ix > 0 && iy > 0) {
    const int64_t b = (int64_t)k + (int64_t)a.npeel * ((ix - 1) + (int64_t)a.nx * (iy - 1));
#pragma unroll
    for (int j = 0; j < 4; ++j) atomicAdd(t.img + j * d.nimg + b, v[j]);
    if (a.imcube) {  // peeloff_3d.f90:271-282: I by the three SED components, Q U V
      const int64_t bc = b + d.nimg * (int64_t)(e.inub - 1);
#pragma unroll
      for (int q = 0; q < 3; ++q) atomicAdd(t.cube + (int64_t)(indx[q] - 1) * d.ncube + bc, v[0]);
#pragma unroll
      for (int j = 1; j < 4; ++j) atomicAdd(t.cube + (int64_t)(kNo + j - 1) * d.ncube + bc, v[j]);
    }
  }
}

// The walk of one peel-off ray of the mixed form (peeloff_3d.f90:52-154).
//
// A peel-off ray is a straight line x(t) = c + t u, with t measured from the
// point c of closest approach to the origin (c.u = 0, |c| = p).  Each wall
// family's crossings along the line follow from invariants of the ray:
//   spheres  |x|^2 = p^2 + t^2 = R^2        t = -+sqrt((R - p)(R + p))
//   cones    C rho^2 = (1 - C) z^2,          a t^2 + 2 h t + q = 0 with
//            C = cos^2 theta                 a = C - uz^2, h = -cz uz, q = C p^2 - cz^2
//   planes   A x + B y = 0                   t = -(A cx + B cy) / (A ux + B uy)
// The walk keeps the next crossing of each family: the sphere bounding the
// cell in the direction of travel, the two roots ahead on each polar wall of
// the cell, and the azimuthal wall the ray turns towards (its azimuth
// changes monotonically).  A step crosses the nearest of them and recomputes
// only that family's next crossing -- one square root or one division --
// instead of the roots of every wall of the cell; the cell index changes
// only at those crossings, so the walk needs no re-location.  Measuring t
// from the point of closest approach keeps the FP32 resolution of t
// proportional to the distance from the origin, where the cells are
// proportionally small.  FP64 enters once per ray (the start point and c)
// and once per round of crossings (the escape tau sum, flush_tau).
//
// Walls the event sits on (PeelRec bits 8-14): a radial wall moves the ray
// into the cell on its side of travel (peeloff_3d.f90:60-87, tested on any
// wall as there); the root of a polar or azimuthal wall at the start point
// is not taken (the on_wall rule of closest_wall.f90:49-58).
constexpr float kInf = 3.402823466e38f;

// A ray set up by PeelWalk::start() (k_peel_mixed keeps these in shared
// memory until a lane takes one): the walk state at its first crossing
// search, its event record e and direction k.
struct PeelStart {
  float cx, cy, cz, p, p2, t, tr, lo1, lo2, hi1, hi2, tp;
  float kap[kSlots];
  int irit;  // ir | it << 16
  int ipup;  // ip | up << 16
  unsigned e;
  int k;
};

struct PeelWalk {
  float cx, cy, cz, ux, uy, uz;  // point of closest approach, direction
  float p, p2;                   // |c| and |c|^2
  float t;                       // parameter of the current point
  float tr;                      // next sphere crossing: the inner sphere when tr < 0, else the outer
  float lo1, lo2, hi1, hi2;      // roots ahead on the lower and upper polar wall of the cell
  float tp;                      // next azimuthal crossing
  int ir, it, ip, nstep;
  bool up;                       // azimuth increases along the ray
  float kap[kSlots];
  float4 rho;                    // peel-masked densities of the current cell, loaded when the ray entered it
  double tsum;  // FP64 escape tau: the FP32 partial sum tpart is added once per round
  float tpart;
  float tf;     // FP32 running tau, for the taumax test only

  enum { GOING = 0, OUT = 1, ENDED = 2 };  // OUT: left the grid, to be tallied

  // Issue the load of the current cell's densities.  Called as soon as the
  // ray enters a cell, before the next crossings of the walls are formed,
  // so that the load's latency overlaps that arithmetic instead of stalling
  // the next step.  An index out of range is caught by the next step.
  __device__ __forceinline__ void fetch_rho(const DevModel& m) {
    if (ir >= 1 && ir <= m.nrg - 1 && it >= 1 && it <= m.ntg - 1 && ip >= 1 && ip <= m.npg - 1)
      rho = __ldg(m.rho4p + (ir - 1) + (m.nrg - 1) * ((it - 1) + (m.ntg - 1) * (ip - 1)));
  }

  // the sphere bounding cell ir in the direction of travel at parameter t
  __device__ __forceinline__ void next_sphere(const DevModel& m) {
    const float rin = __ldg(m.rarrf + ir - 1);
    if (t < 0.f && rin > p) {
      const float ti = -fsqrt_pos((rin - p) * (rin + p));
      if (ti >= t) {
        tr = ti;
        return;
      }
    }
    const float rout = __ldg(m.rarrf + ir);
    const float q = (rout - p) * (rout + p);
    tr = fmaxf(fmaxf(q > 0.f ? fsqrt_pos(q) : 0.f, t), 0.f);
  }

  // The roots r1 <= r2 at or after t of polar wall w (index into conec) on
  // the nappe of its hemisphere, kInf where there are none; own: the ray
  // starts on this wall, so the root nearest t is not taken.  The cone is
  // C rho^2 - (1 - C) z^2 = 0 with C = cos^2 theta, so no coefficient grows
  // like tan^2 theta near the midplane; with |u| = 1 and c.u = 0 the terms
  // are a = C - uz^2, h = -cz uz, q = C p^2 - cz^2, and the discriminant
  // h^2 - a q = C (cz^2 - a p^2) has no cancelling terms.
  __device__ __forceinline__ void cone_roots(const DevModel& m, int w, bool own, float& r1, float& r2) const {
    r1 = r2 = kInf;
    const float2 cw = __ldg(m.conec + w);
    const float C = cw.x, hemi = cw.y;
    if (C < 0.f) {  // the midplane z = 0
      if (!own && uz != 0.f) {
        const float r = __fdividef(-cz, uz);
        if (r >= t) r1 = r;
      }
      return;
    }
    if (hemi == 0.f) return;  // a pole: no crossing
    const float a = fmaf(-uz, uz, C);
    const float h = -cz * uz;
    const float q = fmaf(C, p2, -cz * cz);
    const float D = C * fmaf(-a, p2, cz * cz);
    if (!(D > 0.f)) return;
    const float w_ = -(h + copysignf(fsqrt_pos(D), h));  // |w_| >= sqrt(D) > 0
    const float ra = a != 0.f ? __fdividef(w_, a) : kInf, rb = __fdividef(q, w_);
    const float x1 = fminf(ra, rb), x2 = fmaxf(ra, rb);
    bool v1 = fmaf(x1, uz, cz) * hemi > 0.f;
    bool v2 = x2 < kInf && fmaf(x2, uz, cz) * hemi > 0.f;
    if (own) {
      if (fabsf(x1 - t) <= fabsf(x2 - t)) v1 = false;
      else v2 = false;
    }
    v1 = v1 && x1 >= t;
    v2 = v2 && x2 >= t;
    r1 = v1 ? x1 : (v2 ? x2 : kInf);
    r2 = v1 && v2 ? x2 : kInf;
  }

  // the crossing at or after t of azimuthal wall w (index into planef) on its
  // half-plane, kInf where there is none
  __device__ __forceinline__ float plane_root(const DevModel& m, int w) const {
    const float2 ab = __ldg(m.planef + w);
    const float A = ab.x, B = ab.y;
    const float den = fmaf(A, ux, B * uy);
    if (den == 0.f) return kInf;
    const float r = __fdividef(-fmaf(A, cx, B * cy), den);
    if (!(r >= t)) return kInf;
    // (x, y) . (cos phi, sin phi) > 0 with cos phi = -B, sin phi = A
    if (fmaf(A, fmaf(r, uy, cy), -B * fmaf(r, ux, cx)) <= 0.f) return kInf;
    return r;
  }

  // false when the ray is not walked (the star's far side, or it enters the star)
  __device__ __forceinline__ bool start(const DevModel& m, const PeelRec<float>& r, const PeelDir& dd) {
    const int flags = r.flags;
    if (flags & kRecNoPeel) return false;
    if (flags & 128) {  // newdisktherm.F90:342-360: the star's surface faces the observer
      const float cosnorm = r.d0 * dd.coste + (r.d1 * dd.sinte * (dd.cospe * r.d2 + dd.sinpe * r.d3));
      if (!(cosnorm > 0.f)) return false;
    }
    ir = r.ir; it = r.it; ip = r.ip;
    const int own = (flags >> 8) & 127;
    const double x = dval(r.x), y = dval(r.y), z = dval(r.z);
    const double uxd = dd.ux, uyd = dd.uy, uzd = dd.uz;
    const double b = x * uxd + y * uyd + z * uzd;  // t of the start point
    bool go = true;
    if (own) {  // peeloff_3d.f90:60-87: leave the radial wall the event sits on
      const double rr0 = x * x + y * y + z * z;
      const bool inner_wall = fabs(rr0 - __ldg(m.r2arr + ir - 1)) < fabs(rr0 - __ldg(m.r2arr + ir));
      const bool outwards = b > 0.0;
      if (inner_wall && !outwards) {
        if (ir == 1) go = false;
        ir = ir - 1;
      }
      if (!inner_wall && outwards) ir = ir + 1;
    }
    const double cxd = fma(-b, uxd, x), cyd = fma(-b, uyd, y), czd = fma(-b, uzd, z);
    cx = (float)cxd; cy = (float)cyd; cz = (float)czd;
    ux = dd.ux; uy = dd.uy; uz = dd.uz;
    p2 = (float)(cxd * cxd + cyd * cyd + czd * czd);
    p = sqrtf(p2);
    t = (float)b;
#pragma unroll
    for (int s = 0; s < kSlots; ++s) kap[s] = r.kapd[s];
    tsum = 0.0;
    tpart = 0.f;
    tf = 0.f;
    nstep = 0;
    lo1 = lo2 = hi1 = hi2 = tp = kInf;
    tr = fmaxf(t, 0.f);
    up = x * uyd - y * uxd > 0.0;  // z component of x cross u, constant along the line
    if (!go || ir < 1 || ir > m.nrg - 1) return go;
    next_sphere(m);
    if (m.ntg > 2) {
      cone_roots(m, it - 1, (own >> 3) & 1, lo1, lo2);
      cone_roots(m, it, (own >> 4) & 1, hi1, hi2);
      if (m.npg > 2) {
        const bool mine = up ? ((own >> 6) & 1) : ((own >> 5) & 1);
        tp = mine ? kInf : plane_root(m, up ? ip : ip - 1);
      }
    }
    return go;
  }

  __device__ __forceinline__ int step(const DevModel& m, int cap, PeelCount& pc) {
    if (nstep > cap || it < 1 || it > m.ntg - 1 || ir < 1 || ir > m.nrg - 1) {
      pc.stuck++;
      return ENDED;
    }
    ++nstep;
    const float th = fminf(lo1, hi1);
    const float tn = fminf(tr, fminf(th, tp));
    const float ds = tn - t;
    t = tn;
    const float opac = fmaf(kap[0], rho.x, fmaf(kap[1], rho.y, fmaf(kap[2], rho.z, kap[3] * rho.w)));
    const float dtau = opac * ds;
    tpart += dtau;
    tf += dtau;
    pc.cross++;
    if (tf > (float)kTauMax) return ENDED;
    if (tn == tr) {
      ir += tr < 0.f ? -1 : 1;
      if (ir == m.nrg) return OUT;
      if (ir == 0) return ENDED;
      fetch_rho(m);
      next_sphere(m);
    } else if (tn == th) {
      if (lo1 <= hi1) {  // the lower polar wall: into cell it - 1
        hi1 = lo2;
        hi2 = kInf;
        --it;
        if (it < 1) return GOING;  // caught by the range check of the next step
        fetch_rho(m);
        cone_roots(m, it - 1, false, lo1, lo2);
      } else {           // the upper polar wall: into cell it + 1
        lo1 = hi2;
        lo2 = kInf;
        ++it;
        if (it > m.ntg - 1) return GOING;
        fetch_rho(m);
        cone_roots(m, it, false, hi1, hi2);
      }
    } else {  // the azimuthal wall, with the wrap at 0 / 2 pi
      if (up) {
        ip = ip == m.npg - 1 ? 1 : ip + 1;
        fetch_rho(m);
        tp = plane_root(m, ip);
      } else {
        ip = ip == 1 ? m.npg - 1 : ip - 1;
        fetch_rho(m);
        tp = plane_root(m, ip - 1);
      }
    }
    return GOING;
  }

  // the set-up state of a ray that start() accepted, for a lane to take later
  __device__ __forceinline__ void save(PeelStart& q, unsigned e, int k) const {
    q.cx = cx; q.cy = cy; q.cz = cz; q.p = p; q.p2 = p2; q.t = t; q.tr = tr;
    q.lo1 = lo1; q.lo2 = lo2; q.hi1 = hi1; q.hi2 = hi2; q.tp = tp;
#pragma unroll
    for (int s = 0; s < kSlots; ++s) q.kap[s] = kap[s];
    q.irit = ir | (it << 16);
    q.ipup = ip | ((int)up << 16);
    q.e = e;
    q.k = k;
  }

  __device__ __forceinline__ void load(const DevModel& m, const PeelStart& q, const PeelDir& dd) {
    cx = q.cx; cy = q.cy; cz = q.cz; p = q.p; p2 = q.p2; t = q.t; tr = q.tr;
    lo1 = q.lo1; lo2 = q.lo2; hi1 = q.hi1; hi2 = q.hi2; tp = q.tp;
#pragma unroll
    for (int s = 0; s < kSlots; ++s) kap[s] = q.kap[s];
    ir = q.irit & 0xffff; it = q.irit >> 16;
    ip = q.ipup & 0xffff; up = (q.ipup >> 16) != 0;
    ux = dd.ux; uy = dd.uy; uz = dd.uz;
    tsum = 0.0;
    tpart = 0.f;
    tf = 0.f;
    nstep = 0;
    fetch_rho(m);
  }

  // add the FP32 partial escape tau of the last round to the FP64 sum
  __device__ __forceinline__ void flush_tau() {
    tsum += (double)tpart;
    tpart = 0.f;
  }

  // FP32 point of the ray where it left the grid
  __device__ __forceinline__ void end_point(float& x, float& y, float& z) const {
    x = fmaf(t, ux, cx);
    y = fmaf(t, uy, cy);
    z = fmaf(t, uz, cz);
  }
};

__device__ __forceinline__ PeelDir peel_dir(const RunArgs& a, int k) {
  const double* pd = a.peeldir + 4 * k;
  PeelDir q;
  q.coste = (float)__ldg(pd); q.sinte = (float)__ldg(pd + 1);
  q.cospe = (float)__ldg(pd + 2); q.sinpe = (float)__ldg(pd + 3);
  q.ux = q.sinte * q.cospe; q.uy = q.sinte * q.sinpe; q.uz = q.coste;
  return q;
}

// One peel-off ray of the mixed form walked by one thread (the per-packet
// loop of k_transport: trace harness and unwaved runs)
__device__ __forceinline__ void peel_ray_mixed(const DevModel& m, const DevTallies& t, const TallyDims& d,
                                               const RunArgs& a, const PeelRec<float>& e, int k, Local& L) {
  const PeelDir dd = peel_dir(a, k);
  PeelWalk w;
  if (!w.start(m, e, dd)) return;
  w.fetch_rho(m);
  PeelCount pc{1u, 0u, 0u};
  const int cap = 4 * (m.nrg + m.ntg + m.npg) + 64;
  int st;
  while ((st = w.step(m, cap, pc)) == PeelWalk::GOING) {
    if ((w.nstep & 7) == 0) w.flush_tau();  // the rounds of k_peel_mixed
  }
  w.flush_tau();
  L.add(HC3D_CNT_PEELS);
  L.add(HC3D_CNT_CROSS_PEEL, pc.cross);
  if (pc.stuck) L.add(HC3D_CNT_PEEL_STUCK, pc.stuck);
  if (st == PeelWalk::OUT) {
    float x, y, z;
    w.end_point(x, y, z);
    peel_tally_mixed(t, d, a, e, dd, k, (float)w.tsum, x, y, z);
  }
}

// The peel-off rays of one event walked by the thread that made it (the
// per-packet loop of k_transport)
template <class R>
__device__ __forceinline__ void peel_all(const DevModel& m, const DevTallies& t, const TallyDims& d,
                                         const RunArgs& a, const PeelRec<R>& rec, Local& L) {
  for (int k = 0; k < a.npeel; ++k) {
    if constexpr (sizeof(R) == 4) peel_ray_mixed(m, t, d, a, rec, k, L);
    else peel_ray<R>(m, t, d, a, rec, k, L);
  }
}

// ---- lucydustfreq.f90:19-157 -------------------------------------------------------------
// Mixed form.  The row pair j, j+1 of the Lucy CDF and the weight f follow
// from the cell temperature, which is fixed during a run: they are cached in
// the packet while it stays in the cell and species slot.  The frequency
// index is the same bracket of the interpolated CDF as the reference's
// bisection (the CDF is non-decreasing, so the bracket is unique), found
// from the guide table and a short bisection over the interleaved rows.
__device__ __forceinline__ float lucy_freq_mixed(const DevModel& m, LucyRow& lr, int64_t c, int id, Rng& rng) {
  const int nT = m.nT, nnu = m.nnu;
  const float* nuint = m.nuintf;
  const int key = (int)(4 * c + id);
  if (key != lr.key) {
    const float T0 = __ldg(m.tdustf + 4 * c + id);
    const float* lTint = m.lTintf;
    const float lT0 = logf(T0);
    const float l1 = __ldg(lTint), lN = __ldg(lTint + nT - 1);
    int j = (int)((float)(nT - 1) * (lT0 - l1) / (lN - l1)) + 1;
    j = j < 1 ? 1 : (j > nT - 1 ? nT - 1 : j);
    float f = (lT0 - __ldg(lTint + j - 1)) / (__ldg(lTint + j) - __ldg(lTint + j - 1));
    f = f < 0.f ? 0.f : (f > 1.f ? 1.f : f);
    const int pr = id * (nT - 1) + (j - 1);
    const float2 k1 = __ldg(m.kpairf + (size_t)pr * nnu), kn = __ldg(m.kpairf + (size_t)pr * nnu + nnu - 1);
    lr.key = key;
    lr.pr = pr;
    lr.T0 = T0;
    lr.f = f;
    lr.P0 = fminf((1.f - f) * k1.x + f * k1.y, 1.f);
    lr.P1 = fminf((1.f - f) * kn.x + f * kn.y, 1.f);
  }
  const float T0 = lr.T0, f = lr.f;
  const float xi = ran<float>(rng);
  float P0 = lr.P0, P1 = lr.P1;
  if (xi < P0) return P0 > 0.f ? T0 * xi * __ldg(nuint) / P0 : T0 * __ldg(nuint);
  if (xi >= P1) {
    if (P1 < 1.f && xi < 1.f) return T0 * __ldg(nuint + nnu - 1) * (1.f - P1) / (1.f - xi);
    return T0 * __ldg(nuint + nnu - 1);
  }
  const float2* KP = m.kpairf + (size_t)lr.pr * nnu;
  auto P = [&](int i) { return fminf((1.f - f) * __ldg(KP + i - 1).x + f * __ldg(KP + i - 1).y, 1.f); };
  const short2 g = __ldg(m.kguide + (size_t)lr.pr * kGuide + min((int)(xi * (float)kGuide), kGuide - 1));
  int i0 = g.x, i1 = g.y;
  const float Pa = P(i0), Pb = P(i1);
  if (Pa <= xi) P0 = Pa; else i0 = 1;
  if (Pb > xi) P1 = Pb; else i1 = nnu;
  if (i1 <= i0) { i0 = 1; i1 = nnu; P0 = lr.P0; P1 = lr.P1; }
  while (i1 - i0 > 1) {
    const int i = (i0 + i1) / 2;
    const float v = P(i);
    if (v > xi) { i1 = i; P1 = v; }
    else { i0 = i; P0 = v; }
  }
  float w;
  if (xi < P0) w = 0.f;
  else if (xi > P1) w = 1.f;
  else if (P0 <= 0.f) w = 0.5f;
  else if (P1 <= 0.f || xi <= 0.f) w = f;
  else w = logf(xi / P0) / logf(P1 / P0);
  const float n0 = __ldg(nuint + i0 - 1), n1 = __ldg(nuint + i1 - 1);
  return T0 * n0 * powf(n1 / n0, w);
}

// FP64 form: the reference's bisection.
template <class R> __device__ __forceinline__ R xpow(R a, R b);
template <> __device__ __forceinline__ float xpow<float>(float a, float b) { return powf(a, b); }
template <> __device__ __forceinline__ double xpow<double>(double a, double b) { return pow(a, b); }
__device__ __forceinline__ float xlog10(float x) { return log10f(x); }
__device__ __forceinline__ double xlog10(double x) { return log10(x); }

template <class R>
__device__ __forceinline__ R lucydustfreq(const DevModel& m, R T0, int id, Rng& rng) {
  const int nT = m.nT, nnu = m.nnu;
  const R* lTint = tab<R>(m.lTint, m.lTintf);
  const R* nuint = tab<R>(m.nuint, m.nuintf);
  const R* K = tab<R>(m.kapBint, m.kapBintf) + (size_t)id * nT * nnu;
  const R lT0 = xlog(T0);
  const R xi = ran<R>(rng);
  const R l1 = __ldg(lTint), lN = __ldg(lTint + nT - 1);
  int j = (int)((R)(nT - 1) * (lT0 - l1) / (lN - l1)) + 1;
  j = j < 1 ? 1 : (j > nT - 1 ? nT - 1 : j);
  R f = (lT0 - __ldg(lTint + j - 1)) / (__ldg(lTint + j) - __ldg(lTint + j - 1));
  f = f < R(0) ? R(0) : (f > R(1) ? R(1) : f);
#define KB(jj, ii) __ldg(K + (size_t)((jj) - 1) + (size_t)nT * ((ii) - 1))
  int i0 = 1, i1 = nnu;
  R P0 = (R(1) - f) * KB(j, i0) + f * KB(j + 1, i0);
  if (xi < P0) return (P0 > R(0) ? T0 * xi * __ldg(nuint) / P0 : T0 * __ldg(nuint));
  R P1 = (R(1) - f) * KB(j, i1) + f * KB(j + 1, i1);
  if (P1 > R(1)) P1 = R(1);
  if (xi >= P1) {
    if (P1 < R(1) && xi < R(1)) return (T0 * __ldg(nuint + nnu - 1) * (R(1) - P1) / (R(1) - xi));
    return (T0 * __ldg(nuint + nnu - 1));
  }
  while (i1 - i0 > 1) {
    const int i = (i0 + i1) / 2;
    R P = (R(1) - f) * KB(j, i) + f * KB(j + 1, i);
    if (P > R(1)) P = R(1);
    if (P < P0) { P0 = P; i0 = i; }
    if (P > P1) { P1 = P; i1 = 1; }
    if (P > xi) { i1 = i; P1 = P; }
    else { i0 = i; P0 = P; }
  }
#undef KB
  if (xi < P0) f = R(0);
  else if (xi > P1) f = R(1);
  else if (P0 <= R(0)) f = R(0.5);
  else if (P1 <= R(0) || xi <= R(0)) { }
  else f = xlog(xi / P0) / xlog(P1 / P0);
  const R n0 = __ldg(nuint + i0 - 1), n1 = __ldg(nuint + i1 - 1);
  return (T0 * n0 * xpow<R>(n1 / n0, f));
}

// ---- atmosfreq, starbarb.f90:120-156 ---------------------------------------------------
template <class R>
__device__ R atmosfreq(const DevModel& m, Rng& rng) {
  const R* hnuint = tab<R>(m.hnuint, m.hnuintf);
  const R* lognu = tab<R>(m.lognu, m.lognuf);
  const R* loghnu = tab<R>(m.loghnu, m.loghnuf);
  const R* atmosnu = tab<R>(m.atmosnu, m.atmosnuf);
  const R xi = ran<R>(rng);
  // locate2 (nr.f:152-171) on the increasing hnuint
  const int n = m.nhnu;
  int jl = 0, ju = n + 1;
  while (ju - jl > 1) {
    const int jm = (ju + jl) / 2;
    if (xi > __ldg(hnuint + jm - 1)) jl = jm; else ju = jm;
  }
  int i = jl < 1 ? 1 : (jl > n - 1 ? n - 1 : jl);
  if (i > 1) {
    const R l0 = __ldg(lognu + i - 1), l1 = __ldg(lognu + i);
    const R h0 = __ldg(loghnu + i - 1), h1 = __ldg(loghnu + i);
    return xpow<R>(R(10), l0 + (l1 - l0) * (xlog10(xi) - h0) / (h1 - h0));
  }
  const R a0 = __ldg(atmosnu + i - 1), a1 = __ldg(atmosnu + i);
  const R c0 = __ldg(hnuint + i - 1), c1 = __ldg(hnuint + i);
  return a0 + (a1 - a0) * (xi - c0) / (c1 - c0);
}

__device__ __forceinline__ int locate_dev(const double* xx, int n, double x) {
  int jl = 0, ju = n + 1;
  const bool asc = __ldg(xx + n - 1) > __ldg(xx);
  while (ju - jl > 1) {
    const int jm = (ju + jl) / 2;
    if (asc == (x > __ldg(xx + jm - 1))) jl = jm; else ju = jm;
  }
  if (jl == 0 && x == __ldg(xx)) jl = 1;
  return jl;
}

// ---- rep_draine.f90:1-65: the re-emission frequency of a small grain ---------------
// One uniform picks the bin of the cumulative spectrum of row im (nr
// locate3: the bisection without locate's fix-up at the first row), and of
// row im + 1, each interpolated linearly in log10 cdf against log10 nu; the
// two log frequencies are mixed by jmf (past the last row, row im alone).
// FP64 in both forms: one draw per small-grain absorption.
__device__ __forceinline__ int locate3_dev(const double* xx, int n, double x) {
  int jl = 0, ju = n + 1;
  const bool asc = __ldg(xx + n - 1) > __ldg(xx);
  while (ju - jl > 1) {
    const int jm = (ju + jl) / 2;
    if (asc == (x > __ldg(xx + jm - 1))) jl = jm; else ju = jm;
  }
  return jl;
}

__device__ __forceinline__ double draine_logfreq(const DevModel& m, int j, double xran, double lx) {
  const int nd = m.sg_nd;
  int i = locate3_dev(m.sg_cdf + (size_t)(j - 1) * nd, nd, xran);
  if (i == nd) i = nd - 1;
  if (i == 0) i = 1;
  const double* lc = m.sg_logcdf + (size_t)(j - 1) * nd;
  const double l0 = __ldg(lc + i - 1), l1 = __ldg(lc + i);
  const double f0 = __ldg(m.sg_logfreq + i - 1), f1 = __ldg(m.sg_logfreq + i);
  return (lx - l0) / (l1 - l0) * (f1 - f0) + f0;
}

template <class R>
__device__ __forceinline__ double rep_draine(const DevModel& m, int im, double jmf, Rng& rng) {
  const double xran = (double)ran<R>(rng);
  const double lx = log10(xran);
  const double lf1 = draine_logfreq(m, im, xran, lx);
  double lf = lf1;
  if (im + 1 <= m.sg_nemit) lf = lf1 + jmf * (draine_logfreq(m, im + 1, xran, lx) - lf1);
  return pow(10.0, lf);
}

// ---- propagate.f90:206-319 escape binning ----------------------------------------
template <class R>
__device__ void bin_escape(const DevTallies& t, const TallyDims& d, const RunArgs& a, const Pkt<R>& p, double xpold,
                           double ypold, double zpold, int iflag, int iscat, Local& L) {
  int it = (int)((double)a.nmu * (1.0 - (double)p.cost) / 2.0) + 1;
  it = it > a.nmu ? a.nmu : (it < 1 ? 1 : it);
  double phi = (double)p.phi;
  if (phi < 0.0) phi += kR2p;
  int ip = (int)((double)a.nph * phi / kR2p) + 1;
  ip = ip > a.nph ? a.nph : (ip < 1 ? 1 : ip);
  const double dmu = 2.0 / (double)a.nmu;
  const double u = 1.0 - dmu * ((double)it - 0.5);
  const double sini = sqrt(1.0 - u * u);
  const double cp = (double)p.cosp, sp = (double)p.sinp;
  const double x = ypold * cp - xpold * sp;
  const double y = zpold * sini - ypold * u * sp - xpold * u * cp;
  const double rho2 = x * x + y * y;
  if (rho2 < __ldg(a.aperture2 + a.nap - 1) * 1.0001) {
    L.add(HC3D_CNT_FLUX);
    if (iflag == 1) {
      L.add(HC3D_CNT_SFLUX);
      L.add(HC3D_CNT_NSCAT, (unsigned long long)iscat);
    }
  }
  const int inub = nu_bin<R>(a, p.nub);
  const int i_inter = iflag == 1 ? 2 : (p.i_orig == 1 ? 1 : 3);
  const int indx[3] = {1, 1 + p.i_orig, 5 + i_inter};
  const double si = (double)p.sip, sq = (double)p.sqp, su = (double)p.sup, sv = (double)p.svp;
  const bool count = !(iflag == 0 && p.i_orig == 4);
  // the fixed-point values, converted once for all the bins they go to
  const unsigned long long v[9] = {fx(si, t.stokes_scale), fx(sq, t.stokes_scale), fx(su, t.stokes_scale),
                                   fx(sv, t.stokes_scale), fx(si * si, t.square_scale), fx(sq * sq, t.square_scale),
                                   fx(su * su, t.square_scale), fx(sv * sv, t.square_scale), 1ull};
  for (int ia = 1; ia <= a.nap; ++ia) {
    if (rho2 < __ldg(a.aperture2 + ia - 1) && count) {
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int64_t b = (int64_t)(inub - 1) +
                          (int64_t)a.nfreq * ((it - 1) + (int64_t)a.nmu * ((ip - 1) + (int64_t)a.nph * ((ia - 1) + (int64_t)a.nap * (indx[q] - 1))));
#pragma unroll
        for (int j = 0; j < 9; ++j) atomicAdd(t.sed + j * d.nsed + b, v[j]);
      }
    }
  }
  if (count) L.add(HC3D_CNT_SUMSUB, fx(si, t.stokes_scale));
  L.add(HC3D_CNT_SUMALL, fx(si, t.stokes_scale));
  if (iflag == 1) L.add(HC3D_CNT_SCOUNT);
  L.add(HC3D_CNT_ESCAPED);
}

// ---- the packet history, split at its events ----------------------------------------
// propagate.f90 keeps these in locals; they persist across the waves below.
template <class R>
struct Flow {
  typename PosOf<R>::T xpold, ypold, zpold;
  int iflag, iscat, iint, idust2;
  int64_t ntot;
};

enum { ST_DONE = 0, ST_INTERACT = 1 };

// initp_transform (initp_common.f90:31-94): the direction (cost, phi) drawn
// in the frame of the surface point (cosb, lp), rotated into the grid frame
template <class R>
__device__ __forceinline__ void initp_transform(Pkt<R>& p) {
  if (xabs(p.cosb) < R(0.9999999)) {
    R costi = p.cost * p.cosb - p.sint * p.sinb * p.cosp;
    if (xabs(costi) > R(1)) {
      if (costi > R(1)) costi = R(1);
      if (p.cost < R(-1)) costi = R(-1);
    }
    const R sinti = xsqrt(R(1) - costi * costi);
    R phinew;
    if (sinti > R(0.0000001)) {
      R cospn = (p.cost - costi * p.cosb) / (sinti * p.sinb);
      if (xabs(cospn) > R(1)) cospn = cospn < R(0) ? R(-1) : R(1);
      if (p.phi < (R)kPi) {
        phinew = xacos(cospn);
        if (phinew > (R)kPi) phinew = (R)kPi;
      } else {
        phinew = (R)kR2p - xacos(cospn);
        if (phinew < (R)kPi) phinew = (R)kPi;
      }
    } else {
      phinew = R(0);
    }
    p.phi = phinew; p.cost = costi; p.sint = sinti;
  } else if (p.cosb < R(0)) {
    p.cost = -p.cost;
  }
  p.phi = p.phi + p.lp;
  if (p.phi > (R)kR2p) p.phi -= (R)kR2p;
  if (p.phi < R(0)) p.phi += (R)kR2p;
  p.sinp = xsin(p.phi);
  p.cosp = xcos(p.phi);
}

// darkening (samptabl.f90:29-65): mu from the table of prob(mu) = (mu^3 + mu^2)/2
// (Eddington limb darkening, intensity ~ 1 + mu), interpolated as the Fortran
// does, with the table step delmu = 1/ntab
template <class R>
__device__ __forceinline__ R darkening(const DevModel& m, Rng& rng) {
  const double xi = (double)ran<R>(rng);
  int n = locate_dev(m.limb_prob, m.nlimb, xi);  // 1 <= n <= ntab-1 for 0 < xi < 1
  n = n < 1 ? 1 : (n > m.nlimb - 1 ? m.nlimb - 1 : n);
  const double delmu = 1.0 / (double)m.nlimb;
  const double p1 = __ldg(m.limb_prob + n), p0 = __ldg(m.limb_prob + n - 1);
  return (R)(__ldg(m.limb_xmu + n) - (p1 - xi) / (p1 - p0) * delmu);
}

__device__ __forceinline__ void set_status(const RunArgs& a, int code) {
  if (a.status) atomicCAS(a.status, 0, code);
}

// Record a faulted packet (global id and fault code) in the fault log.
__device__ __forceinline__ void log_fault(const DevTallies& t, const Rng& rng, int code) {
  if (!t.fault_log) return;
  const unsigned long long k = atomicAdd(t.fault_count, 1ull);
  if (k < (unsigned long long)kFaultLog)
    t.fault_log[k] = ((unsigned long long)rng.c2 | ((unsigned long long)rng.c3 << 32)) | ((unsigned long long)code << 56);
}

// bbfreq (random.f90:49-77): a frequency from the Planck function of
// temperature teff (K/11605), drawn as -ln(z1 z2 z3 z4) teff / i, a Gamma(4)
// variate of rate i, with i picked with weight 1/i^4 from the partial sums
// inczeta.  FP64 in both forms (one draw per hot-spot or gas packet).
template <class R>
__device__ double bbfreq(const DevModel& m, double teff, Rng& rng) {
  const double z0 = __ldg(m.inczeta + kIzmax - 1) * (double)ran<R>(rng);
  const double z1 = (double)ran<R>(rng), z2 = (double)ran<R>(rng), z3 = (double)ran<R>(rng),
               z4 = (double)ran<R>(rng);
  int i = 1;
  while (i < kIzmax && z0 > __ldg(m.inczeta + i - 1)) ++i;
  return -log(z1 * z2 * z3 * z4) * teff / (double)i;
}

constexpr int kEmitTries = 1 << 24;  // cap of the rejection loops of an emission point
enum { F_EMIT = 5 };                 // fault code: no emission point within the cap

// Stellar and hot-spot packet emission, newdisktherm.F90:256-337 with
// initpspot (initpspot.f90:33-160), initp_sample (limb = 0, or the Eddington
// table) and initp_transform.  spotph = 1 for a hot-spot packet: with spots
// (ispot) its point is redrawn until it lies in a spot; it radiates at the
// shock temperature, half of the hot-spot packets as X-rays
// (newdisktherm.F90:270-273).  A stellar packet whose point falls in a spot
// also takes the shock temperature when the spots cover less than the star
// (fspot < 1).  The spot geometry is FP64 in both forms (one test per packet).
// rec receives the stellar-surface peel-off event.  Returns false when no
// point was found within the cap (the packet is dropped and logged).
template <class R>
__device__ bool emit_star(const DevModel& m, const DustView<R>& dv, const RunArgs& a, Pkt<R>& p, Rng& rng,
                          PeelRec<R>& rec, Tracer& tr, int spotph) {
  p.on_wall = 0;
  p.safe = 0.f;
  p.lrow.key = -1;
  p.sip = R(1); p.sqp = R(0); p.sup = R(0); p.svp = R(0);
  const bool spots = a.src_on && a.src.ispot;
  for (int tries = 0;; ++tries) {
    for (;;) {
      const R xran = ran<R>(rng);
      p.cosb = R(1) - R(2) * xran;
      p.sinb = xsqrt(R(1) - p.cosb * p.cosb);
      if (p.cosb != R(0) && xabs(p.cosb) < R(1)) break;
    }
    p.lp = (R)kR2p * ran<R>(rng);
    if (!spots) break;
    const hc3d_sources& S = a.src;
    const double cb = (double)p.cosb, sb = (double)p.sinb, lp = (double)p.lp;
    const double cphi = cos(lp), sphi = sin(lp);
    const double d1 = S.spot1[0] * sb * cphi + S.spot1[1] * sb * sphi + S.spot1[2] * cb;
    const double d2 = S.spot2[0] * sb * cphi + S.spot2[1] * sb * sphi + S.spot2[2] * cb;
    if (spotph == 1 && (S.nspot == 1 ? d1 < S.csprad : (d1 < S.csprad && d2 < S.csprad))) {
      if (tries >= kEmitTries) return false;
      continue;
    }
    if (S.fspot < 1.0) {
      double dellon = lp < kPi ? lp : kR2p - lp;
      if (S.spot1[2] * cb + S.spot1[3] * sb * cos(dellon) > S.csprad) spotph = 1;
      if (S.nspot == 2) {
        dellon = lp < kPi ? kPi - lp : lp - kPi;
        if (S.spot2[2] * cb + S.spot2[3] * sb * cos(dellon) > S.csprad) spotph = 1;
      }
    }
    break;
  }
  // initp_sample (initp_common.f90:1-29): cost = sqrt(xi), or the Eddington table
  p.cost = a.limb ? darkening<R>(m, rng) : xsqrt(ran<R>(rng));
  p.sint = xsqrt(R(1) - p.cost * p.cost);
  p.phi = (R)kR2p * ran<R>(rng);
  p.cosp = xcos(p.phi);
  p.sinp = xsin(p.phi);
  initp_transform<R>(p);
  if (spotph) {
    double nu = bbfreq<R>(m, a.src.tshock, rng);
    if (ran<R>(rng) < R(0.5)) nu = 1.2398 / 0.06 + (double)ran<R>(rng) * (1.2398 / 0.015 - 1.2398 / 0.06);
    p.nub = (R)nu;
  } else {
    p.nub = atmosfreq<R>(m, rng);
  }
  p.i_orig = 1;
  opacset<R>(m, dv, p, p.nub, a);
  const R coslp = xcos(p.lp), sinlp = xsin(p.lp);
  const double rp_ = (double)p.sinb;
  set_pos(p.z, (double)p.cosb);
  set_pos(p.x, rp_ * (double)coslp);
  set_pos(p.y, rp_ * (double)sinlp);
  p.ux = p.sint * p.cosp; p.uy = p.sint * p.sinp; p.uz = p.cost;
  p.ir = 1;
  p.on_wall = 1 << 1;  // on the stellar surface: the inner radial wall (id 1) of cell 1
  p.it = locate_dev(m.thetarr, m.ntg, acos((double)p.cosb));
  p.ip = locate_dev(m.phiarr, m.npg, (double)p.lp);
  p.it = p.it < 1 ? 1 : (p.it > m.ntg - 1 ? m.ntg - 1 : p.it);
  p.ip = p.ip < 1 ? 1 : (p.ip > m.npg - 1 ? m.npg - 1 : p.ip);
  tr.add(0, p.ir, p.it, p.ip, 0, 0.0, dval(p.x), dval(p.y), dval(p.z));
  make_rec<R>(rec, p, a, 0, 0, 128);
  rec.d0 = p.cosb; rec.d1 = p.sinb; rec.d2 = coslp; rec.d3 = sinlp;
  return true;
}

// rep_isrf (rep_isrf.f90:1-41): the frequency of an external packet, by
// log-log interpolation in the cumulative distribution of the external field
// (FP64 in both forms: one draw per external packet)
template <class R>
__device__ __forceinline__ R rep_isrf(const DevModel& m, Rng& rng) {
  const double xran = (double)ran<R>(rng);
  const int n = m.nisrf;
  int i = locate_dev(m.isrf_cdf, n, xran);
  if (i == n) i = n - 1;
  if (i == 0) i = 1;
  const double lc0 = __ldg(m.isrf_logcdf + i - 1), lc1 = __ldg(m.isrf_logcdf + i);
  const double lf0 = __ldg(m.isrf_logfreq + i - 1), lf1 = __ldg(m.isrf_logfreq + i);
  return (R)pow(10.0, lf0 + (log10(xran) - lc0) / (lc1 - lc0) * (lf1 - lf0));
}

// External packet, newdisktherm.F90:378-440 with initpout (initpout.f90:3-66):
// a point on the sphere of 0.999999 rmax, a direction drawn inwards with
// cost = -sqrt(xi) in the frame of that point, the frequency from the
// external field.  The packet starts inside the outermost shell (not on a
// wall).  It has no direct peel-off (the Fortran leaves it commented out, so
// that the unprocessed background is not imaged): rec is marked empty.
template <class R>
__device__ void emit_external(const DevModel& m, const DustView<R>& dv, const RunArgs& a, Pkt<R>& p, Rng& rng,
                              PeelRec<R>& rec, Tracer& tr) {
  p.on_wall = 0;
  p.safe = 0.f;
  p.lrow.key = -1;
  p.sip = R(1); p.sqp = R(0); p.sup = R(0); p.svp = R(0);
  p.cosb = R(1) - R(2) * ran<R>(rng);
  p.sinb = xsqrt(R(1) - p.cosb * p.cosb);
  p.cost = -xsqrt(ran<R>(rng));
  p.sint = xsqrt(R(1) - p.cost * p.cost);
  p.phi = (R)kR2p * ran<R>(rng);
  p.cosp = xcos(p.phi);
  p.sinp = xsin(p.phi);
  p.lp = (R)kR2p * ran<R>(rng);
  initp_transform<R>(p);
  p.nub = rep_isrf<R>(m, rng);
  p.i_orig = 4;
  opacset<R>(m, dv, p, p.nub, a);
  const R coslp = xcos(p.lp), sinlp = xsin(p.lp);
  const double zp = (double)p.cosb * a.rmax * 0.999999, rp_ = (double)p.sinb * a.rmax * 0.999999;
  set_pos(p.z, zp);
  set_pos(p.x, rp_ * (double)coslp);
  set_pos(p.y, rp_ * (double)sinlp);
  p.ux = p.sint * p.cosp; p.uy = p.sint * p.sinp; p.uz = p.cost;
  p.ir = m.nrg - 1;
  p.it = locate_dev(m.thetarr, m.ntg, acos((double)p.cosb));
  p.ip = locate_dev(m.phiarr, m.npg, (double)p.lp);
  p.it = p.it < 1 ? 1 : (p.it > m.ntg - 1 ? m.ntg - 1 : p.it);
  p.ip = p.ip < 1 ? 1 : (p.ip > m.npg - 1 ? m.npg - 1 : p.ip);
  tr.add(0, p.ir, p.it, p.ip, 0, 0.0, dval(p.x), dval(p.y), dval(p.z));
  make_rec<R>(rec, p, a, 0, 0, kRecNoPeel);
}

// gasdev (random.f90:140-159): polar Box-Muller pairs, the second deviate of a
// pair returned by the next call.  The reference keeps that deviate in the
// process, so one packet's height uses the deviate its predecessor drew; here
// it is kept in the packet (each packet starts a new pair), which the
// counter-based per-packet streams require.  The deviates are N(0,1) either way.
struct Gauss {
  int have;
  double next;
};
template <class R>
__device__ double gasdev(Gauss& g, Rng& rng) {
  if (g.have) {
    g.have = 0;
    return g.next;
  }
  double v1, v2, rsq;
  do {
    v1 = 2.0 * (double)ran<R>(rng) - 1.0;
    v2 = 2.0 * (double)ran<R>(rng) - 1.0;
    rsq = v1 * v1 + v2 * v2;
  } while (!(rsq < 1.0 && rsq > 0.0));
  const double fac = sqrt(-2.0 * log(rsq) / rsq);
  g.next = v1 * fac;
  g.have = 1;
  return v2 * fac;
}

// Disk accretion packet, newdisktherm.F90:209-251 with initpacc
// (initpacc.f90:24-119), emit_common (emit_common.f90:25-79), emit_gasacc
// (emit_gasacc.f90:26-42) and reemit (reemit.f90:17-34).  The radius is drawn
// from the accretion luminosity profile (w = 1/r with density 1 - sqrt(w),
// in (rddustmin, rmaxdmax)), the azimuth by rantheta, the height as a
// Gaussian of the mass-weighted disk scale height; the point must lie inside
// rmax.  In a cell with thermal disk dust the packet is emitted by a disk
// grain species picked by its V-band opacity (the reference picks with the
// opacities at the previous packet's frequency, a dependence between packets
// that per-packet streams cannot have; with one disk species or one dust file
// the choice is the same) at that species' temperature, and counted as an
// absorption there; otherwise by the gas at the Pringle (1981) accretion
// disk temperature.  The packet starts inside its cell (not on a wall) with
// origin 2 (disk) and an unscattered peel-off.  FP64 set-up in both forms
// (one per accretion packet).  Returns false when no point was found within
// the cap or no species can be picked (the packet is dropped and logged).
template <class R>
__device__ __forceinline__ bool emit_acc(const DevModel& m, const DustView<R>& dv, const DevTallies& t, const RunArgs& a,
                                      Pkt<R>& p, Rng& rng, PeelRec<R>& rec, Tracer& tr) {
  const hc3d_sources& S = a.src;
  p.on_wall = 0;
  p.safe = 0.f;
  p.lrow.key = -1;
  Gauss g{0, 0.0};
  double rp, xp, yp, zp;
  int tries = 0;
  for (;;) {
    rp = 0.0;
    while (rp >= S.rmaxdmax || rp <= S.rddustmin) {
      double winv = (double)ran<R>(rng);
      while ((double)ran<R>(rng) > 1.0 - sqrt(winv)) {
        winv = (double)ran<R>(rng);
        if (++tries > kEmitTries) return false;
      }
      rp = 1.0 / winv;
      if (++tries > kEmitTries) return false;
    }
    // rantheta (random.f90:28-47): a uniform azimuth from a point in the unit disk
    double x, y, r2;
    do {
      x = (double)ran<R>(rng);
      x = x + x - 1.0;
      y = (double)ran<R>(rng);
      y = y + y - 1.0;
      r2 = x * x + y * y;
    } while (r2 > 1.0 || r2 == 0.0);
    const double r = sqrt(r2);
    xp = rp * (x / r);
    yp = rp * (y / r);
    const double h = (0.0 + S.zfac[0] * pow(rp, S.zexp[0])) + S.zfac[1] * pow(rp, S.zexp[1]);
    zp = h * gasdev<R>(g, rng);
    if (zp * zp + rp * rp < S.rmax * S.rmax) break;
    if (++tries > kEmitTries) return false;
  }
  p.sip = R(1); p.sqp = R(0); p.sup = R(0); p.svp = R(0);
  const double rsq = xp * xp + yp * yp + zp * zp;
  const double rtot = sqrt(rsq);
  int ir = locate_dev(m.r2arr, m.nrg, rsq);
  const double cosb = zp / rtot;
  int it = locate_dev(m.costarr, m.ntg, cosb);
  double lp = atan2(yp, xp);
  if (lp < 0.0) lp = lp + kR2p;
  int ip = locate_dev(m.phiarr, m.npg, lp);
  p.ir = ir < 1 ? 1 : (ir > m.nrg - 1 ? m.nrg - 1 : ir);
  p.it = it < 1 ? 1 : (it > m.ntg - 1 ? m.ntg - 1 : it);
  p.ip = ip < 1 ? 1 : (ip > m.npg - 1 ? m.npg - 1 : ip);
  set_pos(p.x, xp);
  set_pos(p.y, yp);
  set_pos(p.z, zp);
  p.cosb = (R)cosb;
  p.lp = (R)lp;
  const int64_t c = cidx(m, p.ir, p.it, p.ip);
  // select_dust over the thermal disk slots (select_dust.f90:16-42)
  const double d0 = __ldg(m.rho4d + 4 * c), d1 = __ldg(m.rho4d + 4 * c + 1);
  int idust2 = -1;
  if (0.0 + d0 + d1 > 0.0) {
    const double xran = (double)ran<R>(rng);
    const double opac = (0.0 + S.kapv[0] * d0) + S.kapv[1] * d1;
    if (opac == 0.0) return false;
    const double eps = (double)1.e-10f;
    double frac = 0.0 + S.kapv[0] * d0 / opac;
    if (xran <= frac + eps) {
      idust2 = 0;
    } else {
      frac = frac + S.kapv[1] * d1 / opac;
      if (xran <= frac + eps) idust2 = 1;
      else return false;
    }
    atomicAdd(t.dbig + c, 1u);
    atomicAdd(t.nabs + (int64_t)idust2 * m.ncell + c, 1ull);
    // reemit at the species' temperature
    p.cost = R(1) - R(2) * ran<R>(rng);
    p.sint = xsqrt(R(1) - p.cost * p.cost);
    p.phi = (R)kR2p * ran<R>(rng);
    p.cosp = xcos(p.phi);
    p.sinp = xsin(p.phi);
    if constexpr (sizeof(R) == 4) p.nub = lucy_freq_mixed(m, p.lrow, c, idust2, rng);
    else p.nub = lucydustfreq<R>(m, __ldg(m.tdust + 4 * c + idust2), idust2, rng);
  } else {
    // gas at the accretion disk temperature (Pringle 1981, eq. 3.23)
    const double t0 = S.gas_num / (S.gas_den * pow(rtot * S.rstar * S.rsun, 3.0));
    const double tgas = pow(t0 * (1.0 - sqrt(1.0 / rtot)), 0.25) / 11605.0;
    p.nub = (R)bbfreq<R>(m, tgas, rng);
    p.cost = R(1) - R(2) * ran<R>(rng);
    p.sint = xsqrt(R(1) - p.cost * p.cost);
    p.phi = (R)kR2p * ran<R>(rng);
    p.cosp = xcos(p.phi);
    p.sinp = xsin(p.phi);
  }
  p.ux = p.sint * p.cosp; p.uy = p.sint * p.sinp; p.uz = p.cost;
  p.i_orig = 2;
  opacset<R>(m, dv, p, p.nub, a);
  tr.add(0, p.ir, p.it, p.ip, 0, 0.0, dval(p.x), dval(p.y), dval(p.z));
  make_rec<R>(rec, p, a, 0, idust2 < 0 ? 0 : idust2);
  return true;
}

// A new packet, by its global id (newdisktherm.F90:207-449: the Fortran
// numbers the accretion packets first, then the hot-spot, stellar and
// external ones).  Returns false when the packet could not be emitted (a
// rejection loop ran out; counted and logged): it is dropped and its peel-off
// record is marked empty.
template <class R>
__device__ __forceinline__ bool emit(const DevModel& m, const DustView<R>& dv, const DevTallies& t, const RunArgs& a,
                                     Pkt<R>& p, Rng& rng, PeelRec<R>& rec, Tracer& tr, Local& L) {
  const int64_t pid = (int64_t)((uint64_t)rng.c2 | ((uint64_t)rng.c3 << 32));
  bool ok = true;
  if (a.ext_illum && pid >= a.n_star) emit_external<R>(m, dv, a, p, rng, rec, tr);
  else if (pid < a.n_acc) ok = emit_acc<R>(m, dv, t, a, p, rng, rec, tr);
  else ok = emit_star<R>(m, dv, a, p, rng, rec, tr, pid < a.n_spot ? 1 : 0);
  if (!ok) {
    L.add(HC3D_CNT_STUCK);
    set_status(a, 2);
    log_fault(t, rng, F_EMIT);
    rec.flags = kRecNoPeel;
  }
  return ok;
}


// tau sample + tauint + outcome, propagate.f90:46-62 (first) and 169-202.
template <class R>
__device__ __forceinline__ int walk(const DevModel& m, const DevTallies& t, const TallyDims& d, const RunArgs& a, Pkt<R>& p, Rng& rng,
                    Flow<R>& f, Local& L, Tracer& tr, bool first) {
  const R tau = -xlog(ran<R>(rng));
  if (!first) {
    f.xpold = p.x; f.ypold = p.y; f.zpold = p.z;
    p.ux = p.sint * p.cosp; p.uy = p.sint * p.sinp; p.uz = p.cost;
  }
  const int pir = p.ir, pit = p.it, pip = p.ip;
  const int st = tauint<R>(m, t, p, tau, L, tr);
  if (st == TI_ESCAPE) {
    tr.add(3, p.ir, p.it, p.ip, 0, 0.0, dval(p.x), dval(p.y), dval(p.z));
    bin_escape<R>(t, d, a, p, dval(f.xpold), dval(f.ypold), dval(f.zpold), f.iflag, f.iscat, L);
    return ST_DONE;
  }
  if (st == TI_STAR) {
    L.add(HC3D_CNT_AFLUX);
    tr.add(4, p.ir, p.it, p.ip, 0, 0.0, dval(p.x), dval(p.y), dval(p.z));
    return ST_DONE;
  }
  if (st == TI_FAULT) {
    L.add(HC3D_CNT_STUCK);
    set_status(a, 1);
    log_fault(t, rng, L.fault);
    return ST_DONE;
  }
  if (!first) {
    if (p.ir != pir || p.it != pit || p.ip != pip) f.iint = 0;
    if (f.iint > a.iintmax || (a.max_interactions > 0 && f.ntot >= a.max_interactions)) {
      atomicAdd(t.killed + cidx(m, p.ir, p.it, p.ip), 1u);
      L.add(HC3D_CNT_ABFLUX);
      tr.add(7, p.ir, p.it, p.ip, 0, 0.0, dval(p.x), dval(p.y), dval(p.z));
      return ST_DONE;
    }
  }
  f.idust2 = select_dust<R>(m, p, rng);
  if (f.idust2 < 0) {
    L.add(HC3D_CNT_STUCK);
    set_status(a, 2);
    log_fault(t, rng, F_SELECT);
    return ST_DONE;
  }
  if (first) L.add(HC3D_CNT_TOT);
  return ST_INTERACT;
}

// Mixed form: the peel-off rays of an event deep in an optically thick cell
// all end inside it.  With s the packet's safe distance (a lower bound on the
// distance to every wall of the cell) and k the peel-masked opacity of the
// cell at the event's frequency, every ray's optical depth at its first wall
// is at least k s; the walk ends a ray whose depth passes taumax = 25
// (peeloff_3d.f90:118) and tallies nothing for it.  When k s exceeds taumax
// by 1 %, and s is large against the FP32 resolution of the ray parameter
// (about 2^-23 |x|), the walk would end every ray at its first wall: no
// record is made and no ray is walked.  The tallies are unchanged; the
// peel-off ray and crossing counters count only the rays walked.
template <class R>
__device__ __forceinline__ bool deep_peel(const DevModel& m, const Pkt<R>& p, int64_t c) {
  if constexpr (sizeof(R) == 4) {
    if (p.safe > 0.f) {
      const float4 q = __ldg(m.rho4p + c);
      const float op = fmaf(p.kapd[0], q.x, fmaf(p.kapd[1], q.y, fmaf(p.kapd[2], q.z, p.kapd[3] * q.w)));
      const float r = fabsf(p.x.hi) + fabsf(p.y.hi) + fabsf(p.z.hi);
      return p.safe * op > 1.01f * (float)kTauMax && p.safe > r * 1.220703125e-4f;
    }
  }
  return false;
}

// One interaction, propagate.f90:70-166: scattering (rec = the state before
// stokes) or absorption and thermal re-emission (rec = the re-emitted packet).
// Returns whether rec was written: only in peeled runs, and not for an event
// whose peel-off rays all end in its cell (deep_peel).
template <class R>
__device__ __forceinline__ bool interact(const DevModel& m, const DustView<R>& dv, const DevTallies& t, const RunArgs& a, Pkt<R>& p, Rng& rng, Flow<R>& f,
                         Local& L, Tracer& tr, PeelRec<R>& rec) {
  const int64_t c = cidx(m, p.ir, p.it, p.ip);
  const int idust2 = f.idust2;
  L.add(HC3D_CNT_EVENTS);
  f.ntot++;
  // issued before the albedo test so that its latency overlaps the draw
  R tave = R(0);
  if constexpr (sizeof(R) == 8) tave = __ldg(m.tdust + 4 * c + idust2);
  bool keep;
  if (ran<R>(rng) <= pick4(p.albedo, idust2)) {  // scattered
    f.iflag = 1; f.iscat++; f.iint++;
    keep = a.ipeel == 1 && !deep_peel<R>(m, p, c);
    if (keep) make_rec<R>(rec, p, a, 1, idust2);
    stokes<R>(p, idust2, rng);
    tr.add(5, p.ir, p.it, p.ip, 0, 0.0, dval(p.x), dval(p.y), dval(p.z));
  } else {  // absorbed + re-emitted (emit_common thermal branch, reemit; small grains: rep_draine, emit_sg)
    const bool sg = (m.sg_mask >> idust2) & 1u;
    atomicAdd((sg ? t.dsg : t.dbig) + c, 1u);
    p.i_orig = ((m.disk_mask >> idust2) & 1u) ? 2 : 3;
    atomicAdd(t.nabs + (int64_t)idust2 * m.ncell + c, 1ull);
    p.sip = R(1); p.sqp = R(0); p.sup = R(0); p.svp = R(0);
    if (sg) {
      // emit_common.f90:31-53: the spectrum row of the cell's mean intensity
      // (row 2, U = 1, in the first iteration), the frequency, then an
      // isotropic direction (emit_sg.f90)
      const int im = a.iter1 ? 2 : __ldg(m.imean + c);
      const double imf = a.iter1 ? 0.0 : __ldg(m.imfract + c);
      p.nub = (R)rep_draine<R>(m, im, imf, rng);
    }
    p.cost = R(1) - R(2) * ran<R>(rng);
    p.sint = xsqrt(R(1) - p.cost * p.cost);
    p.phi = (R)kR2p * ran<R>(rng);
    p.cosp = xcos(p.phi);
    p.sinp = xsin(p.phi);
    if (!sg) {
      if constexpr (sizeof(R) == 4) p.nub = lucy_freq_mixed(m, p.lrow, c, idust2, rng);
      else p.nub = lucydustfreq<R>(m, tave, idust2, rng);
    }
    f.iflag = 0;
    opacset<R>(m, dv, p, p.nub, a);
    keep = a.ipeel == 1 && !deep_peel<R>(m, p, c);
    if (keep) make_rec<R>(rec, p, a, 0, idust2);
    f.iint++;
    tr.add(6, p.ir, p.it, p.ip, 0, 0.0, dval(p.x), dval(p.y), dval(p.z));
  }
  return keep;
}

// every thread of the block calls it, after its last event
__device__ __forceinline__ void flush(const DevTallies& t, Local& L) {
  __syncthreads();
  if (threadIdx.x < 16 && L.sc[threadIdx.x]) atomicAdd(t.counters + threadIdx.x, L.sc[threadIdx.x]);
}

// ---- per-thread form: one packet at a time, its peel-off rays inline --------------
// Used for the trace harness and for runs without peel-off (the Lucy
// iterations), where a packet's history is its only work.
template <class R>
__device__ void run_packet(const DevModel& m, const DustView<R>& dv, const DevTallies& t, const TallyDims& d, const RunArgs& a, Rng& rng,
                           Local& L, Tracer& tr) {
  Pkt<R> p;
  PeelRec<R> rec;
  if (!emit<R>(m, dv, t, a, p, rng, rec, tr, L)) return;
  if (a.ipeel == 1) peel_all<R>(m, t, d, a, rec, L);
  Flow<R> f;
  f.xpold = p.x; f.ypold = p.y; f.zpold = p.z;
  f.iflag = 0; f.iscat = 0; f.iint = 0; f.idust2 = 0; f.ntot = 0;
  int st = walk<R>(m, t, d, a, p, rng, f, L, tr, true);
  while (st == ST_INTERACT) {
    if (interact<R>(m, dv, t, a, p, rng, f, L, tr, rec)) peel_all<R>(m, t, d, a, rec, L);
    st = walk<R>(m, t, d, a, p, rng, f, L, tr, false);
  }
}

template <class R>
__global__ void __launch_bounds__(128) k_transport(DevModel m, DevTallies t, TallyDims d, RunArgs a) {
  extern __shared__ double dust_smem[];
  DustView<R> dv;
  dust_view<R>(m, reinterpret_cast<R*>(dust_smem), dv);
  __shared__ unsigned long long block_counters[16];
  Local L;
  local_init(L, block_counters);
  if (a.inj) {
    // trace harness: one thread per traced packet, draws from the injected list
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < a.np) {
      Rng rng;
      rng_init(rng, a.key0, a.key1, (uint64_t)(a.packet_offset + k));
      rng.inj = a.inj + (size_t)k * a.ninj;
      rng.ninj = a.ninj;
      Tracer tr{reinterpret_cast<TraceRec*>(a.trace) + (size_t)k * a.max_rec, a.max_rec, 0};
      run_packet<R>(m, dv, t, d, a, rng, L, tr);
      a.nrec[k] = tr.n;
    }
  } else {
    Tracer tr{nullptr, 0, 0};
    for (;;) {
      const unsigned long long pid = atomicAdd(a.work, 1ull);
      if (pid >= (unsigned long long)a.np) break;
      Rng rng;
      rng_init(rng, a.key0, a.key1, (uint64_t)(a.packet_offset + (int64_t)pid));
      run_packet<R>(m, dv, t, d, a, rng, L, tr);
    }
  }
  flush(t, L);
}

// ---- batched form: the packets of several models in one persistent launch ------------
// Every thread takes the next packet of the whole batch from one counter,
// finds its model by bisection in the packet ranges, and runs it with that
// model's tables, grid, tallies and run arguments.  Dust tables are read
// from global memory (each model has its own), and the event counters go
// straight to the model's global counters.  A model's packets keep their
// global ids and streams, so a batched run gives the tallies of the model
// run alone.
template <class R>
__global__ void __launch_bounds__(128) k_transport_batch(const BatchItem* items, const int64_t* first, int n,
                                                         unsigned long long* work, int64_t total) {
  __shared__ int64_t sfirst[kMaxBatch + 1];
  for (int i = threadIdx.x; i <= n; i += blockDim.x) sfirst[i] = first[i];
  __syncthreads();
  Tracer tr{nullptr, 0, 0};
  for (;;) {
    const unsigned long long g = atomicAdd(work, 1ull);
    if (g >= (unsigned long long)total) break;
    int lo = 0, hi = n;  // sfirst[lo] <= g < sfirst[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if ((int64_t)g >= sfirst[mid]) lo = mid; else hi = mid;
    }
    const BatchItem& b = items[lo];
    DustView<R> dv;
    dust_view<R>(b.m, nullptr, dv);  // the host set dust_smem = 0: global tables, no barrier
    Local L;
    L.sc = b.t.counters;
    L.fault = 0;
    Rng rng;
    rng_init(rng, b.a.key0, b.a.key1, (uint64_t)(b.a.packet_offset + ((int64_t)g - sfirst[lo])));
    run_packet<R>(b.m, dv, b.t, b.d, b.a, rng, L, tr);
  }
}

// ---- wavefront form: packet pool + peel-off event queue ----------------------------
// Each thread owns one pool slot.  A wave advances every live packet by up
// to E events (taking new packets from the batch as slots free up) and
// appends each event's peel-off record to a queue; k_peel then walks every
// (event, direction) ray of the queue across the whole device.  A packet
// with a very long history therefore costs only its own chain of
// interactions, not that chain times the peel-off rays.
template <class R>
struct Slot {
  Pkt<R> p;
  Flow<R> f;
  uint64_t pid;
  uint32_t c0;
  int left;
  int stage;  // 0 = empty, 1 = an interaction is pending
};

template <class R>
__global__ void __launch_bounds__(128, 3) k_wave(DevModel m, DevTallies t, TallyDims d, RunArgs a, Slot<R>* pool,
                                               PeelRec<R>* queue, unsigned long long* qcount, int E,
                                               unsigned int* alive) {
  extern __shared__ double dust_smem[];
  DustView<R> dv;
  dust_view<R>(m, reinterpret_cast<R*>(dust_smem), dv);
  __shared__ unsigned long long block_counters[16];
  Local L;
  local_init(L, block_counters);
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  Slot<R> s = pool[gid];
  Rng rng;
  rng_init(rng, a.key0, a.key1, s.pid);
  if (s.stage) {
    rng.c0 = s.c0;
    rng.left = s.left;
    if (rng.left > 0) philox(rng.c0 - 1, 0u, rng.c2, rng.c3, rng.k0, rng.k1, rng.b);
  }
  Tracer tr{nullptr, 0, 0};
  // The warp runs its rounds in step (every lane takes part in the ballots).
  // Regeneration threshold: a lane whose packet has ended takes the next one
  // only when at least a.regen lanes of its warp are waiting, or no lane is
  // busy, so that emissions run together instead of beside the other lanes'
  // interactions.  The tallies do not depend on it (each packet's stream is
  // keyed by its id).
  bool done = false;  // the batch has no packet left for this lane
  // Queue slots are reserved a.qchunk at a time, so that the atomic whose
  // result addresses the record is paid once per qchunk events (in the tail
  // of a batch, where a few long histories run alone, it is otherwise a
  // round trip on every event); slots left over are marked empty at the end.
  unsigned long long slot = 0ull, slot_end = 0ull;
  for (int nrec = 0; nrec < E; ++nrec) {
    const unsigned waiting = __ballot_sync(0xffffffffu, s.stage == 0 && !done);
    const unsigned busy = __ballot_sync(0xffffffffu, s.stage != 0);
    if (waiting == 0u && busy == 0u) break;  // warp-uniform
    if (s.stage == 0) {
      if (done || (busy != 0u && __popc(waiting) < a.regen)) continue;
      const unsigned long long pid = atomicAdd(a.work, 1ull);
      if (pid >= (unsigned long long)a.np) {
        done = true;
        continue;
      }
      s.pid = (uint64_t)(a.packet_offset + (int64_t)pid);
      rng_init(rng, a.key0, a.key1, s.pid);
    }
    // The event's record is written field by field into its queue slot as
    // emission or the interaction produces it: the record occupies no
    // registers across the walk.
    if (slot == slot_end) {
      slot = atomicAdd(qcount, (unsigned long long)a.qchunk);
      slot_end = slot + (unsigned long long)a.qchunk;
    }
    PeelRec<R>& rec = queue[slot];
    if (s.stage == 0) {
      ++slot;
      if (!emit<R>(m, dv, t, a, s.p, rng, rec, tr, L)) continue;  // dropped: the lane takes the next packet
      s.f.xpold = s.p.x; s.f.ypold = s.p.y; s.f.zpold = s.p.z;
      s.f.iflag = 0; s.f.iscat = 0; s.f.iint = 0; s.f.idust2 = 0; s.f.ntot = 0;
      s.stage = 2;  // emitted: walk to the first interaction after the record
    } else if (interact<R>(m, dv, t, a, s.p, rng, s.f, L, tr, rec)) {
      ++slot;  // the slot is kept only when the event made a record
    }
    const int st = walk<R>(m, t, d, a, s.p, rng, s.f, L, tr, s.stage == 2);
    s.stage = st == ST_INTERACT ? 1 : 0;
  }
  for (; slot < slot_end; ++slot) queue[slot].flags = kRecNoPeel;
  s.c0 = rng.c0;
  s.left = rng.left;
  pool[gid] = s;
  if (s.stage) atomicAdd(alive, 1u);
  flush(t, L);
}

// Every lane takes its next (event, direction) ray from a counter as soon as
// its current ray ends, so warps stay full although ray lengths differ.
template <class R>
__global__ void __launch_bounds__(256, 3) k_peel(DevModel m, DevTallies t, TallyDims d, RunArgs a,
                                                  const PeelRec<R>* queue, const unsigned long long* qcount,
                                                  unsigned long long* next_ray) {
  __shared__ unsigned long long block_counters[16];
  Local L;
  local_init(L, block_counters);
  const unsigned long long n = *qcount * (unsigned long long)a.npeel;
  for (;;) {
    const unsigned long long i = atomicAdd(next_ray, 1ull);
    if (i >= n) break;
    const unsigned long long e = i / (unsigned)a.npeel;
    const int k = (int)(i - e * (unsigned)a.npeel);
    peel_ray<R>(m, t, d, a, queue[e], k, L);
  }
  flush(t, L);
}


// Set up rays i0 .. i0 + n - 1 (n <= 32) of the warp's staged chunk, one per
// lane, and push those that are walked onto the warp's stack of set-up rays
// (buf, nbuf entries so far).  Every lane of the warp calls it, so the
// set-up -- FP64 closest-approach point and the first crossing of each wall
// family -- runs with the whole warp instead of the few lanes whose ray
// ended; not inlined, so the live walk state of the other lanes stays out of
// its registers.  Returns the number of rays pushed.
static __device__ __noinline__ int prep_rays(const DevModel& m, const PeelRec<float>* st, unsigned e0,
                                             const PeelDir* dirs, unsigned npeel, unsigned i0, unsigned n,
                                             PeelStart* buf, int nbuf) {
  const int lane = threadIdx.x & 31;
  bool ok = false;
  unsigned e = 0;
  int k = 0;
  PeelWalk w;
  if ((unsigned)lane < n) {
    const unsigned i = i0 + (unsigned)lane;
    e = i / npeel;
    k = (int)(i - e * npeel);
    ok = w.start(m, st[e - e0], dirs[k]);
  }
  const unsigned okm = __ballot_sync(0xffffffffu, ok);
  if (ok) w.save(buf[nbuf + __popc(okm & ((1u << lane) - 1u))], e, k);
  __syncwarp();
  return __popc(okm);
}

// Instantiated for two block shapes, between which the autotuner picks:
// 128 threads x 5 blocks per SM and 192 x 3, both held to 96 registers (the
// walk state of a lane, the set-up stack and the 32-ray tally would take
// about 118; the spills are outside the crossing loop).  With one register
// budget the two compile to the same arithmetic, so their tallies agree bit
// for bit.  128 x 5 (20 warps per SM) ran 2 % faster than 256 x 2 at 118
// registers (16 warps); 256 x 3 at 80 registers ran slower.
template <class R, int THREADS, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) k_peel_mixed(DevModel m, DevTallies t, TallyDims d, RunArgs a,
                                                              const PeelRec<R>* queue,
                                                              const unsigned long long* qcount,
                                                              unsigned long long* next_ray) {
  static_assert(sizeof(R) == 4, "the warp-synchronous ray pool is the mixed form");
  __shared__ PeelDir dirs[kMaxPeel];
  __shared__ PeelEsc esc[THREADS / 32][kPeelBuf];
  __shared__ PeelRec<float> stage[THREADS / 32][kPeelStage];
  __shared__ PeelStart prep[THREADS / 32][32];
  static_assert(sizeof(PeelRec<float>) % 4 == 0, "records are staged as 32-bit words");
  for (int k = threadIdx.x; k < a.npeel; k += blockDim.x) dirs[k] = peel_dir(a, k);
  __syncthreads();
  __shared__ unsigned long long block_counters[16];
  Local L;
  local_init(L, block_counters);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  PeelEsc* buf = esc[warp];
  PeelStart* pbuf = prep[warp];
  // ray indices of one wave fit 32 bits: at most 2^22 records x 256 directions
  const unsigned npeel = (unsigned)a.npeel;
  const unsigned n = (unsigned)(*qcount) * npeel;
  // a warp reserves whole records: kPeelStage of them, or fewer when
  // npeel is large, and stages them in shared memory for its lanes
  const unsigned nrec = min((unsigned)kPeelStage, max(1u, (unsigned)kPeelChunk / npeel));
  const unsigned chunk = nrec * npeel;
  PeelRec<float>* st = stage[warp];
  unsigned e0 = 0;  // first record staged
  const int cap = 4 * (m.nrg + m.ntg + m.npg) + 64;
  int nbuf = 0;     // rays parked for the tally
  int nprep = 0;    // rays set up and not yet taken (warp-uniform)
  bool have = false, more = n > 0;
  unsigned rbase = 0, rend = 0;  // rays of the staged chunk not yet set up
  unsigned e = 0;                // the ray of this lane: event e, direction k
  int k = 0;
  PeelWalk w;
  PeelCount pc{0u, 0u, 0u};
  for (;;) {
    const unsigned need = __ballot_sync(0xffffffffu, !have);
    const int nneed = __popc(need);
    // top up the stack of set-up rays, a warp-wide set-up of up to 32 at a time
    while (nprep < nneed && (more || rbase < rend)) {
      if (rbase >= rend) {  // reserve the next chunk of rays for this warp
        unsigned long long b = 0;
        if (lane == 0) b = atomicAdd(next_ray, (unsigned long long)chunk);
        b = __shfl_sync(0xffffffffu, b, 0);
        if (b >= n) {
          more = false;
          break;
        }
        rbase = (unsigned)b;
        rend = b + chunk < n ? (unsigned)b + chunk : n;
        if (rend >= n) more = false;
        // stage the chunk's records (whole records: chunks are multiples of npeel)
        e0 = rbase / npeel;
        const int words = (int)((rend - rbase) / npeel) * (int)(sizeof(PeelRec<float>) / 4);
        const unsigned* src = reinterpret_cast<const unsigned*>(queue + e0);
        unsigned* dst = reinterpret_cast<unsigned*>(st);
        for (int j = lane; j < words; j += 32) dst[j] = __ldg(src + j);
        __syncwarp();
      }
      const unsigned room = 32u - (unsigned)nprep, avail = rend - rbase;
      const unsigned take = room < avail ? room : avail;
      nprep += prep_rays(m, st, e0, dirs, npeel, rbase, take, pbuf, nprep);
      rbase += take;
    }
    if (!have) {  // the lanes without a ray take the top of the stack
      const int idx = __popc(need & lt);
      if (idx < nprep) {
        const PeelStart& q = pbuf[nprep - 1 - idx];
        e = q.e;
        k = q.k;
        w.load(m, q, dirs[k]);
        have = true;
        pc.peels++;
      }
    }
    __syncwarp();
    nprep -= nneed < nprep ? nneed : nprep;
    const bool idle = !__any_sync(0xffffffffu, have) && nprep == 0 && !more && rbase >= rend;
    bool out = false;
    if (have) {
      // up to kPeelSub crossings between refills: the warp-wide refill and
      // parking steps run once per kPeelSub crossings, at the cost of a lane
      // whose ray ends idling for the rest of the round
#pragma unroll 1
      for (int sub = 0; sub < kPeelSub; ++sub) {
        const int s = w.step(m, cap, pc);
        if (s != PeelWalk::GOING) {
          out = s == PeelWalk::OUT;
          have = false;
          break;
        }
      }
      w.flush_tau();  // one FP64 add per round of up to kPeelSub crossings
    }
    // park the rays that left the grid; tally them 32 at a time
    const unsigned outm = __ballot_sync(0xffffffffu, out);
    if (out) {
      PeelEsc& q = buf[nbuf + __popc(outm & lt)];
      q.e = e; q.k = k; q.tsum = (float)w.tsum;
      w.end_point(q.xf, q.yf, q.zf);
    }
    nbuf += __popc(outm);
    // One call site of the tally: a ray's arithmetic does not depend on
    // whether a full buffer or the final drain tallies it, so runs repeat
    // bit for bit.
    if (nbuf >= 32 || (idle && nbuf > 0)) {
      __syncwarp();
      const int take = nbuf < 32 ? nbuf : 32;
      if (lane < take) {
        const PeelEsc q = buf[lane];
        peel_tally_mixed(t, d, a, queue[q.e], dirs[q.k], q.k, q.tsum, q.xf, q.yf, q.zf);
      }
      __syncwarp();
      if (lane < nbuf - take) buf[lane] = buf[lane + take];
      __syncwarp();
      nbuf -= take;
    }
    if (idle && nbuf == 0) break;
  }
  if (pc.peels) L.add(HC3D_CNT_PEELS, pc.peels);
  if (pc.cross) L.add(HC3D_CNT_CROSS_PEEL, pc.cross);
  if (pc.stuck) L.add(HC3D_CNT_PEEL_STUCK, pc.stuck);
  flush(t, L);
}

}  // namespace dev
}  // namespace hc3d
