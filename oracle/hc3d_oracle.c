/*
 * hc3d_oracle.c -- CPU FP64 restatement of the Hochunk3d photon-packet loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle of the GB300
 * library and the timed CPU baseline of bench.py.  Nothing in the product
 * (hochunk3d_gb300/) links, loads or calls it; only tests/, the smoke check
 * of __graft_entry__.py and the cpu_baseline / reference legs of bench.py do.
 *
 * Parity status: UNPINNED at the reference-test level.  The reference ships no
 * tests, golden outputs or runnable build (no Fortran compiler exists here and
 * 14 modules named in Makefile.in are absent), so this restatement is checked
 * only against known answers (closed-form wall roots, the published Philox
 * vectors, analytic escape fractions and phase-function moments) in tests/.
 *
 * It follows the surviving Fortran routine by routine; each function cites
 * the file:line it restates.  The modules that are not shipped (tauint,
 * thetaface, tfinal) are restated from their call sites:
 *   - tauint: the wall machinery of peeloff (peeloff_3d.f90:88-154), stopping
 *     where the integrated optical depth reaches the sampled tau; partial step
 *     ds=(tau-tsum)/opac; tallies dtauabs[id] += kapd(1-albedo)rho*ds and the
 *     path length; escape at ir==nrg; ir==0 ends the packet as absorbed by the
 *     star (the aflux counter of output.F90:378).
 *   - thetaface: cone x^2+y^2 = tan^2(theta) z^2 restricted to the nappe of
 *     the wall's hemisphere; tan2=-1 is the plane z=0, tan2=0 (pole) has no
 *     crossing (gridset.f90:581-604).
 *   - tfinal: the dusttemp fixed point (dusttemp.f90:30-50) with the Lucy
 *     absorbed-path estimator dtauabs in place of the absorption count.
 *   - the small grains' path tally jsg that int_mean reads: ds times the
 *     absorption opacity kappa(nu)/kappa_V (1 - albedo) of one small-grain
 *     species, over the cell's outer radius like the path length.
 *
 * The small-grain inputs (spectra, the species whose opacity weights jsg,
 * the cells' spectrum rows) are module state set by orc_set_sg, read by the
 * runs that follow: one model at a time.
 *
 * Random numbers: Philox4x32-10 streams keyed by (seed, iter, packet id)
 * replace the L'Ecuyer-Cote stream (random.f90:99-118), in the same order of
 * draws as the Fortran, so the GPU kernels can be compared packet by packet.
 */
#include <math.h>
#include <pthread.h>
#include <time.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/hc3d.h"
#include "philox.h"

#define ORC_PI 3.1415926535897932384626433
#define ORC_R2P (2.0 * ORC_PI)
#define ORC_HUGE 1.7976931348623157e308
#define ORC_TAUMAX 25.0 /* peeloff_3d.f90:40 */

/* ------------------------------------------------------------------------ */
/* Inputs, flattened.                                                        */
/* ------------------------------------------------------------------------ */
/* very small grains and PAHs (orc_set_sg) */
typedef struct orc_sg_state {
  int on;                 /* spectra set */
  hc3d_sg_tables sg;      /* cdf and logcdf (nemit,ndraine) Fortran order */
  int jspecies;           /* 0-based species whose opacity weights jsg */
  const int32_t *imean;   /* (nrg,ntg,npg) spectrum rows 1..nemit, NULL before int_mean */
  const double *imfract;  /* (nrg,ntg,npg) */
} orc_sg_state;
static orc_sg_state g_sg;

typedef struct orc_ctx {
  hc3d_dust_tables dt;
  hc3d_grid g;
  int ndg;
  int64_t ncell4; /* nrg*ntg*npg */
  int limb;       /* run parameter limb (0 or 1) */
  double inczeta[145]; /* zetainit partial sums of bbfreq (random.f90:79-97) */
  const orc_sg_state *sg; /* NULL: no small grains */
  int iter1;      /* the first Lucy iteration: small grains use spectrum row 2 */
  double jfac;    /* 1 / (rstar_cm kappa_V) of the jsg species */
} orc_ctx;

/* Tallies: the fixed-point arrays of hc3d_tallies plus FP64 sums of the
 * quantities the reference accumulates in real*8 or real*4. */
typedef struct orc_tallies {
  hc3d_tallies fx;     /* int64 fixed point, same scales as the GPU */
  double *si_d;        /* (nfreq,nmu,nph,nap,no) FP64 Stokes I sums, may be NULL */
  double *ti_d;        /* (nfreq,npeel,nap,no) FP64 peeled I sums, may be NULL */
  double *image_i_d;   /* (npeel,nx,nx) FP64, may be NULL */
  double *dtauabs_d;   /* (nrg,ntg,npg,ndg) FP64 absorbed-path estimator, may be NULL */
  int64_t errors;      /* packets stopped by a geometry or table fault */
  double *image_m2_d;  /* (npeel,nx,nx,4): per pixel the count of peeled rays and the
                          sums of sip^2, sqp^2, sup^2 (variance of the image sums), may be NULL */
} orc_tallies;

typedef struct orc_trace {
  hc3d_trace_rec *recs;
  int max_rec;
  int n;
} orc_trace;

static inline void trace_add(orc_trace *tr, int kind, int ir, int it, int ip, int iface, double tsum,
                             double x, double y, double z) {
  if (!tr || tr->n >= tr->max_rec) return;
  hc3d_trace_rec *r = &tr->recs[tr->n++];
  r->kind = kind; r->ir = ir; r->it = it; r->ip = ip; r->iface = iface; r->pad = 0;
  r->tsum = tsum; r->x = x; r->y = y; r->z = z;
}

/* ------------------------------------------------------------------------ */
/* Packet state: the tts_mod / stokesvar_mod globals one packet touches.     */
/* ------------------------------------------------------------------------ */
typedef struct pkt {
  double xp, yp, zp;
  double ux, uy, uz;
  double cost, sint, cosp, sinp, phi;
  double sip, sqp, sup, svp;
  double nub;
  double cosb, sinb, lp;
  int ir, it, ip;
  int on_wall;
  int i_orig;
  /* opacset outputs for the current frequency (dust_mod) */
  double kapd[HC3D_NDG], albedo[HC3D_NDG], g[HC3D_NDG], pl[HC3D_NDG];
  double g2[HC3D_NDG], g2p1[HC3D_NDG], onemg2[HC3D_NDG], twog[HC3D_NDG];
} pkt;

/* closest_wall module state (closest_wall.f90:7-9) */
typedef struct walls {
  double tn1, tp1, tp2;
  int in1, ip1, ip2;
} walls;

/* ---- nr.f locate (nr.f:131-150) ----------------------------------------- */
static int orc_locate(const double *xx, int n, double x) {
  int jl = 0, ju = n + 1;
  int asc = xx[n - 1] > xx[0];
  while (ju - jl > 1) {
    int jm = (ju + jl) / 2;
    if (asc == (x > xx[jm - 1])) jl = jm; else ju = jm;
  }
  int j = jl;
  if (j == 0 && x == xx[0]) j = 1;
  return j;
}

/* ---- nr.f locate2 (nr.f:152-171): no fix-up at the first element ------- */
static int orc_locate2(const double *xx, int n, double x) {
  int jl = 0, ju = n + 1;
  int asc = xx[n - 1] > xx[0];
  while (ju - jl > 1) {
    int jm = (ju + jl) / 2;
    if (asc == (x > xx[jm - 1])) jl = jm; else ju = jm;
  }
  return jl;
}

/* ---- check.f90:1-30 ----------------------------------------------------- */
static inline double orc_check(double x) {
  if (x > 1.0) return 1.0;
  if (x < -1.0) return -1.0;
  return x;
}

/* ---- opacset, dust.f90:9-80 ---------------------------------------------- */
static void orc_opacset(const orc_ctx *c, pkt *p, double nu, double rstar_cm) {
  const hc3d_dust_tables *d = &c->dt;
  for (int id = 0; id < c->ndg; ++id) {
    const int nl = d->nlambda[id];
    const double *nud = d->nudust + (size_t)id * d->nlammax;
    const double *kap = d->kappad + (size_t)id * d->nlammax;
    const double *alb = d->adust + (size_t)id * d->nlammax;
    const double *gg = d->gdust + (size_t)id * d->nlammax;
    const double *pp = d->pldust + (size_t)id * d->nlammax;
    double g, pl, kappa, albedo;
    if (nu >= nud[0]) {
      g = gg[0]; pl = pp[0]; kappa = kap[0]; albedo = alb[0];
    } else if (nu <= nud[nl - 1]) {
      g = gg[nl - 1]; pl = pp[nl - 1]; kappa = kap[nl - 1]; albedo = alb[nl - 1];
    } else {
      int i0 = 1, i1 = nl;
      while (i1 - i0 > 1) {
        int i = (i1 + i0) / 2;
        if (nu <= nud[i - 1]) i0 = i; else i1 = i;
      }
      double f = (nu - nud[i1 - 1]) / (nud[i0 - 1] - nud[i1 - 1]);
      double fm1 = 1.0 - f;
      g = fm1 * gg[i1 - 1] + f * gg[i0 - 1];
      pl = fm1 * pp[i1 - 1] + f * pp[i0 - 1];
      kappa = fm1 * kap[i1 - 1] + f * kap[i0 - 1];
      albedo = fm1 * alb[i1 - 1] + f * alb[i0 - 1];
    }
    p->g[id] = g; p->pl[id] = pl; p->albedo[id] = albedo;
    p->g2[id] = g * g;
    p->g2p1[id] = p->g2[id] + 1.0;
    p->onemg2[id] = 1.0 - p->g2[id];
    p->twog[id] = 2.0 * g;
    /* newdisktherm.F90:305-311 / propagate.f90:149-151 */
    p->kapd[id] = kappa * rstar_cm * d->kappav[id];
  }
}

/* ---- closest_wall.f90:13-66 ---------------------------------------------- */
static inline void reset_t(walls *w) {
  w->tn1 = -ORC_HUGE; w->tp1 = ORC_HUGE; w->tp2 = ORC_HUGE;
  w->in1 = 0; w->ip1 = 0; w->ip2 = 0;
}
static inline void insert_t(walls *w, double t, int i) {
  if (t < 0.0) {
    if (t > w->tn1) { w->tn1 = t; w->in1 = i; }
  } else {
    if (t < w->tp1) {
      w->tp2 = w->tp1; w->ip2 = w->ip1;
      w->tp1 = t; w->ip1 = i;
    } else if (t < w->tp2) {
      w->tp2 = t; w->ip2 = i;
    }
  }
}
/* returns 0 when no wall was found (the reference stops, closest_wall.f90:65) */
static inline int find_next_wall(const walls *w, int on_wall, double *t, int *i) {
  if (on_wall) {
    if (fabs(w->tn1) < fabs(w->tp1)) { *t = w->tp1; *i = w->ip1; }
    else { *t = w->tp2; *i = w->ip2; }
  } else {
    *t = w->tp1; *i = w->ip1;
  }
  return *t != ORC_HUGE;
}

/* ---- radface.f90:44-62 --------------------------------------------------- */
static inline void radface(walls *w, double ux, double uy, double uz, double x1, double y1, double z1,
                           double R2_1, double R2_2) {
  double bb = 2.0 * (x1 * ux + y1 * uy + uz * z1);
  double cc = x1 * x1 + y1 * y1 + z1 * z1 - R2_1;
  double descr = bb * bb - 4.0 * cc;
  if (descr > 0.0) {
    descr = sqrt(descr);
    insert_t(w, (-bb + descr) * 0.5, 1);
    insert_t(w, (-bb - descr) * 0.5, 1);
  }
  cc = x1 * x1 + y1 * y1 + z1 * z1 - R2_2;
  descr = bb * bb - 4.0 * cc;
  if (descr > 0.0) {
    descr = sqrt(descr);
    insert_t(w, (-bb + descr) * 0.5, 2);
    insert_t(w, (-bb - descr) * 0.5, 2);
  }
}

/* ---- thetaface (module not shipped; restated) ---------------------------
 * One cone wall: tan2 > 0 is the cone x^2+y^2 = tan2*z^2 on the nappe of the
 * wall's hemisphere (hemi = +1 above the midplane, -1 below); tan2 < 0 is the
 * midplane z = 0 (gridset.f90:592-596); tan2 == 0 is a pole, which a ray
 * cannot cross. */
static inline void cone_roots(walls *w, double ux, double uy, double uz, double x, double y, double z,
                              double tan2, double hemi, int id) {
  if (tan2 == 0.0) return;
  if (tan2 < 0.0) {
    if (uz != 0.0) insert_t(w, -z / uz, id);
    return;
  }
  double a = ux * ux + uy * uy - tan2 * uz * uz;
  double b = 2.0 * (x * ux + y * uy - tan2 * z * uz);
  double cq = x * x + y * y - tan2 * z * z;
  if (a == 0.0) {
    if (b != 0.0) {
      double t = -cq / b;
      if ((z + t * uz) * hemi > 0.0) insert_t(w, t, id);
    }
    return;
  }
  double descr = b * b - 4.0 * a * cq;
  if (descr > 0.0) {
    descr = sqrt(descr);
    double t1 = (-b + descr) / (2.0 * a);
    double t2 = (-b - descr) / (2.0 * a);
    if ((z + t1 * uz) * hemi > 0.0) insert_t(w, t1, id);
    if ((z + t2 * uz) * hemi > 0.0) insert_t(w, t2, id);
  }
}
static inline void thetaface(const orc_ctx *c, walls *w, double ux, double uy, double uz, double x, double y,
                             double z, int it) {
  const double *t2 = c->g.tan2arr, *ca = c->g.costarr;
  cone_roots(w, ux, uy, uz, x, y, z, t2[it - 1], ca[it - 1] > 0.0 ? 1.0 : -1.0, 3);
  cone_roots(w, ux, uy, uz, x, y, z, t2[it], ca[it] > 0.0 ? 1.0 : -1.0, 4);
}

/* ---- phiface.f90:48-56 (C=D=0: planes through the z axis) ---------------- */
static inline void phiface(walls *w, double A1, double B1, double A2, double B2, double ux, double uy,
                           double x1, double y1) {
  double denom1 = A1 * ux + B1 * uy;
  if (denom1 != 0.0) insert_t(w, -(A1 * x1 + B1 * y1) / denom1, 5);
  double denom2 = A2 * ux + B2 * uy;
  if (denom2 != 0.0) insert_t(w, -(A2 * x1 + B2 * y1) / denom2, 6);
}

static inline int64_t cidx(const orc_ctx *c, int ir, int it, int ip) {
  return (int64_t)(ir - 1) + (int64_t)c->g.nrg * ((it - 1) + (int64_t)c->g.ntg * (ip - 1));
}
static inline double dens(const orc_ctx *c, int64_t cell, int id) { return c->g.densarr[cell + c->ncell4 * id]; }

/* One step of the shared wall machinery (peeloff_3d.f90:92-115): returns 0
 * when no wall is found. */
static inline int next_wall(const orc_ctx *c, double ux, double uy, double uz, double x, double y, double z,
                            int ir, int it, int ip, int on_wall, double *dt, int *iface) {
  walls w;
  reset_t(&w);
  radface(&w, ux, uy, uz, x, y, z, c->g.r2arr[ir - 1], c->g.r2arr[ir]);
  if (c->g.ntg > 2) thetaface(c, &w, ux, uy, uz, x, y, z, it);
  if (c->g.npg > 2 && c->g.ntg > 2)
    phiface(&w, c->g.aarr[ip - 1], c->g.barr[ip - 1], c->g.aarr[ip], c->g.barr[ip], ux, uy, x, y);
  return find_next_wall(&w, on_wall, dt, iface);
}

/* wall -> index step, peeloff_3d.f90:120-139 */
static inline void step_index(const orc_ctx *c, int iface, int *ir, int *it, int *ip) {
  switch (iface) {
    case 1: (*ir)--; break;
    case 2: (*ir)++; break;
    case 3: (*it)--; break;
    case 4: (*it)++; break;
    case 5: (*ip)--; break;
    case 6: (*ip)++; break;
  }
  if (*ip == 0) *ip = c->g.npg - 1;
  if (*ip == c->g.npg) *ip = 1;
}

static inline int crossing_cap(const orc_ctx *c) { return 4 * (c->g.nrg + c->g.ntg + c->g.npg) + 64; }

static inline int64_t fx_round(double v, double scale) { return llround(v * scale); }

/* ---- tauint (module not shipped; restated, see header) --------------------
 * returns 0 interaction, 1 escape, 2 star, 3 geometry fault */
enum { TI_INTERACT = 0, TI_ESCAPE = 1, TI_STAR = 2, TI_FAULT = 3 };
static int orc_tauint(const orc_ctx *c, pkt *p, double tau, orc_tallies *t, orc_trace *tr) {
  double tsum = 0.0;
  const int cap = crossing_cap(c);
  for (int n = 0;; ++n) {
    if (n > cap) return TI_FAULT;
    if (p->it < 1 || p->it > c->g.ntg - 1 || p->ir < 1 || p->ir > c->g.nrg - 1) return TI_FAULT;
    double dt;
    int iface;
    if (!next_wall(c, p->ux, p->uy, p->uz, p->xp, p->yp, p->zp, p->ir, p->it, p->ip, p->on_wall, &dt, &iface))
      return TI_FAULT;
    const int64_t cell = cidx(c, p->ir, p->it, p->ip);
    double opac = 0.0;
    for (int id = 0; id < c->ndg; ++id) opac += p->kapd[id] * dens(c, cell, id);
    const double dtau = opac * dt;
    const double rout = c->g.rarr[p->ir];
    if (tsum + dtau > tau) {
      const double ds = (tau - tsum) / opac;
      p->xp += ds * p->ux; p->yp += ds * p->uy; p->zp += ds * p->uz;
      p->on_wall = 0;
      for (int id = 0; id < c->ndg; ++id) {
        double rho = dens(c, cell, id);
        if (rho > 0.0) {
          double v = p->kapd[id] * (1.0 - p->albedo[id]) * rho * ds;
          t->fx.dtauabs[cell + c->ncell4 * id] += fx_round(v, t->fx.path_scale);
          if (t->dtauabs_d) t->dtauabs_d[cell + c->ncell4 * id] += v;
        }
      }
      t->fx.jmean[cell] += fx_round(ds / rout, t->fx.path_scale);
      if (c->sg && t->fx.jsg) {
        const int J = c->sg->jspecies;
        t->fx.jsg[cell] += fx_round(ds * (p->kapd[J] * (1.0 - p->albedo[J]) * c->jfac) / rout, t->fx.path_scale);
      }
      t->fx.counters[HC3D_CNT_CROSS_PROP]++;
      trace_add(tr, 2, p->ir, p->it, p->ip, 0, tau, p->xp, p->yp, p->zp);
      return TI_INTERACT;
    }
    for (int id = 0; id < c->ndg; ++id) {
      double rho = dens(c, cell, id);
      if (rho > 0.0) {
        double v = p->kapd[id] * (1.0 - p->albedo[id]) * rho * dt;
        t->fx.dtauabs[cell + c->ncell4 * id] += fx_round(v, t->fx.path_scale);
        if (t->dtauabs_d) t->dtauabs_d[cell + c->ncell4 * id] += v;
      }
    }
    t->fx.jmean[cell] += fx_round(dt / rout, t->fx.path_scale);
    if (c->sg && t->fx.jsg) {
      const int J = c->sg->jspecies;
      t->fx.jsg[cell] += fx_round(dt * (p->kapd[J] * (1.0 - p->albedo[J]) * c->jfac) / rout, t->fx.path_scale);
    }
    t->fx.counters[HC3D_CNT_CROSS_PROP]++;
    tsum += dtau;
    step_index(c, iface, &p->ir, &p->it, &p->ip);
    p->xp += dt * p->ux; p->yp += dt * p->uy; p->zp += dt * p->uz;
    p->on_wall = 1;
    trace_add(tr, 1, p->ir, p->it, p->ip, iface, tsum, p->xp, p->yp, p->zp);
    if (p->ir == c->g.nrg) return TI_ESCAPE;
    if (p->ir == 0) return TI_STAR;
  }
}

/* ---- select_dust.f90:16-42 ------------------------------------------------ */
static int orc_select_dust(const orc_ctx *c, const pkt *p, orc_rng *rng) {
  const double xran = orc_ran(rng);
  const int64_t cell = cidx(c, p->ir, p->it, p->ip);
  double opac = 0.0, frac = 0.0;
  for (int id = 0; id < c->ndg; ++id) opac += p->kapd[id] * dens(c, cell, id);
  if (opac == 0.0) return -1;
  for (int id = 0; id < c->ndg; ++id) {
    frac += p->kapd[id] * dens(c, cell, id) / opac;
    if (xran <= frac + (double)1.e-10f) return id;
  }
  return -1;
}

/* ---- dustmat.f90:40-65 ---------------------------------------------------- */
static inline void orc_dustmat(const pkt *p, int id, double cost, double cost2, double *p1, double *p2,
                               double *p3, double *p4) {
  double temp = p->g2p1[id] - p->twog[id] * cost;
  *p1 = 1.5 * p->onemg2[id] / (2.0 + p->g2[id]) * (1.0 + cost2) / (temp * sqrt(temp));
  *p2 = -p->pl[id] * (*p1) * (1.0 - cost2) / (1.0 + cost2);
  *p3 = (*p1) * 2.0 * cost / (1.0 + cost2);
  *p4 = 0.0;
}

static inline double orc_peak(const pkt *p, int id) {
  double temp, peak;
  if (p->g[id] > 0.0) {
    temp = p->g2p1[id] - p->twog[id];
    peak = 1.5 * p->onemg2[id] / (2.0 + p->g2[id]) * 2.0 / temp / sqrt(temp);
  } else {
    temp = p->g2p1[id] + p->twog[id];
    peak = 1.5 * p->onemg2[id] / (2.0 + p->g2[id]) * 2.0 / temp / sqrt(temp);
  }
  return peak * 1.01;
}

/* ---- stokes.f90:46-388 (idust=1: the dust phase matrix branch) ------------ */
static void orc_stokes(pkt *p, int id, orc_rng *rng) {
  const double costp = p->cost, sintp = p->sint, phip = p->phi;
  double peak = orc_peak(p, id);
  double bmu, cosb2, sinbt, ri1, p1, p2, p3, p4, rprob, a;
  double a11, a12, a13, a21, a22, a23, a24, a31, a32, a33, a34, a42, a43, a44;
  double cosi1 = 0, sini1 = 0, cosi2 = 0, sini2 = 0, cosi3 = 0, sini3 = 0;
  int upper;
  for (;;) {
    bmu = 1.0 - 2.0 * orc_ran(rng);
    cosb2 = bmu * bmu;
    orc_dustmat(p, id, bmu, cosb2, &p1, &p2, &p3, &p4);
    if (fabs(bmu) > 1.0) {
      bmu = bmu > 1.0 ? 1.0 : -1.0;
      cosb2 = 1.0;
    }
    sinbt = sqrt(1.0 - cosb2);
    ri1 = ORC_R2P * orc_ran(rng);
    upper = ri1 > ORC_PI;
    if (upper) {
      double ri3 = ORC_R2P - ri1;
      cosi3 = cos(ri3); sini3 = sin(ri3);
      double sin2i3 = 2.0 * sini3 * cosi3, cos2i3 = 2.0 * cosi3 * cosi3 - 1.0;
      a11 = p1; a12 = p2 * cos2i3; a13 = p2 * sin2i3;
    } else {
      cosi1 = cos(ri1); sini1 = sin(ri1);
      double sin2i1 = 2.0 * sini1 * cosi1, cos2i1 = 2.0 * cosi1 * cosi1 - 1.0;
      a11 = p1; a12 = p2 * cos2i1; a13 = -p2 * sin2i1;
    }
    rprob = (a11 * p->sip + a12 * p->sqp + a13 * p->sup) / p->sip;
    if (rprob > peak) peak = rprob;
    double xran = orc_ran(rng);
    if (!(peak * xran > rprob)) break;
  }
  a = rprob;
  if (bmu == 1.0) return; /* stokes.f90:115-118: direction and Stokes unchanged */
  double ci = upper ? cosi3 : cosi1, si_ = upper ? sini3 : sini1;
  /* double-angle terms of the accepted sample; the bmu=-1 reset below changes
   * only the single-angle terms used by cosdph (stokes.f90:122-130,186-197) */
  const double s2x = 2.0 * si_ * ci, c2x = 2.0 * ci * ci - 1.0;
  if (bmu == -1.0) {
    si_ = 1.0; sini2 = 1.0; ci = 0.0; cosi2 = 0.0;
    p->cost = -costp; p->sint = sintp;
  } else {
    p->cost = costp * bmu + sintp * sinbt * ci;
    if (fabs(p->cost) < 1.0) {
      p->sint = fabs(sqrt(1.0 - p->cost * p->cost));
      sini2 = si_ * sintp / p->sint;
      double bott = p->sint * sinbt;
      cosi2 = costp / bott - p->cost * bmu / bott;
      if (cosi2 >= 1.0) { cosi2 = 1.0; sini2 = 0.0; }
      if (cosi2 <= -1.0) { cosi2 = -1.0; sini2 = 0.0; }
    } else {
      if (p->cost >= 1.0) { p->cost = 1.0; cosi2 = -1.0; }
      if (p->cost <= -1.0) { p->cost = -1.0; cosi2 = 1.0; }
      p->sint = 0.0; sini2 = 0.0;
    }
  }
  double cosdph;
  if (upper) cosdph = -cosi2 * ci + sini2 * si_ * bmu;
  else cosdph = -ci * cosi2 + si_ * sini2 * bmu;
  if (fabs(cosdph) > 1.0) cosdph = cosdph > 1.0 ? 1.0 : -1.0;
  if (upper) p->phi = phip + acos(cosdph);
  else p->phi = phip - acos(cosdph);
  if (p->phi > ORC_R2P) p->phi -= ORC_R2P;
  if (p->phi < 0.0) p->phi += ORC_R2P;
  double sin2i2 = 2.0 * sini2 * cosi2, cos2i2 = 2.0 * cosi2 * cosi2 - 1.0;
  double sin2 = sin2i2 * s2x, cos2 = cos2i2 * c2x;
  double sin2cos1 = sin2i2 * c2x, cos2sin1 = cos2i2 * s2x;
  if (upper) {
    a11 = p1; a12 = p2 * c2x; a13 = p2 * s2x;
    a21 = p2 * cos2i2; a22 = p1 * cos2 - p3 * sin2; a23 = p1 * cos2sin1 + p3 * sin2cos1; a24 = -p4 * sin2i2;
    a31 = -p2 * sin2i2; a32 = -p1 * sin2cos1 - p3 * cos2sin1; a33 = -p1 * sin2 + p3 * cos2; a34 = -p4 * cos2i2;
    a42 = -p4 * s2x; a43 = p4 * c2x; a44 = p3;
  } else {
    a11 = p1; a12 = p2 * c2x; a13 = -p2 * s2x;
    a21 = p2 * cos2i2; a22 = p1 * cos2 - p3 * sin2; a23 = -p1 * cos2sin1 - p3 * sin2cos1; a24 = p4 * sin2i2;
    a31 = p2 * sin2i2; a32 = p1 * sin2cos1 + p3 * cos2sin1; a33 = -p1 * sin2 + p3 * cos2; a34 = -p4 * cos2i2;
    a42 = p4 * s2x; a43 = p4 * c2x; a44 = p3;
  }
  double si = (a11 * p->sip + a12 * p->sqp + a13 * p->sup) / a;
  double sq = (a21 * p->sip + a22 * p->sqp + a23 * p->sup + a24 * p->svp) / a;
  double su = (a31 * p->sip + a32 * p->sqp + a33 * p->sup + a34 * p->svp) / a;
  double sv = (a42 * p->sqp + a43 * p->sup + a44 * p->svp) / a;
  p->sip = si; p->sqp = sq; p->sup = su; p->svp = sv;
  p->cosp = cos(p->phi);
  p->sinp = sin(p->phi);
}

/* ---- findangle3.f90:31-67 -------------------------------------------------
 * The reference passes the module variable phie (set to 0 by reapar) as phi2,
 * not the peel direction's own phi; that is reproduced.  ri1 is left 0 in the
 * two degenerate branches where the Fortran leaves it unset. */
static void orc_findangle3(double cost1, double sint1, double phi1, double cosp1, double sinp1, double cost2,
                           double sint2, double phi2, double cosp2, double sinp2, double *costnew,
                           double *sintnew, double *ri1) {
  *costnew = orc_check(cost1 * cost2 + (sint1 * sint2 * (cosp1 * cosp2 + sinp1 * sinp2)));
  *sintnew = sqrt(1.0 - (*costnew) * (*costnew));
  *ri1 = 0.0;
  if (sint1 > 1.e-8) {
    if (*sintnew > 1.e-8) {
      double cosx = orc_check((cost2 - (cost1 * (*costnew))) / (sint1 * (*sintnew)));
      double x = acos(cosx);
      if (phi2 > phi1) {
        double diff = phi2 - phi1;
        *ri1 = diff > ORC_PI ? x : ORC_R2P - x;
      } else {
        double diff = phi1 - phi2;
        *ri1 = diff > ORC_PI ? ORC_R2P - x : x;
      }
    }
  }
}

/* ---- stokespeel.f90:49-376 ------------------------------------------------
 * cost/sint: peel direction; costp/sintp: incident direction; bmu: cosine of
 * the scattering angle; ri1: rotation angle.  Not normalised by a, so it
 * carries the phase-function weight. */
static void orc_stokespeel(const pkt *p, int id, double *sip, double *sqp, double *sup, double *svp, double cost,
                           double sint, double ri1, double bmu, double costp, double sintp) {
  double cosb2 = bmu * bmu;
  double p1, p2, p3, p4;
  orc_dustmat(p, id, bmu, cosb2, &p1, &p2, &p3, &p4);
  if (fabs(bmu) > 1.0) { bmu = bmu > 1.0 ? 1.0 : -1.0; cosb2 = 1.0; }
  double sinbt = sqrt(1.0 - cosb2);
  int upper = ri1 > ORC_PI;
  double ci, si_;
  if (upper) { double ri3 = ORC_R2P - ri1; ci = cos(ri3); si_ = sin(ri3); }
  else { ci = cos(ri1); si_ = sin(ri1); }
  if (bmu == 1.0) return; /* stokespeel: go to 10, weight unchanged */
  const double s2x = 2.0 * si_ * ci, c2x = 2.0 * ci * ci - 1.0;
  double cosi2 = 0, sini2 = 0;
  if (bmu == -1.0) {
    si_ = 1.0; sini2 = 1.0; ci = 0.0; cosi2 = 0.0;
  } else {
    if (fabs(cost) < 1.0) {
      sini2 = si_ * sintp / sint;
      double bott = sint * sinbt;
      cosi2 = costp / bott - cost * bmu / bott;
      if (cosi2 >= 1.0) { cosi2 = 1.0; sini2 = 0.0; }
      if (cosi2 <= -1.0) { cosi2 = -1.0; sini2 = 0.0; }
    } else {
      if (cost >= 1.0) cosi2 = -1.0;
      if (cost <= -1.0) cosi2 = 1.0;
      sini2 = 0.0;
    }
  }
  double sin2i2 = 2.0 * sini2 * cosi2, cos2i2 = 2.0 * cosi2 * cosi2 - 1.0;
  double sin2 = sin2i2 * s2x, cos2 = cos2i2 * c2x;
  double sin2cos1 = sin2i2 * c2x, cos2sin1 = cos2i2 * s2x;
  double a11, a12, a13, a21, a22, a23, a24, a31, a32, a33, a34, a42, a43, a44;
  if (upper) {
    a11 = p1; a12 = p2 * c2x; a13 = p2 * s2x;
    a21 = p2 * cos2i2; a22 = p1 * cos2 - p3 * sin2; a23 = p1 * cos2sin1 + p3 * sin2cos1; a24 = -p4 * sin2i2;
    a31 = -p2 * sin2i2; a32 = -p1 * sin2cos1 - p3 * cos2sin1; a33 = -p1 * sin2 + p3 * cos2; a34 = -p4 * cos2i2;
    a42 = -p4 * s2x; a43 = p4 * c2x; a44 = p3;
  } else {
    a11 = p1; a12 = p2 * c2x; a13 = -p2 * s2x;
    a21 = p2 * cos2i2; a22 = p1 * cos2 - p3 * sin2; a23 = -p1 * cos2sin1 - p3 * sin2cos1; a24 = p4 * sin2i2;
    a31 = p2 * sin2i2; a32 = p1 * sin2cos1 + p3 * cos2sin1; a33 = -p1 * sin2 + p3 * cos2; a34 = -p4 * cos2i2;
    a42 = p4 * s2x; a43 = p4 * c2x; a44 = p3;
  }
  double si = a11 * (*sip) + a12 * (*sqp) + a13 * (*sup);
  double sq = a21 * (*sip) + a22 * (*sqp) + a23 * (*sup) + a24 * (*svp);
  double su = a31 * (*sip) + a32 * (*sqp) + a33 * (*sup) + a34 * (*svp);
  double sv = a42 * (*sqp) + a43 * (*sup) + a44 * (*svp);
  *sip = si; *sqp = sq; *sup = su; *svp = sv;
}

/* ---- shared SED/peel binning ------------------------------------------------ */
static inline int nu_bin(const hc3d_run_params *rp, double nub) {
  /* propagate.f90:234 / peeloff_3d.f90:219 */
  double lnurat = log(rp->numax / rp->numin);
  int inub = (int)((double)rp->nfreq * log(nub / rp->numin) / lnurat) + 1;
  if (inub < 1) inub = 1;
  if (inub > rp->nfreq) inub = rp->nfreq;
  return inub;
}

/* ---- peeloff_3d.f90:52-286 (one observer direction) ----------------------- */
static void orc_peeloff(const orc_ctx *c, const hc3d_run_params *rp, const pkt *p, double sip_in, int iflag,
                        int idust2, int peelid, orc_tallies *t) {
  double xp1 = p->xp, yp1 = p->yp, zp1 = p->zp;
  int ir = p->ir, it = p->it, ip = p->ip;
  int on_wall = p->on_wall;
  double sip = sip_in, sqp = p->sqp, sup = p->sup, svp = p->svp;
  const double coste = cos(rp->thete[peelid]), sinte = sin(rp->thete[peelid]);
  const double cospe = cos(rp->phie[peelid]), sinpe = sin(rp->phie[peelid]);
  const double ux1 = sinte * cospe, uy1 = sinte * sinpe, uz1 = coste;
  t->fx.counters[HC3D_CNT_PEELS]++;
  if (on_wall) {
    double rsq1 = xp1 * xp1 + yp1 * yp1 + zp1 * zp1;
    int inner_wall = fabs(rsq1 - c->g.r2arr[ir - 1]) < fabs(rsq1 - c->g.r2arr[ir]);
    int outwards = ux1 * xp1 + uy1 * yp1 + uz1 * zp1 > 0.0;
    if (inner_wall && !outwards) {
      if (ir == 1) return;
      ir = ir - 1;
    }
    if (!inner_wall && outwards) ir = ir + 1;
  }
  const double tsub = c->dt.tsub / 11605.0;
  double tsum = 0.0;
  const int cap = crossing_cap(c);
  for (int n = 0;; ++n) {
    if (n > cap || it < 1 || it > c->g.ntg - 1 || ir < 1 || ir > c->g.nrg - 1) {
      t->fx.counters[HC3D_CNT_PEEL_STUCK]++;
      return;
    }
    double dt;
    int iface;
    if (!next_wall(c, ux1, uy1, uz1, xp1, yp1, zp1, ir, it, ip, on_wall, &dt, &iface)) {
      t->fx.counters[HC3D_CNT_PEEL_STUCK]++;
      return;
    }
    const int64_t cell = cidx(c, ir, it, ip);
    double opac = 0.0;
    for (int id = 0; id < c->ndg; ++id)
      if (c->g.tdust[cell + c->ncell4 * id] < tsub) opac += p->kapd[id] * dens(c, cell, id);
    tsum += opac * dt;
    t->fx.counters[HC3D_CNT_CROSS_PEEL]++;
    if (tsum > ORC_TAUMAX) return;
    step_index(c, iface, &ir, &it, &ip);
    xp1 += dt * ux1; yp1 += dt * uy1; zp1 += dt * uz1;
    on_wall = 1;
    if (ir == c->g.nrg) break;
    if (ir == 0) return;
  }
  const double factor = exp(-tsum);
  sip *= factor; sqp *= factor; sup *= factor; svp *= factor;
  if (iflag == 1) {
    double bmu, sinbm, ri1;
    /* phi2 is the module phie = 0 (reapar.f90:500), see orc_findangle3 */
    orc_findangle3(p->cost, p->sint, p->phi, p->cosp, p->sinp, coste, sinte, 0.0, cospe, sinpe, &bmu, &sinbm, &ri1);
    orc_stokespeel(p, idust2, &sip, &sqp, &sup, &svp, coste, sinte, ri1, bmu, p->cost, p->sint);
  }
  const double yimage = zp1 * sinte - yp1 * coste * sinpe - xp1 * coste * cospe;
  const double ximage = yp1 * cospe - xp1 * sinpe;
  const double fractxh = 2.0 * rp->rmaxi / (double)rp->nxhst;
  const int ix = (int)((ximage + rp->rmaxi) / fractxh) + 1;
  const int iy = (int)((yimage + rp->rmaxi) / fractxh) + 1;
  const double rho2 = ximage * ximage + yimage * yimage;
  const int inub = nu_bin(rp, p->nub);
  const int i_inter = iflag == 1 ? 2 : (p->i_orig == 1 ? 1 : 3);
  const int indx[3] = {1, 1 + p->i_orig, 5 + i_inter};
  const double ss = t->fx.stokes_scale, sq = t->fx.square_scale;
  for (int ia = 1; ia <= rp->nap; ++ia) {
    if (rho2 < rp->aperture2[ia - 1]) {
      for (int k = 0; k < 3; ++k) {
        int64_t b = (int64_t)(inub - 1) + (int64_t)rp->nfreq * ((peelid) + (int64_t)rp->npeel * ((ia - 1) + (int64_t)rp->nap * (indx[k] - 1)));
        t->fx.ti[b] += fx_round(sip, ss); t->fx.tq[b] += fx_round(sqp, ss);
        t->fx.tu[b] += fx_round(sup, ss); t->fx.tv[b] += fx_round(svp, ss);
        t->fx.ti2[b] += fx_round(sip * sip, sq); t->fx.tq2[b] += fx_round(sqp * sqp, sq);
        t->fx.tu2[b] += fx_round(sup * sup, sq); t->fx.tv2[b] += fx_round(svp * svp, sq);
        t->fx.numt[b] += 1;
        if (t->ti_d) t->ti_d[b] += sip;
      }
    }
  }
  if (rp->image && ix <= rp->nxhst && iy <= rp->nxhst && ix > 0 && iy > 0) {
    int64_t b = (int64_t)peelid + (int64_t)rp->npeel * ((ix - 1) + (int64_t)rp->nxhst * (iy - 1));
    t->fx.image_i[b] += fx_round(sip, ss); t->fx.image_q[b] += fx_round(sqp, ss);
    t->fx.image_u[b] += fx_round(sup, ss); t->fx.image_v[b] += fx_round(svp, ss);
    if (rp->imcube && t->fx.image_m_i) {
      /* peeloff_3d.f90:271-282: image_m_i(peelid,ix,iy,inub,indx), image_m_q/u/v(peelid,ix,iy,inub) */
      const int64_t nim = (int64_t)rp->npeel * rp->nxhst * rp->nxhst, nc = nim * rp->nfreq;
      const int64_t bc = b + nim * (int64_t)(inub - 1);
      for (int k = 0; k < 3; ++k) t->fx.image_m_i[bc + nc * (indx[k] - 1)] += fx_round(sip, ss);
      t->fx.image_m_q[bc] += fx_round(sqp, ss);
      t->fx.image_m_u[bc] += fx_round(sup, ss);
      t->fx.image_m_v[bc] += fx_round(svp, ss);
    }
    if (t->image_i_d) t->image_i_d[b] += sip;
    if (t->image_m2_d) {
      const int64_t n = (int64_t)rp->npeel * rp->nxhst * rp->nxhst;
      t->image_m2_d[b] += 1.0;
      t->image_m2_d[b + n] += sip * sip;
      t->image_m2_d[b + 2 * n] += sqp * sqp;
      t->image_m2_d[b + 3 * n] += sup * sup;
    }
  }
}

/* ---- lucydustfreq.f90:19-157 ---------------------------------------------- */
static double orc_lucydustfreq(const orc_ctx *c, double T0, int id, orc_rng *rng) {
  const hc3d_dust_tables *d = &c->dt;
  const int nT = d->nT, nnu = d->nnu;
  const double *lTint = d->lTint, *nuint = d->nuint;
  const double *K = d->kapBint + (size_t)id * nT * nnu;
#define KB(j, i) K[(size_t)((j) - 1) + (size_t)nT * ((i) - 1)]
  double lT0 = log(T0);
  double xi = orc_ran(rng);
  int j = (int)((double)(nT - 1) * (lT0 - lTint[0]) / (lTint[nT - 1] - lTint[0])) + 1;
  if (j < 1) j = 1; /* the Fortran reports and reads out of bounds; clamped here */
  if (j > nT - 1) j = nT - 1;
  double f = (lT0 - lTint[j - 1]) / (lTint[j] - lTint[j - 1]);
  if (f < 0.0) f = 0.0;
  if (f > 1.0) f = 1.0;
  int i0 = 1, i1 = nnu;
  double P0 = (1.0 - f) * KB(j, i0) + f * KB(j + 1, i0);
  if (xi < P0) {
    if (P0 > 0.0) return T0 * xi * nuint[0] / P0;
    return T0 * nuint[0];
  }
  double P1 = (1.0 - f) * KB(j, i1) + f * KB(j + 1, i1);
  if (P1 > 1.0) P1 = 1.0;
  if (xi >= P1) {
    if (P1 < 1.0) {
      if (xi < 1.0) return T0 * nuint[nnu - 1] * (1.0 - P1) / (1.0 - xi);
      return T0 * nuint[nnu - 1];
    }
    return T0 * nuint[nnu - 1];
  }
  double P = 0.0;
  while (i1 - i0 > 1) {
    int i = (i0 + i1) / 2;
    P = (1.0 - f) * KB(j, i) + f * KB(j + 1, i);
    if (P > 1.0) P = 1.0;
    if (P < P0) { P0 = P; i0 = i; }
    if (P > P1) { P1 = P; i1 = 1; }
    if (P > xi) { i1 = i; P1 = P; }
    else { i0 = i; P0 = P; }
  }
  if (xi < P0) f = 0.0;
  else if (xi > P1) f = 1.0;
  else if (P0 <= 0.0) f = 0.5;
  else if (P1 <= 0.0) { /* f keeps its value, as in the Fortran */ }
  else if (xi <= 0.0) { }
  else f = log(xi / P0) / log(P1 / P0);
  return T0 * nuint[i0 - 1] * pow(nuint[i1 - 1] / nuint[i0 - 1], f);
#undef KB
}

/* ---- atmosfreq, starbarb.f90:120-156 -------------------------------------- */
static double orc_atmosfreq(const orc_ctx *c, orc_rng *rng) {
  const hc3d_dust_tables *d = &c->dt;
  double xi = orc_ran(rng);
  int i = orc_locate2(d->hnuint, d->nhnu, xi);
  if (i < 1) i = 1; /* hnuint(1)=0 < xi always; guard */
  if (i > d->nhnu - 1) i = d->nhnu - 1;
  if (i > 1) {
    double logatm = d->lognu[i - 1] + (d->lognu[i] - d->lognu[i - 1]) * (log10(xi) - d->loghnu[i - 1]) /
                                          (d->loghnu[i] - d->loghnu[i - 1]);
    return pow(10.0, logatm);
  }
  return d->atmosnu[i - 1] + (d->atmosnu[i] - d->atmosnu[i - 1]) * (xi - d->hnuint[i - 1]) /
                                 (d->hnuint[i] - d->hnuint[i - 1]);
}

/* ---- initp_transform, initp_common.f90:31-94 ----------------------------- */
static void orc_initp_transform(pkt *p) {
  if (fabs(p->cosb) < 0.9999999) {
    double costi = p->cost * p->cosb - p->sint * p->sinb * p->cosp;
    if (fabs(costi) > 1.0) {
      if (costi > 1.0) costi = 1.0;
      if (p->cost < -1.0) costi = -1.0; /* as written in initp_common.f90:45 */
    }
    double sinti = sqrt(1.0 - costi * costi);
    double phinew;
    if (sinti > 0.0000001) {
      double cospn = (p->cost - costi * p->cosb) / (sinti * p->sinb);
      if (fabs(cospn) > 1.0) cospn = cospn < 0.0 ? -1.0 : 1.0;
      if (p->phi < ORC_PI) {
        phinew = acos(cospn);
        if (phinew > ORC_PI) phinew = ORC_PI;
      } else {
        phinew = ORC_R2P - acos(cospn);
        if (phinew < ORC_PI) phinew = ORC_PI;
      }
    } else {
      phinew = 0.0;
    }
    p->phi = phinew; p->cost = costi; p->sint = sinti;
  } else {
    if (p->cosb < 0.0) p->cost = -p->cost;
  }
  p->phi = p->phi + p->lp;
  if (p->phi > ORC_R2P) p->phi -= ORC_R2P;
  if (p->phi < 0.0) p->phi += ORC_R2P;
  p->sinp = sin(p->phi);
  p->cosp = cos(p->phi);
}

/* ---- darkening, samptabl.f90:29-65 (delmu = 1/ntab of tabl_mod) --------- */
static double orc_darkening(const orc_ctx *c, double xi) {
  const hc3d_dust_tables *d = &c->dt;
  int n = orc_locate(d->limb_prob, d->ntab, xi);
  if (n < 1) n = 1;
  if (n > d->ntab - 1) n = d->ntab - 1;
  const double delmu = 1.0 / (double)d->ntab;
  return d->limb_xmu[n] - (d->limb_prob[n] - xi) / (d->limb_prob[n] - d->limb_prob[n - 1]) * delmu;
}

/* ---- bbfreq, random.f90:49-77 ----------------------------------------------- */
static double orc_bbfreq(const orc_ctx *c, double teff, orc_rng *rng) {
  const double z0 = c->inczeta[144] * orc_ran(rng);
  const double z1 = orc_ran(rng), z2 = orc_ran(rng), z3 = orc_ran(rng), z4 = orc_ran(rng);
  int i = 1;
  while (i < 145 && z0 > c->inczeta[i - 1]) i++;
  return -log(z1 * z2 * z3 * z4) * teff / (double)i;
}

#define ORC_EMIT_TRIES (1 << 24) /* cap of the emission rejection loops (the GPU library's) */

/* ---- initpspot, initpspot.f90:33-160, with initp_sample (initp_common.f90:1-29)
 * and the X-ray half of the hot-spot packets (newdisktherm.F90:270-273).
 * spotph: 1 for a hot-spot packet, 0 for a stellar one; *spot_out (when not
 * NULL) receives 1 when the packet radiates at the shock temperature.
 * Returns 0 when the spot rejection ran past the cap. */
static int orc_initpspot(const orc_ctx *c, const hc3d_run_params *rp, pkt *p, orc_rng *rng, int spotph,
                         int *spot_out) {
  const hc3d_sources *S = rp->sources;
  const int spots = S && S->ispot;
  p->sip = 1.0; p->sqp = 0.0; p->sup = 0.0; p->svp = 0.0;
  for (int tries = 0;; tries++) {
    for (;;) {
      double xran = orc_ran(rng);
      p->cosb = 1.0 - 2.0 * xran;
      p->sinb = sqrt(1.0 - p->cosb * p->cosb);
      if (p->cosb != 0.0 && fabs(p->cosb) < 1.0) break;
    }
    p->lp = ORC_R2P * orc_ran(rng);
    if (!spots) break;
    const double cphi = cos(p->lp), sphi = sin(p->lp), sthet = p->sinb, cthet = p->cosb;
    const double dotsp1 = S->spot1[0] * sthet * cphi + S->spot1[1] * sthet * sphi + S->spot1[2] * cthet;
    const double dotsp2 = S->spot2[0] * sthet * cphi + S->spot2[1] * sthet * sphi + S->spot2[2] * cthet;
    if (spotph == 1 && (S->nspot == 1 ? dotsp1 < S->csprad : (dotsp1 < S->csprad && dotsp2 < S->csprad))) {
      if (tries >= ORC_EMIT_TRIES) return 0;
      continue;
    }
    if (S->fspot < 1.0) {
      double dellon = p->lp < ORC_PI ? p->lp : ORC_R2P - p->lp;
      if (S->spot1[2] * p->cosb + S->spot1[3] * p->sinb * cos(dellon) > S->csprad) spotph = 1;
      if (S->nspot == 2) {
        dellon = p->lp < ORC_PI ? ORC_PI - p->lp : p->lp - ORC_PI;
        if (S->spot2[2] * p->cosb + S->spot2[3] * p->sinb * cos(dellon) > S->csprad) spotph = 1;
      }
    }
    break;
  }
  /* initp_sample: uniform disk (limb = 0) or the Eddington table (darkening) */
  p->cost = c->limb ? orc_darkening(c, orc_ran(rng)) : sqrt(orc_ran(rng));
  p->sint = sqrt(1.0 - p->cost * p->cost);
  p->phi = ORC_R2P * orc_ran(rng);
  p->cosp = cos(p->phi);
  p->sinp = sin(p->phi);
  orc_initp_transform(p);
  /* initpspot.f90:146-160: the hot-spot packets (iplanckst = 1) and the
   * stellar packets that fall in a spot when fspot < 1 radiate at tshock; the
   * other stellar packets take the stellar spectrum (atmosfreq) */
  if (spot_out) *spot_out = spotph;
  if (spotph) {
    p->nub = orc_bbfreq(c, S->tshock, rng);
    if (orc_ran(rng) < 0.5) p->nub = 1.2398 / 0.06 + orc_ran(rng) * (1.2398 / 0.015 - 1.2398 / 0.06);
  } else {
    p->nub = orc_atmosfreq(c, rng);
  }
  return 1;
}

/* ---- rep_isrf, rep_isrf.f90:1-41 ------------------------------------------ */
static double orc_rep_isrf(const orc_ctx *c, orc_rng *rng) {
  const hc3d_dust_tables *d = &c->dt;
  const double xran = orc_ran(rng);
  const int n = d->nisrf;
  int i = orc_locate(d->isrf_cdf, n, xran);
  if (i == n) i = n - 1;
  if (i == 0) i = 1;
  const double logfreq = d->isrf_logfreq[i - 1] + (log10(xran) - d->isrf_logcdf[i - 1]) /
                                                      (d->isrf_logcdf[i] - d->isrf_logcdf[i - 1]) *
                                                      (d->isrf_logfreq[i] - d->isrf_logfreq[i - 1]);
  return pow(10.0, logfreq);
}

/* ---- initpout, initpout.f90:3-66 ----------------------------------------- */
static void orc_initpout(const orc_ctx *c, pkt *p, orc_rng *rng) {
  p->sip = 1.0; p->sqp = 0.0; p->sup = 0.0; p->svp = 0.0;
  p->cosb = 1.0 - 2.0 * orc_ran(rng);
  p->sinb = sqrt(1.0 - p->cosb * p->cosb);
  p->cost = -sqrt(orc_ran(rng));
  p->sint = sqrt(1.0 - p->cost * p->cost);
  p->phi = ORC_R2P * orc_ran(rng);
  p->cosp = cos(p->phi);
  p->sinp = sin(p->phi);
  p->lp = ORC_R2P * orc_ran(rng);
  orc_initp_transform(p);
  p->nub = orc_rep_isrf(c, rng);
}

/* ---- propagate.f90:27-319 ------------------------------------------------- */
static void orc_bin_escape(const orc_ctx *c, const hc3d_run_params *rp, const pkt *p, double xpold, double ypold,
                           double zpold, int iflag, int iscat, orc_tallies *t) {
  (void)c;
  int it = (int)((double)rp->nmu * (1.0 - p->cost) / 2.0) + 1;
  if (it > rp->nmu) it = rp->nmu; /* cost = -1 exactly; the Fortran writes one past the end */
  if (it < 1) it = 1;
  double phi = p->phi;
  if (phi < 0.0) phi += ORC_R2P;
  int ip = (int)((double)rp->nph * phi / ORC_R2P) + 1;
  if (ip > rp->nph) ip = rp->nph;
  if (ip < 1) ip = 1;
  const double dmu = 2.0 / (double)rp->nmu;
  const double u = 1.0 - dmu * ((double)it - 0.5);
  const double sini = sqrt(1.0 - u * u);
  const double x = ypold * p->cosp - xpold * p->sinp;
  const double y = zpold * sini - ypold * u * p->sinp - xpold * u * p->cosp;
  const double rho2 = x * x + y * y;
  if (rho2 < rp->aperture2[rp->nap - 1] * 1.0001) {
    t->fx.counters[HC3D_CNT_FLUX]++;
    if (iflag == 1) {
      t->fx.counters[HC3D_CNT_SFLUX]++;
      t->fx.counters[HC3D_CNT_NSCAT] += iscat;
    }
  }
  const int inub = nu_bin(rp, p->nub);
  const int i_inter = iflag == 1 ? 2 : (p->i_orig == 1 ? 1 : 3);
  const int indx[3] = {1, 1 + p->i_orig, 5 + i_inter};
  const double ss = t->fx.stokes_scale, sq = t->fx.square_scale;
  for (int ia = 1; ia <= rp->nap; ++ia) {
    if (rho2 < rp->aperture2[ia - 1]) {
      if (!(iflag == 0 && p->i_orig == 4)) {
        for (int k = 0; k < 3; ++k) {
          int64_t b = (int64_t)(inub - 1) +
                      (int64_t)rp->nfreq * ((it - 1) + (int64_t)rp->nmu * ((ip - 1) + (int64_t)rp->nph * ((ia - 1) + (int64_t)rp->nap * (indx[k] - 1))));
          t->fx.si[b] += fx_round(p->sip, ss); t->fx.sq[b] += fx_round(p->sqp, ss);
          t->fx.su[b] += fx_round(p->sup, ss); t->fx.sv[b] += fx_round(p->svp, ss);
          t->fx.si2[b] += fx_round(p->sip * p->sip, sq); t->fx.sq2[b] += fx_round(p->sqp * p->sqp, sq);
          t->fx.su2[b] += fx_round(p->sup * p->sup, sq); t->fx.sv2[b] += fx_round(p->svp * p->svp, sq);
          t->fx.nums[b] += 1;
          if (t->si_d) t->si_d[b] += p->sip;
        }
      }
    }
  }
  if (!(iflag == 0 && p->i_orig == 4)) t->fx.counters[HC3D_CNT_SUMSUB] += fx_round(p->sip, ss);
  t->fx.counters[HC3D_CNT_SUMALL] += fx_round(p->sip, ss);
  if (iflag == 1) t->fx.counters[HC3D_CNT_SCOUNT]++;
  t->fx.counters[HC3D_CNT_ESCAPED]++;
}

/* ---- rep_draine.f90:1-65 and locate3.f90 ------------------------------------
 * The re-emission frequency of a small grain: bin of the uniform xran in the
 * cumulative spectrum of row jm (locate3: bisection over row jm of cdf_d, no
 * fix-up at the first element; clamped to 1..ndraine-1), log10 cdf against
 * log10 nu interpolation, and the same in row jm + 1 mixed by jmf. */
static int orc_locate3(const double *xx, int n1, int n2, int n3, double x) {
  int jl = 0, ju = n2 + 1;
  const int asc = xx[(n3 - 1) + (size_t)n1 * (n2 - 1)] > xx[n3 - 1];
  while (ju - jl > 1) {
    const int jm = (ju + jl) / 2;
    if (asc == (x > xx[(n3 - 1) + (size_t)n1 * (jm - 1)])) jl = jm; else ju = jm;
  }
  return jl;
}

static double orc_draine_logfreq(const hc3d_sg_tables *s, int jm, double xran) {
  int ifreq = orc_locate3(s->cdf, s->nemit, s->ndraine, jm, xran);
  if (ifreq == s->ndraine) ifreq = s->ndraine - 1;
  if (ifreq == 0) ifreq = 1;
  const double l0 = s->logcdf[(jm - 1) + (size_t)s->nemit * (ifreq - 1)];
  const double l1 = s->logcdf[(jm - 1) + (size_t)s->nemit * ifreq];
  return (log10(xran) - l0) / (l1 - l0) * (s->logfreq[ifreq] - s->logfreq[ifreq - 1]) + s->logfreq[ifreq - 1];
}

static double orc_rep_draine(const hc3d_sg_tables *s, int jm, double jmf, double xran) {
  const double lf1 = orc_draine_logfreq(s, jm, xran);
  double lf = lf1;
  if (jm + 1 <= s->nemit) lf = lf1 + jmf * (orc_draine_logfreq(s, jm + 1, xran) - lf1);
  return pow(10.0, lf);
}

static void orc_propagate(const orc_ctx *c, const hc3d_run_params *rp, pkt *p, orc_rng *rng, orc_tallies *t,
                          orc_trace *tr) {
  double xpold = p->xp, ypold = p->yp, zpold = p->zp;
  int iflag = 0, iscat = 0, iint = 0;
  int64_t ntot = 0;
  double tau = -log(orc_ran(rng));
  int st = orc_tauint(c, p, tau, t, tr);
  if (st == TI_ESCAPE) goto bin;
  if (st == TI_STAR) { t->fx.counters[HC3D_CNT_AFLUX]++; trace_add(tr, 4, p->ir, p->it, p->ip, 0, 0, p->xp, p->yp, p->zp); return; }
  if (st == TI_FAULT) { t->fx.counters[HC3D_CNT_STUCK]++; t->errors++; return; }
  int idust2 = orc_select_dust(c, p, rng);
  if (idust2 < 0) { t->fx.counters[HC3D_CNT_STUCK]++; t->errors++; return; }
  t->fx.counters[HC3D_CNT_TOT]++;
  for (;;) {
    const int64_t cell = cidx(c, p->ir, p->it, p->ip);
    t->fx.counters[HC3D_CNT_EVENTS]++;
    ntot++;
    if (orc_ran(rng) <= p->albedo[idust2]) { /* scattered */
      iflag = 1; iscat++; iint++;
      if (rp->ipeel == 1)
        for (int k = 0; k < rp->npeel; ++k) orc_peeloff(c, rp, p, p->sip, 1, idust2, k, t);
      orc_stokes(p, idust2, rng);
      trace_add(tr, 5, p->ir, p->it, p->ip, 0, 0, p->xp, p->yp, p->zp);
    } else { /* absorbed + re-emitted */
      const int sg = idust2 >= 4; /* is_sg, grid_mod.f90:18 */
      if (sg) { if (t->fx.dsg) t->fx.dsg[cell]++; }
      else t->fx.dbig[cell]++;
      p->i_orig = (idust2 == 0 || idust2 == 1 || idust2 == 4 || idust2 == 5) ? 2 : 3;
      t->fx.nabs[cell + c->ncell4 * idust2] += 1;
      p->sip = 1.0; p->sqp = 0.0; p->sup = 0.0; p->svp = 0.0;
      if (sg) {
        /* emit_common.f90:31-53: the spectrum row of the cell (row 2 in the
         * first iteration), rep_draine, then emit_sg's isotropic direction */
        const int im = c->iter1 ? 2 : c->sg->imean[cell];
        const double imf = c->iter1 ? 0.0 : c->sg->imfract[cell];
        p->nub = orc_rep_draine(&c->sg->sg, im, imf, orc_ran(rng));
        p->cost = 1.0 - 2.0 * orc_ran(rng);
        p->sint = sqrt(1.0 - p->cost * p->cost);
        p->phi = ORC_R2P * orc_ran(rng);
        p->cosp = cos(p->phi);
        p->sinp = sin(p->phi);
      } else {
        /* emit_common.f90:54-79 thermal branch with ilucy=1, reemit.f90:17-34 */
        const double tave = c->g.tdust[cell + c->ncell4 * idust2];
        p->cost = 1.0 - 2.0 * orc_ran(rng);
        p->sint = sqrt(1.0 - p->cost * p->cost);
        p->phi = ORC_R2P * orc_ran(rng);
        p->cosp = cos(p->phi);
        p->sinp = sin(p->phi);
        p->nub = orc_lucydustfreq(c, tave, idust2, rng);
      }
      iflag = 0;
      orc_opacset(c, p, p->nub, rp->rstar_cm);
      if (rp->ipeel == 1)
        for (int k = 0; k < rp->npeel; ++k) orc_peeloff(c, rp, p, p->sip, 0, idust2, k, t);
      iint++;
      trace_add(tr, 6, p->ir, p->it, p->ip, 0, 0, p->xp, p->yp, p->zp);
    }
    tau = -log(orc_ran(rng));
    xpold = p->xp; ypold = p->yp; zpold = p->zp;
    p->ux = p->sint * p->cosp; p->uy = p->sint * p->sinp; p->uz = p->cost;
    const int pir = p->ir, pit = p->it, pip = p->ip;
    st = orc_tauint(c, p, tau, t, tr);
    if (st == TI_ESCAPE) break;
    if (st == TI_STAR) { t->fx.counters[HC3D_CNT_AFLUX]++; trace_add(tr, 4, p->ir, p->it, p->ip, 0, 0, p->xp, p->yp, p->zp); return; }
    if (st == TI_FAULT) { t->fx.counters[HC3D_CNT_STUCK]++; t->errors++; return; }
    if (p->ir != pir || p->it != pit || p->ip != pip) iint = 0;
    if (iint > rp->iintmax || (rp->max_interactions > 0 && ntot >= rp->max_interactions)) {
      t->fx.killed[cidx(c, p->ir, p->it, p->ip)]++;
      t->fx.counters[HC3D_CNT_ABFLUX]++;
      trace_add(tr, 7, p->ir, p->it, p->ip, 0, 0, p->xp, p->yp, p->zp);
      return;
    }
    idust2 = orc_select_dust(c, p, rng);
    if (idust2 < 0) { t->fx.counters[HC3D_CNT_STUCK]++; t->errors++; return; }
  }
bin:
  trace_add(tr, 3, p->ir, p->it, p->ip, 0, 0, p->xp, p->yp, p->zp);
  orc_bin_escape(c, rp, p, xpold, ypold, zpold, iflag, iscat, t);
}

/* ---- one external packet: newdisktherm.F90:378-440 ----------------------- */
/* The packet starts inside the outermost shell at 0.999999 rmax; the walk
 * (tauint, restated) treats it as not on a wall.  No direct peel-off. */
static void orc_external_packet(const orc_ctx *c, const hc3d_run_params *rp, pkt *p, orc_rng *rng, orc_tallies *t,
                                orc_trace *tr) {
  orc_initpout(c, p, rng);
  p->i_orig = 4;
  orc_opacset(c, p, p->nub, rp->rstar_cm);
  const double coslp = cos(p->lp), sinlp = sin(p->lp);
  p->zp = p->cosb * rp->rmax * 0.999999;
  const double rp_ = p->sinb * rp->rmax * 0.999999;
  p->xp = rp_ * coslp;
  p->yp = rp_ * sinlp;
  p->ux = p->sint * p->cosp; p->uy = p->sint * p->sinp; p->uz = p->cost;
  p->ir = c->g.nrg - 1;
  p->on_wall = 0;
  const double thetb = acos(p->cosb);
  p->it = orc_locate(c->g.thetarr, c->g.ntg, thetb);
  p->ip = orc_locate(c->g.phiarr, c->g.npg, p->lp);
  if (p->it < 1) p->it = 1;
  if (p->it > c->g.ntg - 1) p->it = c->g.ntg - 1;
  if (p->ip < 1) p->ip = 1;
  if (p->ip > c->g.npg - 1) p->ip = c->g.npg - 1;
  trace_add(tr, 0, p->ir, p->it, p->ip, 0, 0, p->xp, p->yp, p->zp);
  orc_propagate(c, rp, p, rng, t, tr);
}

/* ---- gasdev, random.f90:140-159, its saved deviate kept per packet -------- */
typedef struct orc_gauss {
  int have;
  double next;
} orc_gauss;

static double orc_gasdev(orc_gauss *g, orc_rng *rng) {
  if (g->have) {
    g->have = 0;
    return g->next;
  }
  double v1, v2, rsq;
  do {
    v1 = 2.0 * orc_ran(rng) - 1.0;
    v2 = 2.0 * orc_ran(rng) - 1.0;
    rsq = v1 * v1 + v2 * v2;
  } while (!(rsq < 1.0 && rsq > 0.0));
  const double fac = sqrt(-2.0 * log(rsq) / rsq);
  g->next = v1 * fac;
  g->have = 1;
  return v2 * fac;
}

/* ---- one disk accretion packet: newdisktherm.F90:209-251 with initpacc
 * (initpacc.f90:24-119), emit_common (emit_common.f90:25-79), emit_gasacc
 * (emit_gasacc.f90:26-42) and reemit (reemit.f90:17-34).  The emitting disk
 * species is picked with the V-band opacities (kapv of hc3d_sources; the
 * reference uses the opacities of the previous packet's frequency).  Returns
 * 0 when no emission point was found within the cap or no species could be
 * picked. */
static int orc_acc_emit(const orc_ctx *c, const hc3d_run_params *rp, pkt *p, orc_rng *rng, orc_tallies *t,
                        int *idust_out) {
  const hc3d_sources *S = rp->sources;
  orc_gauss g = {0, 0.0};
  double rp_, xp, yp, zp;
  int tries = 0;
  for (;;) {
    rp_ = 0.0;
    while (rp_ >= S->rmaxdmax || rp_ <= S->rddustmin) {
      double winv = orc_ran(rng);
      while (orc_ran(rng) > 1.0 - sqrt(winv)) {
        winv = orc_ran(rng);
        if (++tries > ORC_EMIT_TRIES) return 0;
      }
      rp_ = 1.0 / winv;
      if (++tries > ORC_EMIT_TRIES) return 0;
    }
    /* rantheta, random.f90:28-47 */
    double x, y, r2;
    do {
      x = orc_ran(rng);
      x = x + x - 1.0;
      y = orc_ran(rng);
      y = y + y - 1.0;
      r2 = x * x + y * y;
    } while (r2 > 1.0 || r2 == 0.0);
    const double r = sqrt(r2);
    xp = rp_ * (x / r);
    yp = rp_ * (y / r);
    /* sum(fmass*z1*rp**b, mask=is_disk) * gasdev() */
    zp = ((0.0 + S->zfac[0] * pow(rp_, S->zexp[0])) + S->zfac[1] * pow(rp_, S->zexp[1])) * orc_gasdev(&g, rng);
    if (zp * zp + rp_ * rp_ < S->rmax * S->rmax) break;
    if (++tries > ORC_EMIT_TRIES) return 0;
  }
  p->sip = 1.0; p->sqp = 0.0; p->sup = 0.0; p->svp = 0.0;
  const double rsq = xp * xp + yp * yp + zp * zp;
  const double rtot = sqrt(rsq);
  int ir = orc_locate(c->g.r2arr, c->g.nrg, rsq);
  const double cosb = zp / rtot;
  int it = orc_locate(c->g.costarr, c->g.ntg, cosb);
  double lp = atan2(yp, xp);
  if (lp < 0.0) lp = lp + ORC_R2P;
  int ip = orc_locate(c->g.phiarr, c->g.npg, lp);
  p->ir = ir < 1 ? 1 : (ir > c->g.nrg - 1 ? c->g.nrg - 1 : ir);
  p->it = it < 1 ? 1 : (it > c->g.ntg - 1 ? c->g.ntg - 1 : it);
  p->ip = ip < 1 ? 1 : (ip > c->g.npg - 1 ? c->g.npg - 1 : ip);
  p->xp = xp; p->yp = yp; p->zp = zp;
  p->cosb = cosb;
  p->lp = lp;
  p->on_wall = 0;
  const int64_t cell = cidx(c, p->ir, p->it, p->ip);
  const double d0 = dens(c, cell, 0), d1 = dens(c, cell, 1);
  int idust2 = -1;
  if (0.0 + d0 + d1 > 0.0) {
    /* select_dust (select_dust.f90:16-42) over the thermal disk slots */
    const double xran = orc_ran(rng);
    const double opac = (0.0 + S->kapv[0] * d0) + S->kapv[1] * d1;
    if (opac == 0.0) return 0;
    double frac = 0.0;
    const double dd[2] = {d0, d1};
    for (int id = 0; id < 2 && idust2 < 0; ++id) {
      frac = frac + S->kapv[id] * dd[id] / opac;
      if (xran <= frac + (double)1.e-10f) idust2 = id;
    }
    if (idust2 < 0) return 0;
    if (t) {
      t->fx.dbig[cell]++;
      t->fx.nabs[cell + c->ncell4 * idust2] += 1;
    }
    /* emit_common thermal branch (ilucy = 1): reemit at the species' temperature */
    p->cost = 1.0 - 2.0 * orc_ran(rng);
    p->sint = sqrt(1.0 - p->cost * p->cost);
    p->phi = ORC_R2P * orc_ran(rng);
    p->cosp = cos(p->phi);
    p->sinp = sin(p->phi);
    p->nub = orc_lucydustfreq(c, c->g.tdust[cell + c->ncell4 * idust2], idust2, rng);
  } else {
    /* emit_gasacc: the accretion disk temperature of Pringle (1981), eq. 3.23 */
    const double t0 = S->gas_num / (S->gas_den * pow(rtot * S->rstar * S->rsun, 3.0));
    const double tgas = pow(t0 * (1.0 - sqrt(1.0 / rtot)), 0.25) / 11605.0;
    p->nub = orc_bbfreq(c, tgas, rng);
    p->cost = 1.0 - 2.0 * orc_ran(rng);
    p->sint = sqrt(1.0 - p->cost * p->cost);
    p->phi = ORC_R2P * orc_ran(rng);
    p->cosp = cos(p->phi);
    p->sinp = sin(p->phi);
  }
  p->ux = p->sint * p->cosp; p->uy = p->sint * p->sinp; p->uz = p->cost;
  p->i_orig = 2;
  orc_opacset(c, p, p->nub, rp->rstar_cm);
  *idust_out = idust2;
  return 1;
}

static int orc_acc_packet(const orc_ctx *c, const hc3d_run_params *rp, pkt *p, orc_rng *rng, orc_tallies *t,
                          orc_trace *tr) {
  int idust2;
  if (!orc_acc_emit(c, rp, p, rng, t, &idust2)) return 0;
  trace_add(tr, 0, p->ir, p->it, p->ip, 0, 0, p->xp, p->yp, p->zp);
  if (rp->ipeel == 1)
    for (int k = 0; k < rp->npeel; ++k) orc_peeloff(c, rp, p, p->sip, 0, idust2 < 0 ? 0 : idust2, k, t);
  orc_propagate(c, rp, p, rng, t, tr);
  return 1;
}

/* ---- one packet by its global id: newdisktherm.F90:194-449 with ips = 0 --- */
/* Accretion packets first, then hot-spot, stellar and external packets. */
static void orc_packet(const orc_ctx *c, const hc3d_run_params *rp, int64_t pid, orc_rng *rng, orc_tallies *t,
                       orc_trace *tr) {
  pkt p;
  memset(&p, 0, sizeof(p));
  p.on_wall = 0;
  if (rp->ext_illum && pid >= rp->n_star) {
    orc_external_packet(c, rp, &p, rng, t, tr);
    return;
  }
  if (rp->sources && pid < rp->n_acc) {
    if (!orc_acc_packet(c, rp, &p, rng, t, tr)) { t->fx.counters[HC3D_CNT_STUCK]++; t->errors++; }
    return;
  }
  if (!orc_initpspot(c, rp, &p, rng, rp->sources && pid < rp->n_spot ? 1 : 0, NULL)) {
    t->fx.counters[HC3D_CNT_STUCK]++;
    t->errors++;
    return;
  }
  p.i_orig = 1;
  orc_opacset(c, &p, p.nub, rp->rstar_cm);
  const double coslp = cos(p.lp), sinlp = sin(p.lp);
  const double rmin = 1.0;
  p.zp = p.cosb * rmin;
  const double rp_ = p.sinb * rmin;
  p.xp = rp_ * coslp;
  p.yp = rp_ * sinlp;
  p.ux = p.sint * p.cosp; p.uy = p.sint * p.sinp; p.uz = p.cost;
  p.ir = 1;
  p.on_wall = 1;
  const double thetb = acos(p.cosb);
  p.it = orc_locate(c->g.thetarr, c->g.ntg, thetb);
  p.ip = orc_locate(c->g.phiarr, c->g.npg, p.lp);
  if (p.it < 1) p.it = 1;
  if (p.it > c->g.ntg - 1) p.it = c->g.ntg - 1;
  if (p.ip < 1) p.ip = 1;
  if (p.ip > c->g.npg - 1) p.ip = c->g.npg - 1;
  trace_add(tr, 0, p.ir, p.it, p.ip, 0, 0, p.xp, p.yp, p.zp);
  if (rp->ipeel == 1) {
    for (int k = 0; k < rp->npeel; ++k) {
      const double coste = cos(rp->thete[k]), sinte = sin(rp->thete[k]);
      const double cospe = cos(rp->phie[k]), sinpe = sin(rp->phie[k]);
      const double cosnorm = p.cosb * coste + (p.sinb * sinte * (cospe * coslp + sinpe * sinlp));
      /* limb = 0: I constant, energy/sr ~ mu; limb = 1: I ~ 1 + mu (newdisktherm.F90:349-355) */
      const double sipnew = rp->limb ? 12.0 / 5.0 * p.sip * (cosnorm + cosnorm * cosnorm) : 4.0 * p.sip * cosnorm;
      if (cosnorm > 0.0) orc_peeloff(c, rp, &p, sipnew, 0, 0, k, t);
    }
  }
  (void)pid;
  orc_propagate(c, rp, &p, rng, t, tr);
}

/* ------------------------------------------------------------------------ */
/* Public entry points of the oracle (ctypes).                                */
/* ------------------------------------------------------------------------ */
int orc_version(void) { return 1; }

static void orc_ctx_init(orc_ctx *c, const hc3d_dust_tables *dt, const hc3d_grid *g) {
  c->dt = *dt;
  c->g = *g;
  c->limb = 0;
  c->sg = g_sg.on ? &g_sg : NULL;
  c->iter1 = 1;
  c->jfac = 0.0;
  c->ndg = g->ndg;
  c->ncell4 = (int64_t)g->nrg * g->ntg * g->npg;
  /* zetainit (random.f90:79-97): inczeta(i) = sum 1/j^4 over j <= i, added from j = 145 down */
  for (int i = 0; i < 145; ++i) c->inczeta[i] = 0.0;
  for (int j = 145; j >= 1; --j) {
    const double term = 1.0 / (double)(j * j * j * j);
    for (int i = 145; i >= j; --i) c->inczeta[i - 1] = c->inczeta[i - 1] + term;
  }
}

/* The emission of packets [pid0, pid0 + n) of params, without their
 * transport: out[9 k + 0..8] = kind (1 accretion, 2 hot spot, 3 stellar,
 * 4 external, -1 dropped), x, y, z, nu, ir, it, ip, and for an accretion
 * packet the emitting slot (0, 1; -1 the gas) -- for a stellar or hot-spot
 * packet 1 when it radiates at the shock temperature, else 0. */
int orc_sample_emission(const hc3d_dust_tables *dt, const hc3d_grid *g, const hc3d_run_params *rp, int64_t pid0,
                        int64_t n, double *out) {
  orc_ctx c;
  orc_ctx_init(&c, dt, g);
  c.limb = rp->limb;
  for (int64_t k = 0; k < n; ++k) {
    const int64_t pid = rp->packet_offset + pid0 + k;
    orc_rng rng;
    orc_rng_init(&rng, rp->seed, rp->iter, pid);
    pkt p;
    memset(&p, 0, sizeof(p));
    double *o = out + 9 * k;
    int kind, extra = 0, ok = 1;
    if (rp->ext_illum && pid >= rp->n_star) {
      kind = 4;
      orc_initpout(&c, &p, &rng);
    } else if (rp->sources && pid < rp->n_acc) {
      kind = 1;
      ok = orc_acc_emit(&c, rp, &p, &rng, NULL, &extra);
    } else {
      kind = rp->sources && pid < rp->n_spot ? 2 : 3;
      ok = orc_initpspot(&c, rp, &p, &rng, kind == 2, &extra);
      p.xp = p.sinb * cos(p.lp); p.yp = p.sinb * sin(p.lp); p.zp = p.cosb;
    }
    o[0] = ok ? kind : -1;
    o[1] = p.xp; o[2] = p.yp; o[3] = p.zp; o[4] = p.nub;
    o[5] = p.ir; o[6] = p.it; o[7] = p.ip; o[8] = extra;
  }
  return 0;
}

/* n draws of bbfreq(teff), draw k from the counter stream (seed, 1, k). */
int orc_sample_bbfreq(double teff, uint64_t seed, int64_t n, double *out) {
  orc_ctx c;
  memset(&c, 0, sizeof(c));
  for (int j = 145; j >= 1; --j) {
    const double term = 1.0 / (double)(j * j * j * j);
    for (int i = 145; i >= j; --i) c.inczeta[i - 1] = c.inczeta[i - 1] + term;
  }
  for (int64_t k = 0; k < n; ++k) {
    orc_rng rng;
    orc_rng_init(&rng, seed, 1, k);
    out[k] = orc_bbfreq(&c, teff, &rng);
  }
  return 0;
}

/* the run parameters the context reads: limb, and for the small grains the
 * iteration (row 2 in the first) and the jsg weight's kappa_V scale */
static void orc_ctx_params(orc_ctx *c, const hc3d_run_params *rp) {
  c->limb = rp->limb;
  c->iter1 = rp->iter == 1;
  if (c->sg) c->jfac = 1.0 / (rp->rstar_cm * c->dt.kappav[c->sg->jspecies]);
}

/* Run packets [pid_begin, pid_end) of params into t (single thread). */
int orc_run_range(const hc3d_dust_tables *dt, const hc3d_grid *g, const hc3d_run_params *rp, orc_tallies *t,
                  int64_t pid_begin, int64_t pid_end) {
  orc_ctx c;
  orc_ctx_init(&c, dt, g);
  orc_ctx_params(&c, rp);
  for (int64_t pid = pid_begin; pid < pid_end; ++pid) {
    orc_rng rng;
    orc_rng_init(&rng, rp->seed, rp->iter, rp->packet_offset + pid);
    orc_packet(&c, rp, rp->packet_offset + pid, &rng, t, NULL);
  }
  return 0;
}

/* Trace one packet with injected uniforms (or the counter stream when
 * uniforms == NULL).  Returns the number of records written. */
int orc_trace_packet(const hc3d_dust_tables *dt, const hc3d_grid *g, const hc3d_run_params *rp, orc_tallies *t,
                     int64_t pid, const double *uniforms, int nu, hc3d_trace_rec *recs, int max_rec,
                     int *exhausted) {
  orc_ctx c;
  orc_ctx_init(&c, dt, g);
  orc_ctx_params(&c, rp);
  orc_rng rng;
  orc_rng_init(&rng, rp->seed, rp->iter, rp->packet_offset + pid);
  if (uniforms) { rng.inj = uniforms; rng.ninj = nu; rng.pos = 0; }
  orc_trace tr = {recs, max_rec, 0};
  orc_packet(&c, rp, rp->packet_offset + pid, &rng, t, &tr);
  if (exhausted) *exhausted = rng.exhausted;
  return tr.n;
}

/* Draw n uniforms of packet pid's stream (for tests and trace fixtures). */
void orc_stream(uint64_t seed, int iter, int64_t pid, int n, double *out) {
  orc_rng r;
  orc_rng_init(&r, seed, iter, pid);
  for (int i = 0; i < n; ++i) out[i] = orc_ran(&r);
}

void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { orc_philox4x32_10(ctr, key, out); }

/* ---- geometry entry points for known-answer tests ------------------------- */
void orc_radface_roots(double ux, double uy, double uz, double x, double y, double z, double R2_1, double R2_2,
                       double *out6, int *ids3) {
  walls w;
  reset_t(&w);
  radface(&w, ux, uy, uz, x, y, z, R2_1, R2_2);
  out6[0] = w.tn1; out6[1] = w.tp1; out6[2] = w.tp2;
  ids3[0] = w.in1; ids3[1] = w.ip1; ids3[2] = w.ip2;
}

int orc_next_wall(const hc3d_dust_tables *dt, const hc3d_grid *g, double ux, double uy, double uz, double x,
                  double y, double z, int ir, int it, int ip, int on_wall, double *dtout, int *iface) {
  orc_ctx c;
  orc_ctx_init(&c, dt, g);
  return next_wall(&c, ux, uy, uz, x, y, z, ir, it, ip, on_wall, dtout, iface);
}

int orc_locate_c(const double *xx, int n, double x) { return orc_locate(xx, n, x); }

void orc_findangle3_c(double cost1, double sint1, double phi1, double cosp1, double sinp1, double cost2,
                      double sint2, double phi2, double cosp2, double sinp2, double *out3) {
  orc_findangle3(cost1, sint1, phi1, cosp1, sinp1, cost2, sint2, phi2, cosp2, sinp2, &out3[0], &out3[1], &out3[2]);
}

/* ---- single-routine entry points, checked against an independent NumPy
 * restatement of the Fortran routines (tests/golden/ref_routines.py) ------- */

/* closest_wall.f90:13-66: insert n roots (t, id), then find_next_wall.
 * state6 = tn1, tp1, tp2, in1, ip1, ip2; returns 0 when no wall is found. */
int orc_closest_wall_c(int n, const double *t, const int *ids, int on_wall, double *tout, int *iout,
                       double *state6) {
  walls w;
  reset_t(&w);
  for (int k = 0; k < n; ++k) insert_t(&w, t[k], ids[k]);
  state6[0] = w.tn1; state6[1] = w.tp1; state6[2] = w.tp2;
  state6[3] = w.in1; state6[4] = w.ip1; state6[5] = w.ip2;
  return find_next_wall(&w, on_wall, tout, iout);
}

/* phiface.f90:48-56 with C = D = 0 (planes through the z axis) */
void orc_phiface_roots(double A1, double B1, double A2, double B2, double ux, double uy, double x1, double y1,
                       double *out3, int *ids3) {
  walls w;
  reset_t(&w);
  phiface(&w, A1, B1, A2, B2, ux, uy, x1, y1);
  out3[0] = w.tn1; out3[1] = w.tp1; out3[2] = w.tp2;
  ids3[0] = w.in1; ids3[1] = w.ip1; ids3[2] = w.ip2;
}

/* the dust_mod phase-function terms of one species with parameters g, pl
 * (dust.f90:70-74) in slot 0 of a packet */
static void orc_set_phase(pkt *p, double g, double pl) {
  memset(p, 0, sizeof(*p));
  p->g[0] = g; p->pl[0] = pl;
  p->g2[0] = g * g; p->g2p1[0] = p->g2[0] + 1.0; p->onemg2[0] = 1.0 - p->g2[0]; p->twog[0] = 2.0 * g;
}

/* dustmat.f90:40-65: out4 = p1, p2, p3, p4 */
void orc_dustmat_c(double g, double pl, double cost, double cost2, double *out4) {
  pkt p;
  orc_set_phase(&p, g, pl);
  orc_dustmat(&p, 0, cost, cost2, &out4[0], &out4[1], &out4[2], &out4[3]);
}

/* stokespeel.f90:49-376 on s4 = (sip, sqp, sup, svp), in place */
void orc_stokespeel_c(double g, double pl, double *s4, double cost, double sint, double ri1, double bmu,
                      double costp, double sintp) {
  pkt p;
  orc_set_phase(&p, g, pl);
  orc_stokespeel(&p, 0, &s4[0], &s4[1], &s4[2], &s4[3], cost, sint, ri1, bmu, costp, sintp);
}

/* stokes.f90:46-388 with injected uniforms u[0..nu).  st9 = (sip, sqp, sup,
 * svp, cost, sint, phi, cosp, sinp), in place.  Returns the number of
 * uniforms drawn, or -1 when u ran out. */
int orc_stokes_c(double g, double pl, double *st9, const double *u, int nu) {
  pkt p;
  orc_set_phase(&p, g, pl);
  p.sip = st9[0]; p.sqp = st9[1]; p.sup = st9[2]; p.svp = st9[3];
  p.cost = st9[4]; p.sint = st9[5]; p.phi = st9[6]; p.cosp = st9[7]; p.sinp = st9[8];
  orc_rng r;
  orc_rng_init(&r, 0, 0, 0);
  r.inj = u; r.ninj = nu; r.pos = 0;
  orc_stokes(&p, 0, &r);
  st9[0] = p.sip; st9[1] = p.sqp; st9[2] = p.sup; st9[3] = p.svp;
  st9[4] = p.cost; st9[5] = p.sint; st9[6] = p.phi; st9[7] = p.cosp; st9[8] = p.sinp;
  return r.exhausted ? -1 : r.pos;
}

/* opacset (dust.f90:9-80) at frequency nu: out = g[ndg], pl[ndg],
 * albedo[ndg], kappa[ndg] (kappa = kappad interpolated, before the
 * kappav and stellar-radius factors of kapd) */
void orc_opacset_c(const hc3d_dust_tables *dt, const hc3d_grid *g, double nu, double *out) {
  orc_ctx c;
  orc_ctx_init(&c, dt, g);
  pkt p;
  memset(&p, 0, sizeof(p));
  orc_opacset(&c, &p, nu, 1.0);
  const int n = c.ndg;
  for (int id = 0; id < n; ++id) {
    out[id] = p.g[id];
    out[n + id] = p.pl[id];
    out[2 * n + id] = p.albedo[id];
    out[3 * n + id] = p.kapd[id] / dt->kappav[id];
  }
}

/* select_dust.f90:16-42 for one cell whose species densities are dens[ndg],
 * opacities kapd[ndg] and draw xran; returns the 0-based species or -1 */
int orc_select_dust_c(int ndg, const double *kapd, const double *dens, double xran) {
  hc3d_grid g1;
  memset(&g1, 0, sizeof(g1));
  g1.nrg = 1; g1.ntg = 1; g1.npg = 1; g1.ndg = ndg;
  g1.densarr = (double *)dens;
  orc_ctx c;
  memset(&c, 0, sizeof(c));
  c.g = g1; c.ndg = ndg; c.ncell4 = 1;
  pkt p;
  memset(&p, 0, sizeof(p));
  p.ir = 1; p.it = 1; p.ip = 1;
  for (int id = 0; id < ndg; ++id) p.kapd[id] = kapd[id];
  orc_rng r;
  orc_rng_init(&r, 0, 0, 0);
  r.inj = &xran; r.ninj = 1; r.pos = 0;
  return orc_select_dust(&c, &p, &r);
}

/* Sample n scattering events of an unpolarised packet travelling along +z
 * through species 0 at frequency nu, returning the new cos(theta) of each
 * (phase-function moment tests). */
void orc_sample_stokes(const hc3d_dust_tables *dt, const hc3d_grid *g, double nu, uint64_t seed, int n,
                       double *cost_out, double *q_out) {
  orc_ctx c;
  orc_ctx_init(&c, dt, g);
  orc_rng rng;
  orc_rng_init(&rng, seed, 0, 0);
  for (int k = 0; k < n; ++k) {
    pkt p;
    memset(&p, 0, sizeof(p));
    orc_opacset(&c, &p, nu, 1.0);
    p.cost = 0.6; p.sint = 0.8; p.phi = 1.0; p.cosp = cos(1.0); p.sinp = sin(1.0);
    p.sip = 1.0;
    orc_stokes(&p, 0, &rng);
    cost_out[k] = p.cost * 0.6 + p.sint * 0.8 * (p.cosp * cos(1.0) + p.sinp * sin(1.0));
    q_out[k] = p.sqp;
  }
}

double orc_lucydustfreq_c(const hc3d_dust_tables *dt, const hc3d_grid *g, double T0, int id, double xi) {
  orc_ctx c;
  orc_ctx_init(&c, dt, g);
  orc_rng r;
  orc_rng_init(&r, 0, 0, 0);
  r.inj = &xi; r.ninj = 1; r.pos = 0;
  return orc_lucydustfreq(&c, T0, id, &r);
}

/* darkening for one uniform xi (tests) */
double orc_darkening_c(const hc3d_dust_tables *dt, const hc3d_grid *g, double xi) {
  orc_ctx c;
  orc_ctx_init(&c, dt, g);
  return orc_darkening(&c, xi);
}

/* rep_isrf for one injected uniform xi (tests) */
double orc_rep_isrf_c(const hc3d_dust_tables *dt, const hc3d_grid *g, double xi) {
  orc_ctx c;
  orc_ctx_init(&c, dt, g);
  orc_rng r;
  orc_rng_init(&r, 0, 0, 0);
  r.inj = &xi; r.ninj = 1; r.pos = 0;
  return orc_rep_isrf(&c, &r);
}

/* ---- tfinal (restated): Lucy temperature, dusttemp.f90:30-50 form --------- */
static double orc_kapp(const hc3d_dust_tables *d, double T, int id) {
  /* KapP, dust.f90:114-141 */
  const int nT = d->nT;
  double lT = log(T);
  int k = (int)((double)(nT - 1) * (lT - d->lTint[0]) / (d->lTint[nT - 1] - d->lTint[0])) + 1;
  const double *kp = d->kappap + (size_t)id * nT;
  if (k < 1) return kp[0];
  if (k > nT - 1) return kp[nT - 1];
  double f = (lT - d->lTint[k - 1]) / (d->lTint[k] - d->lTint[k - 1]);
  return (1.0 - f) * kp[k - 1] + f * kp[k];
}

#define ORC_SIGT 5.670400e-5
double orc_dusttemp(const hc3d_dust_tables *d, double na, double T0, double ltot, double nphot, int id,
                    double massarr) {
  const double eps = 1.e-5;
  double Td = T0 != 0.0 ? T0 : 0.1 / 11605.0;
  double Told = 0.5 * Td;
  int it = 0;
  while (fabs(Td - Told) > eps * Td && it < 1000) {
    ++it;
    Told = Td;
    Td = pow((na * ltot) / (4.0 * ORC_SIGT * nphot * d->kappav[id] * orc_kapp(d, Td, id)), 0.25) / 11605.0;
    if (massarr > 0.0) Td = Td / massarr;
    else Td = 0.1 / 11605.0;
    if (Td > 1600.0 / 11605.0) Td = 1600.0 / 11605.0;
    if (Td < 0.1 / 11605.0) Td = 0.1 / 11605.0;
  }
  return Td;
}

/* tdust_new(nrg,ntg,npg,ndg) from na(nrg,ntg,npg,ndg) (absorbed-path sums) */
void orc_tfinal(const hc3d_dust_tables *dt, const hc3d_grid *g, const double *na, double ltot, double nphot,
                double *tdust_new) {
  const int64_t n4 = (int64_t)g->nrg * g->ntg * g->npg;
  for (int id = 0; id < g->ndg; ++id)
    for (int ip = 1; ip <= g->npg; ++ip)
      for (int it = 1; it <= g->ntg; ++it)
        for (int ir = 1; ir <= g->nrg; ++ir) {
          int64_t cell = (int64_t)(ir - 1) + (int64_t)g->nrg * ((it - 1) + (int64_t)g->ntg * (ip - 1));
          int64_t k = cell + n4 * id;
          if (ir == g->nrg || it == g->ntg || ip == g->npg || !(g->densarr[k] > 0.0)) {
            tdust_new[k] = g->tdust[k];
            continue;
          }
          tdust_new[k] = orc_dusttemp(dt, na[k], g->tdust[k], ltot, nphot, id, g->massarr[k]);
        }
}

/* ---- very small grains ------------------------------------------------------ */
/* Set (sg != NULL) or clear the small-grain inputs of the runs that follow:
 * the spectra, the 0-based species whose opacity weights the jsg tally, and
 * the cells' spectrum rows and fractions (NULL before the first int_mean).
 * The arrays are not copied. */
void orc_set_sg(const hc3d_sg_tables *sg, int jspecies, const int32_t *imean, const double *imfract) {
  memset(&g_sg, 0, sizeof g_sg);
  if (!sg) return;
  g_sg.sg = *sg;
  g_sg.jspecies = jspecies;
  g_sg.imean = imean;
  g_sg.imfract = imfract;
  g_sg.on = 1;
}

double orc_rep_draine_c(const hc3d_sg_tables *sg, int jm, double jmf, double xran) {
  return orc_rep_draine(sg, jm, jmf, xran);
}

/* int_mean (int_mean.f90:19-94) on the jsg tally of nphot packets: the mean
 * intensity jsg / path_scale x rarr(ir+1) x rstar_cm kappa_V / (4 pi) / vcell
 * / nphot x ltot in units of isrfkap_int, its row in uratio (nr locate,
 * clamped to 1..nemit) and the log10 fraction to the next row.  Cells at the
 * walls' indices (ir = nrg, ...) get row 1, fraction 0. */
void orc_int_mean(const hc3d_grid *g, const hc3d_sg_tables *sg, const int64_t *jsg, double path_scale,
                  double rstar_cm, double kappav, double ltot, double nphot, int32_t *imean, double *imfract) {
  const double jconst = 1.0 / (1.0 / (rstar_cm * kappav)) / (4.0 * ORC_PI);
  for (int ip = 1; ip <= g->npg; ++ip)
    for (int it = 1; it <= g->ntg; ++it)
      for (int ir = 1; ir <= g->nrg; ++ir) {
        const int64_t k = (int64_t)(ir - 1) + (int64_t)g->nrg * ((it - 1) + (int64_t)g->ntg * (ip - 1));
        if (ir == g->nrg || it == g->ntg || ip == g->npg) { imean[k] = 1; imfract[k] = 0.0; continue; }
        double jm = (double)jsg[k] / path_scale;
        jm = jm * g->rarr[ir];
        jm = jm * jconst;
        jm = jm / g->vcell[k] / nphot * ltot;
        const double jratio = jm / sg->isrfkap_int;
        int im = orc_locate(sg->uratio, sg->nemit, jratio);
        if (im > sg->nemit) im = sg->nemit;
        if (im < 1) im = 1;
        double f;
        if (jratio == 0.0) f = 0.0;
        else if (im == sg->nemit) f = 1.0;
        else {
          const double jr1 = log10(sg->uratio[im - 1]), jr2 = log10(sg->uratio[im]);
          f = (log10(jratio) - jr1) / (jr2 - jr1);
        }
        imean[k] = im;
        imfract[k] = f;
      }
}

/* ---- multi-threaded driver (CPU baseline) --------------------------------- */
typedef struct mt_job {
  const hc3d_dust_tables *dt;
  const hc3d_grid *g;
  const hc3d_run_params *rp;
  orc_tallies *t;
  int64_t *next; /* shared: the next packet to claim */
  double deadline; /* CLOCK_MONOTONIC seconds after which no packet is claimed; 0 = none */
  int64_t *done;   /* shared: packets claimed */
} mt_job;

static double orc_now(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* Each thread claims packets one at a time from a shared counter, so a few
 * long histories do not leave the other threads idle; the int64 tallies of
 * the threads sum to the same totals whatever the assignment. */
static void *mt_main(void *arg) {
  mt_job *j = (mt_job *)arg;
  for (;;) {
    if (j->deadline > 0.0 && orc_now() > j->deadline) break;
    const int64_t pid = __atomic_fetch_add(j->next, 1, __ATOMIC_RELAXED);
    if (pid >= j->rp->np) break;
    if (j->done) __atomic_fetch_add(j->done, 1, __ATOMIC_RELAXED);
    orc_run_range(j->dt, j->g, j->rp, j->t, pid, pid + 1);
  }
  return NULL;
}

/* Run np packets on nthreads threads; tls[k] are per-thread tallies that
 * the caller allocated and sums afterwards (int64 sums are exact). */
int orc_run_mt(const hc3d_dust_tables *dt, const hc3d_grid *g, const hc3d_run_params *rp, orc_tallies *tls,
               int nthreads) {
  if (nthreads < 1) nthreads = 1;
  pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
  mt_job *jobs = (mt_job *)calloc((size_t)nthreads, sizeof(mt_job));
  int64_t next = 0;
  if (!th || !jobs) { free(th); free(jobs); return -3; }
  for (int k = 0; k < nthreads; ++k) {
    jobs[k].dt = dt; jobs[k].g = g; jobs[k].rp = rp; jobs[k].t = &tls[k];
    jobs[k].next = &next;
    jobs[k].deadline = 0.0;
    jobs[k].done = NULL;
    pthread_create(&th[k], NULL, mt_main, &jobs[k]);
  }
  for (int k = 0; k < nthreads; ++k) pthread_join(th[k], NULL);
  free(th);
  free(jobs);
  return 0;
}

/* The packets of params claimed by nthreads threads for `seconds` seconds
 * (the threads then finish the packets they hold); *done receives the
 * packets run, the ids [0, *done) of params. */
int orc_run_mt_timed(const hc3d_dust_tables *dt, const hc3d_grid *g, const hc3d_run_params *rp, orc_tallies *tls,
                     int nthreads, double seconds, int64_t *done) {
  if (nthreads < 1) nthreads = 1;
  pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
  mt_job *jobs = (mt_job *)calloc((size_t)nthreads, sizeof(mt_job));
  int64_t next = 0, claimed = 0;
  if (!th || !jobs) { free(th); free(jobs); return -3; }
  const double deadline = orc_now() + seconds;
  for (int k = 0; k < nthreads; ++k) {
    jobs[k].dt = dt; jobs[k].g = g; jobs[k].rp = rp; jobs[k].t = &tls[k];
    jobs[k].next = &next;
    jobs[k].deadline = deadline;
    jobs[k].done = &claimed;
    pthread_create(&th[k], NULL, mt_main, &jobs[k]);
  }
  for (int k = 0; k < nthreads; ++k) pthread_join(th[k], NULL);
  free(th);
  free(jobs);
  if (done) *done = claimed;
  return 0;
}
