/*
 * hc3d.h -- C-ABI of the GB300 photon-packet Monte Carlo loop.
 *
 * This library stands in for one Fortran subroutine of Hochunk3d:
 *
 *     subroutine disk(converge, iter, i1)            (newdisktherm.F90:1)
 *
 * called from the Lucy loop and the final peeled iteration of the driver
 * (newtts.F90:312 and newtts.F90:349).  In the reference every input of
 * disk() reaches it through Fortran module globals (tts_mod, grid_mod,
 * dust_mod, opacin_mod, stokesvar_mod, out_mod).  Here the same data crosses
 * the boundary explicitly, as plain pointers and sizes:
 *
 *   hc3d_load_tables   <- dust_mod / atmos_interp arrays built by dustinit
 *                         (dust.f90:314), setemiss (dust.f90:394) and
 *                         atmosinit (starbarb.f90:3)
 *   hc3d_load_grid     <- grid_mod arrays built by gridset (gridset.f90:1)
 *                         and initarr (initarr.f90:1)
 *   hc3d_run_iteration <- the packet loop of disk() (newdisktherm.F90:194-449)
 *                         with propagate (propagate.f90:1) and peeloff
 *                         (peeloff_3d.f90:5)
 *   hc3d_lucy_update   <- tfinal (called at newdisktherm.F90:557; the module
 *                         is not shipped, restated from dusttemp.f90:30-50)
 *                         followed by initarr(.false.) (initarr.f90:58-89)
 *
 * Conventions (the same as the Fortran arrays they replace):
 *   - arrays are column-major (Fortran order), the first index fastest;
 *   - grid indices are 1-based at the boundary (wall ir = 1..nrg);
 *   - temperatures are in the reference's internal unit K/11605 (eV);
 *   - lengths are in stellar radii, densities in g/cm^3;
 *   - every entry point returns 0 on success and a negative HC3D_ERR_* code
 *     otherwise; no C++ exception crosses the boundary; hc3d_get_error()
 *     returns the last message of a context.
 *
 * Tallies are int64 fixed point: a value v is stored as llround(v * scale),
 * so sums are exact and independent of the order in which packets finish.
 * The scales are reported by hc3d_get_tallies().
 */
#ifndef HC3D_H
#define HC3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HC3D_NDG 8  /* species slots, ndg in grid_mod.f90:13 */
#define HC3D_NO 8   /* SED components all/star/disk/envelope/outside/direct/scattered/thermal, output.F90:232-239 */

#define HC3D_OK 0
#define HC3D_ERR_INVALID (-1)     /* bad argument or size */
#define HC3D_ERR_CUDA (-2)        /* CUDA runtime error */
#define HC3D_ERR_NOMEM (-3)       /* device or host allocation failed */
#define HC3D_ERR_STATE (-4)       /* call out of order (e.g. run before load) */
#define HC3D_ERR_DEVICE (-5)      /* a kernel reported a fault in its status word */
#define HC3D_ERR_IO (-6)          /* file could not be read or written */
#define HC3D_ERR_UNSUPPORTED (-7) /* option of the reference that this build leaves out */
#define HC3D_ERR_TIMEOUT (-8)     /* a bounded wait ran out */
#define HC3D_ERR_CANCELLED (-9)   /* a server request was cancelled (hc3d_server_cancel) */

#define HC3D_PREC_MIXED 0 /* FP32 walk/scatter/peel; FP64 radial quadratic, peel tau sum, Lucy root */
#define HC3D_PREC_FP64 1  /* everything FP64: the all-FP64 GPU form */

typedef struct hc3d_ctx hc3d_ctx;

typedef struct hc3d_device_opts {
  int device;      /* CUDA device ordinal */
  int precision;   /* HC3D_PREC_MIXED or HC3D_PREC_FP64 */
  int block_size;  /* threads per block of the transport kernel; 0 = default */
  int grid_blocks; /* blocks of the persistent transport kernel; 0 = SMs x resident blocks */
} hc3d_device_opts;

/* dust_mod (dust_mod.f90:7-17) plus the stellar-spectrum CDF of atmos_interp
 * (starbarb.f90:57-110).  All species slots 1..ndg must be described; a slot
 * whose density is zero everywhere may repeat another slot's table. */
typedef struct hc3d_dust_tables {
  int ndg;                /* species slots described, 1..8 */
  int nlammax;            /* leading dimension of the per-wavelength tables */
  const int *nlambda;     /* (ndg) rows used per species */
  const double *nudust;   /* (nlammax,ndg) frequency, decreasing with row */
  const double *kappad;   /* (nlammax,ndg) kappa / kappa_V */
  const double *adust;    /* (nlammax,ndg) albedo */
  const double *gdust;    /* (nlammax,ndg) HG asymmetry g */
  const double *pldust;   /* (nlammax,ndg) peak linear polarisation */
  const double *kappav;   /* (ndg) kappa_V in cm^2/g */
  int nT, nnu;            /* 1000, 1025 in the reference */
  const double *lTint;    /* (nT) log temperature grid */
  const double *nuint;    /* (nnu) frequency grid in units of T */
  const double *kapBint;  /* (nT,nnu,ndg) normalised cumulative kappa*B_nu */
  const double *kappap;   /* (nT,ndg) Planck-mean kappa / kappa_V */
  double tsub;            /* dust sublimation temperature, K */
  int nhnu;               /* stellar spectrum samples */
  const double *hnuint;   /* (nhnu) cumulative distribution, increasing */
  const double *atmosnu;  /* (nhnu) frequency */
  const double *lognu;    /* (nhnu) log10 frequency */
  const double *loghnu;   /* (nhnu) log10 cumulative distribution */
  int nisrf;              /* rows of the external-illumination spectrum (isrf_mod, 200); 0 = none */
  const double *isrf_cdf;     /* (nisrf) cdf_i of isrf_cdf.f90: cumulative, 0 .. 1 */
  const double *isrf_logcdf;  /* (nisrf) logcdf_i: log10 cdf_i, -99 at row 1 */
  const double *isrf_logfreq; /* (nisrf) logfreq_i: log10 frequency (1.2398/lambda[um]), 0 at row 1 */
  int ntab;               /* rows of the limb-darkening table (tabl_mod) for limb = 1; 0 = none */
  const double *limb_xmu;     /* (ntab) xmu of samptabl.f90 table: 0, 2d, 3d, .., 1 with d = 1/ntab */
  const double *limb_prob;    /* (ntab) prob: 0.5 (mu^3 + mu^2), 0 at row 1 */
} hc3d_dust_tables;

/* grid_mod (grid_mod.f90:20-50) as gridset leaves it. */
typedef struct hc3d_grid {
  int nrg, ntg, npg;      /* wall counts; cells are (nrg-1)(ntg-1)(npg-1) */
  int ndg;                /* species slots in densarr/tdust/massarr, 1..8 */
  const double *rarr;     /* (nrg) radial walls, R* */
  const double *r2arr;    /* (nrg) squares of rarr */
  const double *thetarr;  /* (ntg) polar walls, rad */
  const double *costarr;  /* (ntg) */
  const double *tan2arr;  /* (ntg) tan^2; 0 at the poles, -1 for the midplane */
  const double *phiarr;   /* (npg) azimuthal walls, rad */
  const double *aarr;     /* (npg) sin(phi) */
  const double *barr;     /* (npg) -cos(phi) */
  const double *densarr;  /* (nrg,ntg,npg,ndg) g/cm^3 */
  const double *massarr;  /* (nrg,ntg,npg,ndg) (rho*V)^(1/4), cgs */
  const double *vcell;    /* (nrg,ntg,npg) cm^3 */
  const double *tdust;    /* (nrg,ntg,npg,ndg) temperature used by re-emission, K/11605 */
} hc3d_grid;

/* Constants of the disk-accretion and stellar hot-spot sources (CDISKACC,
 * CSPOT), as gridset (gridset.f90:72-203) and spotset (spotset.f90:179-206)
 * leave them.  Lengths in stellar radii, temperatures in K/11605. */
typedef struct hc3d_sources {
  /* disk accretion packets (initpacc.f90:24-49, emit_gasacc.f90:26-29) */
  double rddustmin;       /* emission radii lie in (rddustmin, rmaxdmax) */
  double rmaxdmax;        /* max(rmaxd(1), rmaxd(2)), setup.f90:181 */
  double rmax;            /* the emission point lies inside the sphere of radius rmax */
  double zfac[2];         /* fmass*z1 of the two disk slots: height = sum(zfac r^zexp) * gasdev() */
  double zexp[2];         /* b of the two disk slots */
  double kapv[2];         /* kappa_V * rmincgs of the two disk slots: the weights that pick the emitting dust */
  double gas_num;         /* 3 G (Msun Mc) Mdot, cgs */
  double gas_den;         /* 8 pi sigma_SB: T_gas^4 = gas_num / (gas_den (r rstar rsun)^3) (1 - r^-1/2) K^4 */
  double rstar, rsun;     /* stellar radius in Rsun, and Rsun in cm */
  /* hot spots (initpspot.f90:33-160) */
  int ispot;              /* CSPOT: 1 = spots on the stellar surface */
  int nspot;              /* 1 or 2 (the second opposite the first) */
  double spot1[4];        /* sin th0 cos phi0, sin th0 sin phi0, cos th0, sin th0 of spot 1 (scspot1 ..) */
  double spot2[4];        /* the same for spot 2 */
  double csprad;          /* cos of the spot radius: points with dot > csprad lie in a spot */
  double fspot;           /* filling factor of the spots; 1 = stellar packets keep the stellar spectrum */
  double tshock;          /* spot (shock) temperature */
} hc3d_sources;

/* The scalars and small arrays of tts_mod/out_mod that one call of disk()
 * reads (setup.f90:37-43,118-130,196-202; initarr.f90:17-21). */
typedef struct hc3d_run_params {
  int64_t np;             /* packets of this call */
  int64_t packet_offset;  /* global id of the first packet (sharding across processes) */
  uint64_t seed;          /* run seed; packet streams are keyed by (seed, iter, packet id) */
  int iter;               /* Lucy iteration number, 1-based */
  int ipeel;              /* 1 = peel-off images and SEDs (CPEEL) */
  int npeel;              /* peel-off directions */
  const double *thete;    /* (npeel) peel-off theta, rad */
  const double *phie;     /* (npeel) peel-off phi, rad */
  int nfreq, nmu, nph, nap;
  int nxhst;              /* image pixels per side (NXIMG) */
  double rmaxi;           /* image half size, R* */
  const double *aperture2;/* (nap) squared aperture radii, R*^2 */
  double numin, numax;    /* SED frequency range, units of 1.2398/lambda[um] */
  double rstar_cm;        /* stellar radius in cm (rmincgs) */
  double tstar;           /* stellar temperature, K/11605 */
  int limb;               /* 0 = uniform disk; 1 = Eddington limb darkening (the table of hc3d_dust_tables) */
  int iintmax;            /* interactions in one cell before a packet is killed (10000) */
  int64_t max_interactions; /* per-packet cap on interactions; 0 = no cap */
  int image;              /* 1 = accumulate broadband I,Q,U,V images of the peeled packets */
  int ext_illum;          /* 1 = external illumination (COUTILLUM): packets with global id >= n_star
                             enter from the outer sphere (newdisktherm.F90:378-440); needs nisrf > 0 */
  int64_t n_star;         /* packets of the whole iteration with a source inside the grid: global ids
                             >= n_star are external (npacc + ns of newdisktherm.F90:143-175, from
                             hc3d_packet_split; hc3d_star_packets without accretion) */
  double rmax;            /* outer radius of the grid, R* (the external packets start at 0.999999 rmax) */
  int64_t n_acc;          /* global ids < n_acc are disk accretion packets (iphot < npacc,
                             newdisktherm.F90:209); needs sources */
  int64_t n_spot;         /* global ids in [n_acc, n_spot) are hot-spot packets (iphot < npacc + npaccstar,
                             newdisktherm.F90:258); needs sources */
  const hc3d_sources *sources; /* accretion and spot constants; NULL = neither (n_acc = n_spot = 0) */
  int imcube;             /* 1 = also the per-frequency image cube image_m_* of the peeled packets
                             (IMCUBE, peeloff_3d.f90:271-282) in runs with ipeel = 1; needs image */
} hc3d_run_params;

/* Host copies of the device tallies.  Any pointer may be NULL.  Shapes are
 * those of the reference arrays (initarr.f90:24-43, initimages, grid_mod). */
typedef struct hc3d_tallies {
  int64_t *si, *sq, *su, *sv;      /* (nfreq,nmu,nph,nap,no) Stokes sums, x stokes_scale */
  int64_t *si2, *sq2, *su2, *sv2;  /* (nfreq,nmu,nph,nap,no) squares, x square_scale */
  int64_t *nums;                   /* (nfreq,nmu,nph,nap,no) packet counts */
  int64_t *ti, *tq, *tu, *tv;      /* (nfreq,npeel,nap,no) peeled Stokes sums, x stokes_scale */
  int64_t *ti2, *tq2, *tu2, *tv2;  /* (nfreq,npeel,nap,no) peeled squares, x square_scale */
  int64_t *numt;                   /* (nfreq,npeel,nap,no) peeled counts */
  int64_t *image_i, *image_q, *image_u, *image_v; /* (npeel,nxhst,nxhst) broadband, x stokes_scale */
  int64_t *nabs;                   /* (nrg,ntg,npg,ndg) absorption counts */
  int64_t *dtauabs;                /* (nrg,ntg,npg,ndg) absorption path estimator, x path_scale */
  int64_t *jmean;                  /* (nrg,ntg,npg) path length, x path_scale */
  int32_t *killed;                 /* (nrg,ntg,npg) */
  int32_t *dbig;                   /* (nrg,ntg,npg) thermal-grain absorptions */
  int64_t counters[16];            /* see HC3D_CNT_* */
  double stokes_scale;             /* fixed-point scale of Stokes sums and images */
  double square_scale;             /* fixed-point scale of squared Stokes sums */
  double path_scale;               /* fixed-point scale of dtauabs and jmean */
  int64_t *image_m_i;              /* (npeel,nxhst,nxhst,nfreq,no) per-frequency image cube, x stokes_scale
                                      (runs with imcube) */
  int64_t *image_m_q, *image_m_u, *image_m_v; /* (npeel,nxhst,nxhst,nfreq), x stokes_scale */
  int32_t *dsg;                    /* (nrg,ntg,npg) small-grain absorptions (propagate.f90:108-113) */
  int64_t *jsg;                    /* (nrg,ntg,npg) small-grain absorption path, x path_scale: the sum of
                                      ds kappa(nu)/kappa_V (1 - albedo(nu)) / rarr(ir+1) of the sg_slot
                                      species over the cell's steps, the input of int_mean */
} hc3d_tallies;

/* counters[] of hc3d_tallies (newdisktherm.F90:122-141, propagate.f90:296-318) */
#define HC3D_CNT_FLUX 0       /* packets binned inside the largest aperture */
#define HC3D_CNT_SFLUX 1      /* of those, scattered at least once */
#define HC3D_CNT_NSCAT 2      /* scatterings of the packets in SFLUX */
#define HC3D_CNT_SCOUNT 3     /* escaped packets that scattered last */
#define HC3D_CNT_TOT 4        /* packets that interacted at least once */
#define HC3D_CNT_ABFLUX 5     /* packets killed (iint > iintmax or the interaction cap) */
#define HC3D_CNT_AFLUX 6      /* packets absorbed by the star */
#define HC3D_CNT_SUMSUB 7     /* sum of escaping Stokes I, x stokes_scale */
#define HC3D_CNT_SUMALL 8     /* same, including non-interacting external packets */
#define HC3D_CNT_ESCAPED 9    /* packets that left the grid */
#define HC3D_CNT_CROSS_PROP 10 /* cell crossings of the propagation walk */
#define HC3D_CNT_CROSS_PEEL 11 /* cell crossings of the peel-off walks */
#define HC3D_CNT_EVENTS 12    /* scatterings + absorptions */
#define HC3D_CNT_PEELS 13     /* peel-off rays started */
#define HC3D_CNT_STUCK 14     /* packets stopped by a fault (see hc3d_get_fault_log) */
#define HC3D_CNT_PEEL_STUCK 15 /* peel-off rays stopped by a fault (their contribution is dropped) */

/* ---- context ----------------------------------------------------------- */
int hc3d_create(hc3d_ctx **ctx, const hc3d_device_opts *opts);
void hc3d_destroy(hc3d_ctx *ctx);
/* Drop the loaded model (tables, grid, tallies) and keep the stream, the
 * packet pool and the peel-off queue, so that the next model loads without
 * reallocating them (a serving slot runs model after model this way).  No
 * counterpart in the reference, which runs one model per process. */
int hc3d_reset(hc3d_ctx *ctx);
int hc3d_get_error(const hc3d_ctx *ctx, char *buf, size_t len);
/* Library version string and build architecture, e.g. "hc3d 0.1 sm_103a". */
const char *hc3d_version(void);

/* The species (reference numbering 1..8, grid_mod.f90:13-20: 1-2 thermal
 * disk grains, 3 envelope, 4 cavity, 5-8 their very small grains and PAHs)
 * that the device's four species slots carry: species[0] = 1, species[1] =
 * 2, species[2] < species[3] in 3..8.  Default {1, 2, 3, 4}.  Call before
 * hc3d_load_tables and hc3d_load_grid, which read each slot's species from
 * the (.., ndg) host arrays; a species outside the map must hold no density.
 * No counterpart in the reference, which carries all eight species. */
int hc3d_set_species(hc3d_ctx *ctx, const int32_t *species);

/* dustinit/setemiss/atmosinit outputs (dust.f90:314-474, starbarb.f90:3-110) */
int hc3d_load_tables(hc3d_ctx *ctx, const hc3d_dust_tables *tables);

/* draine_mod (draine_mod.f90, draine_cdf.f90:1-79) and the ISRF integral of
 * isrf_cdf.f90:191-214: the emission spectra of the very small grains and
 * PAHs for nemit ratios U of the mean intensity to the ISRF. */
typedef struct hc3d_sg_tables {
  int nemit;              /* spectra (18) */
  int ndraine;            /* frequencies per spectrum (1000) */
  const double *cdf;      /* (nemit,ndraine) cdf_d: cumulative, normalised, increasing frequency */
  const double *logcdf;   /* (nemit,ndraine) logcdf_d: log10 cdf_d, -10 at row 1 */
  const double *logfreq;  /* (ndraine) logfreq_d: log10 frequency (1.2398/lambda[um]), 0 at row 1 */
  const double *uratio;   /* (nemit) uratio_arr: the U of each spectrum, increasing */
  double isrfkap_int;     /* ISRF x absorption opacity of the small grains of sg_slot, integrated over frequency */
  int sg_slot;            /* 1..4: the slot whose opacity weights the jsg tally and isrfkap_int */
} hc3d_sg_tables;
/* Load the small-grain spectra into a context whose species map holds small
 * grains, after hc3d_load_tables.  An absorption by a small-grain slot then
 * re-emits as emit_common.f90:31-53 does: the frequency from the spectrum of
 * the cell's U (rep_draine.f90), an unpolarised isotropic direction
 * (emit_sg.f90); dsg counts it instead of dbig.  hc3d_lucy_update then also
 * runs int_mean (int_mean.f90:19-94) on the jsg tally. */
int hc3d_load_sg_tables(hc3d_ctx *ctx, const hc3d_sg_tables *tables);
/* imean (nrg,ntg,npg): the spectrum row 1..nemit of each cell, and imfract
 * (nrg,ntg,npg): the fraction of the way to the next row, as int_mean of the
 * last hc3d_lucy_update left them (get), or as a host computed them (set).
 * The first iteration (params->iter == 1) uses row 2 with fraction 0 in
 * every cell (emit_common.f90:34-37); later ones need int_mean's result. */
int hc3d_get_imean(hc3d_ctx *ctx, int32_t *imean, double *imfract);
int hc3d_set_imean(hc3d_ctx *ctx, const int32_t *imean, const double *imfract);

/* gridset/initarr outputs (gridset.f90:411-1098, initarr.f90:11-56) */
int hc3d_load_grid(hc3d_ctx *ctx, const hc3d_grid *grid);

/* Replace the dust temperatures of the loaded grid with tdust (nrg,ntg,npg,ndg),
 * K/11605, Fortran order -- the temperature field initarr copies in before
 * an iteration (initarr.f90:78-84), e.g. a field read back from an earlier
 * run.  The sublimation (peel-off) mask follows the new field.  A value of 0
 * stands for the 0.1 K floor of the starting field; a negative, NaN or
 * infinite value is rejected (HC3D_ERR_INVALID). */
int hc3d_set_tdust(hc3d_ctx *ctx, const double *tdust);

/* initarr(.false.) tally reset (initarr.f90:58-89): zero every tally. */
int hc3d_zero_tallies(hc3d_ctx *ctx);

/* One call of the packet loop of disk() (newdisktherm.F90:194-449) for
 * params->np packets, accumulating into the device tallies.  Blocks until the
 * packets are done. */
int hc3d_run_iteration(hc3d_ctx *ctx, const hc3d_run_params *params);

/* One chunk of a peeled iteration of np_iteration packets: the packets
 * [packet_offset, packet_offset + np) of params start here, and with final =
 * 0 the call returns once all of them have started, leaving the packets
 * still in flight in the context; they continue in the next chunk.  The
 * chunk with final = 1 runs every packet to its end.  The chunks of an
 * iteration share its seed and iteration number and accumulate into the same
 * tallies (the fixed-point scales are set for np_iteration packets); their
 * tallies equal those of one hc3d_run_iteration of the whole range, bit for
 * bit.  A long iteration so runs in steps without paying its last, longest
 * histories at the end of every step.  hc3d_run_iteration, hc3d_autotune and
 * hc3d_set_wave_options refuse to run while a chunked iteration is in flight;
 * hc3d_zero_tallies discards it.  Unpeeled runs finish every packet in each
 * chunk.  No counterpart in the reference (its loop runs one iteration in one
 * call). */
int hc3d_run_chunk(hc3d_ctx *ctx, const hc3d_run_params *params, int64_t np_iteration, int final);

/* Copy the device tallies to the non-NULL host buffers of *out. */
int hc3d_get_tallies(hc3d_ctx *ctx, const hc3d_run_params *params, hc3d_tallies *out);

/* tfinal (newdisktherm.F90:557, restated) + initarr(.false.) temperature copy
 * (initarr.f90:78-84): solve the Lucy energy balance of every cell and
 * species in FP64 from the dtauabs tally of the packets run since the last
 * hc3d_zero_tallies(), with ltot in erg/s and np the packets that produced
 * it.  The new temperatures become the device tdust used by the next
 * iteration and are copied to tdust_out (nrg,ntg,npg,ndg) when non-NULL.
 * *max_rel_change receives max |T_new-T_old|/T_new over the cells counted
 * by the convergence test and *converged is 1 when it is below 1%. */
int hc3d_lucy_update(hc3d_ctx *ctx, double ltot, int64_t np, double *tdust_out,
                     double *max_rel_change, int *converged);

/* Replace the context's absorbed-path tally with dtauabs (nrg,ntg,npg,ndg),
 * int64 at the context's path_scale (hc3d_get_tallies reports it): the sum
 * of the shards' tallies when the packets of an iteration ran on several
 * processes (the reference's MPI_ALLREDUCE of newdisktherm.F90:482), so that
 * hc3d_lucy_update then solves the temperatures of the whole iteration.  The
 * shards run their packet ranges with hc3d_run_chunk(final = 1) and the
 * whole iteration's np_iteration, so that every shard tallies at the same
 * scales. */
int hc3d_set_lucy_tally(hc3d_ctx *ctx, const int64_t *dtauabs);

/* The packet loops of n models (1..256) in one persistent launch: ctxs[j]
 * runs params[j] with its own tables, grid and tallies.  Peeled runs
 * (ipeel = 1) walk each event's peel-off rays in the thread that made the
 * event, with the same walk as the wavefront form, so the tallies equal
 * those of hc3d_run_iteration(ctxs[j], &params[j]) bit for bit in the FP64
 * form and within FP32 rounding in the mixed form.  All contexts share one
 * device and precision; the launch runs on the stream of ctxs[0].  No
 * counterpart in the reference (one model per run). */
int hc3d_run_batch(hc3d_ctx *const *ctxs, const hc3d_run_params *params, int n);

/* ---- autotuner (no counterpart in the reference) ---------------------------
 * Times the sample batch under each candidate setting and keeps the fastest
 * in the context (peeled runs: as the second of two such chunks of one
 * iteration, see hc3d_run_chunk).  Peeled runs: the peel-off queue depth (2^20 .. 2^23
 * records), then at the best depth the regeneration threshold of the
 * wavefront kernel (1, 4, 8, 16: how many lanes of a warp must be waiting
 * before they take new packets), then in the mixed form the block shape of
 * the peel-off kernel (128 or 192 threads per block).  Other runs: the transport block
 * size (64, 96, 128).  The settings do not change the tallies.  The tallies
 * are zeroed afterwards. */
typedef struct hc3d_tune_result {
  int n;                      /* candidates timed */
  int best;                   /* index of the setting the context now uses */
  int64_t queue_records[12];  /* per candidate */
  int block_size[12];         /* transport block size */
  int regen[12];
  int peel_shape[12];         /* block shape index of the peel-off kernel */
  int peel_threads[12];       /* its threads per block */
  double ms[12];              /* wall time of the sample batch */
} hc3d_tune_result;
int hc3d_autotune(hc3d_ctx *ctx, const hc3d_run_params *sample, hc3d_tune_result *out);

/* Set the wavefront form's settings by hand (0 keeps a setting): the
 * peel-off queue depth in records (>= 1024), the regeneration threshold
 * (1..32 lanes of a warp), the queue slots a lane reserves per atomic
 * (1..64) and the mixed-form peel-off kernel's block shape (1: 128 threads,
 * 5 blocks per SM; 2: 192 threads, 3 blocks).
 * None of them changes the tallies.  No counterpart in the reference. */
int hc3d_set_wave_options(hc3d_ctx *ctx, int64_t queue_records, int regen, int qchunk, int peel_shape);

/* n_iter Lucy iterations of params->np packets without peel-off
 * (newtts.F90:294-330 with a fixed count), captured as one CUDA graph and
 * launched once: each iteration zeroes the tallies, runs the packet loop
 * with iter = params->iter + k and updates the temperatures, as
 * hc3d_zero_tallies + hc3d_run_iteration + hc3d_lucy_update would, with the
 * same results.  max_rel_change receives n_iter values; tdust_out the last
 * temperatures when non-NULL.  params->ipeel must be 0. */
int hc3d_lucy_iterations(hc3d_ctx *ctx, const hc3d_run_params *params, int n_iter, double ltot,
                         double *max_rel_change, double *tdust_out);

/* ---- Lucy update that allocates nothing (no counterpart in the reference) --
 * hc3d_lucy_update() needs a context, and a context obtains its device
 * buffers with cudaMalloc.  Callers that cannot allocate device memory when
 * the temperatures are due -- a host code that has reserved all of its device
 * memory up front or hands it out from a pool it does not own, or a coupling
 * that runs inside another code's stream work and may not add allocations to
 * it -- call hc3d_lucy_update_noalloc() instead, with every array already on
 * the device.  It computes what hc3d_lucy_update() computes, in the same
 * FP64 arithmetic, from caller-owned buffers in the Fortran layouts above.
 *
 * Its only working memory is a fixed array of 1 MiB + 16 bytes in the
 * library's device image: the per-block maxima of the convergence test and a
 * completion counter.  Every GPU that loads the library holds that array until
 * the process exits.  Grids are limited to nrg*ntg*npg*ndg <=
 * HC3D_NOALLOC_MAX_ELEMENTS; a larger one returns HC3D_ERR_INVALID with a
 * message on stderr.  Every call looks the array's device address up
 * (cudaGetSymbolAddress, which allocates nothing) with the device current,
 * so a context the host recreated after cudaDeviceReset() is found anew; make
 * the first call on a device before any stream capture (it loads the module
 * there).  All calls share the array, which keeps the
 * last call's contents, so calls that overlap on the GPU (different streams
 * without ordering between them) race and must not be issued.  The call
 * returns after the update on `stream` is complete. */
#define HC3D_NOALLOC_MAX_ELEMENTS 134217728LL /* 2^27 grid elements */

typedef struct hc3d_lucy_buffers {
  int device;                /* CUDA device ordinal the buffers live on */
  void *stream;              /* cudaStream_t to run on (NULL = legacy default stream) */
  int nrg, ntg, npg, ndg;    /* wall counts and species slots of the arrays below */
  const int64_t *dtauabs;    /* device (nrg,ntg,npg,ndg) absorbed-path tally, x path_scale */
  double path_scale;         /* fixed-point scale of dtauabs (hc3d_tallies.path_scale) */
  const double *densarr;     /* device (nrg,ntg,npg,ndg) g/cm^3; cells with 0 are left as they are */
  const double *massarr;     /* device (nrg,ntg,npg,ndg) (rho*V)^(1/4) */
  const double *tdust_in;    /* device (nrg,ntg,npg,ndg) temperatures of the last iteration, K/11605 */
  double *tdust_out;         /* device (nrg,ntg,npg,ndg) new temperatures; may equal tdust_in */
  int nT;                    /* rows of lTint */
  const double *lTint;       /* device (nT) log temperature grid */
  const double *kappap;      /* device (nT,ndg) Planck-mean kappa / kappa_V */
  double kappav[HC3D_NDG];   /* kappa_V of each slot, cm^2/g (host values) */
  double ltot;               /* luminosity of the packets, erg/s */
  int64_t np;                /* packets that produced dtauabs */
} hc3d_lucy_buffers;

int hc3d_lucy_update_noalloc(const hc3d_lucy_buffers *buffers, double *max_rel_change,
                             int *converged);

/* ---- measurement helpers (no counterpart in the reference) -------------- */
/* The CUDA stream (cudaStream_t) every kernel of this context is launched on. */
void *hc3d_get_stream(hc3d_ctx *ctx);
/* Device time in ms of the transport kernel of the last hc3d_run_iteration,
 * from CUDA events recorded on that stream around the launch. */
int hc3d_last_kernel_ms(hc3d_ctx *ctx, double *ms);
/* Kernel launches of the last hc3d_run_iteration and their device time, split
 * into packet transport and peel-off ray walks (CUDA events on the stream). */
int hc3d_last_launch_stats(hc3d_ctx *ctx, int *launches, double *transport_ms, double *peel_ms);
/* Packets stopped by a fault since the last hc3d_zero_tallies(): *n receives
 * the count and entries[0..min(n,max,256)-1] the global packet id in the low
 * 56 bits and the fault code in the high 8 (1 index range, 2 no wall found,
 * 3 crossing cap, 4 no opacity to select a species, 5 an accretion or
 * hot-spot packet without an emission point within the sampling cap or
 * without a species to emit it).  Replaying a logged id
 * through hc3d_trace_packets with its counter-based uniforms reproduces it. */
int hc3d_get_fault_log(hc3d_ctx *ctx, uint64_t *entries, int max, int *n);
/* Per wave of the last peeled run: event budget E, threads that could run,
 * packets alive after the wave, transport ms, peel-off ms, interactions
 * (6 doubles each). */
int hc3d_get_wave_log(hc3d_ctx *ctx, double *out, int max_waves, int *n);

/* ---- single-packet trace harness ---------------------------------------- */
/* One record per propagation cell crossing / interaction of a traced packet. */
typedef struct hc3d_trace_rec {
  int32_t kind;    /* 1 = crossing, 2 = interaction point, 3 = escape, 4 = star, 5 = scatter, 6 = absorb, 7 = kill */
  int32_t ir, it, ip; /* cell after the event, 1-based */
  int32_t iface;   /* wall crossed (1..6) or 0 */
  int32_t pad;
  double tsum;     /* optical depth integrated in the current tauint call */
  double x, y, z;  /* position after the event */
} hc3d_trace_rec;

/* Replay packets 0..npkt-1 of params with their uniform draws taken from
 * uniforms[k*nu + j] (packet k, draw j) instead of the counter-based stream,
 * writing up to max_rec trace records per packet to recs[k*max_rec + ...]
 * and the record count to nrec[k].  Tallies are accumulated as usual. */
int hc3d_trace_packets(hc3d_ctx *ctx, const hc3d_run_params *params, int npkt,
                       const double *uniforms, int nu, hc3d_trace_rec *recs,
                       int max_rec, int32_t *nrec);

#ifdef __cplusplus
}
#endif
#endif /* HC3D_H */
