/*
 * hc3d_host.h -- host-side model setup and run driver of the GB300 photon loop.
 *
 * These entry points replace the Fortran caller of disk() -- the work that
 * newtts.F90 does before, between and after the calls of disk():
 *
 *   hc3d_model_create  <- setup (setup.f90:3) + reapar (reapar.f90:1)
 *                         + dustinit/setemiss (dust.f90:314,394)
 *                         + atmosinit (starbarb.f90:3) + setup_wave
 *                         (setup_wave.f90:46-115) + gridset (gridset.f90:1)
 *                         + initarr(.true.) (initarr.f90:11-56)
 *   hc3d_tts           <- program tts (newtts.F90:141-368): Lucy iterations,
 *                         the final peeled iteration, diskflux (flux.f90:1)
 *                         and the ASCII writers of output (output.F90:166-503)
 *
 * The .par format and keys are those of configuration.f90/reapar.f90, with
 * these extensions (all optional):
 *   SEDLMIN, SEDLMAX  SED wavelength range in microns (setup.f90:37-39
 *                     hard-codes 0.01 and 5000)
 *   IMAGE             YES/NO broadband I,Q,U,V peel-off images (default YES)
 *   MAXINT            per-packet interaction cap (default 1000000; 0 = none)
 *   SEED              64-bit run seed of the counter-based packet streams
 *   FRACTLEV, FRACTN, FRACTCONTRAST  levels, clumps per level and density
 *                     contrast of the project fractal generator (CFRACTAL=YES)
 *   ISRF_FILE         with COUTILLUM=YES: the external radiation field, one
 *                     "log10 nu[Hz]  log10 nu*F_nu" pair per line, increasing
 *                     in nu (isrf_cdf.f90 carries its table in the source)
 */
#ifndef HC3D_HOST_H
#define HC3D_HOST_H

#include "hc3d.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hc3d_model hc3d_model;

/* Scalars of tts_mod/opacin_mod that the driver needs besides the views. */
typedef struct hc3d_model_info {
  int64_t np;          /* NP */
  int64_t npmin;       /* NPMIN */
  int64_t np_lucy;     /* packets per Lucy iteration (newtts.F90:159-182) */
  int nimin, nimax;    /* NIMIN, NIMAX */
  int ipeel, ilucy;    /* CPEEL, CLUCY */
  int ndg_active;      /* species slots with nonzero density */
  double ltot;         /* erg/s (gridset.f90:165-180) */
  double tstar_k;      /* K */
  double rstar_rsun;
  double autors;       /* AU in stellar radii */
  double rminsub;      /* sublimation radius, R* */
  double massdisk, massenv; /* Msun on the grid */
  int64_t ncells;      /* (nrg-1)(ntg-1)(npg-1) */
  double density_host_ms; /* wall time of the host density build in gridset */
  double tables_host_ms;  /* wall time of the host setemiss tables */
  double lstar;           /* stellar luminosity, erg/s */
  double l_isrf;          /* external-illumination luminosity, erg/s (newtts.F90:204-228) */
  double isrf_frac;       /* l_isrf / ltot (gridset.f90:208-209) */
  /* disk accretion and hot spots (gridset.f90:72-270); zero without CDISKACC */
  double lacc;            /* accretion luminosity of the disk, erg/s */
  double lacc2;           /* accretion shock luminosity on the star, erg/s */
  double accfrac;         /* lacc / ltot */
  double accfrac2;        /* lacc2 / ltot */
  double mdot_msun_yr;    /* disk accretion rate */
  double tshock_k;        /* hot-spot temperature, K */
  double fspot;           /* spot filling factor (1 without spots) */
  double thspot_deg;      /* spot radius, degrees */
  double tave_k;          /* mean stellar temperature with the shock, K; sets rminsub */
  /* very small grains and PAHs (FSG(1..4) > 0) */
  int32_t slot_species[4]; /* the species each device slot carries (hc3d_set_species) */
  int has_sg;             /* 1: a device slot carries small grains; hc3d_model_sg_tables describes them */
  int ndg;                /* species in the host arrays: 4, or 8 with small grains */
} hc3d_model_info;

/* Build a model from a .par file.  par_dir overrides PARDIR when non-NULL.
 * err receives a message on failure. */
int hc3d_model_create(hc3d_model **m, const char *par_path, const char *par_dir, char *err, size_t errlen);
void hc3d_model_destroy(hc3d_model *m);

/* Views of the model's arrays (owned by the model; valid until destroy). */
int hc3d_model_views(hc3d_model *m, hc3d_dust_tables *tables, hc3d_grid *grid, hc3d_run_params *params,
                     hc3d_model_info *info);

/* The small grains' emission spectra and ISRF integral of a model with FSG >
 * 0 (HC3D_ERR_STATE otherwise), owned by the model. */
int hc3d_model_sg_tables(hc3d_model *m, hc3d_sg_tables *sg);

/* Load the model into a context: its species map, dust tables, grid and,
 * with small grains, their spectra (hc3d_set_species, hc3d_load_tables,
 * hc3d_load_grid, hc3d_load_sg_tables). */
int hc3d_model_load(hc3d_model *m, hc3d_ctx *ctx);

/* Replace the model's tdust (nrg,ntg,npg,ndg), e.g. after hc3d_lucy_update. */
int hc3d_model_set_tdust(hc3d_model *m, const double *tdust);

/* The densities of gridset (gridset.f90:954-1098: disk mass normalisation,
 * densdisk, densenv, the fractal factor -- its clump centres and clump
 * radius too --, cell volumes and (rho V)^(1/4)) on
 * CUDA device `device`, replacing the host-built densarr, massarr, vcell and
 * the grid masses of the model.  *ms receives the device time of the
 * kernels.  Every disk structure option (CGAPD, CSPIRAL, CDISKWARP, CRIMPUFF,
 * CGAPPUFF, CRIMCURVE, CGAPCURVE, CRADEXP) and the envelope gap (CGAPE) are
 * built on the device. */
int hc3d_model_densities_gpu(hc3d_model *m, int device, double *ms, char *err, size_t errlen);

/* setemiss (dust.f90:394-474: the cumulative emissivity tables kapBint and
 * the Planck-mean factors kappap of every distinct dust table) on CUDA device
 * `device`, replacing the host-built kapBint and kappap of the model.  *ms
 * receives the device time of the kernels. */
int hc3d_model_tables_gpu(hc3d_model *m, int device, double *ms, char *err, size_t errlen);

/* The stellar packets ns of an iteration of np packets when a fraction
 * isrf_frac of the luminosity enters from outside (newdisktherm.F90:143-175,
 * without accretion): both shares rounded to the nearest integer, then ns
 * adjusted so that the shares add up to np.  isrf_frac = 0 gives np. */
int64_t hc3d_star_packets(double isrf_frac, int64_t np);

/* The packet shares of an iteration of np packets (newdisktherm.F90:143-175)
 * as the boundaries of hc3d_run_params: global ids < n_acc are accretion
 * packets, [n_acc, n_spot) hot-spot packets, [n_spot, n_star) stellar
 * packets and the rest external.  accfrac, accfrac2 and isrf_frac are the
 * luminosity fractions of hc3d_model_info.  The reference's loop tests
 * iphot < npacc, so its accretion share is npacc - 1 packets and the stellar
 * share one more than ns - npaccstar; the boundaries keep that. */
int hc3d_packet_split(double accfrac, double accfrac2, double isrf_frac, int64_t np, int64_t *n_acc,
                      int64_t *n_spot, int64_t *n_star);

typedef struct hc3d_tts_stats {
  int iterations;            /* Lucy iterations + the final one */
  int converged;
  double max_rel_change;     /* of the last Lucy update */
  double seconds_lucy;       /* wall time of the Lucy iterations */
  double seconds_final;      /* wall time of the final peeled iteration */
  int64_t packets_total;
  int64_t counters[16];      /* final iteration, see HC3D_CNT_* */
} hc3d_tts_stats;

/* program tts: run the whole model on the GPU and write the reference's
 * output files into out_dir (an existing directory): the ASCII files
 * (flux*.dat, peel_flux*.dat, e_ALL_*_img.dat, tmidplane*.dat, tave*.dat)
 * and the .unf grid files of hc3d_write_grid_unf. */
int hc3d_tts(const char *par_path, const char *par_dir, const char *out_dir, const hc3d_device_opts *opts,
             hc3d_tts_stats *stats, char *err, size_t errlen);

/* ---- model-run server -----------------------------------------------------
 * No counterpart in the reference, which runs one model per process.  A
 * server owns `slots` contexts on one device, each driven by a worker thread
 * with its own stream.  Submitted requests are queued; a worker builds the
 * model on the host, waits until the model's device footprint fits the HBM
 * budget, then runs the Lucy iterations and the peeled iteration of
 * newtts.F90:294-368 (no output files).  Runs of different slots overlap on
 * the device.  A request's result does not depend on what else runs. */
typedef struct hc3d_server hc3d_server;

typedef struct hc3d_server_opts {
  int device;          /* CUDA device ordinal */
  int precision;       /* HC3D_PREC_MIXED or HC3D_PREC_FP64 */
  int slots;           /* concurrent model runs, 1..64 */
  int64_t hbm_budget;  /* bytes of model footprints admitted at once; 0 = 80 % of free device memory */
} hc3d_server_opts;

typedef struct hc3d_request {
  const char *par_path;  /* the model's .par file */
  const char *par_dir;   /* overrides PARDIR when non-NULL */
  int n_lucy;            /* Lucy iterations; -1 = the model's NIMIN/NIMAX rule */
  int64_t np_lucy;       /* packets per Lucy iteration; 0 = the model's */
  int64_t np;            /* packets of the peeled iteration; 0 = NP */
  int npeel;             /* peel-off directions of the request; 0 = the model's */
  const double *thete, *phie; /* (npeel) radians */
} hc3d_request;

typedef struct hc3d_result {
  int status;            /* HC3D_OK or the first error */
  char err[256];
  double t_submit, t_admit, t_done; /* seconds since the server started */
  int64_t footprint_bytes;
  int64_t packets;       /* all iterations */
  int iterations;        /* Lucy iterations + 1 */
  double max_rel_change; /* of the last Lucy iteration */
  int nfreq, nmu, nph, nap, npeel;
  int64_t *si, *nums;    /* (nfreq,nmu,nph,nap,8) SED of the peeled iteration, si x stokes_scale */
  int64_t *ti, *numt;    /* (nfreq,npeel,nap,8) peeled SED, ti x stokes_scale */
  double stokes_scale;
} hc3d_result;

typedef struct hc3d_server_stats {
  int64_t budget_bytes, in_use_bytes, peak_in_use_bytes;
  int running, peak_running;
  int64_t queued, completed;
} hc3d_server_stats;

int hc3d_server_create(hc3d_server **s, const hc3d_server_opts *opts);
/* Queue a request (the strings and arrays are copied); *ticket identifies it. */
int hc3d_server_submit(hc3d_server *s, const hc3d_request *req, int64_t *ticket);
/* Block until the request is done; the result's arrays are allocated for the
 * caller and freed by hc3d_result_free.  Returns the request's status, or
 * HC3D_ERR_INVALID for a ticket that was not issued or was already waited
 * for (one wait per ticket). */
int hc3d_server_wait(hc3d_server *s, int64_t ticket, hc3d_result *out);
void hc3d_result_free(hc3d_result *r);
/* Cancel a request (no counterpart in the reference): a queued request is
 * dropped at once; a running one stops before its next iteration, so no
 * kernel of it is in flight when it ends.  Its wait then returns
 * HC3D_ERR_CANCELLED.  Returns HC3D_ERR_STATE when the request has already
 * finished (its result stands) and HC3D_ERR_INVALID for an unknown or
 * already-waited ticket. */
int hc3d_server_cancel(hc3d_server *s, int64_t ticket);
int hc3d_server_get_stats(hc3d_server *s, hc3d_server_stats *st);
/* Finish the queued requests, then release the slots. */
void hc3d_server_destroy(hc3d_server *s);
/* Device bytes a run of the model holds, as the server's admission counts them. */
int64_t hc3d_model_footprint(const hc3d_model *m);

/* diskflux (flux.f90:23-121) and the ASCII writers of output
 * (output.F90:166-503) for tallies the host holds, e.g. after summing the
 * tallies of several ranks: flux*.dat, peel_flux*.dat, e_ALL_*_img.dat
 * (when params->image), tmidplane*.dat and tave*.dat into out_dir.  The
 * tally pointers follow hc3d_tallies (nabs .. dbig are not read); tdust_used
 * and tdust are the (nrg,ntg,npg,ndg) temperatures before and after the
 * last Lucy update.  hc3d_tts calls the same writer. */
int hc3d_write_outputs(const hc3d_model *m, const hc3d_run_params *params, const hc3d_tallies *tallies,
                       const double *tdust_used, const double *tdust, const char *out_dir);

/* output_grid (output.F90:38-150): a Fortran unformatted sequential .unf
 * file (4-byte record lengths around each record) holding the cell counts
 * and lastdim, the cell-centre radii (AU), polar and azimuthal angles, and
 * the array over the cells for id = 1..lastdim.  Exactly one of real_array
 * (real*8) and int_array (integer) is given, shaped (nrg,ntg,npg,lastdim) in
 * Fortran order.  hc3d_tts writes the reference's set: marr, darr, darrtot,
 * tarr, darr_000, diffus, diffdir after the set-up and diffus_NNN,
 * diffdir_NNN, killed_NNN after each iteration. */
int hc3d_write_grid_unf(const hc3d_model *m, const char *path, int lastdim, const double *real_array,
                        const int32_t *int_array);

/* Write a synthetic 7-column dust file (dustinit's format, dust.f90:336)
 * and a 2-column stellar wavelength grid (atmosinit's format,
 * starbarb.f90:24-36): the fixtures of the benchmark models. */
int hc3d_write_synthetic_dust(const char *path);
int hc3d_write_wavelength_grid(const char *path, double tstar_k);
/* Write a synthetic external radiation field in the ISRF_FILE format:
 * three diluted blackbodies (Mathis, Mezger & Panagia 1983 form). */
int hc3d_write_synthetic_isrf(const char *path);
/* Write 18 synthetic small-grain emission spectra emit_draine_<U>.dat into
 * directory dir (draine_cdf.f90's files and format: 1000 rows of lambda [um]
 * and j_nu, lambda increasing): a PAH band set and a warm continuum whose
 * temperature rises with U. */
int hc3d_write_synthetic_draine(const char *dir);

#ifdef __cplusplus
}
#endif
#endif
