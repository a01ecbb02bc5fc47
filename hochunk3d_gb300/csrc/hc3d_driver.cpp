// hc3d_driver.cpp -- program tts (newtts.F90:141-368) over the C-ABI:
// Lucy iterations, the final peeled iteration, diskflux (flux.f90:23-121)
// and the ASCII writers of output (output.F90:166-503).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/hc3d.h"
#include "../../include/hc3d_host.h"
#include "hc3d_model.h"

namespace {

using hc3d::Model;

struct Tallies {
  std::vector<int64_t> sed[9], psed[9], img[4];
  hc3d_tallies t;
};

void alloc_tallies(Tallies* T, const hc3d_run_params& p) {
  const int64_t nsed = (int64_t)p.nfreq * p.nmu * p.nph * p.nap * HC3D_NO;
  const int npeel = p.ipeel ? p.npeel : 0;
  const int64_t npsed = (int64_t)p.nfreq * npeel * p.nap * HC3D_NO;
  const int64_t nimg = (int64_t)npeel * p.nxhst * p.nxhst;
  std::memset(&T->t, 0, sizeof(T->t));
  for (int k = 0; k < 9; ++k) {
    T->sed[k].assign(nsed, 0);
    T->psed[k].assign(std::max<int64_t>(npsed, 1), 0);
  }
  for (int k = 0; k < 4; ++k) T->img[k].assign(std::max<int64_t>(nimg, 1), 0);
  int64_t** s[9] = {&T->t.si, &T->t.sq, &T->t.su, &T->t.sv, &T->t.si2, &T->t.sq2, &T->t.su2, &T->t.sv2, &T->t.nums};
  int64_t** q[9] = {&T->t.ti, &T->t.tq, &T->t.tu, &T->t.tv, &T->t.ti2, &T->t.tq2, &T->t.tu2, &T->t.tv2, &T->t.numt};
  int64_t** im[4] = {&T->t.image_i, &T->t.image_q, &T->t.image_u, &T->t.image_v};
  for (int k = 0; k < 9; ++k) {
    *s[k] = T->sed[k].data();
    *q[k] = T->psed[k].data();
  }
  for (int k = 0; k < 4; ++k) *im[k] = T->img[k].data();
}

// ES11.4 of Fortran: " d.ddddE+xx"
std::string es11(double v) {
  char buf[64];
  if (v == 0.0 || !std::isfinite(v)) {
    std::snprintf(buf, sizeof buf, "%11s", v == 0.0 ? "0.0000E+00" : "NaN");
    return buf;
  }
  std::snprintf(buf, sizeof buf, "%11.4E", v);
  return buf;
}

std::string f51(double v) {
  char buf[32];
  std::snprintf(buf, sizeof buf, "%5.1f", v);
  std::string s = buf;
  size_t b = s.find_first_not_of(' ');
  return s.substr(b);
}

const char* kSuffix[HC3D_NO] = {"", "_star", "_disk", "_enve", "_outi", "_dire", "_scat", "_ther"};

void write_sed_row(FILE* f, double wav, double fi, double fie, double fq, double fqe, double fu, double fue, double fv,
                   double fve) {
  std::fprintf(f, "%10.4f  %s  %s  %s  %s  %s  %s  %s  %s\n", wav, es11(fi).c_str(), es11(fie).c_str(),
               es11(fq).c_str(), es11(fqe).c_str(), es11(fu).c_str(), es11(fue).c_str(), es11(fv).c_str(),
               es11(fve).c_str());
}

const char* kSedHeader =
    "# Lambda         I          I_err         Q/I       (Q/I)_err       U/I       (U/I)_err       V/I       (V/I)_err\n";

// diskflux (flux.f90:23-121) + output (output.F90:166-503), ASCII part
int write_outputs(const Model& m, const hc3d_run_params& p, const hc3d_tallies& t, const double* tdust_used,
                  const double* tdust2, const std::string& dir) {
  // the nine SED and peeled-SED arrays and the four images, in hc3d_tallies order
  const int64_t* sed[9] = {t.si, t.sq, t.su, t.sv, t.si2, t.sq2, t.su2, t.sv2, t.nums};
  const int64_t* psed[9] = {t.ti, t.tq, t.tu, t.tv, t.ti2, t.tq2, t.tu2, t.tv2, t.numt};
  const int64_t* img[4] = {t.image_i, t.image_q, t.image_u, t.image_v};
  for (int k = 0; k < 9; ++k)
    if (!sed[k] || (p.ipeel && !psed[k])) return HC3D_ERR_INVALID;
  for (int k = 0; k < 4; ++k)
    if (p.ipeel && p.image && !img[k]) return HC3D_ERR_INVALID;
  if (!tdust_used || !tdust2) return HC3D_ERR_INVALID;
  const double lsol = hc3d::kLsun;
  const double rnp = (double)p.np;
  const double rnorm = rnp / (double)p.nmu / (double)p.nph / (m.ltot / lsol);
  const double image_norm = rnp / (m.ltot / lsol);
  const double nurat = m.numax / m.numin;
  const double nunorm = std::pow(nurat, 0.5 / p.nfreq) - std::pow(nurat, -0.5 / p.nfreq);
  const double ss = t.stokes_scale, sq = t.square_scale;
  std::vector<double> wav(p.nfreq);
  for (int i = 0; i < p.nfreq; ++i) wav[i] = 1.2398 / (m.numin * std::pow(nurat, ((double)(i + 1) - 0.5) / p.nfreq));
  // ---- flux*.dat ----
  const int64_t nsed = (int64_t)p.nfreq * p.nmu * p.nph * p.nap;
  for (int io = 0; io < HC3D_NO; ++io) {
    std::string fn = dir + "/flux" + kSuffix[io] + ".dat";
    FILE* f = std::fopen(fn.c_str(), "w");
    if (!f) return HC3D_ERR_IO;
    std::fprintf(f, " %11d %11d %11d %11d    nfreq,nph,nmu,nap\n", p.nfreq, p.nph, p.nmu, p.nap);
    std::fputs(kSedHeader, f);
    for (int ia = 0; ia < p.nap; ++ia)
      for (int i = 0; i < p.nmu; ++i)
        for (int ip = 0; ip < p.nph; ++ip)
          for (int inub = 0; inub < p.nfreq; ++inub) {
            const int64_t b = inub + (int64_t)p.nfreq * (i + (int64_t)p.nmu * (ip + (int64_t)p.nph * ia)) + nsed * io;
            const double n = (double)sed[8][b];
            double si = sed[0][b] / ss, sQ = sed[1][b] / ss, sU = sed[2][b] / ss, sV = sed[3][b] / ss;
            double e[4] = {0, 0, 0, 0};
            if (n > 1.0) {
              const double s2[4] = {sed[4][b] / sq, sed[5][b] / sq, sed[6][b] / sq, sed[7][b] / sq};
              const double s1[4] = {si, sQ, sU, sV};
              for (int k = 0; k < 4; ++k) {
                double var = (s2[k] - s1[k] * s1[k] / n) / (n - 1.0) * n;
                e[k] = std::sqrt(std::max(var, 0.0)) / si;
              }
              e[0] += 1.0 / n;
            }
            si /= rnorm; sQ /= rnorm; sU /= rnorm; sV /= rnorm;
            if (si == 0.0) write_sed_row(f, wav[inub], 0, 0, 0, 0, 0, 0, 0, 0);
            else
              write_sed_row(f, wav[inub], si / nunorm, e[0] * si / nunorm, sQ / si, e[1], sU / si, e[2], sV / si, e[3]);
          }
    std::fclose(f);
  }
  // ---- peel_flux*.dat and images ----
  if (p.ipeel) {
    const int64_t npsed = (int64_t)p.nfreq * p.npeel * p.nap;
    for (int io = 0; io < HC3D_NO; ++io)
      for (int k = 0; k < p.npeel; ++k) {
        std::string fn = dir + "/peel_flux" + kSuffix[io] + "_" + f51(m.thete[k] * 180.0 / hc3d::kPi) + "_" +
                         f51(m.phie[k] * 180.0 / hc3d::kPi) + ".dat";
        FILE* f = std::fopen(fn.c_str(), "w");
        if (!f) return HC3D_ERR_IO;
        std::fprintf(f, " %11d %11d %11d    nfreq,npeel,nap\n", p.nfreq, p.npeel, p.nap);
        std::fputs(kSedHeader, f);
        for (int ia = 0; ia < p.nap; ++ia)
          for (int inub = 0; inub < p.nfreq; ++inub) {
            const int64_t b = inub + (int64_t)p.nfreq * (k + (int64_t)p.npeel * ia) + npsed * io;
            const double n = (double)psed[8][b];
            double t1[4] = {psed[0][b] / ss, psed[1][b] / ss, psed[2][b] / ss, psed[3][b] / ss};
            double e[4] = {0, 0, 0, 0};
            if (n > 1.0)
              for (int q = 0; q < 4; ++q) {
                const double t2 = psed[4 + q][b] / sq;
                const double var = t1[q] != 0.0 ? (t2 * n / (t1[q] * t1[q]) - 1.0) / (n - 1.0) : 0.0;
                e[q] = std::sqrt(std::max(var, 0.0));
              }
            for (int q = 0; q < 4; ++q) t1[q] /= image_norm;
            if (t1[0] == 0.0) write_sed_row(f, wav[inub], 0, 0, 0, 0, 0, 0, 0, 0);
            else
              write_sed_row(f, wav[inub], t1[0] / nunorm, e[0] * t1[0] / nunorm, t1[1] / t1[0], e[1], t1[2] / t1[0],
                            e[2], t1[3] / t1[0], e[3]);
          }
        std::fclose(f);
      }
    if (p.image) {
      const double pc2cm = hc3d::kPc;
      const double image_norm_intensity = rnp / m.ltot * 4.0 * hc3d::kPi / 1.e17 *
                                          std::pow(2.0 * m.rmaxi / m.autors / (double)p.nxhst, 2.0) * pc2cm * pc2cm /
                                          std::pow(206265.0, 2.0);
      const int nx = p.nxhst;
      for (int k = 0; k < p.npeel; ++k) {
        const char* st[4] = {"I", "Q", "U", "V"};
        for (int q = 0; q < 4; ++q) {
          std::string fn = dir + "/e_ALL_" + f51(m.thete[k] * 180.0 / hc3d::kPi) + "_" +
                           f51(m.phie[k] * 180.0 / hc3d::kPi) + "_" + st[q] + "_img.dat";
          FILE* f = std::fopen(fn.c_str(), "w");
          if (!f) return HC3D_ERR_IO;
          for (int iy = 0; iy < nx; ++iy) {
            for (int ix = 0; ix < nx; ++ix) {
              const int64_t b = k + (int64_t)p.npeel * (ix + (int64_t)nx * iy);
              const double I = img[0][b] / ss;
              double v;
              if (q == 0) v = I / image_norm_intensity;
              else v = I > 0.0 ? (img[q][b] / ss) / I : 0.0;
              std::fprintf(f, "%s ", es11(v).c_str());
            }
            std::fputc('\n', f);
          }
          std::fclose(f);
        }
      }
    }
  }
  // ---- tmidplane*.dat, tave*.dat ----
  const int64_t n4 = m.n4();
  const int it = (m.ntg + 1) / 2;
  // midplane radial optical depth at V from the star to each cell's outer wall
  std::vector<double> tauarr(m.nrg, 0.0);
  {
    double tau = 0.0;
    const double rcm = m.rstar * hc3d::kRsun;
    for (int ir = 1; ir < m.nrg; ++ir) {
      const int64_t c4 = (int64_t)(ir - 1) + (int64_t)m.nrg * (it - 1);
      for (int s = 0; s < m.ndg; ++s) tau += m.densarr[c4 + n4 * s] * m.kappav[s] * rcm * (m.rarr[ir] - m.rarr[ir - 1]);
      tauarr[ir - 1] = tau;
    }
  }
  for (int s = 0; s < m.ndg; ++s) {
    char fn[512];
    std::snprintf(fn, sizeof fn, "%s/tmidplane%d.dat", dir.c_str(), s + 1);
    FILE* f = std::fopen(fn, "w");
    if (!f) return HC3D_ERR_IO;
    std::fprintf(f, "%9.5f / theta angle at which these values are quoted\n", m.thetarr[it - 1] * 180.0 / hc3d::kPi);
    std::fprintf(f, "%15sr(rstar)%9sr(au)%11stau%8sTdust%5sTdust2\n", "", "", "", "", "");
    for (int ir = 1; ir < m.nrg; ++ir) {
      const int64_t c4 = (int64_t)(ir - 1) + (int64_t)m.nrg * (it - 1) + n4 * s;
      std::fprintf(f, "%6d %15.5f %15.5f %15.5f %10.5f %10.5f\n", ir, m.ravearr[ir - 1], m.ravearr[ir - 1] / m.autors,
                   tauarr[ir - 1], tdust_used[c4] * 11605.0, tdust2[c4] * 11605.0);
    }
    std::fclose(f);
    std::snprintf(fn, sizeof fn, "%s/tave%d.dat", dir.c_str(), s + 1);
    f = std::fopen(fn, "w");
    if (!f) return HC3D_ERR_IO;
    std::fprintf(f, " r(rstar),r(au),  Tave, Tave2\n");
    for (int ir = 1; ir < m.nrg; ++ir) {
      double t1 = 0, t2 = 0, cnt = 0;
      for (int jt = 1; jt < m.ntg; ++jt)
        for (int jp = 1; jp < m.npg; ++jp) {
          const int64_t c4 = (int64_t)(ir - 1) + (int64_t)m.nrg * ((jt - 1) + (int64_t)m.ntg * (jp - 1)) + n4 * s;
          t1 += tdust_used[c4];
          t2 += tdust2[c4];
          cnt += 1.0;
        }
      std::fprintf(f, "%10d %15.5f %15.5f %10.5f %10.5f\n", ir, m.ravearr[ir - 1], m.ravearr[ir - 1] / m.autors,
                   t1 / cnt * 11605.0, t2 / cnt * 11605.0);
    }
    std::fclose(f);
  }
  return HC3D_OK;
}

// output_grid (output.F90:38-150): a Fortran unformatted sequential file,
// each record framed by its length in a 4-byte integer before and after it:
// the cell counts and lastdim, the cell-centre radii in AU, the polar and
// azimuthal cell centres, then the array over the cells (ir fastest) for
// id = 1..lastdim.  real8 (8-byte) or integer (4-byte) arrays, (nrg, ntg, npg,
// lastdim) in Fortran order; the wall entries (ir = nrg, ...) are skipped.
int write_grid_unf(const Model& m, const std::string& path, int lastdim, const double* r8, const int32_t* i4) {
  if (lastdim < 1 || (!r8 && !i4) || (r8 && i4)) return HC3D_ERR_INVALID;
  const int64_t nc = m.ncells(), n4 = m.n4();
  const int64_t body = nc * lastdim * (r8 ? 8 : 4);
  if (body > 0x7fffffffLL) return HC3D_ERR_UNSUPPORTED;  // would need Fortran subrecords
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return HC3D_ERR_IO;
  bool ok = true;
  auto rec = [&](const void* d, int64_t bytes) {
    const uint32_t nb = (uint32_t)bytes;
    ok = ok && std::fwrite(&nb, 4, 1, f) == 1 && (bytes == 0 || std::fwrite(d, 1, (size_t)bytes, f) == (size_t)bytes) &&
         std::fwrite(&nb, 4, 1, f) == 1;
  };
  const int32_t dims[4] = {m.nrg - 1, m.ntg - 1, m.npg - 1, lastdim};
  rec(dims, sizeof dims);
  std::vector<double> v((size_t)std::max(m.nrg, std::max(m.ntg, m.npg)));
  for (int i = 0; i < m.nrg - 1; ++i) v[i] = m.ravearr[i] / m.autors;
  rec(v.data(), 8LL * (m.nrg - 1));
  for (int i = 0; i < m.ntg - 1; ++i) v[i] = m.thetavearr[i];
  rec(v.data(), 8LL * (m.ntg - 1));
  for (int i = 0; i < m.npg - 1; ++i) v[i] = 0.5 * (m.phiarr[i] + m.phiarr[i + 1]);  // phiavearr, gridset.f90:654
  rec(v.data(), 8LL * (m.npg - 1));
  std::vector<unsigned char> buf((size_t)body);
  int64_t k = 0;
  for (int id = 0; id < lastdim; ++id)
    for (int ip = 0; ip < m.npg - 1; ++ip)
      for (int it = 0; it < m.ntg - 1; ++it)
        for (int ir = 0; ir < m.nrg - 1; ++ir, ++k) {
          const int64_t c4 = ir + (int64_t)m.nrg * (it + (int64_t)m.ntg * ip) + n4 * id;
          if (r8) std::memcpy(&buf[(size_t)k * 8], &r8[c4], 8);
          else std::memcpy(&buf[(size_t)k * 4], &i4[c4], 4);
        }
  rec(buf.data(), body);
  ok = std::fclose(f) == 0 && ok;
  return ok ? HC3D_OK : HC3D_ERR_IO;
}

// The grid files of gridset (gridset.f90:1577-1586): marr (rho V), darr,
// darrtot, tarr, darr_000, diffus and diffdir (all zero: no diffusion here).
int write_setup_grids(const Model& m, const std::string& dir) {
  const int64_t n4 = m.n4();
  std::vector<double> rhov((size_t)n4 * m.ndg), tot((size_t)n4, 0.0);
  for (size_t k = 0; k < rhov.size(); ++k) rhov[k] = std::pow(m.massarr[k], 4.0);
  for (int s = 0; s < m.ndg; ++s)
    for (int64_t k = 0; k < n4; ++k) tot[(size_t)k] += m.densarr[(size_t)(k + n4 * s)];
  const std::vector<int32_t> zero((size_t)n4, 0);
  int r;
  if ((r = write_grid_unf(m, dir + "/marr.unf", m.ndg, rhov.data(), nullptr)) ||
      (r = write_grid_unf(m, dir + "/darr.unf", m.ndg, m.densarr.data(), nullptr)) ||
      (r = write_grid_unf(m, dir + "/darrtot.unf", 1, tot.data(), nullptr)) ||
      (r = write_grid_unf(m, dir + "/tarr.unf", m.ndg, m.tdust.data(), nullptr)) ||
      (r = write_grid_unf(m, dir + "/darr_000.unf", m.ndg, m.densarr.data(), nullptr)) ||
      (r = write_grid_unf(m, dir + "/diffus.unf", 1, nullptr, zero.data())) ||
      (r = write_grid_unf(m, dir + "/diffdir.unf", 1, nullptr, zero.data())))
    return r;
  return HC3D_OK;
}

// The grid files that disk() writes after each iteration
// (newdisktherm.F90:605-610): diffus_NNN, diffdir_NNN (zero) and killed_NNN.
int write_iteration_grids(const Model& m, hc3d_ctx* ctx, int iter, const std::string& dir) {
  const int64_t n4 = m.n4();
  std::vector<int32_t> killed((size_t)n4, 0);
  hc3d_tallies k;
  std::memset(&k, 0, sizeof k);
  k.killed = killed.data();
  int r = hc3d_get_tallies(ctx, nullptr, &k);
  if (r) return r;
  char suffix[16];
  std::snprintf(suffix, sizeof suffix, "_%03d", iter);
  const std::vector<int32_t> zero((size_t)n4, 0);
  if ((r = write_grid_unf(m, dir + "/diffus" + suffix + ".unf", 1, nullptr, zero.data())) ||
      (r = write_grid_unf(m, dir + "/diffdir" + suffix + ".unf", 1, nullptr, zero.data())) ||
      (r = write_grid_unf(m, dir + "/killed" + suffix + ".unf", 1, nullptr, killed.data())))
    return r;
  return HC3D_OK;
}

void put_err(char* err, size_t len, const std::string& s) {
  if (err && len) std::snprintf(err, len, "%s", s.c_str());
}

}  // namespace


extern "C" int hc3d_model_load(hc3d_model* hm, hc3d_ctx* ctx) {
  if (!hm || !ctx) return HC3D_ERR_INVALID;
  const Model& m = hm->m;
  int r;
  if ((r = hc3d_set_species(ctx, m.slot_species))) return r;
  hc3d_dust_tables tv = m.tables_view();
  hc3d_grid gv = m.grid_view();
  if ((r = hc3d_load_tables(ctx, &tv)) || (r = hc3d_load_grid(ctx, &gv))) return r;
  if (m.sg_slot >= 0) {
    hc3d_sg_tables sg;
    if ((r = hc3d_model_sg_tables(hm, &sg)) || (r = hc3d_load_sg_tables(ctx, &sg))) return r;
  }
  return HC3D_OK;
}

extern "C" int hc3d_tts(const char* par_path, const char* par_dir, const char* out_dir, const hc3d_device_opts* opts,
                        hc3d_tts_stats* stats, char* err, size_t errlen) {
  if (!par_path || !out_dir) return HC3D_ERR_INVALID;
  hc3d_model* hm = nullptr;
  int r = hc3d_model_create(&hm, par_path, par_dir, err, errlen);
  if (r) return r;
  Model& m = hm->m;
  hc3d_ctx* ctx = nullptr;
  hc3d_device_opts o;
  std::memset(&o, 0, sizeof o);
  if (opts) o = *opts;
  r = hc3d_create(&ctx, &o);
  if (r) {
    put_err(err, errlen, "hc3d_create failed (no CUDA device?)");
    hc3d_model_destroy(hm);
    return r;
  }
  auto bail = [&](int code) {
    char buf[512];
    hc3d_get_error(ctx, buf, sizeof buf);
    put_err(err, errlen, buf);
    hc3d_destroy(ctx);
    hc3d_model_destroy(hm);
    return code;
  };
  if ((r = hc3d_model_load(hm, ctx))) return bail(r);
  hc3d_run_params p = m.params_view();
  const int ipeelorig = p.ipeel;
  auto io_fail = [&](int code, const char* what) {
    put_err(err, errlen, std::string("cannot write ") + what + " into " + out_dir);
    hc3d_destroy(ctx);
    hc3d_model_destroy(hm);
    return code;
  };
  if ((r = write_setup_grids(m, out_dir))) return io_fail(r, "the gridset .unf files");
  hc3d_tts_stats st;
  std::memset(&st, 0, sizeof st);
  using clk = std::chrono::steady_clock;
  auto t0 = clk::now();
  // Lucy iterations (newtts.F90:294-330): no peeling, np_lucy packets
  bool converge = m.ilucy == 0;
  int iter = 0;
  std::vector<double> tdust_used(m.tdust), tdust2(m.tdust);
  while (!converge) {
    ++iter;
    p.np = m.np_lucy;
    m.set_shares(&p, p.np);
    p.ipeel = 0;
    p.iter = iter;
    if ((r = hc3d_zero_tallies(ctx)) || (r = hc3d_run_iteration(ctx, &p))) return bail(r);
    double rel = 0;
    int conv = 0;
    if ((r = hc3d_lucy_update(ctx, m.ltot, p.np, tdust2.data(), &rel, &conv))) return bail(r);
    if ((r = write_iteration_grids(m, ctx, iter, out_dir))) return io_fail(r, "the iteration .unf files");
    st.max_rel_change = rel;
    st.packets_total += p.np;
    converge = conv != 0;
    if (iter < m.nimin) converge = false;
    if (iter >= m.nimax) converge = true;
    tdust_used = tdust2;
  }
  st.converged = iter == 0 ? 1 : (st.max_rel_change < 0.01);
  auto t1 = clk::now();
  // final iteration (newtts.F90:333-368)
  ++iter;
  p.np = m.np;
  m.set_shares(&p, p.np);
  p.ipeel = ipeelorig;
  p.iter = iter;
  Tallies T;
  alloc_tallies(&T, p);
  if ((r = hc3d_zero_tallies(ctx)) || (r = hc3d_run_iteration(ctx, &p))) return bail(r);
  if ((r = hc3d_get_tallies(ctx, &p, &T.t))) return bail(r);
  double rel = 0;
  int conv = 0;
  if ((r = hc3d_lucy_update(ctx, m.ltot, p.np, tdust2.data(), &rel, &conv))) return bail(r);
  if ((r = write_iteration_grids(m, ctx, iter, out_dir))) return io_fail(r, "the iteration .unf files");
  auto t2 = clk::now();
  st.packets_total += p.np;
  st.iterations = iter;
  st.seconds_lucy = std::chrono::duration<double>(t1 - t0).count();
  st.seconds_final = std::chrono::duration<double>(t2 - t1).count();
  for (int k = 0; k < 16; ++k) st.counters[k] = T.t.counters[k];
  r = write_outputs(m, p, T.t, tdust_used.data(), tdust2.data(), out_dir);
  if (r) {
    put_err(err, errlen, std::string("cannot write outputs into ") + out_dir);
    hc3d_destroy(ctx);
    hc3d_model_destroy(hm);
    return r;
  }
  if (stats) *stats = st;
  hc3d_destroy(ctx);
  hc3d_model_destroy(hm);
  return HC3D_OK;
}

extern "C" int hc3d_write_outputs(const hc3d_model* hm, const hc3d_run_params* p, const hc3d_tallies* t,
                                  const double* tdust_used, const double* tdust, const char* out_dir) {
  if (!hm || !p || !t || !tdust_used || !tdust || !out_dir) return HC3D_ERR_INVALID;
  if (!(t->stokes_scale > 0.0) || !(t->square_scale > 0.0)) return HC3D_ERR_INVALID;
  if (p->nfreq < 1 || p->nmu < 1 || p->nph < 1 || p->nap < 1 || (p->ipeel && (p->npeel < 1 || !p->thete)))
    return HC3D_ERR_INVALID;
  return write_outputs(hm->m, *p, *t, tdust_used, tdust, out_dir);
}

extern "C" int hc3d_write_grid_unf(const hc3d_model* hm, const char* path, int lastdim, const double* real_array,
                                   const int32_t* int_array) {
  if (!hm || !path) return HC3D_ERR_INVALID;
  return write_grid_unf(hm->m, path, lastdim, real_array, int_array);
}
