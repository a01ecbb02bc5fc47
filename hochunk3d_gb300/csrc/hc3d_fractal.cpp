// hc3d_fractal.cpp -- the project fractal generator of the host build.
// Compiled without contracted multiply-adds (-ffp-contract=off), so that its
// products and sums round one by one, as the device build of the same factor
// (hc3d_gridbuild.cu) rounds them: both mark the same cells.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "hc3d_model.h"

namespace hc3d {

// ---------------------------------------------------------------------------
// The project fractal generator (CFRACTAL=YES; the reference's fractal_sph is
// not reproduced): fractlev levels of hierarchical clumps, fractn level-1
// centres in cell-index space and fractn/8+1 children per parent, each level
// closer to its parent.  Clump cells get density factor a, the rest b, with
// a/b = fractcontrast, the cell average of the factor 1 (the normalisation of
// gridset.f90:842-851) and a share densratio of the mass in clumps; the clump
// radius is set by bisection to the volume fraction these imply.
// ---------------------------------------------------------------------------

// the final level's clump centres, x = r, t, p in cell-index space, three per centre
std::vector<double> fractal_points(const Model& m) {
  const int total = fractal_total(m.fractn, m.fractlev);
  std::vector<double> buf(3 * (size_t)total);
  const int n = fractal_generate(m.nrg - 1, m.ntg - 1, m.npg - 1, m.fractn, m.fractlev, m.ifseed, buf.data());
  int last = m.fractn;
  for (int lev = 2; lev <= m.fractlev; ++lev) last *= m.fractn / 8 + 1;
  return std::vector<double>(buf.begin() + 3 * (size_t)(n - last), buf.begin() + 3 * (size_t)n);
}

// the bisection's target volume fraction, and the factors a (clumps), b (the rest) of a volume fraction fv
double fractal_target(const Model& m) {
  const double K = m.fractcontrast, fm = m.densratio;
  return fm / (K * (1.0 - fm) + fm);
}
void fractal_factors(const Model& m, double fv, double* a, double* b) {
  const double K = m.fractcontrast;
  *b = 1.0 / (K * fv + 1.0 - fv);
  *a = K * *b;
}

void fractal_field(Model* m) {
  const int nr = m->nrg - 1, nt = m->ntg - 1, np = m->npg - 1;
  const int64_t nc = (int64_t)nr * nt * np;
  const std::vector<double> cur = fractal_points(*m);
  std::vector<uint8_t> in(nc, 0);
  auto mark = [&](double rad) {
    std::fill(in.begin(), in.end(), 0);
    int64_t count = 0;
    for (size_t c = 0; c < cur.size(); c += 3) {
      const FractalBox B = fractal_box(nr, nt, np, rad, cur[c], cur[c + 1], cur[c + 2]);
      for (int ir = B.r0; ir <= B.r1; ++ir)
        for (int it = B.t0; it <= B.t1; ++it)
          for (int ipp = B.p0; ipp <= B.p1; ++ipp) {
            const int ip = ((ipp % np) + np) % np;
            if (fractal_inside(B, ir, it, ipp, cur[c], cur[c + 1], cur[c + 2])) {
              const int64_t k = ir + (int64_t)nr * (it + (int64_t)nt * ip);
              if (!in[k]) { in[k] = 1; ++count; }
            }
          }
    }
    return count;
  };
  const double fv_target = fractal_target(*m);
  double lo = 0.0, hi = 0.5;
  for (int k = 0; k < 30; ++k) {
    double mid = 0.5 * (lo + hi);
    if ((double)mark(mid) / (double)nc < fv_target) lo = mid; else hi = mid;
  }
  const double fv = std::max((double)mark(hi) / (double)nc, 1.0 / (double)nc);
  double a, b;
  fractal_factors(*m, fv, &a, &b);
  m->densvar.assign(nc, 1.0);
  for (int64_t k = 0; k < nc; ++k) m->densvar[k] = in[k] ? a : b;
}

}  // namespace hc3d
