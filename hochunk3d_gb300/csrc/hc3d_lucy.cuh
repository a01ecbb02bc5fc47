// hc3d_lucy.cuh -- the Lucy temperature of one cell and species, shared by
// every kernel that solves it: tfinal (the module is not shipped; restated as
// the fixed point of dusttemp.f90:30-50 with the absorbed-path estimator in
// place of the absorption count), with KapP (dust.f90:114-141).
#pragma once

#include <cuda_runtime.h>

namespace hc3d {

// KapP: Planck-mean kappa/kappa_V at T (K/11605), linear in log T.
__device__ __forceinline__ double lucy_kapp(const double* lTint, int nT, const double* kp, double T) {
  const double lT = log(T);
  const double l1 = lTint[0], lN = lTint[nT - 1];
  const int k = (int)((double)(nT - 1) * (lT - l1) / (lN - l1)) + 1;
  if (k < 1) return kp[0];
  if (k > nT - 1) return kp[nT - 1];
  const double f = (lT - lTint[k - 1]) / (lTint[k] - lTint[k - 1]);
  return (1.0 - f) * kp[k - 1] + f * kp[k];
}

// Energy balance 4 sigma T^4 kappa_V kappa_P(T) (rho V) = na L / N, iterated
// from T0 to 1e-5 relative (at most 1000 steps), clamped to [0.1, 1600] K.
__device__ __forceinline__ double lucy_dusttemp(const double* lTint, int nT, const double* kp, double kappav,
                                                double ltot, double nphot, double na, double T0, double massarr) {
  const double eps = 1.e-5, sigt = 5.670400e-5;
  double Td = T0 != 0.0 ? T0 : 0.1 / 11605.0;
  double Told = 0.5 * Td;
  int it = 0;
  while (fabs(Td - Told) > eps * Td && it < 1000) {
    ++it;
    Told = Td;
    Td = pow((na * ltot) / (4.0 * sigt * nphot * kappav * lucy_kapp(lTint, nT, kp, Td)), 0.25) / 11605.0;
    if (massarr > 0.0) Td = Td / massarr;
    else Td = 0.1 / 11605.0;
    if (Td > 1600.0 / 11605.0) Td = 1600.0 / 11605.0;
    if (Td < 0.1 / 11605.0) Td = 0.1 / 11605.0;
  }
  return Td;
}

}  // namespace hc3d
