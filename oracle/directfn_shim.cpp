// C entry points over the reference's DIRECTFN singular surface-surface
// integrals (create_ST / create_EA / create_VA of its Cpp_Assembly, called by
// singular_{ST,EA,VA}_lin.m through the solve_*_mex gateways), for the
// oracle's checks of the near zone.  TEST INFRASTRUCTURE ONLY: built from the
// reference's own sources into oracle/_ref by oracle/Makefile.
//
// Point conventions (Geometry::ST/EA/VA of the reference's classes.h):
//  ST: one square r1 r2 r3 r4 (cyclic), observation = source;
//  EA: observation square (r4, r3, r6, r5), source square (r3, r4, r1, r2),
//      shared edge r3-r4;
//  VA: observation (r3, r5, r6, r7), source (r3, r4, r1, r2), shared vertex r3.
// ker: DIRECTFN kernel type (1: T_l(r) B_l'(r') e^{-ik0R}/(4 pi R) with
// l = lp = 0 the plain Green function); N: 1D order of each of its four
// quadratures.
#include <complex>

#include "directfn.h"

extern "C" {

void oracle_directfn_st(const double* r1, const double* r2, const double* r3, const double* r4, int N, double k0,
                        double dx, const double* c_src, const double* c_obs, const double* n_src,
                        const double* n_obs, int ker, int l, int lp, double* out) {
  double cq[3], cp[3], nq[3], np[3];
  for (int i = 0; i < 3; ++i) { cq[i] = c_src[i]; cp[i] = c_obs[i]; nq[i] = n_src[i]; np[i] = n_obs[i]; }
  std::complex<double> I[1];
  create_ST(r1, r2, r3, r4, N, N, N, N, k0, dx, cq, cp, nq, np, ker, l, lp, I);
  out[0] = I[0].real();
  out[1] = I[0].imag();
}

void oracle_directfn_ea(const double* r1, const double* r2, const double* r3, const double* r4, const double* r5,
                        const double* r6, int N, double k0, double dx, const double* c_src, const double* c_obs,
                        const double* n_src, const double* n_obs, int ker, int l, int lp, double* out) {
  double cq[3], cp[3], nq[3], np[3];
  for (int i = 0; i < 3; ++i) { cq[i] = c_src[i]; cp[i] = c_obs[i]; nq[i] = n_src[i]; np[i] = n_obs[i]; }
  std::complex<double> I[1];
  create_EA(r1, r2, r3, r4, r5, r6, N, N, N, N, k0, dx, cq, cp, nq, np, ker, l, lp, I);
  out[0] = I[0].real();
  out[1] = I[0].imag();
}

void oracle_directfn_va(const double* r1, const double* r2, const double* r3, const double* r4, const double* r5,
                        const double* r6, const double* r7, int N, double k0, double dx, const double* c_src,
                        const double* c_obs, const double* n_src, const double* n_obs, int ker, int l, int lp,
                        double* out) {
  double cq[3], cp[3], nq[3], np[3];
  for (int i = 0; i < 3; ++i) { cq[i] = c_src[i]; cp[i] = c_obs[i]; nq[i] = n_src[i]; np[i] = n_obs[i]; }
  std::complex<double> I[1];
  create_VA(r1, r2, r3, r4, r5, r6, r7, N, N, N, N, k0, dx, cq, cp, nq, np, ker, l, lp, I);
  out[0] = I[0].real();
  out[1] = I[0].imag();
}

}  // extern "C"
