// Host-side additions to the Green's-tensor assembly (no CUDA): compiled
// into the library by assembly.cu and, for CPU tests, by a g++ shim.
#pragma once

#include <cstdint>

namespace marie {
namespace green_host {

// The point term of the N kernel at the self offset: its six components are
// those of curl curl (g I), and as distributions d_p d_q g = PV(...) -
// (1/3) delta_pq delta(r), lap g = -k0^2 g - delta(r), so curl curl (g I) =
// PV[pointwise kernel] + (2/3) delta_pq delta(r).  Over one voxel pair with
// moments [1, x/res, y/res, z/res] that adds (2/3) Gram_ll' (Gram = diag(res^3,
// res^3/12, res^3/12, res^3/12), the diagonal of mvp_G_pwl.m:5) to the xx, yy,
// zz components (k = 0, 3, 5) of I_V(0,0,0).  The surface-surface near zone
// of assembly_N.m:56-81 contains this term; the cubature of k_vv does not.
inline void add_self_point_term(double* out_host, int64_t nD, int pwx, double res) {
  static const int kL[10] = {0, 1, 2, 3, 0, 0, 0, 1, 1, 2}, kLp[10] = {0, 1, 2, 3, 1, 2, 3, 2, 3, 3};
  const double r3 = res * res * res;
  for (int llp = 0; llp < pwx; ++llp) {
    if (kL[llp] != kLp[llp]) continue;
    const double g = (2.0 / 3.0) * (kL[llp] == 0 ? r3 : r3 / 12.0);
    for (int k : {0, 3, 5}) out_host[2 * ((int64_t)(llp + pwx * k) * nD)] += g;   // (0,0,0) of block (llp, k)
  }
}

}  // namespace green_host
}  // namespace marie
