// Host-side additions to the Green's-tensor assembly (no CUDA): compiled
// into the library by assembly.cu and, for CPU tests, by a g++ shim.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <vector>

namespace marie {
namespace green_host {

// (l, l') of the ten moment products (VV_Nop.m:27-28), 0 = the constant
constexpr int kL10[10] = {0, 1, 2, 3, 0, 0, 0, 1, 1, 2};
constexpr int kLp10[10] = {0, 1, 2, 3, 1, 2, 3, 2, 3, 3};

// The point term of the N kernel at the self offset: its six components are
// those of curl curl (g I), and as distributions d_p d_q g = PV(...) -
// (1/3) delta_pq delta(r), lap g = -k0^2 g - delta(r), so curl curl (g I) =
// PV[pointwise kernel] + (2/3) delta_pq delta(r).  Over one voxel pair with
// moments [1, x/res, y/res, z/res] that adds (2/3) Gram_ll' (Gram = diag(res^3,
// res^3/12, res^3/12, res^3/12), the diagonal of mvp_G_pwl.m:5) to the xx, yy,
// zz components (k = 0, 3, 5) of I_V(0,0,0).  The surface-surface near zone
// of assembly_N.m:56-81 contains this term; the cubature of k_vv does not.
inline void add_self_point_term(double* out_host, int64_t nD, int pwx, double res) {
  const double r3 = res * res * res;
  for (int llp = 0; llp < pwx; ++llp) {
    if (kL10[llp] != kLp10[llp]) continue;
    const double g = (2.0 / 3.0) * (kL10[llp] == 0 ? r3 : r3 / 12.0);
    for (int k : {0, 3, 5}) out_host[2 * ((int64_t)(llp + pwx * k) * nD)] += g;   // (0,0,0) of block (llp, k)
  }
}

using cd = std::complex<double>;

// Gauss-Legendre rule on [0, 1] (Newton iteration on the Legendre recurrence).
inline void gauss01(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double z = std::cos(pi * (i + 0.75) / (n + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[n - 1 - i] = 0.5 * (z + 1.0);
    w[n - 1 - i] = 1.0 / ((1.0 - z * z) * dp * dp);   // 2/((1-z^2) P'^2) on [-1,1], halved on [0,1]
  }
}

// N kernel (the six components of curl curl (g I), G_N.m) or K kernel
// (grad g, G_K.m) at u = r - r'; k0 = 0 gives the static N kernel.
inline void kernel_at(bool isN, double x, double y, double z, double k0, cd* out) {
  const double R2 = x * x + y * y + z * z, R = std::sqrt(R2);
  const double R3 = R2 * R, R4 = R2 * R2, R5 = R4 * R;
  const cd ik(0.0, k0);
  const cd Gexp = std::exp(-ik * R) / (4.0 * 3.14159265358979323846);
  if (!isN) {
    const cd f = Gexp * (1.0 / R3 + ik / R2);
    out[0] = -x * f;
    out[1] = -y * f;
    out[2] = -z * f;
    return;
  }
  const double k2 = k0 * k0;
  auto dd = [&](double a) { return Gexp * (3.0 * a * a / R5 + 3.0 * ik * a * a / R4 - (1.0 + k2 * a * a) / R3 - ik / R2); };
  auto od = [&](double a, double b) { return Gexp * (3.0 * a * b / R5 + 3.0 * ik * a * b / R4 - k2 * a * b / R3); };
  const cd Gxx = dd(x), Gyy = dd(y), Gzz = dd(z);
  out[0] = -Gyy - Gzz;
  out[1] = od(x, y);
  out[2] = od(x, z);
  out[3] = -Gxx - Gzz;
  out[4] = od(y, z);
  out[5] = -Gxx - Gyy;
}

// Per-axis moment overlap w_d(u): the integral over the source voxel's
// x' in [-res/2, res/2], with u + x' inside the observation voxel
// [m res - res/2, m res + res/2], of t(u + x' - m res) b(x'), where t and b
// are s/res on the moment's own axis and 1 otherwise (moments [1, x/res,
// y/res, z/res] of the voxel, VV_Nop.m:18-19).  Exact (quadratic integrand).
inline double moment_overlap(double u, int m, double res, bool l_axis, bool lp_axis) {
  const double lo = std::max(-res / 2, m * res - res / 2 - u);
  const double hi = std::max(lo, std::min(res / 2, m * res + res / 2 - u));
  const double a = l_axis ? (u - m * res) / res : 1.0, b = l_axis ? 1.0 / res : 0.0;
  const double c = lp_axis ? 0.0 : 1.0, d = lp_axis ? 1.0 / res : 0.0;
  const double A = a * c, B = a * d + b * c, C = b * d;
  return A * (hi - lo) + B * (hi * hi - lo * lo) / 2 + C * (hi * hi * hi - lo * lo * lo) / 3;
}

inline void moment_weights(const double u[3], const int m[3], double res, int pwx, double* W) {
  for (int llp = 0; llp < pwx; ++llp) {
    double v = 1.0;
    for (int d = 0; d < 3; ++d)
      v *= moment_overlap(u[d], m[d], res, kL10[llp] == d + 1, kLp10[llp] == d + 1);
    W[llp] = v;
  }
}

// I_V(m) of one near offset m in {0,1}^3, out[llp + pwx*c] (c < 6 for N, 3
// for K): the same integral as the volume cubature of the far zone and as
// the surface-surface near zone of assembly_N.m:56-81 / assembly_K.m:56-81,
// computed here in the relative coordinate u = r - r':
// I(m) = int K(u) W(u) du over prod_d [(m_d - 1) res, (m_d + 1) res], with W
// the moment overlap (piecewise polynomial, kinks at u_d = m_d res).  The box
// is split at the kinks and at 0, so the kernel's singular point u = 0 is a
// corner of every piece that touches it.  Pieces away from 0 take a tensor
// Gauss rule; pieces with that corner take three Duffy pyramids u = t (L_e,
// L_f v, L_g w) (Jacobian L^3 t^2), which cancels the 1/R^2 singularity of K
// and of the dynamic part of N.  The static part K_s of N (homogeneous of
// degree -3) is integrated as K_s(u/t) (W(u) - W(0)) / t; the remaining
// W(0) K_s / t sums to zero over the eight pieces around u = 0 of the self
// offset (the principal value over a cube, by cubic symmetry) and W(0) = 0
// for the other offsets.  The self offset of N then gets the point term of
// the kernel (add_self_point_term).
inline void near_zone_offset(bool isN, double k0, double res, int pwx, const int m[3], int order, cd* out) {
  const int nc = isN ? 6 : 3;
  std::vector<double> gx, gw;
  gauss01(order, gx, gw);
  for (int q = 0; q < pwx * nc; ++q) out[q] = 0.0;
  double lo[3][2], hi[3][2];
  for (int d = 0; d < 3; ++d) {
    lo[d][0] = m[d] == 0 ? -res : 0.0;
    hi[d][0] = m[d] == 0 ? 0.0 : res;
    lo[d][1] = m[d] == 0 ? 0.0 : res;
    hi[d][1] = m[d] == 0 ? res : 2 * res;
  }
  const double zero[3] = {0.0, 0.0, 0.0};
  double W0[10], W[10];
  moment_weights(zero, m, res, pwx, W0);
  cd Kf[6], Ks[6], Kt[6];
  for (int bx = 0; bx < 2; ++bx)
    for (int by = 0; by < 2; ++by)
      for (int bz = 0; bz < 2; ++bz) {
        const int sel[3] = {bx, by, bz};
        double L[3], a[3], sg[3];
        bool corner = true;
        for (int d = 0; d < 3; ++d) {
          a[d] = lo[d][sel[d]];
          L[d] = hi[d][sel[d]] - a[d];
          if (!(lo[d][sel[d]] == 0.0 || hi[d][sel[d]] == 0.0)) corner = false;
          sg[d] = hi[d][sel[d]] > 0.0 ? 1.0 : -1.0;
        }
        const double vol = L[0] * L[1] * L[2];
        if (!corner) {
          for (int i = 0; i < order; ++i)
            for (int j = 0; j < order; ++j)
              for (int k = 0; k < order; ++k) {
                const double u[3] = {a[0] + L[0] * gx[i], a[1] + L[1] * gx[j], a[2] + L[2] * gx[k]};
                const double wt = gw[i] * gw[j] * gw[k] * vol;
                kernel_at(isN, u[0], u[1], u[2], k0, Kf);
                moment_weights(u, m, res, pwx, W);
                for (int c = 0; c < nc; ++c)
                  for (int l = 0; l < pwx; ++l) out[l + pwx * c] += wt * W[l] * Kf[c];
              }
          continue;
        }
        for (int e = 0; e < 3; ++e) {
          const int f = (e + 1) % 3, g = (e + 2) % 3;
          for (int i = 0; i < order; ++i)
            for (int j = 0; j < order; ++j)
              for (int k = 0; k < order; ++k) {
                const double t = gx[i];
                double ut[3];
                ut[e] = sg[e] * L[e];
                ut[f] = sg[f] * L[f] * gx[j];
                ut[g] = sg[g] * L[g] * gx[k];
                const double u[3] = {t * ut[0], t * ut[1], t * ut[2]};
                const double wq = gw[i] * gw[j] * gw[k];
                kernel_at(isN, u[0], u[1], u[2], k0, Kf);
                moment_weights(u, m, res, pwx, W);
                if (isN) {
                  kernel_at(true, u[0], u[1], u[2], 0.0, Ks);
                  kernel_at(true, ut[0], ut[1], ut[2], 0.0, Kt);
                  for (int c = 0; c < nc; ++c)
                    for (int l = 0; l < pwx; ++l)
                      out[l + pwx * c] += wq * vol * ((Kf[c] - Ks[c]) * (W[l] * t * t) + Kt[c] * ((W[l] - W0[l]) / t));
                } else {
                  for (int c = 0; c < nc; ++c)
                    for (int l = 0; l < pwx; ++l) out[l + pwx * c] += wq * vol * t * t * W[l] * Kf[c];
                }
              }
        }
      }
}

// Overwrite the near offsets {0,1}^3 of a dense I_V (n1, n2, n3, pwx, nc),
// interleaved complex, column-major, with near_zone_offset, and add the point
// term of N at the self offset.
inline void near_zone_exact(double* iv, int n1, int n2, int n3, double res, double k0, int pwx, bool isN,
                            int order = 16) {
  const int nc = isN ? 6 : 3;
  const int64_t nD = (int64_t)n1 * n2 * n3;
  std::vector<cd> v((size_t)pwx * nc);
  for (int mz = 0; mz < std::min(2, n3); ++mz)
    for (int my = 0; my < std::min(2, n2); ++my)
      for (int mx = 0; mx < std::min(2, n1); ++mx) {
        const int m[3] = {mx, my, mz};
        near_zone_offset(isN, k0, res, pwx, m, order, v.data());
        const int64_t base = mx + (int64_t)n1 * (my + (int64_t)n2 * mz);
        for (int c = 0; c < nc; ++c)
          for (int l = 0; l < pwx; ++l) {
            const cd z = v[l + pwx * c];
            iv[2 * (base + nD * (l + pwx * c))] = z.real();
            iv[2 * (base + nD * (l + pwx * c)) + 1] = z.imag();
          }
      }
  if (isN) add_self_point_term(iv, nD, pwx, res);   // I_V(0,0,0) only
}

}  // namespace green_host
}  // namespace marie
