// Producers of the hot path's operands, computed on the GPU in FP64:
//  - I_V of assembly_N.m:16-81 / assembly_K.m:16-81 (volume-volume Green's
//    tensor integrals per voxel offset, VV_Nop.m:1-48, VV_Kop.m:1-50,
//    G_N.m:3-19, G_K.m:3-13);
//  - incident fields of unit-current closed loops and of a plane wave, tested
//    onto the PWC/PWL basis (the loop right-hand sides).
#include "green_host.h"
#include <cmath>
#include <vector>

#include "internal.h"

namespace marie {

typedef cplx<double> zd;

struct Rule3 {          // tensor Gauss rule on [-1,1]^3, first variable fastest
  const double* x;      // np*3
  const double* w;      // np
  int np;
};

// G_N.m entries [-Gyy-Gzz, Gxy, Gxz, -Gxx-Gzz, Gyz, -Gxx-Gyy]
__device__ __forceinline__ void gn_kernel(double dx, double dy, double dz, double k0, zd* f) {
  const double R2 = dx * dx + dy * dy + dz * dz;
  const double R = sqrt(R2);
  const double iR = 1.0 / R;
  const double iR2 = iR * iR, iR3 = iR2 * iR, iR4 = iR2 * iR2, iR5 = iR4 * iR;
  double sn, cs;
  sincos(k0 * R, &sn, &cs);
  const double q = 0.25 / 3.14159265358979323846;
  const zd Ge = {cs * q, -sn * q};                 // exp(-i k0 R)/(4 pi)
  const double k2 = k0 * k0;
  // diag: 3d^2/R^5 + 3i k0 d^2/R^4 - (1 + k0^2 d^2)/R^3 - i k0/R^2
  auto diag = [&](double d) -> zd {
    return zd{3 * d * d * iR5 - (1 + k2 * d * d) * iR3, 3 * k0 * d * d * iR4 - k0 * iR2};
  };
  auto off = [&](double a, double b) -> zd {
    return zd{3 * a * b * iR5 - k2 * a * b * iR3, 3 * k0 * a * b * iR4};
  };
  const zd xx = Ge * diag(dx), yy = Ge * diag(dy), zz = Ge * diag(dz);
  f[0] = zd{-(yy.x + zz.x), -(yy.y + zz.y)};
  f[1] = Ge * off(dx, dy);
  f[2] = Ge * off(dx, dz);
  f[3] = zd{-(xx.x + zz.x), -(xx.y + zz.y)};
  f[4] = Ge * off(dy, dz);
  f[5] = zd{-(xx.x + yy.x), -(xx.y + yy.y)};
}

// G_K.m entries [Gx, Gy, Gz] = exp(-ik0R)/(4pi) * (-d) * (1/R^3 + i k0/R^2)
__device__ __forceinline__ void gk_kernel(double dx, double dy, double dz, double k0, zd* f) {
  const double R = sqrt(dx * dx + dy * dy + dz * dz);
  const double iR = 1.0 / R;
  double sn, cs;
  sincos(k0 * R, &sn, &cs);
  const double q = 0.25 / 3.14159265358979323846;
  const zd Ge = {cs * q, -sn * q};
  const zd fac = Ge * zd{iR * iR * iR, k0 * iR * iR};
  f[0] = scale(fac, -dx);
  f[1] = scale(fac, -dy);
  f[2] = scale(fac, -dz);
}

// (l, l') pairs of the 10 PWL moment products, VV_Nop.m:27-28 (0-based)
__constant__ int c_ind_l[10] = {0, 1, 2, 3, 0, 0, 0, 1, 1, 2};
__constant__ int c_ind_lp[10] = {0, 1, 2, 3, 1, 2, 3, 2, 3, 3};

// One CTA per offset.  out[(mx + n1(my + n2 mz)) + nD*(llp + pwx*comp)]
template <int PWX, int NC, bool ISN>
__global__ void __launch_bounds__(128) k_vv(const int* offs, const int* rule_of, int noff, Rule3 r0o, Rule3 r0s,
                                            Rule3 r1o, Rule3 r1s, Rule3 r2o, Rule3 r2s, double dx, double k0,
                                            int n1, int n2, int n3, zd* out) {
  __shared__ zd red[4][PWX * NC];
  const int o = blockIdx.x;
  if (o >= noff) return;
  const int mx = offs[3 * o], my = offs[3 * o + 1], mz = offs[3 * o + 2];
  const int rid = rule_of[o];
  const Rule3 ro = rid == 0 ? r0o : (rid == 1 ? r1o : r2o);
  const Rule3 rs = rid == 0 ? r0s : (rid == 1 ? r1s : r2s);
  const double h = dx / 2;
  const double rmx = mx * dx, rmy = my * dx, rmz = mz * dx;
  zd acc[PWX][NC];
#pragma unroll
  for (int a = 0; a < PWX; ++a)
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[a][c] = zd{0, 0};
  const int npair = ro.np * rs.np;
  for (int p = threadIdx.x; p < npair; p += blockDim.x) {
    const int io = p % ro.np, is = p / ro.np;
    const double X = ro.x[3 * io], Y = ro.x[3 * io + 1], Z = ro.x[3 * io + 2];
    const double Xp = rs.x[3 * is], Yp = rs.x[3 * is + 1], Zp = rs.x[3 * is + 2];
    const double w = ro.w[io] * rs.w[is];
    zd f[NC];
    if (ISN) gn_kernel(rmx + h * (X - Xp), rmy + h * (Y - Yp), rmz + h * (Z - Zp), k0, f);
    else gk_kernel(rmx + h * (X - Xp), rmy + h * (Y - Yp), rmz + h * (Z - Zp), k0, f);
    const double T[4] = {1.0, X * 0.5, Y * 0.5, Z * 0.5};
    const double B[4] = {1.0, Xp * 0.5, Yp * 0.5, Zp * 0.5};
#pragma unroll
    for (int a = 0; a < PWX; ++a) {
      const double tb = w * T[c_ind_l[a]] * B[c_ind_lp[a]];
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        acc[a][c].x += tb * f[c].x;
        acc[a][c].y += tb * f[c].y;
      }
    }
  }
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int a = 0; a < PWX; ++a)
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      zd v = acc[a][c];
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, s);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, s);
      }
      if (lane == 0) red[wid][a * NC + c] = v;
    }
  __syncthreads();
  const double J = h * h * h * h * h * h;
  const int64_t nD = (int64_t)n1 * n2 * n3;
  const int64_t g = mx + (int64_t)n1 * (my + (int64_t)n2 * mz);
  for (int i = threadIdx.x; i < PWX * NC; i += blockDim.x) {
    zd s = {0, 0};
    for (int ww = 0; ww < (int)(blockDim.x >> 5); ++ww) s = s + red[ww][i];
    const int a = i / NC, c = i % NC;
    out[g + nD * (a + PWX * c)] = scale(s, J);
  }
}

void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  // Newton iteration on P_n; nodes ascending.
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < n; ++i) {
    long double z = std::cos(3.141592653589793238462643383279502884L * (i + 0.75L) / (n + 0.5L));
    long double pp = 0;
    for (int it = 0; it < 100; ++it) {
      long double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; ++j) {
        const long double p3 = p2;
        p2 = p1;
        p1 = ((2.0L * j - 1.0L) * z * p2 - (j - 1.0L) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0L);
      const long double z1 = z;
      z = z1 - p1 / pp;
      if (std::fabs((double)(z - z1)) < 1e-19) {
        // recompute derivative at the converged node
        p1 = 1; p2 = 0;
        for (int j = 1; j <= n; ++j) {
          const long double p3 = p2;
          p2 = p1;
          p1 = ((2.0L * j - 1.0L) * z * p2 - (j - 1.0L) * p3) / j;
        }
        pp = n * (z * p1 - p2) / (z * z - 1.0L);
        break;
      }
    }
    x[n - 1 - i] = (double)z;
    w[n - 1 - i] = (double)(2.0L / ((1.0L - z * z) * pp * pp));
  }
}

struct DevRule {
  double* x = nullptr;
  double* w = nullptr;
  int np = 0;
};

static marie_status make_rule(int n, DevRule& r, std::vector<void*>& scratch) {
  std::vector<double> x1, w1;
  gauss_legendre(n, x1, w1);
  const int np = n * n * n;
  std::vector<double> x(3 * np), w(np);
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const int p = i + n * (j + n * k);
        x[3 * p] = x1[i];
        x[3 * p + 1] = x1[j];
        x[3 * p + 2] = x1[k];
        w[p] = w1[i] * w1[j] * w1[k];
      }
  if (cudaMalloc(&r.x, x.size() * sizeof(double)) != cudaSuccess) return MARIE_ERR_OOM;
  scratch.push_back(r.x);
  if (cudaMalloc(&r.w, w.size() * sizeof(double)) != cudaSuccess) return MARIE_ERR_OOM;
  scratch.push_back(r.w);
  cudaMemcpy(r.x, x.data(), x.size() * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(r.w, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice);
  r.np = np;
  return MARIE_OK;
}

// ---------------------------------------------------------------------------
// Incident fields
// ---------------------------------------------------------------------------

// Ue[l][comp*Ns + s] = coef of loop l on voxel s; one thread per (voxel, loop).
// Segments: seg[(l*nseg + i)*6 + {mid xyz, dl xyz}]
template <bool PWL>
__global__ void k_loops(const int64_t* idxS, int64_t Ns, int n1, int n2, double ox, double oy, double oz, double res,
                        const double* seg, int nseg, int nloop, const double* qx, const double* qw, int nq,
                        double k0, double wmu, zd* out) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int l = blockIdx.y;
  if (s >= Ns || l >= nloop) return;
  const int64_t g = idxS[s];
  const int ix = (int)(g % n1), iy = (int)((g / n1) % n2), iz = (int)(g / ((int64_t)n1 * n2));
  const double cx = ox + res * ix, cy = oy + res * iy, cz = oz + res * iz;
  constexpr int L = PWL ? 4 : 1;
  zd acc[3][L];
#pragma unroll
  for (int p = 0; p < 3; ++p)
#pragma unroll
    for (int q = 0; q < L; ++q) acc[p][q] = zd{0, 0};
  const double* sg = seg + (int64_t)l * nseg * 6;
  const double q4 = 0.25 / 3.14159265358979323846;
  for (int a = 0; a < nq; ++a)
    for (int b = 0; b < nq; ++b)
      for (int c = 0; c < nq; ++c) {
        const double px = cx + qx[a] * res * 0.5, py = cy + qx[b] * res * 0.5, pz = cz + qx[c] * res * 0.5;
        const double wt = qw[a] * qw[b] * qw[c] * 0.125;
        zd E[3] = {{0, 0}, {0, 0}, {0, 0}};
        for (int i = 0; i < nseg; ++i) {
          const double dxx = px - sg[6 * i], dyy = py - sg[6 * i + 1], dzz = pz - sg[6 * i + 2];
          const double R = sqrt(dxx * dxx + dyy * dyy + dzz * dzz);
          double sn, cs;
          sincos(k0 * R, &sn, &cs);
          const double gr = q4 / R;
          const zd gg = {cs * gr, -sn * gr};
          E[0] = E[0] + scale(gg, sg[6 * i + 3]);
          E[1] = E[1] + scale(gg, sg[6 * i + 4]);
          E[2] = E[2] + scale(gg, sg[6 * i + 5]);
        }
        // E *= -i * omega * mu0
        const double fl[4] = {1.0, qx[a] * 0.5, qx[b] * 0.5, qx[c] * 0.5};
#pragma unroll
        for (int p = 0; p < 3; ++p) {
          const zd e = {E[p].y * wmu, -E[p].x * wmu};
#pragma unroll
          for (int q = 0; q < L; ++q) acc[p][q] = acc[p][q] + scale(e, wt * fl[q]);
        }
      }
#pragma unroll
  for (int p = 0; p < 3; ++p)
#pragma unroll
    for (int q = 0; q < L; ++q) {
      const double nrm = q == 0 ? 1.0 : 12.0;
      out[(int64_t)l * 3 * L * Ns + (int64_t)(p * L + q) * Ns + s] = scale(acc[p][q], nrm);
    }
}

template <bool PWL>
__global__ void k_plane(const int64_t* idxS, int64_t Ns, int n1, int n2, double ox, double oy, double oz, double res,
                        const double* qx, const double* qw, int nq, double k0, zd* out) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= Ns) return;
  const int64_t g = idxS[s];
  const int ix = (int)(g % n1), iy = (int)((g / n1) % n2), iz = (int)(g / ((int64_t)n1 * n2));
  const double cx = ox + res * ix, cy = oy + res * iy, cz = oz + res * iz;
  (void)cx; (void)cy;
  constexpr int L = PWL ? 4 : 1;
  zd acc[L];
#pragma unroll
  for (int q = 0; q < L; ++q) acc[q] = zd{0, 0};
  for (int a = 0; a < nq; ++a)
    for (int b = 0; b < nq; ++b)
      for (int c = 0; c < nq; ++c) {
        const double pz = cz + qx[c] * res * 0.5;
        const double wt = qw[a] * qw[b] * qw[c] * 0.125;
        double sn, cs;
        sincos(k0 * pz, &sn, &cs);
        const zd e = {cs, -sn};
        const double fl[4] = {1.0, qx[a] * 0.5, qx[b] * 0.5, qx[c] * 0.5};
#pragma unroll
        for (int q = 0; q < L; ++q) acc[q] = acc[q] + scale(e, wt * fl[q]);
      }
  for (int p = 0; p < 3; ++p)
    for (int q = 0; q < L; ++q) {
      const double nrm = q == 0 ? 1.0 : 12.0;
      out[(int64_t)(p * L + q) * Ns + s] = p == 0 ? scale(acc[q], nrm) : zd{0, 0};
    }
}

}  // namespace marie

using namespace marie;

extern "C" marie_status marie_assemble_green_ex(int32_t n1, int32_t n2, int32_t n3, double res, double freq,
                                                int32_t basis, int32_t kernel, int32_t flags, double* out_host) {
  if (flags & ~(MARIE_GREEN_SELF_POINT_TERM | MARIE_GREEN_NEAR_EXACT)) {
    set_error("marie_assemble_green_ex: unknown flags 0x%x", (unsigned)flags);
    return MARIE_ERR_BAD_ARG;
  }
  const marie_status st = marie_assemble_green(n1, n2, n3, res, freq, basis, kernel, out_host);
  if (st != MARIE_OK) return st;
  const int pwx = basis == MARIE_PWL ? 10 : 1;
  if (flags & MARIE_GREEN_NEAR_EXACT) {
    const double k0 = 2 * M_PI / (299792458.0 / freq);
    green_host::near_zone_exact(out_host, n1, n2, n3, res, k0, pwx, kernel == 0);
  } else if ((flags & MARIE_GREEN_SELF_POINT_TERM) && kernel == 0) {
    green_host::add_self_point_term(out_host, (int64_t)n1 * n2 * n3, pwx, res);
  }
  return MARIE_OK;
}

extern "C" marie_status marie_assemble_green(int32_t n1, int32_t n2, int32_t n3, double res, double freq,
                                             int32_t basis, int32_t kernel, double* out_host) {
  if (n1 < 1 || n2 < 1 || n3 < 1 || !(res > 0) || !(freq > 0) || !out_host || (basis != 0 && basis != 1) ||
      (kernel != 0 && kernel != 1)) {
    set_error("marie_assemble_green: invalid argument");
    return MARIE_ERR_BAD_ARG;
  }
  const bool pwl = basis == MARIE_PWL, isN = kernel == 0;
  const int pwx = pwl ? 10 : 1, nc = isN ? 6 : 3;
  const double c0 = 299792458.0;
  const double k0 = 2 * M_PI / (c0 / freq);
  const int64_t nD = (int64_t)n1 * n2 * n3;
  // rules: 0 far (4^3 x 4^3), 1 medium (8^3 x 8^3 or min(n)), 2 near stand-in (8^3 x 7^3)
  const int thr = isN ? 5 : 2;
  const int Npm = (n1 <= thr || n2 <= thr || n3 <= thr) ? std::min(n1, std::min(n2, n3)) : 8;
  std::vector<int> offs, rule;
  offs.reserve(3 * nD);
  rule.reserve(nD);
  for (int mz = 0; mz < n3; ++mz)
    for (int my = 0; my < n2; ++my)
      for (int mx = 0; mx < n1; ++mx) {
        offs.push_back(mx);
        offs.push_back(my);
        offs.push_back(mz);
        int r = 0;
        if (mx < Npm && my < Npm && mz < Npm) r = 1;
        if (mx < std::min(2, n1) && my < std::min(2, n2) && mz < std::min(2, n3)) r = 2;
        rule.push_back(r);
      }
  std::vector<void*> scratch;
  auto done = [&](marie_status s) {
    cudaDeviceSynchronize();
    for (void* p : scratch) cudaFree(p);
    return s;
  };
  DevRule far, med, nearo, nears;
  marie_status st;
  if ((st = make_rule(4, far, scratch)) != MARIE_OK) return done(st);
  if ((st = make_rule(Npm, med, scratch)) != MARIE_OK) return done(st);
  if ((st = make_rule(8, nearo, scratch)) != MARIE_OK) return done(st);
  if ((st = make_rule(7, nears, scratch)) != MARIE_OK) return done(st);
  int *d_offs = nullptr, *d_rule = nullptr;
  zd* d_out = nullptr;
  if (cudaMalloc(&d_offs, offs.size() * sizeof(int)) != cudaSuccess) return done(MARIE_ERR_OOM);
  scratch.push_back(d_offs);
  if (cudaMalloc(&d_rule, rule.size() * sizeof(int)) != cudaSuccess) return done(MARIE_ERR_OOM);
  scratch.push_back(d_rule);
  if (cudaMalloc(&d_out, (size_t)nD * pwx * nc * sizeof(zd)) != cudaSuccess) return done(MARIE_ERR_OOM);
  scratch.push_back(d_out);
  cudaMemcpy(d_offs, offs.data(), offs.size() * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemcpy(d_rule, rule.data(), rule.size() * sizeof(int), cudaMemcpyHostToDevice);
  Rule3 r0o{far.x, far.w, far.np}, r1o{med.x, med.w, med.np}, r2o{nearo.x, nearo.w, nearo.np};
  Rule3 r2s{nears.x, nears.w, nears.np};
  const int noff = (int)nD;
  // launch in slices to keep each grid modest
  const int slice = 1 << 20;
  for (int o0 = 0; o0 < noff; o0 += slice) {
    const int cnt = std::min(slice, noff - o0);
    const int* po = d_offs + 3 * (int64_t)o0;
    const int* pr = d_rule + o0;
    if (pwl && isN) k_vv<10, 6, true><<<cnt, 128>>>(po, pr, cnt, r0o, r0o, r1o, r1o, r2o, r2s, res, k0, n1, n2, n3, d_out);
    else if (pwl) k_vv<10, 3, false><<<cnt, 128>>>(po, pr, cnt, r0o, r0o, r1o, r1o, r2o, r2s, res, k0, n1, n2, n3, d_out);
    else if (isN) k_vv<1, 6, true><<<cnt, 128>>>(po, pr, cnt, r0o, r0o, r1o, r1o, r2o, r2s, res, k0, n1, n2, n3, d_out);
    else k_vv<1, 3, false><<<cnt, 128>>>(po, pr, cnt, r0o, r0o, r1o, r1o, r2o, r2s, res, k0, n1, n2, n3, d_out);
    g_launches++;
    if (cudaGetLastError() != cudaSuccess) {
      set_error("assembly kernel launch failed");
      return done(MARIE_ERR_CUDA);
    }
  }
  if (cudaMemcpy(out_host, d_out, (size_t)nD * pwx * nc * sizeof(zd), cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_error("assembly: device error %s", cudaGetErrorString(cudaGetLastError()));
    return done(MARIE_ERR_CUDA);
  }
  return done(MARIE_OK);
}

static marie_status quad_rule(int nq, double** qx, double** qw, std::vector<void*>& scratch) {
  std::vector<double> x, w;
  gauss_legendre(nq, x, w);
  if (cudaMalloc(qx, nq * sizeof(double)) != cudaSuccess) return MARIE_ERR_OOM;
  scratch.push_back(*qx);
  if (cudaMalloc(qw, nq * sizeof(double)) != cudaSuccess) return MARIE_ERR_OOM;
  scratch.push_back(*qw);
  cudaMemcpy(*qx, x.data(), nq * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(*qw, w.data(), nq * sizeof(double), cudaMemcpyHostToDevice);
  return MARIE_OK;
}

extern "C" marie_status marie_incident_loops(marie_vie* h, const double* origin, const double* loops, int32_t nloop,
                                             double radius, int32_t nseg, void* out_dev, void* stream) {
  if (!h || !origin || !loops || nloop < 1 || !(radius > 0) || nseg < 3 || !out_dev) {
    set_error("marie_incident_loops: invalid argument");
    return MARIE_ERR_BAD_ARG;
  }
  // regular nseg-gon inscribed in each circle: mid-points and chord vectors
  std::vector<double> seg((size_t)nloop * nseg * 6);
  for (int l = 0; l < nloop; ++l) {
    const double* L = loops + 6 * l;
    double nx = L[3], ny = L[4], nz = L[5];
    const double nn = std::sqrt(nx * nx + ny * ny + nz * nz);
    if (!(nn > 0)) { set_error("loop %d has a zero normal", l); return MARIE_ERR_BAD_ARG; }
    nx /= nn; ny /= nn; nz /= nn;
    double ax = 1, ay = 0, az = 0;
    if (std::fabs(nx) >= 0.9) { ax = 0; ay = 1; }
    // e1 = n x a / |.|, e2 = n x e1
    double e1x = ny * az - nz * ay, e1y = nz * ax - nx * az, e1z = nx * ay - ny * ax;
    const double n1 = std::sqrt(e1x * e1x + e1y * e1y + e1z * e1z);
    e1x /= n1; e1y /= n1; e1z /= n1;
    const double e2x = ny * e1z - nz * e1y, e2y = nz * e1x - nx * e1z, e2z = nx * e1y - ny * e1x;
    for (int i = 0; i < nseg; ++i) {
      const double t0 = 2 * M_PI * i / nseg, t1 = 2 * M_PI * (i + 1) / nseg;
      const double p0x = L[0] + radius * (std::cos(t0) * e1x + std::sin(t0) * e2x);
      const double p0y = L[1] + radius * (std::cos(t0) * e1y + std::sin(t0) * e2y);
      const double p0z = L[2] + radius * (std::cos(t0) * e1z + std::sin(t0) * e2z);
      const double p1x = L[0] + radius * (std::cos(t1) * e1x + std::sin(t1) * e2x);
      const double p1y = L[1] + radius * (std::cos(t1) * e1y + std::sin(t1) * e2y);
      const double p1z = L[2] + radius * (std::cos(t1) * e1z + std::sin(t1) * e2z);
      double* sgp = &seg[((size_t)l * nseg + i) * 6];
      sgp[0] = 0.5 * (p0x + p1x); sgp[1] = 0.5 * (p0y + p1y); sgp[2] = 0.5 * (p0z + p1z);
      sgp[3] = p1x - p0x; sgp[4] = p1y - p0y; sgp[5] = p1z - p0z;
    }
  }
  std::vector<void*> scratch;
  auto done = [&](marie_status s) {
    cudaStreamSynchronize((cudaStream_t)stream);
    for (void* p : scratch) cudaFree(p);
    return s;
  };
  double* d_seg = nullptr;
  if (cudaMalloc(&d_seg, seg.size() * sizeof(double)) != cudaSuccess) return done(MARIE_ERR_OOM);
  scratch.push_back(d_seg);
  cudaMemcpy(d_seg, seg.data(), seg.size() * sizeof(double), cudaMemcpyHostToDevice);
  double *qx = nullptr, *qw = nullptr;
  marie_status st;
  if ((st = quad_rule(3, &qx, &qw, scratch)) != MARIE_OK) return done(st);
  const double mu0 = 4e-7 * M_PI;
  dim3 grid((unsigned)((h->Ns + 127) / 128), (unsigned)nloop);
  cudaStream_t s = (cudaStream_t)stream;
  if (h->pwl)
    k_loops<true><<<grid, 128, 0, s>>>(h->idxS, h->Ns, h->n1, h->n2, origin[0], origin[1], origin[2], h->res, d_seg,
                                       nseg, nloop, qx, qw, 3, h->k0, h->omega * mu0, (zd*)out_dev);
  else
    k_loops<false><<<grid, 128, 0, s>>>(h->idxS, h->Ns, h->n1, h->n2, origin[0], origin[1], origin[2], h->res, d_seg,
                                        nseg, nloop, qx, qw, 3, h->k0, h->omega * mu0, (zd*)out_dev);
  g_launches++;
  if (cudaGetLastError() != cudaSuccess) { set_error("incident-field kernel launch failed"); return done(MARIE_ERR_CUDA); }
  return done(MARIE_OK);
}

extern "C" marie_status marie_incident_plane_wave(marie_vie* h, const double* origin, void* out_dev, void* stream) {
  if (!h || !origin || !out_dev) { set_error("marie_incident_plane_wave: invalid argument"); return MARIE_ERR_BAD_ARG; }
  std::vector<void*> scratch;
  auto done = [&](marie_status s) {
    cudaStreamSynchronize((cudaStream_t)stream);
    for (void* p : scratch) cudaFree(p);
    return s;
  };
  double *qx = nullptr, *qw = nullptr;
  marie_status st;
  if ((st = quad_rule(3, &qx, &qw, scratch)) != MARIE_OK) return done(st);
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned gb = (unsigned)((h->Ns + 127) / 128);
  if (h->pwl) k_plane<true><<<gb, 128, 0, s>>>(h->idxS, h->Ns, h->n1, h->n2, origin[0], origin[1], origin[2], h->res, qx, qw, 3, h->k0, (zd*)out_dev);
  else k_plane<false><<<gb, 128, 0, s>>>(h->idxS, h->Ns, h->n1, h->n2, origin[0], origin[1], origin[2], h->res, qx, qw, 3, h->k0, (zd*)out_dev);
  g_launches++;
  if (cudaGetLastError() != cudaSuccess) { set_error("plane-wave kernel launch failed"); return done(MARIE_ERR_CUDA); }
  return done(MARIE_OK);
}
