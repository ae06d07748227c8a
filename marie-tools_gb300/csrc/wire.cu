// Incident fields of wire currents in the reference's wire-basis convention
// (Assemble_tri_coupling_matrix_{N,K}_*.cpp of src_wvie/Cpp_Assembly, scaled
// by res^3 in wvie_mrgf_assembly.m:26-49, applied to the wire currents and
// mapped to coefficients by invG as em_efield_wvie.m:43-47 and
// em_hfield_wvie.m:38 do).
//
// Wire basis i is a pair of straight halves r_p -> r_2 and r_2 -> r_n; on
// each half the Gauss point s = L/2 (x + 1) from the half's start carries
// the current (s/L) * unit tangent (both halves ramp up from their start
// point, as the reference places its source points), weight w * L/2.  The
// host folds the wire currents into a list of source points, each with a
// position and a complex current vector, so a closed loop is a sum over its
// points.  Per body voxel and right-hand side the kernel integrates, with a
// q^3 Gauss rule over the voxel,
//   E (kind 0): -1/(4 pi ce) e^{-ikR}/R^3 [P (R.J) R - (k^2R^2 - ikR - 1) J],
//               P = (k^2R^2 - 3ikR - 3)/R^2  (the dyadic kernel, charges
//               included),
//   H (kind 1): -1/(4 pi) e^{-ikR}/R^3 (1 + ikR) (R x J),
// against 1 and, PWL, the moments x/2, y/2, z/2 of the voxel's local
// coordinates, and divides by the basis Gram (res^3, res^3/12).  FP64
// throughout; the source list of one right-hand side is staged in shared
// memory in tiles.
#include <cmath>
#include <vector>

#include "internal.h"

namespace marie {

typedef cplx<double> zd;

namespace {

constexpr int kWireTile = 256;   // source points per shared-memory tile

struct WireSrc {
  double x, y, z;
  double jxr, jxi, jyr, jyi, jzr, jzi;
};

template <bool PWL, int KIND>
__global__ void __launch_bounds__(128) k_wire(const int64_t* __restrict__ idxS, int64_t Ns, int n1, int n2, double ox,
                                              double oy, double oz, double res, const WireSrc* __restrict__ src,
                                              int nsrc, const double* __restrict__ qx, const double* __restrict__ qw,
                                              int nq, double k0, double scale, const double* __restrict__ invg,
                                              zd* __restrict__ out) {
  __shared__ WireSrc tile[kWireTile];
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int rhs = blockIdx.y;
  const bool on = s < Ns;
  double cx = 0, cy = 0, cz = 0;
  if (on) {
    const int64_t g = idxS[s];
    cx = ox + res * (double)(g % n1);
    cy = oy + res * (double)((g / n1) % n2);
    cz = oz + res * (double)(g / ((int64_t)n1 * n2));
  }
  constexpr int L = PWL ? 4 : 1;
  double ar[3][L], ai[3][L];
#pragma unroll
  for (int p = 0; p < 3; ++p)
#pragma unroll
    for (int l = 0; l < L; ++l) ar[p][l] = ai[p][l] = 0.0;
  const WireSrc* sr = src + (int64_t)rhs * nsrc;
  const double k2 = k0 * k0;
  for (int t0 = 0; t0 < nsrc; t0 += kWireTile) {
    const int nt = min(kWireTile, nsrc - t0);
    __syncthreads();
    for (int i = threadIdx.x; i < nt; i += blockDim.x) tile[i] = sr[t0 + i];
    __syncthreads();
    if (!on) continue;
    for (int a = 0; a < nq; ++a)
      for (int b = 0; b < nq; ++b)
        for (int c = 0; c < nq; ++c) {
          const double px = cx + 0.5 * res * qx[a], py = cy + 0.5 * res * qx[b], pz = cz + 0.5 * res * qx[c];
          double er[3] = {0, 0, 0}, ei[3] = {0, 0, 0};
          for (int i = 0; i < nt; ++i) {
            const WireSrc q = tile[i];
            const double rx = px - q.x, ry = py - q.y, rz = pz - q.z;
            const double R2 = rx * rx + ry * ry + rz * rz;
            const double R = sqrt(R2);
            const double kR = k0 * R;
            double sn, cs;
            sincos(kR, &sn, &cs);
            const double iR3 = 1.0 / (R2 * R);
            // kappa = e^{-ikR}/R^3
            const double kr = cs * iR3, ki = -sn * iR3;
            if constexpr (KIND == 0) {
              // P = (k^2 R^2 - 3 - 3i kR)/R^2; c2 = k^2 R^2 - 1 - i kR
              const double Pr = (k2 * R2 - 3.0) / R2, Pi = -3.0 * kR / R2;
              const double c2r = k2 * R2 - 1.0, c2i = -kR;
              // R.J (complex)
              const double dr = rx * q.jxr + ry * q.jyr + rz * q.jzr;
              const double di = rx * q.jxi + ry * q.jyi + rz * q.jzi;
              // u = P (R.J)
              const double ur = Pr * dr - Pi * di, ui = Pr * di + Pi * dr;
              const double rv[3] = {rx, ry, rz};
              const double jr[3] = {q.jxr, q.jyr, q.jzr}, ji[3] = {q.jxi, q.jyi, q.jzi};
#pragma unroll
              for (int p = 0; p < 3; ++p) {
                // v = u R_p - c2 J_p ; field += kappa v
                const double vr = ur * rv[p] - (c2r * jr[p] - c2i * ji[p]);
                const double vi = ui * rv[p] - (c2r * ji[p] + c2i * jr[p]);
                er[p] += kr * vr - ki * vi;
                ei[p] += kr * vi + ki * vr;
              }
            } else {
              // G = kappa (1 + i kR)
              const double gr = kr - ki * kR, gi = ki + kr * kR;
              const double xr = ry * q.jzr - rz * q.jyr, xi = ry * q.jzi - rz * q.jyi;
              const double yr = rz * q.jxr - rx * q.jzr, yi = rz * q.jxi - rx * q.jzi;
              const double zr = rx * q.jyr - ry * q.jxr, zi = rx * q.jyi - ry * q.jxi;
              er[0] += gr * xr - gi * xi; ei[0] += gr * xi + gi * xr;
              er[1] += gr * yr - gi * yi; ei[1] += gr * yi + gi * yr;
              er[2] += gr * zr - gi * zi; ei[2] += gr * zi + gi * zr;
            }
          }
          const double wt = qw[a] * qw[b] * qw[c] * 0.125;
          const double fl[4] = {1.0, 0.5 * qx[a], 0.5 * qx[b], 0.5 * qx[c]};
#pragma unroll
          for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int l = 0; l < L; ++l) {
              ar[p][l] += wt * fl[l] * er[p];
              ai[p][l] += wt * fl[l] * ei[p];
            }
        }
  }
  if (!on) return;
  // E: times -1/(4 pi ce) = i/(4 pi c) with ce = i c (scale = 1/(4 pi c)); H: times scale = -1/(4 pi);
  // then res^3 (the voxel integral) and invG (coefficients)
#pragma unroll
  for (int p = 0; p < 3; ++p)
#pragma unroll
    for (int l = 0; l < L; ++l) {
      const int comp = p * L + l;
      const double g = invg[comp] * res * res * res;
      double vr, vi;
      if constexpr (KIND == 0) {
        // -1/(4 pi ce), ce = i c: -1/(4 pi i c) = i/(4 pi c) = i*scale
        vr = -ai[p][l] * scale;
        vi = ar[p][l] * scale;
      } else {
        vr = ar[p][l] * scale;
        vi = ai[p][l] * scale;
      }
      out[(int64_t)rhs * 3 * L * Ns + (int64_t)comp * Ns + s] = zd{vr * g, vi * g};
    }
}

}  // namespace
}  // namespace marie

using namespace marie;

extern "C" marie_status marie_incident_wire(marie_vie* h, int32_t kind, const double* origin, const double* r_p,
                                            const double* r_n, const double* r_2, int32_t n_tri, const double* coef,
                                            int32_t nrhs, int32_t q_wire, int32_t q_vox, void* out_dev,
                                            void* stream) {
  if (!h || !origin || !r_p || !r_n || !r_2 || n_tri < 1 || nrhs < 1 || !out_dev || (kind != 0 && kind != 1) ||
      q_wire < 1 || q_wire > 16 || q_vox < 1 || q_vox > 8) {
    set_error("marie_incident_wire: invalid argument");
    return MARIE_ERR_BAD_ARG;
  }
  std::vector<double> xw, ww, xv, wv;
  gauss_legendre(q_wire, xw, ww);
  gauss_legendre(q_vox, xv, wv);
  const int nsrc = n_tri * 2 * q_wire;
  std::vector<WireSrc> src((size_t)nrhs * nsrc);
  for (int t = 0; t < n_tri; ++t) {
    const double* P[3] = {r_p + 3 * t, r_2 + 3 * t, r_n + 3 * t};
    for (int half = 0; half < 2; ++half) {
      const double* a = P[half];
      const double* b = P[half + 1];
      const double d[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
      const double len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      if (!(len > 0)) {
        set_error("marie_incident_wire: wire basis %d has a zero-length half", t);
        return MARIE_ERR_BAD_ARG;
      }
      for (int i = 0; i < q_wire; ++i) {
        const double f = 0.5 * (xw[i] + 1.0);     // s / L
        const double w = ww[i] * 0.5 * f;   // Gauss weight * L/2 * ramp s/L * (1/L: d is not unit)
        for (int r = 0; r < nrhs; ++r) {
          const double cr = coef ? coef[2 * ((size_t)r * n_tri + t)] : 1.0;
          const double ci = coef ? coef[2 * ((size_t)r * n_tri + t) + 1] : 0.0;
          WireSrc& q = src[(size_t)r * nsrc + ((size_t)t * 2 + half) * q_wire + i];
          q.x = a[0] + f * d[0];
          q.y = a[1] + f * d[1];
          q.z = a[2] + f * d[2];
          q.jxr = cr * w * d[0]; q.jxi = ci * w * d[0];
          q.jyr = cr * w * d[1]; q.jyi = ci * w * d[1];
          q.jzr = cr * w * d[2]; q.jzi = ci * w * d[2];
        }
      }
    }
  }
  std::vector<void*> scratch;
  auto done = [&](marie_status st) {
    cudaStreamSynchronize((cudaStream_t)stream);
    for (void* p : scratch) cudaFree(p);
    return st;
  };
  WireSrc* d_src = nullptr;
  double* d_q = nullptr;
  if (cudaMalloc(&d_src, src.size() * sizeof(WireSrc)) != cudaSuccess) { cudaGetLastError(); set_error("marie_incident_wire: out of device memory"); return done(MARIE_ERR_OOM); }
  scratch.push_back(d_src);
  if (cudaMalloc(&d_q, (2 * q_vox + 12) * sizeof(double)) != cudaSuccess) { cudaGetLastError(); set_error("marie_incident_wire: out of device memory"); return done(MARIE_ERR_OOM); }
  scratch.push_back(d_q);
  std::vector<double> qv(2 * q_vox + 12);
  for (int i = 0; i < q_vox; ++i) { qv[i] = xv[i]; qv[q_vox + i] = wv[i]; }
  for (int c = 0; c < h->C; ++c) qv[2 * q_vox + c] = h->invg[c];
  cudaMemcpy(d_src, src.data(), src.size() * sizeof(WireSrc), cudaMemcpyHostToDevice);
  cudaMemcpy(d_q, qv.data(), qv.size() * sizeof(double), cudaMemcpyHostToDevice);
  const double mu0 = 4e-7 * M_PI, c0 = 299792458.0;
  const double e0 = 1.0 / (c0 * c0 * mu0);
  const double ce_im = h->k0 * c0 * e0;                    // ce = i k0 c0 e0 (the reference's own ce)
  const double scale = kind == 0 ? 1.0 / (4.0 * M_PI * ce_im) : -1.0 / (4.0 * M_PI);
  dim3 grid((unsigned)((h->Ns + 127) / 128), (unsigned)nrhs);
  cudaStream_t s = (cudaStream_t)stream;
  const double* qx = d_q;
  const double* qw = d_q + q_vox;
  const double* ig = d_q + 2 * q_vox;
#define MARIE_WIRE_LAUNCH(PW, KD)                                                                             \
  k_wire<PW, KD><<<grid, 128, 0, s>>>(h->idxS, h->Ns, h->n1, h->n2, origin[0], origin[1], origin[2], h->res,    \
                                      d_src, nsrc, qx, qw, q_vox, h->k0, scale, ig, (zd*)out_dev)
  if (h->pwl) {
    if (kind == 0) MARIE_WIRE_LAUNCH(true, 0);
    else MARIE_WIRE_LAUNCH(true, 1);
  } else {
    if (kind == 0) MARIE_WIRE_LAUNCH(false, 0);
    else MARIE_WIRE_LAUNCH(false, 1);
  }
#undef MARIE_WIRE_LAUNCH
  g_launches++;
  if (cudaGetLastError() != cudaSuccess) { set_error("wire incident-field kernel launch failed"); return done(MARIE_ERR_CUDA); }
  return done(MARIE_OK);
}
