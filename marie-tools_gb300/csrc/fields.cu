// Field post-processing on the body: total E and H fields of a batch of
// solved currents (em_efield_vie_excitation.m:17-23,
// em_hfield_vie_excitation.m:16-22, em_ehfield_vie.m:31-41), the
// absorbed-power / noise-covariance matrix (em_ehfield_vie.m:44-52) and
// B1+ maps (em_ehfield_vie.m:67-68).
#include <cstring>

#include "internal.h"

namespace marie {

typedef cplx<double> zd;

constexpr int kPowThreads = 256;
constexpr int kPowRows = 32;       // body rows per shared-memory tile
constexpr int kMaxPowRhs = 64;     // right-hand sides per call of the power kernel

// Per-CTA partial sums P[cta][p*nrhs + q] = sum_i conj(J_ip) w_i g_c(i) J_iq
// over the CTA's rows (FP64; J is rhs-major, rows contiguous per rhs).
__global__ void __launch_bounds__(kPowThreads) k_pow_partial(const zd* J, int64_t Nb, int64_t Ns, int nrhs,
                                                             const double* wpow, const double* gdiag, zd* part) {
  __shared__ zd tile[kPowRows][kMaxPowRhs];
  __shared__ double wt[kPowRows];
  const int npair = nrhs * nrhs;
  constexpr int kMaxPer = kMaxPowRhs * kMaxPowRhs / kPowThreads;
  zd acc[kMaxPer];
#pragma unroll
  for (int u = 0; u < kMaxPer; ++u) acc[u] = zd{0, 0};
  const int64_t rows_per = (Nb + gridDim.x - 1) / gridDim.x;
  const int64_t r0 = (int64_t)blockIdx.x * rows_per;
  const int64_t r1 = r0 + rows_per < Nb ? r0 + rows_per : Nb;
  for (int64_t base = r0; base < r1; base += kPowRows) {
    const int nr = (int)((r1 - base) < kPowRows ? (r1 - base) : kPowRows);
    __syncthreads();
    for (int t = threadIdx.x; t < kPowRows * nrhs; t += blockDim.x) {
      const int i = t % kPowRows, r = t / kPowRows;
      tile[i][r] = i < nr ? J[(int64_t)r * Nb + base + i] : zd{0, 0};
    }
    for (int i = threadIdx.x; i < kPowRows; i += blockDim.x) {
      const int64_t row = base + i;
      wt[i] = i < nr ? wpow[row % Ns] * gdiag[row / Ns] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kMaxPer; ++u) {
      const int pq = threadIdx.x + u * kPowThreads;
      if (pq >= npair) break;
      const int p = pq / nrhs, q = pq - p * nrhs;
      zd a = acc[u];
      for (int i = 0; i < nr; ++i) {
        const zd jp = tile[i][p], jq = tile[i][q];
        const double w = wt[i];
        // conj(jp) * jq * w
        a.x = fma(w, jp.x * jq.x + jp.y * jq.y, a.x);
        a.y = fma(w, jp.x * jq.y - jp.y * jq.x, a.y);
      }
      acc[u] = a;
    }
  }
#pragma unroll
  for (int u = 0; u < kMaxPer; ++u) {
    const int pq = threadIdx.x + u * kPowThreads;
    if (pq < npair) part[(int64_t)blockIdx.x * npair + pq] = acc[u];
  }
}

// phi[p][q] = conj(sum over CTAs in fixed order) (em_ehfield_vie.m:51)
__global__ void k_pow_reduce(const zd* part, int nparts, int npair, zd* phi) {
  const int pq = blockIdx.x * blockDim.x + threadIdx.x;
  if (pq >= npair) return;
  zd s = {0, 0};
  for (int c = 0; c < nparts; ++c) s = s + part[(int64_t)c * npair + pq];
  phi[pq] = zd{s.x, -s.y};
}

// b1p[r][s] = mu0 (H_x + i H_y) at the constant moment of voxel s
// (em_ehfield_vie.m:68: Ub(jj) and Ub(jj + N_scat*l))
__global__ void k_b1_plus(const zd* H, int64_t Nb, int64_t Ns, int l, int nrhs, double mu0, zd* out) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int r = blockIdx.y;
  if (s >= Ns || r >= nrhs) return;
  const zd hx = H[(int64_t)r * Nb + s], hy = H[(int64_t)r * Nb + (int64_t)l * Ns + s];
  out[(int64_t)r * Ns + s] = zd{mu0 * (hx.x - hy.y), mu0 * (hx.y + hy.x)};
}

// Adjoint sensitivities of J_obj = M / P, M = mean over an ROI of |B1+|^2,
// P = (1/2) sum |J|^2 g_c real(Mc_inv/ce) (the absorbed power, phi(p,p)/2),
// with respect to each body voxel's eps_r and sigma.  With the VIE system
// A J = b, A = I - diag(chi) invG N, chi = 1 - 1/Mr, b = ce chi Ue and
// Mr = eps_r + sigma/ce:
//   g      = dJ_obj/dconj(J) = gM / P - (M / P^2) (1/2) D J,   D = g_c real(Mc_inv/ce)
//   A^H lam = g
//   dJ_obj/dp_s = 2 Re( sum_c conj(lam_cs) (ce E_cs + J_cs) (dMr/dp)/Mr_s^2 )
//               + (M / P^2) (1/2) sum_c |J_cs|^2 g_c Re( (dMr/dp) / ((Mr_s - 1)^2 ce) )
// where E is the total field of marie_vie_fields (ce E + J = ce Ue + invG N J)
// and gM = dM/dconj(J) = (mu0/|ROI|) (invG K)^H w (marie_vie_apply_hfield_adjoint).

// g = gM/P - (M/P^2)(1/2) D J
__global__ void k_grad_source(const zd* J, const zd* gM, int64_t Nb, int64_t Ns, const double* wpow,
                              const double* gdiag, double invP, double c2, zd* g) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= Nb) return;
  const double d = wpow[i % Ns] * gdiag[i / Ns] * c2;
  g[i] = zd{gM[i].x * invP - d * J[i].x, gM[i].y * invP - d * J[i].y};
}

__global__ void k_grad(const zd* J, const zd* lam, const zd* E, int64_t Ns, int C, const double* gdiag,
                       const zd* mr, double ce_im, double expl, double* deps, double* dsig) {
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= Ns) return;
  zd q = {0, 0};
  double jj = 0;
  for (int c = 0; c < C; ++c) {
    const int64_t i = (int64_t)c * Ns + s;
    const zd ceE = {-ce_im * E[i].y, ce_im * E[i].x};       // ce = i ce_im
    const zd t = ceE + J[i];
    q = q + zd{lam[i].x * t.x + lam[i].y * t.y, lam[i].x * t.y - lam[i].y * t.x};   // conj(lam) t
    jj += (J[i].x * J[i].x + J[i].y * J[i].y) * gdiag[c];
  }
  const zd m = mr[s];
  const zd m2 = m * m;
  const double n2 = m2.x * m2.x + m2.y * m2.y;
  const zd inv_m2 = {m2.x / n2, -m2.y / n2};                // 1/Mr^2
  const zd inv_ce = {0, -1.0 / ce_im};                      // 1/ce
  const zd a = q * inv_m2;
  deps[s] = 2.0 * a.x;
  dsig[s] = 2.0 * (a * inv_ce).x;
  const zd mc = {m.x - 1.0, m.y};
  const zd mc2 = mc * mc;
  const double nc = mc2.x * mc2.x + mc2.y * mc2.y;
  if (nc > 0) {
    const zd inv_mc2 = {mc2.x / nc, -mc2.y / nc};            // 1/(Mr - 1)^2
    const zd e1 = inv_mc2 * inv_ce;                          // dMr/deps = 1
    const zd e2 = e1 * inv_ce;                               // dMr/dsigma = 1/ce
    deps[s] += expl * jj * e1.x;
    dsig[s] += expl * jj * e2.x;
  }
}

}  // namespace marie

using namespace marie;

extern "C" {

marie_status marie_vie_fields(marie_vie* h, int32_t prec, const void* J, const void* Ue, const void* Ub, void* E,
                              void* H, int32_t nrhs, void* stream) {
  if (!h || !J || (!E && !H) || nrhs < 1) { set_error("marie_vie_fields: invalid argument"); return MARIE_ERR_BAD_ARG; }
  if (prec != MARIE_C128 && prec != MARIE_C64) { set_error("prec must be MARIE_C128 or MARIE_C64"); return MARIE_ERR_BAD_ARG; }
  if (H && !h->has_K) { set_error("the H field needs the K operator (not supplied at create time)"); return MARIE_ERR_BAD_ARG; }
  cudaStream_t s = (cudaStream_t)stream;
  if (prec == MARIE_C128) {
    if (E) MARIE_TRY(launch_matvec_fields<double>(h, MV_EFIELD, OP_N, (const cplx<double>*)J, (cplx<double>*)E,
                                                  (const cplx<double>*)Ue, nrhs, s));
    if (H) MARIE_TRY(launch_matvec_fields<double>(h, MV_HFIELD, OP_K, (const cplx<double>*)J, (cplx<double>*)H,
                                                  (const cplx<double>*)Ub, nrhs, s));
  } else {
    if (E) MARIE_TRY(launch_matvec_fields<float>(h, MV_EFIELD, OP_N, (const cplx<float>*)J, (cplx<float>*)E,
                                                 (const cplx<float>*)Ue, nrhs, s));
    if (H) MARIE_TRY(launch_matvec_fields<float>(h, MV_HFIELD, OP_K, (const cplx<float>*)J, (cplx<float>*)H,
                                                 (const cplx<float>*)Ub, nrhs, s));
  }
  return MARIE_OK;
}

marie_status marie_vie_absorbed_power(marie_vie* h, const void* J, int32_t nrhs, double* phi_host, void* stream) {
  if (!h || !J || !phi_host || nrhs < 1) { set_error("marie_vie_absorbed_power: invalid argument"); return MARIE_ERR_BAD_ARG; }
  if (nrhs > kMaxPowRhs) { set_error("marie_vie_absorbed_power: at most %d right-hand sides per call", kMaxPowRhs); return MARIE_ERR_BAD_ARG; }
  cudaStream_t s = (cudaStream_t)stream;
  const int npair = nrhs * nrhs;
  const int nparts = 2 * 152;
  zd* part = nullptr;
  zd* phi = nullptr;
  double* gd = nullptr;
  auto done = [&](marie_status st) {
    cudaStreamSynchronize(s);
    cudaFree(part);
    cudaFree(phi);
    cudaFree(gd);
    return st;
  };
  if (cudaMalloc((void**)&part, (size_t)nparts * npair * sizeof(zd)) != cudaSuccess ||
      cudaMalloc((void**)&phi, (size_t)npair * sizeof(zd)) != cudaSuccess ||
      cudaMalloc((void**)&gd, (size_t)h->C * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    set_error("marie_vie_absorbed_power: device allocation failed");
    return done(MARIE_ERR_OOM);
  }
  double g[12];
  for (int c = 0; c < h->C; ++c) g[c] = 1.0 / h->invg[c];     // Gram diagonal (mvp_G_pwl.m:5)
  cudaMemcpyAsync(gd, g, h->C * sizeof(double), cudaMemcpyHostToDevice, s);
  k_pow_partial<<<nparts, kPowThreads, 0, s>>>((const zd*)J, h->Nb, h->Ns, nrhs, h->wpow, gd, part);
  g_launches++;
  k_pow_reduce<<<(npair + 255) / 256, 256, 0, s>>>(part, nparts, npair, phi);
  g_launches++;
  if (cudaGetLastError() != cudaSuccess) { set_error("absorbed-power kernel launch failed"); return done(MARIE_ERR_CUDA); }
  if (cudaMemcpyAsync(phi_host, phi, (size_t)npair * sizeof(zd), cudaMemcpyDeviceToHost, s) != cudaSuccess) {
    set_error("absorbed-power copy failed");
    return done(MARIE_ERR_CUDA);
  }
  return done(MARIE_OK);
}

marie_status marie_vie_b1_plus(marie_vie* h, const void* H, int32_t nrhs, void* out, void* stream) {
  if (!h || !H || !out || nrhs < 1) { set_error("marie_vie_b1_plus: invalid argument"); return MARIE_ERR_BAD_ARG; }
  cudaStream_t s = (cudaStream_t)stream;
  const double mu0 = 4e-7 * M_PI;
  dim3 grid((unsigned)((h->Ns + 255) / 256), (unsigned)nrhs);
  k_b1_plus<<<grid, 256, 0, s>>>((const zd*)H, h->Nb, h->Ns, h->pwl ? 4 : 1, nrhs, mu0, (zd*)out);
  g_launches++;
  if (cudaGetLastError() != cudaSuccess) { set_error("B1+ kernel launch failed"); return MARIE_ERR_CUDA; }
  return MARIE_OK;
}

}  // extern "C"

extern "C" {

static marie_status upload_gdiag(marie_vie* h, double** gd, cudaStream_t s) {
  double g[12];
  for (int c = 0; c < h->C; ++c) g[c] = 1.0 / h->invg[c];
  if (cudaMalloc((void**)gd, h->C * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    set_error("device allocation failed");
    return MARIE_ERR_OOM;
  }
  cudaMemcpyAsync(*gd, g, h->C * sizeof(double), cudaMemcpyHostToDevice, s);
  return MARIE_OK;
}

marie_status marie_vie_gradient_source(marie_vie* h, const void* J, const void* gM, double M, double P, void* g,
                                       void* stream) {
  if (!h || !J || !gM || !g || !(P > 0)) { set_error("marie_vie_gradient_source: invalid argument"); return MARIE_ERR_BAD_ARG; }
  cudaStream_t s = (cudaStream_t)stream;
  double* gd = nullptr;
  MARIE_TRY(upload_gdiag(h, &gd, s));
  k_grad_source<<<(unsigned)((h->Nb + 255) / 256), 256, 0, s>>>((const zd*)J, (const zd*)gM, h->Nb, h->Ns, h->wpow,
                                                                gd, 1.0 / P, 0.5 * M / (P * P), (zd*)g);
  g_launches++;
  const cudaError_t e = cudaGetLastError();
  cudaStreamSynchronize(s);
  cudaFree(gd);
  if (e != cudaSuccess) { set_error("gradient-source kernel launch failed"); return MARIE_ERR_CUDA; }
  return MARIE_OK;
}

marie_status marie_vie_gradient(marie_vie* h, const void* J, const void* lam, const void* E, double M, double P,
                                double* d_eps, double* d_sigma, void* stream) {
  if (!h || !J || !lam || !E || !d_eps || !d_sigma || !(P > 0)) {
    set_error("marie_vie_gradient: invalid argument");
    return MARIE_ERR_BAD_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  double* gd = nullptr;
  MARIE_TRY(upload_gdiag(h, &gd, s));
  k_grad<<<(unsigned)((h->Ns + 255) / 256), 256, 0, s>>>((const zd*)J, (const zd*)lam, (const zd*)E, h->Ns, h->C, gd,
                                                         h->mr_body, h->ce_im, 0.5 * M / (P * P), d_eps, d_sigma);
  g_launches++;
  const cudaError_t e = cudaGetLastError();
  cudaStreamSynchronize(s);
  cudaFree(gd);
  if (e != cudaSuccess) { set_error("gradient kernel launch failed"); return MARIE_ERR_CUDA; }
  return MARIE_OK;
}

}  // extern "C"
