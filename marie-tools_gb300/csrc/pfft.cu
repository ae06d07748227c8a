// Coupled coil/body matvec of the pFFT formulation (mvp_svie_pfft.m:1-19).
//
// The unknowns are [Jc; Jb]: N_sie coil currents followed by N_b body
// currents.  The pFFT projection PS (sparse, grid unknowns x (N_sie + N_b))
// puts both on the extended voxel grid, where the N operator of that grid
// (the FFT-VIE matvec of a marie_vie handle, grid mode) couples them;
// sparse near-zone corrections Z_cc and Z_bc_N replace the part of the
// coil-coil and coil-body coupling the grid does not resolve:
//
//   Jb   = PS [0; Jcb_body],  Jtot = PS Jcb                     (:4-5)
//   y1   = (1/ce) M1 .* (PS.' (N Jtot - G Jtot))                 (:8-9)
//   y2   = (1/ce) M2 .* (PS.' G (ext_Mc_inv .* Jb))              (:11-12)
//   y3   = [Z_cc Jc + Z_bc_N.' Jb; -Z_bc_N Jc]                   (:14)
//   y    = y1 + y2 + y3                                           (:17)
//
// with G the Gram diagonal of the basis (mvp_G_pwc.m / mvp_G_pwl.m) and
// M1 = [1; -1], M2 = [0; 1] by block (ie_solver_svie_pfft.m:25-26) unless
// the caller gives its own.  The sparse products run as CSR kernels with
// a group of lanes per row; PS.' and Z_bc_N.' (plain transposes) are formed
// once at create as CSR matrices of their own, so every product reads its
// matrix row by row.  All device memory is owned by the handle.
#include <algorithm>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>

#include "internal.h"

namespace marie {
namespace {

// Device CSR matrix in one precision (int32 columns, int64 row offsets).
template <typename T>
struct DevCsr {
  int64_t rows = 0, cols = 0, nnz = 0;
  int64_t* rp = nullptr;
  int32_t* ci = nullptr;
  cplx<T>* v = nullptr;
};

struct HostCsr {
  int64_t rows = 0, cols = 0;
  std::vector<int64_t> rp;
  std::vector<int32_t> ci;
  std::vector<std::complex<double>> v;
};

}  // namespace
}  // namespace marie

struct marie_svie_pfft {
  marie_vie* grid = nullptr;     // extended-grid operator (not owned)
  int64_t n_sie = 0, n_b = 0, n_grid = 0;   // n_grid = n1*n2*n3*ql of the extended grid
  int64_t nvox = 0;
  int ql = 0;
  double ce_im = 0;
  marie::DevCsr<double> d64[5];  // PS (body columns), PS (coil columns), PS.', Z_cc, Z_bc_N
  marie::DevCsr<float> d32[5];
  marie::DevCsr<double> zbt64;   // Z_bc_N^T
  marie::DevCsr<float> zbt32;
  marie::cplx<double>* mc64 = nullptr;   // ext_Mc_inv (nvox)
  marie::cplx<float>* mc32 = nullptr;
  double* m1 = nullptr;          // multipliers (N_sie + N_b)
  double* m2 = nullptr;          // followed by the Gram diagonal (ql doubles)
  std::vector<void*> allocs;
  // work arrays of one right-hand side: 3 grids + 2 body-length vectors, per precision
  void* work = nullptr;
  size_t work_bytes = 0;
};

namespace marie {
namespace {

enum { M_PSB = 0, M_PSC = 1, M_PST = 2, M_ZCC = 3, M_ZBC = 4 };

marie_status pf_alloc(marie_svie_pfft* h, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) return MARIE_OK;
  if (cudaMalloc(p, bytes) != cudaSuccess) {
    cudaGetLastError();
    set_error("svie_pfft: cudaMalloc(%zu) failed", bytes);
    return MARIE_ERR_OOM;
  }
  h->allocs.push_back(*p);
  return MARIE_OK;
}

bool read_csr(const marie_csr& m, HostCsr& out, const char* name) {
  if (m.rows < 0 || m.cols < 0 || m.nnz < 0 || (m.nnz > 0 && (!m.row_ptr || !m.col_idx || !m.val)) ||
      (m.rows > 0 && !m.row_ptr)) {
    set_error("svie_pfft: %s: invalid CSR descriptor", name);
    return false;
  }
  if (m.cols > INT32_MAX) {
    set_error("svie_pfft: %s has more than 2^31 columns", name);
    return false;
  }
  out.rows = m.rows;
  out.cols = m.cols;
  out.rp.assign(m.rows + 1, 0);
  if (m.rows > 0) {
    if (m.row_ptr[0] != 0 || m.row_ptr[m.rows] != m.nnz) {
      set_error("svie_pfft: %s: row_ptr must start at 0 and end at nnz", name);
      return false;
    }
    for (int64_t r = 0; r <= m.rows; ++r) {
      out.rp[r] = m.row_ptr[r];
      if (r > 0 && out.rp[r] < out.rp[r - 1]) {
        set_error("svie_pfft: %s: row_ptr is not non-decreasing at row %lld", name, (long long)r);
        return false;
      }
    }
  }
  out.ci.resize(m.nnz);
  out.v.resize(m.nnz);
  for (int64_t k = 0; k < m.nnz; ++k) {
    if (m.col_idx[k] < 0 || m.col_idx[k] >= m.cols) {
      set_error("svie_pfft: %s: column index %lld out of range at entry %lld", name, (long long)m.col_idx[k],
                (long long)k);
      return false;
    }
    out.ci[k] = (int32_t)m.col_idx[k];
    out.v[k] = {m.val[2 * k], m.val[2 * k + 1]};
  }
  return true;
}

// Plain transpose (MATLAB .') of a CSR matrix.
HostCsr transpose(const HostCsr& a) {
  HostCsr t;
  t.rows = a.cols;
  t.cols = a.rows;
  t.rp.assign(t.rows + 1, 0);
  for (int32_t c : a.ci) t.rp[c + 1]++;
  for (int64_t r = 0; r < t.rows; ++r) t.rp[r + 1] += t.rp[r];
  t.ci.resize(a.ci.size());
  t.v.resize(a.v.size());
  std::vector<int64_t> next(t.rp.begin(), t.rp.end() - 1);
  for (int64_t r = 0; r < a.rows; ++r)
    for (int64_t k = a.rp[r]; k < a.rp[r + 1]; ++k) {
      const int64_t d = next[a.ci[k]]++;
      t.ci[d] = (int32_t)r;
      t.v[d] = a.v[k];
    }
  return t;
}

// Columns [c0, c1) of a, renumbered from 0.
HostCsr column_range(const HostCsr& a, int64_t c0, int64_t c1) {
  HostCsr o;
  o.rows = a.rows;
  o.cols = c1 - c0;
  o.rp.assign(a.rows + 1, 0);
  for (int64_t r = 0; r < a.rows; ++r) {
    for (int64_t k = a.rp[r]; k < a.rp[r + 1]; ++k)
      if (a.ci[k] >= c0 && a.ci[k] < c1) {
        o.ci.push_back((int32_t)(a.ci[k] - c0));
        o.v.push_back(a.v[k]);
      }
    o.rp[r + 1] = (int64_t)o.ci.size();
  }
  return o;
}

template <typename T>
marie_status upload(marie_svie_pfft* h, const HostCsr& a, DevCsr<T>& d) {
  d.rows = a.rows;
  d.cols = a.cols;
  d.nnz = (int64_t)a.ci.size();
  MARIE_TRY(pf_alloc(h, (void**)&d.rp, (a.rows + 1) * sizeof(int64_t)));
  MARIE_TRY(pf_alloc(h, (void**)&d.ci, std::max<int64_t>(d.nnz, 1) * sizeof(int32_t)));
  MARIE_TRY(pf_alloc(h, (void**)&d.v, std::max<int64_t>(d.nnz, 1) * sizeof(cplx<T>)));
  std::vector<cplx<T>> v(d.nnz);
  for (int64_t k = 0; k < d.nnz; ++k) v[k] = cplx<T>{(T)a.v[k].real(), (T)a.v[k].imag()};
  MARIE_CUDA_TRY(cudaMemcpy(d.rp, a.rp.data(), (a.rows + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
  if (d.nnz) {
    MARIE_CUDA_TRY(cudaMemcpy(d.ci, a.ci.data(), d.nnz * sizeof(int32_t), cudaMemcpyHostToDevice));
    MARIE_CUDA_TRY(cudaMemcpy(d.v, v.data(), d.nnz * sizeof(cplx<T>), cudaMemcpyHostToDevice));
  }
  return MARIE_OK;
}

// y[r] = (add ? add[r] : 0) + sgn * sum_k v[k] x[ci[k]] for row r; a group of
// G lanes per row (strided over the row's entries, shuffle-reduced), rows of
// one right-hand side per grid row y = rhs.  Accumulation in T (FP32 for
// complex64, FP64 for complex128).
constexpr int kSpG = 4;
template <typename T>
__global__ void k_csr(int64_t rows, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
                      const cplx<T>* __restrict__ v, const cplx<T>* __restrict__ x, int64_t x_rs,
                      const cplx<T>* add, int64_t add_rs, cplx<T>* y, int64_t y_rs, T sgn) {
  const int rhs = blockIdx.y;
  const int lane = threadIdx.x % kSpG;
  const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kSpG;
  const bool on = r < rows;
  cplx<T> acc{0, 0};
  if (on) {
    const cplx<T>* xr = x + (int64_t)rhs * x_rs;
    for (int64_t k = rp[r] + lane; k < rp[r + 1]; k += kSpG) acc = acc + v[k] * xr[ci[k]];
  }
#pragma unroll
  for (int o = kSpG / 2; o > 0; o >>= 1) {
    acc.x += __shfl_down_sync(0xffffffffu, acc.x, o, kSpG);
    acc.y += __shfl_down_sync(0xffffffffu, acc.y, o, kSpG);
  }
  if (on && lane == 0) {
    cplx<T> out = scale(acc, sgn);
    if (add) out = out + add[(int64_t)rhs * add_rs + r];
    y[(int64_t)rhs * y_rs + r] = out;
  }
}

template <typename T>
marie_status spmv(const DevCsr<T>& m, const cplx<T>* x, int64_t x_rs, const cplx<T>* add, int64_t add_rs,
                  cplx<T>* y, int64_t y_rs, T sgn, int nrhs, cudaStream_t s) {
  if (m.rows == 0) return MARIE_OK;
  const int threads = 256;
  const int64_t blocks = (m.rows * kSpG + threads - 1) / threads;
  k_csr<T><<<dim3((unsigned)blocks, (unsigned)nrhs), threads, 0, s>>>(m.rows, m.rp, m.ci, m.v, x, x_rs, add, add_rs,
                                                                      y, y_rs, sgn);
  MARIE_LAUNCH_CHECK();
  return MARIE_OK;
}

// e1 = N Jtot - G Jtot (into nj), e2 = G (ext_Mc_inv .* Jb) (into jb), over
// the extended grid (column-major, component slowest).
template <typename T>
__global__ void k_pf_mid(int64_t nvox, int ql, const cplx<T>* __restrict__ mc, const double* __restrict__ gram,
                         const cplx<T>* __restrict__ jtot, cplx<T>* nj, cplx<T>* jb, int64_t rs) {
  const int rhs = blockIdx.y;
  const int64_t n = nvox * ql;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i / nvox);
    const int64_t vx = i - (int64_t)c * nvox;
    const T g = (T)gram[c];
    const int64_t o = (int64_t)rhs * rs + i;
    nj[o] = nj[o] - scale(jtot[o], g);
    jb[o] = scale(mc[vx] * jb[o], g);
  }
}

// y = (1/ce) (m1 .* u + m2 .* w), ce = i*ce_im.
template <typename T>
__global__ void k_pf_combine(int64_t n, const double* __restrict__ m1, const double* __restrict__ m2,
                             const cplx<T>* __restrict__ u, const cplx<T>* __restrict__ w, cplx<T>* y, int64_t rs,
                             double ce_im) {
  const int rhs = blockIdx.y;
  const T inv = (T)(-1.0 / ce_im);   // 1/(i c) = -i/c
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t o = (int64_t)rhs * rs + i;
    const cplx<T> a = scale(u[o], (T)m1[i]) + scale(w[o], (T)m2[i]);
    y[o] = cplx<T>{-a.y * inv, a.x * inv};
  }
}

template <typename T>
marie_status pf_apply(marie_svie_pfft* h, const cplx<T>* x, cplx<T>* y, int nrhs, cudaStream_t s) {
  DevCsr<T>* d;
  DevCsr<T>* zbt;
  cplx<T>* mc;
  if constexpr (sizeof(T) == 8) { d = h->d64; zbt = &h->zbt64; mc = h->mc64; }
  else { d = h->d32; zbt = &h->zbt32; mc = h->mc32; }
  const int64_t nt = h->n_sie + h->n_b, ng = h->n_grid;
  const size_t per = (size_t)(3 * ng + 2 * nt) * sizeof(cplx<T>);
  // work arrays for up to 8 right-hand sides at a time
  const int chunk = std::max(1, std::min(nrhs, 8));
  const size_t need = per * chunk;
  if (need > h->work_bytes) {
    if (h->work) cudaFree(h->work);
    h->work = nullptr;
    h->work_bytes = 0;
    if (cudaMalloc(&h->work, need) != cudaSuccess) {
      cudaGetLastError();
      set_error("svie_pfft: work arrays of %zu bytes could not be allocated", need);
      return MARIE_ERR_OOM;
    }
    h->work_bytes = need;
  }
  const unsigned vb = 1024;
  for (int r0 = 0; r0 < nrhs; r0 += chunk) {
    const int nr = std::min(chunk, nrhs - r0);
    cplx<T>* jb = (cplx<T>*)h->work;            // [nr][ng]
    cplx<T>* jt = jb + (size_t)chunk * ng;       // [nr][ng]
    cplx<T>* nj = jt + (size_t)chunk * ng;       // [nr][ng]
    cplx<T>* u = nj + (size_t)chunk * ng;        // [nr][nt]
    cplx<T>* w = u + (size_t)chunk * nt;         // [nr][nt]
    const cplx<T>* xr = x + (int64_t)r0 * nt;
    cplx<T>* yr = y + (int64_t)r0 * nt;
    // Jb = PS_b Jcb_body; Jtot = Jb + PS_c Jc
    MARIE_TRY(spmv<T>(d[M_PSB], xr + h->n_sie, nt, nullptr, 0, jb, ng, (T)1, nr, s));
    MARIE_TRY(spmv<T>(d[M_PSC], xr, nt, jb, ng, jt, ng, (T)1, nr, s));
    // N Jtot on the extended grid (grid mode of its handle)
    MARIE_TRY(launch_matvec<T>(h->grid, MV_GRID, OP_N, jt, ng, nj, ng, nr, nullptr, s));
    k_pf_mid<T><<<dim3(vb, nr), 256, 0, s>>>(h->nvox, h->ql, mc, h->m1 + 2 * nt, jt, nj, jb, ng);
    MARIE_LAUNCH_CHECK();
    // u = PS.' e1, w = PS.' e2, y = (1/ce)(M1 u + M2 w)
    MARIE_TRY(spmv<T>(d[M_PST], nj, ng, nullptr, 0, u, nt, (T)1, nr, s));
    MARIE_TRY(spmv<T>(d[M_PST], jb, ng, nullptr, 0, w, nt, (T)1, nr, s));
    k_pf_combine<T><<<dim3(vb, nr), 256, 0, s>>>(nt, h->m1, h->m2, u, w, yr, nt, h->ce_im);
    MARIE_LAUNCH_CHECK();
    // near corrections: y_c += Z_cc Jc + Z_bc_N.' Jb; y_b += -Z_bc_N Jc
    MARIE_TRY(spmv<T>(d[M_ZCC], xr, nt, yr, nt, yr, nt, (T)1, nr, s));
    MARIE_TRY(spmv<T>(*zbt, xr + h->n_sie, nt, yr, nt, yr, nt, (T)1, nr, s));
    MARIE_TRY(spmv<T>(d[M_ZBC], xr, nt, yr + h->n_sie, nt, yr + h->n_sie, nt, (T)-1, nr, s));
  }
  return MARIE_OK;
}

}  // namespace
}  // namespace marie

using namespace marie;

extern "C" {

marie_status marie_svie_pfft_create(marie_svie_pfft** out, const marie_svie_pfft_desc* d) {
  if (!out) { set_error("svie_pfft: output handle pointer is NULL"); return MARIE_ERR_BAD_ARG; }
  *out = nullptr;
  if (!d || !d->grid_op) { set_error("svie_pfft: desc or grid_op is NULL"); return MARIE_ERR_BAD_ARG; }
  marie_vie* g = d->grid_op;
  if (g->on1) {
    set_error("svie_pfft: the extended-grid operator must not be embedded (its grid mode is refused)");
    return MARIE_ERR_BAD_ARG;
  }
  if (d->n_sie < 0 || d->n_b < 0 || d->n_sie + d->n_b < 1) { set_error("svie_pfft: n_sie / n_b invalid"); return MARIE_ERR_BAD_ARG; }
  if (!d->ext_Mc_inv) { set_error("svie_pfft: ext_Mc_inv is NULL"); return MARIE_ERR_BAD_ARG; }
  const int64_t nvox = (int64_t)g->n1 * g->n2 * g->n3;
  const int64_t ng = nvox * g->C, nt = d->n_sie + d->n_b;
  HostCsr ps, zcc, zbc;
  if (!read_csr(d->PS, ps, "PS") || !read_csr(d->Z_cc, zcc, "Z_cc") || !read_csr(d->Z_bc_N, zbc, "Z_bc_N"))
    return MARIE_ERR_BAD_ARG;
  if (ps.rows != ng || ps.cols != nt) {
    set_error("svie_pfft: PS must be (n1*n2*n3*ql) x (n_sie + n_b) = %lld x %lld, got %lld x %lld", (long long)ng,
              (long long)nt, (long long)ps.rows, (long long)ps.cols);
    return MARIE_ERR_BAD_ARG;
  }
  if (zcc.rows != d->n_sie || zcc.cols != d->n_sie) { set_error("svie_pfft: Z_cc must be n_sie x n_sie"); return MARIE_ERR_BAD_ARG; }
  if (zbc.rows != d->n_b || zbc.cols != d->n_sie) { set_error("svie_pfft: Z_bc_N must be n_b x n_sie"); return MARIE_ERR_BAD_ARG; }
  if (!g->p64.built && !g->pff.built && !g->p32.built) { set_error("svie_pfft: grid_op has no precision built"); return MARIE_ERR_BAD_ARG; }
  auto* h = new (std::nothrow) marie_svie_pfft();
  if (!h) { set_error("svie_pfft: out of host memory"); return MARIE_ERR_OOM; }
  auto fail = [&](marie_status s) {
    for (void* p : h->allocs) cudaFree(p);
    delete h;
    return s;
  };
  h->grid = g;
  h->n_sie = d->n_sie;
  h->n_b = d->n_b;
  h->n_grid = ng;
  h->nvox = nvox;
  h->ql = g->C;
  h->ce_im = g->ce_im;
  const HostCsr mats[5] = {column_range(ps, d->n_sie, nt), column_range(ps, 0, d->n_sie), transpose(ps), zcc, zbc};
  const HostCsr zbt = transpose(zbc);
  marie_status st;
  for (int i = 0; i < 5; ++i) {
    if ((st = upload<double>(h, mats[i], h->d64[i])) != MARIE_OK) return fail(st);
    if ((st = upload<float>(h, mats[i], h->d32[i])) != MARIE_OK) return fail(st);
  }
  if ((st = upload<double>(h, zbt, h->zbt64)) != MARIE_OK) return fail(st);
  if ((st = upload<float>(h, zbt, h->zbt32)) != MARIE_OK) return fail(st);
  std::vector<cplx<double>> mc(nvox);
  std::vector<cplx<float>> mcf(nvox);
  for (int64_t i = 0; i < nvox; ++i) {
    mc[i] = cplx<double>{d->ext_Mc_inv[2 * i], d->ext_Mc_inv[2 * i + 1]};
    mcf[i] = cplx<float>{(float)mc[i].x, (float)mc[i].y};
  }
  if ((st = pf_alloc(h, (void**)&h->mc64, nvox * sizeof(cplx<double>))) != MARIE_OK) return fail(st);
  if ((st = pf_alloc(h, (void**)&h->mc32, nvox * sizeof(cplx<float>))) != MARIE_OK) return fail(st);
  cudaMemcpy(h->mc64, mc.data(), nvox * sizeof(cplx<double>), cudaMemcpyHostToDevice);
  cudaMemcpy(h->mc32, mcf.data(), nvox * sizeof(cplx<float>), cudaMemcpyHostToDevice);
  // multipliers M1, M2 (default [1; -1] and [0; 1] by block) and the Gram diagonal, in one array
  std::vector<double> mm(2 * nt + 12, 0.0);
  for (int64_t i = 0; i < nt; ++i) {
    mm[i] = d->M1 ? d->M1[i] : (i < d->n_sie ? 1.0 : -1.0);
    mm[nt + i] = d->M2 ? d->M2[i] : (i < d->n_sie ? 0.0 : 1.0);
  }
  const double r3 = g->res * g->res * g->res;
  for (int c = 0; c < g->C; ++c) mm[2 * nt + c] = g->pwl ? ((c % 4) == 0 ? r3 : r3 / 12.0) : r3;
  if ((st = pf_alloc(h, (void**)&h->m1, mm.size() * sizeof(double))) != MARIE_OK) return fail(st);
  h->m2 = h->m1 + nt;
  cudaMemcpy(h->m1, mm.data(), mm.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (cudaDeviceSynchronize() != cudaSuccess) {
    set_error("svie_pfft: device error during create: %s", cudaGetErrorString(cudaGetLastError()));
    return fail(MARIE_ERR_CUDA);
  }
  *out = h;
  return MARIE_OK;
}

marie_status marie_svie_pfft_apply(marie_svie_pfft* h, int32_t prec, const void* x, void* y, int32_t nrhs,
                                   void* stream) {
  if (!h || !x || !y || nrhs < 1) { set_error("svie_pfft_apply: invalid argument"); return MARIE_ERR_BAD_ARG; }
  cudaStream_t s = (cudaStream_t)stream;
  if (prec == MARIE_C128) {
    if (!h->grid->p64.built && !h->grid->pff.built) { set_error("svie_pfft_apply: grid_op has no complex128 state"); return MARIE_ERR_BAD_ARG; }
    return pf_apply<double>(h, (const cplx<double>*)x, (cplx<double>*)y, nrhs, s);
  }
  if (prec == MARIE_C64) {
    if (!h->grid->p32.built) { set_error("svie_pfft_apply: grid_op has no complex64 state"); return MARIE_ERR_BAD_ARG; }
    return pf_apply<float>(h, (const cplx<float>*)x, (cplx<float>*)y, nrhs, s);
  }
  set_error("svie_pfft_apply: prec must be MARIE_C128 or MARIE_C64");
  return MARIE_ERR_BAD_ARG;
}

marie_status marie_svie_pfft_destroy(marie_svie_pfft* h) {
  if (!h) return MARIE_OK;
  cudaDeviceSynchronize();
  for (void* p : h->allocs) cudaFree(p);
  if (h->work) cudaFree(h->work);
  delete h;
  return MARIE_OK;
}

}  // extern "C"
