// Green's-tensor spectra: one-time construction of the octant spectrum of each
// circulant block, either from the reference's Tucker factors (the expansion
// that mvp_N_pwl_tucker.m:31 repeats in every product) or from a dense I_V
// block (assembly_fft_circ_tucker_pwl.m:53 without the HOSVD truncation).
//
// Octant spectrum: for each block, G_hat(kx,ky,kz) for kx in [0,n1], ky in
// [0,n2], kz in [0,n3]; the remaining frequencies follow from the circulant
// symmetry G_hat(2n-k) = s * G_hat(k) per axis (s = +-1 per block and axis,
// see the mirror signs in BlockTab).  Layout [blk][ky][kx][kz], scaled by
// 1/(8 n1 n2 n3) so that the inverse transforms need no normalisation.
#include <cmath>
#include <vector>

#include "internal.h"

namespace marie {

typedef cplx<double> zd;

// out[o][k][i] = sum_j in[o][j][i] * e(j,k),  e(0,k) = 1,
// e(j,k) = w_2n^{jk} + s * w_2n^{-jk}  (j >= 1), k in [0, n]
__global__ void k_circ_axis(const zd* __restrict__ in, zd* __restrict__ out, int n, int s, int64_t inner,
                            int64_t outer, const zd* __restrict__ w2n) {
  const int64_t total = outer * (n + 1) * inner;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ii = idx % inner;
    const int64_t r = idx / inner;
    const int k = (int)(r % (n + 1));
    const int64_t o = r / (n + 1);
    const zd* src = in + o * n * inner + ii;
    zd acc = src[0];
    for (int j = 1; j < n; ++j) {
      const int e = (int)(((int64_t)j * k) % (2 * n));
      const zd w = w2n[e];
      const zd v = src[(int64_t)j * inner];
      // v * (w + s*conj(w))
      const zd ws = {w.x + s * w.x, w.y - s * w.y};
      acc = acc + v * ws;
    }
    out[idx] = acc;
  }
}

// P1[a + r1(b + r2 kz)] = sum_c G[a + r1(b + r2 c)] U3[c + r3 kz]
__global__ void k_tk1(const zd* G, const zd* U3, zd* P1, int r1, int r2, int r3, int nk) {
  const int64_t total = (int64_t)r1 * r2 * nk;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ab = idx % ((int64_t)r1 * r2);
    const int kz = (int)(idx / ((int64_t)r1 * r2));
    zd acc = {0, 0};
    for (int c = 0; c < r3; ++c) acc = acc + G[ab + (int64_t)r1 * r2 * c] * U3[c + (int64_t)r3 * kz];
    P1[idx] = acc;
  }
}

// P2[a + r1(ky + nky kz)] = sum_b P1[a + r1(b + r2 kz)] U2[b + r2 ky]
__global__ void k_tk2(const zd* P1, const zd* U2, zd* P2, int r1, int r2, int nky, int nkz) {
  const int64_t total = (int64_t)r1 * nky * nkz;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(idx % r1);
    const int64_t r = idx / r1;
    const int ky = (int)(r % nky);
    const int kz = (int)(r / nky);
    zd acc = {0, 0};
    for (int b = 0; b < r2; ++b) acc = acc + P1[a + (int64_t)r1 * (b + (int64_t)r2 * kz)] * U2[b + (int64_t)r2 * ky];
    P2[idx] = acc;
  }
}

// tmp[kx + nkx(ky + nky kz)] = sum_a P2[a + r1(ky + nky kz)] U1[a + r1 kx]
__global__ void k_tk3(const zd* P2, const zd* U1, zd* tmp, int r1, int nkx, int nky, int nkz) {
  const int64_t total = (int64_t)nkx * nky * nkz;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int kx = (int)(idx % nkx);
    const int64_t yz = idx / nkx;
    zd acc = {0, 0};
    for (int a = 0; a < r1; ++a) acc = acc + P2[a + (int64_t)r1 * yz] * U1[a + (int64_t)r1 * kx];
    tmp[idx] = acc;
  }
}

// dst[(ky*nkx + kx)*nkz + kz] = scale * tmp[kx + nkx(ky + nky kz)]
template <typename T>
__global__ void k_oct_store(const zd* tmp, cplx<T>* dst, int nkx, int nky, int nkz, double scl) {
  const int64_t total = (int64_t)nkx * nky * nkz;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int kz = (int)(idx % nkz);
    const int64_t r = idx / nkz;
    const int kx = (int)(r % nkx);
    const int ky = (int)(r / nkx);
    const zd v = tmp[kx + (int64_t)nkx * (ky + (int64_t)nky * kz)];
    dst[idx] = cplx<T>{(T)(v.x * scl), (T)(v.y * scl)};
  }
}

// Full spectrum of one block for the four-step z pass, layout
// [ky][kx][kz][blk] over the whole (2n2, 2n1, 2n3) grid with the circulant
// mirror signs applied: dst[((ky*2n1 + kx)*2n3 + kz)*U + blk].
template <typename T>
__global__ void k_full_store(const zd* tmp, cplx<T>* dst, int n1, int n2, int n3, int U, int blk, int s1, int s2,
                             int s3, double scl) {
  const int m1 = 2 * n1, m2 = 2 * n2, m3 = 2 * n3;
  const int nkx = n1 + 1, nky = n2 + 1;
  const int64_t total = (int64_t)m1 * m2 * m3;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int kz = (int)(idx % m3);
    const int64_t r = idx / m3;
    const int kx = (int)(r % m1);
    const int ky = (int)(r / m1);
    const bool mx = kx > n1, my = ky > n2, mz = kz > n3;
    const int kxo = mx ? m1 - kx : kx, kyo = my ? m2 - ky : ky, kzo = mz ? m3 - kz : kz;
    const double sg = (double)((mx ? s1 : 1) * (my ? s2 : 1) * (mz ? s3 : 1)) * scl;
    const zd v = tmp[kxo + (int64_t)nkx * (kyo + (int64_t)nky * kzo)];
    dst[idx * U + blk] = cplx<T>{(T)(v.x * sg), (T)(v.y * sg)};
  }
}

// The same for the complex64 z pass (k4_zp), pair layout: frequencies 2k and
// 2k+1 of a column share one 16-byte entry (re, re, im, im) at
// ((ky*2n1 + kx)*U + blk)*n3 + k.
__global__ void k_full_store_pair(const zd* tmp, float* dst, int n1, int n2, int n3, int U, int blk, int s1, int s2,
                                  int s3, double scl) {
  const int m1 = 2 * n1, m2 = 2 * n2, m3 = 2 * n3;
  const int nkx = n1 + 1, nky = n2 + 1;
  const int64_t total = (int64_t)m1 * m2 * m3;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int kz = (int)(idx % m3);
    const int64_t r = idx / m3;
    const int kx = (int)(r % m1);
    const int ky = (int)(r / m1);
    const bool mx = kx > n1, my = ky > n2, mz = kz > n3;
    const int kxo = mx ? m1 - kx : kx, kyo = my ? m2 - ky : ky, kzo = mz ? m3 - kz : kz;
    const double sg = (double)((mx ? s1 : 1) * (my ? s2 : 1) * (mz ? s3 : 1)) * scl;
    const zd v = tmp[kxo + (int64_t)nkx * (kyo + (int64_t)nky * kzo)];
    float* d = dst + ((r * U + blk) * n3 + (kz >> 1)) * 4 + (kz & 1);
    d[0] = (float)(v.x * sg);
    d[2] = (float)(v.y * sg);
  }
}

static unsigned grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 65535LL * 16) b = 65535LL * 16;
  return (unsigned)std::max<int64_t>(1, b);
}

// The octant storage needs the circulant parity of every block: a block that
// is odd along an axis (mirror sign -1) must vanish on that axis' zero-offset
// plane, otherwise G_hat(2n-k) != -G_hat(k).  Operators assembled by
// assembly_N/K satisfy it to rounding (symmetric Gauss rules); reject others.
static const double kParityTol = 1e-9;

static marie_status check_parity_dense(const double* A, int n1, int n2, int n3, const int8_t s[3], int id) {
  const int64_t nD = (int64_t)n1 * n2 * n3;
  double mx = 0, bad = 0;
  for (int64_t g = 0; g < nD; ++g) {
    const double v = std::hypot(A[2 * g], A[2 * g + 1]);
    mx = std::max(mx, v);
    const int x = (int)(g % n1), y = (int)((g / n1) % n2), z = (int)(g / ((int64_t)n1 * n2));
    if ((s[0] < 0 && x == 0) || (s[1] < 0 && y == 0) || (s[2] < 0 && z == 0)) bad = std::max(bad, v);
  }
  if (bad > kParityTol * mx) {
    set_error("operator block %d violates the circulant parity (odd block nonzero on its zero-offset plane, "
              "relative %.3e)", id, mx > 0 ? bad / mx : bad);
    return MARIE_ERR_BAD_ARG;
  }
  return MARIE_OK;
}

// Tucker block: the zero-offset sample of factor column a along axis d is
// u0[a] = (1/2n) sum_k U_d[a + r k] (inverse FFT at index 0).  Weighted by the
// norm of the core slice it multiplies (the HOSVD singular value), it bounds
// the block's value on the zero-offset plane relative to the block.
static marie_status check_parity_tucker(const marie_tucker_block& t, int n1, int n2, int n3, const int8_t s[3],
                                        int id) {
  const int r[3] = {t.r1, t.r2, t.r3};
  const int n[3] = {n1, n2, n3};
  const double* U[3] = {t.U1, t.U2, t.U3};
  for (int d = 0; d < 3; ++d) {
    if (s[d] > 0) continue;
    std::vector<double> sl(r[d], 0.0);
    for (int c = 0; c < t.r3; ++c)
      for (int b = 0; b < t.r2; ++b)
        for (int a = 0; a < t.r1; ++a) {
          const int64_t g = a + (int64_t)t.r1 * (b + (int64_t)t.r2 * c);
          const double v2 = t.G[2 * g] * t.G[2 * g] + t.G[2 * g + 1] * t.G[2 * g + 1];
          sl[d == 0 ? a : (d == 1 ? b : c)] += v2;
        }
    double smax = 0, worst = 0;
    for (int a = 0; a < r[d]; ++a) smax = std::max(smax, std::sqrt(sl[a]));
    for (int a = 0; a < r[d]; ++a) {
      double sx = 0, sy = 0;
      for (int k = 0; k < 2 * n[d]; ++k) {
        sx += U[d][2 * (a + (int64_t)r[d] * k)];
        sy += U[d][2 * (a + (int64_t)r[d] * k) + 1];
      }
      worst = std::max(worst, std::hypot(sx, sy) / (2.0 * n[d]) * std::sqrt(sl[a]));
    }
    if (worst > kParityTol * std::max(smax, 1e-300)) {
      set_error("Tucker block %d violates the circulant parity along axis %d (odd block nonzero on its "
                "zero-offset plane, relative %.3e)", id, d + 1, worst / smax);
      return MARIE_ERR_BAD_ARG;
    }
  }
  return MARIE_OK;
}

// Build all blocks of one operator (N or K) into the handle's spectra.
// Spectrum destinations of one operator: octant per precision (generic
// path, K) and full block-interleaved (four-step path, N); null = not built.
struct SpecDst {
  cplx<double>* o64 = nullptr;
  cplx<float>* o32 = nullptr;
  cplx<double>* f64 = nullptr;
  cplx<float>* f32 = nullptr;
  cplx<ff>* fff = nullptr;
};

static marie_status build_op(marie_vie* h, const marie_tucker_block* tk, const double* dense, int ncomp,
                             const SpecDst& dst) {
  const int n1 = h->n1, n2 = h->n2, n3 = h->n3;
  const int pwx = h->pwl ? 10 : 1;
  const int nblk = pwx * ncomp;
  const int nkx = n1 + 1, nky = n2 + 1, nkz = n3 + 1;
  const int64_t oct = (int64_t)nkx * nky * nkz;
  const int64_t nD = (int64_t)n1 * n2 * n3;
  const double scl = 1.0 / (8.0 * (double)n1 * (double)n2 * (double)n3);
  // scratch
  zd *tmp = nullptr, *a = nullptr, *b = nullptr, *w1 = nullptr, *w2 = nullptr, *w3 = nullptr;
  zd *dG = nullptr, *dU1 = nullptr, *dU2 = nullptr, *dU3 = nullptr;
  std::vector<void*> scratch;
  auto salloc = [&](zd** p, size_t count) -> marie_status {
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(zd));
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error("scratch allocation of %zu bytes failed", count * sizeof(zd));
      return MARIE_ERR_OOM;
    }
    scratch.push_back(*p);
    return MARIE_OK;
  };
  auto cleanup = [&]() {
    cudaDeviceSynchronize();
    for (void* p : scratch) cudaFree(p);
  };
  marie_status st = MARIE_OK;
  const int tabk = ncomp == 6 ? 0 : 2;   // N or K table (mirror signs)
  const BlockTab& bt = h->tab[tabk];
  const int64_t full = (int64_t)8 * n1 * n2 * n3;
  auto store_block = [&](int id) {
    if (dst.o64) { k_oct_store<double><<<grid_for(oct), 256>>>(tmp, dst.o64 + id * oct, nkx, nky, nkz, scl); g_launches++; }
    if (dst.o32) { k_oct_store<float><<<grid_for(oct), 256>>>(tmp, dst.o32 + id * oct, nkx, nky, nkz, scl); g_launches++; }
    const int s1 = bt.s1[id], s2 = bt.s2[id], s3 = bt.s3[id];
    if (dst.f64) {
      k_full_store<double><<<grid_for(full), 256>>>(tmp, dst.f64, n1, n2, n3, nblk, id, s1, s2, s3, scl);
      g_launches++;
    }
    if (dst.f32) {
      k_full_store_pair<<<grid_for(full), 256>>>(tmp, reinterpret_cast<float*>(dst.f32), n1, n2, n3, nblk, id, s1, s2,
                                                  s3, scl);
      g_launches++;
    }
    if (dst.fff) {
      k_full_store<ff><<<grid_for(full), 256>>>(tmp, dst.fff, n1, n2, n3, nblk, id, s1, s2, s3, scl);
      g_launches++;
    }
  };
  do {
    if ((st = salloc(&tmp, oct)) != MARIE_OK) break;
    if (dense) {
      if ((st = salloc(&a, nD)) != MARIE_OK) break;
      if ((st = salloc(&b, (int64_t)nkx * nky * n3)) != MARIE_OK) break;
      // w_2n tables per axis
      zd* ws[3] = {nullptr, nullptr, nullptr};
      const int ns[3] = {n1, n2, n3};
      for (int d = 0; d < 3 && st == MARIE_OK; ++d) {
        if ((st = salloc(&ws[d], 2 * ns[d])) != MARIE_OK) break;
        std::vector<zd> w(2 * ns[d]);
        for (int k = 0; k < 2 * ns[d]; ++k) {
          const long double ang = -3.141592653589793238462643383279502884L * (long double)k / (long double)ns[d];
          w[k] = zd{(double)std::cos(ang), (double)std::sin(ang)};
        }
        cudaMemcpy(ws[d], w.data(), 2 * ns[d] * sizeof(zd), cudaMemcpyHostToDevice);
      }
      if (st != MARIE_OK) break;
      w1 = ws[0]; w2 = ws[1]; w3 = ws[2];
      zd* c = nullptr;
      if ((st = salloc(&c, (int64_t)nkx * nky * n3)) != MARIE_OK) break;
      for (int id = 0; id < nblk; ++id) {
        // dense I_V is (n1,n2,n3,pwx,ncomp) column-major: block (j,k) at (j + pwx*k)*nD
        const int j = id / ncomp, k = id % ncomp;
        const double* src = dense + 2 * ((int64_t)(j + pwx * k) * nD);
        const int8_t sg[3] = {bt.s1[id], bt.s2[id], bt.s3[id]};
        if ((st = check_parity_dense(src, n1, n2, n3, sg, id)) != MARIE_OK) break;
        if (cudaMemcpy(a, src, nD * sizeof(zd), cudaMemcpyHostToDevice) != cudaSuccess) {
          set_error("upload of dense I_V failed");
          st = MARIE_ERR_CUDA;
          break;
        }
        k_circ_axis<<<grid_for((int64_t)nkx * n2 * n3), 256>>>(a, b, n1, bt.s1[id], 1, (int64_t)n2 * n3, w1);
        g_launches++;
        k_circ_axis<<<grid_for((int64_t)nkx * nky * n3), 256>>>(b, c, n2, bt.s2[id], nkx, n3, w2);
        g_launches++;
        k_circ_axis<<<grid_for(oct), 256>>>(c, tmp, n3, bt.s3[id], (int64_t)nkx * nky, 1, w3);
        g_launches++;
        store_block(id);
        if (cudaGetLastError() != cudaSuccess) { set_error("spectrum kernel launch failed"); st = MARIE_ERR_CUDA; break; }
        cudaDeviceSynchronize();
      }
    } else {
      int mr1 = 1, mr2 = 1, mr3 = 1;
      int64_t mg = 1, mp1 = 1, mp2 = 1;
      for (int id = 0; id < nblk; ++id) {
        const marie_tucker_block& t = tk[id];
        if (t.r1 < 1 || t.r2 < 1 || t.r3 < 1 || !t.G || !t.U1 || !t.U2 || !t.U3) {
          set_error("Tucker block %d is incomplete", id);
          st = MARIE_ERR_BAD_ARG;
          break;
        }
        const int8_t sg[3] = {bt.s1[id], bt.s2[id], bt.s3[id]};
        if ((st = check_parity_tucker(t, n1, n2, n3, sg, id)) != MARIE_OK) break;
        mr1 = std::max(mr1, t.r1); mr2 = std::max(mr2, t.r2); mr3 = std::max(mr3, t.r3);
        mg = std::max<int64_t>(mg, (int64_t)t.r1 * t.r2 * t.r3);
        mp1 = std::max<int64_t>(mp1, (int64_t)t.r1 * t.r2 * nkz);
        mp2 = std::max<int64_t>(mp2, (int64_t)t.r1 * nky * nkz);
      }
      if (st != MARIE_OK) break;
      if ((st = salloc(&dG, mg)) != MARIE_OK) break;
      if ((st = salloc(&dU1, (int64_t)mr1 * 2 * n1)) != MARIE_OK) break;
      if ((st = salloc(&dU2, (int64_t)mr2 * 2 * n2)) != MARIE_OK) break;
      if ((st = salloc(&dU3, (int64_t)mr3 * 2 * n3)) != MARIE_OK) break;
      if ((st = salloc(&a, mp1)) != MARIE_OK) break;
      if ((st = salloc(&b, mp2)) != MARIE_OK) break;
      for (int id = 0; id < nblk; ++id) {
        const marie_tucker_block& t = tk[id];
        cudaMemcpy(dG, t.G, (size_t)t.r1 * t.r2 * t.r3 * sizeof(zd), cudaMemcpyHostToDevice);
        cudaMemcpy(dU1, t.U1, (size_t)t.r1 * 2 * n1 * sizeof(zd), cudaMemcpyHostToDevice);
        cudaMemcpy(dU2, t.U2, (size_t)t.r2 * 2 * n2 * sizeof(zd), cudaMemcpyHostToDevice);
        cudaMemcpy(dU3, t.U3, (size_t)t.r3 * 2 * n3 * sizeof(zd), cudaMemcpyHostToDevice);
        k_tk1<<<grid_for((int64_t)t.r1 * t.r2 * nkz), 256>>>(dG, dU3, a, t.r1, t.r2, t.r3, nkz);
        g_launches++;
        k_tk2<<<grid_for((int64_t)t.r1 * nky * nkz), 256>>>(a, dU2, b, t.r1, t.r2, nky, nkz);
        g_launches++;
        k_tk3<<<grid_for(oct), 256>>>(b, dU1, tmp, t.r1, nkx, nky, nkz);
        g_launches++;
        store_block(id);
        if (cudaGetLastError() != cudaSuccess) { set_error("spectrum kernel launch failed"); st = MARIE_ERR_CUDA; break; }
        cudaDeviceSynchronize();
      }
    }
  } while (0);
  cleanup();
  return st;
}

marie_status build_spectra(marie_vie* h, const marie_vie_desc* d) {
  const int64_t oct = (int64_t)(h->n1 + 1) * (h->n2 + 1) * (h->n3 + 1);
  const int64_t full = (int64_t)8 * h->n1 * h->n2 * h->n3;
  const bool fast = four_step_grid(h);
  if (h->precisions & 1) {
    MARIE_TRY(dev_alloc(h, (void**)&h->p64.GN, (size_t)h->nblkN * oct * sizeof(cplx<double>)));
    if (h->has_K) MARIE_TRY(dev_alloc(h, (void**)&h->p64.GK, (size_t)h->nblkK * oct * sizeof(cplx<double>)));
    if (fast) MARIE_TRY(dev_alloc(h, (void**)&h->p64.GNf, (size_t)h->nblkN * full * sizeof(cplx<double>)));
  }
  if (h->precisions & 2) {
    MARIE_TRY(dev_alloc(h, (void**)&h->p32.GN, (size_t)h->nblkN * oct * sizeof(cplx<float>)));
    if (h->has_K) MARIE_TRY(dev_alloc(h, (void**)&h->p32.GK, (size_t)h->nblkK * oct * sizeof(cplx<float>)));
    if (fast) MARIE_TRY(dev_alloc(h, (void**)&h->p32.GNf, (size_t)h->nblkN * full * sizeof(cplx<float>)));
  }
  if (h->precisions & 4)   // float-float: four-step path only (N and N^H)
    MARIE_TRY(dev_alloc(h, (void**)&h->pff.GNf, (size_t)h->nblkN * full * sizeof(cplx<ff>)));
  SpecDst dN;
  dN.o64 = h->p64.GN;
  dN.o32 = h->p32.GN;
  dN.f64 = h->p64.GNf;
  dN.f32 = h->p32.GNf;
  dN.fff = h->pff.GNf;
  MARIE_TRY(build_op(h, d->tucker_N, d->tucker_N ? nullptr : d->dense_N, 6, dN));
  if (h->has_K) {
    SpecDst dK;
    dK.o64 = h->p64.GK;
    dK.o32 = h->p32.GK;
    MARIE_TRY(build_op(h, d->tucker_K, d->tucker_K ? nullptr : d->dense_K, 3, dK));
  }
  return MARIE_OK;
}

}  // namespace marie
