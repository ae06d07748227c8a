// Per-application Tucker expansion of the complex64 Green's spectrum: the
// reference's form of the operator (mvp_N_pwl_tucker.m:31 re-expands every
// Tucker block inside every product with nmp.m).
//
// With precisions bit 8 (MARIE_PREC_TUCKER_PER_APPLY) a handle built from
// Tucker blocks keeps their factors on the device in FP32 and rebuilds the
// complex64 full spectrum (the pair layout the four-step z pass reads) at the
// start of every complex64 application of N or N^H, once for all the chunks
// of right-hand sides of that application:
//   P1[a, b, kz] = sum_c G[a, b, c] U3[c, kz]             (r1 r2 x 2n3)
//   P2[a, ky, kz] = sum_b P1[a, b, kz] U2[b, ky]          (r1 x 2n2 x 2n3)
//   G(ky, kx, kz) = sum_a P2[a, ky, kz] U1[a, kx] / (8 n1 n2 n3)
// over the whole (2n)^3 grid (the factors are already circulant-extended and
// transformed, assembly_fft_circ_tucker_pwl.m:50-58), written straight into
// the pair layout: ((ky 2n1 + kx) U + blk) n3 + k holds (re G(2k), re
// G(2k+1), im G(2k), im G(2k+1)).  FP32 arithmetic, as the complex64 path.
#include <algorithm>
#include <vector>

#include "internal.h"

namespace marie {
namespace {

// P1[a + r1 (b + r2 kz)] = sum_c G[a + r1 (b + r2 c)] U3[c + r3 kz]
__global__ void k_tkf1(const cplx<float>* __restrict__ G, const cplx<float>* __restrict__ U3, cplx<float>* P1, int r1,
                       int r2, int r3, int m3) {
  const int64_t total = (int64_t)r1 * r2 * m3;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ab = i % ((int64_t)r1 * r2);
    const int kz = (int)(i / ((int64_t)r1 * r2));
    cplx<float> acc{0.f, 0.f};
    for (int c = 0; c < r3; ++c) fma_c(acc, G[ab + (int64_t)r1 * r2 * c], U3[c + (int64_t)r3 * kz]);
    P1[i] = acc;
  }
}

// P2[a + r1 (ky + m2 kz)] = sum_b P1[a + r1 (b + r2 kz)] U2[b + r2 ky]
__global__ void k_tkf2(const cplx<float>* __restrict__ P1, const cplx<float>* __restrict__ U2, cplx<float>* P2, int r1,
                       int r2, int m2, int m3) {
  const int64_t total = (int64_t)r1 * m2 * m3;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(i % r1);
    const int64_t rest = i / r1;
    const int ky = (int)(rest % m2);
    const int kz = (int)(rest / m2);
    cplx<float> acc{0.f, 0.f};
    const cplx<float>* p = P1 + a + (int64_t)r1 * r2 * kz;
    for (int b = 0; b < r2; ++b) fma_c(acc, p[(int64_t)r1 * b], U2[b + (int64_t)r2 * ky]);
    P2[i] = acc;
  }
}

// The last mode product is, for each ky, the product of U1^T (2n1 x r1)
// with the slab P2[:, ky, :] (r1 x 2n3).  A CTA takes one (ky, block) and a
// tile of kTkX consecutive kx: its threads run over the frequency pairs k
// (coalesced 16-byte stores), each holding the slab's two rank vectors for
// its pair in registers, with the tile's U1 columns staged in shared
// memory and read as broadcasts.
constexpr int kTkX = 16;
constexpr int kTkMaxR = 32;     // largest r1 of the per-application mode (checked at create)
__global__ void __launch_bounds__(128) k_tkf3(const cplx<float>* __restrict__ P2, const cplx<float>* __restrict__ U1,
                                              float4* dst, int r1, int m1, int m2, int n3, int U, int blk, float scl) {
  __shared__ cplx<float> u[kTkMaxR * kTkX];
  const int ky = blockIdx.y;
  const int kx0 = blockIdx.x * kTkX;
  const int nkx = min(kTkX, m1 - kx0);
  for (int i = threadIdx.x; i < r1 * nkx; i += blockDim.x) {
    const int a = i % r1, j = i / r1;
    u[j * kTkMaxR + a] = U1[a + (int64_t)r1 * (kx0 + j)];
  }
  __syncthreads();
  for (int k = threadIdx.x; k < n3; k += blockDim.x) {
    cplx<float> p0[kTkMaxR], p1[kTkMaxR];
    const cplx<float>* q0 = P2 + (int64_t)r1 * (ky + (int64_t)m2 * (2 * k));
    const cplx<float>* q1 = q0 + (int64_t)r1 * m2;
#pragma unroll
    for (int a = 0; a < kTkMaxR; ++a) {
      if (a < r1) {
        p0[a] = q0[a];
        p1[a] = q1[a];
      }
    }
    for (int j = 0; j < nkx; ++j) {
      cplx<float> g0{0.f, 0.f}, g1{0.f, 0.f};
      const cplx<float>* uj = u + j * kTkMaxR;
#pragma unroll
      for (int a = 0; a < kTkMaxR; ++a) {
        if (a < r1) {
          fma_c(g0, p0[a], uj[a]);
          fma_c(g1, p1[a], uj[a]);
        }
      }
      const int64_t col = (int64_t)ky * m1 + kx0 + j;
      dst[(col * U + blk) * n3 + k] = make_float4(g0.x * scl, g1.x * scl, g0.y * scl, g1.y * scl);
    }
  }
}

unsigned grid_of(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (unsigned)std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 32);
}

}  // namespace

marie_status tucker_keep_c64(marie_vie* h, const marie_tucker_block* tk) {
  const int nblk = h->nblkN;
  TuckerDev& t = h->tkf;
  t.blocks.assign(nblk, TuckerDev::Block{});
  size_t mp1 = 1, mp2 = 1;
  const int m1 = 2 * h->n1, m2 = 2 * h->n2, m3 = 2 * h->n3;
  for (int id = 0; id < nblk; ++id) {
    const marie_tucker_block& b = tk[id];
    if (b.r1 > kTkMaxR) {
      set_error("per-application Tucker expansion: block %d has rank r1 = %d above %d", id, b.r1, kTkMaxR);
      return MARIE_ERR_NOT_SUPPORTED;
    }
    TuckerDev::Block& d = t.blocks[id];
    d.r1 = b.r1;
    d.r2 = b.r2;
    d.r3 = b.r3;
    const size_t ng = (size_t)b.r1 * b.r2 * b.r3, n1 = (size_t)b.r1 * m1, n2 = (size_t)b.r2 * m2,
                 n3 = (size_t)b.r3 * m3;
    MARIE_TRY(dev_alloc(h, (void**)&d.G, (ng + n1 + n2 + n3) * sizeof(cplx<float>)));
    d.U1 = d.G + ng;
    d.U2 = d.U1 + n1;
    d.U3 = d.U2 + n2;
    std::vector<cplx<float>> host(ng + n1 + n2 + n3);
    const double* srcs[4] = {b.G, b.U1, b.U2, b.U3};
    const size_t cnt[4] = {ng, n1, n2, n3};
    size_t o = 0;
    for (int q = 0; q < 4; ++q)
      for (size_t e = 0; e < cnt[q]; ++e, ++o) host[o] = cplx<float>{(float)srcs[q][2 * e], (float)srcs[q][2 * e + 1]};
    MARIE_CUDA_TRY(cudaMemcpy(d.G, host.data(), host.size() * sizeof(cplx<float>), cudaMemcpyHostToDevice));
    mp1 = std::max(mp1, (size_t)b.r1 * b.r2 * m3);
    mp2 = std::max(mp2, (size_t)b.r1 * m2 * m3);
  }
  MARIE_TRY(dev_alloc(h, (void**)&t.P1, mp1 * sizeof(cplx<float>)));
  MARIE_TRY(dev_alloc(h, (void**)&t.P2, mp2 * sizeof(cplx<float>)));
  t.active = true;
  return MARIE_OK;
}

marie_status tucker_expand_c64(marie_vie* h, cudaStream_t s) {
  TuckerDev& t = h->tkf;
  const int m1 = 2 * h->n1, m2 = 2 * h->n2, m3 = 2 * h->n3, n3 = h->n3;
  const int U = h->nblkN;
  const float scl = (float)(1.0 / (8.0 * (double)h->n1 * (double)h->n2 * (double)h->n3));
  float4* dst = reinterpret_cast<float4*>(h->p32.GNf);
  for (int id = 0; id < U; ++id) {
    const TuckerDev::Block& b = t.blocks[id];
    k_tkf1<<<grid_of((int64_t)b.r1 * b.r2 * m3), 256, 0, s>>>(b.G, b.U3, t.P1, b.r1, b.r2, b.r3, m3);
    MARIE_LAUNCH_CHECK();
    k_tkf2<<<grid_of((int64_t)b.r1 * m2 * m3), 256, 0, s>>>(t.P1, b.U2, t.P2, b.r1, b.r2, m2, m3);
    MARIE_LAUNCH_CHECK();
    k_tkf3<<<dim3((unsigned)((m1 + kTkX - 1) / kTkX), (unsigned)m2), 128, 0, s>>>(t.P2, b.U1, dst, b.r1, m1, m2, n3,
                                                                                U, id, scl);
    MARIE_LAUNCH_CHECK();
  }
  return MARIE_OK;
}

}  // namespace marie
