// FFT-VIE matvec: y = crop(IFFT3( G_hat (.) FFT3(pad(x)) )) over C current
// components, with the circulant Green's tensor applied as a C x C block
// matrix at every frequency, followed (for the VIE operator) by the contrast
// epilogue  y = x - chi * invG(N x).
//
// The zero-padded length-2n DFT along each axis is split into two length-n
// DFTs (even frequencies: DFT(x); odd: DFT(x * w_2n^i)), so every transform
// is an in-place length-n FFT in shared memory.  Spectra in HBM are stored
// per axis as [parity][digit-reversed position] (x and y axes); the z axis
// never leaves shared memory.
//
// Passes (per right-hand side and component):
//   X  : scatter from the body vector (+ optional prologue scale), x-DFT     n^3  -> 2n^3
//   Y  : y-DFT                                                               2n^3 -> 4n^3
//   Z  : z-DFT, Green block multiply, inverse z-DFT (in place)               4n^3 -> 4n^3
//   YI : inverse y-DFT + crop                                                4n^3 -> 2n^3
//   XI : inverse x-DFT + crop + epilogue + gather                            2n^3 -> n^3
#pragma once

#include "common.cuh"

namespace marie {

constexpr int kMaxComp = 12;
constexpr int kMaxBlocks = 60;

enum MvMode : int {
  MV_GRID = 0,      // input/output are full grids (n1,n2,n3,C) column-major
  MV_VIE = 1,       // y = x - chi .* invG(N x) on the body vector
  MV_VIE_ADJ = 2,   // y = x - N^H(invG .* conj(chi) .* x) on the body vector
};

// Per-axis lookup tables (device pointers).
template <typename T>
struct AxisTab {
  const cplx<T>* tw;    // w_n^k, k < n (forward sign)
  const cplx<T>* tw2;   // w_2n^k, k < n
  const int* kofp;      // digit-reversed position -> frequency index (length n)
  const int* pofk;      // frequency index -> position
  FftPlan plan;
};

// Operator block table: out component p, in component q -> (block, sign).
struct BlockTab {
  int8_t blk[kMaxComp * kMaxComp];   // -1: no block
  int8_t sgn[kMaxComp * kMaxComp];
  int8_t s1[kMaxBlocks], s2[kMaxBlocks], s3[kMaxBlocks];  // circulant mirror signs per axis
  int conj;                                               // use conj(G_hat)
  int nblk;
};

template <typename T>
struct MvArgs {
  int n1, n2, n3, C, nrhs;
  int64_t Ns;                 // body voxels
  int mode;
  AxisTab<T> ax, ay, az;
  const int* vox2sol;         // n1*n2*n3 -> body index or -1
  const cplx<T>* chi;         // contrast (Mc/Mr) per body voxel
  T invg[kMaxComp];           // invG diagonal per component
  const cplx<T>* in;          // nrhs x (C*Ns) or nrhs x (C*n^3)
  cplx<T>* out;
  int64_t in_rs, out_rs;      // element stride between right-hand sides
  cplx<T>* T1;                // [rhs][c][z][y][2n1]
  cplx<T>* S;                 // [rhs][c][2n2][z][2n1]
  const cplx<T>* G;           // octant spectra [blk][n2+1][n1+1][n3+1]
  const unsigned char* active;  // per rhs: nonzero = process (may be null)
  int TY, TXY, TX;            // tile sizes of the X, Y, Z passes
};

template <typename T>
__device__ __forceinline__ void load_tw(cplx<T>* dst, const cplx<T>* src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

// ---------------------------------------------------------------------------
// Pass X (forward).  grid (ceil(n2/TY), n3, nrhs*C)
// smem: tw[n1] | buf[TY][2][n1]
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_fwd_x(MvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int rc = blockIdx.z, rhs = rc / a.C, c = rc - rhs * a.C;
  if (a.active && !a.active[rhs]) return;
  const int z = blockIdx.y, y0 = blockIdx.x * a.TY;
  const int n1 = a.n1, n2 = a.n2, n3 = a.n3;
  const int ty = min(a.TY, n2 - y0);
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + n1;
  load_tw(tw, a.ax.tw, n1);
  const int64_t nD = (int64_t)n1 * n2 * n3;
  for (int i = threadIdx.x; i < ty * n1; i += blockDim.x) {
    const int yy = i / n1, x = i - yy * n1;
    const int y = y0 + yy;
    const int64_t g = x + (int64_t)n1 * (y + (int64_t)n2 * z);
    cplx<T> v = {0, 0};
    if (a.mode == MV_GRID) {
      v = a.in[(int64_t)rhs * a.in_rs + (int64_t)c * nD + g];
    } else {
      const int s = a.vox2sol[g];
      if (s >= 0) {
        v = a.in[(int64_t)rhs * a.in_rs + (int64_t)c * a.Ns + s];
        if (a.mode == MV_VIE_ADJ) v = scale(mulc(v, a.chi[s]), a.invg[c]);
      }
    }
    buf[(yy * 2 + 0) * n1 + x] = v;
    buf[(yy * 2 + 1) * n1 + x] = v * a.ax.tw2[x];
  }
  __syncthreads();
  fft_dif<T, false>(buf, 2 * ty, 1, n1, a.ax.plan, tw, false);
  cplx<T>* dst = a.T1 + (((int64_t)rhs * a.C + c) * n3 + z) * (int64_t)n2 * 2 * n1;
  for (int i = threadIdx.x; i < ty * 2 * n1; i += blockDim.x) {
    const int yy = i / (2 * n1), kx = i - yy * 2 * n1;
    dst[(int64_t)(y0 + yy) * 2 * n1 + kx] = buf[i];
  }
}

// ---------------------------------------------------------------------------
// Pass Y (forward).  grid (ceil(2n1/TXY), n3, nrhs*C)
// smem: tw[n2] | buf[n2][2][TXY]
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_fwd_y(MvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int rc = blockIdx.z, rhs = rc / a.C, c = rc - rhs * a.C;
  if (a.active && !a.active[rhs]) return;
  const int z = blockIdx.y, k0 = blockIdx.x * a.TXY;
  const int n1 = a.n1, n2 = a.n2, n3 = a.n3, m1 = 2 * n1;
  const int tx = min(a.TXY, m1 - k0);
  const int TXY = a.TXY;
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + n2;
  load_tw(tw, a.ay.tw, n2);
  const cplx<T>* src = a.T1 + (((int64_t)rhs * a.C + c) * n3 + z) * (int64_t)n2 * m1;
  for (int i = threadIdx.x; i < n2 * TXY; i += blockDim.x) {
    const int y = i / TXY, t = i - y * TXY;
    cplx<T> v = {0, 0};
    if (t < tx) v = src[(int64_t)y * m1 + k0 + t];
    buf[(y * 2 + 0) * TXY + t] = v;
    buf[(y * 2 + 1) * TXY + t] = v * a.ay.tw2[y];
  }
  __syncthreads();
  fft_dif<T, false>(buf, 2 * TXY, 2 * TXY, 1, a.ay.plan, tw, true);
  cplx<T>* dst = a.S + ((int64_t)rhs * a.C + c) * (int64_t)2 * n2 * n3 * m1;
  for (int i = threadIdx.x; i < 2 * n2 * TXY; i += blockDim.x) {
    const int row = i / TXY, t = i - row * TXY;   // row = beta*n2 + p
    const int beta = row / n2, p = row - beta * n2;
    if (t < tx) dst[((int64_t)row * n3 + z) * m1 + k0 + t] = buf[(p * 2 + beta) * TXY + t];
  }
}

// ---------------------------------------------------------------------------
// Pass Z (fused).  grid (ceil(2n1/TX), 2n2, nrhs)
// smem: tw[n3] | buf[n3][2*C*TX + 1]
// row i of buf holds, for each (gamma, c, t), the z-sample / frequency i.
// ---------------------------------------------------------------------------
template <typename T, int CC>
__global__ void k_z(MvArgs<T> a, BlockTab bt) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int rhs = blockIdx.z;
  if (a.active && !a.active[rhs]) return;
  const int kyp = blockIdx.y, k0 = blockIdx.x * a.TX;
  const int n1 = a.n1, n2 = a.n2, n3 = a.n3, m1 = 2 * n1, TX = a.TX;
  constexpr int C = CC;
  const int tx = min(TX, m1 - k0);
  const int rs = 2 * C * TX + 1;   // row stride (padded)
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + n3;
  load_tw(tw, a.az.tw, n3);
  // load: element z of sequence (gamma, c, t) goes to row pofk[z] (DIT input order)
  const int64_t cstride = (int64_t)2 * n2 * n3 * m1;
  const cplx<T>* src = a.S + (int64_t)rhs * C * cstride + ((int64_t)kyp * n3) * m1 + k0;
  for (int i = threadIdx.x; i < C * n3 * TX; i += blockDim.x) {
    const int t = i % TX;
    const int rest = i / TX;
    const int z = rest % n3, c = rest / n3;
    cplx<T> v = {0, 0};
    if (t < tx) v = src[c * cstride + (int64_t)z * m1 + t];
    const int row = a.az.pofk[z];
    buf[row * rs + (0 * C + c) * TX + t] = v;
    buf[row * rs + (1 * C + c) * TX + t] = v * a.az.tw2[z];
  }
  __syncthreads();
  fft_dit<T, false>(buf, 2 * C * TX, rs, 1, a.az.plan, tw, true);

  // Green block multiply, natural frequency order in rows.
  // pencil (kx, ky): kx = 2*kofp[pos] + alpha for kx' = alpha*n1 + pos
  const int beta = kyp / n2, py = kyp - beta * n2;
  const int ky = 2 * a.ay.kofp[py] + beta;
  const bool my = ky > n2;
  const int kyo = my ? 2 * n2 - ky : ky;
  const int nko = n3 + 1;
  for (int i = threadIdx.x; i < TX * nko; i += blockDim.x) {
    const int t = i / nko, ko = i - t * nko;
    if (t >= tx) continue;
    const int kxp = k0 + t;
    const int alpha = kxp / n1, px = kxp - alpha * n1;
    const int kx = 2 * a.ax.kofp[px] + alpha;
    const bool mx = kx > n1;
    const int kxo = mx ? 2 * n1 - kx : kx;
    const int kz0 = ko, kz1 = 2 * n3 - ko;
    const bool two = (ko != 0) && (ko != n3);
    const int r0 = kz0 >> 1, g0 = kz0 & 1;
    const int r1 = (kz1 >> 1) % n3, g1 = kz1 & 1;
    cplx<T> x0[C], x1[C];
#pragma unroll
    for (int q = 0; q < C; ++q) {
      x0[q] = buf[r0 * rs + (g0 * C + q) * TX + t];
      x1[q] = two ? buf[r1 * rs + (g1 * C + q) * TX + t] : cplx<T>{0, 0};
    }
    const int64_t gpen = ((int64_t)kyo * (n1 + 1) + kxo) * nko + ko;
    const int64_t gblk = (int64_t)(n2 + 1) * (n1 + 1) * nko;
#pragma unroll 1
    for (int p = 0; p < C; ++p) {
      cplx<T> acc0 = {0, 0}, acc1 = {0, 0};
#pragma unroll
      for (int q = 0; q < C; ++q) {
        const int b = bt.blk[p * C + q];
        if (b >= 0) {
          cplx<T> g = a.G[b * gblk + gpen];
          if (bt.conj) g = conjg(g);
          T s = (T)bt.sgn[p * C + q];
          if (mx) s *= (T)bt.s1[b];
          if (my) s *= (T)bt.s2[b];
          g = scale(g, s);
          fma_c(acc0, g, x0[q]);
          fma_c(acc1, scale(g, (T)bt.s3[b]), x1[q]);
        }
      }
      buf[r0 * rs + (g0 * C + p) * TX + t] = acc0;
      if (two) buf[r1 * rs + (g1 * C + p) * TX + t] = acc1;
    }
  }
  __syncthreads();
  fft_dif<T, true>(buf, 2 * C * TX, rs, 1, a.az.plan, tw, true);
  // store: z = natural index, read row pofk[z] of both parities and combine
  cplx<T>* dst = a.S + (int64_t)rhs * C * cstride + ((int64_t)kyp * n3) * m1 + k0;
  for (int i = threadIdx.x; i < C * n3 * TX; i += blockDim.x) {
    const int t = i % TX;
    const int rest = i / TX;
    const int z = rest % n3, c = rest / n3;
    if (t >= tx) continue;
    const int row = a.az.pofk[z];
    cplx<T> v0 = buf[row * rs + (0 * C + c) * TX + t];
    cplx<T> v1 = buf[row * rs + (1 * C + c) * TX + t];
    dst[c * cstride + (int64_t)z * m1 + t] = v0 + mulc(v1, a.az.tw2[z]);
  }
}

// ---------------------------------------------------------------------------
// Pass YI (inverse y + crop).  grid (ceil(2n1/TXY), n3, nrhs*C)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_inv_y(MvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int rc = blockIdx.z, rhs = rc / a.C, c = rc - rhs * a.C;
  if (a.active && !a.active[rhs]) return;
  const int z = blockIdx.y, k0 = blockIdx.x * a.TXY;
  const int n1 = a.n1, n2 = a.n2, n3 = a.n3, m1 = 2 * n1;
  const int tx = min(a.TXY, m1 - k0);
  const int TXY = a.TXY;
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + n2;
  load_tw(tw, a.ay.tw, n2);
  const cplx<T>* src = a.S + ((int64_t)rhs * a.C + c) * (int64_t)2 * n2 * n3 * m1;
  for (int i = threadIdx.x; i < 2 * n2 * TXY; i += blockDim.x) {
    const int row = i / TXY, t = i - row * TXY;
    const int beta = row / n2, p = row - beta * n2;
    cplx<T> v = {0, 0};
    if (t < tx) v = src[((int64_t)row * n3 + z) * m1 + k0 + t];
    buf[(p * 2 + beta) * TXY + t] = v;
  }
  __syncthreads();
  fft_dit<T, true>(buf, 2 * TXY, 2 * TXY, 1, a.ay.plan, tw, true);
  cplx<T>* dst = a.T1 + (((int64_t)rhs * a.C + c) * n3 + z) * (int64_t)n2 * m1;
  for (int i = threadIdx.x; i < n2 * TXY; i += blockDim.x) {
    const int y = i / TXY, t = i - y * TXY;
    if (t < tx) {
      cplx<T> v = buf[(y * 2 + 0) * TXY + t] + mulc(buf[(y * 2 + 1) * TXY + t], a.ay.tw2[y]);
      dst[(int64_t)y * m1 + k0 + t] = v;
    }
  }
}

// ---------------------------------------------------------------------------
// Pass XI (inverse x + crop + epilogue).  grid (ceil(n2/TY), n3, nrhs*C)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_inv_x(MvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int rc = blockIdx.z, rhs = rc / a.C, c = rc - rhs * a.C;
  if (a.active && !a.active[rhs]) return;
  const int z = blockIdx.y, y0 = blockIdx.x * a.TY;
  const int n1 = a.n1, n2 = a.n2, n3 = a.n3;
  const int ty = min(a.TY, n2 - y0);
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + n1;
  load_tw(tw, a.ax.tw, n1);
  const cplx<T>* src = a.T1 + (((int64_t)rhs * a.C + c) * n3 + z) * (int64_t)n2 * 2 * n1;
  for (int i = threadIdx.x; i < ty * 2 * n1; i += blockDim.x) {
    const int yy = i / (2 * n1), k = i - yy * 2 * n1;
    buf[i] = src[(int64_t)(y0 + yy) * 2 * n1 + k];
  }
  __syncthreads();
  fft_dit<T, true>(buf, 2 * ty, 1, n1, a.ax.plan, tw, false);
  const int64_t nD = (int64_t)n1 * n2 * n3;
  for (int i = threadIdx.x; i < ty * n1; i += blockDim.x) {
    const int yy = i / n1, x = i - yy * n1;
    const int y = y0 + yy;
    cplx<T> v = buf[(yy * 2 + 0) * n1 + x] + mulc(buf[(yy * 2 + 1) * n1 + x], a.ax.tw2[x]);
    const int64_t g = x + (int64_t)n1 * (y + (int64_t)n2 * z);
    if (a.mode == MV_GRID) {
      a.out[(int64_t)rhs * a.out_rs + (int64_t)c * nD + g] = v;
    } else {
      const int s = a.vox2sol[g];
      if (s >= 0) {
        const int64_t o = (int64_t)c * a.Ns + s;
        cplx<T> xin = a.in[(int64_t)rhs * a.in_rs + o];
        if (a.mode == MV_VIE) v = scale(a.chi[s] * v, a.invg[c]);
        a.out[(int64_t)rhs * a.out_rs + o] = xin - v;
      }
    }
  }
}

}  // namespace marie
