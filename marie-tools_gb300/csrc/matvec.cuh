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
// Right-hand sides are processed in bundles of R, interleaved innermost in
// the work arrays ([bundle][..][kx'][r]): every Green's-tensor value loaded
// by the z pass serves R right-hand sides, and the z-pass tiles of TX pencils
// are contiguous runs of TX*R elements.
//
// Passes (per right-hand side and component):
//   X  : scatter from the body vector (+ optional prologue scale), x-DFT     n^3  -> 2n^3
//   Y  : y-DFT                                                               2n^3 -> 4n^3
//   Z  : z-DFT, Green block multiply, inverse z-DFT (in place)               4n^3 -> 4n^3
//   YI : inverse y-DFT + crop                                                4n^3 -> 2n^3
//   XI : inverse x-DFT + crop + epilogue + gather                            2n^3 -> n^3
//
// Shared-memory layout of every pass: buf[i * es + s], element i of sequence
// s, es = nseq + 1 (odd padding keeps column accesses conflict-free).
#pragma once

#include "common.cuh"
#include "optab.cuh"

#include <utility>

namespace marie {

constexpr int kMaxComp = 12;
constexpr int kMaxBlocks = 60;

enum MvMode : int {
  MV_GRID = 0,      // input/output are full grids (n1,n2,n3,C) column-major
  MV_VIE = 1,       // y = x - chi .* invG(N x) on the body vector
  MV_VIE_ADJ = 2,   // y = x - N^H(invG .* conj(chi) .* x) on the body vector
  MV_EFIELD = 3,    // y = (1/ce) (invG(N x) - x) on the body (em_efield_vie_excitation.m:21)
  MV_HFIELD = 4,    // y = invG(K x) on the body (em_hfield_vie_excitation.m:20)
  MV_HFIELD_ADJ = 5,  // y = K^H(invG x) on the body: the adjoint of the MV_HFIELD map
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
  int n1, n2, n3, C;
  int R;                      // right-hand sides per bundle (interleaved innermost)
  int lgR;                    // log2(R) (R is a power of two)
  int nrhs;                   // right-hand sides in this launch (<= nbundle * R)
  int64_t Ns;                 // body voxels
  int mode;
  AxisTab<T> ax, ay, az;
  const int* vox2sol;         // n1*n2*n3 -> body index or -1
  const cplx<T>* chi;         // contrast (Mc/Mr) per body voxel
  T invg[kMaxComp];           // invG diagonal per component
  const cplx<typename IoOf<T>::type>* in;   // rhs r at in + r*in_rs
  cplx<typename IoOf<T>::type>* out;
  int64_t in_rs, out_rs;      // element stride between right-hand sides
  cplx<T>* T1;                // [bundle][c][z][y][2n1][R]
  cplx<T>* S;                 // [bundle][c][2n2][z][2n1][R]
  const cplx<T>* G;           // octant spectra [blk][n2+1][n1+1][n3+1]
  const unsigned char* active;  // per rhs: nonzero = process (may be null)
  cplx<T> efac;               // 1/ce (MV_EFIELD)
  const cplx<typename IoOf<T>::type>* addend;   // added to the body output (same strides; may be null)
  // Body occupancy for the pruned four-step passes (null: every row live).
  // row_live[z*n2 + y]: the grid row (y, z) holds a body voxel; z_live[z]:
  // slice z does.  Rows and slices that are not live are zero on input and
  // not needed on output, so the passes neither transform nor store them.
  const unsigned char* row_live;
  const unsigned char* z_live;
  // The same occupancy in the four-step index order (edges 16*NB): bit q of
  // rowq[z*8 + b] is row y = NB*q + b of slice z, bit q of zq[b] is slice
  // z = NB*q + b (null: all live).
  const uint16_t* rowq;
  const uint16_t* zq;
  int TY, TXY, TX;            // tile sizes of the X, Y, Z passes
};

template <typename T>
__device__ __forceinline__ void load_tw(cplx<T>* dst, const cplx<T>* src, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

template <typename T>
__device__ __forceinline__ bool lane_active(const MvArgs<T>& a, int rhs) {
  return rhs < a.nrhs && (a.active == nullptr || a.active[rhs]);
}

template <typename T>
__device__ __forceinline__ bool row_is_live(const MvArgs<T>& a, int y, int z) {
  return a.row_live == nullptr || a.row_live[z * a.n2 + y] != 0;
}

template <typename T>
__device__ __forceinline__ bool z_is_live(const MvArgs<T>& a, int z) {
  return a.z_live == nullptr || a.z_live[z] != 0;
}

// Body-vector output of the modes other than MV_GRID for component c, body
// voxel s and right-hand side rhs, given v = (operator x) at that voxel.
template <typename T>
__device__ __forceinline__ void body_store(const MvArgs<T>& a, int c, int s, int rhs, cplx<T> v) {
  const int64_t o = (int64_t)c * a.Ns + s;
  cplx<T> r;
  if (a.mode == MV_HFIELD) {
    r = scale(v, a.invg[c]);
  } else if (a.mode == MV_HFIELD_ADJ) {
    r = v;
  } else {
    const cplx<T> xin = io_load<T>(a.in[(int64_t)rhs * a.in_rs + o]);
    if (a.mode == MV_VIE) r = xin - scale(a.chi[s] * v, a.invg[c]);
    else if (a.mode == MV_VIE_ADJ) r = xin - v;
    else r = a.efac * (scale(v, a.invg[c]) - xin);
  }
  if (a.addend) r = r + io_load<T>(a.addend[(int64_t)rhs * a.out_rs + o]);
  a.out[(int64_t)rhs * a.out_rs + o] = io_store(r);
}

template <typename T>
__device__ __forceinline__ bool bundle_active(const MvArgs<T>& a, int b) {
  for (int r = 0; r < a.R; ++r)
    if (lane_active(a, b * a.R + r)) return true;
  return false;
}

// ---------------------------------------------------------------------------
// Pass X (forward).  grid (ceil(n2/TY), n3, nbundle*C)
// sequences s = (yy*2 + alpha)*R + r, length n1
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_fwd_x(MvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int bc = blockIdx.z, b = bc / a.C, c = bc - b * a.C;
  if (!bundle_active(a, b)) return;
  const int z = blockIdx.y, y0 = blockIdx.x * a.TY;
  const int n1 = a.n1, n2 = a.n2, n3 = a.n3, R = a.R;
  const int ty = min(a.TY, n2 - y0);
  const int nseq = 2 * ty * R, es = nseq + 1;
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + n1;
  load_tw(tw, a.ax.tw, n1);
  const int64_t nD = (int64_t)n1 * n2 * n3;
  for (int i = threadIdx.x; i < ty * R * n1; i += blockDim.x) {
    const int x = i % n1;
    const int rest = i / n1;
    const int r = rest % R, yy = rest / R;
    const int rhs = b * R + r;
    const int64_t g = x + (int64_t)n1 * (y0 + yy + (int64_t)n2 * z);
    cplx<T> v = {0, 0};
    if (lane_active(a, rhs)) {
      const cplx<T>* in = a.in + (int64_t)rhs * a.in_rs;
      if (a.mode == MV_GRID) {
        v = in[(int64_t)c * nD + g];
      } else {
        const int s = a.vox2sol[g];
        if (s >= 0) {
          v = in[(int64_t)c * a.Ns + s];
          if (a.mode == MV_VIE_ADJ) v = scale(mulc(v, a.chi[s]), a.invg[c]);
          else if (a.mode == MV_HFIELD_ADJ) v = scale(v, a.invg[c]);
        }
      }
    }
    buf[x * es + (yy * 2 + 0) * R + r] = v;
    buf[x * es + (yy * 2 + 1) * R + r] = v * a.ax.tw2[x];
  }
  __syncthreads();
  fft_dif<T, false>(buf, nseq, es, 1, a.ax.plan, tw, true);
  // row y of T1: [kx' = alpha*n1 + p][r]
  const int rowlen = 2 * n1 * R;
  cplx<T>* dst = a.T1 + (((int64_t)b * a.C + c) * n3 + z) * (int64_t)n2 * rowlen;
  for (int i = threadIdx.x; i < ty * rowlen; i += blockDim.x) {
    const int yy = i / rowlen, e = i - yy * rowlen;
    const int kx = e / R, r = e - kx * R;
    const int alpha = kx / n1, p = kx - alpha * n1;
    dst[(int64_t)(y0 + yy) * rowlen + e] = buf[p * es + (yy * 2 + alpha) * R + r];
  }
}

// ---------------------------------------------------------------------------
// Pass Y (forward).  grid (ceil(2n1/TXY), n3, nbundle*C)
// sequences s = (beta*TXY + t)*R + r, length n2
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_fwd_y(MvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int bc = blockIdx.z, b = bc / a.C, c = bc - b * a.C;
  if (!bundle_active(a, b)) return;
  const int z = blockIdx.y, k0 = blockIdx.x * a.TXY;
  const int n1 = a.n1, n2 = a.n2, n3 = a.n3, m1 = 2 * n1, R = a.R, TXY = a.TXY;
  const int tx = min(TXY, m1 - k0);
  const int W = TXY * R, nseq = 2 * W, es = nseq + 1;
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + n2;
  load_tw(tw, a.ay.tw, n2);
  const int64_t row = (int64_t)m1 * R;
  const cplx<T>* src = a.T1 + (((int64_t)b * a.C + c) * n3 + z) * (int64_t)n2 * row + (int64_t)k0 * R;
  for (int i = threadIdx.x; i < n2 * W; i += blockDim.x) {
    const int y = i / W, e = i - y * W;
    cplx<T> v = {0, 0};
    if (e < tx * R) v = src[(int64_t)y * row + e];
    buf[y * es + e] = v;
    buf[y * es + W + e] = v * a.ay.tw2[y];
  }
  __syncthreads();
  fft_dif<T, false>(buf, nseq, es, 1, a.ay.plan, tw, true);
  // S[b][c][beta*n2 + p][z][kx'][r]
  cplx<T>* dst = a.S + ((int64_t)b * a.C + c) * (int64_t)2 * n2 * n3 * row + (int64_t)k0 * R;
  for (int i = threadIdx.x; i < 2 * n2 * W; i += blockDim.x) {
    const int ky = i / W, e = i - ky * W;      // ky = beta*n2 + p
    const int beta = ky / n2, p = ky - beta * n2;
    if (e < tx * R) dst[((int64_t)ky * n3 + z) * row + e] = buf[p * es + beta * W + e];
  }
}

// One entry of the z-pass Green multiply, every index a compile-time constant:
// load block blk's value when the entry starts a new block (entries are sorted
// by block), then y[p] += sgn * G_blk * x[q] for both points of the work item.
// TWO: the second point has its own octant value (at gp1) and no z-mirror
// sign; otherwise it is the z-mirror of the first (same value, sign s3).
template <typename T, bool PWL, int OP, int K, bool TWO>
struct ZStep {
  static __device__ __forceinline__ void run(cplx<T>* y0, cplx<T>* y1, const cplx<T>* x0, const cplx<T>* x1,
                                             cplx<T>& g0v, cplx<T>& g1v, const cplx<T>* gp0, const cplx<T>* gp1,
                                             int64_t gblk, bool mx, bool my) {
    using Tab = OpTab<PWL, OP>;
    constexpr int blk = Tab::L.e[K].blk;
    constexpr int p = Tab::L.e[K].p, q = Tab::L.e[K].q, sg = Tab::L.e[K].sgn;
    constexpr bool first = (K == 0) || (Tab::L.e[K == 0 ? 0 : K - 1].blk != blk);
    if constexpr (first) {
      constexpr bool neg1 = Tab::L.s1[blk] < 0, neg2 = Tab::L.s2[blk] < 0, neg3 = Tab::L.s3[blk] < 0;
      cplx<T> gA = ldg_c(gp0 + blk * gblk);
      if constexpr ((OP & 1) != 0) gA = conjg(gA);
      const bool f = (neg1 && mx) != (neg2 && my);    // sign flip from x/y mirrors
      g0v = f ? cplx<T>{-gA.x, -gA.y} : gA;
      if constexpr (TWO) {
        cplx<T> gB = ldg_c(gp1 + blk * gblk);
        if constexpr ((OP & 1) != 0) gB = conjg(gB);
        g1v = f ? cplx<T>{-gB.x, -gB.y} : gB;
      } else {
        g1v = neg3 ? cplx<T>{-g0v.x, -g0v.y} : g0v;
      }
    }
    if constexpr (sg > 0) {
      fma_c(y0[p], g0v, x0[q]);
      fma_c(y1[p], g1v, x1[q]);
    } else {
      fms_c(y0[p], g0v, x0[q]);
      fms_c(y1[p], g1v, x1[q]);
    }
  }
};

template <typename T, bool PWL, int OP, bool TWO, int... Ks>
__device__ __forceinline__ void zmul(std::integer_sequence<int, Ks...>, cplx<T>* y0, cplx<T>* y1, const cplx<T>* x0,
                                     const cplx<T>* x1, const cplx<T>* gp0, const cplx<T>* gp1, int64_t gblk, bool mx,
                                     bool my) {
  cplx<T> g0v = {0, 0}, g1v = {0, 0};
  (ZStep<T, PWL, OP, Ks, TWO>::run(y0, y1, x0, x1, g0v, g1v, gp0, gp1, gblk, mx, my), ...);
}

// Green multiply of one work item: y = G x at two frequencies.
template <typename T, bool PWL, int OP, bool TWO>
__device__ __forceinline__ void zitem(cplx<T>* buf, int o0, int o1, int qstride, const cplx<T>* gp0,
                                      const cplx<T>* gp1, int64_t gblk, bool mx, bool my) {
  constexpr int C = PWL ? 12 : 3;
  cplx<T> x0[C], x1[C], y0[C], y1[C];
#pragma unroll
  for (int q = 0; q < C; ++q) {
    x0[q] = buf[o0 + q * qstride];
    x1[q] = buf[o1 + q * qstride];
    y0[q] = cplx<T>{0, 0};
    y1[q] = cplx<T>{0, 0};
  }
  zmul<T, PWL, OP, TWO>(std::make_integer_sequence<int, OpTab<PWL, OP>::NE>{}, y0, y1, x0, x1, gp0, gp1, gblk, mx,
                        my);
#pragma unroll
  for (int p = 0; p < C; ++p) {
    buf[o0 + p * qstride] = y0[p];
    buf[o1 + p * qstride] = y1[p];
  }
}

// ---------------------------------------------------------------------------
// Pass Z (fused).  grid (ceil(2n1/TX), 2n2, nbundle)
// sequences s = ((gamma*C + c)*TX + t)*R + r, length n3; row i of buf holds
// the z-sample (on load) / frequency (after the DIT) i of every sequence.
// ---------------------------------------------------------------------------
template <typename T, bool PWL, int OP>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 2 : 1) k_z(MvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int b = blockIdx.z;
  if (!bundle_active(a, b)) return;
  const int kyp = blockIdx.y, k0 = blockIdx.x * a.TX;
  const int n1 = a.n1, n2 = a.n2, n3 = a.n3, m1 = 2 * n1, TX = a.TX, R = a.R;
  constexpr int C = PWL ? 12 : 3;
  const int tx = min(TX, m1 - k0);
  const int W = TX * R;                    // contiguous elements per (c, z)
  const int nseq = 2 * C * W, es = nseq + 1;
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + n3;
  load_tw(tw, a.az.tw, n3);
  const int64_t row = (int64_t)m1 * R;
  const int64_t cstride = (int64_t)2 * n2 * n3 * row;
  cplx<T>* base = a.S + (int64_t)b * C * cstride + (int64_t)kyp * n3 * row + (int64_t)k0 * R;
  // load: element z goes to row pofk[z] (DIT input order)
  for (int i = threadIdx.x; i < C * n3 * W; i += blockDim.x) {
    const int e = i % W;
    const int rest = i / W;
    const int z = rest % n3, c = rest / n3;
    cplx<T> v = {0, 0};
    if (e < tx * R) v = base[c * cstride + (int64_t)z * row + e];
    const int rw = a.az.pofk[z];
    buf[rw * es + (0 * C + c) * W + e] = v;
    buf[rw * es + (1 * C + c) * W + e] = v * a.az.tw2[z];
  }
  __syncthreads();
  fft_dit<T, false>(buf, nseq, es, 1, a.az.plan, tw, true);

  // Green block multiply at natural frequencies.  Work item (u, t, r), u in
  // [0, n3): u > 0 handles kz = u and its mirror 2n3 - u (same octant row u,
  // z-mirror sign s3); u = 0 handles the two self-mirror frequencies 0 and n3.
  // Lanes sharing u share every Green load.  The loop runs over Green blocks:
  // each block value is loaded once and applied to all (p, q) pairs using it.
  // Pencil kx' = alpha*n1 + pos has kx = 2*kofp[pos] + alpha.
  const int beta = kyp / n2, py = kyp - beta * n2;
  const int ky = 2 * a.ay.kofp[py] + beta;
  const bool my = ky > n2;
  const int kyo = my ? 2 * n2 - ky : ky;
  const int nko = n3 + 1;
  const int64_t gblk = (int64_t)(n2 + 1) * (n1 + 1) * nko;
  for (int i = threadIdx.x; i < n3 * W; i += blockDim.x) {
    const int e = i % W, u = i / W;
    const int t = e / R;
    if (t >= tx) continue;
    const int kxp = k0 + t;
    const int alpha = kxp / n1, px = kxp - alpha * n1;
    const int kx = 2 * a.ax.kofp[px] + alpha;
    const bool mx = kx > n1;
    const int kxo = mx ? 2 * n1 - kx : kx;
    const int kz0 = u == 0 ? 0 : u;
    const int kz1 = u == 0 ? n3 : 2 * n3 - u;
    const int r0 = kz0 >> 1, g0 = kz0 & 1;
    const int r1 = (kz1 >> 1) % n3, g1 = kz1 & 1;
    const int o0 = r0 * es + g0 * C * W + e, o1 = r1 * es + g1 * C * W + e;
    const cplx<T>* gp0 = a.G + ((int64_t)kyo * (n1 + 1) + kxo) * nko + u;
    // the second point is a z-mirror (sign s3) unless u == 0 (frequency n3)
    if (u != 0) zitem<T, PWL, OP, false>(buf, o0, o1, W, gp0, gp0, gblk, mx, my);
    else zitem<T, PWL, OP, true>(buf, o0, o1, W, gp0, gp0 + n3, gblk, mx, my);
  }
  __syncthreads();
  fft_dif<T, true>(buf, nseq, es, 1, a.az.plan, tw, true);
  // store: z natural, read row pofk[z] of both parities and combine
  for (int i = threadIdx.x; i < C * n3 * W; i += blockDim.x) {
    const int e = i % W;
    const int rest = i / W;
    const int z = rest % n3, c = rest / n3;
    if (e >= tx * R) continue;
    const int rw = a.az.pofk[z];
    const cplx<T> v0 = buf[rw * es + (0 * C + c) * W + e];
    const cplx<T> v1 = buf[rw * es + (1 * C + c) * W + e];
    base[c * cstride + (int64_t)z * row + e] = v0 + mulc(v1, a.az.tw2[z]);
  }
}

// ---------------------------------------------------------------------------
// Pass YI (inverse y + crop).  grid (ceil(2n1/TXY), n3, nbundle*C)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_inv_y(MvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int bc = blockIdx.z, b = bc / a.C, c = bc - b * a.C;
  if (!bundle_active(a, b)) return;
  const int z = blockIdx.y, k0 = blockIdx.x * a.TXY;
  const int n1 = a.n1, n2 = a.n2, n3 = a.n3, m1 = 2 * n1, R = a.R, TXY = a.TXY;
  const int tx = min(TXY, m1 - k0);
  const int W = TXY * R, nseq = 2 * W, es = nseq + 1;
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + n2;
  load_tw(tw, a.ay.tw, n2);
  const int64_t row = (int64_t)m1 * R;
  const cplx<T>* src = a.S + ((int64_t)b * a.C + c) * (int64_t)2 * n2 * n3 * row + (int64_t)k0 * R;
  for (int i = threadIdx.x; i < 2 * n2 * W; i += blockDim.x) {
    const int ky = i / W, e = i - ky * W;
    const int beta = ky / n2, p = ky - beta * n2;
    cplx<T> v = {0, 0};
    if (e < tx * R) v = src[((int64_t)ky * n3 + z) * row + e];
    buf[p * es + beta * W + e] = v;
  }
  __syncthreads();
  fft_dit<T, true>(buf, nseq, es, 1, a.ay.plan, tw, true);
  cplx<T>* dst = a.T1 + (((int64_t)b * a.C + c) * n3 + z) * (int64_t)n2 * row + (int64_t)k0 * R;
  for (int i = threadIdx.x; i < n2 * W; i += blockDim.x) {
    const int y = i / W, e = i - y * W;
    if (e < tx * R) dst[(int64_t)y * row + e] = buf[y * es + e] + mulc(buf[y * es + W + e], a.ay.tw2[y]);
  }
}

// ---------------------------------------------------------------------------
// Pass XI (inverse x + crop + epilogue).  grid (ceil(n2/TY), n3, nbundle*C)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_inv_x(MvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int bc = blockIdx.z, b = bc / a.C, c = bc - b * a.C;
  if (!bundle_active(a, b)) return;
  const int z = blockIdx.y, y0 = blockIdx.x * a.TY;
  const int n1 = a.n1, n2 = a.n2, n3 = a.n3, R = a.R;
  const int ty = min(a.TY, n2 - y0);
  const int nseq = 2 * ty * R, es = nseq + 1;
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + n1;
  load_tw(tw, a.ax.tw, n1);
  const int rowlen = 2 * n1 * R;
  const cplx<T>* src = a.T1 + (((int64_t)b * a.C + c) * n3 + z) * (int64_t)n2 * rowlen;
  for (int i = threadIdx.x; i < ty * rowlen; i += blockDim.x) {
    const int yy = i / rowlen, e = i - yy * rowlen;
    const int kx = e / R, r = e - kx * R;
    const int alpha = kx / n1, p = kx - alpha * n1;
    buf[p * es + (yy * 2 + alpha) * R + r] = src[(int64_t)(y0 + yy) * rowlen + e];
  }
  __syncthreads();
  fft_dit<T, true>(buf, nseq, es, 1, a.ax.plan, tw, true);
  const int64_t nD = (int64_t)n1 * n2 * n3;
  for (int i = threadIdx.x; i < ty * R * n1; i += blockDim.x) {
    const int x = i % n1;
    const int rest = i / n1;
    const int r = rest % R, yy = rest / R;
    const int rhs = b * R + r;
    if (!lane_active(a, rhs)) continue;
    cplx<T> v = buf[x * es + (yy * 2 + 0) * R + r] + mulc(buf[x * es + (yy * 2 + 1) * R + r], a.ax.tw2[x]);
    const int64_t g = x + (int64_t)n1 * (y0 + yy + (int64_t)n2 * z);
    if (a.mode == MV_GRID) {
      a.out[(int64_t)rhs * a.out_rs + (int64_t)c * nD + g] = v;
    } else {
      const int s = a.vox2sol[g];
      if (s >= 0) body_store(a, c, s, rhs, v);
    }
  }
}

}  // namespace marie
