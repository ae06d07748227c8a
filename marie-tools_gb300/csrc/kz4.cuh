// Four-step z pass of the matvec (n3 = 16*NB): z-DFT, Green block multiply
// and inverse z-DFT in shared memory, for W = TX*R contiguous elements of
// every (component, z) row.  k4_z serves native complex128; complex64 and
// float-float complex128 run the packed-pair kernels of kz4p.cuh and
// kz4f.cuh, which keep this layout and work split.
//
// Shared-memory layout.  Half h (0: even frequencies, 1: odd) starts at
// h*H; in it, sequence (c, e) starts at (c*W + e)*S.  Inside a sequence the
// pair (j, k1), j in [0, NB) (b before the NB-point step, k2 after it) and
// k1 in [0, 16), sits at zpos(j, k1) = j*16 + (k1 ^ j).  The stride
// S = N + 16/W (N + 1 for W >= 16) and the half pad 8/W spread the 16 lanes
// of every half-warp phase over distinct bank pairs in all five phases
// (8-byte elements), as checked by enumerating the lane addresses.
//
// Work split: every phase hands each thread the same number of tasks when
// 2*C*NB*W and 2*N*W are multiples of the block size (the 128^3 PWL case:
// 768, 1536 and 1024 tasks for 256 threads).
#pragma once

#include "fastpath.cuh"
#include "matvec4.cuh"

namespace marie {

__device__ __forceinline__ int zpos(int j, int k1) { return j * 16 + (k1 ^ j); }

__device__ __forceinline__ cplx<double> shfl_xor_c(cplx<double> v, int m) {
  return {__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m)};
}
__device__ __forceinline__ cplx<ff> shfl_xor_c(cplx<ff> v, int m) {
  return {ff(__shfl_xor_sync(0xffffffffu, v.x.hi, m), __shfl_xor_sync(0xffffffffu, v.x.lo, m)),
          ff(__shfl_xor_sync(0xffffffffu, v.y.hi, m), __shfl_xor_sync(0xffffffffu, v.y.lo, m))};
}

// One entry of the single-point Green multiply (entries sorted by block;
// every index a compile-time constant).  gp points at the point's U block
// values, contiguous in the full spectrum ([ky][kx][kz][blk], mirror signs
// applied), so block blk sits at the constant offset blk.
template <typename T, bool PWL, int OP, int K>
struct ZPoint {
  static __device__ __forceinline__ void run(cplx<T>* y, const cplx<T>* x, cplx<T>& gv, const cplx<T>* gp) {
    using Tab = OpTab<PWL, OP>;
    constexpr int blk = Tab::L.e[K].blk;
    constexpr int p = Tab::L.e[K].p, q = Tab::L.e[K].q, sg = Tab::L.e[K].sgn;
    constexpr bool first = (K == 0) || (Tab::L.e[K == 0 ? 0 : K - 1].blk != blk);
    if constexpr (first) {
      cplx<T> g = ldg_c(gp + blk);
      if constexpr ((OP & 1) != 0) g = conjg(g);
      gv = g;
    }
    if constexpr (sg > 0) fma_c(y[p], gv, x[q]);
    else fms_c(y[p], gv, x[q]);
  }
};

template <typename T, bool PWL, int OP, int... Ks>
__device__ __forceinline__ void zpoint(std::integer_sequence<int, Ks...>, cplx<T>* v, int qstride,
                                       const cplx<T>* gp) {
  constexpr int C = PWL ? 12 : 3;
  cplx<T> x[C], y[C];
#pragma unroll
  for (int q = 0; q < C; ++q) {
    x[q] = v[q * qstride];
    y[q] = cplx<T>{0, 0};
  }
  cplx<T> gv = {0, 0};
  (ZPoint<T, PWL, OP, Ks>::run(y, x, gv, gp), ...);
#pragma unroll
  for (int p = 0; p < C; ++p) v[p * qstride] = y[p];
}

template <typename T, int NB, bool PWL, int OP>
__global__ void __launch_bounds__(256, 1) k4_z(MvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int N = 16 * NB;
  constexpr int C = PWL ? 12 : 3;
  constexpr int NE = OpTab<PWL, OP>::NE;
  // grid (nbundle, ceil(2n1/TX), 2n2): the bundles of one (ky, kx) tile run
  // back to back and share its Green rows in L2
  const int bu = blockIdx.x;
  if (!bundle_active(a, bu)) return;
  const int kyp = blockIdx.z, k0 = blockIdx.y * a.TX;
  const int n1 = a.n1, n2 = a.n2, m1 = 2 * n1, R = a.R;
  const int W = a.TX * R, wl = min(a.TX, m1 - k0) * R;
  const int lgW = 31 - __clz(W);                // W = TX*R is a power of two
  const int S = kz4_stride(N, W);
  const int H = C * W * S + kz4_halfpad(W);   // start of the odd half
  const int T1 = 2 * C * NB * W;              // tasks of forward step 1 / inverse step B
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + N;
  load_tw(tw, a.az.tw, N);
  __syncthreads();
  const int64_t row = (int64_t)m1 * R;
  const int64_t cstride = (int64_t)2 * n2 * N * row;
  cplx<T>* base = a.S + (int64_t)bu * C * cstride + (int64_t)kyp * N * row + (int64_t)k0 * R;

  // forward step 1: task (e, h, b, c), e fastest; half h of the zero-padded
  // 2N-point transform (h = 1: inputs times w_2N^z), 16-point DFT over a of
  // z = NB*a + b, then the four-step twiddle.
#pragma unroll 1
  for (int t = threadIdx.x; t < T1; t += blockDim.x) {
    const int e = t & (W - 1), r = t >> lgW;
    const int h = r & 1, r2 = r >> 1;
    const int b = r2 % NB, c = r2 / NB;
    const unsigned live = a.zq ? a.zq[b] : 0xffffu;   // slices z = NB*q + b
    cplx<T> u[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      cplx<T> val = (e < wl && ((live >> q) & 1u)) ? base[c * cstride + (int64_t)(NB * q + b) * row + e]
                                                   : cplx<T>{0, 0};
      if (h) val = val * a.az.tw2[NB * q + b];
      u[q] = val;
    }
    dftn<T, false, 16>(u);
    cplx<T>* d = buf + h * H + (c * W + e) * S + b * 16;
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) d[k1 ^ b] = u[k1] * tw[b * k1];
  }
  __syncthreads();
  // forward step 2 (in place): task (s, k1), k1 fastest; NB-point DFT
  for (int t = threadIdx.x; t < 2 * C * W * 16; t += blockDim.x) {
    const int k1 = t & 15, s = t >> 4;
    const int h = s >= C * W ? 1 : 0;
    cplx<T>* p = buf + h * H + (s - h * C * W) * S;
    cplx<T> w[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) w[b] = p[zpos(b, k1)];
    dftn<T, false, NB>(w);
#pragma unroll
    for (int k2 = 0; k2 < NB; ++k2) p[zpos(k2, k1)] = w[k2];
  }
  __syncthreads();

  // Green block multiply, one frequency per item (e, g, k): kz = 2k + g sits
  // in half g at zpos(k >> 4, k & 15); its U block values are contiguous in
  // the full spectrum at ((ky*2n1 + kx)*2N + kz)*U.
  constexpr int U = OpTab<PWL, OP>::L.nblk;
  const int beta = kyp / n2, ky = 2 * (kyp - beta * n2) + beta;
  for (int i = threadIdx.x; i < 2 * N * W; i += blockDim.x) {
    const int e = i & (W - 1), pp = i >> lgW;
    const int kxp = k0 + (e >> a.lgR);
    if (kxp >= m1) continue;
    const int g = pp / N, k = pp - g * N;
    const int kz = 2 * k + g;
    const int alpha = kxp >= n1 ? 1 : 0;
    const int kx = 2 * (kxp - alpha * n1) + alpha;
    const cplx<T>* gp = a.G + (((int64_t)ky * m1 + kx) * (2 * N) + kz) * U;
    cplx<T>* v = buf + g * H + e * S + zpos(k >> 4, k & 15);
    zpoint<T, PWL, OP>(std::make_integer_sequence<int, NE>{}, v, W * S, gp);
  }
  __syncthreads();
  // inverse step A (in place): task (s, k1), k1 fastest
  for (int t = threadIdx.x; t < 2 * C * W * 16; t += blockDim.x) {
    const int k1 = t & 15, s = t >> 4;
    const int h = s >= C * W ? 1 : 0;
    cplx<T>* p = buf + h * H + (s - h * C * W) * S;
    cplx<T> w[NB];
#pragma unroll
    for (int k2 = 0; k2 < NB; ++k2) w[k2] = p[zpos(k2, k1)];
    dftn<T, true, NB>(w);
#pragma unroll
    for (int b = 0; b < NB; ++b) p[zpos(b, k1)] = mulc(w[b], tw[b * k1]);
  }
  __syncthreads();
  // inverse step B: task (e, h, b, c) as in step 1, inverse 16-point DFT of
  // half h (h = 1 then times conj(w_2N^z)).  The partner lane t ^ W holds the
  // other half of the same (e, b, c): the even lane stores q < 8, the odd lane
  // q >= 8, after one exchange.  The loop is warp-uniform so that every lane
  // takes part in the shuffles; lanes past T1 redo a valid task of the first
  // group (tasks come in aligned groups of 2W, so t & (2W - 1) keeps (e, h)
  // and pairs partners again) and store nothing.
  const int lane = threadIdx.x & 31;
#pragma unroll 1
  for (int tb = threadIdx.x - lane; tb < T1; tb += blockDim.x) {
    const int t = tb + lane;
    const bool act = t < T1;
    const int tt = act ? t : (t & (2 * W - 1));   // a valid task with the same (e, h)
    const int e = tt & (W - 1), r = tt >> lgW;
    const int h = r & 1, r2 = r >> 1;
    const int b = r2 % NB, c = r2 / NB;
    const cplx<T>* sp = buf + h * H + (c * W + e) * S + b * 16;
    cplx<T> u[16];
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) u[k1] = sp[k1 ^ b];
    dftn<T, true, 16>(u);
    if (h) {
#pragma unroll
      for (int q = 0; q < 16; ++q) u[q] = mulc(u[q], a.az.tw2[NB * q + b]);
    }
    const bool st = act && e < wl;
    const unsigned live = (a.zq ? a.zq[b] : 0xffffu) >> (8 * h);   // slices z = NB*(8h + j) + b
    cplx<T>* dst = base + c * cstride + (int64_t)(NB * 8 * h + b) * row + e;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const cplx<T> send = h ? u[j] : u[8 + j];
      const cplx<T> recv = shfl_xor_c(send, W);
      const cplx<T> out = h ? recv + u[8 + j] : u[j] + recv;
      if (st && ((live >> j) & 1u)) dst[(int64_t)NB * j * row] = out;
    }
  }
}

}  // namespace marie
