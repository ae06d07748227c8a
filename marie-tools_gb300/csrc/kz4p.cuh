// Four-step z pass of the complex64 operator (n3 = 16*NB) in packed FP32
// pairs: one task carries the even- and odd-frequency halves of the
// zero-padded 2N-point transform in the two lanes of every value (pair.cuh),
// so each complex operation of the z-DFTs and of the Green block product is
// issued once for both halves.
//
// Shared memory: sequence (c, e) of the tile (component c, tile element e)
// starts at (c*W + e)*S; its N positions hold 16-byte pairs
// (re_even, re_odd, im_even, im_odd).  Pair (j, k1), j in [0, NB) and k1 in
// [0, 16), sits at zpos(j, k1) = j*16 + (k1 ^ j); with S = N + 8/W (N + 1
// for W >= 8) the eight lanes of every quarter-warp of a 128-bit access fall
// on distinct 16-byte bank groups in all five phases (even NB).
//
// Green spectrum (full, mirror signs applied) in pair layout: for a column
// (ky, kx), block blk and position k, one 16-byte entry
// (re G(2k), re G(2k+1), im G(2k), im G(2k+1)) at ((ky*2n1 + kx)*U + blk)*N + k.
#pragma once

#include "fastpath.cuh"
#include "matvec4.cuh"
#include "pair.cuh"

namespace marie {

// Bulk prefetch of [p, p + bytes) into L2 (no data returned to the SM);
// p and bytes multiples of 16.
__device__ __forceinline__ void prefetch_l2_bulk(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

__device__ __forceinline__ cp lds_cp(const cp* p) {
  const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(p);
  return cp{f2{v.x}, f2{v.y}};
}
__device__ __forceinline__ void sts_cp(cp* p, cp v) {
  *reinterpret_cast<ulonglong2*>(p) = make_ulonglong2(v.re.v, v.im.v);
}

// Does any entry of block blk carry a negative sign?
template <bool PWL, int OP>
constexpr bool blk_has_neg(int blk) {
  using Tab = OpTab<PWL, OP>;
  for (int i = 0; i < Tab::NE; ++i)
    if (Tab::L.e[i].blk == blk && Tab::L.e[i].sgn < 0) return true;
  return false;
}

// The Green product of one frequency pair runs in two sweeps over the entry
// list, outputs p < C/2 then p >= C/2 (the inputs stay in registers): half
// the accumulators leaves registers for more Green loads in flight, at the
// price of loading blocks that serve both halves twice.  in_half: entry K
// writes output half H; first_in_half: no earlier entry of its block does.
template <bool PWL, int OP>
constexpr bool in_half(int K, int H) {
  using Tab = OpTab<PWL, OP>;
  constexpr int C = PWL ? 12 : 3;
  return (Tab::L.e[K].p < C / 2) == (H == 0);
}
template <bool PWL, int OP>
constexpr bool first_in_half(int K, int H) {
  using Tab = OpTab<PWL, OP>;
  for (int i = 0; i < K; ++i)
    if (Tab::L.e[i].blk == Tab::L.e[K].blk && in_half<PWL, OP>(i, H)) return false;
  return true;
}

// One entry of output half H (entries sorted by block; every index a
// compile-time constant).  y_p += sgn * g * x_q with g (or conj(g) for N^H)
// in the lanes (G(2k), G(2k+1)):
//   re += gr*xr - gi*xi,  im += gr*xi + gi*xr.
template <bool PWL, int OP, int H, int K>
struct ZPointP {
  static __device__ __forceinline__ void run(cp* y, const cp* x, f2& gr, f2& gi, f2& ngi, f2& ngr,
                                             const float4* gp, int gs) {
    using Tab = OpTab<PWL, OP>;
    if constexpr (in_half<PWL, OP>(K, H)) {
      constexpr int blk = Tab::L.e[K].blk;
      constexpr int p = Tab::L.e[K].p, q = Tab::L.e[K].q, sg = Tab::L.e[K].sgn;
      constexpr int C = PWL ? 12 : 3;
      constexpr int pp = p - (H == 0 ? 0 : C / 2);
      if constexpr (first_in_half<PWL, OP>(K, H)) {
        const float4 g = __ldg(gp + (int64_t)blk * gs);
        gr = f2_make(g.x, g.y);
        const f2 gim = f2_make(g.z, g.w);
        if constexpr ((OP & 1) != 0) {   // conj(g)
          ngi = gim;
          gi = f2_neg(gim);
        } else {
          gi = gim;
          ngi = f2_neg(gim);
        }
        if constexpr (blk_has_neg<PWL, OP>(blk)) ngr = f2_neg(gr);
      }
      if constexpr (sg > 0) {
        y[pp].re = fma2(gr, x[q].re, fma2(ngi, x[q].im, y[pp].re));
        y[pp].im = fma2(gr, x[q].im, fma2(gi, x[q].re, y[pp].im));
      } else {
        y[pp].re = fma2(ngr, x[q].re, fma2(gi, x[q].im, y[pp].re));
        y[pp].im = fma2(ngr, x[q].im, fma2(ngi, x[q].re, y[pp].im));
      }
    }
  }
};

template <bool PWL, int OP, int... Ks>
__device__ __forceinline__ void zpoint_pair(std::integer_sequence<int, Ks...>, cp* v, int qstride, const float4* gp,
                                            int gs) {
  constexpr int C = PWL ? 12 : 3;
  constexpr int CH = C / 2;
  cp x[C];
  const f2 zero = f2_make(0.f, 0.f);
#pragma unroll
  for (int q = 0; q < C; ++q) x[q] = lds_cp(v + q * qstride);
  f2 gr = zero, gi = zero, ngi = zero, ngr = zero;
  {
    cp y[CH];
#pragma unroll
    for (int p = 0; p < CH; ++p) y[p] = cp{zero, zero};
    (ZPointP<PWL, OP, 0, Ks>::run(y, x, gr, gi, ngi, ngr, gp, gs), ...);
#pragma unroll
    for (int p = 0; p < CH; ++p) sts_cp(v + p * qstride, y[p]);
  }
  {
    cp y[C - CH];
#pragma unroll
    for (int p = 0; p < C - CH; ++p) y[p] = cp{zero, zero};
    (ZPointP<PWL, OP, 1, Ks>::run(y, x, gr, gi, ngi, ngr, gp, gs), ...);
#pragma unroll
    for (int p = 0; p < C - CH; ++p) sts_cp(v + (CH + p) * qstride, y[p]);
  }
}

// 192 threads: at the 128^3 PWL tile (W = 4) steps 1 and B have 384 tasks,
// steps 2 and A 768, and two CTAs per SM leave 168 registers per thread
// (the product's 12 input and 6 output pairs plus Green loads in flight,
// without spilling).
constexpr int kZpThreads = 192;

template <int NB, bool PWL, int OP>
__global__ void __launch_bounds__(kZpThreads, 2) k4_zp(MvArgs<float> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int N = 16 * NB;
  constexpr int C = PWL ? 12 : 3;
  constexpr int NE = OpTab<PWL, OP>::NE;
  constexpr int U = OpTab<PWL, OP>::L.nblk;
  // grid (nbundle, ceil(2n1/TX), 2n2): the bundles of one (ky, kx) tile run
  // back to back and share its Green rows in L2
  const int bu = blockIdx.x;
  if (!bundle_active(a, bu)) return;
  const int kyp = blockIdx.z, k0 = blockIdx.y * a.TX;
  const int n1 = a.n1, n2 = a.n2, m1 = 2 * n1, R = a.R;
  const int W = a.TX * R, wl = min(a.TX, m1 - k0) * R;
  const int lgW = 31 - __clz(W);                // W = TX*R is a power of two
  const int S = kzp_stride(N, W);
  const int T1 = C * NB * W;                    // tasks of forward step 1 / inverse step B
  // four-step twiddles w_N^(b*k1) at b*18 + k1 (runs of k1 contiguous,
  // consecutive b on different bank groups) as (wr, wr, wi, wi) and
  // (-wi, -wi); w_2N^z; live-slice masks
  ulonglong2* twq = reinterpret_cast<ulonglong2*>(smem_raw);
  unsigned long long* twn = reinterpret_cast<unsigned long long*>(twq + 18 * NB);
  float2* tw2s = reinterpret_cast<float2*>(twn + 18 * NB);
  unsigned* zqs = reinterpret_cast<unsigned*>(tw2s + N);
  cp* buf = reinterpret_cast<cp*>(zqs + 8);
  for (int i = threadIdx.x; i < 18 * NB; i += blockDim.x) {
    const int b = i / 18, k1 = i - 18 * (i / 18);
    const cplx<float> w = k1 < 16 ? a.az.tw[b * k1] : cplx<float>{0.f, 0.f};
    twq[i] = make_ulonglong2(f2_bc(w.x).v, f2_bc(w.y).v);
    twn[i] = f2_bc(-w.y).v;
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const cplx<float> t2 = a.az.tw2[i];
    tw2s[i] = make_float2(t2.x, t2.y);
  }
  if (threadIdx.x < NB) zqs[threadIdx.x] = a.zq ? a.zq[threadIdx.x] : 0xffffu;
  // When several bundles share a column, the first starts the column's
  // Green rows (U blocks x N pairs x 16 bytes, contiguous per column) on
  // their way to L2 while the forward transforms run, so the product finds
  // them there instead of in HBM; the other bundles of the column run right
  // after it and share them.  (With one bundle the prefetch only competes
  // with the step-1 loads: measured 23% slower at 96^3 with one
  // right-hand side.)
  if (bu == 0 && gridDim.x > 1) {
    const int pb = kyp / n2, pky = 2 * (kyp - pb * n2) + pb;
    const int ncol = min(a.TX, m1 - k0);
    const int64_t colb = (int64_t)U * N * 16;
    const unsigned piece = (unsigned)(colb / 8);      // U * N * 2 bytes: a multiple of 16
    for (int c = threadIdx.x; c < ncol * 8; c += blockDim.x) {
      const int kxp = k0 + (c >> 3);
      const int pa = kxp >= n1 ? 1 : 0;
      const int pkx = 2 * (kxp - pa * n1) + pa;
      const char* col = reinterpret_cast<const char*>(a.G) + ((int64_t)pky * m1 + pkx) * colb;
      prefetch_l2_bulk(col + (int64_t)(c & 7) * piece, piece);
    }
  }
  __syncthreads();
  const int64_t row = (int64_t)m1 * R;
  const int64_t cstride = (int64_t)2 * n2 * N * row;
  cplx<float>* base = a.S + (int64_t)bu * C * cstride + (int64_t)kyp * N * row + (int64_t)k0 * R;

  // forward step 1: task (e, b, c), e fastest; lanes (even half, odd half =
  // inputs times w_2N^z) of the 16-point DFT over a of z = NB*a + b, then the
  // four-step twiddle (the same for both halves).
  for (int t = threadIdx.x; t < T1; t += blockDim.x) {
    const int e = t & (W - 1), r = t >> lgW;
    const int b = r % NB, c = r / NB;
    const unsigned live = zqs[b];   // slices z = NB*q + b
    const cplx<float>* src = base + c * cstride + (int64_t)b * row + e;
    cp u[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const cplx<float> v =
          (e < wl && ((live >> q) & 1u)) ? src[(int64_t)NB * q * row] : cplx<float>{0.f, 0.f};
      const float2 w = tw2s[NB * q + b];
      u[q] = cp{f2_make(v.x, v.x * w.x - v.y * w.y), f2_make(v.y, v.x * w.y + v.y * w.x)};
    }
    dftp<false, 16>(u);
    cp* d = buf + (c * W + e) * S + b * 16;
    sts_cp(d + b, u[0]);
#pragma unroll
    for (int k1 = 1; k1 < 16; ++k1) {
      const ulonglong2 w = twq[b * 18 + k1];
      sts_cp(d + (k1 ^ b), tw_mul(u[k1], f2{w.x}, f2{w.y}, f2{twn[b * 18 + k1]}));
    }
  }
  __syncthreads();
  // forward step 2 (in place): task (s, k1), k1 fastest; NB-point DFT
  for (int t = threadIdx.x; t < C * W * 16; t += blockDim.x) {
    const int k1 = t & 15, s = t >> 4;
    cp* p = buf + s * S;
    cp w[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) w[b] = lds_cp(p + zpos(b, k1));
    dftp<false, NB>(w);
#pragma unroll
    for (int k2 = 0; k2 < NB; ++k2) sts_cp(p + zpos(k2, k1), w[k2]);
  }
  __syncthreads();

  // Green block product, item (e, k): frequencies 2k and 2k+1 of every
  // component at zpos(k >> 4, k & 15).
  const int beta = kyp / n2, ky = 2 * (kyp - beta * n2) + beta;
  for (int i = threadIdx.x; i < N * W; i += blockDim.x) {
    const int e = i & (W - 1), k = i >> lgW;
    const int kxp = k0 + (e >> a.lgR);
    if (kxp >= m1) continue;
    const int alpha = kxp >= n1 ? 1 : 0;
    const int kx = 2 * (kxp - alpha * n1) + alpha;
    const float4* gp = reinterpret_cast<const float4*>(a.G) + ((int64_t)ky * m1 + kx) * U * N + k;
    cp* v = buf + e * S + zpos(k >> 4, k & 15);
    zpoint_pair<PWL, OP>(std::make_integer_sequence<int, NE>{}, v, W * S, gp, N);
  }
  __syncthreads();
  // inverse step A (in place): task (s, k1), k1 fastest; inverse NB-point DFT
  // and the conjugate four-step twiddle
  for (int t = threadIdx.x; t < C * W * 16; t += blockDim.x) {
    const int k1 = t & 15, s = t >> 4;
    cp* p = buf + s * S;
    cp w[NB];
#pragma unroll
    for (int k2 = 0; k2 < NB; ++k2) w[k2] = lds_cp(p + zpos(k2, k1));
    dftp<true, NB>(w);
    sts_cp(p + zpos(0, k1), w[0]);
#pragma unroll
    for (int b = 1; b < NB; ++b) {
      const ulonglong2 q = twq[b * 18 + k1];
      sts_cp(p + zpos(b, k1), tw_mulc(w[b], f2{q.x}, f2{q.y}, f2{twn[b * 18 + k1]}));
    }
  }
  __syncthreads();
  // inverse step B: task (e, b, c) as in step 1, inverse 16-point DFT of both
  // halves; output z = NB*q + b is even(q) + odd(q) * conj(w_2N^z).
  for (int t = threadIdx.x; t < T1; t += blockDim.x) {
    const int e = t & (W - 1), r = t >> lgW;
    const int b = r % NB, c = r / NB;
    const cp* sp = buf + (c * W + e) * S + b * 16;
    cp u[16];
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) u[k1] = lds_cp(sp + (k1 ^ b));
    dftp<true, 16>(u);
    const bool st = e < wl;
    const unsigned live = zqs[b];
    cplx<float>* dst = base + c * cstride + (int64_t)b * row + e;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      float ar, br, ai, bi;
      f2_split(u[q].re, ar, br);
      f2_split(u[q].im, ai, bi);
      const float2 w = tw2s[NB * q + b];
      const cplx<float> out{fmaf(br, w.x, fmaf(bi, w.y, ar)), fmaf(bi, w.x, fmaf(-br, w.y, ai))};
      if (st && ((live >> q) & 1u)) dst[(int64_t)NB * q * row] = out;
    }
  }
}

}  // namespace marie
