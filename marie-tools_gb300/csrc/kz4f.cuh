// Four-step z pass of the complex128 operator in float-float arithmetic
// (n3 = 16*NB), every complex value in packed FP32 pairs with (re, im) in the
// two lanes (ffpair.cuh).  Same work split, half layout and half combine as
// k4_z (kz4.cuh), with the stride and pad of 16-byte elements (kzf_stride);
// shared memory holds ffc2 values (re.hi, im.hi, re.lo, im.lo), so the
// z-DFTs, the four-step twiddles and the Green product issue one f32x2
// instruction for both parts of every float-float operation.
#pragma once

#include "fastpath.cuh"
#include "ffpair.cuh"
#include "kz4.cuh"

namespace marie {

// ---------------------------------------------------------------------------
// Float-float PWL multiply of one point for N / N^H.  Unrolled like zpoint,
// the 144 entries are thousands of instructions in float-float and overflow
// the instruction cache, so here the output group P and the input group Q run
// as loops (three trips each) over a body holding the ten Tucker indices j
// unrolled: block (j, k) with k = PQ_N(P, Q) - 1, entries (l, lp) with
// |LLP(l, lp)| = j + 1 (the same for every (P, Q) since PQ_N carries no sign).
// The arithmetic runs in packed FP32 pairs with (re, im) in the two lanes;
// accumulators stay unnormalised (hi, lo) pairs until the end.
// ---------------------------------------------------------------------------
struct PwlPQ {
  int jl[4][4];          // Tucker index j of entry (l, lp)
  int sg[4][4];          // its sign
};

template <int OP>
constexpr PwlPQ make_pwl_pq() {
  using Tab = OpTab<true, OP>;
  PwlPQ t{};
  for (int i = 0; i < Tab::NE; ++i) {
    const OpEntry e = Tab::L.e[i];
    if (e.p < 4 && e.q < 4) {      // (P, Q) = (0, 0): block (j, 0)
      t.jl[e.p][e.q] = e.blk / 6;
      t.sg[e.p][e.q] = e.sgn;
    }
  }
  return t;
}

// acc += a*b per lane (NEG: acc -= a*b) on unnormalised float-float pairs:
// product error by FMA, sum error by two-sum, both collected in acc.lo.  na
// is -a; the error term is accumulated negated (p - a*b) so that every FMA
// adds, which gives the same values as the scalar form a*b - p.
template <bool NEG>
__device__ __forceinline__ void ff_acc2(ffc2& acc, const ffc2& a, const ffc2& na, const ffc2& b) {
  const ffc2& A = NEG ? na : a;
  const ffc2& NA = NEG ? a : na;
  const f2 p = A.hi * b.hi;
  f2 e = fma2(NA.hi, b.hi, p);
  e = fma2(NA.hi, b.lo, e);
  e = fma2(NA.lo, b.hi, e);
  const f2 s = acc.hi + p;
  const f2 bb = s - acc.hi;
  const f2 sl = (acc.hi - (s - bb)) + (p - bb);
  acc.hi = s;
  acc.lo = acc.lo + (sl - e);
}


// y += sgn * g * x for g = gr + i gi: lanes (re, im) += gr * (xr, xi) and
// (re, im) += (-gi, gi) * (xi, xr), in the order of the scalar form (the
// exchanged lanes (xi, xr) are formed at each use: keeping them costs 16
// registers and spills).
template <int OP>
__device__ __forceinline__ void zpoint_pwl_ff(ffc2* v, int qstride, const cplx<ff>* gp) {
  constexpr PwlPQ TB = make_pwl_pq<OP>();
  const f2 zero = f2_make(0.f, 0.f);
  // all inputs in registers first (outputs go back in place); the output
  // group P and the input group Q both run as loops, so the unrolled body
  // is the ten blocks of one (P, Q) pair
  ffc2 xin[12];
#pragma unroll
  for (int q = 0; q < 12; ++q) xin[q] = lds_ffc2(v + q * qstride);
#pragma unroll 1
  for (int P = 0; P < 3; ++P) {
    ffc2 y[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) y[l] = ffc2{zero, zero};
#pragma unroll 1
    for (int Q = 0; Q < 3; ++Q) {
      ffc2 x[4];
#pragma unroll
      for (int lp = 0; lp < 4; ++lp) x[lp] = Q == 0 ? xin[lp] : (Q == 1 ? xin[4 + lp] : xin[8 + lp]);
      const int k = P + Q + ((P > 0 && Q > 0) ? 1 : 0);    // PQ_N(P, Q) - 1
      const cplx<ff>* gk = gp + k;                          // block (j, k) at 6j + k
#pragma unroll
      for (int j = 0; j < 10; ++j) {
        const float4 g = __ldg(reinterpret_cast<const float4*>(gk + 6 * j));   // (gr.hi, gr.lo, gi.hi, gi.lo)
        const ffc2 a1{f2_bc(g.x), f2_bc(g.y)};
        const ffc2 na1{zero - a1.hi, zero - a1.lo};
        ffc2 a2{f2_make(-g.z, g.z), f2_make(-g.w, g.w)};
        ffc2 na2{zero - a2.hi, zero - a2.lo};
        if constexpr ((OP & 1) != 0) {   // conj(g)
          const ffc2 t = a2;
          a2 = na2;
          na2 = t;
        }
#pragma unroll
        for (int l = 0; l < 4; ++l) {
#pragma unroll
          for (int lp = 0; lp < 4; ++lp) {
            if (TB.jl[l][lp] == j) {
              if (TB.sg[l][lp] > 0) {
                ff_acc2<false>(y[l], a1, na1, x[lp]);
                ff_acc2<false>(y[l], a2, na2, ffc2_swap(x[lp]));
              } else {
                ff_acc2<true>(y[l], a1, na1, x[lp]);
                ff_acc2<true>(y[l], a2, na2, ffc2_swap(x[lp]));
              }
            }
          }
        }
      }
    }
#pragma unroll
    for (int l = 0; l < 4; ++l) {
      const f2 s = y[l].hi + y[l].lo;
      sts_ffc2(v + (4 * P + l) * qstride, ffc2{s, y[l].lo - (s - y[l].hi)});
    }
  }
}

// PWC (C = 3): one entry of the 3 x 3 product, entries sorted by block.
template <int OP, int K>
struct ZPointFF {
  static __device__ __forceinline__ void run(ffc2* y, const ffc2* x, const ffc2* xs, ffc2& a1, ffc2& na1, ffc2& a2,
                                             ffc2& na2, const cplx<ff>* gp) {
    using Tab = OpTab<false, OP>;
    constexpr int blk = Tab::L.e[K].blk;
    constexpr int p = Tab::L.e[K].p, q = Tab::L.e[K].q, sg = Tab::L.e[K].sgn;
    constexpr bool first = (K == 0) || (Tab::L.e[K == 0 ? 0 : K - 1].blk != blk);
    if constexpr (first) {
      const f2 zero = f2_make(0.f, 0.f);
      const float4 g = __ldg(reinterpret_cast<const float4*>(gp + blk));
      a1 = ffc2{f2_bc(g.x), f2_bc(g.y)};
      na1 = ffc2{zero - a1.hi, zero - a1.lo};
      a2 = ffc2{f2_make(-g.z, g.z), f2_make(-g.w, g.w)};
      na2 = ffc2{zero - a2.hi, zero - a2.lo};
      if constexpr ((OP & 1) != 0) {
        const ffc2 t = a2;
        a2 = na2;
        na2 = t;
      }
    }
    ff_acc2<(sg < 0)>(y[p], a1, na1, x[q]);
    ff_acc2<(sg < 0)>(y[p], a2, na2, xs[q]);
  }
};

template <int OP, int... Ks>
__device__ __forceinline__ void zpoint_pwc_ff(std::integer_sequence<int, Ks...>, ffc2* v, int qstride,
                                              const cplx<ff>* gp) {
  const f2 zero = f2_make(0.f, 0.f);
  ffc2 x[3], xs[3], y[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    x[q] = lds_ffc2(v + q * qstride);
    xs[q] = ffc2_swap(x[q]);
    y[q] = ffc2{zero, zero};
  }
  ffc2 a1, na1, a2, na2;
  (ZPointFF<OP, Ks>::run(y, x, xs, a1, na1, a2, na2, gp), ...);
#pragma unroll
  for (int p = 0; p < 3; ++p) {
    const f2 s = y[p].hi + y[p].lo;
    sts_ffc2(v + p * qstride, ffc2{s, y[p].lo - (s - y[p].hi)});
  }
}

template <int NB, bool PWL, int OP>
__global__ void __launch_bounds__(256, 2) k4_zf(MvArgs<ff> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int N = 16 * NB;
  constexpr int C = PWL ? 12 : 3;
  constexpr int NE = OpTab<PWL, OP>::NE;
  const int bu = blockIdx.x;
  if (!bundle_active(a, bu)) return;
  const int kyp = blockIdx.z, k0 = blockIdx.y * a.TX;
  const int n1 = a.n1, n2 = a.n2, m1 = 2 * n1, R = a.R;
  const int W = a.TX * R, wl = min(a.TX, m1 - k0) * R;
  const int lgW = 31 - __clz(W);                // W = TX*R is a power of two
  const int S = kzf_stride(N, W);
  const int H = C * W * S + kzf_halfpad(W);   // start of the odd half
  const int T1 = 2 * C * NB * W;              // tasks of forward step 1 / inverse step B
  // four-step twiddles w_N^(b*k1) at b*18 + k1, high and low halves of the
  // 32-byte entries in separate 16-byte arrays
  ulonglong2* twh = reinterpret_cast<ulonglong2*>(smem_raw);
  ulonglong2* twl = twh + 18 * NB;
  ffc2* buf = reinterpret_cast<ffc2*>(twl + 18 * NB);
  for (int i = threadIdx.x; i < 18 * NB; i += blockDim.x) {
    const int b = i / 18, k1 = i - 18 * (i / 18);
    const fftw t = fftw_make(k1 < 16 ? a.az.tw[b * k1] : cplx<ff>{ff(0), ff(0)});
    twh[i] = make_ulonglong2(t.rh.v, t.ih.v);
    twl[i] = make_ulonglong2(t.rl.v, t.il.v);
  }
  auto twf = [&](int i) {
    const ulonglong2 h = twh[i], l = twl[i];
    return fftw{f2{h.x}, f2{h.y}, f2{l.x}, f2{l.y}};
  };
  __syncthreads();
  const int64_t row = (int64_t)m1 * R;
  const int64_t cstride = (int64_t)2 * n2 * N * row;
  cplx<ff>* base = a.S + (int64_t)bu * C * cstride + (int64_t)kyp * N * row + (int64_t)k0 * R;

  // forward step 1: task (e, h, b, c), e fastest; half h of the zero-padded
  // 2N-point transform (h = 1: inputs times w_2N^z), 16-point DFT over a of
  // z = NB*a + b, then the four-step twiddle.
  for (int t = threadIdx.x; t < T1; t += blockDim.x) {
    const int e = t & (W - 1), r = t >> lgW;
    const int h = r & 1, r2 = r >> 1;
    const int b = r2 % NB, c = r2 / NB;
    const unsigned live = a.zq ? a.zq[b] : 0xffffu;   // slices z = NB*q + b
    ffc2 u[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      cplx<ff> val = (e < wl && ((live >> q) & 1u)) ? base[c * cstride + (int64_t)(NB * q + b) * row + e]
                                                    : cplx<ff>{ff(0), ff(0)};
      if (h) val = val * a.az.tw2[NB * q + b];
      u[q] = to_ffc2(val);
    }
    dftf<false, 16>(u);
    ffc2* d = buf + h * H + (c * W + e) * S + b * 16;
    sts_ffc2(d + b, u[0]);
#pragma unroll
    for (int k1 = 1; k1 < 16; ++k1) sts_ffc2(d + (k1 ^ b), tw_mulf<false>(u[k1], twf(b * 18 + k1)));
  }
  __syncthreads();
  // forward step 2 (in place): task (s, k1), k1 fastest; NB-point DFT
  for (int t = threadIdx.x; t < 2 * C * W * 16; t += blockDim.x) {
    const int k1 = t & 15, s = t >> 4;
    const int h = s >= C * W ? 1 : 0;
    ffc2* p = buf + h * H + (s - h * C * W) * S;
    ffc2 w[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) w[b] = lds_ffc2(p + zpos(b, k1));
    dftf<false, NB>(w);
#pragma unroll
    for (int k2 = 0; k2 < NB; ++k2) sts_ffc2(p + zpos(k2, k1), w[k2]);
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
    const cplx<ff>* gp = a.G + (((int64_t)ky * m1 + kx) * (2 * N) + kz) * U;
    ffc2* v = buf + g * H + e * S + zpos(k >> 4, k & 15);
    if constexpr (PWL) zpoint_pwl_ff<OP>(v, W * S, gp);
    else zpoint_pwc_ff<OP>(std::make_integer_sequence<int, NE>{}, v, W * S, gp);
  }
  __syncthreads();
  // inverse step A (in place): task (s, k1), k1 fastest
  for (int t = threadIdx.x; t < 2 * C * W * 16; t += blockDim.x) {
    const int k1 = t & 15, s = t >> 4;
    const int h = s >= C * W ? 1 : 0;
    ffc2* p = buf + h * H + (s - h * C * W) * S;
    ffc2 w[NB];
#pragma unroll
    for (int k2 = 0; k2 < NB; ++k2) w[k2] = lds_ffc2(p + zpos(k2, k1));
    dftf<true, NB>(w);
    sts_ffc2(p + zpos(0, k1), w[0]);
#pragma unroll
    for (int b = 1; b < NB; ++b) sts_ffc2(p + zpos(b, k1), tw_mulf<true>(w[b], twf(b * 18 + k1)));
  }
  __syncthreads();
  // inverse step B: task (e, h, b, c) as in step 1, inverse 16-point DFT of
  // half h (h = 1 then times conj(w_2N^z)); the partner lane t ^ W holds the
  // other half of the same (e, b, c): the even lane stores q < 8, the odd lane
  // q >= 8, after one exchange (the loop is warp-uniform, as in k4_z).
  const int lane = threadIdx.x & 31;
  for (int tb = threadIdx.x - lane; tb < T1; tb += blockDim.x) {
    const int t = tb + lane;
    const bool act = t < T1;
    const int tt = act ? t : (t & (2 * W - 1));   // a valid task with the same (e, h)
    const int e = tt & (W - 1), r = tt >> lgW;
    const int h = r & 1, r2 = r >> 1;
    const int b = r2 % NB, c = r2 / NB;
    const ffc2* sp = buf + h * H + (c * W + e) * S + b * 16;
    ffc2 uf[16];
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) uf[k1] = lds_ffc2(sp + (k1 ^ b));
    dftf<true, 16>(uf);
    cplx<ff> u[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) u[q] = from_ffc2(uf[q]);
    if (h) {
#pragma unroll
      for (int q = 0; q < 16; ++q) u[q] = mulc(u[q], a.az.tw2[NB * q + b]);
    }
    const bool st = act && e < wl;
    const unsigned live = (a.zq ? a.zq[b] : 0xffffu) >> (8 * h);   // slices z = NB*(8h + j) + b
    cplx<ff>* dst = base + c * cstride + (int64_t)(NB * 8 * h + b) * row + e;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const cplx<ff> send = h ? u[j] : u[8 + j];
      const cplx<ff> recv = shfl_xor_c(send, W);
      const cplx<ff> out = h ? recv + u[8 + j] : u[j] + recv;
      if (st && ((live >> j) & 1u)) dst[(int64_t)NB * j * row] = out;
    }
  }
}

}  // namespace marie
