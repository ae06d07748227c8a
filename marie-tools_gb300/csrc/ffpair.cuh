// Complex float-float arithmetic in packed FP32 pairs: a complex value
// (re, im), each part a float-float (hi, lo), is held as ffc2 {hi = (re.hi,
// im.hi), lo = (re.lo, im.lo)}, so the real and imaginary parts of every
// float-float operation go through one f32x2 instruction (pair.cuh).  Each
// operation performs the scalar float-float steps of common.cuh (two-sum,
// fast two-sum, FMA product error) in the same order, written so that every
// FMA adds: a product error is carried negated (p - a*b) and folded back by
// a subtraction, which gives the same values as the scalar form.
#pragma once

#include "pair.cuh"

namespace marie {

struct __align__(16) ffc2 {
  f2 hi, lo;
};

__device__ __forceinline__ f2 f2_swap(f2 a) {
  float x, y;
  f2_split(a, x, y);
  return f2_make(y, x);
}

__device__ __forceinline__ ffc2 to_ffc2(cplx<ff> v) {
  return {f2_make(v.x.hi, v.y.hi), f2_make(v.x.lo, v.y.lo)};
}
__device__ __forceinline__ cplx<ff> from_ffc2(ffc2 v) {
  float rh, ih, rl, il;
  f2_split(v.hi, rh, ih);
  f2_split(v.lo, rl, il);
  return {ff(rh, rl), ff(ih, il)};
}
__device__ __forceinline__ ffc2 lds_ffc2(const ffc2* p) {
  const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(p);
  return {f2{v.x}, f2{v.y}};
}
__device__ __forceinline__ void sts_ffc2(ffc2* p, ffc2 v) {
  *reinterpret_cast<ulonglong2*>(p) = make_ulonglong2(v.hi.v, v.lo.v);
}

// a + b and a - b per lane (the one-pass float-float sum of common.cuh)
__device__ __forceinline__ ffc2 operator+(ffc2 a, ffc2 b) {
  const f2 s = a.hi + b.hi;
  const f2 bb = s - a.hi;
  const f2 e = (a.hi - (s - bb)) + (b.hi - bb);
  const f2 l = e + (a.lo + b.lo);
  const f2 h = s + l;
  return {h, l - (h - s)};
}
__device__ __forceinline__ ffc2 operator-(ffc2 a, ffc2 b) {
  const f2 s = a.hi - b.hi;
  const f2 bb = s - a.hi;
  const f2 e = (a.hi - (s - bb)) - (b.hi + bb);
  const f2 l = e + (a.lo - b.lo);
  const f2 h = s + l;
  return {h, l - (h - s)};
}

// (im, re): the lanes exchanged
__device__ __forceinline__ ffc2 ffc2_swap(ffc2 v) { return {f2_swap(v.hi), f2_swap(v.lo)}; }

// w*b for w = -i (forward) or +i (inverse): lanes (b.im, -b.re) / (-b.im, b.re)
template <bool INV>
__device__ __forceinline__ ffc2 mul_w(ffc2 b) {
  const f2 sg = INV ? f2_make(-1.f, 1.f) : f2_make(1.f, -1.f);
  return {f2_swap(b.hi) * sg, f2_swap(b.lo) * sg};
}

// a times the per-lane float-float constant k, given k.hi and the negated
// -k.hi, -k.lo
__device__ __forceinline__ ffc2 mulk(ffc2 a, f2 khi, f2 nkhi, f2 nklo) {
  const f2 p = a.hi * khi;
  f2 e = fma2(a.hi, nkhi, p);   // p - a.hi*k.hi (exact)
  e = fma2(a.hi, nklo, e);
  e = fma2(a.lo, nkhi, e);
  const f2 h = p - e;
  return {h, (p - h) - e};
}

// Lanes (d0, d1) of two double constants as float-float: hi and the negated
// hi, lo.
struct kff {
  f2 hi, nhi, nlo;
};
__device__ __forceinline__ kff kff_make(double d0, double d1) {
  const ff a(d0), b(d1);
  return {f2_make(a.hi, b.hi), f2_make(-a.hi, -b.hi), f2_make(-a.lo, -b.lo)};
}

// v * exp(-+ i theta) for cos(theta) = c, sin(theta) = s (forward: minus):
// (re, im) = (vr c, vi c) + (-vi ws, vr ws), ws the signed sine
template <bool INV>
__device__ __forceinline__ ffc2 rotf(ffc2 v, double c, double s) {
  const double ws = INV ? s : -s;
  if (c == 0.0) return ws > 0 ? mul_w<true>(v) : mul_w<false>(v);
  const kff C = kff_make(c, c), B = kff_make(-ws, ws);
  const ffc2 a = mulk(v, C.hi, C.nhi, C.nlo);
  const ffc2 b = mulk(ffc2_swap(v), B.hi, B.nhi, B.nlo);
  return a + b;
}

// Twiddle table entry for w = wr + i wi: hi = ((wr.hi, wr.hi), (-wi.hi,
// wi.hi)), lo = the same for the low parts (32 bytes).
struct __align__(16) fftw {
  f2 rh, ih, rl, il;
};
__device__ __forceinline__ fftw fftw_make(cplx<ff> w) {
  return {f2_make(w.x.hi, w.x.hi), f2_make(-w.y.hi, w.y.hi), f2_make(w.x.lo, w.x.lo), f2_make(-w.y.lo, w.y.lo)};
}
// v * w (CONJ: v * conj(w))
template <bool CONJ>
__device__ __forceinline__ ffc2 tw_mulf(ffc2 v, const fftw& t) {
  const f2 zero = f2_make(0.f, 0.f);
  const ffc2 a = mulk(v, t.rh, zero - t.rh, zero - t.rl);
  const ffc2 vs = ffc2_swap(v);
  const ffc2 b = CONJ ? mulk(vs, zero - t.ih, t.ih, t.il) : mulk(vs, t.ih, zero - t.ih, zero - t.il);
  return a + b;
}

// ---------------------------------------------------------------------------
// DFTs of lengths 1-8 and 16, in place, natural order, no scaling.
// ---------------------------------------------------------------------------

template <bool INV>
__device__ __forceinline__ void dftf2(ffc2* v) {
  const ffc2 a = v[0];
  v[0] = a + v[1];
  v[1] = a - v[1];
}

template <bool INV>
__device__ __forceinline__ void dftf4(ffc2* v) {
  const ffc2 t0 = v[0] + v[2], t1 = v[0] - v[2];
  const ffc2 t2 = v[1] + v[3], d = mul_w<INV>(v[1] - v[3]);
  v[0] = t0 + t2;
  v[2] = t0 - t2;
  v[1] = t1 + d;
  v[3] = t1 - d;
}

template <bool INV>
__device__ __forceinline__ void dftf8(ffc2* v) {
  const double h = 0.707106781186547524401;
  ffc2 e[4] = {v[0], v[2], v[4], v[6]};
  ffc2 o[4] = {v[1], v[3], v[5], v[7]};
  dftf4<INV>(e);
  dftf4<INV>(o);
  const ffc2 o1 = rotf<INV>(o[1], h, h);
  const ffc2 o2 = mul_w<INV>(o[2]);
  const ffc2 o3 = rotf<INV>(o[3], -h, h);
  v[0] = e[0] + o[0];
  v[4] = e[0] - o[0];
  v[1] = e[1] + o1;
  v[5] = e[1] - o1;
  v[2] = e[2] + o2;
  v[6] = e[2] - o2;
  v[3] = e[3] + o3;
  v[7] = e[3] - o3;
}

template <bool INV, int R>
__device__ __forceinline__ void dftf_prime(ffc2* v) {
  constexpr int H = (R - 1) / 2;
  ffc2 s[H], d[H];
#pragma unroll
  for (int j = 1; j <= H; ++j) {
    s[j - 1] = v[j] + v[R - j];
    d[j - 1] = v[j] - v[R - j];
  }
  const ffc2 a0 = v[0];
  ffc2 sum = a0;
#pragma unroll
  for (int j = 0; j < H; ++j) sum = sum + s[j];
  v[0] = sum;
#pragma unroll
  for (int k = 1; k <= H; ++k) {
    ffc2 re = a0, im;
#pragma unroll
    for (int j = 1; j <= H; ++j) {
      const int m = (j * k) % R;
      const int mm = m <= H ? m : R - m;
      const double c = PrimeTab<R>::c(mm);
      const double sn = m <= H ? PrimeTab<R>::s(mm) : -PrimeTab<R>::s(mm);
      const kff C = kff_make(c, c), S = kff_make(sn, sn);
      re = re + mulk(s[j - 1], C.hi, C.nhi, C.nlo);
      const ffc2 t = mulk(d[j - 1], S.hi, S.nhi, S.nlo);
      im = j == 1 ? t : im + t;
    }
    const ffc2 wim = mul_w<INV>(im);
    v[k] = re + wim;
    v[R - k] = re - wim;
  }
}

template <bool INV>
__device__ __forceinline__ void dftf6(ffc2* v) {
  const double h3 = 0.866025403784438646764;
  ffc2 A[6];
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    ffc2 t[2] = {v[b], v[3 + b]};
    dftf2<INV>(t);
    A[b * 2 + 0] = t[0];
    A[b * 2 + 1] = b == 0 ? t[1] : (b == 1 ? rotf<INV>(t[1], 0.5, h3) : rotf<INV>(t[1], -0.5, h3));
  }
#pragma unroll
  for (int k1 = 0; k1 < 2; ++k1) {
    ffc2 t[3] = {A[k1], A[2 + k1], A[4 + k1]};
    dftf_prime<INV, 3>(t);
#pragma unroll
    for (int k2 = 0; k2 < 3; ++k2) v[k1 + 2 * k2] = t[k2];
  }
}

template <bool INV>
__device__ __forceinline__ void dftf16(ffc2* v) {
  ffc2 A[16];
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    ffc2 t[4] = {v[b], v[4 + b], v[8 + b], v[12 + b]};
    dftf4<INV>(t);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) A[b * 4 + k1] = (b * k1 == 0) ? t[k1] : rotf<INV>(t[k1], c16(b * k1), s16(b * k1));
  }
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    ffc2 t[4] = {A[k1], A[4 + k1], A[8 + k1], A[12 + k1]};
    dftf4<INV>(t);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[k2];
  }
}

template <bool INV, int N>
__device__ __forceinline__ void dftf(ffc2* v) {
  if constexpr (N == 1) {
  } else if constexpr (N == 2) {
    dftf2<INV>(v);
  } else if constexpr (N == 4) {
    dftf4<INV>(v);
  } else if constexpr (N == 6) {
    dftf6<INV>(v);
  } else if constexpr (N == 8) {
    dftf8<INV>(v);
  } else if constexpr (N == 16) {
    dftf16<INV>(v);
  } else {
    dftf_prime<INV, N>(v);
  }
}

template <bool INV, int N>
__device__ __forceinline__ void dftn_ffc2(cplx<ff>* v) {
  ffc2 u[N];
#pragma unroll
  for (int i = 0; i < N; ++i) u[i] = to_ffc2(v[i]);
  dftf<INV, N>(u);
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = from_ffc2(u[i]);
}

}  // namespace marie
