// Packed FP32 pairs (sm_100 family f32x2 arithmetic) and pair-of-sequence
// complex DFTs.
//
// `f2` holds two floats in one 64-bit register pair; add/sub/mul/fma act on
// both lanes in one instruction (`add.rn.f32x2` etc., PTX ISA 8.6+).  A `cp`
// is a complex value of two independent sequences in structure-of-arrays
// form, (re0, re1) and (im0, im1), so every complex add costs two packed
// instructions for both sequences.  The z pass of the complex64 operator
// keeps the even- and odd-frequency halves of its zero-padded transform in
// the two lanes.  All operations round to nearest like their scalar forms.
#pragma once

#include <cstdint>

#include "matvec4.cuh"

namespace marie {

struct f2 {
  unsigned long long v;
};

__device__ __forceinline__ f2 f2_make(float lo, float hi) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ f2 f2_bc(float c) { return f2_make(c, c); }
__device__ __forceinline__ void f2_split(f2 a, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a.v));
}
__device__ __forceinline__ f2 operator+(f2 a, f2 b) {
  f2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ f2 operator-(f2 a, f2 b) {
  f2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ f2 operator*(f2 a, f2 b) {
  f2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
// a * b + c
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
  f2 r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return r;
}
// -a (as 0 - a: the sign of a zero result may differ from a negation)
__device__ __forceinline__ f2 f2_neg(f2 a) { return f2_make(0.f, 0.f) - a; }

struct __align__(16) cp {
  f2 re, im;
};

__device__ __forceinline__ cp operator+(cp a, cp b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cp operator-(cp a, cp b) { return {a.re - b.re, a.im - b.im}; }

// a + w b and a - w b for w = -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ cp add_w(cp a, cp b) {
  return INV ? cp{a.re - b.im, a.im + b.re} : cp{a.re + b.im, a.im - b.re};
}
template <bool INV>
__device__ __forceinline__ cp sub_w(cp a, cp b) {
  return INV ? cp{a.re + b.im, a.im - b.re} : cp{a.re - b.im, a.im + b.re};
}

// v * exp(-+ i theta) for cos(theta) = c, sin(theta) = s (forward: minus)
template <bool INV>
__device__ __forceinline__ cp rot2(cp v, double c, double s) {
  const float ws = INV ? (float)s : (float)-s;
  if (c == 0.0) {   // multiply by ws * i
    return ws > 0 ? cp{f2_neg(v.im), v.re} : cp{v.im, f2_neg(v.re)};
  }
  const f2 C = f2_bc((float)c), WS = f2_bc(ws), NWS = f2_bc(-ws);
  return {fma2(v.re, C, v.im * NWS), fma2(v.re, WS, v.im * C)};
}

// v * w and v * conj(w) for a twiddle w given as (wr, wr), (wi, wi), (-wi, -wi)
__device__ __forceinline__ cp tw_mul(cp v, f2 wr, f2 wi, f2 nwi) {
  return {fma2(v.re, wr, v.im * nwi), fma2(v.re, wi, v.im * wr)};
}
__device__ __forceinline__ cp tw_mulc(cp v, f2 wr, f2 wi, f2 nwi) {
  return {fma2(v.re, wr, v.im * wi), fma2(v.im, wr, v.re * nwi)};
}

// ---------------------------------------------------------------------------
// DFTs of lengths 1-8 and 16 on pairs, in place, natural order in and out.
// Forward sign exp(-2 pi i j k / R), inverse +, no scaling.
// ---------------------------------------------------------------------------

template <bool INV>
__device__ __forceinline__ void dftp2(cp* v) {
  const cp a = v[0];
  v[0] = a + v[1];
  v[1] = a - v[1];
}

template <bool INV>
__device__ __forceinline__ void dftp4(cp* v) {
  const cp t0 = v[0] + v[2], t1 = v[0] - v[2];
  const cp t2 = v[1] + v[3], d = v[1] - v[3];
  v[0] = t0 + t2;
  v[2] = t0 - t2;
  v[1] = add_w<INV>(t1, d);
  v[3] = sub_w<INV>(t1, d);
}

template <bool INV>
__device__ __forceinline__ void dftp8(cp* v) {
  const double h = 0.707106781186547524401;
  cp e[4] = {v[0], v[2], v[4], v[6]};
  cp o[4] = {v[1], v[3], v[5], v[7]};
  dftp4<INV>(e);
  dftp4<INV>(o);
  const cp o1 = rot2<INV>(o[1], h, h);
  const cp o3 = rot2<INV>(o[3], -h, h);
  v[0] = e[0] + o[0];
  v[4] = e[0] - o[0];
  v[1] = e[1] + o1;
  v[5] = e[1] - o1;
  v[2] = add_w<INV>(e[2], o[2]);
  v[6] = sub_w<INV>(e[2], o[2]);
  v[3] = e[3] + o3;
  v[7] = e[3] - o3;
}

// Odd prime R: X_k = a0 + sum_j s_j cos(2 pi jk/R) -+ i sum_j d_j sin(2 pi jk/R),
// s_j = a_j + a_{R-j}, d_j = a_j - a_{R-j} (j = 1..(R-1)/2).
template <bool INV, int R>
__device__ __forceinline__ void dftp_prime(cp* v) {
  constexpr int H = (R - 1) / 2;
  cp s[H], d[H];
#pragma unroll
  for (int j = 1; j <= H; ++j) {
    s[j - 1] = v[j] + v[R - j];
    d[j - 1] = v[j] - v[R - j];
  }
  const cp a0 = v[0];
  cp sum = a0;
#pragma unroll
  for (int j = 0; j < H; ++j) sum = sum + s[j];
  v[0] = sum;
#pragma unroll
  for (int k = 1; k <= H; ++k) {
    cp re = a0, im;
#pragma unroll
    for (int j = 1; j <= H; ++j) {
      const int m = (j * k) % R;
      const int mm = m <= H ? m : R - m;
      const f2 c = f2_bc((float)PrimeTab<R>::c(mm));
      const f2 sn = f2_bc((float)(m <= H ? PrimeTab<R>::s(mm) : -PrimeTab<R>::s(mm)));
      re = cp{fma2(s[j - 1].re, c, re.re), fma2(s[j - 1].im, c, re.im)};
      im = j == 1 ? cp{d[0].re * sn, d[0].im * sn} : cp{fma2(d[j - 1].re, sn, im.re), fma2(d[j - 1].im, sn, im.im)};
    }
    // X_k = re + w im, X_{R-k} = re - w im (w = -i forward, +i inverse)
    v[k] = add_w<INV>(re, im);
    v[R - k] = sub_w<INV>(re, im);
  }
}

template <bool INV>
__device__ __forceinline__ void dftp6(cp* v) {
  const double h3 = 0.866025403784438646764;
  cp A[6];
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    cp t[2] = {v[b], v[3 + b]};
    dftp2<INV>(t);
    A[b * 2 + 0] = t[0];
    A[b * 2 + 1] = b == 0 ? t[1] : (b == 1 ? rot2<INV>(t[1], 0.5, h3) : rot2<INV>(t[1], -0.5, h3));
  }
#pragma unroll
  for (int k1 = 0; k1 < 2; ++k1) {
    cp t[3] = {A[k1], A[2 + k1], A[4 + k1]};
    dftp_prime<INV, 3>(t);
#pragma unroll
    for (int k2 = 0; k2 < 3; ++k2) v[k1 + 2 * k2] = t[k2];
  }
}

template <bool INV>
__device__ __forceinline__ void dftp16(cp* v) {
  cp A[16];
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    cp t[4] = {v[b], v[4 + b], v[8 + b], v[12 + b]};
    dftp4<INV>(t);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) A[b * 4 + k1] = (b * k1 == 0) ? t[k1] : rot2<INV>(t[k1], c16(b * k1), s16(b * k1));
  }
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    cp t[4] = {A[k1], A[4 + k1], A[8 + k1], A[12 + k1]};
    dftp4<INV>(t);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[k2];
  }
}

template <bool INV, int N>
__device__ __forceinline__ void dftp(cp* v) {
  if constexpr (N == 1) {
  } else if constexpr (N == 2) {
    dftp2<INV>(v);
  } else if constexpr (N == 4) {
    dftp4<INV>(v);
  } else if constexpr (N == 6) {
    dftp6<INV>(v);
  } else if constexpr (N == 8) {
    dftp8<INV>(v);
  } else if constexpr (N == 16) {
    dftp16<INV>(v);
  } else {
    dftp_prime<INV, N>(v);
  }
}

}  // namespace marie
