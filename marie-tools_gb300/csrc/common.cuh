// Common device-side types for the GB300 FFT-VIE library: interleaved
// complex numbers (the layout of MATLAB's R2018a interleaved complex API),
// small-radix DFT butterflies and the in-place mixed-radix FFT used by every
// pass of the matvec.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace marie {

// ---------------------------------------------------------------------------
// Float-float ("ff") numbers: value = hi + lo with |lo| <= ulp(hi)/2, a
// 48-bit significand carried by two FP32 registers (Dekker 1971; Knuth's
// two-sum; products by FMA).  GB300 runs FP32 at 64x its FP64 rate, so the
// complex128 operator evaluated in ff arithmetic beats native FP64 while its
// normwise error (about 1e-13 for a matvec) stays far below any GMRES
// tolerance.  Additions use the one-pass ("sloppy") form: the error bound is
// relative to |a| + |b|, which is what the normwise FFT error analysis uses.
// ---------------------------------------------------------------------------
struct __align__(8) ff {
  float hi, lo;
  ff() = default;
  __host__ __device__ constexpr ff(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr ff(int v) : hi((float)v), lo(0.0f) {}
  // split of a double: hi = round(d), lo = round(d - hi)
  __host__ __device__ constexpr explicit ff(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
};

__device__ __forceinline__ ff ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
// |a| >= |b| (or a == 0)
__device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff operator+(ff a, ff b) {
  const ff s = ff_two_sum(a.hi, b.hi);
  return ff_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ ff operator-(ff a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ ff operator-(ff a, ff b) { return a + (-b); }
__device__ __forceinline__ ff operator*(ff a, ff b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return ff_fast_two_sum(p, e);
}
// a * b + c with one renormalisation
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff c) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const ff s = ff_two_sum(p, c.hi);
  return ff_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(e, c.lo)));
}

// Scalar fused multiply-add in the arithmetic of T.
__device__ __forceinline__ float fmx(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmx(double a, double b, double c) { return ::fma(a, b, c); }
__device__ __forceinline__ ff fmx(ff a, ff b, ff c) { return ff_fma(a, b, c); }

template <typename T>
struct __align__(2 * sizeof(T)) cplx {
  T x, y;
};

// Element type of the operator's inputs and outputs in HBM for arithmetic T:
// the ff operator reads and writes complex128.
template <typename T>
struct IoOf {
  using type = T;
};
template <>
struct IoOf<ff> {
  using type = double;
};

template <typename T>
__device__ __forceinline__ cplx<T> io_load(cplx<typename IoOf<T>::type> v) {
  if constexpr (!std::is_same<T, ff>::value) {
    return v;
  } else {
    return {ff(v.x), ff(v.y)};
  }
}
template <typename T>
__device__ __forceinline__ cplx<typename IoOf<T>::type> io_store(cplx<T> v) {
  if constexpr (std::is_same<T, ff>::value) {
    return {(double)v.x.hi + (double)v.x.lo, (double)v.y.hi + (double)v.y.lo};
  } else {
    return v;
  }
}

template <typename T>
__host__ __device__ __forceinline__ cplx<T> mk(T a, T b) { return cplx<T>{a, b}; }
template <typename T>
__host__ __device__ __forceinline__ cplx<T> operator+(cplx<T> a, cplx<T> b) { return {a.x + b.x, a.y + b.y}; }
template <typename T>
__host__ __device__ __forceinline__ cplx<T> operator-(cplx<T> a, cplx<T> b) { return {a.x - b.x, a.y - b.y}; }
template <typename T>
__host__ __device__ __forceinline__ cplx<T> operator*(cplx<T> a, cplx<T> b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename T>
__host__ __device__ __forceinline__ cplx<T> scale(cplx<T> a, T s) { return {a.x * s, a.y * s}; }
template <typename T>
__host__ __device__ __forceinline__ cplx<T> conjg(cplx<T> a) { return {a.x, -a.y}; }
// a * conj(b)
template <typename T>
__host__ __device__ __forceinline__ cplx<T> mulc(cplx<T> a, cplx<T> b) {
  return {a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}
// acc += a * b
template <typename T>
__device__ __forceinline__ void fma_c(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.x = fmx(a.x, b.x, fmx(-a.y, b.y, acc.x));
  acc.y = fmx(a.x, b.y, fmx(a.y, b.x, acc.y));
}

// Read-only (non-coherent cache) load of a complex value.
__device__ __forceinline__ cplx<float> ldg_c(const cplx<float>* p) {
  const float2 v = __ldg(reinterpret_cast<const float2*>(p));
  return {v.x, v.y};
}
__device__ __forceinline__ cplx<double> ldg_c(const cplx<double>* p) {
  const double2 v = __ldg(reinterpret_cast<const double2*>(p));
  return {v.x, v.y};
}
__device__ __forceinline__ cplx<ff> ldg_c(const cplx<ff>* p) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  return {ff(v.x, v.y), ff(v.z, v.w)};
}

// acc -= a * b
template <typename T>
__device__ __forceinline__ void fms_c(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.x = fmx(-a.x, b.x, fmx(a.y, b.y, acc.x));
  acc.y = fmx(-a.x, b.y, fmx(-a.y, b.x, acc.y));
}

// Multiply by -i (forward transform sign) or +i (inverse).
template <typename T, bool INV>
__device__ __forceinline__ cplx<T> mul_mi(cplx<T> a) {
  return INV ? cplx<T>{-a.y, a.x} : cplx<T>{a.y, -a.x};
}

// ---------------------------------------------------------------------------
// Small DFTs in registers.  Forward sign exp(-2*pi*i*j*k/R), inverse +.
// ---------------------------------------------------------------------------

template <typename T, bool INV>
__device__ __forceinline__ void dft2(cplx<T>* v) {
  cplx<T> a = v[0];
  v[0] = a + v[1];
  v[1] = a - v[1];
}

template <typename T, bool INV>
__device__ __forceinline__ void dft4(cplx<T>* v) {
  cplx<T> t0 = v[0] + v[2], t1 = v[0] - v[2];
  cplx<T> t2 = v[1] + v[3], t3 = mul_mi<T, INV>(v[1] - v[3]);
  v[0] = t0 + t2;
  v[2] = t0 - t2;
  v[1] = t1 + t3;
  v[3] = t1 - t3;
}

template <typename T, bool INV>
__device__ __forceinline__ void dft8(cplx<T>* v) {
  const T h = (T)0.707106781186547524401;
  cplx<T> e[4] = {v[0], v[2], v[4], v[6]};
  cplx<T> o[4] = {v[1], v[3], v[5], v[7]};
  dft4<T, INV>(e);
  dft4<T, INV>(o);
  // twiddles w8^k, w8 = exp(-+ i pi/4)
  cplx<T> o1 = INV ? cplx<T>{h * (o[1].x - o[1].y), h * (o[1].x + o[1].y)}
                   : cplx<T>{h * (o[1].x + o[1].y), h * (o[1].y - o[1].x)};
  cplx<T> o2 = mul_mi<T, INV>(o[2]);
  cplx<T> o3 = INV ? cplx<T>{-h * (o[3].x + o[3].y), h * (o[3].x - o[3].y)}
                   : cplx<T>{h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y)};
  v[0] = e[0] + o[0];
  v[4] = e[0] - o[0];
  v[1] = e[1] + o1;
  v[5] = e[1] - o1;
  v[2] = e[2] + o2;
  v[6] = e[2] - o2;
  v[3] = e[3] + o3;
  v[7] = e[3] - o3;
}

// Odd prime R in {3,5,7}: X_k = a0 + sum_j s_j c_jk -+ i sum_j d_j s_jk,
// s_j = a_j + a_{R-j}, d_j = a_j - a_{R-j}.
template <int R>
struct PrimeTab;
template <>
struct PrimeTab<3> {
  static __device__ __forceinline__ double c(int m) { return -0.5; }
  static __device__ __forceinline__ double s(int m) { return 0.866025403784438646764; }
};
template <>
struct PrimeTab<5> {
  static __device__ __forceinline__ double c(int m) {
    return m == 1 ? 0.309016994374947424102 : -0.809016994374947424102;
  }
  static __device__ __forceinline__ double s(int m) {
    return m == 1 ? 0.951056516295153572116 : 0.587785252292473129169;
  }
};
template <>
struct PrimeTab<7> {
  static __device__ __forceinline__ double c(int m) {
    return m == 1 ? 0.623489801858733530525 : (m == 2 ? -0.222520933956314404289 : -0.900968867902419126236);
  }
  static __device__ __forceinline__ double s(int m) {
    return m == 1 ? 0.781831482468029808708 : (m == 2 ? 0.974927912181823607018 : 0.433883739117558120476);
  }
};

template <typename T, bool INV, int R>
__device__ __forceinline__ void dft_prime(cplx<T>* v) {
  constexpr int H = (R - 1) / 2;
  cplx<T> s[H], d[H];
#pragma unroll
  for (int j = 1; j <= H; ++j) {
    s[j - 1] = v[j] + v[R - j];
    d[j - 1] = v[j] - v[R - j];
  }
  cplx<T> a0 = v[0];
  cplx<T> sum = a0;
#pragma unroll
  for (int j = 0; j < H; ++j) sum = sum + s[j];
  v[0] = sum;
#pragma unroll
  for (int k = 1; k <= H; ++k) {
    cplx<T> re = a0, im = {0, 0};
#pragma unroll
    for (int j = 1; j <= H; ++j) {
      const int m = (j * k) % R;
      // cos(2 pi m/R), sin(2 pi m/R) with m folded into 1..H
      const int mm = m <= H ? m : R - m;
      const T c = (T)PrimeTab<R>::c(mm);
      const T sn = (T)(m <= H ? PrimeTab<R>::s(mm) : -PrimeTab<R>::s(mm));
      re = re + scale(s[j - 1], c);
      im = im + scale(d[j - 1], sn);
    }
    // forward: X_k = re - i*im, X_{R-k} = re + i*im
    cplx<T> iim = {-im.y, im.x};  // i*im
    if (INV) {
      v[k] = re + iim;
      v[R - k] = re - iim;
    } else {
      v[k] = re - iim;
      v[R - k] = re + iim;
    }
  }
}

// Generic prime radix (any R) using the n-th root table tw (tw[k] = w_n^k,
// forward sign): w_R^{u t} = tw[(n/R) * (u t mod R)].  Slow path for sizes
// with prime factors beyond 7.
template <typename T, bool INV>
__device__ __forceinline__ void dft_generic(cplx<T>* v, cplx<T>* out, int R, int n, const cplx<T>* tw) {
  const int step = n / R;
  for (int t = 0; t < R; ++t) {
    cplx<T> acc = {0, 0};
    for (int u = 0; u < R; ++u) {
      cplx<T> w = tw[step * ((u * t) % R)];
      if (INV) w = conjg(w);
      fma_c(acc, v[u], w);
    }
    out[t] = acc;
  }
}

template <typename T, bool INV, int R>
__device__ __forceinline__ void dft_small(cplx<T>* v) {
  if constexpr (R == 2) dft2<T, INV>(v);
  else if constexpr (R == 4) dft4<T, INV>(v);
  else if constexpr (R == 8) dft8<T, INV>(v);
  else dft_prime<T, INV, R>(v);
}

// ---------------------------------------------------------------------------
// FFT plans.  n = r[0]*r[1]*...*r[nst-1]; the DIF pass consumes r[0] first.
// Output of the DIF pass (and input of the DIT pass) is in mixed-radix
// digit-reversed order: position p = sum_i t_i * n/(r0..ri) holds frequency
// k = t0 + r0*t1 + r0*r1*t2 + ...
// ---------------------------------------------------------------------------

constexpr int kMaxStages = 12;
constexpr int kMaxAxis = 1024;   // largest supported grid edge n

struct FftPlan {
  int n;
  int nst;
  int r[kMaxStages];
};

// One DIF stage over all (sequence, butterfly) pairs owned by the CTA.
// buf[seq*ss + i*es] is element i of sequence seq.
template <typename T, bool INV, int R>
__device__ __forceinline__ void dif_stage(cplx<T>* buf, int nseq, int es, int ss, int n, int Lb,
                                          const cplx<T>* tw, bool seq_fast) {
  const int sub = Lb / R;
  const int nb = n / R;
  const int total = nseq * nb;
  const int tstride = n / Lb;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int seq, q;
    if (seq_fast) { seq = idx % nseq; q = idx / nseq; }
    else { q = idx % nb; seq = idx / nb; }
    const int b = q / sub, j = q - b * sub;
    cplx<T>* base = buf + (size_t)seq * ss + (size_t)(b * Lb + j) * es;
    cplx<T> v[R];
#pragma unroll
    for (int u = 0; u < R; ++u) v[u] = base[(size_t)u * sub * es];
    dft_small<T, INV, R>(v);
#pragma unroll
    for (int t = 1; t < R; ++t) {
      cplx<T> w = tw[tstride * j * t];
      if (INV) w = conjg(w);
      v[t] = v[t] * w;
    }
#pragma unroll
    for (int t = 0; t < R; ++t) base[(size_t)t * sub * es] = v[t];
  }
}

template <typename T, bool INV, int R>
__device__ __forceinline__ void dit_stage(cplx<T>* buf, int nseq, int es, int ss, int n, int Lb,
                                          const cplx<T>* tw, bool seq_fast) {
  const int sub = Lb / R;
  const int nb = n / R;
  const int total = nseq * nb;
  const int tstride = n / Lb;
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int seq, q;
    if (seq_fast) { seq = idx % nseq; q = idx / nseq; }
    else { q = idx % nb; seq = idx / nb; }
    const int b = q / sub, j = q - b * sub;
    cplx<T>* base = buf + (size_t)seq * ss + (size_t)(b * Lb + j) * es;
    cplx<T> v[R];
#pragma unroll
    for (int t = 0; t < R; ++t) v[t] = base[(size_t)t * sub * es];
#pragma unroll
    for (int t = 1; t < R; ++t) {
      cplx<T> w = tw[tstride * j * t];
      if (INV) w = conjg(w);
      v[t] = v[t] * w;
    }
    dft_small<T, INV, R>(v);
#pragma unroll
    for (int u = 0; u < R; ++u) base[(size_t)u * sub * es] = v[u];
  }
}

template <typename T, bool INV>
__device__ void generic_stage(cplx<T>* buf, int nseq, int es, int ss, int n, int Lb, int R,
                              const cplx<T>* tw, bool seq_fast, bool dit) {
  const int sub = Lb / R;
  const int nb = n / R;
  const int total = nseq * nb;
  const int tstride = n / Lb;
  cplx<T> v[32], o[32];
  for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
    int seq, q;
    if (seq_fast) { seq = idx % nseq; q = idx / nseq; }
    else { q = idx % nb; seq = idx / nb; }
    const int b = q / sub, j = q - b * sub;
    cplx<T>* base = buf + (size_t)seq * ss + (size_t)(b * Lb + j) * es;
    for (int u = 0; u < R; ++u) v[u] = base[(size_t)u * sub * es];
    if (dit) {
      for (int t = 1; t < R; ++t) {
        cplx<T> w = tw[tstride * j * t];
        if (INV) w = conjg(w);
        v[t] = v[t] * w;
      }
    }
    dft_generic<T, INV>(v, o, R, n, tw);
    if (!dit) {
      for (int t = 1; t < R; ++t) {
        cplx<T> w = tw[tstride * j * t];
        if (INV) w = conjg(w);
        o[t] = o[t] * w;
      }
    }
    for (int t = 0; t < R; ++t) base[(size_t)t * sub * es] = o[t];
  }
}

// In-place DIF: natural-order input -> digit-reversed spectrum.  All threads
// of the CTA must call it; it ends with __syncthreads().
template <typename T, bool INV>
__device__ void fft_dif(cplx<T>* buf, int nseq, int es, int ss, const FftPlan& pl, const cplx<T>* tw,
                        bool seq_fast) {
  int Lb = pl.n;
  for (int s = 0; s < pl.nst; ++s) {
    const int R = pl.r[s];
    switch (R) {
      case 2: dif_stage<T, INV, 2>(buf, nseq, es, ss, pl.n, Lb, tw, seq_fast); break;
      case 3: dif_stage<T, INV, 3>(buf, nseq, es, ss, pl.n, Lb, tw, seq_fast); break;
      case 4: dif_stage<T, INV, 4>(buf, nseq, es, ss, pl.n, Lb, tw, seq_fast); break;
      case 5: dif_stage<T, INV, 5>(buf, nseq, es, ss, pl.n, Lb, tw, seq_fast); break;
      case 7: dif_stage<T, INV, 7>(buf, nseq, es, ss, pl.n, Lb, tw, seq_fast); break;
      case 8: dif_stage<T, INV, 8>(buf, nseq, es, ss, pl.n, Lb, tw, seq_fast); break;
      default: generic_stage<T, INV>(buf, nseq, es, ss, pl.n, Lb, R, tw, seq_fast, false); break;
    }
    Lb /= R;
    __syncthreads();
  }
}

// In-place DIT: digit-reversed input -> natural-order output.
template <typename T, bool INV>
__device__ void fft_dit(cplx<T>* buf, int nseq, int es, int ss, const FftPlan& pl, const cplx<T>* tw,
                        bool seq_fast) {
  int Lb = 1;
  for (int s = pl.nst - 1; s >= 0; --s) {
    const int R = pl.r[s];
    Lb *= R;
    switch (R) {
      case 2: dit_stage<T, INV, 2>(buf, nseq, es, ss, pl.n, Lb, tw, seq_fast); break;
      case 3: dit_stage<T, INV, 3>(buf, nseq, es, ss, pl.n, Lb, tw, seq_fast); break;
      case 4: dit_stage<T, INV, 4>(buf, nseq, es, ss, pl.n, Lb, tw, seq_fast); break;
      case 5: dit_stage<T, INV, 5>(buf, nseq, es, ss, pl.n, Lb, tw, seq_fast); break;
      case 7: dit_stage<T, INV, 7>(buf, nseq, es, ss, pl.n, Lb, tw, seq_fast); break;
      case 8: dit_stage<T, INV, 8>(buf, nseq, es, ss, pl.n, Lb, tw, seq_fast); break;
      default: generic_stage<T, INV>(buf, nseq, es, ss, pl.n, Lb, R, tw, seq_fast, true); break;
    }
    __syncthreads();
  }
}

}  // namespace marie
