// Four-step (register-resident) FFT passes of the matvec for grid edges
// n = 16*NB, NB in [1, 8] (16, 32, ..., 128: every benchmark grid).
//
// A length-n transform is split n = 16 x NB (input index z = NB*a + b,
// output frequency k = k1 + 16*k2):
//   step 1 (per b): 16-point DFT over a in registers, twiddle w_n^(b*k1),
//   step 2 (per k1): NB-point DFT over b in registers,
// with one shared-memory exchange in between.  Inputs are loaded from HBM
// straight into registers and outputs stored from registers, so each pass
// makes one shared-memory round trip (the z pass four: forward, multiply,
// inverse), and every index is a shift or a multiply by a constant.
// Spectra are kept in natural frequency order: position k of half alpha holds
// frequency 2k + alpha.  Layouts in HBM are those of matvec.cuh.
#pragma once

#include "matvec.cuh"

namespace marie {

// cos/sin(2*pi*m/16), m in [0, 9]; cos/sin(2*pi*m/6), m in [0, 2]
__host__ __device__ constexpr double c16(int m) {
  return m == 0 ? 1.0 : m == 1 ? 0.923879532511286756128 : m == 2 ? 0.707106781186547524401
       : m == 3 ? 0.382683432365089771728 : m == 4 ? 0.0 : m == 5 ? -0.382683432365089771728
       : m == 6 ? -0.707106781186547524401 : m == 7 ? -0.923879532511286756128 : m == 8 ? -1.0
       : -0.923879532511286756128;
}
__host__ __device__ constexpr double s16(int m) {
  return m == 0 ? 0.0 : m == 1 ? 0.382683432365089771728 : m == 2 ? 0.707106781186547524401
       : m == 3 ? 0.923879532511286756128 : m == 4 ? 1.0 : m == 5 ? 0.923879532511286756128
       : m == 6 ? 0.707106781186547524401 : m == 7 ? 0.382683432365089771728 : m == 8 ? 0.0
       : -0.382683432365089771728;
}

// v * exp(-+ 2 pi i m / N) given cos and sin of 2 pi m / N (forward: minus)
template <typename T, bool INV>
__device__ __forceinline__ cplx<T> rot(cplx<T> v, double c, double s) {
  const T cc = (T)c, ss = INV ? (T)s : (T)-s;
  return {v.x * cc - v.y * ss, v.x * ss + v.y * cc};
}

template <typename T, bool INV>
__device__ __forceinline__ void dft16(cplx<T>* v) {
  cplx<T> A[16];
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    cplx<T> t[4] = {v[b], v[4 + b], v[8 + b], v[12 + b]};
    dft4<T, INV>(t);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) A[b * 4 + k1] = (b * k1 == 0) ? t[k1] : rot<T, INV>(t[k1], c16(b * k1), s16(b * k1));
  }
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    cplx<T> t[4] = {A[k1], A[4 + k1], A[8 + k1], A[12 + k1]};
    dft4<T, INV>(t);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[k2];
  }
}

template <typename T, bool INV>
__device__ __forceinline__ void dft6(cplx<T>* v) {
  const double h3 = 0.866025403784438646764;
  cplx<T> A[6];
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    cplx<T> t[2] = {v[b], v[3 + b]};
    dft2<T, INV>(t);
    A[b * 2 + 0] = t[0];
    A[b * 2 + 1] = b == 0 ? t[1] : (b == 1 ? rot<T, INV>(t[1], 0.5, h3) : rot<T, INV>(t[1], -0.5, h3));
  }
#pragma unroll
  for (int k1 = 0; k1 < 2; ++k1) {
    cplx<T> t[3] = {A[k1], A[2 + k1], A[4 + k1]};
    dft_prime<T, INV, 3>(t);
#pragma unroll
    for (int k2 = 0; k2 < 3; ++k2) v[k1 + 2 * k2] = t[k2];
  }
}

// Float-float DFTs run in packed (re, im) pairs (ffpair.cuh).
template <bool INV, int N>
__device__ __forceinline__ void dftn_ffc2(cplx<ff>* v);

template <typename T, bool INV, int N>
__device__ __forceinline__ void dftn(cplx<T>* v) {
  if constexpr (std::is_same<T, ff>::value && N > 1) {
    dftn_ffc2<INV, N>(v);
  } else if constexpr (N == 1) {
  } else if constexpr (N == 6) {
    dft6<T, INV>(v);
  } else if constexpr (N == 16) {
    dft16<T, INV>(v);
  } else {
    dft_small<T, INV, N>(v);
  }
}

// ---------------------------------------------------------------------------
// Pass X (forward), n1 = 16*NB.  grid (ceil(n2/TY), n3, nbundle*C)
// buf: sequence s = (yy*R + r)*2 + alpha, stride S = 16*NB + 1, [k1][b]
// ---------------------------------------------------------------------------
template <typename T, int NB>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) k4_fwd_x(MvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int N = 16 * NB, S = N + 1;
  const int bc = blockIdx.z, bu = bc / a.C, c = bc - bu * a.C;
  if (!bundle_active(a, bu)) return;
  const int z = blockIdx.y, y0 = blockIdx.x * a.TY;
  const int n2 = a.n2, n3 = a.n3, R = a.R, lgR = a.lgR;
  const int ty = min(a.TY, n2 - y0);
  bool any = false;
  for (int yy = 0; yy < ty; ++yy) any = any || row_is_live(a, y0 + yy, z);
  if (!any) return;   // rows without body voxels stay unwritten: the y pass reads them as zero
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + N;
  load_tw(tw, a.ax.tw, N);
  __syncthreads();
  const int64_t nD = (int64_t)N * n2 * n3;
  // step 1: task (yy, r, b), b fastest
  for (int t = threadIdx.x; t < ty * R * NB; t += blockDim.x) {
    const int b = t % NB, rr = t / NB;
    const int r = rr & (R - 1), yy = rr >> lgR;
    if (!row_is_live(a, y0 + yy, z)) continue;
    const int rhs = bu * R + r;
    const bool act = lane_active(a, rhs);
    const auto* in = a.in + (int64_t)rhs * a.in_rs;
    const int64_t grow = (int64_t)N * (y0 + yy + (int64_t)n2 * z);
    cplx<T> v[16], u[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int x = NB * q + b;
      cplx<T> val = {0, 0};
      if (act) {
        if (a.mode == MV_GRID) {
          val = io_load<T>(in[(int64_t)c * nD + grow + x]);
        } else {
          const int s = a.vox2sol[grow + x];
          if (s >= 0) {
            val = io_load<T>(in[(int64_t)c * a.Ns + s]);
            if (a.mode == MV_VIE_ADJ) val = scale(mulc(val, a.chi[s]), a.invg[c]);
            else if (a.mode == MV_HFIELD_ADJ) val = scale(val, a.invg[c]);
          }
        }
      }
      v[q] = val;
      u[q] = val;
    }
    cplx<T>* dst0 = buf + ((yy * R + r) * 2) * S + b;
    dftn<T, false, 16>(u);
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) dst0[k1 * NB] = u[k1] * tw[b * k1];
#pragma unroll
    for (int q = 0; q < 16; ++q) u[q] = v[q] * a.ax.tw2[NB * q + b];
    dftn<T, false, 16>(u);
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) dst0[S + k1 * NB] = u[k1] * tw[b * k1];
  }
  __syncthreads();
  // step 2: task (yy, alpha, k1, r), r fastest; output row [kx' = alpha*N + k][r]
  const int rowlen = 2 * N * R;
  cplx<T>* dst = a.T1 + (((int64_t)bu * a.C + c) * n3 + z) * (int64_t)n2 * rowlen;
  for (int t = threadIdx.x; t < ty * 32 * R; t += blockDim.x) {
    const int r = t & (R - 1), q = t >> lgR;
    const int k1 = q & 15, alpha = (q >> 4) & 1, yy = q >> 5;
    if (!row_is_live(a, y0 + yy, z)) continue;
    const cplx<T>* src = buf + ((yy * R + r) * 2 + alpha) * S + k1 * NB;
    cplx<T> w[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) w[b] = src[b];
    dftn<T, false, NB>(w);
    cplx<T>* o = dst + (int64_t)(y0 + yy) * rowlen + (alpha * N + k1) * R + r;
#pragma unroll
    for (int k2 = 0; k2 < NB; ++k2) o[16 * k2 * R] = w[k2];
  }
}

// ---------------------------------------------------------------------------
// Pass XI (inverse x + crop + epilogue), n1 = 16*NB.
// ---------------------------------------------------------------------------
template <typename T, int NB>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) k4_inv_x(MvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int N = 16 * NB, S = N + 1;
  const int bc = blockIdx.z, bu = bc / a.C, c = bc - bu * a.C;
  if (!bundle_active(a, bu)) return;
  const int z = blockIdx.y, y0 = blockIdx.x * a.TY;
  const int n2 = a.n2, n3 = a.n3, R = a.R, lgR = a.lgR;
  const int ty = min(a.TY, n2 - y0);
  bool any = false;
  for (int yy = 0; yy < ty; ++yy) any = any || row_is_live(a, y0 + yy, z);
  if (!any) return;   // no body voxel in these rows: no output
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + N;
  load_tw(tw, a.ax.tw, N);
  __syncthreads();
  const int rowlen = 2 * N * R;
  const cplx<T>* srow = a.T1 + (((int64_t)bu * a.C + c) * n3 + z) * (int64_t)n2 * rowlen;
  // step A: task (yy, alpha, k1, r): inverse NB-point DFT over k2, twiddle
  for (int t = threadIdx.x; t < ty * 32 * R; t += blockDim.x) {
    const int r = t & (R - 1), q = t >> lgR;
    const int k1 = q & 15, alpha = (q >> 4) & 1, yy = q >> 5;
    if (!row_is_live(a, y0 + yy, z)) continue;
    const cplx<T>* in = srow + (int64_t)(y0 + yy) * rowlen + (alpha * N + k1) * R + r;
    cplx<T> w[NB];
#pragma unroll
    for (int k2 = 0; k2 < NB; ++k2) w[k2] = in[16 * k2 * R];
    dftn<T, true, NB>(w);
    cplx<T>* d = buf + ((yy * R + r) * 2 + alpha) * S + k1 * NB;
#pragma unroll
    for (int b = 0; b < NB; ++b) d[b] = mulc(w[b], tw[b * k1]);
  }
  __syncthreads();
  // step B: task (yy, r, b): inverse 16-point DFTs of both halves, combine, epilogue
  const int64_t nD = (int64_t)N * n2 * n3;
  for (int t = threadIdx.x; t < ty * R * NB; t += blockDim.x) {
    const int b = t % NB, rr = t / NB;
    const int r = rr & (R - 1), yy = rr >> lgR;
    const int rhs = bu * R + r;
    if (!lane_active(a, rhs) || !row_is_live(a, y0 + yy, z)) continue;
    const cplx<T>* s0 = buf + ((yy * R + r) * 2) * S + b;
    cplx<T> u0[16], u1[16];
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) {
      u0[k1] = s0[k1 * NB];
      u1[k1] = s0[S + k1 * NB];
    }
    dftn<T, true, 16>(u0);
    dftn<T, true, 16>(u1);
    const int64_t grow = (int64_t)N * (y0 + yy + (int64_t)n2 * z);
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int x = NB * q + b;
      cplx<T> v = u0[q] + mulc(u1[q], a.ax.tw2[x]);
      if (a.mode == MV_GRID) {
        a.out[(int64_t)rhs * a.out_rs + (int64_t)c * nD + grow + x] = io_store(v);
      } else {
        const int s = a.vox2sol[grow + x];
        if (s >= 0) body_store(a, c, s, rhs, v);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Pass Y (forward), n2 = 16*NB.  grid (ceil(2n1/TXY), n3, nbundle*C)
// buf: sequence s = beta*W + e, stride S, [k1][b]
// ---------------------------------------------------------------------------
template <typename T, int NB>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) k4_fwd_y(MvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int N = 16 * NB, S = N + 1;
  const int bc = blockIdx.z, bu = bc / a.C, c = bc - bu * a.C;
  if (!bundle_active(a, bu)) return;
  const int z = blockIdx.y, k0 = blockIdx.x * a.TXY;
  if (!z_is_live(a, z)) return;   // slice without body voxels: the z pass reads it as zero
  const int n1 = a.n1, n3 = a.n3, m1 = 2 * n1, R = a.R;
  const int W = a.TXY * R, wl = min(a.TXY, m1 - k0) * R;
  const int lgW = 31 - __clz(W);   // TXY*R is a power of two
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + N;
  load_tw(tw, a.ay.tw, N);
  __syncthreads();
  const int64_t row = (int64_t)m1 * R;
  const cplx<T>* src = a.T1 + (((int64_t)bu * a.C + c) * n3 + z) * (int64_t)N * row + (int64_t)k0 * R;
  // step 1: task (b, e), e fastest
  for (int t = threadIdx.x; t < W * NB; t += blockDim.x) {
    const int e = t & (W - 1), b = t >> lgW;
    const unsigned live = a.rowq ? a.rowq[z * 8 + b] : 0xffffu;   // rows y = NB*q + b
    cplx<T> v[16], u[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const cplx<T> val =
          (e < wl && ((live >> q) & 1u)) ? src[(int64_t)(NB * q + b) * row + e] : cplx<T>{0, 0};
      v[q] = val;
      u[q] = val;
    }
    dftn<T, false, 16>(u);
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) buf[e * S + k1 * NB + b] = u[k1] * tw[b * k1];
#pragma unroll
    for (int q = 0; q < 16; ++q) u[q] = v[q] * a.ay.tw2[NB * q + b];
    dftn<T, false, 16>(u);
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) buf[(W + e) * S + k1 * NB + b] = u[k1] * tw[b * k1];
  }
  __syncthreads();
  // step 2: task (beta, k1, e), e fastest; S_glob[bu][c][beta*N + k][z][kx'][r]
  cplx<T>* dst = a.S + ((int64_t)bu * a.C + c) * (int64_t)2 * N * n3 * row + (int64_t)k0 * R;
  for (int t = threadIdx.x; t < 2 * 16 * W; t += blockDim.x) {
    const int e = t & (W - 1), q = t >> lgW;
    const int k1 = q & 15, beta = q >> 4;
    cplx<T> w[NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) w[b] = buf[(beta * W + e) * S + k1 * NB + b];
    dftn<T, false, NB>(w);
    if (e < wl) {
#pragma unroll
      for (int k2 = 0; k2 < NB; ++k2) dst[((int64_t)(beta * N + k1 + 16 * k2) * n3 + z) * row + e] = w[k2];
    }
  }
}

// ---------------------------------------------------------------------------
// Pass YI (inverse y + crop), n2 = 16*NB.
// ---------------------------------------------------------------------------
template <typename T, int NB>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) k4_inv_y(MvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int N = 16 * NB, S = N + 1;
  const int bc = blockIdx.z, bu = bc / a.C, c = bc - bu * a.C;
  if (!bundle_active(a, bu)) return;
  const int z = blockIdx.y, k0 = blockIdx.x * a.TXY;
  if (!z_is_live(a, z)) return;   // no body voxel in slice z: no output
  const int n1 = a.n1, n3 = a.n3, m1 = 2 * n1, R = a.R;
  const int W = a.TXY * R, wl = min(a.TXY, m1 - k0) * R;
  const int lgW = 31 - __clz(W);   // TXY*R is a power of two
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + N;
  load_tw(tw, a.ay.tw, N);
  __syncthreads();
  const int64_t row = (int64_t)m1 * R;
  const cplx<T>* src = a.S + ((int64_t)bu * a.C + c) * (int64_t)2 * N * n3 * row + (int64_t)k0 * R;
  // step A: task (beta, k1, e)
  for (int t = threadIdx.x; t < 2 * 16 * W; t += blockDim.x) {
    const int e = t & (W - 1), q = t >> lgW;
    const int k1 = q & 15, beta = q >> 4;
    cplx<T> w[NB];
#pragma unroll
    for (int k2 = 0; k2 < NB; ++k2)
      w[k2] = e < wl ? src[((int64_t)(beta * N + k1 + 16 * k2) * n3 + z) * row + e] : cplx<T>{0, 0};
    dftn<T, true, NB>(w);
#pragma unroll
    for (int b = 0; b < NB; ++b) buf[(beta * W + e) * S + k1 * NB + b] = mulc(w[b], tw[b * k1]);
  }
  __syncthreads();
  // step B: task (b, e): inverse 16-point DFTs of both halves, combine, store
  cplx<T>* dst = a.T1 + (((int64_t)bu * a.C + c) * n3 + z) * (int64_t)N * row + (int64_t)k0 * R;
  for (int t = threadIdx.x; t < W * NB; t += blockDim.x) {
    const int e = t & (W - 1), b = t >> lgW;
    const unsigned live = a.rowq ? a.rowq[z * 8 + b] : 0xffffu;   // rows y = NB*q + b
    cplx<T> u0[16], u1[16];
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) {
      u0[k1] = buf[e * S + k1 * NB + b];
      u1[k1] = buf[(W + e) * S + k1 * NB + b];
    }
    dftn<T, true, 16>(u0);
    dftn<T, true, 16>(u1);
    if (e < wl) {
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int y = NB * q + b;
        if ((live >> q) & 1u) dst[(int64_t)y * row + e] = u0[q] + mulc(u1[q], a.ay.tw2[y]);
      }
    }
  }
}

}  // namespace marie

#include "kz4.cuh"
#include "kz4p.cuh"
#include "kz4f.cuh"
