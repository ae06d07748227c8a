// Batched restarted GMRES for the VIE operator.
//
// One Krylov space per right-hand side (the reference solves ports one at a
// time, ie_solver_vie.m:16-21); all right-hand sides of a batch advance in
// lock-step through the Arnoldi loop and a converged one simply drops out of
// the active mask until the cycle ends.  Per cycle the arithmetic is that of
// is_iter_gmres_vie.m:10-38: classical Gram-Schmidt in a single pass
// (h = V^H w; w -= V h; h_{k+1,k} = ||w||), the (k+1) x k least-squares problem
// for the residual estimate at every k, x += V y and r = V (beta e1 - H y) at
// the end of a cycle.  The least-squares problem is solved by Givens rotations
// in FP64 (same minimiser and residual norm as MATLAB's H \ rhs).
//
// Reductions are deterministic: per-CTA partials (warp shuffles + shared
// memory), then a fixed-order FP64 sum over CTAs.
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"

namespace marie {

constexpr int kMaxRestart = 128;  // largest GMRES restart length


typedef cplx<double> zd;
constexpr int kVT = 256;          // threads per vector CTA
constexpr int kVE = 8;            // elements per thread
constexpr int kCH = kVT * kVE;    // elements per chunk

enum RhsState : int { ST_ACTIVE = 0, ST_DONE = 1, ST_MAXIT = 2, ST_NONFINITE = 3 };

template <typename T>
__device__ __forceinline__ zd to_zd(cplx<T> v) { return zd{(double)v.x, (double)v.y}; }

// Block-wide sum of a complex value held by every thread; result valid in thread 0.
template <typename A>
__device__ __forceinline__ cplx<A> block_sum(cplx<A> v, cplx<A>* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  cplx<A> r = {0, 0};
  if (threadIdx.x < 32) {
    r = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : cplx<A>{0, 0};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      r.x += __shfl_xor_sync(0xffffffffu, r.x, o);
      r.y += __shfl_xor_sync(0xffffffffu, r.y, o);
    }
  }
  __syncthreads();
  return r;
}

// Accumulator type: FP32 for complex64 vectors, FP64 for complex128.
template <typename T>
struct Acc { typedef T type; };

// part[(r*(m+1) + j)*nch + chunk] = sum_i conj(V_j[i]) w[i], j in [0, k]
template <typename T>
__global__ void k_dots(const cplx<T>* V, int64_t ld, int64_t Nb, int k, int mp1, const unsigned char* act,
                       zd* part, int nch) {
  typedef typename Acc<T>::type A;
  __shared__ cplx<A> sh[32];
  const int r = blockIdx.y;
  if (!act[r]) return;
  const int chunk = blockIdx.x;
  const cplx<T>* base = V + (int64_t)r * mp1 * ld;
  const cplx<T>* w = base + (int64_t)(k + 1) * ld;
  cplx<T> wv[kVE];
  const int64_t i0 = (int64_t)chunk * kCH + threadIdx.x;
#pragma unroll
  for (int e = 0; e < kVE; ++e) {
    const int64_t i = i0 + (int64_t)e * kVT;
    wv[e] = i < Nb ? w[i] : cplx<T>{0, 0};
  }
  for (int j = 0; j <= k; ++j) {
    const cplx<T>* vj = base + (int64_t)j * ld;
    cplx<A> acc = {0, 0};
#pragma unroll
    for (int e = 0; e < kVE; ++e) {
      const int64_t i = i0 + (int64_t)e * kVT;
      if (i < Nb) {
        const cplx<T> v = vj[i];
        acc.x += (A)v.x * (A)wv[e].x + (A)v.y * (A)wv[e].y;
        acc.y += (A)v.x * (A)wv[e].y - (A)v.y * (A)wv[e].x;
      }
    }
    cplx<A> s = block_sum(acc, sh);
    if (threadIdx.x == 0) part[((int64_t)r * mp1 + j) * nch + chunk] = zd{(double)s.x, (double)s.y};
  }
}

// Deterministic warp sum of per-CTA partials: lane l adds chunks l, l+32, ...
// in order, then a fixed butterfly tree.
__device__ __forceinline__ zd warp_sum_partials(const zd* p, int nch) {
  const int lane = threadIdx.x & 31;
  double sx = 0, sy = 0;
  for (int c = lane; c < nch; c += 32) { sx += p[c].x; sy += p[c].y; }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, o);
    sy += __shfl_xor_sync(0xffffffffu, sy, o);
  }
  return zd{sx, sy};
}

// H[r][j + (m+1) k] = sum_chunk part, j in [0,k]; one warp per (rhs, j).
// grid (ceil((k+1)/8), nrhs), 256 threads.
__global__ void k_reduce_dots(const zd* part, int nch, int k, int mp1, int m, const unsigned char* act, zd* H) {
  const int r = blockIdx.y;
  if (!act[r]) return;
  const int j = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (j > k) return;
  const zd s = warp_sum_partials(part + ((int64_t)r * mp1 + j) * nch, nch);
  if ((threadIdx.x & 31) == 0) H[(int64_t)r * mp1 * m + j + (int64_t)mp1 * k] = s;
}

// w -= sum_j V_j h_j ; npart[r*nch + chunk] = ||w_chunk||^2
template <typename T>
__global__ void k_update(cplx<T>* V, int64_t ld, int64_t Nb, int k, int mp1, int m, const unsigned char* act,
                         const zd* H, double* npart, int nch) {
  typedef typename Acc<T>::type A;
  __shared__ cplx<T> hs[kMaxRestart];
  __shared__ cplx<A> sh[32];
  const int r = blockIdx.y;
  if (!act[r]) return;
  const int chunk = blockIdx.x;
  for (int j = threadIdx.x; j <= k; j += blockDim.x) {
    const zd hv = H[(int64_t)r * mp1 * m + j + (int64_t)mp1 * k];
    hs[j] = cplx<T>{(T)hv.x, (T)hv.y};
  }
  __syncthreads();
  cplx<T>* base = V + (int64_t)r * mp1 * ld;
  cplx<T>* w = base + (int64_t)(k + 1) * ld;
  const int64_t i0 = (int64_t)chunk * kCH + threadIdx.x;
  cplx<T> wv[kVE];
#pragma unroll
  for (int e = 0; e < kVE; ++e) {
    const int64_t i = i0 + (int64_t)e * kVT;
    wv[e] = i < Nb ? w[i] : cplx<T>{0, 0};
  }
  for (int j = 0; j <= k; ++j) {
    const cplx<T>* vj = base + (int64_t)j * ld;
    const cplx<T> hj = hs[j];
#pragma unroll
    for (int e = 0; e < kVE; ++e) {
      const int64_t i = i0 + (int64_t)e * kVT;
      if (i < Nb) {
        const cplx<T> v = vj[i];
        wv[e].x -= v.x * hj.x - v.y * hj.y;
        wv[e].y -= v.x * hj.y + v.y * hj.x;
      }
    }
  }
  A nrm = 0;
#pragma unroll
  for (int e = 0; e < kVE; ++e) {
    const int64_t i = i0 + (int64_t)e * kVT;
    if (i < Nb) {
      w[i] = wv[e];
      nrm += (A)wv[e].x * (A)wv[e].x + (A)wv[e].y * (A)wv[e].y;
    }
  }
  cplx<A> s = block_sum(cplx<A>{nrm, 0}, sh);
  if (threadIdx.x == 0) npart[(int64_t)r * nch + chunk] = (double)s.x;
}

// npart[r*nch + chunk] = ||v_r chunk||^2 for v_r = base + r*rs
template <typename T>
__global__ void k_norm2(const cplx<T>* v, int64_t rs, int64_t Nb, const unsigned char* act, double* npart, int nch) {
  typedef typename Acc<T>::type A;
  __shared__ cplx<A> sh[32];
  const int r = blockIdx.y;
  if (act && !act[r]) return;
  const cplx<T>* p = v + (int64_t)r * rs;
  const int64_t i0 = (int64_t)blockIdx.x * kCH + threadIdx.x;
  A nrm = 0;
#pragma unroll
  for (int e = 0; e < kVE; ++e) {
    const int64_t i = i0 + (int64_t)e * kVT;
    if (i < Nb) {
      const cplx<T> x = p[i];
      nrm += (A)x.x * (A)x.x + (A)x.y * (A)x.y;
    }
  }
  cplx<A> s = block_sum(cplx<A>{nrm, 0}, sh);
  if (threadIdx.x == 0) npart[(int64_t)r * nch + blockIdx.x] = (double)s.x;
}

// out[r] = sqrt(sum_chunk npart); one warp per rhs, grid (ceil(nrhs/8)), 256 threads.
__global__ void k_reduce_norm(const double* npart, int nch, int nrhs, const unsigned char* act, double* out) {
  const int r = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (r >= nrhs || (act && !act[r])) return;
  const int lane = threadIdx.x & 31;
  const double* p = npart + (int64_t)r * nch;
  double s = 0;
  for (int c = lane; c < nch; c += 32) s += p[c];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[r] = sqrt(s);
}

// v_r *= 1/s_r  (zero when s_r == 0)
template <typename T>
__global__ void k_scale(cplx<T>* v, int64_t rs, int64_t Nb, const unsigned char* act, const double* s) {
  const int r = blockIdx.y;
  if (!act[r]) return;
  const double sv = s[r];
  const T inv = sv > 0 ? (T)(1.0 / sv) : (T)0;
  cplx<T>* p = v + (int64_t)r * rs;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nb; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = scale(p[i], inv);
}

struct GmState {
  zd* H;          // [nrhs][(m+1)*m]   Hessenberg (original)
  zd* R;          // [nrhs][(m+1)*m]   rotated copy
  double* cs;     // [nrhs][m]
  zd* sn;         // [nrhs][m]
  zd* g;          // [nrhs][m+1]
  zd* y;          // [nrhs][m]
  zd* res;        // [nrhs][m+1]
  double* beta;   // [nrhs]
  double* hnorm;  // [nrhs]   h_{k+1,k}
  double* resid;  // [nrhs]   |g_{k+1}|
  double* tolabs; // [nrhs]
  int* kr;        // [nrhs]   Arnoldi steps in the current cycle
  double* hist;   // [nrhs][m] |g_{k+1}| after step k of the current cycle
  unsigned char* incyc;  // [nrhs] in the Arnoldi loop of the current cycle
  zd* part;       // [nrhs][m+1][nch]
  double* npart;  // [nrhs][nch]
};

// Givens step for column k (one thread per rhs).  Sets incyc=0 when the cycle
// ends (converged, breakdown, k+1 == m or non-finite).
__global__ void k_givens(GmState st, int k, int m, int nrhs) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrhs || !st.incyc[r]) return;
  const int mp1 = m + 1;
  zd* H = st.H + (int64_t)r * mp1 * m;
  zd* R = st.R + (int64_t)r * mp1 * m;
  double* cs = st.cs + (int64_t)r * m;
  zd* sn = st.sn + (int64_t)r * m;
  zd* g = st.g + (int64_t)r * mp1;
  const double hk1 = st.hnorm[r];
  H[k + 1 + mp1 * k] = zd{hk1, 0};
  for (int i = 0; i <= k; ++i) R[i + mp1 * k] = H[i + mp1 * k];
  R[k + 1 + mp1 * k] = zd{hk1, 0};
  for (int i = 0; i < k; ++i) {
    const zd a = R[i + mp1 * k], b = R[i + 1 + mp1 * k];
    const double c = cs[i];
    const zd s = sn[i];
    R[i + mp1 * k] = zd{c * a.x + (s.x * b.x - s.y * b.y), c * a.y + (s.x * b.y + s.y * b.x)};
    // -conj(s)*a + c*b
    R[i + 1 + mp1 * k] = zd{-(s.x * a.x + s.y * a.y) + c * b.x, -(s.x * a.y - s.y * a.x) + c * b.y};
  }
  const zd a = R[k + mp1 * k];
  const double b = hk1;
  const double na = sqrt(a.x * a.x + a.y * a.y);
  double c;
  zd s;
  if (na == 0.0) {
    c = 0.0;
    s = zd{1.0, 0.0};
  } else {
    const double t = sqrt(na * na + b * b);
    c = na / t;
    s = zd{a.x / na * b / t, a.y / na * b / t};
  }
  cs[k] = c;
  sn[k] = s;
  R[k + mp1 * k] = zd{c * a.x + s.x * b, c * a.y + s.y * b};
  R[k + 1 + mp1 * k] = zd{0, 0};
  const zd gk = g[k];
  g[k + 1] = zd{-(s.x * gk.x + s.y * gk.y), -(s.x * gk.y - s.y * gk.x)};
  g[k] = zd{c * gk.x, c * gk.y};
  const double res = sqrt(g[k + 1].x * g[k + 1].x + g[k + 1].y * g[k + 1].y);
  st.resid[r] = res;
  st.hist[(int64_t)r * m + k] = res;
  st.kr[r] = k + 1;
  if (!isfinite(res) || !isfinite(hk1)) {
    st.incyc[r] = 0;
    return;
  }
  if (res < st.tolabs[r] || k + 1 == m || hk1 == 0.0) st.incyc[r] = 0;
}

// y = R^{-1} g (k x k), res = beta e1 - H y ((k+1) entries); one thread per rhs.
__global__ void k_solve_y(GmState st, int m, int nrhs, const unsigned char* ran) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrhs || !ran[r]) return;
  const int k = st.kr[r];
  const int mp1 = m + 1;
  const zd* H = st.H + (int64_t)r * mp1 * m;
  const zd* R = st.R + (int64_t)r * mp1 * m;
  const zd* g = st.g + (int64_t)r * mp1;
  zd* y = st.y + (int64_t)r * m;
  zd* res = st.res + (int64_t)r * mp1;
  for (int i = k - 1; i >= 0; --i) {
    zd acc = g[i];
    for (int j = i + 1; j < k; ++j) acc = acc - R[i + mp1 * j] * y[j];
    const zd d = R[i + mp1 * i];
    const double dd = d.x * d.x + d.y * d.y;
    y[i] = dd > 0 ? zd{(acc.x * d.x + acc.y * d.y) / dd, (acc.y * d.x - acc.x * d.y) / dd} : zd{0, 0};
  }
  for (int i = 0; i <= k; ++i) {
    zd acc = i == 0 ? zd{st.beta[r], 0} : zd{0, 0};
    for (int j = 0; j < k; ++j) acc = acc - H[i + mp1 * j] * y[j];
    res[i] = acc;
  }
}

// x_r += sum_{j<k_r} V_j y_j   (x in FP64)
template <typename T>
__global__ void k_xupdate(const cplx<T>* V, int64_t ld, int mp1, int m, int64_t Nb, const unsigned char* ran,
                          GmState st, zd* x, int64_t xrs) {
  const int r = blockIdx.y;
  if (!ran[r]) return;
  const int k = st.kr[r];
  const zd* y = st.y + (int64_t)r * m;
  const cplx<T>* base = V + (int64_t)r * mp1 * ld;
  zd* xr = x + (int64_t)r * xrs;
  if constexpr (std::is_same<T, float>::value) {
    // complex64 basis: the combination in FP32 (the basis' own precision;
    // FP64 arithmetic runs at 1/64 of the FP32 rate here), added to x in FP64
    __shared__ cplx<float> yf[kMaxRestart];
    for (int j = threadIdx.x; j < k; j += blockDim.x) yf[j] = cplx<float>{(float)y[j].x, (float)y[j].y};
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nb; i += (int64_t)gridDim.x * blockDim.x) {
      cplx<float> acc = {0, 0};
      for (int j = 0; j < k; ++j) fma_c(acc, base[(int64_t)j * ld + i], yf[j]);
      xr[i] = xr[i] + zd{(double)acc.x, (double)acc.y};
    }
  } else {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nb; i += (int64_t)gridDim.x * blockDim.x) {
      zd acc = xr[i];
      for (int j = 0; j < k; ++j) acc = acc + to_zd(base[(int64_t)j * ld + i]) * y[j];
      xr[i] = acc;
    }
  }
}

// V_0 <- sum_{j<=k_r} V_j res_j  (the next cycle's residual, is_iter_gmres_vie.m:38)
template <typename T>
__global__ void k_rform(cplx<T>* V, int64_t ld, int mp1, int64_t Nb, const unsigned char* ran, GmState st) {
  const int r = blockIdx.y;
  if (!ran[r]) return;
  const int k = st.kr[r];
  const zd* res = st.res + (int64_t)r * mp1;
  cplx<T>* base = V + (int64_t)r * mp1 * ld;
  if constexpr (std::is_same<T, float>::value) {
    __shared__ cplx<float> rf[kMaxRestart + 1];
    for (int j = threadIdx.x; j <= k; j += blockDim.x) rf[j] = cplx<float>{(float)res[j].x, (float)res[j].y};
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nb; i += (int64_t)gridDim.x * blockDim.x) {
      cplx<float> acc = {0, 0};
      for (int j = 0; j <= k; ++j) fma_c(acc, base[(int64_t)j * ld + i], rf[j]);
      base[i] = acc;
    }
  } else {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nb; i += (int64_t)gridDim.x * blockDim.x) {
      zd acc = {0, 0};
      for (int j = 0; j <= k; ++j) acc = acc + to_zd(base[(int64_t)j * ld + i]) * res[j];
      base[i] = cplx<T>{(T)acc.x, (T)acc.y};
    }
  }
}

// Start a cycle: g = [beta, 0...]; V_0 /= beta.
__global__ void k_cycle_init(GmState st, int m, int nrhs, const unsigned char* start) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrhs || !start[r]) return;
  zd* g = st.g + (int64_t)r * (m + 1);
  for (int i = 0; i <= m; ++i) g[i] = zd{0, 0};
  g[0] = zd{st.beta[r], 0};
  st.kr[r] = 0;
  st.incyc[r] = 1;
}

// dst_r = (Tout) src_r
template <typename Ti, typename To>
__global__ void k_convert(const cplx<Ti>* src, int64_t srs, cplx<To>* dst, int64_t drs, int64_t Nb,
                          const unsigned char* act) {
  const int r = blockIdx.y;
  if (act && !act[r]) return;
  const cplx<Ti>* s = src + (int64_t)r * srs;
  cplx<To>* d = dst + (int64_t)r * drs;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nb; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = cplx<To>{(To)s[i].x, (To)s[i].y};
}

// r = b - r  (r holds A x on entry); FP64
__global__ void k_residual(const zd* b, zd* r, int64_t Nb, const unsigned char* act) {
  const int k = blockIdx.y;
  if (act && !act[k]) return;
  const zd* bb = b + (int64_t)k * Nb;
  zd* rr = r + (int64_t)k * Nb;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nb; i += (int64_t)gridDim.x * blockDim.x)
    rr[i] = bb[i] - rr[i];
}

__global__ void k_zero(zd* x, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = zd{0, 0};
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

// Workspace of one solve, served from the handle's pool: the k-th request
// of a solve reuses the pool's k-th buffer when it is large enough (solves
// with the same shape request the same sequence), else replaces it.
struct Scratch {
  marie_vie* h;
  std::vector<std::pair<void*, size_t>>* pool;
  size_t next = 0;
  bool adjoint = false;   // the solve's operator is A^H (mvp_vie's Hermitian adjoint)
  explicit Scratch(marie_vie* hh) : h(hh), pool(&hh->gm_pool) {}
  Scratch(marie_vie* hh, std::vector<std::pair<void*, size_t>>* p) : h(hh), pool(p) {}
  template <typename P>
  marie_status get(P** p, size_t count) {
    *p = nullptr;
    const size_t bytes = std::max<size_t>(count, 1) * sizeof(P);
    std::vector<std::pair<void*, size_t>>& pl = *pool;
    if (next < pl.size() && pl[next].second >= bytes) {
      *p = (P*)pl[next++].first;
      return MARIE_OK;
    }
    if (next < pl.size()) {     // too small: replace
      cudaFree(pl[next].first);
      h->mem_used -= (int64_t)pl[next].second;
      pl[next] = {nullptr, 0};
    }
    if (h->mem_cap > 0 && h->mem_used + (int64_t)bytes > h->mem_cap) {
      set_error("device memory cap exceeded by GMRES workspace (%zu bytes)", bytes);
      return MARIE_ERR_OOM;
    }
    void* q = nullptr;
    if (cudaMalloc(&q, bytes) != cudaSuccess) {
      cudaGetLastError();
      set_error("GMRES workspace allocation of %zu bytes failed", bytes);
      return MARIE_ERR_OOM;
    }
    h->mem_used += (int64_t)bytes;
    if (next < pl.size()) pl[next] = {q, bytes};
    else pl.push_back({q, bytes});
    ++next;
    *p = (P*)q;
    return MARIE_OK;
  }
};

// ---------------------------------------------------------------------------
// Status channel.  The solver's small host<->device transfers (residual norms,
// active masks, per-rhs counters; a few hundred bytes, several per Arnoldi
// step) go through pinned, device-mapped host memory moved by k_bytes rather
// than through cudaMemcpyAsync: the host-buffer solve keeps the copy engines
// busy with chunk copies, and a small copy queued behind one stalls the
// solve for the chunk copy's duration.  Slot i of 16*nrhs bytes serves one
// transfer; a slot is rewritten by the host only after a stream
// synchronisation that follows the previous kernel reading it.
// ---------------------------------------------------------------------------
enum ChanSlot { SLOT_TOLABS, SLOT_MASK, SLOT_BETA, SLOT_INCYC, SLOT_RESID, SLOT_KR, SLOT_TODO, SLOT_NORM, kSlots };

__global__ void k_bytes(const unsigned char* __restrict__ src, unsigned char* __restrict__ dst, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[i];
}

// Behind the slots: a region of kMaxRestart doubles per rhs for the residual
// history of the Arnoldi steps between two host synchronisations.
static marie_status chan_reserve(marie_vie* h, int nrhs) {
  const size_t need = (size_t)(kSlots * 16 + kMaxRestart * 8) * std::max(nrhs, 1);
  if (h->hio_cap >= need) return MARIE_OK;
  if (h->hio) cudaFreeHost(h->hio);
  h->hio = nullptr;
  h->hio_cap = 0;
  void* p = nullptr;
  if (cudaHostAlloc(&p, need, cudaHostAllocMapped) != cudaSuccess) {
    cudaGetLastError();
    set_error("pinned status buffer allocation of %zu bytes failed", need);
    return MARIE_ERR_OOM;
  }
  h->hio = (unsigned char*)p;
  h->hio_cap = need;
  return MARIE_OK;
}
static unsigned char* chan_slot(marie_vie* h, int slot, int nrhs) {
  return h->hio + (size_t)slot * 16 * std::max(nrhs, 1);
}
// host -> device through the slot
static marie_status chan_put(marie_vie* h, int slot, int nrhs, void* dst, const void* src, size_t bytes,
                             cudaStream_t s) {
  MARIE_TRY(chan_reserve(h, nrhs));
  unsigned char* q = chan_slot(h, slot, nrhs);
  memcpy(q, src, bytes);
  unsigned char* qd = nullptr;
  MARIE_CUDA_TRY(cudaHostGetDevicePointer((void**)&qd, q, 0));
  k_bytes<<<1, 256, 0, s>>>(qd, (unsigned char*)dst, (int)bytes);
  MARIE_LAUNCH_CHECK();
  return MARIE_OK;
}
// device -> slot (read it with chan_take after synchronising the stream)
static marie_status chan_get(marie_vie* h, int slot, int nrhs, const void* src, size_t bytes, cudaStream_t s) {
  MARIE_TRY(chan_reserve(h, nrhs));
  unsigned char* qd = nullptr;
  MARIE_CUDA_TRY(cudaHostGetDevicePointer((void**)&qd, chan_slot(h, slot, nrhs), 0));
  k_bytes<<<1, 256, 0, s>>>((const unsigned char*)src, qd, (int)bytes);
  MARIE_LAUNCH_CHECK();
  return MARIE_OK;
}
static void chan_take(marie_vie* h, int slot, int nrhs, void* dst, size_t bytes) {
  memcpy(dst, chan_slot(h, slot, nrhs), bytes);
}
static unsigned char* chan_hist(marie_vie* h, int nrhs) { return chan_slot(h, kSlots, nrhs); }
static marie_status chan_get_hist(marie_vie* h, int nrhs, const double* src, size_t bytes, cudaStream_t s) {
  MARIE_TRY(chan_reserve(h, nrhs));
  unsigned char* qd = nullptr;
  MARIE_CUDA_TRY(cudaHostGetDevicePointer((void**)&qd, chan_hist(h, nrhs), 0));
  k_bytes<<<8, 256, 0, s>>>((const unsigned char*)src, qd, (int)bytes);
  MARIE_LAUNCH_CHECK();
  return MARIE_OK;
}

// Arnoldi steps between host synchronisations (MARIE_SYNC_STEPS, default 8):
// the device masks stop the work of right-hand sides that leave the cycle,
// the host reads their residual history at each synchronisation.
static int sync_steps() {
  static const int v = [] {
    const char* e = getenv("MARIE_SYNC_STEPS");
    const int n = e ? atoi(e) : 0;
    return n >= 1 ? n : 8;
  }();
  return v;
}

static dim3 vgrid(int64_t Nb, int nrhs) {
  int64_t bx = (Nb + 255) / 256;
  if (bx > 4096) bx = 4096;
  return dim3((unsigned)bx, (unsigned)nrhs);
}

// Every pointer and size an Arnoldi window's launches capture: a graph is
// replayed only for an identical key.
static std::vector<uint64_t> window_key(const marie_vie* h, size_t tsz, bool adjoint, int k0, int k1, int nrhs, int m,
                                        int64_t Nb, const void* V, const GmState& st) {
  return {(uint64_t)tsz, (uint64_t)adjoint, (uint64_t)k0, (uint64_t)k1, (uint64_t)nrhs, (uint64_t)m, (uint64_t)Nb,
          (uint64_t)(uintptr_t)V, (uint64_t)(uintptr_t)st.H, (uint64_t)(uintptr_t)st.R, (uint64_t)(uintptr_t)st.cs,
          (uint64_t)(uintptr_t)st.sn, (uint64_t)(uintptr_t)st.g, (uint64_t)(uintptr_t)st.y,
          (uint64_t)(uintptr_t)st.res, (uint64_t)(uintptr_t)st.beta, (uint64_t)(uintptr_t)st.hnorm,
          (uint64_t)(uintptr_t)st.resid, (uint64_t)(uintptr_t)st.tolabs, (uint64_t)(uintptr_t)st.kr,
          (uint64_t)(uintptr_t)st.hist, (uint64_t)(uintptr_t)st.incyc, (uint64_t)(uintptr_t)st.part,
          (uint64_t)(uintptr_t)st.npart, (uint64_t)(uintptr_t)h->hio, (uint64_t)h->hio_cap,
          (uint64_t)h->p32.TX, (uint64_t)h->p64.TX, (uint64_t)h->pff.TX, (uint64_t)h->p32.ws_rhs,
          (uint64_t)h->p64.ws_rhs, (uint64_t)h->pff.ws_rhs};
}

// MARIE_GMRES_GRAPH=0 turns the window graphs off.
static bool graphs_enabled() {
  static const bool v = [] {
    const char* e = getenv("MARIE_GMRES_GRAPH");
    return !(e && atoi(e) == 0);
  }();
  return v;
}

// Run an Arnoldi window: eagerly on `s` the first time its key is seen (this
// also does the one-time set-up of the kernels it launches), captured into a
// CUDA graph on the handle's own stream the second time, replayed from then
// on.  The graph stream is joined to `s` by events both ways.  A capture that
// fails leaves the window eager for good.
template <typename F>
static marie_status run_window(marie_vie* h, const std::vector<uint64_t>& key, F& window, cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (!graphs_enabled() || cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return window(s);
  }
  auto it = h->graphs.find(key);
  if (it == h->graphs.end()) {
    if (h->graphs.size() >= 4096) graphs_free(h);
    h->graphs[key] = marie_vie::GraphEntry{};
    return window(s);
  }
  marie_vie::GraphEntry& e = it->second;
  if (e.kernels < 0) return window(s);
  if (!h->gstream) {
    if (cudaStreamCreateWithFlags(&h->gstream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->gev[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->gev[1], cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      e.kernels = -1;
      return window(s);
    }
  }
  MARIE_CUDA_TRY(cudaEventRecord(h->gev[0], s));
  MARIE_CUDA_TRY(cudaStreamWaitEvent(h->gstream, h->gev[0], 0));
  if (!e.exec) {
    const int64_t before = t_launches;
    if (cudaStreamBeginCapture(h->gstream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
      cudaGetLastError();
      e.kernels = -1;
      return window(s);
    }
    const marie_status st = window(h->gstream);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(h->gstream, &g);
    const int64_t nk = t_launches - before;
    g_launches -= nk;     // captured, not run
    t_launches -= nk;
    cudaGraphExec_t ex = nullptr;
    if (st != MARIE_OK || ce != cudaSuccess || !g || cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) {
      cudaGetLastError();
      if (g) cudaGraphDestroy(g);
      e.kernels = -1;
      if (st != MARIE_OK) return st;
      return window(s);
    }
    cudaGraphDestroy(g);
    e.exec = ex;
    e.kernels = nk;
  }
  MARIE_CUDA_TRY(cudaGraphLaunch(e.exec, h->gstream));
  g_launches += e.kernels;
  t_launches += e.kernels;
  MARIE_CUDA_TRY(cudaEventRecord(h->gev[1], h->gstream));
  MARIE_CUDA_TRY(cudaStreamWaitEvent(s, h->gev[1], 0));
  return MARIE_OK;
}

struct RhsLog {
  std::vector<double> resvec;   // relative residual history
  int iters = 0, outer = 0, last_inner = 0, status = MARIE_OK;
};

// Run restarted GMRES on A_T for all rhs with todo[r] != 0.  On entry V_0 of
// each such rhs holds its initial residual r0 (unnormalised); bnorm[r] is the
// reference norm for the relative tolerance.  x (FP64) receives += V y.
template <typename T>
static marie_status gmres_core(marie_vie* h, int nrhs, cplx<T>* V, int m, zd* x, const std::vector<double>& bnorm,
                               const std::vector<double>& tolrel, int maxit, const std::vector<unsigned char>& todo,
                               std::vector<RhsLog>& log, int* matvecs, cudaStream_t s, Scratch& sc) {
  const int64_t Nb = h->Nb;
  const int mp1 = m + 1;
  const int nch = (int)((Nb + kCH - 1) / kCH);
  GmState st;
  MARIE_TRY(sc.get(&st.H, (size_t)nrhs * mp1 * m));
  MARIE_TRY(sc.get(&st.R, (size_t)nrhs * mp1 * m));
  MARIE_TRY(sc.get(&st.cs, (size_t)nrhs * m));
  MARIE_TRY(sc.get(&st.sn, (size_t)nrhs * m));
  MARIE_TRY(sc.get(&st.g, (size_t)nrhs * mp1));
  MARIE_TRY(sc.get(&st.y, (size_t)nrhs * m));
  MARIE_TRY(sc.get(&st.res, (size_t)nrhs * mp1));
  MARIE_TRY(sc.get(&st.beta, nrhs));
  MARIE_TRY(sc.get(&st.hnorm, nrhs));
  MARIE_TRY(sc.get(&st.resid, nrhs));
  MARIE_TRY(sc.get(&st.tolabs, nrhs));
  MARIE_TRY(sc.get(&st.kr, nrhs));
  MARIE_TRY(sc.get(&st.hist, (size_t)nrhs * m));
  MARIE_TRY(sc.get(&st.incyc, nrhs));
  MARIE_TRY(sc.get(&st.part, (size_t)nrhs * mp1 * nch));
  MARIE_TRY(sc.get(&st.npart, (size_t)nrhs * nch));
  unsigned char* d_mask = nullptr;
  MARIE_TRY(sc.get(&d_mask, nrhs));
  k_zero<<<vgrid((int64_t)nrhs * mp1 * m, 1), 256, 0, s>>>(st.H, (int64_t)nrhs * mp1 * m);
  MARIE_LAUNCH_CHECK();
  std::vector<double> tolabs(nrhs);
  for (int r = 0; r < nrhs; ++r) tolabs[r] = tolrel[r] * bnorm[r];
  MARIE_TRY(chan_put(h, SLOT_TOLABS, nrhs, st.tolabs, tolabs.data(), nrhs * sizeof(double), s));
  MARIE_TRY(chan_put(h, SLOT_MASK, nrhs, d_mask, todo.data(), nrhs, s));
  const int64_t ld = Nb;
  const int64_t vrs = (int64_t)mp1 * Nb;
  const dim3 cg((unsigned)nch, (unsigned)nrhs);
  const unsigned sb = (unsigned)((nrhs + 127) / 128);
  // beta = ||r0||
  k_norm2<T><<<cg, kVT, 0, s>>>(V, vrs, Nb, d_mask, st.npart, nch);
  MARIE_LAUNCH_CHECK();
  k_reduce_norm<<<(nrhs + 7) / 8, 256, 0, s>>>(st.npart, nch, nrhs, d_mask, st.beta);
  MARIE_LAUNCH_CHECK();
  std::vector<double> beta(nrhs, 0.0);
  MARIE_TRY(chan_get(h, SLOT_BETA, nrhs, st.beta, nrhs * sizeof(double), s));
  MARIE_CUDA_TRY(cudaStreamSynchronize(s));
  chan_take(h, SLOT_BETA, nrhs, beta.data(), nrhs * sizeof(double));
  std::vector<unsigned char> start(nrhs, 0);
  int nstart = 0;
  for (int r = 0; r < nrhs; ++r) {
    if (!todo[r]) continue;
    const double rel = bnorm[r] > 0 ? beta[r] / bnorm[r] : 0.0;
    log[r].resvec.push_back(rel);
    if (!std::isfinite(rel)) { log[r].status = MARIE_ERR_NONFINITE; continue; }
    if (rel > tolrel[r] && maxit > 0) { start[r] = 1; ++nstart; }
  }
  std::vector<unsigned char> incyc(nrhs), prev(nrhs);
  std::vector<int> kr(nrhs);
  int outit = 0;
  while (nstart > 0) {
    ++outit;
    MARIE_TRY(chan_put(h, SLOT_MASK, nrhs, d_mask, start.data(), nrhs, s));
    k_scale<T><<<vgrid(Nb, nrhs), 256, 0, s>>>(V, vrs, Nb, d_mask, st.beta);
    MARIE_LAUNCH_CHECK();
    k_cycle_init<<<sb, 128, 0, s>>>(st, m, nrhs, d_mask);
    MARIE_LAUNCH_CHECK();
    for (int r = 0; r < nrhs; ++r) if (start[r]) log[r].outer = outit;
    incyc = start;
    // The Arnoldi steps run in windows of sync_steps() between host
    // synchronisations; a window's launches (and the status reads that end
    // it) replay as one CUDA graph from its second occurrence on.
    for (int k0 = 0; k0 < m;) {
      const int k1 = std::min(m, (k0 / sync_steps() + 1) * sync_steps());
      auto window = [&](cudaStream_t q) -> marie_status {
        for (int k = k0; k < k1; ++k) {
          MARIE_TRY(launch_matvec<T>(h, sc.adjoint ? MV_VIE_ADJ : MV_VIE, sc.adjoint ? OP_N_ADJ : OP_N,
                                     V + (int64_t)k * ld, vrs, V + (int64_t)(k + 1) * ld, vrs, nrhs, st.incyc, q));
          k_dots<T><<<cg, kVT, 0, q>>>(V, ld, Nb, k, mp1, st.incyc, st.part, nch);
          MARIE_LAUNCH_CHECK();
          k_reduce_dots<<<dim3((k + 8) / 8, nrhs), 256, 0, q>>>(st.part, nch, k, mp1, m, st.incyc, st.H);
          MARIE_LAUNCH_CHECK();
          k_update<T><<<cg, kVT, 0, q>>>(V, ld, Nb, k, mp1, m, st.incyc, st.H, st.npart, nch);
          MARIE_LAUNCH_CHECK();
          k_reduce_norm<<<(nrhs + 7) / 8, 256, 0, q>>>(st.npart, nch, nrhs, st.incyc, st.hnorm);
          MARIE_LAUNCH_CHECK();
          // scale with the mask before the Givens step clears finished rhs
          k_scale<T><<<vgrid(Nb, nrhs), 256, 0, q>>>(V + (int64_t)(k + 1) * ld, vrs, Nb, st.incyc, st.hnorm);
          MARIE_LAUNCH_CHECK();
          k_givens<<<sb, 128, 0, q>>>(st, k, m, nrhs);
          MARIE_LAUNCH_CHECK();
        }
        MARIE_TRY(chan_get(h, SLOT_INCYC, nrhs, st.incyc, nrhs, q));
        MARIE_TRY(chan_get(h, SLOT_KR, nrhs, st.kr, nrhs * sizeof(int), q));
        MARIE_TRY(chan_get_hist(h, nrhs, st.hist, (size_t)nrhs * m * sizeof(double), q));
        return MARIE_OK;
      };
      MARIE_TRY(chan_reserve(h, nrhs));
      const std::vector<uint64_t> key = window_key(h, sizeof(T), sc.adjoint, k0, k1, nrhs, m, Nb, V, st);
      MARIE_TRY(run_window(h, key, window, s));
      *matvecs += k1 - k0;
      prev = incyc;
      MARIE_CUDA_TRY(cudaStreamSynchronize(s));
      chan_take(h, SLOT_INCYC, nrhs, incyc.data(), nrhs);
      chan_take(h, SLOT_KR, nrhs, kr.data(), nrhs * sizeof(int));
      const double* hist = reinterpret_cast<const double*>(chan_hist(h, nrhs));
      int any = 0;
      for (int r = 0; r < nrhs; ++r) {
        if (!prev[r]) continue;
        // steps [k0, kr) of this window ran for r
        for (int j = k0; j < kr[r]; ++j) {
          log[r].resvec.push_back(hist[(size_t)r * m + j] / bnorm[r]);
          log[r].iters++;
        }
        if (incyc[r]) any = 1;
      }
      k0 = k1;
      if (!any) break;
    }
    // finalize the cycle of every rhs that ran it
    MARIE_TRY(chan_get(h, SLOT_KR, nrhs, st.kr, nrhs * sizeof(int), s));
    MARIE_TRY(chan_put(h, SLOT_MASK, nrhs, d_mask, start.data(), nrhs, s));
    k_solve_y<<<sb, 128, 0, s>>>(st, m, nrhs, d_mask);
    MARIE_LAUNCH_CHECK();
    k_xupdate<T><<<vgrid(Nb, nrhs), 256, 0, s>>>(V, ld, mp1, m, Nb, d_mask, st, x, Nb);
    MARIE_LAUNCH_CHECK();
    k_rform<T><<<vgrid(Nb, nrhs), 256, 0, s>>>(V, ld, mp1, Nb, d_mask, st);
    MARIE_LAUNCH_CHECK();
    k_norm2<T><<<cg, kVT, 0, s>>>(V, vrs, Nb, d_mask, st.npart, nch);
    MARIE_LAUNCH_CHECK();
    k_reduce_norm<<<(nrhs + 7) / 8, 256, 0, s>>>(st.npart, nch, nrhs, d_mask, st.beta);
    MARIE_LAUNCH_CHECK();
    MARIE_CUDA_TRY(cudaStreamSynchronize(s));
    chan_take(h, SLOT_KR, nrhs, kr.data(), nrhs * sizeof(int));
    nstart = 0;
    for (int r = 0; r < nrhs; ++r) {
      if (!start[r]) continue;
      log[r].last_inner = kr[r];
      const double rel = log[r].resvec.back();
      start[r] = 0;
      if (!std::isfinite(rel)) { log[r].status = MARIE_ERR_NONFINITE; continue; }
      if (rel > tolrel[r]) {
        if (outit < maxit) { start[r] = 1; ++nstart; }
        else log[r].status = MARIE_ERR_NOT_CONVERGED;
      }
    }
  }
  return MARIE_OK;
}

// r = b - A64 x for rhs in mask; returns ||r||/||b|| per rhs on the host.
static marie_status true_residual(marie_vie* h, int nrhs, const zd* b, const zd* x, zd* r,
                                  const std::vector<unsigned char>& mask, const std::vector<double>& bnorm,
                                  std::vector<double>& rel, int* matvecs, cudaStream_t s, Scratch& sc) {
  const int64_t Nb = h->Nb;
  unsigned char* d_mask = nullptr;
  MARIE_TRY(sc.get(&d_mask, nrhs));
  const int nch = (int)((Nb + kCH - 1) / kCH);
  double *npart = nullptr, *nr = nullptr;
  MARIE_TRY(sc.get(&npart, (size_t)nrhs * nch));
  MARIE_TRY(sc.get(&nr, nrhs));
  MARIE_TRY(chan_put(h, SLOT_NORM, nrhs, d_mask, mask.data(), nrhs, s));
  MARIE_TRY(launch_matvec<double>(h, sc.adjoint ? MV_VIE_ADJ : MV_VIE, sc.adjoint ? OP_N_ADJ : OP_N,
                                  (const cplx<double>*)x, Nb, (cplx<double>*)r, Nb, nrhs, d_mask, s));
  ++*matvecs;
  k_residual<<<vgrid(Nb, nrhs), 256, 0, s>>>(b, r, Nb, d_mask);
  MARIE_LAUNCH_CHECK();
  k_norm2<double><<<dim3(nch, nrhs), kVT, 0, s>>>((const cplx<double>*)r, Nb, Nb, d_mask, npart, nch);
  MARIE_LAUNCH_CHECK();
  k_reduce_norm<<<(nrhs + 7) / 8, 256, 0, s>>>(npart, nch, nrhs, d_mask, nr);
  MARIE_LAUNCH_CHECK();
  std::vector<double> v(nrhs);
  MARIE_TRY(chan_get(h, SLOT_NORM, nrhs, nr, nrhs * sizeof(double), s));
  MARIE_CUDA_TRY(cudaStreamSynchronize(s));
  chan_take(h, SLOT_NORM, nrhs, v.data(), nrhs * sizeof(double));
  rel.resize(nrhs);
  for (int k = 0; k < nrhs; ++k)
    if (mask[k]) rel[k] = bnorm[k] > 0 ? v[k] / bnorm[k] : 0.0;
  return MARIE_OK;
}

static marie_status norms(marie_vie* h, int nrhs, const zd* v, std::vector<double>& out, cudaStream_t s, Scratch& sc) {
  const int64_t Nb = h->Nb;
  const int nch = (int)((Nb + kCH - 1) / kCH);
  double *npart = nullptr, *nr = nullptr;
  MARIE_TRY(sc.get(&npart, (size_t)nrhs * nch));
  MARIE_TRY(sc.get(&nr, nrhs));
  k_norm2<double><<<dim3(nch, nrhs), kVT, 0, s>>>((const cplx<double>*)v, Nb, Nb, nullptr, npart, nch);
  MARIE_LAUNCH_CHECK();
  k_reduce_norm<<<(nrhs + 7) / 8, 256, 0, s>>>(npart, nch, nrhs, nullptr, nr);
  MARIE_LAUNCH_CHECK();
  out.resize(nrhs);
  MARIE_TRY(chan_get(h, SLOT_NORM, nrhs, nr, nrhs * sizeof(double), s));
  MARIE_CUDA_TRY(cudaStreamSynchronize(s));
  chan_take(h, SLOT_NORM, nrhs, out.data(), nrhs * sizeof(double));
  return MARIE_OK;
}

}  // namespace marie

#include "bgmres.cuh"

namespace marie {

static void fill_report(marie_gmres_report* rep, const std::vector<RhsLog>& log, const std::vector<double>& trel,
                        int mv64, int mv32) {
  if (!rep) return;
  const int nrhs = (int)log.size();
  for (int r = 0; r < nrhs; ++r) {
    if (rep->iters) rep->iters[r] = log[r].iters;
    if (rep->outer) rep->outer[r] = log[r].outer;
    if (rep->last_inner) rep->last_inner[r] = log[r].last_inner;
    if (rep->true_resid) rep->true_resid[r] = trel[r];
    if (rep->status) rep->status[r] = log[r].status;
    if (rep->resvec && rep->resvec_cap > 0) {
      const int n = std::min<int>(rep->resvec_cap, (int)log[r].resvec.size());
      for (int i = 0; i < n; ++i) rep->resvec[(int64_t)r * rep->resvec_cap + i] = log[r].resvec[i];
      if (rep->resvec_len) rep->resvec_len[r] = n;
    }
  }
  rep->matvecs_c128 = mv64;
  rep->matvecs_c64 = mv32;
}

}  // namespace marie

using namespace marie;

extern "C" marie_status marie_gmres_vie(marie_vie* h, const void* b_, void* x_, int32_t nrhs,
                                        const marie_gmres_opts* o, marie_gmres_report* rep, void* stream) {
  if (!h || !b_ || !x_ || !o) { set_error("NULL argument"); return MARIE_ERR_BAD_ARG; }
  if (nrhs < 1) { set_error("nrhs must be >= 1"); return MARIE_ERR_BAD_ARG; }
  if (o->restart < 1 || o->restart > kMaxRestart) { set_error("restart must be in [1, %d]", kMaxRestart); return MARIE_ERR_BAD_ARG; }
  if (o->maxit < 0) { set_error("maxit must be >= 0"); return MARIE_ERR_BAD_ARG; }
  if (!(o->tol > 0)) { set_error("tol must be > 0"); return MARIE_ERR_BAD_ARG; }
  if (o->mode != MARIE_SOLVE_FP64 && o->mode != MARIE_SOLVE_MIXED && o->mode != MARIE_SOLVE_MIXED_BLOCK) {
    set_error("unknown solve mode");
    return MARIE_ERR_BAD_ARG;
  }
  if (o->block_steps < 0 || o->block_steps > 200) { set_error("block_steps must be in [0, 200]"); return MARIE_ERR_BAD_ARG; }
  if (!h->p64.built && !h->pff.built) {
    set_error("GMRES needs a complex128 operator (precisions bit 1 or 4)");
    return MARIE_ERR_BAD_ARG;
  }
  if (o->mode != MARIE_SOLVE_FP64 && !h->p32.built) { set_error("mixed mode needs the complex64 operator (precisions bit 2)"); return MARIE_ERR_BAD_ARG; }
  cudaStream_t s = (cudaStream_t)stream;
  const zd* b = (const zd*)b_;
  zd* x = (zd*)x_;
  const int64_t Nb = h->Nb;
  const int m = o->restart;
  Scratch sc(h);
  sc.adjoint = o->adjoint != 0;
  std::vector<RhsLog> log(nrhs);
  std::vector<double> bnorm;
  MARIE_TRY(norms(h, nrhs, b, bnorm, s, sc));
  for (int r = 0; r < nrhs; ++r)
    if (!std::isfinite(bnorm[r])) { set_error("right-hand side %d is not finite", r); return MARIE_ERR_NONFINITE; }
  if (!o->x0_present) {
    k_zero<<<vgrid(Nb * nrhs, 1), 256, 0, s>>>(x, Nb * nrhs);
    MARIE_LAUNCH_CHECK();
  }
  int mv64 = 0, mv32 = 0;
  std::vector<double> trel(nrhs, 0.0);
  std::vector<unsigned char> all(nrhs, 1);
  zd* r64 = nullptr;
  MARIE_TRY(sc.get(&r64, (size_t)nrhs * Nb));
  if (o->mode == MARIE_SOLVE_FP64) {
    cplx<double>* V = nullptr;
    MARIE_TRY(sc.get(&V, (size_t)nrhs * (m + 1) * Nb));
    // r0 into V_0 (is_gmres_vie.m:5-9)
    if (o->x0_present) {
      MARIE_TRY(true_residual(h, nrhs, b, x, r64, all, bnorm, trel, &mv64, s, sc));
      k_convert<double, double><<<vgrid(Nb, nrhs), 256, 0, s>>>((const cplx<double>*)r64, Nb, V, (int64_t)(m + 1) * Nb, Nb, nullptr);
    } else {
      k_convert<double, double><<<vgrid(Nb, nrhs), 256, 0, s>>>((const cplx<double>*)b, Nb, V, (int64_t)(m + 1) * Nb, Nb, nullptr);
    }
    MARIE_LAUNCH_CHECK();
    std::vector<double> tolrel(nrhs, o->tol);
    MARIE_TRY(gmres_core<double>(h, nrhs, V, m, x, bnorm, tolrel, o->maxit, all, log, &mv64, s, sc));
    MARIE_TRY(true_residual(h, nrhs, b, x, r64, all, bnorm, trel, &mv64, s, sc));
  } else {
    const bool block = o->mode == MARIE_SOLVE_MIXED_BLOCK;
    // 30 block steps per cycle: at 128^3 PWL with 64 loop ports 20 / 30 /
    // 40 / 50 / 60 take 185 / 143 / 139 / 142 / 150 block steps, 30 the least time
    const int mb = o->block_steps > 0 ? o->block_steps : 30;
    cplx<float>* V = nullptr;
    BlockWork bw;
    if (!block) {
      MARIE_TRY(sc.get(&V, (size_t)nrhs * (m + 1) * Nb));
    } else {
      // block basis (block_steps + 1) x nrhs vectors, the block W and the
      // small matrices, shared by the refinement steps
      MARIE_TRY(block_work_alloc(h, bw, nrhs, mb, sc));
    }
    std::vector<double> rel(nrhs, 1.0);
    if (o->x0_present) {
      MARIE_TRY(true_residual(h, nrhs, b, x, r64, all, bnorm, rel, &mv64, s, sc));
    } else {
      // a kernel, not a copy-engine transfer (see the status channel above)
      k_convert<double, double><<<vgrid(Nb, nrhs), 256, 0, s>>>((const cplx<double>*)b, Nb, (cplx<double>*)r64, Nb, Nb,
                                                                nullptr);
      MARIE_LAUNCH_CHECK();
      for (int r = 0; r < nrhs; ++r) rel[r] = bnorm[r] > 0 ? 1.0 : 0.0;
    }
    const double floor_tol = o->inner_tol > 0 ? o->inner_tol : 1e-7;
    const int max_refine = o->max_refine > 0 ? o->max_refine : 10;
    // fraction of the outer target the inner solve aims for; a right-hand
    // side that still misses tol gets another (short) inner solve.  With the
    // 64 ring loop ports of the PWL phantom, tol 1e-6: per-RHS GMRES at 96^3
    // takes 238 batched steps for 0.9 against 256 / 266 / 290 for 0.5 / 0.3
    // / 0.15; block GMRES at 128^3 143 block steps against 154 / 175 for
    // 0.5 / 0.2
    const double safety = o->inner_safety > 0 ? o->inner_safety : 0.9;
    for (int it = 0; it < max_refine; ++it) {
      std::vector<unsigned char> todo(nrhs, 0);
      int n = 0;
      for (int r = 0; r < nrhs; ++r)
        if (rel[r] > o->tol && std::isfinite(rel[r]) && log[r].status == MARIE_OK) { todo[r] = 1; ++n; }
      if (n == 0) break;
      // inner problem A d = r: relative tolerance w.r.t. ||r||, asking for just
      // enough reduction to reach the outer target (bounded by the c64 floor)
      std::vector<double> rn(nrhs), tin(nrhs);
      for (int r = 0; r < nrhs; ++r) {
        rn[r] = rel[r] * bnorm[r];
        tin[r] = std::min(0.5, std::max(floor_tol, safety * o->tol / std::max(rel[r], 1e-300)));
      }
      std::vector<RhsLog> ilog(nrhs);
      if (block) {
        // the right-hand sides still above tol share one block Krylov space
        std::vector<int> cols;
        std::vector<double> cn, ct;
        for (int r = 0; r < nrhs; ++r)
          if (todo[r]) {
            cols.push_back(r);
            cn.push_back(rn[r]);
            ct.push_back(tin[r] * rn[r]);
          }
        MARIE_TRY(bgmres_core(h, cols, r64, x, cn, ct, o->maxit, bw, ilog, &mv32, s, sc));
      } else {
        unsigned char* d_todo = nullptr;
        MARIE_TRY(sc.get(&d_todo, nrhs));
        MARIE_TRY(chan_put(h, SLOT_TODO, nrhs, d_todo, todo.data(), nrhs, s));
        k_convert<double, float><<<vgrid(Nb, nrhs), 256, 0, s>>>((const cplx<double>*)r64, Nb, V, (int64_t)(m + 1) * Nb,
                                                                 Nb, d_todo);
        MARIE_LAUNCH_CHECK();
        MARIE_TRY(gmres_core<float>(h, nrhs, V, m, x, rn, tin, o->maxit, todo, ilog, &mv32, s, sc));
      }
      for (int r = 0; r < nrhs; ++r) {
        if (!todo[r]) continue;
        log[r].iters += ilog[r].iters;
        log[r].outer += ilog[r].outer;
        log[r].last_inner = ilog[r].last_inner;
        for (size_t i = 1; i < ilog[r].resvec.size(); ++i) log[r].resvec.push_back(ilog[r].resvec[i] * rel[r]);
        if (ilog[r].status == MARIE_ERR_NONFINITE) log[r].status = MARIE_ERR_NONFINITE;
      }
      MARIE_TRY(true_residual(h, nrhs, b, x, r64, todo, bnorm, rel, &mv64, s, sc));
      for (int r = 0; r < nrhs; ++r)
        if (todo[r]) log[r].resvec.push_back(rel[r]);
    }
    trel = rel;
    for (int r = 0; r < nrhs; ++r)
      if (log[r].status == MARIE_OK && !(rel[r] <= o->tol)) log[r].status = MARIE_ERR_NOT_CONVERGED;
  }
  fill_report(rep, log, trel, mv64, mv32);
  int worst = MARIE_OK;
  for (int r = 0; r < nrhs; ++r)
    if (log[r].status != MARIE_OK) worst = log[r].status;
  if (worst == MARIE_ERR_NOT_CONVERGED) set_error("some right-hand sides did not reach tol");
  if (worst == MARIE_ERR_NONFINITE) set_error("non-finite residual encountered");
  return (marie_status)worst;
}

// Host-buffer form: b and x in host memory (pinned for overlap).  The
// right-hand sides are solved in chunks of at most the matvec chunk size
// through two device buffer pairs: chunk k+1 is copied in before chunk k is
// solved, and chunk k is copied out on a second stream while chunk k+1 is
// solved, so only the first copy in and the last copy out are exposed, and
// those two chunks are made small.
extern "C" marie_status marie_gmres_vie_host(marie_vie* h, const void* b_host, void* x_host, int32_t nrhs,
                                             const marie_gmres_opts* o, marie_gmres_report* rep, void* stream) {
  if (!h || !b_host || !x_host || !o) { set_error("NULL argument"); return MARIE_ERR_BAD_ARG; }
  if (nrhs < 1) { set_error("nrhs must be >= 1"); return MARIE_ERR_BAD_ARG; }
  const int64_t Nb = h->Nb;
  // block mode: one chunk, so that all right-hand sides share the block space
  int cs = o->mode == MARIE_SOLVE_MIXED_BLOCK ? (int)nrhs
           : o->mode == MARIE_SOLVE_MIXED ? h->p32.ws_rhs : (h->p64.built ? h->p64.ws_rhs : h->pff.ws_rhs);
  // MARIE_HOST_CHUNK: right-hand sides per chunk of the host-buffer solve
  if (const char* e = getenv("MARIE_HOST_CHUNK")) {
    if (atoi(e) > 0) cs = atoi(e);
  }
  cs = std::max(1, std::min(cs, (int)nrhs));
  // chunk schedule: only the first copy in and the last copy out are
  // exposed, so the first and last chunks are a quarter chunk and the rest
  // full chunks (64 = 4 + 16 + 16 + 16 + 8 + 4 for chunks of 16)
  std::vector<int> c0, cn;
  {
    const int q = std::max(1, cs / 4);
    int left = nrhs, r0 = 0;
    auto add = [&](int n) { c0.push_back(r0); cn.push_back(n); r0 += n; left -= n; };
    if (nrhs > 2 * q + cs) {
      add(q);
      while (left > cs + q) add(cs);
      if (left > q) add(left - q);
      add(left);
    } else {
      while (left > 0) add(std::min(cs, left));
    }
  }
  const int nch = (int)c0.size();
  cudaStream_t s = (cudaStream_t)stream;
  Scratch sc(h, &h->io_pool);
  zd *bd[2] = {nullptr, nullptr}, *xd[2] = {nullptr, nullptr};
  for (int i = 0; i < 2 && i < nch; ++i) {
    MARIE_TRY(sc.get(&bd[i], (size_t)cs * Nb));
    MARIE_TRY(sc.get(&xd[i], (size_t)cs * Nb));
  }
  cudaStream_t cps = nullptr;
  cudaEvent_t ev_in[2] = {nullptr, nullptr}, ev_done = nullptr;
  MARIE_CUDA_TRY(cudaStreamCreateWithFlags(&cps, cudaStreamNonBlocking));
  for (int i = 0; i < 2; ++i) cudaEventCreateWithFlags(&ev_in[i], cudaEventDisableTiming);
  cudaEventCreateWithFlags(&ev_done, cudaEventDisableTiming);
  auto finish = [&](marie_status st) {
    cudaStreamSynchronize(cps);
    cudaStreamDestroy(cps);
    for (int i = 0; i < 2; ++i) cudaEventDestroy(ev_in[i]);
    cudaEventDestroy(ev_done);
    return st;
  };
  const zd* bh = (const zd*)b_host;
  zd* xh = (zd*)x_host;
  auto copy_in = [&](int k) -> marie_status {
    const int r0 = c0[k], nk = cn[k], u = k & 1;
    const size_t bytes = sizeof(zd) * (size_t)nk * Nb;
    if (cudaMemcpyAsync(bd[u], bh + (int64_t)r0 * Nb, bytes, cudaMemcpyHostToDevice, cps) != cudaSuccess ||
        (o->x0_present && cudaMemcpyAsync(xd[u], xh + (int64_t)r0 * Nb, bytes, cudaMemcpyHostToDevice, cps) != cudaSuccess)) {
      set_error("host-to-device copy of right-hand sides failed");
      return MARIE_ERR_CUDA;
    }
    cudaEventRecord(ev_in[u], cps);
    return MARIE_OK;
  };
  marie_status st = copy_in(0);
  if (st != MARIE_OK) return finish(st);
  int worst = MARIE_OK, mv64 = 0, mv32 = 0;
  for (int k = 0; k < nch; ++k) {
    const int r0 = c0[k], nk = cn[k], u = k & 1;
    if (k + 1 < nch && (st = copy_in(k + 1)) != MARIE_OK) return finish(st);
    cudaStreamWaitEvent(s, ev_in[u], 0);
    marie_gmres_report sub = {};
    if (rep) {
      sub = *rep;
      if (rep->iters) sub.iters = rep->iters + r0;
      if (rep->outer) sub.outer = rep->outer + r0;
      if (rep->last_inner) sub.last_inner = rep->last_inner + r0;
      if (rep->true_resid) sub.true_resid = rep->true_resid + r0;
      if (rep->resvec) sub.resvec = rep->resvec + (int64_t)r0 * rep->resvec_cap;
      if (rep->resvec_len) sub.resvec_len = rep->resvec_len + r0;
      if (rep->status) sub.status = rep->status + r0;
    }
    st = marie_gmres_vie(h, bd[u], xd[u], nk, o, rep ? &sub : nullptr, stream);
    if (st != MARIE_OK && st != MARIE_ERR_NOT_CONVERGED && st != MARIE_ERR_NONFINITE) return finish(st);
    if (st != MARIE_OK) worst = st;
    mv64 += sub.matvecs_c128;
    mv32 += sub.matvecs_c64;
    cudaEventRecord(ev_done, s);
    cudaStreamWaitEvent(cps, ev_done, 0);
    if (cudaMemcpyAsync(xh + (int64_t)r0 * Nb, xd[u], sizeof(zd) * (size_t)nk * Nb, cudaMemcpyDeviceToHost, cps) !=
        cudaSuccess) {
      set_error("device-to-host copy of solutions failed");
      return finish(MARIE_ERR_CUDA);
    }
  }
  if (rep) {
    rep->matvecs_c128 = mv64;
    rep->matvecs_c64 = mv32;
  }
  if (worst == MARIE_ERR_NOT_CONVERGED) set_error("some right-hand sides did not reach tol");
  if (worst == MARIE_ERR_NONFINITE) set_error("non-finite residual encountered");
  return finish((marie_status)worst);
}
