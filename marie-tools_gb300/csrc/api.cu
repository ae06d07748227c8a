// C-ABI entry points of the operator: create/destroy/apply, plus the FFT
// plans, per-axis tables and the matvec launcher.
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <complex>
#include <mutex>
#include <new>

#include "fastpath.cuh"
#include "embed.h"
#include "internal.h"

namespace marie {

static thread_local std::string t_err;
std::atomic<int64_t> g_launches{0};
thread_local int64_t t_launches = 0;

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  t_err = buf;
}

marie_status dev_alloc(marie_vie* h, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) return MARIE_OK;
  if (h->mem_cap > 0 && h->mem_used + (int64_t)bytes > h->mem_cap) {
    set_error("device memory cap exceeded: need %lld more bytes, cap %lld, used %lld",
              (long long)bytes, (long long)h->mem_cap, (long long)h->mem_used);
    return MARIE_ERR_OOM;
  }
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
    *p = nullptr;
    return MARIE_ERR_OOM;
  }
  h->allocs.push_back(*p);
  h->mem_used += (int64_t)bytes;
  return MARIE_OK;
}

void graphs_free(marie_vie* h) {
  for (auto& e : h->graphs)
    if (e.second.exec) cudaGraphExecDestroy(e.second.exec);
  h->graphs.clear();
  if (h->gstream) cudaStreamDestroy(h->gstream);
  for (auto& e : h->gev)
    if (e) cudaEventDestroy(e);
  h->gstream = nullptr;
  h->gev[0] = h->gev[1] = nullptr;
}

void dev_free_all(marie_vie* h) {
  graphs_free(h);
  for (void* p : h->allocs) cudaFree(p);
  h->allocs.clear();
  for (auto& e : h->gm_pool) cudaFree(e.first);
  h->gm_pool.clear();
  for (auto& e : h->io_pool) cudaFree(e.first);
  h->io_pool.clear();
  if (h->hio) cudaFreeHost(h->hio);
  h->hio = nullptr;
  h->hio_cap = 0;
  if (h->bio) cudaFreeHost(h->bio);
  h->bio = nullptr;
  h->bio_cap = 0;
  blas_free(h);
  h->mem_used = 0;
}

template <>
PrecState<double>& prec_state<double>(marie_vie* h) { return h->p64; }
template <>
PrecState<float>& prec_state<float>(marie_vie* h) { return h->p32; }
template <>
PrecState<ff>& prec_state<ff>(marie_vie* h) { return h->pff; }

// Host conversion of a table value to the device arithmetic type.
template <typename T>
static T prec_from(long double v) {
  if constexpr (std::is_same<T, ff>::value) {
    const float hi = (float)v;
    return ff(hi, (float)(v - (long double)hi));
  } else {
    return (T)v;
  }
}

// n = product of radices; 8s first, then 4, 2, then odd primes.
static bool make_plan(int n, FftPlan* pl) {
  pl->n = n;
  pl->nst = 0;
  int m = n;
  auto push = [&](int r) {
    if (pl->nst >= kMaxStages) return false;
    pl->r[pl->nst++] = r;
    m /= r;
    return true;
  };
  while (m % 8 == 0) if (!push(8)) return false;
  if (m % 4 == 0) if (!push(4)) return false;
  if (m % 2 == 0) if (!push(2)) return false;
  for (int p = 3; m > 1 && p <= 31; p += 2) {
    while (m % p == 0) if (!push(p)) return false;
  }
  return m == 1;
}

// kofp[p]: frequency held at digit-reversed position p (see FftPlan).
static void digit_maps(const FftPlan& pl, std::vector<int>& kofp, std::vector<int>& pofk) {
  const int n = pl.n;
  kofp.assign(n, 0);
  pofk.assign(n, 0);
  for (int k = 0; k < n; ++k) {
    int rem = k, p = 0, span = n;
    for (int s = 0; s < pl.nst; ++s) {
      const int r = pl.r[s];
      const int t = rem % r;
      rem /= r;
      span /= r;
      p += t * span;
    }
    kofp[p] = k;
    pofk[k] = p;
  }
}

template <typename T>
static marie_status build_axis(marie_vie* h, int n, AxisDev<T>& ax) {
  if (!make_plan(n, &ax.plan)) {
    set_error("grid edge %d has a prime factor above 31 (unsupported FFT length)", n);
    return MARIE_ERR_NOT_SUPPORTED;
  }
  std::vector<cplx<T>> tw(n), tw2(n);
  for (int k = 0; k < n; ++k) {
    const long double a = -2.0L * 3.141592653589793238462643383279502884L * (long double)k / (long double)n;
    const long double b = a / 2.0L;
    tw[k] = cplx<T>{prec_from<T>(std::cos(a)), prec_from<T>(std::sin(a))};
    tw2[k] = cplx<T>{prec_from<T>(std::cos(b)), prec_from<T>(std::sin(b))};
  }
  std::vector<int> kofp, pofk;
  digit_maps(ax.plan, kofp, pofk);
  MARIE_TRY(dev_alloc(h, (void**)&ax.tw, n * sizeof(cplx<T>)));
  MARIE_TRY(dev_alloc(h, (void**)&ax.tw2, n * sizeof(cplx<T>)));
  MARIE_TRY(dev_alloc(h, (void**)&ax.kofp, n * sizeof(int)));
  MARIE_TRY(dev_alloc(h, (void**)&ax.pofk, n * sizeof(int)));
  MARIE_CUDA_TRY(cudaMemcpy(ax.tw, tw.data(), n * sizeof(cplx<T>), cudaMemcpyHostToDevice));
  MARIE_CUDA_TRY(cudaMemcpy(ax.tw2, tw2.data(), n * sizeof(cplx<T>), cudaMemcpyHostToDevice));
  MARIE_CUDA_TRY(cudaMemcpy(ax.kofp, kofp.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  MARIE_CUDA_TRY(cudaMemcpy(ax.pofk, pofk.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  return MARIE_OK;
}

// Block tables of mvp_{N,K}{,_herm_adj}_{pwc,pwl}_tucker.m.
static const int PQ_N[3][3] = {{1, 2, 3}, {2, 4, 5}, {3, 5, 6}};
static const int PQ_K[3][3] = {{0, -3, 2}, {3, 0, -1}, {-2, 1, 0}};
static const int LLP[4][4] = {{1, 5, 6, 7}, {-5, 2, 8, 9}, {-6, 8, 3, 10}, {-7, 9, 10, 4}};
static const int SLP[4][4] = {{1, -1, -1, -1}, {-1, 1, 1, 1}, {-1, 1, 1, 1}, {-1, 1, 1, 1}};
// circulant mirror signs, assembly_fft_circ_tucker_{pwc,pwl}.m
static const int GN1[6] = {+1, -1, -1, +1, +1, +1}, GN2[6] = {+1, -1, +1, +1, -1, +1},
                 GN3[6] = {+1, +1, -1, +1, -1, +1};
static const int GK1[3] = {-1, +1, +1}, GK2[3] = {+1, -1, +1}, GK3[3] = {+1, +1, -1};
static const int BT1[10] = {+1, +1, +1, +1, -1, +1, +1, -1, -1, +1};
static const int BT2[10] = {+1, +1, +1, +1, +1, -1, +1, -1, +1, -1};
static const int BT3[10] = {+1, +1, +1, +1, +1, +1, -1, +1, -1, -1};

static inline int sgn(int v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }

static void make_tables(marie_vie* h) {
  const int C = h->C, pwl = h->pwl;
  for (int t = 0; t < 4; ++t) {
    BlockTab& b = h->tab[t];
    memset(&b, 0, sizeof(b));
    for (int i = 0; i < kMaxComp * kMaxComp; ++i) b.blk[i] = -1;
    const bool isK = t >= 2, adj = (t & 1) != 0;
    const int ncomp = isK ? 3 : 6;
    const int pwx = pwl ? 10 : 1;
    b.nblk = pwx * ncomp;
    b.conj = adj ? 1 : 0;
    for (int j = 0; j < pwx; ++j)
      for (int k = 0; k < ncomp; ++k) {
        const int id = j * ncomp + k;
        const int bt1 = pwl ? BT1[j] : 1, bt2 = pwl ? BT2[j] : 1, bt3 = pwl ? BT3[j] : 1;
        b.s1[id] = (int8_t)((isK ? GK1[k] : GN1[k]) * bt1);
        b.s2[id] = (int8_t)((isK ? GK2[k] : GN2[k]) * bt2);
        b.s3[id] = (int8_t)((isK ? GK3[k] : GN3[k]) * bt3);
      }
    for (int p = 0; p < 3; ++p)
      for (int q = 0; q < 3; ++q) {
        int k, s_pq;
        if (!isK) {
          k = PQ_N[p][q] - 1;
          s_pq = 1;
        } else {
          if (p == q) continue;
          k = std::abs(PQ_K[p][q]) - 1;
          s_pq = sgn(PQ_K[p][q]);
        }
        if (!pwl) {
          int s = s_pq;
          if (isK && adj) s = -s;  // conj(-nmp(...)), mvp_K_herm_adj_pwc_tucker.m:26
          b.blk[p * C + q] = (int8_t)k;
          b.sgn[p * C + q] = (int8_t)s;
          continue;
        }
        for (int l = 0; l < 4; ++l)
          for (int lp = 0; lp < 4; ++lp) {
            const int j = std::abs(LLP[l][lp]) - 1;
            int s = s_pq * sgn(LLP[l][lp]);
            if (adj) {
              s *= sgn(SLP[l][lp]);
              if (isK) s = -s;  // mvp_K_herm_adj_pwl_tucker.m:34
            }
            const int row = 4 * p + l, col = 4 * q + lp;
            b.blk[row * C + col] = (int8_t)(j * ncomp + k);
            b.sgn[row * C + col] = (int8_t)s;
          }
      }
  }
}

// Z-pass tile width W = TX*R (contiguous elements per (component, z) row):
// the largest power of two whose shared-memory tile fits ~100 KB (two CTAs per
// SM).  The bundle size R is at most W.
static int env_int(const char* name, int dflt) {
  const char* v = getenv(name);
  if (!v || !*v) return dflt;
  return atoi(v);
}

template <typename T>
static marie_status choose_tiles(marie_vie* h, PrecState<T>& ps) {
  const int n3 = h->n3, C = h->C;
  const int sz = (int)sizeof(cplx<T>);
  int W = 16;
  while (W > 1 && (size_t)n3 * (2 * C * W + 1) * sz > 100 * 1024) W /= 2;
  // MARIE_Z_TILE: z-pass tile width (power of two <= 16) if its shared
  // memory fits one CTA (227 KB)
  const int wz = env_int("MARIE_Z_TILE", 0);
  const size_t lim = kSmemOptin;
  if (wz >= 1 && wz <= 16 && (wz & (wz - 1)) == 0 && (size_t)n3 * (2 * C * wz + 2) * sz <= lim &&
      kz4_smem<T>(n3, C, wz) <= lim)
    W = wz;
  // The generic passes (any grid; K and K^H on every grid) with the
  // narrowest row tiles and a bundle of W right-hand sides must fit one CTA's
  // shared memory; narrow W until they do, and refuse the grid at create
  // when even W = 1 does not (a pass would otherwise fail to launch midway
  // through a matvec).  The float-float state runs the four-step passes only.
  if constexpr (!std::is_same<T, ff>::value) {
    auto need = [&](int w) { return generic_smem(h->n1, h->n2, n3, C, sz, 1, 1, 1, w); };
    while (W > 1) {
      const GenericSmem g = need(W);
      if (g.x <= lim && g.y <= lim && g.z <= lim) break;
      W /= 2;
    }
    const GenericSmem g = need(W);
    if (g.x > lim || g.y > lim || g.z > lim) {
      set_error("grid %d x %d x %d (%s, %s) needs %zu / %zu / %zu bytes of shared memory in the x / y / z "
                "passes, more than the %zu a CTA can hold; use smaller edges (complex128 PWL: n3 <= %d)",
                h->n1, h->n2, n3, C == 12 ? "PWL" : "PWC", sz == 16 ? "complex128" : "complex64", g.x, g.y,
                g.z, lim, (int)(lim / ((size_t)(2 * C + 2) * 16)));
      return MARIE_ERR_BAD_ARG;
    }
  }
  ps.TX = W;      // Wz
  ps.TY = 0;
  ps.TXY = 0;
  return MARIE_OK;
}

struct CallTiles {
  int R, TY, TXY, TX;
};

static int pow2floor(int v) {
  int p = 1;
  while (p * 2 <= v) p *= 2;
  return p;
}

// Bundle size R (a power of two, <= the z tile width) and the tiles of one
// chunk of nr right-hand sides.  fast: four-step passes (wider x/y tiles).
template <typename T>
static CallTiles call_tiles(const marie_vie* h, const PrecState<T>& ps, int nr, bool fast) {
  CallTiles t;
  const int Wz = ps.TX;
  t.R = pow2floor(std::max(1, std::min(Wz, nr)));
  const int wxy = (sizeof(T) == 4 ? 16 : 8) * (fast ? 2 : 1);   // row-tile width of the x/y passes
  t.TY = std::max(1, std::min(h->n2, wxy / t.R));
  t.TXY = std::max(1, std::min(2 * h->n1, wxy / t.R));
  t.TX = std::max(1, std::min(2 * h->n1, Wz / t.R));
  if (!fast) {   // generic passes: keep every tile within one CTA's shared memory
    const size_t sz = sizeof(cplx<T>);
    t.TY = std::min(t.TY, generic_tile_cap(h->n1, 1, t.R, sz));
    t.TXY = std::min(t.TXY, generic_tile_cap(h->n2, 1, t.R, sz));
    t.TX = std::min(t.TX, generic_tile_cap(h->n3, h->C, t.R, sz));
  }
  return t;
}


template <typename T>
static void fill_axis(AxisTab<T>& dst, const AxisDev<T>& src) {
  dst.tw = src.tw;
  dst.tw2 = src.tw2;
  dst.kofp = src.kofp;
  dst.pofk = src.pofk;
  dst.plan = src.plan;
}


template <typename T>
static marie_status alloc_workspace(marie_vie* h, PrecState<T>& ps) {
  const int64_t per = (int64_t)h->C * h->n3 * h->n2 * 2 * h->n1;  // T1 per rhs
  int ws = std::max(1, std::min(h->max_rhs, env_int("MARIE_WS_RHS", 16)));
  const int Wz = ps.TX;
  if (ws > Wz) ws = (ws + Wz - 1) / Wz * Wz;   // whole bundles
  ps.ws_rhs = ws;
  const int64_t alloc = (int64_t)(ws + Wz - 1) / Wz * Wz;   // any chunk of <= ws rhs fits whole bundles
  ps.ws_cap = (int)alloc;
  MARIE_TRY(dev_alloc(h, (void**)&ps.T1, (size_t)alloc * per * sizeof(cplx<T>)));
  MARIE_TRY(dev_alloc(h, (void**)&ps.S, (size_t)alloc * per * 2 * sizeof(cplx<T>)));
  return MARIE_OK;
}

template <typename T>
static marie_status launch_matvec_ev(marie_vie* h, int mode, int op, const cplx<typename IoOf<T>::type>* in,
                                     int64_t in_rs, cplx<typename IoOf<T>::type>* out, int64_t out_rs, int nrhs,
                                     const unsigned char* active, cudaStream_t stream, cudaEvent_t* ev,
                                     const cplx<typename IoOf<T>::type>* addend = nullptr);

template <typename T, bool PWL, int OP>
static void launch_z(const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s) {
  static std::atomic<uint64_t> done{0};
  smem_opt_in_device((const void*)k_z<T, PWL, OP>, done);
  k_z<T, PWL, OP><<<g, 256, smem, s>>>(a);
}

template <typename T>
static void dispatch_z(bool pwl, int op, const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s) {
  if (pwl) {
    switch (op) {
      case OP_N: launch_z<T, true, 0>(a, g, smem, s); break;
      case OP_N_ADJ: launch_z<T, true, 1>(a, g, smem, s); break;
      case OP_K: launch_z<T, true, 2>(a, g, smem, s); break;
      default: launch_z<T, true, 3>(a, g, smem, s); break;
    }
  } else {
    switch (op) {
      case OP_N: launch_z<T, false, 0>(a, g, smem, s); break;
      case OP_N_ADJ: launch_z<T, false, 1>(a, g, smem, s); break;
      case OP_K: launch_z<T, false, 2>(a, g, smem, s); break;
      default: launch_z<T, false, 3>(a, g, smem, s); break;
    }
  }
}

// complex128 calls run on the float-float state when the handle was built
// with it instead of native FP64 (precisions bit 4).
static bool c128_is_ff(const marie_vie* h) { return !h->p64.built && h->pff.built; }

template <typename T>
marie_status launch_matvec(marie_vie* h, int mode, int op, const cplx<T>* in, int64_t in_rs, cplx<T>* out,
                           int64_t out_rs, int nrhs, const unsigned char* active, cudaStream_t stream) {
  if constexpr (std::is_same<T, double>::value) {
    if (c128_is_ff(h)) return launch_matvec_ev<ff>(h, mode, op, in, in_rs, out, out_rs, nrhs, active, stream, nullptr);
  }
  return launch_matvec_ev<T>(h, mode, op, in, in_rs, out, out_rs, nrhs, active, stream, nullptr);
}

// ev (optional): 6 events recorded around the 5 passes of the first chunk.
template <typename T>
static marie_status launch_matvec_ev(marie_vie* h, int mode, int op, const cplx<typename IoOf<T>::type>* in,
                                     int64_t in_rs, cplx<typename IoOf<T>::type>* out, int64_t out_rs, int nrhs,
                                     const unsigned char* active, cudaStream_t stream, cudaEvent_t* ev,
                                     const cplx<typename IoOf<T>::type>* addend) {
  PrecState<T>& ps = prec_state<T>(h);
  if (!ps.built) {
    set_error("precision not built for this handle");
    return MARIE_ERR_BAD_ARG;
  }
  const bool isK = op == OP_K || op == OP_K_ADJ;
  if (isK && !h->has_K) {
    set_error("K operator was not supplied at create time");
    return MARIE_ERR_BAD_ARG;
  }
  static std::atomic<uint64_t> done[8];
  smem_opt_in_device((const void*)k_fwd_x<float>, done[0]);
  smem_opt_in_device((const void*)k_fwd_y<float>, done[1]);
  smem_opt_in_device((const void*)k_inv_y<float>, done[2]);
  smem_opt_in_device((const void*)k_inv_x<float>, done[3]);
  smem_opt_in_device((const void*)k_fwd_x<double>, done[4]);
  smem_opt_in_device((const void*)k_fwd_y<double>, done[5]);
  smem_opt_in_device((const void*)k_inv_y<double>, done[6]);
  smem_opt_in_device((const void*)k_inv_x<double>, done[7]);
  MvArgs<T> a;
  memset(&a, 0, sizeof(a));
  a.n1 = h->n1;
  a.n2 = h->n2;
  a.n3 = h->n3;
  a.C = h->C;
  a.Ns = h->Ns;
  a.mode = mode;
  fill_axis(a.ax, ps.ax);
  fill_axis(a.ay, ps.ay);
  fill_axis(a.az, ps.az);
  a.vox2sol = h->vox2sol;
  if (mode != MV_GRID && !env_int("MARIE_NO_PRUNE", 0)) {
    a.row_live = h->row_live;
    a.z_live = h->z_live;
    a.rowq = h->rowq;
    a.zq = h->zq;
  }
  a.chi = ps.chi;
  for (int c = 0; c < h->C; ++c) a.invg[c] = prec_from<T>(h->invg[c]);
  a.efac = cplx<T>{prec_from<T>(0.0L), prec_from<T>(-1.0L / (long double)h->ce_im)};   // 1/ce, ce = i*omega*eps0
  a.T1 = ps.T1;
  a.S = ps.S;
  a.G = isK ? ps.GK : ps.GN;   // octant spectra (generic path); the four-step path below uses GNf
  a.in_rs = in_rs;
  a.out_rs = out_rs;
  const int n1 = h->n1, n2 = h->n2, n3 = h->n3, C = h->C;
  const size_t sz = sizeof(cplx<T>);
  if constexpr (std::is_same<T, float>::value) {
    // the reference's form: the Tucker blocks re-expanded for this application
    if (h->tkf.active && (op == OP_N || op == OP_N_ADJ) && !env_int("MARIE_GENERIC_FFT", 0))
      MARIE_TRY(tucker_expand_c64(h, stream));
  }
  for (int r0 = 0; r0 < nrhs; r0 += ps.ws_rhs) {
    const int nr = std::min(ps.ws_rhs, nrhs - r0);
    const bool fast = four_step_edge(n1) && four_step_edge(n2) && four_step_edge(n3) &&
                      (op == OP_N || op == OP_N_ADJ) && !env_int("MARIE_GENERIC_FFT", 0);
    const CallTiles ct = call_tiles(h, ps, nr, fast);
    const int nb = (nr + ct.R - 1) / ct.R;
    a.R = ct.R;
    a.lgR = 0;
    while ((1 << a.lgR) < a.R) ++a.lgR;
    a.TY = ct.TY;
    a.TXY = ct.TXY;
    a.TX = ct.TX;
    a.nrhs = nr;
    a.in = in + (int64_t)r0 * in_rs;
    a.out = out + (int64_t)r0 * out_rs;
    a.active = active ? active + r0 : nullptr;
    a.addend = addend ? addend + (int64_t)r0 * out_rs : nullptr;
    if (fast) {
      a.G = ps.GNf;
      MARIE_TRY(launch_fast_chunk<T>(h, op, a, nb, stream, (ev && r0 == 0) ? ev : nullptr));
      continue;
    }
    if constexpr (std::is_same<T, ff>::value) {
      set_error("the float-float complex128 operator covers N and N^H on grids with edges 16*NB (NB <= 8); "
                "build the handle with native complex128 (precisions bit 1) for this call");
      return MARIE_ERR_NOT_SUPPORTED;
    } else {
    const size_t smx = (size_t)(n1 + (size_t)n1 * (2 * a.TY * a.R + 1)) * sz;
    const size_t smy = (size_t)(n2 + (size_t)n2 * (2 * a.TXY * a.R + 1)) * sz;
    const size_t smz = (size_t)(n3 + (size_t)n3 * (2 * C * a.TX * a.R + 1)) * sz;
    dim3 gx((n2 + a.TY - 1) / a.TY, n3, nb * C);
    dim3 gy((2 * n1 + a.TXY - 1) / a.TXY, n3, nb * C);
    dim3 gz((2 * n1 + a.TX - 1) / a.TX, 2 * n2, nb);
    const bool rec = ev && r0 == 0;
    if (rec) cudaEventRecord(ev[0], stream);
    k_fwd_x<T><<<gx, 256, smx, stream>>>(a);
    MARIE_LAUNCH_CHECK();
    if (rec) cudaEventRecord(ev[1], stream);
    k_fwd_y<T><<<gy, 256, smy, stream>>>(a);
    MARIE_LAUNCH_CHECK();
    if (rec) cudaEventRecord(ev[2], stream);
    dispatch_z<T>(h->pwl != 0, op, a, gz, smz, stream);
    MARIE_LAUNCH_CHECK();
    if (rec) cudaEventRecord(ev[3], stream);
    k_inv_y<T><<<gy, 256, smy, stream>>>(a);
    MARIE_LAUNCH_CHECK();
    if (rec) cudaEventRecord(ev[4], stream);
    k_inv_x<T><<<gx, 256, smx, stream>>>(a);
    MARIE_LAUNCH_CHECK();
    if (rec) cudaEventRecord(ev[5], stream);
    }
  }
  return MARIE_OK;
}

template <typename T>
marie_status launch_matvec_fields(marie_vie* h, int mode, int op, const cplx<T>* in, cplx<T>* out,
                                  const cplx<T>* addend, int nrhs, cudaStream_t stream) {
  if constexpr (std::is_same<T, double>::value) {
    if (c128_is_ff(h))
      return launch_matvec_ev<ff>(h, mode, op, in, h->Nb, out, h->Nb, nrhs, nullptr, stream, nullptr, addend);
  }
  return launch_matvec_ev<T>(h, mode, op, in, h->Nb, out, h->Nb, nrhs, nullptr, stream, nullptr, addend);
}
template marie_status launch_matvec_fields<float>(marie_vie*, int, int, const cplx<float>*, cplx<float>*,
                                                  const cplx<float>*, int, cudaStream_t);
template marie_status launch_matvec_fields<double>(marie_vie*, int, int, const cplx<double>*, cplx<double>*,
                                                   const cplx<double>*, int, cudaStream_t);

template marie_status launch_matvec<float>(marie_vie*, int, int, const cplx<float>*, int64_t, cplx<float>*, int64_t,
                                           int, const unsigned char*, cudaStream_t);
template marie_status launch_matvec<double>(marie_vie*, int, int, const cplx<double>*, int64_t, cplx<double>*,
                                            int64_t, int, const unsigned char*, cudaStream_t);

// Body-voxel material data from Mr per body voxel: the contrast
// chi = (1./Mr).*Mc (mvp_vie.m:17), the absorbed-power weight
// real(Mc_inv/ce) (em_ehfield_vie.m:46; 0 where Mc = 0) and Mr itself.
static marie_status body_materials(const marie_vie* h, const std::complex<double>* mr, std::vector<cplx<double>>& chi,
                                   std::vector<double>& wpow, std::vector<cplx<double>>& mrb) {
  chi.resize(h->Ns);
  wpow.resize(h->Ns);
  mrb.resize(h->Ns);
  for (int64_t s = 0; s < h->Ns; ++s) {
    const std::complex<double> Mr = mr[s];
    if (!std::isfinite(Mr.real()) || !std::isfinite(Mr.imag()) || Mr == 0.0) {
      set_error("Mr is zero or non-finite at body voxel %lld", (long long)s);
      return MARIE_ERR_NONFINITE;
    }
    const std::complex<double> Mc = Mr - 1.0;
    const std::complex<double> v = (1.0 / Mr) * Mc;
    chi[s] = cplx<double>{v.real(), v.imag()};
    wpow[s] = Mc == 0.0 ? 0.0 : ((1.0 / Mc) / std::complex<double>(0.0, h->ce_im)).real();
    mrb[s] = cplx<double>{Mr.real(), Mr.imag()};
  }
  return MARIE_OK;
}

// Upload the contrast of every built precision (create and material updates).
static marie_status upload_chi(marie_vie* h, const std::vector<cplx<double>>& chi) {
  if (h->p64.chi) MARIE_CUDA_TRY(cudaMemcpy(h->p64.chi, chi.data(), h->Ns * sizeof(cplx<double>), cudaMemcpyHostToDevice));
  if (h->p32.chi) {
    std::vector<cplx<float>> f(h->Ns);
    for (int64_t s = 0; s < h->Ns; ++s) f[s] = cplx<float>{(float)chi[s].x, (float)chi[s].y};
    MARIE_CUDA_TRY(cudaMemcpy(h->p32.chi, f.data(), h->Ns * sizeof(cplx<float>), cudaMemcpyHostToDevice));
  }
  if (h->pff.chi) {
    std::vector<cplx<ff>> f(h->Ns);
    for (int64_t s = 0; s < h->Ns; ++s) f[s] = cplx<ff>{prec_from<ff>(chi[s].x), prec_from<ff>(chi[s].y)};
    MARIE_CUDA_TRY(cudaMemcpy(h->pff.chi, f.data(), h->Ns * sizeof(cplx<ff>), cudaMemcpyHostToDevice));
  }
  return MARIE_OK;
}

}  // namespace marie

using namespace marie;

static marie_status validate_desc(const marie_vie_desc* d, std::vector<int64_t>& idxS) {
  if (!d) { set_error("desc is NULL"); return MARIE_ERR_BAD_ARG; }
  if (d->n1 < 1 || d->n2 < 1 || d->n3 < 1 || d->n1 > kMaxAxis || d->n2 > kMaxAxis || d->n3 > kMaxAxis) {
    set_error("grid edges must be in [1, %d], got %d x %d x %d", kMaxAxis, d->n1, d->n2, d->n3);
    return MARIE_ERR_BAD_ARG;
  }
  if (d->basis != MARIE_PWC && d->basis != MARIE_PWL) { set_error("basis must be 0 (PWC) or 1 (PWL)"); return MARIE_ERR_BAD_ARG; }
  if (!(d->res > 0) || !std::isfinite(d->res)) { set_error("res must be a positive finite number"); return MARIE_ERR_BAD_ARG; }
  if (!(d->freq > 0) || !std::isfinite(d->freq)) { set_error("freq must be a positive finite number"); return MARIE_ERR_BAD_ARG; }
  if (!d->idx_solution || d->n_b <= 0) { set_error("idx_solution is empty"); return MARIE_ERR_BAD_ARG; }
  if (!d->Mr) { set_error("Mr is NULL"); return MARIE_ERR_BAD_ARG; }
  if (!d->tucker_N && !d->dense_N) { set_error("neither tucker_N nor dense_N given"); return MARIE_ERR_BAD_ARG; }
  if (d->precisions < 1 || d->precisions > 15 || !(d->precisions & 7)) {
    set_error("precisions must be a mask of bits 1, 2, 4 (at least one) and 8");
    return MARIE_ERR_BAD_ARG;
  }
  if ((d->precisions & 8) && (!d->tucker_N || !(d->precisions & 2))) {
    set_error("precisions bit 8 (per-application Tucker expansion) needs tucker_N and the complex64 state (bit 2)");
    return MARIE_ERR_BAD_ARG;
  }
  if ((d->precisions & 1) && (d->precisions & 4)) {
    set_error("precisions bits 1 (native complex128) and 4 (float-float complex128) are exclusive");
    return MARIE_ERR_BAD_ARG;
  }
  if ((d->precisions & 4) && !(four_step_edge(d->n1) && four_step_edge(d->n2) && four_step_edge(d->n3))) {
    set_error("float-float complex128 (precisions bit 4) needs grid edges 16*NB with NB <= 8, got %d x %d x %d",
              d->n1, d->n2, d->n3);
    return MARIE_ERR_NOT_SUPPORTED;
  }
  if (d->max_rhs < 1) { set_error("max_rhs must be >= 1"); return MARIE_ERR_BAD_ARG; }
  const int C = d->basis == MARIE_PWL ? 12 : 3;
  if (d->n_b % C != 0) { set_error("n_b=%lld is not a multiple of %d components", (long long)d->n_b, C); return MARIE_ERR_BAD_ARG; }
  const int64_t Ns = d->n_b / C;
  const int64_t nD = (int64_t)d->n1 * d->n2 * d->n3;
  if (Ns > nD) { set_error("more body voxels than grid voxels"); return MARIE_ERR_BAD_ARG; }
  idxS.assign(d->idx_solution, d->idx_solution + Ns);
  for (int64_t s = 0; s < Ns; ++s)
    if (idxS[s] < 0 || idxS[s] >= nD) {
      set_error("idx_solution[%lld]=%lld outside the grid", (long long)s, (long long)idxS[s]);
      return MARIE_ERR_BAD_ARG;
    }
  for (int c = 1; c < C; ++c)
    for (int64_t s = 0; s < Ns; ++s)
      if (d->idx_solution[c * Ns + s] != c * nD + idxS[s]) {
        set_error("idx_solution is not component-major (block %d, entry %lld)", c, (long long)s);
        return MARIE_ERR_BAD_ARG;
      }
  return MARIE_OK;
}

// Handle for a grid the FFT passes take as given (marie_vie_create decides
// whether the caller's grid is first embedded in a larger one, embed.h).
static marie_status create_grid(marie_vie** out, const marie_vie_desc* d) {
  if (!out) { set_error("output handle pointer is NULL"); return MARIE_ERR_BAD_ARG; }
  *out = nullptr;
  std::vector<int64_t> idxS;
  MARIE_TRY(validate_desc(d, idxS));
  marie_vie* h = new (std::nothrow) marie_vie();
  if (!h) { set_error("host allocation failed"); return MARIE_ERR_OOM; }
  h->n1 = d->n1; h->n2 = d->n2; h->n3 = d->n3;
  h->pwl = d->basis == MARIE_PWL;
  h->C = h->pwl ? 12 : 3;
  h->res = d->res;
  h->freq = d->freq;
  const double mu0 = 4e-7 * M_PI, c0 = 299792458.0;
  const double e0 = 1.0 / (c0 * c0 * mu0);
  h->omega = 2 * M_PI * d->freq;
  h->ce_im = h->omega * e0;    // ce = i*omega*eps0 (em_constants.m)
  h->k0 = 2 * M_PI / (c0 / d->freq);
  h->Nb = d->n_b;
  h->Ns = d->n_b / h->C;
  h->max_rhs = d->max_rhs;
  h->precisions = d->precisions;
  h->mem_cap = d->mem_cap_bytes;
  h->has_K = (d->tucker_K || d->dense_K) ? 1 : 0;
  h->nblkN = (h->pwl ? 10 : 1) * 6;
  h->nblkK = (h->pwl ? 10 : 1) * 3;
  h->idxS_host = idxS;
  const double r3 = d->res * d->res * d->res;
  for (int c = 0; c < h->C; ++c) h->invg[c] = (h->pwl && (c % 4) != 0) ? 1.0 / (r3 / 12.0) : 1.0 / r3;
  make_tables(h);
  auto fail = [&](marie_status s) {
    dev_free_all(h);
    delete h;
    return s;
  };
  if (cudaGetDevice(&h->device) != cudaSuccess) {
    cudaGetLastError();
    set_error("no CUDA device available");
    return fail(MARIE_ERR_CUDA);
  }
  // body map
  const int64_t nD = (int64_t)h->n1 * h->n2 * h->n3;
  std::vector<int> vox(nD, -1);
  for (int64_t s = 0; s < h->Ns; ++s) {
    if (vox[idxS[s]] != -1) { set_error("idx_solution lists voxel %lld twice", (long long)idxS[s]); return fail(MARIE_ERR_BAD_ARG); }
    vox[idxS[s]] = (int)s;
  }
  marie_status st;
  if ((st = dev_alloc(h, (void**)&h->vox2sol, nD * sizeof(int))) != MARIE_OK) return fail(st);
  if (cudaMemcpy(h->vox2sol, vox.data(), nD * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
    set_error("upload of the body map failed");
    return fail(MARIE_ERR_CUDA);
  }
  {
    std::vector<unsigned char> rl((size_t)h->n2 * h->n3, 0), zl(h->n3, 0);
    for (int64_t s = 0; s < h->Ns; ++s) {
      const int64_t yz = idxS[s] / h->n1;          // y + n2*z
      rl[yz] = 1;
      zl[yz / h->n2] = 1;
    }
    if ((st = dev_alloc(h, (void**)&h->row_live, rl.size())) != MARIE_OK) return fail(st);
    if ((st = dev_alloc(h, (void**)&h->z_live, zl.size())) != MARIE_OK) return fail(st);
    cudaMemcpy(h->row_live, rl.data(), rl.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(h->z_live, zl.data(), zl.size(), cudaMemcpyHostToDevice);
    if (four_step_edge(h->n2)) {
      const int nb = h->n2 / 16;
      std::vector<uint16_t> rq((size_t)h->n3 * 8, 0);
      for (int z = 0; z < h->n3; ++z)
        for (int b = 0; b < nb; ++b)
          for (int q = 0; q < 16; ++q)
            if (rl[(size_t)z * h->n2 + nb * q + b]) rq[(size_t)z * 8 + b] |= (uint16_t)(1u << q);
      if ((st = dev_alloc(h, (void**)&h->rowq, rq.size() * sizeof(uint16_t))) != MARIE_OK) return fail(st);
      cudaMemcpy(h->rowq, rq.data(), rq.size() * sizeof(uint16_t), cudaMemcpyHostToDevice);
    }
    if (four_step_edge(h->n3)) {
      const int nb = h->n3 / 16;
      std::vector<uint16_t> zq(8, 0);
      for (int b = 0; b < nb; ++b)
        for (int q = 0; q < 16; ++q)
          if (zl[nb * q + b]) zq[b] |= (uint16_t)(1u << q);
      if ((st = dev_alloc(h, (void**)&h->zq, zq.size() * sizeof(uint16_t))) != MARIE_OK) return fail(st);
      cudaMemcpy(h->zq, zq.data(), zq.size() * sizeof(uint16_t), cudaMemcpyHostToDevice);
    }
  }
  if ((st = dev_alloc(h, (void**)&h->idxS, h->Ns * sizeof(int64_t))) != MARIE_OK) return fail(st);
  cudaMemcpy(h->idxS, idxS.data(), h->Ns * sizeof(int64_t), cudaMemcpyHostToDevice);
  // contrast chi = (1./Mr).*Mc on the body (mvp_vie.m:17)
  std::vector<cplx<double>> chi;
  std::vector<double> wpow;
  std::vector<cplx<double>> mrb;
  {
    std::vector<std::complex<double>> mr(h->Ns);
    for (int64_t s = 0; s < h->Ns; ++s) mr[s] = {d->Mr[2 * idxS[s]], d->Mr[2 * idxS[s] + 1]};
    if ((st = body_materials(h, mr.data(), chi, wpow, mrb)) != MARIE_OK) return fail(st);
  }
  if ((st = dev_alloc(h, (void**)&h->mr_body, h->Ns * sizeof(cplx<double>))) != MARIE_OK) return fail(st);
  cudaMemcpy(h->mr_body, mrb.data(), h->Ns * sizeof(cplx<double>), cudaMemcpyHostToDevice);
  if ((st = dev_alloc(h, (void**)&h->wpow, h->Ns * sizeof(double))) != MARIE_OK) return fail(st);
  cudaMemcpy(h->wpow, wpow.data(), h->Ns * sizeof(double), cudaMemcpyHostToDevice);
  (void)e0;
  for (int pr = 0; pr < 3; ++pr) {
    if (!(d->precisions & (1 << pr))) continue;
    if (pr == 2) {
      PrecState<ff>& ps = h->pff;
      if ((st = build_axis(h, h->n1, ps.ax)) != MARIE_OK) return fail(st);
      if ((st = build_axis(h, h->n2, ps.ay)) != MARIE_OK) return fail(st);
      if ((st = build_axis(h, h->n3, ps.az)) != MARIE_OK) return fail(st);
      std::vector<cplx<ff>> chiff(h->Ns);
      for (int64_t s = 0; s < h->Ns; ++s) chiff[s] = cplx<ff>{prec_from<ff>(chi[s].x), prec_from<ff>(chi[s].y)};
      if ((st = dev_alloc(h, (void**)&ps.chi, h->Ns * sizeof(cplx<ff>))) != MARIE_OK) return fail(st);
      cudaMemcpy(ps.chi, chiff.data(), h->Ns * sizeof(cplx<ff>), cudaMemcpyHostToDevice);
      if ((st = choose_tiles(h, ps)) != MARIE_OK) return fail(st);
      if ((st = alloc_workspace(h, ps)) != MARIE_OK) return fail(st);
    } else if (pr == 0) {
      PrecState<double>& ps = h->p64;
      if ((st = build_axis(h, h->n1, ps.ax)) != MARIE_OK) return fail(st);
      if ((st = build_axis(h, h->n2, ps.ay)) != MARIE_OK) return fail(st);
      if ((st = build_axis(h, h->n3, ps.az)) != MARIE_OK) return fail(st);
      if ((st = dev_alloc(h, (void**)&ps.chi, h->Ns * sizeof(cplx<double>))) != MARIE_OK) return fail(st);
      cudaMemcpy(ps.chi, chi.data(), h->Ns * sizeof(cplx<double>), cudaMemcpyHostToDevice);
      if ((st = choose_tiles(h, ps)) != MARIE_OK) return fail(st);
      if ((st = alloc_workspace(h, ps)) != MARIE_OK) return fail(st);
    } else {
      PrecState<float>& ps = h->p32;
      if ((st = build_axis(h, h->n1, ps.ax)) != MARIE_OK) return fail(st);
      if ((st = build_axis(h, h->n2, ps.ay)) != MARIE_OK) return fail(st);
      if ((st = build_axis(h, h->n3, ps.az)) != MARIE_OK) return fail(st);
      std::vector<cplx<float>> chif(h->Ns);
      for (int64_t s = 0; s < h->Ns; ++s) chif[s] = cplx<float>{(float)chi[s].x, (float)chi[s].y};
      if ((st = dev_alloc(h, (void**)&ps.chi, h->Ns * sizeof(cplx<float>))) != MARIE_OK) return fail(st);
      cudaMemcpy(ps.chi, chif.data(), h->Ns * sizeof(cplx<float>), cudaMemcpyHostToDevice);
      if ((st = choose_tiles(h, ps)) != MARIE_OK) return fail(st);
      if ((st = alloc_workspace(h, ps)) != MARIE_OK) return fail(st);
    }
  }
  if ((st = build_spectra(h, d)) != MARIE_OK) return fail(st);
  if (d->precisions & 8) {
    if (!four_step_grid(h)) {
      set_error("precisions bit 8 needs a grid with edges 16*NB, NB <= 8 (the four-step complex64 path)");
      return fail(MARIE_ERR_BAD_ARG);
    }
    if ((st = tucker_keep_c64(h, d->tucker_N)) != MARIE_OK) return fail(st);
  }
  if (h->precisions & 1) h->p64.built = true;
  if (h->precisions & 2) h->p32.built = true;
  if (h->precisions & 4) h->pff.built = true;
  if (cudaDeviceSynchronize() != cudaSuccess) {
    set_error("device error during create: %s", cudaGetErrorString(cudaGetLastError()));
    return fail(MARIE_ERR_CUDA);
  }
  *out = h;
  return MARIE_OK;
}

// Autotuner of the z-pass tile width: time `reps` applications of mvp_vie
// on x (nrhs right-hand sides) for every power-of-two width whose shared
// memory fits a CTA and whose bundles fit the work arrays, keep the fastest.
template <typename T>
static marie_status autotune_state(marie_vie* h, PrecState<T>& ps, const void* x, void* y, int nrhs, int reps,
                                   cudaStream_t s, int32_t* widths, double* ms, int32_t cap, int32_t* count) {
  const int C = h->C;
  const size_t sz = sizeof(cplx<T>);
  const bool fast = four_step_grid(h) && !env_int("MARIE_GENERIC_FFT", 0);
  const int keep = ps.TX;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  int best = keep, n = 0;
  double best_ms = 1e300;
  marie_status st = MARIE_OK;
  for (int W = 1; W <= 16 && st == MARIE_OK; W *= 2) {
    if ((ps.ws_rhs + W - 1) / W * W > ps.ws_cap) continue;
    if (fast) {
      if (kz4_smem<T>(h->n3, C, W) > kSmemOptin) continue;
    } else {
      const GenericSmem g = generic_smem(h->n1, h->n2, h->n3, C, sz, 1, 1, 1, W);
      if (g.x > kSmemOptin || g.y > kSmemOptin || g.z > kSmemOptin) continue;
    }
    ps.TX = W;
    float total = 0;
    for (int r = 0; r <= reps && st == MARIE_OK; ++r) {     // r = 0: warm-up
      cudaEventRecord(t0, s);
      st = launch_matvec_ev<T>(h, MV_VIE, OP_N, (const cplx<typename IoOf<T>::type>*)x, h->Nb,
                               (cplx<typename IoOf<T>::type>*)y, h->Nb, nrhs, nullptr, s, nullptr);
      cudaEventRecord(t1, s);
      if (cudaEventSynchronize(t1) != cudaSuccess) { set_error("autotune: device error"); st = MARIE_ERR_CUDA; }
      float v = 0;
      cudaEventElapsedTime(&v, t0, t1);
      if (r > 0) total += v;
    }
    if (st != MARIE_OK) break;
    const double avg = total / reps;
    if (n < cap) {
      widths[n] = W;
      ms[n] = avg;
    }
    ++n;
    if (avg < best_ms) { best_ms = avg; best = W; }
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  ps.TX = st == MARIE_OK ? best : keep;
  *count = n;
  return st;
}

extern "C" {

marie_status marie_vie_create(marie_vie** out, const marie_vie_desc* d) {
  if (!out) { set_error("output handle pointer is NULL"); return MARIE_ERR_BAD_ARG; }
  *out = nullptr;
  if (!d) { set_error("desc is NULL"); return MARIE_ERR_BAD_ARG; }
  const int n[3] = {d->n1, d->n2, d->n3};
  int m[3] = {d->n1, d->n2, d->n3};
  const bool in_range = n[0] >= 1 && n[1] >= 1 && n[2] >= 1 && n[0] <= kMaxAxis && n[1] <= kMaxAxis &&
                        n[2] <= kMaxAxis;
  // MARIE_EMBED=1: embed every grid with edges <= 128 in the four-step grid
  // (edges rounded up to 16*NB) even where the generic passes would run it
  if (!in_range || !embed::embed_dims(n, env_int("MARIE_EMBED", 0) != 0, m)) return create_grid(out, d);
  // Validate the caller's descriptor on the caller's grid; the float-float
  // edge rule applies to the embedded grid and is checked there.
  marie_vie_desc dv = *d;
  if ((dv.precisions & 4) && !(dv.precisions & 1)) dv.precisions = (dv.precisions & ~4) | 2;
  std::vector<int64_t> idxS;
  MARIE_TRY(validate_desc(&dv, idxS));
  embed::Buffers buf;
  marie_vie_desc e;
  embed::embed_desc(d, m, buf, &e);
  MARIE_TRY(create_grid(out, &e));
  (*out)->on1 = n[0];
  (*out)->on2 = n[1];
  (*out)->on3 = n[2];
  return MARIE_OK;
}

marie_status marie_vie_info(marie_vie* h, int64_t* out) {
  if (!h || !out) { set_error("info: NULL argument"); return MARIE_ERR_BAD_ARG; }
  out[0] = h->on1 ? h->on1 : h->n1;
  out[1] = h->on1 ? h->on2 : h->n2;
  out[2] = h->on1 ? h->on3 : h->n3;
  out[3] = h->C;
  out[4] = h->Ns;
  out[5] = h->Nb;
  return MARIE_OK;
}

marie_status marie_vie_set_materials(marie_vie* h, const double* Mr_body) {
  if (!h || !Mr_body) { set_error("set_materials: NULL argument"); return MARIE_ERR_BAD_ARG; }
  std::vector<std::complex<double>> mr(h->Ns);
  for (int64_t s = 0; s < h->Ns; ++s) mr[s] = {Mr_body[2 * s], Mr_body[2 * s + 1]};
  std::vector<cplx<double>> chi, mrb;
  std::vector<double> wpow;
  MARIE_TRY(body_materials(h, mr.data(), chi, wpow, mrb));
  MARIE_CUDA_TRY(cudaDeviceSynchronize());   // no kernel may still read the old values
  MARIE_TRY(upload_chi(h, chi));
  MARIE_CUDA_TRY(cudaMemcpy(h->wpow, wpow.data(), h->Ns * sizeof(double), cudaMemcpyHostToDevice));
  MARIE_CUDA_TRY(cudaMemcpy(h->mr_body, mrb.data(), h->Ns * sizeof(cplx<double>), cudaMemcpyHostToDevice));
  return MARIE_OK;
}

marie_status marie_vie_release_workspace(marie_vie* h) {
  if (!h) { set_error("handle is NULL"); return MARIE_ERR_BAD_ARG; }
  cudaDeviceSynchronize();
  graphs_free(h);     // they capture workspace pointers
  for (auto* pool : {&h->gm_pool, &h->io_pool}) {
    for (auto& e : *pool) {
      cudaFree(e.first);
      h->mem_used -= (int64_t)e.second;
    }
    pool->clear();
  }
  return MARIE_OK;
}

marie_status marie_vie_destroy(marie_vie* h) {
  if (!h) return MARIE_OK;
  dev_free_all(h);
  delete h;
  return MARIE_OK;
}

static marie_status apply_common(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, void* stream,
                                 int mode, int op) {
  if (!h) { set_error("handle is NULL"); return MARIE_ERR_BAD_ARG; }
  if (!x || !y) { set_error("x or y is NULL"); return MARIE_ERR_BAD_ARG; }
  if (nrhs < 1) { set_error("nrhs must be >= 1"); return MARIE_ERR_BAD_ARG; }
  if (prec != MARIE_C128 && prec != MARIE_C64) { set_error("prec must be MARIE_C128 or MARIE_C64"); return MARIE_ERR_BAD_ARG; }
  if (mode == MV_GRID && h->on1) {
    set_error("operators on full grids are not available on this handle: its %d x %d x %d grid was embedded in "
              "%d x %d x %d (an edge has a prime factor above 31, or MARIE_EMBED was set); body-vector "
              "operators, solves and fields are", h->on1, h->on2, h->on3, h->n1, h->n2, h->n3);
    return MARIE_ERR_NOT_SUPPORTED;
  }
  const int64_t len = mode == MV_GRID ? (int64_t)h->C * h->n1 * h->n2 * h->n3 : h->Nb;
  cudaStream_t s = (cudaStream_t)stream;
  if (prec == MARIE_C128)
    return launch_matvec<double>(h, mode, op, (const cplx<double>*)x, len, (cplx<double>*)y, len, nrhs, nullptr, s);
  return launch_matvec<float>(h, mode, op, (const cplx<float>*)x, len, (cplx<float>*)y, len, nrhs, nullptr, s);
}

marie_status marie_vie_apply(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, void* stream) {
  return apply_common(h, prec, x, y, nrhs, stream, MV_VIE, OP_N);
}
marie_status marie_vie_apply_adjoint(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, void* stream) {
  return apply_common(h, prec, x, y, nrhs, stream, MV_VIE_ADJ, OP_N_ADJ);
}
marie_status marie_vie_apply_N(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, void* stream) {
  return apply_common(h, prec, x, y, nrhs, stream, MV_GRID, OP_N);
}
marie_status marie_vie_apply_N_adj(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, void* stream) {
  return apply_common(h, prec, x, y, nrhs, stream, MV_GRID, OP_N_ADJ);
}
marie_status marie_vie_apply_K(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, void* stream) {
  return apply_common(h, prec, x, y, nrhs, stream, MV_GRID, OP_K);
}
marie_status marie_vie_apply_K_adj(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, void* stream) {
  return apply_common(h, prec, x, y, nrhs, stream, MV_GRID, OP_K_ADJ);
}
marie_status marie_vie_apply_hfield_adjoint(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs,
                                            void* stream) {
  return apply_common(h, prec, x, y, nrhs, stream, MV_HFIELD_ADJ, OP_K_ADJ);
}

marie_status marie_vie_profile(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, int32_t reps,
                               double* ms, void* stream) {
  if (!h || !x || !y || !ms || nrhs < 1 || reps < 1) { set_error("marie_vie_profile: invalid argument"); return MARIE_ERR_BAD_ARG; }
  if (prec != MARIE_C128 && prec != MARIE_C64) { set_error("prec must be MARIE_C128 or MARIE_C64"); return MARIE_ERR_BAD_ARG; }
  cudaStream_t s = (cudaStream_t)stream;
  cudaEvent_t ev[6], t0, t1;
  for (int i = 0; i < 6; ++i) cudaEventCreate(&ev[i]);
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  double acc[6] = {0, 0, 0, 0, 0, 0};
  marie_status st = MARIE_OK;
  for (int r = 0; r < reps && st == MARIE_OK; ++r) {
    cudaEventRecord(t0, s);
    if (prec == MARIE_C128 && c128_is_ff(h))
      st = launch_matvec_ev<ff>(h, MV_VIE, OP_N, (const cplx<double>*)x, h->Nb, (cplx<double>*)y, h->Nb, nrhs,
                                nullptr, s, ev);
    else if (prec == MARIE_C128)
      st = launch_matvec_ev<double>(h, MV_VIE, OP_N, (const cplx<double>*)x, h->Nb, (cplx<double>*)y, h->Nb, nrhs,
                                    nullptr, s, ev);
    else
      st = launch_matvec_ev<float>(h, MV_VIE, OP_N, (const cplx<float>*)x, h->Nb, (cplx<float>*)y, h->Nb, nrhs,
                                   nullptr, s, ev);
    cudaEventRecord(t1, s);
    if (cudaEventSynchronize(t1) != cudaSuccess) { set_error("profile: device error"); st = MARIE_ERR_CUDA; break; }
    for (int i = 0; i < 5; ++i) {
      float v = 0;
      cudaEventElapsedTime(&v, ev[i], ev[i + 1]);
      acc[i] += v;
    }
    float w = 0;
    cudaEventElapsedTime(&w, t0, t1);
    acc[5] += w;
  }
  for (int i = 0; i < 6; ++i) ms[i] = acc[i] / reps;
  for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  return st;
}

marie_status marie_vie_autotune(marie_vie* h, int32_t prec, const void* x, void* y, int32_t nrhs, int32_t reps,
                                int32_t* widths, double* ms, int32_t cap, int32_t* count, void* stream) {
  if (!h || !x || !y || nrhs < 1 || reps < 1 || !count || (cap > 0 && (!widths || !ms))) {
    set_error("marie_vie_autotune: invalid argument");
    return MARIE_ERR_BAD_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (prec == MARIE_C64) {
    if (!h->p32.built) { set_error("autotune: no complex64 state"); return MARIE_ERR_BAD_ARG; }
    return autotune_state<float>(h, h->p32, x, y, nrhs, reps, s, widths, ms, cap, count);
  }
  if (prec != MARIE_C128) { set_error("prec must be MARIE_C128 or MARIE_C64"); return MARIE_ERR_BAD_ARG; }
  if (c128_is_ff(h)) return autotune_state<ff>(h, h->pff, x, y, nrhs, reps, s, widths, ms, cap, count);
  if (!h->p64.built) { set_error("autotune: no complex128 state"); return MARIE_ERR_BAD_ARG; }
  return autotune_state<double>(h, h->p64, x, y, nrhs, reps, s, widths, ms, cap, count);
}

marie_status marie_vie_tiles(marie_vie* h, int32_t prec, int32_t* out) {
  if (!h || !out) { set_error("marie_vie_tiles: invalid argument"); return MARIE_ERR_BAD_ARG; }
  if (prec == MARIE_C128 && c128_is_ff(h)) { out[0] = h->pff.ws_rhs; out[1] = h->pff.TX; out[2] = 1; out[3] = 0; }
  else if (prec == MARIE_C128) { out[0] = h->p64.ws_rhs; out[1] = h->p64.TX; out[2] = 0; out[3] = 0; }
  else { out[0] = h->p32.ws_rhs; out[1] = h->p32.TX; out[2] = 0; out[3] = 0; }
  return MARIE_OK;
}

const char* marie_last_error(void) { return t_err.c_str(); }
const char* marie_version(void) { return "marie_gb300 0.1 (sm_103a)"; }
int64_t marie_launch_count(void) { return g_launches.load(); }

}  // extern "C"
