// Block GMRES: the inner complex64 solver of the mixed-precision refinement
// when the right-hand sides share one block Krylov space (marie_gmres_opts
// mode MARIE_SOLVE_MIXED_BLOCK).  Included by gmres.cu (it uses the solve's
// workspace pool and the true-residual loop there).
//
// The reference solves the ports one at a time (ie_solver_vie.m:16-21) with
// is_gmres_vie; this solver replaces the p per-port Krylov spaces of one
// refinement step by the block space span{R, A R, ..., A^(j) R} of all p
// residuals:
//
//   cycle:  R = V_0 S                      block QR (CholQR2)
//   step j: W = A V_j                      one operator application on p vectors
//           H_{0:j,j} = V_{0:j}^H W; W -= V_{0:j} H_{0:j,j}    block classical
//           Gram-Schmidt (one pass, or two with MARIE_BLOCK_CGS=2)
//           W = V_{j+1} H_{j+1,j}          block QR; H_{j+1,j} upper triangular
//           min_Y || [S;0] - Hbar_j Y ||_F column by column: Householder QR of the
//           block Hessenberg matrix (lower bandwidth p) on the host in FP64, the
//           residual norm of column c is the norm of rows (j+1)p..(j+2)p-1 of
//           the transformed right-hand side
//   end:    D = V_{0:j} Y, x += D (FP64); if not converged R = V_{0:j+1} Z with
//           Z = Q [0; G_bottom] and the next cycle starts from it.
//
// The projections, updates, Gram matrices and combinations are GEMMs of a
// tall (N_b rows) operand with (j+1)p or p columns: cuBLAS complex GEMMs on
// the tensor cores (FP32 emulated by BF16x9 products, FP32 accumulation;
// MARIE_BLOCK_GEMM=fp32 runs them on the FP32 pipe instead;
// MARIE_BLOCK_PROJ=tcgen05 runs the projections on bproj.cu's kernel).  The small
// p x p and (j+2)p x p matrices move through pinned, device-mapped host
// memory by a kernel (the status-channel discipline).
#include <chrono>
#include <cstdio>

#include <cublas_v2.h>

#include "blocklsq.h"

namespace marie {

// dst_c = (complex64) src_{map[c]}
__global__ void k_gather_block(const zd* __restrict__ src, int64_t srs, cplx<float>* __restrict__ dst, int64_t Nb,
                               const int* __restrict__ map) {
  const int c = blockIdx.y;
  const zd* s = src + (int64_t)map[c] * srs;
  cplx<float>* d = dst + (int64_t)c * Nb;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nb; i += (int64_t)gridDim.x * blockDim.x)
    d[i] = cplx<float>{(float)s[i].x, (float)s[i].y};
}

// x_{map[c]} += (FP64) D_c
__global__ void k_add_block(zd* __restrict__ x, int64_t xrs, const cplx<float>* __restrict__ D, int64_t Nb,
                            const int* __restrict__ map) {
  const int c = blockIdx.y;
  zd* xr = x + (int64_t)map[c] * xrs;
  const cplx<float>* d = D + (int64_t)c * Nb;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < Nb; i += (int64_t)gridDim.x * blockDim.x)
    xr[i] = xr[i] + zd{(double)d[i].x, (double)d[i].y};
}

// *flag = 2 if any of the n values is not finite
__global__ void k_check_finite(const float* __restrict__ v, int64_t n, int* flag) {
  bool bad = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    bad |= !isfinite(v[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) *(volatile int*)flag = 2;
}

// 8-byte words between device and pinned, device-mapped host memory
__global__ void k_words(const unsigned long long* __restrict__ src, unsigned long long* __restrict__ dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

static const char* blas_mode() {
  const char* e = getenv("MARIE_BLOCK_GEMM");
  return e && *e ? e : "bf16x9";
}

static void blas_mode_set(cublasHandle_t b) {
  const std::string m = blas_mode();
  if (m == "bf16x9s") {   // with Inf/NaN propagation
    cublasSetMathMode(b, CUBLAS_FP32_EMULATED_BF16X9_MATH);
    cublasSetEmulationStrategy(b, CUBLAS_EMULATION_STRATEGY_EAGER);
  } else if (m == "bf16x9") {
    cublasSetMathMode(b, CUBLAS_FP32_EMULATED_BF16X9_MATH);
    cublasSetEmulationStrategy(b, CUBLAS_EMULATION_STRATEGY_EAGER);
    // no Inf/NaN propagation through the emulated products (it costs a scan
    // of both operands per GEMM): the right-hand sides are checked finite on
    // entry and every operator output W is checked by k_check_finite before
    // it enters a GEMM
    cublasSetEmulationSpecialValuesSupport(b, CUDA_EMULATION_SPECIAL_VALUES_SUPPORT_NONE);
  } else {
    cublasSetMathMode(b, CUBLAS_PEDANTIC_MATH);
  }
}

static marie_status blas_handle(marie_vie* h, cudaStream_t s, cublasHandle_t* out) {
  if (!h->blas) {
    cublasHandle_t b = nullptr;
    if (cublasCreate(&b) != CUBLAS_STATUS_SUCCESS) {
      set_error("cublasCreate failed");
      return MARIE_ERR_CUDA;
    }
    blas_mode_set(b);
    h->blas = b;
  }
  cublasHandle_t b = (cublasHandle_t)h->blas;
  if (cublasSetStream(b, s) != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasSetStream failed");
    return MARIE_ERR_CUDA;
  }
  *out = b;
  return MARIE_OK;
}

void blas_free(marie_vie* h) {
  if (h->blas) cublasDestroy((cublasHandle_t)h->blas);
  h->blas = nullptr;
}

// C (m x n) = alpha op(A) op(B) + beta C, column-major complex64
static marie_status cgemm(cublasHandle_t b, cublasOperation_t ta, cublasOperation_t tb, int64_t m, int64_t n,
                          int64_t k, cuComplex alpha, const cplx<float>* A, int64_t lda, const cplx<float>* B,
                          int64_t ldb, cuComplex beta, cplx<float>* C, int64_t ldc) {
  const cublasStatus_t st = cublasCgemm_64(b, ta, tb, m, n, k, &alpha, (const cuComplex*)A, lda,
                                           (const cuComplex*)B, ldb, &beta, (cuComplex*)C, ldc);
  if (st != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasCgemm (%lld x %lld x %lld) failed with status %d", (long long)m, (long long)n, (long long)k,
              (int)st);
    return MARIE_ERR_CUDA;
  }
  return MARIE_OK;
}

// part[s] summed in a fixed order (FP64) into C (m x n, ldc)
__global__ void k_sum_parts(const cplx<float>* __restrict__ part, int nparts, int64_t m, int64_t n,
                            cplx<float>* __restrict__ C, int64_t ldc) {
  const int64_t mn = m * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < mn; e += (int64_t)gridDim.x * blockDim.x) {
    double x = 0, y = 0;
    for (int q = 0; q < nparts; ++q) {
      const cplx<float> v = part[(int64_t)q * mn + e];
      x += v.x;
      y += v.y;
    }
    C[(e % m) + ldc * (e / m)] = cplx<float>{(float)x, (float)y};
  }
}

// C (m x n) = A^H B with a long contraction (K rows of A and B, m and n
// small): K is split into chunks computed as one strided batch of GEMMs
// (enough tiles to fill the GPU), then the chunk products are summed in a
// fixed order.  part: scratch of part_cap complex64 values.
static marie_status cgemm_cn(cublasHandle_t b, int64_t m, int64_t n, int64_t K, const cplx<float>* A, int64_t lda,
                             const cplx<float>* B, int64_t ldb, cplx<float>* C, int64_t ldc, cplx<float>* part,
                             int64_t part_cap, cudaStream_t s) {
  const cuComplex one = {1.f, 0.f}, zero = {0.f, 0.f};
  const int64_t tiles = ((m + 127) / 128) * ((n + 127) / 128);
  int64_t S = std::min<int64_t>(64, std::max<int64_t>(1, (2 * 152 + tiles - 1) / tiles));
  S = std::min<int64_t>(S, std::max<int64_t>(1, part_cap / (m * n) - 1));
  int64_t Kc = (K + S - 1) / S;
  Kc = (Kc + 63) / 64 * 64;
  const int64_t full = K / Kc, rem = K - full * Kc;
  if (full + (rem > 0) <= 1) return cgemm(b, CUBLAS_OP_C, CUBLAS_OP_N, m, n, K, one, A, lda, B, ldb, zero, C, ldc);
  const cublasStatus_t st = cublasCgemmStridedBatched_64(
      b, CUBLAS_OP_C, CUBLAS_OP_N, m, n, Kc, &one, (const cuComplex*)A, lda, Kc, (const cuComplex*)B, ldb, Kc, &zero,
      (cuComplex*)part, m, m * n, full);
  if (st != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasCgemmStridedBatched (%lld x %lld x %lld, %lld) failed with status %d", (long long)m,
              (long long)n, (long long)Kc, (long long)full, (int)st);
    return MARIE_ERR_CUDA;
  }
  if (rem > 0)
    MARIE_TRY(cgemm(b, CUBLAS_OP_C, CUBLAS_OP_N, m, n, rem, one, A + full * Kc, lda, B + full * Kc, ldb, zero,
                    part + full * m * n, m));
  const int nparts = (int)(full + (rem > 0));
  const unsigned g = (unsigned)std::min<int64_t>(1024, (m * n + 255) / 256);
  k_sum_parts<<<g, 256, 0, s>>>(part, nparts, m, n, C, ldc);
  MARIE_LAUNCH_CHECK();
  return MARIE_OK;
}

// Pinned, device-mapped staging for the block solver's small matrices.
static marie_status bio_reserve(marie_vie* h, size_t bytes) {
  if (h->bio_cap >= bytes) return MARIE_OK;
  if (h->bio) cudaFreeHost(h->bio);
  h->bio = nullptr;
  h->bio_cap = 0;
  void* p = nullptr;
  if (cudaHostAlloc(&p, bytes, cudaHostAllocMapped) != cudaSuccess) {
    cudaGetLastError();
    set_error("pinned block buffer allocation of %zu bytes failed", bytes);
    return MARIE_ERR_OOM;
  }
  h->bio = (unsigned char*)p;
  h->bio_cap = bytes;
  return MARIE_OK;
}

// device <-> pinned buffer at byte offset off (multiples of 8 bytes)
static marie_status bio_move(marie_vie* h, size_t off, void* dev, size_t bytes, bool to_host, cudaStream_t s) {
  unsigned char* qd = nullptr;
  MARIE_CUDA_TRY(cudaHostGetDevicePointer((void**)&qd, h->bio, 0));
  const int64_t n = (int64_t)(bytes / 8);
  const unsigned grid = (unsigned)std::min<int64_t>(64, std::max<int64_t>(1, (n + 255) / 256));
  if (to_host)
    k_words<<<grid, 256, 0, s>>>((const unsigned long long*)dev, (unsigned long long*)(qd + off), n);
  else
    k_words<<<grid, 256, 0, s>>>((const unsigned long long*)(qd + off), (unsigned long long*)dev, n);
  MARIE_LAUNCH_CHECK();
  return MARIE_OK;
}

// MARIE_BLOCK_CGS: block Gram-Schmidt passes per step (1 or 2, default 1:
// single-pass classical Gram-Schmidt as in is_iter_gmres_vie.m:15-16; the
// block QR that follows is CholQR2 either way)
static int cgs_passes() {
  static const int v = [] {
    const char* e = getenv("MARIE_BLOCK_CGS");
    return e && atoi(e) == 2 ? 2 : 1;
  }();
  return v;
}

// MARIE_BLOCK_PROFILE=1: per-phase times of a block solve on stderr
// (operator applications, Gram-Schmidt GEMMs, block QR, host least squares)
struct BlockProfile {
  bool on = false;
  cudaEvent_t ev[4] = {};
  double ms[4] = {0, 0, 0, 0};
  int steps = 0;
  BlockProfile() {
    const char* e = getenv("MARIE_BLOCK_PROFILE");
    on = e && atoi(e) > 0;
    if (on)
      for (auto& x : ev) cudaEventCreate(&x);
  }
  ~BlockProfile() {
    if (!on) return;
    fprintf(stderr, "block gmres profile [ms]: matvec %.1f  gram-schmidt %.1f  block-qr %.1f  host-lsq %.1f\n", ms[0],
            ms[1], ms[2], ms[3]);
    for (auto& x : ev) cudaEventDestroy(x);
  }
};

struct BlockWork {
  int p = 0, mb = 0;
  int64_t Nb = 0;
  cplx<float>* V = nullptr;    // (mb+1) p vectors
  cplx<float>* W = nullptr;    // p vectors
  cplx<float>* H1 = nullptr;   // projections, (mb p) x p
  cplx<float>* H2 = nullptr;   // second Gram-Schmidt pass
  cplx<float>* Gm = nullptr;   // p x p Gram matrix
  cplx<float>* Sm = nullptr;   // uploads: R^{-1}, Y, Z ((mb+1)p x p)
  int* map = nullptr;          // p rhs indices
  cplx<float>* part = nullptr; // split-contraction partial products (cuBLAS path)
  int64_t part_cap = 0;
  float* tpart = nullptr;      // partial sums of the tensor-core path
  int64_t tpart_floats = 0;
  bool tc = false;             // projections on the tensor-core kernel (MARIE_BLOCK_PROJ=tcgen05)
};

// Offsets in the pinned buffer; the last 64 bytes hold the tensor-core
// kernel's error word
static size_t bio_need(int p, int mb) { return (size_t)(2 * mb * p * p + p * p + (mb + 1) * p * p) * 8 + 64; }
static size_t bio_err(int p, int mb) { return bio_need(p, mb) - 64; }
static size_t bio_h1(int, int) { return 0; }
static size_t bio_h2(int p, int mb) { return (size_t)mb * p * p * 8; }
static size_t bio_gm(int p, int mb) { return (size_t)2 * mb * p * p * 8; }
static size_t bio_up(int p, int mb) { return (size_t)(2 * mb * p * p + p * p) * 8; }

// MARIE_BLOCK_PROJ=tcgen05: the projections V^H W on this library's
// tensor-core kernel (bproj.cu, TF32 with three split products, FP32
// accuracy) instead of cuBLAS's emulated FP32.  Off by default: at 128^3
// PWL with 64 ports it reads V at 1.9 TB/s where cuBLAS's kernels are
// faster (22.7 against 21.4 s per solve).
static bool proj_tcgen05() {
  static const bool v = [] {
    const char* e = getenv("MARIE_BLOCK_PROJ");
    return e && std::string(e) == "tcgen05";
  }();
  return v;
}

// H (m x p, ld m) = A^H B for the N_b-row blocks A (m columns) and B (p columns)
static marie_status proj_cn(marie_vie* h, BlockWork& w, cublasHandle_t bl, int64_t m, const cplx<float>* A,
                            const cplx<float>* B, cplx<float>* H, cudaStream_t s) {
  if (w.tc) {
    unsigned char* qd = nullptr;
    MARIE_CUDA_TRY(cudaHostGetDevicePointer((void**)&qd, h->bio, 0));
    return block_gemm_cn(A, w.Nb, B, w.Nb, w.Nb, (int)m, w.p, H, m, w.tpart, w.tpart_floats,
                         (int*)(qd + bio_err(w.p, w.mb)), s);
  }
  return cgemm_cn(bl, m, w.p, w.Nb, A, w.Nb, B, w.Nb, H, m, w.part, w.part_cap, s);
}

// after a synchronisation: the status word (1: a tensor-core wait expired,
// 2: a non-finite operator output)
static marie_status tc_check(marie_vie* h, const BlockWork& w) {
  const int f = *reinterpret_cast<volatile int*>(h->bio + bio_err(w.p, w.mb));
  if (f == 2) {
    set_error("block GMRES: non-finite operator output");
    return MARIE_ERR_NONFINITE;
  }
  if (f) {
    set_error("block GEMM: a bounded tensor-core wait expired");
    return MARIE_ERR_DEVICE_TIMEOUT;
  }
  return MARIE_OK;
}

static void to_c64(const std::vector<zc>& a, cplx<float>* dst) {
  for (size_t i = 0; i < a.size(); ++i) dst[i] = cplx<float>{(float)a[i].real(), (float)a[i].imag()};
}

// dst = src R^{-1} with src = dst R, R (p x p, upper) returned in FP64.
// CholQR2: two Cholesky QR passes (the second restores orthogonality); a
// first pass whose Gram matrix is not numerically positive definite is
// shifted (shifted CholeskyQR) and followed by two plain passes.  src is
// overwritten.
static marie_status block_qr(marie_vie* h, BlockWork& w, cublasHandle_t bl, cplx<float>* src, cplx<float>* dst,
                             std::vector<zc>& R, cudaStream_t s) {
  const int p = w.p;
  const int64_t Nb = w.Nb;
  const cuComplex one = {1.f, 0.f}, zero = {0.f, 0.f};
  const unsigned char* hb = h->bio;
  R.assign((size_t)p * p, zc(0, 0));
  for (int i = 0; i < p; ++i) R[i + (size_t)p * i] = 1.0;
  cplx<float>* a = src;
  cplx<float>* b = dst;
  int passes = 2, shifts = 0;
  for (int pass = 0; pass < passes; ++pass) {
    // the Gram matrix in cuBLAS's FP32-accurate products: the Cholesky
    // factor needs its small eigenvalues (the tensor-core kernel's ~1e-6
    // relative error is enough for the projections, not here)
    MARIE_TRY(cgemm_cn(bl, p, p, Nb, a, Nb, a, Nb, w.Gm, p, w.part, w.part_cap, s));
    MARIE_TRY(bio_move(h, bio_gm(p, w.mb), w.Gm, (size_t)p * p * 8, true, s));
    MARIE_CUDA_TRY(cudaStreamSynchronize(s));
    MARIE_TRY(tc_check(h, w));
    const cplx<float>* g = reinterpret_cast<const cplx<float>*>(hb + bio_gm(p, w.mb));
    std::vector<zc> G((size_t)p * p);
    double tr = 0;
    for (int j = 0; j < p; ++j)
      for (int i = 0; i < p; ++i) {
        // Hermitian part (the GEMM's two triangles differ by rounding)
        const zc gij(g[i + (size_t)p * j].x, g[i + (size_t)p * j].y);
        const zc gji(g[j + (size_t)p * i].x, g[j + (size_t)p * i].y);
        G[i + (size_t)p * j] = 0.5 * (gij + std::conj(gji));
      }
    for (int i = 0; i < p; ++i) tr += G[i + (size_t)p * i].real();
    if (!std::isfinite(tr)) {
      set_error("non-finite Gram matrix in the block QR");
      return MARIE_ERR_NONFINITE;
    }
    std::vector<zc> Rk;
    if (tr == 0.0) {
      set_error("zero block in the block QR");
      return MARIE_ERR_NONFINITE;
    }
    if (!cholesky_upper(G, p, 0.0, Rk)) {
      if (++shifts > 2) {
        set_error("block QR: Gram matrix not positive definite after shifted passes");
        return MARIE_ERR_NONFINITE;
      }
      // shifted pass: Gram rounding is ~1e-6 of the trace in FP32
      if (!cholesky_upper(G, p, 1e-5 * tr / p, Rk)) {
        set_error("block QR: shifted Cholesky failed");
        return MARIE_ERR_NONFINITE;
      }
      passes = pass + 3;
    }
    std::vector<zc> Ri;
    tri_inverse(Rk, p, Ri);
    cplx<float>* up = reinterpret_cast<cplx<float>*>(h->bio + bio_up(p, w.mb));
    to_c64(Ri, up);
    MARIE_TRY(bio_move(h, bio_up(p, w.mb), w.Sm, (size_t)p * p * 8, false, s));
    MARIE_TRY(cgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, Nb, p, p, one, a, Nb, w.Sm, p, zero, b, Nb));
    R = tri_mul(Rk, R, p);
    std::swap(a, b);
    // the pinned upload area is rewritten by the next pass only after the
    // synchronisation that follows its Gram matrix
  }
  if (a != dst) MARIE_CUDA_TRY(cudaMemcpyAsync(dst, a, sizeof(cplx<float>) * (size_t)p * Nb,
                                              cudaMemcpyDeviceToDevice, s));
  return MARIE_OK;
}

// The block solver's device workspace for up to pmax right-hand sides and mb
// block steps, from the solve's pool; allocated once per solve and shared by
// its refinement steps.
static marie_status block_work_alloc(marie_vie* h, BlockWork& w, int pmax, int mb, Scratch& sc) {
  const int64_t Nb = h->Nb;
  w.mb = mb;
  w.Nb = Nb;
  MARIE_TRY(sc.get(&w.V, (size_t)(mb + 1) * pmax * Nb));
  MARIE_TRY(sc.get(&w.W, (size_t)pmax * Nb));
  MARIE_TRY(sc.get(&w.H1, (size_t)mb * pmax * pmax));
  MARIE_TRY(sc.get(&w.H2, (size_t)mb * pmax * pmax));
  MARIE_TRY(sc.get(&w.Gm, (size_t)pmax * pmax));
  MARIE_TRY(sc.get(&w.Sm, (size_t)(mb + 1) * pmax * pmax));
  MARIE_TRY(sc.get(&w.map, (size_t)pmax + 1));
  w.part_cap = (int64_t)65 * mb * pmax * pmax;
  MARIE_TRY(sc.get(&w.part, (size_t)w.part_cap));
  w.tpart_floats = block_gemm_part_floats(Nb, mb * std::min(pmax, 64));
  if (pmax <= 64 && Nb % 2 == 0 && proj_tcgen05()) MARIE_TRY(sc.get(&w.tpart, (size_t)w.tpart_floats));
  return MARIE_OK;
}

// Inner block solve of one refinement step: A D = R for the p right-hand
// sides cols[c] of r64 (FP64), D added to x; w from block_work_alloc with
// pmax >= p.  tolabs[c]: absolute residual target of column c;
// log[cols[c]] receives the residual history relative to rnorm[c] (first
// entry 1), iterations and cycles.
static marie_status bgmres_core(marie_vie* h, const std::vector<int>& cols, const zd* r64, zd* x,
                                const std::vector<double>& rnorm, const std::vector<double>& tolabs, int maxcyc,
                                BlockWork& w, std::vector<RhsLog>& log, int* matvecs, cudaStream_t s, Scratch& sc) {
  const int p = (int)cols.size();
  const int64_t Nb = h->Nb;
  const int mb = w.mb;
  w.p = p;
  w.tc = p <= 64 && Nb % 2 == 0 && w.tpart != nullptr;
  MARIE_TRY(bio_reserve(h, bio_need(p, mb)));
  cublasHandle_t bl = nullptr;
  MARIE_TRY(blas_handle(h, s, &bl));
  const cuComplex one = {1.f, 0.f}, zero = {0.f, 0.f}, mone = {-1.f, 0.f};
  // rhs map and the residual block in complex64
  MARIE_CUDA_TRY(cudaStreamSynchronize(s));
  *reinterpret_cast<volatile int*>(h->bio + bio_err(p, mb)) = 0;
  std::memcpy(h->bio + bio_up(p, mb), cols.data(), (size_t)p * sizeof(int));
  MARIE_TRY(bio_move(h, bio_up(p, mb), w.map, (size_t)((p + 1) / 2) * 8, false, s));
  k_gather_block<<<vgrid(Nb, p), 256, 0, s>>>(r64, Nb, w.W, Nb, w.map);
  MARIE_LAUNCH_CHECK();
  for (int c = 0; c < p; ++c) log[cols[c]].resvec.push_back(1.0);
  std::vector<zc> S0, Rq, Hc, Y, Z;
  MARIE_TRY(block_qr(h, w, bl, w.W, w.V, S0, s));
  BlockLsq lsq;
  std::vector<double> resid;
  bool done = false;
  BlockProfile prof;
  for (int cyc = 0; cyc < maxcyc && !done; ++cyc) {
    for (int c = 0; c < p; ++c) log[cols[c]].outer += 1;
    lsq.init(p, mb, S0);
    int j = 0;
    for (;; ++j) {
      cplx<float>* Vj = w.V + (int64_t)j * p * Nb;
      if (prof.on) cudaEventRecord(prof.ev[0], s);
      MARIE_TRY(launch_matvec<float>(h, sc.adjoint ? MV_VIE_ADJ : MV_VIE, sc.adjoint ? OP_N_ADJ : OP_N, Vj, Nb, w.W,
                                     Nb, p, nullptr, s));
      ++*matvecs;
      {
        unsigned char* qd = nullptr;
        MARIE_CUDA_TRY(cudaHostGetDevicePointer((void**)&qd, h->bio, 0));
        k_check_finite<<<vgrid(2 * (int64_t)p * Nb, 1).x, 256, 0, s>>>(reinterpret_cast<const float*>(w.W),
                                                                       2 * (int64_t)p * Nb,
                                                                       (int*)(qd + bio_err(p, mb)));
        MARIE_LAUNCH_CHECK();
      }
      if (prof.on) cudaEventRecord(prof.ev[1], s);
      const int64_t M = (int64_t)(j + 1) * p;
      MARIE_TRY(proj_cn(h, w, bl, M, w.V, w.W, w.H1, s));
      MARIE_TRY(cgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, Nb, p, M, mone, w.V, Nb, w.H1, M, one, w.W, Nb));
      if (cgs_passes() > 1) {
        MARIE_TRY(proj_cn(h, w, bl, M, w.V, w.W, w.H2, s));
        MARIE_TRY(cgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, Nb, p, M, mone, w.V, Nb, w.H2, M, one, w.W, Nb));
      } else {
        MARIE_CUDA_TRY(cudaMemsetAsync(w.H2, 0, sizeof(cplx<float>) * (size_t)M * p, s));
      }
      MARIE_TRY(bio_move(h, bio_h1(p, mb), w.H1, (size_t)M * p * 8, true, s));
      MARIE_TRY(bio_move(h, bio_h2(p, mb), w.H2, (size_t)M * p * 8, true, s));
      if (prof.on) cudaEventRecord(prof.ev[2], s);
      MARIE_TRY(block_qr(h, w, bl, w.W, w.V + (int64_t)(j + 1) * p * Nb, Rq, s));   // synchronises
      if (prof.on) {
        cudaEventRecord(prof.ev[3], s);
        cudaEventSynchronize(prof.ev[3]);
        float a = 0, b2 = 0, c2 = 0;
        cudaEventElapsedTime(&a, prof.ev[0], prof.ev[1]);
        cudaEventElapsedTime(&b2, prof.ev[1], prof.ev[2]);
        cudaEventElapsedTime(&c2, prof.ev[2], prof.ev[3]);
        prof.ms[0] += a;
        prof.ms[1] += b2;
        prof.ms[2] += c2;
      }
      const auto t_l0 = std::chrono::steady_clock::now();
      const int rows = (int)M + p;
      Hc.assign((size_t)rows * p, zc(0, 0));
      const cplx<float>* h1 = reinterpret_cast<const cplx<float>*>(h->bio + bio_h1(p, mb));
      const cplx<float>* h2 = reinterpret_cast<const cplx<float>*>(h->bio + bio_h2(p, mb));
      for (int c = 0; c < p; ++c) {
        for (int64_t i = 0; i < M; ++i)
          Hc[i + (size_t)rows * c] = zc((double)h1[i + M * c].x + h2[i + M * c].x,
                                        (double)h1[i + M * c].y + h2[i + M * c].y);
        for (int i = 0; i < p; ++i) Hc[M + i + (size_t)rows * c] = Rq[i + (size_t)p * c];
      }
      lsq.add_block(j, Hc, resid);
      if (prof.on) prof.ms[3] += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_l0).count();
      bool all = true, finite = true;
      for (int c = 0; c < p; ++c) {
        RhsLog& L = log[cols[c]];
        L.iters += 1;
        L.resvec.push_back(rnorm[c] > 0 ? resid[c] / rnorm[c] : 0.0);
        if (!std::isfinite(resid[c])) finite = false;
        if (!(resid[c] <= tolabs[c])) all = false;
      }
      if (!finite) {
        for (int c = 0; c < p; ++c) log[cols[c]].status = MARIE_ERR_NONFINITE;
        return MARIE_OK;
      }
      if (all) done = true;
      if (all || j + 1 == mb) break;
    }
    for (int c = 0; c < p; ++c) log[cols[c]].last_inner = j + 1;
    // x += V_{0:j} Y
    const int64_t n = (int64_t)(j + 1) * p;
    lsq.solve(j, Y);
    // the upload area still feeds the last block QR's normalisation until
    // the stream gets there
    MARIE_CUDA_TRY(cudaStreamSynchronize(s));
    cplx<float>* up = reinterpret_cast<cplx<float>*>(h->bio + bio_up(p, mb));
    to_c64(Y, up);
    MARIE_TRY(bio_move(h, bio_up(p, mb), w.Sm, (size_t)n * p * 8, false, s));
    MARIE_TRY(cgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, Nb, p, n, one, w.V, Nb, w.Sm, n, zero, w.W, Nb));
    k_add_block<<<vgrid(Nb, p), 256, 0, s>>>(x, Nb, w.W, Nb, w.map);
    MARIE_LAUNCH_CHECK();
    if (done || cyc + 1 == maxcyc) break;
    // next cycle from R = V_{0:j+1} Z
    lsq.residual(j, Z);
    MARIE_CUDA_TRY(cudaStreamSynchronize(s));     // the upload area held Y
    to_c64(Z, up);
    MARIE_TRY(bio_move(h, bio_up(p, mb), w.Sm, (size_t)(n + p) * p * 8, false, s));
    MARIE_TRY(cgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, Nb, p, n + p, one, w.V, Nb, w.Sm, n + p, zero, w.W, Nb));
    MARIE_TRY(block_qr(h, w, bl, w.W, w.V, S0, s));
  }
  MARIE_CUDA_TRY(cudaStreamSynchronize(s));
  if (!done)
    for (int c = 0; c < p; ++c)
      if (log[cols[c]].status == MARIE_OK) log[cols[c]].status = MARIE_ERR_NOT_CONVERGED;
  return MARIE_OK;
}

}  // namespace marie
