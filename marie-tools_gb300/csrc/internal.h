// Host-side runtime of the GB300 FFT-VIE library: the operator handle,
// error reporting and the launchers shared by the translation units.
#pragma once

#include <atomic>
#include <map>
#include <utility>
#include <string>
#include <vector>
#include <cstdio>

#include "../../include/marie_gb300.h"
#include "matvec.cuh"

namespace marie {

void set_error(const char* fmt, ...);
extern std::atomic<int64_t> g_launches;
extern thread_local int64_t t_launches;   // this thread's share of g_launches

#define MARIE_CUDA_TRY(expr)                                                             \
  do {                                                                                   \
    cudaError_t e_ = (expr);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      ::marie::set_error("CUDA error %d (%s) at %s:%d", (int)e_, cudaGetErrorString(e_), \
                         __FILE__, __LINE__);                                            \
      return e_ == cudaErrorMemoryAllocation ? MARIE_ERR_OOM : MARIE_ERR_CUDA;           \
    }                                                                                    \
  } while (0)

#define MARIE_LAUNCH_CHECK()                 \
  do {                                       \
    ::marie::g_launches.fetch_add(1);        \
    ++::marie::t_launches;                   \
    MARIE_CUDA_TRY(cudaGetLastError());      \
  } while (0)

#define MARIE_TRY(expr)                \
  do {                                 \
    marie_status s_ = (expr);          \
    if (s_ != MARIE_OK) return s_;     \
  } while (0)

// Device tables of one grid axis in one precision.
template <typename T>
struct AxisDev {
  cplx<T>* tw = nullptr;
  cplx<T>* tw2 = nullptr;
  int* kofp = nullptr;
  int* pofk = nullptr;
  FftPlan plan{};
};

// Everything one precision of the operator needs on the device.
template <typename T>
struct PrecState {
  bool built = false;
  AxisDev<T> ax, ay, az;
  cplx<T>* chi = nullptr;     // Ns
  cplx<T>* GN = nullptr;      // nblkN * oct
  cplx<T>* GK = nullptr;      // nblkK * oct
  cplx<T>* GNf = nullptr;     // 8 n1 n2 n3 * nblkN, [ky][kx][kz][blk] (four-step grids; complex64: pair layout)
  cplx<T>* T1 = nullptr;      // ws_rhs * C * n3 * n2 * 2n1
  cplx<T>* S = nullptr;       // ws_rhs * C * 2n2 * n3 * 2n1
  int ws_rhs = 0;             // right-hand sides per matvec chunk
  int ws_cap = 0;             // right-hand sides the work arrays hold (whole z-tile bundles)
  int TY = 1, TXY = 1, TX = 1;
};

// Tucker factors kept on the device (FP32) for the per-application
// expansion of the complex64 spectrum (tucker.cu, precisions bit 8).
struct TuckerDev {
  struct Block {
    int r1 = 0, r2 = 0, r3 = 0;
    cplx<float>* G = nullptr;    // r1 r2 r3, then U1 (r1 x 2n1), U2, U3 in the same allocation
    cplx<float>* U1 = nullptr;
    cplx<float>* U2 = nullptr;
    cplx<float>* U3 = nullptr;
  };
  bool active = false;
  std::vector<Block> blocks;
  cplx<float>* P1 = nullptr;     // work: r1 r2 x 2n3
  cplx<float>* P2 = nullptr;     // work: r1 x 2n2 x 2n3
};

}  // namespace marie

struct marie_vie {
  int n1 = 0, n2 = 0, n3 = 0, C = 0, pwl = 0;
  int on1 = 0, on2 = 0, on3 = 0;     // caller's grid when it was embedded in n1 x n2 x n3 (embed.h); 0 otherwise
  double res = 0, freq = 0, k0 = 0, omega = 0;
  double ce_im = 0;                  // ce = i*ce_im = i*omega*eps0
  int64_t Ns = 0, Nb = 0;
  int device = 0;
  int max_rhs = 1;
  int precisions = 0;
  int has_K = 0;
  int nblkN = 0, nblkK = 0;
  int64_t mem_cap = 0, mem_used = 0;
  double invg[12] = {0};
  int* vox2sol = nullptr;            // device, n1*n2*n3
  unsigned char* row_live = nullptr; // device, n2*n3: grid row (y, z) holds a body voxel
  unsigned char* z_live = nullptr;   // device, n3: slice z holds a body voxel
  uint16_t* rowq = nullptr;          // device, n3*8: row_live in four-step order (n2 = 16*NB)
  uint16_t* zq = nullptr;            // device, 8: z_live in four-step order (n3 = 16*NB)
  int64_t* idxS = nullptr;           // device, Ns (0-based linear voxel index)
  double* wpow = nullptr;            // device, Ns: real(Mc_inv/ce) per body voxel
  marie::cplx<double>* mr_body = nullptr;   // device, Ns: Mr per body voxel
  std::vector<int64_t> idxS_host;
  marie::BlockTab tab[4];            // N, N_adj, K, K_adj
  marie::PrecState<double> p64;
  marie::PrecState<float> p32;
  marie::PrecState<marie::ff> pff;   // complex128 I/O, float-float arithmetic (precisions bit 4)
  marie::TuckerDev tkf;              // precisions bit 8: complex64 spectrum re-expanded per application
  std::vector<void*> allocs;
  // GMRES workspace pool: the buffers a solve requests, in request order,
  // kept across solves and grown on demand (marie_vie_release_workspace
  // frees them; destroy frees everything).
  std::vector<std::pair<void*, size_t>> gm_pool;
  std::vector<std::pair<void*, size_t>> io_pool;   // device buffers of the host-buffer solve
  // Pinned, device-mapped host memory for the solver's per-iteration status
  // (residuals, masks): moved by a kernel, so it never queues on a copy
  // engine behind the chunk copies of the host-buffer solve.
  unsigned char* hio = nullptr;
  size_t hio_cap = 0;
  // the block solver's small matrices (pinned, device-mapped) and its cuBLAS handle
  unsigned char* bio = nullptr;
  size_t bio_cap = 0;
  void* blas = nullptr;
  // CUDA graphs of Arnoldi windows (the launches between two host
  // synchronisations of the GMRES loop), keyed by every pointer and size the
  // launches capture; replayed by later cycles and solves of the same shape.
  struct GraphEntry {
    cudaGraphExec_t exec = nullptr;
    int64_t kernels = 0;
  };
  std::map<std::vector<uint64_t>, GraphEntry> graphs;
  cudaStream_t gstream = nullptr;    // the graphs run here, joined to the caller's stream by events
  cudaEvent_t gev[2] = {nullptr, nullptr};
};

namespace marie {

marie_status dev_alloc(marie_vie* h, void** p, size_t bytes);
void dev_free_all(marie_vie* h);
void graphs_free(marie_vie* h);
void blas_free(marie_vie* h);

// H (M x p, ldh) = V^H W on the tensor cores (bproj.cu); p <= 64; part:
// block_gemm_part_floats(K, M) floats of scratch; err: device-visible word
// set to 1 if a bounded wait expired.
marie_status block_gemm_cn(const cplx<float>* V, int64_t ldv, const cplx<float>* W, int64_t ldw, int64_t K, int M,
                           int p, cplx<float>* H, int64_t ldh, float* part, int64_t part_floats, int* err,
                           cudaStream_t s);
int64_t block_gemm_part_floats(int64_t K, int M);

enum OpKind { OP_N = 0, OP_N_ADJ = 1, OP_K = 2, OP_K_ADJ = 3 };

// Enqueue one operator application on `stream`.
//  mode: MV_GRID / MV_VIE / MV_VIE_ADJ; op: OP_*.
//  in/out: device arrays in precision T; in_rs/out_rs: element strides between
//  consecutive right-hand sides; active: optional per-rhs mask (device).
template <typename T>
marie_status launch_matvec(marie_vie* h, int mode, int op, const cplx<T>* in, int64_t in_rs,
                           cplx<T>* out, int64_t out_rs, int nrhs, const unsigned char* active,
                           cudaStream_t stream);

template <typename T>
PrecState<T>& prec_state(marie_vie* h);

// Field modes (MV_EFIELD / MV_HFIELD) on body vectors of length N_b, with an
// optional addend (incident field) of the same layout.
template <typename T>
marie_status launch_matvec_fields(marie_vie* h, int mode, int op, const cplx<T>* in, cplx<T>* out,
                                  const cplx<T>* addend, int nrhs, cudaStream_t stream);

// Four-step passes (grid edges 16*NB, NB <= 8) for one chunk of nb bundles;
// tiles and bundle size are set in `a` by the caller.
template <typename T>
marie_status launch_fast_chunk(marie_vie* h, int op, MvArgs<T>& a, int nb, cudaStream_t stream, cudaEvent_t* ev);

marie_status build_spectra(marie_vie* h, const marie_vie_desc* d);

// Per-application Tucker expansion (tucker.cu): keep the N operator's
// factors at create; rebuild the complex64 full spectrum on `s`.
marie_status tucker_keep_c64(marie_vie* h, const marie_tucker_block* tk);
marie_status tucker_expand_c64(marie_vie* h, cudaStream_t s);

// n-point Gauss-Legendre rule on [-1, 1], nodes ascending (host).
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w);

// Largest dynamic shared memory a CTA may opt into on sm_100-family GPUs.
constexpr size_t kSmemOptin = 227 * 1024;

// Opt a kernel into the large dynamic shared-memory carve-out once per
// device (the attribute is per device; a process may drive several).
// `done` is the kernel's own flag word: bit d set once device d is done.
constexpr int kMaxDevices = 64;
inline void smem_opt_in_device(const void* fn, std::atomic<uint64_t>& done) {
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t bit = 1ull << (dev & (kMaxDevices - 1));
  if (done.load(std::memory_order_acquire) & bit) return;
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemOptin);
  done.fetch_or(bit, std::memory_order_acq_rel);
}

// Dynamic shared memory of the generic x, y and z passes (matvec.cuh) with
// row tiles TY / TXY / TX and bundle size R: each holds its axis' twiddles
// plus 2*tile*R (times C for z) padded sequences of length n.
struct GenericSmem {
  size_t x, y, z;
};
inline GenericSmem generic_smem(int n1, int n2, int n3, int C, size_t sz, int TY, int TXY, int TX, int R) {
  return {(size_t)(n1 + (size_t)n1 * (2 * (size_t)TY * R + 1)) * sz,
          (size_t)(n2 + (size_t)n2 * (2 * (size_t)TXY * R + 1)) * sz,
          (size_t)(n3 + (size_t)n3 * (2 * (size_t)C * TX * R + 1)) * sz};
}
// Largest row tile t (>= 1) with n * (2 * mult * t * R + 2) elements of sz
// bytes within kSmemOptin; 1 when even t = 1 does not fit (the caller checks).
inline int generic_tile_cap(int n, int mult, int R, size_t sz) {
  const long v = ((long)(kSmemOptin / sz / (size_t)n) - 2) / (2L * mult * R);
  return (int)(v < 1 ? 1 : (v > (1 << 20) ? (1 << 20) : v));
}

// Every grid edge is 16*NB with NB <= 8: the four-step passes apply.
inline bool four_step_edge(int n) { return n % 16 == 0 && n / 16 >= 1 && n / 16 <= 8; }
inline bool four_step_grid(const marie_vie* h) {
  return four_step_edge(h->n1) && four_step_edge(h->n2) && four_step_edge(h->n3);
}

}  // namespace marie
