// Allocation-free N-operator apply.
//
// marie_vie_apply_N_noalloc computes y = mvp_N(x) for one right-hand side in
// complex64 without a handle and without allocating device memory: the
// caller passes the grid, the Green's-tensor octant spectrum, x and y, and the
// FFT work arrays live in a fixed file-scope __device__ array.  It exists for
// callers that must not allocate on the device, e.g. code running where a
// memory allocator is forbidden (inside another framework's allocator-free
// region, a real-time loop, or a process that pre-reserves all device memory),
// and cannot go through marie_vie_create, which allocates its workspaces.
//
// Limits and sharing:
//  - scratch: kNoAllocScratchBytes (64 MiB) of work arrays, i.e.
//    6 * n1*n2*n3 * C * 8 bytes <= 64 MiB (C = 3 PWC, 12 PWL); larger grids are
//    rejected with MARIE_ERR_BAD_ARG.  Grid edges <= 1024.
//  - the scratch and the per-axis tables are shared by every call in the
//    process on a given device and keep the last call's contents; calls that
//    overlap on the GPU (different streams, or threads) race on them.
//    Nothing needs clearing between calls: every pass writes all it reads.
//  - the first call on a device resolves the scratch symbols' device
//    addresses (cudaGetSymbolAddress, once per device, with that device
//    current); make that first call before any stream capture.
#include <cstring>
#include <mutex>

#include "internal.h"

namespace marie {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;

static __device__ __align__(256) unsigned char g_na_scratch[kNoAllocScratchBytes];
// per axis: [tw (n) | tw2 (n)] complex64 and [kofp (n) | pofk (n)]
static __device__ __align__(256) cplx<float> g_na_tw[3][2 * kMaxAxis];
static __device__ __align__(256) int g_na_maps[3][2 * kMaxAxis];

struct NaPtrs {
  bool ready = false;
  unsigned char* scratch = nullptr;
  cplx<float>* tw = nullptr;
  int* maps = nullptr;
};
std::mutex g_na_mu;
NaPtrs g_na[kMaxDevices];

// Twiddles (w_n^k, w_2n^k) and digit-reversal maps of the three axes.
__global__ void k_na_tables(FftPlan p0, FftPlan p1, FftPlan p2, cplx<float>* tw, int* maps) {
  const int a = blockIdx.x;
  const FftPlan pl = a == 0 ? p0 : (a == 1 ? p1 : p2);
  const int n = pl.n;
  cplx<float>* t = tw + (size_t)a * 2 * kMaxAxis;
  int* m = maps + (size_t)a * 2 * kMaxAxis;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    double s, c;
    sincospi(-2.0 * k / n, &s, &c);
    t[k] = cplx<float>{(float)c, (float)s};
    sincospi(-1.0 * k / n, &s, &c);
    t[n + k] = cplx<float>{(float)c, (float)s};
    int rem = k, p = 0, span = n;
    for (int st = 0; st < pl.nst; ++st) {
      const int r = pl.r[st];
      const int d = rem % r;
      rem /= r;
      span /= r;
      p += d * span;
    }
    m[p] = k;       // kofp
    m[n + k] = p;   // pofk
  }
}

bool na_plan(int n, FftPlan* pl) {
  pl->n = n;
  pl->nst = 0;
  int m = n;
  while (m % 8 == 0 && pl->nst < kMaxStages) { pl->r[pl->nst++] = 8; m /= 8; }
  if (m % 4 == 0 && pl->nst < kMaxStages) { pl->r[pl->nst++] = 4; m /= 4; }
  if (m % 2 == 0 && pl->nst < kMaxStages) { pl->r[pl->nst++] = 2; m /= 2; }
  for (int p = 3; m > 1 && p <= 31; p += 2)
    while (m % p == 0 && pl->nst < kMaxStages) { pl->r[pl->nst++] = p; m /= p; }
  return m == 1;
}

marie_status na_setup(int dev, NaPtrs** out) {
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("noalloc: device ordinal %d out of range", dev);
    return MARIE_ERR_NOT_SUPPORTED;
  }
  std::lock_guard<std::mutex> lk(g_na_mu);
  NaPtrs& P = g_na[dev];
  if (!P.ready) {
    cudaError_t e = cudaGetSymbolAddress((void**)&P.scratch, g_na_scratch);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&P.tw, g_na_tw);
    if (e == cudaSuccess) e = cudaGetSymbolAddress((void**)&P.maps, g_na_maps);
    if (e != cudaSuccess) {
      cudaGetLastError();
      set_error("noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return MARIE_ERR_CUDA;
    }
    const void* fns[] = {(const void*)k_fwd_x<float>, (const void*)k_fwd_y<float>,
                         (const void*)k_inv_y<float>, (const void*)k_inv_x<float>,
                         (const void*)k_z<float, true, 0>, (const void*)k_z<float, false, 0>};
    for (const void* f : fns) {
      e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemOptin);
      if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("noalloc: cudaFuncSetAttribute (shared-memory opt-in) failed: %s", cudaGetErrorString(e));
        return MARIE_ERR_CUDA;
      }
    }
    P.ready = true;
  }
  *out = &P;
  return MARIE_OK;
}

}  // namespace
}  // namespace marie

using namespace marie;

extern "C" marie_status marie_vie_apply_N_noalloc(int32_t n1, int32_t n2, int32_t n3, int32_t basis,
                                                  const void* green_octant, const void* x, void* y,
                                                  void* stream) {
  if (n1 < 1 || n2 < 1 || n3 < 1 || n1 > kMaxAxis || n2 > kMaxAxis || n3 > kMaxAxis) {
    set_error("noalloc: grid edges must be in [1, %d]", kMaxAxis);
    return MARIE_ERR_BAD_ARG;
  }
  if (basis != MARIE_PWC && basis != MARIE_PWL) { set_error("noalloc: basis must be 0 or 1"); return MARIE_ERR_BAD_ARG; }
  if (!green_octant || !x || !y) { set_error("noalloc: NULL pointer argument"); return MARIE_ERR_BAD_ARG; }
  const bool pwl = basis == MARIE_PWL;
  const int C = pwl ? 12 : 3;
  const size_t per = (size_t)C * n3 * n2 * 2 * n1;   // T1 elements; S is twice that
  const size_t need = 3 * per * sizeof(cplx<float>);
  if (need > kNoAllocScratchBytes) {
    set_error("noalloc: grid %dx%dx%d (%s) needs %zu bytes of scratch, more than the fixed %zu bytes "
              "(6*n1*n2*n3*C*8 must not exceed 64 MiB)", n1, n2, n3, pwl ? "PWL" : "PWC", need,
              kNoAllocScratchBytes);
    return MARIE_ERR_BAD_ARG;
  }
  FftPlan px, py, pz;
  if (!na_plan(n1, &px) || !na_plan(n2, &py) || !na_plan(n3, &pz)) {
    set_error("noalloc: grid edge with a prime factor above 31 (unsupported FFT length)");
    return MARIE_ERR_NOT_SUPPORTED;
  }
  // tiles: the same rule as the handle path for one complex64 right-hand
  // side, narrowed where a pass would not fit one CTA's shared memory; a
  // grid that does not fit even with one-row tiles is refused before any
  // launch
  const size_t sz = sizeof(cplx<float>);
  int W = 16;
  while (W > 1 && (size_t)n3 * (2 * C * W + 1) * sz > 100 * 1024) W /= 2;
  const int TY = std::min(std::max(1, std::min(n2, 16)), generic_tile_cap(n1, 1, 1, sz));
  const int TXY = std::min(std::max(1, std::min(2 * n1, 16)), generic_tile_cap(n2, 1, 1, sz));
  const int TX = std::min(std::max(1, std::min(2 * n1, W)), generic_tile_cap(n3, C, 1, sz));
  const GenericSmem sm = generic_smem(n1, n2, n3, C, sz, TY, TXY, TX, 1);
  if (sm.x > kSmemOptin || sm.y > kSmemOptin || sm.z > kSmemOptin) {
    set_error("noalloc: grid %dx%dx%d (%s) needs %zu / %zu / %zu bytes of shared memory in the x / y / z passes, "
              "more than the %zu a CTA can hold", n1, n2, n3, pwl ? "PWL" : "PWC", sm.x, sm.y, sm.z, kSmemOptin);
    return MARIE_ERR_BAD_ARG;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    set_error("noalloc: no CUDA device");
    return MARIE_ERR_CUDA;
  }
  NaPtrs* P = nullptr;
  MARIE_TRY(na_setup(dev, &P));
  cudaStream_t s = (cudaStream_t)stream;
  k_na_tables<<<3, 256, 0, s>>>(px, py, pz, P->tw, P->maps);
  MARIE_LAUNCH_CHECK();

  MvArgs<float> a;
  memset(&a, 0, sizeof(a));
  a.n1 = n1; a.n2 = n2; a.n3 = n3; a.C = C;
  a.R = 1;
  a.nrhs = 1;
  a.mode = MV_GRID;
  const FftPlan* pls[3] = {&px, &py, &pz};
  AxisTab<float>* axs[3] = {&a.ax, &a.ay, &a.az};
  for (int d = 0; d < 3; ++d) {
    const int n = pls[d]->n;
    axs[d]->tw = P->tw + (size_t)d * 2 * kMaxAxis;
    axs[d]->tw2 = axs[d]->tw + n;
    axs[d]->kofp = P->maps + (size_t)d * 2 * kMaxAxis;
    axs[d]->pofk = axs[d]->kofp + n;
    axs[d]->plan = *pls[d];
  }
  a.in = (const cplx<float>*)x;
  a.out = (cplx<float>*)y;
  a.in_rs = a.out_rs = (int64_t)C * n1 * n2 * n3;
  a.T1 = (cplx<float>*)P->scratch;
  a.S = a.T1 + per;
  a.G = (const cplx<float>*)green_octant;
  a.TY = TY;
  a.TXY = TXY;
  a.TX = TX;
  const size_t smx = sm.x, smy = sm.y, smz = sm.z;
  dim3 gx((n2 + a.TY - 1) / a.TY, n3, C);
  dim3 gy((2 * n1 + a.TXY - 1) / a.TXY, n3, C);
  dim3 gz((2 * n1 + a.TX - 1) / a.TX, 2 * n2, 1);
  k_fwd_x<float><<<gx, 256, smx, s>>>(a);
  MARIE_LAUNCH_CHECK();
  k_fwd_y<float><<<gy, 256, smy, s>>>(a);
  MARIE_LAUNCH_CHECK();
  if (pwl) k_z<float, true, 0><<<gz, 256, smz, s>>>(a);
  else k_z<float, false, 0><<<gz, 256, smz, s>>>(a);
  MARIE_LAUNCH_CHECK();
  k_inv_y<float><<<gy, 256, smy, s>>>(a);
  MARIE_LAUNCH_CHECK();
  k_inv_x<float><<<gx, 256, smx, s>>>(a);
  MARIE_LAUNCH_CHECK();
  return MARIE_OK;
}
