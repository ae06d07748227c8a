// Tall-skinny complex GEMM H = V^H W on the tensor cores (tcgen05,
// kind::tf32, three split products per product), for the block GMRES
// projections V_{0:j}^H W and Gram matrices W^H W (bgmres.cuh).
//
// V: M complex64 columns of K rows (column a at V + a*ldv), W: p <= 64
// complex64 columns (column c at W + c*ldw), H: M x p (column-major, ldh).
// Real form: with the complex rows interleaved (re, im) along the
// contraction,
//   Re H[a,c] = sum_i (wr vr + wi vi) = sum_k W'[c,k]  V'[a,k]
//   Im H[a,c] = sum_i (wi vr - wr vi) = sum_k W''[c,k] V'[a,k],  W'' = (wi, -wr)
// so one MMA with A = [W'; W''] (128 rows: c and 64 + c) and B = V' (basis
// vectors as its N rows) leaves Re H[a,c] in tensor-memory lane c and Im
// H[a,c] in lane 64 + c, column a.  Every operand value x is split into
// hi = rna_tf32(x) and lo = rna_tf32(x - hi); D += A_hi B_hi + A_hi B_lo +
// A_lo B_hi (the dropped lo x lo term is ~2^-22 of the product).
//
// CTA: 256 threads, one slice of the contraction (complex rows [i0, i1)) x
// up to 512 basis vectors (two accumulators of 256 tensor-memory columns).
// Chunks of 8 complex rows in two shared-memory stages: the threads convert
// the chunk held in registers into one stage's operand tiles (8-row x
// 16-byte core matrices, K-major, no swizzle) while the tensor core
// multiplies the other stage; one thread issues a chunk's MMAs and commits
// them to the stage's mbarrier, and all threads then load the next chunk
// into registers.  Every 256 chunks the accumulators are added into the
// CTA's FP32 partial sums and restarted (short accumulation chains in the
// tensor core); k_bproj_sum adds the slices in a fixed order (FP64).  Every
// wait is bounded: on expiry the CTA sets the error word, waits (bounded)
// for its own MMAs, frees its tensor memory and returns.
#include <cstdint>

#include "internal.h"

namespace marie {

constexpr int kBpThreads = 256;
constexpr int kBpChunk = 8;                     // complex rows per chunk (16 floats = 64 B per operand row)
constexpr int kBpN = 512;                       // basis vectors per CTA
constexpr int kBpA = 128 * 64;                  // bytes of one A tile (128 rows x 64 B)
constexpr int kBpB = kBpN * 64;                 // bytes of one B tile
constexpr int kBpStage = 2 * kBpA + 2 * kBpB;   // A_hi, A_lo, B_hi, B_lo
constexpr int kBpSmem = 2 * kBpStage;           // two stages
constexpr int kBpChain = 256;                   // chunks accumulated in tensor memory between flushes
constexpr long long kBpWaitLimit = 1ll << 22;   // mbarrier polls before giving up

__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// hi / lo split of four values: hi = rna_tf32(x), lo = x - hi exactly in
// FP32 (|lo| <= 2^-12 |x|; the tensor core reads its top 19 bits, so lo
// carries x to within 2^-23 |x|)
__device__ __forceinline__ void split4(float4 v, uint4& hi, uint4& lo) {
  hi.x = tf32_rna(v.x);
  hi.y = tf32_rna(v.y);
  hi.z = tf32_rna(v.z);
  hi.w = tf32_rna(v.w);
  lo.x = __float_as_uint(v.x - __uint_as_float(hi.x));
  lo.y = __float_as_uint(v.y - __uint_as_float(hi.y));
  lo.z = __float_as_uint(v.z - __uint_as_float(hi.z));
  lo.w = __float_as_uint(v.w - __uint_as_float(hi.w));
}

// byte offset of (row, 16-byte column kq) in a K-major core-matrix tile with
// 4 core matrices along K (64 bytes of K per row)
__device__ __forceinline__ uint32_t core_off(int row, int kq) {
  return (uint32_t)((((row >> 3) << 2) + kq) << 7) + (uint32_t)((row & 7) << 4);
}

// shared-memory matrix descriptor: K-major, no swizzle; core matrices 128 B
// apart along K (leading byte offset) and 512 B apart along M/N (stride byte
// offset); descriptor version 1 (sm_100 family)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(512 >> 4) << 32) |
         (1ull << 46);
}

// instruction descriptor: D F32, A and B TF32, both K-major, M = 128, N
__device__ __forceinline__ uint32_t idesc_tf32(int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(id), "r"(acc)
      : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long long it = 0; it < kBpWaitLimit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

struct BprojArgs {
  const float* V;      // interleaved complex64
  const float* W;
  int64_t ldv, ldw;    // complex elements between columns
  int64_t K;           // complex rows
  int64_t rows;        // complex rows per slice (multiple of kBpChunk)
  int M, p;
  int64_t Mpad;        // basis vectors per slice in part (tiles x 512)
  float* part;         // [slice][Mpad][128]
  int* err;
};

__global__ void __launch_bounds__(kBpThreads, 1) k_bproj(BprojArgs g) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ __align__(8) unsigned long long bars[2];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int slice = blockIdx.x, tile = blockIdx.y;
  const int64_t i0 = (int64_t)slice * g.rows;
  const int64_t i1 = min(g.K, i0 + g.rows);
  const int a0 = tile * kBpN;
  const int nvalid = min(kBpN, g.M - a0);
  const int nB = (nvalid + 15) & ~15;                 // MMA N (multiple of 16)
  const uint32_t ncols = nB <= 32 ? 32 : nB <= 64 ? 64 : nB <= 128 ? 128 : nB <= 256 ? 256 : 512;
  const uint32_t s0 = (uint32_t)__cvta_generic_to_shared(sm);
  const uint32_t sbar0 = (uint32_t)__cvta_generic_to_shared(&bars[0]);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(&tmem_slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sbar0) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sbar0 + 8) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_slot;

  const int64_t nch = (i1 - i0 + kBpChunk - 1) / kBpChunk;
  // per-thread float4 loads of a chunk: B rows q = tid + 256 u (u < 8), A (W)
  // rows q = tid; q -> row = (q >> 5) * 8 + (q & 7), kq = (q >> 3) & 3, so
  // the 8 threads of a quarter warp store 8 rows of one core-matrix column
  // (distinct banks) and a warp reads 8 rows x 64 contiguous bytes
  // three register sets: chunks ch+1 and ch+2 are in flight while chunk ch
  // is converted (one CTA per SM: the loads in flight set the bandwidth)
  float4 rb0[8], rb1[8], rb2[8], ra0, ra1, ra2;
  // the thread's rows: base pointers at the slice start (row and column
  // fixed for the whole slice), advanced by 16 floats per chunk
  const float* bp[8];
  unsigned bvalid = 0;
#pragma unroll
  for (int u = 0; u < 8; ++u) {
    const int q = tid + kBpThreads * u;
    const int row = ((q >> 5) << 3) + (q & 7), kq = (q >> 3) & 3;
    if (row < nvalid) bvalid |= 1u << u;
    bp[u] = g.V + 2 * ((int64_t)(a0 + (row < nvalid ? row : 0)) * g.ldv + i0) + 4 * kq;
  }
  const int ac = ((tid >> 5) << 3) + (tid & 7), akq = (tid >> 3) & 3;
  const bool avalid = ac < g.p;
  const float* ap = g.W + 2 * ((int64_t)(avalid ? ac : 0) * g.ldw + i0) + 4 * akq;
  const int64_t nfull = (i1 - i0) / kBpChunk;         // chunks without a ragged end
  auto load = [&](int64_t ch, float4 (&rb)[8], float4& ra) {
    const int64_t off = ch * 2 * kBpChunk;
    if (ch < nfull) {
#pragma unroll
      for (int u = 0; u < 8; ++u)
        rb[u] = (bvalid >> u) & 1u ? __ldg(reinterpret_cast<const float4*>(bp[u] + off))
                                   : make_float4(0.f, 0.f, 0.f, 0.f);
      ra = avalid ? __ldg(reinterpret_cast<const float4*>(ap + off)) : make_float4(0.f, 0.f, 0.f, 0.f);
      return;
    }
    // the ragged last chunk: complex rows i and i + 1 of each float4 checked
    const int64_t ib = i0 + ch * kBpChunk;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = tid + kBpThreads * u;
      const int kq = (q >> 3) & 3;
      const int64_t i = ib + 2 * kq;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (((bvalid >> u) & 1u) && i < i1) {
        if (i + 1 < i1) {
          v = __ldg(reinterpret_cast<const float4*>(bp[u] + off));
        } else {
          const float2 h = __ldg(reinterpret_cast<const float2*>(bp[u] + off));
          v = make_float4(h.x, h.y, 0.f, 0.f);
        }
      }
      rb[u] = v;
    }
    {
      const int64_t i = ib + 2 * akq;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (avalid && i < i1) {
        if (i + 1 < i1) {
          v = __ldg(reinterpret_cast<const float4*>(ap + off));
        } else {
          const float2 h = __ldg(reinterpret_cast<const float2*>(ap + off));
          v = make_float4(h.x, h.y, 0.f, 0.f);
        }
      }
      ra = v;
    }
  };
  auto store = [&](int st, const float4 (&rb)[8], const float4& ra) {
    unsigned char* base = sm + st * kBpStage;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = tid + kBpThreads * u;
      const int row = ((q >> 5) << 3) + (q & 7), kq = (q >> 3) & 3;
      if (row < nB) {
        uint4 hi, lo;
        split4(rb[u], hi, lo);
        const uint32_t off = core_off(row, kq);
        *reinterpret_cast<uint4*>(base + 2 * kBpA + off) = hi;
        *reinterpret_cast<uint4*>(base + 2 * kBpA + kBpB + off) = lo;
      }
    }
    {
      const int c = ((tid >> 5) << 3) + (tid & 7), kq = (tid >> 3) & 3;
      const float4 w2 = make_float4(ra.y, -ra.x, ra.w, -ra.z);   // (wi, -wr) of the two complex rows
      uint4 hi, lo;
      split4(ra, hi, lo);
      uint32_t off = core_off(c, kq);
      *reinterpret_cast<uint4*>(base + off) = hi;
      *reinterpret_cast<uint4*>(base + kBpA + off) = lo;
      split4(w2, hi, lo);
      off = core_off(64 + c, kq);
      *reinterpret_cast<uint4*>(base + off) = hi;
      *reinterpret_cast<uint4*>(base + kBpA + off) = lo;
    }
  };
  // tensor memory -> partial sums (the CTA's own rows of part): the first
  // flush stores, later ones add in FP32
  const int lane_base = (warp & 3) * 32;
  const int m = lane_base + (tid & 31);
  const int half = (nB + 63) / 64 * 32;               // columns per warp half, multiple of 32
  const int fc0 = (warp >> 2) * half, fc1 = min(nB, fc0 + half);
  float* dst = g.part + ((int64_t)slice * g.Mpad + a0) * 128 + m;
  auto flush = [&](bool first) {
    for (int cb = fc0; cb < fc1; cb += 32) {
      uint32_t r[32];
      const uint32_t taddr = tmem + ((uint32_t)lane_base << 16) + (uint32_t)cb;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
            "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (cb + j < fc1) {
          float* q = dst + (int64_t)(cb + j) * 128;
          *q = first ? __uint_as_float(r[j]) : *q + __uint_as_float(r[j]);
        }
    }
  };

  bool ok = true;
  int64_t last = -1;                                  // last committed chunk
  int64_t chain0 = 0;                                 // first chunk of the current accumulation chain
  // one chunk: convert it into its stage, multiply, refill its register set
  // with chunk ch + 3, and at the end of a chain move the sums out; false
  // after an expired wait (the same for every thread)
  auto step = [&](int64_t ch, float4 (&rb)[8], float4& ra) -> bool {
    const int st = (int)(ch & 1);
    // the stage's previous chunk (ch - 2) must be multiplied before it is
    // overwritten; the barrier makes an expired wait everyone's decision
    const bool ready = ch < 2 || mbar_wait(sbar0 + 8 * st, (uint32_t)(((ch - 2) >> 1) & 1));
    if (ready) store(st, rb, ra);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (!__syncthreads_and(ready)) return false;
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sA_hi = s0 + st * kBpStage, sA_lo = sA_hi + kBpA;
      const uint32_t sB_hi = sA_hi + 2 * kBpA, sB_lo = sB_hi + kBpB;
      const int n0 = min(nB, 256), n1 = nB - n0;
#pragma unroll
      for (int s = 0; s < 2; ++s) {         // two K steps of 8 values (two core matrices)
#pragma unroll
        for (int t = 0; t < 3; ++t) {       // hi.hi, hi.lo, lo.hi
          const uint64_t ad = smem_desc((t == 2 ? sA_lo : sA_hi) + s * 256);
          const uint32_t bb = (t == 1 ? sB_lo : sB_hi) + s * 256;
          const uint32_t acc = (ch > chain0 || s > 0 || t > 0) ? 1u : 0u;
          mma_tf32(tmem, ad, smem_desc(bb), idesc_tf32(n0), acc);
          if (n1 > 0) mma_tf32(tmem + 256, ad, smem_desc(bb + 32 * 512), idesc_tf32(n1), acc);
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       sbar0 + 8 * st)
                   : "memory");
    }
    last = ch;
    if (ch + 3 < nch) load(ch + 3, rb, ra);
    if (ch + 1 == nch || ch + 1 - chain0 == kBpChain) {
      // end of an accumulation chain: wait for its products, move them out
      const bool done = mbar_wait(sbar0 + 8 * st, (uint32_t)((ch >> 1) & 1));
      if (!__syncthreads_and(done)) return false;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      flush(chain0 == 0);
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      chain0 = ch + 1;
    }
    return true;
  };
  if (nch > 0) load(0, rb0, ra0);
  if (nch > 1) load(1, rb1, ra1);
  if (nch > 2) load(2, rb2, ra2);
  for (int64_t ch = 0; ch < nch && ok; ch += 3) {
    ok = step(ch, rb0, ra0);
    if (ok && ch + 1 < nch) ok = step(ch + 1, rb1, ra1);
    if (ok && ch + 2 < nch) ok = step(ch + 2, rb2, ra2);
  }
  if (!ok) {
    // an expired wait: one more bounded wait for the products in flight
    *(volatile int*)g.err = 1;
    if (last >= 0 && !mbar_wait(sbar0 + 8 * (int)(last & 1), (uint32_t)((last >> 1) & 1)))
      *(volatile int*)g.err = 1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols) : "memory");
  }
}

// H[a + ldh c] = sum over slices of (part[s][a][c], part[s][a][64 + c]), in
// slice order (FP64 sums)
__global__ void k_bproj_sum(const float* __restrict__ part, int nslices, int64_t Mpad, int M, int p,
                            cplx<float>* __restrict__ H, int64_t ldh) {
  const int64_t n = (int64_t)M * p;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(e % p);
    const int64_t a = e / p;
    double x = 0, y = 0;
    for (int s = 0; s < nslices; ++s) {
      const float* q = part + ((int64_t)s * Mpad + a) * 128;
      x += q[c];
      y += q[64 + c];
    }
    H[a + ldh * c] = cplx<float>{(float)x, (float)y};
  }
}

int64_t block_gemm_part_floats(int64_t K, int M) {
  const int tiles = (M + kBpN - 1) / kBpN;
  const int64_t S = std::max<int64_t>(1, std::min<int64_t>(152 / tiles, (K + kBpChunk - 1) / kBpChunk));
  return S * (int64_t)tiles * kBpN * 128;
}

marie_status block_gemm_cn(const cplx<float>* V, int64_t ldv, const cplx<float>* W, int64_t ldw, int64_t K, int M,
                           int p, cplx<float>* H, int64_t ldh, float* part, int64_t part_floats, int* err,
                           cudaStream_t s) {
  if (p < 1 || p > 64 || M < 1 || K < 1) {
    set_error("block GEMM: p must be in [1, 64] (got %d), M and K positive", p);
    return MARIE_ERR_BAD_ARG;
  }
  // 16-byte loads of two complex rows: columns must start on 16 bytes
  if ((((uintptr_t)V | (uintptr_t)W) & 15) || (ldv & 1) || (ldw & 1)) {
    set_error("block GEMM: columns must start on 16-byte boundaries (even leading dimensions)");
    return MARIE_ERR_BAD_ARG;
  }
  static std::atomic<uint64_t> done{0};
  {
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = 1ull << (dev & 63);
    if (!(done.load() & bit)) {
      MARIE_CUDA_TRY(cudaFuncSetAttribute((const void*)k_bproj, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          kBpSmem));
      done.fetch_or(bit);
    }
  }
  const int tiles = (M + kBpN - 1) / kBpN;
  int64_t S = std::max<int64_t>(1, std::min<int64_t>(152 / tiles, (K + kBpChunk - 1) / kBpChunk));
  int64_t rows = (K + S - 1) / S;
  rows = (rows + kBpChunk - 1) / kBpChunk * kBpChunk;
  S = (K + rows - 1) / rows;
  const int64_t Mpad = (int64_t)tiles * kBpN;
  if (S * Mpad * 128 > part_floats) {
    set_error("block GEMM: partial-sum scratch too small");
    return MARIE_ERR_BAD_ARG;
  }
  BprojArgs g;
  g.V = reinterpret_cast<const float*>(V);
  g.W = reinterpret_cast<const float*>(W);
  g.ldv = ldv;
  g.ldw = ldw;
  g.K = K;
  g.rows = rows;
  g.M = M;
  g.p = p;
  g.Mpad = Mpad;
  g.part = part;
  g.err = err;
  k_bproj<<<dim3((unsigned)S, (unsigned)tiles), kBpThreads, kBpSmem, s>>>(g);
  MARIE_LAUNCH_CHECK();
  const int64_t n = (int64_t)M * p;
  k_bproj_sum<<<(unsigned)std::min<int64_t>(1024, (n + 255) / 256), 256, 0, s>>>(part, (int)S, Mpad, M, p, H, ldh);
  MARIE_LAUNCH_CHECK();
  return MARIE_OK;
}

}  // namespace marie

using namespace marie;

// Test hook: H (M x p, column-major, ldh) = V^H W for complex64 device
// arrays, on the tensor cores; err: device int set to 1 if a bounded wait
// expired.  No counterpart in the reference.
extern "C" marie_status marie_block_gemm_cn(const void* V, int64_t ldv, const void* W, int64_t ldw, int64_t K,
                                            int32_t M, int32_t p, void* H, int64_t ldh, void* part,
                                            int64_t part_floats, void* err, void* stream) {
  if (!V || !W || !H || !part || !err) {
    set_error("NULL argument");
    return MARIE_ERR_BAD_ARG;
  }
  return block_gemm_cn((const cplx<float>*)V, ldv, (const cplx<float>*)W, ldw, K, M, p, (cplx<float>*)H, ldh,
                       (float*)part, part_floats, (int*)err, (cudaStream_t)stream);
}

extern "C" int64_t marie_block_gemm_part_floats(int64_t K, int32_t M) { return block_gemm_part_floats(K, M); }
