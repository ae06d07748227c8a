// Launch code of the four-step matvec passes (matvec4.cuh, kz4.cuh).
//
// The per-pass launchers (switch over NB = n/16) are declared here and
// defined in fastpath_impl.cuh, so that one precision's kernels can be spread
// over several translation units that compile in parallel (the float-float
// kernels: x and y passes in two units, the z pass in one object per NB).
#pragma once

#include "internal.h"

namespace marie {

__host__ __device__ constexpr int kz4_stride(int N, int W) { return N + (W >= 16 ? 1 : 16 / W); }
__host__ __device__ constexpr int kz4_halfpad(int W) { return W >= 16 ? 0 : 8 / W; }

// Sequence stride of k4_zp (complex64, packed pairs) in 16-byte pairs.
__host__ __device__ constexpr int kzp_stride(int N, int W) { return N + (W >= 8 ? 1 : 8 / W); }
// k4_zf (float-float, 16-byte elements): the same stride and an odd-half pad
// of 4/W, which put the eight lanes of every quarter-warp of its five phases
// on distinct 16-byte bank groups (checked by enumerating lane addresses).
__host__ __device__ constexpr int kzf_stride(int N, int W) { return N + (W >= 8 ? 1 : 8 / W); }
__host__ __device__ constexpr int kzf_halfpad(int W) { return W >= 8 ? 0 : 4 / W; }

// Shared-memory bytes of the z pass: k4_z (native complex128: twiddles +
// both halves), k4_zf (float-float: 32-byte twiddle entries + both halves)
// or k4_zp (complex64: twiddle tables, slice masks, pairs).
template <typename T>
__host__ inline size_t kz4_smem(int N, int C, int W) {
  const size_t NB = N / 16;
  if (sizeof(T) == 4) return 560 * NB + 32 + (size_t)C * W * kzp_stride(N, W) * 16;
  if (std::is_same<T, ff>::value) return (36 * NB + 2 * (size_t)C * W * kzf_stride(N, W) + kzf_halfpad(W)) * 16;
  const size_t half = (size_t)C * W * kz4_stride(N, W);
  return (N + 2 * half + kz4_halfpad(W)) * sizeof(cplx<T>);
}

template <typename T>
void launch_x_nb(int nb, bool inv, const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s);
template <typename T>
void launch_y_nb(int nb, bool inv, const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s);
template <typename T, bool PWL, int NB>
void launch_z_one(int op, const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s);

#define MARIE_NB_SWITCH(nb, CALL) \
  switch (nb) {                   \
    case 1: CALL(1); break;       \
    case 2: CALL(2); break;       \
    case 3: CALL(3); break;       \
    case 4: CALL(4); break;       \
    case 5: CALL(5); break;       \
    case 6: CALL(6); break;       \
    case 7: CALL(7); break;       \
    default: CALL(8); break;      \
  }

template <typename T, bool PWL>
void launch_z_nb(int nb, int op, const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s) {
#define Z_CALL(NB) launch_z_one<T, PWL, NB>(op, a, g, smem, s)
  MARIE_NB_SWITCH(nb, Z_CALL);
#undef Z_CALL
}

// The five passes of one chunk on the four-step path; ev (optional) as in
// launch_matvec_ev.  Tiles in `a` are set by the caller.
template <typename T>
marie_status launch_fast_chunk(marie_vie* h, int op, MvArgs<T>& a, int nb, cudaStream_t stream, cudaEvent_t* ev) {
  const int n1 = h->n1, n2 = h->n2, n3 = h->n3, C = h->C;
  const size_t sz = sizeof(cplx<T>);
  const size_t smx = (size_t)(n1 + (size_t)2 * a.TY * a.R * (n1 + 1)) * sz;
  const size_t smy = (size_t)(n2 + (size_t)2 * a.TXY * a.R * (n2 + 1)) * sz;
  const size_t smz = kz4_smem<T>(n3, C, a.TX * a.R);
  dim3 gx((n2 + a.TY - 1) / a.TY, n3, nb * C);
  dim3 gy((2 * n1 + a.TXY - 1) / a.TXY, n3, nb * C);
  dim3 gz(nb, (2 * n1 + a.TX - 1) / a.TX, 2 * n2);
  if (ev) cudaEventRecord(ev[0], stream);
  launch_x_nb<T>(n1 / 16, false, a, gx, smx, stream);
  MARIE_LAUNCH_CHECK();
  if (ev) cudaEventRecord(ev[1], stream);
  launch_y_nb<T>(n2 / 16, false, a, gy, smy, stream);
  MARIE_LAUNCH_CHECK();
  if (ev) cudaEventRecord(ev[2], stream);
  if (h->pwl) launch_z_nb<T, true>(n3 / 16, op, a, gz, smz, stream);
  else launch_z_nb<T, false>(n3 / 16, op, a, gz, smz, stream);
  MARIE_LAUNCH_CHECK();
  if (ev) cudaEventRecord(ev[3], stream);
  launch_y_nb<T>(n2 / 16, true, a, gy, smy, stream);
  MARIE_LAUNCH_CHECK();
  if (ev) cudaEventRecord(ev[4], stream);
  launch_x_nb<T>(n1 / 16, true, a, gx, smx, stream);
  MARIE_LAUNCH_CHECK();
  if (ev) cudaEventRecord(ev[5], stream);
  return MARIE_OK;
}

}  // namespace marie
