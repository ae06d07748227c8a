// Launch code of the four-step matvec passes (matvec4.cuh), instantiated per
// precision in fast_f32.cu / fast_f64.cu.
#pragma once

#include <mutex>

#include "internal.h"
#include "matvec4.cuh"

namespace marie {

template <typename KernelFn>
static void smem_opt_in(KernelFn fn, std::once_flag& once) {
  std::call_once(once, [fn] {
    cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  });
}

template <typename T, int NB>
static void launch_x(bool inv, const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s) {
  static std::once_flag of, oi;
  if (!inv) {
    smem_opt_in(k4_fwd_x<T, NB>, of);
    k4_fwd_x<T, NB><<<g, 256, smem, s>>>(a);
  } else {
    smem_opt_in(k4_inv_x<T, NB>, oi);
    k4_inv_x<T, NB><<<g, 256, smem, s>>>(a);
  }
}

template <typename T, int NB>
static void launch_y(bool inv, const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s) {
  static std::once_flag of, oi;
  if (!inv) {
    smem_opt_in(k4_fwd_y<T, NB>, of);
    k4_fwd_y<T, NB><<<g, 256, smem, s>>>(a);
  } else {
    smem_opt_in(k4_inv_y<T, NB>, oi);
    k4_inv_y<T, NB><<<g, 256, smem, s>>>(a);
  }
}

template <typename T, int NB, bool PWL, int OP>
static void launch_z4(const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s) {
  static std::once_flag o;
  smem_opt_in(k4_z<T, NB, PWL, OP>, o);
  k4_z<T, NB, PWL, OP><<<g, 256, smem, s>>>(a);
}

template <typename T, int NB>
static void launch_z_nb(bool pwl, int op, const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s) {
  if (pwl) {
    if (op == OP_N) launch_z4<T, NB, true, 0>(a, g, smem, s);
    else launch_z4<T, NB, true, 1>(a, g, smem, s);
  } else {
    if (op == OP_N) launch_z4<T, NB, false, 0>(a, g, smem, s);
    else launch_z4<T, NB, false, 1>(a, g, smem, s);
  }
}

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
  dim3 gz((2 * n1 + a.TX - 1) / a.TX, 2 * n2, nb);
  const bool pwl = h->pwl != 0;
  if (ev) cudaEventRecord(ev[0], stream);
#define X_FWD(NB) launch_x<T, NB>(false, a, gx, smx, stream)
  MARIE_NB_SWITCH(n1 / 16, X_FWD);
#undef X_FWD
  MARIE_LAUNCH_CHECK();
  if (ev) cudaEventRecord(ev[1], stream);
#define Y_FWD(NB) launch_y<T, NB>(false, a, gy, smy, stream)
  MARIE_NB_SWITCH(n2 / 16, Y_FWD);
#undef Y_FWD
  MARIE_LAUNCH_CHECK();
  if (ev) cudaEventRecord(ev[2], stream);
#define Z_ALL(NB) launch_z_nb<T, NB>(pwl, op, a, gz, smz, stream)
  MARIE_NB_SWITCH(n3 / 16, Z_ALL);
#undef Z_ALL
  MARIE_LAUNCH_CHECK();
  if (ev) cudaEventRecord(ev[3], stream);
#define Y_INV(NB) launch_y<T, NB>(true, a, gy, smy, stream)
  MARIE_NB_SWITCH(n2 / 16, Y_INV);
#undef Y_INV
  MARIE_LAUNCH_CHECK();
  if (ev) cudaEventRecord(ev[4], stream);
#define X_INV(NB) launch_x<T, NB>(true, a, gx, smx, stream)
  MARIE_NB_SWITCH(n1 / 16, X_INV);
#undef X_INV
  MARIE_LAUNCH_CHECK();
  if (ev) cudaEventRecord(ev[5], stream);
  return MARIE_OK;
}

}  // namespace marie
