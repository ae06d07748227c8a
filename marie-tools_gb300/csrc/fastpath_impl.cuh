// Definitions of the four-step pass launchers declared in fastpath.cuh.
#pragma once

#include <atomic>

#include "fastpath.cuh"
#include "matvec4.cuh"

namespace marie {

template <typename KernelFn>
static void smem_opt_in(KernelFn fn, std::atomic<uint64_t>& done) {
  smem_opt_in_device((const void*)fn, done);
}

template <typename T, int NB>
static void launch_x(bool inv, const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s) {
  static std::atomic<uint64_t> of{0}, oi{0};
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
  static std::atomic<uint64_t> of{0}, oi{0};
  if (!inv) {
    smem_opt_in(k4_fwd_y<T, NB>, of);
    k4_fwd_y<T, NB><<<g, 256, smem, s>>>(a);
  } else {
    smem_opt_in(k4_inv_y<T, NB>, oi);
    k4_inv_y<T, NB><<<g, 256, smem, s>>>(a);
  }
}

// complex64: the packed-pair kernel k4_zp; complex128 in float-float: k4_zf
// (packed (re, im) pairs); native complex128: k4_z
template <typename T, int NB, bool PWL, int OP>
static void launch_z4(const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s) {
  static std::atomic<uint64_t> o{0};
  if constexpr (std::is_same<T, float>::value) {
    smem_opt_in(k4_zp<NB, PWL, OP>, o);
    k4_zp<NB, PWL, OP><<<g, kZpThreads, smem, s>>>(a);
  } else if constexpr (std::is_same<T, ff>::value) {
    smem_opt_in(k4_zf<NB, PWL, OP>, o);
    k4_zf<NB, PWL, OP><<<g, 256, smem, s>>>(a);
  } else {
    smem_opt_in(k4_z<T, NB, PWL, OP>, o);
    k4_z<T, NB, PWL, OP><<<g, 256, smem, s>>>(a);
  }
}

template <typename T>
void launch_x_nb(int nb, bool inv, const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s) {
#define X_CALL(NB) launch_x<T, NB>(inv, a, g, smem, s)
  MARIE_NB_SWITCH(nb, X_CALL);
#undef X_CALL
}

template <typename T>
void launch_y_nb(int nb, bool inv, const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s) {
#define Y_CALL(NB) launch_y<T, NB>(inv, a, g, smem, s)
  MARIE_NB_SWITCH(nb, Y_CALL);
#undef Y_CALL
}

// The four-step path serves N (op 0) and N^H (op 1).
template <typename T, bool PWL, int NB>
void launch_z_one(int op, const MvArgs<T>& a, dim3 g, size_t smem, cudaStream_t s) {
  if (op == OP_N) launch_z4<T, NB, PWL, 0>(a, g, smem, s);
  else launch_z4<T, NB, PWL, 1>(a, g, smem, s);
}

}  // namespace marie
