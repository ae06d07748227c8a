// Four-step x passes, float-float instantiation.
#include "fastpath_impl.cuh"

namespace marie {
template void launch_x_nb<ff>(int, bool, const MvArgs<ff>&, dim3, size_t, cudaStream_t);
}  // namespace marie
