// Four-step y passes, float-float instantiation.
#include "fastpath_impl.cuh"

namespace marie {
template void launch_y_nb<ff>(int, bool, const MvArgs<ff>&, dim3, size_t, cudaStream_t);
}  // namespace marie
