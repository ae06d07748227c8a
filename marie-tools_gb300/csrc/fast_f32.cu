// Four-step matvec passes, float instantiation.
#include "fastpath_impl.cuh"

namespace marie {
template void launch_x_nb<float>(int, bool, const MvArgs<float>&, dim3, size_t, cudaStream_t);
template void launch_y_nb<float>(int, bool, const MvArgs<float>&, dim3, size_t, cudaStream_t);
template void launch_z_nb<float, true>(int, int, const MvArgs<float>&, dim3, size_t, cudaStream_t);
template void launch_z_nb<float, false>(int, int, const MvArgs<float>&, dim3, size_t, cudaStream_t);
template marie_status launch_fast_chunk<float>(marie_vie*, int, MvArgs<float>&, int, cudaStream_t, cudaEvent_t*);
}  // namespace marie
