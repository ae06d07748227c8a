// Four-step matvec passes, double instantiation.
#include "fastpath_impl.cuh"

namespace marie {
template void launch_x_nb<double>(int, bool, const MvArgs<double>&, dim3, size_t, cudaStream_t);
template void launch_y_nb<double>(int, bool, const MvArgs<double>&, dim3, size_t, cudaStream_t);
template void launch_z_nb<double, true>(int, int, const MvArgs<double>&, dim3, size_t, cudaStream_t);
template void launch_z_nb<double, false>(int, int, const MvArgs<double>&, dim3, size_t, cudaStream_t);
template marie_status launch_fast_chunk<double>(marie_vie*, int, MvArgs<double>&, int, cudaStream_t, cudaEvent_t*);
}  // namespace marie
