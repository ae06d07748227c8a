// Four-step matvec passes, double instantiation.
#include "fastpath.cuh"

namespace marie {
template marie_status launch_fast_chunk<double>(marie_vie*, int, MvArgs<double>&, int, cudaStream_t, cudaEvent_t*);
}  // namespace marie
