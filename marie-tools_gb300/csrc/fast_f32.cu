// Four-step matvec passes, float instantiation.
#include "fastpath.cuh"

namespace marie {
template marie_status launch_fast_chunk<float>(marie_vie*, int, MvArgs<float>&, int, cudaStream_t, cudaEvent_t*);
}  // namespace marie
