// Four-step matvec passes, float-float (complex128 in and out): the chunk
// driver; the kernels are instantiated in fast_ff_x.cu, fast_ff_y.cu,
// fast_ff_zl.cu and fast_ff_zc.cu.
#include "fastpath.cuh"

namespace marie {
template marie_status launch_fast_chunk<ff>(marie_vie*, int, MvArgs<ff>&, int, cudaStream_t, cudaEvent_t*);
}  // namespace marie
