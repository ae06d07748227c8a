// Four-step z pass, float-float instantiation for one NB = n3/16 (both bases,
// N and N^H).  Compiled once per NB in [1, 8] with -DMARIE_FF_NB=<NB>: the
// float-float z kernels take long to compile together, so each NB is its own
// object and the eight compile in parallel.
#include "fastpath_impl.cuh"

#ifndef MARIE_FF_NB
#error "compile with -DMARIE_FF_NB=<1..8>"
#endif

namespace marie {
template void launch_z_one<ff, true, MARIE_FF_NB>(int, const MvArgs<ff>&, dim3, size_t, cudaStream_t);
template void launch_z_one<ff, false, MARIE_FF_NB>(int, const MvArgs<ff>&, dim3, size_t, cudaStream_t);
}  // namespace marie
