// C entry point over one of the reference's wire-to-voxel coupling kernels
// (Assemble_tri_coupling_matrix_<V>.cpp of its src_wvie/Cpp_Assembly, called
// by wvie_mrgf_assembly.m:26-49), for the oracle's checks of the loop
// right-hand sides.  TEST INFRASTRUCTURE ONLY: oracle/Makefile compiles it
// together with the reference source into oracle/_ref, once per variant V
// (the macro ORACLE_TRI_FN names the kernel).
#include <cstddef>

#include "mex.h"

void ORACLE_TRI_FN(mxComplexDouble* Zbc, double* Scoord, double* r_p, double* r_n, double* r_2, double* wie_quads,
                   double* vie_quads, double res, const size_t N_vox, const size_t N_tri, double ko);

extern "C" void oracle_tri_coupling(double* Z, double* Scoord, double* r_p, double* r_n, double* r_2,
                                    double* wie_quads, double* vie_quads, double res, size_t n_vox, size_t n_tri,
                                    double k0) {
  ORACLE_TRI_FN(reinterpret_cast<mxComplexDouble*>(Z), Scoord, r_p, r_n, r_2, wie_quads, vie_quads, res, n_vox,
                n_tri, k0);
}
