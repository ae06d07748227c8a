/* Minimal stand-in for MATLAB's mex.h: only the interleaved-complex element
 * type that the reference's wire-coupling kernels write
 * (Assemble_tri_coupling_matrix_*.cpp).  For oracle/Makefile only. */
#ifndef ORACLE_MEX_STUB_H
#define ORACLE_MEX_STUB_H
typedef struct { double real, imag; } mxComplexDouble;
#endif
