/* Declaration-only stand-in for MATLAB's mex.h (R2018a interleaved complex
 * API), used to compile-check the MEX gateway where MATLAB is absent.  Only
 * the names and signatures the gateway uses are declared. */
#ifndef MARIE_MEX_STUB_H
#define MARIE_MEX_STUB_H
#include <stddef.h>
#include <stdbool.h>
typedef struct mxArray_tag mxArray;
typedef size_t mwSize;
typedef size_t mwIndex;
typedef enum { mxUNKNOWN_CLASS, mxDOUBLE_CLASS, mxSINGLE_CLASS, mxUINT64_CLASS } mxClassID;
typedef enum { mxREAL, mxCOMPLEX } mxComplexity;
typedef struct { double real, imag; } mxComplexDouble;
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
bool mxIsUint64(const mxArray*);
bool mxIsDouble(const mxArray*);
bool mxIsComplex(const mxArray*);
bool mxIsStruct(const mxArray*);
bool mxIsChar(const mxArray*);
bool mxIsEmpty(const mxArray*);
bool mxIsSparse(const mxArray*);
size_t mxGetN(const mxArray*);
mwIndex* mxGetIr(const mxArray*);
mwIndex* mxGetJc(const mxArray*);
size_t mxGetNumberOfElements(const mxArray*);
size_t mxGetM(const mxArray*);
void* mxGetData(const mxArray*);
double mxGetScalar(const mxArray*);
double* mxGetDoubles(const mxArray*);
mxComplexDouble* mxGetComplexDoubles(const mxArray*);
mxArray* mxGetField(const mxArray*, mwIndex, const char*);
const mwSize* mxGetDimensions(const mxArray*);
mwSize mxGetNumberOfDimensions(const mxArray*);
void* mxCalloc(size_t, size_t);
mxArray* mxCreateNumericMatrix(mwSize, mwSize, mxClassID, mxComplexity);
mxArray* mxCreateNumericArray(mwSize, const mwSize*, mxClassID, mxComplexity);
mxArray* mxCreateDoubleMatrix(mwSize, mwSize, mxComplexity);
int mxGetString(const mxArray*, char*, mwSize);
#endif
