/* Declaration-only stand-in for MATLAB's gpu/mxGPUArray.h (compile check). */
#ifndef MARIE_MXGPU_STUB_H
#define MARIE_MXGPU_STUB_H
#include "mex.h"
typedef struct mxGPUArray_tag mxGPUArray;
typedef enum { MX_GPU_INITIALIZE_VALUES, MX_GPU_DO_NOT_INITIALIZE } mxGPUInitialize;
bool mxIsGPUArray(const mxArray*);
int mxInitGPU(void);
const mxGPUArray* mxGPUCreateFromMxArray(const mxArray*);
mxClassID mxGPUGetClassID(const mxGPUArray*);
mxComplexity mxGPUGetComplexity(const mxGPUArray*);
mwSize mxGPUGetNumberOfElements(const mxGPUArray*);
mwSize mxGPUGetNumberOfDimensions(const mxGPUArray*);
const mwSize* mxGPUGetDimensions(const mxGPUArray*);
mxGPUArray* mxGPUCreateGPUArray(mwSize, const mwSize*, mxClassID, mxComplexity, mxGPUInitialize);
const void* mxGPUGetDataReadOnly(const mxGPUArray*);
void* mxGPUGetData(mxGPUArray*);
mxArray* mxGPUCreateMxArrayOnGPU(const mxGPUArray*);
void mxGPUDestroyGPUArray(const mxGPUArray*);
#endif
