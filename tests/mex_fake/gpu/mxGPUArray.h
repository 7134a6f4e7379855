/* Minimal stand-in for MATLAB's gpu/mxGPUArray.h (see ../mex.h). */
#ifndef MLF_FAKE_MXGPUARRAY_H
#define MLF_FAKE_MXGPUARRAY_H
#include "mex.h"
typedef struct mxGPUArray_tag mxGPUArray;
typedef enum { MX_GPU_DO_NOT_INITIALIZE = 0, MX_GPU_INITIALIZE_VALUES = 1 } mxGPUInitialize;
int mxInitGPU(void);
const mxGPUArray* mxGPUCreateFromMxArray(const mxArray* a);
mwSize mxGPUGetNumberOfDimensions(const mxGPUArray* a);
const mwSize* mxGPUGetDimensions(const mxGPUArray* a);
mxClassID mxGPUGetClassID(const mxGPUArray* a);
const void* mxGPUGetDataReadOnly(const mxGPUArray* a);
void* mxGPUGetData(mxGPUArray* a);
mxGPUArray* mxGPUCreateGPUArray(mwSize nd, const mwSize* dims, mxClassID cls, mxComplexity cx, mxGPUInitialize init);
mxArray* mxGPUCreateMxArrayOnGPU(const mxGPUArray* a);
void mxGPUDestroyGPUArray(const mxGPUArray* a);
#endif
