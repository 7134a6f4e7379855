/* Minimal stand-in for MATLAB's mex.h: only what the MEX shims in this repository use,
 * so that they can be compiled and exercised by the tests without MATLAB. */
#ifndef MLF_FAKE_MEX_H
#define MLF_FAKE_MEX_H
#include <stddef.h>
#include <stdint.h>
typedef size_t mwSize;
typedef enum { mxUNKNOWN_CLASS = 0, mxDOUBLE_CLASS = 6, mxSINGLE_CLASS = 7 } mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef struct mxArray_tag mxArray;
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
void mxFree(void* p);
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);
#endif
