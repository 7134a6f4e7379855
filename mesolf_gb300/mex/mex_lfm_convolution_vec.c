/* MEX shim: out = mex_lfm_convolution_vec(bitmap, kernels), a drop-in for the reference's
 * src/cuda/mex_lfm_convolution_vec.cu (mexFunction :276-421) over libmesolf_lf.so.
 *
 * Build inside MATLAB:  mex -R2018a mex_lfm_convolution_vec.c -I<include> -L<lib> -lmesolf_lf
 *
 * Same arguments and validation as the reference: exactly two inputs; a 2-D or 3-D single
 * bitmap (W x H [x n], CPU or gpuArray); 4-D single kernels (kw x kw x 15 x 15, kw <= 341);
 * errors raise "parallel:gpu:mexGPUExample:InvalidInput" (:296-297, :305-347), library
 * errors carry the library's message under the same id.  Returns a new single gpuArray with
 * the bitmap's dimensions; synchronous like the reference (:406,420). */
#include "mex.h"
#include "gpu/mxGPUArray.h"
#include "mesolf_lf.h"

static const char* kInvalid = "parallel:gpu:mexGPUExample:InvalidInput";

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  const mxGPUArray* bm;
  const mxGPUArray* kr;
  const mwSize* bd;
  const mwSize* kd;
  mwSize nd;
  mxGPUArray* out;
  int st;
  (void)nlhs;
  mxInitGPU();
  if (nrhs != 2) mexErrMsgIdAndTxt(kInvalid, "Invalid input to mex_lfm_convolution_vec()");
  bm = mxGPUCreateFromMxArray(prhs[0]);
  kr = mxGPUCreateFromMxArray(prhs[1]);
  bd = mxGPUGetDimensions(bm);
  kd = mxGPUGetDimensions(kr);
  nd = mxGPUGetNumberOfDimensions(bm);
  if (nd < 2 || nd > 3 || mxGPUGetNumberOfDimensions(kr) != 4 || mxGPUGetClassID(bm) != mxSINGLE_CLASS ||
      mxGPUGetClassID(kr) != mxSINGLE_CLASS)
    mexErrMsgIdAndTxt(kInvalid, "Invalid input to mex_lfm_convolution_vec()");
  out = mxGPUCreateGPUArray(nd, bd, mxSINGLE_CLASS, mxREAL, MX_GPU_DO_NOT_INITIALIZE);
  st = mlf_conv_vec((const float*)mxGPUGetDataReadOnly(bm), (int64_t)bd[0], (int64_t)bd[1],
                    nd == 3 ? (int64_t)bd[2] : 1, (const float*)mxGPUGetDataReadOnly(kr), (int64_t)kd[0],
                    (int32_t)kd[2], (float*)mxGPUGetData(out), NULL);
  if (st != MLF_OK) {
    char msg[512];
    mlf_last_error(msg, sizeof msg);
    mexErrMsgIdAndTxt(kInvalid, "%s", msg);
  }
  plhs[0] = mxGPUCreateMxArrayOnGPU(out);
  mxFree((void*)bd);
  mxFree((void*)kd);
  mxGPUDestroyGPUArray(bm);
  mxGPUDestroyGPUArray(kr);
  mxGPUDestroyGPUArray(out);
}
