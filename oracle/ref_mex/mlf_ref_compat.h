/*
 * mlf_ref_compat.h -- force-included (nvcc -include) when the reference's own MEX source,
 * src/cuda/mex_lfm_convolution_vec.cu, is compiled unchanged into a cubin for the parity
 * tests (recipe: oracle/refbuild.py).  Test infrastructure only: nothing in the product
 * includes it.
 *
 * The reference reads its bitmap and kernels through legacy texture references
 * (`texture<float, 1, cudaReadModeElementType>`, tex1Dfetch, cudaBindTexture:
 * mex_lfm_convolution_vec.cu:22,25,153-181,375-385,415-416).  CUDA 12 removed texture
 * references, so this header supplies a stand-in with the same spelling: `texture<...>`
 * becomes a __device__ struct holding the bound pointer and its element count, and
 * tex1Dfetch becomes a plain global load that returns 0 outside the bound range (what a
 * 1-D fetch from linear memory returns out of range).  Every other line of the reference
 * file compiles as written.  The host side (mexFunction) is parsed but never run: the
 * launcher oracle/ref_mex_launch.cu loads the cubin and launches the kernel with the
 * reference's own launch geometry, writing the bound pointers with cudaLibraryGetGlobal.
 */
#ifndef MLF_REF_COMPAT_H
#define MLF_REF_COMPAT_H

/* Headers the reference includes, included before the `texture` macro below exists. */
#include <cublas_v2.h>
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>

/* MATLAB's MEX headers: the declaration-only stand-ins of the MEX shim tests. */
#include "mex.h"
#include "gpu/mxGPUArray.h"
int mexPrintf(const char* fmt, ...);
mxComplexity mxGPUGetComplexity(const mxGPUArray* a);

/* Layout shared with the launcher: the launcher writes {ptr, n} into the two globals. */
template <class T, int dim, enum cudaTextureReadMode mode>
struct mlf_ref_texref {
  const T* ptr;
  long long n;
};

#define texture __device__ mlf_ref_texref

template <class T, int dim, enum cudaTextureReadMode mode>
__device__ __forceinline__ T tex1Dfetch(const mlf_ref_texref<T, dim, mode>& t, int i) {
  return (i >= 0 && (long long)i < t.n) ? t.ptr[i] : T(0);
}

/* Host-side binders, parsed for mexFunction only (the launcher never calls mexFunction). */
template <class T, int dim, enum cudaTextureReadMode mode>
static cudaError_t cudaBindTexture(size_t*, const mlf_ref_texref<T, dim, mode>&, const void*,
                                   cudaChannelFormatDesc, size_t) {
  return cudaErrorNotSupported;
}
template <class T, int dim, enum cudaTextureReadMode mode>
static cudaError_t cudaUnbindTexture(const mlf_ref_texref<T, dim, mode>&) {
  return cudaSuccess;
}

#endif /* MLF_REF_COMPAT_H */
