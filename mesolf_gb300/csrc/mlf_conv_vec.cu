// Position-variant light-field correlation with the semantics of the reference MEX
// (src/cuda/mex_lfm_convolution_vec.cu:43-266):
//
//   out[i][y][x] = sum_{ky,kx < kw} in[i][y+ky-kw/2][x+kx-kw/2] * K[(y%nn)*nn + x%nn][ky][kx]
//
// (x is MATLAB dims[0], the fast axis; kernel slot (x%nn, y%nn) is taken from the bitmap
// origin), zero outside the bitmap.  The reference clips the tap window at the edges
// (:55-78); for odd kw that is exactly zero padding.  For even kw its clip
// (bitmap_end = x + kw/2 + 1) never reaches the last input column / row, so those are
// treated as zero here too.
//
// All slices and output phases run in one launch (the reference issues one launch per
// slice on 16 streams, :396-405).  Each CTA computes a 32 x 8 output tile of one slice
// from a shared-memory input tile (tile + kernel halo, staged in row strips).
#include "mlf_internal.h"

namespace mlf {

namespace {

constexpr int CV_TX = 32, CV_TY = 8;   // output tile per CTA
constexpr int CV_STRIP = 16;           // input rows staged per step

__global__ void __launch_bounds__(CV_TX * CV_TY)
k_conv_vec(const float* __restrict__ in, int W, int H, const float* __restrict__ K, int kw, int nn,
           float* __restrict__ out) {
  extern __shared__ float tile[];  // [CV_STRIP + CV_TY - 1][CV_TX + kw - 1]
  const int hk = kw / 2;
  const int x0 = blockIdx.x * CV_TX, y0 = blockIdx.y * CV_TY;
  const int i = blockIdx.z;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x = x0 + tx, y = y0 + ty;
  const int tw = CV_TX + kw - 1;
  const int Wv = (kw % 2 == 0) ? W - 1 : W;  // even kw: last column / row never used
  const int Hv = (kw % 2 == 0) ? H - 1 : H;
  const float* src = in + (int64_t)i * W * H;
  const float* Kp = K + (int64_t)((y % nn) * nn + (x % nn)) * kw * kw;
  const int nthr = CV_TX * CV_TY, tid = ty * CV_TX + tx;
  float acc = 0.f;
  // input row for kernel row ky of output row y: y + ky - hk
  for (int ky0 = 0; ky0 < kw; ky0 += CV_STRIP) {
    const int nk = min(CV_STRIP, kw - ky0);
    const int rows = nk + CV_TY - 1;
    __syncthreads();
    for (int e = tid; e < rows * tw; e += nthr) {
      const int r = e / tw, c = e - r * tw;
      const int gy = y0 + ky0 + r - hk, gx = x0 + c - hk;
      float v = 0.f;
      if (gy >= 0 && gy < Hv && gx >= 0 && gx < Wv) v = __ldg(src + (int64_t)gy * W + gx);
      tile[e] = v;
    }
    __syncthreads();
    if (x < W && y < H) {
      for (int k = 0; k < nk; ++k) {
        const float* trow = tile + (ty + k) * tw + tx;
        const float* krow = Kp + (int64_t)(ky0 + k) * kw;
#pragma unroll 8
        for (int kx = 0; kx < kw; ++kx) acc = fmaf(trow[kx], __ldg(krow + kx), acc);
      }
    }
  }
  if (x < W && y < H) out[(int64_t)i * W * H + (int64_t)y * W + x] = acc;
}

}  // namespace

int conv_vec_run(const float* d_bitmap, int64_t W, int64_t H, int64_t n, const float* d_kernels,
                 int64_t kw, int nnum, float* d_out, cudaStream_t st) {
  const size_t smem = sizeof(float) * (size_t)(CV_STRIP + CV_TY - 1) * (CV_TX + kw - 1);
  MLF_TRY(allow_max_dyn_smem((const void*)k_conv_vec));
  const dim3 grid((unsigned)((W + CV_TX - 1) / CV_TX), (unsigned)((H + CV_TY - 1) / CV_TY), (unsigned)n);
  k_conv_vec<<<grid, dim3(CV_TX, CV_TY), smem, st>>>(d_bitmap, (int)W, (int)H, d_kernels, (int)kw,
                                                     nnum, d_out);
  MLF_LAUNCHED();
  return MLF_OK;
}

}  // namespace mlf
