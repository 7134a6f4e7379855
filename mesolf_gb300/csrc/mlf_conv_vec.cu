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

// ---- tensor-core route: the correlation above (kernel slot from the OUTPUT pixel's phase)
// equals the full light-field forward projection (PSF slice from the SOURCE pixel's phase,
// forwardProjectGPU.m) of the re-indexed kernel
//   H'[d][psi] = K[c - d + hk][(psi - (c - d)) mod 15]   per axis, c = (K0-1)/2, hk = kw/2,
// embedded in K0 = 15 + 30 m >= kw + 14 so that every tap lies inside the phase-space crop.
__global__ void k_mex_reindex(const float* __restrict__ K, int kw, int K0, int nn, float* __restrict__ Hp) {
  const int c = (K0 - 1) / 2, hk = kw / 2;
  const int64_t total = (int64_t)K0 * K0 * nn * nn;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int dx = (int)(e % K0);
    const int dy = (int)((e / K0) % K0);
    const int px = (int)((e / ((int64_t)K0 * K0)) % nn);
    const int py = (int)(e / ((int64_t)K0 * K0 * nn));
    const int kx = c - dx + hk, ky = c - dy + hk;
    float v = 0.f;
    if (kx >= 0 && kx < kw && ky >= 0 && ky < kw) {
      const int fx = ((px - (c - dx)) % nn + nn) % nn, fy = ((py - (c - dy)) % nn + nn) % nn;
      v = K[(int64_t)kx + (int64_t)kw * (ky + (int64_t)kw * (fx + (int64_t)nn * fy))];
    }
    Hp[e] = v;
  }
}

// slices of the bitmap -> zero-padded Wp x Hq slices; for even kw the reference never reads
// the last input row / column, so they are zeroed
__global__ void k_mex_pad(const float* __restrict__ bm, int64_t W, int64_t H, int64_t n, int64_t Wp, int64_t Hq,
                          int zero_last, float* __restrict__ dst) {
  const int64_t total = Wp * Hq * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = e % Wp, y = (e / Wp) % Hq, i = e / (Wp * Hq);
    float v = 0.f;
    if (x < W && y < H && !(zero_last && (x == W - 1 || y == H - 1))) v = bm[x + W * (y + H * i)];
    dst[e] = v;
  }
}

// dst += src zero-padded to Wp x Hq (one slice; last row / column dropped for even kw)
__global__ void k_mex_pad_add(const float* __restrict__ src, int64_t W, int64_t H, int64_t Wp, int64_t Hq,
                              int zero_last, float* __restrict__ dst) {
  const int64_t total = W * H;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = e % W, y = e / W;
    if (zero_last && (x == W - 1 || y == H - 1)) continue;
    dst[x + Wp * y] += src[e];
  }
}

__global__ void k_mex_crop(const float* __restrict__ src, int64_t Wp, int64_t Hq, int64_t W, int64_t H, int64_t n,
                           float* __restrict__ out) {
  const int64_t total = W * H * n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = e % W, y = (e / W) % H, i = e / (W * H);
    out[e] = src[x + Wp * (y + Hq * i)];
  }
}

}  // namespace

int launch_mex_reindex(const float* K, int kw, int K0, int nn, float* Hp, cudaStream_t st) {
  k_mex_reindex<<<2048, 256, 0, st>>>(K, kw, K0, nn, Hp);
  MLF_LAUNCHED();
  return MLF_OK;
}
int launch_mex_pad(const float* bm, int64_t W, int64_t H, int64_t n, int64_t Wp, int64_t Hq, bool zero_last,
                   float* dst, cudaStream_t st) {
  k_mex_pad<<<2048, 256, 0, st>>>(bm, W, H, n, Wp, Hq, zero_last ? 1 : 0, dst);
  MLF_LAUNCHED();
  return MLF_OK;
}
int launch_mex_pad_add(const float* src, int64_t W, int64_t H, int64_t Wp, int64_t Hq, bool zero_last, float* dst,
                       cudaStream_t st) {
  k_mex_pad_add<<<512, 256, 0, st>>>(src, W, H, Wp, Hq, zero_last ? 1 : 0, dst);
  MLF_LAUNCHED();
  return MLF_OK;
}
int launch_mex_crop(const float* src, int64_t Wp, int64_t Hq, int64_t W, int64_t H, int64_t n, float* out,
                    cudaStream_t st) {
  k_mex_crop<<<2048, 256, 0, st>>>(src, Wp, Hq, W, H, n, out);
  MLF_LAUNCHED();
  return MLF_OK;
}

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
