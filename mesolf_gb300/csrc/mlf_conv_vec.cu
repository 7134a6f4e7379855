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
// Direct kernel (k_conv_vec_rows).  The outputs of one row phase b = y % 15 share one set
// of 15 kernels (one per x phase), so a CTA takes rows y = b + 15 j of one slice and a
// thread owns a segment of 15 consecutive outputs x = 15 i + a, a = 0..14 -- one per x
// phase.  Per kernel row ky the CTA stages its input rows and the 15 kernels' row ky
// ([kx][a], padded to 16) in shared memory with zero-filling cp.async, double buffered so
// that row ky + 1 loads while row ky is computed.  Along kx the thread slides a window of
// 15 inputs in registers (one new shared load per step) and reads the step's 15 taps as
// broadcast 16-byte loads shared by the whole CTA; kw is padded to a multiple of 15 with
// zero taps so that the 15-step rotation of the window needs no tail.  Every output still adds its products in
// the reference's order -- kernel rows in order, each row left to right, one FP32 FMA chain
// (mex_lfm_convolution_vec.cu:147-251) -- and the products it adds beyond the reference's
// clipped window multiply zero-filled inputs, which adds exactly 0 for finite kernels; so
// the output equals the reference kernel's bit for bit (tests/test_gpu_ref_mex.py).
#include <algorithm>

#include "mlf_internal.h"

namespace mlf {

namespace {

constexpr int CV_NN = 15;            // kernels per axis (the reference's num_kernels)
constexpr int CV_MAX_THREADS = 768;  // rows a CTA's threads own at most (RPT rows per thread)
constexpr int CV_RPT = 2;            // output rows per thread

__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 4 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

struct ConvRowsArgs {
  const float* in;   // W x H x n slices (x fastest)
  const float* K;    // kw x kw x 15 x 15 (kx fastest; kernel (a, b) at kw*kw*(a + 15 b))
  float* out;
  int W, H, kw, hk, Wv, Hv;  // Wv, Hv: columns / rows that can contribute (even kw: W-1, H-1)
  int kwp;                   // kw rounded up to a multiple of 15 (the extra taps are zero)
  int sx, sy, tilesX;        // CTA tile: sx segments of 15 outputs x sy rows of one row phase
  int width, pitch;          // staged input row: 15 sx + kw - 1 floats, pitch odd
  int64_t slice0;            // first slice of this launch
};

// Stage input rows (row phase b, rows j0.., kernel row ky) and the 15 kernels' row ky into
// buffer sel (zero where the reference reads nothing), then commit the copies.
__device__ __forceinline__ void conv_rows_stage(const ConvRowsArgs& A, float* sm, float* rows0, int rowbuf,
                                                const float* src, const float* kb, int64_t kplane, int b,
                                                int j0, int nJ, int cstart, int ky, int sel) {
  const int tid = threadIdx.x, nthr = blockDim.x;
  float* rb = rows0 + sel * rowbuf;
  // element e = r_l * width + c, advanced by nthr per step without a division
  int r_l = tid / A.width, c = tid - r_l * A.width;
  for (int e = tid; e < A.sy * A.width; e += nthr) {
    const int r = b + CV_NN * (j0 + r_l) + ky - A.hk, col = cstart + c;
    const bool ok = (j0 + r_l) < nJ && r >= 0 && r < A.Hv && col >= 0 && col < A.Wv;
    cp_async4(rb + r_l * A.pitch + c, ok ? src + (int64_t)r * A.W + col : src, ok);
    c += nthr;
    while (c >= A.width) {
      c -= A.width;
      ++r_l;
    }
  }
  float* tb = sm + sel * 16 * A.kwp;
  const float* krow = kb + (int64_t)A.kw * ky;
  for (int e = tid; e < 16 * A.kwp; e += nthr) {
    const int kx = e >> 4, a = e & 15;
    const bool ok = a < CV_NN && kx < A.kw;
    cp_async4(tb + e, ok ? krow + kplane * a + kx : kb, ok);
  }
  cp_async_commit();
}

// RPT output rows per thread (rows jl*RPT .. jl*RPT + RPT-1 of the CTA's tile): the taps
// of a step, loaded once, serve RPT rows.
template <int RPT>
__global__ void __launch_bounds__(CV_MAX_THREADS / RPT, 1) k_conv_vec_rows(ConvRowsArgs A) {
  extern __shared__ __align__(16) float sm[];
  const int b = blockIdx.y;                      // row phase
  const int64_t slice = A.slice0 + blockIdx.z;
  const int i0 = (blockIdx.x % A.tilesX) * A.sx; // first segment
  const int j0 = (blockIdx.x / A.tilesX) * A.sy; // first row index of phase b
  const int nJ = b < A.H ? (A.H - b + CV_NN - 1) / CV_NN : 0;
  if (j0 >= nJ) return;                           // CTA-uniform
  const int tid = threadIdx.x;
  const int il = tid % A.sx, jl = (tid / A.sx) * RPT;
  const int x_seg = CV_NN * (i0 + il);
  bool mine[RPT];
  int yr[RPT];
#pragma unroll
  for (int r = 0; r < RPT; ++r) {
    yr[r] = b + CV_NN * (j0 + jl + r);
    mine[r] = jl + r < A.sy && x_seg < A.W && yr[r] < A.H;
  }
  const int cstart = CV_NN * i0 - A.hk;          // input column of staged column 0
  // taps first (16-byte aligned for the float4 loads), then the two row buffers
  const int rowbuf = A.sy * A.pitch;
  float* const rows0 = sm + 32 * A.kwp;  // buffer sel: taps sm + sel*16*kwp, rows rows0 + sel*rowbuf
  const float* src = A.in + slice * (int64_t)A.W * A.H;
  const int64_t kplane = (int64_t)A.kw * A.kw;
  const float* kb = A.K + kplane * CV_NN * b;    // kernels (a, b), a = 0..14

  float acc[RPT][CV_NN];
#pragma unroll
  for (int r = 0; r < RPT; ++r)
#pragma unroll
    for (int a = 0; a < CV_NN; ++a) acc[r][a] = 0.f;
  conv_rows_stage(A, sm, rows0, rowbuf, src, kb, kplane, b, j0, nJ, cstart, 0, 0);
  cp_async_wait0();
  __syncthreads();
  for (int ky = 0; ky < A.kw; ++ky) {
    const int sel = ky & 1;
    if (ky + 1 < A.kw) conv_rows_stage(A, sm, rows0, rowbuf, src, kb, kplane, b, j0, nJ, cstart, ky + 1, sel ^ 1);
    if (mine[0]) {
      // rows past the tile read staged rows that exist (jl + r < sy is not required for the
      // read: the buffer holds sy rows, so clamp) and are not stored
      const float* rowp[RPT];
#pragma unroll
      for (int r = 0; r < RPT; ++r) rowp[r] = rows0 + sel * rowbuf + min(jl + r, A.sy - 1) * A.pitch + CV_NN * il;
      const float* tp = sm + sel * 16 * A.kwp;
      float w[RPT][CV_NN];  // w[r][(m + a) % 15] holds rowp[r][kx0 + m + a]
#pragma unroll
      for (int r = 0; r < RPT; ++r)
#pragma unroll
        for (int a = 0; a < CV_NN - 1; ++a) w[r][a] = rowp[r][a];
      for (int kx0 = 0; kx0 < A.kwp; kx0 += CV_NN) {
#pragma unroll
        for (int m = 0; m < CV_NN; ++m) {
#pragma unroll
          for (int r = 0; r < RPT; ++r) w[r][(m + CV_NN - 1) % CV_NN] = rowp[r][kx0 + m + CV_NN - 1];
          const float4* t4 = reinterpret_cast<const float4*>(tp + 16 * (kx0 + m));
          float t[16];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float4 v = t4[q];
            t[4 * q] = v.x;
            t[4 * q + 1] = v.y;
            t[4 * q + 2] = v.z;
            t[4 * q + 3] = v.w;
          }
#pragma unroll
          for (int r = 0; r < RPT; ++r)
#pragma unroll
            for (int a = 0; a < CV_NN; ++a) acc[r][a] = fmaf(w[r][(m + a) % CV_NN], t[a], acc[r][a]);
        }
      }
    }
    cp_async_wait0();
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < RPT; ++r) {
    if (!mine[r]) continue;
    float* o = A.out + slice * (int64_t)A.W * A.H + (int64_t)yr[r] * A.W;
#pragma unroll
    for (int a = 0; a < CV_NN; ++a)
      if (x_seg + a < A.W) o[x_seg + a] = acc[r][a];
  }
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
  if (nnum != CV_NN) return fail(MLF_ERR_INVALID, "direct MEX projector: the kernel grid must be 15 x 15");
  if (W > (1 << 24) || H > (1 << 24) || W * H > ((int64_t)1 << 31))
    return fail(MLF_ERR_UNSUPPORTED, "direct MEX projector: slice larger than 2^31 pixels");
  int dev = 0, optin = 0;
  MLF_CUDA(cudaGetDevice(&dev));
  MLF_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  MLF_TRY(allow_max_dyn_smem((const void*)k_conv_vec_rows<CV_RPT>));
  ConvRowsArgs a{};
  a.in = d_bitmap;
  a.K = d_kernels;
  a.out = d_out;
  a.W = (int)W;
  a.H = (int)H;
  a.kw = (int)kw;
  a.hk = (int)(kw / 2);
  a.kwp = (a.kw + CV_NN - 1) / CV_NN * CV_NN;
  a.Wv = (kw % 2 == 0) ? a.W - 1 : a.W;  // even kw: the reference's clip never reaches the last column / row
  a.Hv = (kw % 2 == 0) ? a.H - 1 : a.H;
  const int nI = (a.W + CV_NN - 1) / CV_NN, nJ = (a.H + CV_NN - 1) / CV_NN;
  a.sx = std::min(nI, 32);
  a.width = CV_NN * a.sx + a.kwp - 1;
  a.pitch = a.width | 1;  // odd: rows of a warp fall on different banks
  const size_t tap_bytes = sizeof(float) * 2 * 16 * (size_t)a.kwp;
  const size_t budget = (size_t)optin - 1024;
  a.sy = std::max(1, std::min(nJ, CV_RPT * (CV_MAX_THREADS / CV_RPT / a.sx)));
  while (a.sy > 1 && sizeof(float) * 2 * (size_t)a.sy * a.pitch + tap_bytes > budget) --a.sy;
  const size_t smem = sizeof(float) * 2 * (size_t)a.sy * a.pitch + tap_bytes;
  if (smem > budget) return fail(MLF_ERR_UNSUPPORTED, "direct MEX projector: kernel row does not fit in shared memory");
  a.tilesX = (nI + a.sx - 1) / a.sx;
  const int tilesY = (nJ + a.sy - 1) / a.sy;
  const int threads = (a.sx * ((a.sy + CV_RPT - 1) / CV_RPT) + 31) / 32 * 32;
  for (int64_t s0 = 0; s0 < n; s0 += 65535) {
    a.slice0 = s0;
    const dim3 grid((unsigned)(a.tilesX * tilesY), CV_NN, (unsigned)std::min<int64_t>(65535, n - s0));
    k_conv_vec_rows<CV_RPT><<<grid, threads, smem, st>>>(a);
    MLF_LAUNCHED();
  }
  return MLF_OK;
}

}  // namespace mlf
