// Rectification of raw sensor frames onto the lenslet-aligned grid, the input step of the
// pipeline: src/module/image_load_module_aug.m:19-164 (frame selection and averaging,
// raw-patch cut, img_rectify_mod, division by the movie max).
//
// img_rectify_mod (:126-164) resamples a raw patch with griddedInterpolant (bilinear, linear
// extrapolation, 1-based sample coordinates 1..H, 1..W) onto the grid
//   R = [fliplr(c : -dx/M : -dx/M), c+dx/M : dx/M : size+0.9]
// per axis (c = lenslet centre inside the patch), drops the first mod(idx(c) - floor(M/2), M)
// grid points so that lenslets start on a multiple of M, evaluates, and keeps the first
// M*floor(n/M) rows and columns.  The grids are computed here on the host in FP64 and turned
// into per-row and per-column (cell, weight) tables; the kernel gathers the four neighbours of
// every output pixel of every output frame, averaging the selected input frames first (the
// interpolation is linear, so this is the reference's mean-then-rectify).
//
// One launch covers all output frames.  Frame averaging (k_rectify): thread per output row
// of one column (coalesced along the fast axis of the output, which maps to
// near-consecutive raw rows) and 8 output frames, with all 32 neighbour loads of the 8
// frames in flight before the interpolation.  One input frame per output frame
// (k_rectify_staged): the raw tile of a block is staged in shared memory by 16-byte copies
// and the next frame chunk is prefetched while the current one is interpolated.  The raw
// data is read once from HBM.
#include "mlf_internal.h"

#include <algorithm>
#include <cmath>

namespace mlf {

namespace {


template <typename TIn>
__device__ __forceinline__ float ldv(const TIn* p) {
  return (float)__ldg(p);
}

// out[(r + oh*c) + P*i] = bilinear(mean of frames f0 + i*fstep + j, j < navg_i) at row cell
// iy[r] (weight wy[r]) and column cell ix[c] (weight wx[c]).  Frame f of the input is at
// raw + f*fstride; element (row, col) of the cut at (row0 + row) + cstride*(col0 + col).
// Block: RC_ROWS output rows x RC_COLS columns (threadIdx.y), output frames in chunks of
// RC_FCH (all 4*RC_FCH neighbour loads of a chunk in flight before the interpolation), RC_NCH
// chunks per block; the tables are read once per thread.
constexpr int RC_ROWS = 128, RC_COLS = 4, RC_FCH = 8, RC_NCH = 8;

template <typename TIn>
__global__ void __launch_bounds__(RC_ROWS * RC_COLS)
k_rectify(const TIn* __restrict__ raw, int64_t fstride, int64_t cstride, int64_t row0, int64_t col0,
          const int* __restrict__ iy, const float* __restrict__ wy, int oh, const int* __restrict__ ix,
          const float* __restrict__ wx, int ow, int64_t f0, int64_t fstep, int navg, int64_t flast, int64_t n_out,
          float* __restrict__ out) {
  const int r = blockIdx.x * RC_ROWS + threadIdx.x;
  const int c = blockIdx.y * RC_COLS + threadIdx.y;
  if (r >= oh || c >= ow) return;
  const int64_t P = (int64_t)oh * ow;
  const int i0 = __ldg(iy + r), j0 = __ldg(ix + c);
  const float fy = __ldg(wy + r), fx = __ldg(wx + c);
  const int64_t o00 = (row0 + i0) + cstride * (col0 + j0);
  const int64_t o01 = o00 + cstride;
  float* op = out + r + (int64_t)oh * c;
  for (int ch = 0; ch < RC_NCH; ++ch) {
    const int64_t ib = ((int64_t)blockIdx.z * RC_NCH + ch) * RC_FCH;
    if (ib >= n_out) return;
    const int ni = (int)(n_out - ib < RC_FCH ? n_out - ib : RC_FCH);
    if (navg == 1) {
      float v[RC_FCH][4];
#pragma unroll
      for (int q = 0; q < RC_FCH; ++q) {
        if (q < ni) {
          const TIn* fr = raw + (f0 + (ib + q) * fstep) * fstride;
          v[q][0] = ldv(fr + o00);
          v[q][1] = ldv(fr + o00 + 1);
          v[q][2] = ldv(fr + o01);
          v[q][3] = ldv(fr + o01 + 1);
        }
      }
#pragma unroll
      for (int q = 0; q < RC_FCH; ++q) {
        if (q < ni) {
          const float a = fmaf(fx, v[q][2] - v[q][0], v[q][0]), b = fmaf(fx, v[q][3] - v[q][1], v[q][1]);
          __stcs(op + P * (ib + q), fmaf(fy, b - a, a));
        }
      }
      continue;
    }
    for (int q = 0; q < ni; ++q) {
      const int64_t fa = f0 + (ib + q) * fstep;
      const int64_t fb = min(fa + navg - 1, flast);
      float v00 = 0.f, v10 = 0.f, v01 = 0.f, v11 = 0.f;
      for (int64_t f = fa; f <= fb; ++f) {
        const TIn* fr = raw + f * fstride;
        v00 += ldv(fr + o00);
        v10 += ldv(fr + o00 + 1);
        v01 += ldv(fr + o01);
        v11 += ldv(fr + o01 + 1);
      }
      const float rn = 1.f / (float)(fb - fa + 1);
      const float a = fmaf(fx, v01 - v00, v00), b = fmaf(fx, v11 - v10, v10);
      __stcs(op + P * (ib + q), fmaf(fy, b - a, a) * rn);
    }
  }
}

// The same for one input frame per output frame (navg = 1), with the raw tile of each block
// staged in shared memory by 16-byte loads: block = RC_ROWS x RC_COLS output pixels, chunks of
// SF output frames (blockIdx.z).  For frame q and raw column k of the block's footprint (raw
// columns ix[c0] .. ix[c1]+1, rows iy[r0] .. iy[r1]+1) the column segment is loaded from the
// 16-byte boundary at or below its first element into slot [q][k] (`slot` elements), its
// start at off[q][k] inside the slot.  A few wide loads per thread replace four narrow
// gathers per output pixel and frame.  raw must be 16-byte aligned; `total` = elements of
// the frame buffer (vectors that would cross its end are loaded per element).
constexpr int SF = 16;

// exact uint16 -> float with one logic op and one add: the bits 0x4B000000 | x are the float
// 2^23 + x (x < 2^23 fits the mantissa)
__device__ __forceinline__ float to_f(uint16_t x) { return __uint_as_float(0x4B000000u | x) - 8388608.f; }
__device__ __forceinline__ float to_f(float x) { return x; }

__device__ __forceinline__ void rc_cp_async16(void* smem, const void* gmem, int src_bytes) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(gmem), "r"(src_bytes) : "memory");
}

// Persistent over frame chunks z = blockIdx.z, blockIdx.z + gridDim.z, ...: the raw tile of
// chunk z+1 is copied into the second buffer (16-byte zero-filling cp.async, no register
// round trip) while chunk z is interpolated, so DRAM loads stay in flight.
template <typename TIn>
__global__ void __launch_bounds__(RC_ROWS * RC_COLS, 3)
k_rectify_staged(const TIn* __restrict__ raw, int64_t total, int64_t fstride, int64_t cstride, int64_t row0,
                 int64_t col0, const int* __restrict__ iy, const float* __restrict__ wy, int oh,
                 const int* __restrict__ ix, const float* __restrict__ wx, int ow, int64_t f0, int64_t fstep,
                 int64_t n_out, int slot, int maxc, int same_align, float* __restrict__ out) {
  constexpr int VEC = 16 / sizeof(TIn);
  constexpr int NT = RC_ROWS * RC_COLS;
  extern __shared__ __align__(16) unsigned char rc_smem[];
  TIn* tiles = reinterpret_cast<TIn*>(rc_smem);  // [2 buffers][SF][maxc][slot]
  __shared__ int off[2][SF][8];
  const int tid = threadIdx.y * RC_ROWS + threadIdx.x;
  const int r0 = blockIdx.x * RC_ROWS, c0 = blockIdx.y * RC_COLS;
  const int r1 = min(r0 + RC_ROWS, oh) - 1, c1 = min(c0 + RC_COLS, ow) - 1;
  const int rlo = __ldg(iy + r0), nrow = __ldg(iy + r1) + 2 - rlo;
  const int clo = __ldg(ix + c0), ncol = __ldg(ix + c1) + 2 - clo;  // <= maxc (host bound)
  const int nv = (nrow + 2 * VEC - 2) / VEC;                         // vectors per column segment
  const int64_t chunks = (n_out + SF - 1) / SF;
  const int64_t fs = (int64_t)SF * maxc * slot;                    // elements per buffer
  // staging role of this thread: one (column k, vector v) of the footprint, frames q = g, g+G, ...
  const int cnv = ncol * nv;
  const int G = NT / cnv;  // >= 1: the host bounds nrow and maxc
  const int sg = tid / cnv, srem = tid - sg * cnv;
  const int sk = srem / nv, sv = srem - sk * nv;
  const int64_t colbase = (row0 + rlo) + cstride * (col0 + clo + sk);
  auto stage = [&](int64_t z, int b) {
    if (sg >= G) return;
    const int64_t ib = z * SF;
    const int nf = (int)(n_out - ib < SF ? n_out - ib : SF);
    const int64_t fdelta = (int64_t)G * fstep * fstride;
    int64_t e = (f0 + (ib + sg) * fstep) * fstride + colbase;
    for (int q = sg; q < nf; q += G, e += fdelta) {
      const int64_t ea = e & ~(int64_t)(VEC - 1);
      if (sv == 0) off[b][q][sk] = (int)(e - ea);
      TIn* dst = tiles + b * fs + ((int64_t)q * maxc + sk) * slot + (int64_t)sv * VEC;
      const int64_t src = ea + (int64_t)sv * VEC;
      const int64_t avail = total - src;  // elements of the frame buffer left from src
      const int nbytes = avail >= VEC ? 16 : (avail > 0 ? (int)avail * (int)sizeof(TIn) : 0);
      rc_cp_async16(dst, nbytes > 0 ? (const void*)(raw + src) : (const void*)raw, nbytes);
    }
  };
  const int r = r0 + threadIdx.x, c = c0 + threadIdx.y;
  const bool mine = r < oh && c < ow;
  const int lr = mine ? __ldg(iy + r) - rlo : 0, lc = mine ? __ldg(ix + c) - clo : 0;
  const float fy = mine ? __ldg(wy + r) : 0.f, fx = mine ? __ldg(wx + c) : 0.f;
  const int64_t P = (int64_t)oh * ow;
  const int per = maxc * slot;  // elements per staged frame
  int b = 0;
  if (blockIdx.z < chunks) stage(blockIdx.z, 0);
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  for (int64_t z = blockIdx.z; z < chunks; z += gridDim.z, b ^= 1) {
    const int64_t zn = z + gridDim.z;
    if (zn < chunks) stage(zn, b ^ 1);  // the other buffer was last read before the barrier below
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 1;\n" ::: "memory");
    __syncthreads();  // chunk z staged by every thread
    if (mine) {
      const int64_t ib = z * SF;
      const int nf = (int)(n_out - ib < SF ? n_out - ib : SF);
      float* op = out + r + (int64_t)oh * c + P * ib;
      const TIn* base = tiles + b * fs + (int64_t)lc * slot + lr;
      if (same_align) {
        // every frame has the same 16-byte alignment: the column offsets of frame 0 serve all
        const TIn* ca = base + off[b][0][lc];
        const TIn* cb = base + slot + off[b][0][lc + 1];
#pragma unroll
        for (int q = 0; q < SF; ++q) {
          if (q < nf) {
            const float v00 = to_f(ca[q * per]), v10 = to_f(ca[q * per + 1]);
            const float v01 = to_f(cb[q * per]), v11 = to_f(cb[q * per + 1]);
            const float a = fmaf(fx, v01 - v00, v00), bb = fmaf(fx, v11 - v10, v10);
            __stcs(op + P * q, fmaf(fy, bb - a, a));
          }
        }
      } else {
#pragma unroll 4
        for (int q = 0; q < nf; ++q) {
          const TIn* ca = base + (int64_t)q * per + off[b][q][lc];
          const TIn* cb = base + (int64_t)q * per + slot + off[b][q][lc + 1];
          const float v00 = to_f(ca[0]), v10 = to_f(ca[1]), v01 = to_f(cb[0]), v11 = to_f(cb[1]);
          const float a = fmaf(fx, v01 - v00, v00), bb = fmaf(fx, v11 - v10, v10);
          __stcs(op + P * q, fmaf(fy, bb - a, a));
        }
      }
    }
    __syncthreads();  // buffer b is read: the next iteration may stage into it
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

__global__ void k_rc_max(const float* __restrict__ a, int64_t n, float* __restrict__ part) {
  __shared__ float sh[32];
  float m = -INFINITY;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, a[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, sh[w]);
    part[blockIdx.x] = m;
  }
}

__global__ void k_rc_scale(float* __restrict__ a, int64_t n, const float* __restrict__ part, int nparts) {
  __shared__ float mx;
  if (threadIdx.x == 0) {
    float m = -INFINITY;
    for (int i = 0; i < nparts; ++i) m = fmaxf(m, part[i]);
    mx = m;
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = a[i] / mx;
}

// MATLAB a:d:b (d != 0): count floor((b-a)/d) + 1 with a relative tolerance of 1e-10
int64_t colon_count(double a, double d, double b) {
  const double q = (b - a) / d;
  const double tol = 1e-10 * std::max(1.0, std::fabs(q));
  if (q < -tol) return 0;
  return (int64_t)std::floor(q + tol) + 1;
}

}  // namespace

// One axis of img_rectify_mod: query coordinates of the kept grid (before the cut to whole
// lenslets), 1-based.  lo = -dx/M, hi = n + 0.9.
std::vector<double> rectify_axis_query(double center, double lo, double hi, int M, double dx) {
  const double s = dx / M;
  const int64_t nl = colon_count(center, -s, lo), nr = colon_count(center + s, s, hi);
  std::vector<double> R;
  R.reserve((size_t)(nl + nr));
  for (int64_t k = nl - 1; k >= 0; --k) R.push_back(center - s * (double)k);
  for (int64_t k = 0; k < nr; ++k) R.push_back(center + s + s * (double)k);
  const int64_t c0 = nl - M / 2;  // find(R == center) = nl (1-based)
  const int64_t qinit = c0 - (int64_t)M * (int64_t)std::floor((double)c0 / M);
  if (qinit > (int64_t)R.size()) return {};
  return std::vector<double>(R.begin() + qinit, R.end());
}

int rectify_run(const void* d_raw, int dtype, int64_t total, int64_t fstride, int64_t cstride, int64_t row0, int64_t col0,
                int64_t h, int64_t w, double xc, double yc, int M, double dx, int64_t out_h, int64_t out_w,
                int64_t f0, int64_t fstep, int navg, int64_t flast, int64_t n_out, float* d_out, bool normalize,
                cudaStream_t st) {
  std::vector<double> xq = rectify_axis_query(xc, -dx / M, (double)w + 0.9, M, dx);
  std::vector<double> yq = rectify_axis_query(yc, -dx / M, (double)h + 0.9, M, dx);
  const int64_t kh = M * ((int64_t)yq.size() / M), kw = M * ((int64_t)xq.size() / M);
  if (kh != out_h || kw != out_w)
    return fail(MLF_ERR_INVALID, "After raw patch read and rectification, the shape is different from what was "
                                 "expected. (" + std::to_string(kh) + " x " + std::to_string(kw) + " vs " +
                                 std::to_string(out_h) + " x " + std::to_string(out_w) + ")");
  // per-row / per-column cell (0-based, clamped to [0, n-2]) and weight inside the cell
  std::vector<int> iy(out_h), ix(out_w);
  std::vector<float> wy(out_h), wx(out_w);
  for (int64_t r = 0; r < out_h; ++r) {
    const double c = std::min(std::max(std::floor(yq[r]), 1.0), (double)(h - 1));
    iy[r] = (int)c - 1;
    wy[r] = (float)(yq[r] - c);
  }
  for (int64_t c = 0; c < out_w; ++c) {
    const double cc = std::min(std::max(std::floor(xq[c]), 1.0), (double)(w - 1));
    ix[c] = (int)cc - 1;
    wx[c] = (float)(xq[c] - cc);
  }
  DevBuf tabs;
  const size_t tb = sizeof(int) * (out_h + out_w) + sizeof(float) * (out_h + out_w);
  MLF_TRY(tabs.alloc(tb, "rectification tables"));
  char* base = static_cast<char*>(tabs.p);
  int* d_iy = reinterpret_cast<int*>(base);
  int* d_ix = d_iy + out_h;
  float* d_wy = reinterpret_cast<float*>(d_ix + out_w);
  float* d_wx = d_wy + out_h;
  MLF_CUDA(cudaMemcpyAsync(d_iy, iy.data(), sizeof(int) * out_h, cudaMemcpyHostToDevice, st));
  MLF_CUDA(cudaMemcpyAsync(d_ix, ix.data(), sizeof(int) * out_w, cudaMemcpyHostToDevice, st));
  MLF_CUDA(cudaMemcpyAsync(d_wy, wy.data(), sizeof(float) * out_h, cudaMemcpyHostToDevice, st));
  MLF_CUDA(cudaMemcpyAsync(d_wx, wx.data(), sizeof(float) * out_w, cudaMemcpyHostToDevice, st));
  const int64_t P = out_h * out_w;
  // largest raw tile of a block (rows and columns of the four-neighbour footprint)
  int maxr = 0, maxc = 0;
  for (int64_t r0 = 0; r0 < out_h; r0 += RC_ROWS)
    maxr = std::max(maxr, iy[std::min<int64_t>(r0 + RC_ROWS, out_h) - 1] + 2 - iy[r0]);
  for (int64_t c0 = 0; c0 < out_w; c0 += RC_COLS)
    maxc = std::max(maxc, ix[std::min<int64_t>(c0 + RC_COLS, out_w) - 1] + 2 - ix[c0]);
  const int es = dtype == MLF_DTYPE_U16 ? 2 : 4, vec = 16 / es;
  const int slot = ((maxr + 2 * vec - 2) / vec) * vec;
  const size_t smem = 2 * (size_t)SF * maxc * slot * es;  // two chunk buffers
  const bool staged = navg == 1 && reinterpret_cast<uintptr_t>(d_raw) % 16 == 0 && maxc <= 8 &&
                      smem <= 112 * 1024 && (out_w + RC_COLS - 1) / RC_COLS <= 65535;
  const dim3 block(RC_ROWS, RC_COLS);
  if (staged) {
    const void* kf = dtype == MLF_DTYPE_U16 ? (const void*)k_rectify_staged<uint16_t> : (const void*)k_rectify_staged<float>;
    MLF_TRY(allow_max_dyn_smem(kf));
    const int64_t chunks = (n_out + SF - 1) / SF;
    // frames whose starts differ by multiples of 16 bytes share the staged column offsets
    const int same_align = ((fstep * fstride) % vec == 0) ? 1 : 0;
    if (chunks > 65535) return fail(MLF_ERR_UNSUPPORTED, "mlf_rectify_frames: more than 1048560 output frames");
    // blocks loop over frame chunks (prefetching the next one): enough z-slices for about
    // sixteen waves of resident blocks (a short last wave), each slice walking its chunks
    int dev = 0, nsm = 0;
    MLF_CUDA(cudaGetDevice(&dev));
    MLF_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int64_t gxy = ((out_h + RC_ROWS - 1) / RC_ROWS) * ((out_w + RC_COLS - 1) / RC_COLS);
    const int64_t zb = std::max<int64_t>(1, std::min<int64_t>(chunks, (16 * 3 * (int64_t)nsm + gxy - 1) / gxy));
    const dim3 grid((unsigned)((out_h + RC_ROWS - 1) / RC_ROWS), (unsigned)((out_w + RC_COLS - 1) / RC_COLS),
                    (unsigned)zb);
    if (dtype == MLF_DTYPE_U16)
      k_rectify_staged<uint16_t><<<grid, block, smem, st>>>(static_cast<const uint16_t*>(d_raw), total, fstride,
                                                            cstride, row0, col0, d_iy, d_wy, (int)out_h, d_ix, d_wx,
                                                            (int)out_w, f0, fstep, n_out, slot, maxc, same_align,
                                                            d_out);
    else
      k_rectify_staged<float><<<grid, block, smem, st>>>(static_cast<const float*>(d_raw), total, fstride, cstride,
                                                         row0, col0, d_iy, d_wy, (int)out_h, d_ix, d_wx, (int)out_w,
                                                         f0, fstep, n_out, slot, maxc, same_align, d_out);
    MLF_LAUNCHED();
  } else {
  const int64_t per_block = (int64_t)RC_FCH * RC_NCH;
  if ((n_out + per_block - 1) / per_block > 65535 || (out_w + RC_COLS - 1) / RC_COLS > 65535)
    return fail(MLF_ERR_UNSUPPORTED, "mlf_rectify_frames: too many output frames or columns for one launch");
  const dim3 grid((unsigned)((out_h + RC_ROWS - 1) / RC_ROWS), (unsigned)((out_w + RC_COLS - 1) / RC_COLS),
                  (unsigned)((n_out + per_block - 1) / per_block));
  if (dtype == MLF_DTYPE_U16)
    k_rectify<uint16_t><<<grid, block, 0, st>>>(static_cast<const uint16_t*>(d_raw), fstride, cstride, row0, col0,
                                                  d_iy, d_wy, (int)out_h, d_ix, d_wx, (int)out_w, f0, fstep, navg,
                                                  flast, n_out, d_out);
  else
    k_rectify<float><<<grid, block, 0, st>>>(static_cast<const float*>(d_raw), fstride, cstride, row0, col0, d_iy,
                                               d_wy, (int)out_h, d_ix, d_wx, (int)out_w, f0, fstep, navg, flast, n_out,
                                               d_out);
  }
  MLF_LAUNCHED();
  if (normalize) {
    constexpr int NB = 1024;
    DevBuf part;
    MLF_TRY(part.alloc(sizeof(float) * NB, "rectification max partials"));
    k_rc_max<<<NB, 256, 0, st>>>(d_out, P * n_out, part.as<float>());
    k_rc_scale<<<NB, 256, 0, st>>>(d_out, P * n_out, part.as<float>(), NB);
    MLF_LAUNCHED();
    MLF_CUDA(cudaStreamSynchronize(st));
  } else {
    MLF_CUDA(cudaStreamSynchronize(st));  // tables are released on return
  }
  return MLF_OK;
}

}  // namespace mlf
