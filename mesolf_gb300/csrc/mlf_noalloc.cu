// Forward projection of one view that allocates no device memory.
//
// Who needs it: callers that cannot call cudaMalloc / cudaFree.  A MATLAB MEX function
// that works on gpuArrays runs inside MATLAB's own GPU memory manager, which owns the
// device heap and may have it fully reserved; a frame callback of the 18 Hz acquisition
// loop must not block on the implicit device-wide synchronisation that cudaMalloc /
// cudaFree can cause.  Both already hold every input (the resident mlf_psf, the volume)
// and the output buffer; what the regular forward projection adds on top is scratch --
// the per-CTA partial sums of the projection and a phase-major copy of the volume.
//
// This variant reads the volume in its MATLAB layout directly (no phase-major copy) and
// keeps the per-CTA partial sums in a file-scope static device array,
// g_static_partials, of kStaticPartialFloats floats (8 MiB).  Every GPU that loads this
// library holds that array until the process exits.  Its device address is looked up with
// cudaGetSymbolAddress on every call, with the caller's device current: the lookup
// allocates nothing, and a cached address would go stale when the caller resets the device
// (MATLAB's reset(gpuDevice) runs cudaDeviceReset; the next context loads the module again,
// possibly at another address).  The first call on a device, and the first after a reset,
// makes the runtime load this library's device code, so it must come before any stream
// capture.  All calls on a device share the one array: every CTA overwrites the whole
// partial plane it owns before the reduction reads it, so no clearing is needed, but two
// calls whose kernels overlap on the GPU (different streams, or different host threads)
// race on the array and must be serialised by the caller.
//
// The projection is the per-channel forward correlation of k_view's MODE_FWD (mlf_view.cuh)
// with a tiling of its own: 8 x 4 tiles (VT_TY x VT_TX) through conv_tile on unswizzled
// planes, the plane gathered from the MATLAB-layout volume, taps at pitch T, partials
// reduced per CTA in shared memory.  It shares view_nw, view_qpad and conv_tile with
// mlf_view.cuh, not k_view's 4 x 8 tile, swizzled planes or slot partial planes; both add
// each output's products in the order (tap row, tap column), and tests/test_zz_no_alloc.py
// compares the two on every tap count it covers.
#include <cuda_runtime.h>

#include <algorithm>

#include "mlf_view.cuh"

struct mlf_psf;  // opaque: an mlf::Psf created by mlf_psf_create

namespace mlf {
namespace {

constexpr int64_t kStaticPartialFloats = int64_t(2) << 20;  // 2 Mi floats = 8 MiB
static __device__ __align__(256) float g_static_partials[kStaticPartialFloats];

// Device address of g_static_partials in the current context.
int static_partials(float** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_static_partials);
  if (e != cudaSuccess || p == nullptr)
    return fail(MLF_ERR_CUDA, std::string("cudaGetSymbolAddress(g_static_partials): ") + cudaGetErrorString(e));
  *out = static_cast<float*>(p);
  return MLF_OK;
}

struct StaticFwdArgs {
  const float* vol;  // (Xr, Xc, Z) column-major
  const float* wf;   // forward taps of the view [nch][T*T]
  float* part;       // [gridDim.x][Lj*Li] in the static array
  int64_t Xr, Xc, nch;
  int N, Z, Li, Lj, tilesA, tilesB, tps, slots, XP, XProws, slot_floats;
};

// Same per-channel forward correlation as k_view (MODE_FWD), with the plane gathered
// from the MATLAB-layout volume: P_ch[b][a] = vol(N a + alpha, N b + beta, z).
template <int T>
__global__ void __launch_bounds__(256, 2) k_fwd_static(StaticFwdArgs A) {
  extern __shared__ __align__(16) float sm[];
  constexpr int TT = T * T;
  constexpr int Q = (T - 1) / 2;
  constexpr int QP = view_qpad(Q);
  const int tid = threadIdx.x;
  const int slot = tid / A.tps;
  const int lt = tid - slot * A.tps;
  const bool slot_ok = slot < A.slots;
  const bool tile_ok = slot_ok && lt < A.tps;
  const int a0 = (lt % A.tilesA) * VT_TX, b0 = (lt / A.tilesA) * VT_TY;
  float* xin = sm + (slot_ok ? slot : 0) * A.slot_floats;
  float* wfs = xin + A.XProws * A.XP;
  for (int i = tid; i < A.slots * A.slot_floats; i += blockDim.x) sm[i] = 0.f;
  __syncthreads();
  float hx[VT_TY][VT_TX];
#pragma unroll
  for (int y = 0; y < VT_TY; ++y)
#pragma unroll
    for (int x = 0; x < VT_TX; ++x) hx[y][x] = 0.f;
  const int64_t step = (int64_t)gridDim.x * A.slots;
  for (int64_t base = (int64_t)blockIdx.x * A.slots; base < A.nch; base += step) {
    const int64_t ch = base + slot;
    const bool active = slot_ok && ch < A.nch;
    if (active) {
      const int z = (int)(ch % A.Z);
      const int alpha = (int)((ch / A.Z) % A.N);
      const int beta = (int)(ch / ((int64_t)A.Z * A.N));
      for (int i = lt; i < TT; i += A.tps) wfs[i] = __ldg(A.wf + ch * TT + i);
      if (lt < A.tps) {
        const float* src = A.vol + (int64_t)z * A.Xr * A.Xc + alpha + A.Xr * beta;
#pragma unroll
        for (int y = 0; y < VT_TY; ++y) {
          const int b = b0 + y;
          if (b >= A.Lj) continue;
#pragma unroll
          for (int x = 0; x < VT_TX; ++x) {
            const int a = a0 + x;
            xin[(b + Q) * A.XP + a0 + QP + x] =
                a < A.Li ? __ldg(src + (int64_t)A.N * a + A.Xr * (int64_t)A.N * b) : 0.f;
          }
        }
      }
    }
    __syncthreads();
    if (active && lt < A.tps) conv_tile<T, QP - Q>(xin + b0 * A.XP + a0, A.XP, wfs, hx);
    __syncthreads();
  }
  float* red = sm;  // [slots][Lj*Li]
  const int LL = A.Li * A.Lj;
  if (tile_ok) {
#pragma unroll
    for (int y = 0; y < VT_TY; ++y) {
      const int b = b0 + y;
      if (b >= A.Lj) continue;
#pragma unroll
      for (int x = 0; x < VT_TX; ++x)
        if (a0 + x < A.Li) red[slot * LL + b * A.Li + a0 + x] = hx[y][x];
    }
  }
  __syncthreads();
  float* out = A.part + (int64_t)blockIdx.x * LL;
  for (int i = tid; i < LL; i += blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < A.slots; ++k) s += red[k * LL + i];
    out[i] = s;
  }
}

// hx[i] = sum over CTAs of the partial planes, fixed order.
__global__ void k_static_reduce(const float* __restrict__ part, int nparts, int LL, float* hx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= LL) return;
  float s = 0.f;
  for (int k = 0; k < nparts; ++k) s += part[(int64_t)k * LL + i];
  hx[i] = s;
}

template <int T>
int run_static(const StaticFwdArgs& a, int nsm, size_t smem, int threads, int max_grid, cudaStream_t st,
               int* grid_out) {
  if (smem > 48 * 1024) MLF_TRY(allow_max_dyn_smem((const void*)k_fwd_static<T>));
  int per_sm = 1;
  MLF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fwd_static<T>, threads, smem));
  const int64_t want = (a.nch + a.slots - 1) / a.slots;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>({want, (int64_t)nsm * std::max(1, per_sm),
                                                                  (int64_t)max_grid}));
  k_fwd_static<T><<<grid, threads, smem, st>>>(a);
  MLF_LAUNCHED();
  *grid_out = grid;
  return MLF_OK;
}

}  // namespace
}  // namespace mlf

extern "C" int mlf_forward_view_static(const mlf_psf* psf_handle, const float* vol, int64_t Xr, int64_t Xc,
                                       int32_t u, int32_t v, float* hx, void* stream) {
  using namespace mlf;
  clear_error();
  if (!psf_handle || !vol || !hx) return fail(MLF_ERR_INVALID, "mlf_forward_view_static: null pointer");
  const Psf* psf = reinterpret_cast<const Psf*>(psf_handle);
  const int N = psf->N;
  if (Xr < N || Xc < N || Xr % N || Xc % N)
    return fail(MLF_ERR_INVALID, "mlf_forward_view_static: image sides must be positive multiples of Nnum");
  if (u < 0 || v < 0 || u >= N || v >= N) return fail(MLF_ERR_INVALID, "mlf_forward_view_static: view out of range");
  if (!is_device_ptr(vol) || !is_device_ptr(hx))
    return fail(MLF_ERR_INVALID, "mlf_forward_view_static: vol and hx must be device memory");
  int dev = 0, nsm = 0, dev_smem = 0;
  MLF_CUDA(cudaGetDevice(&dev));
  if (dev != psf->device) return fail(MLF_ERR_INVALID, "mlf_forward_view_static: the PSF lives on another device");
  MLF_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  MLF_CUDA(cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const int Li = (int)(Xr / N), Lj = (int)(Xc / N), T = psf->T;
  const int64_t LL = (int64_t)Li * Lj;
  if (LL > kStaticPartialFloats)
    return fail(MLF_ERR_INVALID, "mlf_forward_view_static: " + std::to_string(Li) + " x " + std::to_string(Lj) +
                                     " lenslets exceed the static scratch of " +
                                     std::to_string(kStaticPartialFloats) + " floats");
  StaticFwdArgs a{};
  a.vol = vol;
  a.wf = psf->wf.as<float>() + (int64_t)(u + N * v) * psf->taps_per_view;
  a.Xr = Xr; a.Xc = Xc; a.nch = psf->nch; a.N = N; a.Z = psf->Z; a.Li = Li; a.Lj = Lj;
  a.tilesA = (Li + 3) / 4;
  a.tilesB = (Lj + 7) / 8;
  a.tps = a.tilesA * a.tilesB;
  if (a.tps > 256)
    return fail(MLF_ERR_UNSUPPORTED, "mlf_forward_view_static: " + std::to_string(Li) + " x " + std::to_string(Lj) +
                                         " lenslets need ceil(Li/4)*ceil(Lj/8) = " + std::to_string(a.tps) +
                                         " tiles per CTA; the limit is 256");
  const int NW = view_nw(T);
  a.XP = ((4 * (a.tilesA - 1) + 4 * NW) + 3) / 4 * 4;
  a.XProws = a.tilesB * 8 + T - 1;
  a.slot_floats = (a.XProws * a.XP + T * T + 3) / 4 * 4;
  a.slots = a.tps >= 128 ? 1 : std::max(1, std::min(32, 192 / a.tps));
  const int threads = (a.slots * a.tps + 31) / 32 * 32;
  const size_t smem = sizeof(float) * (size_t)a.slots * std::max<int64_t>(a.slot_floats, LL);
  if ((int)smem > dev_smem) return fail(MLF_ERR_UNSUPPORTED, "mlf_forward_view_static: shared memory limit");
  MLF_TRY(static_partials(&a.part));
  const int max_grid = (int)(kStaticPartialFloats / LL);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int grid = 0;
  switch (T) {
    case 3: MLF_TRY(run_static<3>(a, nsm, smem, threads, max_grid, st, &grid)); break;
    case 5: MLF_TRY(run_static<5>(a, nsm, smem, threads, max_grid, st, &grid)); break;
    case 7: MLF_TRY(run_static<7>(a, nsm, smem, threads, max_grid, st, &grid)); break;
    case 9: MLF_TRY(run_static<9>(a, nsm, smem, threads, max_grid, st, &grid)); break;
    case 11: MLF_TRY(run_static<11>(a, nsm, smem, threads, max_grid, st, &grid)); break;
    case 13: MLF_TRY(run_static<13>(a, nsm, smem, threads, max_grid, st, &grid)); break;
    case 15: MLF_TRY(run_static<15>(a, nsm, smem, threads, max_grid, st, &grid)); break;
    case 17: MLF_TRY(run_static<17>(a, nsm, smem, threads, max_grid, st, &grid)); break;
    default: return fail(MLF_ERR_UNSUPPORTED, "mlf_forward_view_static: unsupported tap count");
  }
  k_static_reduce<<<(int)((LL + 255) / 256), 256, 0, st>>>(a.part, grid, (int)LL, hx);
  MLF_LAUNCHED();
  return MLF_OK;
}
