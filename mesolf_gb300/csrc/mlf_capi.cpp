// extern "C" entry points of libmesolf_lf.so (declared in include/mesolf_lf.h).
//
// Argument validation mirrors the reference's own checks (the MEX at
// src/cuda/mex_lfm_convolution_vec.cu:301-355 and the shape assumptions of
// recon_theory_phase_space_LFM_with_filter.m); failures return a status code and set a
// per-thread message instead of aborting.  Pointers may be device or host memory: host
// arrays are staged through device buffers owned by the call or the solver.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "mlf_internal.h"

namespace mlf {

namespace {
// NVTX range for the duration of an entry point (visible to nsys / ncu --nvtx; a no-op
// when no tool is attached).
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
};
}  // namespace

namespace {
thread_local int g_code = MLF_OK;
thread_local std::string g_msg;
}  // namespace

int fail(int code, const std::string& msg) {
  g_code = code;
  g_msg = msg;
  return code;
}

void clear_error() {
  g_code = MLF_OK;
  g_msg.clear();
}

int DevBuf::alloc(size_t n, const char* what) {
  release();
  if (n == 0) n = 16;
  std::lock_guard<std::recursive_mutex> lk(device_mutex());
  cudaError_t e = cudaMalloc(&p, n);
  if (e != cudaSuccess) {
    cudaGetLastError();
    p = nullptr;
    return fail(MLF_ERR_NOMEM, std::string("cudaMalloc(") + std::to_string(n) + " B) for " + what +
                                   ": " + cudaGetErrorString(e));
  }
  bytes = n;
  return MLF_OK;
}

std::recursive_mutex& device_mutex() {
  static std::recursive_mutex m;
  return m;
}

void DevBuf::release() {
  if (p) {
    std::lock_guard<std::recursive_mutex> lk(device_mutex());
    cudaFree(p);
  }
  p = nullptr;
  bytes = 0;
}

int allow_max_dyn_smem(const void* func) {
  int dev = 0, optin = 0;
  MLF_CUDA(cudaGetDevice(&dev));
  MLF_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  MLF_CUDA(cudaFuncGetAttributes(&fa, func));
  MLF_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
  return MLF_OK;
}

bool is_device_ptr(const void* ptr) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

}  // namespace mlf

using namespace mlf;

struct mlf_psf : public mlf::Psf {};
struct mlf_solver : public mlf::Solver {};
struct mlf_batch {
  mlf::Psf* psf = nullptr;
  std::vector<std::unique_ptr<mlf::Solver>> members;  // per-patch geometry, filter plan, scratch
  mlf::TcSolverState* work = nullptr;
  ~mlf_batch() { mlf::tc_solver_free(work); }
};

namespace {

// Device view of an "any" input array: the pointer itself, or a staged copy.
int stage_in(const float* p, size_t n, DevBuf& tmp, const float** dev, cudaStream_t st) {
  if (p == nullptr) {
    *dev = nullptr;
    return MLF_OK;
  }
  if (is_device_ptr(p)) {
    *dev = p;
    return MLF_OK;
  }
  if (tmp.bytes < n * sizeof(float)) MLF_TRY(tmp.alloc(n * sizeof(float), "input staging"));
  MLF_CUDA(cudaMemcpyAsync(tmp.p, p, n * sizeof(float), cudaMemcpyHostToDevice, st));
  *dev = tmp.as<float>();
  return MLF_OK;
}

struct OutStage {
  float* user = nullptr;
  float* dev = nullptr;
  size_t n = 0;
  bool host = false;
};

int stage_out(float* p, size_t n, DevBuf& tmp, OutStage* o) {
  o->user = p;
  o->n = n;
  o->host = !is_device_ptr(p);
  if (!o->host) {
    o->dev = p;
    return MLF_OK;
  }
  if (tmp.bytes < n * sizeof(float)) MLF_TRY(tmp.alloc(n * sizeof(float), "output staging"));
  o->dev = tmp.as<float>();
  return MLF_OK;
}

int finish_out(const OutStage& o, cudaStream_t st) {
  if (o.host) MLF_CUDA(cudaMemcpyAsync(o.user, o.dev, o.n * sizeof(float), cudaMemcpyDeviceToHost, st));
  return MLF_OK;
}

int current_device(int* dev) {
  MLF_CUDA(cudaGetDevice(dev));
  return MLF_OK;
}

}  // namespace

extern "C" {

int mlf_version(void) { return MLF_ABI_VERSION; }

int mlf_last_error(char* buf, size_t len) {
  if (buf && len) {
    std::strncpy(buf, g_msg.c_str(), len - 1);
    buf[len - 1] = '\0';
  }
  return g_code;
}

// The MEX projector on the tensor cores: the correlation of mlf_conv_vec equals the full
// forward projection of the re-indexed kernels (launch_mex_reindex), so a one-plane PSF made
// of them, every slice a patch of a batch, and the batched forward projection in
// MLF_PREC_BF16X3 (FP32-class accuracy) give the output after padding each slice to a
// multiple of 15 and cropping back.  MLF_ERR_UNSUPPORTED when the route does not apply
// (kernels wider than 241, kernel sum zero or not finite).
static int conv_vec_tc(const float* db, int64_t W, int64_t H, int64_t n, const float* dk, int64_t kw, float* dout,
                       cudaStream_t st) {
  const int nn = 15;
  int K0 = 15;
  while (K0 < kw + 14) K0 += 30;
  if (K0 > 255) return fail(MLF_ERR_UNSUPPORTED, "tensor-core MEX projector: kernels wider than 241");
  if (n > (1 << 20)) return fail(MLF_ERR_UNSUPPORTED, "tensor-core MEX projector: too many slices");
  DevBuf hp;
  MLF_TRY(hp.alloc(sizeof(float) * K0 * K0 * nn * nn, "MEX re-indexed kernels"));
  MLF_TRY(launch_mex_reindex(dk, (int)kw, K0, nn, hp.as<float>(), st));
  mlf_psf* psf = nullptr;
  MLF_TRY(mlf_psf_create(hp.as<float>(), hp.as<float>(), K0, nn, 1, &psf, st));
  std::unique_ptr<mlf_psf> pg(psf);
  const double hs = psf->hsum_z[0];
  if (!std::isfinite(hs) || hs == 0.0)
    return fail(MLF_ERR_UNSUPPORTED, "tensor-core MEX projector: kernel sum is zero or not finite");
  const int64_t Wp = (W + nn - 1) / nn * nn, Hq = (H + nn - 1) / nn * nn;
  std::vector<int64_t> xr(n, Wp), xc(n, Hq);
  std::vector<int32_t> z0(n, 0), nz(n, 1);
  mlf_batch* b = nullptr;
  MLF_TRY(mlf_batch_create(psf, (int32_t)n, xr.data(), xc.data(), z0.data(), nz.data(), &b));
  std::unique_ptr<mlf_batch> bg(b);
  DevBuf pin, pout;
  MLF_TRY(pin.alloc(sizeof(float) * Wp * Hq * n, "MEX padded slices"));
  MLF_TRY(pout.alloc(sizeof(float) * Wp * Hq * n, "MEX padded output"));
  MLF_TRY(launch_mex_pad(db, W, H, n, Wp, Hq, kw % 2 == 0, pin.as<float>(), st));
  std::vector<const float*> vp(n);
  std::vector<float*> op(n);
  for (int64_t i = 0; i < n; ++i) {
    vp[i] = pin.as<float>() + i * Wp * Hq;
    op[i] = pout.as<float>() + i * Wp * Hq;
  }
  MLF_TRY(mlf_batch_forward_project(b, vp.data(), op.data(), 1, MLF_PREC_BF16X3, st));
  MLF_TRY(launch_mex_crop(pout.as<float>(), Wp, Hq, W, H, n, dout, st));
  MLF_CUDA(cudaStreamSynchronize(st));
  return MLF_OK;
}

int mlf_conv_vec(const float* bitmap, int64_t W, int64_t H, int64_t n, const float* kernels,
                 int64_t kw, int32_t nnum, float* out, void* stream) {
  return mlf_conv_vec_ex(bitmap, W, H, n, kernels, kw, nnum, out, MLF_CONV_AUTO, stream);
}

int mlf_conv_vec_ex(const float* bitmap, int64_t W, int64_t H, int64_t n, const float* kernels,
                    int64_t kw, int32_t nnum, float* out, int32_t method, void* stream) {
  mlf::Range nvtx_range("mlf_conv_vec_ex");
  clear_error();
  if (method != MLF_CONV_AUTO && method != MLF_CONV_DIRECT && method != MLF_CONV_TENSOR)
    return fail(MLF_ERR_INVALID, "mlf_conv_vec_ex: unknown method");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // src/cuda/mex_lfm_convolution_vec.cu:313-347 -- 2-D/3-D single bitmap, n >= 1,
  // 4-D single kernels with kw <= 341; the kernel count per axis is fixed at 15 (:35).
  if (!bitmap || !kernels || !out) return fail(MLF_ERR_INVALID, "Invalid input to mex_lfm_convolution_vec(): null pointer");
  if (W < 1 || H < 1) return fail(MLF_ERR_INVALID, "Invalid input to mex_lfm_convolution_vec(): empty bitmap");
  if (n < 1) return fail(MLF_ERR_INVALID, "Invalid input to mex_lfm_convolution_vec(): bitmap_n has to be at least 1");
  if (kw < 1 || kw > 341) return fail(MLF_ERR_INVALID, "Invalid input to mex_lfm_convolution_vec(): kernel_width exceeds kernel_width_limit=341");
  if (nnum != 15) return fail(MLF_ERR_INVALID, "Invalid input to mex_lfm_convolution_vec(): the kernel grid must be 15 x 15");
  if (W * H * n > ((int64_t)1 << 40)) return fail(MLF_ERR_INVALID, "bitmap too large");
  DevBuf bin, kin, bout;
  const float *db = nullptr, *dk = nullptr;
  MLF_TRY(stage_in(bitmap, (size_t)(W * H * n), bin, &db, st));
  MLF_TRY(stage_in(kernels, (size_t)(kw * kw * nnum * nnum), kin, &dk, st));
  OutStage o;
  MLF_TRY(stage_out(out, (size_t)(W * H * n), bout, &o));
  const double flop = 2.0 * (double)W * H * n * kw * kw;
  bool done = false;
  if (method == MLF_CONV_TENSOR || (method == MLF_CONV_AUTO && flop >= 1e11)) {
    const int rc = conv_vec_tc(db, W, H, n, dk, kw, o.dev, st);
    if (rc == MLF_OK)
      done = true;
    else if (rc != MLF_ERR_UNSUPPORTED || method == MLF_CONV_TENSOR)
      return rc;
    else
      clear_error();
  }
  if (!done) MLF_TRY(conv_vec_run(db, W, H, n, dk, kw, nnum, o.dev, st));
  MLF_TRY(finish_out(o, st));
  MLF_CUDA(cudaStreamSynchronize(st));
  return MLF_OK;
}

int mlf_summary_image(const float* movie, int64_t P, int64_t T, int32_t mode, int32_t bg_iter, int32_t window_1,
                      int32_t window_2, int32_t poly_index, float* summary_out, float* bg_spatial_out,
                      float* bg_temporal_out, void* stream) {
  return mlf_summary_image_ex(movie, P, T, mode, bg_iter, window_1, window_2, poly_index, summary_out,
                              bg_spatial_out, bg_temporal_out, nullptr, stream);
}

int mlf_summary_image_ex(const float* movie, int64_t P, int64_t T, int32_t mode, int32_t bg_iter,
                         int32_t window_1, int32_t window_2, int32_t poly_index, float* summary_out,
                         float* bg_spatial_out, float* bg_temporal_out, double* pass_ms, void* stream) {
  mlf::Range nvtx_range("mlf_summary_image_ex");
  clear_error();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!movie || !summary_out) return fail(MLF_ERR_INVALID, "mlf_summary_image: null pointer");
  if (P < 1 || T < 1) return fail(MLF_ERR_INVALID, "mlf_summary_image: empty movie");
  if (T > INT32_MAX / 8) return fail(MLF_ERR_INVALID, "mlf_summary_image: too many frames");
  if (mode != MLF_DETREND_PIXELWISE && mode != MLF_DETREND_GLOBAL)
    return fail(MLF_ERR_INVALID, "mlf_summary_image: Invalid value for param \"detrend_mode\"");
  if (bg_iter < 1) return fail(MLF_ERR_INVALID, "mlf_summary_image: bg_iter must be at least 1");
  if (mode == MLF_DETREND_PIXELWISE && (window_1 < 1 || window_2 < 1 || poly_index < 0))
    return fail(MLF_ERR_INVALID, "mlf_summary_image: windows must be positive and poly_index non-negative");
  DevBuf bin, bimg, bs, bt;
  const float* dy = nullptr;
  MLF_TRY(stage_in(movie, (size_t)(P * T), bin, &dy, st));
  OutStage oi, os, ot;
  MLF_TRY(stage_out(summary_out, (size_t)P, bimg, &oi));
  DevBuf s_own, t_own;
  float* ds = nullptr;
  float* dt = nullptr;
  if (bg_spatial_out) {
    MLF_TRY(stage_out(bg_spatial_out, (size_t)P, bs, &os));
    ds = os.dev;
  } else {
    MLF_TRY(s_own.alloc(sizeof(float) * P, "summary: spatial background"));
    ds = s_own.as<float>();
  }
  if (bg_temporal_out) {
    MLF_TRY(stage_out(bg_temporal_out, (size_t)T, bt, &ot));
    dt = ot.dev;
  } else {
    MLF_TRY(t_own.alloc(sizeof(float) * T, "summary: temporal background"));
    dt = t_own.as<float>();
  }
  MLF_TRY(summary_run(dy, P, T, mode, bg_iter, window_1, window_2, poly_index, oi.dev, ds, dt, pass_ms, st));
  MLF_TRY(finish_out(oi, st));
  if (bg_spatial_out) MLF_TRY(finish_out(os, st));
  if (bg_temporal_out) MLF_TRY(finish_out(ot, st));
  MLF_CUDA(cudaStreamSynchronize(st));
  return MLF_OK;
}

int mlf_rectify_frames(const void* frames, int32_t dtype, int64_t H, int64_t W, int64_t n_frames,
                       const int64_t* raw_cut, double raw_cut_xCenter, double raw_cut_yCenter, int32_t Nnum,
                       double frames_dx, int64_t size_h, int64_t size_w, int64_t frames_start, int64_t frames_step,
                       int64_t frames_end, int32_t frames_average, int32_t normalize, float* movie_out,
                       int64_t* n_out, void* stream) {
  mlf::Range nvtx_range("mlf_rectify_frames");
  clear_error();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!frames || !raw_cut || !movie_out) return fail(MLF_ERR_INVALID, "mlf_rectify_frames: null pointer");
  if (dtype != MLF_DTYPE_F32 && dtype != MLF_DTYPE_U16) return fail(MLF_ERR_INVALID, "mlf_rectify_frames: dtype");
  if (H < 1 || W < 1 || n_frames < 1) return fail(MLF_ERR_INVALID, "mlf_rectify_frames: empty frames");
  const int64_t y0 = raw_cut[0], y1 = raw_cut[1], x0 = raw_cut[2], x1 = raw_cut[3];
  if (y0 < 1 || y1 > H || x0 < 1 || x1 > W || y1 - y0 < 1 || x1 - x0 < 1)
    return fail(MLF_ERR_INVALID, "mlf_rectify_frames: raw_cut outside the frame or narrower than 2 pixels");
  if (Nnum < 1 || !(frames_dx > 0) || !std::isfinite(raw_cut_xCenter) || !std::isfinite(raw_cut_yCenter))
    return fail(MLF_ERR_INVALID, "mlf_rectify_frames: Nnum, frames_dx or the lenslet centre");
  if (size_h < 1 || size_w < 1 || frames_start < 1 || frames_step < 1)
    return fail(MLF_ERR_INVALID, "mlf_rectify_frames: size or frame range");
  const int64_t last = frames_end < 0 ? n_frames : std::min(n_frames, frames_end);  // 1-based
  if (last < frames_start) return fail(MLF_ERR_INVALID, "mlf_rectify_frames: no frame selected");
  const int64_t n_final = (last - frames_start) / frames_step + 1;
  const int navg = frames_average ? (int)std::min<int64_t>(frames_step, INT32_MAX) : 1;
  const int64_t h = y1 - y0 + 1, w = x1 - x0 + 1;
  const size_t es = dtype == MLF_DTYPE_U16 ? 2 : 4;
  const int64_t P = size_h * size_w;
  OutStage o;
  DevBuf bout, bin;
  MLF_TRY(stage_out(movie_out, (size_t)(P * n_final), bout, &o));
  if (is_device_ptr(frames)) {
    // read the frames in place: 0-based first frame, step, last frame
    MLF_TRY(rectify_run(frames, dtype, H * W * n_frames, H * W, H, y0 - 1, x0 - 1, h, w, raw_cut_xCenter, raw_cut_yCenter, Nnum,
                        frames_dx, size_h, size_w, frames_start - 1, frames_step, navg, last - 1, n_final, o.dev,
                        normalize != 0, st));
  } else {
    // copy the cut region of the frames used (every frame of the range when averaging)
    const int64_t n_used = frames_average ? last - frames_start + 1 : n_final;
    MLF_TRY(bin.alloc(es * h * w * n_used, "rectification input staging"));
    const char* src = static_cast<const char*>(frames);
    for (int64_t k = 0; k < n_used; ++k) {
      const int64_t f = frames_average ? frames_start - 1 + k : frames_start - 1 + k * frames_step;
      const char* s0 = src + es * ((size_t)f * H * W + (size_t)(x0 - 1) * H + (size_t)(y0 - 1));
      MLF_CUDA(cudaMemcpy2DAsync(static_cast<char*>(bin.p) + es * h * w * k, es * h, s0, es * H, es * h, w,
                                 cudaMemcpyHostToDevice, st));
    }
    MLF_TRY(rectify_run(bin.p, dtype, h * w * n_used, h * w, h, 0, 0, h, w, raw_cut_xCenter, raw_cut_yCenter, Nnum, frames_dx,
                        size_h, size_w, 0, frames_average ? frames_step : 1, navg, n_used - 1, n_final, o.dev,
                        normalize != 0, st));
  }
  MLF_TRY(finish_out(o, st));
  MLF_CUDA(cudaStreamSynchronize(st));
  if (n_out) *n_out = n_final;
  return MLF_OK;
}

int mlf_conv_vec_accumulate(const float* bitmaps, int64_t W, int64_t H, int64_t n, const int32_t* plane,
                            const int32_t* slot, int64_t n_out, const float* kernels, int64_t kw, int32_t nnum,
                            int64_t Z, float* out, void* stream) {
  mlf::Range nvtx_range("mlf_conv_vec_accumulate");
  clear_error();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!bitmaps || !plane || !slot || !kernels || !out) return fail(MLF_ERR_INVALID, "mlf_conv_vec_accumulate: null pointer");
  if (W < 1 || H < 1 || n < 1 || n_out < 1 || Z < 1) return fail(MLF_ERR_INVALID, "mlf_conv_vec_accumulate: empty input");
  if (kw < 1 || kw > 341) return fail(MLF_ERR_INVALID, "mlf_conv_vec_accumulate: kernel_width exceeds kernel_width_limit=341");
  if (nnum != 15) return fail(MLF_ERR_INVALID, "mlf_conv_vec_accumulate: the kernel grid must be 15 x 15");
  std::vector<int> zmin(n_out, (int)Z), zmax(n_out, -1);
  for (int64_t j = 0; j < n; ++j) {
    if (plane[j] < 0 || plane[j] >= Z || slot[j] < 0 || slot[j] >= n_out)
      return fail(MLF_ERR_INVALID, "mlf_conv_vec_accumulate: slice " + std::to_string(j) + ": plane or slot out of range");
    zmin[slot[j]] = std::min(zmin[slot[j]], plane[j]);
    zmax[slot[j]] = std::max(zmax[slot[j]], plane[j]);
  }
  const int64_t img = W * H, kz = kw * kw * nnum * nnum;
  DevBuf bin, kin, bout;
  const float *db = nullptr, *dk = nullptr;
  MLF_TRY(stage_in(bitmaps, (size_t)(img * n), bin, &db, st));
  MLF_TRY(stage_in(kernels, (size_t)(kz * Z), kin, &dk, st));
  OutStage o;
  MLF_TRY(stage_out(out, (size_t)(img * n_out), bout, &o));
  MLF_CUDA(cudaMemsetAsync(o.dev, 0, sizeof(float) * img * n_out, st));
  const bool even = kw % 2 == 0;
  // tensor-core route: one PSF of the re-indexed kernels of every plane, one patch per output
  // slot spanning its planes, one batched forward projection
  int K0 = 15;
  while (K0 < kw + 14) K0 += 30;
  bool done = false;
  if (K0 <= 255) {
    const int nn = 15;
    DevBuf hp;
    MLF_TRY(hp.alloc(sizeof(float) * K0 * K0 * nn * nn * Z, "MEX re-indexed kernels"));
    for (int64_t z = 0; z < Z; ++z)
      MLF_TRY(launch_mex_reindex(dk + z * kz, (int)kw, K0, nn, hp.as<float>() + z * K0 * K0 * nn * nn, st));
    mlf_psf* psf = nullptr;
    MLF_TRY(mlf_psf_create(hp.as<float>(), hp.as<float>(), K0, nn, Z, &psf, st));
    std::unique_ptr<mlf_psf> pg(psf);
    bool sums_ok = true;
    for (int64_t z = 0; z < Z; ++z) sums_ok = sums_ok && std::isfinite(psf->hsum_z[z]) && psf->hsum_z[z] != 0.0;
    if (sums_ok) {
      const int64_t Wp = (W + nn - 1) / nn * nn, Hq = (H + nn - 1) / nn * nn;
      std::vector<int64_t> xr, xc;
      std::vector<int32_t> z0, nz, patch_of(n_out, -1);
      std::vector<int64_t> voff;
      int64_t vtot = 0;
      for (int64_t s = 0; s < n_out; ++s) {
        if (zmax[s] < 0) continue;  // nothing projected into this slot: stays zero
        patch_of[s] = (int32_t)xr.size();
        xr.push_back(Wp);
        xc.push_back(Hq);
        z0.push_back(zmin[s]);
        nz.push_back(zmax[s] - zmin[s] + 1);
        voff.push_back(vtot);
        vtot += Wp * Hq * nz.back();
      }
      mlf_batch* b = nullptr;
      MLF_TRY(mlf_batch_create(psf, (int32_t)xr.size(), xr.data(), xc.data(), z0.data(), nz.data(), &b));
      std::unique_ptr<mlf_batch> bg(b);
      DevBuf vols, lfo;
      MLF_TRY(vols.alloc(sizeof(float) * vtot, "accumulated slice volumes"));
      MLF_TRY(lfo.alloc(sizeof(float) * Wp * Hq * xr.size(), "accumulated projections"));
      MLF_CUDA(cudaMemsetAsync(vols.p, 0, sizeof(float) * vtot, st));
      for (int64_t j = 0; j < n; ++j) {
        const int p = patch_of[slot[j]];
        float* dst = vols.as<float>() + voff[p] + Wp * Hq * (plane[j] - zmin[slot[j]]);
        MLF_TRY(launch_mex_pad_add(db + j * img, W, H, Wp, Hq, even, dst, st));
      }
      std::vector<const float*> vp(xr.size());
      std::vector<float*> op(xr.size());
      for (size_t p = 0; p < xr.size(); ++p) {
        vp[p] = vols.as<float>() + voff[p];
        op[p] = lfo.as<float>() + (int64_t)p * Wp * Hq;
      }
      MLF_TRY(mlf_batch_forward_project(b, vp.data(), op.data(), 1, MLF_PREC_BF16X3, st));
      for (int64_t s = 0; s < n_out; ++s)
        if (patch_of[s] >= 0)
          MLF_TRY(launch_mex_crop(lfo.as<float>() + (int64_t)patch_of[s] * Wp * Hq, Wp, Hq, W, H, 1,
                                  o.dev + s * img, st));
      MLF_CUDA(cudaStreamSynchronize(st));
      done = true;
    }
  }
  if (!done) {
    // direct route: every slice projected on its own and added to its slot
    DevBuf tmp;
    MLF_TRY(tmp.alloc(sizeof(float) * img, "projection scratch"));
    for (int64_t j = 0; j < n; ++j) {
      MLF_TRY(conv_vec_run(db + j * img, W, H, 1, dk + plane[j] * kz, kw, nnum, tmp.as<float>(), st));
      MLF_TRY(launch_mex_pad_add(tmp.as<float>(), W, H, W, H, false, o.dev + slot[j] * img, st));
    }
  }
  MLF_TRY(finish_out(o, st));
  MLF_CUDA(cudaStreamSynchronize(st));
  return MLF_OK;
}

int mlf_psf_create(const float* H, const float* Ht, int64_t K0, int32_t N, int64_t Z, mlf_psf** out,
                   void* stream) {
  mlf::Range nvtx_range("mlf_psf_create");
  clear_error();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!H || !Ht || !out) return fail(MLF_ERR_INVALID, "mlf_psf_create: null pointer");
  *out = nullptr;
  if (N < 3 || N % 2 == 0) return fail(MLF_ERR_INVALID, "mlf_psf_create: Nnum must be odd and >= 3");
  if (K0 < N || K0 % 2 == 0) return fail(MLF_ERR_INVALID, "mlf_psf_create: PSF side K0 must be odd and >= Nnum");
  if (Z < 1) return fail(MLF_ERR_INVALID, "mlf_psf_create: need at least one depth plane");
  const int64_t S = K0 - ((K0 - N) % (2 * N));
  const int64_t T = S / N;
  if (!view_taps_supported((int)T))
    return fail(MLF_ERR_UNSUPPORTED, "mlf_psf_create: phase-space PSF side S = " + std::to_string(S) +
                                         " gives S/N = " + std::to_string(T) + " (supported: 3..17, odd)");
  std::unique_ptr<mlf_psf> p(new mlf_psf());
  MLF_TRY(current_device(&p->device));
  p->N = N;
  p->Z = (int)Z;
  p->K0 = (int)K0;
  const size_t nel = (size_t)K0 * K0 * N * N * Z;
  DevBuf sh, sht;
  const float *dH = nullptr, *dHt = nullptr;
  MLF_TRY(stage_in(H, nel, sh, &dH, st));
  MLF_TRY(stage_in(Ht, nel, sht, &dHt, st));
  MLF_TRY(psf_build(p.get(), dH, dHt, st));
  MLF_CUDA(cudaStreamSynchronize(st));
  *out = p.release();
  return MLF_OK;
}

int mlf_psf_destroy(mlf_psf* psf) {
  clear_error();
  delete psf;
  return MLF_OK;
}

int mlf_psf_info(const mlf_psf* psf, int32_t* N, int64_t* Z, int64_t* S) {
  clear_error();
  if (!psf) return fail(MLF_ERR_INVALID, "mlf_psf_info: null psf");
  if (N) *N = psf->N;
  if (Z) *Z = psf->Z;
  if (S) *S = psf->S;
  return MLF_OK;
}

int mlf_psf_weights(const mlf_psf* psf, double* w) {
  clear_error();
  if (!psf || !w) return fail(MLF_ERR_INVALID, "mlf_psf_weights: null pointer");
  std::memcpy(w, psf->weights.data(), sizeof(double) * psf->weights.size());
  return MLF_OK;
}

int64_t mlf_psf_device_bytes(const mlf_psf* psf) { return psf ? (int64_t)psf->bytes() : 0; }

int mlf_solver_create(mlf_psf* psf, int64_t Xr, int64_t Xc, mlf_solver** out) {
  clear_error();
  if (!psf || !out) return fail(MLF_ERR_INVALID, "mlf_solver_create: null pointer");
  *out = nullptr;
  if (Xr < psf->N || Xc < psf->N || Xr % psf->N || Xc % psf->N)
    return fail(MLF_ERR_INVALID, "mlf_solver_create: image sides must be positive multiples of Nnum");
  std::unique_ptr<mlf_solver> s(new mlf_solver());
  s->psf = psf;
  s->Xr = Xr;
  s->Xc = Xc;
  MLF_TRY(current_device(&s->device));
  if (s->device != psf->device) return fail(MLF_ERR_INVALID, "mlf_solver_create: PSF lives on another device");
  MLF_TRY(solver_init(s.get()));
  *out = s.release();
  return MLF_OK;
}

int mlf_solver_create_variant(mlf_psf* psf, int64_t Xr, int64_t Xc, int32_t variant, mlf_solver** out) {
  clear_error();
  if (variant != MLF_VARIANT_BASE && variant != MLF_VARIANT_PEELING)
    return fail(MLF_ERR_INVALID, "mlf_solver_create_variant: unknown variant");
  if (!psf || !out) return fail(MLF_ERR_INVALID, "mlf_solver_create_variant: null pointer");
  *out = nullptr;
  if (Xr < psf->N || Xc < psf->N || Xr % psf->N || Xc % psf->N)
    return fail(MLF_ERR_INVALID, "mlf_solver_create_variant: image sides must be positive multiples of Nnum");
  std::unique_ptr<mlf_solver> s(new mlf_solver());
  s->psf = psf;
  s->Xr = Xr;
  s->Xc = Xc;
  s->variant = variant;
  MLF_TRY(current_device(&s->device));
  if (s->device != psf->device) return fail(MLF_ERR_INVALID, "mlf_solver_create_variant: PSF lives on another device");
  MLF_TRY(solver_init(s.get()));
  *out = s.release();
  return MLF_OK;
}

int mlf_solver_run_peeling(mlf_solver* s, const float* lfimg, int32_t max_iter, int32_t precision, float* vol_out,
                           float* lf_peeled_out, float* proj_sensor_out, mlf_stats* stats, void* stream) {
  mlf::Range nvtx_range("mlf_solver_run_peeling");
  clear_error();
  if (!s || !lfimg || !vol_out) return fail(MLF_ERR_INVALID, "mlf_solver_run_peeling: null pointer");
  if (max_iter < 0) return fail(MLF_ERR_INVALID, "mlf_solver_run_peeling: maxIter must be >= 0");
  if (!prec_valid(precision))
    return fail(MLF_ERR_INVALID, "mlf_solver_run_peeling: unknown precision");
  for (const void* p : {(const void*)lfimg, (const void*)vol_out, (const void*)lf_peeled_out, (const void*)proj_sensor_out})
    if (p && !is_device_ptr(p)) return fail(MLF_ERR_INVALID, "mlf_solver_run_peeling: device pointers required");
  return peel_solve(s, lfimg, max_iter, precision, vol_out, lf_peeled_out, proj_sensor_out, stats,
                    static_cast<cudaStream_t>(stream));
}

int mlf_solver_destroy(mlf_solver* s) {
  clear_error();
  delete s;
  return MLF_OK;
}

int64_t mlf_solver_device_bytes(const mlf_solver* s) { return s ? (int64_t)s->bytes() : 0; }

int mlf_solver_run(mlf_solver* s, const float* lfimg, int32_t max_iter, int32_t precision,
                   const float* warm_start, float* vol_out, mlf_stats* stats, void* stream) {
  mlf::Range nvtx_range("mlf_solver_run");
  clear_error();
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!s || !lfimg || !vol_out) return fail(MLF_ERR_INVALID, "mlf_solver_run: null pointer");
  if (max_iter < 0) return fail(MLF_ERR_INVALID, "mlf_solver_run: maxIter must be >= 0");
  if (!prec_valid(precision))
    return fail(MLF_ERR_INVALID, "mlf_solver_run: unknown precision");
  const size_t n_img = (size_t)(s->Xr * s->Xc), n_vol = n_img * s->Z;
  const float *dlf = nullptr, *dwarm = nullptr;
  MLF_TRY(stage_in(lfimg, n_img, s->stage_in, &dlf, st));
  DevBuf warm_tmp;
  MLF_TRY(stage_in(warm_start, n_vol, warm_tmp, &dwarm, st));
  OutStage o;
  MLF_TRY(stage_out(vol_out, n_vol, s->stage_out, &o));
  MLF_TRY(solver_run(s, dlf, max_iter, precision, dwarm, o.dev, stats, st));
  MLF_TRY(finish_out(o, st));
  if (o.host || warm_tmp.p || dlf != lfimg) MLF_CUDA(cudaStreamSynchronize(st));
  return MLF_OK;
}

int mlf_batch_create(mlf_psf* psf, int32_t npatch, const int64_t* Xr, const int64_t* Xc, const int32_t* z0,
                     const int32_t* nz, mlf_batch** out) {
  clear_error();
  if (!psf || !Xr || !Xc || !z0 || !nz || !out) return fail(MLF_ERR_INVALID, "mlf_batch_create: null pointer");
  *out = nullptr;
  if (npatch < 1) return fail(MLF_ERR_INVALID, "mlf_batch_create: need at least one patch");
  std::unique_ptr<mlf_batch> b(new mlf_batch());
  b->psf = psf;
  int dev = 0;
  MLF_CUDA(cudaGetDevice(&dev));
  if (dev != psf->device) return fail(MLF_ERR_INVALID, "mlf_batch_create: PSF lives on another device");
  for (int k = 0; k < npatch; ++k) {
    if (Xr[k] < psf->N || Xc[k] < psf->N || Xr[k] % psf->N || Xc[k] % psf->N)
      return fail(MLF_ERR_INVALID, "mlf_batch_create: patch " + std::to_string(k) +
                                       ": image sides must be positive multiples of Nnum");
    if (z0[k] < 0 || nz[k] < 1 || z0[k] + nz[k] > psf->Z)
      return fail(MLF_ERR_INVALID, "mlf_batch_create: patch " + std::to_string(k) + ": plane range outside the PSF");
    std::unique_ptr<mlf::Solver> m(new mlf::Solver());
    m->psf = psf;
    m->device = dev;
    m->lite = true;
    m->Xr = Xr[k];
    m->Xc = Xc[k];
    m->Z = nz[k];
    m->z0 = z0[k];
    MLF_TRY(solver_init(m.get()));
    b->members.push_back(std::move(m));
  }
  std::vector<mlf::Solver*> ms;
  for (auto& m : b->members) ms.push_back(m.get());
  MLF_TRY(tc_work_create(psf, ms, &b->work, nullptr));
  MLF_CUDA(cudaStreamSynchronize(nullptr));
  *out = b.release();
  return MLF_OK;
}

int mlf_batch_plan_bytes(const mlf_psf* psf, int32_t npatch, const int64_t* Xr, const int64_t* Xc,
                         const int32_t* z0, const int32_t* nz, int64_t* bytes) {
  clear_error();
  if (!psf || npatch < 1 || !Xr || !Xc || !z0 || !nz || !bytes) return fail(MLF_ERR_INVALID, "mlf_batch_plan_bytes: bad argument");
  int nsm = 0;
  MLF_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, psf->device));
  std::vector<int> li, lj;
  size_t members = 0;
  for (int k = 0; k < npatch; ++k) {
    if (Xr[k] < psf->N || Xc[k] < psf->N || Xr[k] % psf->N || Xc[k] % psf->N || z0[k] < 0 || nz[k] < 1 ||
        z0[k] + nz[k] > psf->Z)
      return fail(MLF_ERR_INVALID, "mlf_batch_plan_bytes: patch " + std::to_string(k) + ": bad geometry");
    li.push_back((int)(Xr[k] / psf->N));
    lj.push_back((int)(Xc[k] / psf->N));
    // filter scratch volume, reduction scratch, filter kernels and sums (upper bounds)
    const int64_t gmax = (std::max(Xr[k], Xc[k]) + 31) / 32;
    members += (size_t)(Xr[k] * Xc[k] * nz[k] * 4 + 4096 * 8 + (int64_t)nz[k] * (Xr[k] + Xc[k]) * 4 +
                        6 * (int64_t)nz[k] * 4 + (2 * (int64_t)nz[k] * gmax + nz[k]) * 8);
  }
  *bytes = (int64_t)(members + tc_work_plan_bytes(psf, li, lj, nsm));
  return MLF_OK;
}

int mlf_batch_destroy(mlf_batch* b) {
  clear_error();
  delete b;
  return MLF_OK;
}

int64_t mlf_batch_device_bytes(const mlf_batch* b) {
  if (!b) return 0;
  size_t n = tc_work_bytes(b->work);
  for (auto& m : b->members) n += m->bytes();
  return (int64_t)n;
}

int mlf_batch_run(mlf_batch* b, const float* const* lfimg, int32_t max_iter, int32_t precision,
                  const float* const* warm, float* const* vol_out, mlf_stats* stats, void* stream) {
  mlf::Range nvtx_range("mlf_batch_run");
  clear_error();
  if (!b || !lfimg || !vol_out) return fail(MLF_ERR_INVALID, "mlf_batch_run: null pointer");
  if (max_iter < 0) return fail(MLF_ERR_INVALID, "mlf_batch_run: maxIter must be >= 0");
  if (!prec_tensor(precision))
    return fail(MLF_ERR_UNSUPPORTED, "mlf_batch_run: batches run on the tensor cores (MLF_PREC_BF16* / "
                                     "MLF_PREC_FP16*); use mlf_solver_run per patch for MLF_PREC_FP32");
  const size_t P = b->members.size();
  std::vector<const float*> lf(P), wm(P);
  std::vector<float*> out(P);
  std::vector<mlf::Solver*> ms;
  size_t active = 0;
  for (size_t k = 0; k < P; ++k) {
    lf[k] = lfimg[k];
    ms.push_back(b->members[k].get());
    if (!lf[k]) continue;  // patch k sits this run out
    ++active;
    wm[k] = warm ? warm[k] : nullptr;
    out[k] = vol_out[k];
    if (!out[k]) return fail(MLF_ERR_INVALID, "mlf_batch_run: null output pointer for a patch with an image");
    if (!is_device_ptr(lf[k]) || !is_device_ptr(out[k]) || (wm[k] && !is_device_ptr(wm[k])))
      return fail(MLF_ERR_INVALID, "mlf_batch_run: device pointers required");
  }
  if (active == 0) return fail(MLF_ERR_INVALID, "mlf_batch_run: no patch has an image");
  return tc_run(b->work, ms, lf, wm, out, max_iter, precision, stats, ms[0], static_cast<cudaStream_t>(stream));
}

int mlf_batch_cancel(mlf_batch* b) {
  if (!b) return fail(MLF_ERR_INVALID, "mlf_batch_cancel: null batch");
  tc_cancel_state(b->work).request();
  return MLF_OK;
}

int mlf_batch_cancelled(const mlf_batch* b) {
  return (b && tc_cancel_state(b->work).stopped()) ? 1 : 0;
}

int mlf_solver_cancel(mlf_solver* s) {
  if (!s) return fail(MLF_ERR_INVALID, "mlf_solver_cancel: null solver");
  s->cancel.request();
  if (s->tc) tc_cancel_state(s->tc).request();
  return MLF_OK;
}

int mlf_solver_cancelled(const mlf_solver* s) {
  if (!s) return 0;
  if (s->last_run_tc) return (s->tc && tc_cancel_state(s->tc).stopped()) ? 1 : 0;
  return s->cancel.stopped() ? 1 : 0;
}

int mlf_rl_solve(const float* lfimg, int64_t Xr, int64_t Xc, const float* H, const float* Ht,
                 int64_t K0, int32_t N, int64_t Z, int32_t max_iter, int32_t precision, float* vol_out,
                 mlf_stats* stats, void* stream) {
  mlf::Range nvtx_range("mlf_rl_solve");
  mlf_psf* psf = nullptr;
  MLF_TRY(mlf_psf_create(H, Ht, K0, N, Z, &psf, stream));
  std::unique_ptr<mlf_psf> guard(psf);
  mlf_solver* s = nullptr;
  MLF_TRY(mlf_solver_create(psf, Xr, Xc, &s));
  std::unique_ptr<mlf_solver> sguard(s);
  MLF_TRY(mlf_solver_run(s, lfimg, max_iter, precision, nullptr, vol_out, stats, stream));
  MLF_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
  return MLF_OK;
}

int mlf_forward_view(mlf_solver* s, const float* vol, int32_t u, int32_t v, float* hx, void* stream) {
  clear_error();
  if (!s || !vol || !hx) return fail(MLF_ERR_INVALID, "mlf_forward_view: null pointer");
  if (u < 0 || v < 0 || u >= s->N || v >= s->N) return fail(MLF_ERR_INVALID, "mlf_forward_view: view out of range");
  if (!is_device_ptr(vol) || !is_device_ptr(hx)) return fail(MLF_ERR_INVALID, "mlf_forward_view: device pointers required");
  return forward_view(s, vol, u, v, hx, static_cast<cudaStream_t>(stream));
}

int mlf_backward_view(mlf_solver* s, const float* proj, int32_t u, int32_t v, float* out, void* stream) {
  clear_error();
  if (!s || !proj || !out) return fail(MLF_ERR_INVALID, "mlf_backward_view: null pointer");
  if (u < 0 || v < 0 || u >= s->N || v >= s->N) return fail(MLF_ERR_INVALID, "mlf_backward_view: view out of range");
  if (!is_device_ptr(proj) || !is_device_ptr(out)) return fail(MLF_ERR_INVALID, "mlf_backward_view: device pointers required");
  return backward_view(s, proj, u, v, out, static_cast<cudaStream_t>(stream));
}

int mlf_rl_view_step(mlf_solver* s, const float* lfimg, float* vol, int32_t u, int32_t v, double w,
                     void* stream) {
  return mlf_rl_view_step_prec(s, lfimg, vol, u, v, w, MLF_PREC_FP32, stream);
}

int mlf_rl_view_step_prec(mlf_solver* s, const float* lfimg, float* vol, int32_t u, int32_t v, double w,
                          int32_t precision, void* stream) {
  clear_error();
  if (!s || !lfimg || !vol) return fail(MLF_ERR_INVALID, "mlf_rl_view_step: null pointer");
  if (u < 0 || v < 0 || u >= s->N || v >= s->N) return fail(MLF_ERR_INVALID, "mlf_rl_view_step: view out of range");
  if (!prec_valid(precision)) return fail(MLF_ERR_INVALID, "mlf_rl_view_step: unknown precision");
  if (!is_device_ptr(lfimg) || !is_device_ptr(vol)) return fail(MLF_ERR_INVALID, "mlf_rl_view_step: device pointers required");
  return rl_view_step(s, lfimg, vol, u, v, w, precision, static_cast<cudaStream_t>(stream));
}

int mlf_forward_view_prec(mlf_solver* s, const float* vol, int32_t u, int32_t v, int32_t precision, float* hx,
                          void* stream) {
  clear_error();
  if (!s || !vol || !hx) return fail(MLF_ERR_INVALID, "mlf_forward_view_prec: null pointer");
  if (u < 0 || v < 0 || u >= s->N || v >= s->N) return fail(MLF_ERR_INVALID, "mlf_forward_view_prec: view out of range");
  if (!prec_valid(precision)) return fail(MLF_ERR_INVALID, "mlf_forward_view_prec: unknown precision");
  if (!is_device_ptr(vol) || !is_device_ptr(hx)) return fail(MLF_ERR_INVALID, "mlf_forward_view_prec: device pointers required");
  return forward_view_prec(s, vol, u, v, precision, hx, static_cast<cudaStream_t>(stream));
}

int mlf_forward_project(mlf_solver* s, const float* vol, float* lf_out, int32_t raw_psf, int32_t precision,
                        void* stream) {
  mlf::Range nvtx_range("mlf_forward_project");
  clear_error();
  if (!s || !vol || !lf_out) return fail(MLF_ERR_INVALID, "mlf_forward_project: null pointer");
  if (!prec_valid(precision)) return fail(MLF_ERR_INVALID, "mlf_forward_project: unknown precision");
  if (!is_device_ptr(vol) || !is_device_ptr(lf_out)) return fail(MLF_ERR_INVALID, "mlf_forward_project: device pointers required");
  return forward_project(s, vol, lf_out, raw_psf ? s->psf->hsum_dev.as<float>() : nullptr, precision,
                         static_cast<cudaStream_t>(stream));
}

int mlf_batch_forward_project(mlf_batch* b, const float* const* vols, float* const* lf_out, int32_t raw_psf,
                              int32_t precision, void* stream) {
  mlf::Range nvtx_range("mlf_batch_forward_project");
  clear_error();
  if (!b || !vols || !lf_out) return fail(MLF_ERR_INVALID, "mlf_batch_forward_project: null pointer");
  if (!prec_tensor(precision))
    return fail(MLF_ERR_UNSUPPORTED, "mlf_batch_forward_project: batches run on the tensor cores "
                                     "(MLF_PREC_BF16* / MLF_PREC_FP16*)");
  const size_t P = b->members.size();
  std::vector<const float*> v(P);
  std::vector<float*> o(P);
  std::vector<mlf::Solver*> ms;
  for (size_t k = 0; k < P; ++k) {
    v[k] = vols[k];
    o[k] = lf_out[k];
    if (!v[k] || !o[k] || !is_device_ptr(v[k]) || !is_device_ptr(o[k]))
      return fail(MLF_ERR_INVALID, "mlf_batch_forward_project: device pointers required");
    ms.push_back(b->members[k].get());
  }
  return tc_forward_project(b->work, ms, v, o, precision, raw_psf ? b->psf->hsum_dev.as<float>() : nullptr,
                            static_cast<cudaStream_t>(stream));
}

int mlf_sample_filter(mlf_solver* s, float* vol, void* stream) {
  clear_error();
  if (!s || !vol) return fail(MLF_ERR_INVALID, "mlf_sample_filter: null pointer");
  if (!is_device_ptr(vol)) return fail(MLF_ERR_INVALID, "mlf_sample_filter: device pointer required");
  return sample_filter(s, vol, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
