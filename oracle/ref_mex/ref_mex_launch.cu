// Launcher for the reference's own MEX kernel, lfm_convolution_kernel_vec
// (src/cuda/mex_lfm_convolution_vec.cu:43-266), compiled unchanged into a cubin by
// oracle/refbuild.py (texture references replaced by plain loads through
// oracle/ref_mex/mlf_ref_compat.h).  Test infrastructure: the parity tests run the
// reference kernel and the library's mlf_conv_vec on the same device inputs.
//
// mlf_ref_mex_run reproduces the host side of mexFunction (:356-406) without MATLAB: the
// output is zero-initialised (MX_GPU_INITIALIZE_VALUES, :365-369), the two "texture
// bindings" cover bitmap_width*bitmap_height*bitmap_n and kw*kw*15*15 floats (:375,381),
// the grid is (bitmap_width/1024 + 1, bitmap_height) x 1024 threads (:391-392), one launch
// per slice with kernel_width = max_kernel_width = kw (:341-342,402-405), then a device
// synchronisation (:406).  The reference spreads the slices over 16 streams; the slices
// write disjoint outputs, so one stream gives the same result.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

namespace {

struct TexRef {  // mlf_ref_texref<float, 1, cudaReadModeElementType>
  const float* ptr;
  long long n;
};

std::mutex g_mu;
cudaLibrary_t g_lib = nullptr;
cudaKernel_t g_kernel = nullptr;
TexRef* g_tex_bitmap = nullptr;   // device address of the reference's texture_bitmap
TexRef* g_tex_kernels = nullptr;  // device address of texture_kernels
char g_err[512];

int fail(const char* what, cudaError_t e) {
  snprintf(g_err, sizeof g_err, "%s: %s", what, cudaGetErrorString(e));
  return 1;
}

}  // namespace

extern "C" const char* mlf_ref_mex_error(void) { return g_err; }

// Load the cubin on the current device.  Returns 0 on success.
extern "C" int mlf_ref_mex_load(const char* cubin_path) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_lib) return 0;
  cudaError_t e = cudaLibraryLoadFromFile(&g_lib, cubin_path, nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (e != cudaSuccess) return fail("cudaLibraryLoadFromFile", e);
  e = cudaLibraryGetKernel(&g_kernel, g_lib, "_Z26lfm_convolution_kernel_veciiiiiPKfPf");
  if (e != cudaSuccess) return fail("cudaLibraryGetKernel(lfm_convolution_kernel_vec)", e);
  size_t bytes = 0;
  e = cudaLibraryGetGlobal((void**)&g_tex_bitmap, &bytes, g_lib, "texture_bitmap");
  if (e != cudaSuccess) return fail("cudaLibraryGetGlobal(texture_bitmap)", e);
  if (bytes != sizeof(TexRef)) {
    snprintf(g_err, sizeof g_err, "texture_bitmap has %zu bytes, expected %zu", bytes, sizeof(TexRef));
    return 1;
  }
  e = cudaLibraryGetGlobal((void**)&g_tex_kernels, &bytes, g_lib, "texture_kernels");
  if (e != cudaSuccess) return fail("cudaLibraryGetGlobal(texture_kernels)", e);
  if (bytes != sizeof(TexRef)) {
    snprintf(g_err, sizeof g_err, "texture_kernels has %zu bytes, expected %zu", bytes, sizeof(TexRef));
    return 1;
  }
  return 0;
}

// out (W x H x n, device) = the reference kernel applied to bitmap (W x H x n, device) with
// kernels (kw x kw x 15 x 15, device).  Synchronous.  Returns 0 on success.  Optional
// ms_out receives the device time of the n launches (CUDA events).
extern "C" int mlf_ref_mex_run(const float* bitmap, int W, int H, int n, const float* kernels, int kw,
                               float* out, double* ms_out) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_lib) {
    snprintf(g_err, sizeof g_err, "mlf_ref_mex_load was not called");
    return 1;
  }
  if (W < 1 || H < 1 || n < 1 || kw < 1 || kw > 341) {
    snprintf(g_err, sizeof g_err, "invalid shape W=%d H=%d n=%d kw=%d", W, H, n, kw);
    return 1;
  }
  cudaError_t e = cudaMemset(out, 0, sizeof(float) * (size_t)W * H * n);
  if (e != cudaSuccess) return fail("cudaMemset", e);
  const TexRef tb{bitmap, (long long)W * H * n};
  const TexRef tk{kernels, (long long)kw * kw * 15 * 15};
  e = cudaMemcpy(g_tex_bitmap, &tb, sizeof tb, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail("cudaMemcpy(texture_bitmap)", e);
  e = cudaMemcpy(g_tex_kernels, &tk, sizeof tk, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail("cudaMemcpy(texture_kernels)", e);
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return fail("cudaDeviceSynchronize", e);
  const dim3 grid(W / 1024 + 1, H), block(1024, 1);
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0, 0);
  for (int i = 0; i < n; ++i) {
    int bw = W, bh = H, ix = i, kwid = kw, kmax = kw;
    const float* kp = kernels;
    float* op = out;
    void* args[] = {&bw, &bh, &ix, &kwid, &kmax, &kp, &op};
    e = cudaLaunchKernel((const void*)g_kernel, grid, block, args, 0, 0);
    if (e != cudaSuccess) {
      cudaEventDestroy(t0);
      cudaEventDestroy(t1);
      return fail("cudaLaunchKernel(lfm_convolution_kernel_vec)", e);
    }
  }
  cudaEventRecord(t1, 0);
  e = cudaDeviceSynchronize();
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (e != cudaSuccess) return fail("lfm_convolution_kernel_vec", e);
  if (ms_out) *ms_out = ms;
  return 0;
}
