// Device characterisation helper: achieved FP32 FMA rate of the current device.
//
// A register-only kernel (8 independent FMA chains per thread, no memory traffic in the
// loop) sized to fill every SM; the rate it reaches under the current clocks is the
// denominator used for the plain FP32 projector's roofline fraction.
#include "mlf_internal.h"
#include "mlf_tc.cuh"

namespace mlf {
namespace {

__global__ void __launch_bounds__(256) k_fma_probe(float* sink, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-7f, x1 = x0 + 1e-7f, x2 = x0 + 2e-7f, x3 = x0 + 3e-7f;
  float x4 = x0 + 4e-7f, x5 = x0 + 5e-7f, x6 = x0 + 6e-7f, x7 = x0 + 7e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
      x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
    }
  }
  const float r = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (r == 123.456f) sink[blockIdx.x] = r;  // keeps the chains alive
}

// One thread waits, with the same bounded mbarrier wait the tensor-core kernels use, on a
// barrier that nothing arrives at; when the wait gives up it records the timeout in
// `status` and the kernel returns normally.
__global__ void k_wait_probe(int* status, uint32_t limit) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  tc::mbar_init(&bar, 1);
  tc::fence_mbar_init();
  *status = tc::mbar_wait(&bar, 0, limit) ? 0 : 1;
}

}  // namespace
}  // namespace mlf

extern "C" int mlf_probe_wait_timeout(uint32_t limit, void* stream) {
  using namespace mlf;
  clear_error();
  if (limit == 0 || limit > (1u << 20)) return fail(MLF_ERR_INVALID, "mlf_probe_wait_timeout: limit outside [1, 2^20]");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  DevBuf status;
  MLF_TRY(status.alloc(sizeof(int), "wait probe status"));
  MLF_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), st));
  k_wait_probe<<<1, 32, 0, st>>>(status.as<int>(), limit);
  MLF_LAUNCHED();
  int h = 0;
  MLF_CUDA(cudaMemcpyAsync(&h, status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  MLF_CUDA(cudaStreamSynchronize(st));
  if (h) return fail(MLF_ERR_TIMEOUT, "mlf_probe_wait_timeout: the bounded wait expired (as intended)");
  return MLF_OK;
}

extern "C" int mlf_probe_fp32_peak(double ms, double* tflops, void* stream) {
  using namespace mlf;
  clear_error();
  if (!tflops) return fail(MLF_ERR_INVALID, "mlf_probe_fp32_peak: null output");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int dev = 0, nsm = 0;
  MLF_CUDA(cudaGetDevice(&dev));
  MLF_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  DevBuf sink;
  MLF_TRY(sink.alloc(sizeof(float) * nsm * 8, "probe sink"));
  const int blocks = nsm * 8, threads = 256;
  cudaEvent_t e0, e1;
  MLF_CUDA(cudaEventCreate(&e0));
  MLF_CUDA(cudaEventCreate(&e1));
  int iters = 2048;
  float t = 0.f;
  for (int pass = 0; pass < 8; ++pass) {  // grow until the kernel runs for ~ms
    MLF_CUDA(cudaEventRecord(e0, st));
    k_fma_probe<<<blocks, threads, 0, st>>>(sink.as<float>(), iters, 0.999999f, 1e-7f);
    MLF_CUDA(cudaEventRecord(e1, st));
    MLF_CUDA(cudaEventSynchronize(e1));
    MLF_CUDA(cudaEventElapsedTime(&t, e0, e1));
    if (t >= ms || pass == 7) break;
    iters = (int)std::min<double>(1 << 26, iters * std::max(2.0, 1.2 * ms / std::max(1e-3f, t)));
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double flop = 2.0 * 8 * 16 * (double)iters * blocks * threads;
  *tflops = flop / (t * 1e-3) / 1e12;
  return MLF_OK;
}
