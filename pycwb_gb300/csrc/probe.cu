// FP32 FMA throughput probe: the measured denominator of the sky loop's
// FP32 roofline.  Every thread runs 8 independent chains of fused
// multiply-adds on registers (no memory traffic inside the loop); the host
// times the launch with CUDA events.
#include <cuda_runtime.h>

#include <string>

#include "../../include/pycwb_gb300.h"

namespace pgw {
int fail(int code, const std::string& msg);
}

namespace {

__global__ void __launch_bounds__(256) fma_chains_kernel(int iters, float a, float b, float* sink) {
  float x0 = threadIdx.x * 1e-7f, x1 = x0 + 1e-7f, x2 = x0 + 2e-7f, x3 = x0 + 3e-7f;
  float x4 = x0 + 4e-7f, x5 = x0 + 5e-7f, x6 = x0 + 6e-7f, x7 = x0 + 7e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
      x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
    }
  }
  const float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 12345.678f) sink[threadIdx.x] = s;  // keeps the chains alive
}

}  // namespace

extern "C" int pgw_fp32_fma_peak(int iters, double* out_tflops, double* out_ms, void* stream) {
  if (iters < 1 || !out_tflops) return pgw::fail(PGW_ERR_BAD_ARGUMENT, "iters >= 1 and an output");
  int dev = 0, n_sm = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return pgw::fail(PGW_ERR_CUDA, "device query failed");
  const int blocks = n_sm * 8, threads = 256;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chains_kernel<<<blocks, threads, 0, s>>>(iters / 4 + 1, 0.999999f, 1e-7f, nullptr);  // warm-up
  cudaEventRecord(e0, s);
  fma_chains_kernel<<<blocks, threads, 0, s>>>(iters, 0.999999f, 1e-7f, nullptr);
  cudaEventRecord(e1, s);
  const cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return pgw::fail(PGW_ERR_CUDA, std::string("fma probe: ") + cudaGetErrorString(e));
  const double fmas = static_cast<double>(blocks) * threads * iters * 16.0 * 8.0;
  *out_tflops = 2.0 * fmas / (ms * 1e-3) / 1e12;
  if (out_ms) *out_ms = ms;
  return PGW_OK;
}
