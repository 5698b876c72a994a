// Arithmetic throughput probes, the measured denominators of the rooflines:
// FP32 FMA (the sky loop) and float64 multiply/add issued as separate,
// separately rounded instructions (the td-amplitude build).  Every thread
// runs 8 independent register chains (no memory traffic inside the loop);
// the host times the launch with CUDA events.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
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

// Chains of __dmul_rn then __dadd_rn: one multiply and one add per step, the
// instruction mix of td_vecs_kernel's FIRs.
__global__ void __launch_bounds__(256) dmul_dadd_chains_kernel(int iters, double a, double b,
                                                               double* sink) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-9 + k * 1e-9;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
#pragma unroll
      for (int k = 0; k < 8; ++k) x[k] = __dadd_rn(__dmul_rn(x[k], a), b);
    }
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 12345.678) sink[threadIdx.x] = s;
}

template <typename Kernel, typename T>
int time_probe(Kernel kernel, int iters, T a, T b, void* stream, int* n_sm_out, float* ms_out) {
  int dev = 0, n_sm = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return pgw::fail(PGW_ERR_CUDA, "device query failed");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  kernel<<<n_sm * 8, 256, 0, s>>>(iters / 4 + 1, a, b, nullptr);  // warm-up
  cudaEventRecord(e0, s);
  kernel<<<n_sm * 8, 256, 0, s>>>(iters, a, b, nullptr);
  cudaEventRecord(e1, s);
  const cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return pgw::fail(PGW_ERR_CUDA, std::string("probe: ") + cudaGetErrorString(e));
  if (ms <= 0.f) return pgw::fail(PGW_ERR_CUDA, "probe: no elapsed time");
  *n_sm_out = n_sm;
  *ms_out = ms;
  return PGW_OK;
}

}  // namespace

extern "C" int pgw_fp64_mul_add_peak(int iters, double* out_gops, double* out_ms, void* stream) {
  if (iters < 1 || !out_gops) return pgw::fail(PGW_ERR_BAD_ARGUMENT, "iters >= 1 and an output");
  int n_sm = 0;
  float ms = 0.f;
  const int rc = time_probe(dmul_dadd_chains_kernel, iters, 0.999999999, 1e-9, stream, &n_sm, &ms);
  if (rc != PGW_OK) return rc;
  const double ops = 2.0 * n_sm * 8.0 * 256.0 * iters * 8.0 * 8.0;  // one mul + one add per step
  *out_gops = ops / (ms * 1e-3) / 1e9;
  if (out_ms) *out_ms = ms;
  return PGW_OK;
}

extern "C" int pgw_fp32_fma_peak(int iters, double* out_tflops, double* out_ms, void* stream) {
  if (iters < 1 || !out_tflops) return pgw::fail(PGW_ERR_BAD_ARGUMENT, "iters >= 1 and an output");
  int n_sm = 0;
  float ms = 0.f;
  const int rc = time_probe(fma_chains_kernel, iters, 0.999999f, 1e-7f, stream, &n_sm, &ms);
  if (rc != PGW_OK) return rc;
  const double fmas = static_cast<double>(n_sm) * 8 * 256 * iters * 16.0 * 8.0;
  *out_tflops = 2.0 * fmas / (ms * 1e-3) / 1e12;
  if (out_ms) *out_ms = ms;
  return PGW_OK;
}

// Device-driven copy from page-locked host memory: every thread moves 16-byte
// words (grid-stride), so the SMs keep many host-page translations in flight
// at once.  Used by the batched loop's upload; the copy engine's path was
// measured at 5-11 GB/s on its first pass over a buffer after a large sky-loop
// launch (210 GB/s otherwise).
namespace {
__global__ void __launch_bounds__(256) copy_from_host_kernel(uint4* __restrict__ dst,
                                                             const uint4* __restrict__ src,
                                                             size_t n16) {
  const size_t stride = static_cast<size_t>(gridDim.x) * blockDim.x;
  for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n16; i += stride)
    dst[i] = src[i];
}
__global__ void copy_tail_kernel(unsigned char* dst, const unsigned char* src, size_t n) {
  const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i];
}
}  // namespace

extern "C" int pgw_copy_from_host(void* dst, const void* host_src, size_t bytes, void* stream) {
  if (bytes == 0) return PGW_OK;
  if (!dst || !host_src) return pgw::fail(PGW_ERR_BAD_ARGUMENT, "NULL pointer");
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, host_src) != cudaSuccess || at.type != cudaMemoryTypeHost)
    return pgw::fail(PGW_ERR_BAD_ARGUMENT, "source is not page-locked host memory");
  const void* dev_src = at.devicePointer ? at.devicePointer : host_src;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0, n_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return pgw::fail(PGW_ERR_CUDA, "device query failed");
  const bool aligned = (reinterpret_cast<uintptr_t>(dst) % 16 == 0) &&
                       (reinterpret_cast<uintptr_t>(dev_src) % 16 == 0);
  size_t head = 0;
  if (aligned) {
    const size_t n16 = bytes / 16;
    head = n16 * 16;
    if (n16) {
      const unsigned blocks = static_cast<unsigned>(
          std::min<size_t>((n16 + 255) / 256, static_cast<size_t>(n_sm) * 8));
      copy_from_host_kernel<<<blocks, 256, 0, s>>>(static_cast<uint4*>(dst),
                                                   static_cast<const uint4*>(dev_src), n16);
    }
  }
  const size_t tail = bytes - head;
  if (tail)
    copy_tail_kernel<<<static_cast<unsigned>((tail + 255) / 256), 256, 0, s>>>(
        static_cast<unsigned char*>(dst) + head, static_cast<const unsigned char*>(dev_src) + head,
        tail);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return pgw::fail(PGW_ERR_CUDA, std::string("copy_from_host: ") + cudaGetErrorString(e));
  return PGW_OK;
}
