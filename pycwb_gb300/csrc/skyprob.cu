// Normalised sky probability of each cluster, on the device (sm_103a).
//
// The reference's caller turns the sky-statistic map into a probability
// map right after the scan (pycwb/modules/likelihoodWP/likelihood.py:
// 338-342):
//     s = nSkyStat.astype(float64);  e = exp(s - max(s));
//     nProbability = (e / sum(e)).astype(float32)
// over all n_sky entries (masked directions hold 0 and take part).  Here
// one CTA per selected cluster reads that cluster's map where the sky loop
// left it (stats block (11, n_sky), row 6) and writes the float32
// probabilities; the maximum, the sum and the normalisation are float64 as
// in the reference (the sum is a block reduction, so it agrees with NumPy's
// pairwise sum to float64 rounding), the exponentials float32-accurate
// (exp_neg), so a probability agrees with the reference's to a few float32
// ulp.  NaN anywhere in the map makes every probability NaN,
// as NumPy's max and sum propagate it.  Alongside, per cluster: the maximum,
// the sum and the number of directions whose probabilities, taken largest
// first, reach 50 % and 90 % of the total -- the inputs of an error region
// (cWB's getSkyArea), found by bisection on the probability threshold.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/pycwb_gb300.h"

namespace pgw {
int fail(int code, const std::string& msg);
}

namespace {

constexpr int kThreads = 1024;
constexpr int kStatRow = 6;        // nSkyStat in the (11, n_sky) block

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < (blockDim.x >> 5) ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[0] = v;
  }
  __syncthreads();
  return red[0];
}

__device__ __forceinline__ double block_max(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < (blockDim.x >> 5) ? red[lane] : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) red[0] = v;
  }
  __syncthreads();
  return red[0];
}

__device__ __forceinline__ int block_or(int v) { return __syncthreads_or(v); }

// exp(d) for d <= 0 to float32 accuracy without a float64 exponential (the
// float64 pipe is narrow on this GPU): Cody-Waite range reduction in float64,
// d = k ln2 + r with k = rint(d / ln2) and |r| <= ln2 / 2 (r exact to about
// 1e-16 |d| by one FMA with the double nearest ln2), then exp(r) in float32
// and the exact scaling by 2^k.  Within about 2 ulp of float(exp(d)); 0 below
// the smallest float32 (d < -104).
__device__ __forceinline__ float exp_neg(double d) {
  if (!(d > -104.0)) return 0.0f;
  const double k = rint(d * 1.4426950408889634);       // 1 / ln 2
  const float r = static_cast<float>(fma(-k, 0.6931471805599453, d));
  return ldexpf(expf(r), static_cast<int>(k));
}

__global__ void __launch_bounds__(kThreads) sky_probability_kernel(
    int64_t n_sky, const float* __restrict__ stats, int64_t stats_stride,
    const int32_t* __restrict__ clusters, float* __restrict__ prob, double* __restrict__ summary) {
  __shared__ double red[32];
  const int c = clusters ? clusters[blockIdx.x] : static_cast<int>(blockIdx.x);
  const float* s = stats + static_cast<int64_t>(c) * stats_stride + kStatRow * n_sky;
  float* out = prob + static_cast<int64_t>(blockIdx.x) * n_sky;

  double mx = -INFINITY;
  int nan = 0;
  for (int64_t l = threadIdx.x; l < n_sky; l += blockDim.x) {
    const double v = static_cast<double>(s[l]);
    nan |= isnan(v);
    mx = fmax(mx, v);
  }
  nan = block_or(nan);
  mx = block_max(mx, red);
  // the exponentials are float32-accurate (exp_neg); the sum and the
  // normalisation stay float64, as the reference's
  double sum = 0.0;
  if (!nan)
    for (int64_t l = threadIdx.x; l < n_sky; l += blockDim.x)
      sum += static_cast<double>(exp_neg(static_cast<double>(s[l]) - mx));
  sum = nan ? NAN : block_sum(sum, red);
  for (int64_t l = threadIdx.x; l < n_sky; l += blockDim.x)
    out[l] = nan ? NAN
                 : static_cast<float>(static_cast<double>(exp_neg(static_cast<double>(s[l]) - mx)) / sum);

  // Error-region inputs: the smallest set of directions, largest
  // probabilities first, holding at least 50 % / 90 % of the total.  The
  // probabilities are non-negative floats, whose bit patterns order as
  // unsigned integers, so the threshold is bisected over the bit patterns:
  // the largest pattern lo with mass(p >= lo) >= level, exact after about
  // 30 steps.  Each step sums the mass above the trial pattern in float32
  // per thread (the FP64 pipe is narrow on this GPU) and in float64 across
  // the block.
  __syncthreads();
  const double levels[2] = {0.5, 0.9};
  double counts[2] = {0.0, 0.0};
  if (!nan) {
    for (int q = 0; q < 2; ++q) {
      unsigned lo = 0u, hi = 0x7f800000u;   // mass(>= hi) = 0 < level <= mass(>= lo)
      while (hi - lo > 1u) {
        const unsigned mid = lo + ((hi - lo) >> 1);
        float m = 0.0f;
        for (int64_t l = threadIdx.x; l < n_sky; l += blockDim.x) {
          const float p = out[l];
          if (__float_as_uint(p) >= mid) m += p;
        }
        const double tot = block_sum(static_cast<double>(m), red);
        if (tot >= levels[q]) lo = mid; else hi = mid;
      }
      double n = 0.0;
      for (int64_t l = threadIdx.x; l < n_sky; l += blockDim.x) n += __float_as_uint(out[l]) >= lo;
      counts[q] = block_sum(n, red);
    }
  }
  if (threadIdx.x == 0 && summary) {
    double* o = summary + 4 * static_cast<int64_t>(blockIdx.x);
    o[0] = nan ? NAN : mx;
    o[1] = sum;
    o[2] = nan ? NAN : counts[0];
    o[3] = nan ? NAN : counts[1];
  }
}

}  // namespace

extern "C" int pgw_sky_probability(int n_select, int64_t n_sky, const float* stats,
                                   int64_t stats_stride, const int32_t* clusters,
                                   float* out_probability, double* out_summary, void* stream) {
  if (n_select < 0 || n_sky < 1 || stats_stride < PGW_N_STATS * n_sky)
    return pgw::fail(PGW_ERR_BAD_SHAPE,
                     "pgw_sky_probability: need n_select >= 0, n_sky >= 1, stats_stride >= 11 n_sky");
  if (n_select == 0) return PGW_OK;
  if (!stats || !out_probability)
    return pgw::fail(PGW_ERR_BAD_ARGUMENT, "pgw_sky_probability: NULL device pointer");
  sky_probability_kernel<<<n_select, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      n_sky, stats, stats_stride, clusters, out_probability, out_summary);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return pgw::fail(PGW_ERR_CUDA, std::string("sky_probability_kernel: ") + cudaGetErrorString(e));
  return PGW_OK;
}
