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
// probabilities.  The maximum of floats is a float (exact); each
// exponential is float32-accurate with no float64 operation (exp_diff); the
// sum is compensated (Kahan) per thread and float64 across the block, so it
// agrees with NumPy's float64 sum to about 1e-14; the normalisation is the
// product with the float32 reciprocal of that sum.  A probability agrees
// with the reference's float64 result cast to float32 within a few float32
// ulp.  NaN anywhere in the map makes every probability NaN, as NumPy's max
// and sum propagate it.  Alongside, per cluster: the maximum, the sum and
// the number of directions whose probabilities, taken largest first, reach
// 50 % and 90 % of the total -- the inputs of an error region (cWB's
// getSkyArea).
//
// The error-region counts need the largest probability p* such that the
// directions with p >= p* hold at least the level.  Probabilities are
// non-negative floats, whose bit patterns order as unsigned integers: a
// histogram over the exponent byte (mass and count per binade, built while
// the probabilities are written) finds the binade holding p* for both
// levels; that binade's probabilities are compacted into shared memory and
// p* is bisected over their 23 mantissa bits there.  Four passes over the
// map in all (one more per level whose binade holds more than kCap
// directions, which is then bisected over the map itself).  The float64
// pipe, narrow on this GPU, does a few operations per direction only in the
// block reductions.

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
constexpr int kBins = 256;         // exponent byte of a float32 probability
constexpr int kCap = 8192;         // probabilities of one binade kept in shared memory
constexpr size_t kSmem = sizeof(float) * 2 * kCap;

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

__device__ __forceinline__ float block_max(float v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < (blockDim.x >> 5) ? static_cast<float>(red[lane]) : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) red[0] = v;
  }
  __syncthreads();
  return static_cast<float>(red[0]);
}

// exp(s - m) for floats s <= m, to float32 accuracy in float32 arithmetic:
// the difference as an exact pair x + lo (Knuth's TwoSum), Cody-Waite
// reduction (W. J. Cody and W. Waite, Software Manual for the Elementary
// Functions, 1980) x + lo = k ln2 + r with ln2 split into a 16-bit head,
// so that k * head is exact for |k| < 2^8, and a tail, then expf(r) for
// |r| <= ln2 / 2 and the exact scaling by 2^k.  Within about 3 ulp of
// float(exp(s - m)); 0 below the smallest float32 (s - m < -104).
__device__ __forceinline__ float exp_diff(float s, float m) {
  const float b = -m;
  const float x = s + b;
  if (!(x > -104.0f)) return 0.0f;
  const float bv = x - s;
  const float lo = (s - (x - bv)) + (b - bv);
  constexpr float kLn2Hi = 0.693145751953125f;     // 45426 / 2^16
  constexpr float kLn2Lo = 1.42860682e-06f;        // ln 2 - kLn2Hi
  constexpr float kLog2e = 1.44269502f;
  const float k = rintf(x * kLog2e);
  float r = fmaf(-k, kLn2Hi, x);
  r = fmaf(-k, kLn2Lo, r) + lo;
  return ldexpf(expf(r), static_cast<int>(k));
}

__device__ __forceinline__ unsigned bits(float p) { return __float_as_uint(p); }

// The largest pattern lo in [lo, hi) of binade `bin` with
// above + mass(p >= lo, p in the binade) >= level, from the n compacted
// probabilities in `list` (or, when list is null, from the whole map).
__device__ unsigned bisect_binade(unsigned lo, unsigned hi, double above, double level,
                                  const float* list, int n, const float* out, int64_t n_sky,
                                  double* red) {
  const unsigned top = hi;                       // the binade's end
  while (hi - lo > 1u) {
    const unsigned mid = lo + ((hi - lo) >> 1);
    float m = 0.0f;
    if (list) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float p = list[i];
        if (bits(p) >= mid) m += p;
      }
    } else {
      for (int64_t l = threadIdx.x; l < n_sky; l += blockDim.x) {
        const float p = out[l];
        const unsigned q = bits(p);
        if (q >= mid && q < top) m += p;
      }
    }
    const double tot = above + block_sum(static_cast<double>(m), red);
    if (tot >= level) lo = mid; else hi = mid;
  }
  return lo;
}

__global__ void __launch_bounds__(kThreads, 2) sky_probability_kernel(
    int64_t n_sky, const float* __restrict__ stats, int64_t stats_stride,
    const int32_t* __restrict__ clusters, float* __restrict__ prob, double* __restrict__ summary) {
  extern __shared__ float lists[];             // [2][kCap]
  __shared__ double red[32];
  __shared__ float hmass[kBins];
  __shared__ int hcnt[kBins];
  __shared__ int n_list[2];
  __shared__ int sel_bin[2];
  __shared__ double sel_above[2];
  __shared__ double sel_count[2];
  const int c = clusters ? clusters[blockIdx.x] : static_cast<int>(blockIdx.x);
  const float* s = stats + static_cast<int64_t>(c) * stats_stride + kStatRow * n_sky;
  float* out = prob + static_cast<int64_t>(blockIdx.x) * n_sky;
  const int tid = threadIdx.x;

  for (int b = tid; b < kBins; b += blockDim.x) {
    hmass[b] = 0.0f;
    hcnt[b] = 0;
  }
  if (tid < 2) n_list[tid] = 0;

  // pass 1: NaN and maximum (the maximum of floats is a float)
  float mx = -INFINITY;
  int nan = 0;
  for (int64_t l = tid; l < n_sky; l += blockDim.x) {
    const float v = s[l];
    nan |= isnan(v);
    mx = fmaxf(mx, v);
  }
  nan = __syncthreads_or(nan);
  if (nan) {
    for (int64_t l = tid; l < n_sky; l += blockDim.x) out[l] = NAN;
    if (tid == 0 && summary) {
      double* o = summary + 4 * static_cast<int64_t>(blockIdx.x);
      o[0] = o[1] = o[2] = o[3] = NAN;
    }
    return;
  }
  mx = block_max(mx, red);

  // pass 2: the sum of the exponentials, compensated per thread
  float sh = 0.0f, sc = 0.0f;
  for (int64_t l = tid; l < n_sky; l += blockDim.x) {
    const float y = exp_diff(s[l], mx) - sc;
    const float t = sh + y;
    sc = (t - sh) - y;
    sh = t;
  }
  const double sum = block_sum(static_cast<double>(sh) - static_cast<double>(sc), red);
  const float inv = static_cast<float>(1.0 / sum);

  // pass 3: the probabilities, and their mass and count per binade (a
  // thread's run of one binade goes to shared memory in one update)
  {
    int cur = -1, cnt = 0;
    float mass = 0.0f;
    for (int64_t l = tid; l < n_sky; l += blockDim.x) {
      const float p = exp_diff(s[l], mx) * inv;
      out[l] = p;
      const int b = static_cast<int>(bits(p) >> 23);
      if (b != cur) {
        if (cnt) {
          atomicAdd(&hmass[cur], mass);
          atomicAdd(&hcnt[cur], cnt);
        }
        cur = b;
        mass = 0.0f;
        cnt = 0;
      }
      mass += p;
      ++cnt;
    }
    if (cnt) {
      atomicAdd(&hmass[cur], mass);
      atomicAdd(&hcnt[cur], cnt);
    }
  }
  __syncthreads();
  // the binade of p* for each level: the mass of the binades above it is
  // below the level, with it at or above
  if (tid < 2) {
    const double level = tid == 0 ? 0.5 : 0.9;
    double cum = 0.0, above = 0.0, cabove = 0.0, ccum = 0.0;
    int sel = 0;
    for (int b = kBins - 1; b >= 0; --b) {
      above = cum;
      cabove = ccum;
      cum += static_cast<double>(hmass[b]);
      ccum += static_cast<double>(hcnt[b]);
      sel = b;
      if (cum >= level) break;
    }
    sel_bin[tid] = sel;
    sel_above[tid] = above;
    sel_count[tid] = cabove;
  }
  __syncthreads();

  // pass 4: the selected binades' probabilities into shared memory
  const int b0 = sel_bin[0], b1 = sel_bin[1];
  for (int64_t l = tid; l < n_sky; l += blockDim.x) {
    const float p = out[l];
    const int b = static_cast<int>(bits(p) >> 23);
    if (b == b0) {
      const int i = atomicAdd(&n_list[0], 1);
      if (i < kCap) lists[i] = p;
    }
    if (b == b1) {
      const int i = atomicAdd(&n_list[1], 1);
      if (i < kCap) lists[kCap + i] = p;
    }
  }
  __syncthreads();

  double counts[2];
  for (int q = 0; q < 2; ++q) {
    const unsigned blo = static_cast<unsigned>(sel_bin[q]) << 23;
    const unsigned bhi = static_cast<unsigned>(sel_bin[q] + 1) << 23;
    const int n = n_list[q];
    const bool fits = n <= kCap;
    const float* list = fits ? lists + q * kCap : nullptr;
    const unsigned lo = bisect_binade(blo, bhi, sel_above[q], q == 0 ? 0.5 : 0.9, list,
                                      fits ? n : 0, out, n_sky, red);
    double m = 0.0;
    if (fits) {
      for (int i = tid; i < n; i += blockDim.x) m += bits(list[i]) >= lo;
    } else {
      for (int64_t l = tid; l < n_sky; l += blockDim.x) {
        const unsigned v = bits(out[l]);
        m += (v >= lo && v < bhi);
      }
    }
    counts[q] = sel_count[q] + block_sum(m, red);
  }
  if (tid == 0 && summary) {
    double* o = summary + 4 * static_cast<int64_t>(blockIdx.x);
    o[0] = static_cast<double>(mx);
    o[1] = sum;
    o[2] = counts[0];
    o[3] = counts[1];
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
  // per device and per call (a few microseconds): callers may use several
  // devices and threads
  const cudaError_t ea = cudaFuncSetAttribute(
      sky_probability_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kSmem));
  if (ea != cudaSuccess)
    return pgw::fail(PGW_ERR_CUDA, std::string("sky_probability_kernel smem: ") + cudaGetErrorString(ea));
  sky_probability_kernel<<<n_select, kThreads, kSmem, static_cast<cudaStream_t>(stream)>>>(
      n_sky, stats, stats_stride, clusters, out_probability, out_summary);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return pgw::fail(PGW_ERR_CUDA, std::string("sky_probability_kernel: ") + cudaGetErrorString(e));
  return PGW_OK;
}
