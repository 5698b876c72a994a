// WDM forward transform (both quadratures) for GB300 (sm_103a).
//
// cWB's WDM::t2w(MM = -1) (cwb-core/WDM.cc:1384-1535), which the reference
// reaches through wdm_wavelet's t2w (pycwb/utils/td_vector_batch.py:80):
// the series x (n_ts samples) is extended by mirroring at both ends
// (x(-k) = x(k), x(n_ts + k) = x(n_ts - 1 - k)) and cut into N = ceil(n_ts/M)
// time slices.  For slice n the window (filter f of odd length nW,
// (nW - 1) a multiple of 2M) centred on sample nM is folded modulo 2M,
//
//     r[m] = sum_{t = m mod 2M, |t| <= nW - 1} x(nM + t) f(|t|),  m < 2M,
//
// a real DFT X[k] = sum_m r[m] exp(-2 pi i k m / 2M) (FFTW's forward sign)
// gives layers k = 0..M, the two edge layers scaled by 1/sqrt(2) in both
// parts (re = im = Re X / sqrt 2), and the quadratures are
//
//     (k + n) odd:  a00 = sqrt2 Im X,  a90 = sqrt2 Re X
//     (k + n) even: a00 = sqrt2 Re X,  a90 = -sqrt2 Im X.
//
// One CTA transforms G = max(1, 2048 / 2M) consecutive slices: the fold
// reads the series coalesced along m and writes the folded values in
// bit-reversed order to shared memory; a radix-2 decimation-in-time FFT of
// length 2M runs there in float64 with twiddles from one table per device
// (W_8192^j, j < 4096, from sincospi; the twiddle W_2M^k of any M <= 4096 is
// entry k 4096/M, the same angle to the last bit); the M+1
// outputs of each slice are written as float64 maps (n, m) and/or as the
// zero-padded float32 planes that the td-amplitude build reads.  All work is
// float64; the fold costs 2 nW / M FMAs per input sample and the FFT
// ~5 log2(2M) flops per sample, so the kernel is bound by FP64 issue for
// long filters and by DRAM for short ones, at a few GB per second of
// strain either way.

#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/pycwb_gb300.h"

namespace pgw {
int fail(int code, const std::string& msg);
}

namespace {

constexpr double kSqrt2 = 1.4142135623730951;  // the double nearest sqrt(2)
constexpr int kSlicePoints = 2048;              // complex points per CTA (G * 2M)
constexpr int kThreads = 256;
constexpr int kMaxM = 4096;

// W_8192^j = exp(-2 pi i j / 8192), j < 4096, on every device that loads the
// library (64 KB), filled once per device by twiddle_init_kernel.
__device__ double2 g_wdm_twiddle[kMaxM];

__global__ void twiddle_init_kernel() {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= kMaxM) return;
  double s, c;
  sincospi(static_cast<double>(j) / static_cast<double>(kMaxM), &s, &c);
  g_wdm_twiddle[j] = make_double2(c, -s);
}

__device__ __forceinline__ double series_at(const double* __restrict__ x, int64_t n_ts, int64_t s) {
  if (s < 0) s = -s;                    // x(-k) = x(k)
  else if (s >= n_ts) s = 2 * n_ts - 1 - s;  // x(n_ts + k) = x(n_ts - 1 - k)
  return __ldg(x + s);
}

__global__ void __launch_bounds__(kThreads)
wdm_t2w_kernel(const double* __restrict__ x, int64_t n_ts, int M, int log2M2,
               const double* __restrict__ filt, int64_t n_filter, int64_t n_time, int G,
               double* __restrict__ map00, double* __restrict__ map90,
               float* __restrict__ pad00, float* __restrict__ pad90, int n_pad) {
  extern __shared__ double2 smem[];
  const int M2 = 2 * M;
  const int half = M;                         // twiddles W^k, k < M
  double2* tw = smem;                         // [M]
  double2* buf = smem + half;                 // [G * M2]
  const int64_t n0 = static_cast<int64_t>(blockIdx.x) * G;
  const int64_t kfold = (n_filter - 1) / M2;  // filter spans t in [-kfold*M2, kfold*M2]

  const int tw_step = kMaxM / M;               // W_2M^k = W_8192^(k 4096 / M)
  for (int k = threadIdx.x; k < half; k += blockDim.x) tw[k] = g_wdm_twiddle[k * tw_step];

  // fold, stored bit-reversed for the in-place decimation-in-time FFT
  const int shift = 32 - log2M2;
  for (int e = threadIdx.x; e < G * M2; e += blockDim.x) {
    const int g = e / M2;
    const int m = e - g * M2;
    const int64_t n = n0 + g;
    double acc = 0.0;
    if (n < n_time) {
      const int64_t centre = n * M;
      const int64_t q_hi = (m == 0) ? kfold : kfold - 1;
      for (int64_t q = -kfold; q <= q_hi; ++q) {
        const int64_t t = m + q * M2;
        const int64_t at = t < 0 ? -t : t;
        acc = fma(series_at(x, n_ts, centre + t), __ldg(filt + at), acc);
      }
    }
    const int r = static_cast<int>(__brev(static_cast<unsigned>(m)) >> shift);
    buf[g * M2 + r] = make_double2(acc, 0.0);
  }

  for (int h = 1; h < M2; h <<= 1) {
    __syncthreads();
    const int stride = M / h;                 // twiddle step: 2M / (2h)
    for (int b = threadIdx.x; b < G * M; b += blockDim.x) {
      const int g = b / M;
      const int bb = b - g * M;
      const int k = bb & (h - 1);
      const int pos = g * M2 + ((bb - k) << 1) + k;
      const double2 w = tw[k * stride];
      const double2 u = buf[pos];
      const double2 v0 = buf[pos + h];
      const double2 v = make_double2(v0.x * w.x - v0.y * w.y, v0.x * w.y + v0.y * w.x);
      buf[pos] = make_double2(u.x + v.x, u.y + v.y);
      buf[pos + h] = make_double2(u.x - v.x, u.y - v.y);
    }
  }
  __syncthreads();

  const int M1 = M + 1;
  for (int e = threadIdx.x; e < G * M1; e += blockDim.x) {
    const int g = e / M1;
    const int m = e - g * M1;
    const int64_t n = n0 + g;
    if (n >= n_time) continue;
    const double2 X = buf[g * M2 + m];
    double re = X.x, im = X.y;
    if (m == 0 || m == M) {
      re = __ddiv_rn(re, kSqrt2);
      im = re;
    }
    double a00, a90;
    if (((m + static_cast<int>(n & 1)) & 1) != 0) {
      a00 = __dmul_rn(kSqrt2, im);
      a90 = __dmul_rn(kSqrt2, re);
    } else {
      a00 = __dmul_rn(kSqrt2, re);
      a90 = -__dmul_rn(kSqrt2, im);
    }
    const int64_t o = n * M1 + m;
    if (map00) {
      map00[o] = a00;
      map90[o] = a90;
    }
    if (pad00) {
      const int64_t op = (n + n_pad) * M1 + m;
      pad00[op] = static_cast<float>(a00);
      pad90[op] = static_cast<float>(a90);
    }
  }
}

}  // namespace

extern "C" int64_t pgw_wdm_n_time(int64_t n_samples, int M) {
  if (M < 1 || n_samples < 0) return -1;
  return (n_samples + M - 1) / M;
}

extern "C" int pgw_wdm_t2w(const double* ts, int64_t n_ts, int M, const double* filter,
                           int64_t n_filter, double* map00, double* map90, float* padded00,
                           float* padded90, int n_pad, void* stream) {
  if (M < 1 || M > 4096 || (M & (M - 1)) != 0)
    return pgw::fail(PGW_ERR_BAD_SHAPE, "WDM layers M must be a power of two in [1, 4096]");
  if (n_filter < 1 || (n_filter - 1) % (2 * static_cast<int64_t>(M)) != 0)
    return pgw::fail(PGW_ERR_BAD_SHAPE, "WDM filter length must be 1 + a multiple of 2M");
  if (n_ts <= n_filter)
    return pgw::fail(PGW_ERR_BAD_SHAPE, "series must be longer than the WDM filter");
  if (n_pad < 0) return pgw::fail(PGW_ERR_BAD_SHAPE, "n_pad must be >= 0");
  if (!ts || !filter) return pgw::fail(PGW_ERR_BAD_ARGUMENT, "NULL device pointer");
  if ((map00 == nullptr) != (map90 == nullptr) || (padded00 == nullptr) != (padded90 == nullptr))
    return pgw::fail(PGW_ERR_BAD_ARGUMENT, "give both maps (or neither) of each output");
  if (!map00 && !padded00) return pgw::fail(PGW_ERR_BAD_ARGUMENT, "no output requested");
  const int64_t n_time = (n_ts + M - 1) / M;
  const int M2 = 2 * M;
  const int G = M2 >= kSlicePoints ? 1 : kSlicePoints / M2;
  int log2M2 = 0;
  while ((1 << log2M2) < M2) ++log2M2;
  const int64_t blocks = (n_time + G - 1) / G;
  if (blocks > 0x7fffffffLL) return pgw::fail(PGW_ERR_BAD_SHAPE, "series too long");
  const size_t smem = sizeof(double2) * (static_cast<size_t>(M) + static_cast<size_t>(G) * M2);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // The twiddle table, once per device: filled on the caller's stream and
  // waited for, so later calls on any stream find it complete.  A first call
  // made while the stream is being captured puts the fill in the graph and
  // leaves the table marked empty, so the next ordinary call fills it again.
  {
    static std::mutex mu;
    static bool ready[256] = {false};
    int dev = 0;
    cudaError_t de = cudaGetDevice(&dev);
    if (de != cudaSuccess || dev < 0 || dev >= 256)
      return pgw::fail(PGW_ERR_CUDA, "cudaGetDevice failed for the WDM twiddle table");
    std::lock_guard<std::mutex> lock(mu);
    if (!ready[dev]) {
      cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
      de = cudaStreamIsCapturing(s, &cap);
      if (de != cudaSuccess)
        return pgw::fail(PGW_ERR_CUDA, std::string("wdm twiddles: ") + cudaGetErrorString(de));
      twiddle_init_kernel<<<kMaxM / kThreads, kThreads, 0, s>>>();
      de = cudaGetLastError();
      if (de == cudaSuccess && cap == cudaStreamCaptureStatusNone) {
        de = cudaStreamSynchronize(s);
        if (de == cudaSuccess) ready[dev] = true;
      }
      if (de != cudaSuccess)
        return pgw::fail(PGW_ERR_CUDA, std::string("wdm twiddles: ") + cudaGetErrorString(de));
    }
  }
  cudaError_t e = cudaFuncSetAttribute(wdm_t2w_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
  if (e != cudaSuccess)
    return pgw::fail(PGW_ERR_CUDA, std::string("wdm_t2w_kernel smem: ") + cudaGetErrorString(e));
  if (padded00 && n_pad > 0) {
    const size_t pad_bytes = sizeof(float) * static_cast<size_t>(n_pad) * (M + 1);
    const size_t tail = sizeof(float) * static_cast<size_t>(n_time + n_pad) * (M + 1);
    for (float* p : {padded00, padded90}) {
      e = cudaMemsetAsync(p, 0, pad_bytes, s);
      if (e == cudaSuccess) e = cudaMemsetAsync(reinterpret_cast<char*>(p) + tail, 0, pad_bytes, s);
      if (e != cudaSuccess)
        return pgw::fail(PGW_ERR_CUDA, std::string("wdm padding: ") + cudaGetErrorString(e));
    }
  }
  wdm_t2w_kernel<<<static_cast<unsigned>(blocks), kThreads, smem, s>>>(
      ts, n_ts, M, log2M2, filter, n_filter, n_time, G, map00, map90, padded00, padded90, n_pad);
  e = cudaGetLastError();
  if (e != cudaSuccess) return pgw::fail(PGW_ERR_CUDA, std::string("wdm_t2w_kernel: ") + cudaGetErrorString(e));
  return PGW_OK;
}
