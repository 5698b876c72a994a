// td-amplitude build (WDM time-delay vectors) for GB300 (sm_103a).
//
// For a pixel (time bin n, layer m) of one detector's WDM plane and a delay
// dT in [-K, K], the amplitude of the delayed pixel is a same-layer FIR of
// the 00 (or 90) plane with the T0 filter plus FIRs of the two neighbouring
// layers with Tx, each split into even and odd taps and multiplied by the
// phase factors of (m, dT); delays of a whole pixel or more swap the
// quadratures (pycwb/utils/td_vector_kernels.py:15-199, the form of cWB's
// WDM::getTDamp, cwb-core/WDM.cc:1103-1196).
//
// One thread computes one (pixel, delay) pair: both quadratures, six FIRs
// of 2*n_coeffs+1 taps.  Accumulation is float64 with every multiply and add
// rounded separately, in the reference's order, and the phase factors come
// precomputed from the host's libm, so the float32 results are bit-identical
// to the reference's.

#include <cuda_runtime.h>

#include <string>

#include "../../include/pycwb_gb300.h"

namespace pgw {
int fail(int code, const std::string& msg);
}

namespace {

constexpr double kSqrt2 = 1.4142135623730951;  // the double nearest sqrt(2)

__device__ __forceinline__ double plane_at(const float* __restrict__ plane, int64_t rows, int M1,
                                           int64_t r, int m) {
  return (r < 0 || r >= rows) ? 0.0 : static_cast<double>(__ldg(plane + r * M1 + m));
}

__device__ __forceinline__ void fir(const float* __restrict__ plane, int64_t rows, int M1,
                                    int64_t n, int m, const double* __restrict__ T, int win,
                                    double& even, double& odd) {
  even = 0.0;
  odd = 0.0;
  for (int k = 0; k < win; ++k) {
    const double v = __dmul_rn(plane_at(plane, rows, M1, n + k, m), __ldg(T + k));
    if (k & 1) odd = __dadd_rn(odd, v); else even = __dadd_rn(even, v);
  }
}

__device__ double pixel_amplitude(int64_t n, int m, int dT, const float* __restrict__ plane,
                                  int64_t rows, const double* __restrict__ T0,
                                  const double* __restrict__ Tx, int M, int nc, int J, bool quad,
                                  const double* __restrict__ phase) {
  const bool odd_n = (n & 1) != 0;
  const bool odd_mn = ((m + n) & 1) != 0;
  const bool cancel_even = odd_n != quad;
  const bool edge = (m == 0) || (m == M);
  const int M1 = M + 1;
  const int idx = dT + J;
  const int win = 2 * nc + 1;
  const double* ph = phase + (static_cast<int64_t>(m) * (2 * J + 1) + idx) * 4;
  const double* t0 = T0 + static_cast<int64_t>(idx) * win;
  const double* tx = Tx + static_cast<int64_t>(idx) * win;

  double se, so;
  fir(plane, rows, M1, n, m, t0, win, se, so);
  if (edge && cancel_even) se = 0.0;
  if (edge && !cancel_even) so = 0.0;
  const double a = __dmul_rn(se, __ldg(ph + 0)), b = __dmul_rn(so, __ldg(ph + 1));
  double result = odd_n ? __dsub_rn(a, b) : __dadd_rn(a, b);

  if (m > 0) {
    double le, lo;
    fir(plane, rows, M1, n, m - 1, tx, win, le, lo);
    if (m == 1 && cancel_even) le = 0.0;
    if (m == 1 && !cancel_even) lo = 0.0;
    double low = __dmul_rn(odd_n ? __dsub_rn(le, lo) : __dadd_rn(le, lo), __ldg(ph + 2));
    if (m == 1 || m == M) low = __dmul_rn(low, kSqrt2);
    result = odd_mn ? __dsub_rn(result, low) : __dadd_rn(result, low);
  }
  if (m < M) {
    double he, ho;
    fir(plane, rows, M1, n, m + 1, tx, win, he, ho);
    if (m == M - 1 && cancel_even) he = 0.0;
    if (m == M - 1 && !cancel_even) ho = 0.0;
    double high = __dmul_rn(odd_n ? __dadd_rn(he, ho) : __dsub_rn(he, ho), __ldg(ph + 3));
    if (m == 0 || m == M - 1) high = __dmul_rn(high, kSqrt2);
    result = odd_mn ? __dsub_rn(result, high) : __dadd_rn(result, high);
  }
  return (edge && cancel_even) ? 0.0 : result;
}

__global__ void td_vecs_kernel(const int32_t* __restrict__ pixel_indices, int64_t n_pixels,
                               const float* __restrict__ p00, const float* __restrict__ p90,
                               int64_t rows, const double* __restrict__ T0,
                               const double* __restrict__ Tx, const double* __restrict__ phase,
                               int M, int nc, int K, int J, float* __restrict__ out) {
  const int half = 2 * K + 1;
  const int64_t gid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= n_pixels * half) return;
  const int64_t p = gid / half;
  const int ki = static_cast<int>(gid % half);
  const int64_t idx = pixel_indices[p];
  const int64_t n = idx / (M + 1);
  const int m = static_cast<int>(idx % (M + 1));
  const int dT = ki - K;
  const int shift = dT >= 0 ? dT / J : -((-dT) / J);
  const int sub = dT - shift * J;
  const int64_t ne = n - shift;
  double a00, a90;
  if (shift % 2 != 0) {
    const double x = pixel_amplitude(ne, m, sub, p90, rows, T0, Tx, M, nc, J, true, phase);
    const double y = pixel_amplitude(ne, m, sub, p00, rows, T0, Tx, M, nc, J, false, phase);
    if ((n + m) % 2 != 0) { a00 = -x; a90 = y; } else { a00 = x; a90 = -y; }
  } else {
    a00 = pixel_amplitude(ne, m, sub, p00, rows, T0, Tx, M, nc, J, false, phase);
    a90 = pixel_amplitude(ne, m, sub, p90, rows, T0, Tx, M, nc, J, true, phase);
  }
  out[p * 2 * half + ki] = static_cast<float>(a00);
  out[p * 2 * half + half + ki] = static_cast<float>(a90);
}

// Same amplitudes, written into the batched scan's cluster layout: pixel p
// of this (plane, detector) belongs to cluster dst_cluster[p] at local
// position dst_pixel[p]; a00(dT) goes to td00_all[td_off[c] + ((dT+K) *
// n_ifo + ifo) * P_c + j], as the reference's set_td_amp_from_dense and the
// transposes of likelihood.py:303-304 would arrange it.
__global__ void td_vecs_scatter_kernel(const int32_t* __restrict__ pixel_indices, int64_t n_pixels,
                                       const int32_t* __restrict__ dst_cluster,
                                       const int32_t* __restrict__ dst_pixel, int n_clusters,
                                       const int64_t* __restrict__ pix_offsets,
                                       const int64_t* __restrict__ td_offsets, int ifo, int n_ifo,
                                       const float* __restrict__ p00, const float* __restrict__ p90,
                                       int64_t rows, const double* __restrict__ T0,
                                       const double* __restrict__ Tx,
                                       const double* __restrict__ phase, int M, int nc, int K,
                                       int J, float* __restrict__ td00_all,
                                       float* __restrict__ td90_all) {
  const int half = 2 * K + 1;
  const int64_t gid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= n_pixels * half) return;
  const int64_t p = gid / half;
  const int ki = static_cast<int>(gid % half);
  const int64_t idx = pixel_indices[p];
  const int64_t n = idx / (M + 1);
  const int m = static_cast<int>(idx % (M + 1));
  const int dT = ki - K;
  const int shift = dT >= 0 ? dT / J : -((-dT) / J);
  const int sub = dT - shift * J;
  const int64_t ne = n - shift;
  double a00, a90;
  if (shift % 2 != 0) {
    const double x = pixel_amplitude(ne, m, sub, p90, rows, T0, Tx, M, nc, J, true, phase);
    const double y = pixel_amplitude(ne, m, sub, p00, rows, T0, Tx, M, nc, J, false, phase);
    if ((n + m) % 2 != 0) { a00 = -x; a90 = y; } else { a00 = x; a90 = -y; }
  } else {
    a00 = pixel_amplitude(ne, m, sub, p00, rows, T0, Tx, M, nc, J, false, phase);
    a90 = pixel_amplitude(ne, m, sub, p90, rows, T0, Tx, M, nc, J, true, phase);
  }
  const int c = dst_cluster[p];
  if (c < 0 || c >= n_clusters) return;  // a bad destination is dropped, never written
  const int64_t P = pix_offsets[c + 1] - pix_offsets[c];
  const int64_t j = dst_pixel[p];
  if (j < 0 || j >= P) return;
  const int64_t o = td_offsets[c] + (static_cast<int64_t>(ki) * n_ifo + ifo) * P + j;
  td00_all[o] = static_cast<float>(a00);
  td90_all[o] = static_cast<float>(a90);
}

}  // namespace

extern "C" int pgw_td_vecs_to_clusters(const int32_t* pixel_indices, int64_t n_pixels,
                                       const int32_t* dst_cluster, const int32_t* dst_pixel,
                                       int n_clusters, const int64_t* pix_offsets, const int64_t* td_offsets,
                                       int ifo, int n_ifo, const float* padded00,
                                       const float* padded90, int64_t rows, const double* T0,
                                       const double* Tx, const double* phase, int M, int n_coeffs,
                                       int K, int J, float* td00_all, float* td90_all,
                                       void* stream) {
  if (M < 1 || n_coeffs < 0 || K < 0 || J < 1 || rows < 0 || n_pixels < 0)
    return pgw::fail(PGW_ERR_BAD_SHAPE, "td vectors need M >= 1, J >= 1, K >= 0, n_coeffs >= 0");
  if (n_clusters < 0) return pgw::fail(PGW_ERR_BAD_SHAPE, "n_clusters must be >= 0");
  if (ifo < 0 || ifo >= n_ifo || n_ifo > PGW_MAX_IFO)
    return pgw::fail(PGW_ERR_BAD_SHAPE, "ifo must be in [0, n_ifo), n_ifo <= 8");
  if (n_pixels == 0) return PGW_OK;
  if (!pixel_indices || !dst_cluster || !dst_pixel || !pix_offsets || !td_offsets || !padded00 ||
      !padded90 || !T0 || !Tx || !phase || !td00_all || !td90_all)
    return pgw::fail(PGW_ERR_BAD_ARGUMENT, "NULL device pointer");
  const int64_t total = n_pixels * (2 * K + 1);
  const int threads = 256;
  const int64_t blocks = (total + threads - 1) / threads;
  if (blocks > 0x7fffffffLL) return pgw::fail(PGW_ERR_BAD_SHAPE, "too many pixels");
  td_vecs_scatter_kernel<<<static_cast<unsigned>(blocks), threads, 0,
                           static_cast<cudaStream_t>(stream)>>>(
      pixel_indices, n_pixels, dst_cluster, dst_pixel, n_clusters, pix_offsets, td_offsets, ifo, n_ifo,
      padded00, padded90, rows, T0, Tx, phase, M, n_coeffs, K, J, td00_all, td90_all);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return pgw::fail(PGW_ERR_CUDA, std::string("td_vecs_scatter_kernel: ") + cudaGetErrorString(e));
  return PGW_OK;
}

extern "C" int pgw_batch_get_td_vecs(const int32_t* pixel_indices, int64_t n_pixels,
                                     const float* padded00, const float* padded90, int64_t rows,
                                     const double* T0, const double* Tx, const double* phase, int M,
                                     int n_coeffs, int K, int J, float* out, void* stream) {
  if (M < 1 || n_coeffs < 0 || K < 0 || J < 1 || rows < 0 || n_pixels < 0)
    return pgw::fail(PGW_ERR_BAD_SHAPE, "td vectors need M >= 1, J >= 1, K >= 0, n_coeffs >= 0");
  if (n_pixels == 0) return PGW_OK;
  if (!pixel_indices || !padded00 || !padded90 || !T0 || !Tx || !phase || !out)
    return pgw::fail(PGW_ERR_BAD_ARGUMENT, "NULL device pointer");
  const int64_t total = n_pixels * (2 * K + 1);
  const int threads = 256;
  const int64_t blocks = (total + threads - 1) / threads;
  if (blocks > 0x7fffffffLL) return pgw::fail(PGW_ERR_BAD_SHAPE, "too many pixels");
  td_vecs_kernel<<<static_cast<unsigned>(blocks), threads, 0, static_cast<cudaStream_t>(stream)>>>(
      pixel_indices, n_pixels, padded00, padded90, rows, T0, Tx, phase, M, n_coeffs, K, J, out);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return pgw::fail(PGW_ERR_CUDA, std::string("td_vecs_kernel: ") + cudaGetErrorString(e));
  return PGW_OK;
}
