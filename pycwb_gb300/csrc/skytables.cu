// Sky tables on the device: HEALPix RING directions, per-detector antenna
// patterns and delay indices, the per-segment tables of the sky scan
// (compute_sky_delay_and_patterns, pycwb/types/detector.py:1243-1329 with
// _build_sky_directions :1220-1240 and atenna_pattern :272-358).
//
// One thread per sky pixel.  pix2ang follows the RING scheme's closed forms
// (integer ring/pixel arithmetic, then z and phi in float64); the antenna
// patterns contract each detector's response tensor with the wave frame at
// gha = -phi_geo, dec = latitude, psi = 0 (float64, stored as float32 in the
// scan's (n_sky, n_ifo) layout); the delay index is
// clip(rint((n . b_i) / c * rate), -K, K) with b_i the detector's baseline to
// the reference detector in metres.

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/pycwb_gb300.h"

namespace pgw {
int fail(int code, const std::string& msg);
}

namespace {

struct SkyGeom {
  double response[PGW_MAX_IFO][9];  // row-major 3x3 response tensor
  double baseline[PGW_MAX_IFO][3];  // R_i - R_ref, metres
};

// floor(sqrt(v)) for v >= 0, exact for the sizes of a HEALPix grid
__device__ __forceinline__ int64_t isqrt64(int64_t v) {
  int64_t r = static_cast<int64_t>(sqrt(static_cast<double>(v)));
  while (r * r > v) --r;
  while ((r + 1) * (r + 1) <= v) ++r;
  return r;
}

__global__ void sky_tables_kernel(int64_t nside, int n_ifo, SkyGeom g, double c_light, double rate,
                                  int K,
                                  float* __restrict__ FP, float* __restrict__ FX,
                                  int32_t* __restrict__ ml) {
  const int64_t npix = 12 * nside * nside;
  const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const int64_t ncap = 2 * nside * (nside - 1);
  const double pi = 3.14159265358979323846;
  double z, phi;
  if (p < ncap) {                          // north polar cap
    const int64_t iring = (1 + isqrt64(1 + 2 * p)) >> 1;
    const int64_t iphi = (p + 1) - 2 * iring * (iring - 1);
    z = 1.0 - static_cast<double>(iring * iring) * (4.0 / static_cast<double>(npix));
    phi = (static_cast<double>(iphi) - 0.5) * (0.5 * pi) / static_cast<double>(iring);
  } else if (p < npix - ncap) {            // equatorial belt
    const int64_t ip = p - ncap;
    const int64_t nl4 = 4 * nside;
    const int64_t tmp = ip / nl4;
    const int64_t iring = tmp + nside;
    const int64_t iphi = ip - nl4 * tmp + 1;
    const double fodd = ((iring + nside) & 1) ? 1.0 : 0.5;
    z = static_cast<double>(2 * nside - iring) * (2.0 / (3.0 * static_cast<double>(nside)));
    phi = (static_cast<double>(iphi) - fodd) * pi / (2.0 * static_cast<double>(nside));
  } else {                                  // south polar cap
    const int64_t ip = npix - p;
    const int64_t iring = (1 + isqrt64(2 * ip - 1)) >> 1;
    const int64_t iphi = 4 * iring + 1 - (ip - 2 * iring * (iring - 1));
    z = static_cast<double>(iring * iring) * (4.0 / static_cast<double>(npix)) - 1.0;
    phi = (static_cast<double>(iphi) - 0.5) * (0.5 * pi) / static_cast<double>(iring);
  }
  const double theta = acos(z);
  const double lat = 0.5 * pi - theta;
  // wave frame at gha = -phi, dec = lat, psi = 0
  const double singha = sin(-phi), cosgha = cos(-phi);
  const double sindec = sin(lat), cosdec = cos(lat);
  const double x[3] = {-singha, -cosgha, 0.0};
  const double y[3] = {-cosgha * sindec, singha * sindec, cosdec};
  const double n[3] = {cos(lat) * cos(phi), cos(lat) * sin(phi), sin(lat)};
  for (int i = 0; i < n_ifo; ++i) {
    const double* D = g.response[i];
    double fp = 0.0, fx = 0.0;
    for (int r = 0; r < 3; ++r) {
      const double dx = D[3 * r] * x[0] + D[3 * r + 1] * x[1] + D[3 * r + 2] * x[2];
      const double dy = D[3 * r] * y[0] + D[3 * r + 1] * y[1] + D[3 * r + 2] * y[2];
      fp += x[r] * dx - y[r] * dy;
      fx += x[r] * dy + y[r] * dx;
    }
    FP[p * n_ifo + i] = static_cast<float>(fp);
    FX[p * n_ifo + i] = static_cast<float>(fx);
    const double shift =
        (n[0] * g.baseline[i][0] + n[1] * g.baseline[i][1] + n[2] * g.baseline[i][2]) / c_light;
    double d = rint(shift * rate);
    d = d < -K ? -K : (d > K ? K : d);
    ml[static_cast<int64_t>(i) * npix + p] = static_cast<int32_t>(d);
  }
}

}  // namespace

extern "C" int pgw_sky_tables_healpix(int healpix_order, int n_ifo, const double* response,
                                      const double* baseline, double c_light, double sample_rate,
                                      int td_size, float* FP, float* FX, int32_t* ml,
                                      void* stream) {
  if (healpix_order < 0 || healpix_order > 13)
    return pgw::fail(PGW_ERR_BAD_SHAPE, "healpix_order must be in [0, 13]");
  if (n_ifo < 1 || n_ifo > PGW_MAX_IFO) return pgw::fail(PGW_ERR_BAD_SHAPE, "n_ifo must be in [1, 8]");
  if (!response || !baseline || !FP || !FX || !ml)
    return pgw::fail(PGW_ERR_BAD_ARGUMENT, "NULL pointer");
  if (td_size < 1) return pgw::fail(PGW_ERR_BAD_ARGUMENT, "td_size must be >= 1");
  SkyGeom g{};
  for (int i = 0; i < n_ifo; ++i) {
    for (int q = 0; q < 9; ++q) g.response[i][q] = response[i * 9 + q];
    for (int q = 0; q < 3; ++q) g.baseline[i][q] = baseline[i * 3 + q];
  }
  const int64_t nside = int64_t{1} << healpix_order;
  const int64_t npix = 12 * nside * nside;
  sky_tables_kernel<<<static_cast<unsigned>((npix + 255) / 256), 256, 0,
                      static_cast<cudaStream_t>(stream)>>>(nside, n_ifo, g, c_light, sample_rate,
                                                           td_size, FP, FX, ml);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return pgw::fail(PGW_ERR_CUDA, std::string("sky tables: ") + cudaGetErrorString(e));
  return PGW_OK;
}
