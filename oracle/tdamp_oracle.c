/*
 * td-amplitude oracle: CPU restatement of PycWB's batch time-delay vector
 * extraction (the WDM getTDamp equivalent that feeds the sky scan).
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/ and by bench.py's CPU baseline,
 * never by the product.  Follows
 *
 *   _get_pixel_amplitude_nb  pycwb/utils/td_vector_kernels.py:15-130
 *   batch_get_td_vecs        pycwb/utils/td_vector_kernels.py:133-199
 *
 * in double precision with the same summation order and no fused
 * multiply-add (build with -ffp-contract=off), so the float32 outputs are
 * bit-identical to the reference's.  The trigonometric phase factors depend
 * only on (layer, delay); the caller passes them precomputed (cos/sin of
 * the same float64 phase expressions, evaluated with the host libm) as the
 * table ``phase[(m * (2J+1) + dT + J) * 4 + {0,1,2,3}] =
 * {cos(same), sin(same), sin(low), sin(high)}``.
 *
 * Rows of the padded plane outside [0, rows) read as zero.  The reference
 * reads out of bounds there (numba does not bounds-check); inside the
 * padded range both agree.
 */
#include <math.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline double plane_at(const float* plane, int64_t rows, int M1, int64_t r, int m) {
  if (r < 0 || r >= rows) return 0.0;
  return (double)plane[r * M1 + m];
}

static double pixel_amplitude(int64_t n, int m, int dT, const float* plane, int64_t rows,
                              const double* T0, const double* Tx, int M, int nc, int J, int quad,
                              const double* phase) {
  const int is_odd_n = (n & 1) != 0;
  const int is_odd_mn = ((m + n) & 1) != 0;
  const int cancel_even = is_odd_n ^ quad;
  const int edge = (m == 0) || (m == M);
  const int M1 = M + 1;
  const int idx = dT + J;
  const int win = 2 * nc + 1;
  const double* ph = phase + ((int64_t)m * (2 * J + 1) + idx) * 4;

  double se = 0.0, so = 0.0;                              /* :46-52 */
  for (int k = 0; k < win; ++k) {
    double v = plane_at(plane, rows, M1, n + k, m) * T0[(int64_t)idx * win + k];
    if (k % 2 == 0) se += v; else so += v;
  }
  if (edge && cancel_even) se = 0.0;                      /* :54-57 */
  if (edge && !cancel_even) so = 0.0;
  double result = is_odd_n ? se * ph[0] - so * ph[1] : se * ph[0] + so * ph[1];   /* :59-63 */

  if (m > 0) {                                            /* :66-94 */
    double le = 0.0, lo = 0.0;
    for (int k = 0; k < win; ++k) {
      double v = plane_at(plane, rows, M1, n + k, m - 1) * Tx[(int64_t)idx * win + k];
      if (k % 2 == 0) le += v; else lo += v;
    }
    if (m == 1 && cancel_even) le = 0.0;
    if (m == 1 && !cancel_even) lo = 0.0;
    double low = is_odd_n ? (le - lo) * ph[2] : (le + lo) * ph[2];
    if (m == 1 || m == M) low *= sqrt(2.0);
    result = is_odd_mn ? result - low : result + low;
  }
  if (m < M) {                                            /* :97-125 */
    double he = 0.0, ho = 0.0;
    for (int k = 0; k < win; ++k) {
      double v = plane_at(plane, rows, M1, n + k, m + 1) * Tx[(int64_t)idx * win + k];
      if (k % 2 == 0) he += v; else ho += v;
    }
    if (m == M - 1 && cancel_even) he = 0.0;
    if (m == M - 1 && !cancel_even) ho = 0.0;
    double high = is_odd_n ? (he + ho) * ph[3] : (he - ho) * ph[3];
    if (m == 0 || m == M - 1) high *= sqrt(2.0);
    result = is_odd_mn ? result - high : result + high;
  }
  if (edge && cancel_even) return 0.0;                    /* :128-129 */
  return result;
}

int oracle_batch_get_td_vecs(const int32_t* pixel_indices, int64_t n_pixels, const float* padded00,
                             const float* padded90, int64_t rows, const double* T0,
                             const double* Tx, int M, int n_coeffs, int K, int J,
                             const double* phase, int n_threads, float* out) {
  if (M < 1 || n_coeffs < 0 || K < 0 || J < 1) return 1;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#else
  (void)n_threads;
#endif
  const int M1 = M + 1;
  const int half = 2 * K + 1;
#pragma omp parallel for schedule(static)
  for (int64_t p = 0; p < n_pixels; ++p) {               /* :166-198 */
    const int64_t idx = pixel_indices[p];
    const int64_t n = idx / M1;
    const int m = (int)(idx % M1);
    for (int ki = 0; ki < half; ++ki) {
      const int dT = ki - K;
      const int shift = dT >= 0 ? dT / J : -((-dT) / J);  /* C-style truncation, :176-180 */
      const int sub = dT - shift * J;
      const int64_t ne = n - shift;
      double a00, a90;
      if (shift % 2 != 0) {
        if ((n + m) % 2 != 0) {
          a00 = -pixel_amplitude(ne, m, sub, padded90, rows, T0, Tx, M, n_coeffs, J, 1, phase);
          a90 = pixel_amplitude(ne, m, sub, padded00, rows, T0, Tx, M, n_coeffs, J, 0, phase);
        } else {
          a00 = pixel_amplitude(ne, m, sub, padded90, rows, T0, Tx, M, n_coeffs, J, 1, phase);
          a90 = -pixel_amplitude(ne, m, sub, padded00, rows, T0, Tx, M, n_coeffs, J, 0, phase);
        }
      } else {
        a00 = pixel_amplitude(ne, m, sub, padded00, rows, T0, Tx, M, n_coeffs, J, 0, phase);
        a90 = pixel_amplitude(ne, m, sub, padded90, rows, T0, Tx, M, n_coeffs, J, 1, phase);
      }
      out[p * 2 * half + ki] = (float)a00;
      out[p * 2 * half + half + ki] = (float)a90;
    }
  }
  return 0;
}
