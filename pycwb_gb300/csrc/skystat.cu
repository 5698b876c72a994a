// Statistics at the sky maximum for GB300 (sm_103a): the reference's
// compute_statistics_at_sky_position (pycwb/modules/likelihoodWP/
// sky_statistics.py:94-262 with the packet operations of packet_ops.py) for
// every cluster of a lag in one launch.
//
// One CTA per cluster, at the cluster's direction l (its sky maximum):
//   1. every thread takes pixels: delayed data, DPF frame, energy mask, GW
//      projection, orthogonalisation and coherent statistics of the pixel
//      (sky_stat.py:74-89, 157-189, 264-288, 357-405; dpf.py:396-446), all
//      float32 operations rounded separately as the reference's;
//   2. thread 0 sums the data and signal packets over the pixels in pixel
//      order (avx_packet_ps, packet_ops.py:659-753) and derives their
//      rotations and amplitudes;
//   3. pixels again: packet amplitudes; xtalk-corrected norms of the data
//      packet (packet_norm_numpy, :814-901) in float64;
//   4. thread 0: detector norms, signal SNRs (gw_norm_numpy, :905-948), the
//      noise correction (avx_noise_ps, :93-231);
//   5. pixels: float64 packet amplitudes (avx_setAMP_ps, :234-330), null
//      packet (avx_loadNULL_ps), xtalk energies of data and null
//      (xtalk_energy_sum_numpy, :756-810);
//   6. thread 0: the event statistics (sky_statistics.py:196-262).
// Per-pixel intermediates live in the caller's workspace
// (pgw_skystat_workspace_bytes).  The reference's float64 sums use NumPy's
// pairwise order; here they run in pixel order, so float64 results agree to
// rounding.  xtalk rows out of range set PGW_ERR_BAD_SHAPE in the cluster's
// status and are skipped.

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/pycwb_gb300.h"

namespace pgw {
int fail(int code, const std::string& msg);
}

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float M(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float A(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float S(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float D(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double dM(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dA(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dS(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dD(double a, double b) { return __ddiv_rn(a, b); }

struct StatArgs {
  const float* FP;
  const float* FX;
  const int32_t* ml;
  int64_t n_sky;
  int n_delay;
  const int64_t* pix_offsets;
  const int64_t* td_offsets;
  const float* rms;
  const float* td00;
  const float* td90;
  const int64_t* sky_idx;
  const float* regulator;  // REG[1] per cluster
  float REG0, ethr;
  const float* xtalk;      // rows of 8: neighbour index, 3 unused, 4 coefficients
  int64_t n_xtalk;
  const int64_t* xtalk_lookup;  // per pixel [start, end) rows
  int xgb;
  float* wf;               // float workspace
  double* wd;              // double workspace
  pgw_skystat_result* out;
};

// float workspace per pixel (stride in floats, I detectors)
template <int I> struct FW {
  static constexpr int v0 = 0, v9 = I, s = 2 * I, Sg = 3 * I, f = 4 * I, F = 5 * I, pd = 6 * I,
                       pD = 7 * I, ps = 8 * I, pS = 9 * I, fp = 10 * I, fx = fp + 1, et = fp + 2,
                       msk = fp + 3, ec = fp + 4, gn = fp + 5, ee = fp + 6, EE = fp + 7,
                       pr0 = fp + 8, pa0 = fp + 9, pr9 = fp + 10, pa9 = fp + 11, stride = fp + 12;
};
// double workspace per pixel
template <int I> struct DW {
  static constexpr int tcl = 0, qn = I, pdd = 2 * I, pDd = 3 * I, psd = 4 * I, pSd = 5 * I,
                       gdat = 6 * I, gnul = 7 * I, rnx = 8 * I, stride = 8 * I + 1;
};

// Sum over the CTA of N float64 values per thread; every thread gets the
// totals.  The order differs from a pixel-order loop, so results agree with
// it to float64 rounding.
template <int N>
__device__ __forceinline__ void block_sum(double (&v)[N], double (*red)[kThreads / 32]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; ++k) red[k][w] = v[k];
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; ++k) {
    double t = 0.0;
    for (int u = 0; u < kThreads / 32; ++u) t += red[k][u];
    v[k] = t;
  }
  __syncthreads();
}

template <int I>
__device__ void xtalk_terms(const StatArgs& a, int64_t gp, int64_t P, const double* pv,
                            const double* qv, int pstride, double (&x0)[I], double (&x1)[I],
                            double (&x2)[I], double (&x3)[I], int& bad) {
  for (int i = 0; i < I; ++i) x0[i] = x1[i] = x2[i] = x3[i] = 0.0;
  const int64_t r0 = a.xtalk_lookup[2 * gp], r1 = a.xtalk_lookup[2 * gp + 1];
  if (r0 < 0 || r1 < r0 || r1 > a.n_xtalk) { bad = 1; return; }
  for (int64_t r = r0; r < r1; ++r) {
    const float* row = a.xtalk + 8 * r;
    const int64_t k = static_cast<int64_t>(row[0]);
    if (k < 0 || k >= P) { bad = 1; continue; }
    const double c0 = row[4], c1 = row[5], c2 = row[6], c3 = row[7];
    for (int i = 0; i < I; ++i) {
      const double p = pv[k * pstride + i], q = qv[k * pstride + i];
      x0[i] = dA(x0[i], dM(p, c0));
      x1[i] = dA(x1[i], dM(p, c1));
      x2[i] = dA(x2[i], dM(q, c2));
      x3[i] = dA(x3[i], dM(q, c3));
    }
  }
}

template <int I>
__global__ void __launch_bounds__(kThreads) skystat_kernel(StatArgs a) {
  using W = FW<I>;
  using Q = DW<I>;
  const int c = blockIdx.x;
  const int64_t p0 = a.pix_offsets[c];
  const int64_t P = a.pix_offsets[c + 1] - p0;
  const int64_t l = a.sky_idx[c];
  __shared__ int s_row[8];
  __shared__ int s_bad;
  __shared__ float s_pk[4][8];      // data si, co, 1/a, 1/A
  __shared__ float s_sk[4][8];      // signal si, co, 1/a, 1/A
  __shared__ float s_aA[2][8];      // a + A of data and signal
  __shared__ int s_go;
  if (threadIdx.x == 0) {
    s_bad = 0;
    s_go = (P > 0 && l >= 0 && l < a.n_sky) ? 1 : 0;
    for (int i = 0; i < I && s_go; ++i) {
      const int d = a.ml[i * a.n_sky + l] + a.n_delay / 2;
      if (d < 0 || d >= a.n_delay) s_go = 0;
      s_row[i] = d;
    }
    if (!s_go) {
      pgw_skystat_result r{};
      r.status = (P > 0) ? PGW_ERR_DELAY_RANGE : 0;
      r.n_pix = static_cast<int32_t>(P);
      a.out[c] = r;
    }
  }
  __syncthreads();
  if (!s_go) return;
  float* wf = a.wf + p0 * W::stride;
  double* wd = a.wd + p0 * Q::stride;
  const int64_t td0 = a.td_offsets[c];
  float Fp[I], Fx[I];
  for (int i = 0; i < I; ++i) { Fp[i] = a.FP[l * I + i]; Fx[i] = a.FX[l * I + i]; }
  const float rr = a.REG0, RR = a.regulator[c];

  // 1. per pixel (sky_statistics.py:94-133)
  for (int64_t j = threadIdx.x; j < P; j += blockDim.x) {
    float* w = wf + j * W::stride;
    float v0[I], v9[I];
    for (int i = 0; i < I; ++i) {
      v0[i] = a.td00[td0 + (static_cast<int64_t>(s_row[i]) * I + i) * P + j];
      v9[i] = a.td90[td0 + (static_cast<int64_t>(s_row[i]) * I + i) * P + j];
    }
    // dpf.py:396-446
    const float* r = a.rms + (p0 + j) * I;
    float f[I], F[I], ff = 0.f, FF = 0.f, fF = 0.f;
    for (int i = 0; i < I; ++i) { f[i] = M(r[i], Fp[i]); F[i] = M(r[i], Fx[i]); }
    for (int i = 0; i < I; ++i) { ff = A(ff, M(f[i], f[i])); FF = A(FF, M(F[i], F[i])); fF = A(fF, M(F[i], f[i])); }
    const float si2 = M(2.0f, fF), co2 = S(ff, FF), AP = A(ff, FF);
    const float nn = __fsqrt_rn(A(M(co2, co2), M(si2, si2)));
    const float cc = D(co2, A(nn, 1e-9f));
    const float fp = D(A(AP, nn), 2.0f);
    const float si = __fsqrt_rn(D(S(1.0f, cc), 2.0f));
    const float cq = __fsqrt_rn(D(A(1.0f, cc), 2.0f));
    const float co = si2 > 0.0f ? cq : -cq;
    for (int i = 0; i < I; ++i) {
      const float x = A(M(f[i], co), M(F[i], si));
      const float y = S(M(F[i], co), M(f[i], si));
      f[i] = x; F[i] = y;
    }
    float fFn = 0.f;
    for (int i = 0; i < I; ++i) fFn = A(fFn, M(f[i], F[i]));
    fFn = D(fFn, A(fp, 1e-9f));
    float fx = 0.f, ni = 0.f;
    for (int i = 0; i < I; ++i) {
      F[i] = S(F[i], M(f[i], fFn));
      fx = A(fx, M(F[i], F[i]));
      const float f2 = M(f[i], f[i]);
      ni = A(ni, M(f2, f2));
    }
    ni = D(ni, A(M(fp, fp), 1e-9f));
    // load_data_from_td
    float aa = 0.f, AA = 0.f;
    for (int i = 0; i < I; ++i) { aa = A(aa, M(v0[i], v0[i])); AA = A(AA, M(v9[i], v9[i])); }
    const float e = A(A(aa, AA), 1e-12f);
    const int mk = e > a.ethr ? 1 : 0;
    const float et = mk ? e : 0.0f;
    // avx_GW_ps
    float xp = 0.f, XP = 0.f, xx = 0.f, XX = 0.f;
    for (int i = 0; i < I; ++i) {
      xp = A(xp, M(v0[i], f[i])); XP = A(XP, M(v9[i], f[i]));
      xx = A(xx, M(v0[i], F[i])); XX = A(XX, M(v9[i], F[i]));
    }
    float t = M(ni, A(M(xp, xp), M(XP, XP)));
    t = D(t, A(et, 1e-9f));
    float g = S(M(__fsqrt_rn(t), rr), fp);
    g = g > 0.0f ? g : 0.0f;
    const double fd = dD(static_cast<double>(mk), static_cast<double>(A(A(fp, g), 1e-9f)));
    double h = dM(static_cast<double>(xp), fd), Hh = dM(static_cast<double>(XP), fd);
    h = dA(dM(h, h), dM(Hh, Hh));
    const float H2 = A(M(xx, xx), M(XX, XX));
    const double Fd = __dsqrt_rn(dD(static_cast<double>(H2), dA(h, static_cast<double>(1e-9f))));
    const float Rg = A(0.1f, D(RR, A(et, 1e-9f)));
    float G = S(M(static_cast<float>(Fd), Rg), fx);
    G = G > 0.0f ? G : 0.0f;
    const double Gd = dD(static_cast<double>(mk), static_cast<double>(A(A(fx, G), 1e-9f)));
    const float au = static_cast<float>(dM(static_cast<double>(xp), fd));
    const float AU = static_cast<float>(dM(static_cast<double>(XP), fd));
    const float av = static_cast<float>(dM(static_cast<double>(xx), Gd));
    const float AV = static_cast<float>(dM(static_cast<double>(XX), Gd));
    const double a_ = dA(dM(fd, static_cast<double>(fp)), dM(Gd, static_cast<double>(fx)));
    const float msk = static_cast<float>(dS(dA(a_, static_cast<double>(mk)), 1.0));
    float s[I], Sg[I];
    for (int i = 0; i < I; ++i) {
      s[i] = A(M(f[i], au), M(F[i], av));
      Sg[i] = A(M(f[i], AU), M(F[i], AV));
    }
    // avx_ort_ps
    float a2 = 0.f, A2 = 0.f, aA = 0.f;
    for (int i = 0; i < I; ++i) { a2 = A(a2, M(s[i], s[i])); A2 = A(A2, M(Sg[i], Sg[i])); aA = A(aA, M(s[i], Sg[i])); }
    float osi = M(aA, 2.0f), oco = S(a2, A2);
    const float onn = __fsqrt_rn(A(M(oco, oco), M(osi, osi)));
    {   // the per-pixel plus / cross energies of the signal (sky_stat.py:279-281)
      const float eo = A(A(a2, A2), 1e-21f);
      w[W::ee] = D(A(eo, onn), 2.0f);
      w[W::EE] = D(S(eo, onn), 2.0f);
    }
    const float occ = D(oco, A(onn, 1e-21f));
    const float sg = osi > 0.0f ? 1.0f : -1.0f;
    osi = __fsqrt_rn(D(S(1.0f, occ), 2.0f));
    oco = M(__fsqrt_rn(D(A(1.0f, occ), 2.0f)), sg);
    // avx_stat_ps
    float cs = 0.f, Cs = 0.f, ss = 0.f, SS = 0.f, r0 = 0.f, R0 = 0.f, xs = 0.f, XS = 0.f;
    for (int i = 0; i < I; ++i) {
      const float s_ = A(M(s[i], oco), M(Sg[i], osi));
      const float x_ = A(M(v0[i], oco), M(v9[i], osi));
      const float S_ = S(M(Sg[i], oco), M(s[i], osi));
      const float X_ = S(M(v9[i], oco), M(v0[i], osi));
      const float p = M(s_, x_), q = M(S_, X_);
      xs = A(xs, p); XS = A(XS, q);
      cs = A(cs, M(p, p)); Cs = A(Cs, M(q, q));
      ss = A(ss, M(s_, s_)); SS = A(SS, M(S_, S_));
      const float q0 = S(s[i], v0[i]), q9 = S(Sg[i], v9[i]);
      r0 = A(r0, M(q0, q0)); R0 = A(R0, M(q9, q9));
    }
    const int mks = msk >= 0.0f ? 1 : 0;
    cs = D(cs, A(M(xs, xs), 1e-9f));
    Cs = D(Cs, A(M(XS, XS), 1e-9f));
    ss = M(ss, S(1.0f, cs));
    SS = M(SS, S(1.0f, Cs));
    for (int i = 0; i < I; ++i) {
      w[W::v0 + i] = v0[i]; w[W::v9 + i] = v9[i];
      w[W::s + i] = s[i]; w[W::Sg + i] = Sg[i];
      w[W::f + i] = f[i]; w[W::F + i] = F[i];
    }
    w[W::fp] = fp; w[W::fx] = fx; w[W::et] = et; w[W::msk] = msk;
    w[W::ec] = M(static_cast<float>(mks), A(ss, SS));
    w[W::gn] = M(static_cast<float>(mks * 2.0), msk);
    // the network-plane radius and angle of both quadratures (avx_pol_ps,
    // packet_ops.py:564-655), float64 as the reference's sums
    {
      const double mkp = msk > 0.0f ? 1.0 : 0.0;
      double xp = 0.0, XP = 0.0, xx = 0.0, XX = 0.0;
      for (int i = 0; i < I; ++i) {
        const double p0v = static_cast<double>(v0[i]) * mkp, p9v = static_cast<double>(v9[i]) * mkp;
        xp += static_cast<double>(f[i]) * p0v;
        XP += static_cast<double>(f[i]) * p9v;
        xx += static_cast<double>(F[i]) * p0v;
        XX += static_cast<double>(F[i]) * p9v;
      }
      const double o = 1e-9, fpd = fp, fxd = fx;
      const double sfp = sqrt(fpd) + o, sfx = sqrt(fxd) + o;
      w[W::pr0] = static_cast<float>(sqrt(xp * xp / (fpd + o) + xx * xx / (fxd + o)));
      w[W::pa0] = static_cast<float>(atan2(xx / sfx, xp / sfp));
      w[W::pr9] = static_cast<float>(sqrt(XP * XP / (fpd + o) + XX * XX / (fxd + o)));
      w[W::pa9] = static_cast<float>(atan2(XX / sfx, XP / sfp));
    }
  }
  __syncthreads();

  // 2. packet rotations of data and signal (avx_packet_ps).  The packet sums
  // are float32 loops over the pixels in pixel order in the reference; each of
  // the 2 x I (packet, detector) loops runs on its own thread, in that order.
  __shared__ float s_E[2][8];       // per-detector packet energies (data, signal)
  if (threadIdx.x < 2 * I) {
    const int which = threadIdx.x / I, i = threadIdx.x % I;
    const int o0 = which == 0 ? W::v0 : W::s, o9 = which == 0 ? W::v9 : W::Sg;
    float (*k)[8] = which == 0 ? s_pk : s_sk;
    float aa = 0.f, AA = 0.f, aA = 0.f;
    for (int64_t j = 0; j < P; ++j) {
      const float* w = wf + j * W::stride;
      const float m = w[W::msk] > 0.0f ? 1.0f : 0.0f;
      const float x = w[o0 + i], y = w[o9 + i];
      aa = A(aa, M(m, M(x, x)));
      AA = A(AA, M(m, M(y, y)));
      aA = A(aA, M(m, M(x, y)));
    }
    const float s2 = M(2.0f, aA), c2 = S(aa, AA);
    const float x = A(A(aa, AA), 1e-9f);
    // the norm is a float64 (Python) value; float32 operands round it first
    const double nn = __dsqrt_rn(static_cast<double>(A(M(c2, c2), M(s2, s2))));
    const float nnf = static_cast<float>(nn);
    const float av = static_cast<float>(__dsqrt_rn(static_cast<double>(D(A(x, nnf), 2.0f))));
    const float Av = static_cast<float>(
        __dsqrt_rn(static_cast<double>(fabsf(D(S(x, nnf), 2.0f)))));
    const float cc = D(c2, static_cast<float>(dA(nn, 1e-9)));
    const float sgn = s2 > 0.0f ? 1.0f : -1.0f;
    k[0][i] = static_cast<float>(__dsqrt_rn(static_cast<double>(D(S(1.0f, cc), 2.0f))));
    k[1][i] = M(static_cast<float>(__dsqrt_rn(static_cast<double>(D(A(1.0f, cc), 2.0f)))), sgn);
    k[2][i] = D(1.0f, A(av, 1e-9f));
    k[3][i] = D(1.0f, A(Av, 1e-9f));
    const float sum = A(av, Av);
    s_aA[which][i] = sum;
    s_E[which][i] = D(M(sum, sum), 2.0f);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int which = 0; which < 2; ++which) {
      float Ep = 0.f;
      for (int i = 0; i < I; ++i) Ep = A(Ep, s_E[which][i]);
      if (which == 0) a.out[c].Eo = D(Ep, 2.0f);
      else a.out[c].Lo = D(Ep, 2.0f);
    }
  }
  __syncthreads();

  // 3. packet amplitudes (float32) and the data packet's xtalk norms
  for (int64_t j = threadIdx.x; j < P; j += blockDim.x) {
    float* w = wf + j * W::stride;
    const float m = w[W::msk] > 0.0f ? 1.0f : 0.0f;
    for (int i = 0; i < I; ++i) {
      const float x = w[W::v0 + i], y = w[W::v9 + i];
      const float pa = A(M(x, s_pk[1][i]), M(y, s_pk[0][i]));
      const float pA = S(M(y, s_pk[1][i]), M(x, s_pk[0][i]));
      w[W::pd + i] = M(M(m, pa), s_pk[2][i]);
      w[W::pD + i] = M(M(m, pA), s_pk[3][i]);
      const float u = w[W::s + i], v = w[W::Sg + i];
      const float sa = A(M(u, s_sk[1][i]), M(v, s_sk[0][i]));
      const float sA = S(M(v, s_sk[1][i]), M(u, s_sk[0][i]));
      w[W::ps + i] = M(M(m, sa), s_sk[2][i]);
      w[W::pS + i] = M(M(m, sA), s_sk[3][i]);
      double* d = wd + j * Q::stride;
      d[Q::pdd + i] = w[W::pd + i];
      d[Q::pDd + i] = w[W::pD + i];
    }
  }
  __syncthreads();
  for (int64_t j = threadIdx.x; j < P; j += blockDim.x) {
    const float* w = wf + j * W::stride;
    double* d = wd + j * Q::stride;
    for (int i = 0; i < I; ++i) { d[Q::tcl + i] = 0.0; d[Q::qn + i] = 0.0; }
    d[Q::rnx] = 0.0;
    if (!(w[W::msk] > 0.0f)) continue;
    double x0[I], x1[I], x2[I], x3[I];
    int bad = 0;
    xtalk_terms<I>(a, p0 + j, P, wd + Q::pdd, wd + Q::pDd, Q::stride, x0, x1, x2, x3, bad);
    if (bad) atomicOr(&s_bad, 1);
    double rn = 0.0;
    for (int i = 0; i < I; ++i) {
      const double pi = d[Q::pdd + i], qi = d[Q::pDd + i];
      double t = dA(dA(dA(dM(x0[i], pi), dM(x1[i], qi)), dM(x2[i], pi)), dM(x3[i], qi));
      t = t < 0.0 ? 0.0 : t;
      d[Q::tcl + i] = t;
      const double e = dD(dA(dM(pi, pi), dM(qi, qi)), dA(t, 1e-12));
      d[Q::qn + i] = e >= 1.0 ? 0.0 : e;
      const double u = dA(x0[i], x2[i]), v = dA(x1[i], x3[i]);
      rn = dA(rn, dA(dM(u, u), dM(v, v)));
    }
    d[Q::rnx] = rn;
  }
  __syncthreads();

  // 4. detector norms, signal SNR, noise correction: per-pixel terms on every
  // thread, float64 sums as block reductions
  __shared__ double s_red[16][kThreads / 32];
  __shared__ double s_norm[8];
  __shared__ double s_sc[8];   // GN, EC, SC, RC, NC, NS, EH, ES
  {
    double v[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = 0.0;
    for (int64_t j = threadIdx.x; j < P; j += blockDim.x) {
      float* w = wf + j * W::stride;
      const double* d = wd + j * Q::stride;
#pragma unroll
      for (int i = 0; i < I; ++i) v[8 + i] = dA(v[8 + i], d[Q::tcl + i]);
      const float ec = w[W::ec];
      double ns = 0.0, nx = 0.0;
      for (int i = 0; i < I; ++i) {
        nx = dA(nx, d[Q::qn + i]);
        ns = dA(ns, ec > 0.0f ? d[Q::qn + i] : 0.0);
      }
      ns = dD(ns, static_cast<double>(I));
      nx = dD(nx, static_cast<double>(I));
      const double mk = w[W::msk] > 0.0f ? 1.0 : 0.0;
      const double core = dM(mk, nx > 0.0 ? 1.0 : 0.0);
      v[1] = dA(v[1], dM(core, ec));                     // EC
      v[4] = dA(v[4], core);                             // NC
      v[7] = dA(v[7], dM(dS(mk, core), d[Q::rnx]));      // ES
      const double gn = w[W::gn];
      double rc = gn < 2.0 ? 1.0 : 0.0;
      rc = dA(rc, dM(dM(gn, dS(1.0, rc)), 0.5));
      rc = dD(static_cast<double>(ec), dA(rc, 1e-9));
      const double sig = dM(mk, ns > 0.0 ? 1.0 : 0.0);
      const float gnew = static_cast<float>(dM(dM(mk, gn), nx));
      w[W::gn] = gnew;
      v[2] = dA(v[2], dM(sig, ec));                      // SC
      v[3] = dA(v[3], dM(sig, rc));                      // RC
      v[0] = dA(v[0], dM(sig, static_cast<double>(gnew)));  // GN
      v[5] = dA(v[5], sig);                              // NS
      v[6] = dA(v[6], dM(dS(mk, sig), static_cast<double>(w[W::et])));  // EH
    }
    block_sum<16>(v, s_red);
    if (threadIdx.x == 0) {
      for (int i = 0; i < I; ++i) s_norm[i] = v[8 + i] < 2.0 ? 2.0 : v[8 + i];
      for (int i = 0; i < PGW_MAX_IFO; ++i)   // gw_norm_numpy: 2 E_signal / data norm
        a.out[c].S_snr[i] = i < I ? static_cast<float>(
            dD(static_cast<double>(M(s_E[1][i], 2.0f)), s_norm[i])) : 0.0f;
      for (int k = 0; k < 8; ++k) s_sc[k] = v[k];
    }
  }
  __syncthreads();

  // 5. float64 packet amplitudes, null packet, xtalk energies
  for (int64_t j = threadIdx.x; j < P; j += blockDim.x) {
    const float* w = wf + j * W::stride;
    double* d = wd + j * Q::stride;
    const float mk = w[W::msk] > 0.0f ? 0.5f : 0.0f;
    const float ec = w[W::ec];
    for (int i = 0; i < I; ++i) {
      const double qn = d[Q::qn + i];
      const double pn = ec > 0.0f ? qn : 0.0;
      const double nd = dM(static_cast<double>(M(s_aA[0][i], mk)), qn);
      const double ns = dM(static_cast<double>(M(s_aA[1][i], mk)), pn);
      const float x = w[W::pd + i], y = w[W::pD + i];
      d[Q::psd + i] = dM(ns, static_cast<double>(S(M(w[W::ps + i], s_sk[1][i]), M(w[W::pS + i], s_sk[0][i]))));
      d[Q::pSd + i] = dM(ns, static_cast<double>(A(M(w[W::pS + i], s_sk[1][i]), M(w[W::ps + i], s_sk[0][i]))));
      d[Q::pdd + i] = dM(nd, static_cast<double>(S(M(x, s_pk[1][i]), M(y, s_pk[0][i]))));
      d[Q::pDd + i] = dM(nd, static_cast<double>(A(M(y, s_pk[1][i]), M(x, s_pk[0][i]))));
    }
  }
  __syncthreads();
  for (int64_t j = threadIdx.x; j < P; j += blockDim.x) {
    // null packet amplitudes, kept in the float workspace slots ps/pS (float32)
    float* w = wf + j * W::stride;
    const double* d = wd + j * Q::stride;
    for (int i = 0; i < I; ++i) {
      w[W::ps + i] = S(static_cast<float>(d[Q::pdd + i]), static_cast<float>(d[Q::psd + i]));
      w[W::pS + i] = S(static_cast<float>(d[Q::pDd + i]), static_cast<float>(d[Q::pSd + i]));
    }
  }
  __syncthreads();
  for (int64_t j = threadIdx.x; j < P; j += blockDim.x) {
    const float* w = wf + j * W::stride;
    double* d = wd + j * Q::stride;
    for (int i = 0; i < I; ++i) { d[Q::gdat + i] = 0.0; d[Q::gnul + i] = 0.0; }
    if (!(w[W::msk] > 0.0f)) continue;
    int bad = 0;
    double x0[I], x1[I], x2[I], x3[I];
    xtalk_terms<I>(a, p0 + j, P, wd + Q::pdd, wd + Q::pDd, Q::stride, x0, x1, x2, x3, bad);
    for (int i = 0; i < I; ++i) {
      const double pi = d[Q::pdd + i], qi = d[Q::pDd + i];
      const double t = dA(dA(dA(dM(x0[i], pi), dM(x1[i], qi)), dM(x2[i], pi)), dM(x3[i], qi));
      d[Q::gdat + i] = t > 0.0 ? t : 0.0;
    }
    // the null packet's float32 amplitudes, read through a float64 view of the row
    for (int i = 0; i < I; ++i) x0[i] = x1[i] = x2[i] = x3[i] = 0.0;
    const int64_t r0 = a.xtalk_lookup[2 * (p0 + j)], r1 = a.xtalk_lookup[2 * (p0 + j) + 1];
    if (r0 >= 0 && r1 >= r0 && r1 <= a.n_xtalk) {
      for (int64_t r = r0; r < r1; ++r) {
        const float* row = a.xtalk + 8 * r;
        const int64_t k = static_cast<int64_t>(row[0]);
        if (k < 0 || k >= P) continue;
        const float* wk = wf + k * W::stride;
        for (int i = 0; i < I; ++i) {
          const double p = wk[W::ps + i], q = wk[W::pS + i];
          x0[i] = dA(x0[i], dM(p, static_cast<double>(row[4])));
          x1[i] = dA(x1[i], dM(p, static_cast<double>(row[5])));
          x2[i] = dA(x2[i], dM(q, static_cast<double>(row[6])));
          x3[i] = dA(x3[i], dM(q, static_cast<double>(row[7])));
        }
      }
    }
    for (int i = 0; i < I; ++i) {
      const double pi = w[W::ps + i], qi = w[W::pS + i];
      const double t = dA(dA(dA(dM(x0[i], pi), dM(x1[i], qi)), dM(x2[i], pi)), dM(x3[i], qi));
      d[Q::gnul + i] = t > 0.0 ? t : 0.0;
    }
  }
  __syncthreads();

  // 6. event statistics (sky_statistics.py:196-262): the per-detector sums of
  // the xtalk energies and the effective pixel count as block reductions
  double v6[17];
#pragma unroll
  for (int k = 0; k < 17; ++k) v6[k] = 0.0;
  for (int64_t j = threadIdx.x; j < P; j += blockDim.x) {
    const float* w = wf + j * W::stride;
    const double* d = wd + j * Q::stride;
    double q = 0.0;
#pragma unroll
    for (int i = 0; i < I; ++i) {
      v6[i] = dA(v6[i], d[Q::gdat + i]);
      v6[8 + i] = dA(v6[8 + i], d[Q::gnul + i]);
      q = dA(q, d[Q::qn + i]);
    }
    v6[16] = dA(v6[16], dM(q, w[W::msk] > 0.0f ? 0.5 : 0.0));
  }
  {
    double lo[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) lo[k] = v6[k];
    block_sum<16>(lo, s_red);
#pragma unroll
    for (int k = 0; k < 16; ++k) v6[k] = lo[k];
    double one[1] = {v6[16]};
    block_sum<1>(one, s_red);
    v6[16] = one[0];
  }
  if (threadIdx.x == 0) {
    double Em = 0.0, Np = 0.0;
    for (int i = 0; i < I; ++i) {
      Em = dA(Em, v6[i]);
      Np = dA(Np, v6[8 + i]);
    }
    const double Npix = v6[16];
    const double Neff = dS(dD(dM(Npix, 4.0), static_cast<double>(I)), 1.0);
    const double GN = s_sc[0], EC = s_sc[1], SC = s_sc[2], RC = s_sc[3];
    const double EH = dD(s_sc[6], 2.0), ES = dD(s_sc[7], 2.0);
    const double Rc = dD(RC, dA(SC, 0.01));
    double Ec = EC, Dc = dS(SC, EC);
    const float Eo = a.out[c].Eo;
    // norm: a float32 ratio when Em > 0 (NumPy scalar rules) and Ec, Dc with
    // it; the int 1 or the float 1e9 otherwise, Ec and Dc staying float64
    double norm;
    bool f32 = false;
    if (Em > 0.0) {
      const float nf = D(S(Eo, static_cast<float>(EH)), static_cast<float>(Em));
      if (nf < 1.0f) {
        norm = 1.0;
      } else {
        norm = nf;
        f32 = true;
        Ec = D(static_cast<float>(Ec), nf);
        Dc = D(static_cast<float>(Dc), nf);
      }
    } else {
      norm = 1.e9;
      Ec = dD(Ec, norm);
      Dc = dD(Dc, norm);
    }
    const double Lm = dS(dS(Em, Np), GN);
    const double ch = dD(dA(Np, GN), dM(Neff, static_cast<double>(I)));
    const double cc = ch > 1.0 ? ch : 1.0;
    // sqrt(Ec Rc / 2): float32 arithmetic when Ec is a float32
    const double r2 = f32 ? static_cast<double>(__fsqrt_rn(D(M(static_cast<float>(Ec),
                                                               static_cast<float>(Rc)), 2.0f)))
                          : __dsqrt_rn(dD(dM(Ec, Rc), 2.0));
    double rho = 0.0, xrho = 0.0;
    if (!a.xgb) {
      rho = Ec > 0.0 ? r2 : 0.0;
    } else {
      const double den = dA(1.0, dM(ch, dS(ch > 1.0 ? ch : 1.0, 1.0)));
      rho = Ec > 0.0 ? (f32 ? static_cast<double>(__fsqrt_rn(D(static_cast<float>(Ec),
                                                               static_cast<float>(den))))
                            : __dsqrt_rn(dD(Ec, den)))
                     : 0.0;
      xrho = Ec > 0.0 ? r2 : 0.0;
    }
    pgw_skystat_result& r = a.out[c];
    r.N_pix_effective = Neff;
    r.Gn = static_cast<float>(GN); r.Ec = static_cast<float>(Ec); r.Dc = static_cast<float>(Dc);
    r.Rc = static_cast<float>(Rc); r.Eh = static_cast<float>(EH); r.Es = static_cast<float>(ES);
    r.Np = static_cast<float>(Np); r.Em = static_cast<float>(Em); r.Lm = static_cast<float>(Lm);
    r.norm = static_cast<float>(norm); r.cc = static_cast<float>(cc);
    r.rho = static_cast<float>(rho); r.xrho = static_cast<float>(xrho);
    r.status = s_bad ? PGW_ERR_BAD_SHAPE : 0;
    r.n_pix = static_cast<int32_t>(P);
    r.reserved = 0;
  }
}

template <int I>
cudaError_t launch(const StatArgs& a, int n_clusters, cudaStream_t s) {
  skystat_kernel<I><<<n_clusters, kThreads, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

extern "C" size_t pgw_skystat_workspace_bytes(int n_ifo, int64_t total_pix) {
  if (n_ifo < 1 || n_ifo > PGW_MAX_IFO || total_pix < 0) return 0;
  const size_t fl = static_cast<size_t>(10 * n_ifo + 12) * 4;
  const size_t db = static_cast<size_t>(8 * n_ifo + 1) * 8;
  return 256 + static_cast<size_t>(total_pix) * (fl + db) + 256;
}

extern "C" int pgw_skystat_batched(int n_ifo, int n_clusters, const int64_t* pix_offsets,
                                   const int64_t* td_offsets, int64_t total_pix, int64_t n_sky,
                                   const float* FP, const float* FX, const float* rms_all,
                                   const float* td00_all, const float* td90_all, int n_delay,
                                   const int32_t* ml, const int64_t* sky_idx,
                                   const float* regulators, float REG0,
                                   float network_energy_threshold, const float* xtalk,
                                   int64_t n_xtalk, const int64_t* xtalk_lookup, int xgb_rho_mode,
                                   void* ws, size_t ws_bytes, pgw_skystat_result* out,
                                   void* stream) {
  if (n_ifo < 2 || n_ifo > PGW_MAX_IFO) return pgw::fail(PGW_ERR_BAD_SHAPE, "n_ifo must be in [2, 8]");
  if (n_clusters < 1 || n_clusters > 0x7fffffff || total_pix < 0 || n_sky < 1 || n_delay < 1 ||
      (n_delay & 1) == 0 || n_xtalk < 0)
    return pgw::fail(PGW_ERR_BAD_SHAPE, "bad cluster, sky, delay or xtalk sizes");
  if (!pix_offsets || !td_offsets || !FP || !FX || !ml || !sky_idx || !regulators || !out || !ws ||
      (total_pix > 0 && (!rms_all || !td00_all || !td90_all || !xtalk_lookup)) ||
      (n_xtalk > 0 && !xtalk))
    return pgw::fail(PGW_ERR_BAD_ARGUMENT, "NULL device pointer");
  const size_t need = pgw_skystat_workspace_bytes(n_ifo, total_pix);
  if (ws_bytes < need) return pgw::fail(PGW_ERR_WORKSPACE, "workspace smaller than pgw_skystat_workspace_bytes");
  char* base = static_cast<char*>(ws);
  const uintptr_t al = (reinterpret_cast<uintptr_t>(base) + 255) & ~static_cast<uintptr_t>(255);
  char* b = reinterpret_cast<char*>(al);
  StatArgs a{};
  a.FP = FP; a.FX = FX; a.ml = ml; a.n_sky = n_sky; a.n_delay = n_delay;
  a.pix_offsets = pix_offsets; a.td_offsets = td_offsets; a.rms = rms_all;
  a.td00 = td00_all; a.td90 = td90_all; a.sky_idx = sky_idx; a.regulator = regulators;
  a.REG0 = REG0; a.ethr = network_energy_threshold; a.xtalk = xtalk; a.n_xtalk = n_xtalk;
  a.xtalk_lookup = xtalk_lookup; a.xgb = xgb_rho_mode ? 1 : 0; a.out = out;
  a.wd = reinterpret_cast<double*>(b);
  a.wf = reinterpret_cast<float*>(b + static_cast<size_t>(8 * n_ifo + 1) * 8 *
                                          static_cast<size_t>(total_pix));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  switch (n_ifo) {
    case 2: e = launch<2>(a, n_clusters, s); break;
    case 3: e = launch<3>(a, n_clusters, s); break;
    case 4: e = launch<4>(a, n_clusters, s); break;
    case 5: e = launch<5>(a, n_clusters, s); break;
    case 6: e = launch<6>(a, n_clusters, s); break;
    case 7: e = launch<7>(a, n_clusters, s); break;
    default: e = launch<8>(a, n_clusters, s); break;
  }
  if (e != cudaSuccess) return pgw::fail(PGW_ERR_CUDA, std::string("skystat_kernel: ") + cudaGetErrorString(e));
  return PGW_OK;
}

// ----------------------------------------------------------------------------
// The per-pixel arrays of the reference's SkyStatistics, from the workspace of
// the last pgw_skystat_batched call (sky_statistics.py:264-292).
// ----------------------------------------------------------------------------
namespace {

template <int I>
__global__ void skystat_pixels_kernel(int64_t total_pix, const float* __restrict__ wf,
                                      const double* __restrict__ wd, float* __restrict__ out32,
                                      double* __restrict__ out64) {
  using W = FW<I>;
  using Q = DW<I>;
  const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= total_pix) return;
  const float* w = wf + p * W::stride;
  const double* d = wd + p * Q::stride;
  constexpr int NF = 9 + 4 * I;
  float* o = out32 + p * NF;
  o[0] = w[W::ee];
  o[1] = w[W::EE];
  o[2] = w[W::msk];
  o[3] = w[W::gn];
  o[4] = w[W::ec];
  o[5] = w[W::pr0];
  o[6] = w[W::pa0];
  o[7] = w[W::pr9];
  o[8] = w[W::pa9];
  for (int i = 0; i < I; ++i) {
    o[9 + i] = w[W::ps + i];           // null packet, 00 (the slots hold it after phase 5)
    o[9 + I + i] = w[W::pS + i];       // null packet, 90
    o[9 + 2 * I + i] = w[W::f + i];
    o[9 + 3 * I + i] = w[W::F + i];
  }
  double* o64 = out64 + p * (4 * I);
  for (int i = 0; i < I; ++i) {
    o64[i] = d[Q::pdd + i];
    o64[I + i] = d[Q::pDd + i];
    o64[2 * I + i] = d[Q::psd + i];
    o64[3 * I + i] = d[Q::pSd + i];
  }
}

}  // namespace

extern "C" int pgw_skystat_pixel_arrays(int n_ifo, int64_t total_pix, const void* ws,
                                        size_t ws_bytes, float* out32, double* out64,
                                        void* stream) {
  if (n_ifo < 2 || n_ifo > PGW_MAX_IFO || total_pix < 0)
    return pgw::fail(PGW_ERR_BAD_SHAPE, "n_ifo must be in [2, 8] and total_pix >= 0");
  if (total_pix == 0) return PGW_OK;
  if (!ws || !out32 || !out64) return pgw::fail(PGW_ERR_BAD_ARGUMENT, "NULL device pointer");
  if (ws_bytes < pgw_skystat_workspace_bytes(n_ifo, total_pix))
    return pgw::fail(PGW_ERR_WORKSPACE, "workspace smaller than pgw_skystat_workspace_bytes");
  const char* base = static_cast<const char*>(ws);
  const uintptr_t al = (reinterpret_cast<uintptr_t>(base) + 255) & ~static_cast<uintptr_t>(255);
  const char* b = reinterpret_cast<const char*>(al);
  const double* wd = reinterpret_cast<const double*>(b);
  const float* wf = reinterpret_cast<const float*>(b + static_cast<size_t>(8 * n_ifo + 1) * 8 *
                                                          static_cast<size_t>(total_pix));
  const unsigned blocks = static_cast<unsigned>((total_pix + 255) / 256);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (n_ifo) {
    case 2: skystat_pixels_kernel<2><<<blocks, 256, 0, s>>>(total_pix, wf, wd, out32, out64); break;
    case 3: skystat_pixels_kernel<3><<<blocks, 256, 0, s>>>(total_pix, wf, wd, out32, out64); break;
    case 4: skystat_pixels_kernel<4><<<blocks, 256, 0, s>>>(total_pix, wf, wd, out32, out64); break;
    case 5: skystat_pixels_kernel<5><<<blocks, 256, 0, s>>>(total_pix, wf, wd, out32, out64); break;
    case 6: skystat_pixels_kernel<6><<<blocks, 256, 0, s>>>(total_pix, wf, wd, out32, out64); break;
    case 7: skystat_pixels_kernel<7><<<blocks, 256, 0, s>>>(total_pix, wf, wd, out32, out64); break;
    default: skystat_pixels_kernel<8><<<blocks, 256, 0, s>>>(total_pix, wf, wd, out32, out64); break;
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return pgw::fail(PGW_ERR_CUDA, std::string("skystat_pixels_kernel: ") + cudaGetErrorString(e));
  return PGW_OK;
}
