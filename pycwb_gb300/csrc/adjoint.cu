// Sky statistic at continuous (theta, phi) and its gradient, for off-grid
// refinement of the sky maximum (GB300, sm_103a).
//
// The grid scan evaluates the statistic only at HEALPix directions with
// delays rounded to whole samples (pycwb/types/detector.py:1317-1321).  Here
// the direction is continuous: F+ and Fx come from each detector's response
// tensor D at gha = -phi, dec = pi/2 - theta, psi = 0 (detector.py:301-358),
// and the delay of detector i, tau_i = n(theta, phi) . b_i with b_i the
// baseline to the reference detector in TD samples, is made continuous by
// linear interpolation between the td-amplitude samples that bracket it.
// The per-pixel pipeline and the per-direction tail are the sky scan's
// (sky_stat.py:37-410, dpf.py:343-453, sky_scan.py:100-141).
//
// The derivative with respect to (theta, phi) is taken in the same pass:
// every quantity carries its two tangents (forward-mode dual numbers), the
// natural form of the adjoint when the Jacobian has one row and two columns.
// Kinks of the statistic (the energy threshold, max(., 0) regulators,
// interpolation knots) give one-sided derivatives, as any adjoint would.
//
// Arithmetic: float32 values and tangents, float32 accumulation.

#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "../../include/pycwb_gb300.h"

namespace pgw {
int fail(int code, const std::string& msg);
}

namespace {

struct D2 {  // value and d/dtheta, d/dphi
  float v, a, b;
};

__device__ __forceinline__ D2 mk(float v) { return {v, 0.f, 0.f}; }
__device__ __forceinline__ D2 operator+(D2 x, D2 y) { return {x.v + y.v, x.a + y.a, x.b + y.b}; }
__device__ __forceinline__ D2 operator-(D2 x, D2 y) { return {x.v - y.v, x.a - y.a, x.b - y.b}; }
__device__ __forceinline__ D2 operator-(D2 x) { return {-x.v, -x.a, -x.b}; }
__device__ __forceinline__ D2 operator*(D2 x, D2 y) {
  return {x.v * y.v, x.v * y.a + x.a * y.v, x.v * y.b + x.b * y.v};
}
__device__ __forceinline__ D2 operator*(D2 x, float s) { return {x.v * s, x.a * s, x.b * s}; }
__device__ __forceinline__ D2 operator*(float s, D2 x) { return x * s; }
__device__ __forceinline__ D2 operator+(D2 x, float s) { return {x.v + s, x.a, x.b}; }
__device__ __forceinline__ D2 operator+(float s, D2 x) { return {x.v + s, x.a, x.b}; }
__device__ __forceinline__ D2 operator-(D2 x, float s) { return {x.v - s, x.a, x.b}; }
__device__ __forceinline__ D2 operator-(float s, D2 x) { return {s - x.v, -x.a, -x.b}; }
__device__ __forceinline__ D2 operator/(D2 x, D2 y) {
  const float q = x.v / y.v;
  const float r = 1.0f / y.v;
  return {q, (x.a - q * y.a) * r, (x.b - q * y.b) * r};
}
__device__ __forceinline__ D2 dsqrt(D2 x) {
  const float s = sqrtf(x.v);
  const float h = s > 0.f ? 0.5f / s : 0.f;  // one-sided at 0
  return {s, x.a * h, x.b * h};
}
__device__ __forceinline__ D2 dmax0(D2 x) { return x.v > 0.f ? x : mk(0.f); }

// Rotation (cos psi, sin psi) with 2 psi = atan2(s2, c2), times sign(s2 > 0).
// Mathematically the reference's (±sqrt((1+cos2psi)/2), sqrt((1-cos2psi)/2))
// (dpf.py:419-420, sky_stat.py:283-288); everything downstream is invariant
// to the overall sign.  The half-angle square roots have derivatives that
// blow up where cos2psi -> ±1 and cancel only in exact arithmetic; the angle
// form has a smooth derivative.
__device__ __forceinline__ void drot(D2 s2, D2 c2, D2& co, D2& si) {
  const float r2 = c2.v * c2.v + s2.v * s2.v;
  const float inv = r2 > 0.f ? 0.5f / r2 : 0.f;
  const float psi = 0.5f * atan2f(s2.v, c2.v);
  const D2 ps = {psi, (c2.v * s2.a - s2.v * c2.a) * inv, (c2.v * s2.b - s2.v * c2.b) * inv};
  float sn, cs;
  sincosf(ps.v, &sn, &cs);
  const float sg = s2.v > 0.f ? 1.f : -1.f;
  co = {sg * cs, -sg * sn * ps.a, -sg * sn * ps.b};
  si = {sg * sn, sg * cs * ps.a, sg * cs * ps.b};
}
__device__ __forceinline__ D2 dabs(D2 x) { return x.v < 0.f ? -x : x; }

// per-detector geometry: response tensor (row major, 9) and baseline to the
// reference detector in TD samples (3)
constexpr int kGeom = 12;

template <int I>
struct DirInputs {
  D2 Fp[I], Fx[I], tau[I];
};

// F+, Fx and delays of direction (theta, phi); tangents d/dtheta, d/dphi.
template <int I>
__device__ void direction_inputs(float theta, float phi, const float* __restrict__ geom,
                                 DirInputs<I>& o) {
  float st, ct, sp, cp;
  sincosf(theta, &st, &ct);
  sincosf(phi, &sp, &cp);
  // gha = -phi, dec = pi/2 - theta: sin(dec) = cos(theta), cos(dec) = sin(theta)
  const D2 sgha = {-sp, 0.f, -cp};   // sin(-phi)
  const D2 cgha = {cp, 0.f, -sp};    // cos(-phi)
  const D2 sdec = {ct, -st, 0.f};
  const D2 cdec = {st, ct, 0.f};
  const D2 x[3] = {-sgha, -cgha, mk(0.f)};
  const D2 y[3] = {-(cgha * sdec), sgha * sdec, cdec};
  // unit vector n = (sin t cos p, sin t sin p, cos t)
  const D2 n[3] = {D2{st * cp, ct * cp, -st * sp}, D2{st * sp, ct * sp, st * cp},
                   D2{ct, -st, 0.f}};
#pragma unroll
  for (int i = 0; i < I; ++i) {
    const float* D = geom + i * kGeom;
    D2 dx[3], dy[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      dx[r] = x[0] * D[3 * r] + x[1] * D[3 * r + 1] + x[2] * D[3 * r + 2];
      dy[r] = y[0] * D[3 * r] + y[1] * D[3 * r + 1] + y[2] * D[3 * r + 2];
    }
    D2 fp = mk(0.f), fc = mk(0.f);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      fp = fp + x[r] * dx[r] - y[r] * dy[r];
      fc = fc + x[r] * dy[r] + y[r] * dx[r];
    }
    o.Fp[i] = fp;
    o.Fx[i] = fc;
    o.tau[i] = n[0] * geom[i * kGeom + 9] + n[1] * geom[i * kGeom + 10] +
               n[2] * geom[i * kGeom + 11];
  }
}

struct Acc {
  D2 EE, LL, Lr, EC, GN, RN;
  int Mo;
};

// One pixel of the scan pipeline in dual arithmetic (sky_stat.py:74-405).
template <int I>
__device__ void pixel_dual(const float* __restrict__ r, const D2 (&v0)[I], const D2 (&v9)[I],
                           const DirInputs<I>& d, float rr, float RR, float ethr, Acc& acc) {
  D2 e = mk(1e-12f);
#pragma unroll
  for (int i = 0; i < I; ++i) e = e + v0[i] * v0[i] + v9[i] * v9[i];
  const bool mask = e.v > ethr;
  if (!mask) return;  // contributes nothing (sky_stat.py:83-86, 166, 176, 385-393)
  const D2 et = e;
  acc.EE = acc.EE + et;
  acc.Mo += 1;
  // DPF (dpf.py:396-446)
  D2 f[I], F[I], ff = mk(0.f), FF = mk(0.f), fF = mk(0.f);
#pragma unroll
  for (int i = 0; i < I; ++i) {
    f[i] = d.Fp[i] * r[i];
    F[i] = d.Fx[i] * r[i];
    ff = ff + f[i] * f[i];
    FF = FF + F[i] * F[i];
    fF = fF + F[i] * f[i];
  }
  const D2 si2 = 2.0f * fF, co2 = ff - FF, AP = ff + FF;
  const D2 nn = dsqrt(co2 * co2 + si2 * si2);
  const D2 fp = (AP + nn) * 0.5f;
  D2 co, si;
  drot(si2, co2, co, si);
  D2 fFn = mk(0.f);
#pragma unroll
  for (int i = 0; i < I; ++i) {
    const D2 a = f[i] * co + F[i] * si;
    const D2 b = F[i] * co - f[i] * si;
    f[i] = a;
    F[i] = b;
    fFn = fFn + a * b;
  }
  fFn = fFn / (fp + 1e-9f);
  D2 fx = mk(0.f), ni = mk(0.f);
#pragma unroll
  for (int i = 0; i < I; ++i) {
    F[i] = F[i] - f[i] * fFn;
    fx = fx + F[i] * F[i];
    const D2 f2 = f[i] * f[i];
    ni = ni + f2 * f2;
  }
  ni = ni / (fp * fp + 1e-9f);
  // avx_GW_ps (sky_stat.py:157-189)
  D2 xp = mk(0.f), XP = mk(0.f), xx = mk(0.f), XX = mk(0.f);
#pragma unroll
  for (int i = 0; i < I; ++i) {
    xp = xp + v0[i] * f[i];
    XP = XP + v9[i] * f[i];
    xx = xx + v0[i] * F[i];
    XX = XX + v9[i] * F[i];
  }
  const D2 eto = et + 1e-9f;
  const D2 g = dmax0(dsqrt(ni * (xp * xp + XP * XP) / eto) * rr - fp);
  const D2 fd = mk(1.0f) / (fp + g + 1e-9f);
  D2 h = xp * fd, Hh = XP * fd;
  h = h * h + Hh * Hh;
  const D2 H2 = xx * xx + XX * XX;
  const D2 Fd = dsqrt(H2 / (h + 1e-9f));
  const D2 R = mk(0.1f) + mk(RR) / eto;
  const D2 G = dmax0(Fd * R - fx);
  const D2 Gd = mk(1.0f) / (fx + G + 1e-9f);
  const D2 au = xp * fd, AU = XP * fd, av = xx * Gd, AV = XX * Gd;
  const D2 msk = fd * fp + Gd * fx;
  D2 s[I], S[I], a2 = mk(0.f), A2 = mk(0.f), aA = mk(0.f);
#pragma unroll
  for (int i = 0; i < I; ++i) {
    s[i] = f[i] * au + F[i] * av;
    S[i] = f[i] * AU + F[i] * AV;
    a2 = a2 + s[i] * s[i];
    A2 = A2 + S[i] * S[i];
    aA = aA + s[i] * S[i];
  }
  // avx_ort_ps (sky_stat.py:264-288)
  D2 oco, osi;
  drot(aA * 2.0f, a2 - A2, oco, osi);
  // avx_stat_ps (sky_stat.py:357-405)
  D2 c = mk(0.f), C = mk(0.f), ss = mk(0.f), SS = mk(0.f), r0 = mk(0.f), R0 = mk(0.f);
  D2 xs = mk(0.f), XS = mk(0.f);
#pragma unroll
  for (int i = 0; i < I; ++i) {
    const D2 s_ = s[i] * oco + S[i] * osi;
    const D2 x_ = v0[i] * oco + v9[i] * osi;
    const D2 S_ = S[i] * oco - s[i] * osi;
    const D2 X_ = v9[i] * oco - v0[i] * osi;
    const D2 q = s_ * x_, Q = S_ * X_;
    xs = xs + q;
    XS = XS + Q;
    c = c + q * q;
    C = C + Q * Q;
    ss = ss + s_ * s_;
    SS = SS + S_ * S_;
    const D2 d0 = s[i] - v0[i], d9 = S[i] - v9[i];
    r0 = r0 + d0 * d0;
    R0 = R0 + d9 * d9;
  }
  c = c / (xs * xs + 1e-9f);
  C = C / (XS * XS + 1e-9f);
  const D2 ll = ss + SS;
  const D2 ec = ss * (1.0f - c) + SS * (1.0f - C);
  const D2 gn = msk * 2.0f;
  const D2 rn = r0 + R0;
  const D2 ccn = ec / (2.0f * dabs(ec) + (rn + gn + 1e-9f));
  acc.Lr = acc.Lr + ll * ccn;
  acc.LL = acc.LL + ll;
  acc.EC = acc.EC + ec;
  acc.GN = acc.GN + gn;
  acc.RN = acc.RN + rn;
}

// Per-query inputs of one cluster
struct Query {
  const float* rms;   // (P, I)
  const float* td00;  // (D, I, P)
  const float* td90;
  int P;
};

constexpr int kThreads = 256;
constexpr int kOut = 8;  // AA, dAA/dtheta, dAA/dphi, likelihood, correlation, ellipticity, Ec, No

template <int I>
__device__ void block_stat(const Query& q, float theta, float phi, const float* geom, int K,
                           float rr, float RR, float ethr, float* out, float* red) {
  DirInputs<I> d;
  direction_inputs<I>(theta, phi, geom, d);
  const int D = 2 * K + 1;
  // interpolation weights per detector (tangent carried by the fraction)
  int d0[I];
  D2 fr[I];
#pragma unroll
  for (int i = 0; i < I; ++i) {
    D2 t = d.tau[i];
    if (t.v < -K) t = mk(static_cast<float>(-K));
    if (t.v > K) t = mk(static_cast<float>(K));
    const D2 pos = t + static_cast<float>(K);
    int k0 = static_cast<int>(floorf(pos.v));
    k0 = k0 < 0 ? 0 : (k0 > D - 2 ? D - 2 : k0);
    d0[i] = k0;
    fr[i] = pos - static_cast<float>(k0);
  }
  Acc acc{mk(0.f), mk(0.f), mk(0.f), mk(0.f), mk(0.f), mk(0.f), 0};
  for (int j = threadIdx.x; j < q.P; j += blockDim.x) {
    float r[I];
    D2 v0[I], v9[I];
#pragma unroll
    for (int i = 0; i < I; ++i) {
      r[i] = q.rms[static_cast<int64_t>(j) * I + i];
      const int64_t a = (static_cast<int64_t>(d0[i]) * I + i) * q.P + j;
      const int64_t b = a + static_cast<int64_t>(I) * q.P;
      const float lo0 = q.td00[a], hi0 = q.td00[b], lo9 = q.td90[a], hi9 = q.td90[b];
      v0[i] = mk(lo0) + fr[i] * (hi0 - lo0);
      v9[i] = mk(lo9) + fr[i] * (hi9 - lo9);
    }
    pixel_dual<I>(r, v0, v9, d, rr, RR, ethr, acc);
  }
  // block reduction of 6 duals (18 floats) and Mo
  float vals[19] = {acc.EE.v, acc.EE.a, acc.EE.b, acc.LL.v, acc.LL.a, acc.LL.b,
                    acc.Lr.v, acc.Lr.a, acc.Lr.b, acc.EC.v, acc.EC.a, acc.EC.b,
                    acc.GN.v, acc.GN.a, acc.GN.b, acc.RN.v, acc.RN.a, acc.RN.b,
                    static_cast<float>(acc.Mo)};
#pragma unroll
  for (int k = 0; k < 19; ++k) {
    float v = vals[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    vals[k] = v;
  }
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < 19; ++k) red[warp * 19 + k] = vals[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    float t[19];
    for (int k = 0; k < 19; ++k) {
      t[k] = 0.f;
      for (int w = 0; w < nw; ++w) t[k] += red[w * 19 + k];
    }
    const D2 EE{t[0], t[1], t[2]}, LL{t[3], t[4], t[5]}, Lr{t[6], t[7], t[8]};
    const D2 EC{t[9], t[10], t[11]}, GN{t[12], t[13], t[14]}, RN{t[15], t[16], t[17]};
    const float Mo = t[18];
    // per-direction tail (sky_scan.py:131-140)
    const D2 Eo = EE * 0.5f;
    const D2 Cr = 2.0f * Lr / (LL + 1e-9f);
    const D2 No = (GN + RN) * 0.5f;
    const float den = I * Mo + sqrtf(Mo);
    const D2 CH = No / mk(den);
    const D2 cc = CH.v > 1.f ? CH : mk(1.f);
    const D2 Co = EC / (EC + No * cc - Mo * (I - 1));
    const D2 Lk = Eo.v > 0.f ? Eo - No : mk(0.f);
    const D2 AA = Lk * Co;
    out[0] = AA.v; out[1] = AA.a; out[2] = AA.b;
    out[3] = (Eo - No).v; out[4] = Co.v; out[5] = Cr.v; out[6] = EC.v; out[7] = No.v;
  }
  __syncthreads();
}

struct GradArgs {
  int n_queries, K;
  const int32_t* qc;          // cluster of each query
  const double* theta;
  const double* phi;
  const int64_t* pix_off;
  const int64_t* td_off;
  const float* rms;
  const float* td00;
  const float* td90;
  const float* geom;
  float rr;
  const float* reg1;          // per cluster
  float ethr;
  float* out;                 // (n_queries, kOut)
};

template <int I>
__global__ void __launch_bounds__(kThreads) sky_stat_grad_kernel(GradArgs g) {
  __shared__ float red[kThreads / 32 * 19];
  __shared__ float geom[I * kGeom];
  for (int k = threadIdx.x; k < I * kGeom; k += blockDim.x) geom[k] = g.geom[k];
  __syncthreads();
  for (int qi = blockIdx.x; qi < g.n_queries; qi += gridDim.x) {
    const int c = g.qc[qi];
    Query q;
    q.P = static_cast<int>(g.pix_off[c + 1] - g.pix_off[c]);
    q.rms = g.rms + g.pix_off[c] * I;
    q.td00 = g.td00 + g.td_off[c];
    q.td90 = g.td90 + g.td_off[c];
    block_stat<I>(q, static_cast<float>(g.theta[qi]), static_cast<float>(g.phi[qi]), geom, g.K,
                  g.rr, g.reg1[c], g.ethr, g.out + static_cast<int64_t>(qi) * kOut, red);
  }
}

struct RefineArgs {
  GradArgs base;
  int n_steps;
  float step0;                // initial step (radians of arc)
  double* theta_out;          // refined (theta, phi) per query
  double* phi_out;
  float* trace;               // (n_queries, n_steps + 1, 3): AA, theta, phi
};

// Gradient ascent on the sky statistic: one CTA per query; a step along the
// gradient (in arc length) is kept when the statistic does not decrease,
// otherwise the step is halved.
template <int I>
__global__ void __launch_bounds__(kThreads) refine_kernel(RefineArgs r) {
  __shared__ float red[kThreads / 32 * 19];
  __shared__ float geom[I * kGeom];
  __shared__ float cur[kOut], trial[kOut];
  __shared__ float s_th, s_ph, s_step;
  const GradArgs& g = r.base;
  for (int k = threadIdx.x; k < I * kGeom; k += blockDim.x) geom[k] = g.geom[k];
  for (int qi = blockIdx.x; qi < g.n_queries; qi += gridDim.x) {
    const int c = g.qc[qi];
    Query q;
    q.P = static_cast<int>(g.pix_off[c + 1] - g.pix_off[c]);
    q.rms = g.rms + g.pix_off[c] * I;
    q.td00 = g.td00 + g.td_off[c];
    q.td90 = g.td90 + g.td_off[c];
    if (threadIdx.x == 0) {
      s_th = static_cast<float>(g.theta[qi]);
      s_ph = static_cast<float>(g.phi[qi]);
      s_step = r.step0;
    }
    __syncthreads();
    block_stat<I>(q, s_th, s_ph, geom, g.K, g.rr, g.reg1[c], g.ethr, cur, red);
    float* tr = r.trace ? r.trace + static_cast<int64_t>(qi) * (r.n_steps + 1) * 3 : nullptr;
    if (threadIdx.x == 0 && tr) { tr[0] = cur[0]; tr[1] = s_th; tr[2] = s_ph; }
    for (int it = 0; it < r.n_steps; ++it) {
      __shared__ float t_th, t_ph;
      if (threadIdx.x == 0) {
        const float st = fmaxf(sinf(s_th), 1e-6f);
        const float gt = cur[1], gp = cur[2] / st;  // per unit arc length
        const float gn = sqrtf(gt * gt + gp * gp);
        const float h = gn > 0.f ? s_step / gn : 0.f;
        t_th = fminf(fmaxf(s_th + h * gt, 1e-6f), 3.14159265f - 1e-6f);
        t_ph = s_ph + h * gp / st;
      }
      __syncthreads();
      block_stat<I>(q, t_th, t_ph, geom, g.K, g.rr, g.reg1[c], g.ethr, trial, red);
      if (threadIdx.x == 0) {
        if (trial[0] >= cur[0]) {
          for (int k = 0; k < kOut; ++k) cur[k] = trial[k];
          s_th = t_th;
          s_ph = t_ph;
        } else {
          s_step *= 0.5f;
        }
        if (tr) {
          tr[3 * (it + 1)] = cur[0];
          tr[3 * (it + 1) + 1] = s_th;
          tr[3 * (it + 1) + 2] = s_ph;
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      r.theta_out[qi] = s_th;
      r.phi_out[qi] = s_ph;
      for (int k = 0; k < kOut; ++k) g.out[static_cast<int64_t>(qi) * kOut + k] = cur[k];
    }
    __syncthreads();
  }
}

int grad_launch(int n_ifo, const GradArgs& g, cudaStream_t s) {
  const int grid = g.n_queries < 65535 ? g.n_queries : 65535;
  switch (n_ifo) {
    case 1: sky_stat_grad_kernel<1><<<grid, kThreads, 0, s>>>(g); break;
    case 2: sky_stat_grad_kernel<2><<<grid, kThreads, 0, s>>>(g); break;
    case 3: sky_stat_grad_kernel<3><<<grid, kThreads, 0, s>>>(g); break;
    case 4: sky_stat_grad_kernel<4><<<grid, kThreads, 0, s>>>(g); break;
    case 5: sky_stat_grad_kernel<5><<<grid, kThreads, 0, s>>>(g); break;
    case 6: sky_stat_grad_kernel<6><<<grid, kThreads, 0, s>>>(g); break;
    case 7: sky_stat_grad_kernel<7><<<grid, kThreads, 0, s>>>(g); break;
    case 8: sky_stat_grad_kernel<8><<<grid, kThreads, 0, s>>>(g); break;
    default: return pgw::fail(PGW_ERR_BAD_SHAPE, "n_ifo must be in [1, 8]");
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return pgw::fail(PGW_ERR_CUDA, std::string("sky_stat_grad: ") + cudaGetErrorString(e));
  return PGW_OK;
}

int refine_launch(int n_ifo, const RefineArgs& r, cudaStream_t s) {
  const int grid = r.base.n_queries < 65535 ? r.base.n_queries : 65535;
  switch (n_ifo) {
    case 1: refine_kernel<1><<<grid, kThreads, 0, s>>>(r); break;
    case 2: refine_kernel<2><<<grid, kThreads, 0, s>>>(r); break;
    case 3: refine_kernel<3><<<grid, kThreads, 0, s>>>(r); break;
    case 4: refine_kernel<4><<<grid, kThreads, 0, s>>>(r); break;
    case 5: refine_kernel<5><<<grid, kThreads, 0, s>>>(r); break;
    case 6: refine_kernel<6><<<grid, kThreads, 0, s>>>(r); break;
    case 7: refine_kernel<7><<<grid, kThreads, 0, s>>>(r); break;
    case 8: refine_kernel<8><<<grid, kThreads, 0, s>>>(r); break;
    default: return pgw::fail(PGW_ERR_BAD_SHAPE, "n_ifo must be in [1, 8]");
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return pgw::fail(PGW_ERR_CUDA, std::string("refine: ") + cudaGetErrorString(e));
  return PGW_OK;
}

int fill_grad_args(GradArgs& g, int n_ifo, int n_queries, const int32_t* query_cluster,
                   const double* theta, const double* phi, const int64_t* pix_offsets,
                   const int64_t* td_offsets, const float* rms_all, const float* td00_all,
                   const float* td90_all, int n_delay, const float* geometry, float REG0,
                   const float* reg1, double network_energy_threshold, float* out) {
  if (n_ifo < 1 || n_ifo > PGW_MAX_IFO) return pgw::fail(PGW_ERR_BAD_SHAPE, "n_ifo must be in [1, 8]");
  if (n_delay < 3 || (n_delay & 1) == 0)
    return pgw::fail(PGW_ERR_BAD_SHAPE, "n_delay must be odd and >= 3 (2K+1, K >= 1)");
  if (n_queries < 0) return pgw::fail(PGW_ERR_BAD_SHAPE, "n_queries must be >= 0");
  if (n_queries > 0 && (!query_cluster || !theta || !phi || !pix_offsets || !td_offsets ||
                        !rms_all || !td00_all || !td90_all || !geometry || !reg1 || !out))
    return pgw::fail(PGW_ERR_BAD_ARGUMENT, "NULL device pointer");
  g.n_queries = n_queries;
  g.K = n_delay / 2;
  g.qc = query_cluster; g.theta = theta; g.phi = phi;
  g.pix_off = pix_offsets; g.td_off = td_offsets;
  g.rms = rms_all; g.td00 = td00_all; g.td90 = td90_all;
  g.geom = geometry;
  g.rr = REG0; g.reg1 = reg1;
  g.ethr = static_cast<float>(network_energy_threshold);
  g.out = out;
  return PGW_OK;
}

}  // namespace

extern "C" int pgw_sky_stat_grad(int n_ifo, int n_queries, const int32_t* query_cluster,
                                 const double* theta, const double* phi,
                                 const int64_t* pix_offsets, const int64_t* td_offsets,
                                 const float* rms_all, const float* td00_all,
                                 const float* td90_all, int n_delay, const float* geometry,
                                 float REG0, const float* reg1, double network_energy_threshold,
                                 float* out, void* stream) {
  GradArgs g{};
  int rc = fill_grad_args(g, n_ifo, n_queries, query_cluster, theta, phi, pix_offsets, td_offsets,
                          rms_all, td00_all, td90_all, n_delay, geometry, REG0, reg1,
                          network_energy_threshold, out);
  if (rc || n_queries == 0) return rc;
  return grad_launch(n_ifo, g, static_cast<cudaStream_t>(stream));
}

extern "C" int pgw_refine_sky(int n_ifo, int n_queries, const int32_t* query_cluster,
                              const double* theta0, const double* phi0,
                              const int64_t* pix_offsets, const int64_t* td_offsets,
                              const float* rms_all, const float* td00_all, const float* td90_all,
                              int n_delay, const float* geometry, float REG0, const float* reg1,
                              double network_energy_threshold, int n_steps, float step0,
                              double* theta_out, double* phi_out, float* out, float* trace,
                              void* stream) {
  RefineArgs r{};
  int rc = fill_grad_args(r.base, n_ifo, n_queries, query_cluster, theta0, phi0, pix_offsets,
                          td_offsets, rms_all, td00_all, td90_all, n_delay, geometry, REG0, reg1,
                          network_energy_threshold, out);
  if (rc || n_queries == 0) return rc;
  if (n_steps < 0 || !(step0 > 0.f)) return pgw::fail(PGW_ERR_BAD_ARGUMENT, "n_steps >= 0, step0 > 0");
  if (!theta_out || !phi_out) return pgw::fail(PGW_ERR_BAD_ARGUMENT, "NULL device pointer");
  r.n_steps = n_steps;
  r.step0 = step0;
  r.theta_out = theta_out;
  r.phi_out = phi_out;
  r.trace = trace;
  return refine_launch(n_ifo, r, static_cast<cudaStream_t>(stream));
}
