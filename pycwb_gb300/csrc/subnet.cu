// Sub-network-cut sky loop for GB300 (sm_103a): optimze_sky_loc_from_td of
// pycwb/modules/super_cluster_native/sub_net_cut.py:404-517, for many clusters
// in one launch.
//
// For every cluster and every sky direction l: the per-pixel network energy
// at the direction's delays, the gate on the sub-network fraction (when
// subcut >= 0), the DPF projection of the pixels above the energy threshold
// (sse_like_ps) and the direction's statistic AA; the cluster keeps the
// direction with the largest AA > 0, the first one on ties (the reference's
// strict `>` over l = 0, 1, ...).
//
// One thread per (cluster, direction); a cluster's td block (a few hundred
// of its loudest pixels, (2K+1, nIFO, P) float32) stays in L1/L2 while the
// CTA's directions read it.  Every float32 operation is rounded separately
// (no contraction) in the reference's order, and np.dot is evaluated as
// NumPy does it (float32 products summed in float64), so a direction's values
// are those of the reference run with NumPy scalar semantics, bit for bit.
// The winning direction's outputs are recomputed by one thread per cluster
// after the sweep.

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/pycwb_gb300.h"

namespace pgw {
int fail(int code, const std::string& msg);
}

namespace {

constexpr int kMaxIfo = PGW_MAX_IFO;

__device__ __forceinline__ float M(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float A(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float S(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float D(float a, float b) { return __fdiv_rn(a, b); }

struct SubnetArgs {
  const float* FP;
  const float* FX;
  const int32_t* ml;
  int64_t n_sky;
  int n_ifo, n_delay, offset, n_clusters;
  int64_t total_pix;
  const int64_t* pix_offsets;  // null: one cluster of total_pix pixels
  const int64_t* td_offsets;
  const float* rms;
  const float* td00;
  const float* td90;
  float thr, Es, subcut;
  int gate;
  pgw_subnet_result* out;
};

struct DirStats {
  float AA, Eo, aa2, ee, em;
  int m;
  bool ok;  // passed the gate and Eo > 0
};

// np.dot of float32 vectors as NumPy evaluates it: float32 products, float64 sum
template <int I>
__device__ __forceinline__ float dot32(const float (&a)[I], const float (&b)[I]) {
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < I; ++j) s = __dadd_rn(s, static_cast<double>(M(a[j], b[j])));
  return static_cast<float>(s);
}

// One direction of one cluster (sub_net_cut.py:432-507).
template <int I>
__device__ DirStats direction_stats(const SubnetArgs& a, int64_t P, int64_t td0, int64_t p0,
                                    int64_t l, const int (&d)[kMaxIfo]) {
  DirStats r{};
  float m_gt = 0.f, Eo_gt = 0.f, Ls_gt = 0.f, Ln_gt = 0.f, Eo_ge = 0.f, Ls_ge = 0.f, Ln_ge = 0.f;
  int m = 0;
  for (int64_t j = 0; j < P; ++j) {  // :436-465
    float rE = 0.f, em = 0.f;
#pragma unroll
    for (int i = 0; i < I; ++i) {
      const int64_t q = td0 + (static_cast<int64_t>(d[i]) * I + i) * P + j;
      const float x = __ldg(a.td00 + q), y = __ldg(a.td90 + q);
      const float de = A(M(x, x), M(y, y));
      rE = A(rE, de);
      if (de > em) em = de;
    }
    const float sub = S(rE, em);
    if (rE >= a.thr) {
      Eo_ge = A(Eo_ge, rE);
      Ls_ge = A(Ls_ge, sub);
      if (sub > a.Es) Ln_ge = A(Ln_ge, rE);
      ++m;
    }
    if (rE > a.thr) {
      m_gt = A(m_gt, 1.0f);
      Eo_gt = A(Eo_gt, rE);
      Ls_gt = A(Ls_gt, sub);
      if (sub > a.Es) Ln_gt = A(Ln_gt, rE);
    }
  }
  const float Eo_cut = A(Eo_gt, 0.01f);                              // :467
  const float m_cut = static_cast<float>(static_cast<int64_t>(A(M(2.0f, m_gt), 0.01f)));  // :468
  const float aa = D(M(Ls_gt, Ln_gt), S(Eo_cut, Ls_gt));            // :469
  if (a.gate && D(S(aa, m_cut), A(A(aa, m_cut), 1e-16f)) < a.subcut) return r;  // :470
  const float Eo = Eo_ge, Ls = Ls_ge, Ln = Ln_ge;
  if (Eo <= 0.f) return r;                                           // :488
  float Fp[I], Fx[I];
  for (int i = 0; i < I; ++i) {
    Fp[i] = __ldg(a.FP + l * I + i);
    Fx[i] = __ldg(a.FX + l * I + i);
  }
  float Lo = 0.f;
  for (int64_t j = 0; j < P; ++j) {  // the pixels above the threshold, in order (:474-497)
    float am[I], AM[I];
    float rE = 0.f;
#pragma unroll
    for (int i = 0; i < I; ++i) {
      const int64_t q = td0 + (static_cast<int64_t>(d[i]) * I + i) * P + j;
      am[i] = __ldg(a.td00 + q);
      AM[i] = __ldg(a.td90 + q);
      rE = A(rE, A(M(am[i], am[i]), M(AM[i], AM[i])));
    }
    if (rE < a.thr) continue;
    // _dpf_np_loops_vec_into for this pixel (:521-563)
    float f[I], F[I];
    for (int i = 0; i < I; ++i) {
      const float w = __ldg(a.rms + (p0 + j) * I + i);
      f[i] = M(w, Fp[i]);
      F[i] = M(w, Fx[i]);
    }
    float ff = 0.f, FF = 0.f, fF = 0.f;
    for (int i = 0; i < I; ++i) {
      ff = A(ff, M(f[i], f[i]));
      FF = A(FF, M(F[i], F[i]));
      fF = A(fF, M(F[i], f[i]));
    }
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
      f[i] = x;
      F[i] = y;
    }
    float fFn = 0.f;
    for (int i = 0; i < I; ++i) fFn = A(fFn, M(f[i], F[i]));
    fFn = D(fFn, A(fp, 1e-9f));
    for (int i = 0; i < I; ++i) F[i] = S(F[i], M(f[i], fFn));
    // sse_like_ps (:728-742)
    const float xp = dot32<I>(f, am), XP = dot32<I>(f, AM);
    const float xx = dot32<I>(F, am), XX = dot32<I>(F, AM);
    const float gp = A(dot32<I>(f, f), 1e-12f), gx = A(dot32<I>(F, F), 1e-12f);
    const float p2 = A(M(xp, xp), M(XP, XP)), x2 = A(M(xx, xx), M(XX, XX));
    Lo = A(Lo, A(D(p2, gp), D(x2, gx)));
  }
  const float mf = static_cast<float>(m);
  const float den = A(A(fabsf(aa), fabsf(S(Eo, Lo))), D(M(M(2.0f, mf), S(Eo, Ln)), Eo));  // :503
  r.AA = D(aa, den);
  float ee = D(M(Ls, Eo), S(Eo, Ls));                                // :504
  r.em = A(fabsf(S(Eo, Lo)), M(2.0f, mf));                           // :505
  r.ee = D(ee, A(ee, r.em));                                         // :506
  r.aa2 = D(S(aa, mf), A(aa, mf));                                   // :507
  r.Eo = Eo;
  r.m = m;
  r.ok = true;
  return r;
}

__device__ __forceinline__ bool direction_delays(const SubnetArgs& a, int64_t l, int (&d)[kMaxIfo]) {
  for (int i = 0; i < a.n_ifo; ++i) {
    d[i] = a.ml[static_cast<int64_t>(i) * a.n_sky + l] + a.offset;
    if (d[i] < 0 || d[i] >= a.n_delay) return false;
  }
  return true;
}

__global__ void subnet_init_kernel(pgw_subnet_result* out, int n_clusters) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n_clusters) {
    out[c].key = 0ull;
    out[c].status = 0;
  }
}

template <int I>
__global__ void __launch_bounds__(256) subnet_sweep_kernel(SubnetArgs a) {
  const int c = blockIdx.y;
  const int64_t p0 = a.pix_offsets ? a.pix_offsets[c] : 0;
  const int64_t P = a.pix_offsets ? a.pix_offsets[c + 1] - p0 : a.total_pix;
  const int64_t td0 = (a.pix_offsets && a.td_offsets) ? a.td_offsets[c] : 0;
  const int64_t l = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  unsigned long long key = 0ull;
  if (l < a.n_sky && P > 0) {
    int d[kMaxIfo];
    if (!direction_delays(a, l, d)) {
      atomicOr(&a.out[c].status, 1 << PGW_ERR_DELAY_RANGE);
    } else {
      const DirStats s = direction_stats<I>(a, P, td0, p0, l, d);
      // AA > 0 (NaN never qualifies); larger AA first, then the smaller l
      if (s.ok && s.AA > 0.0f)
        key = (static_cast<unsigned long long>(__float_as_uint(s.AA)) << 32) |
              static_cast<unsigned long long>(0xffffffffu - static_cast<unsigned>(l));
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(0xffffffffu, key, o);
    key = other > key ? other : key;
  }
  if ((threadIdx.x & 31) == 0 && key)
    atomicMax(reinterpret_cast<unsigned long long*>(&a.out[c].key), key);
}

template <int I>
__global__ void subnet_finalize_kernel(SubnetArgs a) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= a.n_clusters) return;
  pgw_subnet_result& r = a.out[c];
  const unsigned long long key = r.key;
  r.l_max = 0;
  r.stat = r.Em = r.Am = r.suball = r.EE = 0.0f;
  r.Vm = 0;
  if (!key) return;
  const int64_t l = static_cast<int64_t>(0xffffffffu - static_cast<unsigned>(key & 0xffffffffull));
  const int64_t p0 = a.pix_offsets ? a.pix_offsets[c] : 0;
  const int64_t P = a.pix_offsets ? a.pix_offsets[c + 1] - p0 : a.total_pix;
  const int64_t td0 = (a.pix_offsets && a.td_offsets) ? a.td_offsets[c] : 0;
  int d[kMaxIfo];
  if (!direction_delays(a, l, d)) return;
  const DirStats s = direction_stats<I>(a, P, td0, p0, l, d);
  r.l_max = l;
  r.stat = s.AA;
  r.Em = s.Eo;
  r.Am = s.aa2;
  r.Vm = s.m;
  r.suball = s.ee;
  r.EE = s.em;
}

template <int I>
void launch_subnet(const SubnetArgs& a, cudaStream_t s) {
  const dim3 grid(static_cast<unsigned>((a.n_sky + 255) / 256), static_cast<unsigned>(a.n_clusters));
  subnet_sweep_kernel<I><<<grid, 256, 0, s>>>(a);
  subnet_finalize_kernel<I><<<(a.n_clusters + 127) / 128, 128, 0, s>>>(a);
}

}  // namespace

extern "C" int pgw_subnet_sky_batched(int n_ifo, int n_clusters, const int64_t* pix_offsets,
                                      const int64_t* td_offsets, int64_t total_pix,
                                      int64_t n_sky, const float* FP, const float* FX,
                                      const float* rms_all, const float* td00_all,
                                      const float* td90_all, int n_delay, const int32_t* ml,
                                      float network_energy_threshold, double e2or,
                                      double subcut, pgw_subnet_result* out, void* stream) {
  if (n_ifo < 1 || n_ifo > PGW_MAX_IFO) return pgw::fail(PGW_ERR_BAD_SHAPE, "n_ifo must be in [1, 8]");
  if (n_clusters < 1 || n_clusters > 65535)
    return pgw::fail(PGW_ERR_BAD_SHAPE, "n_clusters must be in [1, 65535]");
  if (n_delay < 1 || (n_delay & 1) == 0)
    return pgw::fail(PGW_ERR_BAD_SHAPE, "n_delay must be odd and >= 1 (2K+1)");
  if (n_sky < 1 || n_sky > 0x7fffffffLL || total_pix < 0)
    return pgw::fail(PGW_ERR_BAD_SHAPE, "need 1 <= n_sky < 2^31 and total_pix >= 0");
  if (!FP || !FX || !ml || !out || (total_pix > 0 && (!rms_all || !td00_all || !td90_all)))
    return pgw::fail(PGW_ERR_BAD_ARGUMENT, "NULL device pointer");
  if (n_clusters > 1 && (!pix_offsets || !td_offsets))
    return pgw::fail(PGW_ERR_BAD_ARGUMENT, "offsets are required for more than one cluster");
  SubnetArgs a{};
  a.FP = FP; a.FX = FX; a.ml = ml; a.n_sky = n_sky;
  a.n_ifo = n_ifo; a.n_delay = n_delay; a.offset = n_delay / 2; a.n_clusters = n_clusters;
  a.total_pix = total_pix; a.pix_offsets = pix_offsets; a.td_offsets = td_offsets;
  a.rms = rms_all; a.td00 = td00_all; a.td90 = td90_all;
  a.thr = network_energy_threshold;
  a.Es = static_cast<float>(2.0 * e2or);        // sub_net_cut.py:407
  a.subcut = static_cast<float>(subcut);
  a.gate = subcut >= 0.0;
  a.out = out;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  subnet_init_kernel<<<(n_clusters + 255) / 256, 256, 0, s>>>(out, n_clusters);
  switch (n_ifo) {
    case 1: launch_subnet<1>(a, s); break;
    case 2: launch_subnet<2>(a, s); break;
    case 3: launch_subnet<3>(a, s); break;
    case 4: launch_subnet<4>(a, s); break;
    case 5: launch_subnet<5>(a, s); break;
    case 6: launch_subnet<6>(a, s); break;
    case 7: launch_subnet<7>(a, s); break;
    default: launch_subnet<8>(a, s); break;
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return pgw::fail(PGW_ERR_CUDA, std::string("subnet sky loop: ") + cudaGetErrorString(e));
  return PGW_OK;
}
