/*
 * Sky-scan oracle: a CPU restatement of PycWB's coherent sky-scan likelihood.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product imports or links this
 * file: it is the checker that the CUDA path is compared against (tests/),
 * and the timed CPU baseline of bench.py.  It follows, line by line,
 *
 *   calculate_dpf            pycwb/modules/likelihoodWP/dpf.py:7-34
 *   dpf_np_loops_vec         pycwb/modules/likelihoodWP/dpf.py:343-453
 *   load_data_from_td        pycwb/modules/likelihoodWP/sky_stat.py:37-89
 *   avx_GW_ps                pycwb/modules/likelihoodWP/sky_stat.py:93-219
 *   avx_ort_ps               pycwb/modules/likelihoodWP/sky_stat.py:223-294
 *   avx_stat_ps              pycwb/modules/likelihoodWP/sky_stat.py:298-410
 *   scan_sky_for_best_fit    pycwb/modules/likelihoodWP/sky_scan.py:17-192
 *
 * Two precisions:
 *
 *   *_f32  reproduces the reference's own arithmetic: float32 everywhere the
 *          reference declares float32, float64 exactly where NumPy scalar
 *          promotion makes the reference compute in float64 (int32/float32
 *          divisions in avx_GW_ps, the disbalance/correlation tail of the
 *          scan).  Pixel energies are compared against (float)E_thr, as the
 *          NumPy scalars and cWB's _avx_loadata_ps (cwb-core/watavx.hh:648)
 *          do.  Sums run in pixel order, as in the reference.  Build with
 *          -ffp-contract=off so no multiply-add is fused (the reference never
 *          fuses).  Pinned against the golden vectors in tests/golden/.
 *   *_f64  the same loop entirely in double precision: the FP64 yardstick
 *          for error figures.  Not a parity target.
 *
 * The oracle is parallelised over sky directions with OpenMP, like the
 * reference's numba prange over the sky (sky_scan.py:97, dpf.py:27).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAXIFO 8
#define N_STATS 11

enum { ORC_OK = 0, ORC_BAD_SHAPE = 1, ORC_BAD_DELAY = 2 };

static inline void set_threads(int n_threads) {
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#else
  (void)n_threads;
#endif
}

/* ------------------------------------------------------------------------ */
/* float32 restatement (reference arithmetic)                                */
/* ------------------------------------------------------------------------ */

typedef struct {
  float f[ORC_MAXIFO], F[ORC_MAXIFO];
  float fp, fx, ni;
} dpf32_t;

/* dpf.py:396-438 for one pixel; returns the rotated f, orthogonalised F,
 * |f+|^2 (fp), |fx|^2 (fx) and the network index (ni, already divided by
 * fp^2 as in dpf.py:446). */
static inline void dpf_pixel32(const float* Fp, const float* Fx, const float* r, int I, dpf32_t* o) {
  float f[ORC_MAXIFO], F[ORC_MAXIFO];
  for (int j = 0; j < I; ++j) { f[j] = r[j] * Fp[j]; F[j] = r[j] * Fx[j]; }    /* :396-399 */
  float ff = 0.f, FF = 0.f, fF = 0.f;
  for (int j = 0; j < I; ++j) { ff += f[j] * f[j]; FF += F[j] * F[j]; fF += F[j] * f[j]; }  /* :407-410 */
  float si2 = 2.0f * fF;                                 /* :413 */
  float co2 = ff - FF;                                   /* :414 */
  float AP = ff + FF;                                    /* :415 */
  float nn = sqrtf(co2 * co2 + si2 * si2);               /* :416 */
  float cc = co2 / (nn + 1e-9f);                         /* :417 */
  float fp = (AP + nn) / 2.0f;                           /* :418 */
  float si = sqrtf((1.0f - cc) / 2.0f);                  /* :419 */
  float cq = sqrtf((1.0f + cc) / 2.0f);
  float co = si2 > 0.0f ? cq : -cq;                      /* :420 */
  for (int j = 0; j < I; ++j) {                          /* :424-425 */
    float a = f[j] * co + F[j] * si;
    float b = F[j] * co - f[j] * si;
    f[j] = a; F[j] = b;
  }
  float fFn = 0.f;
  for (int j = 0; j < I; ++j) fFn += f[j] * F[j];        /* :429-431 */
  fFn = fFn / (fp + 1e-9f);                              /* :433 */
  float fx = 0.f, ni = 0.f;
  for (int j = 0; j < I; ++j) {                          /* :435-438 */
    F[j] -= f[j] * fFn;
    fx += F[j] * F[j];
    ni += powf(f[j], 4.0f);
  }
  ni = ni / (fp * fp + 1e-9f);                           /* :446 */
  for (int j = 0; j < I; ++j) { o->f[j] = f[j]; o->F[j] = F[j]; }
  o->fp = fp; o->fx = fx; o->ni = ni;
}

int oracle_calculate_dpf_f32(const float* FP, const float* FX, const float* rms,
                             int64_t n_sky, int n_ifo, int64_t n_pix,
                             double gamma_regulator, double network_energy_threshold,
                             const int64_t* valid, int64_t n_valid, int n_threads,
                             double* out_regulator) {
  if (n_ifo < 1 || n_ifo > ORC_MAXIFO || n_pix < 0 || n_sky < 1) return ORC_BAD_SHAPE;
  set_threads(n_threads);
  int64_t n_pass = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : n_pass)
  for (int64_t k = 0; k < n_valid; ++k) {
    const int64_t l = valid[k];
    const float* Fp = FP + l * n_ifo;
    const float* Fx = FX + l * n_ifo;
    float NI = 0.f;
    uint32_t NN = 0;
    for (int64_t p = 0; p < n_pix; ++p) {                /* dpf.py:444-450 */
      dpf32_t d;
      dpf_pixel32(Fp, Fx, rms + p * n_ifo, n_ifo, &d);
      NI += d.fx / (d.ni + 1e-9f);
      NN += d.fp > 0.0f ? 1u : 0u;
    }
    double q = sqrt((double)NI / ((double)NN + 0.01));   /* dpf.py:453 */
    if (q > gamma_regulator) n_pass += 1;                /* dpf.py:32 */
  }
  double FF = (double)n_valid, ff = (double)n_pass;
  *out_regulator = (FF * FF / (ff * ff + 1.e-9) - 1) * network_energy_threshold;  /* dpf.py:34 */
  return ORC_OK;
}

/* One pixel of one direction through load_data_from_td, avx_GW_ps,
 * avx_ort_ps and avx_stat_ps (sky_stat.py:74-89, 157-189, 264-288, 357-405):
 * every per-pixel quantity the scan accumulates and the statistics at l_max
 * read back. */
typedef struct {
  float et, msk, ee, EE, osi, oco, ec, gn, rn, ll;
  int32_t mk;
  float s[ORC_MAXIFO], S[ORC_MAXIFO];
} pix32_t;

static inline void pixel32(int I, const float* v0, const float* v9, const dpf32_t* dp,
                           float rr, float RR, float ethr32, pix32_t* o) {
  const dpf32_t d = *dp;
  /* load_data_from_td, sky_stat.py:74-89 */
  float aa = 0.f, AA = 0.f;
  for (int i = 0; i < I; ++i) { aa += v0[i] * v0[i]; AA += v9[i] * v9[i]; }
  float e = aa + AA + 1e-12f;
  int32_t mk = e > ethr32 ? 1 : 0;
  float et = mk ? e : 0.0f;

  /* avx_GW_ps, sky_stat.py:157-189 */
  float xp = 0.f, XP = 0.f, xx = 0.f, XX = 0.f;
  for (int i = 0; i < I; ++i) {
    xp += v0[i] * d.f[i]; XP += v9[i] * d.f[i];
    xx += v0[i] * d.F[i]; XX += v9[i] * d.F[i];
  }
  float t = d.ni * (xp * xp + XP * XP);
  t = t / (et + 1e-9f);
  float g = sqrtf(t) * rr - d.fp;                        /* :164 */
  g = g > 0.0f ? g : 0.0f;                               /* :165 */
  double fd = (double)mk / (double)((d.fp + g) + 1e-9f); /* :166, int32/float32 -> float64 */
  double h = (double)xp * fd, Hh = (double)XP * fd;      /* :168-169 */
  h = h * h + Hh * Hh;                                   /* :170 */
  float H2 = xx * xx + XX * XX;                          /* :171 */
  double Fd = sqrt((double)H2 / (h + (double)1e-9f));    /* :172 */
  float R = 0.1f + RR / (et + 1e-9f);                    /* :173 */
  float G = (float)Fd * R - d.fx;                        /* :174 */
  G = G > 0.0f ? G : 0.0f;                               /* :175 */
  double Gd = (double)mk / (double)((d.fx + G) + 1e-9f); /* :176 */
  float au = (float)((double)xp * fd), AU = (float)((double)XP * fd);   /* :178-179 */
  float av = (float)((double)xx * Gd), AV = (float)((double)XX * Gd);   /* :180-181 */
  double a_ = fd * (double)d.fp + Gd * (double)d.fx;     /* :183 */
  float msk = (float)((a_ + (double)mk) - (double)1.0f); /* :185 */
  for (int i = 0; i < I; ++i) {                          /* :187-189 */
    o->s[i] = d.f[i] * au + d.F[i] * av;
    o->S[i] = d.f[i] * AU + d.F[i] * AV;
  }
  const float* s = o->s;
  const float* S = o->S;

  /* avx_ort_ps, sky_stat.py:264-288 */
  float a2 = 0.f, A2 = 0.f, aA = 0.f;
  for (int i = 0; i < I; ++i) { a2 += s[i] * s[i]; A2 += S[i] * S[i]; aA += s[i] * S[i]; }
  float osi = aA * 2.0f;
  float oco = a2 - A2;
  float oet = a2 + A2 + 1e-21f;
  float occ = oco * oco, oss = osi * osi;
  float onn = sqrtf(occ + oss);
  o->ee = (oet + onn) / 2.0f;
  o->EE = (oet - onn) / 2.0f;
  occ = oco / (onn + 1e-21f);
  float sgn = osi > 0.0f ? 1.0f : -1.0f;
  osi = sqrtf((1.0f - occ) / 2.0f);
  oco = sqrtf((1.0f + occ) / 2.0f) * sgn;

  /* avx_stat_ps, sky_stat.py:357-405 */
  float c = 0.f, C = 0.f, ss = 0.f, SS = 0.f, r0 = 0.f, R0 = 0.f, xs = 0.f, XS = 0.f;
  for (int i = 0; i < I; ++i) {
    float s_ = s[i] * oco + S[i] * osi;
    float x_ = v0[i] * oco + v9[i] * osi;
    float S_ = S[i] * oco - s[i] * osi;
    float X_ = v9[i] * oco - v0[i] * osi;
    float a = s_ * x_, A = S_ * X_;
    xs += a; XS += A;
    c += a * a; C += A * A;
    ss += s_ * s_; SS += S_ * S_;
    float q0 = s[i] - v0[i], q9 = S[i] - v9[i];
    r0 += q0 * q0; R0 += q9 * q9;
  }
  int mks = msk >= 0.0f ? 1 : 0;                         /* :385 */
  c = c / (xs * xs + 1e-9f);
  C = C / (XS * XS + 1e-9f);
  o->ll = (float)mks * (ss + SS);
  ss = ss * (1.0f - c);
  SS = SS * (1.0f - C);
  o->ec = (float)mks * (ss + SS);
  o->gn = (float)(mks * 2.0) * msk;
  o->rn = (float)mks * (r0 + R0);
  o->et = et; o->mk = mk; o->msk = msk; o->osi = osi; o->oco = oco;
}

/* One sky direction of scan_sky_for_best_fit (sky_scan.py:98-179) fused into
 * a single pass over the pixels; every accumulator keeps pixel order. */
static inline int scan_sky32(int I, int64_t P, int64_t l, const float* FP, const float* FX,
                             const float* rms, const float* td00, const float* td90,
                             int n_delay, int64_t n_sky, const int32_t* ml, float rr, float RR,
                             double netCC, double delta_regulator, float ethr32,
                             float* stats /* N_STATS x n_sky */, float* best, float* cr_all) {
  const int off = n_delay / 2;                           /* sky_scan.py:92 */
  int row[ORC_MAXIFO];
  for (int i = 0; i < I; ++i) {
    int d = ml[(int64_t)i * n_sky + l] + off;
    if (d < 0 || d >= n_delay) return ORC_BAD_DELAY;
    row[i] = d;
  }
  const float* Fp = FP + l * I;
  const float* Fx = FX + l * I;

  float EE = 0.f;               /* load_data_from_td: sum of thresholded energy */
  int32_t Mo = 0;               /* avx_GW_ps: NN, pixels above threshold */
  float LL = 0.f, Lr = 0.f, EC = 0.f, GN = 0.f, RN = 0.f, NNc = 0.f;   /* avx_stat_ps */
  float ee = 0.f, ffw = 0.f, FFw = 0.f;                  /* sky_scan.py:144-153 */

  for (int64_t j = 0; j < P; ++j) {
    float v0[ORC_MAXIFO], v9[ORC_MAXIFO];
    for (int i = 0; i < I; ++i) {                        /* sky_scan.py:102-104 */
      v0[i] = td00[((int64_t)row[i] * I + i) * P + j];
      v9[i] = td90[((int64_t)row[i] * I + i) * P + j];
    }
    dpf32_t d;                                           /* dpf_np_loops_vec, dpf.py:396-446 */
    dpf_pixel32(Fp, Fx, rms + j * I, I, &d);
    pix32_t q;
    pixel32(I, v0, v9, &d, rr, RR, ethr32, &q);
    EE += q.et;
    Mo += q.mk;                                          /* sky_stat.py:184 */
    float a2e = 2.0f * fabsf(q.ec);
    float An = q.rn + q.gn + 1e-9f;
    float ccn = q.ec / (a2e + An);
    Lr += q.ll * ccn;
    LL += q.ll; EC += q.ec; GN += q.gn; RN += q.rn;
    NNc += q.ec > 1e-9f ? 1.0f : 0.0f;

    /* sky_scan.py:148-153 */
    if (q.msk > 0.0f) { ee += q.et; ffw += d.fp * q.et; FFw += d.fx * q.et; }
  }
  const float Eo = EE / 2.0f;                            /* sky_stat.py:89 */
  const float Cr = 2.0f * Lr / (LL + 1e-9f);             /* sky_stat.py:407 */
  const float No = (GN + RN) / 2.0f;                     /* sky_stat.py:408 */

  /* sky_scan.py:131-133 */
  double den = (double)(I * Mo) + sqrt((double)Mo);
  double CH = (double)No / den;
  double corr, ccor;
  if (CH > 1.0) {
    ccor = CH;
    corr = (double)EC / ((double)EC + (double)No * CH - (double)(Mo * (I - 1)));
  } else {
    ccor = 1.0;   /* Python float 1.0: null*1.0 stays float32 and (Ec+No) rounds to float32 */
    corr = (double)EC / ((double)(EC + No) - (double)(Mo * (I - 1)));
  }
  if (cr_all) cr_all[l] = Cr;  /* ellipticity of every valid direction (diagnostic) */
  if (!isfinite(Cr) || (double)Cr < netCC) return ORC_OK;  /* :135-136 */

  float Lk = Eo > 0.0f ? Eo - No : 0.0f;                 /* :139 */
  double AA = (double)Lk * corr;                         /* :140 */
  (void)delta_regulator;                                 /* :141 probability map is not returned */
  ffw = ee > 0.0f ? ffw / ee : 0.0f;                     /* :154-161 */
  FFw = ee > 0.0f ? FFw / ee : 0.0f;
  stats[0 * n_sky + l] = sqrtf(ffw + FFw);               /* :163 */
  stats[1 * n_sky + l] = ffw > 0.0f ? sqrtf(FFw / ffw) : 0.0f;   /* :164-167 */
  stats[2 * n_sky + l] = Eo - No;                        /* :169 */
  stats[3 * n_sky + l] = No;
  stats[4 * n_sky + l] = EC;
  stats[5 * n_sky + l] = (float)corr;
  stats[6 * n_sky + l] = (float)AA;
  stats[7 * n_sky + l] = (float)CH;
  stats[8 * n_sky + l] = (float)ccor;
  stats[9 * n_sky + l] = Cr;
  stats[10 * n_sky + l] = NNc;
  best[l] = (float)AA;                                   /* :179 */
  return ORC_OK;
}

/* Forward scan with >=, last tie wins, over valid indices in list order
 * (sky_scan.py:183-189).  *found = 0 reproduces the reference's untouched
 * initial state: l_max = valid[0], sky_stat_max = 0. */
static void argmax_ties_last(const float* best, const int64_t* valid, int64_t n_valid,
                             int64_t* l_max, double* sky_stat_max, int* found) {
  double cur = 0.0;
  int64_t lm = valid[0];
  int fnd = 0;
  for (int64_t k = 0; k < n_valid; ++k) {
    const int64_t l = valid[k];
    if ((double)best[l] >= cur) { cur = (double)best[l]; lm = l; fnd = 1; }
  }
  *l_max = lm; *sky_stat_max = cur;
  if (found) *found = fnd;
}

int oracle_scan_sky_f32(int n_ifo, int64_t n_pix, int64_t n_sky, const float* FP, const float* FX,
                        const float* rms, const float* td00, const float* td90, int n_delay,
                        const int32_t* ml, const float* REG, double netCC, double delta_regulator,
                        double network_energy_threshold, const int64_t* valid, int64_t n_valid,
                        int n_threads, float* stats, int64_t* l_max, double* sky_stat_max,
                        int* found, float* cr_all) {
  if (n_ifo < 1 || n_ifo > ORC_MAXIFO || n_pix < 0 || n_sky < 1 || n_valid < 1 || n_delay < 1)
    return ORC_BAD_SHAPE;
  set_threads(n_threads);
  memset(stats, 0, sizeof(float) * N_STATS * (size_t)n_sky);
  float* best = (float*)malloc(sizeof(float) * (size_t)n_sky);
  if (!best) return ORC_BAD_SHAPE;
  for (int64_t l = 0; l < n_sky; ++l) best[l] = -1.e12f;
  const float rr = REG[0], RR = REG[1];
  const float ethr32 = (float)network_energy_threshold;
  int err = ORC_OK;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t k = 0; k < n_valid; ++k) {
    int e = scan_sky32(n_ifo, n_pix, valid[k], FP, FX, rms, td00, td90, n_delay, n_sky, ml, rr,
                       RR, netCC, delta_regulator, ethr32, stats, best, cr_all);
    if (e) {
#pragma omp atomic write
      err = e;
    }
  }
  if (err == ORC_OK) argmax_ties_last(best, valid, n_valid, l_max, sky_stat_max, found);
  free(best);
  return err;
}

/* ------------------------------------------------------------------------ */
/* float64 yardstick: the same loop with every operation in double           */
/* ------------------------------------------------------------------------ */

typedef struct {
  double f[ORC_MAXIFO], F[ORC_MAXIFO];
  double fp, fx, ni;
} dpf64_t;

static inline void dpf_pixel64(const float* Fp, const float* Fx, const float* r, int I, dpf64_t* o) {
  double f[ORC_MAXIFO], F[ORC_MAXIFO];
  for (int j = 0; j < I; ++j) { f[j] = (double)r[j] * Fp[j]; F[j] = (double)r[j] * Fx[j]; }
  double ff = 0, FF = 0, fF = 0;
  for (int j = 0; j < I; ++j) { ff += f[j] * f[j]; FF += F[j] * F[j]; fF += F[j] * f[j]; }
  double si2 = 2.0 * fF, co2 = ff - FF, AP = ff + FF;
  double nn = sqrt(co2 * co2 + si2 * si2);
  double cc = co2 / (nn + 1e-9);
  double fp = (AP + nn) / 2.0;
  double si = sqrt((1.0 - cc) / 2.0);
  double cq = sqrt((1.0 + cc) / 2.0);
  double co = si2 > 0.0 ? cq : -cq;
  for (int j = 0; j < I; ++j) {
    double a = f[j] * co + F[j] * si, b = F[j] * co - f[j] * si;
    f[j] = a; F[j] = b;
  }
  double fFn = 0;
  for (int j = 0; j < I; ++j) fFn += f[j] * F[j];
  fFn = fFn / (fp + 1e-9);
  double fx = 0, ni = 0;
  for (int j = 0; j < I; ++j) {
    F[j] -= f[j] * fFn;
    fx += F[j] * F[j];
    ni += (f[j] * f[j]) * (f[j] * f[j]);
  }
  ni = ni / (fp * fp + 1e-9);
  for (int j = 0; j < I; ++j) { o->f[j] = f[j]; o->F[j] = F[j]; }
  o->fp = fp; o->fx = fx; o->ni = ni;
}

int oracle_calculate_dpf_f64(const float* FP, const float* FX, const float* rms,
                             int64_t n_sky, int n_ifo, int64_t n_pix,
                             double gamma_regulator, double network_energy_threshold,
                             const int64_t* valid, int64_t n_valid, int n_threads,
                             double* out_regulator) {
  if (n_ifo < 1 || n_ifo > ORC_MAXIFO || n_pix < 0 || n_sky < 1) return ORC_BAD_SHAPE;
  set_threads(n_threads);
  int64_t n_pass = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : n_pass)
  for (int64_t k = 0; k < n_valid; ++k) {
    const int64_t l = valid[k];
    double NI = 0;
    int64_t NN = 0;
    for (int64_t p = 0; p < n_pix; ++p) {
      dpf64_t d;
      dpf_pixel64(FP + l * n_ifo, FX + l * n_ifo, rms + p * n_ifo, n_ifo, &d);
      NI += d.fx / (d.ni + 1e-9);
      NN += d.fp > 0.0 ? 1 : 0;
    }
    if (sqrt(NI / ((double)NN + 0.01)) > gamma_regulator) n_pass += 1;
  }
  double FF = (double)n_valid, ff = (double)n_pass;
  *out_regulator = (FF * FF / (ff * ff + 1.e-9) - 1) * network_energy_threshold;
  return ORC_OK;
}

static inline int scan_sky64(int I, int64_t P, int64_t l, const float* FP, const float* FX,
                             const float* rms, const float* td00, const float* td90,
                             int n_delay, int64_t n_sky, const int32_t* ml, double rr, double RR,
                             double netCC, double ethr, double* stats, double* best,
                             double* cr_all) {
  const int off = n_delay / 2;
  int row[ORC_MAXIFO];
  for (int i = 0; i < I; ++i) {
    int d = ml[(int64_t)i * n_sky + l] + off;
    if (d < 0 || d >= n_delay) return ORC_BAD_DELAY;
    row[i] = d;
  }
  double EE = 0, LL = 0, Lr = 0, EC = 0, GN = 0, RN = 0, NNc = 0, ee = 0, ffw = 0, FFw = 0;
  int64_t Mo = 0;
  for (int64_t j = 0; j < P; ++j) {
    double v0[ORC_MAXIFO], v9[ORC_MAXIFO];
    for (int i = 0; i < I; ++i) {
      v0[i] = td00[((int64_t)row[i] * I + i) * P + j];
      v9[i] = td90[((int64_t)row[i] * I + i) * P + j];
    }
    double aa = 0, AA = 0;
    for (int i = 0; i < I; ++i) { aa += v0[i] * v0[i]; AA += v9[i] * v9[i]; }
    double e = aa + AA + 1e-12;
    int mk = e > ethr ? 1 : 0;
    double et = mk ? e : 0.0;
    EE += et;
    dpf64_t d;
    dpf_pixel64(FP + l * I, FX + l * I, rms + j * I, I, &d);
    double xp = 0, XP = 0, xx = 0, XX = 0;
    for (int i = 0; i < I; ++i) {
      xp += v0[i] * d.f[i]; XP += v9[i] * d.f[i];
      xx += v0[i] * d.F[i]; XX += v9[i] * d.F[i];
    }
    double g = sqrt(d.ni * (xp * xp + XP * XP) / (et + 1e-9)) * rr - d.fp;
    g = g > 0 ? g : 0;
    double fd = mk / (d.fp + g + 1e-9);
    double h = xp * fd, Hh = XP * fd;
    h = h * h + Hh * Hh;
    double H2 = xx * xx + XX * XX;
    double G = sqrt(H2 / (h + 1e-9)) * (0.1 + RR / (et + 1e-9)) - d.fx;
    G = G > 0 ? G : 0;
    double Gd = mk / (d.fx + G + 1e-9);
    double au = xp * fd, AU = XP * fd, av = xx * Gd, AV = XX * Gd;
    Mo += mk;
    double msk = fd * d.fp + Gd * d.fx + mk - 1.0;
    double s[ORC_MAXIFO], S[ORC_MAXIFO];
    for (int i = 0; i < I; ++i) { s[i] = d.f[i] * au + d.F[i] * av; S[i] = d.f[i] * AU + d.F[i] * AV; }
    double a2 = 0, A2 = 0, aA = 0;
    for (int i = 0; i < I; ++i) { a2 += s[i] * s[i]; A2 += S[i] * S[i]; aA += s[i] * S[i]; }
    double osi = aA * 2.0, oco = a2 - A2;
    double onn = sqrt(oco * oco + osi * osi);
    double occ = oco / (onn + 1e-21);
    double sgn = osi > 0 ? 1.0 : -1.0;
    osi = sqrt((1.0 - occ) / 2.0);
    oco = sqrt((1.0 + occ) / 2.0) * sgn;
    double c = 0, C = 0, ss = 0, SS = 0, r0 = 0, R0 = 0, xs = 0, XS = 0;
    for (int i = 0; i < I; ++i) {
      double s_ = s[i] * oco + S[i] * osi, x_ = v0[i] * oco + v9[i] * osi;
      double S_ = S[i] * oco - s[i] * osi, X_ = v9[i] * oco - v0[i] * osi;
      double a = s_ * x_, A = S_ * X_;
      xs += a; XS += A; c += a * a; C += A * A; ss += s_ * s_; SS += S_ * S_;
      r0 += (s[i] - v0[i]) * (s[i] - v0[i]); R0 += (S[i] - v9[i]) * (S[i] - v9[i]);
    }
    int mks = msk >= 0 ? 1 : 0;
    c = c / (xs * xs + 1e-9);
    C = C / (XS * XS + 1e-9);
    double ll = mks * (ss + SS);
    double ec = mks * (ss * (1.0 - c) + SS * (1.0 - C));
    double gn = mks * 2.0 * msk;
    double rn = mks * (r0 + R0);
    Lr += ll * ec / (2.0 * fabs(ec) + rn + gn + 1e-9);
    LL += ll; EC += ec; GN += gn; RN += rn; NNc += ec > 1e-9 ? 1.0 : 0.0;
    if (msk > 0) { ee += et; ffw += d.fp * et; FFw += d.fx * et; }
  }
  double Eo = EE / 2.0, Cr = 2.0 * Lr / (LL + 1e-9), No = (GN + RN) / 2.0;
  double CH = No / ((double)(I * Mo) + sqrt((double)Mo));
  double ccor = CH > 1.0 ? CH : 1.0;
  double corr = EC / (EC + No * ccor - (double)(Mo * (I - 1)));
  if (cr_all) cr_all[l] = Cr;
  if (!isfinite(Cr) || Cr < netCC) return ORC_OK;
  double Lk = Eo > 0 ? Eo - No : 0.0;
  double AA = Lk * corr;
  ffw = ee > 0 ? ffw / ee : 0.0;
  FFw = ee > 0 ? FFw / ee : 0.0;
  stats[0 * n_sky + l] = sqrt(ffw + FFw);
  stats[1 * n_sky + l] = ffw > 0 ? sqrt(FFw / ffw) : 0.0;
  stats[2 * n_sky + l] = Eo - No;
  stats[3 * n_sky + l] = No;
  stats[4 * n_sky + l] = EC;
  stats[5 * n_sky + l] = corr;
  stats[6 * n_sky + l] = AA;
  stats[7 * n_sky + l] = CH;
  stats[8 * n_sky + l] = ccor;
  stats[9 * n_sky + l] = Cr;
  stats[10 * n_sky + l] = NNc;
  best[l] = AA;
  return ORC_OK;
}

int oracle_scan_sky_f64(int n_ifo, int64_t n_pix, int64_t n_sky, const float* FP, const float* FX,
                        const float* rms, const float* td00, const float* td90, int n_delay,
                        const int32_t* ml, const double* REG, double netCC,
                        double network_energy_threshold, const int64_t* valid, int64_t n_valid,
                        int n_threads, double* stats, int64_t* l_max, double* sky_stat_max,
                        double* cr_all) {
  if (n_ifo < 1 || n_ifo > ORC_MAXIFO || n_pix < 0 || n_sky < 1 || n_valid < 1 || n_delay < 1)
    return ORC_BAD_SHAPE;
  set_threads(n_threads);
  memset(stats, 0, sizeof(double) * N_STATS * (size_t)n_sky);
  double* best = (double*)malloc(sizeof(double) * (size_t)n_sky);
  if (!best) return ORC_BAD_SHAPE;
  for (int64_t l = 0; l < n_sky; ++l) best[l] = -1.e12;
  int err = ORC_OK;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t k = 0; k < n_valid; ++k) {
    int e = scan_sky64(n_ifo, n_pix, valid[k], FP, FX, rms, td00, td90, n_delay, n_sky, ml,
                       REG[0], REG[1], netCC, network_energy_threshold, stats, best, cr_all);
    if (e) {
#pragma omp atomic write
      err = e;
    }
  }
  if (err == ORC_OK) {
    double cur = 0.0;
    int64_t lm = valid[0];
    for (int64_t k = 0; k < n_valid; ++k)
      if (best[valid[k]] >= cur) { cur = best[valid[k]]; lm = valid[k]; }
    *l_max = lm; *sky_stat_max = cur;
  }
  free(best);
  return err;
}

/* Every per-pixel quantity of one direction l (float32 reference arithmetic),
 * for the statistics at the sky maximum (sky_statistics.py:94-133): the
 * delayed data v0/v9 (I x P), the DPF vectors f/F (P x I) and norms fp/fx/ni,
 * the thresholded energy et and mask mk (load_data_from_td), the float mask
 * msk and signal s/S (I x P, avx_GW_ps), the packet energies ee/EE and
 * rotation osi/oco (avx_ort_ps), and ec/gn/rn (avx_stat_ps). */
int oracle_direction_pixels_f32(int n_ifo, int64_t n_pix, int64_t l, const float* FP,
                                const float* FX, const float* rms, const float* td00,
                                const float* td90, int n_delay, int64_t n_sky, const int32_t* ml,
                                const float* REG, double network_energy_threshold,
                                float* v0o, float* v9o, float* fo, float* Fo, float* fpo, float* fxo,
                                float* nio, float* eto, int32_t* mko, float* msko, float* so,
                                float* So, float* eeo, float* EEo, float* osio, float* ocoo,
                                float* eco, float* gno, float* rno) {
  const int I = n_ifo;
  const int64_t P = n_pix;
  if (I < 1 || I > ORC_MAXIFO || P < 0 || n_sky < 1 || l < 0 || l >= n_sky) return ORC_BAD_SHAPE;
  const int off = n_delay / 2;
  int row[ORC_MAXIFO];
  for (int i = 0; i < I; ++i) {
    int d = ml[(int64_t)i * n_sky + l] + off;
    if (d < 0 || d >= n_delay) return ORC_BAD_DELAY;
    row[i] = d;
  }
  const float ethr32 = (float)network_energy_threshold;
  for (int64_t j = 0; j < P; ++j) {
    float v0[ORC_MAXIFO], v9[ORC_MAXIFO];
    for (int i = 0; i < I; ++i) {
      v0[i] = td00[((int64_t)row[i] * I + i) * P + j];
      v9[i] = td90[((int64_t)row[i] * I + i) * P + j];
      v0o[i * P + j] = v0[i];
      v9o[i * P + j] = v9[i];
    }
    dpf32_t d;
    dpf_pixel32(FP + l * I, FX + l * I, rms + j * I, I, &d);
    pix32_t q;
    pixel32(I, v0, v9, &d, REG[0], REG[1], ethr32, &q);
    for (int i = 0; i < I; ++i) {
      fo[j * I + i] = d.f[i];
      Fo[j * I + i] = d.F[i];
      so[i * P + j] = q.s[i];
      So[i * P + j] = q.S[i];
    }
    fpo[j] = d.fp; fxo[j] = d.fx; nio[j] = d.ni;
    eto[j] = q.et; mko[j] = q.mk; msko[j] = q.msk;
    eeo[j] = q.ee; EEo[j] = q.EE; osio[j] = q.osi; ocoo[j] = q.oco;
    eco[j] = q.ec; gno[j] = q.gn; rno[j] = q.rn;
  }
  return ORC_OK;
}
