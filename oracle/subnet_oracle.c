/* CPU restatement of the sub-network-cut sky loop, optimze_sky_loc_from_td
 * (pycwb/modules/super_cluster_native/sub_net_cut.py:404-517) with its helpers
 * sse_like_ps (:728-742) and _dpf_np_loops_vec_into (:521-563).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU kernel and a timed CPU
 * baseline.  Never linked into the product.
 *
 * The float32 form follows the reference run with NumPy scalar semantics (the
 * way tests/golden/make_golden.py executes it): every float32 operation is
 * rounded to float32, and Python integers (the pixel counts m, m_cut) mix
 * into float32 expressions without promotion.  The float64 form is the
 * yardstick for error figures. */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define SUB_MAXIFO 8

typedef struct {
  float f[SUB_MAXIFO], F[SUB_MAXIFO];
} subdpf32_t;

/* _dpf_np_loops_vec_into for one pixel (sub_net_cut.py:521-563): the DPF
 * rotation of f = r F+, F = r Fx and the orthogonalisation of F against f. */
static inline void sub_dpf32(const float* Fp, const float* Fx, const float* r, int I,
                             subdpf32_t* o) {
  float f[SUB_MAXIFO], F[SUB_MAXIFO];
  for (int j = 0; j < I; ++j) { f[j] = r[j] * Fp[j]; F[j] = r[j] * Fx[j]; }
  float ff = 0.f, FF = 0.f, fF = 0.f;
  for (int j = 0; j < I; ++j) { ff += f[j] * f[j]; FF += F[j] * F[j]; fF += F[j] * f[j]; }
  const float si2 = 2.0f * fF, co2 = ff - FF, AP = ff + FF;
  const float nn = sqrtf(co2 * co2 + si2 * si2);
  const float cc = co2 / (nn + 1e-9f);
  const float fp = (AP + nn) / 2.0f;
  const float si = sqrtf((1.0f - cc) / 2.0f);
  const float cq = sqrtf((1.0f + cc) / 2.0f);
  const float co = si2 > 0.0f ? cq : -cq;
  for (int j = 0; j < I; ++j) {
    const float a = f[j] * co + F[j] * si, b = F[j] * co - f[j] * si;
    f[j] = a; F[j] = b;
  }
  float fFn = 0.f;
  for (int j = 0; j < I; ++j) fFn += f[j] * F[j];
  fFn = fFn / (fp + 1e-9f);
  for (int j = 0; j < I; ++j) { F[j] -= f[j] * fFn; o->f[j] = f[j]; o->F[j] = F[j]; }
}

/* np.dot of two float32 vectors as NumPy evaluates it (checked against
 * NumPy on 20,000 random 3-vectors): float32 products, summed in float64,
 * rounded to float32 once. */
static inline float dot32(const float* a, const float* b, int I) {
  double s = 0.0;
  for (int j = 0; j < I; ++j) s += (double)(a[j] * b[j]);
  return (float)s;
}

/* sse_like_ps (:728-742): projected energy of (am, AM) on the DPF vectors */
static inline float sse_like32(const float* f, const float* F, const float* am, const float* AM,
                               int I) {
  float xp = dot32(f, am, I), XP = dot32(f, AM, I);
  float xx = dot32(F, am, I), XX = dot32(F, AM, I);
  const float gp = dot32(f, f, I) + 1e-12f, gx = dot32(F, F, I) + 1e-12f;
  xp = xp * xp + XP * XP;
  xx = xx * xx + XX * XX;
  return xp / gp + xx / gx;
}

/* out[8] = (l_max, stat, Em, Am, lm, Vm, suball, EE) as the reference returns */
int oracle_subnet_sky_f32(int I, int64_t P, int64_t n_sky, const float* FP, const float* FX,
                          const float* rms, const float* td00, const float* td90, int n_delay,
                          const int32_t* ml, float thr, double e2or, double subcut, double* out) {
  if (I < 1 || I > SUB_MAXIFO || P < 0 || n_sky < 1 || n_delay < 1) return 1;
  const float Es = (float)(2.0 * e2or);                         /* :407 */
  const int offset = n_delay / 2;                               /* :409 */
  int64_t l_max = 0, lm = 0, Vm = 0;
  float stat = 0.f, Em = 0.f, Am = 0.f, suball = 0.f, EE = 0.f, AA_max = 0.f;
  for (int64_t l = 0; l < n_sky; ++l) {
    float m_gt = 0.f, Eo_gt = 0.f, Ls_gt = 0.f, Ln_gt = 0.f, Eo_ge = 0.f, Ls_ge = 0.f, Ln_ge = 0.f;
    int64_t m = 0;
    for (int64_t j = 0; j < P; ++j) {                           /* :436-465 */
      float rE = 0.f, em = 0.f;
      for (int i = 0; i < I; ++i) {
        const int d = ml[(int64_t)i * n_sky + l] + offset;
        if (d < 0 || d >= n_delay) return 2;
        const float a = td00[((int64_t)d * I + i) * P + j], b = td90[((int64_t)d * I + i) * P + j];
        const float de = a * a + b * b;
        rE += de;
        if (de > em) em = de;
      }
      const float sub = rE - em;
      if (rE >= thr) {
        Eo_ge += rE; Ls_ge += sub;
        if (sub > Es) Ln_ge += rE;
        ++m;
      }
      if (rE > thr) {
        m_gt += 1.0f; Eo_gt += rE; Ls_gt += sub;
        if (sub > Es) Ln_gt += rE;
      }
    }
    const float Eo_cut = Eo_gt + 0.01f;                         /* :467 */
    const int64_t m_cut = (int64_t)(2.0f * m_gt + 0.01f);       /* :468 */
    float aa = Ls_gt * Ln_gt / (Eo_cut - Ls_gt);                /* :469 */
    if (subcut >= 0.0 &&
        (aa - (float)m_cut) / (aa + (float)m_cut + 1e-16f) < (float)subcut)  /* :470 */
      continue;
    const float Eo = Eo_ge, Ls = Ls_ge, Ln = Ln_ge;
    if (Eo <= 0.f) continue;                                    /* :488 */
    float Lo = 0.f;
    for (int64_t j = 0; j < P; ++j) {                           /* :474-497: pixels >= thr, in order */
      float r[SUB_MAXIFO], am[SUB_MAXIFO], AM[SUB_MAXIFO], Fp[SUB_MAXIFO], Fx[SUB_MAXIFO];
      float rE = 0.f;
      for (int i = 0; i < I; ++i) {
        const int d = ml[(int64_t)i * n_sky + l] + offset;
        am[i] = td00[((int64_t)d * I + i) * P + j];
        AM[i] = td90[((int64_t)d * I + i) * P + j];
        rE += am[i] * am[i] + AM[i] * AM[i];
      }
      if (rE < thr) continue;
      for (int i = 0; i < I; ++i) {
        r[i] = rms[j * I + i];
        Fp[i] = FP[l * I + i];
        Fx[i] = FX[l * I + i];
      }
      subdpf32_t o;
      sub_dpf32(Fp, Fx, r, I, &o);
      Lo += sse_like32(o.f, o.F, am, AM, I);
    }
    const float mf = (float)m;
    const float AA = aa / (fabsf(aa) + fabsf(Eo - Lo) + 2.0f * mf * (Eo - Ln) / Eo);  /* :503 */
    float ee = Ls * Eo / (Eo - Ls);                             /* :504 */
    const float emv = fabsf(Eo - Lo) + 2.0f * mf;               /* :505 */
    ee = ee / (ee + emv);                                       /* :506 */
    const float aa2 = (aa - mf) / (aa + mf);                    /* :507 */
    if (AA > AA_max) {                                          /* :508-517 */
      AA_max = AA; l_max = l; stat = AA; Em = Eo; Am = aa2; lm = l; Vm = m; suball = ee; EE = emv;
    }
  }
  out[0] = (double)l_max; out[1] = stat; out[2] = Em; out[3] = Am;
  out[4] = (double)lm; out[5] = (double)Vm; out[6] = suball; out[7] = EE;
  return 0;
}

/* the same loop in float64 (yardstick) */
int oracle_subnet_sky_f64(int I, int64_t P, int64_t n_sky, const float* FP, const float* FX,
                          const float* rms, const float* td00, const float* td90, int n_delay,
                          const int32_t* ml, float thr, double e2or, double subcut, double* out) {
  if (I < 1 || I > SUB_MAXIFO || P < 0 || n_sky < 1 || n_delay < 1) return 1;
  const double Es = 2.0 * e2or, th = (double)thr;
  const int offset = n_delay / 2;
  int64_t l_max = 0, lm = 0, Vm = 0;
  double stat = 0, Em = 0, Am = 0, suball = 0, EE = 0, AA_max = 0;
  for (int64_t l = 0; l < n_sky; ++l) {
    double m_gt = 0, Eo_gt = 0, Ls_gt = 0, Ln_gt = 0, Eo_ge = 0, Ls_ge = 0, Ln_ge = 0;
    int64_t m = 0;
    for (int64_t j = 0; j < P; ++j) {
      double rE = 0, em = 0;
      for (int i = 0; i < I; ++i) {
        const int d = ml[(int64_t)i * n_sky + l] + offset;
        if (d < 0 || d >= n_delay) return 2;
        const double a = td00[((int64_t)d * I + i) * P + j], b = td90[((int64_t)d * I + i) * P + j];
        const double de = a * a + b * b;
        rE += de;
        if (de > em) em = de;
      }
      const double sub = rE - em;
      if (rE >= th) { Eo_ge += rE; Ls_ge += sub; if (sub > Es) Ln_ge += rE; ++m; }
      if (rE > th) { m_gt += 1.0; Eo_gt += rE; Ls_gt += sub; if (sub > Es) Ln_gt += rE; }
    }
    const double Eo_cut = Eo_gt + 0.01;
    const int64_t m_cut = (int64_t)(2.0 * m_gt + 0.01);
    double aa = Ls_gt * Ln_gt / (Eo_cut - Ls_gt);
    if (subcut >= 0.0 && (aa - (double)m_cut) / (aa + (double)m_cut + 1e-16) < subcut) continue;
    const double Eo = Eo_ge, Ls = Ls_ge, Ln = Ln_ge;
    if (Eo <= 0) continue;
    double Lo = 0;
    for (int64_t j = 0; j < P; ++j) {
      double am[SUB_MAXIFO], AM[SUB_MAXIFO], f[SUB_MAXIFO], F[SUB_MAXIFO];
      double rE = 0;
      for (int i = 0; i < I; ++i) {
        const int d = ml[(int64_t)i * n_sky + l] + offset;
        am[i] = td00[((int64_t)d * I + i) * P + j];
        AM[i] = td90[((int64_t)d * I + i) * P + j];
        rE += am[i] * am[i] + AM[i] * AM[i];
      }
      if (rE < th) continue;
      for (int i = 0; i < I; ++i) {
        f[i] = (double)rms[j * I + i] * FP[l * I + i];
        F[i] = (double)rms[j * I + i] * FX[l * I + i];
      }
      double ff = 0, FF = 0, fF = 0;
      for (int i = 0; i < I; ++i) { ff += f[i] * f[i]; FF += F[i] * F[i]; fF += F[i] * f[i]; }
      const double si2 = 2 * fF, co2 = ff - FF, AP = ff + FF;
      const double nn = sqrt(co2 * co2 + si2 * si2), cc = co2 / (nn + 1e-9), fp = (AP + nn) / 2;
      const double si = sqrt((1 - cc) / 2), cq = sqrt((1 + cc) / 2), co = si2 > 0 ? cq : -cq;
      for (int i = 0; i < I; ++i) {
        const double a = f[i] * co + F[i] * si, b = F[i] * co - f[i] * si;
        f[i] = a; F[i] = b;
      }
      double fFn = 0;
      for (int i = 0; i < I; ++i) fFn += f[i] * F[i];
      fFn /= (fp + 1e-9);
      for (int i = 0; i < I; ++i) F[i] -= f[i] * fFn;
      double xp = 0, XP = 0, xx = 0, XX = 0, gp = 0, gx = 0;
      for (int i = 0; i < I; ++i) {
        xp += f[i] * am[i]; XP += f[i] * AM[i]; xx += F[i] * am[i]; XX += F[i] * AM[i];
        gp += f[i] * f[i]; gx += F[i] * F[i];
      }
      gp += 1e-12; gx += 1e-12;
      Lo += (xp * xp + XP * XP) / gp + (xx * xx + XX * XX) / gx;
    }
    const double mf = (double)m;
    const double AA = aa / (fabs(aa) + fabs(Eo - Lo) + 2 * mf * (Eo - Ln) / Eo);
    double ee = Ls * Eo / (Eo - Ls);
    const double emv = fabs(Eo - Lo) + 2 * mf;
    ee = ee / (ee + emv);
    const double aa2 = (aa - mf) / (aa + mf);
    if (AA > AA_max) {
      AA_max = AA; l_max = l; stat = AA; Em = Eo; Am = aa2; lm = l; Vm = m; suball = ee; EE = emv;
    }
  }
  out[0] = (double)l_max; out[1] = stat; out[2] = Em; out[3] = Am;
  out[4] = (double)lm; out[5] = (double)Vm; out[6] = suball; out[7] = EE;
  return 0;
}
