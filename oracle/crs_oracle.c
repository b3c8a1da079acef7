/*
 * CPU oracle for the wdot path (TEST INFRASTRUCTURE -- never shipped, never
 * measured as the product; only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py load it).
 *
 * A table-driven restatement, in plain C at FP64, of the straight-line code
 * create_rate_subs emits.  Every expression keeps the emitted operand order
 * so that, compiled with -ffp-contract=off against the same libm, results
 * are bit-identical to the reference's own emitted C (pinned by the golden
 * vectors in tests/golden/).  Tables come from the blob built by
 * create_rate_subs_gb300/tables.py.
 *
 *   oracle_eval_conc         rate_subs.py:1295-1391
 *   oracle_eval_rxn_rates    rate_subs.py:283-704 (rate constants :20-135)
 *   oracle_get_rxn_pres_mod  rate_subs.py:757-1073
 *   oracle_eval_spec_rates   rate_subs.py:1121-1235
 *   oracle_thermo            eval_h / eval_u / eval_cv / eval_cp,
 *                            rate_subs.py:1497-1776
 *   oracle_eval_conc_rho     rate_subs.py:1396-1490
 *   oracle_dydt              dydt, constant pressure rate_subs.py:1829-1946
 *                            and constant volume :1951-2067 (the constant
 *                            volume branch as its emitter means it: the
 *                            emitted text misses a comma at :1967-1969 and a
 *                            '+' at :2024-2025 and does not compile)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { RATE_CONST = 0, RATE_EXP = 1, RATE_NEGEXP = 2, RATE_POW = 3, RATE_PLOG = 4,
       RATE_CHEB = 5 };
#define CHEB_MAX 16
enum { PM_THD = 0, PM_FALL_LOW = 1, PM_FALL_HIGH = 2 };
enum { FORM_LINDEMANN = 0, FORM_TROE = 1, FORM_SRI = 2 };

typedef struct {
  int N, R, NREV, NPM, NRATE;
  const double *inv_mw;
  const int32_t *rate_kind, *rate_npow;
  const double *rate_par;
  const int32_t *rx_ptr, *rx_sp, *rx_nint;
  const double *rx_nu;
  const int32_t *px_ptr, *px_sp, *px_nint;
  const double *px_nu;
  const int32_t *rev_idx, *kc_ptr;
  const double *kc_tmid, *kc_lo, *kc_hi, *kc_pref;
  const int32_t *pm_idx, *pm_rxn, *pm_kind, *pm_form, *pm_sp, *pm_eff_ptr,
      *pm_eff_sp, *pm_k0, *pm_kinf, *pm_troe_t2, *pm_sri_de;
  const double *pm_eff_val, *pm_troe, *pm_sri;
  const int32_t *nu_ptr, *nu_sp;
  const double *nu_val;
  const double *sp_mw, *sp_tmid, *sp_lo, *sp_hi;
  const int32_t *rate_aux, *plog_ptr, *plog_row, *cheb_ptr, *cheb_nt, *cheb_np;
  const double *plog_p, *plog_lp, *plog_dlp, *cheb_par, *cheb_tp;
  unsigned char *blob; /* owned copy */
} omech;

static const void *section(const unsigned char *b, size_t n, const char *name,
                           uint32_t want_dt, uint64_t *count) {
  uint32_t nsec;
  memcpy(&nsec, b + 12, 4);
  for (uint32_t i = 0; i < nsec; ++i) {
    const unsigned char *e = b + 16 + (size_t)i * 48;
    char nm[25];
    uint32_t dt;
    uint64_t cnt, off;
    memcpy(nm, e, 24);
    nm[24] = 0;
    memcpy(&dt, e + 24, 4);
    memcpy(&cnt, e + 32, 8);
    memcpy(&off, e + 40, 8);
    if (strcmp(nm, name) == 0) {
      size_t es = (dt == 1 || dt == 3) ? 8 : (dt == 2 ? 4 : 1);
      if (dt != want_dt || off + cnt * es > n) return NULL;
      if (count) *count = cnt;
      return b + off;
    }
  }
  return NULL;
}

void oracle_free(omech *m) {
  if (!m) return;
  free(m->blob);
  free(m);
}

int oracle_load(const void *blob, size_t n, omech **out) {
  if (!blob || !out || n < 16 || memcmp(blob, "CRSMECH1", 8) != 0) return 1;
  omech *m = (omech *)calloc(1, sizeof(omech));
  m->blob = (unsigned char *)malloc(n);
  memcpy(m->blob, blob, n);
  const unsigned char *b = m->blob;
  uint64_t c;
  const int64_t *dims = (const int64_t *)section(b, n, "dims", 3, &c);
  if (!dims || c < 5) { oracle_free(m); return 2; }
  m->N = (int)dims[0]; m->R = (int)dims[1]; m->NREV = (int)dims[2];
  m->NPM = (int)dims[3]; m->NRATE = (int)dims[4];
#define F64(field, nm) m->field = (const double *)section(b, n, nm, 1, NULL)
#define I32(field, nm) m->field = (const int32_t *)section(b, n, nm, 2, NULL)
  F64(inv_mw, "sp_inv_mw");
  I32(rate_kind, "rate_kind"); I32(rate_npow, "rate_npow"); F64(rate_par, "rate_par");
  I32(rx_ptr, "rx_ptr"); I32(rx_sp, "rx_sp"); I32(rx_nint, "rx_nint"); F64(rx_nu, "rx_nu");
  I32(px_ptr, "px_ptr"); I32(px_sp, "px_sp"); I32(px_nint, "px_nint"); F64(px_nu, "px_nu");
  I32(rev_idx, "rev_idx"); I32(kc_ptr, "kc_ptr");
  F64(kc_tmid, "kc_tmid"); F64(kc_lo, "kc_lo"); F64(kc_hi, "kc_hi"); F64(kc_pref, "kc_pref");
  I32(pm_idx, "pm_idx"); I32(pm_rxn, "pm_rxn"); I32(pm_kind, "pm_kind");
  I32(pm_form, "pm_form"); I32(pm_sp, "pm_sp"); I32(pm_eff_ptr, "pm_eff_ptr");
  I32(pm_eff_sp, "pm_eff_sp"); I32(pm_k0, "pm_k0"); I32(pm_kinf, "pm_kinf");
  I32(pm_troe_t2, "pm_troe_t2"); I32(pm_sri_de, "pm_sri_de");
  F64(pm_eff_val, "pm_eff_val"); F64(pm_troe, "pm_troe"); F64(pm_sri, "pm_sri");
  I32(nu_ptr, "nu_ptr"); I32(nu_sp, "nu_sp"); F64(nu_val, "nu_val");
  F64(sp_mw, "sp_mw"); F64(sp_tmid, "sp_tmid"); F64(sp_lo, "sp_lo"); F64(sp_hi, "sp_hi");
  I32(rate_aux, "rate_aux"); I32(plog_ptr, "plog_ptr"); I32(plog_row, "plog_row");
  I32(cheb_ptr, "cheb_ptr"); I32(cheb_nt, "cheb_nt"); I32(cheb_np, "cheb_np");
  F64(plog_p, "plog_p"); F64(plog_lp, "plog_lp"); F64(plog_dlp, "plog_dlp");
  F64(cheb_par, "cheb_par"); F64(cheb_tp, "cheb_tp");
#undef F64
#undef I32
  if (!m->inv_mw || !m->rate_kind || !m->rx_ptr || !m->px_ptr || !m->rev_idx ||
      !m->pm_idx || !m->nu_ptr || !m->kc_ptr || !m->pm_eff_ptr || !m->sp_mw ||
      !m->sp_tmid || !m->sp_lo || !m->sp_hi || !m->rate_aux || !m->plog_ptr ||
      !m->cheb_ptr) {
    oracle_free(m);
    return 3;
  }
  *out = m;
  return 0;
}

int oracle_dims(const omech *m, int64_t *out5) {
  out5[0] = m->N; out5[1] = m->R; out5[2] = m->NREV; out5[3] = m->NPM;
  out5[4] = m->NRATE;
  return 0;
}

/* rxn_rate_const as a standalone expression (rate_subs.py:60-135). */
static double rate_const(const omech *m, int row, double T, double logT) {
  const double *p = m->rate_par + 4 * row; /* A, logA, b, Ta */
  double k;
  switch (m->rate_kind[row]) {
    case RATE_CONST: return p[0];
    case RATE_EXP: return exp(p[1] + p[2] * logT - (p[3] / T));
    case RATE_NEGEXP: return p[0] * exp(p[2] * logT - (p[3] / T));
    default:
      k = p[0];
      for (int i = 0; i < m->rate_npow[row]; ++i) k = k * T;
      return k;
  }
}

/* PLOG (rate_subs.py:444-485) and Chebyshev (rate_subs.py:136-223) forward
 * rate constants, in the emitted order: PLOG branches on the pressures as
 * printed with %.4e and interpolates log-linearly in ln P; Chebyshev forms
 * the reduced T and P, the pressure dot products by the Chebyshev
 * recursion, the temperature sum and 10^kf. */
static double pdep_kf(const omech *m, int row, double T, double logT, double pres) {
  const int a = m->rate_aux[row];
  if (m->rate_kind[row] == RATE_PLOG) {
    const int e0 = m->plog_ptr[a], e1 = m->plog_ptr[a + 1];
    if (pres <= m->plog_p[e0]) return rate_const(m, m->plog_row[e0], T, logT);
    for (int e = e0; e < e1 - 1; ++e)
      if ((pres > m->plog_p[e]) && (pres <= m->plog_p[e + 1])) {
        double kf = log(rate_const(m, m->plog_row[e], T, logT));
        double kf2 = log(rate_const(m, m->plog_row[e + 1], T, logT));
        return exp(kf + (kf2 - kf) * (log(pres) - m->plog_lp[e]) / m->plog_dlp[e]);
      }
    if (pres > m->plog_p[e1 - 1]) return rate_const(m, m->plog_row[e1 - 1], T, logT);
    return NAN;
  }
  const double *tp = m->cheb_tp + 4 * a;
  const int nt = m->cheb_nt[a], np = m->cheb_np[a];
  const double *c = m->cheb_par + m->cheb_ptr[a];
  double Tred = ((2.0 / T) - tp[0]) / tp[1];
  double Pred = (2.0 * log10(pres) - tp[2]) / tp[3];
  double dp[CHEB_MAX];
  for (int i = 0; i < nt; ++i) dp[i] = c[i * np] + Pred * c[i * np + 1];
  double ct0 = 1, ct1 = Pred;
  int upd = 1;
  for (int j = 2; j < np; ++j) {
    if (upd) {
      ct0 = 2 * Pred * ct1 - ct0;
      for (int i = 0; i < nt; ++i) dp[i] += c[i * np + j] * ct0;
    } else {
      ct1 = 2 * Pred * ct0 - ct1;
      for (int i = 0; i < nt; ++i) dp[i] += c[i * np + j] * ct1;
    }
    upd = !upd;
  }
  ct0 = 1;
  ct1 = Tred;
  double kf = dp[0] + Tred * dp[1];
  upd = 1;
  for (int i = 2; i < nt; ++i) {
    if (upd) {
      ct0 = 2 * Tred * ct1 - ct0;
      kf += dp[i] * ct0;
    } else {
      ct1 = 2 * Tred * ct0 - ct1;
      kf += dp[i] * ct1;
    }
    upd = !upd;
  }
  return pow(10.0, kf);
}

/* Product of concentrations C[k]^nu over one side, left to right, integral
 * nu as repeated multiplication and others as pow (rate_subs.py:487-501,
 * 668-681).  *have = 0 if the side printed no factor. */
static double conc_product(const int32_t *sp, const int32_t *nint,
                           const double *nu, int a, int b, const double *C,
                           int *have) {
  double p = 0.0;
  int first = 1;
  for (int j = a; j < b; ++j) {
    if (nint[j] >= 0) {
      for (int t = 0; t < nint[j]; ++t) {
        p = first ? C[sp[j]] : p * C[sp[j]];
        first = 0;
      }
    } else {
      double f = pow(C[sp[j]], nu[j]);
      p = first ? f : p * f;
      first = 0;
    }
  }
  *have = !first;
  return p;
}

/* Kc exponent of one reversible reaction: sum over T_common groups of
 * (c0 + c1*logT + T*(c2 + T*(c3 + T*(c4 + c5*T))) - c6/T)
 * (rate_subs.py:592-655). */
static double kc_exponent(const omech *m, int j, double T, double logT) {
  double kc = 0.0;
  for (int g = m->kc_ptr[j]; g < m->kc_ptr[j + 1]; ++g) {
    const double *c = (T <= m->kc_tmid[g]) ? m->kc_lo + 7 * g : m->kc_hi + 7 * g;
    double v = (c[0] + c[1] * logT + T * (c[2] + T * (c[3] + T * (c[4] + c[5] * T)))
                - c[6] / T);
    kc = (g == m->kc_ptr[j]) ? v : kc + v;
  }
  return kc;
}

void oracle_eval_rxn_rates(const omech *m, double T, double pres,
                           const double *C, double *fwd, double *rev) {
  double logT = log(T);
  for (int r = 0; r < m->R; ++r) {
    int have;
    double p = conc_product(m->rx_sp, m->rx_nint, m->rx_nu, m->rx_ptr[r],
                            m->rx_ptr[r + 1], C, &have);
    int j = m->rev_idx[r];
    const int pdep = m->rate_kind[r] >= RATE_PLOG;
    if (pdep && j < 0) {
      /* PLOG / Chebyshev print kf first, then C... * kf (:437-448, 503-505) */
      double kf = pdep_kf(m, r, T, logT, pres);
      fwd[r] = have ? p * kf : kf;
    } else if (j >= 0) {
      double kf = pdep ? pdep_kf(m, r, T, logT, pres) : rate_const(m, r, T, logT);
      fwd[r] = have ? p * kf : kf;
      double Kc = kc_exponent(m, j, T, logT);
      Kc = m->kc_pref[j] * exp(Kc);
      double q = conc_product(m->px_sp, m->px_nint, m->px_nu, m->px_ptr[r],
                              m->px_ptr[r + 1], C, &have);
      rev[j] = have ? q * kf / Kc : kf / Kc;
    } else if (!have) {
      fwd[r] = rate_const(m, r, T, logT);
    } else {
      /* irreversible: the rate expression is printed inline after the
       * concentration factors, so its own factors multiply in order */
      const double *a = m->rate_par + 4 * r;
      switch (m->rate_kind[r]) {
        case RATE_CONST: fwd[r] = p * a[0]; break;
        case RATE_EXP: fwd[r] = p * exp(a[1] + a[2] * logT - (a[3] / T)); break;
        case RATE_NEGEXP: fwd[r] = p * a[0] * exp(a[2] * logT - (a[3] / T)); break;
        default:
          p = p * a[0];
          for (int i = 0; i < m->rate_npow[r]; ++i) p = p * T;
          fwd[r] = p;
      }
    }
  }
}

static double third_body(const omech *m, int p, double mix, const double *C) {
  double t = mix;
  for (int e = m->pm_eff_ptr[p]; e < m->pm_eff_ptr[p + 1]; ++e)
    t = t + m->pm_eff_val[e] * C[m->pm_eff_sp[e]];
  return t;
}

void oracle_get_rxn_pres_mod(const omech *m, double T, double pres,
                             const double *C, double *pres_mod) {
  double logT = log(T);
  double mix = pres / (8.31446210e+03 * T);
  for (int p = 0; p < m->NPM; ++p) {
    if (m->pm_kind[p] == PM_THD) {
      pres_mod[p] = third_body(m, p, mix, C);
      continue;
    }
    double thd = 0.0;
    if (m->pm_sp[p] < 0) thd = third_body(m, p, mix, C);
    double k0 = rate_const(m, m->pm_k0[p], T, logT);
    double kinf = rate_const(m, m->pm_kinf[p], T, logT);
    double Pr = (m->pm_sp[p] >= 0) ? k0 * C[m->pm_sp[p]] / kinf : k0 * thd / kinf;
    int low = (m->pm_kind[p] == PM_FALL_LOW);
    double F;
    if (m->pm_form[p] == FORM_TROE) {
      const double *c = m->pm_troe + 5 * p;
      double s = c[0] * exp(-T / c[1]) + c[2] * exp(-T / c[3]);
      if (m->pm_troe_t2[p]) s = s + exp(-c[4] / T);
      double logFcent = log10(fmax(s, 1.0e-300));
      double A = log10(fmax(Pr, 1.0e-300)) - 0.67 * logFcent - 0.4;
      double B = 0.806 - 1.1762 * logFcent - 0.14 * log10(fmax(Pr, 1.0e-300));
      F = pow(10.0, logFcent / (1.0 + A * A / (B * B)));
      pres_mod[p] = low ? F * Pr / (1.0 + Pr) : F / (1.0 + Pr);
    } else if (m->pm_form[p] == FORM_SRI) {
      const double *c = m->pm_sri + 5 * p;
      double X = 1.0 / (1.0 + log10(fmax(Pr, 1.0e-300)) * log10(fmax(Pr, 1.0e-300)));
      F = pow(c[0] * exp(-c[1] / T) + exp(-T / c[2]), X);
      if (m->pm_sri_de[p]) F = F * c[3] * pow(T, c[4]);
      pres_mod[p] = low ? F * Pr / (1.0 + Pr) : F / (1.0 + Pr);
    } else {
      pres_mod[p] = low ? Pr / (1.0 + Pr) : 1.0 / (1.0 + Pr);
    }
  }
}

void oracle_eval_spec_rates(const omech *m, const double *fwd,
                            const double *rev, const double *pres_mod,
                            double *sp_rates, double *dy_N) {
  int N = m->N;
  double *acc = (double *)alloca(sizeof(double) * N);
  char *seen = (char *)alloca(N);
  memset(seen, 0, N);
  for (int r = 0; r < m->R; ++r) {
    int j = m->rev_idx[r], p = m->pm_idx[r];
    for (int e = m->nu_ptr[r]; e < m->nu_ptr[r + 1]; ++e) {
      int k = m->nu_sp[e];
      double nu = m->nu_val[e];
      double a = fabs(nu);
      double t = (j >= 0) ? (fwd[r] - rev[j]) : fwd[r];
      if (a != 1.0) t = a * t;
      if (p >= 0) t = t * pres_mod[p];
      if (!seen[k]) acc[k] = (nu < 0) ? -t : t;
      else acc[k] = (nu < 0) ? acc[k] - t : acc[k] + t;
      seen[k] = 1;
    }
  }
  for (int k = 0; k < N; ++k) {
    double v = seen[k] ? acc[k] : 0.0;
    if (k == N - 1) *dy_N = v;
    else sp_rates[k] = v;
  }
}

void oracle_eval_conc(const omech *m, double T, double pres, const double *y,
                      double *y_N, double *mw_avg, double *rho, double *conc) {
  int N = m->N;
  double s = y[0];
  for (int k = 1; k < N - 1; ++k) s = s + y[k];
  *y_N = (N > 1) ? 1.0 - s : 1.0;
  double mw = 0.0;
  for (int k = 0; k < N - 1; ++k) {
    double t = y[k] * m->inv_mw[k];
    mw = (k == 0) ? t : mw + t;
  }
  mw = (N > 1) ? mw + (*y_N) * m->inv_mw[N - 1] : (*y_N) * m->inv_mw[N - 1];
  *mw_avg = 1.0 / mw;
  *rho = pres * (*mw_avg) / (8.31446210e+03 * T);
  for (int k = 0; k < N - 1; ++k) conc[k] = (*rho) * y[k] * m->inv_mw[k];
  conc[N - 1] = (*rho) * (*y_N) * m->inv_mw[N - 1];
}

static void one_state(const omech *m, int64_t i, const double *T,
                      const double *P, const double *Y, int64_t ld,
                      double *conc_o, double *fwd_o, double *rev_o,
                      double *pm_o, double *wdot_o, double *misc_o) {
  int N = m->N;
  double *y = (double *)alloca(sizeof(double) * (N + 1));
  double *C = (double *)alloca(sizeof(double) * N);
  double *fwd = (double *)alloca(sizeof(double) * (m->R + 1));
  double *rev = (double *)alloca(sizeof(double) * (m->NREV + 1));
  double *pm = (double *)alloca(sizeof(double) * (m->NPM + 1));
  double *sp = (double *)alloca(sizeof(double) * N);
  double y_N, mw_avg, rho;
  for (int k = 0; k < N - 1; ++k) y[k] = Y[(int64_t)k * ld + i];
  oracle_eval_conc(m, T[i], P[i], y, &y_N, &mw_avg, &rho, C);
  oracle_eval_rxn_rates(m, T[i], P[i], C, fwd, rev);
  oracle_get_rxn_pres_mod(m, T[i], P[i], C, pm);
  oracle_eval_spec_rates(m, fwd, rev, pm, sp, &sp[N - 1]);
  if (conc_o) for (int k = 0; k < N; ++k) conc_o[(int64_t)k * ld + i] = C[k];
  if (fwd_o) for (int k = 0; k < m->R; ++k) fwd_o[(int64_t)k * ld + i] = fwd[k];
  if (rev_o) for (int k = 0; k < m->NREV; ++k) rev_o[(int64_t)k * ld + i] = rev[k];
  if (pm_o) for (int k = 0; k < m->NPM; ++k) pm_o[(int64_t)k * ld + i] = pm[k];
  if (wdot_o) for (int k = 0; k < N; ++k) wdot_o[(int64_t)k * ld + i] = sp[k];
  if (misc_o) {
    misc_o[i] = y_N;
    misc_o[ld + i] = mw_avg;
    misc_o[2 * ld + i] = rho;
  }
}

/* Every stage for n SoA states (entry k of state i at [k*ld + i]). */
int oracle_eval(const omech *m, int64_t n, const double *T, const double *P,
                const double *Y, int64_t ld, double *conc, double *fwd,
                double *rev, double *pm, double *wdot, double *misc) {
  if (!m || n < 0 || ld < n) return 1;
  for (int64_t i = 0; i < n; ++i)
    one_state(m, i, T, P, Y, ld, conc, fwd, rev, pm, wdot, misc);
  return 0;
}

/* wdot for n states with OpenMP over states; returns threads used. */
int oracle_wdot_omp(const omech *m, int64_t n, const double *T,
                    const double *P, const double *Y, int64_t ld, double *wdot,
                    int nthreads) {
  int used = 1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
  {
#pragma omp single
    used = omp_get_num_threads();
#pragma omp for schedule(static)
    for (int64_t i = 0; i < n; ++i)
      one_state(m, i, T, P, Y, ld, NULL, NULL, NULL, NULL, wdot, NULL);
  }
#else
  (void)nthreads;
  for (int64_t i = 0; i < n; ++i)
    one_state(m, i, T, P, Y, ld, NULL, NULL, NULL, NULL, wdot, NULL);
#endif
  return used;
}


/* ---- thermodynamic utilities and the ODE right-hand side ---------------- */

#define RU_J 8314.4621 /* chem.RU, J/(kmol K) */

/* Per-species h [J/kg] (which 0), u (1), cv [J/(kg K)] (2), cp (3) at T, in
 * the emitted form: RU/mw times a Horner polynomial whose coefficients are
 * the NASA-7 a_j, divided by 2..5 for h and u (rate_subs.py:1513-1776). */
void oracle_thermo(const omech *m, int which, double T, double *out) {
  for (int k = 0; k < m->N; ++k) {
    const double *a = (T <= m->sp_tmid[k]) ? m->sp_lo + 7 * k : m->sp_hi + 7 * k;
    const double rm = RU_J / m->sp_mw[k];
    double v;
    switch (which) {
      case 0:
        v = rm * (a[5] + T * (a[0] + T * (a[1] / 2.0 + T * (a[2] / 3.0 +
                  T * (a[3] / 4.0 + a[4] / 5.0 * T)))));
        break;
      case 1:
        v = rm * (a[5] + T * (a[0] - 1.0 + T * (a[1] / 2.0 + T * (a[2] / 3.0 +
                  T * (a[3] / 4.0 + a[4] / 5.0 * T)))));
        break;
      case 2:
        v = rm * (a[0] - 1.0 + T * (a[1] + T * (a[2] + T * (a[3] + a[4] * T))));
        break;
      default:
        v = rm * (a[0] + T * (a[1] + T * (a[2] + T * (a[3] + a[4] * T))));
        break;
    }
    out[k] = v;
  }
}

/* eval_conc_rho: concentrations and pressure from density (:1396-1490). */
void oracle_eval_conc_rho(const omech *m, double T, double rho, const double *y,
                          double *y_N, double *mw_avg, double *pres,
                          double *conc) {
  int N = m->N;
  double s = y[0];
  for (int k = 1; k < N - 1; ++k) s = s + y[k];
  *y_N = (N > 1) ? 1.0 - s : 1.0;
  double mw = 0.0;
  for (int k = 0; k < N - 1; ++k) {
    double t = y[k] * m->inv_mw[k];
    mw = (k == 0) ? t : mw + t;
  }
  mw = (N > 1) ? mw + (*y_N) * m->inv_mw[N - 1] : (*y_N) * m->inv_mw[N - 1];
  *mw_avg = 1.0 / mw;
  *pres = rho * 8.31446210e+03 * T / (*mw_avg);
  for (int k = 0; k < N - 1; ++k) conc[k] = rho * y[k] * m->inv_mw[k];
  conc[N - 1] = rho * (*y_N) * m->inv_mw[N - 1];
}

/* dydt for y = [T, Y_0 .. Y_{N-2}] and dy the same; conv = 0: p_or_rho is
 * the pressure (constant pressure, cp and h), conv = 1: the density
 * (constant volume, cv and u). */
void oracle_dydt(const omech *m, int conv, double p_or_rho, const double *y,
                 double *dy) {
  const int N = m->N;
  double *C = (double *)alloca(sizeof(double) * N);
  double *fwd = (double *)alloca(sizeof(double) * (m->R + 1));
  double *rev = (double *)alloca(sizeof(double) * (m->NREV + 1));
  double *pm = (double *)alloca(sizeof(double) * (m->NPM + 1));
  double *c = (double *)alloca(sizeof(double) * N);
  double *e = (double *)alloca(sizeof(double) * N);
  const double T = y[0];
  double y_N, mw_avg, rho, pres;
  if (conv) {
    rho = p_or_rho;
    oracle_eval_conc_rho(m, T, rho, y + 1, &y_N, &mw_avg, &pres, C);
  } else {
    pres = p_or_rho;
    oracle_eval_conc(m, T, pres, y + 1, &y_N, &mw_avg, &rho, C);
  }
  oracle_eval_rxn_rates(m, T, pres, C, fwd, rev);
  oracle_get_rxn_pres_mod(m, T, pres, C, pm);
  double dy_N;
  oracle_eval_spec_rates(m, fwd, rev, pm, dy + 1, &dy_N);
  oracle_thermo(m, conv ? 2 : 3, T, c);
  double avg = 0.0;
  for (int k = 0; k < N - 1; ++k) {
    double t = c[k] * y[k + 1];
    avg = (k == 0) ? t : avg + t;
  }
  avg = (N > 1) ? avg + c[N - 1] * y_N : c[N - 1] * y_N;
  oracle_thermo(m, conv ? 1 : 0, T, e);
  double sum = 0.0;
  for (int k = 0; k < N - 1; ++k) {
    double t = dy[k + 1] * e[k] * m->sp_mw[k];
    sum = (k == 0) ? t : sum + t;
  }
  sum = (N > 1) ? sum + dy_N * e[N - 1] * m->sp_mw[N - 1] : dy_N * e[N - 1] * m->sp_mw[N - 1];
  dy[0] = (-1.0 / (rho * avg)) * sum;
  for (int k = 0; k < N - 1; ++k) dy[k + 1] *= (m->sp_mw[k] / rho);
}

/* SoA batches: y and dy [N][ld], thermo out [N][ld], misc (y_N, mw_avg,
 * pres) [3][ld]. */
int oracle_dydt_batch(const omech *m, int conv, int64_t n, const double *p_or_rho,
                      const double *y, int64_t ld, double *dy) {
  if (!m || n < 0 || ld < n) return 1;
  const int N = m->N;
  double *ys = (double *)malloc(sizeof(double) * 2 * N);
  double *ds = ys + N;
  for (int64_t i = 0; i < n; ++i) {
    for (int k = 0; k < N; ++k) ys[k] = y[(int64_t)k * ld + i];
    oracle_dydt(m, conv, p_or_rho[i], ys, ds);
    for (int k = 0; k < N; ++k) dy[(int64_t)k * ld + i] = ds[k];
  }
  free(ys);
  return 0;
}

int oracle_thermo_batch(const omech *m, int which, int64_t n, const double *T,
                        int64_t ld, double *out) {
  if (!m || n < 0 || ld < n || which < 0 || which > 3) return 1;
  double *v = (double *)malloc(sizeof(double) * m->N);
  for (int64_t i = 0; i < n; ++i) {
    oracle_thermo(m, which, T[i], v);
    for (int k = 0; k < m->N; ++k) out[(int64_t)k * ld + i] = v[k];
  }
  free(v);
  return 0;
}

int oracle_conc_rho_batch(const omech *m, int64_t n, const double *T,
                          const double *rho, const double *Y, int64_t ld,
                          double *misc, double *conc) {
  if (!m || n < 0 || ld < n) return 1;
  const int N = m->N;
  double *y = (double *)malloc(sizeof(double) * 2 * N);
  double *c = y + N;
  for (int64_t i = 0; i < n; ++i) {
    double y_N, mw, p;
    for (int k = 0; k < N - 1; ++k) y[k] = Y[(int64_t)k * ld + i];
    oracle_eval_conc_rho(m, T[i], rho[i], y, &y_N, &mw, &p, c);
    if (conc) for (int k = 0; k < N; ++k) conc[(int64_t)k * ld + i] = c[k];
    if (misc) { misc[i] = y_N; misc[ld + i] = mw; misc[2 * ld + i] = p; }
  }
  free(y);
  return 0;
}
