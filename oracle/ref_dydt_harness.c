/*
 * Batch driver for create_rate_subs' emitted dydt and thermo utilities
 * (TEST INFRASTRUCTURE).
 *
 * Compiled together with the emitted chem_utils.c, rxn_rates.c,
 * rxn_rates_pres_mod.c, spec_rates.c and dydt.c of one mechanism, with
 * -DCONP: the emitted header defines CONV, whose branch of dydt.c does not
 * compile (rate_subs.py:1967-1969 drops a comma, :2024-2025 a '+'), and the
 * constant-pressure branch is selected first when CONP is defined.  This
 * file owns none of the arithmetic; it loops the emitted per-state calls
 * over structure-of-arrays states:
 *
 *   refd_dydt        dydt(t, pres, y, dy)           rate_subs.py:1829-1946
 *   refd_thermo      eval_h / eval_u / eval_cv / eval_cp   :1497-1776
 *   refd_conc_rho    eval_conc_rho                  :1396-1490
 *
 * State layout of dydt (the emitted one): y = [T, Y_0 .. Y_{N-2}], dy the
 * same (dT/dt, dY_k/dt).  SoA here: entry k of state i at [k*ld + i].
 * Sizes come from the build: CRS_NSP.
 */
#include <stdint.h>

#ifndef CRS_NSP
#error "CRS_NSP must be defined"
#endif

void dydt(const double t, const double pres, const double* y, double* dy);
void eval_conc_rho(const double T, const double rho, const double* y,
                   double* y_N, double* mw_avg, double* pres, double* conc);
void eval_h(const double T, double* h);
void eval_u(const double T, double* u);
void eval_cv(const double T, double* cv);
void eval_cp(const double T, double* cp);

int refd_dydt(int64_t n, const double* P, const double* y, int64_t ld,
              double* dy) {
  if (n < 0 || ld < n) return 1;
  for (int64_t i = 0; i < n; ++i) {
    double ys[CRS_NSP], d[CRS_NSP];
    for (int k = 0; k < CRS_NSP; ++k) ys[k] = y[(int64_t)k * ld + i];
    dydt(0.0, P[i], ys, d);
    for (int k = 0; k < CRS_NSP; ++k) dy[(int64_t)k * ld + i] = d[k];
  }
  return 0;
}

/* which: 0 h [J/kg], 1 u, 2 cv [J/(kg K)], 3 cp; out [N][ld]. */
int refd_thermo(int which, int64_t n, const double* T, int64_t ld,
                double* out) {
  if (n < 0 || ld < n || which < 0 || which > 3) return 1;
  for (int64_t i = 0; i < n; ++i) {
    double v[CRS_NSP];
    switch (which) {
      case 0: eval_h(T[i], v); break;
      case 1: eval_u(T[i], v); break;
      case 2: eval_cv(T[i], v); break;
      default: eval_cp(T[i], v); break;
    }
    for (int k = 0; k < CRS_NSP; ++k) out[(int64_t)k * ld + i] = v[k];
  }
  return 0;
}

/* misc (may be NULL): y_N, mw_avg, pres at [0*ld+i], [1*ld+i], [2*ld+i]. */
int refd_conc_rho(int64_t n, const double* T, const double* rho,
                  const double* Y, int64_t ld, double* misc, double* conc) {
  if (n < 0 || ld < n) return 1;
  for (int64_t i = 0; i < n; ++i) {
    double y[CRS_NSP], c[CRS_NSP];
    double y_N, mw, p;
    for (int k = 0; k < CRS_NSP - 1; ++k) y[k] = Y[(int64_t)k * ld + i];
    eval_conc_rho(T[i], rho[i], y, &y_N, &mw, &p, c);
    if (conc)
      for (int k = 0; k < CRS_NSP; ++k) conc[(int64_t)k * ld + i] = c[k];
    if (misc) {
      misc[i] = y_N;
      misc[ld + i] = mw;
      misc[2 * ld + i] = p;
    }
  }
  return 0;
}
