/*
 * Batch driver for create_rate_subs' emitted C (TEST INFRASTRUCTURE).
 *
 * The reference's runtime for this path is the straight-line C that its
 * generator prints (rate_subs.py:226-1391): eval_conc, eval_rxn_rates,
 * get_rxn_pres_mod (only when the mechanism has third-body/fall-off
 * reactions), eval_spec_rates.  This file owns none of that arithmetic.  It
 * is compiled together with the emitted files of one mechanism and loops
 * the four per-state calls over structure-of-arrays states, the way the
 * emitted dydt calls them (rate_subs.py:1845-1880).
 *
 * Sizes come from the build: CRS_NSP (species), CRS_NR (reactions),
 * CRS_NREV (reversible reactions), CRS_NPM (pres_mod entries).
 *
 * Only tests, the golden-vector script and bench.py's CPU baseline use this.
 */
#include <stddef.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef CRS_NSP
#error "CRS_NSP must be defined"
#endif

void eval_conc(const double T, const double pres, const double* y,
               double* y_N, double* mw_avg, double* rho, double* conc);
void eval_rxn_rates(const double T, const double pres, const double* C,
                    double* fwd_rxn_rates, double* rev_rxn_rates);
#if CRS_NPM > 0
void get_rxn_pres_mod(const double T, const double pres, const double* C,
                      double* pres_mod);
#endif
void eval_spec_rates(const double* fwd_rates, const double* rev_rates,
                     const double* pres_mod, double* sp_rates, double* dy_N);

#define NREV_ (CRS_NREV > 0 ? CRS_NREV : 1)
#define NPM_ (CRS_NPM > 0 ? CRS_NPM : 1)

int ref_dims(int64_t* out4) {
  out4[0] = CRS_NSP;
  out4[1] = CRS_NR;
  out4[2] = CRS_NREV;
  out4[3] = CRS_NPM;
  return 0;
}

/* One state i of an SoA batch.  Output arrays are SoA with leading
 * dimension ld (entry k of state i at [k*ld + i]); any may be NULL.
 * misc (if not NULL) receives y_N, mw_avg, rho at [0*ld+i], [1*ld+i],
 * [2*ld+i]. */
static void one_state(int64_t i, const double* T, const double* P,
                      const double* Y, int64_t ld, double* conc_o,
                      double* fwd_o, double* rev_o, double* pm_o,
                      double* wdot_o, double* misc_o) {
  double y[CRS_NSP], C[CRS_NSP], fwd[CRS_NR], rev[NREV_], pm[NPM_];
  double sp[CRS_NSP];
  double y_N, mw_avg, rho;
  for (int k = 0; k < CRS_NSP - 1; ++k) y[k] = Y[(int64_t)k * ld + i];
  eval_conc(T[i], P[i], y, &y_N, &mw_avg, &rho, C);
  eval_rxn_rates(T[i], P[i], C, fwd, rev);
#if CRS_NPM > 0
  get_rxn_pres_mod(T[i], P[i], C, pm);
#else
  pm[0] = 0.0;
#endif
  eval_spec_rates(fwd, rev, pm, sp, &sp[CRS_NSP - 1]);
  if (conc_o)
    for (int k = 0; k < CRS_NSP; ++k) conc_o[(int64_t)k * ld + i] = C[k];
  if (fwd_o)
    for (int k = 0; k < CRS_NR; ++k) fwd_o[(int64_t)k * ld + i] = fwd[k];
  if (rev_o)
    for (int k = 0; k < CRS_NREV; ++k) rev_o[(int64_t)k * ld + i] = rev[k];
  if (pm_o)
    for (int k = 0; k < CRS_NPM; ++k) pm_o[(int64_t)k * ld + i] = pm[k];
  if (wdot_o)
    for (int k = 0; k < CRS_NSP; ++k) wdot_o[(int64_t)k * ld + i] = sp[k];
  if (misc_o) {
    misc_o[i] = y_N;
    misc_o[ld + i] = mw_avg;
    misc_o[2 * ld + i] = rho;
  }
}

/* All stages for n states.  States are independent and each is evaluated
 * by the same per-state calls, so an OpenMP build (the parity build is one)
 * spreads them over threads without changing any result. */
int ref_eval(int64_t n, const double* T, const double* P, const double* Y,
             int64_t ld, double* conc, double* fwd, double* rev, double* pm,
             double* wdot, double* misc) {
  if (n < 0 || ld < n) return 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int64_t i = 0; i < n; ++i)
    one_state(i, T, P, Y, ld, conc, fwd, rev, pm, wdot, misc);
  return 0;
}

/* wdot only, OpenMP over states (the CPU baseline).  nthreads <= 0 keeps
 * the OpenMP default.  Returns the thread count used. */
int ref_wdot_omp(int64_t n, const double* T, const double* P,
                 const double* Y, int64_t ld, double* wdot, int nthreads) {
  int used = 1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
  {
#pragma omp single
    used = omp_get_num_threads();
#pragma omp for schedule(static)
    for (int64_t i = 0; i < n; ++i)
      one_state(i, T, P, Y, ld, NULL, NULL, NULL, NULL, wdot, NULL);
  }
#else
  (void)nthreads;
  for (int64_t i = 0; i < n; ++i)
    one_state(i, T, P, Y, ld, NULL, NULL, NULL, NULL, wdot, NULL);
#endif
  return used;
}
