/*
 * crs_device.cuh -- the reference's per-state functions as CUDA device
 * functions, for a user's own kernels (the 'cuda' target of the CLI).
 *
 * create_rate_subs -l cuda emits eval_conc, eval_rxn_rates,
 * get_rxn_pres_mod and eval_spec_rates (and the thermo utilities and dydt)
 * as __device__ functions with the mechanism compiled in
 * (rate_subs.py:256, 283, 757-763, 1121-1127); an integrator kernel calls
 * them once per thread, one state per thread (create_rate_subs.py:57-102).
 * Here the same signatures evaluate a table image that the CLI writes as
 * mech_image.cuh, in the reference's operation order (crs_eval.h).
 *
 * Use: include the CLI's out/rates.cuh (or mech_image.cuh and then this
 * header) in the translation unit of the kernel that calls them; every
 * definition is inline, so no relocatable device code is needed.  Compile
 * that unit with -fmad=false to get the reference's rounding (results then
 * equal CRS_MODE_FP64_STRICT's bit for bit); with FMA contraction they
 * stay within 1e-12 of the reference on the gross-rate scale.  The host
 * functions of crs.h have the same names: do not include crs.h in the same
 * translation unit.  Buffers are the caller's (no allocation); dydt needs
 * crs_device_dydt_scratch() doubles of scratch per thread.
 */
#ifndef CRS_DEVICE_CUH
#define CRS_DEVICE_CUH

#include "crs_eval.h"

#ifndef CRS_MECH_IMAGE_DEFINED
#error "include the mechanism image (mech_image.cuh, written by the CLI's cuda target) first"
#endif

// The compiled-in mechanism as a table view.
__device__ inline crs::Tab crs_device_tab() {
  return crs::make_tab(crs_mech_image, crs_mech_layout);
}

__device__ inline void eval_conc(const double T, const double pres, const double *y,
                                 double *y_N, double *mw_avg, double *rho, double *conc) {
  crs::ref::state_eval_conc(crs_device_tab(), T, pres, y, y_N, mw_avg, rho, conc);
}

__device__ inline void eval_rxn_rates(const double T, const double pres, const double *C,
                                      double *fwd_rxn_rates, double *rev_rxn_rates) {
  crs::ref::state_eval_rxn_rates(crs_device_tab(), T, pres, C, fwd_rxn_rates, rev_rxn_rates);
}

__device__ inline void get_rxn_pres_mod(const double T, const double pres, const double *C,
                                        double *pres_mod) {
  crs::ref::state_get_rxn_pres_mod(crs_device_tab(), T, pres, C, pres_mod);
}

__device__ inline void eval_spec_rates(const double *fwd_rates, const double *rev_rates,
                                       const double *pres_mod, double *sp_rates,
                                       double *dy_N) {
  crs::ref::state_eval_spec_rates(crs_device_tab(), fwd_rates, rev_rates, pres_mod, sp_rates,
                                  dy_N);
}

__device__ inline void eval_h(const double T, double *h) {
  crs::ref::state_eval_thermo(crs_device_tab(), 0, T, h);
}
__device__ inline void eval_u(const double T, double *u) {
  crs::ref::state_eval_thermo(crs_device_tab(), 1, T, u);
}
__device__ inline void eval_cv(const double T, double *cv) {
  crs::ref::state_eval_thermo(crs_device_tab(), 2, T, cv);
}
__device__ inline void eval_cp(const double T, double *cp) {
  crs::ref::state_eval_thermo(crs_device_tab(), 3, T, cp);
}

__device__ inline void eval_conc_rho(const double T, const double rho, const double *y,
                                     double *y_N, double *mw_avg, double *pres,
                                     double *conc) {
  crs::ref::state_eval_conc_rho(crs_device_tab(), T, rho, y, y_N, mw_avg, pres, conc);
}

// Doubles of per-thread scratch that dydt needs for this mechanism.
__host__ __device__ inline int crs_device_dydt_scratch() {
  return (int)(3 * CRS_MECH_NSP + CRS_MECH_NRXN + (CRS_MECH_NREV > 0 ? CRS_MECH_NREV : 1) +
               (CRS_MECH_NPDEP > 0 ? CRS_MECH_NPDEP : 1));
}

// dydt (rate_subs.py:1829-2067) for y = [T, Y_0 .. Y_{N-2}]: constant
// pressure (pres = P) unless CRS_CONV is defined (pres = the density), as
// the emitted -DCONP / -DCONV builds read it.  scratch: per-thread space
// of crs_device_dydt_scratch() doubles.
__device__ inline void dydt(const double t, const double pres, const double *y, double *dy,
                            double *scratch) {
  (void)t;
#ifdef CRS_CONV
  crs::ref::state_dydt(crs_device_tab(), 1, pres, y, dy, scratch);
#else
  crs::ref::state_dydt(crs_device_tab(), 0, pres, y, dy, scratch);
#endif
}

#endif /* CRS_DEVICE_CUH */
