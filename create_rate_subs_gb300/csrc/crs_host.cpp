// Reentrant per-state evaluation on the host: the reference's per-state
// functions (eval_conc, eval_rxn_rates, get_rxn_pres_mod, eval_spec_rates,
// the thermo utilities and dydt; rate_subs.py:287-290, 761-763, 1124-1127,
// 1297-1299, 1396-2067) over a mechanism's host table image.
//
// The arithmetic is include/crs_eval.h, the same code the reference-order
// GPU kernel runs.  This file is compiled by the host C++ compiler with
// -ffp-contract=off (create_rate_subs_gb300/build.py), so every operation
// is rounded once in the emitted order and the C library's exp/log/pow are
// the ones the reference's emitted C calls: the results equal the emitted
// C's bit for bit.  No function here locks, allocates after a thread's
// first dydt call, or touches a GPU; the table image is immutable, so any
// number of threads may call at once.
#include <vector>

#include "../../include/crs_eval.h"

namespace crs {
namespace host {

void eval_conc(const Tab &t, double T, double pres, const double *y, double *y_N,
               double *mw_avg, double *rho, double *conc) {
  ref::state_eval_conc(t, T, pres, y, y_N, mw_avg, rho, conc);
}

void eval_rxn_rates(const Tab &t, double T, double pres, const double *C, double *fwd,
                    double *rev) {
  ref::state_eval_rxn_rates(t, T, pres, C, fwd, rev);
}

void get_rxn_pres_mod(const Tab &t, double T, double pres, const double *C, double *pm) {
  ref::state_get_rxn_pres_mod(t, T, pres, C, pm);
}

void eval_spec_rates(const Tab &t, const double *fwd, const double *rev, const double *pm,
                     double *sp_rates, double *dy_N) {
  ref::state_eval_spec_rates(t, fwd, rev, pm, sp_rates, dy_N);
}

void eval_thermo(const Tab &t, int which, double T, double *out) {
  ref::state_eval_thermo(t, which, T, out);
}

void eval_conc_rho(const Tab &t, double T, double rho, const double *y, double *y_N,
                   double *mw_avg, double *pres, double *conc) {
  ref::state_eval_conc_rho(t, T, rho, y, y_N, mw_avg, pres, conc);
}

// Scratch of the calling thread (concentrations, rates, thermo columns),
// grown on its first call for the largest mechanism it has seen.
void dydt(const Tab &t, int conv, double p_or_rho, const double *y, double *dy) {
  thread_local std::vector<double> scratch;
  const size_t need = (size_t)ref::dydt_scratch(t);
  if (scratch.size() < need) scratch.resize(need);
  ref::state_dydt(t, conv, p_or_rho, y, dy, scratch.data());
}

}  // namespace host
}  // namespace crs
