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
// first call, or touches a GPU; the table image is immutable, so any
// number of threads may call at once.
//
// eval_rxn_rates and eval_spec_rates run over per-mechanism lists (Aux,
// built once at load) that take the data-dependent branches out of their
// inner loops, with results identical by exact identities: each side's
// concentration factors in the emitted order padded to a fixed width with
// a slot holding 1.0 (x * 1.0 == x), a missing reverse rate read as 0.0
// (f - 0.0 == f), a missing pres_mod as 1.0, and the signed accumulation
// W -/+ (|nu| * net) * pm written as W + (nu * net) * pm (rounding to
// nearest is symmetric under negation, and W - v == W + (-v)).
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/crs_eval.h"

namespace crs {
namespace host {

// Widest padded factor list of the fast path; longer sides (and
// non-integer coefficients, PLOG / Chebyshev rows, irreversible rows of
// the A < 0 and integer-power forms, whose emitted expressions group the
// factors differently) take the generic path of crs_eval.h.
constexpr int MAX_FACTORS = 4;

struct Aux {
  int N = 0, R = 0, NREV = 0, NPM = 0, W = 1;
  std::vector<int32_t> fac;     // [R][2][W]: reactant then product factors, N = the 1.0 slot
  std::vector<uint8_t> fast;    // per reaction: 1 when the padded lists apply
  std::vector<int32_t> jrev;    // per reaction: rev index, or NREV (a 0.0 slot)
  std::vector<int32_t> jpm;     // per reaction: pres_mod index, or NPM (a 1.0 slot)
  std::vector<int32_t> pm_order;  // pres_mod entries grouped by kind and form
};

namespace {

// Expanded factor species of one side of reaction r in the emitted order
// (integer nu repeated), or false when a coefficient is not an integer.
bool expand(const int32_t *ptr, const int32_t *sp, const int32_t *nint, int r,
            std::vector<int32_t> &out) {
  out.clear();
  for (int e = ptr[r]; e < ptr[r + 1]; ++e) {
    if (nint[e] < 0) return false;
    for (int q = 0; q < nint[e]; ++q) out.push_back(sp[e]);
  }
  return true;
}

// The calling thread's scratch, grown for the largest mechanism it has seen.
double *scratch(std::vector<double> &v, size_t n) {
  if (v.size() < n) v.resize(n);
  return v.data();
}

}  // namespace

Aux *make_aux(const Tab &t) {
  Aux *a = new Aux();
  a->N = t.N;
  a->R = t.R;
  a->NREV = t.NREV;
  a->NPM = t.NPM;
  std::vector<int32_t> rf, pf;
  std::vector<std::vector<int32_t>> sides(2 * (size_t)t.R);
  a->fast.assign(t.R, 0);
  for (int r = 0; r < t.R; ++r) {
    const int kind = t.rate_kind[r];
    const bool ok_r = expand(t.rx_ptr, t.rx_sp, t.rx_nint, r, rf);
    const bool ok_p = expand(t.px_ptr, t.px_sp, t.px_nint, r, pf);
    const bool irrev_ok = kind == RATE_EXP || kind == RATE_CONST;
    const bool ok = ok_r && ok_p && kind < RATE_PLOG && (t.rev_idx[r] >= 0 || irrev_ok) &&
                    (int)rf.size() <= MAX_FACTORS && (int)pf.size() <= MAX_FACTORS;
    if (!ok) continue;
    a->fast[r] = 1;
    a->W = std::max(a->W, (int)std::max(rf.size(), pf.size()));
    sides[2 * (size_t)r] = rf;
    sides[2 * (size_t)r + 1] = pf;
  }
  a->fac.assign(2 * (size_t)t.R * a->W, t.N);
  for (int r = 0; r < t.R; ++r)
    for (int h = 0; h < 2; ++h) {
      const std::vector<int32_t> &f = sides[2 * (size_t)r + h];
      for (size_t q = 0; q < f.size(); ++q) a->fac[(2 * (size_t)r + h) * a->W + q] = f[q];
    }
  a->jrev.resize(t.R);
  a->jpm.resize(t.R);
  for (int r = 0; r < t.R; ++r) {
    a->jrev[r] = t.rev_idx[r] >= 0 ? t.rev_idx[r] : t.NREV;
    a->jpm[r] = t.pm_idx[r] >= 0 ? t.pm_idx[r] : t.NPM;
  }
  // third bodies first, then the fall-off entries by form: each entry is
  // computed alone, so the order changes no result, only how well the
  // branches on kind and form predict
  for (int pass = 0; pass < 4; ++pass)
    for (int p = 0; p < t.NPM; ++p) {
      const int g = t.pm_kind[p] == PM_THD ? 0 : t.pm_form[p] == FORM_TROE ? 2
                    : t.pm_form[p] == FORM_SRI ? 3 : 1;
      if (g == pass) a->pm_order.push_back(p);
    }
  return a;
}

void free_aux(Aux *a) { delete a; }

void eval_conc(const Tab &t, double T, double pres, const double *y, double *y_N,
               double *mw_avg, double *rho, double *conc) {
  ref::state_eval_conc(t, T, pres, y, y_N, mw_avg, rho, conc);
}

// eval_rxn_rates (rate_subs.py:287-290, 433-693): ref::rxn_rates for the
// rows the padded lists do not cover, else the same operations: fwd =
// (factors) * kf; rev = ((factors) * kf) / (prefactor * exp(Kc exponent)).
void eval_rxn_rates(const Tab &t, const Aux *a, double T, double pres, const double *C,
                    double *fwd, double *rev) {
  if (!a) {
    ref::state_eval_rxn_rates(t, T, pres, C, fwd, rev);
    return;
  }
  thread_local std::vector<double> buf;
  const int N = a->N, W = a->W;
  double *Cx = scratch(buf, (size_t)N + 1);
  for (int k = 0; k < N; ++k) Cx[k] = C[k];
  Cx[N] = 1.0;
  const ref::Strided<const double> Cc{C, 1};
  const double logT = log(T);
  for (int r = 0; r < a->R; ++r) {
    const int j = t.rev_idx[r];
    if (!a->fast[r]) {
      double f, rv;
      ref::rxn_rates(t, r, T, logT, pres, Cc, f, rv);
      fwd[r] = f;
      if (j >= 0) rev[j] = rv;
      continue;
    }
    const int32_t *fr = a->fac.data() + 2 * (size_t)r * W, *fp = fr + W;
    double p = Cx[fr[0]];
    for (int q = 1; q < W; ++q) p = p * Cx[fr[q]];
    const double kf = ref::rate_const(t, r, T, logT);
    fwd[r] = p * kf;
    if (j >= 0) {
      double Kc = ref::kc_exponent(t, j, T, logT);
      Kc = t.kc_pref[j] * exp(Kc);
      double q = Cx[fp[0]];
      for (int u = 1; u < W; ++u) q = q * Cx[fp[u]];
      rev[j] = q * kf / Kc;
    }
  }
}

// get_rxn_pres_mod (rate_subs.py:761-763): every entry as ref::pres_mod
// computes it, visited in the grouped order.
void get_rxn_pres_mod(const Tab &t, const Aux *a, double T, double pres, const double *C,
                      double *pm) {
  if (!a) {
    ref::state_get_rxn_pres_mod(t, T, pres, C, pm);
    return;
  }
  const ref::Strided<const double> Cc{C, 1};
  const double logT = log(T);
  const double mix = pres / (ref::RU_PRINTED * T);
  for (const int p : a->pm_order) pm[p] = ref::pres_mod(t, p, T, logT, mix, Cc);
}

// eval_spec_rates (rate_subs.py:1121-1235): per net-nu entry, in reaction
// order, W_k += (nu * net) * pres_mod, which equals the emitted
// W_k -/+ (|nu| * (fwd - rev)) * pres_mod bit for bit.
void eval_spec_rates(const Tab &t, const Aux *a, const double *fwd, const double *rev,
                     const double *pm, double *sp_rates, double *dy_N) {
  if (!a) {
    ref::state_eval_spec_rates(t, fwd, rev, pm, sp_rates, dy_N);
    return;
  }
  thread_local std::vector<double> buf;
  const int N = a->N, NREV = a->NREV, NPM = a->NPM;
  double *Wk = scratch(buf, (size_t)N + NREV + NPM + 2);
  double *rv = Wk + N, *pmx = rv + NREV + 1;
  for (int k = 0; k < N; ++k) Wk[k] = 0.0;
  for (int j = 0; j < NREV; ++j) rv[j] = rev[j];
  rv[NREV] = 0.0;
  for (int p = 0; p < NPM; ++p) pmx[p] = pm[p];
  pmx[NPM] = 1.0;
  for (int r = 0; r < a->R; ++r) {
    const double net = fwd[r] - rv[a->jrev[r]];
    const double m = pmx[a->jpm[r]];
    for (int e = t.nu_ptr[r]; e < t.nu_ptr[r + 1]; ++e) {
      const int k = t.nu_sp[e];
      Wk[k] = Wk[k] + (t.nu_val[e] * net) * m;
    }
  }
  for (int k = 0; k < N - 1; ++k) sp_rates[k] = Wk[k];
  *dy_N = Wk[N - 1];
}

void eval_thermo(const Tab &t, int which, double T, double *out) {
  ref::state_eval_thermo(t, which, T, out);
}

void eval_conc_rho(const Tab &t, double T, double rho, const double *y, double *y_N,
                   double *mw_avg, double *pres, double *conc) {
  ref::state_eval_conc_rho(t, T, rho, y, y_N, mw_avg, pres, conc);
}

// dydt (rate_subs.py:1829-2067): ref::state_dydt's sequence with the
// three rate functions above in place of the generic ones.  Scratch of the
// calling thread (concentrations, rates, thermo columns), grown on its
// first call for the largest mechanism it has seen.
void dydt(const Tab &t, const Aux *a, int conv, double p_or_rho, const double *y,
          double *dy) {
  thread_local std::vector<double> scratch;
  double *s = crs::host::scratch(scratch, (size_t)ref::dydt_scratch(t));
  if (!a) {
    ref::state_dydt(t, conv, p_or_rho, y, dy, s);
    return;
  }
  const int N = t.N;
  double *C = s, *fwd = C + N, *rev = fwd + t.R;
  double *pm = rev + (t.NREV > 0 ? t.NREV : 1);
  double *c = pm + (t.NPM > 0 ? t.NPM : 1), *e = c + N;
  const double T = y[0];
  double y_N, mw_avg, rho, pres;
  if (conv) {
    rho = p_or_rho;
    ref::state_eval_conc_rho(t, T, rho, y + 1, &y_N, &mw_avg, &pres, C);
  } else {
    pres = p_or_rho;
    ref::state_eval_conc(t, T, pres, y + 1, &y_N, &mw_avg, &rho, C);
  }
  eval_rxn_rates(t, a, T, pres, C, fwd, rev);
  get_rxn_pres_mod(t, a, T, pres, C, pm);
  double dy_N;
  eval_spec_rates(t, a, fwd, rev, pm, dy + 1, &dy_N);
  ref::state_eval_thermo(t, conv ? 2 : 3, T, c);
  double avg = 0.0;
  for (int k = 0; k < N - 1; ++k) {
    const double v = c[k] * y[k + 1];
    avg = (k == 0) ? v : avg + v;
  }
  avg = (N > 1) ? avg + c[N - 1] * y_N : c[N - 1] * y_N;
  ref::state_eval_thermo(t, conv ? 1 : 0, T, e);
  double sum = 0.0;
  for (int k = 0; k < N - 1; ++k) {
    const double v = dy[k + 1] * e[k] * t.sp_mw[k];
    sum = (k == 0) ? v : sum + v;
  }
  sum = (N > 1) ? sum + dy_N * e[N - 1] * t.sp_mw[N - 1] : dy_N * e[N - 1] * t.sp_mw[N - 1];
  dy[0] = (-1.0 / (rho * avg)) * sum;
  for (int k = 0; k < N - 1; ++k) dy[k + 1] *= (t.sp_mw[k] / rho);
}

}  // namespace host
}  // namespace crs
