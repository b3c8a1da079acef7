/*
 * crs_eval.h -- the FP64 arithmetic of one thermochemical state in the
 * reference's own operation order (C++, host and device).
 *
 * create_rate_subs emits this arithmetic as straight-line C per mechanism
 * (rate_subs.py:20-1391 for the rates, :1396-1776 for the thermo
 * utilities, :1829-2067 for dydt).  Here it is written once over the table
 * image of crs_tables.h, with one rounding per operation in the emitted
 * order, so that compiled without floating-point contraction
 * (g++ -ffp-contract=off on the host, nvcc -fmad=false on the device) it
 * reproduces the emitted C up to the last bits of exp/log/log10/pow (none
 * at all on the host, where the C library is the same).
 *
 * Three places compile it: libcrs's reentrant per-state host functions
 * (eval_conc ... in crs.h), the reference-order GPU kernel
 * (CRS_MODE_FP64_STRICT) and the per-state device functions of
 * crs_device.cuh.  Everything here has internal linkage, so that each
 * translation unit keeps the copy its own flags compiled.
 */
#ifndef CRS_EVAL_H
#define CRS_EVAL_H

#include <math.h>

#include "crs_tables.h"

namespace crs {
namespace ref {
namespace {

// The gas constant as eval_conc prints it (%.8e, rate_subs.py:1364).
constexpr double RU_PRINTED = 8.31446210e+03;

// Element k of a column at p[k * stride] (the kernels' per-thread columns
// and SoA arrays; stride 1 for one state's contiguous array).
template <class V>
struct Strided {
  V *p;
  int64_t stride;
  CRS_HD V &operator[](int k) const { return p[(int64_t)k * stride]; }
};

// rxn_rate_const (rate_subs.py:60-135): A > 0 as exp(logA + b ln T - Ta/T),
// A < 0 as A exp(b ln T - Ta/T), integer b with zero Ta as repeated
// multiplication, a constant.
CRS_HD inline double rate_const(const Tab &t, int row, double T, double logT) {
  const double *p = t.rate_par + 4 * row;  // A, logA, b, Ta
  switch (t.rate_kind[row]) {
    case RATE_CONST:
      return p[0];
    case RATE_EXP:
      return exp(p[1] + p[2] * logT - (p[3] / T));
    case RATE_NEGEXP:
      return p[0] * exp(p[2] * logT - (p[3] / T));
    default: {
      double k = p[0];
      for (int j = 0; j < t.rate_npow[row]; ++j) k = k * T;
      return k;
    }
  }
}

// Forward rate constant of a PLOG row (rate_subs.py:444-485: branch
// thresholds as printed with %.4e, log-linear interpolation in ln P between
// the bracketing points) or a Chebyshev row (rate_subs.py:136-223: reduced
// temperature and pressure, the pressure dot products by the Chebyshev
// recursion, then the temperature sum, 10^kf), in the emitted order.
CRS_HD inline double pdep_kf(const Tab &t, int row, double T, double logT, double pres) {
  const int a = t.rate_aux[row];
  if (t.rate_kind[row] == RATE_PLOG) {
    const int e0 = t.plog_ptr[a], e1 = t.plog_ptr[a + 1];
    if (pres <= t.plog_p[e0]) return rate_const(t, t.plog_row[e0], T, logT);
    for (int e = e0; e < e1 - 1; ++e)
      if ((pres > t.plog_p[e]) && (pres <= t.plog_p[e + 1])) {
        const double k1 = log(rate_const(t, t.plog_row[e], T, logT));
        const double k2 = log(rate_const(t, t.plog_row[e + 1], T, logT));
        return exp(k1 + (k2 - k1) * (log(pres) - t.plog_lp[e]) / t.plog_dlp[e]);
      }
    if (pres > t.plog_p[e1 - 1]) return rate_const(t, t.plog_row[e1 - 1], T, logT);
    return nan("");  // no branch taken (NaN pressure)
  }
  const double *tp = t.cheb_tp + 4 * a;
  const int nt = t.cheb_nt[a], np = t.cheb_np[a];
  const double *c = t.cheb_par + t.cheb_ptr[a];  // [nt][np]
  const double Tred = ((2.0 / T) - tp[0]) / tp[1];
  const double Pred = (2.0 * log10(pres) - tp[2]) / tp[3];
  double dp[CHEB_MAX];
  for (int i = 0; i < nt; ++i) dp[i] = c[i * np] + Pred * c[i * np + 1];
  double ct0 = 1.0, ct1 = Pred;
  bool upd = true;
  for (int j = 2; j < np; ++j) {
    if (upd) {
      ct0 = 2.0 * Pred * ct1 - ct0;
      for (int i = 0; i < nt; ++i) dp[i] += c[i * np + j] * ct0;
    } else {
      ct1 = 2.0 * Pred * ct0 - ct1;
      for (int i = 0; i < nt; ++i) dp[i] += c[i * np + j] * ct1;
    }
    upd = !upd;
  }
  ct0 = 1.0;
  ct1 = Tred;
  double kf = dp[0] + Tred * dp[1];
  upd = true;
  for (int i = 2; i < nt; ++i) {
    if (upd) {
      ct0 = 2.0 * Tred * ct1 - ct0;
      kf += dp[i] * ct0;
    } else {
      ct1 = 2.0 * Tred * ct0 - ct1;
      kf += dp[i] * ct1;
    }
    upd = !upd;
  }
  return pow(10.0, kf);
}

// Product of concentrations over one side of a reaction, in the emitted
// factor order (rate_subs.py:490-501): integer nu as repeated
// multiplication, other nu through pow.  have = false for an empty side.
template <class CS>
CRS_HD inline double conc_product(const int32_t *sp, const int32_t *nint, const double *nu,
                                  int a, int b, const CS &C, bool &have) {
  double p = 0.0;
  bool first = true;
  for (int j = a; j < b; ++j) {
    const int s = sp[j];
    if (nint[j] >= 0) {
      for (int q = 0; q < nint[j]; ++q) {
        const double c = C[s];
        p = first ? c : p * c;
        first = false;
      }
    } else {
      const double f = pow(C[s], nu[j]);
      p = first ? f : p * f;
      first = false;
    }
  }
  have = !first;
  return p;
}

// Exponent of the equilibrium constant of reversible reaction j, summed
// over its T_common groups (rate_subs.py:592-655).
CRS_HD inline double kc_exponent(const Tab &t, int j, double T, double logT) {
  double kc = 0.0;
  const int g0 = t.kc_ptr[j], g1 = t.kc_ptr[j + 1];
  for (int g = g0; g < g1; ++g) {
    const double *c = (T <= t.kc_tmid[g]) ? t.kc_lo + 7 * g : t.kc_hi + 7 * g;
    const double v =
        (c[0] + c[1] * logT + T * (c[2] + T * (c[3] + T * (c[4] + c[5] * T))) - c[6] / T);
    kc = (g == g0) ? v : kc + v;
  }
  return kc;
}

// fwd (and rev when reversible) of reaction r (rate_subs.py:433-693).
// PLOG / Chebyshev rows print kf first and use it like a reversible
// reaction's kf (rate_subs.py:437-448, 503-505).
template <class CS>
CRS_HD inline void rxn_rates(const Tab &t, int r, double T, double logT, double pres,
                             const CS &C, double &fwd, double &rev) {
  bool have;
  const double p =
      conc_product(t.rx_sp, t.rx_nint, t.rx_nu, t.rx_ptr[r], t.rx_ptr[r + 1], C, have);
  const int j = t.rev_idx[r];
  const bool pdep = t.rate_kind[r] >= RATE_PLOG;
  if (j >= 0 || pdep) {
    const double kf = pdep ? pdep_kf(t, r, T, logT, pres) : rate_const(t, r, T, logT);
    fwd = have ? p * kf : kf;
    if (j < 0) {
      rev = 0.0;
      return;
    }
    double Kc = kc_exponent(t, j, T, logT);
    Kc = t.kc_pref[j] * exp(Kc);
    bool hq;
    const double q =
        conc_product(t.px_sp, t.px_nint, t.px_nu, t.px_ptr[r], t.px_ptr[r + 1], C, hq);
    rev = hq ? q * kf / Kc : kf / Kc;
  } else {
    rev = 0.0;
    if (!have) {
      fwd = rate_const(t, r, T, logT);
      return;
    }
    // irreversible: the rate expression is printed inline after the
    // concentration factors (rate_subs.py:503-510)
    const double *a = t.rate_par + 4 * r;
    switch (t.rate_kind[r]) {
      case RATE_CONST: fwd = p * a[0]; break;
      case RATE_EXP: fwd = p * exp(a[1] + a[2] * logT - (a[3] / T)); break;
      case RATE_NEGEXP: fwd = p * a[0] * exp(a[2] * logT - (a[3] / T)); break;
      default: {
        double v = p * a[0];
        for (int q = 0; q < t.rate_npow[r]; ++q) v = v * T;
        fwd = v;
      }
    }
  }
}

// Third-body concentration of pres_mod entry p: m + sum (eff - 1) C_k
// (rate_subs.py:901-915).
template <class CS>
CRS_HD inline double third_body(const Tab &t, int p, double mix, const CS &C) {
  double v = mix;
  for (int e = t.pm_eff_ptr[p]; e < t.pm_eff_ptr[p + 1]; ++e)
    v = v + t.pm_eff_val[e] * C[t.pm_eff_sp[e]];
  return v;
}

// pres_mod entry p (rate_subs.py:881-1064): third body, or the Lindemann /
// Troe / SRI fall-off factor with LOW or HIGH.
template <class CS>
CRS_HD inline double pres_mod(const Tab &t, int p, double T, double logT, double mix,
                              const CS &C) {
  if (t.pm_kind[p] == PM_THD) return third_body(t, p, mix, C);
  const int sp = t.pm_sp[p];
  const double thd = (sp < 0) ? third_body(t, p, mix, C) : 0.0;
  const double k0 = rate_const(t, t.pm_k0[p], T, logT);
  const double kinf = rate_const(t, t.pm_kinf[p], T, logT);
  const double Pr = (sp >= 0) ? k0 * C[sp] / kinf : k0 * thd / kinf;
  const bool low = t.pm_kind[p] == PM_FALL_LOW;
  const int form = t.pm_form[p];
  if (form == FORM_TROE) {
    const double *c = t.pm_troe + 5 * p;
    double s = c[0] * exp(-T / c[1]) + c[2] * exp(-T / c[3]);
    if (t.pm_troe_t2[p]) s = s + exp(-c[4] / T);
    const double logFcent = log10(fmax(s, 1.0e-300));
    const double A = log10(fmax(Pr, 1.0e-300)) - 0.67 * logFcent - 0.4;
    const double B = 0.806 - 1.1762 * logFcent - 0.14 * log10(fmax(Pr, 1.0e-300));
    const double F = pow(10.0, logFcent / (1.0 + A * A / (B * B)));
    return low ? F * Pr / (1.0 + Pr) : F / (1.0 + Pr);
  }
  if (form == FORM_SRI) {
    const double *c = t.pm_sri + 5 * p;
    const double X = 1.0 / (1.0 + log10(fmax(Pr, 1.0e-300)) * log10(fmax(Pr, 1.0e-300)));
    double F = pow(c[0] * exp(-c[1] / T) + exp(-T / c[2]), X);
    if (t.pm_sri_de[p]) F = F * c[3] * pow(T, c[4]);
    return low ? F * Pr / (1.0 + Pr) : F / (1.0 + Pr);
  }
  return low ? Pr / (1.0 + Pr) : 1.0 / (1.0 + Pr);
}

// Net term of reaction r for species entry e, accumulated into W
// (rate_subs.py:1183-1216): sign * ((|nu| * (fwd - rev)) * pres_mod).
template <class WA>
CRS_HD inline void accumulate(const Tab &t, int e, double net, double pm, bool has_pm,
                              const WA &W) {
  const int k = t.nu_sp[e];
  const double nu = t.nu_val[e];
  const double a = fabs(nu);
  double v = net;
  if (a != 1.0) v = a * v;
  if (has_pm) v = v * pm;
  W[k] = (nu < 0.0) ? W[k] - v : W[k] + v;
}

// Net rate of every reaction into W (W zeroed first): eval_spec_rates
// (rate_subs.py:1121-1235) from fwd [R], rev [R_rev] and pres_mod [N_pm].
template <class FA, class WA>
CRS_HD inline void spec_rates(const Tab &t, const FA &fwd, const FA &rev, const FA &pm,
                              const WA &W) {
  for (int k = 0; k < t.N; ++k) W[k] = 0.0;
  for (int r = 0; r < t.R; ++r) {
    const int j = t.rev_idx[r], p = t.pm_idx[r];
    const double f = fwd[r];
    const double net = (j >= 0) ? f - rev[j] : f;
    const double m = (p >= 0) ? pm[p] : 0.0;
    for (int e = t.nu_ptr[r]; e < t.nu_ptr[r + 1]; ++e) accumulate(t, e, net, m, p >= 0, W);
  }
}

// eval_conc for one state (rate_subs.py:1295-1391) up to the
// concentrations: y_N = 1 - sum y, mw_avg, and the returned density.
// Y[k] is the k-th mass fraction, k < N-1.
template <class YA>
CRS_HD inline double eval_conc(const Tab &t, double T, double P, const YA &Y, double &y_N,
                               double &mw_avg) {
  const int N = t.N;
  double s = (N > 1) ? Y[0] : 0.0;
  for (int k = 1; k < N - 1; ++k) s = s + Y[k];
  y_N = 1.0 - s;
  double mw = 0.0;
  for (int k = 0; k < N - 1; ++k) {
    const double v = Y[k] * t.inv_mw[k];
    mw = (k == 0) ? v : mw + v;
  }
  mw = (N > 1) ? mw + y_N * t.inv_mw[N - 1] : y_N * t.inv_mw[N - 1];
  mw_avg = 1.0 / mw;
  return P * mw_avg / (RU_PRINTED * T);
}

// h (which 0), u (1), cv (2), cp (3) of one species at T, J/kg or
// J/(kg K), from its 24-entry sp_thermo record (RU/mw, mw, T_common, 0,
// low-range a0..a5, a1/2, a2/3, a3/4, a4/5, high range the same), in the
// emitted form (rate_subs.py:1513-1776).
CRS_HD inline double thermo_value(const double *c, int which, double T) {
  const double *a = c + ((T <= c[2]) ? 4 : 14);
  const double rm = c[0];
  switch (which) {
    case 0:
      return rm * (a[5] + T * (a[0] + T * (a[6] + T * (a[7] + T * (a[8] + a[9] * T)))));
    case 1:
      return rm * (a[5] + T * (a[0] - 1.0 + T * (a[6] + T * (a[7] + T * (a[8] + a[9] * T)))));
    case 2:
      return rm * (a[0] - 1.0 + T * (a[1] + T * (a[2] + T * (a[3] + a[4] * T))));
    default:
      return rm * (a[0] + T * (a[1] + T * (a[2] + T * (a[3] + a[4] * T))));
  }
}

// ---- one state, with the reference's per-state signatures --------------

// eval_conc (rate_subs.py:1297-1299): y holds the first N-1 mass fractions.
CRS_HD inline void state_eval_conc(const Tab &t, double T, double pres, const double *y,
                                   double *y_N, double *mw_avg, double *rho, double *conc) {
  const int N = t.N;
  const Strided<const double> Y{y, 1};
  double yN, mw;
  const double r = eval_conc(t, T, pres, Y, yN, mw);
  for (int k = 0; k < N - 1; ++k) conc[k] = r * y[k] * t.inv_mw[k];
  conc[N - 1] = r * yN * t.inv_mw[N - 1];
  *y_N = yN;
  *mw_avg = mw;
  *rho = r;
}

// eval_rxn_rates (rate_subs.py:287-290): fwd [R], rev [R_rev].
CRS_HD inline void state_eval_rxn_rates(const Tab &t, double T, double pres, const double *C,
                                        double *fwd, double *rev) {
  const Strided<const double> Cc{C, 1};
  const double logT = log(T);
  for (int r = 0; r < t.R; ++r) {
    double f, rv;
    rxn_rates(t, r, T, logT, pres, Cc, f, rv);
    fwd[r] = f;
    const int j = t.rev_idx[r];
    if (j >= 0) rev[j] = rv;
  }
}

// get_rxn_pres_mod (rate_subs.py:761-763): pres_mod [N_pm].
CRS_HD inline void state_get_rxn_pres_mod(const Tab &t, double T, double pres, const double *C,
                                          double *pres_mod_out) {
  const Strided<const double> Cc{C, 1};
  const double logT = log(T);
  const double mix = pres / (RU_PRINTED * T);
  for (int p = 0; p < t.NPM; ++p) pres_mod_out[p] = pres_mod(t, p, T, logT, mix, Cc);
}

// The reference's sp_rates [N-1] + *dy_N as one species-indexed array.
struct SpecOut {
  double *sp, *dy_N;
  int last;
  CRS_HD double &operator[](int k) const { return k == last ? *dy_N : sp[k]; }
};

// eval_spec_rates (rate_subs.py:1124-1127): sp_rates [N-1], *dy_N.
CRS_HD inline void state_eval_spec_rates(const Tab &t, const double *fwd, const double *rev,
                                         const double *pm, double *sp_rates, double *dy_N) {
  const Strided<const double> F{fwd, 1}, Rv{rev, 1}, PM{pm, 1};
  spec_rates(t, F, Rv, PM, SpecOut{sp_rates, dy_N, t.N - 1});
}

// eval_h / eval_u / eval_cv / eval_cp (rate_subs.py:1497-1776): out [N].
CRS_HD inline void state_eval_thermo(const Tab &t, int which, double T, double *out) {
  for (int k = 0; k < t.N; ++k) out[k] = thermo_value(t.sp_thermo + 24 * k, which, T);
}

// eval_conc_rho (rate_subs.py:1396-1490): concentrations and pressure from
// the density.
CRS_HD inline void state_eval_conc_rho(const Tab &t, double T, double rho, const double *y,
                                       double *y_N, double *mw_avg, double *pres,
                                       double *conc) {
  const int N = t.N;
  const Strided<const double> Y{y, 1};
  double yN, mw;
  eval_conc(t, T, 0.0, Y, yN, mw);
  if (N <= 1) yN = 1.0;
  *y_N = yN;
  *mw_avg = mw;
  *pres = rho * RU_PRINTED * T / mw;
  for (int k = 0; k < N - 1; ++k) conc[k] = rho * y[k] * t.inv_mw[k];
  conc[N - 1] = rho * yN * t.inv_mw[N - 1];
}

// Doubles of scratch that state_dydt needs: C [N], fwd [R], rev [R_rev],
// pres_mod [N_pm], two thermo columns [N] each.
CRS_HD inline int64_t dydt_scratch(const Tab &t) {
  return 3 * (int64_t)t.N + t.R + (t.NREV > 0 ? t.NREV : 1) + (t.NPM > 0 ? t.NPM : 1);
}

// dydt (rate_subs.py:1829-2067) for y = [T, Y_0 .. Y_{N-2}], dy the same:
// conv = 0 constant pressure (p_or_rho = P; cp, h), conv = 1 constant
// volume (p_or_rho = rho; pressure and concentrations from eval_conc_rho;
// cv, u).  dT/dt = -(sum wdot_k e_k mw_k) / (rho c_avg),
// dY_k/dt = wdot_k (mw_k / rho).  `scratch` holds dydt_scratch(t) doubles.
CRS_HD inline void state_dydt(const Tab &t, int conv, double p_or_rho, const double *y,
                              double *dy, double *scratch) {
  const int N = t.N;
  double *C = scratch, *fwd = C + N, *rev = fwd + t.R;
  double *pm = rev + (t.NREV > 0 ? t.NREV : 1);
  double *c = pm + (t.NPM > 0 ? t.NPM : 1), *e = c + N;
  const double T = y[0];
  double y_N, mw_avg, rho, pres;
  if (conv) {
    rho = p_or_rho;
    state_eval_conc_rho(t, T, rho, y + 1, &y_N, &mw_avg, &pres, C);
  } else {
    pres = p_or_rho;
    state_eval_conc(t, T, pres, y + 1, &y_N, &mw_avg, &rho, C);
  }
  state_eval_rxn_rates(t, T, pres, C, fwd, rev);
  state_get_rxn_pres_mod(t, T, pres, C, pm);
  double dy_N;
  state_eval_spec_rates(t, fwd, rev, pm, dy + 1, &dy_N);
  state_eval_thermo(t, conv ? 2 : 3, T, c);
  double avg = 0.0;
  for (int k = 0; k < N - 1; ++k) {
    const double v = c[k] * y[k + 1];
    avg = (k == 0) ? v : avg + v;
  }
  avg = (N > 1) ? avg + c[N - 1] * y_N : c[N - 1] * y_N;
  state_eval_thermo(t, conv ? 1 : 0, T, e);
  double sum = 0.0;
  for (int k = 0; k < N - 1; ++k) {
    const double v = dy[k + 1] * e[k] * t.sp_mw[k];
    sum = (k == 0) ? v : sum + v;
  }
  sum = (N > 1) ? sum + dy_N * e[N - 1] * t.sp_mw[N - 1] : dy_N * e[N - 1] * t.sp_mw[N - 1];
  dy[0] = (-1.0 / (rho * avg)) * sum;
  for (int k = 0; k < N - 1; ++k) dy[k + 1] *= (t.sp_mw[k] / rho);
}

}  // namespace
}  // namespace ref
}  // namespace crs

#endif /* CRS_EVAL_H */
