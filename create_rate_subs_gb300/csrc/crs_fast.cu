// CRS_MODE_FP64: FP64 throughout, restructured for GB300's FP64 pipe.
//
// On this part an FP64 instruction costs ~70 FP32 instructions, so the
// kernel is bound by the number of FP64 instructions per state.  Compared
// with the reference's operation order (crs_fp64_strict.cu) it
//  * evaluates exp with a table-driven method (Tang, ACM TOMS 15(2), 1989:
//    x = (256 k + j) ln2/256 + r, exp(x) = 2^k 2^(j/256) p(r), |r| <=
//    ln2/512, p the degree-4 Taylor polynomial; error below 1 ulp plus the
//    table rounding) -- 9 FP64 instructions instead of ~19 for CUDA's exp;
//  * multiplies by 1/T (one division per state) instead of dividing;
//  * forms the equilibrium constant from per-species Gibbs terms
//    S_k = s_k/R - h_k/RT - ln T evaluated once per state (the reference
//    sums the same NASA-7 coefficients per reaction on the host), and folds
//    1/Kc into the reverse rate constant: kr = exp(x_f - sum nu S - ln p),
//    one exponential instead of exp + exp + divide;
//  * computes the fall-off reduced pressure as exp(x_0 - x_inf) * [M].
// Results stay within 1e-12 (gross-rate scaled) of the reference.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <type_traits>

#include "crs_exp.cuh"
#include "crs_internal.cuh"
#include "crs_shapes.cuh"
#include "crs_tile.cuh"

namespace crs {

// ---- derived tables (host) ----------------------------------------------
namespace {
template <class T>
void put(std::vector<Derived> &v, int ImgLayout::*field, const std::vector<T> &src) {
  Derived d;
  d.field = field;
  d.bytes.resize(src.size() * sizeof(T));
  if (!src.empty()) memcpy(d.bytes.data(), src.data(), d.bytes.size());
  v.push_back(std::move(d));
}
}  // namespace

bool build_fast_tables(const std::vector<unsigned char> &img,
                       const ImgLayout &L, std::vector<Derived> &extra) {
  const Tab t = make_tab(img.data(), L);
  extra.clear();
  // per rate row: logA, b, -Ta (EXP kind); A, b, -Ta (other kinds)
  std::vector<double> rx(3 * (size_t)L.NRATE);
  for (int r = 0; r < L.NRATE; ++r) {
    const double *p = t.rate_par + 4 * r;
    rx[3 * r + 0] = (t.rate_kind[r] == RATE_EXP) ? p[1] : p[0];
    rx[3 * r + 1] = p[2];
    rx[3 * r + 2] = -p[3];
  }
  std::vector<double> lp(L.NREV > 0 ? L.NREV : 1);
  for (int j = 0; j < L.NREV; ++j) lp[j] = std::log(t.kc_pref[j]);
  std::vector<double> tx(5 * (size_t)(L.NPM > 0 ? L.NPM : 1), 0.0);
  std::vector<double> sx(5 * (size_t)(L.NPM > 0 ? L.NPM : 1), 0.0);
  for (int p = 0; p < L.NPM; ++p) {
    const double *c = t.pm_troe + 5 * p;
    tx[5 * p + 0] = c[0];
    tx[5 * p + 1] = -1.0 / c[1];
    tx[5 * p + 2] = c[2];
    tx[5 * p + 3] = -1.0 / c[3];
    tx[5 * p + 4] = -c[4];
    const double *s = t.pm_sri + 5 * p;
    sx[5 * p + 0] = s[0];
    sx[5 * p + 1] = -s[1];
    sx[5 * p + 2] = -1.0 / s[2];
    sx[5 * p + 3] = s[3];
    sx[5 * p + 4] = s[4];
  }
  // S_k(T) = g0 + g1 ln T + T (g2 + T (g3 + T (g4 + g5 T))) + g6 / T
  std::vector<double> g(14 * (size_t)L.N);
  for (int k = 0; k < L.N; ++k) {
    for (int h = 0; h < 2; ++h) {
      const double *a = (h ? t.sp_hi : t.sp_lo) + 7 * k;
      double *o = g.data() + 14 * k + 7 * h;
      o[0] = a[6] - a[0];
      o[1] = a[0] - 1.0;
      o[2] = a[1] / 2.0;
      o[3] = a[2] / 6.0;
      o[4] = a[3] / 12.0;
      o[5] = a[4] / 20.0;
      o[6] = -a[5];
    }
  }
  std::vector<double> et(256);
  for (int j = 0; j < 256; ++j) et[j] = (double)exp2l((long double)j / 256.0L);
  // (1/F, log F) for F = 1 + j/128 of the table logarithm (texp::log_t)
  std::vector<double> lt(2 * texp::LOG_TAB_ENTRIES);
  for (int j = 0; j < texp::LOG_TAB_ENTRIES; ++j) {
    const long double F = 1.0L + (long double)j / 128.0L;
    lt[2 * j] = (double)(1.0L / F);
    lt[2 * j + 1] = (double)logl(F);
  }
  put(extra, &ImgLayout::rate_x, rx);
  put(extra, &ImgLayout::kc_lpref, lp);
  // Kc polynomials with the prefactor folded in (single T_common group)
  bool single = true;
  for (int j = 0; j < L.NREV; ++j) single &= (t.kc_ptr[j + 1] - t.kc_ptr[j]) <= 1;
  std::vector<double> kp(16 * (size_t)(single && L.NREV > 0 ? L.NREV : 1), 0.0);
  if (single) {
    for (int j = 0; j < L.NREV; ++j) {
      double *o = kp.data() + 16 * j;
      o[0] = INFINITY;  // no group: the zero polynomial on both sides
      if (t.kc_ptr[j + 1] > t.kc_ptr[j]) {
        const int g = t.kc_ptr[j];
        o[0] = t.kc_tmid[g];
        for (int c = 0; c < 7; ++c) {
          o[2 + c] = t.kc_lo[7 * g + c];
          o[9 + c] = t.kc_hi[7 * g + c];
        }
      }
      o[2] += lp[j];
      o[9] += lp[j];
    }
  }
  put(extra, &ImgLayout::kc_poly, kp);
  // thermo utilities: RU/mw, mw, T_common and the NASA-7 coefficients in the
  // forms the emitted eval_h/u/cv/cp print (rate_subs.py:1513-1776)
  std::vector<double> th(24 * (size_t)L.N, 0.0);
  for (int k = 0; k < L.N; ++k) {
    double *o = th.data() + 24 * k;
    o[0] = 8314.4621 / t.sp_mw[k];  // chem.RU / mw, as the emitter prints it
    o[1] = t.sp_mw[k];
    o[2] = t.sp_tmid[k];
    for (int h = 0; h < 2; ++h) {
      const double *a = (h ? t.sp_hi : t.sp_lo) + 7 * k;
      double *c = o + 4 + 10 * h;
      for (int j = 0; j < 6; ++j) c[j] = a[j];
      c[6] = a[1] / 2.0;
      c[7] = a[2] / 3.0;
      c[8] = a[3] / 4.0;
      c[9] = a[4] / 5.0;
    }
  }
  put(extra, &ImgLayout::sp_thermo, th);
  put(extra, &ImgLayout::troe_x, tx);
  put(extra, &ImgLayout::sri_x, sx);
  put(extra, &ImgLayout::sp_gibbs, g);
  put(extra, &ImgLayout::exptab, et);
  put(extra, &ImgLayout::logtab, lt);
  // mixed-precision tables
  auto split = [](double v, float *h, float *l) {
    *h = (float)v;
    *l = (float)(v - (double)*h);
  };
  std::vector<float> rf(8 * (size_t)L.NRATE, 0.0f);
  for (int r = 0; r < L.NRATE; ++r) {
    const double *p = t.rate_par + 4 * r;  // A, logA, b, Ta
    double lnA = std::log(std::fabs(p[0]));
    double bb = p[2];
    if (t.rate_kind[r] == RATE_POW) bb = (double)t.rate_npow[r];
    if (t.rate_kind[r] == RATE_CONST) bb = 0.0;
    const double nTa = (t.rate_kind[r] == RATE_POW || t.rate_kind[r] == RATE_CONST) ? 0.0 : -p[3];
    split(lnA, &rf[8 * r + 0], &rf[8 * r + 1]);
    split(bb, &rf[8 * r + 2], &rf[8 * r + 3]);
    split(nTa, &rf[8 * r + 4], &rf[8 * r + 5]);
    rf[8 * r + 6] = p[0] < 0 ? -1.0f : 1.0f;
  }
  std::vector<float> imf(L.N);
  for (int k = 0; k < L.N; ++k) imf[k] = (float)t.inv_mw[k];
  std::vector<float> tf(8 * (size_t)(L.NPM > 0 ? L.NPM : 1), 0.0f);
  std::vector<float> sf(8 * (size_t)(L.NPM > 0 ? L.NPM : 1), 0.0f);
  for (int p = 0; p < L.NPM; ++p) {
    const double *c = tx.data() + 5 * p;  // P0, -1/T3, P2, -1/T1, -T2
    tf[8 * p + 0] = (float)c[0];
    split(c[1], &tf[8 * p + 1], &tf[8 * p + 2]);
    tf[8 * p + 3] = (float)c[2];
    split(c[3], &tf[8 * p + 4], &tf[8 * p + 5]);
    split(c[4], &tf[8 * p + 6], &tf[8 * p + 7]);
    const double *d = sx.data() + 5 * p;  // a, -b, -1/c, d, e
    sf[8 * p + 0] = (float)d[0];
    split(d[1], &sf[8 * p + 1], &sf[8 * p + 2]);
    split(d[2], &sf[8 * p + 3], &sf[8 * p + 4]);
    sf[8 * p + 5] = (float)d[3];
    sf[8 * p + 6] = (float)d[4];
  }
  const int ne = t.pm_eff_ptr[L.NPM];
  std::vector<float> ef(ne > 0 ? ne : 1, 0.0f);
  for (int e = 0; e < ne; ++e) ef[e] = (float)t.pm_eff_val[e];
  // the Kc polynomials (kc_poly, prefactor folded into c0) as float-float
  // pairs for the mixed kernels, -c6 stored so that every Horner step is a
  // multiply-add; T_common kept as a double for the same bit-pattern test
  std::vector<float> km(32 * (size_t)(single && L.NREV > 0 ? L.NREV : 1), 0.0f);
  if (single) {
    for (int j = 0; j < L.NREV; ++j) {
      for (int h = 0; h < 2; ++h) {
        const double *c = kp.data() + 16 * j + 2 + 7 * h;
        float *o = km.data() + 32 * j + 16 * h;
        for (int q = 0; q < 6; ++q) split(c[q], &o[2 * q], &o[2 * q + 1]);
        split(-c[6], &o[12], &o[13]);
        memcpy(o + 14, kp.data() + 16 * j, sizeof(double));
      }
    }
  }
  put(extra, &ImgLayout::kc_mix, km);
  put(extra, &ImgLayout::rate_ff, rf);
  put(extra, &ImgLayout::inv_mw_f, imf);
  put(extra, &ImgLayout::troe_ff, tf);
  put(extra, &ImgLayout::sri_ff, sf);
  put(extra, &ImgLayout::eff_f, ef);
  // reaction order for the shape-specialised paths and expanded factors
  // species indices as int16 (the mechanism is checked to have fewer than
  // 32768 species): half the shared memory of int32
  std::vector<int16_t> rfac((size_t)MAXF * (L.R > 0 ? L.R : 1), 0),
      pfac((size_t)MAXF * (L.R > 0 ? L.R : 1), 0);
  std::vector<int32_t> shape(L.R, NSHAPE);
  for (int r = 0; r < L.R; ++r) {
    bool ok = t.rate_kind[r] == RATE_EXP && t.pm_idx[r] < 0;
    int nr = 0, np = 0;
    for (int q = t.rx_ptr[r]; q < t.rx_ptr[r + 1]; ++q) {
      if (t.rx_nint[q] < 0) ok = false;
      for (int c = 0; c < t.rx_nint[q] && ok; ++c) {
        if (nr < MAXF) rfac[(size_t)MAXF * r + nr] = (int16_t)t.rx_sp[q];
        ++nr;
      }
    }
    for (int q = t.px_ptr[r]; q < t.px_ptr[r + 1]; ++q) {
      if (t.px_nint[q] < 0) ok = false;
      for (int c = 0; c < t.px_nint[q] && ok; ++c) {
        if (np < MAXF) pfac[(size_t)MAXF * r + np] = (int16_t)t.px_sp[q];
        ++np;
      }
    }
    const int nnu = t.nu_ptr[r + 1] - t.nu_ptr[r];
    const int rev = t.rev_idx[r] >= 0;
    if (!ok) continue;
    for (int sh = 0; sh < NSHAPE; ++sh) {
      const Shape d = shape_of(sh);
      if (d.nr == nr && d.np == np && d.nnu == nnu && d.rev == rev) {
        shape[r] = sh;
        break;
      }
    }
  }
  // seg[NSHAPE] .. seg[NSHAPE + 1]: the other reactions of exponential
  // form; seg[NSHAPE + 1] .. R: PLOG and Chebyshev reactions, last, so that
  // the hot general loop of the one-state-per-thread kernels has no code
  // for them
  std::vector<int32_t> perm, seg(NSHAPE + 2);
  for (int sh = 0; sh <= NSHAPE; ++sh) {
    seg[sh] = (int32_t)perm.size();
    for (int r = 0; r < L.R; ++r)
      if (shape[r] == sh && (sh < NSHAPE || t.rate_kind[r] < RATE_PLOG)) perm.push_back(r);
  }
  seg[NSHAPE + 1] = (int32_t)perm.size();
  for (int r = 0; r < L.R; ++r)
    if (shape[r] == NSHAPE && t.rate_kind[r] >= RATE_PLOG) perm.push_back(r);
  if (perm.empty()) perm.push_back(0);
  put(extra, &ImgLayout::perm, perm);
  // net-nu entries in compact form for the mixed one-state-per-thread kernel
  {
    const int nnz = t.nu_ptr[L.R];
    std::vector<int16_t> sp16(nnz > 0 ? nnz : 1, 0);
    std::vector<uint16_t> hi(nnz > 0 ? nnz : 1, 0);
    for (int e = 0; e < nnz; ++e) {
      uint64_t u;
      memcpy(&u, &t.nu_val[e], 8);
      sp16[e] = (int16_t)t.nu_sp[e];
      hi[e] = (uint16_t)(u >> 48);  // the top 16 bits of the double
    }
    put(extra, &ImgLayout::nu_sp16, sp16);
    put(extra, &ImgLayout::nu_hi, hi);
  }
  // warp-per-state kernels: reactions ordered so that 32 consecutive ones
  // mostly take the same code path (rate form, pressure modification,
  // broadening, reversibility, factor counts)
  std::vector<int32_t> dperm(L.R > 0 ? L.R : 1);
  {
    std::vector<std::pair<long long, int>> key;
    for (int r = 0; r < L.R; ++r) {
      const int p = t.pm_idx[r];
      const long long pmk = p < 0 ? 0 : 1 + t.pm_kind[p] * 3 + t.pm_form[p];
      const long long nr = t.rx_ptr[r + 1] - t.rx_ptr[r];
      const long long np = t.px_ptr[r + 1] - t.px_ptr[r];
      const long long k = ((((long long)(t.rate_kind[r] != RATE_EXP) * 16 + pmk) * 2 +
                            (t.rev_idx[r] >= 0)) * 8 + nr) * 8 + np;
      key.emplace_back(k, r);
    }
    std::stable_sort(key.begin(), key.end(),
                     [](const std::pair<long long, int> &a,
                        const std::pair<long long, int> &b) { return a.first < b.first; });
    for (int r = 0; r < L.R; ++r) dperm[r] = key[r].second;
  }
  // species-major net-nu CSR, entries in reaction order (the order in which
  // the reference adds the terms of each species)
  const int nnz = t.nu_ptr[L.R];
  std::vector<int32_t> sptr(L.N + 1, 0), sr(nnz > 0 ? nnz : 1), cnt(L.N, 0);
  std::vector<double> snu(nnz > 0 ? nnz : 1);
  for (int e = 0; e < nnz; ++e) sptr[t.nu_sp[e] + 1]++;
  for (int k = 0; k < L.N; ++k) sptr[k + 1] += sptr[k];
  for (int r = 0; r < L.R; ++r)
    for (int e = t.nu_ptr[r]; e < t.nu_ptr[r + 1]; ++e) {
      const int k = t.nu_sp[e];
      const int at = sptr[k] + cnt[k]++;
      sr[at] = r;
      snu[at] = t.nu_val[e];
    }
  // species to lanes, balancing the number of terms per lane (longest
  // first onto the least loaded lane)
  std::vector<int> order(L.N);
  for (int k = 0; k < L.N; ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return sptr[a + 1] - sptr[a] > sptr[b + 1] - sptr[b];
  });
  std::vector<std::vector<int>> bins(32);
  std::vector<long long> load(32, 0);
  for (int k : order) {
    int best = 0;
    for (int l = 1; l < 32; ++l)
      if (load[l] < load[best]) best = l;
    bins[best].push_back(k);
    load[best] += 1 + (sptr[k + 1] - sptr[k]);
  }
  std::vector<int32_t> lptr(33, 0), lsp;
  for (int l = 0; l < 32; ++l) {
    for (int k : bins[l]) lsp.push_back(k);
    lptr[l + 1] = (int32_t)lsp.size();
  }
  put(extra, &ImgLayout::dperm, dperm);
  put(extra, &ImgLayout::spc_ptr, sptr);
  put(extra, &ImgLayout::spc_r, sr);
  put(extra, &ImgLayout::spc_nu, snu);
  put(extra, &ImgLayout::lane_ptr, lptr);
  put(extra, &ImgLayout::lane_sp, lsp);
  put(extra, &ImgLayout::seg, seg);
  put(extra, &ImgLayout::rfac, rfac);
  put(extra, &ImgLayout::pfac, pfac);
  return true;
}

namespace fast {

using texp::exp_core;
using texp::exp_fix;
using texp::exp_t;
using texp::log_t;
constexpr double INV_RU = 0.0001202723625380408;
constexpr double LN10 = 2.302585092994046;
constexpr double INV_LN10 = 0.4342944819032518;

struct Col {
  double *p;
  int64_t stride;
  __device__ double &operator[](int k) const { return p[(int64_t)k * stride]; }
};

// Contiguous per-warp array (warp-per-state kernels).
struct Arr {
  double *p;
  __device__ double &operator[](int k) const { return p[k]; }
};

// Kc exponent from the per-species Gibbs column S: ln(prefactor) +
// sum_k nu_k S_k (the layouts that keep S on chip).
template <class CS>
struct KcCol {
  CS S;
  __device__ __forceinline__ double operator()(const Tab &t, int r, int j) const {
    double g = t.kc_lpref[j];
    for (int e = t.nu_ptr[r]; e < t.nu_ptr[r + 1]; ++e) g = fma(t.nu_val[e], S[t.nu_sp[e]], g);
    return g;
  }
};
template <class T>
struct IsKcCol { static constexpr bool value = false; };
template <class CS>
struct IsKcCol<KcCol<CS>> { static constexpr bool value = true; };

struct State {
  double T, invT, logT, P;
  const double *tab;   // 2^(j/256), exp_t
  const double *ltab;  // (1/F, log F), log_t
};

// Rate constant of row `row`; *x receives its exponent for the EXP kind.
__device__ __forceinline__ double rate(const Tab &t, int row, const State &s,
                                       double &x) {
  const double *c = t.rate_x + 3 * row;  // (logA | A), b, -Ta
  switch (t.rate_kind[row]) {
    case RATE_EXP:
      x = fma(c[2], s.invT, fma(c[1], s.logT, c[0]));
      return exp_t(x, s.tab);
    case RATE_CONST:
      return c[0];
    case RATE_NEGEXP:
      return c[0] * exp_t(fma(c[2], s.invT, c[1] * s.logT), s.tab);
    case RATE_POW: {
      double k = c[0];
      for (int j = 0; j < t.rate_npow[row]; ++j) k *= s.T;
      return k;
    }
    default:  // PLOG, Chebyshev
      return pdep_kf(t, row, s.T, s.logT, s.P);
  }
}

template <class CS>
__device__ __forceinline__ double product(const int32_t *sp, const int32_t *nint,
                                          const double *nu, int a, int b,
                                          const CS &C) {
  double p = 1.0;
  for (int j = a; j < b; ++j) {
    const double c = C[sp[j]];
    const int n = nint[j];
    if (n == 1) p *= c;
    else if (n == 2) p *= c * c;
    else if (n >= 0) for (int q = 0; q < n; ++q) p *= c;
    else p *= pow(c, nu[j]);
  }
  return p;
}

template <class CS>
__device__ double pres_mod(const Tab &t, int p, const State &s, double mix,
                           const CS &C) {
  double thd = mix;
  const int sp = t.pm_sp[p];
  if (t.pm_kind[p] == PM_THD || sp < 0) {
    for (int e = t.pm_eff_ptr[p]; e < t.pm_eff_ptr[p + 1]; ++e)
      thd = fma(t.pm_eff_val[e], C[t.pm_eff_sp[e]], thd);
    if (t.pm_kind[p] == PM_THD) return thd;
  } else {
    thd = C[sp];
  }
  const int r0 = t.pm_k0[p], ri = t.pm_kinf[p];
  double Pr;
  if (t.rate_kind[r0] == RATE_EXP && t.rate_kind[ri] == RATE_EXP) {
    const double *a = t.rate_x + 3 * r0, *b = t.rate_x + 3 * ri;
    const double x0 = fma(a[2], s.invT, fma(a[1], s.logT, a[0]));
    const double xi = fma(b[2], s.invT, fma(b[1], s.logT, b[0]));
    Pr = exp_t(x0 - xi, s.tab) * thd;
  } else {
    double x;
    const double k0 = rate(t, r0, s, x);
    const double ki = rate(t, ri, s, x);
    Pr = k0 * thd / ki;
  }
  const bool low = t.pm_kind[p] == PM_FALL_LOW;
  const double inv1p = 1.0 / (1.0 + Pr);
  const int form = t.pm_form[p];
  if (form == FORM_LINDEMANN) return low ? Pr * inv1p : inv1p;
  const double lP = log_t(fmax(Pr, 1.0e-300), s.ltab) * INV_LN10;
  double F;
  if (form == FORM_TROE) {
    const double *c = t.troe_x + 5 * p;  // P0, -1/T3, P2, -1/T1, -T2
    double f = c[0] * exp_t(s.T * c[1], s.tab) + c[2] * exp_t(s.T * c[3], s.tab);
    if (t.pm_troe_t2[p]) f += exp_t(c[4] * s.invT, s.tab);
    const double lF = log_t(fmax(f, 1.0e-300), s.ltab) * INV_LN10;
    const double A = lP - 0.67 * lF - 0.4;
    const double B = 0.806 - 1.1762 * lF - 0.14 * lP;
    // log10 F = log10 Fcent / (1 + A^2/B^2) = log10 Fcent B^2 / (B^2 + A^2):
    // one division
    const double B2 = B * B;
    F = exp_t(LN10 * lF * B2 / fma(A, A, B2), s.tab);
  } else {
    const double *c = t.sri_x + 5 * p;  // a, -b, -1/c, d, e
    const double X = 1.0 / (1.0 + lP * lP);
    const double base = c[0] * exp_t(c[1] * s.invT, s.tab) + exp_t(s.T * c[2], s.tab);
    F = exp_t(X * log_t(base, s.ltab), s.tab);
    if (t.pm_sri_de[p]) F *= c[3] * exp_t(c[4] * s.logT, s.tab);
  }
  return low ? F * Pr * inv1p : F * inv1p;
}

// wdot[k] += nu * net for the reactions of one block, in order.
template <int NNU, class DC>
__device__ __forceinline__ void accumulate(const Tab &t, const int *rr, int cnt,
                                           const double (&net)[4], const DC &W) {
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    if (u >= cnt) break;
    const int e0 = t.nu_ptr[rr[u]];
    // the species of one reaction are distinct: all its loads go before its
    // stores, so that they overlap instead of waiting on each other
    int k[NNU];
    double w[NNU];
#pragma unroll
    for (int q = 0; q < NNU; ++q) {
      k[q] = t.nu_sp[e0 + q];
      w[q] = W[k[q]];
    }
#pragma unroll
    for (int q = 0; q < NNU; ++q) W[k[q]] = fma(t.nu_val[e0 + q], net[u], w[q]);
  }
}

// Four reactions of one shape (crs_shapes.cuh): rate constants, products
// and net rates with compile-time trip counts, so that the four dependency
// chains interleave; then their wdot contributions in order.
// Sink of the on-chip kernels: net rates accumulate into the state's wdot
// column, block by block or one reaction at a time, in order.
struct WSink {
  Col W;
  template <int NNU>
  __device__ __forceinline__ void block(const Tab &t, const int *rr, int cnt,
                                        const double (&net)[4]) const {
    accumulate<NNU>(t, rr, cnt, net, W);
  }
  __device__ __forceinline__ void one(const Tab &t, int r, double net) const {
    for (int e = t.nu_ptr[r]; e < t.nu_ptr[r + 1]; ++e) {
      const int k = t.nu_sp[e];
      W[k] = fma(t.nu_val[e], net, W[k]);
    }
  }
};

template <int NR, int NP, int NNU, int REV, bool STAGES, class KC, class CC, class SINK>
__device__ __forceinline__ void shape_block(const Tab &t, const int *rr,
                                            int cnt, const State &s,
                                            const CC &C, const KC &kc,
                                            const SINK &sink, const Batch &b,
                                            int64_t i) {
  double net[4], x[4], e[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const double *c = t.rate_x + 3 * rr[u];
    x[u] = fma(c[2], s.invT, fma(c[1], s.logT, c[0]));
    e[u] = exp_core(x[u], s.tab);
  }
  double fwd[4], rev[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int r = rr[u];
    double f = exp_fix(x[u], e[u]);
#pragma unroll
    for (int q = 0; q < NR; ++q) f *= C[t.rfac[MAXF * r + q]];
    fwd[u] = f;
    rev[u] = 0.0;
    if (REV) {
      double g;
      if constexpr (IsKcCol<KC>::value) {
        const int e0 = t.nu_ptr[r];
        g = t.kc_lpref[t.rev_idx[r]];
#pragma unroll
        for (int q = 0; q < NNU; ++q) g = fma(t.nu_val[e0 + q], kc.S[t.nu_sp[e0 + q]], g);
      } else {
        g = kc(t, r, t.rev_idx[r]);
      }
      x[u] = x[u] - g;
      e[u] = exp_core(x[u], s.tab);
    }
  }
  if (REV) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int r = rr[u];
      double v = exp_fix(x[u], e[u]);
#pragma unroll
      for (int q = 0; q < NP; ++q) v *= C[t.pfac[MAXF * r + q]];
      rev[u] = v;
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) net[u] = fwd[u] - rev[u];
  if (STAGES) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (u >= cnt) break;
      if (b.fwd) b.fwd[(int64_t)rr[u] * b.ld + i] = fwd[u];
      if (REV && b.rev) b.rev[(int64_t)t.rev_idx[rr[u]] * b.ld + i] = rev[u];
    }
  }
  sink.template block<NNU>(t, rr, cnt, net);
}

// The shape groups' blocks of four reactions, in order; a caller that
// splits the blocks among npart workers evaluates blocks part, part +
// npart, ... of every group.
template <int SH, bool STAGES, class KC, class CC, class SINK>
struct Shapes {
  __device__ __forceinline__ static void run(const Tab &t, const State &s,
                                             const CC &C, const KC &S,
                                             const SINK &sink, const Batch &b,
                                             int64_t i, int part = 0, int npart = 1) {
    constexpr Shape d = shape_of(SH);
    const int p0 = t.seg[SH], p1 = t.seg[SH + 1];
    for (int p = p0 + 4 * part; p < p1; p += 4 * npart) {
      const int cnt = p1 - p < 4 ? p1 - p : 4;
      int rr[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) rr[u] = t.perm[p + (u < cnt ? u : cnt - 1)];
      shape_block<d.nr, d.np, d.nnu, d.rev, STAGES>(t, rr, cnt, s, C, S, sink, b, i);
    }
    Shapes<SH + 1, STAGES, KC, CC, SINK>::run(t, s, C, S, sink, b, i, part, npart);
  }
};
template <bool STAGES, class KC, class CC, class SINK>
struct Shapes<NSHAPE, STAGES, KC, CC, SINK> {
  __device__ __forceinline__ static void run(const Tab &, const State &,
                                             const CC &, const KC &,
                                             const SINK &, const Batch &,
                                             int64_t, int = 0, int = 1) {}
};

// Net rate (fwd - rev) * pres_mod of any reaction: general rate forms,
// pressure modification, non-integer coefficients.
template <class CS, class KC>
__device__ __forceinline__ double rxn_net(const Tab &t, int r, const State &s,
                                          double mix, const CS &C, const KC &kc,
                                          double &fwd, double &rev, double &pm) {
  double xf = 0.0;
  const double kf = rate(t, r, s, xf);
  fwd = kf * product(t.rx_sp, t.rx_nint, t.rx_nu, t.rx_ptr[r], t.rx_ptr[r + 1], C);
  const int j = t.rev_idx[r];
  double net = fwd;
  rev = 0.0;
  if (j >= 0) {
    const double gsum = kc(t, r, j);
    const double kr = (t.rate_kind[r] == RATE_EXP) ? exp_t(xf - gsum, s.tab)
                                                   : kf * exp_t(-gsum, s.tab);
    rev = kr * product(t.px_sp, t.px_nint, t.px_nu, t.px_ptr[r], t.px_ptr[r + 1], C);
    net = fwd - rev;
  }
  const int p = t.pm_idx[r];
  pm = 1.0;
  if (p >= 0) {
    pm = pres_mod(t, p, s, mix, C);
    net *= pm;
  }
  return net;
}

template <bool STAGES, class KC, class CC, class SINK>
__device__ __forceinline__ void general(const Tab &t, int r, const State &s,
                                        double mix, const CC &C,
                                        const KC &S, const SINK &sink,
                                        const Batch &b, int64_t i) {
  double fwd, rev, pm;
  const double net = rxn_net(t, r, s, mix, C, S, fwd, rev, pm);
  if (STAGES) {
    const int j = t.rev_idx[r], p = t.pm_idx[r];
    if (b.fwd) b.fwd[(int64_t)r * b.ld + i] = fwd;
    if (b.rev && j >= 0) b.rev[(int64_t)j * b.ld + i] = rev;
    if (b.pm && p >= 0) b.pm[(int64_t)p * b.ld + i] = pm;
  }
  sink.one(t, r, net);
}

// KCM 0: Kc from a per-species Gibbs column S (3 columns of 8 B per
// species and thread); 1 / 2: from the per-reaction Kc polynomials (single /
// several T_common groups; 2 columns, so more threads fit next to the
// tables).
template <bool STAGES, int KCM>
__global__ void __launch_bounds__(256, 1)
    k_wdot(const unsigned char *__restrict__ img, ImgLayout L, Batch b) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  const unsigned amask = __activemask();
  const int lane = threadIdx.x & 31;
  Tab t;
  int nb;
  if (!stage_ranges(smem, img, L, 0, &bar, b.status, t, nb)) {
    sched_done(b.sched, amask, lane);
    return;
  }
  const int N = t.N;
  double *base = reinterpret_cast<double *>(smem + nb);
  const int64_t st = blockDim.x;
  const Col C{base + threadIdx.x, st};
  const Col W{base + (int64_t)N * st + threadIdx.x, st};
  const Col S{base + (int64_t)2 * N * st + threadIdx.x, st};  // KCM 0 only
  int bad = 0;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - (int64_t)gridDim.x * blockDim.x;
  for (;;) {
    if (b.sched) {
      i = sched_next(b.sched, b.n, amask, lane);
      if (i < 0) break;
      if (i >= b.n) continue;
    } else {
      i += (int64_t)gridDim.x * blockDim.x;
      if (i >= b.n) break;
    }
    State s;
    s.T = b.T[i];
    const double P = b.P[i];
    s.P = P;
    s.invT = 1.0 / s.T;
    s.logT = log_t(s.T, t.logtab);
    s.tab = t.exptab;
    s.ltab = t.logtab;
    // eval_conc
    double ysum = 0.0, mwi = 0.0;
    for (int k = 0; k < N - 1; ++k) {
      const double y = b.Y[(int64_t)k * b.ld + i];
      C[k] = y;
      ysum += y;
      mwi = fma(y, t.inv_mw[k], mwi);
    }
    const double yN = 1.0 - ysum;
    mwi = fma(yN, t.inv_mw[N - 1], mwi);
    const double rho = P / mwi * (s.invT * INV_RU);
    for (int k = 0; k < N - 1; ++k) C[k] = C[k] * (rho * t.inv_mw[k]);
    C[N - 1] = yN * (rho * t.inv_mw[N - 1]);
    const long long Tbits = __double_as_longlong(s.T);
    for (int k = 0; k < N; ++k) {
      if (KCM == 0) {
        // per-species Gibbs terms (T <= T_common on the positive doubles'
        // bit patterns)
        const double *g = t.sp_gibbs + 14 * k +
                          ((Tbits <= __double_as_longlong(t.sp_tmid[k])) ? 0 : 7);
        const double h = fma(fma(fma(g[5], s.T, g[4]), s.T, g[3]), s.T, g[2]);
        double v = fma(h, s.T, g[0]);
        v = fma(g[1], s.logT, v);
        S[k] = fma(g[6], s.invT, v);
      }
      W[k] = 0.0;
    }
    if (STAGES && b.conc)
      for (int k = 0; k < N; ++k) b.conc[(int64_t)k * b.ld + i] = C[k];
    const double mix = P * s.invT * INV_RU;
    const WSink sink{W};
    if constexpr (KCM == 0) {
      const KcCol<Col> kc{S};
      Shapes<0, STAGES, KcCol<Col>, Col, WSink>::run(t, s, C, kc, sink, b, i);
      for (int p = t.seg[NSHAPE]; p < t.R; ++p)
        general<STAGES>(t, t.perm[p], s, mix, C, kc, sink, b, i);
    } else {
      using KC = typename std::conditional<KCM == 1, KcPoly1, KcPolyG>::type;
      KC kc;
      kc.T = s.T;
      kc.logT = s.logT;
      kc.invT = s.invT;
      if constexpr (KCM == 1) kc.Tbits = Tbits;
      Shapes<0, STAGES, KC, Col, WSink>::run(t, s, C, kc, sink, b, i);
      for (int p = t.seg[NSHAPE]; p < t.R; ++p)
        general<STAGES>(t, t.perm[p], s, mix, C, kc, sink, b, i);
    }
    for (int k = 0; k < N; ++k) {
      const double v = W[k];
      bad += ((__double2hiint(v) >> 20) & 0x7ff) == 0x7ff;  // inf or NaN, integer test
      b.wdot[(int64_t)k * b.ld + i] = v;
    }
  }
  if (bad && b.status) atomicAdd(&b.status[1], bad);
  sched_done(b.sched, amask, lane);
}

// ---- state tiles (two passes over HBM; see crs_large.cu) ---------------
// FP64 concentrations of a tile of 32 states in shared memory ([N][32],
// 256 B per species), FTW warps taking the shape blocks round-robin, every
// net rate written to HBM for the species sums.  For mechanisms whose
// per-thread columns do not fit on chip.
// 12 warps at 168 registers (8: 4.59, 12: 4.81, 16: 4.76 M states/s at 561/2539;
// 4.90 at 12 with the state sums on two warps)
constexpr int FTW = 12;
static_assert(FTW >= 2, "tile::state_sums runs on warps 0 and 1");

template <bool KC1>
__global__ void __launch_bounds__(FTW * 32, 1)
    k_rates_tile64(const unsigned char *__restrict__ img, ImgLayout L, Batch b,
                   tile::RatesOut o) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ double s_rho[32], s_yN[32];
  __shared__ int64_t s_tile;
  const Tab t = make_tab(img, L);
  const int N = t.N, R = t.R;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Col C{reinterpret_cast<double *>(smem) + lane, 32};
  const int64_t ntiles = (b.n + 31) / 32;
  for (;;) {
    const int64_t tile = tile::next_tile(b.sched, &s_tile);
    if (tile >= ntiles) break;
    const int64_t i = tile * 32 + lane;
    const bool valid = i < b.n;
    const int64_t ic = valid ? i : tile * 32;  // idle lanes repeat a valid state
    State s;
    s.T = b.T[ic];
    const double P = b.P[ic];
    s.P = P;
    s.invT = 1.0 / s.T;
    s.logT = log_t(s.T, t.logtab);
    s.tab = t.exptab;
    s.ltab = t.logtab;
    tile::state_sums(t, b, ic, warp, lane, P, s.invT * INV_RU, s_yN, s_rho);
    __syncthreads();
    const double rho = s_rho[lane];
    for (int k = warp; k < N; k += FTW) {
      const double y = k == N - 1 ? s_yN[lane] : b.Y[(int64_t)k * b.ld + ic];
      C[k] = y * (rho * t.inv_mw[k]);
    }
    __syncthreads();
    const double mix = P * s.invT * INV_RU;
    using KC = typename std::conditional<KC1, KcPoly1, KcPolyG>::type;
    KC kc;
    kc.T = s.T;
    kc.logT = s.logT;
    kc.invT = s.invT;
    if constexpr (KC1) kc.Tbits = __double_as_longlong(s.T);
    int esum = 0, ecnt = 0;
    const tile::QSink sink{o.q + i, o.ldq, valid, esum, ecnt};
    Shapes<0, false, KC, Col, tile::QSink>::run(t, s, C, kc, sink, b, i, warp, FTW);
    for (int p = t.seg[NSHAPE] + warp; p < R; p += FTW)
      general<false>(t, t.perm[p], s, mix, C, kc, sink, b, i);
    // the next tile replaces C only after every warp is done with this one
    __syncthreads();
  }
  tile::tiles_done(b.sched);
}

// ---- warp per state -----------------------------------------------------
// A warp evaluates one state at a time: lanes split the species for the
// concentrations and Gibbs terms, the reactions (in dperm order) for the
// net rates, which go to a per-warp buffer q[R], and then the species
// again -- balanced lane bins over the species-major CSR -- to sum wdot in
// reaction order.  Per-state scalars (1/T, ln T) are computed once per
// state by one lane of a 32-state batch.  With no per-thread arrays, many
// more warps fit on an SM than with one state per thread.
constexpr int DW = 8;  // most warps per CTA

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <bool STAGES, bool SMEM_TAB>
__global__ void __launch_bounds__(DW * 32)
    k_wdot_warp(const unsigned char *__restrict__ img, ImgLayout L, Batch b,
                int per_warp) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  int nb = 0;
  Tab t;
  if (SMEM_TAB) {
    if (!stage_ranges(smem, img, L, 1, &bar, b.status, t, nb)) return;
  } else {
    t = make_tab(img, L);
  }
  const int N = t.N, R = t.R;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *wb = reinterpret_cast<double *>(smem + nb) + (size_t)warp * per_warp;
  double *bT = wb, *bP = wb + 32, *biT = wb + 64, *blT = wb + 96;
  const Arr C{wb + 128};
  const Arr S{wb + 128 + N};
  double *q = wb + 128 + 2 * N;
  const int l0 = t.lane_ptr[lane], l1 = t.lane_ptr[lane + 1];
  int bad = 0;
  const int nw = blockDim.x >> 5;
  const int64_t nwarp = (int64_t)gridDim.x * nw;
  for (int64_t i0 = ((int64_t)blockIdx.x * nw + warp) * 32; i0 < b.n; i0 += nwarp * 32) {
    // per-state scalars of a batch of 32 consecutive states, one per lane
    {
      const int64_t i = i0 + lane;
      const double T = i < b.n ? b.T[i] : 1000.0;
      bT[lane] = T;
      bP[lane] = i < b.n ? b.P[i] : 101325.0;
      biT[lane] = 1.0 / T;
      blT[lane] = log_t(T, t.logtab);
    }
    __syncwarp();
    const int jn = (b.n - i0) < 32 ? (int)(b.n - i0) : 32;
    for (int j = 0; j < jn; ++j) {
      const int64_t i = i0 + j;
      State s;
      s.T = bT[j];
      s.invT = biT[j];
      s.logT = blT[j];
      s.tab = t.exptab;
      s.ltab = t.logtab;
      const double P = bP[j];
      s.P = P;
      // concentrations (lanes over species)
      double mw = 0.0;
      for (int k = lane; k < N - 1; k += 32) {
        const double y = b.Y[(int64_t)k * b.ld + i];
        C[k] = y;
        mw = fma(y, t.inv_mw[k], mw);
      }
      mw = warp_sum(mw);
      __syncwarp();
      // y_N = 1 - sum y in the reference's left-to-right order on every
      // lane (rate_subs.py:1312-1320): where the bath gas is scarce, the
      // rounding of this difference is a large relative error of C_N
      double ys = N > 1 ? C[0] : 0.0;
      for (int k = 1; k < N - 1; ++k) ys += C[k];
      const double yN = 1.0 - ys;
      mw = fma(yN, t.inv_mw[N - 1], mw);
      const double rho = P / mw * (s.invT * INV_RU);
      __syncwarp();
      for (int k = lane; k < N; k += 32) {
        const double y = (k == N - 1) ? yN : C[k];
        const double c = y * (rho * t.inv_mw[k]);
        C[k] = c;
        if (STAGES && b.conc) b.conc[(int64_t)k * b.ld + i] = c;
        const double *g = t.sp_gibbs + 14 * k + ((s.T <= t.sp_tmid[k]) ? 0 : 7);
        const double h = fma(fma(fma(g[5], s.T, g[4]), s.T, g[3]), s.T, g[2]);
        double v = fma(h, s.T, g[0]);
        v = fma(g[1], s.logT, v);
        S[k] = fma(g[6], s.invT, v);
      }
      __syncwarp();
      // net rates (lanes over reactions)
      const double mix = P * s.invT * INV_RU;
      for (int p = lane; p < R; p += 32) {
        const int r = t.dperm[p];
        double fwd, rev, pm;
        q[r] = rxn_net(t, r, s, mix, C, KcCol<Arr>{S}, fwd, rev, pm);
        if (STAGES) {
          const int jr = t.rev_idx[r], pp = t.pm_idx[r];
          if (b.fwd) b.fwd[(int64_t)r * b.ld + i] = fwd;
          if (b.rev && jr >= 0) b.rev[(int64_t)jr * b.ld + i] = rev;
          if (b.pm && pp >= 0) b.pm[(int64_t)pp * b.ld + i] = pm;
        }
      }
      __syncwarp();
      // wdot (lanes over species, terms in reaction order)
      for (int a = l0; a < l1; ++a) {
        const int k = t.lane_sp[a];
        double w = 0.0;
        for (int e = t.spc_ptr[k]; e < t.spc_ptr[k + 1]; ++e)
          w = fma(t.spc_nu[e], q[t.spc_r[e]], w);
        bad += !isfinite(w);
        b.wdot[(int64_t)k * b.ld + i] = w;
      }
      __syncwarp();
    }
  }
  if (bad && b.status) atomicAdd(&b.status[1], bad);
}

}  // namespace fast

int grid_for(int64_t n, int block, int max_ctas);

// Thread-per-state variant (kept for comparison: CRS_MODE_FP64_TPS).
cudaError_t launch_wdot_fp64_tps(const unsigned char *img, const ImgLayout &L,
                                 const Batch &b, int sm_count, int smem_optin,
                                 cudaStream_t s) {
  const size_t tab = (size_t)(L.rng[0][1] - L.rng[0][0] + L.rng[0][3] - L.rng[0][2]);
  auto fit = [&](int cols) {
    const long long room = (long long)smem_optin - (long long)tab;
    int nt = room > 0 ? (int)(room / ((long long)cols * L.N * 8)) / 32 * 32 : 0;
    return nt > 256 ? 256 : nt;
  };
  // the polynomial layout when it buys more threads than the Gibbs column
  const int nt2 = fit(2), nt3 = fit(3);
  const int kcm = (nt2 > nt3 && nt2 >= 64) ? (L.kc_single ? 1 : 2) : 0;
  const int block = kcm ? nt2 : nt3;
  if (block < 32) return cudaErrorNotSupported;
  const size_t bytes = tab + (size_t)(kcm ? 2 : 3) * L.N * block * sizeof(double);
  const bool stages = b.conc || b.fwd || b.rev || b.pm;
  void (*k)(const unsigned char *, ImgLayout, Batch);
  if (kcm == 0) k = stages ? fast::k_wdot<true, 0> : fast::k_wdot<false, 0>;
  else if (kcm == 1) k = stages ? fast::k_wdot<true, 1> : fast::k_wdot<false, 1>;
  else k = stages ? fast::k_wdot<true, 2> : fast::k_wdot<false, 2>;
  const cudaError_t e = set_smem_limit(k, bytes);
  if (e != cudaSuccess) return e;
  k<<<grid_for(b.n, block, sm_count), block, bytes, s>>>(img, L, b);
  return cudaGetLastError();
}

// FP64 rates of n states (b: chunk-local, no intermediates) into q [R][ldq]
// by state tiles; b.sched must be a free counter pair.
cudaError_t launch_rates_tile64(const unsigned char *img, const ImgLayout &L, const Batch &b,
                                int sm_count, int smem_optin, cudaStream_t s, double *q,
                                int64_t ldq) {
  const size_t bytes = (size_t)L.N * 32 * sizeof(double);
  if (bytes > (size_t)smem_optin || !b.sched) return cudaErrorNotSupported;
  auto k = L.kc_single ? fast::k_rates_tile64<true> : fast::k_rates_tile64<false>;
  cudaError_t e = set_smem_limit(k, bytes);
  if (e != cudaSuccess) return e;
  int per_sm = 1;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, fast::FTW * 32, bytes);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorNotSupported;
  const int grid = grid_for((b.n + 31) / 32, 1, sm_count * per_sm);
  k<<<grid, fast::FTW * 32, bytes, s>>>(img, L, b, tile::RatesOut{q, ldq, nullptr});
  return cudaGetLastError();
}

cudaError_t launch_wdot_fp64(const unsigned char *img, const ImgLayout &L,
                             const Batch &b, int sm_count, int smem_optin,
                             cudaStream_t s) {
  const int per_warp = 128 + 2 * L.N + L.R + 1;  // doubles
  const size_t pw = (size_t)per_warp * sizeof(double);
  const size_t tab = (size_t)(L.rng[1][1] - L.rng[1][0] + L.rng[1][3] - L.rng[1][2]);
  const bool stages = b.conc || b.fwd || b.rev || b.pm;
  const int64_t nbatch = (b.n + 31) / 32;
  // tables on chip with 8 warps if they fit, else tables in global memory
  // and as many warps (up to 8) as the per-warp buffers allow
  bool smem_tab = tab + fast::DW * pw <= (size_t)smem_optin;
  int nw = fast::DW;
  if (!smem_tab) {
    nw = (int)((size_t)smem_optin / pw);
    if (nw > fast::DW) nw = fast::DW;
    if (nw < 1) return cudaErrorNotSupported;
  }
  const size_t bytes = (smem_tab ? tab : 0) + nw * pw;
  auto k = smem_tab ? (stages ? fast::k_wdot_warp<true, true> : fast::k_wdot_warp<false, true>)
                    : (stages ? fast::k_wdot_warp<true, false> : fast::k_wdot_warp<false, false>);
  cudaError_t e = set_smem_limit(k, bytes);
  if (e != cudaSuccess) return e;
  int per_sm = 1;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, nw * 32, bytes);
  if (e != cudaSuccess) return e;
  const int grid = grid_for(nbatch, nw, sm_count * (per_sm > 0 ? per_sm : 1));
  k<<<grid, nw * 32, bytes, s>>>(img, L, b, per_warp);
  return cudaGetLastError();
}

}  // namespace crs
