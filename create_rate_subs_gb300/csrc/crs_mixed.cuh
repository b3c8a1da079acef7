// Mixed-precision arithmetic of one reaction for one state (CRS_MODE_MIXED
// and the contraction producer; see crs_mixed.cu for the precision split).
// Shared by the one-state-per-thread and warp kernels (crs_mixed.cu) and
// the state-tile rates producer of large mechanisms (crs_large.cu).  The
// shape blocks hand their net rates to a sink: accumulation into the
// state's wdot column on chip (WSink), or the rates themselves to HBM.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <type_traits>

#include "crs_internal.cuh"
#include "crs_shapes.cuh"

namespace crs {
namespace mixed {

constexpr float LOG2E_F = 1.4426950216293335f;
constexpr float LN2_HI_F = 0.693145751953125f;  // 16 significant bits
constexpr float LN2_LO_F = 1.428606765330187e-06f;
constexpr float SHIFT_F = 12582912.0f;          // 1.5 * 2^23
constexpr double INV_RU = 0.0001202723625380408;
constexpr float INV_LN10_F = 0.4342944920063019f;       // 1/ln 10 = INV_LN10_F + INV_LN10_LO_F
constexpr float INV_LN10_LO_F = -1.0103049952192578e-08f;
constexpr float LN2_H12_F = 0.693115234375f;            // ln 2, 12 significant bits
constexpr float LN2_L12_F = 3.194618329871446e-05f;     // ln 2 - LN2_H12_F

struct ff {
  float h, l;
};

__device__ __forceinline__ ff ff_norm(float s, float e) {
  const float h = s + e;
  return ff{h, e - (h - s)};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const float s = a.h + b.h;
  const float bb = s - a.h;
  float e = (a.h - (s - bb)) + (b.h - bb);
  e += a.l + b.l;
  return ff_norm(s, e);
}
__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.h, -a.l}; }
__device__ __forceinline__ ff ff_mul(ff a, ff b);
// a / b: one fp32 quotient, its residual a - q b in float-float, a
// correction quotient
__device__ __forceinline__ ff ff_div(ff a, ff b) {
  const float q1 = a.h / b.h;
  const ff r = ff_add(a, ff_neg(ff_mul(b, ff{q1, 0.0f})));
  const float q2 = r.h / b.h;
  return ff_norm(q1, q2);
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return ff_norm(p, e);
}

// exact float -> double for normal numbers, by integer operations
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0u || e == 0xffu) return (double)f;
  const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3);
  return __hiloint2double((int)hi, (int)(u << 29));
}

// double -> float, round to nearest even, by integer operations when the
// result is a normal float
__device__ __forceinline__ float d2f_rn(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
  if (e <= 0 || e >= 255) return __double2float_rn(d);
  const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned rest = lo & 0x1fffffffu;
  unsigned u = (hi & 0x80000000u) | ((unsigned)e << 23) | mant;
  u += (rest > 0x10000000u) || (rest == 0x10000000u && (mant & 1u));
  return __uint_as_float(u);
}

__device__ __forceinline__ ff ff_from_double(double d) {
  const float h = d2f_rn(d);
  return ff{h, d2f_rn(d - f2d_exact(h))};
}

// The same split by integer operations only (no FP64 instruction): h = d
// truncated to 24 significant bits, l = the remaining 29 bits of the
// significand converted once to fp32.  |d| below 2^-100 gives (0, 0), an
// absolute error far below what an exponent argument can notice.
__device__ __forceinline__ ff ff_from_double_int(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023;
  if (e < -100 || e > 127) return e > 127 ? ff{d2f_rn(d), 0.0f} : ff{0.0f, 0.0f};
  const unsigned sign = hi & 0x80000000u;
  const float h = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | ((hi & 0xfffffu) << 3) |
                                  (lo >> 29));
  const float m = (float)(lo & 0x1fffffffu);  // exact below 2^24, else rounded once
  // times 2^(e - 52): one normal power of two for e >= -74, else two
  const float l = (e >= -74) ? m * __uint_as_float((unsigned)(e + 75) << 23)
                             : m * __uint_as_float((unsigned)(e + 139) << 23) *
                                   5.421010862427522e-20f;  // 2^-64
  return ff{h, sign ? -l : l};
}

// value m * 2^E as a double, by integer operations (selects, no branches);
// m is an FP32 number whose magnitude stays within [2^-8, 2^8] or is zero
// / non-finite.  Zero and underflow give +0, overflow +-inf, inf / NaN m
// the same as a double.
__device__ __forceinline__ double assemble(float m, int E) {
  const unsigned u = __float_as_uint(m);
  const int fe = (int)((u >> 23) & 0xffu);
  const unsigned sign = u & 0x80000000u, mant = u & 0x7fffffu;
  const int de = fe - 127 + 1023 + E;
  unsigned hi = sign | ((unsigned)de << 20) | (mant >> 3), lo = u << 29;
  const bool special = fe == 0xff;
  const bool ovf = !special && de >= 2047;
  const bool unf = !special && (fe == 0 || de <= 0);
  hi = ovf ? (sign | 0x7ff00000u) : hi;
  lo = ovf ? 0u : lo;
  hi = special ? (sign | 0x7ff00000u | (mant >> 3)) : hi;
  hi = unf ? 0u : hi;
  lo = unf ? 0u : lo;
  return __hiloint2double((int)hi, (int)lo);
}

// exp(x) for a float-float x, as (p, k) with exp(x) = p * 2^k,
// p in [0.70, 1.42]
__device__ __forceinline__ float ff_exp(ff x, int &k) {
  // far outside the FP64 range: clamp (selects, no branches); NaN passes
  const bool nan = x.h != x.h;
  const bool big = !(fabsf(x.h) <= 3.0e3f);
  const float xh = big ? copysignf(3.0e3f, x.h) : x.h;
  const float xl = big ? 0.0f : x.l;
  const float t = fmaf(xh, LOG2E_F, SHIFT_F);
  const float kf = t - SHIFT_F;
  k = nan ? 0 : __float_as_int(t) - 0x4b400000;
  float r = fmaf(kf, -LN2_HI_F, xh);
  r = fmaf(kf, -LN2_LO_F, r);
  r = r + xl;
  float p = fmaf(r, 1.0f / 5040.0f, 1.0f / 720.0f);
  p = fmaf(p, r, 1.0f / 120.0f);
  p = fmaf(p, r, 1.0f / 24.0f);
  p = fmaf(p, r, 1.0f / 6.0f);
  p = fmaf(p, r, 0.5f);
  p = fmaf(p, r, 1.0f);
  p = fmaf(p, r, 1.0f);
  return nan ? x.h : p;
}

// exp of a float-float argument as a plain float (saturating)
__device__ __forceinline__ float ff_expf(ff x) {
  if (x.h > 88.0f) return INFINITY;
  if (x.h < -103.0f) return 0.0f;
  int k;
  const float p = ff_exp(x, k);
  return ldexpf(p, k);
}

// split a float into mantissa in [1,2) (sign kept) and exponent; zero and
// subnormal values give m = 0
__device__ __forceinline__ float fsplit(float c, int &e) {
  const unsigned u = __float_as_uint(c);
  const unsigned fe = (u >> 23) & 0xffu;
  const bool z = fe == 0u;  // selects, not branches: keeps callers straight-line
  e = z ? 0 : (int)fe - 127;
  return z ? 0.0f : __uint_as_float((u & 0x807fffffu) | 0x3f800000u);
}

struct FCol {
  float *p;
  int stride;
  __device__ float &operator[](int k) const { return p[k * stride]; }
};
struct DCol {
  double *p;
  int stride;
  __device__ double &operator[](int k) const { return p[k * stride]; }
};

// Contiguous per-warp arrays (warp-per-state kernel).
struct FArr {
  float *p;
  __device__ float &operator[](int k) const { return p[k]; }
};
struct DArr {
  double *p;
  __device__ double &operator[](int k) const { return p[k]; }
};

struct State {
  double T, invT, logT, P;
  float Tf;
  ff Tff, lTff, iTff;
};

// Arrhenius exponent of a rate row as float-float, and the sign of A.
__device__ __forceinline__ ff rate_exponent(const Tab &t, int row,
                                            const State &s, float &sign) {
  const float *c = t.rate_ff + 8 * row;
  ff x = ff_add(ff{c[0], c[1]}, ff_mul(ff{c[2], c[3]}, s.lTff));
  x = ff_add(x, ff_mul(ff{c[4], c[5]}, s.iTff));
  sign = c[6];
  return x;
}

// Exponent of the equilibrium constant of reversible reaction j (with
// ln of its prefactor), in FP64, from the per-species Gibbs column S:
// sum_k nu_k S_k.
template <class DC>
struct KcFromGibbs {
  DC S;
  __device__ __forceinline__ double operator()(const Tab &t, int r, int j) const {
    double g = t.kc_lpref[j];
    for (int e = t.nu_ptr[r]; e < t.nu_ptr[r + 1]; ++e) g = fma(t.nu_val[e], S[t.nu_sp[e]], g);
    return g;
  }
};

// a * b + c in float-float: the FP32 product with its FMA residuals, the
// head of c added exactly (TwoSum, by operations that are never contracted
// into an FMA) and every low-order term added once.  The result is left
// unnormalised (its low part may exceed half an ulp of the head), which a
// following ff_fma or ff_add takes as it is.  Error about 2^-44 of
// |a b| + |c|.
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff c) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  const float s = __fadd_rn(p, c.h);
  const float bb = __fsub_rn(s, p);
  const float err = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bb)), __fsub_rn(c.h, bb));
  return ff{s, __fadd_rn(err, __fadd_rn(e, c.l))};
}

// Exponent of the equilibrium constant of reversible reaction j (with ln
// of its prefactor) as float-float, entirely on the FP32 pipe, for the
// mixed one-state-per-thread kernel when every reaction has a single
// T_common group: the polynomial of KcPoly1 in the same Horner order,
//   c0 + c1 ln T + T (c2 + T (c3 + T (c4 + c5 T))) - c6 / T,
// with float-float coefficients (kc_mix) and float-float T, ln T and 1/T.
// Seven multiply-adds of ~2^-44 relative error: an absolute error of a few
// 1e-12 for exponents of a few hundred, against FP32 rates that notice
// 1e-7; the FP64 pipe, which retires 1/64 of the FP32 pipe's operations on
// GB300, does none of it.
struct KcMix {
  long long Tbits;  // T's bit pattern: T <= T_common as an integer test
  ff T, logT, invT;
};
__device__ __forceinline__ ff kc_exponent(const KcMix &kc, const Tab &t, int, int j) {
  const float4 *p = reinterpret_cast<const float4 *>(t.kc_mix + 32 * j);
  const float4 lo3 = p[3];  // -c6 of the low block and T_common
  const long long tc =
      (long long)(((unsigned long long)__float_as_uint(lo3.w) << 32) | __float_as_uint(lo3.z));
  const float4 *c = kc.Tbits <= tc ? p : p + 4;
  const float4 a = c[0], b = c[1], d = c[2], e = c[3];
  ff v = ff{d.z, d.w};                      // c5
  v = ff_fma(v, kc.T, ff{d.x, d.y});        // c4
  v = ff_fma(v, kc.T, ff{b.z, b.w});        // c3
  v = ff_fma(v, kc.T, ff{b.x, b.y});        // c2
  v = ff_fma(v, kc.T, ff{a.x, a.y});        // c0
  v = ff_fma(ff{a.z, a.w}, kc.logT, v);     // c1 ln T
  return ff_fma(ff{e.x, e.y}, kc.invT, v);  // -c6 / T
}
// Any other form (FP64 polynomials, Gibbs columns): its FP64 exponent,
// kept as a double until the exponential needs it (kc_ff), so that the
// FP64 chain overlaps the forward-rate work in between.
template <class KC>
__device__ __forceinline__ double kc_exponent(const KC &kc, const Tab &t, int r, int j) {
  return kc(t, r, j);
}
template <class KC>
struct KcOut {
  using type = double;
};
template <>
struct KcOut<KcMix> {
  using type = ff;
};
__device__ __forceinline__ ff kc_ff(ff g) { return g; }
__device__ __forceinline__ ff kc_ff(double g) { return ff_from_double_int(g); }

// product of concentration factors as mantissa * 2^E
// Product of concentration factors, times the mantissa m0 of the rate
// constant, as mantissa * 2^E; the FP32 rounding of every multiply is kept
// (FMA error terms) and added back once at the end.
template <class FC>
__device__ __forceinline__ float product(float m0, const int32_t *sp,
                                         const int32_t *nint, const double *nu,
                                         int a, int b, const FC &C, int &E) {
  float m = m0, err = 0.0f;
  for (int j = a; j < b; ++j) {
    const float c = C[sp[j]];
    int n = nint[j];
    int e;
    const float f = fsplit(n < 0 ? powf(c, (float)nu[j]) : c, e);
    if (n < 0) n = 1;
    for (; n > 0; --n) {
      const float mm = m * f;
      err = fmaf(err, f, fmaf(m, f, -mm));
      // keep the mantissa inside [2^-8, 2^8]: rescale by a power of two
      int e2;
      const float ms = fsplit(mm, e2);
      err = ldexpf(err, -e2);
      m = ms;
      E += e + e2;
    }
  }
  return m + err;
}

// pres_mod entry p in FP32.  The reduced pressure enters through
// ln Pr = (x_0 - x_inf) + ln [M], so that it never overflows.
template <class FC>
__device__ float pres_mod(const Tab &t, int p, const State &s, float mix,
                          const FC &C) {
  float thd = mix;
  const int sp = t.pm_sp[p];
  if (t.pm_kind[p] == PM_THD || sp < 0) {
    for (int e = t.pm_eff_ptr[p]; e < t.pm_eff_ptr[p + 1]; ++e)
      thd = fmaf(t.eff_f[e], C[t.pm_eff_sp[e]], thd);
    if (t.pm_kind[p] == PM_THD) return thd;
  } else {
    thd = C[sp];
  }
  float sg0, sgi;
  const ff x0 = rate_exponent(t, t.pm_k0[p], s, sg0);
  const ff xi = rate_exponent(t, t.pm_kinf[p], s, sgi);
  // Pr = exp(x_0 - x_inf) * [M] as mantissa * 2^E: no overflow, and the
  // float-float exponent difference keeps its precision
  int E;
  const float pe = ff_exp(ff_add(x0, ff_neg(xi)), E);
  int et;
  const float mt = fsplit(thd * sg0 * sgi, et);
  float m = pe * mt;
  E += et;
  int e2;
  m = fsplit(m, e2);
  E += e2;
  const bool low = t.pm_kind[p] == PM_FALL_LOW;
  float frac, inv1p;  // Pr/(1+Pr), 1/(1+Pr)
  if (m <= 0.0f) {
    frac = 0.0f;
    inv1p = 1.0f;
  } else if (E >= 0) {
    const float q = ldexpf(1.0f / m, -E);  // 1/Pr <= 1
    frac = 1.0f / (1.0f + q);
    inv1p = q * frac;
  } else {
    const float pr = ldexpf(m, E);  // Pr < 1
    inv1p = 1.0f / (1.0f + pr);
    frac = pr * inv1p;
  }
  const int form = t.pm_form[p];
  if (form == FORM_LINDEMANN) return low ? frac : inv1p;
  // Broadening in float-float where magnitudes demand it: log10 Pr reaches
  // +-300, so A, B and the exponent of F are formed as float-float pairs
  // (fp32 alone would leave F with ~1e-6 relative error).
  // ln Pr = E ln2 + ln m (m in [1, 2)), E ln2 split as an exact 12-bit head
  // times E plus a small tail.
  ff lnPr = ff{-1.0e30f, 0.0f};
  if (m > 0.0f) {
    const float Ef = (float)E;
    lnPr = ff_add(ff{Ef * LN2_H12_F, 0.0f}, ff{fmaf(Ef, LN2_L12_F, logf(m)), 0.0f});
  }
  // log10(fmax(Pr, 1e-300))
  ff lP = ff_mul(lnPr, ff{INV_LN10_F, INV_LN10_LO_F});
  if (lP.h < -300.0f) lP = ff{-300.0f, 0.0f};
  float F;
  if (form == FORM_TROE) {
    const float *c = t.troe_ff + 8 * p;  // P0, -1/T3 (ff), P2, -1/T1 (ff), -T2 (ff)
    float f = c[0] * ff_expf(ff_mul(s.Tff, ff{c[1], c[2]})) +
              c[3] * ff_expf(ff_mul(s.Tff, ff{c[4], c[5]}));
    if (t.pm_troe_t2[p]) f += ff_expf(ff_mul(s.iTff, ff{c[6], c[7]}));
    const float lnf = logf(fmaxf(f, 1.0e-37f));
    const ff lF = ff_mul(ff{lnf, 0.0f}, ff{INV_LN10_F, INV_LN10_LO_F});  // log10 Fcent
    // A = log10 Pr - 0.67 log10 Fcent - 0.4, B = 0.806 - 1.1762 log10 Fcent
    // - 0.14 log10 Pr (rate_subs.py:993-1003)
    const ff A = ff_add(ff_add(lP, ff_neg(ff_mul(ff{0.6700000166893005f, -1.668930060816365e-08f}, lF))),
                        ff{-0.4000000059604645f, 5.9604645663569045e-09f});
    const ff B = ff_add(ff_add(ff{0.8059999942779541f, 5.7220459481754915e-09f},
                               ff_neg(ff_mul(ff{1.176200032234192f, -3.2234190427971043e-08f}, lF))),
                        ff_neg(ff_mul(ff{0.14000000059604645f, -5.9604643443123e-10f}, lP)));
    // F = 10^(log10 Fcent / (1 + A^2/B^2)) = exp(ln Fcent * B^2 / (A^2 + B^2))
    const ff B2 = ff_mul(B, B);
    const ff w = ff_div(B2, ff_add(ff_mul(A, A), B2));
    F = ff_expf(ff_mul(ff{lnf, 0.0f}, w));
  } else {
    const float *c = t.sri_ff + 8 * p;  // a, -b (ff), -1/c (ff), d, e
    // X = 1 / (1 + log10^2 Pr); F = base^X
    const ff X = ff_div(ff{1.0f, 0.0f}, ff_add(ff{1.0f, 0.0f}, ff_mul(lP, lP)));
    const float base = c[0] * ff_expf(ff_mul(s.iTff, ff{c[1], c[2]})) +
                       ff_expf(ff_mul(s.Tff, ff{c[3], c[4]}));
    F = ff_expf(ff_mul(X, ff{logf(base), 0.0f}));
    if (t.pm_sri_de[p]) F *= c[5] * ff_expf(ff_mul(ff{c[6], 0.0f}, s.lTff));
  }
  return low ? F * frac : F * inv1p;
}

// The stoichiometric coefficient of a compact nu-list entry: its top 16
// bits, the rest zero (integer operations only).
__device__ __forceinline__ double nu_of(uint16_t top) {
  return __hiloint2double((int)((unsigned)top << 16), 0);
}

// wdot[k] += nu * net (FP64) for the reactions of one block, in order.
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
      k[q] = t.nu_sp16[e0 + q];
      w[q] = W[k[q]];
    }
#pragma unroll
    for (int q = 0; q < NNU; ++q)
      W[k[q]] = fma(nu_of(t.nu_hi[e0 + q]), net[u], w[q]);  // FP64
  }
}

// Sink of the on-chip kernels: net rates accumulate into the state's wdot
// column (FP64), block by block or one reaction at a time, in order.
template <class DC>
struct WSink {
  DC W;
  template <int NNU>
  __device__ __forceinline__ void block(const Tab &t, const int *rr, int cnt,
                                        const double (&net)[4]) const {
    accumulate<NNU>(t, rr, cnt, net, W);
  }
  __device__ __forceinline__ void one(const Tab &t, int r, double net) const {
    for (int e = t.nu_ptr[r]; e < t.nu_ptr[r + 1]; ++e) {
      const int k = t.nu_sp16[e];
      W[k] = fma(nu_of(t.nu_hi[e]), net, W[k]);  // FP64 accumulation
    }
  }
};

template <int NR, int NP, int NNU, int REV, bool STAGES, class KC, class SINK>
__device__ __forceinline__ void shape_block(const Tab &t, const int *rr,
                                            int cnt, const State &s,
                                            const FCol &C, const KC &kc,
                                            const SINK &sink, const Batch &b,
                                            int64_t i) {
  // Kc exponents first: independent of the rate work below, so the
  // scheduler can overlap them with it (the block is straight-line code)
  typename KcOut<KC>::type g[4];
  if (REV) {
#pragma unroll
    for (int u = 0; u < 4; ++u) g[u] = kc_exponent(kc, t, rr[u], t.rev_idx[rr[u]]);
  }
  ff x[4];
  double fwd[4], rev[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const int r = rr[u];
    float sg;
    x[u] = rate_exponent(t, r, s, sg);
    int E;
    float m = ff_exp(x[u], E), err = 0.0f;
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      int e;
      const float f = fsplit(C[t.rfac[MAXF * r + q]], e);
      const float mm = m * f;  // exact rounding error kept in err
      err = fmaf(err, f, fmaf(m, f, -mm));
      m = mm;
      E += e;
    }
    fwd[u] = assemble(m + err, E);
    rev[u] = 0.0;
  }
  if (REV) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int r = rr[u];
      int E;
      float m = ff_exp(ff_add(x[u], ff_neg(kc_ff(g[u]))), E), err = 0.0f;
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        int e;
        const float f = fsplit(C[t.pfac[MAXF * r + q]], e);
        const float mm = m * f;
        err = fmaf(err, f, fmaf(m, f, -mm));
        m = mm;
        E += e;
      }
      rev[u] = assemble(m + err, E);
    }
  }
  double net[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) net[u] = fwd[u] - rev[u];  // FP64
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

// The shape groups' blocks of four reactions, in order.  A caller that
// splits the blocks among NPART workers passes its part (0 <= part <
// NPART): it evaluates blocks part, part + NPART, ... of every group.
template <int SH, bool STAGES, class KC, class SINK>
struct Shapes {
  __device__ __forceinline__ static void run(const Tab &t, const State &s,
                                             const FCol &C, const KC &S,
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
    Shapes<SH + 1, STAGES, KC, SINK>::run(t, s, C, S, sink, b, i, part, npart);
  }
};
template <bool STAGES, class KC, class SINK>
struct Shapes<NSHAPE, STAGES, KC, SINK> {
  __device__ __forceinline__ static void run(const Tab &, const State &,
                                             const FCol &, const KC &,
                                             const SINK &, const Batch &,
                                             int64_t, int = 0, int = 1) {}
};

// Net rate (fwd - rev) * pres_mod of any reaction, as FP64.  PD: the
// reaction may be PLOG or Chebyshev (false: exponential form known).
template <bool PD = true, class FC, class KC>
__device__ __forceinline__ double rxn_net(const Tab &t, int r, const State &s,
                                          float mix, const FC &C, const KC &kc,
                                          double &fwd, double &rev, float &pm) {
  const int j = t.rev_idx[r];
  // the Kc exponent first, to overlap with the forward rate
  const typename KcOut<KC>::type g = j >= 0 ? kc_exponent(kc, t, r, j) : typename KcOut<KC>::type{};
  float sgn;
  ff xf;
  if (PD && t.rate_kind[r] >= RATE_PLOG) {
    // PLOG / Chebyshev: kf in FP64 in the emitted form, then its log
    const double kf = pdep_kf(t, r, s.T, s.logT, s.P);
    sgn = kf < 0.0 ? -1.0f : 1.0f;
    xf = ff_from_double(log(fabs(kf)));
  } else {
    xf = rate_exponent(t, r, s, sgn);
  }
  int Ef;
  const float pf = ff_exp(xf, Ef);
  const float mf = sgn * product(pf, t.rx_sp, t.rx_nint, t.rx_nu, t.rx_ptr[r],
                                 t.rx_ptr[r + 1], C, Ef);
  fwd = assemble(mf, Ef);
  double net = fwd;
  rev = 0.0;
  if (j >= 0) {
    int Er;
    const float pr = ff_exp(ff_add(xf, ff_neg(kc_ff(g))), Er);
    const float mr = sgn * product(pr, t.px_sp, t.px_nint, t.px_nu, t.px_ptr[r],
                                   t.px_ptr[r + 1], C, Er);
    rev = assemble(mr, Er);
    net = fwd - rev;  // FP64
  }
  const int p = t.pm_idx[r];
  pm = 1.0f;
  if (p >= 0) {
    pm = pres_mod(t, p, s, mix, C);
    net *= f2d_exact(pm);
  }
  return net;
}

template <bool STAGES, bool PD, class KC, class SINK>
__device__ __forceinline__ void general(const Tab &t, int r, const State &s,
                                        float mix, const FCol &C,
                                        const KC &S, const SINK &sink,
                                        const Batch &b, int64_t i) {
  double fwd, rev;
  float pm;
  const double net = rxn_net<PD>(t, r, s, mix, C, S, fwd, rev, pm);
  if (STAGES) {
    const int j = t.rev_idx[r], p = t.pm_idx[r];
    if (b.fwd) b.fwd[(int64_t)r * b.ld + i] = fwd;
    if (b.rev && j >= 0) b.rev[(int64_t)j * b.ld + i] = rev;
    if (b.pm && p >= 0) b.pm[(int64_t)p * b.ld + i] = (double)pm;
  }
  sink.one(t, r, net);
}

}  // namespace mixed
}  // namespace crs
