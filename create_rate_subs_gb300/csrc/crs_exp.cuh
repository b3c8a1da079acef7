// Table-driven FP64 exponential of the CRS_MODE_FP64 kernels (Tang, ACM
// TOMS 15(2), 1989): x = (256 k + j) ln2/256 + r, exp(x) = 2^k 2^(j/256)
// p(r) with |r| <= ln2/512 and p the degree-4 Taylor polynomial; error below
// 1 ulp plus the table rounding.  exp_core costs 9 FP64 instructions (two
// FMA reductions, the shifted-integer rounding and its subtraction, three
// FMAs and one multiply for p, the final FMA); the table index, the 2^k
// scaling and the range test are integer work.  The in-run probe times this
// same function to price an exponential in the FP64 roofline.
#pragma once

#include <cuda_runtime.h>

namespace crs {
namespace texp {

constexpr double INV_L = 369.3299304675746;     // 256 / ln 2
constexpr double L_HI = 0x1.62e42fefa0000p-9;   // ln2/256, 35 bits
constexpr double L_LO = 0x1.cf79abc9e3b3ap-48;  // ln2/256 - L_HI
constexpr double SHIFT = 6755399441055744.0;    // 1.5 * 2^52
// FP64 instructions of exp_core (the count above)
constexpr int EXP_CORE_FP64_OPS = 9;

// exp(x) from the 2^(j/256) table `tab`, without the range check:
// arguments beyond +-700 and NaN give garbage here and are replaced by
// exp_fix.  The table index stays in [0, 255] for any input.
__device__ __forceinline__ double exp_core(double x, const double *tab) {
  const double t = fma(x, INV_L, SHIFT);
  const double kd = t - SHIFT;
  const int k = __double2loint(t);
  double r = fma(kd, -L_HI, x);
  r = fma(kd, -L_LO, r);
  const double q = fma(fma(r, 1.0 / 24.0, 1.0 / 6.0), r, 0.5);
  const double p = fma(q, r * r, r);
  const double tj = tab[k & 255];
  const int m = k >> 8;  // arithmetic shift: floor(k / 256)
  const double s = __hiloint2double(__double2hiint(tj) + m * (1 << 20),
                                    __double2loint(tj));
  return fma(s, p, s);
}
// Overflow, underflow and NaN go to CUDA's exp.  |x| <= 700 is tested on
// the high word as an integer (0x4085E000 = high word of 700.0; a larger
// low word still leaves x below 700.0001): no FP64 instruction.
__device__ __forceinline__ double exp_fix(double x, double e) {
  return ((unsigned)__double2hiint(x) & 0x7fffffffu) <= 0x4085E000u ? e : exp(x);
}
__device__ __forceinline__ double exp_t(double x, const double *tab) {
  return exp_fix(x, exp_core(x, tab));
}

// Table-driven FP64 natural logarithm of the CRS_MODE_FP64 kernels (Tang,
// ACM TOMS 16(4), 1990): x = 2^e m with m in [1, 2), F = 1 + j/128 the
// grid point nearest m (|m - F| <= 1/256, exact difference), and
//   log x = e ln2 + log F + log1p(u),  u = (m - F) / F,  |u| < 2^-8,
// log1p by its degree-6 Taylor polynomial (truncation below 2^-58).  The
// table holds 1/F and log F for j = 0..128 (tab[2j], tab[2j+1]); e ln2 is
// split so that e times its head is exact.  Error about 1 ulp; 12 FP64
// instructions against roughly 30 for CUDA's log.  Zero, negative,
// subnormal, infinite and NaN arguments go to CUDA's log.
constexpr double LN2_HI = 0x1.62e42fefa3800p-1;  // ln 2 to 42 bits
constexpr double LN2_LO = 0x1.ef35793c76730p-45; // ln 2 - LN2_HI
constexpr int LOG_TAB_ENTRIES = 129;

__device__ __forceinline__ double log_t(double x, const double *tab) {
  const int hi = __double2hiint(x);
  // positive normal finite x: high word in [0x00100000, 0x7fefffff]
  if ((unsigned)(hi - 0x00100000) >= 0x7fe00000u) return log(x);
  const int mh = hi & 0x000fffff;
  const int j = (mh + (1 << 12)) >> 13;  // 0..128: the nearest 1/128 step
  const double m = __hiloint2double(mh | 0x3ff00000, __double2loint(x));
  const double F = __hiloint2double(0x3ff00000 + (j << 13), 0);
  const double2 c = *reinterpret_cast<const double2 *>(tab + 2 * j);
  const double u = (m - F) * c.x;
  double q = fma(fma(fma(fma(u, -1.0 / 6.0, 0.2), u, -0.25), u, 1.0 / 3.0), u, -0.5);
  q = fma(q, u * u, u);
  const double ed = (double)((hi >> 20) - 1023);
  return fma(ed, LN2_HI, c.y) + fma(ed, LN2_LO, q);
}

}  // namespace texp
}  // namespace crs
