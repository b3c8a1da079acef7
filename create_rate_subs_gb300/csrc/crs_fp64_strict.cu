// FP64 evaluation in the reference's operation order (CRS_MODE_FP64_STRICT)
// and the batched per-stage kernels.
//
// This translation unit is compiled with -fmad=false: every expression is
// evaluated as the reference's emitted C writes it (rate_subs.py), one
// rounding per operation, so the only differences to the emitted C compiled
// on a CPU are the last-bit differences of exp/log/log10/pow between CUDA's
// math library and the host libm.
//
// Layout: one thread per state (grid-stride loop); the CTA stages the
// mechanism tables into shared memory with cp.async.bulk; each thread keeps
// its concentrations and wdot accumulators in its own shared-memory column
// (entry k at [k*blockDim + tid]).  When a mechanism is too large for that,
// tables stay in global memory, concentrations are recomputed from Y and
// wdot accumulates in place in the output.
#include <cstdint>
#include <cuda_runtime.h>
#include <math.h>

#include "crs_internal.cuh"

namespace crs {
namespace strict {

// A per-thread column: element k at p[k * stride].
struct Col {
  double *p;
  int64_t stride;
  __device__ double &operator[](int k) const { return p[(int64_t)k * stride]; }
};

// Concentrations either stored in a column, or recomputed from Y exactly as
// eval_conc computes them (rate_subs.py:1386-1390): (rho * y_k) * (1/mw_k).
struct ConcSrc {
  Col col;
  bool stored;
  const double *Y;
  int64_t ld, i;
  double rho, y_N;
  const double *inv_mw;
  int N;
  __device__ double operator[](int k) const {
    if (stored) return col[k];
    double y = (k == N - 1) ? y_N : Y[(int64_t)k * ld + i];
    return rho * y * inv_mw[k];
  }
};

// rxn_rate_const, standalone (rate_subs.py:60-135).
__device__ double rate_const(const Tab &t, int row, double T, double logT) {
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

template <class CS>
__device__ double conc_product(const int32_t *sp, const int32_t *nint,
                               const double *nu, int a, int b, const CS &C,
                               bool &have) {
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

// Kc exponent over the T_common groups (rate_subs.py:592-655).
__device__ double kc_exponent(const Tab &t, int j, double T, double logT) {
  double kc = 0.0;
  const int g0 = t.kc_ptr[j], g1 = t.kc_ptr[j + 1];
  for (int g = g0; g < g1; ++g) {
    const double *c = (T <= t.kc_tmid[g]) ? t.kc_lo + 7 * g : t.kc_hi + 7 * g;
    const double v =
        (c[0] + c[1] * logT + T * (c[2] + T * (c[3] + T * (c[4] + c[5] * T))) -
         c[6] / T);
    kc = (g == g0) ? v : kc + v;
  }
  return kc;
}

// fwd (and rev when reversible) of reaction r (rate_subs.py:433-693).
// PLOG / Chebyshev rows print kf first and use it like a reversible
// reaction's kf (rate_subs.py:437-448, 503-505).
template <class CS>
__device__ void rxn_rates(const Tab &t, int r, double T, double logT, double pres,
                          const CS &C, double &fwd, double &rev) {
  bool have;
  const double p = conc_product(t.rx_sp, t.rx_nint, t.rx_nu, t.rx_ptr[r],
                                t.rx_ptr[r + 1], C, have);
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
    const double q = conc_product(t.px_sp, t.px_nint, t.px_nu, t.px_ptr[r],
                                  t.px_ptr[r + 1], C, hq);
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

template <class CS>
__device__ double third_body(const Tab &t, int p, double mix, const CS &C) {
  double v = mix;
  for (int e = t.pm_eff_ptr[p]; e < t.pm_eff_ptr[p + 1]; ++e)
    v = v + t.pm_eff_val[e] * C[t.pm_eff_sp[e]];
  return v;
}

// pres_mod entry p (rate_subs.py:881-1064).
template <class CS>
__device__ double pres_mod(const Tab &t, int p, double T, double logT,
                           double mix, const CS &C) {
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
    const double X =
        1.0 / (1.0 + log10(fmax(Pr, 1.0e-300)) * log10(fmax(Pr, 1.0e-300)));
    double F = pow(c[0] * exp(-c[1] / T) + exp(-T / c[2]), X);
    if (t.pm_sri_de[p]) F = F * c[3] * pow(T, c[4]);
    return low ? F * Pr / (1.0 + Pr) : F / (1.0 + Pr);
  }
  return low ? Pr / (1.0 + Pr) : 1.0 / (1.0 + Pr);
}

// Net term of reaction r for species entry e, accumulated into W
// (rate_subs.py:1183-1216): sign * ((|nu| * (fwd - rev)) * pres_mod).
__device__ __forceinline__ void accumulate(const Tab &t, int e, double net,
                                           double pm, bool has_pm,
                                           const Col &W) {
  const int k = t.nu_sp[e];
  const double nu = t.nu_val[e];
  const double a = fabs(nu);
  double v = net;
  if (a != 1.0) v = a * v;
  if (has_pm) v = v * pm;
  W[k] = (nu < 0.0) ? W[k] - v : W[k] + v;
}

// eval_conc for one state (rate_subs.py:1295-1391).  Writes y into C first
// when C is a stored column.  Returns rho; y_N / mw_avg through refs.
__device__ double eval_conc(const Tab &t, double T, double P, const double *Y,
                            int64_t ld, int64_t i, double &y_N,
                            double &mw_avg) {
  const int N = t.N;
  double s = (N > 1) ? Y[i] : 0.0;
  for (int k = 1; k < N - 1; ++k) s = s + Y[(int64_t)k * ld + i];
  y_N = 1.0 - s;
  double mw = 0.0;
  for (int k = 0; k < N - 1; ++k) {
    const double v = Y[(int64_t)k * ld + i] * t.inv_mw[k];
    mw = (k == 0) ? v : mw + v;
  }
  mw = (N > 1) ? mw + y_N * t.inv_mw[N - 1] : y_N * t.inv_mw[N - 1];
  mw_avg = 1.0 / mw;
  return P * mw_avg / (8.31446210e+03 * T);
}

template <bool SMEM_TAB, bool SMEM_COL>
__global__ void __launch_bounds__(128)
    k_wdot(const unsigned char *__restrict__ img, ImgLayout L, Batch b) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  const unsigned char *tb = img;
  if (SMEM_TAB) {
    if (!stage_to_smem(smem, img, L.bytes, &bar, b.status)) return;
    tb = smem;
  }
  const Tab t = make_tab(tb, L);
  const int N = t.N;
  double *colbase =
      reinterpret_cast<double *>(smem + (SMEM_TAB ? L.bytes : 0));
  const int64_t stride = blockDim.x;
  Col Cc{colbase + threadIdx.x, stride};
  Col Wc{colbase + (int64_t)N * stride + threadIdx.x, stride};
  int bad = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double T = b.T[i], P = b.P[i];
    double y_N, mw_avg;
    const double rho = eval_conc(t, T, P, b.Y, b.ld, i, y_N, mw_avg);
    ConcSrc C{Cc, SMEM_COL, b.Y, b.ld, i, rho, y_N, t.inv_mw, N};
    Col W = SMEM_COL ? Wc : Col{b.wdot + i, b.ld};
    if (SMEM_COL) {
      for (int k = 0; k < N - 1; ++k)
        Cc[k] = rho * b.Y[(int64_t)k * b.ld + i] * t.inv_mw[k];
      Cc[N - 1] = rho * y_N * t.inv_mw[N - 1];
    }
    for (int k = 0; k < N; ++k) W[k] = 0.0;
    if (b.conc)
      for (int k = 0; k < N; ++k) b.conc[(int64_t)k * b.ld + i] = C[k];
    const double logT = log(T);
    const double mix = P / (8.31446210e+03 * T);
    for (int r = 0; r < t.R; ++r) {
      double fwd, rev;
      rxn_rates(t, r, T, logT, P, C, fwd, rev);
      const int j = t.rev_idx[r];
      const int p = t.pm_idx[r];
      double pm = 0.0;
      if (p >= 0) pm = pres_mod(t, p, T, logT, mix, C);
      if (b.fwd) b.fwd[(int64_t)r * b.ld + i] = fwd;
      if (b.rev && j >= 0) b.rev[(int64_t)j * b.ld + i] = rev;
      if (b.pm && p >= 0) b.pm[(int64_t)p * b.ld + i] = pm;
      const double net = (j >= 0) ? fwd - rev : fwd;
      for (int e = t.nu_ptr[r]; e < t.nu_ptr[r + 1]; ++e)
        accumulate(t, e, net, pm, p >= 0, W);
    }
    for (int k = 0; k < N; ++k) {
      const double v = W[k];
      if (!isfinite(v)) ++bad;
      if (SMEM_COL) b.wdot[(int64_t)k * b.ld + i] = v;
    }
  }
  if (bad && b.status) atomicAdd(&b.status[1], bad);
}

// ---- per-stage kernels (tables read from global memory) ----------------

__global__ void k_conc(const unsigned char *__restrict__ img, ImgLayout L,
                       Batch b, double *y_N_o, double *mw_o, double *rho_o) {
  const Tab t = make_tab(img, L);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double T = b.T[i], P = b.P[i];
    double y_N, mw_avg;
    const double rho = eval_conc(t, T, P, b.Y, b.ld, i, y_N, mw_avg);
    for (int k = 0; k < t.N - 1; ++k)
      b.conc[(int64_t)k * b.ld + i] = rho * b.Y[(int64_t)k * b.ld + i] * t.inv_mw[k];
    b.conc[(int64_t)(t.N - 1) * b.ld + i] = rho * y_N * t.inv_mw[t.N - 1];
    if (y_N_o) y_N_o[i] = y_N;
    if (mw_o) mw_o[i] = mw_avg;
    if (rho_o) rho_o[i] = rho;
  }
}

// b.conc holds C (input).
__global__ void k_rxn_rates(const unsigned char *__restrict__ img, ImgLayout L,
                            Batch b) {
  const Tab t = make_tab(img, L);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double T = b.T[i], P = b.P[i];
    Col C{b.conc + i, b.ld};
    const double logT = log(T);
    for (int r = 0; r < t.R; ++r) {
      double fwd, rev;
      rxn_rates(t, r, T, logT, P, C, fwd, rev);
      b.fwd[(int64_t)r * b.ld + i] = fwd;
      const int j = t.rev_idx[r];
      if (j >= 0 && b.rev) b.rev[(int64_t)j * b.ld + i] = rev;
    }
  }
}

__global__ void k_pres_mod(const unsigned char *__restrict__ img, ImgLayout L,
                           Batch b) {
  const Tab t = make_tab(img, L);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double T = b.T[i], P = b.P[i];
    Col C{b.conc + i, b.ld};
    const double logT = log(T);
    const double mix = P / (8.31446210e+03 * T);
    for (int p = 0; p < t.NPM; ++p)
      b.pm[(int64_t)p * b.ld + i] = pres_mod(t, p, T, logT, mix, C);
  }
}

// b.fwd / b.rev / b.pm are inputs; wdot accumulates in place.
__global__ void k_spec_rates(const unsigned char *__restrict__ img,
                             ImgLayout L, Batch b) {
  const Tab t = make_tab(img, L);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    Col W{b.wdot + i, b.ld};
    for (int k = 0; k < t.N; ++k) W[k] = 0.0;
    for (int r = 0; r < t.R; ++r) {
      const int j = t.rev_idx[r], p = t.pm_idx[r];
      const double f = b.fwd[(int64_t)r * b.ld + i];
      const double net = (j >= 0) ? f - b.rev[(int64_t)j * b.ld + i] : f;
      const double pm = (p >= 0) ? b.pm[(int64_t)p * b.ld + i] : 0.0;
      for (int e = t.nu_ptr[r]; e < t.nu_ptr[r + 1]; ++e)
        accumulate(t, e, net, pm, p >= 0, W);
    }
  }
}

}  // namespace strict

// ---- launchers ----------------------------------------------------------

int grid_for(int64_t n, int block, int max_ctas) {
  int64_t g = (n + block - 1) / block;
  if (g > max_ctas) g = max_ctas;
  if (g < 1) g = 1;
  return (int)g;
}

cudaError_t launch_wdot_strict(const unsigned char *img, const ImgLayout &L,
                               const Batch &b, int sm_count, int smem_optin,
                               cudaStream_t s) {
  const int block = 128;
  const size_t tab = (size_t)L.bytes;
  const size_t cols = (size_t)2 * L.N * block * sizeof(double);
  const int ctas_per_sm = 1;
  const int grid = grid_for(b.n, block, sm_count * ctas_per_sm);
  if (tab + cols <= (size_t)smem_optin) {
    auto k = strict::k_wdot<true, true>;
    const cudaError_t e = set_smem_limit(k, tab + cols);
    if (e != cudaSuccess) return e;
    k<<<grid, block, tab + cols, s>>>(img, L, b);
  } else if (tab <= (size_t)smem_optin) {
    auto k = strict::k_wdot<true, false>;
    const cudaError_t e = set_smem_limit(k, tab);
    if (e != cudaSuccess) return e;
    k<<<sm_count * 4 < grid ? sm_count * 4 : grid, block, tab, s>>>(img, L, b);
  } else {
    auto k = strict::k_wdot<false, false>;
    k<<<grid_for(b.n, block, sm_count * 8), block, 0, s>>>(img, L, b);
  }
  return cudaGetLastError();
}

cudaError_t launch_stage(int which, const unsigned char *img,
                         const ImgLayout &L, const Batch &b, double *y_N,
                         double *mw, double *rho, int sm_count,
                         cudaStream_t s) {
  const int block = 128;
  const int grid = grid_for(b.n, block, sm_count * 16);
  switch (which) {
    case 0: strict::k_conc<<<grid, block, 0, s>>>(img, L, b, y_N, mw, rho); break;
    case 1: strict::k_rxn_rates<<<grid, block, 0, s>>>(img, L, b); break;
    case 2: strict::k_pres_mod<<<grid, block, 0, s>>>(img, L, b); break;
    default: strict::k_spec_rates<<<grid, block, 0, s>>>(img, L, b); break;
  }
  return cudaGetLastError();
}

}  // namespace crs
