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

// The arithmetic itself is include/crs_eval.h (shared with the per-state
// host and device functions); this file adds the batched layouts.
using ref::accumulate;
using ref::pres_mod;
using ref::rxn_rates;

// A per-thread column: element k at p[k * stride].
using Col = ref::Strided<double>;

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
  CRS_HD double operator[](int k) const {
    if (stored) return col[k];
    double y = (k == N - 1) ? y_N : Y[(int64_t)k * ld + i];
    return rho * y * inv_mw[k];
  }
};

// eval_conc for state i of an SoA batch (rate_subs.py:1295-1391): returns
// rho; y_N / mw_avg through refs.
__device__ double eval_conc(const Tab &t, double T, double P, const double *Y,
                            int64_t ld, int64_t i, double &y_N, double &mw_avg) {
  return ref::eval_conc(t, T, P, ref::Strided<const double>{Y + i, ld}, y_N, mw_avg);
}

// Tables in global memory: four CTAs per SM at 128 registers ran 10%
// faster than three at the 168 registers the compiler may pick by itself.
// Staged tables: one CTA per SM (shared memory).
template <bool SMEM_TAB, bool SMEM_COL>
__global__ void __launch_bounds__(128, SMEM_TAB ? 1 : 4)
    k_wdot(const unsigned char *__restrict__ img, ImgLayout L, Batch b) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  const unsigned char *tb = img;
  if (SMEM_TAB) {
    // the image up to the mixed kernels' trailing section (kc_mix)
    if (!stage_to_smem(smem, img, L.kc_mix, &bar, b.status)) return;
    tb = smem;
  }
  const Tab t = make_tab(tb, L);
  const int N = t.N;
  double *colbase =
      reinterpret_cast<double *>(smem + (SMEM_TAB ? L.kc_mix : 0));
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
  const size_t tab = (size_t)L.kc_mix;  // staged: every section before kc_mix
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
