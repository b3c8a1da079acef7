// Thermodynamic utilities and the ODE right-hand side around wdot.
//
// The reference emits, per mechanism, eval_h / eval_u / eval_cv / eval_cp
// and eval_conc_rho (rate_subs.py:1396-1776) and a dydt that combines them
// with the rate functions (rate_subs.py:1829-2067): for y = [T, Y_0 ..
// Y_{N-2}],
//   constant pressure:  dT/dt = -(sum_k wdot_k h_k mw_k) / (rho cp_avg)
//   constant volume:    dT/dt = -(sum_k wdot_k u_k mw_k) / (rho cv_avg)
//   dY_k/dt = wdot_k mw_k / rho,
// cp_avg / cv_avg = sum_k c_k Y_k (the bath gas Y_N = 1 - sum).  Here the
// same arithmetic, in the emitted operand order and FP64, runs one state per
// thread over SoA batches; wdot itself comes from the wdot kernels (any
// precision mode), so dydt = the wdot launch + one pass of this file.  The
// per-species coefficients sit in the sp_thermo table (RU/mw, mw, T_common,
// NASA-7 a_j and a_j / (j+1)) and are read through L1: every thread of a warp
// reads the same entry.
#include <cuda_runtime.h>

#include "crs_internal.cuh"

namespace crs {
namespace thermo {

using ref::RU_PRINTED;  // RU as eval_conc prints it (%.8e)

// h (which 0), u (1), cv (2), cp (3) of species k at T (include/crs_eval.h)
__device__ __forceinline__ double value(const double *c, int which, double T) {
  return ref::thermo_value(c, which, T);
}

__global__ void k_thermo(const unsigned char *__restrict__ img, ImgLayout L, int which,
                         int64_t n, const double *__restrict__ T, int64_t ld,
                         double *__restrict__ out) {
  const Tab t = make_tab(img, L);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double Ti = T[i];
    for (int k = 0; k < t.N; ++k) out[(int64_t)k * ld + i] = value(t.sp_thermo + 24 * k, which, Ti);
  }
}

// y_N = 1 - sum Y (left to right), 1 / mw_avg = sum Y_k / mw_k
__device__ __forceinline__ double mix(const Tab &t, const double *Y, int64_t ld, int64_t i,
                                      double &y_N) {
  const int N = t.N;
  double s = N > 1 ? Y[i] : 0.0;
  for (int k = 1; k < N - 1; ++k) s = s + Y[(int64_t)k * ld + i];
  y_N = N > 1 ? 1.0 - s : 1.0;
  double mw = 0.0;
  for (int k = 0; k < N - 1; ++k) {
    const double v = Y[(int64_t)k * ld + i] * t.inv_mw[k];
    mw = k == 0 ? v : mw + v;
  }
  return N > 1 ? mw + y_N * t.inv_mw[N - 1] : y_N * t.inv_mw[N - 1];
}

__global__ void k_conc_rho(const unsigned char *__restrict__ img, ImgLayout L, int64_t n,
                           const double *__restrict__ T, const double *__restrict__ rho,
                           const double *__restrict__ Y, int64_t ld, double *y_N_o,
                           double *mw_o, double *pres_o, double *conc) {
  const Tab t = make_tab(img, L);
  const int N = t.N;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double y_N;
    const double mw_avg = 1.0 / mix(t, Y, ld, i, y_N);
    const double r = rho[i];
    if (y_N_o) y_N_o[i] = y_N;
    if (mw_o) mw_o[i] = mw_avg;
    if (pres_o) pres_o[i] = r * RU_PRINTED * T[i] / mw_avg;
    if (conc) {
      for (int k = 0; k < N - 1; ++k)
        conc[(int64_t)k * ld + i] = r * Y[(int64_t)k * ld + i] * t.inv_mw[k];
      conc[(int64_t)(N - 1) * ld + i] = r * y_N * t.inv_mw[N - 1];
    }
  }
}

template <bool CONV>
__global__ void k_dydt_finish(const unsigned char *__restrict__ img, ImgLayout L, int64_t n,
                              const double *__restrict__ y, int64_t ld,
                              const double *__restrict__ p_or_rho,
                              const double *__restrict__ W, double *__restrict__ dy) {
  const Tab t = make_tab(img, L);
  const int N = t.N;
  const double *Y = y + ld;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double T = y[i];
    double y_N;
    const double m = mix(t, Y, ld, i, y_N);
    // constant pressure: rho as eval_conc forms it; constant volume: given
    const double rho = CONV ? p_or_rho[i] : p_or_rho[i] * (1.0 / m) / (RU_PRINTED * T);
    double avg = 0.0, sum = 0.0;
    for (int k = 0; k < N; ++k) {
      const double *c = t.sp_thermo + 24 * k;
      const double yk = k < N - 1 ? Y[(int64_t)k * ld + i] : y_N;
      const double ck = value(c, CONV ? 2 : 3, T);
      const double ek = value(c, CONV ? 1 : 0, T);
      const double w = W[(int64_t)k * ld + i];
      avg = k == 0 ? ck * yk : avg + ck * yk;
      sum = k == 0 ? w * ek * c[1] : sum + w * ek * c[1];
      if (k < N - 1) dy[(int64_t)(k + 1) * ld + i] = w * (c[1] / rho);
    }
    dy[i] = (-1.0 / (rho * avg)) * sum;
  }
}

inline int grid(int64_t n, int sm_count) {
  int64_t g = (n + 255) / 256;
  const int64_t cap = (int64_t)sm_count * 8;
  if (g > cap) g = cap;
  return (int)(g < 1 ? 1 : g);
}

}  // namespace thermo

cudaError_t launch_thermo(const unsigned char *img, const ImgLayout &L, int which, int64_t n,
                          const double *T, int64_t ld, double *out, int sm_count,
                          cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  thermo::k_thermo<<<thermo::grid(n, sm_count), 256, 0, s>>>(img, L, which, n, T, ld, out);
  return cudaGetLastError();
}

cudaError_t launch_conc_rho(const unsigned char *img, const ImgLayout &L, int64_t n,
                            const double *T, const double *rho, const double *Y, int64_t ld,
                            double *y_N, double *mw_avg, double *pres, double *conc,
                            int sm_count, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  thermo::k_conc_rho<<<thermo::grid(n, sm_count), 256, 0, s>>>(img, L, n, T, rho, Y, ld, y_N,
                                                               mw_avg, pres, conc);
  return cudaGetLastError();
}

cudaError_t launch_dydt_finish(const unsigned char *img, const ImgLayout &L, int conv,
                               int64_t n, const double *y, int64_t ld, const double *p_or_rho,
                               const double *W, double *dy, int sm_count, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  if (conv)
    thermo::k_dydt_finish<true><<<thermo::grid(n, sm_count), 256, 0, s>>>(img, L, n, y, ld,
                                                                          p_or_rho, W, dy);
  else
    thermo::k_dydt_finish<false><<<thermo::grid(n, sm_count), 256, 0, s>>>(img, L, n, y, ld,
                                                                           p_or_rho, W, dy);
  return cudaGetLastError();
}

}  // namespace crs
