// Surrogate network kernels: a BF16 MLP trained and evaluated on the
// tensor cores.
//
// Layers are Y = act(X W^T + b) computed by the tcgen05 GEMM of
// crs_gemm.cuh with fused epilogues:
//   forward          z = acc + b; a = silu(z); store z (fp32, for the
//                    backward pass), a row-major (bf16, the next layer's X)
//                    and a transposed (bf16, the operand of the weight
//                    gradient), or the fp32 output of the last layer;
//   backward, data   dz_prev = (dz W) * silu'(z_prev), stored row-major and
//                    transposed (bf16);
//   backward, weight dW = dz^T a_prev, split over K (the batch) into fp32
//                    partial sums reduced in a fixed order.
// Element-wise kernels: input features and the training-set box check,
// loss and its gradient, bias gradients, Adam (fp32 master weights, bf16
// copies W and W^T), and the surrogate's output transform with the
// element-conservation check that routes states back to the exact kernel.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

#include "../../include/crs.h"
#include "crs_gemm.cuh"
#include "crs_internal.cuh"

namespace crs {
namespace mlp {

__device__ __forceinline__ float sigmoidf(float z) { return __fdividef(1.0f, 1.0f + __expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigmoidf(z); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = sigmoidf(z);
  return s * (1.0f + z * (1.0f - s));
}

// Stores of one thread's 32 consecutive values of a row: four or eight
// 16-byte stores when all 32 are wanted and the address allows it (rows of
// a warp are a row stride apart, so per-element stores would cost a memory
// sector each), element by element otherwise.
__device__ __forceinline__ void store32(float *dst, const float (&x)[32], int nvalid) {
  if (nvalid >= 32 && !(reinterpret_cast<uintptr_t>(dst) & 15)) {
    float4 *d = reinterpret_cast<float4 *>(dst);
#pragma unroll
    for (int q = 0; q < 8; ++q) d[q] = make_float4(x[4 * q], x[4 * q + 1], x[4 * q + 2], x[4 * q + 3]);
  } else {
#pragma unroll
    for (int j = 0; j < 32; ++j)
      if (j < nvalid) dst[j] = x[j];
  }
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&h);
}

__device__ __forceinline__ void store32(__nv_bfloat16 *dst, const float (&x)[32], int nvalid) {
  if (nvalid >= 32 && !(reinterpret_cast<uintptr_t>(dst) & 15)) {
    uint4 *d = reinterpret_cast<uint4 *>(dst);
#pragma unroll
    for (int q = 0; q < 4; ++q)
      d[q] = make_uint4(pack_bf16(x[8 * q], x[8 * q + 1]), pack_bf16(x[8 * q + 2], x[8 * q + 3]),
                        pack_bf16(x[8 * q + 4], x[8 * q + 5]),
                        pack_bf16(x[8 * q + 6], x[8 * q + 7]));
  } else {
#pragma unroll
    for (int j = 0; j < 32; ++j)
      if (j < nvalid) dst[j] = __float2bfloat16_rn(x[j]);
  }
}

struct EpiForward {
  const float *bias;  // [N] or nullptr
  int act;
  int m_valid, n_valid;
  float *Z;
  int64_t ldz;
  __nv_bfloat16 *A;
  int64_t lda;
  __nv_bfloat16 *AT;
  int64_t ldat;
  float *Y;
  int64_t ldy;
  __device__ void operator()(int row, int col0, const uint32_t (&v)[32]) const {
    if (row >= m_valid || col0 >= n_valid) return;
    const int nv = n_valid - col0;
    float z[32], a[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      z[j] = __uint_as_float(v[j]) + ((bias && j < nv) ? bias[col0 + j] : 0.0f);
      a[j] = act == CRS_ACT_SILU ? silu(z[j]) : z[j];
    }
    if (Z) store32(Z + (int64_t)row * ldz + col0, z, nv);
    if (A) store32(A + (int64_t)row * lda + col0, a, nv);
    if (Y) store32(Y + (int64_t)row * ldy + col0, a, nv);
    if (AT) {
      // consecutive lanes hold consecutive rows: these stores coalesce
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (j < nv) AT[(int64_t)(col0 + j) * ldat + row] = __float2bfloat16_rn(a[j]);
    }
  }
};

struct EpiBackwardData {
  const float *Zprev;
  int64_t ldz;
  int m_valid, n_valid;
  __nv_bfloat16 *dZ;
  int64_t ld;
  __nv_bfloat16 *dZT;
  int64_t ldt;
  __device__ void operator()(int row, int col0, const uint32_t (&v)[32]) const {
    if (row >= m_valid || col0 >= n_valid) return;
    const int nv = n_valid - col0;
    const float *zp = Zprev + (int64_t)row * ldz + col0;
    float zv[32], d[32];
    if (nv >= 32 && !(reinterpret_cast<uintptr_t>(zp) & 15)) {
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float4 t = reinterpret_cast<const float4 *>(zp)[q];
        zv[4 * q] = t.x;
        zv[4 * q + 1] = t.y;
        zv[4 * q + 2] = t.z;
        zv[4 * q + 3] = t.w;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 32; ++j) zv[j] = j < nv ? zp[j] : 0.0f;
    }
#pragma unroll
    for (int j = 0; j < 32; ++j) d[j] = __uint_as_float(v[j]) * dsilu(zv[j]);
    store32(dZ + (int64_t)row * ld + col0, d, nv);
    if (dZT) {
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (j < nv) dZT[(int64_t)(col0 + j) * ldt + row] = __float2bfloat16_rn(d[j]);
    }
  }
};

// split-K partial: P[z][row][col]
struct EpiPartial {
  float *P;
  int64_t rows_pad, cols_pad;
  __device__ void operator()(int row, int col0, const uint32_t (&v)[32]) const {
    float x[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) x[j] = __uint_as_float(v[j]);
    store32(P + ((int64_t)blockIdx.z * rows_pad + row) * cols_pad + col0, x, 32);
  }
};

__global__ void k_reduce_partials(const float *P, int splits, int64_t rows_pad,
                                  int64_t cols_pad, int64_t rows, int64_t cols, float *dW) {
  const int64_t n = rows * cols;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx / cols, c = idx % cols;
    float s = 0.0f;
    for (int z = 0; z < splits; ++z) s += P[((int64_t)z * rows_pad + r) * cols_pad + c];
    dW[idx] = s;
  }
}

// Row sums of a [rows][ld] bf16 matrix over its first m columns (one warp
// per row, fixed order).
__global__ void k_row_sums(const __nv_bfloat16 *X, int64_t ld, int64_t rows, int64_t m,
                           float *out) {
  const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= rows) return;
  float s = 0.0f;
  for (int64_t i = lane; i < m; i += 32) s += __bfloat162float(X[row * ld + i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[row] = s;
}

// loss = sum (y - t)^2 * scale, dY = 2 scale (y - t) (bf16, row-major and
// transposed); columns >= n are zero in dY.
__global__ void k_loss_grad(const float *Yh, int64_t ldy, const float *Tg, int64_t ldt,
                            int64_t m, int64_t n, int64_t n_pad, float scale,
                            __nv_bfloat16 *dY, int64_t ld, __nv_bfloat16 *dYT, int64_t ldtt,
                            float *loss) {
  float acc = 0.0f;
  const int64_t total = m * n_pad;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = idx / n_pad, c = idx % n_pad;
    float g = 0.0f;
    if (c < n) {
      const float d = Yh[r * ldy + c] - Tg[r * ldt + c];
      acc += d * d;
      g = 2.0f * scale * d;
    }
    const __nv_bfloat16 gb = __float2bfloat16_rn(g);
    dY[r * ld + c] = gb;
    dYT[c * ldtt + r] = gb;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, acc * scale);
}

__global__ void k_adam(float *p, const float *g, float *mo, float *ve, int64_t rows,
                       int64_t cols, float lr, float b1, float b2, float eps, float c1,
                       float c2, __nv_bfloat16 *W, int64_t ldw, __nv_bfloat16 *WT,
                       int64_t ldwt) {
  const int64_t n = rows * cols;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[idx];
    const float m = b1 * mo[idx] + (1.0f - b1) * gi;
    const float v = b2 * ve[idx] + (1.0f - b2) * gi * gi;
    mo[idx] = m;
    ve[idx] = v;
    const float w = p[idx] - lr * (m * c1) / (sqrtf(v * c2) + eps);
    p[idx] = w;
    const int64_t r = idx / cols, c = idx % cols;
    if (W) W[r * ldw + c] = __float2bfloat16_rn(w);
    if (WT) WT[c * ldwt + r] = __float2bfloat16_rn(w);
  }
}

// Features of state i: [(T - mu0)/sd0, (ln P - mu1)/sd1,
// (ln(Y_k + 1e-12) - mu_k)/sd_k for the N species], zero padding to ldx.
// out_of_box[i] = 1 when a feature leaves the training box [lo, hi].
__global__ void k_features(int64_t n, const double *T, const double *P, const double *Y,
                           int64_t ld, int nsp, const float *mu, const float *sd,
                           const float *lo, const float *hi, __nv_bfloat16 *X, int64_t ldx,
                           __nv_bfloat16 *XT, int64_t ldxt, int nfeat_pad,
                           unsigned char *out_of_box, float *raw) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    bool out = false;
    double ysum = 0.0;
    // eight features at a time: one 16-byte store of the row
    for (int f0 = 0; f0 < nfeat_pad; f0 += 8) {
      float x[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int f = f0 + j;
        float v = 0.0f;
        if (f == 0) {
          v = (float)T[i];
        } else if (f == 1) {
          v = logf((float)P[i]);
        } else if (f < 2 + nsp) {
          const int k = f - 2;
          double y;
          if (k < nsp - 1) {
            y = Y[(int64_t)k * ld + i];
            ysum += y;
          } else {
            y = 1.0 - ysum;
          }
          v = logf(fmaxf((float)y, 0.0f) + 1.0e-12f);
        }
        if (f < 2 + nsp) {
          if (raw) raw[i * (2 + nsp) + f] = v;
          if (lo && (v < lo[f] || v > hi[f])) out = true;
          v = (v - mu[f]) / sd[f];
        }
        x[j] = v;
        if (XT) XT[(int64_t)f * ldxt + i] = __float2bfloat16_rn(v);
      }
      *reinterpret_cast<uint4 *>(X + i * ldx + f0) =
          make_uint4(pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(x[4], x[5]),
                     pack_bf16(x[6], x[7]));
    }
    if (out_of_box) out_of_box[i] = out;
  }
}

// v * 2^e as a double, by integer operations on v's fields (exact); values
// below the fp32 normal range give zero.
__device__ __forceinline__ double scale_to_double(float v, int e) {
  const uint32_t b = __float_as_uint(v);
  const int ef = (int)((b >> 23) & 0xFF);
  if (ef == 0) return 0.0;
  if (ef == 0xFF) return (double)v;
  const int ed = ef - 127 + 1023 + e;
  const uint64_t sign = (uint64_t)(b >> 31) << 63;
  if (ed >= 0x7FF) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
  if (ed <= 0) return __longlong_as_double((long long)sign);
  return __longlong_as_double(
      (long long)(sign | ((uint64_t)ed << 52) | ((uint64_t)(b & 0x7FFFFF) << 29)));
}

constexpr int MAX_ELEM = 8;

// Network output -> wdot.  With u_k = sign(y_k) expm1(|y_k|) (the rate in
// units of its scale s_k = sm_k 2^se_k), w_k = (u_k sm_k) 2^se_k in FP64.
// The state goes to the exact kernel when it is outside the training box or
// when its element residual
//   max_e |sum_k a_ek w_k| / sum_k a_ek (|w_k| + s_k)
// exceeds tol: conservation violated by more than tol of the rates' own
// size, or of their typical size where the rates are small.  The residual
// is formed in fp32 from cons[e][k] = a_ek s_k / max_j a_ej s_j, which
// keeps every term in range (rates reach 1e50 and beyond).
__global__ void k_output(int64_t n, const float *Yh, int64_t ldy, int nsp, const float *sm,
                         const int *se, const float *cons, int nelem, float tol,
                         const unsigned char *out_of_box, double *wdot, int64_t ld,
                         unsigned char *fallback) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float sum[MAX_ELEM], mag[MAX_ELEM];
#pragma unroll
    for (int e = 0; e < MAX_ELEM; ++e) sum[e] = mag[e] = 0.0f;
    for (int k = 0; k < nsp; ++k) {
      const float y = Yh[i * ldy + k];
      const float u = copysignf(expm1f(fabsf(y)), y);
      wdot[(int64_t)k * ld + i] = scale_to_double(u * sm[k], se[k]);
#pragma unroll
      for (int e = 0; e < MAX_ELEM; ++e) {
        if (e < nelem) {
          const float c = cons[e * nsp + k];
          sum[e] = fmaf(c, u, sum[e]);
          mag[e] = fmaf(c, fabsf(u) + 1.0f, mag[e]);
        }
      }
    }
    float worst = 0.0f;
#pragma unroll
    for (int e = 0; e < MAX_ELEM; ++e)
      if (e < nelem && mag[e] > 0.0f) worst = fmaxf(worst, fabsf(sum[e]) / mag[e]);
    const bool fb = !(worst <= tol) || (out_of_box && out_of_box[i]);
    fallback[i] = fb;
  }
}

// Two-member output with an error gate.  The served y_k is the mean of the
// members' outputs; in y = sign(u) log1p|u| space a change dy moves w by
// |dy| (|w| + s) to first order, so an error in y is the reported error
// e = max_k |w_k - w_k,exact| / (|w_k,exact| + s_k).  The gate score of a
// state is
//   g = dweight log10(D + 1e-4) + E,   D = max_k |y_k,a - y_k,b|,
// the members' disagreement plus E = est[i * lde], the output of a network
// trained to predict log10(e + 1e-4) (omitted when est is NULL); the
// disagreement term is weighted by dweight (0 when the error network takes
// D as an input, see k_disagreement).  A state
// goes back to the exact kernel as in k_output, or when g > stol (NaN
// included).  gate[i] (optional) receives g, for calibrating stol.
__global__ void k_output2(int64_t n, const float *Ya, const float *Yb, int64_t ldy, int nsp,
                          const float *sm, const int *se, const float *cons, int nelem,
                          float tol, float dweight, const float *est, int64_t lde,
                          float stol, const unsigned char *out_of_box, double *wdot,
                          int64_t ld, unsigned char *fallback, float *gate) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float sum[MAX_ELEM], mag[MAX_ELEM];
#pragma unroll
    for (int e = 0; e < MAX_ELEM; ++e) sum[e] = mag[e] = 0.0f;
    float d = 0.0f;
    for (int k = 0; k < nsp; ++k) {
      const float ya = Ya[i * ldy + k], yb = Yb[i * ldy + k];
      d = fmaxf(d, fabsf(ya - yb));
      const float y = 0.5f * (ya + yb);
      const float u = copysignf(expm1f(fabsf(y)), y);
      wdot[(int64_t)k * ld + i] = scale_to_double(u * sm[k], se[k]);
#pragma unroll
      for (int e = 0; e < MAX_ELEM; ++e) {
        if (e < nelem) {
          const float c = cons[e * nsp + k];
          sum[e] = fmaf(c, u, sum[e]);
          mag[e] = fmaf(c, fabsf(u) + 1.0f, mag[e]);
        }
      }
    }
    float worst = 0.0f;
#pragma unroll
    for (int e = 0; e < MAX_ELEM; ++e)
      if (e < nelem && mag[e] > 0.0f) worst = fmaxf(worst, fabsf(sum[e]) / mag[e]);
    const float g = dweight * log10f(d + 1.0e-4f) + (est ? est[i * lde] : 0.0f);
    const bool fb = !(worst <= tol) || !(g <= stol) || (out_of_box && out_of_box[i]);
    fallback[i] = fb;
    if (gate) gate[i] = g;
  }
}

// The members' disagreement D = max_k |y_k,a - y_k,b| as an input of the
// error network: X[i][col] = bf16((log10(D + 1e-4) - mu) / sd).
__global__ void k_disagreement(int64_t n, const float *Ya, const float *Yb, int64_t ldy,
                               int nsp, float mu, float sd, __nv_bfloat16 *X, int64_t ldx,
                               int col) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float d = 0.0f;
    for (int k = 0; k < nsp; ++k) d = fmaxf(d, fabsf(Ya[i * ldy + k] - Yb[i * ldy + k]));
    X[i * ldx + col] = __float2bfloat16_rn((log10f(d + 1.0e-4f) - mu) / sd);
  }
}

// Indices of flagged states (order unspecified; one warp-aggregated atomic
// per warp).  count must be zero on entry.
__global__ void k_compact(int64_t n, const unsigned char *flag, int64_t *idx,
                          unsigned long long *count) {
  const int lane = threadIdx.x & 31;
  for (int64_t c0 = (int64_t)blockIdx.x * blockDim.x; c0 < n;
       c0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = c0 + threadIdx.x;
    const bool f = i < n && flag[i];
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    if (!bal) continue;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(count, (unsigned long long)__popc(bal));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (f) idx[base + __popc(bal & ((1u << lane) - 1u))] = i;
  }
}

__global__ void k_gather(int64_t m, const int64_t *idx, const double *T, const double *P,
                         const double *Y, int64_t ld, int rows, double *Tc, double *Pc,
                         double *Yc, int64_t ldc) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m;
       j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx[j];
    Tc[j] = T[i];
    Pc[j] = P[i];
    for (int k = 0; k < rows; ++k) Yc[(int64_t)k * ldc + j] = Y[(int64_t)k * ld + i];
  }
}

__global__ void k_scatter(int64_t m, const int64_t *idx, const double *Wc, int64_t ldc,
                          int rows, double *W, int64_t ld) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m;
       j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx[j];
    for (int k = 0; k < rows; ++k) W[(int64_t)k * ld + i] = Wc[(int64_t)k * ldc + j];
  }
}

inline int grid1(int64_t n, int per = 256) {
  int64_t g = (n + per - 1) / per;
  if (g > 65535) g = 65535;
  return (int)(g < 1 ? 1 : g);
}

template <class Epi>
cudaError_t gemm_bn(const CUtensorMap &ta, const CUtensorMap &tb, int64_t M_pad, int64_t N_pad,
                    int64_t K, int bn, const Epi &epi, cudaStream_t s, int splits = 1) {
  // two-stage ring, 8 warps: two CTAs per SM (the network's K is small)
  switch (bn) {
    case 64: return launch_gemm<64, Epi, 2, 256>(ta, tb, M_pad, N_pad, K, epi, nullptr, s, splits);
    case 128: return launch_gemm<128, Epi, 2, 256>(ta, tb, M_pad, N_pad, K, epi, nullptr, s, splits);
    case 256: return launch_gemm<256, Epi, 2, 256>(ta, tb, M_pad, N_pad, K, epi, nullptr, s, splits);
    default: return cudaErrorInvalidValue;
  }
}

inline int pick_bn(int64_t n_pad) {
  return n_pad % 256 == 0 ? 256 : n_pad % 128 == 0 ? 128 : n_pad % 64 == 0 ? 64 : 0;
}

inline int bad(const char *fn) {
  char buf[160];
  snprintf(buf, sizeof buf, "%s: invalid argument (null pointer, size or alignment)", fn);
  return report(CRS_ERR_ARG, buf);
}

inline int done(cudaError_t e, const char *fn) {
  if (e == cudaSuccess) return CRS_OK;
  char buf[200];
  snprintf(buf, sizeof buf, "%s: %s", fn, cudaGetErrorString(e));
  return report(CRS_ERR_CUDA, buf);
}

}  // namespace mlp
}  // namespace crs

using namespace crs;
using mlp::bad;
using mlp::done;

extern "C" {

int crs_mlp_forward(const void *X, const void *W, const float *b, int64_t M_pad, int64_t N_pad,
                    int64_t K, int64_t M, int64_t N, int act, float *Z, int64_t ldz, void *A,
                    int64_t lda, void *AT, int64_t ldat, float *Y32, int64_t ldy,
                    void *stream) {
  const int bn = mlp::pick_bn(N_pad);
  if (!X || !W || M_pad % 128 || K % 64 || !bn || M > M_pad || N > N_pad) return bad(__func__);
  CUtensorMap ta, tb;
  if (!make_tmap_bf16(&ta, X, M_pad, K, 128) || !make_tmap_bf16(&tb, W, N_pad, K, bn))
    return bad(__func__);
  mlp::EpiForward epi{b, act, (int)M, (int)N, Z, ldz, static_cast<__nv_bfloat16 *>(A), lda,
                      static_cast<__nv_bfloat16 *>(AT), ldat, Y32, ldy};
  cudaError_t e = mlp::gemm_bn(ta, tb, M_pad, N_pad, K, bn, epi, static_cast<cudaStream_t>(stream));
  return done(e, __func__);
}

int crs_mlp_backward_data(const void *dZ, const void *WT, int64_t M_pad, int64_t Nin_pad,
                          int64_t Kout, int64_t M, int64_t Nin, const float *Zprev,
                          int64_t ldz, void *dZprev, int64_t ld, void *dZprevT, int64_t ldt,
                          void *stream) {
  const int bn = mlp::pick_bn(Nin_pad);
  if (!dZ || !WT || !Zprev || !dZprev || M_pad % 128 || Kout % 64 || !bn) return bad(__func__);
  CUtensorMap ta, tb;
  if (!make_tmap_bf16(&ta, dZ, M_pad, Kout, 128) || !make_tmap_bf16(&tb, WT, Nin_pad, Kout, bn))
    return bad(__func__);
  mlp::EpiBackwardData epi{Zprev, ldz, (int)M, (int)Nin, static_cast<__nv_bfloat16 *>(dZprev),
                           ld, static_cast<__nv_bfloat16 *>(dZprevT), ldt};
  cudaError_t e = mlp::gemm_bn(ta, tb, M_pad, Nin_pad, Kout, bn, epi, static_cast<cudaStream_t>(stream));
  return done(e, __func__);
}

int crs_mlp_backward_weight(const void *dZT, const void *AT, int64_t Nout_pad, int64_t Nin_pad,
                            int64_t M_pad, int64_t Nout, int64_t Nin, int splits,
                            float *partial, float *dW, void *stream) {
  const int bn = mlp::pick_bn(Nin_pad);
  if (!dZT || !AT || !partial || !dW || Nout_pad % 128 || M_pad % 64 || !bn || splits < 1 ||
      (M_pad / 64) % splits)
    return bad(__func__);
  CUtensorMap ta, tb;
  if (!make_tmap_bf16(&ta, dZT, Nout_pad, M_pad, 128) || !make_tmap_bf16(&tb, AT, Nin_pad, M_pad, bn))
    return bad(__func__);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  mlp::EpiPartial epi{partial, Nout_pad, Nin_pad};
  cudaError_t e = mlp::gemm_bn(ta, tb, Nout_pad, Nin_pad, M_pad, bn, epi, s, splits);
  if (e != cudaSuccess) return done(e, __func__);
  mlp::k_reduce_partials<<<mlp::grid1(Nout * Nin), 256, 0, s>>>(partial, splits, Nout_pad,
                                                                 Nin_pad, Nout, Nin, dW);
  return done(cudaGetLastError(), __func__);
}

int crs_mlp_row_sums(const void *X, int64_t ld, int64_t rows, int64_t m, float *out,
                     void *stream) {
  if (!X || !out || rows < 0 || m < 0 || ld < m) return bad(__func__);
  if (rows == 0) return CRS_OK;
  mlp::k_row_sums<<<(unsigned)((rows + 7) / 8), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16 *>(X), ld, rows, m, out);
  return done(cudaGetLastError(), __func__);
}

int crs_mlp_loss_grad(const float *Yh, int64_t ldy, const float *Tg, int64_t ldt, int64_t m,
                      int64_t n, int64_t n_pad, float scale, void *dY, int64_t ld, void *dYT,
                      int64_t ldtt, float *loss, void *stream) {
  if (!Yh || !Tg || !dY || !dYT || m < 0 || n > n_pad) return bad(__func__);
  mlp::k_loss_grad<<<mlp::grid1(m * n_pad), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      Yh, ldy, Tg, ldt, m, n, n_pad, scale, static_cast<__nv_bfloat16 *>(dY), ld,
      static_cast<__nv_bfloat16 *>(dYT), ldtt, loss);
  return done(cudaGetLastError(), __func__);
}

int crs_adam_step(float *p, const float *g, float *m, float *v, int64_t rows, int64_t cols,
                  float lr, float b1, float b2, float eps, int step, void *W, int64_t ldw,
                  void *WT, int64_t ldwt, void *stream) {
  if (!p || !g || !m || !v || rows < 0 || cols < 0 || step < 1) return bad(__func__);
  const float c1 = 1.0f / (1.0f - powf(b1, (float)step));
  const float c2 = 1.0f / (1.0f - powf(b2, (float)step));
  mlp::k_adam<<<mlp::grid1(rows * cols), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      p, g, m, v, rows, cols, lr, b1, b2, eps, c1, c2, static_cast<__nv_bfloat16 *>(W), ldw,
      static_cast<__nv_bfloat16 *>(WT), ldwt);
  return done(cudaGetLastError(), __func__);
}

int crs_surrogate_features(int64_t n, const double *T, const double *P, const double *Y,
                           int64_t ld, int nsp, const float *mu, const float *sd,
                           const float *lo, const float *hi, void *X, int64_t ldx, void *XT,
                           int64_t ldxt, int nfeat_pad, unsigned char *out_of_box, float *raw,
                           void *stream) {
  if (n < 0 || !T || !P || !Y || !mu || !sd || !X || nfeat_pad < 2 + nsp || nfeat_pad % 8 ||
      ldx % 8 || ldx < nfeat_pad || (reinterpret_cast<uintptr_t>(X) & 15) || ld < n)
    return bad(__func__);
  if (n == 0) return CRS_OK;
  mlp::k_features<<<mlp::grid1(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      n, T, P, Y, ld, nsp, mu, sd, lo, hi, static_cast<__nv_bfloat16 *>(X), ldx,
      static_cast<__nv_bfloat16 *>(XT), ldxt, nfeat_pad, out_of_box, raw);
  return done(cudaGetLastError(), __func__);
}

int crs_surrogate_output(int64_t n, const float *Yh, int64_t ldy, int nsp, const float *scale_m,
                         const int *scale_e, const float *cons, int nelem, float tol,
                         const unsigned char *out_of_box, double *wdot, int64_t ld,
                         unsigned char *fallback, void *stream) {
  if (n < 0 || !Yh || !scale_m || !scale_e || !wdot || !fallback || (nelem && !cons) ||
      nelem < 0 || nelem > mlp::MAX_ELEM || ld < n || ldy < nsp)
    return bad(__func__);
  if (n == 0) return CRS_OK;
  mlp::k_output<<<mlp::grid1(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      n, Yh, ldy, nsp, scale_m, scale_e, cons, nelem, tol, out_of_box, wdot, ld, fallback);
  return done(cudaGetLastError(), __func__);
}

int crs_surrogate_output2(int64_t n, const float *Ya, const float *Yb, int64_t ldy, int nsp,
                          const float *scale_m, const int *scale_e, const float *cons, int nelem,
                          float tol, float dweight, const float *est, int64_t lde, float stol,
                          const unsigned char *out_of_box, double *wdot, int64_t ld,
                          unsigned char *fallback, float *gate, void *stream) {
  if (n < 0 || !Ya || !Yb || !scale_m || !scale_e || !wdot || !fallback ||
      (nelem && !cons) || nelem < 0 || nelem > mlp::MAX_ELEM || ld < n || ldy < nsp ||
      (est && lde < 1))
    return bad(__func__);
  if (n == 0) return CRS_OK;
  mlp::k_output2<<<mlp::grid1(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      n, Ya, Yb, ldy, nsp, scale_m, scale_e, cons, nelem, tol, dweight, est, lde, stol,
      out_of_box, wdot, ld, fallback, gate);
  return done(cudaGetLastError(), __func__);
}

int crs_surrogate_disagreement(int64_t n, const float *Ya, const float *Yb, int64_t ldy,
                               int nsp, float mu, float sd, void *X, int64_t ldx, int col,
                               void *stream) {
  if (n < 0 || !Ya || !Yb || !X || ldy < nsp || col < 0 || col >= ldx || !(sd > 0.0f))
    return bad(__func__);
  if (n == 0) return CRS_OK;
  mlp::k_disagreement<<<mlp::grid1(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      n, Ya, Yb, ldy, nsp, mu, sd, static_cast<__nv_bfloat16 *>(X), ldx, col);
  return done(cudaGetLastError(), __func__);
}

int crs_select(int64_t n, const unsigned char *flag, int64_t *idx, int64_t *count, void *stream) {
  if (n < 0 || !flag || !idx || !count) return bad(__func__);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int64_t), s);
  if (e != cudaSuccess || n == 0) return done(e, __func__);
  mlp::k_compact<<<mlp::grid1(n), 256, 0, s>>>(n, flag, idx,
                                               reinterpret_cast<unsigned long long *>(count));
  return done(cudaGetLastError(), __func__);
}

int crs_gather_states(int64_t m, const int64_t *idx, const double *T, const double *P,
                      const double *Y, int64_t ld, int rows, double *Tc, double *Pc, double *Yc,
                      int64_t ldc, void *stream) {
  if (m < 0 || !idx || ldc < m) return bad(__func__);
  if (m == 0) return CRS_OK;
  mlp::k_gather<<<mlp::grid1(m), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      m, idx, T, P, Y, ld, rows, Tc, Pc, Yc, ldc);
  return done(cudaGetLastError(), __func__);
}

int crs_scatter_wdot(int64_t m, const int64_t *idx, const double *Wc, int64_t ldc, int rows,
                     double *W, int64_t ld, void *stream) {
  if (m < 0 || !idx || ldc < m) return bad(__func__);
  if (m == 0) return CRS_OK;
  mlp::k_scatter<<<mlp::grid1(m), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      m, idx, Wc, ldc, rows, W, ld);
  return done(cudaGetLastError(), __func__);
}

}  // extern "C"
