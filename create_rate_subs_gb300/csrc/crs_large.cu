// Mixed precision for mechanisms whose per-state columns do not fit on chip
// (hundreds of species, thousands of reactions): the rates and the species
// sums as separate passes over HBM.
//
// The one-state-per-thread kernel keeps a state's concentrations and wdot
// accumulators in shared memory (12 B per species and thread); at 561
// species that leaves room for ~30 states per SM.  The warp-per-state
// kernel fits but reads every reaction's tables per lane, scattered, with
// 8 warps per SM.  Here:
//
//  k_rates_tile  a CTA holds a tile of 32 states (lane = state) and their
//                FP32 concentrations in shared memory ([N][32], 128 B per
//                species); its warps take the shape blocks (four reactions
//                of one stoichiometric shape) round-robin, so every table
//                read is uniform across a warp, and write each net rate
//                (fwd - rev) * pres_mod in FP64 to HBM, q[r][state]:
//                256 B per warp store.  The arithmetic is the one-state-
//                per-thread kernel's (crs_mixed.cuh); tiles are handed out
//                from a per-launch counter.  Per state it also forms the
//                scale exponent of the tensor-core contraction.
//  k_spec_sum    wdot[k][i] = sum over species k's net coefficients, in
//                reaction order, of nu * q[r][i] in FP64 (lane = state);
//                or only the terms outside the bf16 window (the
//                contraction adds the rest).
//  k_pack_bf16   q[r][i] * 2^-c_i split into bf16 hi + lo rows [i][r] for
//                the contraction GEMM, through a shared-memory transpose.
//
// Traffic per state: R doubles written and read once (20 KB at 2539
// reactions), against ~17 k FP64 instructions of rates: the FP64 pipe, not
// HBM, stays the bound.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "crs_mixed.cuh"
#include "crs_tile.cuh"

namespace crs {
namespace large {

using namespace mixed;

// warps per CTA of the rates kernel: two CTAs of 8 warps fit an SM (two
// 72 KB concentration tiles at 561 species, 128 registers per thread), 16
// warps against 12 with three CTAs of 4 (+15% for the mixed rates pass)
constexpr int TW = 8;
static_assert(TW >= 2, "tile::state_sums runs on warps 0 and 1");
constexpr int WINDOW = 100;  // binary orders around c_s carried by bf16 hi + lo

using tile::QSink;
using tile::RatesOut;

template <bool KC1>
__global__ void __launch_bounds__(TW * 32, 2)
    k_rates_tile(const unsigned char *__restrict__ img, ImgLayout L, Batch b, RatesOut o) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ double s_rho[32], s_yN[32];
  __shared__ int s_es[TW][32], s_ec[TW][32];
  __shared__ int64_t s_tile;
  const Tab t = make_tab(img, L);
  const int N = t.N, R = t.R;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float *Cs = reinterpret_cast<float *>(smem);  // [N][32]
  const FCol C{Cs + lane, 32};
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
    s.logT = log(s.T);
    s.Tf = (float)s.T;
    s.Tff = ff_from_double(s.T);
    s.lTff = ff_from_double(s.logT);
    s.iTff = ff_from_double(s.invT);
    tile::state_sums(t, b, ic, warp, lane, P, s.invT * INV_RU, s_yN, s_rho);
    __syncthreads();
    const double rho = s_rho[lane];
    for (int k = warp; k < N; k += TW) {
      const double y = k == N - 1 ? s_yN[lane] : b.Y[(int64_t)k * b.ld + ic];
      C[k] = d2f_rn(y * (rho * t.inv_mw[k]));
    }
    __syncthreads();
    const float mix = d2f_rn(P * s.invT * INV_RU);
    // FP64 Kc polynomials here: the float-float form (KcMix) ran 12% slower
    // in this kernel (128 registers per thread at 16 warps per SM)
    using KC = typename std::conditional<KC1, KcPoly1, KcPolyG>::type;
    KC kc;
    kc.T = s.T;
    kc.logT = s.logT;
    kc.invT = s.invT;
    if constexpr (KC1) kc.Tbits = __double_as_longlong(s.T);
    int esum = 0, ecnt = 0;
    const QSink sink{o.q + i, o.ldq, valid, esum, ecnt};
    Shapes<0, false, KC, QSink>::run(t, s, C, kc, sink, b, i, warp, TW);
    for (int p = t.seg[NSHAPE] + warp; p < t.seg[NSHAPE + 1]; p += TW)
      general<false, false>(t, t.perm[p], s, mix, C, kc, sink, b, i);
    for (int p = t.seg[NSHAPE + 1] + warp; p < R; p += TW)  // PLOG / Chebyshev
      general<false, true>(t, t.perm[p], s, mix, C, kc, sink, b, i);
    s_es[warp][lane] = esum;
    s_ec[warp][lane] = ecnt;
    __syncthreads();
    if (warp == 0 && valid && o.escale) {
      int es = 0, ec = 0;
#pragma unroll
      for (int w = 0; w < TW; ++w) {
        es += s_es[w][lane];
        ec += s_ec[w][lane];
      }
      o.escale[i] = tile::scale_exponent(es, ec);
    }
    // the next tile replaces C and the tile number only after every warp
    // is done with this one
    __syncthreads();
  }
  tile::tiles_done(b.sched);
}

__device__ __forceinline__ bool in_window(double v, int c) {
  const int hi = __double2hiint(v), lo = __double2loint(v);
  const int e = (hi >> 20) & 0x7ff;
  const bool zero = ((hi & 0x7fffffff) | lo) == 0;
  return zero || (e != 0 && e != 0x7ff && abs(e - 1023 - c) <= WINDOW);
}

// wdot[k][i] (FP64) = sum over the net coefficients of species k, in
// reaction order, of nu * q[r][i]; OUTWIN: only the terms outside the bf16
// window of state i (zero when there are none).  CTA: one tile of 32
// states, warps over species.
template <bool OUTWIN>
__global__ void __launch_bounds__(256)
    k_spec_sum(const unsigned char *__restrict__ img, ImgLayout L, const double *__restrict__ q,
               int64_t ldq, int64_t n, const int *__restrict__ escale,
               const unsigned *__restrict__ outflag, double *__restrict__ wdot, int64_t ld,
               int32_t *status) {
  const Tab t = make_tab(img, L);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int bad = 0;
  for (int64_t tile = blockIdx.x; tile * 32 < n; tile += gridDim.x) {
    const int64_t i = tile * 32 + lane;
    const bool valid = i < n;
    const int64_t ic = valid ? i : tile * 32;
    const int c = OUTWIN ? escale[ic] : 0;
    const double *qi = q + ic;
    if (OUTWIN && !__any_sync(0xffffffffu, valid && outflag[ic] != 0u)) {
      // no term of these states lies outside the window: the sums are zero
      // (the contraction's epilogue adds the rest)
      if (valid)
        for (int k = warp; k < t.N; k += nw) wdot[(int64_t)k * ld + i] = 0.0;
      continue;
    }
    for (int k = warp; k < t.N; k += nw) {
      double w = 0.0;
      const int e1 = t.spc_ptr[k + 1];
      int e = t.spc_ptr[k];
      // four loads in flight ahead of the dependent FMAs
      for (; e + 4 <= e1; e += 4) {
        double v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = qi[(int64_t)t.spc_r[e + u] * ldq];
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (!OUTWIN || !in_window(v[u], c)) w = fma(t.spc_nu[e + u], v[u], w);
      }
      for (; e < e1; ++e) {
        const double v = qi[(int64_t)t.spc_r[e] * ldq];
        if (!OUTWIN || !in_window(v, c)) w = fma(t.spc_nu[e], v, w);
      }
      if (valid) {
        if (!OUTWIN) bad += ((__double2hiint(w) >> 20) & 0x7ff) == 0x7ff;
        wdot[(int64_t)k * ld + i] = w;
      }
    }
  }
  if (bad && status) atomicAdd(&status[1], bad);
}

// A[i][r] = bf16 hi of q[r][i] * 2^-c_i, A[i][Kh + r] = bf16 lo, for the
// terms within the window (others 0: k_spec_sum<true> sums them in FP64,
// and outflag[i], zero on entry, marks state i); columns R..Kh-1 zero.  CTA: 32 states x 64 reactions through shared
// memory, so that both the reads (256 B per reaction row) and the writes
// (128 B per state row) are contiguous.
__global__ void __launch_bounds__(256)
    k_pack_bf16(const double *__restrict__ q, int64_t ldq, int64_t n, int R, int Kh,
                const int *__restrict__ escale, __nv_bfloat16 *__restrict__ A, int64_t lda,
                unsigned *__restrict__ outflag) {
  __shared__ float f[64][33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t ntile = (n + 31) / 32;
  const int rtiles = Kh / 64;
  for (int64_t tt = blockIdx.x; tt < ntile * rtiles; tt += gridDim.x) {
    const int64_t s0 = (tt / rtiles) * 32;
    const int r0 = (int)(tt % rtiles) * 64;
    const int64_t i = s0 + lane;
    const bool valid = i < n;
    const int c = valid ? escale[i] : 0;
    for (int rr = warp; rr < 64; rr += 8) {
      const int r = r0 + rr;
      const double v = (valid && r < R) ? q[(int64_t)r * ldq + i] : 0.0;
      float x = 0.0f;
      if (!in_window(v, c)) atomicOr(&outflag[i], 1u);  // rare: marks the state
      else if (v != 0.0) {
        const int hi = __double2hiint(v), lo = __double2loint(v);
        // v * 2^-c exactly through the exponent field (the result stays a
        // normal number within 2^+-WINDOW), then rounded to fp32
        x = d2f_rn(__hiloint2double(hi - c * (1 << 20), lo));
      }
      f[rr][lane] = x;
    }
    __syncthreads();
    // thread = (state j, 8 reactions): one 16-byte store of hi and one of lo
    const int j = threadIdx.x >> 3, seg = threadIdx.x & 7;
    if (s0 + j < n) {
      __align__(16) __nv_bfloat16 h[8], l[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const float x = f[seg * 8 + u][j];
        h[u] = __float2bfloat16_rn(x);
        l[u] = __float2bfloat16_rn(x - __bfloat162float(h[u]));
      }
      __nv_bfloat16 *row = A + (s0 + j) * lda + r0 + seg * 8;
      *reinterpret_cast<uint4 *>(row) = *reinterpret_cast<const uint4 *>(h);
      *reinterpret_cast<uint4 *>(row + Kh) = *reinterpret_cast<const uint4 *>(l);
    }
    __syncthreads();
  }
}

}  // namespace large

int grid_for(int64_t n, int block, int max_ctas);

// Shared memory of the rates kernel for N species (the concentration tile).
size_t large_rates_smem(const ImgLayout &L) { return (size_t)L.N * 32 * sizeof(float); }

// Rates of n states (b: chunk-local, no intermediates requested) into
// q [R][ldq] and escale [n].  b.sched must be a free counter pair.
cudaError_t launch_rates_tile(const unsigned char *img, const ImgLayout &L, const Batch &b,
                              int sm_count, int smem_optin, cudaStream_t s, double *q,
                              int64_t ldq, int *escale) {
  const size_t bytes = large_rates_smem(L);
  if (bytes > (size_t)smem_optin || !b.sched) return cudaErrorNotSupported;
  auto k = L.kc_single ? large::k_rates_tile<true> : large::k_rates_tile<false>;
  cudaError_t e = set_smem_limit(k, bytes);
  if (e != cudaSuccess) return e;
  int per_sm = 1;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, large::TW * 32, bytes);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorNotSupported;
  const int64_t ntiles = (b.n + 31) / 32;
  const int grid = grid_for(ntiles, 1, sm_count * per_sm);
  k<<<grid, large::TW * 32, bytes, s>>>(img, L, b, tile::RatesOut{q, ldq, escale});
  return cudaGetLastError();
}

// outflag: NULL for the full sums; else the per-state marks of
// k_pack_bf16, and only the terms outside the window are summed.
cudaError_t launch_spec_sum(const unsigned char *img, const ImgLayout &L, const double *q,
                            int64_t ldq, int64_t n, const int *escale, const unsigned *outflag,
                            double *wdot, int64_t ld, int32_t *status, int sm_count,
                            cudaStream_t s) {
  const int64_t ntiles = (n + 31) / 32;
  const int grid = grid_for(ntiles, 1, sm_count * 8);
  if (outflag)
    large::k_spec_sum<true><<<grid, 256, 0, s>>>(img, L, q, ldq, n, escale, outflag, wdot, ld,
                                                 status);
  else
    large::k_spec_sum<false><<<grid, 256, 0, s>>>(img, L, q, ldq, n, escale, nullptr, wdot, ld,
                                                  status);
  return cudaGetLastError();
}

// outflag: n words, cleared here before the pack.
cudaError_t launch_pack_bf16(const double *q, int64_t ldq, int64_t n, int R, int Kh,
                             const int *escale, void *A, int64_t lda, unsigned *outflag,
                             int sm_count, cudaStream_t s) {
  if (Kh % 64 || lda % 8) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(outflag, 0, (size_t)n * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  const int64_t tiles = (n + 31) / 32 * (Kh / 64);
  const int grid = grid_for(tiles, 1, sm_count * 8);
  large::k_pack_bf16<<<grid, 256, 0, s>>>(q, ldq, n, R, Kh, escale,
                                          static_cast<__nv_bfloat16 *>(A), lda, outflag);
  return cudaGetLastError();
}

}  // namespace crs
