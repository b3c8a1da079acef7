// CRS_MODE_MIXED: FP32 bulk arithmetic, FP64 where stability needs it.
//
// FP64 instructions are kept for
//   * the net rate fwd - rev (cancels near equilibrium);
//   * the accumulation of wdot;
//   * per-state scalars (1/T, ln T, the mass-fraction sums behind rho).
// Everything else runs on the FP32 pipe, which on GB300 issues ~70x more
// operations per clock than the FP64 pipe:
//   * Arrhenius exponents ln|A| + b ln T - Ta/T as float-float pairs
//     (~44 significant bits), so that |x| up to ~300 keeps an absolute
//     error near 1e-12;
//   * exp(x) = 2^k exp(r): Cody-Waite reduction in FP32 with a 16-bit
//     ln2 head (exact through fmaf), r in [-ln2/2, ln2/2], degree-7 Taylor
//     polynomial (truncation 6e-9);
//   * rates kept as an FP32 mantissa times 2^E with an integer E, so that
//     rates far outside the FP32 range (1/Kc can reach e^150 with random
//     thermochemistry) neither overflow nor underflow; the FP64 value is
//     assembled with integer operations only;
//   * concentrations, third-body sums and fall-off broadening in FP32;
//   * the exponent of the equilibrium constant, ln(prefactor) + the
//     reaction's Kc polynomial in T, ln T and 1/T, as float-float multiply-
//     adds (KcMix: within ~3e-12 of the FP64 polynomial for exponents up to
//     ~400, where the FP32 rates notice 1e-7).  The warp-per-state kernel,
//     the large mechanisms' state tile (crs_large.cu) and mechanisms with
//     several T_common groups per reaction form it in FP64 (per-species
//     Gibbs terms S_k, or the polynomials).
// The error against FP64, scaled by the gross rate of each species, is
// measured by the tests and reported by bench.py.
#include <cuda_runtime.h>
#include <math.h>
#include <type_traits>

#include <cuda_bf16.h>

#include "crs_exp.cuh"
#include "crs_mixed.cuh"

namespace crs {
namespace mixed {

// One state per thread.  Per-state shared-memory columns: C (fp32) and
// the wdot accumulators W (FP64; only for the species below L.nw, the
// others never accumulate), 12 B per species and thread; the Kc
// exponents come from the per-reaction polynomials (no Gibbs column, the
// polynomials read through L1), and only the tables of this kernel's hot
// loop are staged, so that ~300 threads fit.  KC1: one T_common group per
// reaction (float-float polynomials, kc_mix).
template <bool STAGES, bool KC1>
__global__ void __launch_bounds__(352, 1)
    k_wdot(const unsigned char *__restrict__ img, ImgLayout L, Batch b) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  const unsigned amask = __activemask();
  const int lane = threadIdx.x & 31;
  Tab t;
  int nb = 0;
  if (!stage_ranges(smem, img, L, 2, &bar, b.status, t, nb)) {
    sched_done(b.sched, amask, lane);
    return;
  }
  const int N = t.N, NW = L.nw;
  const int st = blockDim.x;
  double *dbase = reinterpret_cast<double *>(smem + nb);
  const DCol W{dbase + threadIdx.x, st};
  const FCol C{reinterpret_cast<float *>(dbase + NW * st) + threadIdx.x, st};
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
    s.logT = texp::log_t(s.T, t.logtab);  // table logarithm (12 FP64 instructions)
    s.Tf = (float)s.T;
    s.Tff = ff_from_double_int(s.T);  // splits by integer operations
    s.lTff = ff_from_double_int(s.logT);
    s.iTff = ff_from_double_int(s.invT);
    // concentrations: sums and C = y * (rho / mw) in FP64, each C rounded
    // once to FP32
    double ysum = 0.0, mwi = 0.0;
    for (int k = 0; k < N - 1; ++k) {
      // streamed: read once, evict first, so that L1 keeps the rate rows
      const double y = __ldcs(b.Y + (int64_t)k * b.ld + i);
      ysum += y;
      mwi = fma(y, t.inv_mw[k], mwi);
      if (k < NW) W[k] = y;  // parked in the accumulator column until C is formed
    }
    const double yN = 1.0 - ysum;
    mwi = fma(yN, t.inv_mw[N - 1], mwi);
    const double rho = P / mwi * (s.invT * INV_RU);
    for (int k = 0; k < N - 1; ++k) {
      const double y = k < NW ? W[k] : b.Y[(int64_t)k * b.ld + i];  // no column: read again
      C[k] = d2f_rn(y * (rho * t.inv_mw[k]));
      if (k < NW) W[k] = 0.0;
    }
    C[N - 1] = d2f_rn(yN * (rho * t.inv_mw[N - 1]));
    if (N - 1 < NW) W[N - 1] = 0.0;
    if (STAGES && b.conc)
      for (int k = 0; k < N; ++k) b.conc[(int64_t)k * b.ld + i] = (double)C[k];
    const float mix = d2f_rn(P * s.invT * INV_RU);
    using KC = typename std::conditional<KC1, KcMix, KcPolyG>::type;
    KC kc;
    if constexpr (KC1) {
      kc.Tbits = __double_as_longlong(s.T);
      kc.T = s.Tff;
      kc.logT = s.lTff;
      kc.invT = s.iTff;
    } else {
      kc.T = s.T;
      kc.logT = s.logT;
      kc.invT = s.invT;
    }
    const WSink<DCol> sink{W};
    Shapes<0, STAGES, KC, WSink<DCol>>::run(t, s, C, kc, sink, b, i);
    for (int p = t.seg[NSHAPE]; p < t.seg[NSHAPE + 1]; ++p)
      general<STAGES, false>(t, t.perm[p], s, mix, C, kc, sink, b, i);
    for (int p = t.seg[NSHAPE + 1]; p < t.R; ++p)  // PLOG / Chebyshev
      general<STAGES, true>(t, t.perm[p], s, mix, C, kc, sink, b, i);
    for (int k = 0; k < N; ++k) {
      const double v = k < NW ? W[k] : 0.0;
      bad += ((__double2hiint(v) >> 20) & 0x7ff) == 0x7ff;  // inf or NaN, integer test
      __stcs(b.wdot + (int64_t)k * b.ld + i, v);  // streamed out
    }
  }
  if (bad && b.status) atomicAdd(&b.status[1], bad);
  sched_done(b.sched, amask, lane);
}

// ---- warp per state (see crs_fast.cu for the layout) --------------------
constexpr int DW = 8;  // most warps per CTA

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Rates-only variant (OUTQ, see QOut): terms whose binary exponent lies
// more than WINDOW from the state's scale c_s are summed here in FP64
// instead and written to wdot, to which the contraction then adds.
constexpr int WINDOW = 100;

__device__ __forceinline__ int dexp2(double v) {
  return (int)((__double2hiint(v) >> 20) & 0x7ff) - 1023;
}

template <bool STAGES, bool SMEM_TAB, bool OUTQ>
__global__ void __launch_bounds__(DW * 32)
    k_wdot_warp(const unsigned char *__restrict__ img, ImgLayout L, Batch b,
                int per_warp, QOut qo) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  int nb = 0;
  Tab t;
  if (SMEM_TAB) {
    if (!stage_ranges(smem, img, L, 3, &bar, b.status, t, nb)) return;
  } else {
    t = make_tab(img, L);
  }
  const int N = t.N, R = t.R;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *wb = reinterpret_cast<double *>(smem + nb) + (size_t)warp * per_warp;
  double *bT = wb, *bP = wb + 32, *biT = wb + 64, *blT = wb + 96;
  const DArr S{wb + 128};
  double *q = wb + 128 + N;
  const FArr C{reinterpret_cast<float *>(wb + 128 + N + R)};
  uint32_t *mask = reinterpret_cast<uint32_t *>(wb + 128 + N + R + (N + 1) / 2);
  const int l0 = t.lane_ptr[lane], l1 = t.lane_ptr[lane + 1];
  int bad = 0;
  const int nw = blockDim.x >> 5;
  const int64_t nwarp = (int64_t)gridDim.x * nw;
  for (int64_t i0 = ((int64_t)blockIdx.x * nw + warp) * 32; i0 < b.n; i0 += nwarp * 32) {
    {
      const int64_t i = i0 + lane;
      const double T = i < b.n ? b.T[i] : 1000.0;
      bT[lane] = T;
      bP[lane] = i < b.n ? b.P[i] : 101325.0;
      biT[lane] = 1.0 / T;
      blT[lane] = log(T);
    }
    __syncwarp();
    const int jn = (b.n - i0) < 32 ? (int)(b.n - i0) : 32;
    for (int j = 0; j < jn; ++j) {
      const int64_t i = i0 + j;
      State s;
      s.T = bT[j];
      s.invT = biT[j];
      s.logT = blT[j];
      s.Tf = (float)s.T;
      s.Tff = ff_from_double(s.T);
      s.lTff = ff_from_double(s.logT);
      s.iTff = ff_from_double(s.invT);
      const double P = bP[j];
      s.P = P;
      double mw = 0.0;
      for (int k = lane; k < N - 1; k += 32) {
        const double y = b.Y[(int64_t)k * b.ld + i];
        S[k] = y;  // parked in the Gibbs column until C is formed
        mw = fma(y, t.inv_mw[k], mw);
      }
      mw = warp_sum(mw);
      __syncwarp();
      // y_N = 1 - sum y in the reference's left-to-right order on every
      // lane (rate_subs.py:1312-1320): where the bath gas is scarce, the
      // rounding of this difference is a large relative error of C_N
      double ys = N > 1 ? S[0] : 0.0;
      for (int k = 1; k < N - 1; ++k) ys += S[k];
      const double yN = 1.0 - ys;
      mw = fma(yN, t.inv_mw[N - 1], mw);
      const double rho = P / mw * (s.invT * INV_RU);
      __syncwarp();  // every lane has read the parked y before any is replaced
      for (int k = lane; k < N; k += 32) {
        const double y = (k == N - 1) ? yN : S[k];
        const float c = d2f_rn(y * (rho * t.inv_mw[k]));
        C[k] = c;
        if (STAGES && b.conc) b.conc[(int64_t)k * b.ld + i] = (double)c;
        const double *g = t.sp_gibbs + 14 * k + ((s.T <= t.sp_tmid[k]) ? 0 : 7);
        const double h = fma(fma(fma(g[5], s.T, g[4]), s.T, g[3]), s.T, g[2]);
        double v = fma(h, s.T, g[0]);
        v = fma(g[1], s.logT, v);
        S[k] = fma(g[6], s.invT, v);  // FP64 Gibbs term
      }
      __syncwarp();
      const float mix = d2f_rn(P * s.invT * INV_RU);
      for (int p = lane; p < R; p += 32) {
        const int r = t.dperm[p];
        double fwd, rev;
        float pm;
        q[r] = rxn_net(t, r, s, mix, C, KcFromGibbs<DArr>{S}, fwd, rev, pm);
        if (STAGES) {
          const int jr = t.rev_idx[r], pp = t.pm_idx[r];
          if (b.fwd) b.fwd[(int64_t)r * b.ld + i] = fwd;
          if (b.rev && jr >= 0) b.rev[(int64_t)jr * b.ld + i] = rev;
          if (b.pm && pp >= 0) b.pm[(int64_t)pp * b.ld + i] = (double)pm;
        }
      }
      __syncwarp();
      if (!OUTQ) {
        for (int a = l0; a < l1; ++a) {
          const int k = t.lane_sp[a];
          double w = 0.0;
          for (int e = t.spc_ptr[k]; e < t.spc_ptr[k + 1]; ++e)
            w = fma(t.spc_nu[e], q[t.spc_r[e]], w);  // FP64 accumulation
          bad += !isfinite(w);
          b.wdot[(int64_t)k * b.ld + i] = w;
        }
      } else {
        // scale centre: mean binary exponent of the nonzero finite terms
        // (tests on the bit pattern: no FP64 instruction)
        int esum = 0, ecnt = 0;
        for (int r = lane; r < R; r += 32) {
          const int hi = __double2hiint(q[r]);
          const int e = (hi >> 20) & 0x7ff;
          if (e != 0x7ff && ((hi & 0x7fffffff) | __double2loint(q[r])) != 0) {
            esum += e - 1023;
            ++ecnt;
          }
        }
        for (int w = lane; w < (R + 31) / 32; w += 32) mask[w] = 0u;
        esum = __reduce_add_sync(0xffffffffu, esum);
        ecnt = __reduce_add_sync(0xffffffffu, ecnt);
        const int c = ecnt ? (int)lrint((double)esum / ecnt) : 0;
        if (lane == 0) qo.escale[i] = c;
        __syncwarp();
        __nv_bfloat16 *row = static_cast<__nv_bfloat16 *>(qo.A) + (int64_t)i * qo.lda;
        bool any_out = false;
        for (int r = lane; r < qo.Kh; r += 32) {
          const double v = r < R ? q[r] : 0.0;
          const int hi = __double2hiint(v), lo = __double2loint(v);
          const int e = (hi >> 20) & 0x7ff;
          // zero, or a normal number within WINDOW binary orders of c
          const bool zero = ((hi & 0x7fffffff) | lo) == 0;
          const bool inwin = zero || (e != 0 && e != 0x7ff && abs(e - 1023 - c) <= WINDOW);
          float f = 0.0f;
          if (!inwin) {
            atomicOr(&mask[r >> 5], 1u << (r & 31));
            any_out = true;
          } else if (!zero) {
            // v * 2^-c exactly, by the exponent field (the result stays a
            // normal number within 2^+-WINDOW), then rounded to fp32
            f = d2f_rn(__hiloint2double(hi - c * (1 << 20), lo));
          }
          const __nv_bfloat16 bh = __float2bfloat16_rn(f);
          row[r] = bh;
          row[qo.Kh + r] = __float2bfloat16_rn(f - __bfloat162float(bh));
        }
        any_out = __any_sync(0xffffffffu, any_out);
        __syncwarp();
        // out-of-window terms in FP64, in reaction order per species (the
        // contraction's epilogue adds the rest); zeros when there are none
        for (int a = l0; a < l1; ++a) {
          const int k = t.lane_sp[a];
          double w = 0.0;
          if (any_out)
            for (int e = t.spc_ptr[k]; e < t.spc_ptr[k + 1]; ++e) {
              const int r = t.spc_r[e];
              if (mask[r >> 5] & (1u << (r & 31))) w = fma(t.spc_nu[e], q[r], w);
            }
          b.wdot[(int64_t)k * b.ld + i] = w;
        }
      }
      __syncwarp();
    }
  }
  if (bad && b.status) atomicAdd(&b.status[1], bad);
}

}  // namespace mixed

int grid_for(int64_t n, int block, int max_ctas);

// Thread-per-state mixed kernel (CRS_MODE_MIXED_TPS, and CRS_MODE_MIXED
// when it fits): as many threads per CTA (at most 352) as the shared
// memory left by the tables allows.
cudaError_t launch_wdot_mixed_tps(const unsigned char *img, const ImgLayout &L,
                                  const Batch &b, int sm_count, int smem_optin,
                                  cudaStream_t s) {
  const bool stages = b.conc || b.fwd || b.rev || b.pm;
  auto k = L.kc_single ? (stages ? mixed::k_wdot<true, true> : mixed::k_wdot<false, true>)
                       : (stages ? mixed::k_wdot<true, false> : mixed::k_wdot<false, false>);
  const size_t tab = (size_t)(L.rng[2][1] - L.rng[2][0] + L.rng[2][3] - L.rng[2][2]);
  const size_t per = (size_t)L.nw * 8 + (size_t)L.N * 4;
  const long long room = (long long)smem_optin - (long long)tab;
  // any thread count, but a last warp under half full is dropped: the FP64
  // pipe charges a whole warp instruction whatever the active lanes, so a
  // sparse warp costs more pipe time than its states are worth (321 threads
  // ran 4% slower than 317, the tenth warp holding 1 thread against 29)
  int block = room > 0 ? (int)(room / (long long)per) : 0;
  if (block > 352) block = 352;
  if (block % 32 < 16) block -= block % 32;
  // the compact nu lists must be exact (else the warp kernel runs)
  if (block < 32 || !L.nu_hi_exact) return cudaErrorNotSupported;
  const size_t bytes = tab + per * block;
  const cudaError_t e = set_smem_limit(k, bytes);
  if (e != cudaSuccess) return e;
  k<<<grid_for(b.n, block, sm_count), block, bytes, s>>>(img, L, b);
  return cudaGetLastError();
}

// Warp-per-state mixed kernel.  qo.A == nullptr: full wdot (CSR sum in
// FP64); else the rates-only variant for the tensor-core contraction.
cudaError_t launch_wdot_mixed_q(const unsigned char *img, const ImgLayout &L,
                                const Batch &b, int sm_count, int smem_optin,
                                cudaStream_t s, const mixed::QOut &qo) {
  // doubles: 4 x 32 scalars, S[N], q[R], C[N] floats, R-bit mask
  const int per_warp = 128 + L.N + L.R + (L.N + 1) / 2 + (L.R + 63) / 64 + 1;
  const size_t pw = (size_t)per_warp * sizeof(double);
  const size_t tab = (size_t)(L.rng[3][1] - L.rng[3][0] + L.rng[3][3] - L.rng[3][2]);
  const bool stages = b.conc || b.fwd || b.rev || b.pm;
  const bool outq = qo.A != nullptr;
  const int64_t nbatch = (b.n + 31) / 32;
  bool smem_tab = tab + mixed::DW * pw <= (size_t)smem_optin;
  int nw = mixed::DW;
  if (!smem_tab) {
    nw = (int)((size_t)smem_optin / pw);
    if (nw > mixed::DW) nw = mixed::DW;
    if (nw < 1) return cudaErrorNotSupported;
  }
  const size_t bytes = (smem_tab ? tab : 0) + nw * pw;
  auto k = outq ? (smem_tab ? mixed::k_wdot_warp<false, true, true>
                            : mixed::k_wdot_warp<false, false, true>)
                : smem_tab ? (stages ? mixed::k_wdot_warp<true, true, false>
                                     : mixed::k_wdot_warp<false, true, false>)
                           : (stages ? mixed::k_wdot_warp<true, false, false>
                                     : mixed::k_wdot_warp<false, false, false>);
  cudaError_t e = set_smem_limit(k, bytes);
  if (e != cudaSuccess) return e;
  int per_sm = 1;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, nw * 32, bytes);
  if (e != cudaSuccess) return e;
  const int grid = grid_for(nbatch, nw, sm_count * (per_sm > 0 ? per_sm : 1));
  k<<<grid, nw * 32, bytes, s>>>(img, L, b, per_warp, qo);
  return cudaGetLastError();
}

cudaError_t launch_wdot_mixed(const unsigned char *img, const ImgLayout &L,
                              const Batch &b, int sm_count, int smem_optin,
                              cudaStream_t s) {
  return launch_wdot_mixed_q(img, L, b, sm_count, smem_optin, s, mixed::QOut{});
}

}  // namespace crs
