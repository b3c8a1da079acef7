// State tiles of the two-pass path (crs_large.cu, crs_fast.cu): a CTA
// holds 32 states (lane = state) and its warps split the reactions; every
// net rate goes to HBM, q[r][state], for the species sums or the
// contraction that follow.
#pragma once

#include "crs_internal.cuh"

namespace crs {
namespace tile {

// Per-chunk outputs of a rates-tile kernel.
struct RatesOut {
  double *q;    // [R][ldq]: net rate of reaction r for chunk state i
  int64_t ldq;
  int *escale;  // [n] or NULL: scale exponent c_i (mean binary exponent of the nonzero rates)
};

// Sink of a rates-tile kernel: the lane's net rates to HBM, and the running
// sum / count of their binary exponents (integer work on the bit pattern).
struct QSink {
  double *q;  // this lane's column
  int64_t ldq;
  bool valid;
  int &esum, &ecnt;
  __device__ __forceinline__ void put(int r, double v) const {
    if (valid) q[(int64_t)r * ldq] = v;
    const int hi = __double2hiint(v);
    const int e = (hi >> 20) & 0x7ff;
    if (e != 0x7ff && ((hi & 0x7fffffff) | __double2loint(v)) != 0) {
      esum += e - 1023;
      ++ecnt;
    }
  }
  template <int NNU>
  __device__ __forceinline__ void block(const Tab &, const int *rr, int cnt,
                                        const double (&net)[4]) const {
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (u < cnt) put(rr[u], net[u]);
  }
  __device__ __forceinline__ void one(const Tab &, int r, double net) const { put(r, net); }
};

// Next tile of the launch for the calling CTA (all threads), from the
// launch's counter pair sched ([0] tiles handed out, [1] CTAs finished).
__device__ __forceinline__ int64_t next_tile(unsigned long long *sched, int64_t *s_tile) {
  if (threadIdx.x == 0) *s_tile = (int64_t)atomicAdd(sched, 1ULL);
  __syncthreads();
  return *s_tile;
}

// Called by every CTA once, after its last tile: the launch's last CTA puts
// the counter pair back to zero for the next launch that draws it.
__device__ __forceinline__ void tiles_done(unsigned long long *sched) {
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(sched + 1, 1ULL) == (unsigned long long)gridDim.x - 1) {
      atomicExch(sched, 0ULL);
      atomicExch(sched + 1, 0ULL);
    }
  }
}

// Scale exponent of state (lane) from the warps' partial exponent sums and
// counts: the nearest integer to sum / count, by integer arithmetic.
__device__ __forceinline__ int scale_exponent(int es, int ec) {
  if (!ec) return 0;
  const int a = es >= 0 ? es : -es;
  const int c = (2 * a + ec) / (2 * ec);
  return es < 0 ? -c : c;
}

// The tile's per-state sums (lane = state, ic its column): warp 0 forms
// y_N = 1 - the sum of the first N-1 mass fractions in the reference's
// left-to-right order (rate_subs.py:1312-1320) into s_yN; warp 1 the sum of
// y_k / W_k over the first N-1 species and, once y_N is known, the density
// P / (that sum + y_N / W_N) * scale into s_rho.  The two dependent FP64
// chains (N-2 additions, N-1 FMAs) run side by side on two warps, with the
// operations and their order of one warp doing both; the two warps meet at
// named barrier 1, and the caller's __syncthreads publishes the results
// to the other warps.  Needs a CTA of two or more warps.
__device__ __forceinline__ void state_sums(const Tab &t, const Batch &b, int64_t ic, int warp,
                                           int lane, double P, double scale, double *s_yN,
                                           double *s_rho) {
  const int N = t.N;
  if (warp == 0) {
    double ys = N > 1 ? b.Y[ic] : 0.0;
    for (int k = 1; k < N - 1; ++k) ys += b.Y[(int64_t)k * b.ld + ic];
    s_yN[lane] = 1.0 - ys;
    asm volatile("bar.sync 1, 64;" ::: "memory");
  } else if (warp == 1) {
    double mwi = 0.0;
    for (int k = 0; k < N - 1; ++k) mwi = fma(b.Y[(int64_t)k * b.ld + ic], t.inv_mw[k], mwi);
    asm volatile("bar.sync 1, 64;" ::: "memory");
    mwi = fma(s_yN[lane], t.inv_mw[N - 1], mwi);
    s_rho[lane] = P / mwi * scale;
  }
}

}  // namespace tile
}  // namespace crs
