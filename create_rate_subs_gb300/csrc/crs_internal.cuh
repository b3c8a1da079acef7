// Internal declarations shared by the libcrs kernels and the host ABI.
//
// The table image (include/crs_tables.h) is staged whole or in ranges into
// shared memory with cp.async.bulk, each section 16-byte aligned;
// ImgLayout is passed by value as a kernel parameter.
#pragma once

#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/crs_eval.h"
#include "../../include/crs_tables.h"

namespace crs {

// Status word bits (device, one per mechanism handle).
enum { STATUS_STAGE_TIMEOUT = 1, STATUS_GEMM_TIMEOUT = 2 };

namespace mixed {
// Output of the mixed rates-only kernel that feeds the tensor-core
// contraction: per state s a bf16 row A[s] = [hi(q_0..q_R-1), 0.., lo(...)]
// of q * 2^-c_s (Kh columns each), c_s in escale[s].
struct QOut {
  void *A;        // __nv_bfloat16 rows
  int64_t lda;    // 2 * Kh
  int Kh;
  int *escale;
};
}  // namespace mixed

// A derived table computed on the host at load time.
struct Derived {
  int ImgLayout::*field;
  std::vector<unsigned char> bytes;
};

// Arguments of one batched evaluation (device pointers, SoA with ld).
struct Batch {
  int64_t n, ld;
  const double *T, *P, *Y;
  double *wdot, *conc, *fwd, *rev, *pm;
  int32_t *status;  // [0] flag bits, [1] non-finite wdot count
  // dynamic scheduling slot of the one-state-per-thread kernels: [0] states
  // handed out, [1] warps finished (both zero between launches); null: a
  // static grid stride
  unsigned long long *sched;
};

#ifdef __CUDACC__
// ---- dynamic state scheduling -------------------------------------------
// The one-state-per-thread kernels run one CTA per SM whose thread count is
// set by shared memory, rarely a multiple of 4 warps, so the SM's four
// sub-partitions hold unequal numbers of warps.  With a static grid stride
// every warp evaluates the same number of states and the sub-partitions
// with more warps finish last; handing out states one warp-sized chunk at a
// time from a global counter lets the faster warps take more.

// Next chunk of states for the calling warp: its first state + lane (past n
// for some lanes of the last chunk), or -1 for every lane when the batch is
// exhausted.  amask: the
// warp's lanes (taken at kernel entry, when the warp is converged).
__device__ __forceinline__ int64_t sched_next(unsigned long long *sched, int64_t n,
                                              unsigned amask, int lane) {
  unsigned long long got = 0;
  if (lane == 0) got = atomicAdd(sched, (unsigned long long)__popc(amask));
  got = __shfl_sync(amask, got, 0);
  return got >= (unsigned long long)n ? -1 : (int64_t)got + lane;
}

// Called once by every warp of the launch when it is done (also on early
// exits): the last one puts the slot back to zero for the next launch that
// draws it.  Counters only; no wait.
__device__ __forceinline__ void sched_done(unsigned long long *sched, unsigned amask, int lane) {
  if (!sched) return;
  __syncwarp(amask);
  if (lane == 0) {
    const unsigned long long warps =
        (unsigned long long)gridDim.x * ((blockDim.x + 31) / 32);
    __threadfence();
    if (atomicAdd(sched + 1, 1ULL) == warps - 1) {
      atomicExch(sched, 0ULL);
      atomicExch(sched + 1, 0ULL);
    }
  }
}

// ---- shared-memory staging with cp.async.bulk + mbarrier ---------------
// Every wait is bounded: on expiry the CTA records STATUS_STAGE_TIMEOUT and
// the caller skips its work.
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Stage `bytes` (multiple of 16, both pointers 16-byte aligned) from global
// to shared memory, followed by `bytes2` from `gsrc2` when given.  Must be
// called by all threads of the CTA.  Returns false (for every thread) when
// the copies did not complete in time.
__device__ inline bool stage_to_smem(void *sdst, const void *gsrc, int bytes,
                                     uint64_t *bar, int32_t *status,
                                     const void *gsrc2 = nullptr,
                                     int bytes2 = 0) {
  const uint32_t b = smem_u32(bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile(
        "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b),
        "r"(bytes + bytes2)
        : "memory");
    const int CH = 32768;
    for (int part = 0; part < 2; ++part) {
      const char *src = static_cast<const char *>(part ? gsrc2 : gsrc);
      char *dst = static_cast<char *>(sdst) + (part ? bytes : 0);
      const int nbytes = part ? bytes2 : bytes;
      for (int off = 0; off < nbytes; off += CH) {
        int sz = nbytes - off < CH ? nbytes - off : CH;
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
            "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst + off)),
            "l"(src + off), "r"(sz), "r"(b)
            : "memory");
      }
    }
  }
  bool done = false;
  for (int it = 0; it < (1 << 22); ++it) {
    if (mbar_try_wait(b, 0)) {
      done = true;
      break;
    }
  }
  // every thread must agree before anyone leaves
  int all = __syncthreads_and(done ? 1 : 0);
  if (!all) {
    // give up, but not while the copies may still be writing this CTA's
    // shared memory: wait for them once more (bounded, 16x longer)
    if (threadIdx.x == 0 && status) atomicOr(&status[0], STATUS_STAGE_TIMEOUT);
    for (int it = 0; it < (1 << 26); ++it)
      if (mbar_try_wait(b, 0)) break;
    __syncthreads();
  }
  return all != 0;
}

// Stage ranges r of the image into shared memory and return the view.
__device__ inline bool stage_ranges(unsigned char *smem,
                                    const unsigned char *img,
                                    const ImgLayout &L, int r, uint64_t *bar,
                                    int32_t *status, Tab &t, int &nbytes) {
  const int *g = L.rng[r];
  nbytes = (g[1] - g[0]) + (g[3] - g[2]);
  if (!stage_to_smem(smem, img + g[0], g[1] - g[0], bar, status, img + g[2],
                     g[3] - g[2]))
    return false;
  t = make_tab2(smem, img, L, g[0], g[1], g[2], g[3]);
  return true;
}

#endif

// Thermo utilities and the ODE right-hand side (crs_dydt.cu).
// which: 0 h, 1 u, 2 cv, 3 cp (per species, [N][ld]).
cudaError_t launch_thermo(const unsigned char *img, const ImgLayout &L, int which, int64_t n,
                          const double *T, int64_t ld, double *out, int sm_count,
                          cudaStream_t s);
// eval_conc_rho over n states; any output may be NULL.
cudaError_t launch_conc_rho(const unsigned char *img, const ImgLayout &L, int64_t n,
                            const double *T, const double *rho, const double *Y, int64_t ld,
                            double *y_N, double *mw_avg, double *pres, double *conc,
                            int sm_count, cudaStream_t s);
// dy from y = [T; Y_0..Y_{N-2}] ([N][ld]) and wdot W ([N][ld]): the energy
// equation and dY/dt; conv = 1: p_or_rho is the density, else the pressure.
cudaError_t launch_dydt_finish(const unsigned char *img, const ImgLayout &L, int conv,
                               int64_t n, const double *y, int64_t ld, const double *p_or_rho,
                               const double *W, double *dy, int sm_count, cudaStream_t s);

// The PLOG / Chebyshev forward rate constant in the emitted order, shared
// by every kernel (these reactions are rare; FP64 in every mode).
using ref::pdep_kf;

#ifdef __CUDACC__
// Exponent of the equilibrium constant of reversible reaction j (with ln
// of its prefactor) from the reaction's own polynomial in T, summed over
// its T_common groups (rate_subs.py:592-655 forms these coefficients):
// c0 + c1 ln T + T (c2 + T (c3 + T (c4 + c5 T))) - c6 / T, in FP64.  Needs
// no per-state column.  KcPoly1: one group per reaction (kc_poly), the
// prefactor folded into c0 and the T <= T_common test made on the positive
// doubles' bit patterns as integers, so that only the polynomial's six
// FMAs use the FP64 pipe and the code has no branch.
struct KcPoly1 {
  double T, logT, invT;
  long long Tbits;
  __device__ __forceinline__ double operator()(const Tab &t, int, int j) const {
    const double *p = t.kc_poly + 16 * j;
    const double *c = (Tbits <= __double_as_longlong(p[0])) ? p + 2 : p + 9;
    double h = fma(fma(fma(c[5], T, c[4]), T, c[3]), T, c[2]);
    h = fma(h, T, c[0]);
    h = fma(c[1], logT, h);
    return fma(-c[6], invT, h);
  }
};

// Several T_common groups in a reaction: sum the groups' polynomials.
struct KcPolyG {
  double T, logT, invT;
  __device__ __forceinline__ double operator()(const Tab &t, int, int j) const {
    double g = t.kc_lpref[j];
    for (int q = t.kc_ptr[j]; q < t.kc_ptr[j + 1]; ++q) {
      const double *c = (T <= t.kc_tmid[q]) ? t.kc_lo + 7 * q : t.kc_hi + 7 * q;
      double h = fma(fma(fma(c[5], T, c[4]), T, c[3]), T, c[2]);
      h = fma(h, T, c[0]);
      h = fma(c[1], logT, h);
      g += fma(-c[6], invT, h);
    }
    return g;
  }
};

#endif

// Sets the text returned by crs_last_error() and returns code.
int report(int code, const char *msg);

#ifdef __CUDACC__
// Raise kernel k's dynamic shared-memory limit to `bytes`.  Every launcher
// returns this error instead of launching when the limit was not applied.
template <class K>
inline cudaError_t set_smem_limit(K k, size_t bytes) {
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}
#endif

}  // namespace crs
