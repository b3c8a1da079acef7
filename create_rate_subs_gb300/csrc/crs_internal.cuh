// Internal layout shared by the libcrs kernels and the host ABI.
//
// A mechanism lives on the device as one contiguous "table image": every
// table of create_rate_subs_gb300/tables.py, each section 16-byte aligned,
// so that one CTA can stage the whole image into shared memory with
// cp.async.bulk.  ImgLayout carries the byte offsets (it is passed by value
// as a kernel parameter).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace crs {

enum { RATE_CONST = 0, RATE_EXP = 1, RATE_NEGEXP = 2, RATE_POW = 3 };
enum { PM_THD = 0, PM_FALL_LOW = 1, PM_FALL_HIGH = 2 };
enum { FORM_LINDEMANN = 0, FORM_TROE = 1, FORM_SRI = 2 };

// Status word bits (device, one per mechanism handle).
enum { STATUS_STAGE_TIMEOUT = 1 };

struct ImgLayout {
  int N, R, NREV, NPM, NRATE, NKC;
  int bytes;  // image size, multiple of 16
  // f64 sections
  int inv_mw, rate_par, rx_nu, px_nu, kc_tmid, kc_lo, kc_hi, kc_pref,
      pm_eff_val, pm_troe, pm_sri, nu_val, sp_tmid, sp_lo, sp_hi, kc_dnu;
  // i32 sections
  int rate_kind, rate_npow, rx_ptr, rx_sp, rx_nint, px_ptr, px_sp, px_nint,
      rev_idx, kc_ptr, pm_idx, pm_kind, pm_form, pm_sp, pm_eff_ptr,
      pm_eff_sp, pm_k0, pm_kinf, pm_troe_t2, pm_sri_de, nu_ptr, nu_sp;
};

// Typed view of an image (in shared or global memory).
struct Tab {
  const double *inv_mw, *rate_par, *rx_nu, *px_nu, *kc_tmid, *kc_lo, *kc_hi,
      *kc_pref, *pm_eff_val, *pm_troe, *pm_sri, *nu_val, *sp_tmid, *sp_lo,
      *sp_hi, *kc_dnu;
  const int32_t *rate_kind, *rate_npow, *rx_ptr, *rx_sp, *rx_nint, *px_ptr,
      *px_sp, *px_nint, *rev_idx, *kc_ptr, *pm_idx, *pm_kind, *pm_form,
      *pm_sp, *pm_eff_ptr, *pm_eff_sp, *pm_k0, *pm_kinf, *pm_troe_t2,
      *pm_sri_de, *nu_ptr, *nu_sp;
  int N, R, NREV, NPM;
};

__host__ __device__ inline Tab make_tab(const unsigned char *b,
                                        const ImgLayout &L) {
  Tab t;
#define CRS_F(x) t.x = reinterpret_cast<const double *>(b + L.x)
#define CRS_I(x) t.x = reinterpret_cast<const int32_t *>(b + L.x)
  CRS_F(inv_mw); CRS_F(rate_par); CRS_F(rx_nu); CRS_F(px_nu); CRS_F(kc_tmid);
  CRS_F(kc_lo); CRS_F(kc_hi); CRS_F(kc_pref); CRS_F(pm_eff_val);
  CRS_F(pm_troe); CRS_F(pm_sri); CRS_F(nu_val); CRS_F(sp_tmid); CRS_F(sp_lo);
  CRS_F(sp_hi); CRS_F(kc_dnu);
  CRS_I(rate_kind); CRS_I(rate_npow); CRS_I(rx_ptr); CRS_I(rx_sp);
  CRS_I(rx_nint); CRS_I(px_ptr); CRS_I(px_sp); CRS_I(px_nint); CRS_I(rev_idx);
  CRS_I(kc_ptr); CRS_I(pm_idx); CRS_I(pm_kind); CRS_I(pm_form); CRS_I(pm_sp);
  CRS_I(pm_eff_ptr); CRS_I(pm_eff_sp); CRS_I(pm_k0); CRS_I(pm_kinf);
  CRS_I(pm_troe_t2); CRS_I(pm_sri_de); CRS_I(nu_ptr); CRS_I(nu_sp);
#undef CRS_F
#undef CRS_I
  t.N = L.N; t.R = L.R; t.NREV = L.NREV; t.NPM = L.NPM;
  return t;
}

// Arguments of one batched evaluation (device pointers, SoA with ld).
struct Batch {
  int64_t n, ld;
  const double *T, *P, *Y;
  double *wdot, *conc, *fwd, *rev, *pm;
  int32_t *status;  // [0] flag bits, [1] non-finite wdot count
};

#ifdef __CUDACC__
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
// to shared memory.  Must be called by all threads of the CTA.  Returns
// false (for every thread) when the copy did not complete in time.
__device__ inline bool stage_to_smem(void *sdst, const void *gsrc, int bytes,
                                     uint64_t *bar, int32_t *status) {
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
        "r"(bytes)
        : "memory");
    const int CH = 32768;
    for (int off = 0; off < bytes; off += CH) {
      int sz = bytes - off < CH ? bytes - off : CH;
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
          "[%0], [%1], %2, [%3];" ::"r"(smem_u32(static_cast<char *>(sdst) + off)),
          "l"(static_cast<const char *>(gsrc) + off), "r"(sz), "r"(b)
          : "memory");
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
  if (!all && threadIdx.x == 0 && status) atomicOr(&status[0], STATUS_STAGE_TIMEOUT);
  return all != 0;
}
#endif

}  // namespace crs
