// Internal layout shared by the libcrs kernels and the host ABI.
//
// A mechanism lives on the device as one contiguous "table image": every
// table of create_rate_subs_gb300/tables.py, each section 16-byte aligned,
// so that one CTA can stage the whole image into shared memory with
// cp.async.bulk.  ImgLayout carries the byte offsets (it is passed by value
// as a kernel parameter).
#pragma once

#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

namespace crs {

enum { RATE_CONST = 0, RATE_EXP = 1, RATE_NEGEXP = 2, RATE_POW = 3, RATE_PLOG = 4,
       RATE_CHEB = 5 };
constexpr int CHEB_MAX = 16;  // most Chebyshev temperature terms (checked at load)
enum { PM_THD = 0, PM_FALL_LOW = 1, PM_FALL_HIGH = 2 };
enum { FORM_LINDEMANN = 0, FORM_TROE = 1, FORM_SRI = 2 };

// Status word bits (device, one per mechanism handle).
enum { STATUS_STAGE_TIMEOUT = 1, STATUS_GEMM_TIMEOUT = 2 };

struct ImgLayout {
  int N, R, NREV, NPM, NRATE, NKC;
  int bytes;  // image size, multiple of 16
  // Byte ranges [lo, hi) of the image that each fast kernel stages into
  // shared memory (two ranges per kernel, copied back to back); sections
  // outside them are read from global memory through L1.
  //   [0] FP64 one state per thread   [1] FP64 one state per warp
  //   [2] mixed one state per thread, Kc polynomials read through L1
  //   [3] mixed one state per warp
  //   [4] mixed one state per thread, Kc polynomials in shared memory
  int rng[5][4];
  // derived f64 sections (fast kernels): per rate row (logA, b, -Ta); per
  // reversible reaction log(Kc prefactor); per pres_mod entry the Troe and
  // SRI constants in multiply form; per species the 2x7 Gibbs
  // coefficients; the 256-entry 2^(j/256) table of the exponential.
  int rate_x, kc_lpref, troe_x, sri_x, sp_gibbs, exptab;
  // derived f32 sections (mixed kernel): per rate row ln|A|, b, -Ta as
  // float-float pairs and sign(A); 1/mw; Troe and SRI constants (exponent
  // factors as float-float pairs); efficiencies minus one.
  int rate_ff, inv_mw_f, troe_ff, sri_ff, eff_f;
  // derived f64 section (mixed, one state per thread): per reversible
  // reaction 16 doubles [T_common, 0, lo c0..c6, hi c0..c6] of its Kc
  // exponent polynomial with ln(prefactor) folded into c0; built when every
  // reaction has a single T_common group (kc_single = 1)
  int kc_poly, kc_single;
  // derived sections (mixed, one state per thread): the net-nu species as
  // int16 and each nu as the high word of its double (nu_hi_exact = 1 when
  // every nu's low word is zero, i.e. the pair is exact)
  int nu_sp16, nu_hi, nu_hi_exact;
  // derived f64 section (thermo utilities): per species 24 doubles
  // [RU/mw, mw, T_common, 0, lo: a0..a5, a1/2, a2/3, a3/4, a4/5, hi: same]
  int sp_thermo;
  // derived i32 sections: reaction processing order, start of each shape
  // group in it (crs_shapes.cuh), expanded reactant / product factors
  int perm, seg, rfac, pfac;
  // warp-per-state kernels: reaction order (dperm), species-major net-nu
  // CSR in reaction order (spc_ptr/spc_r/spc_nu), species per lane
  // (lane_ptr/lane_sp)
  int dperm, spc_ptr, spc_r, spc_nu, lane_ptr, lane_sp;
  // f64 sections
  int inv_mw, rate_par, rx_nu, px_nu, kc_tmid, kc_lo, kc_hi, kc_pref,
      pm_eff_val, pm_troe, pm_sri, nu_val, sp_tmid, sp_lo, sp_hi, kc_dnu, sp_mw;
  // PLOG and Chebyshev rate forms: per rate row an index into their tables
  // (rate_aux), PLOG points (printed pressure, ln P, ln-P spacing, rate row)
  // and Chebyshev coefficient blocks with their reduced-T/P constants
  int rate_aux, plog_ptr, plog_row, plog_p, plog_lp, plog_dlp, cheb_ptr, cheb_nt, cheb_np,
      cheb_par, cheb_tp;
  // i32 sections
  int rate_kind, rate_npow, rx_ptr, rx_sp, rx_nint, px_ptr, px_sp, px_nint,
      rev_idx, kc_ptr, pm_idx, pm_kind, pm_form, pm_sp, pm_eff_ptr,
      pm_eff_sp, pm_k0, pm_kinf, pm_troe_t2, pm_sri_de, nu_ptr, nu_sp;
};

// Typed view of an image (in shared or global memory).
struct Tab {
  const int32_t *perm, *seg;
  const int16_t *rfac, *pfac;
  const int32_t *dperm, *spc_ptr, *spc_r, *lane_ptr, *lane_sp;
  const double *spc_nu;
  const float *rate_ff, *inv_mw_f, *troe_ff, *sri_ff, *eff_f;
  const double *rate_x, *kc_lpref, *troe_x, *sri_x, *sp_gibbs, *exptab, *kc_poly, *sp_thermo;
  int kc_single;
  const int16_t *nu_sp16;
  const int32_t *nu_hi;
  const double *inv_mw, *rate_par, *rx_nu, *px_nu, *kc_tmid, *kc_lo, *kc_hi,
      *kc_pref, *pm_eff_val, *pm_troe, *pm_sri, *nu_val, *sp_tmid, *sp_lo,
      *sp_hi, *kc_dnu, *sp_mw;
  const int32_t *rate_aux, *plog_ptr, *plog_row, *cheb_ptr, *cheb_nt, *cheb_np;
  const double *plog_p, *plog_lp, *plog_dlp, *cheb_par, *cheb_tp;
  const int32_t *rate_kind, *rate_npow, *rx_ptr, *rx_sp, *rx_nint, *px_ptr,
      *px_sp, *px_nint, *rev_idx, *kc_ptr, *pm_idx, *pm_kind, *pm_form,
      *pm_sp, *pm_eff_ptr, *pm_eff_sp, *pm_k0, *pm_kinf, *pm_troe_t2,
      *pm_sri_de, *nu_ptr, *nu_sp;
  int N, R, NREV, NPM;
};

// View of an image whose byte ranges [lo, hi) and [lo2, hi2) have been
// copied back to back to `near` (shared memory); every other section is
// read at `far` (global memory).
__host__ __device__ inline Tab make_tab2(const unsigned char *near,
                                         const unsigned char *far,
                                         const ImgLayout &L, int lo, int hi,
                                         int lo2 = 0, int hi2 = 0) {
  Tab t;
#define CRS_P(x)                                                      \
  ((L.x >= lo && L.x < hi)     ? near + (L.x - lo)                    \
   : (L.x >= lo2 && L.x < hi2) ? near + (hi - lo) + (L.x - lo2)       \
                               : far + L.x)
#define CRS_F(x) t.x = reinterpret_cast<const double *>(CRS_P(x))
#define CRS_S(x) t.x = reinterpret_cast<const float *>(CRS_P(x))
#define CRS_I(x) t.x = reinterpret_cast<const int32_t *>(CRS_P(x))
  CRS_F(rate_x); CRS_F(kc_lpref); CRS_F(troe_x); CRS_F(sri_x); CRS_F(sp_gibbs);
  CRS_F(exptab); CRS_F(kc_poly); CRS_F(sp_thermo);
  CRS_I(perm); CRS_I(seg);
  t.rfac = reinterpret_cast<const int16_t *>(CRS_P(rfac));
  t.pfac = reinterpret_cast<const int16_t *>(CRS_P(pfac));
  t.nu_sp16 = reinterpret_cast<const int16_t *>(CRS_P(nu_sp16));
  CRS_I(nu_hi);
  CRS_I(dperm); CRS_I(spc_ptr); CRS_I(spc_r); CRS_I(lane_ptr); CRS_I(lane_sp);
  CRS_F(spc_nu);
  CRS_S(rate_ff); CRS_S(inv_mw_f); CRS_S(troe_ff); CRS_S(sri_ff); CRS_S(eff_f);
  CRS_F(inv_mw); CRS_F(rate_par); CRS_F(rx_nu); CRS_F(px_nu); CRS_F(kc_tmid);
  CRS_F(kc_lo); CRS_F(kc_hi); CRS_F(kc_pref); CRS_F(pm_eff_val);
  CRS_F(pm_troe); CRS_F(pm_sri); CRS_F(nu_val); CRS_F(sp_tmid); CRS_F(sp_lo);
  CRS_F(sp_hi); CRS_F(kc_dnu); CRS_F(sp_mw);
  CRS_I(rate_aux); CRS_I(plog_ptr); CRS_I(plog_row); CRS_I(cheb_ptr); CRS_I(cheb_nt);
  CRS_I(cheb_np); CRS_F(plog_p); CRS_F(plog_lp); CRS_F(plog_dlp); CRS_F(cheb_par);
  CRS_F(cheb_tp);
  CRS_I(rate_kind); CRS_I(rate_npow); CRS_I(rx_ptr); CRS_I(rx_sp);
  CRS_I(rx_nint); CRS_I(px_ptr); CRS_I(px_sp); CRS_I(px_nint); CRS_I(rev_idx);
  CRS_I(kc_ptr); CRS_I(pm_idx); CRS_I(pm_kind); CRS_I(pm_form); CRS_I(pm_sp);
  CRS_I(pm_eff_ptr); CRS_I(pm_eff_sp); CRS_I(pm_k0); CRS_I(pm_kinf);
  CRS_I(pm_troe_t2); CRS_I(pm_sri_de); CRS_I(nu_ptr); CRS_I(nu_sp);
#undef CRS_P
#undef CRS_F
#undef CRS_S
#undef CRS_I
  t.N = L.N; t.R = L.R; t.NREV = L.NREV; t.NPM = L.NPM;
  t.kc_single = L.kc_single;
  return t;
}

__host__ __device__ inline Tab make_tab(const unsigned char *b,
                                        const ImgLayout &L) {
  return make_tab2(b, b, L, 0, 0);
}

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

#ifdef __CUDACC__
// rxn_rate_const in the emitted form (rate_subs.py:60-135), CUDA exp.
__device__ inline double ref_rate_const(const Tab &t, int row, double T, double logT) {
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

// Forward rate constant of a PLOG row (rate_subs.py:444-485: branch
// thresholds as printed with %.4e, log-linear interpolation in ln P between
// the bracketing points) or a Chebyshev row (rate_subs.py:136-223: reduced
// temperature and pressure, the pressure dot products by the Chebyshev
// recursion, then the temperature sum, 10^kf), in the emitted order.
__device__ inline double pdep_kf(const Tab &t, int row, double T, double logT, double pres) {
  const int a = t.rate_aux[row];
  if (t.rate_kind[row] == RATE_PLOG) {
    const int e0 = t.plog_ptr[a], e1 = t.plog_ptr[a + 1];
    if (pres <= t.plog_p[e0]) return ref_rate_const(t, t.plog_row[e0], T, logT);
    for (int e = e0; e < e1 - 1; ++e)
      if ((pres > t.plog_p[e]) && (pres <= t.plog_p[e + 1])) {
        const double k1 = log(ref_rate_const(t, t.plog_row[e], T, logT));
        const double k2 = log(ref_rate_const(t, t.plog_row[e + 1], T, logT));
        return exp(k1 + (k2 - k1) * (log(pres) - t.plog_lp[e]) / t.plog_dlp[e]);
      }
    if (pres > t.plog_p[e1 - 1]) return ref_rate_const(t, t.plog_row[e1 - 1], T, logT);
    return __longlong_as_double(0x7ff8000000000000ll);  // no branch (NaN pressure)
  }
  const double *tp = t.cheb_tp + 4 * a;
  const int nt = t.cheb_nt[a], np = t.cheb_np[a];
  const double *c = t.cheb_par + t.cheb_ptr[a];  // [nt][np]
  const double Tred = ((2.0 / T) - tp[0]) / tp[1];
  const double Pred = (2.0 * log10(pres) - tp[2]) / tp[3];
  double dp[CHEB_MAX];
  for (int i = 0; i < nt; ++i) dp[i] = c[i * np] + Pred * c[i * np + 1];
  double ct0 = 1.0, ct1 = Pred;
  bool upd = true;
  for (int j = 2; j < np; ++j) {
    if (upd) {
      ct0 = 2.0 * Pred * ct1 - ct0;
      for (int i = 0; i < nt; ++i) dp[i] += c[i * np + j] * ct0;
    } else {
      ct1 = 2.0 * Pred * ct0 - ct1;
      for (int i = 0; i < nt; ++i) dp[i] += c[i * np + j] * ct1;
    }
    upd = !upd;
  }
  ct0 = 1.0;
  ct1 = Tred;
  double kf = dp[0] + Tred * dp[1];
  upd = true;
  for (int i = 2; i < nt; ++i) {
    if (upd) {
      ct0 = 2.0 * Tred * ct1 - ct0;
      kf += dp[i] * ct0;
    } else {
      ct1 = 2.0 * Tred * ct0 - ct1;
      kf += dp[i] * ct1;
    }
    upd = !upd;
  }
  return pow(10.0, kf);
}
#endif

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
