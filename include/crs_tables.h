/*
 * crs_tables.h -- the mechanism table image of libcrs (C++, host and
 * device).
 *
 * A mechanism lives as one contiguous "table image": every table that
 * create_rate_subs_gb300.tables packs (Arrhenius rows, reactant / product
 * lists, equilibrium-constant coefficients, third-body and fall-off
 * constants, NASA-7 coefficients, net stoichiometric lists) plus the
 * tables libcrs derives from them at load time, each section 16-byte
 * aligned.  ImgLayout holds the byte offset of each section; Tab is a typed
 * view of an image in host, global or shared memory.  The reference bakes
 * the same constants into its emitted code as literals (rate_subs.py:
 * 226-1391); here they are data, so that one evaluator serves any
 * mechanism.
 *
 * libcrs builds images (crs_mech_load, crs_mech_image in crs.h); the
 * per-state device functions of crs_device.cuh read the image that the
 * 'cuda' CLI target compiles into a user's program.
 */
#ifndef CRS_TABLES_H
#define CRS_TABLES_H

#include <stdint.h>

#if defined(__CUDACC__)
#define CRS_HD __host__ __device__
#else
#define CRS_HD
#endif

namespace crs {

enum { RATE_CONST = 0, RATE_EXP = 1, RATE_NEGEXP = 2, RATE_POW = 3, RATE_PLOG = 4,
       RATE_CHEB = 5 };
constexpr int CHEB_MAX = 16;  // most Chebyshev temperature terms (checked at load)
enum { PM_THD = 0, PM_FALL_LOW = 1, PM_FALL_HIGH = 2 };
enum { FORM_LINDEMANN = 0, FORM_TROE = 1, FORM_SRI = 2 };


struct ImgLayout {
  int N, R, NREV, NPM, NRATE, NKC;
  int bytes;  // image size, multiple of 16
  // Byte ranges [lo, hi) of the image that each fast kernel stages into
  // shared memory (two ranges per kernel, copied back to back); sections
  // outside them are read from global memory through L1.
  //   [0] FP64 one state per thread   [1] FP64 one state per warp
  //   [2] mixed one state per thread, Kc polynomials and rate rows read
  //       through L1
  //   [3] mixed one state per warp
  //   [4] mixed one state per thread, Kc polynomials in shared memory
  int rng[5][4];
  // derived f64 sections (fast kernels): per rate row (logA, b, -Ta); per
  // reversible reaction log(Kc prefactor); per pres_mod entry the Troe and
  // SRI constants in multiply form; per species the 2x7 Gibbs
  // coefficients; the 256-entry 2^(j/256) table of the exponential; the
  // 129 pairs (1/F, log F), F = 1 + j/128, of the logarithm.
  int rate_x, kc_lpref, troe_x, sri_x, sp_gibbs, exptab, logtab;
  // derived f32 sections (mixed kernel): per rate row ln|A|, b, -Ta as
  // float-float pairs and sign(A); 1/mw; Troe and SRI constants (exponent
  // factors as float-float pairs); efficiencies minus one.
  int rate_ff, inv_mw_f, troe_ff, sri_ff, eff_f;
  // derived f64 section (mixed, one state per thread): per reversible
  // reaction 16 doubles [T_common, 0, lo c0..c6, hi c0..c6] of its Kc
  // exponent polynomial with ln(prefactor) folded into c0; built when every
  // reaction has a single T_common group (kc_single = 1)
  int kc_poly, kc_single;
  // derived f32 section (mixed kernels): the same polynomials as float-
  // float pairs, per reversible reaction two 16-float blocks (lo, hi), each
  // [c0..c5 as (h, l), -c6 as (h, l), T_common as a double]; built with
  // kc_poly
  int kc_mix;
  // derived sections (mixed, one state per thread): the net-nu species as
  // int16 and each nu as the top 16 bits of its double (nu_hi_exact = 1 when
  // every nu's other 48 bits are zero, i.e. the pair is exact)
  int nu_sp16, nu_hi, nu_hi_exact;
  // 1 + the highest species index with a nonzero net nu: species at or
  // above it (bath gases listed last) never accumulate a rate
  int nw;
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
  const float *rate_ff, *inv_mw_f, *troe_ff, *sri_ff, *eff_f, *kc_mix;
  const double *rate_x, *kc_lpref, *troe_x, *sri_x, *sp_gibbs, *exptab, *logtab, *kc_poly,
      *sp_thermo;
  int kc_single;
  const int16_t *nu_sp16;
  const uint16_t *nu_hi;
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
CRS_HD inline Tab make_tab2(const unsigned char *near,
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
  CRS_F(exptab); CRS_F(logtab); CRS_F(kc_poly); CRS_F(sp_thermo);
  CRS_I(perm); CRS_I(seg);
  t.rfac = reinterpret_cast<const int16_t *>(CRS_P(rfac));
  t.pfac = reinterpret_cast<const int16_t *>(CRS_P(pfac));
  t.nu_sp16 = reinterpret_cast<const int16_t *>(CRS_P(nu_sp16));
  t.nu_hi = reinterpret_cast<const uint16_t *>(CRS_P(nu_hi));
  CRS_I(dperm); CRS_I(spc_ptr); CRS_I(spc_r); CRS_I(lane_ptr); CRS_I(lane_sp);
  CRS_F(spc_nu);
  CRS_S(rate_ff); CRS_S(inv_mw_f); CRS_S(troe_ff); CRS_S(sri_ff); CRS_S(eff_f);
  CRS_S(kc_mix);
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

CRS_HD inline Tab make_tab(const unsigned char *b,
                                        const ImgLayout &L) {
  return make_tab2(b, b, L, 0, 0);
}


}  // namespace crs

#endif /* CRS_TABLES_H */
