// libcrs C ABI: mechanism loading, argument checking, kernel dispatch and
// the reference's four per-state entry points.  See include/crs.h.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "../../include/crs.h"
#include "crs_internal.cuh"

namespace crs {
cudaError_t launch_wdot_strict(const unsigned char *img, const ImgLayout &L,
                               const Batch &b, int sm_count, int smem_optin,
                               cudaStream_t s);
cudaError_t launch_wdot_fp64(const unsigned char *img, const ImgLayout &L,
                             const Batch &b, int sm_count, int smem_optin,
                             cudaStream_t s);
cudaError_t launch_wdot_mixed(const unsigned char *img, const ImgLayout &L,
                              const Batch &b, int sm_count, int smem_optin,
                              cudaStream_t s);
cudaError_t launch_wdot_fp64_tps(const unsigned char *img, const ImgLayout &L,
                                 const Batch &b, int sm_count, int smem_optin,
                                 cudaStream_t s);
cudaError_t launch_wdot_mixed_tps(const unsigned char *img, const ImgLayout &L,
                                  const Batch &b, int sm_count, int smem_optin,
                                  cudaStream_t s);
cudaError_t launch_stage(int which, const unsigned char *img,
                         const ImgLayout &L, const Batch &b, double *y_N,
                         double *mw, double *rho, int sm_count, cudaStream_t s);
cudaError_t launch_wdot_mixed_q(const unsigned char *img, const ImgLayout &L,
                                const Batch &b, int sm_count, int smem_optin,
                                cudaStream_t s, const mixed::QOut &qo);
cudaError_t launch_gemm_wdot(const void *A, const void *B, int64_t M_pad, int64_t N_pad,
                             int64_t K, int block_n, double *out, int64_t ld, int m_valid,
                             int n_valid, const int *escale, int32_t *status,
                             cudaStream_t s);
// Mixed precision for large mechanisms in two passes over HBM (crs_large.cu).
size_t large_rates_smem(const ImgLayout &L);
cudaError_t launch_rates_tile(const unsigned char *img, const ImgLayout &L, const Batch &b,
                              int sm_count, int smem_optin, cudaStream_t s, double *q,
                              int64_t ldq, int *escale);
cudaError_t launch_rates_tile64(const unsigned char *img, const ImgLayout &L, const Batch &b,
                                int sm_count, int smem_optin, cudaStream_t s, double *q,
                                int64_t ldq);
cudaError_t launch_spec_sum(const unsigned char *img, const ImgLayout &L, const double *q,
                            int64_t ldq, int64_t n, const int *escale, const unsigned *outflag,
                            double *wdot, int64_t ld, int32_t *status, int sm_count,
                            cudaStream_t s);
cudaError_t launch_pack_bf16(const double *q, int64_t ldq, int64_t n, int R, int Kh,
                             const int *escale, void *A, int64_t lda, unsigned *outflag,
                             int sm_count, cudaStream_t s);
// Tables the fast kernels derive from the blob's tables at load time.
bool build_fast_tables(const std::vector<unsigned char> &img,
                       const ImgLayout &L, std::vector<Derived> &extra);
// Reentrant per-state evaluation on the host (crs_host.cpp).
namespace host {
void eval_conc(const Tab &t, double T, double pres, const double *y, double *y_N,
               double *mw_avg, double *rho, double *conc);
// Lists of the branch-free host paths, built once per mechanism (NULL: the
// generic path).
struct Aux;
Aux *make_aux(const Tab &t);
void free_aux(Aux *a);
void eval_rxn_rates(const Tab &t, const Aux *a, double T, double pres, const double *C,
                    double *fwd, double *rev);
void get_rxn_pres_mod(const Tab &t, const Aux *a, double T, double pres, const double *C,
                      double *pm);
void eval_spec_rates(const Tab &t, const Aux *a, const double *fwd, const double *rev,
                     const double *pm, double *sp_rates, double *dy_N);
void eval_thermo(const Tab &t, int which, double T, double *out);
void eval_conc_rho(const Tab &t, double T, double rho, const double *y, double *y_N,
                   double *mw_avg, double *pres, double *conc);
void dydt(const Tab &t, const Aux *a, int conv, double p_or_rho, const double *y,
          double *dy);
}  // namespace host
}  // namespace crs

// Dynamic-scheduling slots per mechanism handle: the most launches of the
// one-state-per-thread kernels that may run at the same time on one handle.
constexpr unsigned SCHED_SLOTS = 256;

struct crs_mech {
  int device = 0;
  int sm_count = 0;
  int smem_optin = 0;
  crs::ImgLayout L{};
  unsigned char *d_img = nullptr;  // device table image
  int32_t *d_status = nullptr;     // [0] flags, [1] non-finite count
  // dynamic-scheduling counter pairs of the one-state-per-thread kernels;
  // each launch draws the next slot, so launches in flight at the same time
  // (several streams) use different counters
  unsigned long long *d_sched = nullptr;
  mutable std::atomic<unsigned> sched_next{0};
  std::vector<unsigned char> h_img;
  crs::Tab htab{};  // view of h_img for the per-state host functions
  crs::host::Aux *haux = nullptr;  // their branch-free lists
  // tensor-core contraction (CRS_MODE_GEMM): nu as a bf16 matrix
  // [N_pad][2*Kh] (each row nu_k, then nu_k again for the lo half), and a
  // workspace for one chunk of states (bf16 rows + per-state exponents),
  // allocated on first use and reused by later calls
  std::mutex ws_mu;
  int gemm_state = 0;  // 0 unknown, 1 ready, -1 unsupported
  int Kh = 0, N_pad = 0, block_n = 64;
  void *d_nuB = nullptr;
  void *d_ws = nullptr;
  int *d_escale = nullptr;
  unsigned *d_outflag = nullptr;  // states with terms outside the bf16 window
  int64_t ws_rows = 0;
  // two-pass mixed precision of large mechanisms (and the contraction's
  // producer): FP64 net rates of one chunk of states [R][q_rows]
  double *d_q = nullptr;
  int64_t q_rows = 0;
  // recorded after the last kernel that used the workspaces, waited on by
  // the next call's stream: calls on several streams take turns on the GPU
  cudaEvent_t ws_done = nullptr;
  bool ws_used = false;
  // crs_wdot_host: two streams and two device buffers of one chunk of
  // states each (T, P, Y, wdot), allocated on first use
  std::mutex host_mu;
  cudaStream_t hs[2] = {nullptr, nullptr};
  double *d_host = nullptr;
  int64_t host_chunk = 0;
};

void unbind(const crs_mech *m);

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(CRS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

}  // namespace

// Message for crs_last_error() from the other translation units.
int crs::report(int code, const char *msg) { return fail(code, "%s", msg); }

namespace {

struct Section {
  uint32_t dtype;
  uint64_t count, offset;
};

bool find_section(const unsigned char *b, size_t n, const char *name,
                  Section &out) {
  uint32_t nsec;
  memcpy(&nsec, b + 12, 4);
  if (16 + (size_t)nsec * 48 > n) return false;
  for (uint32_t i = 0; i < nsec; ++i) {
    const unsigned char *e = b + 16 + (size_t)i * 48;
    char nm[25];
    memcpy(nm, e, 24);
    nm[24] = 0;
    if (strcmp(nm, name) != 0) continue;
    memcpy(&out.dtype, e + 24, 4);
    memcpy(&out.count, e + 32, 8);
    memcpy(&out.offset, e + 40, 8);
    const size_t es = (out.dtype == 1 || out.dtype == 3) ? 8 : (out.dtype == 2 ? 4 : 1);
    return out.offset + out.count * es <= n;
  }
  return false;
}

// Table sections copied into the device image: name, dtype, expected count
// expressed through the dims (-1 = any).
struct Want {
  const char *name;
  int *field;
  uint32_t dtype;
};

int build_image(const unsigned char *b, size_t n, crs_mech *m) {
  if (n < 16 || memcmp(b, "CRSMECH1", 8) != 0)
    return fail(CRS_ERR_BLOB, "not a mechanism blob (bad magic)");
  uint32_t ver;
  memcpy(&ver, b + 8, 4);
  if (ver != 1) return fail(CRS_ERR_BLOB, "unsupported blob version %u", ver);
  Section s;
  if (!find_section(b, n, "dims", s) || s.dtype != 3 || s.count < 5)
    return fail(CRS_ERR_BLOB, "blob has no dims section");
  int64_t dims[5];
  memcpy(dims, b + s.offset, sizeof dims);
  crs::ImgLayout &L = m->L;
  L.N = (int)dims[0];
  L.R = (int)dims[1];
  L.NREV = (int)dims[2];
  L.NPM = (int)dims[3];
  L.NRATE = (int)dims[4];
  if (L.N < 2 || L.N > 32767 || L.R < 0 || L.NREV < 0 || L.NPM < 0 || L.NRATE < L.R)
    return fail(CRS_ERR_BLOB, "bad dims");
  // Sections the fast kernels read come first; the ones only the
  // reference-order kernels read (per-reaction Kc polynomials, raw NASA-7
  // coefficients) come last, so that fast kernels stage a prefix.
  Want want[] = {
      {"sp_inv_mw", &L.inv_mw, 1}, {"rate_par", &L.rate_par, 1},
      {"rx_nu", &L.rx_nu, 1}, {"px_nu", &L.px_nu, 1},
      {"kc_pref", &L.kc_pref, 1},
      {"pm_eff_val", &L.pm_eff_val, 1}, {"pm_troe", &L.pm_troe, 1},
      {"pm_sri", &L.pm_sri, 1}, {"nu_val", &L.nu_val, 1},
      {"sp_tmid", &L.sp_tmid, 1}, {"kc_dnu", &L.kc_dnu, 1},
      {"rate_kind", &L.rate_kind, 2}, {"rate_npow", &L.rate_npow, 2},
      {"rx_ptr", &L.rx_ptr, 2}, {"rx_sp", &L.rx_sp, 2},
      {"rx_nint", &L.rx_nint, 2}, {"px_ptr", &L.px_ptr, 2},
      {"px_sp", &L.px_sp, 2}, {"px_nint", &L.px_nint, 2},
      {"rev_idx", &L.rev_idx, 2}, {"kc_ptr", &L.kc_ptr, 2},
      {"pm_idx", &L.pm_idx, 2}, {"pm_kind", &L.pm_kind, 2},
      {"pm_form", &L.pm_form, 2}, {"pm_sp", &L.pm_sp, 2},
      {"pm_eff_ptr", &L.pm_eff_ptr, 2}, {"pm_eff_sp", &L.pm_eff_sp, 2},
      {"pm_k0", &L.pm_k0, 2}, {"pm_kinf", &L.pm_kinf, 2},
      {"pm_troe_t2", &L.pm_troe_t2, 2}, {"pm_sri_de", &L.pm_sri_de, 2},
      {"nu_ptr", &L.nu_ptr, 2}, {"nu_sp", &L.nu_sp, 2},
      // reference-order only
      {"kc_tmid", &L.kc_tmid, 1}, {"kc_lo", &L.kc_lo, 1},
      {"kc_hi", &L.kc_hi, 1}, {"sp_lo", &L.sp_lo, 1},
      {"sp_hi", &L.sp_hi, 1}, {"sp_mw", &L.sp_mw, 1},
      {"rate_aux", &L.rate_aux, 2}, {"plog_ptr", &L.plog_ptr, 2},
      {"plog_row", &L.plog_row, 2}, {"plog_p", &L.plog_p, 1},
      {"plog_lp", &L.plog_lp, 1}, {"plog_dlp", &L.plog_dlp, 1},
      {"cheb_ptr", &L.cheb_ptr, 2}, {"cheb_nt", &L.cheb_nt, 2},
      {"cheb_np", &L.cheb_np, 2}, {"cheb_par", &L.cheb_par, 1},
      {"cheb_tp", &L.cheb_tp, 1},
  };
  std::vector<unsigned char> &img = m->h_img;
  img.clear();
  std::vector<std::pair<const char *, Section>> got;
  for (auto &w : want) {
    if (!find_section(b, n, w.name, s))
      return fail(CRS_ERR_BLOB, "blob lacks section %s", w.name);
    if (s.dtype != w.dtype)
      return fail(CRS_ERR_BLOB, "section %s has the wrong type", w.name);
    const size_t es = w.dtype == 1 ? 8 : 4;
    size_t off = (img.size() + 15) / 16 * 16;
    img.resize(off + s.count * es + 16);  // +16: keeps empty sections valid
    memcpy(img.data() + off, b + s.offset, s.count * es);
    *w.field = (int)off;
    got.emplace_back(w.name, s);
  }
  img.resize((img.size() + 15) / 16 * 16);
  // Index sanity: every index stored in the tables must be in range, so
  // that no kernel can read outside its tables or state columns.
  const crs::Tab t = crs::make_tab(img.data(), L);
  auto cnt = [&](const char *name) -> int64_t {
    for (auto &g : got)
      if (strcmp(g.first, name) == 0) return (int64_t)g.second.count;
    return -1;
  };
  auto ptr_ok = [&](const int32_t *p, int len, int64_t total) {
    if (p[0] != 0) return false;
    for (int i = 0; i < len; ++i)
      if (p[i + 1] < p[i]) return false;
    return p[len] == total;
  };
  if (cnt("rate_par") != 4LL * L.NRATE || cnt("rate_kind") != L.NRATE ||
      cnt("rx_ptr") != L.R + 1 || cnt("px_ptr") != L.R + 1 ||
      cnt("nu_ptr") != L.R + 1 || cnt("rev_idx") != L.R ||
      cnt("pm_idx") != L.R || cnt("kc_ptr") != L.NREV + 1 ||
      cnt("pm_eff_ptr") != L.NPM + 1 || cnt("pm_kind") != L.NPM ||
      cnt("sp_inv_mw") != L.N || cnt("sp_lo") != 7LL * L.N ||
      cnt("sp_hi") != 7LL * L.N || cnt("sp_mw") != L.N || cnt("sp_tmid") != L.N)
    return fail(CRS_ERR_BLOB, "table sizes disagree with dims");
  if (!ptr_ok(t.rx_ptr, L.R, cnt("rx_sp")) || !ptr_ok(t.px_ptr, L.R, cnt("px_sp")) ||
      !ptr_ok(t.nu_ptr, L.R, cnt("nu_sp")) ||
      !ptr_ok(t.kc_ptr, L.NREV, cnt("kc_tmid")) ||
      !ptr_ok(t.pm_eff_ptr, L.NPM, cnt("pm_eff_sp")))
    return fail(CRS_ERR_BLOB, "bad CSR pointers");
  L.NKC = (int)cnt("kc_tmid");
  auto in = [](int64_t v, int64_t lo, int64_t hi) { return v >= lo && v < hi; };
  for (int64_t e = 0; e < cnt("rx_sp"); ++e)
    if (!in(t.rx_sp[e], 0, L.N) || t.rx_nint[e] > 64) return fail(CRS_ERR_BLOB, "bad reactant");
  for (int64_t e = 0; e < cnt("px_sp"); ++e)
    if (!in(t.px_sp[e], 0, L.N) || t.px_nint[e] > 64) return fail(CRS_ERR_BLOB, "bad product");
  for (int64_t e = 0; e < cnt("nu_sp"); ++e)
    if (!in(t.nu_sp[e], 0, L.N)) return fail(CRS_ERR_BLOB, "bad nu species");
  for (int64_t e = 0; e < cnt("pm_eff_sp"); ++e)
    if (!in(t.pm_eff_sp[e], 0, L.N)) return fail(CRS_ERR_BLOB, "bad efficiency species");
  int nrev = 0, npm = 0;
  for (int r = 0; r < L.R; ++r) {
    if (t.rev_idx[r] >= 0 && t.rev_idx[r] != nrev++) return fail(CRS_ERR_BLOB, "bad rev_idx");
    if (t.pm_idx[r] >= 0 && t.pm_idx[r] != npm++) return fail(CRS_ERR_BLOB, "bad pm_idx");
    if (!in(t.rate_kind[r], 0, 6) || t.rate_npow[r] > 64) return fail(CRS_ERR_BLOB, "bad rate");
  }
  if (nrev != L.NREV || npm != L.NPM) return fail(CRS_ERR_BLOB, "rev/pm counts disagree");
  // PLOG / Chebyshev rows: indices in range, PLOG points plain Arrhenius rows
  const int64_t nplog = cnt("plog_ptr") - 1, ncheb = cnt("cheb_nt");
  if (cnt("rate_aux") != L.NRATE || nplog < 0 || cnt("cheb_ptr") != ncheb + 1 ||
      cnt("cheb_np") != ncheb || cnt("cheb_tp") != 4 * ncheb ||
      cnt("plog_row") != cnt("plog_p") || cnt("plog_lp") != cnt("plog_p") ||
      cnt("plog_dlp") != cnt("plog_p"))
    return fail(CRS_ERR_BLOB, "PLOG/Chebyshev table sizes disagree");
  if (!ptr_ok(t.plog_ptr, (int)nplog, cnt("plog_p")) || !ptr_ok(t.cheb_ptr, (int)ncheb, cnt("cheb_par")))
    return fail(CRS_ERR_BLOB, "bad PLOG/Chebyshev pointers");
  for (int64_t q = 0; q < nplog; ++q)
    if (t.plog_ptr[q + 1] - t.plog_ptr[q] < 1) return fail(CRS_ERR_BLOB, "empty PLOG entry");
  for (int64_t e = 0; e < cnt("plog_row"); ++e)
    if (!in(t.plog_row[e], 0, L.NRATE) || t.rate_kind[t.plog_row[e]] > crs::RATE_POW)
      return fail(CRS_ERR_BLOB, "bad PLOG rate row");
  for (int64_t q = 0; q < ncheb; ++q)
    if (t.cheb_nt[q] < 2 || t.cheb_nt[q] > crs::CHEB_MAX || t.cheb_np[q] < 2 ||
        (int64_t)t.cheb_nt[q] * t.cheb_np[q] != t.cheb_ptr[q + 1] - t.cheb_ptr[q])
      return fail(CRS_ERR_BLOB, "bad Chebyshev block");
  for (int r = 0; r < L.NRATE; ++r) {
    const int k = t.rate_kind[r];
    if (!in(k, 0, 6)) return fail(CRS_ERR_BLOB, "bad rate kind");
    if (k == crs::RATE_PLOG && !in(t.rate_aux[r], 0, nplog)) return fail(CRS_ERR_BLOB, "bad PLOG index");
    if (k == crs::RATE_CHEB && !in(t.rate_aux[r], 0, ncheb)) return fail(CRS_ERR_BLOB, "bad Chebyshev index");
    if ((k == crs::RATE_PLOG || k == crs::RATE_CHEB) && r >= L.R)
      return fail(CRS_ERR_BLOB, "PLOG/Chebyshev only as reaction rows");
  }
  for (int p = 0; p < L.NPM; ++p) {
    if (!in(t.pm_kind[p], 0, 3) || !in(t.pm_form[p], 0, 3) || t.pm_sp[p] >= L.N)
      return fail(CRS_ERR_BLOB, "bad pres_mod entry");
    if (t.pm_kind[p] != crs::PM_THD &&
        (!in(t.pm_k0[p], 0, L.NRATE) || !in(t.pm_kinf[p], 0, L.NRATE)))
      return fail(CRS_ERR_BLOB, "bad fall-off rate rows");
  }
  // Final image: sections in the order the kernels stage them.  [F] is
  // read only by the FP64 kernel, [S] by both fast kernels, [M] only by the
  // mixed kernel; all of them are per-reaction tables that go to shared
  // memory.  The rest (fall-off constants, raw NASA-7 data, per-reaction Kc
  // polynomials of the reference-order kernel) stays in global memory.
  std::vector<crs::Derived> derived;
  if (!crs::build_fast_tables(img, L, derived))
    return fail(CRS_ERR_BLOB, "could not derive fast tables");
  L.kc_single = 1;
  for (int j = 0; j < L.NREV; ++j) L.kc_single &= (t.kc_ptr[j + 1] - t.kc_ptr[j]) <= 1;
  L.nw = 0;
  for (int e = 0; e < t.nu_ptr[L.R]; ++e) L.nw = std::max(L.nw, (int)t.nu_sp[e] + 1);
  L.nu_hi_exact = 1;
  for (int e = 0; e < t.nu_ptr[L.R]; ++e) {
    uint64_t u;
    memcpy(&u, &t.nu_val[e], 8);
    // the double is its top 16 bits followed by zeros (small integers,
    // halves, ...): the compact nu list holds exactly those 16 bits
    L.nu_hi_exact &= (u & 0x0000ffffffffffffull) == 0;
  }
  using M = int crs::ImgLayout::*;
  std::vector<std::pair<M, std::vector<unsigned char>>> secs;
  auto raw = [&](M f, const char *name) {
    const int64_t c = cnt(name);
    size_t es = 8;
    for (auto &w : want)
      if (strcmp(w.name, name) == 0) es = w.dtype == 1 ? 8 : 4;
    const unsigned char *src = img.data() + (L.*f);
    secs.emplace_back(f, std::vector<unsigned char>(src, src + c * es));
  };
  auto der = [&](M f) {
    for (auto &d : derived)
      if (d.field == f) secs.emplace_back(f, d.bytes);
  };
  using IL = crs::ImgLayout;
  // Region order T F S2 S1 M K D (see ImgLayout::rng):
  // [T] one-state-per-thread tables
  der(&IL::perm); der(&IL::seg); der(&IL::rfac); der(&IL::pfac);
  const size_t iF = secs.size();
  // [F] FP64 only
  der(&IL::exptab); der(&IL::rate_x);
  const size_t iS = secs.size();
  // [S2] shared by the fast kernels except the mixed one-state-per-thread
  // kernel (Gibbs terms, generic reactant / product lists)
  der(&IL::sp_gibbs); raw(&IL::sp_tmid, "sp_tmid");
  raw(&IL::rate_kind, "rate_kind"); raw(&IL::rx_ptr, "rx_ptr");
  raw(&IL::rx_sp, "rx_sp"); raw(&IL::rx_nint, "rx_nint");
  raw(&IL::px_ptr, "px_ptr"); raw(&IL::px_sp, "px_sp");
  raw(&IL::px_nint, "px_nint");
  raw(&IL::nu_sp, "nu_sp"); raw(&IL::nu_val, "nu_val");
  const size_t iS1 = secs.size();
  // [S1] shared by all fast kernels
  raw(&IL::inv_mw, "sp_inv_mw");
  raw(&IL::rev_idx, "rev_idx"); raw(&IL::pm_idx, "pm_idx");
  raw(&IL::nu_ptr, "nu_ptr");
  const size_t iM = secs.size();
  // [M] mixed only (the net-nu lists in their compact form)
  der(&IL::inv_mw_f); der(&IL::nu_sp16); der(&IL::nu_hi);
  // the mixed one-state-per-thread kernel reads the rate rows (last in the
  // region) through L1: the shared memory they would take holds a third
  // of a warp more of per-thread columns (+1.7% at 53 species)
  const size_t iRF = secs.size();
  der(&IL::rate_ff);
  const size_t iK = secs.size();
  // [K] per-reaction Kc polynomials (mixed, one state per thread) and the
  // ln Kc prefactors (read through L1 by the Gibbs-column layouts)
  der(&IL::kc_poly); der(&IL::kc_lpref);
  raw(&IL::kc_ptr, "kc_ptr"); raw(&IL::kc_tmid, "kc_tmid");
  raw(&IL::kc_lo, "kc_lo"); raw(&IL::kc_hi, "kc_hi");
  const size_t iD = secs.size();
  // [D] one-state-per-warp tables
  der(&IL::dperm); der(&IL::spc_ptr); der(&IL::spc_r); der(&IL::spc_nu);
  der(&IL::lane_ptr); der(&IL::lane_sp);
  const size_t iC = secs.size();
  // cold: read from global memory
  raw(&IL::rate_npow, "rate_npow"); raw(&IL::rx_nu, "rx_nu");
  raw(&IL::px_nu, "px_nu"); raw(&IL::pm_eff_val, "pm_eff_val");
  raw(&IL::pm_kind, "pm_kind"); raw(&IL::pm_form, "pm_form");
  raw(&IL::pm_sp, "pm_sp"); raw(&IL::pm_eff_ptr, "pm_eff_ptr");
  raw(&IL::pm_eff_sp, "pm_eff_sp"); raw(&IL::pm_k0, "pm_k0");
  raw(&IL::pm_kinf, "pm_kinf"); raw(&IL::pm_troe_t2, "pm_troe_t2");
  raw(&IL::pm_sri_de, "pm_sri_de");
  der(&IL::troe_x); der(&IL::sri_x); der(&IL::troe_ff); der(&IL::sri_ff);
  der(&IL::eff_f); der(&IL::logtab);
  raw(&IL::rate_par, "rate_par"); raw(&IL::kc_pref, "kc_pref");
  raw(&IL::pm_troe, "pm_troe"); raw(&IL::pm_sri, "pm_sri");
  raw(&IL::kc_dnu, "kc_dnu"); raw(&IL::sp_lo, "sp_lo"); raw(&IL::sp_hi, "sp_hi");
  raw(&IL::sp_mw, "sp_mw"); der(&IL::sp_thermo);
  raw(&IL::rate_aux, "rate_aux"); raw(&IL::plog_ptr, "plog_ptr"); raw(&IL::plog_row, "plog_row");
  raw(&IL::plog_p, "plog_p"); raw(&IL::plog_lp, "plog_lp"); raw(&IL::plog_dlp, "plog_dlp");
  raw(&IL::cheb_ptr, "cheb_ptr"); raw(&IL::cheb_nt, "cheb_nt"); raw(&IL::cheb_np, "cheb_np");
  raw(&IL::cheb_par, "cheb_par"); raw(&IL::cheb_tp, "cheb_tp");
  // last: the mixed kernels' float-float Kc polynomials (read through L1).
  // Every other section keeps the offset it has without them, and the
  // strict kernel stages only the bytes before them (ImgLayout::kc_mix)
  der(&IL::kc_mix);
  // every blob section and every derived table must have been placed
  for (auto &w : want) {
    bool found = false;
    for (auto &sec : secs) found |= (sec.first == (M)nullptr) ? false : (&(L.*(sec.first)) == w.field);
    if (!found) return fail(CRS_ERR_BLOB, "internal: section %s not placed", w.name);
  }
  for (auto &d : derived) {
    bool found = false;
    for (auto &sec : secs) found |= sec.first == d.field;
    if (!found) return fail(CRS_ERR_BLOB, "internal: derived table not placed");
  }
  std::vector<unsigned char> out;
  crs::ImgLayout L2 = L;
  std::vector<int> starts;
  for (auto &sec : secs) {
    const size_t off = (out.size() + 15) / 16 * 16;
    out.resize(off + sec.second.size() + 16);  // +16 keeps empty sections valid
    if (!sec.second.empty()) memcpy(out.data() + off, sec.second.data(), sec.second.size());
    L2.*(sec.first) = (int)off;
    starts.push_back((int)off);
  }
  out.resize((out.size() + 15) / 16 * 16);
  L2.bytes = (int)out.size();
  starts.push_back((int)out.size());
  const int RF0 = starts[iRF];
  const int T0 = starts[0], F0 = starts[iF], S0 = starts[iS], S1 = starts[iS1],
            M0 = starts[iM], K0 = starts[iK], D0 = starts[iD], C0 = starts[iC];
  const int rng[5][4] = {{T0, M0, 0, 0},    // FP64 per thread: T F S2 S1
                         {F0, M0, D0, C0},  // FP64 per warp: F S2 S1 + D
                         {T0, F0, S1, RF0}, // mixed per thread: T + S1 M, rate rows via L1
                         {S0, K0, D0, C0},  // mixed per warp: S2 S1 M + D
                         {T0, F0, S1, D0}}; // mixed per thread: T + S1 M K
  memcpy(L2.rng, rng, sizeof rng);
  img.swap(out);
  L = L2;
  return CRS_OK;
}

bool check_device(const crs_mech *m) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev != m->device) {
    fail(CRS_ERR_ARG, "current device %d is not the mechanism's device %d",
         dev, m->device);
    return false;
  }
  return true;
}

int check_batch(const crs_mech *m, int64_t n, int64_t ld) {
  if (!m) return fail(CRS_ERR_ARG, "mechanism is NULL");
  if (!m->d_img)
    return fail(CRS_ERR_ARG, "mechanism has no device tables (loaded with crs_mech_load_host)");
  if (n < 0) return fail(CRS_ERR_ARG, "n < 0");
  if (ld < n) return fail(CRS_ERR_ARG, "ld < n");
  if (!check_device(m)) return CRS_ERR_ARG;
  return CRS_OK;
}

crs::Batch make_batch(const crs_mech *m, int64_t n, int64_t ld) {
  crs::Batch b{};
  b.n = n;
  b.ld = ld;
  b.status = m->d_status;
  b.sched = m->d_sched ? m->d_sched + 2 * (m->sched_next.fetch_add(1) % SCHED_SLOTS) : nullptr;
  return b;
}

// Chunk of states per contraction pass (workspace rows).
constexpr int64_t GEMM_CHUNK = 1 << 17;

int gemm_prepare(crs_mech *m) {
  if (m->gemm_state) return m->gemm_state > 0 ? CRS_OK : CRS_ERR_UNSUPPORTED;
  const crs::ImgLayout &L = m->L;
  const crs::Tab t = crs::make_tab(m->h_img.data(), L);
  m->Kh = (L.R + 63) / 64 * 64;
  m->block_n = L.N <= 64 ? 64 : L.N <= 128 ? 128 : L.N <= 192 ? 192 : L.N <= 256 ? 256 : 192;
  m->N_pad = (L.N + m->block_n - 1) / m->block_n * m->block_n;
  const int64_t K = 2 * (int64_t)m->Kh;
  std::vector<__nv_bfloat16> B((size_t)m->N_pad * K, __float2bfloat16(0.0f));
  for (int r = 0; r < L.R; ++r)
    for (int e = t.nu_ptr[r]; e < t.nu_ptr[r + 1]; ++e) {
      const double nu = t.nu_val[e];
      const __nv_bfloat16 v = __float2bfloat16((float)nu);
      if ((double)__bfloat162float(v) != nu) {
        m->gemm_state = -1;
        return fail(CRS_ERR_UNSUPPORTED,
                    "a stoichiometric coefficient is not exact in bf16 (reaction %d)", r);
      }
      const int k = t.nu_sp[e];
      B[(size_t)k * K + r] = v;
      B[(size_t)k * K + m->Kh + r] = v;
    }
  cudaError_t e = cudaMalloc(&m->d_nuB, B.size() * sizeof(__nv_bfloat16));
  if (e == cudaSuccess)
    e = cudaMemcpy(m->d_nuB, B.data(), B.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "gemm tables");
  m->gemm_state = 1;
  return CRS_OK;
}

// Largest chunk of states whose FP64 net rates fit in ~2 GiB (a multiple
// of 128, at most GEMM_CHUNK).
int64_t q_chunk(const crs::ImgLayout &L, int64_t n) {
  int64_t c = ((int64_t)2 << 30) / ((int64_t)8 * (L.R > 0 ? L.R : 1));
  c = std::min<int64_t>(c, GEMM_CHUNK) / 128 * 128;
  if (c < 128) c = 128;
  return std::min<int64_t>(c, (n + 127) / 128 * 128);
}

// Workspace of the two-pass paths for chunks of `rows` states (caller
// holds ws_mu); with_ws: also the contraction's bf16 rows and exponents.
int ensure_q(crs_mech *m, int64_t rows, bool with_ws) {
  cudaError_t e = cudaSuccess;
  if (m->q_rows < rows) {
    if (m->d_q) cudaFree(m->d_q);
    m->d_q = nullptr;
    m->q_rows = 0;
    e = cudaMalloc(&m->d_q, (size_t)rows * (m->L.R > 0 ? m->L.R : 1) * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(e, "rates workspace");
    m->q_rows = rows;
  }
  if (with_ws && m->ws_rows < rows) {
    if (m->d_ws) cudaFree(m->d_ws);
    if (m->d_escale) cudaFree(m->d_escale);
    if (m->d_outflag) cudaFree(m->d_outflag);
    m->d_ws = nullptr;
    m->d_escale = nullptr;
    m->d_outflag = nullptr;
    m->ws_rows = 0;
    const int64_t K = 2 * (int64_t)m->Kh;
    e = cudaMalloc(&m->d_ws, (size_t)rows * K * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc(&m->d_escale, (size_t)rows * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&m->d_outflag, (size_t)rows * sizeof(unsigned));
    if (e != cudaSuccess) return cuda_fail(e, "gemm workspace");
    m->ws_rows = rows;
  }
  if (!m->ws_done) {
    e = cudaEventCreateWithFlags(&m->ws_done, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(e, "workspace event");
  }
  return CRS_OK;
}

// Order this call's use of the workspaces after the previous call's, on
// whatever stream that ran (not while the stream is being captured into a
// graph, where the caller orders the work).
int ws_begin(crs_mech *m, cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &cs);
  if (e != cudaSuccess) return cuda_fail(e, "workspace ordering");
  if (m->ws_used && cs == cudaStreamCaptureStatusNone) {
    e = cudaStreamWaitEvent(s, m->ws_done, 0);
    if (e != cudaSuccess) return cuda_fail(e, "workspace ordering");
  }
  return CRS_OK;
}

int ws_end(crs_mech *m, cudaStream_t s) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &cs);
  if (e == cudaSuccess && cs == cudaStreamCaptureStatusNone) {
    e = cudaEventRecord(m->ws_done, s);
    m->ws_used = e == cudaSuccess;
  }
  return e == cudaSuccess ? CRS_OK : cuda_fail(e, "workspace ordering");
}

// Shared memory of a rates tile: FP32 (mixed) or FP64 concentrations of
// 32 states.
size_t tile_smem(const crs::ImgLayout &L, bool fp64) {
  return fp64 ? (size_t)L.N * 32 * sizeof(double) : crs::large_rates_smem(L);
}

// Two passes (large mechanisms): per chunk, the state-tile rates kernel
// (mixed precision, or FP64 throughout) writes the FP64 net rates, the
// species sums read them.
int wdot_two_pass(crs_mech *m, const crs::Batch &b, cudaStream_t s, bool fp64) {
  if (tile_smem(m->L, fp64) > (size_t)m->smem_optin)
    return fail(CRS_ERR_UNSUPPORTED, "mechanism too large for the rates tile");
  std::lock_guard<std::mutex> lk(m->ws_mu);
  const int64_t rows = q_chunk(m->L, b.n);
  int rc = ensure_q(m, rows, false);
  if (rc == CRS_OK) rc = ws_begin(m, s);
  if (rc != CRS_OK) return rc;
  for (int64_t c0 = 0; c0 < b.n && rc == CRS_OK; c0 += rows) {
    const int64_t cnt = std::min<int64_t>(rows, b.n - c0);
    crs::Batch bc = b;
    bc.n = cnt;
    bc.T = b.T + c0;
    bc.P = b.P + c0;
    bc.Y = b.Y + c0;
    cudaError_t e =
        fp64 ? crs::launch_rates_tile64(m->d_img, m->L, bc, m->sm_count, m->smem_optin, s,
                                        m->d_q, rows)
             : crs::launch_rates_tile(m->d_img, m->L, bc, m->sm_count, m->smem_optin, s,
                                      m->d_q, rows, nullptr);
    if (e == cudaSuccess)
      e = crs::launch_spec_sum(m->d_img, m->L, m->d_q, rows, cnt, nullptr, nullptr,
                               b.wdot + c0, b.ld, m->d_status, m->sm_count, s);
    if (e == cudaErrorNotSupported) rc = fail(CRS_ERR_UNSUPPORTED, "rates tile not available");
    else if (e != cudaSuccess) rc = cuda_fail(e, "two-pass mixed launch");
  }
  const int rc2 = ws_end(m, s);
  return rc != CRS_OK ? rc : rc2;
}

// CRS_MODE_GEMM: per chunk, the FP64 net rates (state tiles), their bf16
// hi + lo rows scaled per state, the terms outside the bf16 window summed
// in FP64 into wdot, and the contraction GEMM adding the rest.
int wdot_gemm(crs_mech *m, const crs::Batch &b, cudaStream_t s) {
  if ((size_t)crs::large_rates_smem(m->L) > (size_t)m->smem_optin)
    return fail(CRS_ERR_UNSUPPORTED, "mechanism too large for the rates tile");
  std::lock_guard<std::mutex> lk(m->ws_mu);
  int rc = gemm_prepare(m);
  if (rc != CRS_OK) return rc;
  const int64_t K = 2 * (int64_t)m->Kh;
  const int64_t rows = q_chunk(m->L, b.n);
  rc = ensure_q(m, rows, true);
  if (rc == CRS_OK) rc = ws_begin(m, s);
  if (rc != CRS_OK) return rc;
  for (int64_t c0 = 0; c0 < b.n && rc == CRS_OK; c0 += rows) {
    const int64_t cnt = std::min<int64_t>(rows, b.n - c0);
    crs::Batch bc = b;
    bc.n = cnt;
    bc.T = b.T + c0;
    bc.P = b.P + c0;
    bc.Y = b.Y + c0;
    bc.wdot = b.wdot + c0;
    cudaError_t e = crs::launch_rates_tile(m->d_img, m->L, bc, m->sm_count, m->smem_optin, s,
                                           m->d_q, rows, m->d_escale);
    if (e == cudaSuccess)
      e = crs::launch_pack_bf16(m->d_q, rows, cnt, m->L.R, m->Kh, m->d_escale, m->d_ws, K,
                                m->d_outflag, m->sm_count, s);
    if (e == cudaSuccess)
      e = crs::launch_spec_sum(m->d_img, m->L, m->d_q, rows, cnt, m->d_escale, m->d_outflag,
                               bc.wdot, b.ld, m->d_status, m->sm_count, s);
    const int64_t M_pad = (cnt + 127) / 128 * 128;
    if (e == cudaSuccess)
      e = crs::launch_gemm_wdot(m->d_ws, m->d_nuB, M_pad, m->N_pad, K, m->block_n, bc.wdot,
                                b.ld, (int)cnt, m->L.N, m->d_escale, m->d_status, s);
    if (e == cudaErrorNotSupported) rc = fail(CRS_ERR_UNSUPPORTED, "rates tile not available");
    else if (e != cudaSuccess) rc = cuda_fail(e, "gemm launch");
  }
  const int rc2 = ws_end(m, s);
  return rc != CRS_OK ? rc : rc2;
}

}  // namespace

namespace {
// Launch the kernel of `mode` on one batch (the switch behind every
// batched entry point).
int launch_mode(const crs_mech *m, crs::Batch &b, int mode, cudaStream_t s) {
  cudaError_t e;
  switch (mode) {
    case CRS_MODE_FP64_STRICT:
      e = crs::launch_wdot_strict(m->d_img, m->L, b, m->sm_count, m->smem_optin, s);
      break;
    case CRS_MODE_FP64:
      // one state per thread when its columns fit on chip; else the
      // two-pass state-tile path (per warp when intermediates are asked for)
      e = crs::launch_wdot_fp64_tps(m->d_img, m->L, b, m->sm_count, m->smem_optin, s);
      if (e == cudaErrorNotSupported) {
        if (!(b.conc || b.fwd || b.rev || b.pm) && tile_smem(m->L, true) <= (size_t)m->smem_optin)
          return wdot_two_pass(const_cast<crs_mech *>(m), b, s, true);
        e = crs::launch_wdot_fp64(m->d_img, m->L, b, m->sm_count, m->smem_optin, s);
      }
      break;
    case CRS_MODE_FP64_TILE:
      if (b.conc || b.fwd || b.rev || b.pm)
        return fail(CRS_ERR_UNSUPPORTED, "CRS_MODE_FP64_TILE does not write intermediates");
      return wdot_two_pass(const_cast<crs_mech *>(m), b, s, true);
    case CRS_MODE_MIXED:
      // one state per thread when its columns fit on chip; else the
      // two-pass state-tile path (per warp when intermediates are asked for)
      e = crs::launch_wdot_mixed_tps(m->d_img, m->L, b, m->sm_count, m->smem_optin, s);
      if (e == cudaErrorNotSupported) {
        if (!(b.conc || b.fwd || b.rev || b.pm) && tile_smem(m->L, false) <= (size_t)m->smem_optin)
          return wdot_two_pass(const_cast<crs_mech *>(m), b, s, false);
        e = crs::launch_wdot_mixed(m->d_img, m->L, b, m->sm_count, m->smem_optin, s);
      }
      break;
    case CRS_MODE_MIXED_TILE:
      if (b.conc || b.fwd || b.rev || b.pm)
        return fail(CRS_ERR_UNSUPPORTED, "CRS_MODE_MIXED_TILE does not write intermediates");
      return wdot_two_pass(const_cast<crs_mech *>(m), b, s, false);
    case CRS_MODE_FP64_TPS:
      e = crs::launch_wdot_fp64_tps(m->d_img, m->L, b, m->sm_count, m->smem_optin, s);
      break;
    case CRS_MODE_MIXED_TPS:
      e = crs::launch_wdot_mixed_tps(m->d_img, m->L, b, m->sm_count, m->smem_optin, s);
      break;
    case CRS_MODE_FP64_WARP:
      e = crs::launch_wdot_fp64(m->d_img, m->L, b, m->sm_count, m->smem_optin, s);
      break;
    case CRS_MODE_MIXED_WARP:
      e = crs::launch_wdot_mixed(m->d_img, m->L, b, m->sm_count, m->smem_optin, s);
      break;
    case CRS_MODE_GEMM: {
      if (b.conc || b.fwd || b.rev || b.pm)
        return fail(CRS_ERR_UNSUPPORTED, "CRS_MODE_GEMM does not write intermediates");
      int rc2 = wdot_gemm(const_cast<crs_mech *>(m), b, s);
      if (rc2 != CRS_OK) return rc2;
      e = cudaSuccess;
      break;
    }
    default:
      return fail(CRS_ERR_ARG, "unknown mode %d", mode);
  }
  if (e == cudaErrorNotSupported)
    return fail(CRS_ERR_UNSUPPORTED, "mode %d is not available for this mechanism", mode);
  return e == cudaSuccess ? CRS_OK : cuda_fail(e, "crs_wdot launch");
}

}  // namespace

extern "C" {

const char *crs_last_error(void) { return g_err.c_str(); }

int crs_mech_load(const void *blob, size_t nbytes, crs_mech **out) {
  if (!blob || !out) return fail(CRS_ERR_ARG, "NULL argument");
  *out = nullptr;
  crs_mech *m = new crs_mech();
  int rc = build_image(static_cast<const unsigned char *>(blob), nbytes, m);
  if (rc != CRS_OK) {
    delete m;
    return rc;
  }
  m->htab = crs::make_tab(m->h_img.data(), m->L);
  m->haux = crs::host::make_aux(m->htab);
  cudaError_t e = cudaGetDevice(&m->device);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, m->device);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&m->smem_optin,
                               cudaDevAttrMaxSharedMemoryPerBlockOptin, m->device);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_img, m->h_img.size());
  if (e == cudaSuccess)
    e = cudaMemcpy(m->d_img, m->h_img.data(), m->h_img.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&m->d_status, 4 * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMemset(m->d_status, 0, 4 * sizeof(int32_t));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_sched, 2 * SCHED_SLOTS * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(m->d_sched, 0, 2 * SCHED_SLOTS * sizeof(unsigned long long));
  if (e != cudaSuccess) {
    int r = cuda_fail(e, "crs_mech_load");
    crs_mech_free(m);
    return r;
  }
  // dynamic shared memory of the launchers: the opt-in limit less the
  // kernels' static __shared__ part (the staging mbarrier, which the
  // 128-byte alignment of the dynamic part pads to 128 bytes) and slack
  m->smem_optin -= 256;
  *out = m;
  return CRS_OK;
}

int crs_mech_load_host(const void *blob, size_t nbytes, crs_mech **out) {
  if (!blob || !out) return fail(CRS_ERR_ARG, "NULL argument");
  *out = nullptr;
  crs_mech *m = new crs_mech();
  int rc = build_image(static_cast<const unsigned char *>(blob), nbytes, m);
  if (rc != CRS_OK) {
    delete m;
    return rc;
  }
  m->device = -1;
  m->htab = crs::make_tab(m->h_img.data(), m->L);
  m->haux = crs::host::make_aux(m->htab);
  *out = m;
  return CRS_OK;
}

int crs_mech_image(const void *blob, size_t nbytes, void *img, size_t img_cap,
                   int32_t *layout, size_t layout_cap, size_t sizes[2]) {
  if (!blob || !sizes) return fail(CRS_ERR_ARG, "NULL argument");
  crs_mech m;
  int rc = build_image(static_cast<const unsigned char *>(blob), nbytes, &m);
  if (rc != CRS_OK) return rc;
  static_assert(sizeof(crs::ImgLayout) % sizeof(int32_t) == 0, "layout of int32 words");
  sizes[0] = m.h_img.size();
  sizes[1] = sizeof(crs::ImgLayout) / sizeof(int32_t);
  if (img) {
    if (img_cap < sizes[0]) return fail(CRS_ERR_ARG, "image buffer too small");
    memcpy(img, m.h_img.data(), sizes[0]);
  }
  if (layout) {
    if (layout_cap < sizes[1]) return fail(CRS_ERR_ARG, "layout buffer too small");
    memcpy(layout, &m.L, sizeof(crs::ImgLayout));
  }
  return CRS_OK;
}

int crs_mech_inspect(const void *blob, size_t nbytes, int64_t out[6]) {
  if (!blob || !out) return fail(CRS_ERR_ARG, "NULL argument");
  crs_mech m;
  int rc = build_image(static_cast<const unsigned char *>(blob), nbytes, &m);
  if (rc != CRS_OK) return rc;
  const int64_t block = 128, N = m.L.N;
  out[0] = m.L.bytes;
  auto span = [&](int r) {
    return (int64_t)(m.L.rng[r][1] - m.L.rng[r][0] + m.L.rng[r][3] - m.L.rng[r][2]);
  };
  const int64_t R = m.L.R;
  out[1] = span(1);
  out[2] = span(3);
  out[3] = span(1) + 8 * 8 * (128 + 2 * N + R + 1);          // CRS_MODE_FP64 per CTA
  out[4] = span(3) + 8 * 8 * (128 + N + R + (N + 1) / 2 + 1);  // CRS_MODE_MIXED per CTA
  out[5] = m.L.kc_mix + 2 * N * block * 8;   // CRS_MODE_FP64_STRICT, all on chip
  return CRS_OK;
}

int crs_mech_load_file(const char *path, crs_mech **out) {
  if (!path || !out) return fail(CRS_ERR_ARG, "NULL argument");
  std::ifstream f(path, std::ios::binary);
  if (!f) return fail(CRS_ERR_ARG, "cannot open %s", path);
  std::vector<char> buf((std::istreambuf_iterator<char>(f)),
                        std::istreambuf_iterator<char>());
  return crs_mech_load(buf.data(), buf.size(), out);
}

int crs_mech_free(crs_mech *m) {
  if (!m) return CRS_OK;
  unbind(m);
  if (m->d_img) cudaFree(m->d_img);
  if (m->d_status) cudaFree(m->d_status);
  if (m->d_sched) cudaFree(m->d_sched);
  if (m->d_nuB) cudaFree(m->d_nuB);
  if (m->d_ws) cudaFree(m->d_ws);
  if (m->d_escale) cudaFree(m->d_escale);
  if (m->d_outflag) cudaFree(m->d_outflag);
  if (m->d_q) cudaFree(m->d_q);
  if (m->ws_done) cudaEventDestroy(m->ws_done);
  if (m->d_host) cudaFree(m->d_host);
  for (cudaStream_t st : m->hs)
    if (st) cudaStreamDestroy(st);
  crs::host::free_aux(m->haux);
  delete m;
  return CRS_OK;
}

int crs_mech_dims(const crs_mech *m, int64_t out[5]) {
  if (!m || !out) return fail(CRS_ERR_ARG, "NULL argument");
  out[0] = m->L.N;
  out[1] = m->L.R;
  out[2] = m->L.NREV;
  out[3] = m->L.NPM;
  out[4] = m->L.NRATE;
  return CRS_OK;
}

int crs_status(const crs_mech *m, void *stream, int32_t out[2]) {
  if (!m || !out) return fail(CRS_ERR_ARG, "NULL argument");
  if (!m->d_status) return fail(CRS_ERR_ARG, "mechanism has no device tables");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(out, m->d_status, 2 * sizeof(int32_t),
                                  cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? CRS_OK : cuda_fail(e, "crs_status");
}

int crs_status_reset(const crs_mech *m, void *stream) {
  if (!m) return fail(CRS_ERR_ARG, "NULL argument");
  if (!m->d_status) return fail(CRS_ERR_ARG, "mechanism has no device tables");
  cudaError_t e = cudaMemsetAsync(m->d_status, 0, 2 * sizeof(int32_t),
                                  static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? CRS_OK : cuda_fail(e, "crs_status_reset");
}

int crs_eval_conc_batch(const crs_mech *m, int64_t n, const double *T,
                        const double *P, const double *Y, int64_t ld,
                        double *y_N, double *mw_avg, double *rho, double *conc,
                        void *stream) {
  int rc = check_batch(m, n, ld);
  if (rc) return rc;
  if (n == 0) return CRS_OK;
  if (!T || !P || !Y || !conc) return fail(CRS_ERR_ARG, "NULL array");
  crs::Batch b = make_batch(m, n, ld);
  b.T = T; b.P = P; b.Y = Y; b.conc = conc;
  cudaError_t e = crs::launch_stage(0, m->d_img, m->L, b, y_N, mw_avg, rho,
                                    m->sm_count, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? CRS_OK : cuda_fail(e, "eval_conc launch");
}

int crs_eval_rxn_rates_batch(const crs_mech *m, int64_t n, const double *T,
                             const double *P, const double *C, int64_t ld,
                             double *fwd, double *rev, void *stream) {
  int rc = check_batch(m, n, ld);
  if (rc) return rc;
  if (n == 0) return CRS_OK;
  if (!T || !P || !C || !fwd || (m->L.NREV > 0 && !rev))
    return fail(CRS_ERR_ARG, "NULL array");
  crs::Batch b = make_batch(m, n, ld);
  b.T = T; b.P = P; b.conc = const_cast<double *>(C); b.fwd = fwd; b.rev = rev;
  cudaError_t e = crs::launch_stage(1, m->d_img, m->L, b, nullptr, nullptr,
                                    nullptr, m->sm_count, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? CRS_OK : cuda_fail(e, "eval_rxn_rates launch");
}

int crs_get_rxn_pres_mod_batch(const crs_mech *m, int64_t n, const double *T,
                               const double *P, const double *C, int64_t ld,
                               double *pres_mod, void *stream) {
  int rc = check_batch(m, n, ld);
  if (rc) return rc;
  if (n == 0 || m->L.NPM == 0) return CRS_OK;
  if (!T || !P || !C || !pres_mod) return fail(CRS_ERR_ARG, "NULL array");
  crs::Batch b = make_batch(m, n, ld);
  b.T = T; b.P = P; b.conc = const_cast<double *>(C); b.pm = pres_mod;
  cudaError_t e = crs::launch_stage(2, m->d_img, m->L, b, nullptr, nullptr,
                                    nullptr, m->sm_count, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? CRS_OK : cuda_fail(e, "get_rxn_pres_mod launch");
}

int crs_eval_spec_rates_batch(const crs_mech *m, int64_t n, const double *fwd,
                              const double *rev, const double *pres_mod,
                              int64_t ld, double *wdot, void *stream) {
  int rc = check_batch(m, n, ld);
  if (rc) return rc;
  if (n == 0) return CRS_OK;
  if (!fwd || !wdot || (m->L.NREV > 0 && !rev) || (m->L.NPM > 0 && !pres_mod))
    return fail(CRS_ERR_ARG, "NULL array");
  crs::Batch b = make_batch(m, n, ld);
  b.fwd = const_cast<double *>(fwd); b.rev = const_cast<double *>(rev);
  b.pm = const_cast<double *>(pres_mod); b.wdot = wdot;
  cudaError_t e = crs::launch_stage(3, m->d_img, m->L, b, nullptr, nullptr,
                                    nullptr, m->sm_count, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? CRS_OK : cuda_fail(e, "eval_spec_rates launch");
}

int crs_wdot_stages(const crs_mech *m, int64_t n, const double *T,
                    const double *P, const double *Y, int64_t ld, double *wdot,
                    double *conc, double *fwd, double *rev, double *pres_mod,
                    int mode, void *stream) {
  int rc = check_batch(m, n, ld);
  if (rc) return rc;
  if (n == 0) return CRS_OK;
  if (!T || !P || !Y || !wdot) return fail(CRS_ERR_ARG, "NULL array");
  crs::Batch b = make_batch(m, n, ld);
  b.T = T; b.P = P; b.Y = Y; b.wdot = wdot;
  b.conc = conc; b.fwd = fwd; b.rev = rev; b.pm = pres_mod;
  return launch_mode(m, b, mode, static_cast<cudaStream_t>(stream));
}

int crs_wdot(const crs_mech *m, int64_t n, const double *T, const double *P,
             const double *Y, int64_t ld, double *wdot, int mode, void *stream) {
  return crs_wdot_stages(m, n, T, P, Y, ld, wdot, nullptr, nullptr, nullptr,
                         nullptr, mode, stream);
}

int crs_eval_thermo_batch(const crs_mech *m, int64_t n, const double *T, int64_t ld,
                          int which, double *out, void *stream) {
  int rc = check_batch(m, n, ld);
  if (rc) return rc;
  if (which < 0 || which > 3) return fail(CRS_ERR_ARG, "which must be 0..3 (h, u, cv, cp)");
  if (n == 0) return CRS_OK;
  if (!T || !out) return fail(CRS_ERR_ARG, "NULL array");
  cudaError_t e = crs::launch_thermo(m->d_img, m->L, which, n, T, ld, out, m->sm_count,
                                     static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? CRS_OK : cuda_fail(e, "crs_eval_thermo_batch");
}

int crs_eval_conc_rho_batch(const crs_mech *m, int64_t n, const double *T, const double *rho,
                            const double *Y, int64_t ld, double *y_N, double *mw_avg,
                            double *pres, double *conc, void *stream) {
  int rc = check_batch(m, n, ld);
  if (rc) return rc;
  if (n == 0) return CRS_OK;
  if (!T || !rho || !Y) return fail(CRS_ERR_ARG, "NULL array");
  cudaError_t e = crs::launch_conc_rho(m->d_img, m->L, n, T, rho, Y, ld, y_N, mw_avg, pres,
                                       conc, m->sm_count, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? CRS_OK : cuda_fail(e, "crs_eval_conc_rho_batch");
}

int crs_dydt(const crs_mech *m, int64_t n, const double *p_or_rho, const double *y,
             int64_t ld, double *dy, int conv, int mode, void *stream) {
  int rc = check_batch(m, n, ld);
  if (rc) return rc;
  if (conv != 0 && conv != 1) return fail(CRS_ERR_ARG, "conv must be 0 or 1");
  if (n == 0) return CRS_OK;
  if (!p_or_rho || !y || !dy) return fail(CRS_ERR_ARG, "NULL array");
  const int64_t N = m->L.N;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // stream-ordered scratch: wdot [N][ld] and, for constant volume, the
  // pressure row
  double *ws = nullptr;
  const size_t bytes = ((size_t)N * ld + (conv ? (size_t)ld : 0)) * sizeof(double);
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&ws), bytes, s);
  if (e != cudaSuccess) return cuda_fail(e, "crs_dydt scratch");
  double *W = ws, *Pw = ws + (size_t)N * ld;
  if (conv)
    e = crs::launch_conc_rho(m->d_img, m->L, n, y, p_or_rho, y + ld, ld, nullptr, nullptr, Pw,
                             nullptr, m->sm_count, s);
  int result = e == cudaSuccess ? CRS_OK : cuda_fail(e, "crs_dydt pressure");
  if (result == CRS_OK) {
    crs::Batch b = make_batch(m, n, ld);
    b.T = y; b.P = conv ? Pw : p_or_rho; b.Y = y + ld; b.wdot = W;
    result = launch_mode(m, b, mode, s);
  }
  if (result == CRS_OK) {
    e = crs::launch_dydt_finish(m->d_img, m->L, conv, n, y, ld, p_or_rho, W, dy, m->sm_count, s);
    if (e != cudaSuccess) result = cuda_fail(e, "crs_dydt");
  }
  e = cudaFreeAsync(ws, s);
  if (e != cudaSuccess && result == CRS_OK) result = cuda_fail(e, "crs_dydt scratch");
  return result;
}

}  // extern "C"

namespace {
// The device address of a host array that the current device can read and
// write in place (page-locked memory mapped into its address space), else
// null.
void *mapped_view(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // an unregistered pointer is not an error here
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}
}  // namespace

extern "C" {

int crs_wdot_host(const crs_mech *m, int64_t n, const double *T, const double *P,
                  const double *Y, int64_t ld, double *wdot, int mode) {
  int rc = check_batch(m, n, ld);
  if (rc) return rc;
  if (n == 0) return CRS_OK;
  if (!T || !P || !Y || !wdot) return fail(CRS_ERR_ARG, "NULL array");
  const bool staged_only = (mode & CRS_HOST_STAGED) != 0;
  mode &= ~CRS_HOST_STAGED;
  crs_mech *mm = const_cast<crs_mech *>(m);
  std::lock_guard<std::mutex> lock(mm->host_mu);
  const int64_t N = m->L.N;
  cudaError_t e = cudaSuccess;
  if (!mm->hs[0]) e = cudaStreamCreateWithFlags(&mm->hs[0], cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(e, "crs_wdot_host streams");
  if (!staged_only) {
    // arrays the device addresses in place: one launch reads the states
    // from host memory and writes wdot back over the host link (NVLink-C2C
    // on Grace), without staging copies or per-chunk launches
    void *vT = mapped_view(T), *vP = mapped_view(P), *vY = mapped_view(Y),
         *vW = mapped_view(wdot);
    if (vT && vP && vY && vW) {
      crs::Batch b = make_batch(m, n, ld);
      b.T = static_cast<const double *>(vT);
      b.P = static_cast<const double *>(vP);
      b.Y = static_cast<const double *>(vY);
      b.wdot = static_cast<double *>(vW);
      int result = launch_mode(m, b, mode, mm->hs[0]);
      const cudaError_t es = cudaStreamSynchronize(mm->hs[0]);
      if (es != cudaSuccess && result == CRS_OK) result = cuda_fail(es, "crs_wdot_host");
      return result;
    }
  }
  const int64_t per = 2 + (N - 1) + N;  // doubles per state: T, P, Y, wdot
  // chunks of up to 2^17 states, at most 256 MB per buffer
  int64_t chunk = ((int64_t)256 << 20) / (per * 8);
  if (chunk > ((int64_t)1 << 17)) chunk = (int64_t)1 << 17;
  if (chunk < 128) chunk = 128;
  if (mm->host_chunk < chunk) {
    if (mm->d_host) cudaFree(mm->d_host);
    mm->d_host = nullptr;
    mm->host_chunk = 0;
    e = cudaMalloc(&mm->d_host, (size_t)2 * chunk * per * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(e, "crs_wdot_host buffers");
    mm->host_chunk = chunk;
  }
  for (int j = 0; j < 2 && e == cudaSuccess; ++j)
    if (!mm->hs[j]) e = cudaStreamCreateWithFlags(&mm->hs[j], cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(e, "crs_wdot_host streams");
  // chunk c on stream c % 2: its copies in overlap the other stream's
  // kernel, its copies out the next kernel; a buffer is reused only after
  // the same stream has finished with it
  int result = CRS_OK;
  for (int64_t c0 = 0, c = 0; c0 < n && result == CRS_OK; c0 += chunk, ++c) {
    const int64_t cn = n - c0 < chunk ? n - c0 : chunk;
    cudaStream_t s = mm->hs[c & 1];
    double *dT = mm->d_host + (size_t)(c & 1) * chunk * per;
    double *dP = dT + cn, *dY = dP + cn, *dW = dY + (N - 1) * cn;
    const size_t row = (size_t)cn * sizeof(double);
    e = cudaMemcpyAsync(dT, T + c0, row, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dP, P + c0, row, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && N > 1)
      e = cudaMemcpy2DAsync(dY, row, Y + c0, (size_t)ld * sizeof(double), row, N - 1,
                            cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
      result = cuda_fail(e, "crs_wdot_host copy in");
      break;
    }
    crs::Batch b = make_batch(m, cn, cn);
    b.T = dT; b.P = dP; b.Y = dY; b.wdot = dW;
    result = launch_mode(m, b, mode, s);
    if (result != CRS_OK) break;
    e = cudaMemcpy2DAsync(wdot + c0, (size_t)ld * sizeof(double), dW, row, row, N,
                          cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) result = cuda_fail(e, "crs_wdot_host copy out");
  }
  for (int j = 0; j < 2; ++j) {
    const cudaError_t es = cudaStreamSynchronize(mm->hs[j]);
    if (es != cudaSuccess && result == CRS_OK) result = cuda_fail(es, "crs_wdot_host");
  }
  return result;
}

}  // extern "C"

// ---- per-state drop-in ---------------------------------------------------
//
// The reference's per-state functions are pure host functions with the
// mechanism baked in.  Here they evaluate the bound mechanism's host table
// image on the calling thread (crs_host.cpp): no lock, no device, no
// allocation, safe from any number of threads at once.

extern "C" {

#define CRS_STATE_CHECK(m, name)                                        \
  do {                                                                  \
    if (!(m)) return fail(CRS_ERR_ARG, "%s: mechanism is NULL", name);  \
  } while (0)

int crs_state_eval_conc(const crs_mech *m, double T, double pres, const double *y,
                        double *y_N, double *mw_avg, double *rho, double *conc) {
  CRS_STATE_CHECK(m, "crs_state_eval_conc");
  if ((!y && m->L.N > 1) || !y_N || !mw_avg || !rho || !conc)
    return fail(CRS_ERR_ARG, "crs_state_eval_conc: NULL array");
  crs::host::eval_conc(m->htab, T, pres, y, y_N, mw_avg, rho, conc);
  return CRS_OK;
}

int crs_state_eval_rxn_rates(const crs_mech *m, double T, double pres, const double *C,
                             double *fwd, double *rev) {
  CRS_STATE_CHECK(m, "crs_state_eval_rxn_rates");
  if (!C || (!fwd && m->L.R > 0) || (!rev && m->L.NREV > 0))
    return fail(CRS_ERR_ARG, "crs_state_eval_rxn_rates: NULL array");
  crs::host::eval_rxn_rates(m->htab, m->haux, T, pres, C, fwd, rev);
  return CRS_OK;
}

int crs_state_get_rxn_pres_mod(const crs_mech *m, double T, double pres, const double *C,
                               double *pres_mod) {
  CRS_STATE_CHECK(m, "crs_state_get_rxn_pres_mod");
  if (!C || (!pres_mod && m->L.NPM > 0))
    return fail(CRS_ERR_ARG, "crs_state_get_rxn_pres_mod: NULL array");
  crs::host::get_rxn_pres_mod(m->htab, m->haux, T, pres, C, pres_mod);
  return CRS_OK;
}

int crs_state_eval_spec_rates(const crs_mech *m, const double *fwd, const double *rev,
                              const double *pres_mod, double *sp_rates, double *dy_N) {
  CRS_STATE_CHECK(m, "crs_state_eval_spec_rates");
  if ((!fwd && m->L.R > 0) || (!rev && m->L.NREV > 0) || (!pres_mod && m->L.NPM > 0) ||
      (!sp_rates && m->L.N > 1) || !dy_N)
    return fail(CRS_ERR_ARG, "crs_state_eval_spec_rates: NULL array");
  crs::host::eval_spec_rates(m->htab, m->haux, fwd, rev, pres_mod, sp_rates, dy_N);
  return CRS_OK;
}

int crs_state_eval_thermo(const crs_mech *m, int which, double T, double *out) {
  CRS_STATE_CHECK(m, "crs_state_eval_thermo");
  if (which < 0 || which > 3) return fail(CRS_ERR_ARG, "which must be 0..3 (h, u, cv, cp)");
  if (!out) return fail(CRS_ERR_ARG, "crs_state_eval_thermo: NULL array");
  crs::host::eval_thermo(m->htab, which, T, out);
  return CRS_OK;
}

int crs_state_eval_conc_rho(const crs_mech *m, double T, double rho, const double *y,
                            double *y_N, double *mw_avg, double *pres, double *conc) {
  CRS_STATE_CHECK(m, "crs_state_eval_conc_rho");
  if ((!y && m->L.N > 1) || !y_N || !mw_avg || !pres || !conc)
    return fail(CRS_ERR_ARG, "crs_state_eval_conc_rho: NULL array");
  crs::host::eval_conc_rho(m->htab, T, rho, y, y_N, mw_avg, pres, conc);
  return CRS_OK;
}

int crs_state_dydt(const crs_mech *m, int conv, double p_or_rho, const double *y, double *dy) {
  CRS_STATE_CHECK(m, "crs_state_dydt");
  if (conv != 0 && conv != 1) return fail(CRS_ERR_ARG, "conv must be 0 or 1");
  if (!y || !dy) return fail(CRS_ERR_ARG, "crs_state_dydt: NULL array");
  crs::host::dydt(m->htab, m->haux, conv, p_or_rho, y, dy);
  return CRS_OK;
}

#undef CRS_STATE_CHECK

}  // extern "C"

namespace {
// The mechanism of the reference-signature functions: the calling thread's
// own binding (crs_bind_thread) if it has one, else the process-wide one
// (crs_bind).  Reads are lock-free; a handle is immutable after load.
std::atomic<const crs_mech *> g_bound{nullptr};
thread_local const crs_mech *t_bound = nullptr;
std::atomic<int> g_dydt_conv{0};  // form of the per-state dydt (crs_dydt_form)

const crs_mech *bound(const char *name) {
  const crs_mech *m = t_bound ? t_bound : g_bound.load(std::memory_order_acquire);
  if (!m) fail(CRS_ERR_NOMECH, "%s: no mechanism bound (crs_bind / crs_bind_thread)", name);
  return m;
}
}  // namespace

// Called by crs_mech_free: a freed handle stays bound nowhere that this
// thread or the process-wide binding can reach.
void unbind(const crs_mech *m) {
  const crs_mech *expected = m;
  g_bound.compare_exchange_strong(expected, nullptr);
  if (t_bound == m) t_bound = nullptr;
}

extern "C" {

int crs_bind(const crs_mech *m) {
  g_bound.store(m, std::memory_order_release);
  return CRS_OK;
}

int crs_bind_thread(const crs_mech *m) {
  t_bound = m;
  return CRS_OK;
}

// rate_subs.py:1297-1299 (chem_utils.h)
void eval_conc(const double T, const double pres, const double *y, double *y_N,
               double *mw_avg, double *rho, double *conc) {
  if (const crs_mech *m = bound("eval_conc"))
    crs::host::eval_conc(m->htab, T, pres, y, y_N, mw_avg, rho, conc);
}

// rate_subs.py:287-290 (rates.h)
void eval_rxn_rates(const double T, const double pres, const double *C,
                    double *fwd_rxn_rates, double *rev_rxn_rates) {
  if (const crs_mech *m = bound("eval_rxn_rates"))
    crs::host::eval_rxn_rates(m->htab, m->haux, T, pres, C, fwd_rxn_rates, rev_rxn_rates);
}

// rate_subs.py:761-763 (rates.h)
void get_rxn_pres_mod(const double T, const double pres, const double *C,
                      double *pres_mod) {
  if (const crs_mech *m = bound("get_rxn_pres_mod"))
    crs::host::get_rxn_pres_mod(m->htab, m->haux, T, pres, C, pres_mod);
}

// rate_subs.py:1124-1127 (rates.h)
void eval_spec_rates(const double *fwd_rates, const double *rev_rates,
                     const double *pres_mod, double *sp_rates, double *dy_N) {
  if (const crs_mech *m = bound("eval_spec_rates"))
    crs::host::eval_spec_rates(m->htab, m->haux, fwd_rates, rev_rates, pres_mod, sp_rates, dy_N);
}

// rate_subs.py:1497-1776 (chem_utils.h :1276-1279)
void eval_h(const double T, double *h) {
  if (const crs_mech *m = bound("eval_h")) crs::host::eval_thermo(m->htab, 0, T, h);
}
void eval_u(const double T, double *u) {
  if (const crs_mech *m = bound("eval_u")) crs::host::eval_thermo(m->htab, 1, T, u);
}
void eval_cv(const double T, double *cv) {
  if (const crs_mech *m = bound("eval_cv")) crs::host::eval_thermo(m->htab, 2, T, cv);
}
void eval_cp(const double T, double *cp) {
  if (const crs_mech *m = bound("eval_cp")) crs::host::eval_thermo(m->htab, 3, T, cp);
}

// rate_subs.py:1396-1490 (chem_utils.h :1274-1275)
void eval_conc_rho(const double T, const double rho, const double *y, double *y_N,
                   double *mw_avg, double *pres, double *conc) {
  if (const crs_mech *m = bound("eval_conc_rho"))
    crs::host::eval_conc_rho(m->htab, T, rho, y, y_N, mw_avg, pres, conc);
}

int crs_dydt_form(int conv) {
  if (conv != 0 && conv != 1) return fail(CRS_ERR_ARG, "conv must be 0 or 1");
  g_dydt_conv.store(conv);
  return CRS_OK;
}

// rate_subs.py:1829-2067 (dydt.h): y = [T, Y_0 .. Y_{N-2}]; `pres` is the
// pressure (constant pressure, the default) or the density (constant
// volume, after crs_dydt_form(1)), as the emitted CONP / CONV builds read it.
void dydt(const double t, const double pres, const double *y, double *dy) {
  (void)t;
  if (const crs_mech *m = bound("dydt"))
    crs::host::dydt(m->htab, m->haux, g_dydt_conv.load(), pres, y, dy);
}

}  // extern "C"

// ---- allocation-free variant of the tensor-core contraction path ----------
//
// Some callers cannot allocate device memory at the moment they evaluate
// rates: solvers that run inside a memory pool or framework that owns every
// device allocation, code embedded in another runtime whose allocator must
// not be bypassed, or integrator loops that must not block on cudaMalloc
// (it can synchronise the device).  crs_wdot_gemm_noalloc serves them: it
// evaluates exactly what crs_wdot(..., CRS_MODE_GEMM, ...) evaluates, but all
// of its scratch lives in the array below, which the library's module holds
// on every device it is loaded on, until the process exits.
namespace {

constexpr size_t kNoallocScratchBytes = (size_t)32 << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Device address of the array, looked up once per device.  In host code
// g_noalloc_scratch names a host-side stand-in, never a device address.
struct NoallocDevice {
  bool ready = false;
  unsigned char *ptr = nullptr;
};
std::mutex g_noalloc_mu;
NoallocDevice g_noalloc_dev[64];

int noalloc_scratch(int device, unsigned char **out) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (device < 0 || device >= 64) return fail(CRS_ERR_ARG, "device ordinal %d out of range", device);
  NoallocDevice &d = g_noalloc_dev[device];
  if (!d.ready) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "crs_wdot_gemm_noalloc: scratch address");
    d.ptr = static_cast<unsigned char *>(p);
    d.ready = true;
  }
  *out = d.ptr;
  return CRS_OK;
}

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

// B[k][r] = B[k][Kh + r] = nu_kr for the reactions' net coefficients; the
// rest of B must already be zero.
__global__ void k_noalloc_nu(const unsigned char *__restrict__ img, crs::ImgLayout L,
                             __nv_bfloat16 *B, int64_t K, int Kh) {
  const crs::Tab t = crs::make_tab(img, L);
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < L.R; r += gridDim.x * blockDim.x)
    for (int e = t.nu_ptr[r]; e < t.nu_ptr[r + 1]; ++e) {
      const __nv_bfloat16 v = __float2bfloat16((float)t.nu_val[e]);
      const int64_t k = t.nu_sp[e];
      B[k * K + r] = v;
      B[k * K + Kh + r] = v;
    }
}

}  // namespace

extern "C" int crs_wdot_gemm_noalloc(const crs_mech *m, int64_t n, const double *T,
                                     const double *P, const double *Y, int64_t ld,
                                     double *wdot, void *stream) {
  int rc = check_batch(m, n, ld);
  if (rc) return rc;
  if (n == 0) return CRS_OK;
  if (!T || !P || !Y || !wdot) return fail(CRS_ERR_ARG, "NULL array");
  const crs::ImgLayout &L = m->L;
  // the stoichiometric matrix must be exact in bf16
  const crs::Tab th = crs::make_tab(m->h_img.data(), L);
  for (int e = 0; e < th.nu_ptr[L.R]; ++e) {
    const double nu = th.nu_val[e];
    if ((double)__bfloat162float(__float2bfloat16((float)nu)) != nu)
      return fail(CRS_ERR_UNSUPPORTED, "a stoichiometric coefficient is not exact in bf16");
  }
  const int Kh = (L.R + 63) / 64 * 64;
  const int64_t K = 2 * (int64_t)Kh;
  const int block_n = L.N <= 64 ? 64 : L.N <= 128 ? 128 : L.N <= 192 ? 192 : L.N <= 256 ? 256 : 192;
  const int64_t N_pad = (L.N + block_n - 1) / block_n * block_n;
  // scratch layout: B [N_pad][K] | escale [rows] | bf16 rows [rows][K]
  const size_t b_bytes = align256((size_t)N_pad * K * sizeof(__nv_bfloat16));
  const size_t per_row = (size_t)K * sizeof(__nv_bfloat16) + sizeof(int);
  int64_t rows = 0;
  if (b_bytes + 256 < kNoallocScratchBytes)
    rows = (int64_t)((kNoallocScratchBytes - b_bytes - 256) / per_row) / 128 * 128;
  if (rows < 128)
    return fail(CRS_ERR_UNSUPPORTED,
                "crs_wdot_gemm_noalloc: the mechanism needs %zu bytes of scratch for "
                "128 states, more than the fixed %zu",
                b_bytes + 256 + 128 * per_row, kNoallocScratchBytes);
  rows = std::min<int64_t>(rows, (n + 127) / 128 * 128);
  unsigned char *base = nullptr;
  rc = noalloc_scratch(m->device, &base);
  if (rc) return rc;
  __nv_bfloat16 *B = reinterpret_cast<__nv_bfloat16 *>(base);
  int *escale = reinterpret_cast<int *>(base + b_bytes);
  void *A = base + b_bytes + align256((size_t)rows * sizeof(int));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the array keeps the previous call's contents: rebuild B from zero
  cudaError_t e = cudaMemsetAsync(B, 0, (size_t)N_pad * K * sizeof(__nv_bfloat16), s);
  if (e != cudaSuccess) return cuda_fail(e, "crs_wdot_gemm_noalloc: clear");
  k_noalloc_nu<<<(L.R + 127) / 128 > 0 ? (L.R + 127) / 128 : 1, 128, 0, s>>>(m->d_img, L, B, K, Kh);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "crs_wdot_gemm_noalloc: nu");
  crs::Batch b = make_batch(m, n, ld);
  b.T = T; b.P = P; b.Y = Y; b.wdot = wdot;
  for (int64_t c0 = 0; c0 < n; c0 += rows) {
    const int64_t cnt = std::min<int64_t>(rows, n - c0);
    crs::Batch bc = b;
    bc.n = cnt;
    bc.T = T + c0;
    bc.P = P + c0;
    bc.Y = Y + c0;
    bc.wdot = wdot + c0;
    crs::mixed::QOut qo{A, K, Kh, escale};
    e = crs::launch_wdot_mixed_q(m->d_img, L, bc, m->sm_count, m->smem_optin, s, qo);
    if (e == cudaErrorNotSupported)
      return fail(CRS_ERR_UNSUPPORTED, "mechanism too large for the rates kernel");
    if (e != cudaSuccess) return cuda_fail(e, "crs_wdot_gemm_noalloc: rates");
    const int64_t M_pad = (cnt + 127) / 128 * 128;
    e = crs::launch_gemm_wdot(A, B, M_pad, N_pad, K, block_n, bc.wdot, ld, (int)cnt, L.N,
                              escale, m->d_status, s);
    if (e != cudaSuccess) return cuda_fail(e, "crs_wdot_gemm_noalloc: contraction");
  }
  return CRS_OK;
}
