/*
 * crs.h -- C ABI of libcrs, the sm_103a (GB300) evaluation library behind
 * create_rate_subs_gb300.
 *
 * The reference (kyleniemeyer/create_rate_subs) emits, per mechanism, four
 * per-state C functions that an integrator calls once per thermochemical
 * state.  libcrs keeps those four signatures (bottom of this file) and adds
 * batched, stream-ordered entry points over millions of states held in
 * device memory in structure-of-arrays layout.
 *
 * Conventions for the batched entry points
 *  - every array argument is a DEVICE pointer owned by the caller;
 *  - SoA layout: entry k of state i lives at [k*ld + i]; ld >= n;
 *  - Y holds the first N-1 mass fractions (species order of the mechanism);
 *    the last one is implied, as in the reference's eval_conc;
 *  - calls are asynchronous on `stream` (a cudaStream_t, NULL = legacy
 *    default stream) and do not synchronise;
 *  - return 0 on success or a CRS_ERR_* code; crs_last_error() describes
 *    the last failure of the calling thread;
 *  - a crs_mech is immutable after crs_mech_load and may be used from
 *    several host threads at once; each handle owns one device status word
 *    that concurrent launches on the same handle share, and 256 scheduling
 *    counters that its one-state-per-thread launches draw in turn: at most
 *    256 such launches of one handle may be in flight at the same time
 *    (several streams; a captured CUDA graph replayed on several streams at
 *    once counts every replay).
 * Units are the reference's: T [K], P [Pa], C [kmol/m^3], rates
 * [kmol/(m^3 s)].
 */
#ifndef CRS_H
#define CRS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct crs_mech crs_mech;

#define CRS_OK 0
#define CRS_ERR_ARG 1         /* NULL pointer, n < 0, ld < n, bad mode */
#define CRS_ERR_BLOB 2        /* malformed mechanism tables */
#define CRS_ERR_CUDA 3        /* CUDA runtime error (text in crs_last_error) */
#define CRS_ERR_UNSUPPORTED 4 /* mode not available for this mechanism */
#define CRS_ERR_TIMEOUT 5     /* a bounded device or host wait expired */
#define CRS_ERR_NOMECH 6      /* per-state call without a bound mechanism */

/* Evaluation modes of crs_wdot. */
#define CRS_MODE_FP64 0        /* FP64 throughout; <=1e-12 of the reference */
#define CRS_MODE_FP64_STRICT 1 /* FP64 in the reference's operation order */
#define CRS_MODE_MIXED 2       /* FP32 bulk, float-float Kc exponent, FP64 net rate/sum */
/* The arithmetic of CRS_MODE_FP64 / CRS_MODE_MIXED with a fixed thread
 * layout: one state per thread (TPS) or one state per warp (WARP).  The
 * default modes pick the faster layout that fits the mechanism.
 * CRS_MODE_MIXED_TPS also needs every stoichiometric coefficient to be
 * exact in 5 significant bits (integers up to 31, halves, ...); else, like a
 * mechanism whose per-thread columns do not fit, it returns
 * CRS_ERR_UNSUPPORTED and CRS_MODE_MIXED runs the warp layout. */
#define CRS_MODE_FP64_TPS 3
#define CRS_MODE_MIXED_TPS 4
#define CRS_MODE_FP64_WARP 5
#define CRS_MODE_MIXED_WARP 6
/* Mixed-precision rates, then the stoichiometric contraction
 * wdot = q . nu as a BF16 tensor-core GEMM (q split into bf16 hi + lo,
 * scaled per state; terms far outside the scale summed in FP64; FP32
 * accumulation).  For large mechanisms.  No intermediates. */
#define CRS_MODE_GEMM 7
/* The arithmetic of CRS_MODE_MIXED in two passes: net rates of tiles of 32
 * states (all warps of a CTA on one tile) to HBM in FP64, then the species
 * sums.  CRS_MODE_MIXED takes this path when a mechanism's per-thread
 * columns do not fit on chip and no intermediates are asked for.  No
 * intermediates.
 * CRS_MODE_GEMM and the two-pass paths use a workspace owned by the handle,
 * allocated on first use (FP64 rates of up to 2^17 states, <= ~2 GiB, plus
 * 4 bytes per reaction and state for the contraction): calls on one handle
 * take turns on the GPU, whatever their streams. */
#define CRS_MODE_MIXED_TILE 8
/* The arithmetic of CRS_MODE_FP64 in the same two passes (FP64
 * concentrations of the tile in shared memory); CRS_MODE_FP64 takes this
 * path when the per-thread columns do not fit and no intermediates are
 * asked for. */
#define CRS_MODE_FP64_TILE 9

/* ---- mechanism tables ------------------------------------------------ */

/* Load the table blob written by create_rate_subs_gb300 (tables.pack; the
 * 'gb300' CLI target writes it to out/mech.crs) and stage it on the current
 * device.  Replaces the constants the reference bakes into its emitted
 * code (rate_subs.py:226-1391). */
int crs_mech_load(const void *blob, size_t nbytes, crs_mech **out);
int crs_mech_load_file(const char *path, crs_mech **out);
/* Validate a blob and report, without touching a GPU: out[0] device table
 * bytes, out[1] / out[2] bytes the FP64 / mixed kernels stage into shared
 * memory, out[3] / out[4] / out[5] shared memory per 128-thread CTA of
 * CRS_MODE_FP64 / CRS_MODE_MIXED / CRS_MODE_FP64_STRICT (all on chip). */
int crs_mech_inspect(const void *blob, size_t nbytes, int64_t out[6]);
int crs_mech_free(crs_mech *mech);
/* out[0..4] = species, reactions, reversible reactions, pres_mod entries,
 * rate-constant rows. */
int crs_mech_dims(const crs_mech *mech, int64_t out[5]);
const char *crs_last_error(void);
/* Non-finite outputs and device-wait timeouts recorded since the last
 * crs_status_reset on this handle: out[0] = flag bits (1 = table staging
 * timed out, 2 = a tensor-core GEMM wait timed out), out[1] = count of
 * non-finite wdot values.  Synchronises
 * `stream`. */
int crs_status(const crs_mech *mech, void *stream, int32_t out[2]);
int crs_status_reset(const crs_mech *mech, void *stream);

/* ---- batched stages (reference functions, many states) ---------------- */

/* eval_conc over n states (rate_subs.py:1295-1391).  y_N, mw_avg, rho may
 * be NULL; conc is [N][ld]. */
int crs_eval_conc_batch(const crs_mech *mech, int64_t n, const double *T,
                        const double *P, const double *Y, int64_t ld,
                        double *y_N, double *mw_avg, double *rho,
                        double *conc, void *stream);
/* eval_rxn_rates (rate_subs.py:283-704): fwd [R][ld], rev [R_rev][ld]. */
int crs_eval_rxn_rates_batch(const crs_mech *mech, int64_t n, const double *T,
                             const double *P, const double *C, int64_t ld,
                             double *fwd, double *rev, void *stream);
/* get_rxn_pres_mod (rate_subs.py:757-1073): pres_mod [N_pm][ld]. */
int crs_get_rxn_pres_mod_batch(const crs_mech *mech, int64_t n,
                               const double *T, const double *P,
                               const double *C, int64_t ld, double *pres_mod,
                               void *stream);
/* eval_spec_rates (rate_subs.py:1121-1235): wdot [N][ld] (row N-1 is the
 * reference's *dy_N). */
int crs_eval_spec_rates_batch(const crs_mech *mech, int64_t n,
                              const double *fwd, const double *rev,
                              const double *pres_mod, int64_t ld, double *wdot,
                              void *stream);

/* ---- fused hot path --------------------------------------------------- */

/* wdot [N][ld] for n states in one launch: eval_conc -> eval_rxn_rates ->
 * get_rxn_pres_mod -> eval_spec_rates fused, intermediates on chip. */
int crs_wdot(const crs_mech *mech, int64_t n, const double *T,
             const double *P, const double *Y, int64_t ld, double *wdot,
             int mode, void *stream);
/* crs_wdot that also writes the intermediates (any may be NULL): conc
 * [N][ld], fwd [R][ld], rev [R_rev][ld], pres_mod [N_pm][ld].  For
 * per-stage parity checks. */
int crs_wdot_stages(const crs_mech *mech, int64_t n, const double *T,
                    const double *P, const double *Y, int64_t ld,
                    double *wdot, double *conc, double *fwd, double *rev,
                    double *pres_mod, int mode, void *stream);

/* ---- thermo utilities and the ODE right-hand side ------------------------ */

/* eval_h / eval_u / eval_cv / eval_cp over n states (rate_subs.py:1497-1776):
 * which 0 h [J/kg], 1 u [J/kg], 2 cv [J/(kg K)], 3 cp; out [N][ld]. */
int crs_eval_thermo_batch(const crs_mech *mech, int64_t n, const double *T,
                          int64_t ld, int which, double *out, void *stream);
/* eval_conc_rho over n states (rate_subs.py:1396-1490): concentrations and
 * pressure from density; y_N, mw_avg, pres, conc may be NULL. */
int crs_eval_conc_rho_batch(const crs_mech *mech, int64_t n, const double *T,
                            const double *rho, const double *Y, int64_t ld,
                            double *y_N, double *mw_avg, double *pres,
                            double *conc, void *stream);
/* dydt over n states (rate_subs.py:1829-2067): y [N][ld] holds T in row 0
 * and Y_0..Y_{N-2} in rows 1..N-1 (the emitted state vector), dy the same
 * (dT/dt, dY_k/dt).  conv = 0: constant pressure, p_or_rho[n] = P [Pa];
 * conv = 1: constant volume, p_or_rho = rho [kg/m^3] (the form the
 * reference means; its emitted constant-volume text does not compile).
 * wdot comes from `mode` (CRS_MODE_*); the energy equation is FP64.  Uses
 * N*ld (+ ld) doubles of stream-ordered scratch (cudaMallocAsync). */
int crs_dydt(const crs_mech *mech, int64_t n, const double *p_or_rho,
             const double *y, int64_t ld, double *dy, int conv, int mode,
             void *stream);

/* wdot from HOST arrays (same SoA layout and ld as crs_wdot): the batched
 * form of the reference's per-state host functions (rate_subs.py:1297-1299,
 * 287-290, 761-763, 1124-1127 evaluated for every state).  When all four
 * arrays are page-locked host memory that the current device can address
 * (cudaHostAlloc, torch's pin_memory, cudaHostRegister), one launch reads
 * the states and writes wdot in place over the host link (NVLink-C2C on
 * Grace).  Otherwise, or with CRS_HOST_STAGED or'ed into `mode`, states go
 * through device buffers in chunks on two streams owned by the handle, so
 * that the copies of one chunk overlap the kernel of the other (pinned
 * memory is needed for that overlap; the buffers, <= 2 x 256 MB, are
 * allocated on first use and kept by the handle).  Returns when wdot is on
 * the host; calls on one handle are serialised. */
#define CRS_HOST_STAGED 0x100
int crs_wdot_host(const crs_mech *mech, int64_t n, const double *T,
                  const double *P, const double *Y, int64_t ld,
                  double *wdot, int mode);

/* ---- allocation-free contraction (no counterpart in the reference) ----- */

/* The evaluation of crs_wdot(..., CRS_MODE_GEMM, ...) for callers that must
 * not allocate device memory while they run: solvers inside a memory pool
 * or framework that owns every device allocation, code embedded in another
 * runtime whose allocator must not be bypassed, or time-stepping loops that
 * cannot afford cudaMalloc's device synchronisation.  All scratch (the bf16
 * stoichiometric matrix, per-state scale exponents and bf16 rate rows for
 * one chunk of states) lives in one fixed 32 MiB array inside libcrs, which
 * every GPU that loads the library keeps until the process exits; states
 * are processed in chunks that fit it.  Mechanisms whose matrix plus 128
 * states do not fit are refused with CRS_ERR_UNSUPPORTED and a message.
 * The first call on a device looks the array's device address up; make
 * that first call before any stream capture.  Every call rebuilds what must
 * start from zero, but all calls share the one array: calls whose work
 * overlaps on the GPU (other streams, other host threads) race on it and
 * must be serialised by the caller.  Arguments as crs_wdot. */
int crs_wdot_gemm_noalloc(const crs_mech *mech, int64_t n, const double *T,
                          const double *P, const double *Y, int64_t ld,
                          double *wdot, void *stream);

/* ---- building blocks (no counterpart in the reference) ----------------- */

/* D[m*ldd + n] = sum_k A[m*K + k] * B[n*K + k]: bf16 inputs (device,
 * row-major, K contiguous), fp32 output, on the tensor cores (tcgen05, TMA
 * operand staging).  M a multiple of 128, K of 64, N of block_n, block_n in
 * {64, 128, 192, 256}.  status (may be NULL): device int32[2], bit 2 of
 * status[0] is set when a bounded device wait expires. */
int crs_gemm_bf16(const void *A, const void *B, float *D, int64_t M, int64_t N,
                  int64_t K, int64_t ldd, int block_n, int32_t *status,
                  void *stream);

/* ---- surrogate network (no counterpart in the reference) -------------- */

/* A BF16 multilayer perceptron for wdot(T, ln P, ln Y), trained and run on
 * the tensor cores.  Matrices are device, row-major, bf16 unless stated;
 * "pad" sizes are the allocated extents (zero-filled by the caller), the
 * unpadded sizes say which outputs are written.  M (states) pads to 128,
 * K to 64, layer widths to 64 (and to 128 where they are GEMM rows). */
#define CRS_ACT_NONE 0
#define CRS_ACT_SILU 1

/* Z = X[M_pad][K] W[N_pad][K]^T + b; A = act(Z).  Each output may be NULL:
 * Z fp32 [M][ldz] (kept for the backward pass), A bf16 [M][lda] (next
 * layer's input), AT bf16 [N][ldat] (A transposed, for the weight
 * gradient), Y32 fp32 [M][ldy] (the network's output layer). */
int crs_mlp_forward(const void *X, const void *W, const float *b,
                    int64_t M_pad, int64_t N_pad, int64_t K, int64_t M,
                    int64_t N, int act, float *Z, int64_t ldz, void *A,
                    int64_t lda, void *AT, int64_t ldat, float *Y32,
                    int64_t ldy, void *stream);
/* Inference through the whole network in one kernel: Y32[:M][:dims[L]]
 * (fp32, row stride ldy) = layer L-1(... SiLU(layer 0(X))), X bf16
 * [M_pad][pads[0]] (M_pad a multiple of 128).  Layer l: W[l] bf16
 * [pads[l+1]][pads[l]] (zero outside dims), b[l] fp32 [dims[l+1]]; SiLU
 * after every layer but the last.  1 <= L <= 6, every pads[l] a multiple of
 * 64 and <= 256.  Each CTA keeps its 128 states' activations in shared
 * memory between layers.  status (may be NULL): device int32[2], bit 2 of
 * status[0] is set when a bounded device wait expires. */
int crs_mlp_infer(const void *X, int64_t M_pad, int64_t M, int L,
                  const int64_t *dims, const int64_t *pads, const void *const *W,
                  const float *const *b, float *Y32, int64_t ldy, int32_t *status,
                  void *stream);
/* dZprev = (dZ[M_pad][Kout] WT[Nin_pad][Kout]^T) * silu'(Zprev): the
 * gradient through a layer's weights and the previous SiLU; written
 * row-major [M][ld] and transposed [Nin][ldt] (dZprevT may be NULL). */
int crs_mlp_backward_data(const void *dZ, const void *WT, int64_t M_pad,
                          int64_t Nin_pad, int64_t Kout, int64_t M,
                          int64_t Nin, const float *Zprev, int64_t ldz,
                          void *dZprev, int64_t ld, void *dZprevT,
                          int64_t ldt, void *stream);
/* dW[Nout][Nin] (fp32, dense) = dZT[Nout_pad][M_pad] AT[Nin_pad][M_pad]^T,
 * the batch split into `splits` slices whose fp32 partial products
 * (partial: splits * Nout_pad * Nin_pad floats) are summed in slice order.
 * Nout_pad a multiple of 128; M_pad / 64 a multiple of splits. */
int crs_mlp_backward_weight(const void *dZT, const void *AT, int64_t Nout_pad,
                            int64_t Nin_pad, int64_t M_pad, int64_t Nout,
                            int64_t Nin, int splits, float *partial,
                            float *dW, void *stream);
/* out[r] = sum_{i<m} X[r*ld + i] (fp32; the bias gradient from dZT). */
int crs_mlp_row_sums(const void *X, int64_t ld, int64_t rows, int64_t m,
                     float *out, void *stream);
/* loss += scale * sum (Yh - Tg)^2 over [m][n]; dY = 2 scale (Yh - Tg) as
 * bf16 [m][ld] and transposed [n_pad][ldtt] (columns n..n_pad zero). */
int crs_mlp_loss_grad(const float *Yh, int64_t ldy, const float *Tg,
                      int64_t ldt, int64_t m, int64_t n, int64_t n_pad,
                      float scale, void *dY, int64_t ld, void *dYT,
                      int64_t ldtt, float *loss, void *stream);
/* Adam on fp32 master weights p[rows][cols] (moments m, v), bias-corrected
 * for `step` (1-based); refreshes the bf16 copies W [rows][ldw] and
 * WT [cols][ldwt] when not NULL. */
int crs_adam_step(float *p, const float *g, float *m, float *v, int64_t rows,
                  int64_t cols, float lr, float b1, float b2, float eps,
                  int step, void *W, int64_t ldw, void *WT, int64_t ldwt,
                  void *stream);
/* Network input of n states (SoA as crs_wdot): features T, ln P and
 * ln(Y_k + 1e-12) for all nsp species (Y_N = 1 - sum), standardised by
 * mu/sd, as bf16 X [n][ldx] (zero to nfeat_pad; nfeat_pad and ldx
 * multiples of 8, X 16-byte aligned) and XT [nfeat_pad][ldxt]
 * (may be NULL).  out_of_box[i] = 1 when a raw feature is outside
 * [lo, hi] (lo/hi/out_of_box may be NULL); raw (may be NULL) receives the
 * unstandardised features [n][2 + nsp]. */
int crs_surrogate_features(int64_t n, const double *T, const double *P,
                           const double *Y, int64_t ld, int nsp,
                           const float *mu, const float *sd, const float *lo,
                           const float *hi, void *X, int64_t ldx, void *XT,
                           int64_t ldxt, int nfeat_pad,
                           unsigned char *out_of_box, float *raw,
                           void *stream);
/* wdot[k][i] = s_k sign(y) expm1(|y|) in FP64 from the network output
 * Yh[i][k], the species scale given as s_k = scale_m[k] * 2^scale_e[k]
 * (fp32 mantissa, int exponent: scales exceed the fp32 range).
 * fallback[i] = 1 when out_of_box[i] or the element residual
 * max_e |sum_k a_ek w_k| / sum_k a_ek (|w_k| + s_k) exceeds tol; cons
 * [nelem][nsp] (nelem <= 8) = a_ek s_k / max_j a_ej s_j, a_ek the atoms
 * of element e in species k. */
int crs_surrogate_output(int64_t n, const float *Yh, int64_t ldy, int nsp,
                         const float *scale_m, const int *scale_e,
                         const float *cons, int nelem, float tol,
                         const unsigned char *out_of_box, double *wdot,
                         int64_t ld, unsigned char *fallback, void *stream);
/* Two-network form of crs_surrogate_output with an error gate (no
 * counterpart in the reference).  Ya and Yb are two networks' outputs
 * (same layout); the served y is their mean.  Gate score of state i:
 * g = dweight log10(D + 1e-4) + est[i * lde], D = max_k |Ya[i][k] -
 * Yb[i][k]| (the networks' disagreement) and est the output of an error
 * network trained to predict log10 of the served error + 1e-4 (may be NULL:
 * term omitted).  fallback[i] = 1 as in crs_surrogate_output, or when
 * g > stol (NaN included).  gate (may be NULL) receives g. */
int crs_surrogate_output2(int64_t n, const float *Ya, const float *Yb,
                          int64_t ldy, int nsp, const float *scale_m,
                          const int *scale_e, const float *cons, int nelem,
                          float tol, float dweight, const float *est,
                          int64_t lde, float stol,
                          const unsigned char *out_of_box, double *wdot,
                          int64_t ld, unsigned char *fallback, float *gate,
                          void *stream);
/* The networks' disagreement as an input of the error network (no
 * counterpart in the reference): X[i * ldx + col] (bf16 feature rows) =
 * (log10(D + 1e-4) - mu) / sd, D as in crs_surrogate_output2. */
int crs_surrogate_disagreement(int64_t n, const float *Ya, const float *Yb,
                               int64_t ldy, int nsp, float mu, float sd,
                               void *X, int64_t ldx, int col, void *stream);
/* idx[0..count) = the i < n with flag[i] != 0, in no particular order
 * (count: device int64, set by the call). */
int crs_select(int64_t n, const unsigned char *flag, int64_t *idx,
               int64_t *count, void *stream);
/* Copy the m states idx[j] into compact SoA arrays (rows = species rows of
 * Y), and compact wdot rows back to their places. */
int crs_gather_states(int64_t m, const int64_t *idx, const double *T,
                      const double *P, const double *Y, int64_t ld, int rows,
                      double *Tc, double *Pc, double *Yc, int64_t ldc,
                      void *stream);
int crs_scatter_wdot(int64_t m, const int64_t *idx, const double *Wc,
                     int64_t ldc, int rows, double *W, int64_t ld,
                     void *stream);

/* ---- per-state drop-in (the reference's emitted signatures) ----------- */

/* The reference emits these as pure host functions with the mechanism
 * compiled in; an integrator calls them once per state, often from many
 * OpenMP threads.  Here they evaluate a mechanism's host table image on the
 * calling thread in FP64, in the reference's operation order
 * (include/crs_eval.h, compiled without floating-point contraction): the
 * results equal the emitted C's bit for bit.  They lock nothing, launch
 * nothing, need no GPU, and may run on any number of threads at once.
 *
 * The mechanism is the calling thread's own binding (crs_bind_thread) when
 * it has one, else the process-wide binding (crs_bind).  A handle must stay
 * loaded while calls may use it; crs_mech_free removes it from the
 * process-wide binding and from the calling thread's.  Without a binding
 * the outputs are left untouched and crs_last_error() says so. */

/* Host-only load: the table image for the per-state functions and the
 * crs_state_* calls, without a GPU.  Batched entry points refuse such a
 * handle (CRS_ERR_ARG).  Free with crs_mech_free. */
int crs_mech_load_host(const void *blob, size_t nbytes, crs_mech **out);
/* The table image of a blob (host only), for code that compiles it into a
 * program (the per-state device functions of include/crs_device.cuh):
 * sizes[0] = image bytes, sizes[1] = int32 words of crs::ImgLayout
 * (include/crs_tables.h).  img / layout may be NULL (sizes only); else they
 * receive the image and the layout words. */
int crs_mech_image(const void *blob, size_t nbytes, void *img, size_t img_cap,
                   int32_t *layout, size_t layout_cap, size_t sizes[2]);
/* Process-wide mechanism of the functions below (NULL unbinds). */
int crs_bind(const crs_mech *mech);
/* The calling thread's own mechanism, ahead of the process-wide one (NULL
 * returns the thread to the process-wide binding). */
int crs_bind_thread(const crs_mech *mech);

/* rate_subs.py:1297-1299 (chem_utils.h) */
void eval_conc(const double T, const double pres, const double *y,
               double *y_N, double *mw_avg, double *rho, double *conc);
/* rate_subs.py:287-290 (rates.h) */
void eval_rxn_rates(const double T, const double pres, const double *C,
                    double *fwd_rxn_rates, double *rev_rxn_rates);
/* rate_subs.py:761-763 (rates.h; emitted only when N_pm > 0) */
void get_rxn_pres_mod(const double T, const double pres, const double *C,
                      double *pres_mod);
/* rate_subs.py:1124-1127 (rates.h) */
void eval_spec_rates(const double *fwd_rates, const double *rev_rates,
                     const double *pres_mod, double *sp_rates, double *dy_N);

/* rate_subs.py:1497-1776 (chem_utils.h): per-species h, u, cv, cp at T */
void eval_h(const double T, double *h);
void eval_u(const double T, double *u);
void eval_cv(const double T, double *cv);
void eval_cp(const double T, double *cp);
/* rate_subs.py:1396-1490 (chem_utils.h) */
void eval_conc_rho(const double T, const double rho, const double *y,
                   double *y_N, double *mw_avg, double *pres, double *conc);
/* rate_subs.py:1829-2067 (dydt.h): y = [T, Y_0 .. Y_{N-2}], dy the same;
 * `pres` is the pressure (constant pressure, the default) or the density
 * after crs_dydt_form(1) (constant volume), as the emitted -DCONP / -DCONV
 * builds read it.  The constant-volume form takes the pressure and the
 * concentrations from eval_conc_rho (the reference's constant-volume text
 * does not compile, rate_subs.py:1967-1969, 2024-2025). */
void dydt(const double t, const double pres, const double *y, double *dy);
/* Form of the per-state dydt, process-wide: 0 constant pressure, 1
 * constant volume. */
int crs_dydt_form(int conv);

/* The same functions with the mechanism passed explicitly (no binding) and
 * an error code returned: CRS_ERR_ARG for a NULL handle or array. */
int crs_state_eval_conc(const crs_mech *mech, double T, double pres, const double *y,
                        double *y_N, double *mw_avg, double *rho, double *conc);
int crs_state_eval_rxn_rates(const crs_mech *mech, double T, double pres, const double *C,
                             double *fwd, double *rev);
int crs_state_get_rxn_pres_mod(const crs_mech *mech, double T, double pres,
                               const double *C, double *pres_mod);
int crs_state_eval_spec_rates(const crs_mech *mech, const double *fwd, const double *rev,
                              const double *pres_mod, double *sp_rates, double *dy_N);
/* which: 0 h, 1 u, 2 cv, 3 cp; out [N] */
int crs_state_eval_thermo(const crs_mech *mech, int which, double T, double *out);
int crs_state_eval_conc_rho(const crs_mech *mech, double T, double rho, const double *y,
                            double *y_N, double *mw_avg, double *pres, double *conc);
/* conv 0: p_or_rho = P (constant pressure); 1: p_or_rho = rho */
int crs_state_dydt(const crs_mech *mech, int conv, double p_or_rho, const double *y,
                   double *dy);

#ifdef __cplusplus
}
#endif

#endif /* CRS_H */
