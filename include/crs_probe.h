/*
 * crs_probe.h -- measurement helper of libcrs (no counterpart in the
 * reference; not part of the evaluation API).
 *
 * bench.py takes its FP64 roofline denominators from this probe, because
 * the measured peaks cover HBM bandwidth and the bf16 tensor rate
 * only.
 */
#ifndef CRS_PROBE_H
#define CRS_PROBE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Issue-rate probes of the current device, operations per second:
 * out[0] FP64 FMA, out[1] CUDA double exp(), out[2] FP32 FMA, out[3] SFU
 * ex2.approx, out[4] the table exponential of the FP64 kernels (9 FP64
 * instructions each).  out[0] / out[4] is the FP64-pipe price of one
 * exponential in the roofline of the FP64 kernels. */
int crs_probe_peaks(double out[5]);

#ifdef __cplusplus
}
#endif

#endif /* CRS_PROBE_H */
