/* cardiomech_gb300_diag.h -- measurement helper of libcmgb300.so (no counterpart in the
 * reference, which has no GPU code). The FP64 cell-model kernels are bound by the FP64
 * pipe; this gives the measured denominator of their roofline. */
#ifndef CARDIOMECH_GB300_DIAG_H
#define CARDIOMECH_GB300_DIAG_H
#ifdef __cplusplus
extern "C" {
#endif

#define CM_DIAG_ERR (-5)

/* Dense FMA throughput of the current device in TFLOP/s (2 flops per FMA), FP64 (fp64 != 0)
 * or FP32, measured with independent FMA chains on the given stream (NULL = default). */
int cm_diag_fma_peak(int fp64, double *tflops, void *stream);

#ifdef __cplusplus
}
#endif
#endif
