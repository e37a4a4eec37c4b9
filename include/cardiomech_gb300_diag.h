/* cardiomech_gb300_diag.h -- measurement helper of libcmgb300.so (no counterpart in the
 * reference, which has no GPU code). The FP64 cell-model kernels are bound by the FP64
 * pipe; this gives the measured denominator of their roofline. */
#ifndef CARDIOMECH_GB300_DIAG_H
#define CARDIOMECH_GB300_DIAG_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define CM_DIAG_ERR (-5)

/* Dense FMA throughput of the current device in TFLOP/s (2 flops per FMA), FP64 (fp64 != 0)
 * or FP32, measured with independent FMA chains on the given stream (NULL = default). */
int cm_diag_fma_peak(int fp64, double *tflops, void *stream);

/* One 128 x n tile D = A * B^T on the tcgen05 tensor core (BF16 operands, FP32 accumulation in
 * tensor memory), with the operand layout and descriptors of the learned macro step: A is
 * 128 x k and B n x k, row-major BF16 device arrays; D is 128 x n FP32 (device). n in {32, 64,
 * 128}, k in {32, 64, 128}. Checks the tensor-core path against a host product. */
int cm_diag_umma_tile(const void *A, const void *B, int n, int k, float *D, void *stream);

/* Test hook for the bounded waits (a cm_batch_t as `batch`): the batch's next launches of the
 * staged pipeline (mixed batches, launch shapes 7 and 8) and of the learned macro step issue no
 * bulk copy for tile skip_tile (-1: none), so the wait for that tile's data runs out, and every
 * such wait gives up after spin_limit polls (0: the default, 2^26). A wait that runs out sets
 * CM_AUDIT_TIMEOUT in the batch's audit mask; the kernel then waits (bounded) for the copies it
 * did issue, frees what it holds and returns, leaving that tile's work undone. Nothing faults
 * or hangs. Call with (-1, 0) to restore normal operation. */
int cm_diag_batch_wait_check(void *batch, int64_t skip_tile, uint32_t spin_limit);

/* Rows of allocated workspace a network (cm_mlp_t) holds for its forward and training passes:
 * lets a test see that an entry point which must not allocate left it unchanged. */
int cm_diag_mlp_workspace_rows(void *mlp, int64_t *rows);

/* The FP64 exp, log and division of the FP64 cell-model steps (table-driven exp and log, Newton
 * division from the approximate reciprocal) beside the CUDA library's, on device arrays x, y of
 * n values: out (device, 6 n values) holds, per i, exp64(x), log64(y), div64(x, y), exp(x),
 * log(y), x / y. For accuracy tests. */
int cm_diag_fp64_math(const double *x, const double *y, int64_t n, double *out, void *stream);

/* The compensated FP32 pair conversions of the mixed kernels, on device arrays of n values: hi,
 * lo = the pair of x (FP32 head rounded to nearest, FP32 remainder), back = hi + lo in FP64,
 * widened = (double)(float)x, computed with the integer bit-pattern forms the kernels use.
 * For tests. */
int cm_diag_pair_convert(const double *x, int64_t n, float *hi, float *lo, double *back, double *widened,
                         void *stream);

#ifdef __cplusplus
}
#endif
#endif
