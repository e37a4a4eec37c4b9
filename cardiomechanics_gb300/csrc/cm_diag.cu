// Pipe-peak measurement kernels: the FP64 plain kernels are bound by the FP64 pipe, whose
// GB300 rate is not in the driver's measured peaks. Each thread runs 8 independent FMA
// chains (enough to cover the pipe latency at full occupancy); the result is written so the
// chains are not dead code.
#include <cuda_runtime.h>

#include "../../include/cardiomech_gb300_diag.h"

namespace {

template <typename R>
__global__ void __launch_bounds__(256) fma_chains(R *out, int iters, R a, R b) {
  R x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = (R)(threadIdx.x + k);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = x[k] * a + b;
  }
  R s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  if (s == (R)1.2345) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // practically never
}

template <typename R>
int measure(double *tflops, void *stream, int iters) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return CM_DIAG_ERR;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256;
  R *out = nullptr;
  cudaEvent_t e0, e1;
  if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(R)) != cudaSuccess) return CM_DIAG_ERR;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaStream_t s = (cudaStream_t)stream;
  fma_chains<R><<<blocks, threads, 0, s>>>(out, iters / 10, (R)0.999999, (R)1e-7);
  cudaEventRecord(e0, s);
  fma_chains<R><<<blocks, threads, 0, s>>>(out, iters, (R)0.999999, (R)1e-7);
  cudaEventRecord(e1, s);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess || ms <= 0) return CM_DIAG_ERR;
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return 0;
}

}  // namespace

extern "C" int cm_diag_fma_peak(int fp64, double *tflops, void *stream) {
  if (!tflops) return CM_DIAG_ERR;
  return fp64 ? measure<double>(tflops, stream, 4096) : measure<float>(tflops, stream, 65536);
}
