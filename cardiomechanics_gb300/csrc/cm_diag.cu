// Pipe-peak measurement kernels: the FP64 plain kernels are bound by the FP64 pipe, whose
// GB300 rate the measured copy-bandwidth and GEMM peaks do not give. Each thread runs 8 independent FMA
// chains (enough to cover the pipe latency at full occupancy); the result is written so the
// chains are not dead code.
#include <algorithm>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/cardiomech_gb300_diag.h"
#include "cm_bulk.cuh"
#include "cm_fp64_math.cuh"
#include "cm_umma.cuh"

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

// out[6 i + ...]: exp64(x), log64(y), div64(x, y), then the library's exp(x), log(y), x / y
__global__ void fp64_math_kernel(const double *__restrict__ x, const double *__restrict__ y, int64_t n,
                                 double *__restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double a = x[i], b = y[i];
    double *o = out + 6 * i;
    o[0] = cm::fp64::exp64(a);
    o[1] = cm::fp64::log64(b);
    o[2] = cm::fp64::div64(a, b);
    o[3] = exp(a);
    o[4] = log(b);
    o[5] = a / b;
  }
}

// The compensated-pair conversions of the mixed kernels (integer forms on the device)
__global__ void pair_kernel(const double *__restrict__ x, int64_t n, float *__restrict__ hi, float *__restrict__ lo,
                            double *__restrict__ back, double *__restrict__ widened) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const cm::Acc a = cm::acc_from_double(x[i]);
    hi[i] = a.hi;
    lo[i] = a.lo;
    back[i] = cm::acc_to_double(a);
    widened[i] = cm::f32_widen((float)x[i]);
  }
}

}  // namespace

// D (128 x N, FP32) = A (128 x K) * B (N x K)^T on the tcgen05 tensor core, operands staged in
// shared memory in the learned macro step's layout, accumulator in TMEM read back with
// tcgen05.ld: one tile, one block of 128 threads (thread i owns row i = TMEM lane i).
__global__ void __launch_bounds__(128) umma_tile_kernel(const __nv_bfloat16 *__restrict__ A,
                                                        const __nv_bfloat16 *__restrict__ B, int N, int K,
                                                        float *__restrict__ D, unsigned int *err) {
  using namespace cm;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  __nv_bfloat16 *sA = (__nv_bfloat16 *)smem;
  __nv_bfloat16 *sB = sA + 128 * K;
  const int warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < 128 * K; i += 128) sA[umma::kmajor_index(i / K, i % K, K)] = A[i];
  for (int i = threadIdx.x; i < N * K; i += 128) sB[umma::kmajor_index(i / K, i % K, K)] = B[i];
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) umma::tmem_alloc(&tslot, 128);
  umma::fence_smem_to_async();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tslot;
  if (threadIdx.x == 0) {
    const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB), sbo = (uint32_t)(K / 8) * 128u;
    const uint32_t idesc = umma::idesc_bf16_f32(128, N);
    for (int s = 0; s < K / 16; s++)
      umma::mma_bf16(tmem, umma::smem_desc(a0 + s * 256u, 128u, sbo), umma::smem_desc(b0 + s * 256u, 128u, sbo),
                     idesc, s > 0);
    umma::commit(&bar);
  }
  bool ok = mbar_wait(&bar, 0);
  ok = __syncthreads_and(ok);
  umma::fence_after_sync();
  if (ok) {
    for (int c0 = 0; c0 < N; c0 += 32) {
      float v[32];
      umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int j = 0; j < 32; j++) D[(size_t)threadIdx.x * N + c0 + j] = v[j];
    }
  } else {
    if (threadIdx.x == 0) atomicOr(err, 1u);
    mbar_wait(&bar, 0);  // one more bounded wait for the MMAs before their TMEM is released
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_free(tmem, 128);
}

extern "C" int cm_diag_umma_tile(const void *A, const void *B, int n, int k, float *D, void *stream) {
  if (!A || !B || !D || (n != 32 && n != 64 && n != 128) || (k != 32 && k != 64 && k != 128)) return CM_DIAG_ERR;
  const size_t smem = (size_t)(128 + n) * k * sizeof(__nv_bfloat16);
  if (cudaFuncSetAttribute(umma_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return CM_DIAG_ERR;
  unsigned int *err = nullptr;
  if (cudaMalloc(&err, sizeof(unsigned int)) != cudaSuccess) return CM_DIAG_ERR;
  cudaStream_t s = (cudaStream_t)stream;
  unsigned int h = 0;
  cudaError_t e = cudaMemsetAsync(err, 0, sizeof(unsigned int), s);
  if (e == cudaSuccess) {
    umma_tile_kernel<<<1, 128, smem, s>>>((const __nv_bfloat16 *)A, (const __nv_bfloat16 *)B, n, k, D, err);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, err, sizeof(unsigned int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(err);
  return (e == cudaSuccess && h == 0) ? 0 : CM_DIAG_ERR;
}

extern "C" int cm_diag_fma_peak(int fp64, double *tflops, void *stream) {
  if (!tflops) return CM_DIAG_ERR;
  return fp64 ? measure<double>(tflops, stream, 4096) : measure<float>(tflops, stream, 65536);
}

extern "C" int cm_diag_fp64_math(const double *x, const double *y, int64_t n, double *out, void *stream) {
  if (!x || !y || !out || n < 0) return CM_DIAG_ERR;
  if (n == 0) return 0;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
  fp64_math_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(x, y, n, out);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  return e == cudaSuccess ? 0 : CM_DIAG_ERR;
}

extern "C" int cm_diag_pair_convert(const double *x, int64_t n, float *hi, float *lo, double *back, double *widened,
                                    void *stream) {
  if (!x || !hi || !lo || !back || !widened || n < 0) return CM_DIAG_ERR;
  if (n == 0) return 0;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
  pair_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(x, n, hi, lo, back, widened);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  return e == cudaSuccess ? 0 : CM_DIAG_ERR;
}
