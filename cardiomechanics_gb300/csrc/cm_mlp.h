// The surrogate's MLP on the tensor cores (cm_mlp.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace cm {

struct Mlp {
  int n_in = 0, H = 0, n_out = 0, in_pad = 0, out_pad = 0;
  cudaStream_t stream = nullptr;
  // FP32 master parameters, gradients, Adam moments; BF16 operand copies and transposes
  float *w = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;
  __nv_bfloat16 *wb = nullptr, *wt = nullptr;
  size_t off[6] = {}, size[6] = {}, n_params = 0;  // W1 b1 W2 b2 W3 b3 (padded shapes)
  uint64_t version = 0;  // advanced by every change of the weights (reset, sync_bf16, adam_step)
  float *loss = nullptr;
  void *ws = nullptr;
  float *part = nullptr;  // partial sums of the split weight-gradient GEMMs and column sums
  unsigned int *tc_err = nullptr;  // set by a tensor-core GEMM whose bounded wait ran out
  // cudaErrorLaunchTimeout if a tensor-core GEMM since the last check ran out of its wait
  cudaError_t check_tc();
  int ws_rows = 0;
  int step = 0;

  struct Buffers {
    __nv_bfloat16 *X, *XT, *H1, *H1T, *H2, *H2T, *dZ1, *dZ1T, *dZ2, *dZ2T, *dY, *dYT;
    float *Y, *Xf, *Tf;
  };

  cudaError_t init(int n_in, int n_hidden, int n_out, uint64_t seed, cudaStream_t s);
  // fresh Glorot-uniform weights from seed, zero biases, optimiser state cleared
  cudaError_t reset(uint64_t seed);
  void release();
  cudaError_t sync_bf16();  // after host-side weight changes
  // X: n x n_in (device, FP32); Y: n x n_out (device, FP32)
  cudaError_t forward(const float *X, int64_t n, float *Y);
  // Bytes of scratch forward_in_scratch needs per row of a 64-row-padded batch: packed BF16
  // inputs, both BF16 hidden activations and the padded FP32 outputs.
  size_t forward_scratch_bytes_per_row() const;
  // forward() with its intermediates in caller-provided device scratch (256-byte aligned, at
  // least rows_pad x forward_scratch_bytes_per_row() bytes, rows_pad = n rounded up to 64);
  // allocates nothing. Every byte of scratch it reads it has written first.
  cudaError_t forward_in_scratch(void *scratch, const float *X, int64_t n, float *Y);
  // forward + backward on n samples (device FP32 X, T); gradients in g, mean loss in *loss
  cudaError_t loss_grad(const float *X, const float *T, int64_t n);
  cudaError_t adam_step(float lr, float b1, float b2, float eps);
  // minibatch Adam over a device dataset of n samples
  cudaError_t train(const float *X, const float *T, int64_t n, int batch, int steps, float lr, uint64_t seed,
                    float *final_loss);

 private:
  cudaError_t workspace(int rows);
  Buffers buffers(int rows) const;
  cudaError_t forward_rows(const Buffers &B, int rows);
};

}  // namespace cm
