// Kernel launch interface between the C-ABI layer (cm_capi.cpp) and the CUDA kernels
// (cm_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "cm_common.cuh"

namespace cm {

// Device memory of one batch of cells of one model in one precision.
//   FP64:  s64[k * ld + c], k < n_state (SOA order of the model)
//   MIXED: s32[k * ld + c] for the FP32 variables, s64[k * ld + c] for the FP64 accumulators
//          TT2  FP32: m h j xr1 xr2 xs r s d f f2 fCa Rq Ca_i CaSS     FP64: CaSR Na_i K_i
//          CRN  FP32: h j oi ui Xr Xs u v w m oa ua d f f_Ca Ca_i Ca_TRPN  FP64: Ca_up Ca_rel Na_i K_i
struct DevBatch {
  int model = 0;      // 2 Courtemanche, 5 TenTusscher2
  int precision = 0;  // 0 FP64, 1 mixed
  int64_t n = 0, ld = 0;
  double *s64 = nullptr;
  float *s32 = nullptr;
  const double *rows64 = nullptr, *eca64 = nullptr;
  const float *rows32 = nullptr, *eca32 = nullptr;
  const void *het[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // double* (FP64) / float* (mixed)
  uint32_t *audit_cell = nullptr;
  unsigned int *audit_or = nullptr;
  double *diag = nullptr;  // TT2 FP64: 17 x ld diagnostic currents; CRN FP64: 1 x ld (I_SAC)
  int variant = 0, grid_mode = 0;  // launch shape chosen by cm_batch_autotune
  TT2Consts<double> tt2_64;
  TT2Consts<float> tt2_32;
  CRNConsts<double> crn_64;
  CRNConsts<float> crn_32;
};

// Per-launch inputs/outputs (device pointers).
struct StepIO {
  const double *vm = nullptr;  // Vm in
  double *vm_out = nullptr;    // fused Vm += dV (run mode) or nullptr
  double *dvm = nullptr;       // dV out (step mode) or nullptr
  const double *iext = nullptr;  // per-cell i_ext, or nullptr
  double iext_uniform = 0.0;     // used when iext == nullptr and tb_cell == nullptr
  const double *stretch = nullptr;
  // per-cell stimulus protocol (run mode with per-cell first stimulus times)
  double *tb_cell = nullptr;
  double t = 0.0, textlen = 0.0, bcl = 0.0, amp = 0.0;
  double vm_range = 0.0;  // > 0: flag cells whose new |Vm| exceeds it (fused update only)
};

int n_fp32_vars(int model);
int n_fp64_vars(int model, int precision);

// variant: mixed-kernel launch shape (0 .. n_shape_variants()-1); grid_mode 0 = one thread
// per cell, k > 0 = grid-stride loop over k blocks per SM.
cudaError_t launch_step(const DevBatch &b, const StepIO &io, int variant, int grid_mode, cudaStream_t s);
int n_shape_variants();
// Copies Vm[probe[i]] into out[i * stride + k] for i < n_probe.
cudaError_t launch_probe(const double *vm, const int64_t *probe, int64_t n_probe, double *out, int64_t stride,
                         int64_t k, cudaStream_t s);
int sm_count();

}  // namespace cm
