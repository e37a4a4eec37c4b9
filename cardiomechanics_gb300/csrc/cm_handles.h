// Handle structures and shared helpers of the C ABI implementation (cm_capi.cpp, cm_sur_api.cpp).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/cardiomech_gb300.h"
#include "cm_launch.h"
#include "cm_params.h"

struct cm_params_s {
  cm::ParamSet ps;
};

struct cm_batch_s {
  cm::ParamSet ps;
  cm::DevBatch d;
  cudaStream_t stream = nullptr;
  void *state_mem = nullptr;   // one allocation: FP64 block then FP32 block
  void *table_mem = nullptr;   // rows/eca in FP64 (FP64 batches) or FP32 (mixed)
  void *het_mem[6] = {};
  uint32_t *audit_cell = nullptr;
  unsigned int *audit_or = nullptr;
  double *diag = nullptr;
  bool diag_on = false;
  // staging buffers for host arrays, grown on demand
  double *stage[4] = {};
  int64_t stage_n = 0;
  double *tb_cell = nullptr;
  float *vm_planes = nullptr;  // mixed batches: Vm as hi/lo planes during fused runs (2 x n)
  float *vm_planes2 = nullptr; // the second pair of Vm planes of coupled runs (cm_batch_run_diffuse)
  int64_t *probe_idx = nullptr;
  int64_t probe_cap = 0;
  double *probe_out = nullptr;
  int64_t probe_out_cap = 0;
};


// A monodomain operator in 32-row slices (cm_diffusion.cpp): entry k of row 32 s + r at
// sl_ptr[s] + 32 k + r, each row's entries in CSR order, padding entries value 0 / own column.
struct cm_diffusion_s {
  int64_t n = 0, n_slices = 0, entries = 0;
  int wmax = 0;  // widest slice
  int64_t *sl_ptr = nullptr;  // n_slices + 1 entry offsets
  int32_t *sl_col = nullptr;
  double *val64 = nullptr;
  float *val32 = nullptr;     // off-diagonal entries only (the diagonal is in rowsum32)
  float *rowsum32 = nullptr;  // sum of the row's entries, formed in FP64
  double *scale64 = nullptr;
  float *scale32 = nullptr;
  double uniform = 0.0;
  void fill(cm::StepIO &io, bool fp32) const {
    io.sl_ptr = sl_ptr;
    io.sl_col = sl_col;
    io.sl_val64 = fp32 ? nullptr : val64;
    io.sl_val32 = fp32 ? val32 : nullptr;
    io.rowsum32 = rowsum32;
    io.dscale64 = scale64;
    io.dscale32 = scale32;
    io.dscale_u = uniform;
    io.sl_wmax = wmax;
  }
};

namespace cm {

std::string &last_error();

inline int fail(int code, const std::string &msg) {
  last_error() = msg;
  return code;
}

inline int cuda_fail(cudaError_t e, const char *what) {
  last_error() = std::string(what) + ": " + cudaGetErrorString(e);
  return CM_ERR_CUDA;
}

#define CK(call)                                        \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cm::cuda_fail(e_, #call); \
  } while (0)

inline bool is_device_ptr(const void *p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// The device's address of page-locked host memory (cudaHostAlloc / cudaHostRegister, mapped
// into the device's address space), or nullptr for any other pointer. Kernels read and write such
// memory directly over the host link, with no staging copy.
inline double *mapped_host_ptr(void *p) {
  if (!p) return nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  return static_cast<double *>(at.devicePointer);
}

// Grows the batch's four staging buffers to n doubles each.
inline int ensure_stage(cm_batch_s *b, int64_t n) {
  if (b->stage_n >= n) return CM_OK;
  for (auto &p : b->stage) {
    if (p) cudaFree(p);
    p = nullptr;
  }
  b->stage_n = 0;
  for (auto &p : b->stage) CK(cudaMalloc(&p, std::max<int64_t>(n, 1) * sizeof(double)));
  b->stage_n = n;
  return CM_OK;
}

// The driver's per-cell first stimulus times for a run: a device array is used (and advanced)
// in place; a host array is copied to the batch's own buffer, which the run advances.
inline int per_cell_times(cm_batch_s *b, const double *src, cudaStream_t s, double **out) {
  if (is_device_ptr(src)) {
    *out = const_cast<double *>(src);
    return CM_OK;
  }
  if (!b->tb_cell) CK(cudaMalloc(&b->tb_cell, std::max<int64_t>(1, b->d.n) * sizeof(double)));
  CK(cudaMemcpyAsync(b->tb_cell, src, b->d.n * sizeof(double), cudaMemcpyHostToDevice, s));
  *out = b->tb_cell;
  return CM_OK;
}

}  // namespace cm
