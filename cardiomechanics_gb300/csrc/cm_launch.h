// Kernel launch interface between the C-ABI layer (cm_capi.cpp) and the CUDA kernels
// (cm_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "cm_common.cuh"

namespace cm {

// Device memory of one batch of cells of one model in one precision.
//   FP64:  s64[k * ld + c], k < n_state (SOA order of the model)
//   MIXED: s32[k * ld + c], every variable a 32-bit word; compensated accumulators take two
//          (hi, lo) planes:
//          TT2  m h j xr1 xr2 xs r s d f f2 fCa Rq Ca_i CaSS | CaSR Na_i K_i (hi, lo each)
//          CRN  h j oi ui Xr Xs u v w m oa ua d f f_Ca Ca_i Ca_TRPN | Ca_up Ca_rel Na_i K_i (hi, lo)
//          ORd  the 35 states of ORDState other than the six below, in that order |
//               Na_i Na_ss K_i K_ss Ca_nsr Ca_jsr (hi, lo)
//          Tom  the 38 states of TOMState other than the same six, in that order | the six (hi, lo)
struct alignas(16) DevBatch {
  int model = 0;      // 2 Courtemanche, 5 TenTusscher2, 12 OHaraRudy, 14 Tomek
  int precision = 0;  // 0 FP64, 1 mixed
  int64_t n = 0, ld = 0;
  double *s64 = nullptr;
  float *s32 = nullptr;
  const double *rows64 = nullptr, *eca64 = nullptr;
  const float *rows32 = nullptr, *eca32 = nullptr;
  const void *het[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // double* (FP64) / float* (mixed)
  uint32_t *audit_cell = nullptr;
  unsigned int *audit_or = nullptr;
  double *diag = nullptr;  // FP64 only: TT2 and ORd 17 x ld diagnostic currents; CRN 1 x ld (I_SAC); Tomek 40 x ld
  int variant = 0, grid_mode = 0;  // launch shape chosen by cm_batch_autotune
  // Bounded waits of the bulk-copy kernels: polls before a wait gives up (CM_AUDIT_TIMEOUT).
  uint32_t spin_limit = 1u << 26;
  // Test hook (cm_diag_batch_wait_check): the staged pipeline and the learned macro step issue
  // no copy for this tile, so the wait for it runs out; -1: every tile is copied.
  int64_t fault_skip_tile = -1;
  TT2Consts<double> tt2_64;
  TT2Consts<float> tt2_32;
  CRNConsts<double> crn_64;
  CRNConsts<float> crn_32;
  ORDConsts<double> ord_64;
  ORDConsts<float> ord_32;
  TOMConsts<double> tom_64;
  TOMConsts<float> tom_32;
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
  // mixed batches in run mode: Vm as compensated FP32 planes (vm_hi + vm_lo), updated in place
  float *vm_hi = nullptr, *vm_lo = nullptr;
  double vm_range = 0.0;  // > 0: flag cells whose new |Vm| exceeds it (fused update only)
  // fused update only: activation times (acCELLerate.cpp:1997-2005): a cell whose entry is still
  // -1 and whose new Vm reaches act_threshold gets act_time
  double *act = nullptr;
  double act_time = 0.0, act_threshold = 0.0;
  // monodomain coupling (cm_batch_run_diffuse): i_ext += scale * (A x), A in 32-row slices
  // (slice s: entries sl_ptr[s] .. sl_ptr[s+1], entry k of row 32 s + r at sl_ptr[s] + 32 k + r).
  // FP64 batches: x = vm (the previous step's Vm; the new one goes to vm_out), sum in CSR order.
  // Mixed batches: x = the previous step's hi plane, rowsum32 * x_l + sum val32 (x_j - x_l)
  // (val32 holds the off-diagonal entries only); the new Vm goes to vm_hi_out / vm_lo_out.
  const int64_t *sl_ptr = nullptr;
  const int32_t *sl_col = nullptr;
  const double *sl_val64 = nullptr;
  const float *sl_val32 = nullptr, *rowsum32 = nullptr;
  const double *dscale64 = nullptr;  // per node, or nullptr for dscale_u
  const float *dscale32 = nullptr;
  double dscale_u = 0.0;
  int sl_wmax = 0;  // widest slice (entries per row); rowsum32 / dscale32 padded to whole 256-cell tiles
  float *vm_hi_out = nullptr, *vm_lo_out = nullptr;  // mixed: new Vm planes (nullptr: in place)
};

// Coupled runs of mixed batches through the staged kernels (cm_staged.cu): the tile's operator
// slices are staged with its state; the producer/consumer pipeline unless a TT2 / Courtemanche
// batch chose the double-buffered kernel (variant 5 or 6). false when the batch or the operator
// does not fit (then the register kernel runs).
bool coupled_staged_supported(const DevBatch &b, const StepIO &io);
cudaError_t launch_coupled_staged(const DevBatch &b, const StepIO &io, int variant, cudaStream_t s);

// y = scale * (A x) for a coupling operator (cm_diffusion_apply); io carries the operator.
cudaError_t launch_diffusion_apply(const StepIO &io, const double *x, double *y, int64_t n, cudaStream_t s);

int n_fp32_vars(int model);
int n_fp64_vars(int model, int precision);

// variant: mixed-kernel launch shape (0 .. n_shape_variants()-1); grid_mode 0 = one thread
// per cell, k > 0 = grid-stride loop over k blocks per SM.
cudaError_t launch_step(const DevBatch &b, const StepIO &io, int variant, int grid_mode, cudaStream_t s);
int n_shape_variants();
// Shared-memory-staged mixed kernels (cm_staged.cu): fused runs only (Vm planes, uniform
// stimulus, leading dimension a multiple of 256, planes lo = hi + ld).
bool staged_supported(const DevBatch &b, const StepIO &io);
cudaError_t launch_staged(const DevBatch &b, const StepIO &io, int threads, int blocks_per_sm, cudaStream_t s);
// The staged kernel as a producer/consumer pipeline (one bulk-copy warp, mbarrier hand-over).
cudaError_t launch_pipe(const DevBatch &b, const StepIO &io, int threads, int blocks_per_sm, cudaStream_t s);
int n_register_shapes();  // variants below this index are the register kernels

// The implicit finite-element step's solver (cm_theta.cu): operators in the 32-row slices of
// cm_diffusion_s, the conjugate-gradient vectors, per-block partial sums (G blocks; rz and zz
// double-buffered by iteration parity), the tolerances and the device-side outcome.
struct ThetaOp {
  const int64_t *ptr = nullptr;
  const int32_t *col = nullptr;
  const double *val = nullptr;
  int64_t n = 0;
};
struct ThetaVecs {
  double *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;
  const double *dinv = nullptr;
};
struct ThetaPart {
  double *bb = nullptr, *pq = nullptr, *rz = nullptr, *zz = nullptr;  // G, G, 2 G, 2 G
  int G = 0;
};
struct ThetaCfg {
  double rtol = 1e-6, atol = 1e-6, dtol = 1e4;
};
struct ThetaStat {
  int done;   // 0 running or out of iterations, 1 converged, 2 diverged, 3 breakdown
  int iters;  // iterations taken
  double znorm;  // the last preconditioned residual norm
  int ka, kb;    // the iteration index, handed from kernel a to b and from b to the next a
};
int theta_grid();
cudaError_t launch_theta_dinv(const ThetaOp &A, double *dinv, int *bad, cudaStream_t s);
// r, z, p from x (b = R x), q = A p, and the test on the initial residual
cudaError_t launch_theta_init(const ThetaOp &A, const ThetaOp &R, const ThetaVecs &v, const ThetaPart &P,
                              const ThetaCfg &cfg, ThetaStat *st, cudaStream_t s);
// count more iterations (each a no-op once the device-side outcome is set)
cudaError_t launch_theta_iters(const ThetaOp &A, const ThetaVecs &v, const ThetaPart &P, const ThetaCfg &cfg,
                               ThetaStat *st, int max_iter, int count, cudaStream_t s);
// the iterations as a conditional while node of a graph: launched once per solve, no host reads
cudaError_t build_theta_graph(const ThetaOp &A, const ThetaVecs &v, const ThetaPart &P, const ThetaCfg &cfg,
                              ThetaStat *st, int max_iter, cudaGraphExec_t *exec);
// activation times after the solve (acCELLerate.cpp:1997-2005)
cudaError_t launch_theta_act(const double *x, double *act, int64_t n, double thr, double t, cudaStream_t s);
// Copies Vm[probe[i]] into out[i * stride + k] for i < n_probe.
cudaError_t launch_probe(const double *vm, const float *vm_hi, const float *vm_lo, const int64_t *probe,
                         int64_t n_probe, double *out, int64_t stride, int64_t k, cudaStream_t s);
// Vm planes <-> doubles (the mixed form's Vm between fused runs and the caller's array).
cudaError_t launch_vm_split(const double *v, float *hi, float *lo, int64_t n, cudaStream_t s);
cudaError_t launch_vm_join(const float *hi, const float *lo, double *v, int64_t n, cudaStream_t s);
int sm_count();

// Raises a kernel's dynamic shared-memory limit to `bytes` on the current device, once per
// device for the call site that owns `done` (the attribute belongs to the device's module).
inline cudaError_t smem_limit(const void *func, int bytes, std::atomic<uint64_t> &done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (bit && (done.load() & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) done.fetch_or(bit);
  return e;
}

}  // namespace cm
