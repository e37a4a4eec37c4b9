// Learned macro-step for ten Tusscher 2006 cells (cm_surrogate.cu).
//
// One macro step advances a cell by S fine steps (S * dt, e.g. 10 x 0.01 ms). It is the coarse
// physics step -- the mixed-form update once with tables built for S * dt -- plus an MLP
// correction trained on the residual between S fine steps of the plain integrator and that
// coarse step:   x(t + S dt) = coarse(x) + sigma_y * MLP((f(x) - mu_x) / sigma_x).
// Cells whose stimulus is on during the macro step, whose |dVm/dt| exceeds the gate (5 mV/ms,
// the upstroke), that fail the range audit, or that fall in the rotating audit sample are
// integrated by the plain integrator instead (S fine steps); audited cells also record how far
// the surrogate's prediction was from the plain result.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "cm_launch.h"
#include "cm_mlp.h"

namespace cm {

constexpr int kSurIn = 22;   // features
constexpr int kSurOut = 19;  // corrected quantities
constexpr int kSurH = 128;   // hidden width (the inference kernel is built for 128)

// Features: Vm [mV], 13 gates, log Ca_i, log CaSS, CaSR, Na_i, K_i, log(g/g0) of g_Na, g_Kr, g_K1.
// Outputs: residuals of Vm [mV], the 13 gates, Ca_i, CaSS, CaSR, Na_i, K_i.
// Feature normalisation, target scales, the scale at which each output's correction is applied
// (sd_y where the network predicts that output's residual better than its mean, R^2 >= kSurMinR2
// on the training data; 0 where it does not, and the coarse step's value is kept), and the R^2.
// Corrections the network predicts poorly are biased noise that accumulates over macro steps;
// the gates' clamp into [0, 1] (apply() in cm_surrogate.cu) bounds what remains of that.
constexpr float kSurMinR2 = 0.0f;
struct SurNorm {
  float mu_x[kSurIn], inv_sd_x[kSurIn], sd_y[kSurOut], apply_y[kSurOut], r2[kSurOut];
};

struct SurKernelArgs {
  DevBatch fine;       // the batch (state, fine tables, per-cell conductances)
  TT2Consts<float> coarse;       // constants for the macro step S * dt
  const float *rows_coarse;      // FP32 voltage table rows for S * dt
  const float *eca;              // ECa table (dt independent)
  // Vm [V], one of two forms: the caller's FP64 array in page-locked host memory, read and
  // written once per macro step (vm != nullptr), or device FP32 planes holding the compensated
  // pair (vm_hi, vm_lo; split from and joined into the caller's array once per call)
  double *vm;
  float *vm_hi, *vm_lo;
  SurNorm norm;
  const __nv_bfloat16 *w1, *w2, *w3;  // BF16 network: W1 [128][32], W2 [128][128], W3 [32][128]
  const float *bias;             // b1 [128], b2 [128], b3 [32]
  int mode;                      // 0: coarse + MLP, 1: coarse only
  int stim_on;                   // stimulus during this macro step: every cell takes the plain path
  float gate_mv_per_ms;          // |dVm/dt| above this: plain path
  int audit_mod, audit_phase;    // cells with c % audit_mod == audit_phase are audited
  int *fallback;                 // compacted list of cells for the plain integrator
  unsigned int *n_fallback;
  unsigned long long *n_fallback_total;  // over all macro steps
  // audit sample: cells with c % audit_mod == audit_phase whose surrogate step was accepted are
  // copied, with their initial state and the prediction, into a snapshot for the audit kernel
  float *snap;                   // kSnapPlanes planes of snap_cap entries
  unsigned int *n_snap;
  int snap_cap;
  unsigned long long *n_sur;     // cells advanced by the surrogate (over all macro steps)
  float inv_g0_Na, inv_g0_Kr, inv_g0_K1;  // 1 / the parameter-set conductances (feature reference)
  // per-cell stimulus protocol (else stim_on for all cells): first stimulus time by cell, and
  // the time of the macro step's last fine step; a cell is stimulated when t_last >= tb_cell[c]
  const double *tb_cell;
  double t_last;
};

// Snapshot of an audited cell: 21 state planes, Vm hi / lo, the six conductances, the
// surrogate's prediction of Vm [mV] after the macro step.
constexpr int kSnapPlanes = 21 + 2 + 6 + 1;

struct SurPlainArgs {
  DevBatch fine;
  double *vm;                    // as SurKernelArgs
  float *vm_hi, *vm_lo;
  const int *list;               // the cells to advance; null: cells 0 .. n_all - 1
  const unsigned int *n_list;
  int n_all;
  int substeps;
  float iext[64];                // per fine step of the macro step
  // per-cell stimulus protocol (else iext[] for all cells): the reference driver's logic per
  // fine step k at time tk[k], advancing tb_cell in place
  double *tb_cell;
  double tk[64];
  double textlen, bcl, amp;
};

// The audit of one macro step: every snapshot integrated by the plain method over the S fine
// steps (no stimulus: stimulated cells never take the surrogate) in FP64 (the reference
// arithmetic, FP64 tables) or in the mixed form, and compared with the prediction.
struct SurAuditArgs {
  const float *snap;
  const unsigned int *n_snap;
  int snap_cap, substeps, fp64;
  TT2Consts<double> c64;
  const double *rows64, *eca64;
  TT2Consts<float> c32;
  const float *rows32, *eca32;
  float *audit_err;              // max |prediction - plain| Vm [mV] (atomicMax on the float bits)
  unsigned long long *n_audit;
};

struct SurGenArgs {
  DevBatch fine;
  TT2Consts<float> coarse;
  const float *rows_coarse, *eca;
  const float *vm_hi, *vm_lo;
  int64_t stride, offset;        // sampled cells: c = offset + k * stride
  int64_t n_sample;
  float *X, *C;                  // features and coarse result per sample (kSurIn, kSurOut)
  float *Old;                    // Vm, CaSR, Na_i, K_i hi/lo words at the macro-step start (8)
  float inv_g0_Na, inv_g0_Kr, inv_g0_K1;
};

struct SurPostArgs {
  DevBatch fine;
  const float *vm_hi, *vm_lo;
  int64_t stride, offset, n_sample;
  const float *C;                // coarse result (accumulator quantities: coarse increments)
  const float *Old;              // accumulator words at the macro-step start
  float *T;                      // residual targets (kSurOut)
  uint8_t *keep;                 // 1: usable pair (not stimulated, not in the upstroke)
  float gate_mv_per_ms, macro_ms;
  int stim_on;
};

// prev: the previous macro step's audit, run by an extra warp group of the same launch (the
// macro step then uses 3 MLP groups); NULL: no audit group, 4 MLP groups.
cudaError_t launch_sur_step(const SurKernelArgs &a, const SurAuditArgs *prev, int64_t n, cudaStream_t s);
cudaError_t launch_sur_plain(const SurPlainArgs &a, int max_cells, cudaStream_t s);
// the audit of the last macro step of a run
cudaError_t launch_sur_audit(const SurAuditArgs &a, cudaStream_t s);
cudaError_t launch_sur_gen(const SurGenArgs &a, cudaStream_t s);
cudaError_t launch_sur_post(const SurPostArgs &a, cudaStream_t s);
// Ordered append of the kept pairs; chunk_scratch holds sur_append_scratch_words(n) words.
int64_t sur_append_scratch_words(int64_t n);
cudaError_t launch_sur_append(const float *X, const float *T, const uint8_t *keep, int64_t n, float *dX, float *dT,
                              unsigned long long *count, int64_t cap, int64_t *chunk_scratch, cudaStream_t s);
cudaError_t launch_sur_normalize(const float *X, const float *T, int64_t n, const SurNorm &norm, float *nX, float *nT,
                                 cudaStream_t s);

}  // namespace cm
