// Surrogate macro step for ten Tusscher 2006 cells (see cm_surrogate.h): coarse physics in
// registers, the MLP on the tensor cores per warp (mma.sync m16n8k16 BF16, FP32 accumulate,
// weights resident in shared memory), residual add, gating and audit, compaction of the cells
// that take the plain integrator.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "cm_bulk.cuh"
#include "cm_cells.cuh"
#include "cm_surrogate.h"

namespace cm {

namespace {

struct Cell {
  TT2Cell<float> x;
  Acc CaSR, Na, K;
  TT2Het_<float> g;
};

__device__ __forceinline__ void load_cell(const DevBatch &b, int c, Cell &q) {
  const int64_t ld = b.ld;
  const float *s = b.s32 + c;
  const float *const *het = (const float *const *)b.het;
  const TT2Consts<float> &C = b.tt2_32;
  q.x.m = s[0]; q.x.h = s[ld]; q.x.j = s[2 * ld]; q.x.xr1 = s[3 * ld]; q.x.xr2 = s[4 * ld]; q.x.xs = s[5 * ld];
  q.x.r = s[6 * ld]; q.x.s = s[7 * ld]; q.x.d = s[8 * ld]; q.x.f = s[9 * ld]; q.x.f2 = s[10 * ld];
  q.x.fCa = s[11 * ld]; q.x.Rq = s[12 * ld]; q.x.Ca_i = s[13 * ld]; q.x.CaSS = s[14 * ld];
  q.CaSR = Acc{s[15 * ld], s[16 * ld]};
  q.Na = Acc{s[17 * ld], s[18 * ld]};
  q.K = Acc{s[19 * ld], s[20 * ld]};
  q.g.g_Na = het[H2_g_Na] ? het[H2_g_Na][c] : C.g_Na;
  q.g.g_Kr = het[H2_g_Kr] ? het[H2_g_Kr][c] : C.g_Kr;
  q.g.g_K1 = het[H2_g_K1] ? het[H2_g_K1][c] : C.g_K1;
  q.g.g_Ks = het[H2_g_Ks] ? het[H2_g_Ks][c] : C.g_Ks;
  q.g.g_to = het[H2_g_to] ? het[H2_g_to][c] : C.g_to;
  q.g.g_CaL = het[H2_g_CaL] ? het[H2_g_CaL][c] : C.g_CaL;
}

__device__ __forceinline__ void store_cell(const DevBatch &b, int c, const Cell &q) {
  const int64_t ld = b.ld;
  float *s = b.s32 + c;
  s[0] = q.x.m; s[ld] = q.x.h; s[2 * ld] = q.x.j; s[3 * ld] = q.x.xr1; s[4 * ld] = q.x.xr2; s[5 * ld] = q.x.xs;
  s[6 * ld] = q.x.r; s[7 * ld] = q.x.s; s[8 * ld] = q.x.d; s[9 * ld] = q.x.f; s[10 * ld] = q.x.f2;
  s[11 * ld] = q.x.fCa; s[12 * ld] = q.x.Rq; s[13 * ld] = q.x.Ca_i; s[14 * ld] = q.x.CaSS;
  s[15 * ld] = q.CaSR.hi; s[16 * ld] = q.CaSR.lo; s[17 * ld] = q.Na.hi; s[18 * ld] = q.Na.lo;
  s[19 * ld] = q.K.hi; s[20 * ld] = q.K.lo;
}

// Output vector order: Vm [mV], m h j xr1 xr2 xs r s d f f2 fCa Rq, Ca_i, CaSS, CaSR, Na_i, K_i.
__device__ __forceinline__ void outputs(const Cell &q, const Acc &vm, float o[kSurOut]) {
  o[0] = (vm.hi + vm.lo) * 1000.f;
  o[1] = q.x.m; o[2] = q.x.h; o[3] = q.x.j; o[4] = q.x.xr1; o[5] = q.x.xr2; o[6] = q.x.xs; o[7] = q.x.r;
  o[8] = q.x.s; o[9] = q.x.d; o[10] = q.x.f; o[11] = q.x.f2; o[12] = q.x.fCa; o[13] = q.x.Rq;
  o[14] = q.x.Ca_i; o[15] = q.x.CaSS; o[16] = q.CaSR.hi; o[17] = q.Na.hi; o[18] = q.K.hi;
}

__device__ __forceinline__ void features(const Cell &q, float vm_mv, float g0_Na, float g0_Kr, float g0_K1,
                                         float f[kSurIn]) {
  f[0] = vm_mv;
  f[1] = q.x.m; f[2] = q.x.h; f[3] = q.x.j; f[4] = q.x.xr1; f[5] = q.x.xr2; f[6] = q.x.xs; f[7] = q.x.r;
  f[8] = q.x.s; f[9] = q.x.d; f[10] = q.x.f; f[11] = q.x.f2; f[12] = q.x.fCa; f[13] = q.x.Rq;
  f[14] = logf(fmaxf(q.x.Ca_i, 1e-12f));
  f[15] = logf(fmaxf(q.x.CaSS, 1e-12f));
  f[16] = q.CaSR.hi; f[17] = q.Na.hi; f[18] = q.K.hi;
  f[19] = logf(q.g.g_Na / g0_Na);
  f[20] = logf(q.g.g_Kr / g0_Kr);
  f[21] = logf(q.g.g_K1 / g0_K1);
}

// Exact-ish increment of a compensated accumulator: the hi difference is exact for nearby
// values (Sterbenz), the lo difference is tiny.
__device__ __forceinline__ float acc_delta(const Acc &n, const Acc &o) { return (n.hi - o.hi) + (n.lo - o.lo); }

// The coarse macro step on a copy of the cell (no stimulus: stimulated cells take the plain
// path). oc: absolute outputs; inc: increments of Vm [mV], CaSR, Na_i, K_i.
__device__ __forceinline__ void coarse(const TT2Consts<float> &Cc, const float *rows_c, const float *eca, Cell q,
                                       Acc vm, float oc[kSurOut], float inc[4]) {
  uint32_t audit = 0;
  const Cell q0 = q;
  const Acc v0 = vm;
  const int vi = vrow_fp32(vm.hi * 1000.f, audit);
  const float dV = tt2_calc_mixed(Cc, rows_c + (size_t)vi * T2_COLS, eca, q.x, q.CaSR, q.Na, q.K, q.g, vm.hi, 0.f, audit);
  acc_add(vm, dV);
  outputs(q, vm, oc);
  inc[0] = acc_delta(vm, v0) * 1000.f;
  inc[1] = acc_delta(q.CaSR, q0.CaSR);
  inc[2] = acc_delta(q.Na, q0.Na);
  inc[3] = acc_delta(q.K, q0.K);
}

// The surrogate result: gates and fast Ca from oc + correction; Vm, CaSR, Na_i, K_i advanced by
// their coarse increment + correction in their accumulators.
__device__ __forceinline__ void apply(Cell &q, Acc &vm, const float on[kSurOut], const float inc[4],
                                      const float corr[kSurOut]) {
  acc_add(vm, (inc[0] + corr[0]) * 1e-3f);
  q.x.m = on[1]; q.x.h = on[2]; q.x.j = on[3]; q.x.xr1 = on[4]; q.x.xr2 = on[5]; q.x.xs = on[6]; q.x.r = on[7];
  q.x.s = on[8]; q.x.d = on[9]; q.x.f = on[10]; q.x.f2 = on[11]; q.x.fCa = on[12]; q.x.Rq = on[13];
  q.x.Ca_i = on[14]; q.x.CaSS = on[15];
  acc_add(q.CaSR, inc[1] + corr[16]);
  acc_add(q.Na, inc[2] + corr[17]);
  acc_add(q.K, inc[3] + corr[18]);
}

__device__ __forceinline__ uint32_t lds_u32(const __nv_bfloat16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// shared-memory strides (BF16 elements), chosen so fragment loads hit 32 distinct banks
constexpr int kLdX = 40, kLdH = 136;
constexpr int kWarps = 8, kThreads = kWarps * 32;
constexpr int kSmemW = (128 * kLdX + 128 * kLdH + 32 * kLdH) * 2;  // bytes
constexpr int kSmemB = (128 + 128 + 32) * 4;
constexpr int kSmemWarp = 32 * kLdX * 2 + 2 * 16 * kLdH * 2 + 32 * 33 * 4;
constexpr int kStageVars = 21 + 2 + 6;                   // state planes, Vm hi/lo, hetero slots
constexpr int kSmemStage = kStageVars * kThreads * 4;
constexpr int kSmemTotal = kSmemW + kSmemB + kWarps * kSmemWarp + kSmemStage;

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void *p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}

// tanh of two FP32 values as one packed BF16 pair (tanh.approx.bf16x2: one SFU operation)
__device__ __forceinline__ uint32_t tanh2_bf16(float x, float y) {
  uint32_t p, r;
  asm("cvt.rn.bf16x2.f32 %0, %2, %1;" : "=r"(p) : "f"(x), "f"(y));
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(r) : "r"(p));
  return r;
}

// One hidden layer for an m16 tile: OUT[16][128] = tanh(IN[16][K] W^T + b), fragments by
// ldmatrix.x4 (A: rows r, k halves; B: two n8 tiles x k16 per load).
template <int K, int LDI>
__device__ __forceinline__ void hidden_layer(const __nv_bfloat16 *W, int ldw, const float *bias,
                                             const __nv_bfloat16 *IN, __nv_bfloat16 *OUT, int lane) {
  const int g = lane >> 2, t = lane & 3;
  const int ar = lane & 15, ac = (lane >> 4) * 8;                          // A lane address
  const int br = (lane & 7) + ((lane >> 4) << 3), bc = ((lane >> 3) & 1) * 8;  // B lane address
#pragma unroll 1
  for (int nc = 0; nc < 128; nc += 32) {
    float acc[4][4] = {};
#pragma unroll
    for (int k = 0; k < K; k += 16) {
      uint32_t a[4], b01[4], b23[4];
      ldsm_x4(a, IN + ar * LDI + k + ac);
      ldsm_x4(b01, W + (nc + br) * ldw + k + bc);
      ldsm_x4(b23, W + (nc + 16 + br) * ldw + k + bc);
      mma16816(acc[0], a, b01[0], b01[1]);
      mma16816(acc[1], a, b01[2], b01[3]);
      mma16816(acc[2], a, b23[0], b23[1]);
      mma16816(acc[3], a, b23[2], b23[3]);
    }
#pragma unroll
    for (int ni = 0; ni < 4; ni++) {
      const int n = nc + ni * 8 + 2 * t;
      const float b0 = bias[n], b1 = bias[n + 1];
      *reinterpret_cast<uint32_t *>(OUT + g * kLdH + n) = tanh2_bf16(acc[ni][0] + b0, acc[ni][1] + b1);
      *reinterpret_cast<uint32_t *>(OUT + (g + 8) * kLdH + n) = tanh2_bf16(acc[ni][2] + b0, acc[ni][3] + b1);
    }
  }
}

// One m16 tile: rows [r0, r0+16) of X (K = 32) through the three layers into Y (FP32).
__device__ __forceinline__ void mlp_tile(const __nv_bfloat16 *W1, const __nv_bfloat16 *W2, const __nv_bfloat16 *W3,
                                         const float *b1, const float *b2, const float *b3, const __nv_bfloat16 *X,
                                         __nv_bfloat16 *H1, __nv_bfloat16 *H2, float *Y, int r0, int lane) {
  hidden_layer<32, kLdX>(W1, kLdX, b1, X + r0 * kLdX, H1, lane);
  __syncwarp();
  hidden_layer<128, kLdH>(W2, kLdH, b2, H1, H2, lane);
  __syncwarp();
  // output layer: Y = H2 W3^T + b3, N = 32
  const int g = lane >> 2, t = lane & 3;
  const int ar = lane & 15, ac = (lane >> 4) * 8;
  const int br = (lane & 7) + ((lane >> 4) << 3), bc = ((lane >> 3) & 1) * 8;
  float acc[4][4] = {};
#pragma unroll
  for (int k = 0; k < 128; k += 16) {
    uint32_t a[4], b01[4], b23[4];
    ldsm_x4(a, H2 + ar * kLdH + k + ac);
    ldsm_x4(b01, W3 + br * kLdH + k + bc);
    ldsm_x4(b23, W3 + (16 + br) * kLdH + k + bc);
    mma16816(acc[0], a, b01[0], b01[1]);
    mma16816(acc[1], a, b01[2], b01[3]);
    mma16816(acc[2], a, b23[0], b23[1]);
    mma16816(acc[3], a, b23[2], b23[3]);
  }
#pragma unroll
  for (int ni = 0; ni < 4; ni++)
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int r = g + (q >> 1) * 8, n = ni * 8 + 2 * t + (q & 1);
      Y[(r0 + r) * 33 + n] = acc[ni][q] + b3[n];
    }
  __syncwarp();
}

// Tiles of kThreads cells: the tile's state planes, Vm planes and conductances arrive in shared
// memory by bulk async copies (one mbarrier); every thread takes its cell into registers, then
// thread 0 issues the next tile's copies, which land while this tile's coarse step and MLP run.
__global__ void __launch_bounds__(kThreads, 1) sur_step_kernel(const SurKernelArgs a, int n) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ int s_abort;
  __nv_bfloat16 *W1 = (__nv_bfloat16 *)smem;
  __nv_bfloat16 *W2 = W1 + 128 * kLdX;
  __nv_bfloat16 *W3 = W2 + 128 * kLdH;
  float *bias = (float *)(smem + kSmemW);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char *wbase = smem + kSmemW + kSmemB + warp * kSmemWarp;
  __nv_bfloat16 *X = (__nv_bfloat16 *)wbase;
  __nv_bfloat16 *H1 = X + 32 * kLdX;
  __nv_bfloat16 *H2 = H1 + 16 * kLdH;
  float *Y = (float *)(H2 + 16 * kLdH);
  float *stage = (float *)(smem + kSmemW + kSmemB + kWarps * kSmemWarp);
  const DevBatch &fb = a.fine;
  const int64_t ld = fb.ld;
  int het_pos[6];
  int nv = 23;
#pragma unroll
  for (int k = 0; k < 6; k++) het_pos[k] = fb.het[k] ? nv++ : -1;
  const uint32_t tile_bytes = (uint32_t)nv * kThreads * 4u;
  const int n_tiles = (n + kThreads - 1) / kThreads;
  auto issue = [&](int tile) {
    const int64_t c0 = (int64_t)tile * kThreads;
    mbar_expect_tx(&bar, tile_bytes);
    for (int v = 0; v < 21; v++) bulk_g2s(stage + v * kThreads, fb.s32 + v * ld + c0, kThreads * 4u, &bar);
    bulk_g2s(stage + 21 * kThreads, a.vm_hi + c0, kThreads * 4u, &bar);
    bulk_g2s(stage + 22 * kThreads, a.vm_lo + c0, kThreads * 4u, &bar);
    for (int k = 0; k < 6; k++)
      if (het_pos[k] >= 0) bulk_g2s(stage + het_pos[k] * kThreads, (const float *)fb.het[k] + c0, kThreads * 4u, &bar);
  };
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  // network into shared memory (padded rows): W1 [128][32], W2 [128][128], W3 [32][128]
  for (int i = threadIdx.x; i < 128 * 32; i += kThreads) W1[(i >> 5) * kLdX + (i & 31)] = a.w1[i];
  for (int i = threadIdx.x; i < 128 * 128; i += kThreads) W2[(i >> 7) * kLdH + (i & 127)] = a.w2[i];
  for (int i = threadIdx.x; i < 32 * 128; i += kThreads) W3[(i >> 7) * kLdH + (i & 127)] = a.w3[i];
  for (int i = threadIdx.x; i < 288; i += kThreads) bias[i] = a.bias[i];
  __syncthreads();
  if (threadIdx.x == 0 && (int)blockIdx.x < n_tiles) issue(blockIdx.x);
  const float macro_ms = a.coarse.dt * 1000.f;
  const TT2Consts<float> &C = fb.tt2_32;
  int it = 0;
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, it++) {
    if (!mbar_wait(&bar, (uint32_t)(it & 1))) {
      s_abort = 1;
      atomicOr(fb.audit_or, kAuditTimeout);
    }
    __syncthreads();
    if (s_abort) {  // the only copy in flight is the one that timed out: give it one more bounded wait
      mbar_wait(&bar, (uint32_t)(it & 1));
      return;
    }
    const int c = t * kThreads + threadIdx.x;
    const bool valid = c < n;
    const float *S = stage + threadIdx.x;
    Cell q;
    q.x.m = S[0]; q.x.h = S[kThreads]; q.x.j = S[2 * kThreads]; q.x.xr1 = S[3 * kThreads];
    q.x.xr2 = S[4 * kThreads]; q.x.xs = S[5 * kThreads]; q.x.r = S[6 * kThreads]; q.x.s = S[7 * kThreads];
    q.x.d = S[8 * kThreads]; q.x.f = S[9 * kThreads]; q.x.f2 = S[10 * kThreads]; q.x.fCa = S[11 * kThreads];
    q.x.Rq = S[12 * kThreads]; q.x.Ca_i = S[13 * kThreads]; q.x.CaSS = S[14 * kThreads];
    q.CaSR = Acc{S[15 * kThreads], S[16 * kThreads]};
    q.Na = Acc{S[17 * kThreads], S[18 * kThreads]};
    q.K = Acc{S[19 * kThreads], S[20 * kThreads]};
    Acc vm{S[21 * kThreads], S[22 * kThreads]};
    q.g.g_Na = het_pos[H2_g_Na] >= 0 ? S[het_pos[H2_g_Na] * kThreads] : C.g_Na;
    q.g.g_Kr = het_pos[H2_g_Kr] >= 0 ? S[het_pos[H2_g_Kr] * kThreads] : C.g_Kr;
    q.g.g_K1 = het_pos[H2_g_K1] >= 0 ? S[het_pos[H2_g_K1] * kThreads] : C.g_K1;
    q.g.g_Ks = het_pos[H2_g_Ks] >= 0 ? S[het_pos[H2_g_Ks] * kThreads] : C.g_Ks;
    q.g.g_to = het_pos[H2_g_to] >= 0 ? S[het_pos[H2_g_to] * kThreads] : C.g_to;
    q.g.g_CaL = het_pos[H2_g_CaL] >= 0 ? S[het_pos[H2_g_CaL] * kThreads] : C.g_CaL;
    __syncthreads();  // the stage buffer is free: the next tile's copies overlap this tile's work
    if (threadIdx.x == 0 && t + (int)gridDim.x < n_tiles) {
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      issue(t + gridDim.x);
    }
    float oc[kSurOut], inc[4], f[kSurIn];
    bool fall = !valid;
    if (valid) {
      coarse(a.coarse, a.rows_coarse, a.eca, q, vm, oc, inc);
      const float rate = fabsf(inc[0]) / macro_ms;
      fall = a.stim_on || !(rate <= a.gate_mv_per_ms);
      features(q, (vm.hi + vm.lo) * 1000.f, a.g0_Na, a.g0_Kr, a.g0_K1, f);
    } else {
#pragma unroll
      for (int k = 0; k < kSurIn; k++) f[k] = a.norm.mu_x[k];
    }
    // normalised features into this warp's X rows (row = lane), K padded to 32 with zeros
#pragma unroll
    for (int k = 0; k < kSurIn; k++) X[lane * kLdX + k] = __float2bfloat16((f[k] - a.norm.mu_x[k]) * a.norm.inv_sd_x[k]);
#pragma unroll
    for (int k = kSurIn; k < 32; k++) X[lane * kLdX + k] = __float2bfloat16(0.f);
    __syncwarp();
    const bool any = __any_sync(0xffffffffu, !fall);
    if (a.mode == 0 && any) {
      mlp_tile(W1, W2, W3, bias, bias + 128, bias + 256, X, H1, H2, Y, 0, lane);
      mlp_tile(W1, W2, W3, bias, bias + 128, bias + 256, X, H1, H2, Y, 16, lane);
    }
    if (valid) {
      const bool audited = a.audit_mod > 0 && (c % a.audit_mod) == a.audit_phase;
      if (audited) a.pred[c] = __int_as_float(0x7fc00000);  // NaN unless the surrogate predicts below
      if (!fall) {
        float on[kSurOut], corr[kSurOut];
#pragma unroll
        for (int k = 0; k < kSurOut; k++) {
          corr[k] = a.mode == 0 ? a.norm.sd_y[k] * Y[lane * 33 + k] : 0.f;
          on[k] = oc[k] + corr[k];
        }
        // range audit: gates in [0, 1], concentrations positive, everything finite
        bool ok = isfinite(on[0]);
#pragma unroll
        for (int k = 1; k <= 13; k++) ok = ok && on[k] >= -1e-3f && on[k] <= 1.001f;
#pragma unroll
        for (int k = 14; k < kSurOut; k++) ok = ok && on[k] > 0.f && isfinite(on[k]);
        if (!ok) {
          fall = true;
          atomicOr(fb.audit_cell + c, 16u);
          atomicOr(fb.audit_or, 16u);
        } else if (audited) {
          a.pred[c] = on[0];
          fall = true;
        } else {
          Cell nq = q;
          Acc nv = vm;
          apply(nq, nv, on, inc, corr);
          store_cell(fb, c, nq);
          a.vm_hi[c] = nv.hi;
          a.vm_lo[c] = nv.lo;
        }
      }
      if (fall) {
        const unsigned int slot = atomicAdd(a.n_fallback, 1u);
        a.fallback[slot] = c;
        atomicAdd(a.n_fallback_total, 1ull);
      } else {
        atomicAdd(a.n_sur, 1ull);
      }
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(128) sur_plain_kernel(const SurPlainArgs a) {
  const unsigned int n = *a.n_list;
  for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int c = a.list[i];
    Acc v{a.vm_hi[c], a.vm_lo[c]};
    uint32_t audit = 0;
    for (int k = 0; k < a.substeps; k++) acc_add(v, tt2_mixed_cell<int>(a.fine, c, v.hi, a.iext[k], audit));
    a.vm_hi[c] = v.hi;
    a.vm_lo[c] = v.lo;
    if (!isfinite(v.hi)) audit |= 1u;
    if (audit) {
      atomicOr(a.fine.audit_cell + c, audit);
      atomicOr(a.fine.audit_or, audit);
    }
    if (a.audit_mod > 0 && (c % a.audit_mod) == a.audit_phase) {
      const float p = a.pred[c];
      if (isfinite(p)) {
        const float err = fabsf(p - (v.hi + v.lo) * 1000.f);
        atomicMax((int *)a.audit_err, __float_as_int(err));  // non-negative floats order as ints
        atomicAdd(a.n_audit, 1ull);
      }
    }
  }
}

__global__ void __launch_bounds__(128) sur_gen_kernel(const SurGenArgs a) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < a.n_sample; k += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(a.offset + k * a.stride);
    Cell q;
    load_cell(a.fine, c, q);
    const Acc vm{a.vm_hi[c], a.vm_lo[c]};
    float f[kSurIn], oc[kSurOut], inc[4];
    features(q, (vm.hi + vm.lo) * 1000.f, a.g0_Na, a.g0_Kr, a.g0_K1, f);
    coarse(a.coarse, a.rows_coarse, a.eca, q, vm, oc, inc);
    // accumulator quantities carry their coarse increment; the others their coarse value
    oc[0] = inc[0];
    oc[16] = inc[1];
    oc[17] = inc[2];
    oc[18] = inc[3];
    for (int i = 0; i < kSurIn; i++) a.X[k * kSurIn + i] = f[i];
    for (int i = 0; i < kSurOut; i++) a.C[k * kSurOut + i] = oc[i];
    float *old = a.Old + k * 8;
    old[0] = vm.hi; old[1] = vm.lo; old[2] = q.CaSR.hi; old[3] = q.CaSR.lo;
    old[4] = q.Na.hi; old[5] = q.Na.lo; old[6] = q.K.hi; old[7] = q.K.lo;
  }
}

__global__ void __launch_bounds__(128) sur_post_kernel(const SurPostArgs a) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < a.n_sample; k += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(a.offset + k * a.stride);
    Cell q;
    load_cell(a.fine, c, q);
    const Acc vm{a.vm_hi[c], a.vm_lo[c]};
    float o[kSurOut];
    outputs(q, vm, o);
    const float *old = a.Old + k * 8;
    // fine increments of the accumulator quantities, from their hi/lo words
    o[0] = acc_delta(vm, Acc{old[0], old[1]}) * 1000.f;
    o[16] = acc_delta(q.CaSR, Acc{old[2], old[3]});
    o[17] = acc_delta(q.Na, Acc{old[4], old[5]});
    o[18] = acc_delta(q.K, Acc{old[6], old[7]});
    bool keep = !a.stim_on;
    const float rate = fabsf(a.C[k * kSurOut]) / a.macro_ms;  // the inference gate (coarse dVm)
    keep = keep && rate <= a.gate_mv_per_ms;
    for (int i = 0; i < kSurOut; i++) {
      const float r = o[i] - a.C[k * kSurOut + i];
      keep = keep && isfinite(r);
      a.T[k * kSurOut + i] = r;
    }
    a.keep[k] = keep ? 1 : 0;
  }
}

// Appends the kept (feature, target) pairs of one generation step to the dataset.
__global__ void sur_append_kernel(const float *__restrict__ X, const float *__restrict__ T,
                                  const uint8_t *__restrict__ keep, int64_t n, float *__restrict__ dX,
                                  float *__restrict__ dT, unsigned long long *count, int64_t cap) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    if (!keep[k]) continue;
    const unsigned long long slot = atomicAdd(count, 1ull);
    if ((int64_t)slot >= cap) continue;
    for (int i = 0; i < kSurIn; i++) dX[slot * kSurIn + i] = X[k * kSurIn + i];
    for (int i = 0; i < kSurOut; i++) dT[slot * kSurOut + i] = T[k * kSurOut + i];
  }
}

__global__ void sur_normalize_kernel(const float *__restrict__ X, const float *__restrict__ T, int64_t n,
                                     const SurNorm norm, float *__restrict__ nX, float *__restrict__ nT) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    for (int i = 0; i < kSurIn; i++) nX[k * kSurIn + i] = (X[k * kSurIn + i] - norm.mu_x[i]) * norm.inv_sd_x[i];
    for (int i = 0; i < kSurOut; i++) nT[k * kSurOut + i] = T[k * kSurOut + i] / norm.sd_y[i];
  }
}

}  // namespace

cudaError_t launch_sur_append(const float *X, const float *T, const uint8_t *keep, int64_t n, float *dX, float *dT,
                              unsigned long long *count, int64_t cap, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t g = (n + 127) / 128;
  sur_append_kernel<<<(unsigned)(g < 4096 ? g : 4096), 128, 0, s>>>(X, T, keep, n, dX, dT, count, cap);
  return cudaGetLastError();
}

cudaError_t launch_sur_normalize(const float *X, const float *T, int64_t n, const SurNorm &norm, float *nX, float *nT,
                                 cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t g = (n + 255) / 256;
  sur_normalize_kernel<<<(unsigned)(g < 8192 ? g : 8192), 256, 0, s>>>(X, T, n, norm, nX, nT);
  return cudaGetLastError();
}

cudaError_t launch_sur_step(const SurKernelArgs &a, int64_t n, cudaStream_t s) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(sur_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemTotal);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  if (n <= 0) return cudaSuccess;
  const int64_t need = (n + kThreads - 1) / kThreads;
  const int64_t cap = (int64_t)sm_count();
  const int grid = (int)(need < cap ? need : cap);
  sur_step_kernel<<<grid, kThreads, kSmemTotal, s>>>(a, (int)n);
  return cudaGetLastError();
}

cudaError_t launch_sur_plain(const SurPlainArgs &a, int max_cells, cudaStream_t s) {
  if (max_cells <= 0) return cudaSuccess;
  const int grid = (max_cells + 127) / 128 < sm_count() * 8 ? (max_cells + 127) / 128 : sm_count() * 8;
  sur_plain_kernel<<<grid, 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_sur_gen(const SurGenArgs &a, cudaStream_t s) {
  if (a.n_sample <= 0) return cudaSuccess;
  const int64_t g = (a.n_sample + 127) / 128;
  sur_gen_kernel<<<(unsigned)(g < 4096 ? g : 4096), 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_sur_post(const SurPostArgs &a, cudaStream_t s) {
  if (a.n_sample <= 0) return cudaSuccess;
  const int64_t g = (a.n_sample + 127) / 128;
  sur_post_kernel<<<(unsigned)(g < 4096 ? g : 4096), 128, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace cm
