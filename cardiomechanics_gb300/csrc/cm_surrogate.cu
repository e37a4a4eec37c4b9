// Surrogate macro step for ten Tusscher 2006 cells (see cm_surrogate.h): coarse physics in
// registers, the MLP on the fifth-generation tensor cores (tcgen05.mma, BF16 operands in shared
// memory, FP32 accumulators in tensor memory), residual add, gating and audit, compaction of the
// cells that take the plain integrator; the plain integrator for those cells; training-data
// generation kernels.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "cm_bulk.cuh"
#include "cm_cells.cuh"
#include "cm_surrogate.h"
#include "cm_umma.cuh"

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

// The logarithms are the SFU's (relative error ~2^-21): the features reach the network as BF16
// (8 significant bits), and the library logf and division cost the issue-bound macro step ~5 %
// of its instructions.
__device__ __forceinline__ void features(const Cell &q, float vm_mv, float inv_g0_Na, float inv_g0_Kr,
                                         float inv_g0_K1, float f[kSurIn]) {
  f[0] = vm_mv;
  f[1] = q.x.m; f[2] = q.x.h; f[3] = q.x.j; f[4] = q.x.xr1; f[5] = q.x.xr2; f[6] = q.x.xs; f[7] = q.x.r;
  f[8] = q.x.s; f[9] = q.x.d; f[10] = q.x.f; f[11] = q.x.f2; f[12] = q.x.fCa; f[13] = q.x.Rq;
  f[14] = __logf(fmaxf(q.x.Ca_i, 1e-12f));
  f[15] = __logf(fmaxf(q.x.CaSS, 1e-12f));
  f[16] = q.CaSR.hi; f[17] = q.Na.hi; f[18] = q.K.hi;
  f[19] = __logf(q.g.g_Na * inv_g0_Na);
  f[20] = __logf(q.g.g_Kr * inv_g0_Kr);
  f[21] = __logf(q.g.g_K1 * inv_g0_K1);
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
// their coarse increment + correction in their accumulators. Gates are probabilities: values the
// range audit let through (within 1e-3 of [0, 1]) are clamped into it, so a small bias in a
// correction cannot accumulate past the bounds over many macro steps.
__device__ __forceinline__ float unit(float x) { return fminf(fmaxf(x, 0.f), 1.f); }
__device__ __forceinline__ void apply(Cell &q, Acc &vm, const float on[kSurOut], const float inc[4],
                                      const float corr[kSurOut]) {
  acc_add(vm, (inc[0] + corr[0]) * 1e-3f);
  q.x.m = unit(on[1]); q.x.h = unit(on[2]); q.x.j = unit(on[3]); q.x.xr1 = unit(on[4]); q.x.xr2 = unit(on[5]);
  q.x.xs = unit(on[6]); q.x.r = unit(on[7]); q.x.s = unit(on[8]); q.x.d = unit(on[9]); q.x.f = unit(on[10]);
  q.x.f2 = unit(on[11]); q.x.fCa = unit(on[12]); q.x.Rq = unit(on[13]);
  q.x.Ca_i = on[14]; q.x.CaSS = on[15];
  acc_add(q.CaSR, inc[1] + corr[16]);
  acc_add(q.Na, inc[2] + corr[17]);
  acc_add(q.K, inc[3] + corr[18]);
}

// tanh of two FP32 values as one packed BF16 pair (tanh.approx.bf16x2: one SFU operation)
__device__ __forceinline__ uint32_t tanh2_bf16(float x, float y) {
  uint32_t p, r;
  asm("cvt.rn.bf16x2.f32 %0, %2, %1;" : "=r"(p) : "f"(x), "f"(y));
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(r) : "r"(p));
  return r;
}

__global__ void __launch_bounds__(128) sur_plain_kernel(const SurPlainArgs a) {
  const unsigned int n = a.list ? *a.n_list : (unsigned int)a.n_all;
  for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int c = a.list ? a.list[i] : (int)i;
    Acc v = a.vm ? acc_from_double(a.vm[c]) : Acc{a.vm_hi[c], a.vm_lo[c]};
    uint32_t audit = 0;
    double tb = a.tb_cell ? a.tb_cell[c] : 0.0;
    for (int k = 0; k < a.substeps; k++) {
      float iext = a.iext[k];
      if (a.tb_cell) {  // reference driver stimulus (CellModel.h:405-419), per cell
        iext = 0.f;
        if (a.tk[k] >= tb) {
          iext = (float)a.amp;
          if (a.tk[k] >= tb + a.textlen) tb += a.bcl;
        }
      }
      acc_add(v, tt2_mixed_cell<int>(a.fine, c, v.hi, iext, audit));
    }
    if (a.tb_cell) a.tb_cell[c] = tb;
    if (a.vm) {
      a.vm[c] = acc_to_double(v);
    } else {
      a.vm_hi[c] = v.hi;
      a.vm_lo[c] = v.lo;
    }
    if (!isfinite(v.hi)) audit |= 1u;
    if (audit) {
      atomicOr(a.fine.audit_cell + c, audit);
      atomicOr(a.fine.audit_or, audit);
    }
  }
}

// The audit of one snapshot: the audited cell integrated over the macro step by the plain method
// in FP64 (the reference arithmetic: the FP32 state widened, FP64 tables and constants) or in the
// mixed form; returns |prediction - plain| for Vm [mV] (a NaN counts as the largest error).
__device__ __forceinline__ float audit_entry(const SurAuditArgs &a, unsigned int i) {
  const int64_t cap = a.snap_cap;
  const float *S = a.snap + i;
  uint32_t audit = 0;
  float err;
  if (a.fp64) {
    TT2Cell<double> x;
    x.m = S[0]; x.h = S[cap]; x.j = S[2 * cap]; x.xr1 = S[3 * cap]; x.xr2 = S[4 * cap]; x.xs = S[5 * cap];
    x.r = S[6 * cap]; x.s = S[7 * cap]; x.d = S[8 * cap]; x.f = S[9 * cap]; x.f2 = S[10 * cap];
    x.fCa = S[11 * cap]; x.Rq = S[12 * cap]; x.Ca_i = S[13 * cap]; x.CaSS = S[14 * cap];
    double CaSR = acc_to_double(Acc{S[15 * cap], S[16 * cap]});
    double Na_i = acc_to_double(Acc{S[17 * cap], S[18 * cap]});
    double K_i = acc_to_double(Acc{S[19 * cap], S[20 * cap]});
    double V = acc_to_double(Acc{S[21 * cap], S[22 * cap]});
    TT2Het_<double> g;
    g.g_Na = S[23 * cap]; g.g_Kr = S[24 * cap]; g.g_K1 = S[25 * cap];
    g.g_Ks = S[26 * cap]; g.g_to = S[27 * cap]; g.g_CaL = S[28 * cap];
    for (int k = 0; k < a.substeps; k++) {
      const int vi = vrow_fp64(V * 1000.0, audit);
      V += tt2_calc_fp64<false>(a.c64, a.rows64 + (size_t)vi * T2_COLS, a.eca64, x, CaSR, Na_i, K_i, g, V, 0.0, audit,
                                nullptr);
    }
    err = fabsf(S[29 * cap] - (float)(V * 1000.0));
  } else {
    TT2Cell<float> x;
    x.m = S[0]; x.h = S[cap]; x.j = S[2 * cap]; x.xr1 = S[3 * cap]; x.xr2 = S[4 * cap]; x.xs = S[5 * cap];
    x.r = S[6 * cap]; x.s = S[7 * cap]; x.d = S[8 * cap]; x.f = S[9 * cap]; x.f2 = S[10 * cap];
    x.fCa = S[11 * cap]; x.Rq = S[12 * cap]; x.Ca_i = S[13 * cap]; x.CaSS = S[14 * cap];
    Acc CaSR{S[15 * cap], S[16 * cap]}, Na_i{S[17 * cap], S[18 * cap]}, K_i{S[19 * cap], S[20 * cap]};
    Acc V{S[21 * cap], S[22 * cap]};
    TT2Het_<float> g;
    g.g_Na = S[23 * cap]; g.g_Kr = S[24 * cap]; g.g_K1 = S[25 * cap];
    g.g_Ks = S[26 * cap]; g.g_to = S[27 * cap]; g.g_CaL = S[28 * cap];
    for (int k = 0; k < a.substeps; k++) {
      const int vi = vrow_fp32(V.hi * 1000.f, audit);
      acc_add(V, tt2_calc_mixed(a.c32, a.rows32 + (size_t)vi * T2_COLS, a.eca32, x, CaSR, Na_i, K_i, g, V.hi, 0.f,
                                audit));
    }
    err = fabsf(S[29 * cap] - (V.hi + V.lo) * 1000.f);
  }
  return err == err ? err : 3.4e38f;
}

// Audits of entries [first, n) with stride `stride` by a set of threads that form whole warps:
// one atomic maximum and one count per warp and round.
__device__ __forceinline__ void audit_range(const SurAuditArgs &a, unsigned int first, unsigned int stride) {
  const unsigned int n = min(*a.n_snap, (unsigned int)a.snap_cap);
  const int lane = threadIdx.x & 31;
  const unsigned int wfirst = first - (unsigned int)lane;  // the warp's first entry
  for (unsigned int i0 = wfirst; i0 < n; i0 += stride) {
    const unsigned int i = i0 + lane;
    const bool valid = i < n;
    float err = valid ? audit_entry(a, i) : 0.f;
    for (int o = 16; o > 0; o >>= 1) err = fmaxf(err, __shfl_xor_sync(0xffffffffu, err, o));
    const unsigned int cnt = __popc(__ballot_sync(0xffffffffu, valid));
    if (lane == 0 && cnt) {
      atomicMax((int *)a.audit_err, __float_as_int(err));  // non-negative floats order as ints
      atomicAdd(a.n_audit, (unsigned long long)cnt);
    }
  }
}

// The audit of the last macro step of a run (the others run inside the next macro step).
__global__ void __launch_bounds__(128) sur_audit_kernel(const SurAuditArgs a) {
  audit_range(a, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

__global__ void __launch_bounds__(128) sur_gen_kernel(const SurGenArgs a) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < a.n_sample; k += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(a.offset + k * a.stride);
    Cell q;
    load_cell(a.fine, c, q);
    const Acc vm{a.vm_hi[c], a.vm_lo[c]};
    float f[kSurIn], oc[kSurOut], inc[4];
    features(q, (vm.hi + vm.lo) * 1000.f, a.inv_g0_Na, a.inv_g0_Kr, a.inv_g0_K1, f);
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

// Appends the kept (feature, target) pairs of one generation step to the dataset in sample
// order, so the dataset (and the cut at its capacity) is the same on every run: pass 1 counts the
// kept pairs of each chunk of kAppendChunk samples, pass 2 (one block) turns the counts into
// dataset offsets after the pairs already held, pass 3 writes each chunk's pairs at its offset.
constexpr int kAppendThreads = 128, kAppendPer = 8, kAppendChunk = kAppendThreads * kAppendPer;

__global__ void __launch_bounds__(kAppendThreads) sur_append_count_kernel(const uint8_t *__restrict__ keep, int64_t n,
                                                                          int64_t *__restrict__ chunk_count) {
  const int64_t n_chunks = (n + kAppendChunk - 1) / kAppendChunk;
  for (int64_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
    int cnt = 0;
    for (int i = threadIdx.x; i < kAppendChunk; i += kAppendThreads) {
      const int64_t k = c * kAppendChunk + i;
      cnt += (k < n && keep[k]) ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    __shared__ int warp_cnt[kAppendThreads / 32];
    if ((threadIdx.x & 31) == 0) warp_cnt[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int w = 0; w < kAppendThreads / 32; w++) t += warp_cnt[w];
      chunk_count[c] = t;
    }
    __syncthreads();
  }
}

// One block of 1024 threads: exclusive prefix sums of the chunk counts, offset by the pairs
// the dataset already holds; the total is added to the dataset count.
__global__ void __launch_bounds__(1024) sur_append_scan_kernel(int64_t *__restrict__ chunk_count, int64_t n_chunks,
                                                               unsigned long long *count) {
  __shared__ int64_t part[1024];
  __shared__ int64_t base;
  if (threadIdx.x == 0) base = (int64_t)*count;
  __syncthreads();
  for (int64_t c0 = 0; c0 < n_chunks; c0 += 1024) {
    const int64_t c = c0 + threadIdx.x;
    const int64_t v = c < n_chunks ? chunk_count[c] : 0;
    part[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // Hillis-Steele inclusive scan
      const int64_t add = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
      __syncthreads();
      part[threadIdx.x] += add;
      __syncthreads();
    }
    if (c < n_chunks) chunk_count[c] = base + part[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 0) base += part[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = (unsigned long long)base;
}

__global__ void __launch_bounds__(kAppendThreads) sur_append_kernel(
    const float *__restrict__ X, const float *__restrict__ T, const uint8_t *__restrict__ keep, int64_t n,
    const int64_t *__restrict__ chunk_offset, float *__restrict__ dX, float *__restrict__ dT, int64_t cap) {
  __shared__ int warp_cnt[kAppendThreads / 32];
  const int64_t n_chunks = (n + kAppendChunk - 1) / kAppendChunk;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
    // thread t owns samples [t * kAppendPer, (t + 1) * kAppendPer) of the chunk
    const int64_t k0 = c * kAppendChunk + (int64_t)threadIdx.x * kAppendPer;
    int mine = 0;
    for (int i = 0; i < kAppendPer; i++) mine += (k0 + i < n && keep[k0 + i]) ? 1 : 0;
    int incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) warp_cnt[warp] = incl;
    __syncthreads();
    int before = incl - mine;
    for (int w = 0; w < warp; w++) before += warp_cnt[w];
    int64_t slot = chunk_offset[c] + before;
    for (int i = 0; i < kAppendPer; i++) {
      const int64_t k = k0 + i;
      if (k >= n || !keep[k]) continue;
      if (slot < cap) {
        for (int j = 0; j < kSurIn; j++) dX[slot * kSurIn + j] = X[k * kSurIn + j];
        for (int j = 0; j < kSurOut; j++) dT[slot * kSurOut + j] = T[k * kSurOut + j];
      }
      slot++;
    }
    __syncthreads();
  }
}

__global__ void sur_normalize_kernel(const float *__restrict__ X, const float *__restrict__ T, int64_t n,
                                     const SurNorm norm, float *__restrict__ nX, float *__restrict__ nT) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    for (int i = 0; i < kSurIn; i++) nX[k * kSurIn + i] = (X[k * kSurIn + i] - norm.mu_x[i]) * norm.inv_sd_x[i];
    for (int i = 0; i < kSurOut; i++) nT[k * kSurOut + i] = T[k * kSurOut + i] / norm.sd_y[i];
  }
}

// ---------------------------------------------------------------- tcgen05 inference kernel
// kGroups groups of 4 warps per block; a group owns tiles of 128 cells (one cell per thread,
// thread i of the group = row i of the MLP tile = TMEM lane i). The network is resident in
// shared memory once per block in the tensor core's K-major layout; each group has a 32 KB
// activation tile (features, then hidden layer 1, then hidden layer 2, each overwritten once the
// MMA that read it has completed), a bulk-copy stage for its next cell tile, and 128 TMEM
// columns for the FP32 accumulators of the three layers (each layer's accumulator is read back
// by tcgen05.ld before the next layer's MMA overwrites it). One elected thread per group issues
// the MMAs; completion is signalled through an mbarrier by tcgen05.commit.
// The hidden biases are added on the tensor core: b1 as column 22 of W1 against a constant 1 in
// column 22 of the input tile, b2 by one more MMA of a constant 128 x 16 tile whose column 0 is 1
// against a 128 x 16 tile whose column 0 is b2. b3 (19 values) is added in the epilogue.
constexpr int kTcCells = 128;
constexpr int kTcStageVars = 21;  // the tile's state planes (Vm is read with plain loads)
constexpr int kTcW1 = 128 * 32 * 2, kTcW2 = 128 * 128 * 2, kTcW3 = 32 * 128 * 2;
constexpr int kTcOnes = 128 * 16 * 2, kTcB2 = 128 * 16 * 2, kTcB3 = 32 * 4;
constexpr int kTcHead = kTcW1 + kTcW2 + kTcW3 + kTcOnes + kTcB2 + kTcB3;
constexpr int kTcAct = kTcCells * 128 * 2;          // activation tile (BF16)
constexpr int kTcStage = kTcStageVars * kTcCells * 4;
constexpr int kTcGroupBytes = kTcAct + kTcStage;
__host__ __device__ constexpr int tc_smem_bytes(int groups) { return kTcHead + groups * kTcGroupBytes; }

__device__ __forceinline__ void group_sync(int g) { asm volatile("bar.sync %0, 128;\n" ::"r"(g + 1) : "memory"); }

__device__ __forceinline__ void sts128(void *p, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1,%2,%3,%4};\n" ::"r"((uint32_t)__cvta_generic_to_shared(p)), "r"(a), "r"(b),
               "r"(c), "r"(d)
               : "memory");
}

// bf16 pair (lo = x, hi = y) without activation
__device__ __forceinline__ uint32_t pack_bf16(float x, float y) {
  uint32_t p;
  asm("cvt.rn.bf16x2.f32 %0, %2, %1;" : "=r"(p) : "f"(x), "f"(y));
  return p;
}

// One hidden-layer epilogue for this thread's row: TMEM columns [0, 128) of the group's
// accumulator (bias included) -> tanh -> BF16, written as row r of a 128 x 128 K-major tile.
__device__ __forceinline__ void tc_hidden_epilogue(uint32_t tacc, __nv_bfloat16 *act, int r) {
#pragma unroll 1
  for (int c0 = 0; c0 < 128; c0 += 32) {
    float v[32];
    umma::tmem_ld32(tacc + (uint32_t)c0, v);
    uint32_t h[16];
#pragma unroll
    for (int j = 0; j < 16; j++) h[j] = tanh2_bf16(v[2 * j], v[2 * j + 1]);
#pragma unroll
    for (int q = 0; q < 4; q++)
      sts128(act + umma::kmajor_index(r, c0 + 8 * q, 128), h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]);
  }
}

// Appends this lane to a warp-aggregated list: one atomic per warp; returns the lane's slot
// (meaningful where pred). Every lane of the warp calls it.
__device__ __forceinline__ unsigned int warp_slot(unsigned int *counter, bool pred, int lane) {
  const unsigned int mask = __ballot_sync(0xffffffffu, pred);
  if (!mask) return 0u;
  const int first = __ffs(mask) - 1;
  unsigned int base = 0;
  if (lane == first) base = atomicAdd(counter, (unsigned int)__popc(mask));
  base = __shfl_sync(0xffffffffu, base, first);
  return base + (unsigned int)__popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ void warp_count(unsigned long long *counter, bool pred, int lane) {
  const unsigned int mask = __ballot_sync(0xffffffffu, pred);
  if (mask && lane == __ffs(mask) - 1) atomicAdd(counter, (unsigned long long)__popc(mask));
}

// Per group and tile: the features of the cells' initial state go to the tensor core first
// (layer-1 MMA), then the layers' epilogues and MMAs alternate, with the coarse physics step
// computed while the tensor core runs layer 2 (the longest product); the network's correction is
// applied to the coarse result.
// The block's tiles (blockIdx.x + k * gridDim.x) go to its groups through a shared-memory counter,
// so a group that starts late still takes an even share. kAudit: group kGroups - 1 first audits
// the previous macro step's snapshots (prev) -- on the FP64 pipe the MLP groups leave idle --
// and then takes tiles like the others.
template <int kGroups, bool kAudit>
__global__ void __launch_bounds__(512, 1) sur_step_tc_kernel(const SurKernelArgs a, const SurAuditArgs prev, int n) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar_stage[kGroups], bar_mma[kGroups];
  __shared__ uint32_t tslot;
  __shared__ int s_abort[kGroups], s_tile[kGroups], s_next;
  __nv_bfloat16 *W1 = (__nv_bfloat16 *)smem;
  __nv_bfloat16 *W2 = (__nv_bfloat16 *)(smem + kTcW1);
  __nv_bfloat16 *W3 = (__nv_bfloat16 *)(smem + kTcW1 + kTcW2);
  __nv_bfloat16 *ONES = (__nv_bfloat16 *)(smem + kTcW1 + kTcW2 + kTcW3);
  __nv_bfloat16 *B2T = (__nv_bfloat16 *)(smem + kTcW1 + kTcW2 + kTcW3 + kTcOnes);
  float *b3 = (float *)(smem + kTcW1 + kTcW2 + kTcW3 + kTcOnes + kTcB2);
  const int g = threadIdx.x >> 7, r = threadIdx.x & 127, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char *gbase = smem + kTcHead + g * kTcGroupBytes;
  __nv_bfloat16 *act = (__nv_bfloat16 *)gbase;
  float *stage = (float *)(gbase + kTcAct);
  const bool leader = r == 0;
  const DevBatch &fb = a.fine;
  const int64_t ld = fb.ld;
  const float *const *het = (const float *const *)fb.het;
  const int n_tiles = (n + kTcCells - 1) / kTcCells;
  auto grab = [&]() -> int {  // the block's next tile (leader threads)
    return (int)blockIdx.x + atomicAdd(&s_next, 1) * (int)gridDim.x;
  };
  // The tile's 21 state planes, issued by the group's first warp: lane 0 posts the byte count,
  // then lane v copies plane v (one bulk copy per lane instead of 21 from one thread).
  auto issue = [&](int tile) {
    if (tile == fb.fault_skip_tile) return;  // test hook: this tile's copy is never issued
    const int64_t c0 = (int64_t)tile * kTcCells;
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    if (lane == 0) mbar_expect_tx(&bar_stage[g], (uint32_t)kTcStageVars * kTcCells * 4u);
    __syncwarp();
    if (lane < kTcStageVars) bulk_g2s(stage + lane * kTcCells, fb.s32 + lane * ld + c0, kTcCells * 4u, &bar_stage[g]);
  };
  const bool issuer = (threadIdx.x & 127) < 32;  // the group's first warp
  auto next_tile = [&]() {  // the issuing warp takes the group's next tile and starts its copies
    int tn = 0;
    if (lane == 0) {
      tn = grab();
      s_tile[g] = tn;
    }
    tn = __shfl_sync(0xffffffffu, tn, 0);
    if (tn < n_tiles) issue(tn);
  };
  if (threadIdx.x == 0) s_next = 0;
  if (leader && g < kGroups) {
    mbar_init(&bar_stage[g], 1);
    mbar_init(&bar_mma[g], 1);
    s_abort[g] = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  // network into shared memory in the K-major layout; consecutive threads take consecutive rows
  // of one 16-byte K chunk, so each quarter-warp stores 128 contiguous bytes
  {
    const uint4 *w1 = (const uint4 *)a.w1, *w2 = (const uint4 *)a.w2, *w3 = (const uint4 *)a.w3;
    for (int i = threadIdx.x; i < 128 * 4; i += blockDim.x) {
      const int row = i & 127, ch = i >> 7;
      *(uint4 *)(W1 + umma::kmajor_index(row, ch * 8, 32)) = w1[row * 4 + ch];
    }
    for (int i = threadIdx.x; i < 128 * 16; i += blockDim.x) {
      const int row = i & 127, ch = i >> 7;
      *(uint4 *)(W2 + umma::kmajor_index(row, ch * 8, 128)) = w2[row * 16 + ch];
    }
    for (int i = threadIdx.x; i < 32 * 16; i += blockDim.x) {
      const int row = i & 31, ch = i >> 5;
      *(uint4 *)(W3 + umma::kmajor_index(row, ch * 8, 128)) = w3[row * 16 + ch];
    }
    // the bias operands: ONES (column 0 = 1), B2T (column 0 = b2), b3 in FP32
    const __nv_bfloat16 one = __float2bfloat16(1.f), zero = __float2bfloat16(0.f);
    for (int i = threadIdx.x; i < 128 * 16; i += blockDim.x) {
      const int row = i >> 4, k = i & 15;
      ONES[umma::kmajor_index(row, k, 16)] = k == 0 ? one : zero;
      B2T[umma::kmajor_index(row, k, 16)] = k == 0 ? __float2bfloat16(a.bias[128 + row]) : zero;
    }
    for (int i = threadIdx.x; i < 32; i += blockDim.x) b3[i] = a.bias[256 + i];
    __syncthreads();  // W1's rows are in place: column 22 (padding, zero) takes b1
    for (int i = threadIdx.x; i < 128; i += blockDim.x) W1[umma::kmajor_index(i, kSurIn, 32)] = __float2bfloat16(a.bias[i]);
  }
  const bool mlp_on = a.mode == 0 && !a.stim_on;
  constexpr uint32_t kCols = kGroups == 1 ? 128 : (kGroups == 2 ? 256 : 512);
  if (mlp_on && warp == 0) umma::tmem_alloc(&tslot, kCols);
  umma::fence_smem_to_async();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tbase = mlp_on ? tslot : 0u;
  const uint32_t tacc = tbase + (uint32_t)(g * 128) + ((uint32_t)((warp & 3) * 32) << 16);  // this warp's lanes
  const uint32_t tacc_mma = tbase + (uint32_t)(g * 128);
  if (kAudit && g == kGroups - 1) {  // the audit group: entries of the previous step's snapshot
    audit_range(prev, blockIdx.x * 128 + r, gridDim.x * 128);
  }
  if (issuer) next_tile();
  group_sync(g);
  int t = s_tile[g];
  const float macro_ms = a.coarse.dt * 1000.f;
  const TT2Consts<float> &C = fb.tt2_32;
  uint32_t ps = 0, pm = 0;  // mbarrier phase parities
  const uint32_t act_s = smem_u32(act), w1_s = smem_u32(W1), w2_s = smem_u32(W2), w3_s = smem_u32(W3);
  const uint32_t ones_s = smem_u32(ONES), b2_s = smem_u32(B2T);
  auto wait_mma = [&]() {
    if (!mbar_wait(&bar_mma[g], pm, fb.spin_limit)) {
      s_abort[g] = 1;
      atomicOr(fb.audit_or, kAuditTimeout);
    }
    pm ^= 1u;
    umma::fence_after_sync();
  };
  auto operands_ready = [&]() {  // this group's act rows written -> the leader may issue the next MMA
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    group_sync(g);
  };
  int t_next = n_tiles;
  double vm_pf = 0.0;    // page-locked host Vm of this thread's cell of the next tile, loaded early
  bool have_pf = false;
  while (t < n_tiles) {
    const int c = t * kTcCells + r;
    const bool valid = c < n;
    // loads that do not come through the stage go first: their latency overlaps the stage wait
    // Vm: the device planes (c < ld: padding cells too), or the caller's page-locked host array
    // (plain load, or the one issued during the last tile; padding cells 0)
    const Acc vm = a.vm ? acc_from_double(have_pf ? vm_pf : (valid ? a.vm[c] : 0.0))
                        : Acc{__ldg(a.vm_hi + c), __ldg(a.vm_lo + c)};
    have_pf = false;
    const int cc = valid ? c : 0;  // conductance planes: the tile's padding cells read cell 0
    TT2Het_<float> g6;
    g6.g_Na = het[H2_g_Na] ? __ldg(het[H2_g_Na] + cc) : C.g_Na;
    g6.g_Kr = het[H2_g_Kr] ? __ldg(het[H2_g_Kr] + cc) : C.g_Kr;
    g6.g_K1 = het[H2_g_K1] ? __ldg(het[H2_g_K1] + cc) : C.g_K1;
    g6.g_Ks = het[H2_g_Ks] ? __ldg(het[H2_g_Ks] + cc) : C.g_Ks;
    g6.g_to = het[H2_g_to] ? __ldg(het[H2_g_to] + cc) : C.g_to;
    g6.g_CaL = het[H2_g_CaL] ? __ldg(het[H2_g_CaL] + cc) : C.g_CaL;
    if (!mbar_wait(&bar_stage[g], ps, fb.spin_limit)) {
      s_abort[g] = 1;
      atomicOr(fb.audit_or, kAuditTimeout);
    }
    ps ^= 1u;
    // the group agrees on a timeout at its next barrier: here without the network, after the
    // features in the learned mode (a thread whose wait ran out computes them from whatever the
    // stage holds; nothing of it leaves shared memory)
    if (!mlp_on) {
      group_sync(g);
      if (s_abort[g]) {
        mbar_wait(&bar_stage[g], ps ^ 1u, fb.spin_limit);  // the copy that timed out: one more bounded wait
        break;
      }
    }
    const float *S = stage + r;
    Cell q;
    q.x.m = S[0]; q.x.h = S[kTcCells]; q.x.j = S[2 * kTcCells]; q.x.xr1 = S[3 * kTcCells];
    q.x.xr2 = S[4 * kTcCells]; q.x.xs = S[5 * kTcCells]; q.x.r = S[6 * kTcCells]; q.x.s = S[7 * kTcCells];
    q.x.d = S[8 * kTcCells]; q.x.f = S[9 * kTcCells]; q.x.f2 = S[10 * kTcCells]; q.x.fCa = S[11 * kTcCells];
    q.x.Rq = S[12 * kTcCells]; q.x.Ca_i = S[13 * kTcCells]; q.x.CaSS = S[14 * kTcCells];
    q.CaSR = Acc{S[15 * kTcCells], S[16 * kTcCells]};
    q.Na = Acc{S[17 * kTcCells], S[18 * kTcCells]};
    q.K = Acc{S[19 * kTcCells], S[20 * kTcCells]};
    q.g = g6;
    if (!mlp_on) {  // the stage is free: the next tile's copies overlap this tile's work
      group_sync(g);
      if (issuer) next_tile();
    }
    if (mlp_on) {  // features of the initial state -> row r of the 128 x 32 input tile
      float f[kSurIn];
      features(q, (vm.hi + vm.lo) * 1000.f, a.inv_g0_Na, a.inv_g0_Kr, a.inv_g0_K1, f);
      uint32_t xb[16];
#pragma unroll
      for (int j = 0; j < 16; j++) {
        const int k0 = 2 * j, k1 = 2 * j + 1;
        // column kSurIn = 1 carries b1; padding 0
        const float x0 = k0 < kSurIn ? (valid ? (f[k0] - a.norm.mu_x[k0]) * a.norm.inv_sd_x[k0] : 0.f)
                                     : (k0 == kSurIn ? 1.f : 0.f);
        const float x1 = k1 < kSurIn ? (valid ? (f[k1] - a.norm.mu_x[k1]) * a.norm.inv_sd_x[k1] : 0.f)
                                     : (k1 == kSurIn ? 1.f : 0.f);
        xb[j] = pack_bf16(x0, x1);
      }
#pragma unroll
      for (int qd = 0; qd < 4; qd++)
        sts128(act + umma::kmajor_index(r, 8 * qd, 32), xb[4 * qd], xb[4 * qd + 1], xb[4 * qd + 2], xb[4 * qd + 3]);
      operands_ready();  // also: every thread has read its state from the stage
      if (s_abort[g]) {
        mbar_wait(&bar_stage[g], ps ^ 1u, fb.spin_limit);  // the copy that timed out: one more bounded wait
        break;
      }
      if (leader) {  // layer 1: D = X W1^T (K = 32)
        umma::fence_after_sync();
        constexpr uint32_t id = umma::idesc_bf16_f32(128, 128);
#pragma unroll
        for (int s = 0; s < 2; s++)
          umma::mma_bf16(tacc_mma, umma::smem_desc(act_s + s * 256u, 128u, 512u), umma::smem_desc(w1_s + s * 256u, 128u, 512u), id, s);
        umma::commit(&bar_mma[g]);
      }
      if (issuer) next_tile();  // the stage is free: the next tile's copies overlap this tile's work
    }
    // coarse physics step (registers only): in the learned mode while the tensor core computes
    // hidden layer 2, the longest of the three products
    float oc[kSurOut], inc[4];
    bool fall = !valid;
    auto coarse_step = [&]() {
      if (valid) {
        coarse(a.coarse, a.rows_coarse, a.eca, q, vm, oc, inc);
        const float rate = fabsf(inc[0]) / macro_ms;
        const bool stim = a.stim_on || (a.tb_cell && f64_ge(a.t_last, a.tb_cell[c]));
        fall = stim || !(rate <= a.gate_mv_per_ms);
      }
    };
    if (!mlp_on) coarse_step();
    float y[32];
    if (mlp_on) {
      wait_mma();
      tc_hidden_epilogue(tacc, act, r);
      operands_ready();
      // the issuing warp wrote the group's next tile index before it reached this barrier (and
      // writes the one after only past the next tile's first barrier, which this warp must reach)
      t_next = s_tile[g];
      if (a.vm) {  // host Vm of the next tile: the link's latency overlaps layers 2 and 3
        const int cn = t_next * kTcCells + r;
        vm_pf = (t_next < n_tiles && cn < n) ? a.vm[cn] : 0.0;
        have_pf = true;
      }
      if (leader) {  // layer 2: D = H1 W2^T, K = 128
        umma::fence_after_sync();
        constexpr uint32_t id = umma::idesc_bf16_f32(128, 128);
#pragma unroll
        for (int s = 0; s < 8; s++)
          umma::mma_bf16(tacc_mma, umma::smem_desc(act_s + s * 256u, 128u, 2048u), umma::smem_desc(w2_s + s * 256u, 128u, 2048u), id, s);
        // + ONES (128 x 16) B2T^T: every row gets b2
        umma::mma_bf16(tacc_mma, umma::smem_desc(ones_s, 128u, 256u), umma::smem_desc(b2_s, 128u, 256u), id, 1u);
        umma::commit(&bar_mma[g]);
      }
      coarse_step();
      wait_mma();
      tc_hidden_epilogue(tacc, act, r);
      operands_ready();
      if (leader) {  // output layer: D = H2 W3^T, N = 32
        umma::fence_after_sync();
        constexpr uint32_t id = umma::idesc_bf16_f32(128, 32);
#pragma unroll
        for (int s = 0; s < 8; s++)
          umma::mma_bf16(tacc_mma, umma::smem_desc(act_s + s * 256u, 128u, 2048u), umma::smem_desc(w3_s + s * 256u, 128u, 2048u), id, s);
        umma::commit(&bar_mma[g]);
      }
      wait_mma();
      umma::tmem_ld32(tacc, y);
      umma::fence_before_sync();
#pragma unroll
      for (int k = 0; k < kSurOut; k++) y[k] += b3[k];
    } else {
#pragma unroll
      for (int k = 0; k < 32; k++) y[k] = 0.f;
    }
    bool took = false;
    float pred = 0.f;
    if (valid) {
      if (!fall) {
        float on[kSurOut], corr[kSurOut];
#pragma unroll
        for (int k = 0; k < kSurOut; k++) {
          corr[k] = a.mode == 0 ? a.norm.apply_y[k] * y[k] : 0.f;
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
        } else {
          Cell nq = q;
          Acc nvm = vm;
          apply(nq, nvm, on, inc, corr);
          store_cell(fb, c, nq);
          if (a.vm) {
            a.vm[c] = acc_to_double(nvm);
          } else {
            a.vm_hi[c] = nvm.hi;
            a.vm_lo[c] = nvm.lo;
          }
          pred = (nvm.hi + nvm.lo) * 1000.f;
          took = true;
        }
      }
    }
    // audit sample: the accepted steps of this step's audited cells, with their initial state
    const bool snap = took && a.audit_mod > 0 && (c % a.audit_mod) == a.audit_phase;
    const unsigned int si = warp_slot(a.n_snap, snap, lane);
    if (snap && si < (unsigned int)a.snap_cap) {
      float *D = a.snap + si;
      const int64_t cap = a.snap_cap;
      D[0] = q.x.m; D[cap] = q.x.h; D[2 * cap] = q.x.j; D[3 * cap] = q.x.xr1; D[4 * cap] = q.x.xr2;
      D[5 * cap] = q.x.xs; D[6 * cap] = q.x.r; D[7 * cap] = q.x.s; D[8 * cap] = q.x.d; D[9 * cap] = q.x.f;
      D[10 * cap] = q.x.f2; D[11 * cap] = q.x.fCa; D[12 * cap] = q.x.Rq; D[13 * cap] = q.x.Ca_i;
      D[14 * cap] = q.x.CaSS; D[15 * cap] = q.CaSR.hi; D[16 * cap] = q.CaSR.lo; D[17 * cap] = q.Na.hi;
      D[18 * cap] = q.Na.lo; D[19 * cap] = q.K.hi; D[20 * cap] = q.K.lo; D[21 * cap] = vm.hi; D[22 * cap] = vm.lo;
      D[23 * cap] = q.g.g_Na; D[24 * cap] = q.g.g_Kr; D[25 * cap] = q.g.g_K1; D[26 * cap] = q.g.g_Ks;
      D[27 * cap] = q.g.g_to; D[28 * cap] = q.g.g_CaL; D[29 * cap] = pred;
    }
    const bool listed = valid && fall;
    const unsigned int slot = warp_slot(a.n_fallback, listed, lane);
    if (listed) a.fallback[slot] = c;
    warp_count(a.n_fallback_total, listed, lane);
    warp_count(a.n_sur, took, lane);
    if (mlp_on) {
      t = t_next;
    } else {
      group_sync(g);  // the issuing warp's next tile index is visible
      t = s_tile[g];
    }
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  if (mlp_on && warp == 0) umma::tmem_free(tslot, kCols);
}


}  // namespace

int64_t sur_append_scratch_words(int64_t n) { return (n + kAppendChunk - 1) / kAppendChunk; }

cudaError_t launch_sur_append(const float *X, const float *T, const uint8_t *keep, int64_t n, float *dX, float *dT,
                              unsigned long long *count, int64_t cap, int64_t *chunk_scratch, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t n_chunks = sur_append_scratch_words(n);
  const unsigned g = (unsigned)(n_chunks < 4096 ? n_chunks : 4096);
  sur_append_count_kernel<<<g, kAppendThreads, 0, s>>>(keep, n, chunk_scratch);
  sur_append_scan_kernel<<<1, 1024, 0, s>>>(chunk_scratch, n_chunks, count);
  sur_append_kernel<<<g, kAppendThreads, 0, s>>>(X, T, keep, n, chunk_scratch, dX, dT, cap);
  return cudaGetLastError();
}

cudaError_t launch_sur_normalize(const float *X, const float *T, int64_t n, const SurNorm &norm, float *nX, float *nT,
                                 cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t g = (n + 255) / 256;
  sur_normalize_kernel<<<(unsigned)(g < 8192 ? g : 8192), 256, 0, s>>>(X, T, n, norm, nX, nT);
  return cudaGetLastError();
}

template <bool kAudit>
cudaError_t launch_sur_step_t(const SurKernelArgs &a, const SurAuditArgs &prev, int64_t n, cudaStream_t s) {
  constexpr int kG = 4;
  constexpr int smem = tc_smem_bytes(kG);
  static std::atomic<uint64_t> done{0};
  cudaError_t e = smem_limit((const void *)sur_step_tc_kernel<kG, kAudit>, smem, done);
  if (e != cudaSuccess) return e;
  if (n <= 0) return cudaSuccess;
  const int64_t need = (n + kTcCells * kG - 1) / (kTcCells * kG);
  const int64_t cap = (int64_t)sm_count();
  const int grid = (int)(need < cap ? need : cap);
  sur_step_tc_kernel<kG, kAudit><<<grid, kG * 128, smem, s>>>(a, prev, (int)n);
  return cudaGetLastError();
}

cudaError_t launch_sur_step(const SurKernelArgs &a, const SurAuditArgs *prev, int64_t n, cudaStream_t s) {
  if (prev) return launch_sur_step_t<true>(a, *prev, n, s);
  return launch_sur_step_t<false>(a, SurAuditArgs{}, n, s);
}

cudaError_t launch_sur_audit(const SurAuditArgs &a, cudaStream_t s) {
  sur_audit_kernel<<<sm_count() * 4, 128, 0, s>>>(a);
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
