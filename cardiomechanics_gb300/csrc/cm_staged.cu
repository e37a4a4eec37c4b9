// Mixed-form kernels that stage each tile's state through shared memory with bulk async copies
// (cp.async.bulk on the TMA engine, completion counted by an mbarrier), double-buffered: while a
// block integrates tile t from one buffer, the copies of its next tile land in the other. Each
// state variable of a tile of kThreads consecutive cells is one contiguous kThreads*4-byte run of
// the structure-of-arrays state, so a tile is ~30 bulk copies issued by one thread. Results go
// straight back to global memory. Used for fused runs (Vm as compensated planes), where the
// library owns every staged array and pads it to the batch's leading dimension (a multiple of
// 256 cells), so whole tiles stay inside the allocations.
//
// Every wait is bounded: a wait that runs out sets CM_AUDIT_TIMEOUT in the batch's audit word,
// waits (bounded) for the block's other copy in flight, and the block returns.
#include <cuda_runtime.h>

#include "cm_bulk.cuh"
#include "cm_cells.cuh"
#include "cm_launch.h"

namespace cm {

namespace {

template <int kModel>
struct Vars;
template <>
struct Vars<5> {
  static constexpr int kState = 21;  // tt2 mixed planes
};
template <>
struct Vars<2> {
  static constexpr int kState = 25;
};

// Staged variables of a tile: state planes, Vm hi, Vm lo, then the present hetero slots.
template <int kModel, int kThreads>
__global__ void __launch_bounds__(kThreads, 2) mixed_staged_kernel(const DevBatch b, const StepIO io) {
  constexpr int NS = Vars<kModel>::kState;
  constexpr int NVMAX = NS + 2 + 6;
  extern __shared__ __align__(128) float stage[];  // [2][NVMAX][kThreads]
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ int s_abort;
  const int64_t ld = b.ld;
  const int n = (int)b.n;
  const int n_tiles = (n + kThreads - 1) / kThreads;
  // which hetero slots are staged, and where
  int het_pos[6];
  int nv = NS + 2;
#pragma unroll
  for (int k = 0; k < 6; k++) het_pos[k] = b.het[k] ? nv++ : -1;
  const uint32_t tile_bytes = (uint32_t)nv * kThreads * 4u;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int tile, int buf) {
    float *dst = stage + (size_t)buf * NVMAX * kThreads;
    const int64_t c0 = (int64_t)tile * kThreads;
    mbar_expect_tx(&bar[buf], tile_bytes);
    for (int v = 0; v < NS; v++) bulk_g2s(dst + v * kThreads, b.s32 + v * ld + c0, kThreads * 4u, &bar[buf]);
    bulk_g2s(dst + NS * kThreads, io.vm_hi + c0, kThreads * 4u, &bar[buf]);
    bulk_g2s(dst + (NS + 1) * kThreads, io.vm_lo + c0, kThreads * 4u, &bar[buf]);
    for (int k = 0; k < 6; k++)
      if (het_pos[k] >= 0)
        bulk_g2s(dst + het_pos[k] * kThreads, (const float *)b.het[k] + c0, kThreads * 4u, &bar[buf]);
  };
  int it = 0;
  int t = blockIdx.x;
  if (t < n_tiles && threadIdx.x == 0) issue(t, 0);
  for (; t < n_tiles; t += gridDim.x, it++) {
    const int buf = it & 1;
    const int next = t + gridDim.x;
    __syncthreads();  // every thread is done with buffer buf ^ 1 (used two tiles ago)
    if (next < n_tiles && threadIdx.x == 0) {
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      issue(next, buf ^ 1);
    }
    if (!mbar_wait(&bar[buf], (uint32_t)((it >> 1) & 1))) {
      s_abort = 1;
      atomicOr(b.audit_or, kAuditTimeout);
    }
    __syncthreads();
    if (s_abort) {
      if (next < n_tiles) mbar_wait(&bar[buf ^ 1], (uint32_t)(((it + 1) >> 1) & 1));
      return;
    }
    const float *S = stage + (size_t)buf * NVMAX * kThreads + threadIdx.x;
    const int c = t * kThreads + threadIdx.x;
    if (c >= n) continue;
    const float iext = (float)io.iext_uniform;
    uint32_t audit = 0;
    Acc vm{S[NS * kThreads], S[(NS + 1) * kThreads]};
    float *s = b.s32 + c;
    if (kModel == 5) {
      const TT2Consts<float> &C = b.tt2_32;
      TT2Cell<float> x;
      x.m = S[0]; x.h = S[kThreads]; x.j = S[2 * kThreads]; x.xr1 = S[3 * kThreads]; x.xr2 = S[4 * kThreads];
      x.xs = S[5 * kThreads]; x.r = S[6 * kThreads]; x.s = S[7 * kThreads]; x.d = S[8 * kThreads];
      x.f = S[9 * kThreads]; x.f2 = S[10 * kThreads]; x.fCa = S[11 * kThreads]; x.Rq = S[12 * kThreads];
      x.Ca_i = S[13 * kThreads]; x.CaSS = S[14 * kThreads];
      Acc CaSR{S[15 * kThreads], S[16 * kThreads]}, Na_i{S[17 * kThreads], S[18 * kThreads]},
          K_i{S[19 * kThreads], S[20 * kThreads]};
      TT2Het_<float> g;
      g.g_Na = het_pos[H2_g_Na] >= 0 ? S[het_pos[H2_g_Na] * kThreads] : C.g_Na;
      g.g_Kr = het_pos[H2_g_Kr] >= 0 ? S[het_pos[H2_g_Kr] * kThreads] : C.g_Kr;
      g.g_K1 = het_pos[H2_g_K1] >= 0 ? S[het_pos[H2_g_K1] * kThreads] : C.g_K1;
      g.g_Ks = het_pos[H2_g_Ks] >= 0 ? S[het_pos[H2_g_Ks] * kThreads] : C.g_Ks;
      g.g_to = het_pos[H2_g_to] >= 0 ? S[het_pos[H2_g_to] * kThreads] : C.g_to;
      g.g_CaL = het_pos[H2_g_CaL] >= 0 ? S[het_pos[H2_g_CaL] * kThreads] : C.g_CaL;
      const int vi = vrow_fp32(vm.hi * 1000.f, audit);
      const float dV = tt2_calc_mixed(C, b.rows32 + (size_t)vi * T2_COLS, b.eca32, x, CaSR, Na_i, K_i, g, vm.hi,
                                      iext, audit);
      s[0] = x.m; s[ld] = x.h; s[2 * ld] = x.j; s[3 * ld] = x.xr1; s[4 * ld] = x.xr2; s[5 * ld] = x.xs;
      s[6 * ld] = x.r; s[7 * ld] = x.s; s[8 * ld] = x.d; s[9 * ld] = x.f; s[10 * ld] = x.f2;
      s[11 * ld] = x.fCa; s[12 * ld] = x.Rq; s[13 * ld] = x.Ca_i; s[14 * ld] = x.CaSS;
      s[15 * ld] = CaSR.hi; s[16 * ld] = CaSR.lo; s[17 * ld] = Na_i.hi; s[18 * ld] = Na_i.lo;
      s[19 * ld] = K_i.hi; s[20 * ld] = K_i.lo;
      acc_add(vm, dV);
    } else {
      const CRNConsts<float> &C = b.crn_32;
      CRNCell<float> x;
      x.h = S[0]; x.j = S[kThreads]; x.oi = S[2 * kThreads]; x.ui = S[3 * kThreads]; x.Xr = S[4 * kThreads];
      x.Xs = S[5 * kThreads]; x.u = S[6 * kThreads]; x.v = S[7 * kThreads]; x.w = S[8 * kThreads];
      x.m = S[9 * kThreads]; x.oa = S[10 * kThreads]; x.ua = S[11 * kThreads]; x.d = S[12 * kThreads];
      x.f = S[13 * kThreads]; x.f_Ca = S[14 * kThreads]; x.Ca_i = S[15 * kThreads]; x.Ca_TRPN = S[16 * kThreads];
      Acc Ca_up{S[17 * kThreads], S[18 * kThreads]}, Ca_rel{S[19 * kThreads], S[20 * kThreads]},
          Na_i{S[21 * kThreads], S[22 * kThreads]}, K_i{S[23 * kThreads], S[24 * kThreads]};
      CRNHet_<float> g;
      g.g_Na = het_pos[HC_g_Na] >= 0 ? S[het_pos[HC_g_Na] * kThreads] : C.g_Na;
      g.g_to = het_pos[HC_g_to] >= 0 ? S[het_pos[HC_g_to] * kThreads] : C.g_to;
      g.g_Ks = het_pos[HC_g_Ks] >= 0 ? S[het_pos[HC_g_Ks] * kThreads] : C.g_Ks;
      g.g_CaL = het_pos[HC_g_CaL] >= 0 ? S[het_pos[HC_g_CaL] * kThreads] : C.g_CaL;
      g.g_bNa = het_pos[HC_g_bNa] >= 0 ? S[het_pos[HC_g_bNa] * kThreads] : C.g_bNa;
      g.g_bCa = het_pos[HC_g_bCa] >= 0 ? S[het_pos[HC_g_bCa] * kThreads] : C.g_bCa;
      const int vi = vrow_fp32(vm.hi * 1000.f, audit);
      const float dV = crn_calc_mixed(C, b.rows32 + (size_t)vi * CR_COLS, x, Ca_up, Ca_rel, Na_i, K_i, g, vm.hi,
                                      iext, 1.f, audit);
      s[0] = x.h; s[ld] = x.j; s[2 * ld] = x.oi; s[3 * ld] = x.ui; s[4 * ld] = x.Xr; s[5 * ld] = x.Xs;
      s[6 * ld] = x.u; s[7 * ld] = x.v; s[8 * ld] = x.w; s[9 * ld] = x.m; s[10 * ld] = x.oa; s[11 * ld] = x.ua;
      s[12 * ld] = x.d; s[13 * ld] = x.f; s[14 * ld] = x.f_Ca; s[15 * ld] = x.Ca_i; s[16 * ld] = x.Ca_TRPN;
      s[17 * ld] = Ca_up.hi; s[18 * ld] = Ca_up.lo; s[19 * ld] = Ca_rel.hi; s[20 * ld] = Ca_rel.lo;
      s[21 * ld] = Na_i.hi; s[22 * ld] = Na_i.lo; s[23 * ld] = K_i.hi; s[24 * ld] = K_i.lo;
      acc_add(vm, dV);
    }
    io.vm_hi[c] = vm.hi;
    io.vm_lo[c] = vm.lo;
    if (!isfinite(vm.hi)) audit |= 1u;
    if (audit) {
      atomicOr(b.audit_cell + c, audit);
      atomicOr(b.audit_or, audit);
    }
  }
}

template <int kModel, int kThreads>
cudaError_t launch_staged_t(const DevBatch &b, const StepIO &io, int blocks_per_sm, cudaStream_t s) {
  constexpr int NVMAX = Vars<kModel>::kState + 2 + 6;
  const size_t smem = (size_t)2 * NVMAX * kThreads * sizeof(float);
  static bool configured = false;  // one attribute call per instantiation and process
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(mixed_staged_kernel<kModel, kThreads>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const int n_tiles = (int)((b.n + kThreads - 1) / kThreads);
  int grid = sm_count() * (blocks_per_sm > 0 ? blocks_per_sm : 2);
  if (grid > n_tiles) grid = n_tiles;
  if (grid < 1) grid = 1;
  mixed_staged_kernel<kModel, kThreads><<<grid, kThreads, smem, s>>>(b, io);
  return cudaGetLastError();
}

}  // namespace

bool staged_supported(const DevBatch &b, const StepIO &io) {
  return b.precision == 1 && io.vm_hi && io.vm_lo && !io.tb_cell && !io.iext && b.ld % 256 == 0 &&
         io.vm_lo == io.vm_hi + b.ld && b.n < (int64_t)1 << 30;
}

cudaError_t launch_staged(const DevBatch &b, const StepIO &io, int threads, int blocks_per_sm, cudaStream_t s) {
  if (b.n == 0) return cudaSuccess;
  if (b.model == 5) {
    if (threads == 128) return launch_staged_t<5, 128>(b, io, blocks_per_sm, s);
    return launch_staged_t<5, 256>(b, io, blocks_per_sm, s);
  }
  if (threads == 128) return launch_staged_t<2, 128>(b, io, blocks_per_sm, s);
  return launch_staged_t<2, 256>(b, io, blocks_per_sm, s);
}

}  // namespace cm
