// Batched form: many batches (instances) of uneven size and mixed model, advanced by one
// persistent launch per time step. The cells of all instances are cut into tiles of
// `tile_cells`; blocks take tiles from an atomic counter until none are left, so large and
// small instances, and the costlier Courtemanche tiles, balance across the 152 SMs by
// themselves. Each instance carries its own stimulus clock on the device (double-buffered by
// step parity), so consecutive steps are identical launches that a CUDA graph can replay.
#include <cuda_runtime.h>

#include "cm_bulk.cuh"
#include "cm_cells.cuh"
#include "cm_multi.h"
#include "cm_staged_cell.cuh"

namespace cm {

namespace {

template <int kBlock, int kMinB>
__global__ void __launch_bounds__(kBlock, kMinB)
    multi_kernel(const MultiInst *__restrict__ insts, const MultiTile *__restrict__ tiles, int n_tiles,
                 const MultiClock *__restrict__ clk_cur, MultiClock *__restrict__ clk_next,
                 unsigned int *__restrict__ counter, unsigned int *__restrict__ counter_next) {
  __shared__ DevBatch sb;
  __shared__ int s_tile;
  if (blockIdx.x == 0 && threadIdx.x == 0) *counter_next = 0;  // the next step's counter
  for (;;) {
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int tile = s_tile;
    if (tile >= n_tiles) break;
    const MultiTile T = tiles[tile];
    const MultiInst *I = insts + T.inst;
    {  // the instance's batch descriptor (pointers + constants) into shared memory
      const int4 *src = reinterpret_cast<const int4 *>(&I->d);
      int4 *dst = reinterpret_cast<int4 *>(&sb);
      for (int k = threadIdx.x; k < (int)(sizeof(DevBatch) / sizeof(int4)); k += kBlock) dst[k] = src[k];
    }
    const MultiClock ck = clk_cur[T.inst];
    const double amp = I->amp, textlen = I->textlen, bcl = I->bcl, dt = I->dt;
    float *vm_hi = I->vm_hi, *vm_lo = I->vm_lo;
    __syncthreads();
    // reference driver stimulus (CellModel.h:405-419) with this instance's clock
    const float iext = ck.t >= ck.tb ? (float)amp : 0.f;
    if (T.start == 0 && threadIdx.x == 0) {
      MultiClock nx;
      nx.t = ck.t + dt;
      nx.tb = (ck.t >= ck.tb && ck.t >= ck.tb + textlen) ? ck.tb + bcl : ck.tb;
      clk_next[T.inst] = nx;
    }
    const int end = T.start + T.count;
    if (sb.model == 5) {
      for (int c = T.start + threadIdx.x; c < end; c += kBlock) {
        Acc v{vm_hi[c], vm_lo[c]};
        uint32_t audit = 0;
        acc_add(v, tt2_mixed_cell<int>(sb, c, v.hi, iext, audit));
        vm_hi[c] = v.hi;
        vm_lo[c] = v.lo;
        if (!isfinite(v.hi)) audit |= 1u;
        if (audit) {
          atomicOr(sb.audit_cell + c, audit);
          atomicOr(sb.audit_or, audit);
        }
      }
    } else {
      for (int c = T.start + threadIdx.x; c < end; c += kBlock) {
        Acc v{vm_hi[c], vm_lo[c]};
        uint32_t audit = 0;
        acc_add(v, crn_mixed_cell<int>(sb, c, v.hi, iext, 1.f, audit));
        vm_hi[c] = v.hi;
        vm_lo[c] = v.lo;
        if (!isfinite(v.hi)) audit |= 1u;
        if (audit) {
          atomicOr(sb.audit_cell + c, audit);
          atomicOr(sb.audit_or, audit);
        }
      }
    }
    __syncthreads();  // sb and s_tile are rewritten for the next tile
  }
}

// The same step with each tile's cells staged through shared memory by bulk async copies in
// sub-tiles of kT cells, double-buffered: thread 0 schedules the block's next sub-tile (the next
// one of its tile, or a new tile from the counter) and issues its copies before the block
// integrates the current one. The instance's descriptor is copied to shared memory when the
// block moves to another instance. Requires tile starts and sizes in whole sub-tiles, which the
// launcher checks. Bounded waits as in the single-batch staged kernel.
template <int kT>
__global__ void __launch_bounds__(kT, 2)
    multi_staged_kernel(const MultiInst *__restrict__ insts, const MultiTile *__restrict__ tiles, int n_tiles,
                        const MultiClock *__restrict__ clk_cur, MultiClock *__restrict__ clk_next,
                        unsigned int *__restrict__ counter, unsigned int *__restrict__ counter_next) {
  constexpr int NVMAX = StagedVars<2>::kState + 2 + 6;  // the larger model
  extern __shared__ __align__(128) float stage[];      // [2][NVMAX][kT]
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ DevBatch sb;
  __shared__ int s_tile[2], s_sub[2], s_abort;
  if (blockIdx.x == 0 && threadIdx.x == 0) *counter_next = 0;  // the next step's counter
  auto issue = [&](int tile, int sub, int buf) {  // thread 0
    const MultiTile T = tiles[tile];
    const MultiInst *I = insts + T.inst;
    const int64_t ld = I->d.ld;
    const int ns = I->d.model == 5 ? StagedVars<5>::kState : StagedVars<2>::kState;
    int nh = 0;
    for (int k = 0; k < 6; k++) nh += I->d.het[k] ? 1 : 0;
    const int64_t c0 = (int64_t)T.start + (int64_t)sub * kT;
    float *dst = stage + (size_t)buf * NVMAX * kT;
    mbar_expect_tx(&bar[buf], (uint32_t)(ns + 2 + nh) * kT * 4u);
    for (int v = 0; v < ns; v++) bulk_g2s(dst + v * kT, I->d.s32 + v * ld + c0, kT * 4u, &bar[buf]);
    bulk_g2s(dst + ns * kT, I->vm_hi + c0, kT * 4u, &bar[buf]);
    bulk_g2s(dst + (ns + 1) * kT, I->vm_lo + c0, kT * 4u, &bar[buf]);
    int pos = ns + 2;
    for (int k = 0; k < 6; k++)
      if (I->d.het[k]) bulk_g2s(dst + (pos++) * kT, (const float *)I->d.het[k] + c0, kT * 4u, &bar[buf]);
  };
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    const int t0 = (int)atomicAdd(counter, 1u);
    s_tile[0] = t0 < n_tiles ? t0 : -1;
    s_sub[0] = 0;
    if (t0 < n_tiles) issue(t0, 0, 0);
  }
  int cur_inst = -1;
  int het_pos[6] = {-1, -1, -1, -1, -1, -1};
  for (int it = 0;; it++) {
    const int buf = it & 1;
    __syncthreads();  // s_tile[buf] is visible; buffer buf ^ 1 and sb are free
    const int tile = s_tile[buf];
    if (tile < 0) break;
    const int sub = s_sub[buf];
    const MultiTile T = tiles[tile];
    if (threadIdx.x == 0) {  // the block's next sub-tile, prefetched into the other buffer
      int nt = tile, nsub = sub + 1;
      if ((int64_t)nsub * kT >= T.count) {
        const int a = (int)atomicAdd(counter, 1u);
        nt = a < n_tiles ? a : -1;
        nsub = 0;
      }
      s_tile[buf ^ 1] = nt;
      s_sub[buf ^ 1] = nsub;
      if (nt >= 0) {
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        issue(nt, nsub, buf ^ 1);
      }
    }
    const MultiInst *I = insts + T.inst;
    if (T.inst != cur_inst) {  // block-uniform
      const int4 *src = reinterpret_cast<const int4 *>(&I->d);
      int4 *dst = reinterpret_cast<int4 *>(&sb);
      for (int k = threadIdx.x; k < (int)(sizeof(DevBatch) / sizeof(int4)); k += kT) dst[k] = src[k];
      __syncthreads();
      cur_inst = T.inst;
      int pos = sb.model == 5 ? StagedVars<5>::kState + 2 : StagedVars<2>::kState + 2;
#pragma unroll
      for (int k = 0; k < 6; k++) het_pos[k] = sb.het[k] ? pos++ : -1;
    }
    const MultiClock ck = clk_cur[T.inst];
    const float iext = ck.t >= ck.tb ? (float)I->amp : 0.f;
    if (T.start == 0 && sub == 0 && threadIdx.x == 0) {  // reference driver clock (CellModel.h:405-419)
      MultiClock nx;
      nx.t = ck.t + I->dt;
      nx.tb = (ck.t >= ck.tb && ck.t >= ck.tb + I->textlen) ? ck.tb + I->bcl : ck.tb;
      clk_next[T.inst] = nx;
    }
    if (!mbar_wait(&bar[buf], (uint32_t)((it >> 1) & 1))) {
      s_abort = 1;
      atomicOr(sb.audit_or, kAuditTimeout);
    }
    __syncthreads();
    if (s_abort) {
      if (s_tile[buf ^ 1] >= 0) mbar_wait(&bar[buf ^ 1], (uint32_t)(((it + 1) >> 1) & 1));
      return;
    }
    const float *S = stage + (size_t)buf * NVMAX * kT + threadIdx.x;
    const int c = T.start + sub * kT + (int)threadIdx.x;
    if (c < T.start + T.count) {
      if (sb.model == 5) staged_cell<5, kT>(sb, S, het_pos, c, iext, I->vm_hi, I->vm_lo);
      else staged_cell<2, kT>(sb, S, het_pos, c, iext, I->vm_hi, I->vm_lo);
    }
  }
}

// The staged step as a producer/consumer pipeline (as mixed_pipe_kernel): one extra warp
// schedules the block's sub-tiles (the next one of its tile, or a new tile from the counter),
// copies the instance's descriptor into the stage's descriptor slot when the instance changes,
// advances the instance's stimulus clock, and issues the sub-tile's bulk copies; the kT / 32
// consumer warps integrate. Stages pass through `full` and `empty` mbarriers; the end of the
// work is a stage whose tile index is -1. Every wait is bounded: a consumer whose `full` wait
// runs out sets CM_AUDIT_TIMEOUT in the first instance's audit word and leaves; the producer then
// runs out on `empty`, does the same, waits (bounded) for the copies nobody took and leaves.
// Two consistency checks skip work instead of touching memory outside an instance: the producer
// issues no copy for a sub-tile outside its instance (audit bit 256), a consumer warp integrates
// no cell when its stage's descriptor is not its tile's instance's (audit bit 128).
template <int kT, int kStages>
__global__ void __launch_bounds__(kT + 32, 2)
    multi_pipe_kernel(const MultiInst *__restrict__ insts, const MultiTile *__restrict__ tiles, int n_tiles,
                      const MultiClock *__restrict__ clk_cur, MultiClock *__restrict__ clk_next,
                      unsigned int *__restrict__ counter, unsigned int *__restrict__ counter_next) {
  constexpr int NVMAX = StagedVars<2>::kState + 2 + 6;  // the larger model
  constexpr int kWarps = kT / 32;
  extern __shared__ __align__(128) float stage[];      // [kStages][NVMAX][kT]
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages];
  __shared__ __align__(16) DevBatch sd[kStages];
  __shared__ int s_tile[kStages], s_sub[kStages], s_inst[kStages];
  __shared__ float s_iext[kStages];
  if (blockIdx.x == 0 && threadIdx.x == 0) *counter_next = 0;  // the next step's counter
  if (threadIdx.x == 0) {
    for (int k = 0; k < kStages; k++) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], kWarps);
      s_inst[k] = -1;
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x >= kT) {  // the producer warp
    const int lane = threadIdx.x - kT;
    int tile = -1, sub = 0;
    // the current tile's records (lane 0), read once per tile, before the stage wait
    MultiTile T{};
    int64_t ld = 0;
    int ns = 0, nh = 0;
    bool bad = false;
    const float *s32 = nullptr, *vhi = nullptr, *vlo = nullptr;
    const float *hp[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    float iext = 0.f;
    for (int it = 0;; it++) {
      const int st = it % kStages;
      int nt = tile, nsub = sub + 1;
      if (lane == 0 && (tile < 0 || (int64_t)nsub * kT >= T.count)) {
        const int a = (int)atomicAdd(counter, 1u);
        nt = a < n_tiles ? a : -1;
        nsub = 0;
        if (nt >= 0) {
          T = tiles[nt];
          const MultiInst *I = insts + T.inst;
          ld = I->d.ld;
          const int model = I->d.model;
          ns = model == 5 ? StagedVars<5>::kState : StagedVars<2>::kState;
          bad = model != 5 && model != 2;
          s32 = I->d.s32;
          vhi = I->vm_hi;
          vlo = I->vm_lo;
          nh = 0;
#pragma unroll
          for (int k = 0; k < 6; k++) {
            hp[k] = (const float *)I->d.het[k];
            nh += hp[k] ? 1 : 0;
          }
          const MultiClock ck = clk_cur[T.inst];
          iext = ck.t >= ck.tb ? (float)I->amp : 0.f;
          if (T.start == 0) {  // reference driver clock (CellModel.h:405-419), once per instance
            MultiClock nx;
            nx.t = ck.t + I->dt;
            nx.tb = (ck.t >= ck.tb && ck.t >= ck.tb + I->textlen) ? ck.tb + I->bcl : ck.tb;
            clk_next[T.inst] = nx;
          }
        }
      }
      nt = __shfl_sync(0xffffffffu, nt, 0);
      nsub = __shfl_sync(0xffffffffu, nsub, 0);
      const int inst = __shfl_sync(0xffffffffu, T.inst, 0);
      int ok = 1;
      if (lane == 0 && it >= kStages) ok = mbar_wait(&empty[st], (uint32_t)((it / kStages - 1) & 1)) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok) {
        if (lane == 0) {
          atomicOr(insts[0].d.audit_or, kAuditTimeout);
          for (int j = it - kStages; j < it; j++)
            if (j >= 0) mbar_wait(&full[j % kStages], (uint32_t)((j / kStages) & 1));
        }
        return;
      }
      if (nt < 0) {  // no work left: an empty stage tells the consumers
        if (lane == 0) {
          s_tile[st] = -1;
          mbar_arrive(&full[st]);
        }
        return;
      }
      // lane 0 decides whether the stage's descriptor slot needs this instance's descriptor and
      // tells the warp: a lane that read s_inst itself could see lane 0's update of it below
      // and skip its share of the copy
      int need = lane == 0 ? (s_inst[st] != inst) : 0;
      need = __shfl_sync(0xffffffffu, need, 0);
      if (need) {  // the instance's descriptor into this stage's slot
        const int4 *src = reinterpret_cast<const int4 *>(&insts[inst].d);
        int4 *dst = reinterpret_cast<int4 *>(&sd[st]);
        for (int k = lane; k < (int)(sizeof(DevBatch) / sizeof(int4)); k += 32) dst[k] = src[k];
      }
      if (lane == 0) {
        s_inst[st] = inst;
        s_tile[st] = nt;
        s_sub[st] = nsub;
        s_iext[st] = iext;
      }
      __syncwarp();
      if (lane == 0) {
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        const int64_t c0 = (int64_t)T.start + (int64_t)nsub * kT;
        float *dst = stage + (size_t)st * NVMAX * kT;
        if (c0 < 0 || c0 + kT > ld || bad) {  // a sub-tile outside its instance
          atomicOr(insts[inst].d.audit_or, kAuditInternal << 1);
          s_tile[st] = -2;  // the consumers skip it
          mbar_arrive(&full[st]);
        } else {
          mbar_expect_tx(&full[st], (uint32_t)(ns + 2 + nh) * kT * 4u);
          for (int v = 0; v < ns; v++) bulk_g2s(dst + v * kT, s32 + v * ld + c0, kT * 4u, &full[st]);
          bulk_g2s(dst + ns * kT, vhi + c0, kT * 4u, &full[st]);
          bulk_g2s(dst + (ns + 1) * kT, vlo + c0, kT * 4u, &full[st]);
          int pos = ns + 2;
#pragma unroll
          for (int k = 0; k < 6; k++)
            if (hp[k]) bulk_g2s(dst + (pos++) * kT, hp[k] + c0, kT * 4u, &full[st]);
        }
      }
      tile = nt;
      sub = nsub;
    }
  }
  const int lane = threadIdx.x & 31;
  for (int it = 0;; it++) {
    const int st = it % kStages;
    if (!mbar_wait(&full[st], (uint32_t)((it / kStages) & 1))) {
      atomicOr(insts[0].d.audit_or, kAuditTimeout);
      return;
    }
    const int tile = s_tile[st];
    if (tile == -1) break;
    if (tile < 0) {  // skipped by the producer's check
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[st]);
      continue;
    }
    const DevBatch &b = sd[st];
    const MultiTile T = tiles[tile];
    const MultiInst *I = insts + T.inst;
    // the stage's descriptor must be its tile's instance's (decided for the whole warp)
    const bool bad = b.s32 != I->d.s32 || b.ld != I->d.ld || b.model != I->d.model ||
                     b.audit_cell != I->d.audit_cell || b.rows32 != I->d.rows32 || b.eca32 != I->d.eca32 || b.audit_or != I->d.audit_or;
    if (__any_sync(0xffffffffu, bad)) {
      if (lane == 0) {
        atomicOr(I->d.audit_or, kAuditInternal);
        mbar_arrive(&empty[st]);
      }
      continue;
    }
    int het_pos[6];
    int pos = b.model == 5 ? StagedVars<5>::kState + 2 : StagedVars<2>::kState + 2;
#pragma unroll
    for (int k = 0; k < 6; k++) het_pos[k] = b.het[k] ? pos++ : -1;
    const float *S = stage + (size_t)st * NVMAX * kT + threadIdx.x;
    const int c = T.start + s_sub[st] * kT + (int)threadIdx.x;
    if (c < T.start + T.count) {
      if (b.model == 5) staged_cell<5, kT>(b, S, het_pos, c, s_iext[st], I->vm_hi, I->vm_lo);
      else staged_cell<2, kT>(b, S, het_pos, c, s_iext[st], I->vm_hi, I->vm_lo);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[st]);
  }
}

struct MShape {
  int block, minb;
  bool staged, pipe;
  int stages;  // the pipelines' stage count
};
constexpr MShape kMShapes[] = {{256, 2, false, false, 0}, {128, 5, false, false, 0}, {512, 1, false, false, 0},
                               {128, 2, true, false, 0},  {256, 2, true, false, 0},  {256, 2, true, true, 2},
                               {128, 2, true, true, 3},   {256, 2, true, true, 3},   {128, 2, true, true, 4}};

template <int kT>
cudaError_t launch_multi_staged(const MultiLaunch &L, const MultiClock *cur, MultiClock *nxt, unsigned int *cnt,
                                unsigned int *cnt_next, cudaStream_t s) {
  constexpr size_t smem = (size_t)2 * (StagedVars<2>::kState + 2 + 6) * kT * sizeof(float);
  static std::atomic<uint64_t> done{0};
  cudaError_t e = smem_limit((const void *)multi_staged_kernel<kT>, (int)smem, done);
  if (e != cudaSuccess) return e;
  multi_staged_kernel<kT><<<L.grid, kT, smem, s>>>(L.insts, L.tiles, L.n_tiles, cur, nxt, cnt, cnt_next);
  return cudaGetLastError();
}

template <int kT, int kStages>
cudaError_t launch_multi_pipe(const MultiLaunch &L, const MultiClock *cur, MultiClock *nxt, unsigned int *cnt,
                              unsigned int *cnt_next, cudaStream_t s) {
  constexpr size_t smem = (size_t)kStages * (StagedVars<2>::kState + 2 + 6) * kT * sizeof(float);
  static std::atomic<uint64_t> done{0};
  cudaError_t e = smem_limit((const void *)multi_pipe_kernel<kT, kStages>, (int)smem, done);
  if (e != cudaSuccess) return e;
  multi_pipe_kernel<kT, kStages><<<L.grid, kT + 32, smem, s>>>(L.insts, L.tiles, L.n_tiles, cur, nxt, cnt, cnt_next);
  return cudaGetLastError();
}

}  // namespace

int n_multi_shapes() { return (int)(sizeof(kMShapes) / sizeof(kMShapes[0])); }
int multi_block(int shape) { return kMShapes[(shape >= 0 && shape < n_multi_shapes()) ? shape : 0].block; }

cudaError_t launch_multi(const MultiLaunch &L, int parity, cudaStream_t s) {
  const MultiClock *cur = L.clk + (parity & 1) * L.n_inst;
  MultiClock *nxt = L.clk + ((parity & 1) ^ 1) * L.n_inst;
  unsigned int *cnt = L.counters + (parity & 1);
  unsigned int *cnt_next = L.counters + ((parity & 1) ^ 1);
  const int grid = L.grid;
  int shape = L.shape;
  if (shape >= 0 && shape < n_multi_shapes() && kMShapes[shape].staged) {
    if (L.tile_cells % kMShapes[shape].block == 0) {
      if (kMShapes[shape].pipe) {
        const bool b128 = kMShapes[shape].block == 128;
        switch (kMShapes[shape].stages) {
          case 2: return launch_multi_pipe<256, 2>(L, cur, nxt, cnt, cnt_next, s);
          case 3: return b128 ? launch_multi_pipe<128, 3>(L, cur, nxt, cnt, cnt_next, s)
                              : launch_multi_pipe<256, 3>(L, cur, nxt, cnt, cnt_next, s);
          default: return launch_multi_pipe<128, 4>(L, cur, nxt, cnt, cnt_next, s);
        }
      }
      return kMShapes[shape].block == 128 ? launch_multi_staged<128>(L, cur, nxt, cnt, cnt_next, s)
                                          : launch_multi_staged<256>(L, cur, nxt, cnt, cnt_next, s);
    }
    shape = 0;  // tiles not in whole sub-tiles: the unstaged kernel
  }
  switch (shape) {
    case 1: multi_kernel<128, 5><<<grid, 128, 0, s>>>(L.insts, L.tiles, L.n_tiles, cur, nxt, cnt, cnt_next); break;
    case 2: multi_kernel<512, 1><<<grid, 512, 0, s>>>(L.insts, L.tiles, L.n_tiles, cur, nxt, cnt, cnt_next); break;
    default: multi_kernel<256, 2><<<grid, 256, 0, s>>>(L.insts, L.tiles, L.n_tiles, cur, nxt, cnt, cnt_next); break;
  }
  return cudaGetLastError();
}

}  // namespace cm
