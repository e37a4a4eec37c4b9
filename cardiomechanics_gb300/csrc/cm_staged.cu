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
#include "cm_launch.h"
#include "cm_staged_cell.cuh"

namespace cm {

namespace {

// Staged variables of a tile: state planes, Vm hi, Vm lo, then the present hetero slots.
template <int kModel, int kThreads>
__global__ void __launch_bounds__(kThreads, 2) mixed_staged_kernel(const DevBatch b, const StepIO io) {
  constexpr int NS = StagedVars<kModel>::kState;
  extern __shared__ __align__(128) float stage[];  // [2][nv][kThreads]
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
  const size_t buf_floats = (size_t)nv * kThreads;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int tile, int buf) {
    float *dst = stage + buf * buf_floats;
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
    const float *S = stage + buf * buf_floats + threadIdx.x;
    const int c = t * kThreads + threadIdx.x;
    if (c >= n) continue;
    staged_cell<kModel, kThreads>(b, S, het_pos, c, (float)io.iext_uniform, io.vm_hi, io.vm_lo);
  }
}

template <int kModel, int kThreads>
cudaError_t launch_staged_t(const DevBatch &b, const StepIO &io, int blocks_per_sm, cudaStream_t s) {
  // the stage holds the state planes, the Vm pair and the present hetero planes, twice; the
  // attribute allows all six hetero planes, a launch takes what its batch stages
  constexpr int NVMAX = StagedVars<kModel>::kState + 2 + 6;
  int nv = StagedVars<kModel>::kState + 2;
  for (int k = 0; k < 6; k++) nv += b.het[k] ? 1 : 0;
  const size_t smem = (size_t)2 * nv * kThreads * sizeof(float);
  static std::atomic<uint64_t> done{0};  // one attribute call per instantiation and device
  cudaError_t e = smem_limit((const void *)mixed_staged_kernel<kModel, kThreads>,
                             (int)((size_t)2 * NVMAX * kThreads * sizeof(float)), done);
  if (e != cudaSuccess) return e;
  const int n_tiles = (int)((b.n + kThreads - 1) / kThreads);
  int grid = sm_count() * (blocks_per_sm > 0 ? blocks_per_sm : 2);
  if (grid > n_tiles) grid = n_tiles;
  if (grid < 1) grid = 1;
  mixed_staged_kernel<kModel, kThreads><<<grid, kThreads, smem, s>>>(b, io);
  return cudaGetLastError();
}

// The staged kernel as a producer/consumer pipeline: one extra warp only issues the tiles' bulk
// copies into kStages stage buffers; the kThreads / 32 consumer warps integrate. A stage is
// handed over by two mbarriers: `full` (the producer's expect_tx plus the copies' bytes) and
// `empty` (one arrival per consumer warp when it is done with the stage). No block-wide barrier
// inside the loop: a warp that finishes its part of a tile moves on to the next staged tile
// while slower warps still work on this one.
//
// Every wait is bounded. A consumer whose `full` wait runs out sets CM_AUDIT_TIMEOUT and leaves;
// the producer then runs out on `empty`, sets the same bit, waits (bounded) for the copies it
// issued that no consumer took, and leaves.
template <int kModel, int kThreads, int kStages>
__global__ void __launch_bounds__(kThreads + 32, 2) mixed_pipe_kernel(const DevBatch b, const StepIO io) {
  constexpr int NS = StagedVars<kModel>::kState;
  constexpr int kWarps = kThreads / 32;
  extern __shared__ __align__(128) float stage[];  // [kStages][nv][kThreads]
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages];
  const int64_t ld = b.ld;
  const int n = (int)b.n;
  const int n_tiles = (n + kThreads - 1) / kThreads;
  int het_pos[6];
  int nv = NS + 2;
#pragma unroll
  for (int k = 0; k < 6; k++) het_pos[k] = b.het[k] ? nv++ : -1;
  const uint32_t tile_bytes = (uint32_t)nv * kThreads * 4u;
  const size_t buf_floats = (size_t)nv * kThreads;
  if (threadIdx.x == 0) {
    for (int k = 0; k < kStages; k++) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], kWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x >= kThreads) {  // the producer warp: lane 0 issues, the other lanes leave
    if (threadIdx.x != kThreads) return;
    int it = 0;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, it++) {
      const int st = it % kStages;
      if (it >= kStages && !mbar_wait(&empty[st], (uint32_t)((it / kStages - 1) & 1), b.spin_limit)) {
        atomicOr(b.audit_or, kAuditTimeout);
        // the copies of the last kStages tiles may still be landing: wait for them, bounded
        for (int j = it - kStages; j < it; j++)
          if (j >= 0) mbar_wait(&full[j % kStages], (uint32_t)((j / kStages) & 1), b.spin_limit);
        return;
      }
      if (t == b.fault_skip_tile) continue;  // test hook: this stage's copy is never issued
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      float *dst = stage + st * buf_floats;
      const int64_t c0 = (int64_t)t * kThreads;
      mbar_expect_tx(&full[st], tile_bytes);
      for (int v = 0; v < NS; v++) bulk_g2s(dst + v * kThreads, b.s32 + v * ld + c0, kThreads * 4u, &full[st]);
      bulk_g2s(dst + NS * kThreads, io.vm_hi + c0, kThreads * 4u, &full[st]);
      bulk_g2s(dst + (NS + 1) * kThreads, io.vm_lo + c0, kThreads * 4u, &full[st]);
      for (int k = 0; k < 6; k++)
        if (het_pos[k] >= 0)
          bulk_g2s(dst + het_pos[k] * kThreads, (const float *)b.het[k] + c0, kThreads * 4u, &full[st]);
    }
    return;
  }
  const int lane = threadIdx.x & 31;
  int it = 0;
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, it++) {
    const int st = it % kStages;
    if (!mbar_wait(&full[st], (uint32_t)((it / kStages) & 1), b.spin_limit)) {
      atomicOr(b.audit_or, kAuditTimeout);
      return;
    }
    const int c = t * kThreads + threadIdx.x;
    if (c < n)
      staged_cell<kModel, kThreads>(b, stage + st * buf_floats + threadIdx.x, het_pos, c, (float)io.iext_uniform,
                                    io.vm_hi, io.vm_lo);
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[st]);
  }
}

template <int kModel, int kThreads, int kStages>
cudaError_t launch_pipe_t(const DevBatch &b, const StepIO &io, int blocks_per_sm, cudaStream_t s) {
  constexpr int NVMAX = StagedVars<kModel>::kState + 2 + 6;
  int nv = StagedVars<kModel>::kState + 2;
  for (int k = 0; k < 6; k++) nv += b.het[k] ? 1 : 0;
  const size_t smem = (size_t)kStages * nv * kThreads * sizeof(float);
  static std::atomic<uint64_t> done{0};
  cudaError_t e = smem_limit((const void *)mixed_pipe_kernel<kModel, kThreads, kStages>,
                             (int)((size_t)kStages * NVMAX * kThreads * sizeof(float)), done);
  if (e != cudaSuccess) return e;
  const int n_tiles = (int)((b.n + kThreads - 1) / kThreads);
  int grid = sm_count() * (blocks_per_sm > 0 ? blocks_per_sm : 2);
  if (grid > n_tiles) grid = n_tiles;
  if (grid < 1) grid = 1;
  mixed_pipe_kernel<kModel, kThreads, kStages><<<grid, kThreads + 32, smem, s>>>(b, io);
  return cudaGetLastError();
}

template <int kThreads, int kStages>
cudaError_t launch_pipe_m(const DevBatch &b, const StepIO &io, int blocks_per_sm, cudaStream_t s) {
  switch (b.model) {
    case 5: return launch_pipe_t<5, kThreads, kStages>(b, io, blocks_per_sm, s);
    case 2: return launch_pipe_t<2, kThreads, kStages>(b, io, blocks_per_sm, s);
    case 12: return launch_pipe_t<12, kThreads, kStages>(b, io, blocks_per_sm, s);
    default: return launch_pipe_t<14, kThreads, kStages>(b, io, blocks_per_sm, s);
  }
}

// Coupled runs (cm_batch_run_diffuse): the staged kernel plus the tile's monodomain operator.
// A tile of kThreads cells is kThreads / 32 consecutive slices, whose entries are one contiguous
// run of the operator's column and value arrays (each slice 32 * width entries, so the run starts
// and ends on 128-byte boundaries); both runs are bulk-copied with the state, next to the row
// sums and the per-node scales (padded to whole tiles by cm_diffusion_create). Only the
// neighbours' potentials are read from global memory (the previous step's hi plane); the new Vm
// pair goes to the other pair of planes.
constexpr int kCoupledWmax = 16;  // widest operator slice staged (entries per row)

// The update of one cell of a staged coupled tile: the stimulus by the driver's rule
// (CellModel.h:405-419) with per-cell times, the cell update with i_external = stimulus +
// coupling current `cpl`, the range check and the activation time. tb, a0: the cell's stimulus
// time and activation entry, read before the stage wait.
template <int kModel, int kThreads>
__device__ __forceinline__ void coupled_update(const DevBatch &b, const StepIO &io, const float *S,
                                               const int (&het_pos)[6], int c, double tb, double a0, float cpl) {
  float stim = (float)io.iext_uniform;
  if (io.tb_cell) {
    stim = 0.f;
    if (f64_ge(io.t, tb)) {  // integer compare: no FP64-pipe instruction per cell
      stim = (float)io.amp;
      if (io.t >= tb + io.textlen) io.tb_cell[c] = tb + io.bcl;
    }
  }
  const Acc v = staged_cell<kModel, kThreads>(b, S, het_pos, c, stim + cpl, io.vm_hi_out, io.vm_lo_out);
  uint32_t audit = 0;
  if (io.vm_range > 0.0 && fabsf(v.hi) > (float)io.vm_range) audit |= 32u;
  // a0 == -1.0 (not yet activated), compared on the bit pattern
  if (io.act && __double_as_longlong(a0) == (long long)0xbff0000000000000ull && v.hi >= (float)io.act_threshold)
    io.act[c] = io.act_time;
  if (audit) {
    atomicOr(b.audit_cell + c, audit);
    atomicOr(b.audit_or, audit);
  }
}

// One cell of a staged coupled tile whose operator entries are staged too (base + NVMAX *
// kThreads: columns, then values; off: the tile's slice entry offsets): the coupling current
// rowsum x_c + sum_j A_cj (x_j - x_c) from the stage and the neighbours' previous hi words, then
// coupled_update.
template <int kModel, int kThreads>
__device__ __forceinline__ void coupled_cell(const DevBatch &b, const StepIO &io, const float *base, const int *off,
                                             const int (&het_pos)[6], int rs_pos, int sc_pos, int c, double tb,
                                             double a0) {
  constexpr int NS = StagedVars<kModel>::kState;
  constexpr int NVMAX = NS + 2 + 6 + 2;
  const int W = io.sl_wmax;
  const int tid = threadIdx.x;
  const float *S = base + tid;
  const int32_t *ecol = (const int32_t *)(base + (size_t)NVMAX * kThreads);
  const float *eval = base + (size_t)NVMAX * kThreads + (size_t)W * kThreads;
  const int sl = tid >> 5, lane = tid & 31;
  const int o0 = off[sl] + lane, o1 = off[sl + 1];
  const float xc = S[NS * kThreads];
  int32_t cj[kCoupledWmax];
  float aj[kCoupledWmax], xj[kCoupledWmax];
#pragma unroll
  for (int k = 0; k < kCoupledWmax; k++) {
    const int e = o0 + 32 * k;
    cj[k] = e < o1 ? ecol[e] : c;
    aj[k] = e < o1 ? eval[e] : 0.f;
  }
#pragma unroll
  for (int k = 0; k < kCoupledWmax; k++) xj[k] = io.vm_hi[cj[k]];
  float acc = S[rs_pos * kThreads] * xc;
#pragma unroll
  for (int k = 0; k < kCoupledWmax; k++) acc += aj[k] * (xj[k] - xc);
  const float scale = sc_pos >= 0 ? S[sc_pos * kThreads] : (float)io.dscale_u;
  coupled_update<kModel, kThreads>(b, io, S, het_pos, c, tb, a0, acc * scale);
}

template <int kModel, int kThreads>
__global__ void __launch_bounds__(kThreads, 2) coupled_staged_kernel(const DevBatch b, const StepIO io) {
  constexpr int NS = StagedVars<kModel>::kState;
  constexpr int NVMAX = NS + 2 + 6 + 2;
  constexpr int kSlices = kThreads / 32;
  extern __shared__ __align__(128) float stage[];  // [2][NVMAX * kThreads + 2 * W * kThreads]
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ int s_abort;
  __shared__ int s_off[2][kSlices + 1];  // slice entry offsets from the tile's first entry
  const int64_t ld = b.ld;
  const int n = (int)b.n;
  const int n_tiles = (n + kThreads - 1) / kThreads;
  const int64_t n_slices = ((int64_t)n + 31) / 32;
  const int W = io.sl_wmax;
  const size_t buf_floats = (size_t)NVMAX * kThreads + 2 * (size_t)W * kThreads;
  int het_pos[6];
  int nv = NS + 2;
#pragma unroll
  for (int k = 0; k < 6; k++) het_pos[k] = b.het[k] ? nv++ : -1;
  const int rs_pos = nv++;
  const int sc_pos = io.dscale32 ? nv++ : -1;
  const uint32_t plane_bytes = (uint32_t)nv * kThreads * 4u;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int tile, int buf) {
    float *dst = stage + (size_t)buf * buf_floats;
    const int64_t c0 = (int64_t)tile * kThreads;
    const int64_t s0 = c0 / 32, s1 = s0 + kSlices < n_slices ? s0 + kSlices : n_slices;
    const int64_t e0 = io.sl_ptr[s0], e1 = io.sl_ptr[s1];
    for (int k = 0; k <= kSlices; k++) s_off[buf][k] = (int)(io.sl_ptr[s0 + k < s1 ? s0 + k : s1] - e0);
    const uint32_t ent_bytes = (uint32_t)(e1 - e0) * 4u;
    mbar_expect_tx(&bar[buf], plane_bytes + 2u * ent_bytes);
    for (int v = 0; v < NS; v++) bulk_g2s(dst + v * kThreads, b.s32 + v * ld + c0, kThreads * 4u, &bar[buf]);
    bulk_g2s(dst + NS * kThreads, io.vm_hi + c0, kThreads * 4u, &bar[buf]);
    bulk_g2s(dst + (NS + 1) * kThreads, io.vm_lo + c0, kThreads * 4u, &bar[buf]);
    for (int k = 0; k < 6; k++)
      if (het_pos[k] >= 0)
        bulk_g2s(dst + het_pos[k] * kThreads, (const float *)b.het[k] + c0, kThreads * 4u, &bar[buf]);
    bulk_g2s(dst + rs_pos * kThreads, io.rowsum32 + c0, kThreads * 4u, &bar[buf]);
    if (sc_pos >= 0) bulk_g2s(dst + sc_pos * kThreads, io.dscale32 + c0, kThreads * 4u, &bar[buf]);
    if (ent_bytes) {
      float *ent = dst + (size_t)NVMAX * kThreads;
      bulk_g2s(ent, io.sl_col + e0, ent_bytes, &bar[buf]);
      bulk_g2s(ent + (size_t)W * kThreads, io.sl_val32 + e0, ent_bytes, &bar[buf]);
    }
  };
  int it = 0;
  int t = blockIdx.x;
  if (t < n_tiles && threadIdx.x == 0) issue(t, 0);
  for (; t < n_tiles; t += gridDim.x, it++) {
    const int buf = it & 1;
    const int next = t + gridDim.x;
    // the cell's stimulus time and activation entry do not depend on the stage: read them now,
    // while the tile's copies may still be landing
    const int c = t * kThreads + threadIdx.x;
    const double tb = (io.tb_cell && c < n) ? io.tb_cell[c] : 0.0;
    const double a0 = (io.act && c < n) ? io.act[c] : 0.0;
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
    if (c >= n) continue;
    coupled_cell<kModel, kThreads>(b, io, stage + (size_t)buf * buf_floats, s_off[buf], het_pos, rs_pos, sc_pos, c,
                                   tb, a0);
  }
}

// Coupled runs through the producer/consumer pipeline of mixed_pipe_kernel. kStagedOps: the
// tile's operator entries, row sums and scales are staged too (the producer reads the tile's
// slice offsets and writes them to the stage's offset row before the stage's `full` arrival,
// which releases them to the consumers). Otherwise a consumer forms its cell's coupling current
// from global memory (coupling_f32) before it waits for the stage, so the entry and neighbour
// reads overlap the stage's copies, and the stage holds the state, Vm and conductances only.
template <int kModel, int kThreads, int kStages, bool kStagedOps>
__global__ void __launch_bounds__(kThreads + 32, kThreads == 256 ? 2 : 3) coupled_pipe_kernel(const DevBatch b,
                                                                                           const StepIO io) {
  constexpr int NS = StagedVars<kModel>::kState;
  constexpr int NVMAX = NS + 2 + 6 + 2;
  constexpr int kSlices = kThreads / 32;
  constexpr int kWarps = kThreads / 32;
  extern __shared__ __align__(128) float stage[];  // [kStages][buf_floats]
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages];
  __shared__ int s_off[kStages][kSlices + 1];
  const int64_t ld = b.ld;
  const int n = (int)b.n;
  const int n_tiles = (n + kThreads - 1) / kThreads;
  const int64_t n_slices = ((int64_t)n + 31) / 32;
  const int W = io.sl_wmax;
  int het_pos[6];
  int nv = NS + 2;
#pragma unroll
  for (int k = 0; k < 6; k++) het_pos[k] = b.het[k] ? nv++ : -1;
  const int rs_pos = kStagedOps ? nv++ : -1;
  const int sc_pos = (kStagedOps && io.dscale32) ? nv++ : -1;
  const uint32_t plane_bytes = (uint32_t)nv * kThreads * 4u;
  const size_t buf_floats =
      kStagedOps ? (size_t)NVMAX * kThreads + 2 * (size_t)W * kThreads : (size_t)nv * kThreads;
  if (threadIdx.x == 0) {
    for (int k = 0; k < kStages; k++) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], kWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x >= kThreads) {  // the producer warp: lane 0 issues, the other lanes leave
    if (threadIdx.x != kThreads) return;
    int it = 0;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, it++) {
      const int st = it % kStages;
      const int64_t c0 = (int64_t)t * kThreads;
      int64_t so[kSlices + 1];  // read before the wait: the offsets do not depend on the stage
      {
        const int64_t s0 = c0 / 32, s1 = s0 + kSlices < n_slices ? s0 + kSlices : n_slices;
#pragma unroll
        for (int k = 0; k <= kSlices; k++) so[k] = io.sl_ptr[s0 + k < s1 ? s0 + k : s1];
      }
      if (!kStagedOps) {
        // the consumers read the tile's operator entries, row sums and scales themselves: bring
        // them into L2 ahead of them (each run starts on a 128-byte boundary, whole slices)
        const uint32_t eb = (uint32_t)(so[kSlices] - so[0]) * 4u;
        if (eb) {
          bulk_prefetch_l2(io.sl_col + so[0], eb);
          bulk_prefetch_l2(io.sl_val32 + so[0], eb);
        }
        bulk_prefetch_l2(io.rowsum32 + c0, kThreads * 4u);
        if (io.dscale32) bulk_prefetch_l2(io.dscale32 + c0, kThreads * 4u);
      }
      if (it >= kStages && !mbar_wait(&empty[st], (uint32_t)((it / kStages - 1) & 1))) {
        atomicOr(b.audit_or, kAuditTimeout);
        for (int j = it - kStages; j < it; j++)
          if (j >= 0) mbar_wait(&full[j % kStages], (uint32_t)((j / kStages) & 1));
        return;
      }
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      float *dst = stage + st * buf_floats;
      uint32_t ent_bytes = 0;
      if (kStagedOps) {
        for (int k = 0; k <= kSlices; k++) s_off[st][k] = (int)(so[k] - so[0]);
        ent_bytes = (uint32_t)(so[kSlices] - so[0]) * 4u;
      }
      mbar_expect_tx(&full[st], plane_bytes + 2u * ent_bytes);
      for (int v = 0; v < NS; v++) bulk_g2s(dst + v * kThreads, b.s32 + v * ld + c0, kThreads * 4u, &full[st]);
      bulk_g2s(dst + NS * kThreads, io.vm_hi + c0, kThreads * 4u, &full[st]);
      bulk_g2s(dst + (NS + 1) * kThreads, io.vm_lo + c0, kThreads * 4u, &full[st]);
      for (int k = 0; k < 6; k++)
        if (het_pos[k] >= 0)
          bulk_g2s(dst + het_pos[k] * kThreads, (const float *)b.het[k] + c0, kThreads * 4u, &full[st]);
      if (kStagedOps) {
        bulk_g2s(dst + rs_pos * kThreads, io.rowsum32 + c0, kThreads * 4u, &full[st]);
        if (sc_pos >= 0) bulk_g2s(dst + sc_pos * kThreads, io.dscale32 + c0, kThreads * 4u, &full[st]);
        if (ent_bytes) {
          float *ent = dst + (size_t)NVMAX * kThreads;
          bulk_g2s(ent, io.sl_col + so[0], ent_bytes, &full[st]);
          bulk_g2s(ent + (size_t)W * kThreads, io.sl_val32 + so[0], ent_bytes, &full[st]);
        }
      }
    }
    return;
  }
  const int lane = threadIdx.x & 31;
  int it = 0;
  for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, it++) {
    const int st = it % kStages;
    const int c = t * kThreads + threadIdx.x;
    const double tb = (io.tb_cell && c < n) ? io.tb_cell[c] : 0.0;
    const double a0 = (io.act && c < n) ? io.act[c] : 0.0;
    float cpl = 0.f;
    if (!kStagedOps && c < n) cpl = coupling_f32<int>(io, c);
    if (!mbar_wait(&full[st], (uint32_t)((it / kStages) & 1))) {
      atomicOr(b.audit_or, kAuditTimeout);
      return;
    }
    if (c < n) {
      if (kStagedOps)
        coupled_cell<kModel, kThreads>(b, io, stage + st * buf_floats, s_off[st], het_pos, rs_pos, sc_pos, c, tb,
                                       a0);
      else
        coupled_update<kModel, kThreads>(b, io, stage + st * buf_floats + threadIdx.x, het_pos, c, tb, a0, cpl);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[st]);
  }
}

template <int kModel, int kThreads, int kStages, bool kStagedOps>
cudaError_t launch_coupled_pipe_t(const DevBatch &b, const StepIO &io, cudaStream_t s) {
  constexpr int NS = StagedVars<kModel>::kState;
  constexpr int NVMAX = NS + 2 + 6 + 2;
  int nv = NS + 2;
  for (int k = 0; k < 6; k++) nv += b.het[k] ? 1 : 0;
  const size_t smem = kStagedOps ? (size_t)kStages * ((size_t)NVMAX * kThreads + 2 * (size_t)io.sl_wmax * kThreads) *
                                       sizeof(float)
                                 : (size_t)kStages * nv * kThreads * sizeof(float);
  const size_t smem_max =
      kStagedOps ? (size_t)kStages * ((size_t)NVMAX * kThreads + 2 * (size_t)kCoupledWmax * kThreads) * sizeof(float)
                 : (size_t)kStages * (NS + 2 + 6) * kThreads * sizeof(float);
  auto kern = coupled_pipe_kernel<kModel, kThreads, kStages, kStagedOps>;
  static std::atomic<uint64_t> done{0};
  cudaError_t e = smem_limit((const void *)kern, (int)smem_max, done);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads + 32, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const int n_tiles = (int)((b.n + kThreads - 1) / kThreads);
  int grid = sm_count() * per_sm;
  if (grid > n_tiles) grid = n_tiles;
  if (grid < 1) grid = 1;
  kern<<<grid, kThreads + 32, smem, s>>>(b, io);
  return cudaGetLastError();
}

template <int kModel>
cudaError_t launch_coupled_t(const DevBatch &b, const StepIO &io, cudaStream_t s) {
  constexpr int kThreads = 256;
  constexpr int NVMAX = StagedVars<kModel>::kState + 2 + 6 + 2;
  const size_t smem = (size_t)2 * ((size_t)NVMAX * kThreads + 2 * (size_t)io.sl_wmax * kThreads) * sizeof(float);
  const size_t smem_max = (size_t)2 * ((size_t)NVMAX * kThreads + 2 * (size_t)kCoupledWmax * kThreads) * sizeof(float);
  static std::atomic<uint64_t> done{0};
  cudaError_t e = smem_limit((const void *)coupled_staged_kernel<kModel, kThreads>, (int)smem_max, done);
  if (e != cudaSuccess) return e;
  const int n_tiles = (int)((b.n + kThreads - 1) / kThreads);
  int grid = sm_count() * 2;
  if (grid > n_tiles) grid = n_tiles;
  if (grid < 1) grid = 1;
  coupled_staged_kernel<kModel, kThreads><<<grid, kThreads, smem, s>>>(b, io);
  return cudaGetLastError();
}

}  // namespace

bool coupled_staged_supported(const DevBatch &b, const StepIO &io) {
  return (b.model == 5 || b.model == 2 || b.model == 12 || b.model == 14) && b.precision == 1 && io.sl_ptr && io.sl_val32 && io.rowsum32 &&
         io.sl_wmax >= 1 && io.sl_wmax <= kCoupledWmax && io.vm_hi && io.vm_hi_out && io.vm_lo == io.vm_hi + b.ld &&
         io.vm_lo_out == io.vm_hi_out + b.ld && !io.iext && b.ld % 256 == 0 && b.n < (int64_t)1 << 30;
}

cudaError_t launch_coupled_staged(const DevBatch &b, const StepIO &io, int variant, cudaStream_t s) {
  if (b.n == 0) return cudaSuccess;
  // variant (cm_batch_set_launch) past the register shapes: 0, 1 the double-buffered kernel
  // (TT2 / Courtemanche); 2 the pipeline with the operator staged; 3 the pipeline with the
  // coupling current from global memory. Otherwise the faster of the two pipelines on a
  // 4,194,304-node slab: operator staged for TT2 / Courtemanche (92 % of measured HBM against
  // 74 %), coupling from global memory with 256-cell tiles for O'Hara-Rudy and Tomek (their
  // stages with the operator fit two blocks per SM only with 128-cell tiles: 79 % against 78 %,
  // 77 % against 73 %).
  const int k = variant - n_register_shapes();
  const bool staged_ops = k == 2 || (k != 3 && (b.model == 5 || b.model == 2));
  switch (b.model) {
    case 12:
      return staged_ops ? launch_coupled_pipe_t<12, 128, 2, true>(b, io, s) : launch_coupled_pipe_t<12, 256, 2, false>(b, io, s);
    case 14:
      return staged_ops ? launch_coupled_pipe_t<14, 128, 2, true>(b, io, s) : launch_coupled_pipe_t<14, 256, 2, false>(b, io, s);
    case 5:
      if (k == 0 || k == 1) return launch_coupled_t<5>(b, io, s);
      return staged_ops ? launch_coupled_pipe_t<5, 256, 2, true>(b, io, s) : launch_coupled_pipe_t<5, 256, 2, false>(b, io, s);
    default:
      if (k == 0 || k == 1) return launch_coupled_t<2>(b, io, s);
      return staged_ops ? launch_coupled_pipe_t<2, 256, 2, true>(b, io, s) : launch_coupled_pipe_t<2, 256, 2, false>(b, io, s);
  }
}

bool staged_supported(const DevBatch &b, const StepIO &io) {
  return (b.model == 5 || b.model == 2 || b.model == 12 || b.model == 14) && b.precision == 1 && io.vm_hi && io.vm_lo && !io.tb_cell && !io.iext &&
         !io.sl_ptr && !io.vm_hi_out && !io.act && io.vm_range <= 0.0 &&
         b.ld % 256 == 0 &&
         io.vm_lo == io.vm_hi + b.ld && b.n < (int64_t)1 << 30;
}

cudaError_t launch_pipe(const DevBatch &b, const StepIO &io, int threads, int blocks_per_sm, cudaStream_t s) {
  if (b.n == 0) return cudaSuccess;
  return threads == 128 ? launch_pipe_m<128, 3>(b, io, blocks_per_sm, s) : launch_pipe_m<256, 2>(b, io, blocks_per_sm, s);
}

cudaError_t launch_staged(const DevBatch &b, const StepIO &io, int threads, int blocks_per_sm, cudaStream_t s) {
  if (b.n == 0) return cudaSuccess;
  if (b.model == 5) {
    if (threads == 128) return launch_staged_t<5, 128>(b, io, blocks_per_sm, s);
    return launch_staged_t<5, 256>(b, io, blocks_per_sm, s);
  }
  if (b.model == 12) {
    if (threads == 128) return launch_staged_t<12, 128>(b, io, blocks_per_sm, s);
    return launch_staged_t<12, 256>(b, io, blocks_per_sm, s);
  }
  if (b.model == 14) {
    if (threads == 128) return launch_staged_t<14, 128>(b, io, blocks_per_sm, s);
    return launch_staged_t<14, 256>(b, io, blocks_per_sm, s);
  }
  if (threads == 128) return launch_staged_t<2, 128>(b, io, blocks_per_sm, s);
  return launch_staged_t<2, 256>(b, io, blocks_per_sm, s);
}

}  // namespace cm
