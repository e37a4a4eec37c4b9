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
    staged_cell<kModel, kThreads>(b, S, het_pos, c, (float)io.iext_uniform, io.vm_hi, io.vm_lo);
  }
}

template <int kModel, int kThreads>
cudaError_t launch_staged_t(const DevBatch &b, const StepIO &io, int blocks_per_sm, cudaStream_t s) {
  constexpr int NVMAX = StagedVars<kModel>::kState + 2 + 6;
  const size_t smem = (size_t)2 * NVMAX * kThreads * sizeof(float);
  static std::atomic<uint64_t> done{0};  // one attribute call per instantiation and device
  cudaError_t e = smem_limit((const void *)mixed_staged_kernel<kModel, kThreads>, (int)smem, done);
  if (e != cudaSuccess) return e;
  const int n_tiles = (int)((b.n + kThreads - 1) / kThreads);
  int grid = sm_count() * (blocks_per_sm > 0 ? blocks_per_sm : 2);
  if (grid > n_tiles) grid = n_tiles;
  if (grid < 1) grid = 1;
  mixed_staged_kernel<kModel, kThreads><<<grid, kThreads, smem, s>>>(b, io);
  return cudaGetLastError();
}

}  // namespace

bool staged_supported(const DevBatch &b, const StepIO &io) {
  return (b.model == 5 || b.model == 2) && b.precision == 1 && io.vm_hi && io.vm_lo && !io.tb_cell && !io.iext &&
         !io.sl_ptr && !io.vm_hi_out && !io.act && io.vm_range <= 0.0 &&
         b.ld % 256 == 0 &&
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
