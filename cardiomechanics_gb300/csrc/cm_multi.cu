// Batched form: many batches (instances) of uneven size and mixed model, advanced by one
// persistent launch per time step. The cells of all instances are cut into tiles of
// `tile_cells`; blocks take tiles from an atomic counter until none are left, so large and
// small instances, and the costlier Courtemanche tiles, balance across the 152 SMs by
// themselves. Each instance carries its own stimulus clock on the device (double-buffered by
// step parity), so consecutive steps are identical launches that a CUDA graph can replay.
#include <cuda_runtime.h>

#include "cm_cells.cuh"
#include "cm_multi.h"

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

struct MShape {
  int block, minb;
};
constexpr MShape kMShapes[] = {{256, 2}, {128, 5}, {512, 1}};

}  // namespace

int n_multi_shapes() { return (int)(sizeof(kMShapes) / sizeof(kMShapes[0])); }
int multi_block(int shape) { return kMShapes[(shape >= 0 && shape < n_multi_shapes()) ? shape : 0].block; }

cudaError_t launch_multi(const MultiLaunch &L, int parity, cudaStream_t s) {
  const MultiClock *cur = L.clk + (parity & 1) * L.n_inst;
  MultiClock *nxt = L.clk + ((parity & 1) ^ 1) * L.n_inst;
  unsigned int *cnt = L.counters + (parity & 1);
  unsigned int *cnt_next = L.counters + ((parity & 1) ^ 1);
  const int grid = L.grid;
  switch (L.shape) {
    case 1: multi_kernel<128, 5><<<grid, 128, 0, s>>>(L.insts, L.tiles, L.n_tiles, cur, nxt, cnt, cnt_next); break;
    case 2: multi_kernel<512, 1><<<grid, 512, 0, s>>>(L.insts, L.tiles, L.n_tiles, cur, nxt, cnt, cnt_next); break;
    default: multi_kernel<256, 2><<<grid, 256, 0, s>>>(L.insts, L.tiles, L.n_tiles, cur, nxt, cnt, cnt_next); break;
  }
  return cudaGetLastError();
}

}  // namespace cm
