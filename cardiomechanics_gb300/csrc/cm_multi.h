// Device layout of the batched (multi-instance) form; see cm_multi.cu.
#pragma once

#include <cuda_runtime.h>

#include "cm_launch.h"

namespace cm {

struct alignas(16) MultiInst {
  DevBatch d;      // the instance's batch (state, tables, per-cell conductances, audit)
  float *vm_hi, *vm_lo;  // its cells' Vm as compensated FP32 planes
  double textlen, bcl, amp, dt;
};

struct MultiTile {
  int inst, start, count, pad;
};

struct MultiClock {
  double t, tb;  // time and current first-stimulus time (reference driver's t, textbegin)
};

struct MultiLaunch {
  const MultiInst *insts = nullptr;
  const MultiTile *tiles = nullptr;
  int n_tiles = 0, n_inst = 0;
  MultiClock *clk = nullptr;          // 2 x n_inst, by step parity
  unsigned int *counters = nullptr;   // 2, by step parity
  int shape = 0, grid = 0;
  int tile_cells = 0;                 // every tile starts at a multiple of it within its instance
};

int n_multi_shapes();
int multi_block(int shape);
cudaError_t launch_multi(const MultiLaunch &L, int parity, cudaStream_t s);

}  // namespace cm
