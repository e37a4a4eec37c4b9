// The surrogate's MLP (n_in -> H -> H -> n_out, tanh): BF16 operands with FP32 accumulation on
// the tcgen05 tensor cores (accumulators in tensor memory), FP32 master weights and Adam. Training runs as a
// sequence of small GEMMs with fused epilogues:
//   forward   Z1 = X W1^T + b1, H1 = tanh Z1;  Z2 = H1 W2^T + b2, H2 = tanh Z2;  Y = H2 W3^T + b3
//   loss      L = mean over samples and real outputs of (Y - T)^2, dY = dL/dY (padding masked)
//   backward  dZ2 = (dY W3) * (1 - H2^2);  dZ1 = (dZ2 W2) * (1 - H1^2)
//             dW3 = dY^T H2, dW2 = dZ2^T H1, dW1 = dZ1^T X, db = column sums
// Every GEMM is C[m][n] = sum_k A[m][k] B[n][k] over row-major BF16 operands ("NT"), so the
// backward products first transpose their operands with a small kernel. Dimensions are padded:
// n_in to 32, n_out to 32, the batch to a multiple of 64.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "cm_bulk.cuh"
#include "cm_mlp.h"
#include "cm_umma.cuh"

namespace cm {

namespace {

// tanh of two FP32 values as one packed BF16 pair (tanh.approx.bf16x2), low half = x
__device__ __forceinline__ uint32_t tanh2_bf16(float x, float y) {
  uint32_t p, r;
  asm("cvt.rn.bf16x2.f32 %0, %2, %1;" : "=r"(p) : "f"(x), "f"(y));
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(r) : "r"(p));
  return r;
}

enum Epi { EPI_BIAS_TANH = 0, EPI_BIAS_F32 = 1, EPI_DTANH = 2, EPI_F32 = 3 };

struct EpiArgs {
  const float *bias;           // EPI_BIAS_*: per column n
  __nv_bfloat16 *out_bf16;     // EPI_BIAS_TANH, EPI_DTANH
  float *out_f32;              // EPI_BIAS_F32, EPI_F32
  const __nv_bfloat16 *h;      // EPI_DTANH: tanh output of the layer, same shape as C
  int ldc;
};

// The products on the tcgen05 tensor core: C = A B^T over K-major BF16 rows in global
// memory. A block of 128 threads owns a 128-row tile of C and up to 128 of its columns; K is
// staged slice by slice (kTcKs at a time) into shared memory in the tensor core's K-major,
// no-swizzle layout (the learned macro step's; checked by cm_diag_umma_tile), one thread issues
// the slice's MMAs into a tensor-memory accumulator and commits them to an mbarrier, and after
// the last slice each thread reads its row back (tcgen05.ld: thread i = row i = TMEM lane i) into
// the epilogue. gridDim.z > 1 (EPI_F32): split K, one partial product per z slice of out_f32.
// kTrans (EPI_F32): the block computes C^T's tile and stores it transposed, for products whose
// own M is below 128 (dW3 = dY^T H2 as (H2^T dY)^T). Waits are bounded; a timeout sets *err.
constexpr int kTcKs = 64;

template <int EPI, bool kTrans>
__global__ void __launch_bounds__(128) gemm_tc(const __nv_bfloat16 *__restrict__ A, int lda,
                                               const __nv_bfloat16 *__restrict__ B, int ldb, int M, int N, int K,
                                               EpiArgs e, unsigned int *err) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  __nv_bfloat16 *sA = (__nv_bfloat16 *)smem;
  __nv_bfloat16 *sB = sA + 128 * kTcKs;
  const int warp = threadIdx.x >> 5;
  const int m0 = blockIdx.y * 128, n0 = blockIdx.x * 128;
  const int nt = min(128, N - n0);                                   // columns of this tile
  const uint32_t ncols = nt <= 32 ? 32u : (nt <= 64 ? 64u : 128u);   // MMA N = TMEM columns
  const int kc = K / (int)gridDim.z, kbeg = (int)blockIdx.z * kc, kend = kbeg + kc;
  const int ks = kc % kTcKs == 0 ? kTcKs : 32;                        // kc is a multiple of 32
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) umma::tmem_alloc(&tslot, ncols);
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tslot;
  uint32_t phase = 0;
  bool ok = true;
  const int chunks = ks / 8;  // 16-byte chunks of a staged row
  for (int k0 = kbeg; k0 < kend && ok; k0 += ks) {
    for (int i = threadIdx.x; i < 128 * chunks; i += 128) {
      const int r = i / chunks, c = i - r * chunks;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (m0 + r < M) v = *reinterpret_cast<const uint4 *>(A + (size_t)(m0 + r) * lda + k0 + 8 * c);
      *reinterpret_cast<uint4 *>(sA + umma::kmajor_index(r, 8 * c, ks)) = v;
    }
    for (int i = threadIdx.x; i < (int)ncols * chunks; i += 128) {
      const int r = i / chunks, c = i - r * chunks;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (r < nt) v = *reinterpret_cast<const uint4 *>(B + (size_t)(n0 + r) * ldb + k0 + 8 * c);
      *reinterpret_cast<uint4 *>(sB + umma::kmajor_index(r, 8 * c, ks)) = v;
    }
    umma::fence_smem_to_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    if (threadIdx.x == 0) {
      const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB), sbo = (uint32_t)(ks / 8) * 128u;
      const uint32_t idesc = umma::idesc_bf16_f32(128, (int)ncols);
      for (int st = 0; st < ks / 16; st++)
        umma::mma_bf16(tmem, umma::smem_desc(a0 + st * 256u, 128u, sbo), umma::smem_desc(b0 + st * 256u, 128u, sbo),
                       idesc, (k0 > kbeg || st > 0) ? 1u : 0u);
      umma::commit(&bar);
    }
    // the slice's MMAs are complete: their sums are in TMEM and the stage may be rewritten
    ok = __syncthreads_and(mbar_wait(&bar, phase) ? 1 : 0) != 0;
    phase ^= 1u;
    umma::fence_after_sync();
  }
  if (ok) {
    // thread = row m: each 32-column chunk of the row is one contiguous 64 or 128 B run, written
    // (and, for EPI_DTANH, read) with 16-byte accesses; N is a multiple of 32, so chunks are whole
    const int m = m0 + warp * 32 + (int)(threadIdx.x & 31);  // this thread's row = TMEM lane
    for (int c0 = 0; c0 < nt; c0 += 32) {
      float v[32];
      umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (m >= M) continue;
      const int n = n0 + c0;
      if (EPI == EPI_BIAS_TANH || EPI == EPI_DTANH) {
        uint32_t w[16];
        if (EPI == EPI_BIAS_TANH) {  // hidden biases in BF16, as the inference kernel feeds them
#pragma unroll
          for (int j = 0; j < 32; j += 2) {
            const float b0 = __bfloat162float(__float2bfloat16(e.bias[n + j]));
            const float b1 = __bfloat162float(__float2bfloat16(e.bias[n + j + 1]));
            w[j / 2] = tanh2_bf16(v[j] + b0, v[j + 1] + b1);
          }
        } else {
          uint4 hv[4];
          const uint4 *hp = reinterpret_cast<const uint4 *>(e.h + (size_t)m * e.ldc + n);
#pragma unroll
          for (int q = 0; q < 4; q++) hv[q] = hp[q];
          const __nv_bfloat16 *hb = reinterpret_cast<const __nv_bfloat16 *>(hv);
#pragma unroll
          for (int j = 0; j < 32; j += 2) {
            const float h0 = __bfloat162float(hb[j]), h1 = __bfloat162float(hb[j + 1]);
            const __nv_bfloat16 o0 = __float2bfloat16(v[j] * (1.f - h0 * h0));
            const __nv_bfloat16 o1 = __float2bfloat16(v[j + 1] * (1.f - h1 * h1));
            w[j / 2] = (uint32_t)__bfloat16_as_ushort(o0) | ((uint32_t)__bfloat16_as_ushort(o1) << 16);
          }
        }
        uint4 *op = reinterpret_cast<uint4 *>(e.out_bf16 + (size_t)m * e.ldc + n);
#pragma unroll
        for (int q = 0; q < 4; q++) op[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
      } else if (kTrans) {  // C^T's element (m, n + j) is C's (n + j, m); C has N rows: coalesced over m
#pragma unroll
        for (int j = 0; j < 32; j++)
          e.out_f32[(size_t)blockIdx.z * (size_t)N * e.ldc + (size_t)(n + j) * e.ldc + m] = v[j];
      } else {
        float *op = EPI == EPI_BIAS_F32 ? e.out_f32 + (size_t)m * e.ldc + n
                                        : e.out_f32 + (size_t)blockIdx.z * (size_t)M * e.ldc + (size_t)m * e.ldc + n;
#pragma unroll
        for (int q = 0; q < 8; q++) {
          float4 o = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
          if (EPI == EPI_BIAS_F32) {
            o.x += e.bias[n + 4 * q];
            o.y += e.bias[n + 4 * q + 1];
            o.z += e.bias[n + 4 * q + 2];
            o.w += e.bias[n + 4 * q + 3];
          }
          reinterpret_cast<float4 *>(op)[q] = o;
        }
      }
    }
  } else {
    if (threadIdx.x == 0) atomicOr(err, 1u);
    mbar_wait(&bar, phase ^ 1u);  // the slice that ran out: one more bounded wait before TMEM is freed
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_free(tmem, ncols);
}

// out[c][r] = in[r][c] for a rows x cols BF16 matrix.
__global__ void transpose_bf16(const __nv_bfloat16 *__restrict__ in, __nv_bfloat16 *__restrict__ out, int rows,
                               int cols) {
  __shared__ __nv_bfloat16 tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int r = by + j, c = bx + threadIdx.x;
    tile[j][threadIdx.x] = (r < rows && c < cols) ? in[(size_t)r * cols + c] : __float2bfloat16(0.f);
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int c = bx + j, r = by + threadIdx.x;
    if (c < cols && r < rows) out[(size_t)c * rows + r] = tile[threadIdx.x][j];
  }
}

// dY = 2 (Y - T) / (n * n_out) on the real outputs (padding columns and rows masked); each
// block's share of the loss goes to loss_part[block] (summed in block order by mse_total, so the
// reported loss is the same on every run).
constexpr int kMseBlocks = 256;
// Weight-gradient GEMMs split K (the minibatch rows) into up to kMaxSplits parts of 256 rows;
// column sums use up to kColsumParts row blocks. Partial sums live in Mlp::part.
constexpr int kMaxSplits = 32, kColsumParts = 64;
constexpr size_t kPartFloats = (size_t)kMaxSplits * 128 * 128;
__global__ void mse_grad(const float *__restrict__ Y, const float *__restrict__ T, int n, int n_real_rows, int n_out,
                         int ldy, __nv_bfloat16 *__restrict__ dY, float *loss_part) {
  __shared__ float red[256];
  float s = 0.f;
  const float scale = 2.f / ((float)n_real_rows * (float)n_out);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n * ldy; i += gridDim.x * blockDim.x) {
    const int r = i / ldy, c = i - r * ldy;
    float d = 0.f;
    if (r < n_real_rows && c < n_out) {
      d = Y[i] - T[(size_t)r * n_out + c];
      s += d * d;
    }
    dY[i] = __float2bfloat16(d * scale);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_part[blockIdx.x] = red[0] / ((float)n_real_rows * (float)n_out);
}

__global__ void mse_total(float *__restrict__ loss_part, int n_part, float *__restrict__ loss) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float s = 0.f;
  for (int i = 0; i < n_part; i++) s += loss_part[i];
  *loss = s;
}

// db[c] = sum_r dZ[r][c] in two passes with a fixed order: block b sums rows [b R, (b + 1) R)
// of every column into part[b][c], then one block sums the parts in block order.
__global__ void colsum_part(const __nv_bfloat16 *__restrict__ dZ, int rows, int cols, int rows_per_block,
                            float *__restrict__ part) {
  const int r0 = blockIdx.x * rows_per_block, r1 = min(rows, r0 + rows_per_block);
  for (int c = threadIdx.x; c < cols; c += blockDim.x) {
    float s = 0.f;
    for (int r = r0; r < r1; r++) s += __bfloat162float(dZ[(size_t)r * cols + c]);
    part[(size_t)blockIdx.x * cols + c] = s;
  }
}

__global__ void sum_parts(const float *__restrict__ part, int n_parts, int n, float *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int z = 0; z < n_parts; z++) s += part[(size_t)z * n + i];
    out[i] = s;
  }
}

// Adam on FP32 master weights (Kingma & Ba 2015), then the BF16 operand copy.
__global__ void adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                     __nv_bfloat16 *__restrict__ wb, int n, float lr, float b1, float b2, float eps, float c1,
                     float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  if (wb) wb[i] = __float2bfloat16(wi);
}

__global__ void to_bf16(const float *__restrict__ in, __nv_bfloat16 *__restrict__ out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = __float2bfloat16(in[i]);
}

// X rows (n_in real features, fp32) -> padded BF16 rows (ld = in_pad); rows beyond n zero.
__global__ void pack_inputs(const float *__restrict__ X, int n, int n_in, int rows_pad, int in_pad,
                            __nv_bfloat16 *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows_pad * in_pad; i += gridDim.x * blockDim.x) {
    const int r = i / in_pad, c = i - r * in_pad;
    out[i] = __float2bfloat16((r < n && c < n_in) ? X[(size_t)r * n_in + c] : 0.f);
  }
}

// Gather a minibatch: rows idx[k] of X (n_in) and T (n_out).
__global__ void gather_rows(const float *__restrict__ X, const float *__restrict__ T, const int64_t *__restrict__ idx,
                            int nb, int n_in, int n_out, float *__restrict__ Xb, float *__restrict__ Tb) {
  const int r = blockIdx.x;
  if (r >= nb) return;
  const int64_t s = idx[r];
  for (int c = threadIdx.x; c < n_in; c += blockDim.x) Xb[(size_t)r * n_in + c] = X[s * n_in + c];
  for (int c = threadIdx.x; c < n_out; c += blockDim.x) Tb[(size_t)r * n_out + c] = T[s * n_out + c];
}

// C = A B^T on the tcgen05 tensor core (gemm_tc); rows of A and B 16-byte aligned, N a multiple
// of 32, K a multiple of 32 * splits.
template <int EPI, bool kTrans = false>
cudaError_t gemm_tcgen05(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K,
                         EpiArgs e, int splits, unsigned int *err, cudaStream_t s) {
  if (splits < 1 || K % (32 * splits) || lda % 8 || ldb % 8 || N % 32) return cudaErrorInvalidValue;
  // the epilogue's 16-byte row accesses
  if ((uintptr_t)e.out_bf16 % 16 || (uintptr_t)e.out_f32 % 16 || (uintptr_t)e.h % 16 || e.ldc % 8)
    return cudaErrorInvalidValue;
  dim3 grid((N + 127) / 128, (M + 127) / 128, splits);
  gemm_tc<EPI, kTrans><<<grid, 128, 2 * 128 * kTcKs * sizeof(__nv_bfloat16), s>>>(A, lda, B, ldb, M, N, K, e, err);
  return cudaGetLastError();
}

// C (M x ldc, FP32) = A B^T with K split over `splits` blocks per tile (weight gradients: K = the
// minibatch rows, M and N at most 128), partial products in `part`, summed in split order. A
// product with fewer than 128 rows but more columns is computed as its transpose (a full
// 128-row tensor-core tile) and stored transposed.
cudaError_t gemm_f32_split(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb, int M, int N, int K,
                           float *C, int ldc, float *part, int splits, unsigned int *tc_err, cudaStream_t s) {
  splits = std::min(splits, (int)(kPartFloats / ((size_t)M * ldc)));
  if (splits < 1 || K % (32 * splits)) splits = 1;
  EpiArgs e{};
  e.out_f32 = splits > 1 ? part : C;
  e.ldc = ldc;
  cudaError_t err = M < 128 && N > M
                        ? gemm_tcgen05<EPI_F32, true>(B, ldb, A, lda, N, M, K, e, splits, tc_err, s)
                        : gemm_tcgen05<EPI_F32, false>(A, lda, B, ldb, M, N, K, e, splits, tc_err, s);
  if (err != cudaSuccess || splits == 1) return err;
  const int n = M * ldc;
  sum_parts<<<(n + 255) / 256, 256, 0, s>>>(part, splits, n, C);
  return cudaGetLastError();
}

cudaError_t colsum(const __nv_bfloat16 *dZ, int rows, int cols, float *db, float *part, cudaStream_t s) {
  const int rows_per_block = rows > 64 * kColsumParts ? (rows + kColsumParts - 1) / kColsumParts : 64;
  const int blocks = (rows + rows_per_block - 1) / rows_per_block;
  colsum_part<<<blocks, 128, 0, s>>>(dZ, rows, cols, rows_per_block, part);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  sum_parts<<<1, 128, 0, s>>>(part, blocks, cols, db);
  return cudaGetLastError();
}

cudaError_t transpose(const __nv_bfloat16 *in, __nv_bfloat16 *out, int rows, int cols, cudaStream_t s) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  transpose_bf16<<<grid, block, 0, s>>>(in, out, rows, cols);
  return cudaGetLastError();
}

}  // namespace

#define MCK(x)                            \
  do {                                    \
    cudaError_t e_ = (x);                 \
    if (e_ != cudaSuccess) return e_;     \
  } while (0)

cudaError_t Mlp::init(int n_in_, int n_hidden_, int n_out_, uint64_t seed, cudaStream_t s) {
  n_in = n_in_;
  H = n_hidden_;
  n_out = n_out_;
  stream = s;
  in_pad = ((n_in + 31) / 32) * 32;
  out_pad = ((n_out + 31) / 32) * 32;
  // parameter block (FP32 masters, padded shapes): W1 H x in_pad, b1 H, W2 H x H, b2 H, W3 out_pad x H, b3 out_pad
  off[0] = 0;
  size[0] = (size_t)H * in_pad;
  size[1] = H;
  size[2] = (size_t)H * H;
  size[3] = H;
  size[4] = (size_t)out_pad * H;
  size[5] = out_pad;
  for (int k = 1; k < 6; k++) off[k] = off[k - 1] + size[k - 1];
  n_params = off[5] + size[5];
  MCK(cudaMalloc(&w, n_params * sizeof(float)));
  MCK(cudaMalloc(&g, n_params * sizeof(float)));
  MCK(cudaMalloc(&m1, n_params * sizeof(float)));
  MCK(cudaMalloc(&m2, n_params * sizeof(float)));
  MCK(cudaMalloc(&wb, n_params * sizeof(__nv_bfloat16)));
  MCK(cudaMalloc(&wt, n_params * sizeof(__nv_bfloat16)));
  MCK(cudaMalloc(&loss, (1 + kMseBlocks) * sizeof(float)));
  MCK(cudaMalloc(&part, kPartFloats * sizeof(float)));
  MCK(cudaMalloc(&tc_err, sizeof(unsigned int)));
  MCK(cudaMemsetAsync(tc_err, 0, sizeof(unsigned int), stream));
  return reset(seed);
}

cudaError_t Mlp::reset(uint64_t seed) {
  MCK(cudaMemsetAsync(m1, 0, n_params * sizeof(float), stream));
  MCK(cudaMemsetAsync(m2, 0, n_params * sizeof(float), stream));
  // Glorot-uniform weights from a counter-based generator, zero biases; padded rows/cols zero
  std::vector<float> h(n_params, 0.f);
  auto u01 = [&](uint64_t k) {
    uint64_t z = (seed << 32) + k + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  uint64_t ctr = 0;
  auto fill = [&](int blk, int rows, int cols, int real_rows, int real_cols, int fan_in, int fan_out) {
    const double a = std::sqrt(6.0 / (fan_in + fan_out));
    for (int r = 0; r < rows; r++)
      for (int c = 0; c < cols; c++) {
        const double u = u01(ctr++);
        h[off[blk] + (size_t)r * cols + c] = (r < real_rows && c < real_cols) ? (float)((2 * u - 1) * a) : 0.f;
      }
  };
  fill(0, H, in_pad, H, n_in, n_in, H);
  fill(2, H, H, H, H, H, H);
  fill(4, out_pad, H, n_out, H, H, n_out);
  MCK(cudaMemcpyAsync(w, h.data(), n_params * sizeof(float), cudaMemcpyHostToDevice, stream));
  step = 0;
  return sync_bf16();
}

cudaError_t Mlp::sync_bf16() {
  version++;
  to_bf16<<<(unsigned)((n_params + 255) / 256), 256, 0, stream>>>(w, wb, (int)n_params);
  MCK(cudaGetLastError());
  // transposed copies for the backward products: W3^T (H x out_pad), W2^T (H x H)
  MCK(transpose(wb + off[4], wt + off[4], out_pad, H, stream));
  MCK(transpose(wb + off[2], wt + off[2], H, H, stream));
  return cudaSuccess;
}

void Mlp::release() {
  for (void *p : {(void *)w, (void *)g, (void *)m1, (void *)m2, (void *)wb, (void *)wt, (void *)loss, (void *)ws,
                  (void *)part, (void *)tc_err})
    cudaFree(p);
  part = nullptr;
  tc_err = nullptr;
  w = g = m1 = m2 = nullptr;
  wb = wt = nullptr;
  loss = nullptr;
  ws = nullptr;
  ws_rows = 0;
}

cudaError_t Mlp::workspace(int rows) {
  if (rows <= ws_rows) return cudaSuccess;
  cudaFree(ws);
  ws = nullptr;
  ws_rows = 0;
  // X, XT, H1, H1T, H2, H2T, dZ1, dZ1T, dZ2, dZ2T, dY, dYT (bf16) + Y, Xf, Tf (f32)
  const size_t b16 = (size_t)rows * (2 * in_pad + 8 * H + 2 * out_pad);
  const size_t f32 = (size_t)rows * (out_pad + n_in + n_out);
  MCK(cudaMalloc(&ws, b16 * 2 + f32 * 4 + 64));
  ws_rows = rows;
  return cudaSuccess;
}

Mlp::Buffers Mlp::buffers(int rows) const {
  Buffers B;
  __nv_bfloat16 *p = (__nv_bfloat16 *)ws;
  auto take = [&](size_t n) {
    __nv_bfloat16 *q = p;
    p += n;
    return q;
  };
  B.X = take((size_t)rows * in_pad);
  B.XT = take((size_t)rows * in_pad);
  B.H1 = take((size_t)rows * H);
  B.H1T = take((size_t)rows * H);
  B.H2 = take((size_t)rows * H);
  B.H2T = take((size_t)rows * H);
  B.dZ1 = take((size_t)rows * H);
  B.dZ1T = take((size_t)rows * H);
  B.dZ2 = take((size_t)rows * H);
  B.dZ2T = take((size_t)rows * H);
  B.dY = take((size_t)rows * out_pad);
  B.dYT = take((size_t)rows * out_pad);
  float *f = reinterpret_cast<float *>(p);
  B.Y = f;
  B.Xf = f + (size_t)rows * out_pad;
  B.Tf = B.Xf + (size_t)rows * n_in;
  return B;
}

cudaError_t Mlp::forward_rows(const Buffers &B, int rows) {
  EpiArgs e{};
  e.bias = w + off[1];
  e.out_bf16 = B.H1;
  e.ldc = H;
  MCK(gemm_tcgen05<EPI_BIAS_TANH>(B.X, in_pad, wb + off[0], in_pad, rows, H, in_pad, e, 1, tc_err, stream));
  e.bias = w + off[3];
  e.out_bf16 = B.H2;
  MCK(gemm_tcgen05<EPI_BIAS_TANH>(B.H1, H, wb + off[2], H, rows, H, H, e, 1, tc_err, stream));
  EpiArgs e3{};
  e3.bias = w + off[5];
  e3.out_f32 = B.Y;
  e3.ldc = out_pad;
  return gemm_tcgen05<EPI_BIAS_F32>(B.H2, H, wb + off[4], H, rows, out_pad, H, e3, 1, tc_err, stream);
}

cudaError_t Mlp::check_tc() {
  unsigned int h = 0;
  MCK(cudaMemcpyAsync(&h, tc_err, sizeof(h), cudaMemcpyDeviceToHost, stream));
  MCK(cudaStreamSynchronize(stream));
  if (!h) return cudaSuccess;
  MCK(cudaMemsetAsync(tc_err, 0, sizeof(unsigned int), stream));
  return cudaErrorLaunchTimeout;
}

cudaError_t Mlp::forward(const float *X, int64_t n, float *Y) {
  const int rows = (int)(((n + 63) / 64) * 64);
  MCK(workspace(rows));
  Buffers B = buffers(rows);
  pack_inputs<<<1024, 256, 0, stream>>>(X, (int)n, n_in, rows, in_pad, B.X);
  MCK(cudaGetLastError());
  MCK(forward_rows(B, rows));
  // Y (rows x out_pad) -> caller's n x n_out
  MCK(cudaMemcpy2DAsync(Y, n_out * sizeof(float), B.Y, out_pad * sizeof(float), n_out * sizeof(float), n,
                        cudaMemcpyDeviceToDevice, stream));
  return check_tc();
}

size_t Mlp::forward_scratch_bytes_per_row() const {
  return (size_t)(in_pad + 2 * H) * sizeof(__nv_bfloat16) + (size_t)out_pad * sizeof(float);
}

cudaError_t Mlp::forward_in_scratch(void *scratch, const float *X, int64_t n, float *Y) {
  const int rows = (int)(((n + 63) / 64) * 64);
  // X | H1 | H2 (BF16) | Y (FP32); rows is a multiple of 64, so every part starts 256-byte aligned
  Buffers B{};
  B.X = (__nv_bfloat16 *)scratch;
  B.H1 = B.X + (size_t)rows * in_pad;
  B.H2 = B.H1 + (size_t)rows * H;
  B.Y = (float *)(B.H2 + (size_t)rows * H);
  pack_inputs<<<1024, 256, 0, stream>>>(X, (int)n, n_in, rows, in_pad, B.X);  // writes the padding too
  MCK(cudaGetLastError());
  MCK(forward_rows(B, rows));
  MCK(cudaMemcpy2DAsync(Y, n_out * sizeof(float), B.Y, out_pad * sizeof(float), n_out * sizeof(float), n,
                        cudaMemcpyDeviceToDevice, stream));
  return check_tc();
}

cudaError_t Mlp::loss_grad(const float *X, const float *T, int64_t n) {
  const int rows = (int)(((n + 63) / 64) * 64);
  MCK(workspace(rows));
  Buffers B = buffers(rows);
  pack_inputs<<<1024, 256, 0, stream>>>(X, (int)n, n_in, rows, in_pad, B.X);
  MCK(cudaGetLastError());
  MCK(forward_rows(B, rows));
  mse_grad<<<kMseBlocks, 256, 0, stream>>>(B.Y, T, rows, (int)n, n_out, out_pad, B.dY, loss + 1);
  MCK(cudaGetLastError());
  mse_total<<<1, 32, 0, stream>>>(loss + 1, kMseBlocks, loss);
  MCK(cudaGetLastError());
  // dZ2 = (dY W3) * (1 - H2^2): A = dY (rows x out_pad), B-operand rows = W3^T (H x out_pad)
  EpiArgs e{};
  e.out_bf16 = B.dZ2;
  e.h = B.H2;
  e.ldc = H;
  MCK(gemm_tcgen05<EPI_DTANH>(B.dY, out_pad, wt + off[4], out_pad, rows, H, out_pad, e, 1, tc_err, stream));
  e.out_bf16 = B.dZ1;
  e.h = B.H1;
  MCK(gemm_tcgen05<EPI_DTANH>(B.dZ2, H, wt + off[2], H, rows, H, H, e, 1, tc_err, stream));
  // weight gradients: dW = dZ^T A_prev, K = rows
  MCK(transpose(B.dY, B.dYT, rows, out_pad, stream));
  MCK(transpose(B.H2, B.H2T, rows, H, stream));
  MCK(transpose(B.dZ2, B.dZ2T, rows, H, stream));
  MCK(transpose(B.H1, B.H1T, rows, H, stream));
  MCK(transpose(B.dZ1, B.dZ1T, rows, H, stream));
  MCK(transpose(B.X, B.XT, rows, in_pad, stream));
  const int splits = rows >= 512 ? std::min(kMaxSplits, rows / 256) : 1;
  MCK(gemm_f32_split(B.dYT, rows, B.H2T, rows, out_pad, H, rows, g + off[4], H, part, splits, tc_err, stream));
  MCK(gemm_f32_split(B.dZ2T, rows, B.H1T, rows, H, H, rows, g + off[2], H, part, splits, tc_err, stream));
  MCK(gemm_f32_split(B.dZ1T, rows, B.XT, rows, H, in_pad, rows, g + off[0], in_pad, part, splits, tc_err, stream));
  MCK(colsum(B.dY, rows, out_pad, g + off[5], part, stream));
  MCK(colsum(B.dZ2, rows, H, g + off[3], part, stream));
  MCK(colsum(B.dZ1, rows, H, g + off[1], part, stream));
  return cudaGetLastError();
}

cudaError_t Mlp::adam_step(float lr, float b1, float b2, float eps) {
  step++;
  version++;
  const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
  adam<<<(unsigned)((n_params + 255) / 256), 256, 0, stream>>>(w, g, m1, m2, wb, (int)n_params, lr, b1, b2, eps, c1,
                                                                 c2);
  MCK(cudaGetLastError());
  // padded weight entries have zero gradients and stay zero
  MCK(transpose(wb + off[4], wt + off[4], out_pad, H, stream));
  MCK(transpose(wb + off[2], wt + off[2], H, H, stream));
  return cudaSuccess;
}

cudaError_t Mlp::train(const float *X, const float *T, int64_t n, int batch, int steps, float lr, uint64_t seed,
                       float *final_loss) {
  batch = (batch / 64) * 64;
  if (batch < 64) batch = 64;
  MCK(workspace(batch));
  Buffers B = buffers(batch);
  int64_t *idx = nullptr;
  MCK(cudaMalloc(&idx, batch * sizeof(int64_t)));
  std::vector<int64_t> hidx(batch);
  uint64_t state = seed * 0x9E3779B97F4A7C15ull + 1;
  float lsum = 0.f;
  int lcnt = 0;
  cudaError_t err = cudaSuccess;
  for (int it = 0; it < steps && err == cudaSuccess; it++) {
    for (int k = 0; k < batch; k++) {  // xorshift sampling with replacement
      state ^= state << 13;
      state ^= state >> 7;
      state ^= state << 17;
      hidx[k] = (int64_t)(state % (uint64_t)n);
    }
    err = cudaMemcpyAsync(idx, hidx.data(), batch * sizeof(int64_t), cudaMemcpyHostToDevice, stream);
    if (err == cudaSuccess) {
      gather_rows<<<batch, 32, 0, stream>>>(X, T, idx, batch, n_in, n_out, B.Xf, B.Tf);
      err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = loss_grad(B.Xf, B.Tf, batch);
    if (err == cudaSuccess) err = adam_step(lr, 0.9f, 0.999f, 1e-8f);
    if (err == cudaSuccess && it >= steps - 20) {
      float l = 0;
      err = cudaMemcpyAsync(&l, loss, sizeof(float), cudaMemcpyDeviceToHost, stream);
      if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
      lsum += l;
      lcnt++;
    }
  }
  cudaFree(idx);
  if (final_loss) *final_loss = lcnt ? lsum / lcnt : 0.f;
  if (err == cudaSuccess) err = check_tc();
  return err;
}

}  // namespace cm
