// The implicit finite-element step of acCELLerate::IntraStep (acCELLerate.cpp:1951-1993): after
// the cell update, b = R x and the solve A x = b, A = C_m beta/dt M + theta K, R = C_m beta/dt M -
// (1 - theta) K (set up at acCELLerate.cpp:541-653). A is symmetric positive definite, so the
// solve is conjugate gradients with the Jacobi preconditioner, from the current x as initial guess
// (the reference sets KSPSetInitialGuessNonzero, PETScLSE.h:376), in FP64.
//
// One iteration is two launches. Kernel a: alpha from the partial sums of p.q and r.z, x += alpha
// p, r -= alpha q, z = D^-1 r, partial sums of r.z and z.z. Kernel b: the convergence test, beta,
// p = z + beta p and q = A z + beta q (= A p without a dependence of the product on this kernel's
// own writes), partial sums of p.q. Partial sums are per block, and every block of the next
// kernel adds them in the same order: no atomics, the same scalars everywhere, deterministic
// results. The test is PETSc's default (KSPConvergedDefault) with the preconditioned norm:
// ||z|| < max(rtol ||D^-1 b||, atol); ||z|| > dtol ||D^-1 b|| stops as divergence.
#include <cuda_runtime.h>

#include "cm_launch.h"

namespace cm {

namespace {

// Resident blocks per SM: 3 (80 registers) measured 2-3 % faster per step than 4 (64 registers,
// spills in the iteration kernels), 6 and 8 15-30 % slower (the entry rounds spill).
#ifndef CM_THETA_BLOCKS_PER_SM
#define CM_THETA_BLOCKS_PER_SM 3
#endif
#ifndef CM_THETA_ROUND
#define CM_THETA_ROUND 8
#endif
constexpr int kThetaThreads = 256;
constexpr int kThetaBlocks = CM_THETA_BLOCKS_PER_SM;  // resident blocks per SM (register budget)

// Row l of a sliced operator times x, entries added in CSR order. The entries are fetched in
// rounds of kRound (all columns and values, then all gathered x), so a row of 27 entries costs
// about eight memory latencies rather than 54.
constexpr int kRound = CM_THETA_ROUND;
__device__ __forceinline__ double sell_row(const ThetaOp &A, const double *x, int64_t l) {
  const int64_t s = l >> 5;
  const int64_t e1 = A.ptr[s + 1];
  double acc = 0.0;
  for (int64_t e0 = A.ptr[s] + (l & 31); e0 < e1; e0 += 32 * kRound) {
    int32_t c[kRound];
    double v[kRound], xv[kRound];
#pragma unroll
    for (int k = 0; k < kRound; k++) {
      const int64_t e = e0 + 32 * k;
      c[k] = e < e1 ? A.col[e] : (int32_t)l;
      v[k] = e < e1 ? A.val[e] : 0.0;
    }
#pragma unroll
    for (int k = 0; k < kRound; k++) xv[k] = x[c[k]];
#pragma unroll
    for (int k = 0; k < kRound; k++)
      if (e0 + 32 * k < e1) acc += v[k] * xv[k];
  }
  return acc;
}

// Adds N values over the block; thread 0 writes value k to dst[k][blockIdx.x].
template <int N>
__device__ __forceinline__ void block_partials(double (&v)[N], double *const (&dst)[N]) {
  __shared__ double red[N][kThetaThreads / 32];
#pragma unroll
  for (int k = 0; k < N; k++)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; k++) red[k][w] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < N; k++) {
      double s = 0.0;
      for (int i = 0; i < kThetaThreads / 32; i++) s += red[k][i];
      dst[k][blockIdx.x] = s;
    }
  }
}

// The sums of N arrays of G partials, every block the same reduction tree (so the same scalars
// everywhere): strided per thread, then over the warp, then over the warps.
template <int N>
__device__ __forceinline__ void totals(const double *const (&src)[N], int G, double (&out)[N]) {
  __shared__ double red[N][kThetaThreads / 32];
  __shared__ double res[N];
  double v[N];
#pragma unroll
  for (int k = 0; k < N; k++) {
    v[k] = 0.0;
    for (int i = threadIdx.x; i < G; i += kThetaThreads) v[k] += src[k][i];
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; k++) red[k][w] = v[k];
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < N; k++) {
      double t = 0.0;
      for (int i = 0; i < kThetaThreads / 32; i++) t += red[k][i];
      res[k] = t;
    }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; k++) out[k] = res[k];
}

// r = R x - A x, z = D^-1 r, p = z; partials ||D^-1 R x||^2, r.z, z.z
__global__ void __launch_bounds__(kThetaThreads, kThetaBlocks) theta_init_kernel(ThetaOp A, ThetaOp R, ThetaVecs v, ThetaPart P) {
  double acc[3] = {0.0, 0.0, 0.0};
  for (int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; l < A.n; l += (int64_t)gridDim.x * blockDim.x) {
    const double b = sell_row(R, v.x, l);
    const double r = b - sell_row(A, v.x, l);
    const double d = v.dinv[l];
    const double z = d * r, zb = d * b;
    v.r[l] = r;
    v.z[l] = z;
    v.p[l] = z;
    acc[0] += zb * zb;
    acc[1] += r * z;
    acc[2] += z * z;
  }
  // bb, rz and zz into buffer 1 (the "previous iteration" of iteration 0)
  double *const dst[3] = {P.bb, P.rz + P.G, P.zz + P.G};
  block_partials<3>(acc, dst);
}

// q = A z (p = z); partial p.q; the test on the initial residual
__global__ void __launch_bounds__(kThetaThreads, kThetaBlocks) theta_q0_kernel(ThetaOp A, ThetaVecs v, ThetaPart P, ThetaCfg cfg,
                                                                 ThetaStat *st) {
  const double *const src[2] = {P.bb, P.zz + P.G};
  double tot[2];
  totals<2>(src, P.G, tot);
  const double rnorm0 = sqrt(tot[0]);
  const double zn = sqrt(tot[1]);
  const double tol = fmax(cfg.rtol * rnorm0, cfg.atol);
  if (zn < tol || !(zn == zn)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->done = zn < tol ? 1 : 3;
      st->iters = 0;
      st->znorm = zn;
    }
    return;
  }
  double acc[1] = {0.0};
  for (int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; l < A.n; l += (int64_t)gridDim.x * blockDim.x) {
    const double q = sell_row(A, v.z, l);
    v.q[l] = q;
    acc[0] += v.p[l] * q;
  }
  double *const dst[1] = {P.pq};
  block_partials<1>(acc, dst);
}

// iteration k, kernel a. k comes from st->kb, which only the previous kernel b writes; block 0
// passes it on in st->ka, which only the next kernel b reads (a block never reads a word that
// another block of the same launch writes).
__global__ void __launch_bounds__(kThetaThreads, kThetaBlocks) theta_a_kernel(ThetaVecs v, ThetaPart P, ThetaStat *st, int64_t n) {
  if (st->done) return;
  const int k = st->kb;
  if (blockIdx.x == 0 && threadIdx.x == 0) st->ka = k;
  const double *const src[2] = {P.rz + (size_t)((k + 1) & 1) * P.G, P.pq};
  double tot[2];
  totals<2>(src, P.G, tot);
  const double rz = tot[0], pq = tot[1];
  if (!(pq > 0.0) || !(rz == rz)) {  // breakdown: A not positive definite, or non-finite values
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->done = 3;
      st->iters = k;
    }
    return;
  }
  const double alpha = rz / pq;
  double acc[2] = {0.0, 0.0};
  // four rows per thread and pass, all their loads ahead of the stores (the vectors could alias
  // as far as the compiler knows, so it would not move a load above an earlier store)
  constexpr int U = 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t l0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; l0 < n; l0 += U * stride) {
    double xv[U], pv[U], rv[U], qv[U], dv[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int64_t l = l0 + u * stride;
      const bool in = l < n;
      xv[u] = in ? v.x[l] : 0.0;
      pv[u] = in ? v.p[l] : 0.0;
      rv[u] = in ? v.r[l] : 0.0;
      qv[u] = in ? v.q[l] : 0.0;
      dv[u] = in ? v.dinv[l] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int64_t l = l0 + u * stride;
      if (l < n) {
        const double r = rv[u] - alpha * qv[u];
        const double z = dv[u] * r;
        v.x[l] = xv[u] + alpha * pv[u];
        v.r[l] = r;
        v.z[l] = z;
        acc[0] += r * z;
        acc[1] += z * z;
      }
    }
  }
  double *const dst[2] = {P.rz + (size_t)(k & 1) * P.G, P.zz + (size_t)(k & 1) * P.G};
  block_partials<2>(acc, dst);
}

// iteration k, kernel b: the test, and the end of the loop of a conditional graph node (h != 0)
// when the solve converged, diverged, broke down or reached max_iter
__global__ void __launch_bounds__(kThetaThreads, kThetaBlocks) theta_b_kernel(ThetaOp A, ThetaVecs v, ThetaPart P, ThetaCfg cfg,
                                                                ThetaStat *st, int max_iter,
                                                                cudaGraphConditionalHandle h) {
  if (st->done) {
    if (h && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(h, 0);
    return;
  }
  const int k = st->ka;
  const double *const src[4] = {P.bb, P.rz + (size_t)(k & 1) * P.G, P.rz + (size_t)((k + 1) & 1) * P.G,
                                P.zz + (size_t)(k & 1) * P.G};
  double tot[4];
  totals<4>(src, P.G, tot);
  const double rnorm0 = sqrt(tot[0]);
  const double rz_new = tot[1], rz_old = tot[2];
  const double zn = sqrt(tot[3]);
  const double tol = fmax(cfg.rtol * rnorm0, cfg.atol);
  const bool conv = zn < tol;
  const bool div = !(zn == zn) || zn > cfg.dtol * rnorm0;
  if (conv || div || k + 1 >= max_iter) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->done = conv ? 1 : (div ? 2 : 0);
      st->iters = k + 1;
      st->znorm = zn;
      st->kb = k + 1;
      if (h) cudaGraphSetConditional(h, 0);
    }
    return;
  }
  const double beta = rz_new / rz_old;
  double acc[1] = {0.0};
  constexpr int U = 2;  // two rows per thread and pass: their products' rounds overlap
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t l0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; l0 < A.n; l0 += U * stride) {
    double az[U], zv[U], pv[U], qv[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int64_t l = l0 + u * stride;
      const bool in = l < A.n;
      zv[u] = in ? v.z[l] : 0.0;
      pv[u] = in ? v.p[l] : 0.0;
      qv[u] = in ? v.q[l] : 0.0;
      az[u] = in ? sell_row(A, v.z, l) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int64_t l = l0 + u * stride;
      if (l < A.n) {
        const double p = zv[u] + beta * pv[u];
        const double q = az[u] + beta * qv[u];
        v.p[l] = p;
        v.q[l] = q;
        acc[0] += p * q;
      }
    }
  }
  double *const dst[1] = {P.pq};
  block_partials<1>(acc, dst);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->iters = k + 1;
    st->znorm = zn;
    st->kb = k + 1;
  }
}

__global__ void theta_act_kernel(const double *x, double *act, int64_t n, double thr, double t) {
  for (int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x)
    if (act[l] == -1.0 && x[l] >= thr) act[l] = t;
}

__global__ void theta_dinv_kernel(ThetaOp A, double *dinv, int *bad) {
  for (int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; l < A.n; l += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = l >> 5;
    double d = 0.0;
    for (int64_t e = A.ptr[s] + (l & 31); e < A.ptr[s + 1]; e += 32)
      if (A.col[e] == l) d += A.val[e];
    if (!(d > 0.0)) atomicOr(bad, 1);
    dinv[l] = d > 0.0 ? 1.0 / d : 0.0;
  }
}

}  // namespace

int theta_grid() { return sm_count() * kThetaBlocks; }

cudaError_t launch_theta_dinv(const ThetaOp &A, double *dinv, int *bad, cudaStream_t s) {
  if (A.n == 0) return cudaSuccess;
  theta_dinv_kernel<<<theta_grid(), kThetaThreads, 0, s>>>(A, dinv, bad);
  return cudaGetLastError();
}

cudaError_t launch_theta_init(const ThetaOp &A, const ThetaOp &R, const ThetaVecs &v, const ThetaPart &P,
                              const ThetaCfg &cfg, ThetaStat *st, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(st, 0, sizeof(ThetaStat), s);
  if (e != cudaSuccess) return e;
  theta_init_kernel<<<P.G, kThetaThreads, 0, s>>>(A, R, v, P);
  theta_q0_kernel<<<P.G, kThetaThreads, 0, s>>>(A, v, P, cfg, st);
  return cudaGetLastError();
}

cudaError_t launch_theta_iters(const ThetaOp &A, const ThetaVecs &v, const ThetaPart &P, const ThetaCfg &cfg,
                               ThetaStat *st, int max_iter, int count, cudaStream_t s) {
  for (int k = 0; k < count; k++) {
    theta_a_kernel<<<P.G, kThetaThreads, 0, s>>>(v, P, st, A.n);
    theta_b_kernel<<<P.G, kThetaThreads, 0, s>>>(A, v, P, cfg, st, max_iter, 0);
  }
  return cudaGetLastError();
}

// A graph whose one node is a conditional while loop over [kernel a, kernel b]; kernel b ends
// the loop. Replaces the host's reads of the outcome between chunks of iterations.
cudaError_t build_theta_graph(const ThetaOp &A, const ThetaVecs &v, const ThetaPart &P, const ThetaCfg &cfg,
                              ThetaStat *st, int max_iter, cudaGraphExec_t *exec) {
  *exec = nullptr;
  cudaGraph_t g = nullptr;
  cudaStream_t cap = nullptr;
  cudaError_t e = cudaGraphCreate(&g, 0);
  cudaGraphConditionalHandle h = 0;
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
  if (e == cudaSuccess)
    e = cudaStreamBeginCaptureToGraph(cap, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    theta_a_kernel<<<P.G, kThetaThreads, 0, cap>>>(v, P, st, A.n);
    theta_b_kernel<<<P.G, kThetaThreads, 0, cap>>>(A, v, P, cfg, st, max_iter, h);
    cudaGraph_t body = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(cap, &body);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = e2;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(exec, g, 0);
  if (cap) cudaStreamDestroy(cap);
  if (g) cudaGraphDestroy(g);
  return e;
}

cudaError_t launch_theta_act(const double *x, double *act, int64_t n, double thr, double t, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  theta_act_kernel<<<theta_grid(), kThetaThreads, 0, s>>>(x, act, n, thr, t);
  return cudaGetLastError();
}

}  // namespace cm
