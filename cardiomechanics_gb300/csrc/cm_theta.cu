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

constexpr int kThetaThreads = 256;

__device__ __forceinline__ double sell_row(const ThetaOp &A, const double *x, int64_t l) {
  const int64_t s = l >> 5;
  const int64_t e1 = A.ptr[s + 1];
  double acc = 0.0;
  for (int64_t e = A.ptr[s] + (l & 31); e < e1; e += 32) acc += A.val[e] * x[A.col[e]];
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

// The sum of G partials, in the same order in every block.
__device__ __forceinline__ double total(const double *part, int G) {
  __shared__ double s_tot;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < G; i++) s += part[i];
    s_tot = s;
  }
  __syncthreads();
  return s_tot;
}

// r = R x - A x, z = D^-1 r, p = z; partials ||D^-1 R x||^2, r.z, z.z
__global__ void __launch_bounds__(kThetaThreads) theta_init_kernel(ThetaOp A, ThetaOp R, ThetaVecs v, ThetaPart P) {
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
__global__ void __launch_bounds__(kThetaThreads) theta_q0_kernel(ThetaOp A, ThetaVecs v, ThetaPart P, ThetaCfg cfg,
                                                                 ThetaStat *st) {
  const double rnorm0 = sqrt(total(P.bb, P.G));
  const double zn = sqrt(total(P.zz + P.G, P.G));
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

// iteration k, kernel a
__global__ void __launch_bounds__(kThetaThreads) theta_a_kernel(ThetaVecs v, ThetaPart P, ThetaStat *st, int64_t n,
                                                                int k) {
  if (st->done) return;
  const double rz = total(P.rz + (size_t)((k + 1) & 1) * P.G, P.G);
  const double pq = total(P.pq, P.G);
  if (!(pq > 0.0) || !(rz == rz)) {  // breakdown: A not positive definite, or non-finite values
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->done = 3;
      st->iters = k;
    }
    return;
  }
  const double alpha = rz / pq;
  double acc[2] = {0.0, 0.0};
  for (int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; l < n; l += (int64_t)gridDim.x * blockDim.x) {
    v.x[l] += alpha * v.p[l];
    const double r = v.r[l] - alpha * v.q[l];
    const double z = v.dinv[l] * r;
    v.r[l] = r;
    v.z[l] = z;
    acc[0] += r * z;
    acc[1] += z * z;
  }
  double *const dst[2] = {P.rz + (size_t)(k & 1) * P.G, P.zz + (size_t)(k & 1) * P.G};
  block_partials<2>(acc, dst);
}

// iteration k, kernel b
__global__ void __launch_bounds__(kThetaThreads) theta_b_kernel(ThetaOp A, ThetaVecs v, ThetaPart P, ThetaCfg cfg,
                                                                ThetaStat *st, int k) {
  if (st->done) return;
  const double rnorm0 = sqrt(total(P.bb, P.G));
  const double rz_new = total(P.rz + (size_t)(k & 1) * P.G, P.G);
  const double rz_old = total(P.rz + (size_t)((k + 1) & 1) * P.G, P.G);
  const double zn = sqrt(total(P.zz + (size_t)(k & 1) * P.G, P.G));
  const double tol = fmax(cfg.rtol * rnorm0, cfg.atol);
  const bool conv = zn < tol;
  const bool div = !(zn == zn) || zn > cfg.dtol * rnorm0;
  if (conv || div) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->done = conv ? 1 : 2;
      st->iters = k + 1;
      st->znorm = zn;
    }
    return;
  }
  const double beta = rz_new / rz_old;
  double acc[1] = {0.0};
  for (int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; l < A.n; l += (int64_t)gridDim.x * blockDim.x) {
    const double p = v.z[l] + beta * v.p[l];
    const double q = sell_row(A, v.z, l) + beta * v.q[l];
    v.p[l] = p;
    v.q[l] = q;
    acc[0] += p * q;
  }
  double *const dst[1] = {P.pq};
  block_partials<1>(acc, dst);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->iters = k + 1;
    st->znorm = zn;
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

int theta_grid() { return sm_count() * 4; }

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
                               ThetaStat *st, int k0, int count, cudaStream_t s) {
  for (int k = k0; k < k0 + count; k++) {
    theta_a_kernel<<<P.G, kThetaThreads, 0, s>>>(v, P, st, A.n, k);
    theta_b_kernel<<<P.G, kThetaThreads, 0, s>>>(A, v, P, cfg, st, k);
  }
  return cudaGetLastError();
}

cudaError_t launch_theta_act(const double *x, double *act, int64_t n, double thr, double t, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  theta_act_kernel<<<theta_grid(), kThetaThreads, 0, s>>>(x, act, n, thr, t);
  return cudaGetLastError();
}

}  // namespace cm
