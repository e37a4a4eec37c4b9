// Per-timestep cell-model kernels for sm_103a: one thread per cell, structure-of-arrays
// state (coalesced: a warp touches 256 contiguous bytes per FP64 variable, 128 per FP32
// one), voltage lookup rows read through the read-only path (cells of a tissue or of a
// synchronously paced population share a few rows, which stay L1-resident).
//
// The FP64 kernels do all arithmetic in FP64 (the reference's arithmetic; the GB300 FP64
// pipe bounds them). The mixed kernels do gates and currents in FP32 and keep four FP64
// accumulators; they are bound by HBM bandwidth.
#include <cuda_runtime.h>

#include "cm_cells.cuh"

namespace cm {

namespace {

// i_external of a cell update: the stimulus plus, in coupled kernels (kCoupled, launched for
// cm_batch_run_diffuse only), the coupling current.
template <bool kCoupled>
__device__ __forceinline__ double iext_fp64(const StepIO &io, int64_t c) {
  double i = stim_for_cell(io, c);
  if (kCoupled) i += coupling_fp64(io, io.vm, c);
  return i;
}

template <bool kCoupled, typename I>
__device__ __forceinline__ float iext_f32(const StepIO &io, I c) {
  float i = (float)stim_for_cell(io, c);
  if (kCoupled) i += coupling_f32<I>(io, c);
  return i;
}

__device__ __forceinline__ void finish(const DevBatch &b, const StepIO &io, int64_t c, double V, double dV,
                                       uint32_t audit) {
  const double vn = V + dV;
  if (io.vm_out) io.vm_out[c] = vn;
  if (io.dvm) io.dvm[c] = dV;
  if (!isfinite(vn)) audit |= 1u;
  if (io.vm_range > 0.0 && fabs(vn) > io.vm_range) audit |= 32u;
  if (io.act && io.act[c] == -1.0 && vn >= io.act_threshold) io.act[c] = io.act_time;
  if (audit) {
    atomicOr(b.audit_cell + c, audit);
    atomicOr(b.audit_or, audit);
  }
}

template <typename I>
__device__ __forceinline__ void finish_acc(const DevBatch &b, I c, Acc v, uint32_t audit, const StepIO &io) {
  (io.vm_hi_out ? io.vm_hi_out : io.vm_hi)[c] = v.hi;
  (io.vm_lo_out ? io.vm_lo_out : io.vm_lo)[c] = v.lo;
  if (!isfinite(v.hi)) audit |= 1u;
  if (io.vm_range > 0.0 && fabsf(v.hi) > (float)io.vm_range) audit |= 32u;
  if (io.act && io.act[c] == -1.0 && v.hi >= (float)io.act_threshold) io.act[c] = io.act_time;
  if (audit) {
    atomicOr(b.audit_cell + c, audit);
    atomicOr(b.audit_or, audit);
  }
}

template <bool kDiag, bool kCoupled>
__global__ void __launch_bounds__(128) tt2_fp64_kernel(const DevBatch b, const StepIO io) {
  const int64_t ld = b.ld;
  const double *const *het = (const double *const *)b.het;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < b.n; c += (int64_t)gridDim.x * blockDim.x) {
    double *s = b.s64 + c;
    TT2Cell<double> x;
    x.Ca_i = s[S2_Cai * ld];
    double CaSR = s[S2_CaSR * ld];
    x.CaSS = s[S2_CaSS * ld];
    double Na_i = s[S2_Nai * ld], K_i = s[S2_Ki * ld];
    x.m = s[S2_m * ld]; x.h = s[S2_h * ld]; x.j = s[S2_j * ld]; x.xr1 = s[S2_xr1 * ld];
    x.xr2 = s[S2_xr2 * ld]; x.xs = s[S2_xs * ld]; x.r = s[S2_r * ld]; x.s = s[S2_s * ld];
    x.d = s[S2_d * ld]; x.f = s[S2_f * ld]; x.f2 = s[S2_f2 * ld]; x.fCa = s[S2_fCa * ld];
    x.Rq = s[S2_Rq * ld];
    const TT2Consts<double> &C = b.tt2_64;
    TT2Het_<double> g;
    g.g_Na = het[H2_g_Na] ? __ldg(het[H2_g_Na] + c) : C.g_Na;
    g.g_Kr = het[H2_g_Kr] ? __ldg(het[H2_g_Kr] + c) : C.g_Kr;
    g.g_K1 = het[H2_g_K1] ? __ldg(het[H2_g_K1] + c) : C.g_K1;
    g.g_Ks = het[H2_g_Ks] ? __ldg(het[H2_g_Ks] + c) : C.g_Ks;
    g.g_to = het[H2_g_to] ? __ldg(het[H2_g_to] + c) : C.g_to;
    g.g_CaL = het[H2_g_CaL] ? __ldg(het[H2_g_CaL] + c) : C.g_CaL;
    const double V = __ldg(io.vm + c);
    const double iext = iext_fp64<kCoupled>(io, c);
    uint32_t audit = 0;
    const int vi = vrow_fp64(V * 1000, audit);
    TT2Diag<double> dg;
    const double dV = tt2_calc_fp64<kDiag>(C, b.rows64 + (size_t)vi * T2_COLS, b.eca64, x, CaSR, Na_i, K_i, g, V,
                                           iext, audit, &dg);
    s[S2_Cai * ld] = x.Ca_i; s[S2_CaSR * ld] = CaSR; s[S2_CaSS * ld] = x.CaSS; s[S2_Nai * ld] = Na_i;
    s[S2_Ki * ld] = K_i; s[S2_m * ld] = x.m; s[S2_h * ld] = x.h; s[S2_j * ld] = x.j; s[S2_xr1 * ld] = x.xr1;
    s[S2_xr2 * ld] = x.xr2; s[S2_xs * ld] = x.xs; s[S2_r * ld] = x.r; s[S2_s * ld] = x.s; s[S2_d * ld] = x.d;
    s[S2_f * ld] = x.f; s[S2_f2 * ld] = x.f2; s[S2_fCa * ld] = x.fCa; s[S2_Rq * ld] = x.Rq;
    if (kDiag)
      for (int k = 0; k < 17; k++) b.diag[k * ld + c] = dg.v[k];
    finish(b, io, c, V, dV, audit);
  }
}

template <typename I, int kBlock, int kMinB, bool kCoupled = false>
__global__ void __launch_bounds__(kBlock, kMinB) tt2_mixed_kernel(const DevBatch b, const StepIO io) {
  for (I c = (I)blockIdx.x * blockDim.x + threadIdx.x; c < (I)b.n; c += (I)gridDim.x * blockDim.x) {
    const float iext = iext_f32<kCoupled>(io, c);
    uint32_t audit = 0;
    if (io.vm_hi) {
      Acc v{io.vm_hi[c], io.vm_lo[c]};
      acc_add(v, tt2_mixed_cell<I>(b, c, v.hi, iext, audit));
      finish_acc(b, c, v, audit, io);
    } else {
      const double V = __ldg(io.vm + c);
      const float dV = tt2_mixed_cell<I>(b, c, (float)V, iext, audit);
      finish(b, io, c, V, (double)dV, audit);
    }
  }
}

template <bool kDiag, bool kCoupled>
__global__ void __launch_bounds__(128) crn_fp64_kernel(const DevBatch b, const StepIO io) {
  const int64_t ld = b.ld;
  const double *const *het = (const double *const *)b.het;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < b.n; c += (int64_t)gridDim.x * blockDim.x) {
    double *s = b.s64 + c;
    CRNCell<double> x;
    x.Ca_i = s[SC_Cai * ld];
    double Ca_up = s[SC_Caup * ld], Ca_rel = s[SC_Carel * ld];
    x.h = s[SC_h * ld]; x.j = s[SC_j * ld]; x.oi = s[SC_oi * ld]; x.ui = s[SC_ui * ld]; x.Xr = s[SC_Xr * ld];
    x.Xs = s[SC_Xs * ld]; x.u = s[SC_u * ld]; x.v = s[SC_v * ld]; x.w = s[SC_w * ld];
    double Na_i = s[SC_Nai * ld], K_i = s[SC_Ki * ld];
    x.m = s[SC_m * ld]; x.oa = s[SC_oa * ld]; x.ua = s[SC_ua * ld]; x.d = s[SC_d * ld]; x.f = s[SC_f * ld];
    x.f_Ca = s[SC_fCa * ld]; x.Ca_TRPN = s[SC_CaTRPN * ld];
    const CRNConsts<double> &C = b.crn_64;
    CRNHet_<double> g;
    g.g_Na = het[HC_g_Na] ? __ldg(het[HC_g_Na] + c) : C.g_Na;
    g.g_to = het[HC_g_to] ? __ldg(het[HC_g_to] + c) : C.g_to;
    g.g_Ks = het[HC_g_Ks] ? __ldg(het[HC_g_Ks] + c) : C.g_Ks;
    g.g_CaL = het[HC_g_CaL] ? __ldg(het[HC_g_CaL] + c) : C.g_CaL;
    g.g_bNa = het[HC_g_bNa] ? __ldg(het[HC_g_bNa] + c) : C.g_bNa;
    g.g_bCa = het[HC_g_bCa] ? __ldg(het[HC_g_bCa] + c) : C.g_bCa;
    const double V = __ldg(io.vm + c);
    const double iext = iext_fp64<kCoupled>(io, c);
    const double stretch = io.stretch ? __ldg(io.stretch + c) : 1.0;
    uint32_t audit = 0;
    const int vi = vrow_fp64(V * 1000.0, audit);
    double isac;
    const double dV = crn_calc_fp64(C, b.rows64 + (size_t)vi * CR_COLS, x, Ca_up, Ca_rel, Na_i, K_i, g, V, iext,
                                    stretch, isac, audit);
    s[SC_Cai * ld] = x.Ca_i; s[SC_Caup * ld] = Ca_up; s[SC_Carel * ld] = Ca_rel; s[SC_h * ld] = x.h;
    s[SC_j * ld] = x.j; s[SC_oi * ld] = x.oi; s[SC_ui * ld] = x.ui; s[SC_Xr * ld] = x.Xr; s[SC_Xs * ld] = x.Xs;
    s[SC_u * ld] = x.u; s[SC_v * ld] = x.v; s[SC_w * ld] = x.w; s[SC_Nai * ld] = Na_i; s[SC_Ki * ld] = K_i;
    s[SC_m * ld] = x.m; s[SC_oa * ld] = x.oa; s[SC_ua * ld] = x.ua; s[SC_d * ld] = x.d; s[SC_f * ld] = x.f;
    s[SC_fCa * ld] = x.f_Ca; s[SC_CaTRPN * ld] = x.Ca_TRPN;
    if (kDiag) b.diag[c] = isac;
    finish(b, io, c, V, dV, audit);
  }
}

template <typename I, int kBlock, int kMinB, bool kCoupled = false>
__global__ void __launch_bounds__(kBlock, kMinB) crn_mixed_kernel(const DevBatch b, const StepIO io) {
  for (I c = (I)blockIdx.x * blockDim.x + threadIdx.x; c < (I)b.n; c += (I)gridDim.x * blockDim.x) {
    const float iext = iext_f32<kCoupled>(io, c);
    const float stretch = io.stretch ? (float)__ldg(io.stretch + c) : 1.f;
    uint32_t audit = 0;
    if (io.vm_hi) {
      Acc v{io.vm_hi[c], io.vm_lo[c]};
      acc_add(v, crn_mixed_cell<I>(b, c, v.hi, iext, stretch, audit));
      finish_acc(b, c, v, audit, io);
    } else {
      const double V = __ldg(io.vm + c);
      const float dV = crn_mixed_cell<I>(b, c, (float)V, iext, stretch, audit);
      finish(b, io, c, V, (double)dV, audit);
    }
  }
}

template <bool kDiag, bool kCoupled>
__global__ void __launch_bounds__(128) ord_fp64_kernel(const DevBatch b, const StepIO io) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < b.n; c += (int64_t)gridDim.x * blockDim.x) {
    ORDStore64 x{b.s64 + c, b.ld, kDiag ? b.diag + c : nullptr};
    const double V = __ldg(io.vm + c);
    const double iext = iext_fp64<kCoupled>(io, c);
    const double stretch = io.stretch ? __ldg(io.stretch + c) : 1.0;
    const double dV = ord_calc<double>(b.ord_64, x, ord_het<double>(b, b.ord_64, c), V, iext, stretch);
    finish(b, io, c, V, dV, 0u);
  }
}

template <typename I, int kBlock, int kMinB, bool kCoupled = false>
__global__ void __launch_bounds__(kBlock, kMinB) ord_mixed_kernel(const DevBatch b, const StepIO io) {
  for (I c = (I)blockIdx.x * blockDim.x + threadIdx.x; c < (I)b.n; c += (I)gridDim.x * blockDim.x) {
    const float iext = iext_f32<kCoupled>(io, c);
    const float stretch = io.stretch ? (float)__ldg(io.stretch + c) : 1.f;
    if (io.vm_hi) {
      Acc v{io.vm_hi[c], io.vm_lo[c]};
      acc_add(v, ord_mixed_cell<I>(b, c, v.hi, iext, stretch));
      finish_acc(b, c, v, 0u, io);
    } else {
      const double V = __ldg(io.vm + c);
      const float dV = ord_mixed_cell<I>(b, c, (float)V, iext, stretch);
      finish(b, io, c, V, (double)dV, 0u);
    }
  }
}

template <bool kDiag, bool kCoupled>
__global__ void __launch_bounds__(128) tom_fp64_kernel(const DevBatch b, const StepIO io) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < b.n; c += (int64_t)gridDim.x * blockDim.x) {
    ORDStore64 x{b.s64 + c, b.ld, kDiag ? b.diag + c : nullptr};
    const double V = __ldg(io.vm + c);
    const double iext = iext_fp64<kCoupled>(io, c);
    const double stretch = io.stretch ? __ldg(io.stretch + c) : 1.0;
    const double dV = tom_calc<double>(b.tom_64, x, ord_het<double>(b, b.tom_64, c), V, iext, stretch);
    finish(b, io, c, V, dV, 0u);
  }
}

template <typename I, int kBlock, int kMinB, bool kCoupled = false>
__global__ void __launch_bounds__(kBlock, kMinB) tom_mixed_kernel(const DevBatch b, const StepIO io) {
  for (I c = (I)blockIdx.x * blockDim.x + threadIdx.x; c < (I)b.n; c += (I)gridDim.x * blockDim.x) {
    const float iext = iext_f32<kCoupled>(io, c);
    const float stretch = io.stretch ? (float)__ldg(io.stretch + c) : 1.f;
    if (io.vm_hi) {
      Acc v{io.vm_hi[c], io.vm_lo[c]};
      acc_add(v, tom_mixed_cell<I>(b, c, v.hi, iext, stretch));
      finish_acc(b, c, v, 0u, io);
    } else {
      const double V = __ldg(io.vm + c);
      const float dV = tom_mixed_cell<I>(b, c, (float)V, iext, stretch);
      finish(b, io, c, V, (double)dV, 0u);
    }
  }
}

__global__ void diffusion_apply_kernel(const StepIO io, const double *x, double *y, int64_t n) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    y[c] = coupling_fp64(io, x, c);
}

__global__ void probe_kernel(const double *vm, const float *vm_hi, const float *vm_lo, const int64_t *probe,
                             int64_t n_probe, double *out, int64_t stride, int64_t k) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_probe) {
    const int64_t c = probe[i];
    out[i * stride + k] = vm ? vm[c] : acc_to_double(Acc{vm_hi[c], vm_lo[c]});
  }
}

__global__ void vm_split_kernel(const double *v, float *hi, float *lo, int64_t n) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const Acc a = acc_from_double(v[c]);
    hi[c] = a.hi;
    lo[c] = a.lo;
  }
}

__global__ void vm_join_kernel(const float *hi, const float *lo, double *v, int64_t n) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x)
    v[c] = acc_to_double(Acc{hi[c], lo[c]});
}

// The same two conversions two cells per thread with 16-byte accesses of Vm (fewer, wider
// transactions where Vm is host memory read or written over the host link).
__global__ void vm_split2_kernel(const double2 *v, float2 *hi, float2 *lo, int64_t n2) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n2; c += (int64_t)gridDim.x * blockDim.x) {
    const double2 x = v[c];
    const Acc a = acc_from_double(x.x), b = acc_from_double(x.y);
    hi[c] = make_float2(a.hi, b.hi);
    lo[c] = make_float2(a.lo, b.lo);
  }
}

__global__ void vm_join2_kernel(const float2 *hi, const float2 *lo, double2 *v, int64_t n2) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n2; c += (int64_t)gridDim.x * blockDim.x) {
    const float2 h = hi[c], l = lo[c];
    v[c] = make_double2(acc_to_double(Acc{h.x, l.x}), acc_to_double(Acc{h.y, l.y}));
  }
}

bool aligned_pair(const void *v, const void *hi, const void *lo) {
  return ((uintptr_t)v % 16 == 0) && ((uintptr_t)hi % 8 == 0) && ((uintptr_t)lo % 8 == 0);
}

}  // namespace

int n_fp32_vars(int model) {
  return model == 5 ? 21 : (model == 12 ? kORDPlain + 12 : (model == 14 ? kTOMPlain + 12 : 25));
}
int n_fp64_vars(int model, int precision) {
  if (precision == 0) return model == 5 ? S2_N : (model == 12 ? SO_N : (model == 14 ? SM_N : SC_N));
  return 0;
}

int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

// Launch shapes of the mixed kernels the autotuner chooses from: (threads per block,
// minimum resident blocks per SM as a register-allocation hint).
namespace {
struct Shape {
  int block, minb;
};
// register budgets: (256,2) and (512,1) -> 128, (128,5) and (64,10) -> 96, (256,3) -> 80
constexpr Shape kShapes[] = {{256, 2}, {128, 5}, {256, 3}, {512, 1}, {64, 10}};

template <typename I, int B, int M>
void launch_mixed(const DevBatch &b, const StepIO &io, int grid, cudaStream_t s) {
  if (b.model == 5) tt2_mixed_kernel<I, B, M><<<grid, B, 0, s>>>(b, io);
  else if (b.model == 12) ord_mixed_kernel<I, B, M><<<grid, B, 0, s>>>(b, io);
  else if (b.model == 14) tom_mixed_kernel<I, B, M><<<grid, B, 0, s>>>(b, io);
  else crn_mixed_kernel<I, B, M><<<grid, B, 0, s>>>(b, io);
}

template <typename I>
void launch_mixed_variant(const DevBatch &b, const StepIO &io, int v, int grid, cudaStream_t s) {
  if (io.sl_ptr) {  // coupled runs: one shape (256 threads, 128 registers)
    if (b.model == 5) tt2_mixed_kernel<I, 256, 2, true><<<grid, 256, 0, s>>>(b, io);
    else if (b.model == 12) ord_mixed_kernel<I, 256, 2, true><<<grid, 256, 0, s>>>(b, io);
    else if (b.model == 14) tom_mixed_kernel<I, 256, 2, true><<<grid, 256, 0, s>>>(b, io);
    else crn_mixed_kernel<I, 256, 2, true><<<grid, 256, 0, s>>>(b, io);
    return;
  }
  switch (v) {
    case 1: launch_mixed<I, 128, 5>(b, io, grid, s); break;
    case 2: launch_mixed<I, 256, 3>(b, io, grid, s); break;
    case 3: launch_mixed<I, 512, 1>(b, io, grid, s); break;
    case 4: launch_mixed<I, 64, 10>(b, io, grid, s); break;
    default: launch_mixed<I, 256, 2>(b, io, grid, s); break;
  }
}
}  // namespace

// Variants past the register-budget shapes are the shared-memory-staged kernels: the
// double-buffered block (256 and 128 threads per block), then the producer/consumer pipeline
// (256 consumer threads with 2 stages, 128 with 3). They apply to fused runs and fall back to
// shape 0 elsewhere.
int n_register_shapes() { return (int)(sizeof(kShapes) / sizeof(kShapes[0])); }
int n_shape_variants() { return n_register_shapes() + 4; }

cudaError_t launch_step(const DevBatch &b, const StepIO &io, int variant, int grid_mode, cudaStream_t s) {
  if (b.n == 0) return cudaSuccess;
  const bool diag = b.diag != nullptr;
  // 32-bit offsets when every state index fits (ld * variables < 2^31)
  const bool small = b.ld * (n_fp32_vars(b.model) + 1) < (int64_t)2147483647;
  if (b.precision == 0) {
    const int block = 128;
    const int64_t need = (b.n + block - 1) / block;
    const int64_t cap = (int64_t)sm_count() * 16;
    const int grid = (int)(need < cap ? need : cap);
    if (b.model == 5) {
      if (diag) if (io.sl_ptr) tt2_fp64_kernel<true, true><<<grid, block, 0, s>>>(b, io); else tt2_fp64_kernel<true, false><<<grid, block, 0, s>>>(b, io);
      else if (io.sl_ptr) tt2_fp64_kernel<false, true><<<grid, block, 0, s>>>(b, io); else tt2_fp64_kernel<false, false><<<grid, block, 0, s>>>(b, io);
    } else if (b.model == 12) {
      if (diag) if (io.sl_ptr) ord_fp64_kernel<true, true><<<grid, block, 0, s>>>(b, io); else ord_fp64_kernel<true, false><<<grid, block, 0, s>>>(b, io);
      else if (io.sl_ptr) ord_fp64_kernel<false, true><<<grid, block, 0, s>>>(b, io); else ord_fp64_kernel<false, false><<<grid, block, 0, s>>>(b, io);
    } else if (b.model == 14) {
      if (diag) if (io.sl_ptr) tom_fp64_kernel<true, true><<<grid, block, 0, s>>>(b, io); else tom_fp64_kernel<true, false><<<grid, block, 0, s>>>(b, io);
      else if (io.sl_ptr) tom_fp64_kernel<false, true><<<grid, block, 0, s>>>(b, io); else tom_fp64_kernel<false, false><<<grid, block, 0, s>>>(b, io);
    } else {
      if (diag) if (io.sl_ptr) crn_fp64_kernel<true, true><<<grid, block, 0, s>>>(b, io); else crn_fp64_kernel<true, false><<<grid, block, 0, s>>>(b, io);
      else if (io.sl_ptr) crn_fp64_kernel<false, true><<<grid, block, 0, s>>>(b, io); else crn_fp64_kernel<false, false><<<grid, block, 0, s>>>(b, io);
    }
    return cudaGetLastError();
  }
  // coupled runs of TT2 / Courtemanche: the staged kernel with the operator staged too
  if (io.sl_ptr && coupled_staged_supported(b, io)) return launch_coupled_staged(b, io, variant, s);
  if (variant < 0 || variant >= n_shape_variants()) variant = 0;
  const int n_plain = n_register_shapes();
  if (variant >= n_plain) {
    if (staged_supported(b, io)) {
      const int k = variant - n_plain;
      return k < 2 ? launch_staged(b, io, k == 0 ? 256 : 128, grid_mode, s)
                   : launch_pipe(b, io, k == 2 ? 256 : 128, grid_mode, s);
    }
    variant = 0;
  }
  const Shape sh = io.sl_ptr ? Shape{256, 2} : kShapes[variant];  // coupled runs: one shape
  const int64_t need = (b.n + sh.block - 1) / sh.block;
  // grid_mode 0: one thread per cell; k > 0: grid-stride over k blocks per SM
  const int64_t cap = grid_mode > 0 ? (int64_t)sm_count() * grid_mode : need;
  const int grid = (int)(need < cap ? need : cap);
  if (small) launch_mixed_variant<int>(b, io, variant, grid, s);
  else launch_mixed_variant<int64_t>(b, io, variant, grid, s);
  return cudaGetLastError();
}

cudaError_t launch_diffusion_apply(const StepIO &io, const double *x, double *y, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t g = (n + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 16;
  diffusion_apply_kernel<<<(unsigned)(g < cap ? g : cap), 256, 0, s>>>(io, x, y, n);
  return cudaGetLastError();
}

cudaError_t launch_probe(const double *vm, const float *vm_hi, const float *vm_lo, const int64_t *probe,
                         int64_t n_probe, double *out, int64_t stride, int64_t k, cudaStream_t s) {
  if (n_probe <= 0) return cudaSuccess;
  probe_kernel<<<(unsigned)((n_probe + 127) / 128), 128, 0, s>>>(vm, vm_hi, vm_lo, probe, n_probe, out, stride, k);
  return cudaGetLastError();
}

cudaError_t launch_vm_split(const double *v, float *hi, float *lo, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t g = (n + 255) / 256;
  if (n >= 2 && aligned_pair(v, hi, lo)) {
    const int64_t n2 = n / 2, g2 = (n2 + 255) / 256;
    vm_split2_kernel<<<(unsigned)(g2 < 65535 ? g2 : 65535), 256, 0, s>>>((const double2 *)v, (float2 *)hi,
                                                                          (float2 *)lo, n2);
    if (n % 2) vm_split_kernel<<<1, 32, 0, s>>>(v + 2 * n2, hi + 2 * n2, lo + 2 * n2, 1);
    return cudaGetLastError();
  }
  vm_split_kernel<<<(unsigned)(g < 65535 ? g : 65535), 256, 0, s>>>(v, hi, lo, n);
  return cudaGetLastError();
}

cudaError_t launch_vm_join(const float *hi, const float *lo, double *v, int64_t n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t g = (n + 255) / 256;
  if (n >= 2 && aligned_pair(v, hi, lo)) {
    const int64_t n2 = n / 2, g2 = (n2 + 255) / 256;
    vm_join2_kernel<<<(unsigned)(g2 < 65535 ? g2 : 65535), 256, 0, s>>>((const float2 *)hi, (const float2 *)lo,
                                                                         (double2 *)v, n2);
    if (n % 2) vm_join_kernel<<<1, 32, 0, s>>>(hi + 2 * n2, lo + 2 * n2, v + 2 * n2, 1);
    return cudaGetLastError();
  }
  vm_join_kernel<<<(unsigned)(g < 65535 ? g : 65535), 256, 0, s>>>(hi, lo, v, n);
  return cudaGetLastError();
}

}  // namespace cm
