// Per-cell bodies of the mixed kernels: load one cell's state from its batch, advance it one
// step and store it back. Shared by the single-batch kernels (cm_kernels.cu) and the
// multi-instance kernel (cm_multi.cu).
#pragma once

#include "cm_crn.cuh"
#include "cm_launch.h"
#include "cm_tom.cuh"
#include "cm_tt2.cuh"

namespace cm {

// Stimulus current of cell c: the reference driver's rule (CellModel.h:405-419) with per-cell
// first stimulus times, advanced in place; else the per-cell array or the uniform value.
__device__ __forceinline__ double stim_for_cell(const StepIO &io, int64_t c) {
  if (io.tb_cell) {
    const double tb = io.tb_cell[c];
    double i_ext = 0.0;
    if (f64_ge(io.t, tb)) {  // integer compare: no FP64-pipe instruction per cell
      i_ext = io.amp;
      if (io.t >= tb + io.textlen) io.tb_cell[c] = tb + io.bcl;
    }
    return i_ext;
  }
  return io.iext ? __ldg(io.iext + c) : io.iext_uniform;
}

template <typename I>
__device__ __forceinline__ float tt2_mixed_cell(const DevBatch &b, I c, float V, float iext, uint32_t &audit) {
  const I ld = (I)b.ld;
  const float *const *het = (const float *const *)b.het;
  float *s = b.s32 + c;
  TT2Cell<float> x;
  x.m = s[0]; x.h = s[ld]; x.j = s[2 * ld]; x.xr1 = s[3 * ld]; x.xr2 = s[4 * ld]; x.xs = s[5 * ld];
  x.r = s[6 * ld]; x.s = s[7 * ld]; x.d = s[8 * ld]; x.f = s[9 * ld]; x.f2 = s[10 * ld]; x.fCa = s[11 * ld];
  x.Rq = s[12 * ld]; x.Ca_i = s[13 * ld]; x.CaSS = s[14 * ld];
  Acc CaSR{s[15 * ld], s[16 * ld]}, Na_i{s[17 * ld], s[18 * ld]}, K_i{s[19 * ld], s[20 * ld]};
  const TT2Consts<float> &C = b.tt2_32;
  TT2Het_<float> g;
  g.g_Na = het[H2_g_Na] ? __ldg(het[H2_g_Na] + c) : C.g_Na;
  g.g_Kr = het[H2_g_Kr] ? __ldg(het[H2_g_Kr] + c) : C.g_Kr;
  g.g_K1 = het[H2_g_K1] ? __ldg(het[H2_g_K1] + c) : C.g_K1;
  g.g_Ks = het[H2_g_Ks] ? __ldg(het[H2_g_Ks] + c) : C.g_Ks;
  g.g_to = het[H2_g_to] ? __ldg(het[H2_g_to] + c) : C.g_to;
  g.g_CaL = het[H2_g_CaL] ? __ldg(het[H2_g_CaL] + c) : C.g_CaL;
  const int vi = vrow_fp32(V * 1000.f, audit);
  const float dV = tt2_calc_mixed(C, b.rows32 + (size_t)vi * T2_COLS, b.eca32, x, CaSR, Na_i, K_i, g, V, iext, audit);
  s[0] = x.m; s[ld] = x.h; s[2 * ld] = x.j; s[3 * ld] = x.xr1; s[4 * ld] = x.xr2; s[5 * ld] = x.xs;
  s[6 * ld] = x.r; s[7 * ld] = x.s; s[8 * ld] = x.d; s[9 * ld] = x.f; s[10 * ld] = x.f2; s[11 * ld] = x.fCa;
  s[12 * ld] = x.Rq; s[13 * ld] = x.Ca_i; s[14 * ld] = x.CaSS;
  s[15 * ld] = CaSR.hi; s[16 * ld] = CaSR.lo; s[17 * ld] = Na_i.hi; s[18 * ld] = Na_i.lo;
  s[19 * ld] = K_i.hi; s[20 * ld] = K_i.lo;
  return dV;
}

template <typename I>
__device__ __forceinline__ float crn_mixed_cell(const DevBatch &b, I c, float V, float iext, float stretch,
                                                uint32_t &audit) {
  const I ld = (I)b.ld;
  const float *const *het = (const float *const *)b.het;
  float *s = b.s32 + c;
  CRNCell<float> x;
  x.h = s[0]; x.j = s[ld]; x.oi = s[2 * ld]; x.ui = s[3 * ld]; x.Xr = s[4 * ld]; x.Xs = s[5 * ld];
  x.u = s[6 * ld]; x.v = s[7 * ld]; x.w = s[8 * ld]; x.m = s[9 * ld]; x.oa = s[10 * ld]; x.ua = s[11 * ld];
  x.d = s[12 * ld]; x.f = s[13 * ld]; x.f_Ca = s[14 * ld]; x.Ca_i = s[15 * ld]; x.Ca_TRPN = s[16 * ld];
  Acc Ca_up{s[17 * ld], s[18 * ld]}, Ca_rel{s[19 * ld], s[20 * ld]}, Na_i{s[21 * ld], s[22 * ld]},
      K_i{s[23 * ld], s[24 * ld]};
  const CRNConsts<float> &C = b.crn_32;
  CRNHet_<float> g;
  g.g_Na = het[HC_g_Na] ? __ldg(het[HC_g_Na] + c) : C.g_Na;
  g.g_to = het[HC_g_to] ? __ldg(het[HC_g_to] + c) : C.g_to;
  g.g_Ks = het[HC_g_Ks] ? __ldg(het[HC_g_Ks] + c) : C.g_Ks;
  g.g_CaL = het[HC_g_CaL] ? __ldg(het[HC_g_CaL] + c) : C.g_CaL;
  g.g_bNa = het[HC_g_bNa] ? __ldg(het[HC_g_bNa] + c) : C.g_bNa;
  g.g_bCa = het[HC_g_bCa] ? __ldg(het[HC_g_bCa] + c) : C.g_bCa;
  const int vi = vrow_fp32(V * 1000.f, audit);
  const float dV = crn_calc_mixed(C, b.rows32 + (size_t)vi * CR_COLS, x, Ca_up, Ca_rel, Na_i, K_i, g, V, iext,
                                  stretch, audit);
  s[0] = x.h; s[ld] = x.j; s[2 * ld] = x.oi; s[3 * ld] = x.ui; s[4 * ld] = x.Xr; s[5 * ld] = x.Xs;
  s[6 * ld] = x.u; s[7 * ld] = x.v; s[8 * ld] = x.w; s[9 * ld] = x.m; s[10 * ld] = x.oa; s[11 * ld] = x.ua;
  s[12 * ld] = x.d; s[13 * ld] = x.f; s[14 * ld] = x.f_Ca; s[15 * ld] = x.Ca_i; s[16 * ld] = x.Ca_TRPN;
  s[17 * ld] = Ca_up.hi; s[18 * ld] = Ca_up.lo; s[19 * ld] = Ca_rel.hi; s[20 * ld] = Ca_rel.lo;
  s[21 * ld] = Na_i.hi; s[22 * ld] = Na_i.lo; s[23 * ld] = K_i.hi; s[24 * ld] = K_i.lo;
  return dV;
}

// Monodomain coupling current of cell c: scale_c * (A x)_c with A's row c in its 32-row slice
// (acCELLerate.cpp:1849 MatMult and 1880-1887 conversion). Padding entries of a slice carry
// value 0 and the row's own column. The first kCouplingBatch entries of the row are fetched in
// two rounds -- all columns and values, then all neighbour potentials -- so a row costs two
// memory latencies rather than two per entry; longer rows continue entry by entry.
constexpr int kCouplingBatch = 8;

// FP64: entries summed in CSR order.
__device__ __forceinline__ double coupling_fp64(const StepIO &io, const double *x, int64_t c) {
  const int64_t s = c >> 5;
  const int64_t e0 = io.sl_ptr[s] + (c & 31), e1 = io.sl_ptr[s + 1];
  int32_t cj[kCouplingBatch];
  double aj[kCouplingBatch];
#pragma unroll
  for (int k = 0; k < kCouplingBatch; k++) {
    const int64_t e = e0 + 32 * k;
    cj[k] = e < e1 ? io.sl_col[e] : (int32_t)c;
    aj[k] = e < e1 ? io.sl_val64[e] : 0.0;
  }
  double xj[kCouplingBatch];
#pragma unroll
  for (int k = 0; k < kCouplingBatch; k++) xj[k] = __ldg(x + cj[k]);
  double acc = 0.0;
#pragma unroll
  for (int k = 0; k < kCouplingBatch; k++)
    if (e0 + 32 * k < e1) acc += aj[k] * xj[k];
  for (int64_t e = e0 + 32 * kCouplingBatch; e < e1; e += 32) acc += io.sl_val64[e] * __ldg(x + io.sl_col[e]);
  return acc * (io.dscale64 ? __ldg(io.dscale64 + c) : io.dscale_u);
}

// Mixed form: rowsum_c x_c + sum_j A_cj (x_j - x_c) on the previous step's hi plane; the
// differences of neighbouring potentials are small, so FP32 keeps them (the plain sum would
// cancel a diagonal ~6 orders above the result at rest).
template <typename I>
__device__ __forceinline__ float coupling_f32(const StepIO &io, I c) {
  const float *x = io.vm_hi;
  const int64_t s = (int64_t)c >> 5;
  const int64_t e0 = io.sl_ptr[s] + (c & 31), e1 = io.sl_ptr[s + 1];
  int32_t cj[kCouplingBatch];
  float aj[kCouplingBatch];
#pragma unroll
  for (int k = 0; k < kCouplingBatch; k++) {
    const int64_t e = e0 + 32 * k;
    cj[k] = e < e1 ? io.sl_col[e] : (int32_t)c;
    aj[k] = e < e1 ? io.sl_val32[e] : 0.f;
  }
  const float xc = x[c];
  float xj[kCouplingBatch];
#pragma unroll
  for (int k = 0; k < kCouplingBatch; k++) xj[k] = x[cj[k]];
  float acc = __ldg(io.rowsum32 + c) * xc;
#pragma unroll
  for (int k = 0; k < kCouplingBatch; k++) acc += aj[k] * (xj[k] - xc);
  for (int64_t e = e0 + 32 * kCouplingBatch; e < e1; e += 32) acc += io.sl_val32[e] * (x[io.sl_col[e]] - xc);
  return acc * (io.dscale32 ? __ldg(io.dscale32 + c) : (float)io.dscale_u);
}

// O'Hara-Rudy state stores over a batch's device memory (see ord_calc): every state read
// and written in place as ord_calc reaches it.
struct ORDStore64 {
  double *s;     // state of this cell: s[k * ld]
  int64_t ld;
  double *diag;  // 17 x ld currents of this cell, or nullptr
  __device__ __forceinline__ void fetch(int) {}
  __device__ __forceinline__ double get(int k) const { return s[k * ld]; }
  __device__ __forceinline__ void set(int k, double v) { s[k * ld] = v; }
  // the reference's `X += tinc * dX` (OHaraRudy.cpp:597-659)
  __device__ __forceinline__ void add(int k, double x, double d) { s[k * ld] = x + d; }
  __device__ __forceinline__ void cur(int k, double v) {
    if (diag) diag[k * ld] = v;
  }
};

// The FP32 store reads the cell's words in two batches, each before any write that could
// precede it: a load placed after a store to the same planes could not be moved above it (the
// planes might alias), so loads taken one by one as ord_calc reaches them would each wait out
// the full memory latency, and loading all 47 words at once would not fit the registers.
// Batch 0 (when the store is made): CaMK, the I_Na/I_NaL/I_to gates, Na_i, K_i, Ca_ss; batch 1
// (fetch(1), before I_CaL): everything else.
template <typename I>
struct ORDStore32 {
  float *s;  // mixed planes of this cell: s[plane * ld]
  I ld;
  float v[SO_N];  // this step's inputs (hi words for the pairs)
  float lo[6];    // lo words of the pairs, ord_pair_var order
  __device__ __forceinline__ static bool first(int k) {
    return k <= SO_i_CaMK_slow || k == SO_Na_i || k == SO_K_i || k == SO_Ca_ss || k == SO_CaMK_trap;
  }
  __device__ __forceinline__ ORDStore32(float *s_, I ld_) : s(s_), ld(ld_) { fetch(0); }
  __device__ __forceinline__ void fetch(int part) {
#pragma unroll
    for (int k = 0; k < SO_N; k++) {
      bool pair;
      if (first(k) == (part == 0)) v[k] = s[ord_mixed_plane(k, pair) * ld];
    }
    if (part == 1) {
#pragma unroll
      for (int q = 0; q < 6; q++) lo[q] = s[(kORDPlain + 2 * q + 1) * ld];
    }
  }
  __device__ __forceinline__ float get(int k) const { return v[k]; }
  __device__ __forceinline__ void set(int k, float x) {
    bool pair;
    s[ord_mixed_plane(k, pair) * ld] = x;
  }
  // compensated add on the (hi, lo) pair; x is the hi word get() returned
  __device__ __forceinline__ void add(int k, float x, float d) {
    const int q = k <= SO_K_ss ? k - SO_Na_i : 4 + (k - SO_Ca_nsr);
    Acc a{x, lo[q]};
    acc_add(a, d);
    s[(kORDPlain + 2 * q) * ld] = a.hi;
    s[(kORDPlain + 2 * q + 1) * ld] = a.lo;
  }
  __device__ __forceinline__ void cur(int, float) {}
};

// The six per-cell multiplier slots (INaF, INaL, Ito, IKr, IKs, IK1) of O'Hara-Rudy and Tomek:
// the cell's own value where a slot is set, else the parameter set's.
template <typename R, typename CT, typename I>
__device__ __forceinline__ ORDHet_<R> ord_het(const DevBatch &b, const CT &C, I c) {
  const R *const *het = (const R *const *)b.het;
  ORDHet_<R> g;
  g.INaF = het[HO_INaF] ? __ldg(het[HO_INaF] + c) : C.INaF;
  g.INaL = het[HO_INaL] ? __ldg(het[HO_INaL] + c) : C.INaL;
  g.Ito = het[HO_Ito] ? __ldg(het[HO_Ito] + c) : C.Ito;
  g.IKr = het[HO_IKr] ? __ldg(het[HO_IKr] + c) : C.IKr;
  g.IKs = het[HO_IKs] ? __ldg(het[HO_IKs] + c) : C.IKs;
  g.IK1 = het[HO_IK1] ? __ldg(het[HO_IK1] + c) : C.IK1;
  return g;
}

// Tomek FP32 store: the O'Hara-Rudy store's two-batch loads over the Tomek planes. Batch 0:
// CaMK, the I_Na/I_NaL/I_to gates, Na_i, K_i, Ca_ss, Cl_i; batch 1 (before I_CaL): the rest.
template <typename I>
struct TOMStore32 {
  float *s;  // mixed planes of this cell: s[plane * ld]
  I ld;
  float v[SM_N];  // this step's inputs (hi words for the pairs)
  float lo[6];    // lo words of Na_i, Na_ss, K_i, K_ss, Ca_nsr, Ca_jsr
  __device__ __forceinline__ static bool first(int k) {
    return k <= SM_i_CaMK_slow || k == SM_Na_i || k == SM_K_i || k == SM_Ca_ss || k == SM_Cl_i ||
           k == SM_CaMK_trap;
  }
  __device__ __forceinline__ TOMStore32(float *s_, I ld_) : s(s_), ld(ld_) { fetch(0); }
  __device__ __forceinline__ void fetch(int part) {
#pragma unroll
    for (int k = 0; k < SM_N; k++) {
      bool pair;
      if (first(k) == (part == 0)) v[k] = s[tom_mixed_plane(k, pair) * ld];
    }
    if (part == 1) {
#pragma unroll
      for (int q = 0; q < 6; q++) lo[q] = s[(kTOMPlain + 2 * q + 1) * ld];
    }
  }
  __device__ __forceinline__ float get(int k) const { return v[k]; }
  __device__ __forceinline__ void set(int k, float x) {
    bool pair;
    s[tom_mixed_plane(k, pair) * ld] = x;
  }
  __device__ __forceinline__ void add(int k, float x, float d) {
    const int q = k <= SM_K_ss ? k - SM_Na_i : 4 + (k - SM_Ca_nsr);
    Acc a{x, lo[q]};
    acc_add(a, d);
    s[(kTOMPlain + 2 * q) * ld] = a.hi;
    s[(kTOMPlain + 2 * q + 1) * ld] = a.lo;
  }
  __device__ __forceinline__ void cur(int, float) {}
};

template <typename I>
__device__ __forceinline__ float tom_mixed_cell(const DevBatch &b, I c, float V, float iext, float stretch) {
  TOMStore32<I> x(b.s32 + c, (I)b.ld);
  return tom_calc<float>(b.tom_32, x, ord_het<float>(b, b.tom_32, c), V, iext, stretch);
}

template <typename I>
__device__ __forceinline__ float ord_mixed_cell(const DevBatch &b, I c, float V, float iext, float stretch) {
  ORDStore32<I> x(b.s32 + c, (I)b.ld);
  return ord_calc<float>(b.ord_32, x, ord_het<float>(b, b.ord_32, c), V, iext, stretch);
}

}  // namespace cm
