// One cell of a staged tile (cm_staged.cu, cm_multi.cu): the cell's state, Vm pair and present
// conductance planes are read from the tile's shared-memory stage S (this thread's column,
// plane stride kT), the mixed update runs in registers, and the results go straight to global
// memory (state planes, Vm pair, audit bits).
#pragma once

#include "cm_cells.cuh"

namespace cm {

template <int kModel>
struct StagedVars;
template <>
struct StagedVars<5> {
  static constexpr int kState = 21;  // tt2 mixed planes
};
template <>
struct StagedVars<2> {
  static constexpr int kState = 25;
};
template <>
struct StagedVars<12> {
  static constexpr int kState = kORDPlain + 12;  // O'Hara-Rudy mixed planes
};
template <>
struct StagedVars<14> {
  static constexpr int kState = kTOMPlain + 12;  // Tomek mixed planes
};

// O'Hara-Rudy (12) / Tomek (14) state store over a staged tile: every state is read from the
// stage when ord_calc / tom_calc reaches it (a shared-memory load, no long wait), every new value
// goes straight to its global plane.
template <int kModel, int kT>
struct StagedStore {
  const float *S;  // this cell's column of the stage (plane stride kT)
  float *s;        // this cell's global planes (stride ld)
  int64_t ld;
  __device__ __forceinline__ static int plane(int k, bool &pair) {
    return kModel == 12 ? ord_mixed_plane(k, pair) : tom_mixed_plane(k, pair);
  }
  __device__ __forceinline__ void fetch(int) {}
  __device__ __forceinline__ float get(int k) const {
    bool pair;
    return S[plane(k, pair) * kT];
  }
  __device__ __forceinline__ void set(int k, float x) {
    bool pair;
    s[plane(k, pair) * ld] = x;
  }
  // compensated add on the (hi, lo) pair; x is the hi word get() returned
  __device__ __forceinline__ void add(int k, float x, float d) {
    bool pair;
    const int q = plane(k, pair);
    Acc a{x, S[(q + 1) * kT]};
    acc_add(a, d);
    s[q * ld] = a.hi;
    s[(q + 1) * ld] = a.lo;
  }
  __device__ __forceinline__ void cur(int, float) {}
};

template <int kT, typename CT>
__device__ __forceinline__ ORDHet_<float> staged_ord_het(const CT &C, const float *S, const int (&het_pos)[6]) {
  ORDHet_<float> g;
  g.INaF = het_pos[HO_INaF] >= 0 ? S[het_pos[HO_INaF] * kT] : C.INaF;
  g.INaL = het_pos[HO_INaL] >= 0 ? S[het_pos[HO_INaL] * kT] : C.INaL;
  g.Ito = het_pos[HO_Ito] >= 0 ? S[het_pos[HO_Ito] * kT] : C.Ito;
  g.IKr = het_pos[HO_IKr] >= 0 ? S[het_pos[HO_IKr] * kT] : C.IKr;
  g.IKs = het_pos[HO_IKs] >= 0 ? S[het_pos[HO_IKs] * kT] : C.IKs;
  g.IK1 = het_pos[HO_IK1] >= 0 ? S[het_pos[HO_IK1] * kT] : C.IK1;
  return g;
}

// S: stage + threadIdx.x; planes 0..NS-1 state, NS / NS+1 Vm hi / lo, het_pos[k] the present
// conductance slots (-1: parameter-set value).
// Returns the new Vm pair (also written to vm_hi / vm_lo).
template <int kModel, int kT>
__device__ __forceinline__ Acc staged_cell(const DevBatch &b, const float *S, const int (&het_pos)[6], int c,
                                           float iext, float *vm_hi, float *vm_lo) {
  constexpr int NS = StagedVars<kModel>::kState;
  constexpr int kThreads = kT;
  const int64_t ld = b.ld;
  uint32_t audit = 0;
  Acc vm{S[NS * kThreads], S[(NS + 1) * kThreads]};
  float *s = b.s32 + c;
  if constexpr (kModel == 12) {
    StagedStore<12, kThreads> x{S, s, ld};
    acc_add(vm, ord_calc<float>(b.ord_32, x, staged_ord_het<kThreads>(b.ord_32, S, het_pos), vm.hi, iext, 1.f));
  } else if constexpr (kModel == 14) {
    StagedStore<14, kThreads> x{S, s, ld};
    acc_add(vm, tom_calc<float>(b.tom_32, x, staged_ord_het<kThreads>(b.tom_32, S, het_pos), vm.hi, iext, 1.f));
  } else if constexpr (kModel == 5) {
    const TT2Consts<float> &C = b.tt2_32;
    TT2Cell<float> x;
    x.m = S[0]; x.h = S[kThreads]; x.j = S[2 * kThreads]; x.xr1 = S[3 * kThreads]; x.xr2 = S[4 * kThreads];
    x.xs = S[5 * kThreads]; x.r = S[6 * kThreads]; x.s = S[7 * kThreads]; x.d = S[8 * kThreads];
    x.f = S[9 * kThreads]; x.f2 = S[10 * kThreads]; x.fCa = S[11 * kThreads]; x.Rq = S[12 * kThreads];
    x.Ca_i = S[13 * kThreads]; x.CaSS = S[14 * kThreads];
    Acc CaSR{S[15 * kThreads], S[16 * kThreads]}, Na_i{S[17 * kThreads], S[18 * kThreads]},
        K_i{S[19 * kThreads], S[20 * kThreads]};
    TT2Het_<float> g;
    g.g_Na = het_pos[H2_g_Na] >= 0 ? S[het_pos[H2_g_Na] * kThreads] : C.g_Na;
    g.g_Kr = het_pos[H2_g_Kr] >= 0 ? S[het_pos[H2_g_Kr] * kThreads] : C.g_Kr;
    g.g_K1 = het_pos[H2_g_K1] >= 0 ? S[het_pos[H2_g_K1] * kThreads] : C.g_K1;
    g.g_Ks = het_pos[H2_g_Ks] >= 0 ? S[het_pos[H2_g_Ks] * kThreads] : C.g_Ks;
    g.g_to = het_pos[H2_g_to] >= 0 ? S[het_pos[H2_g_to] * kThreads] : C.g_to;
    g.g_CaL = het_pos[H2_g_CaL] >= 0 ? S[het_pos[H2_g_CaL] * kThreads] : C.g_CaL;
    const int vi = vrow_fp32(vm.hi * 1000.f, audit);
    const float dV = tt2_calc_mixed(C, b.rows32 + (size_t)vi * T2_COLS, b.eca32, x, CaSR, Na_i, K_i, g, vm.hi,
                                    iext, audit);
    s[0] = x.m; s[ld] = x.h; s[2 * ld] = x.j; s[3 * ld] = x.xr1; s[4 * ld] = x.xr2; s[5 * ld] = x.xs;
    s[6 * ld] = x.r; s[7 * ld] = x.s; s[8 * ld] = x.d; s[9 * ld] = x.f; s[10 * ld] = x.f2;
    s[11 * ld] = x.fCa; s[12 * ld] = x.Rq; s[13 * ld] = x.Ca_i; s[14 * ld] = x.CaSS;
    s[15 * ld] = CaSR.hi; s[16 * ld] = CaSR.lo; s[17 * ld] = Na_i.hi; s[18 * ld] = Na_i.lo;
    s[19 * ld] = K_i.hi; s[20 * ld] = K_i.lo;
    acc_add(vm, dV);
  } else {
    const CRNConsts<float> &C = b.crn_32;
    CRNCell<float> x;
    x.h = S[0]; x.j = S[kThreads]; x.oi = S[2 * kThreads]; x.ui = S[3 * kThreads]; x.Xr = S[4 * kThreads];
    x.Xs = S[5 * kThreads]; x.u = S[6 * kThreads]; x.v = S[7 * kThreads]; x.w = S[8 * kThreads];
    x.m = S[9 * kThreads]; x.oa = S[10 * kThreads]; x.ua = S[11 * kThreads]; x.d = S[12 * kThreads];
    x.f = S[13 * kThreads]; x.f_Ca = S[14 * kThreads]; x.Ca_i = S[15 * kThreads]; x.Ca_TRPN = S[16 * kThreads];
    Acc Ca_up{S[17 * kThreads], S[18 * kThreads]}, Ca_rel{S[19 * kThreads], S[20 * kThreads]},
        Na_i{S[21 * kThreads], S[22 * kThreads]}, K_i{S[23 * kThreads], S[24 * kThreads]};
    CRNHet_<float> g;
    g.g_Na = het_pos[HC_g_Na] >= 0 ? S[het_pos[HC_g_Na] * kThreads] : C.g_Na;
    g.g_to = het_pos[HC_g_to] >= 0 ? S[het_pos[HC_g_to] * kThreads] : C.g_to;
    g.g_Ks = het_pos[HC_g_Ks] >= 0 ? S[het_pos[HC_g_Ks] * kThreads] : C.g_Ks;
    g.g_CaL = het_pos[HC_g_CaL] >= 0 ? S[het_pos[HC_g_CaL] * kThreads] : C.g_CaL;
    g.g_bNa = het_pos[HC_g_bNa] >= 0 ? S[het_pos[HC_g_bNa] * kThreads] : C.g_bNa;
    g.g_bCa = het_pos[HC_g_bCa] >= 0 ? S[het_pos[HC_g_bCa] * kThreads] : C.g_bCa;
    const int vi = vrow_fp32(vm.hi * 1000.f, audit);
    const float dV = crn_calc_mixed(C, b.rows32 + (size_t)vi * CR_COLS, x, Ca_up, Ca_rel, Na_i, K_i, g, vm.hi,
                                    iext, 1.f, audit);
    s[0] = x.h; s[ld] = x.j; s[2 * ld] = x.oi; s[3 * ld] = x.ui; s[4 * ld] = x.Xr; s[5 * ld] = x.Xs;
    s[6 * ld] = x.u; s[7 * ld] = x.v; s[8 * ld] = x.w; s[9 * ld] = x.m; s[10 * ld] = x.oa; s[11 * ld] = x.ua;
    s[12 * ld] = x.d; s[13 * ld] = x.f; s[14 * ld] = x.f_Ca; s[15 * ld] = x.Ca_i; s[16 * ld] = x.Ca_TRPN;
    s[17 * ld] = Ca_up.hi; s[18 * ld] = Ca_up.lo; s[19 * ld] = Ca_rel.hi; s[20 * ld] = Ca_rel.lo;
    s[21 * ld] = Na_i.hi; s[22 * ld] = Na_i.lo; s[23 * ld] = K_i.hi; s[24 * ld] = K_i.lo;
    acc_add(vm, dV);
  }
  vm_hi[c] = vm.hi;
  vm_lo[c] = vm.lo;
  if (!isfinite(vm.hi)) audit |= 1u;
  if (audit) {
    atomicOr(b.audit_cell + c, audit);
    atomicOr(b.audit_or, audit);
  }
  return vm;
}

}  // namespace cm
