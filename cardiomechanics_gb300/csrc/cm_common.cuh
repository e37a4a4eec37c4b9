// Shared definitions for the cell-model kernels: table geometry, per-model device
// parameter blocks, state layouts and small numeric helpers.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define CM_HD __host__ __device__ __forceinline__
#else
#define CM_HD inline
#include <cmath>
#endif

namespace cm {

// Voltage-table geometry (reference ElphyModelBasis.h:46-56): 4000 rows, row
// Vi = int(10 * (200 + V[mV]) + 0.5), built on V = -199.9999 + k * 0.1 (accumulated).
constexpr int kRows = 4000;
constexpr int kRangeHalf = 200;
constexpr int kDivision = 10;

// Row layout of the TT2 voltage table on the device (one row = 28 values, 224 B in FP64).
// Gates are stored as (x_inf, exp(-dt/tau_x)) pairs; j_inf repeats h_inf as in the reference
// (TenTusscher2Parameters.cpp:420).
enum TT2Col {
  T2_m_inf, T2_exptau_m, T2_h_inf, T2_exptau_h, T2_j_inf, T2_exptau_j, T2_Xr1_inf, T2_exptau_Xr1,
  T2_Xr2_inf, T2_exptau_Xr2, T2_Xs_inf, T2_exptau_Xs, T2_r_inf, T2_exptau_r, T2_s_inf, T2_exptau_s,
  T2_d_inf, T2_exptau_d, T2_f_inf, T2_exptau_f, T2_f2_inf, T2_exptau_f2, T2_rec_ipK, T2_CaL_P1,
  T2_CaL_P2, T2_NaCa_P1, T2_NaCa_P2, T2_NaK_P1, T2_COLS
};

// Row layout of the Courtemanche voltage table (30 values, 240 B in FP64).
enum CRNCol {
  CR_m_m, CR_exptau_m, CR_m_h, CR_exptau_h, CR_m_j, CR_exptau_j, CR_m_oa, CR_exptau_oa, CR_m_oi,
  CR_exptau_oi, CR_m_ua, CR_exptau_ua, CR_m_ui, CR_exptau_ui, CR_m_Xr, CR_exptau_Xr, CR_m_Xs,
  CR_exptau_Xs, CR_m_d, CR_exptau_d, CR_m_f, CR_exptau_f, CR_m_w, CR_exptau_w, CR_expVm, CR_CK1,
  CR_g_Kur, CR_CKr, CR_CNaK, CR_CNaCa, CR_COLS
};

// Per-cell state variables in SOA order (Vm is the caller's).
enum TT2State {
  S2_Cai, S2_CaSR, S2_CaSS, S2_Nai, S2_Ki, S2_m, S2_h, S2_j, S2_xr1, S2_xr2, S2_xs, S2_r, S2_s, S2_d,
  S2_f, S2_f2, S2_fCa, S2_Rq, S2_N
};
enum CRNState {
  SC_Cai, SC_Caup, SC_Carel, SC_h, SC_j, SC_oi, SC_ui, SC_Xr, SC_Xs, SC_u, SC_v, SC_w, SC_Nai, SC_Ki,
  SC_m, SC_oa, SC_ua, SC_d, SC_f, SC_fCa, SC_CaTRPN, SC_N
};

// O'Hara-Rudy: the reference block order (OHaraRudy.h:31-43) without h_CaMK_fast, which the
// reference declares but never sets or reads.
enum ORDState {
  SO_m, SO_h_fast, SO_h_slow, SO_j, SO_h_CaMK_slow, SO_j_CaMK, SO_m_L, SO_h_L, SO_h_L_CaMK, SO_a, SO_i_fast,
  SO_i_slow, SO_a_CaMK, SO_i_CaMK_fast, SO_i_CaMK_slow, SO_d, SO_f_fast, SO_f_slow, SO_f_Ca_fast, SO_f_Ca_slow,
  SO_j_Ca, SO_n, SO_f_CaMK_fast, SO_f_Ca_CaMK_fast, SO_x_r_fast, SO_x_r_slow, SO_x_s1, SO_x_s2, SO_x_K1,
  SO_Na_i, SO_Na_ss, SO_K_i, SO_K_ss, SO_Ca_i, SO_Ca_ss, SO_Ca_nsr, SO_Ca_jsr, SO_CaMK_trap, SO_J_rel_NP,
  SO_J_rel_CaMK, SO_Ca_TRPN, SO_N
};
// The 17 currents the reference keeps after the states (OHaraRudy.h:48-52); the FP64
// kernel writes them when diagnostics are on.
constexpr int kORDCurrents = 17;

// O'Hara-Rudy mixed form: planes 0..34 are the FP32 states (ORDState order, the six
// compensated concentrations left out), planes 35..46 the (hi, lo) pairs of Na_i, Na_ss, K_i,
// K_ss, Ca_nsr and Ca_jsr.
constexpr int kORDPlain = 35;

// ORDState variable of pair q (Na_i, Na_ss, K_i, K_ss, Ca_nsr, Ca_jsr).
CM_HD int ord_pair_var(int q) { return q < 4 ? SO_Na_i + q : SO_Ca_nsr + (q - 4); }

// Plane of ORDState variable k in the mixed layout (for a pair, its hi plane; lo follows).
CM_HD int ord_mixed_plane(int k, bool &pair) {
  pair = false;
  if (k < SO_Na_i) return k;
  if (k == SO_Ca_i || k == SO_Ca_ss) return k - 4;
  if (k >= SO_CaMK_trap) return k - 6;
  pair = true;
  return k <= SO_K_ss ? kORDPlain + 2 * (k - SO_Na_i) : kORDPlain + 8 + 2 * (k - SO_Ca_nsr);
}

// Tomek 2019: the reference block's states (Tomek.h:33-44) without A_h, B_h, A_j, B_j, which
// Calc recomputes from Vm every step before using them.
enum TOMState {
  SM_m, SM_h, SM_j, SM_h_p, SM_j_p, SM_m_L, SM_h_L, SM_h_L_CaMK, SM_a, SM_i_fast, SM_i_slow, SM_a_CaMK,
  SM_i_CaMK_fast, SM_i_CaMK_slow, SM_d, SM_f_fast, SM_f_slow, SM_f_Ca_fast, SM_f_Ca_slow, SM_j_Ca,
  SM_f_CaMK_fast, SM_f_Ca_CaMK_fast, SM_n_ss, SM_n_i, SM_C_0, SM_C_1, SM_C_2, SM_O, SM_I, SM_x_s1, SM_x_s2,
  SM_Na_i, SM_Na_ss, SM_K_i, SM_K_ss, SM_Ca_i, SM_Ca_ss, SM_Ca_nsr, SM_Ca_jsr, SM_Cl_i, SM_CaMK_trap, SM_J_rel_NP,
  SM_J_rel_CaMK, SM_Ca_TRPN, SM_N
};
// Diagnostic values of a Tomek FP64 batch: the 36 values Calc stores after the states
// (Tomek.h:47-52, block slots 48..83), then the rates A_h, B_h, A_j, B_j (block slots 1, 2, 4, 5).
constexpr int kTOMStored = 36;
constexpr int kTOMDiag = kTOMStored + 4;

// Tomek mixed form: planes 0..37 the FP32 states (TOMState order without the six compensated
// concentrations), planes 38..49 the (hi, lo) pairs of Na_i, Na_ss, K_i, K_ss, Ca_nsr, Ca_jsr.
constexpr int kTOMPlain = 38;
CM_HD int tom_mixed_plane(int k, bool &pair) {
  pair = false;
  if (k < SM_Na_i) return k;
  if (k == SM_Ca_i || k == SM_Ca_ss) return k - 4;
  if (k >= SM_Cl_i) return k - 6;
  pair = true;
  return k <= SM_K_ss ? kTOMPlain + 2 * (k - SM_Na_i) : kTOMPlain + 8 + 2 * (k - SM_Ca_nsr);
}

// Hetero (per-cell parameter) slots. Each slot either points at n_cells per-cell values
// or is null (the parameter set's value applies).
enum TT2Het { H2_g_Na, H2_g_Kr, H2_g_K1, H2_g_Ks, H2_g_to, H2_g_CaL, H2_N };
enum CRNHet { HC_g_Na, HC_g_to, HC_g_Ks, HC_g_CaL, HC_g_bNa, HC_g_bCa, HC_N };
enum ORDHet { HO_INaF, HO_INaL, HO_Ito, HO_IKr, HO_IKs, HO_IK1, HO_N };

// Constants of TenTusscherEtAl2::Calc (TenTusscher2.cpp:615-906) prepared on the host.
// Quantities the reference recomputes every call from parameters alone
// (sqrt(K_o/5.4), K_o/(K_o+KmK), Vc/Vss, ...) are evaluated once, in FP64.
template <typename R>
struct TT2Consts {
  R RTONF, K_o, Na_o, pKNa, pKNaNao, sqrtKo54, KoKmK, KmNa;
  R g_pCa, KpCa, g_to, g_Kr, g_Ks, g_K1, g_bNa, g_bCa, g_Na, g_CaL, kNaCa, knak;
  R CaiTabConst1, CaiTabConst2;
  R Cm, max_sr, min_sr, EC, ks1, ks2, k3, k4, Vrel, Vxfer, Vmaxup, Kupsquare;
  R Bufsr, Kbufsr, Bufss, Kbufss, Bufc, Kbufc, BufcPKbufc;
  R VcVss, VsrVss, inversevssF2, inverseviF, inverseviF2, invVcdVsr;
  R dt, dt1000, inv_stim_unit;  // inv_stim_unit = 1 / 2.29656e-2 (nA -> pA/pF, line 630)
  R logKo, logNao, logKoNao;    // log K_o, log Na_o, log(K_o + pKNa Na_o) (mixed form)
};

// Constants of Courtemanche::Calc (CourtemancheEtAl.cpp:85-187).
template <typename R>
struct CRNConsts {
  R RTdF, RTd2F, Na_o, K_o, Ca_o, g_Na, g_to, g_Ks, g_CaL, E_rL, g_bNa, g_bCa, k_mNai, I_pCamax,
      k_mpCa, k_rel, I_upmax, k_up, kupleak, dt_tr, G_sac, E_sac, K_sac, alpha, ISAC_SWITCH, Ca_T50,
      beta1, k_TRPN, n_TRPN, VreldVup, csqnkm, kmcsqnm2, kkmcsqn, CmdFvi, VupdVi, VreldVi, TRPNmax,
      cmdnkm, kmcmdnm2, kkmcmdn, Vrel, Cmd2F, exp250, exp50;
  R dt_ms;  // tinc * 1000 (line 87)
  R logNao, logKo, logCao;  // mixed form
};

// Constants of OHaraRudy::Calc (OHaraRudy.cpp:105-663) prepared on the host: every value
// that depends on parameters alone (F/RT, volume ratios, sqrt(K_o), the cell-type factors,
// products of multipliers) is evaluated once in FP64. The heterogeneity slots' multipliers
// (INaF, INaL, Ito, IKr, IKs, IK1) stay separate because they may be per cell.
template <typename R>
struct ORDConsts {
  R dt_ms;                                      // tinc * 1000 (line 106)
  R RToverF, FoRT, FFoRT, Na_o, K_o, Ca_o;      // F/(R T) and F^2/(R T)
  R util_1, util_2, util_3, vnsr_vmyo, vjsr_vss, vjsr_vnsr;
  R A_h_fast, A_h_slow, A_f_fast, A_f_slow, tau_h_L_mod, tau_h_L_CaMK;  // tau_h_L scaled by HF_Gomez_2
  R INaF, INaL, Ito, IKr, IKs, IK1;  // the multipliers a cell may replace
  R HF1, HF3, HF4, HF5, INaCa_HF6, INaK_HF7, IKb, INab, ICab, IpCa;
  R P_Ca, P_CaNa, P_CaK, P_Ca_CaMK, P_CaNa_CaMK, P_CaK_CaMK;
  R k_Na1, k_Na2, k_Ca_on, h_11, k_1, k_2, k_5, beta_1, alpha_2, alpha_4, MgATP1;  // MgATP1 = 1 + MgATP
  R alpha_rel, alpha_rel_CaMK, beta_tau, beta_tau_CaMK, rel_scale, HF8x15;  // rel_scale 1.7 for M cells; 1.5 HF8
  R up_scale, HF9, HF0, cmdnmax;                      // up_scale 1.3 epicardial; cmdnmax 0.05 (x1.3 epi)
  R epi;                                              // 1 for celltype 1 (delta_epi applies), else 0
  R sqrtKo54, sqrtKo, EKs_num, xK1_shift, xK1_slope, RK1_shift;  // K_o-only terms of I_Kr, I_Ks, I_K1
  R G_sac, E_sac, K_sac, alpha_sac, ISAC_SWITCH;
  R Ca_T50, beta1, HFM, k_TRPN, n_TRPN;
  R logNao, logKo, logEKs_num;  // mixed form
};

// Constants of Tomek::Calc (Tomek.cpp:110-656) prepared on the host, as ORDConsts. The
// outside activity coefficients depend on the bath alone (lines 271-279).
template <typename R>
struct TOMConsts {
  R dt_ms, RToverF, FoRT, FFoRT, RToF, Na_o, K_o, Ca_o, Cl_o;
  R util_1, util_2, util_3, vnsr_vmyo, vjsr_vss, vjsr_vnsr;
  R A_h, A_f_fast, A_f_slow, tau_h_L, tau_h_L_CaMK;
  R INaF, INaL, Ito, IKr, IKs, IK1;  // the multipliers a cell may replace
  R INaCa, INaK, IKb, INab, ICab, IpCa, PCa;  // PCa = IpCa_Multiplier * 8.3757e-5 (line 292)
  R k_Na1, k_Na2, k_Ca_on, h_11, k_1, k_2, k_5, beta_1, alpha_2, alpha_4, MgATP1;
  R alpha_rel, alpha_rel_CaMK, beta_tau, beta_tau_CaMK, rel_scale, up_scale, cmdnmax, epi;
  R sqrtKo5, EKs_num, constA, gamma_Ca_o, gamma_Na_o, gamma_K_o;
  R G_sac, E_sac, K_sac, alpha_sac, ISAC_SWITCH, Ca_T50, beta1, k_TRPN, n_TRPN;
};

// Voltage row index exactly as the reference computes it (TenTusscher2.cpp:618,
// CourtemancheEtAl.cpp:89), clamped to the table; out-of-table rows raise an audit bit
// instead of reading out of bounds.
CM_HD int vrow_fp64(double vmv, uint32_t &audit) {
  const double x = kDivision * (kRangeHalf + vmv) + .5;
  int vi = (x > -1.0 && x < 2147483647.0) ? (int)x : -1;  // (int) truncates toward 0
  if (vi < 0 || vi >= kRows || x != x) {
    audit |= 2u;
    vi = (x != x || vi < 0) ? 0 : kRows - 1;
  }
  return vi;
}

CM_HD int vrow_fp32(float vmv, uint32_t &audit) {
  const float x = kDivision * (kRangeHalf + vmv) + .5f;
  int vi = (x > -1.0f && x < 1.0e9f) ? (int)x : -1;
  if (vi < 0 || vi >= kRows || x != x) {
    audit |= 2u;
    vi = (x != x || vi < 0) ? 0 : kRows - 1;
  }
  return vi;
}

// FP32 helpers of the mixed form. On the device they map to the SFU (MUFU.EX2/LG2/RCP/RSQ)
// with one or two FMA-pipe instructions around them instead of the ~10-20 instruction
// IEEE-exact library sequences; their relative errors (~1e-7 .. 1e-6) are far below the
// mixed form's tolerance, which the parity tests check against the FP64 oracle.
CM_HD float fexp(float x) {
#ifdef __CUDA_ARCH__
  return __expf(x);
#else
  return expf(x);
#endif
}
CM_HD float flog(float x) {
#ifdef __CUDA_ARCH__
  return __logf(x);
#else
  return logf(x);
#endif
}
CM_HD float fdiv(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdividef(a, b);
#else
  return a / b;
#endif
}
CM_HD float fsqrt(float x) {
#ifdef __CUDA_ARCH__
  return x > 0.f ? x * rsqrtf(x) : 0.f;
#else
  return x > 0.f ? sqrtf(x) : 0.f;
#endif
}

// Compensated FP32 accumulator (value = hi + lo, |lo| <= ulp(hi)/2): about 48 significant
// bits with FP32-pipe instructions only. The mixed form keeps Vm, [Na]i, [K]i and [Ca]SR in
// it: their per-step increments are 1e-7..1e-9 of their values and would vanish in plain FP32,
// and GB300's FP64 pipe (1/64 of the FP32 rate) would bound the kernel if they were doubles.
struct Acc {
  float hi, lo;
};

// hi + lo += d with Knuth's two-sum (no magnitude precondition, so it also holds where Vm
// crosses zero) followed by a fast renormalisation.
CM_HD void acc_add(Acc &a, float d) {
  const float s = a.hi + d;
  const float bp = s - a.hi;
  const float e = (a.hi - (s - bp)) + (d - bp);
  const float t = a.lo + e;
  const float h = s + t;
  a.lo = t - (h - s);
  a.hi = h;
}

// Double <-> compensated pair. On the device the conversions are done on the bit patterns with
// integer instructions and selects, with no branch: on GB300 every FP64-pipe instruction,
// conversions included, issues at 2 per clock per SM (1/64 of the FP32 rate), so the four
// conversions and the subtraction of the plain form cost a kernel that reads FP64 Vm every step
// more than its memory traffic does (and a rare-case branch to the plain form is if-converted by
// the compiler into running it always). acc_from_double gives the plain form's pair (hi = x
// rounded to FP32, lo = the remainder rounded to FP32) for 2^-74 <= |x| < 2^128, except that a
// remainder of exactly half an FP32 ulp of x rounds hi away from zero instead of to even (the pair
// still sums to x); below that lo is 0 (|x| < 2^-74) and hi a signed zero (|x| < 2^-126); where
// hi rounds past the FP32 range it is infinite and lo 0; NaN stays NaN. acc_to_double widens both halves exactly and adds them once: the plain form's
// result.
CM_HD Acc acc_from_double(double x) {
#ifdef __CUDA_ARCH__
  const uint32_t hw = (uint32_t)__double2hiint(x), lw = (uint32_t)__double2loint(x);
  const uint32_t s = hw & 0x80000000u;
  const int E = (int)((hw >> 20) & 0x7ffu);  // biased FP64 exponent
  const uint32_t lr = lw + 0x10000000u;      // + half an ulp of the 24-bit significand
  const uint32_t hr = hw + (lr < lw ? 1u : 0u);
  const uint32_t er = (hr >> 20) & 0x7ffu;   // one more than E where the significand carried out
  uint32_t hi = s | ((er - 896u) << 23) | ((hr & 0xfffffu) << 3) | (lr >> 29);
  // the low 29 significand bits as a signed remainder in [-2^28, 2^28), in units of 2^(E-1075)
  int rem = ((int)((lw & 0x1fffffffu) << 3)) >> 3;
  rem = s ? -rem : rem;
  float lo = __int2float_rn(rem) * __uint_as_float((uint32_t)(E - 948) << 23);
  const bool inf_or_nan = E == 0x7ff, nan = inf_or_nan && ((hw & 0xfffffu) | lw);
  lo = (E >= 949 && er <= 1150u) ? lo : 0.f;
  hi = E < 897 ? s : hi;
  hi = er > 1150u || inf_or_nan ? (s | 0x7f800000u) : hi;
  hi = nan ? (s | 0x7fc00000u) : hi;
  return Acc{__uint_as_float(hi), lo};
#else
  Acc a;
  a.hi = (float)x;
  a.lo = (float)(x - (double)a.hi);
  return a;
#endif
}

// FP32 -> FP64 widening on the bit pattern (exact, zero, subnormal, inf and NaN included).
CM_HD double f32_widen(float f) {
#ifdef __CUDA_ARCH__
  const uint32_t u = __float_as_uint(f), e = (u >> 23) & 0xffu, s = u & 0x80000000u, m = u & 0x7fffffu;
  uint32_t h = s | ((e + 896u) << 20) | (m >> 3), l = m << 29;  // normal: exponent + 1023 - 127
  // subnormal: m 2^-149 = 2^(p-149) (1 + fraction), p = the index of m's leading one
  const int p = 31 - __clz(m | 1u);
  const uint32_t fs = (m << (23 - p)) & 0x7fffffu;
  const uint32_t hs = s | ((uint32_t)(p + 874) << 20) | (fs >> 3), ls = fs << 29;
  h = e == 255u ? (s | 0x7ff00000u | (m >> 3)) : h;
  h = e == 0u ? (m ? hs : s) : h;
  l = e == 0u ? (m ? ls : 0u) : l;
  return __hiloint2double((int)h, (int)l);
#else
  return (double)f;
#endif
}

CM_HD double acc_to_double(Acc a) { return f32_widen(a.hi) + f32_widen(a.lo); }

// a >= b for non-NaN doubles, on the bit patterns (no FP64 instruction): the sign-magnitude
// patterns mapped to a two's-complement order; +0 and -0 compare equal.
CM_HD bool f64_ge(double a, double b) {
#ifdef __CUDA_ARCH__
  long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
  if (((ia | ib) & 0x7fffffffffffffffll) == 0) return true;
  ia ^= (ia >> 63) & 0x7fffffffffffffffll;
  ib ^= (ib >> 63) & 0x7fffffffffffffffll;
  return ia >= ib;
#else
  return a >= b;
#endif
}

// New free concentration increment of a rapidly buffered species. The reference solves
// x^2 + b x - c = 0 for the new free value x given total = x_old + B x_old/(x_old+K) + dT
// (TenTusscher2.cpp:814-836). Writing x = x_old + d, the same conservation law gives
//   a d^2 + (a^2 + B K - dT a) d - dT a^2 = 0,  a = x_old + K,
// whose root is taken in the form without cancellation. Used by the mixed form in FP32,
// where the reference form loses most digits of d (sqrt(b^2+4c) - b with b >> d).
CM_HD float buffered_increment(float x, float dT, float B, float K) {
  const float a = x + K;
  const float Bq = a * a + B * K - dT * a;
  const float s = fsqrt(Bq * Bq + 4.f * a * a * a * dT);
  return Bq > 0.f ? fdiv(2.f * dT * a * a, Bq + s) : fdiv(s - Bq, 2.f * a);
}

}  // namespace cm
