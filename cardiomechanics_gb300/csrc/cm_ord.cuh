// O'Hara-Rudy 2011 human ventricular model as the reference compiles it (OHaraRudy.cpp:105-663
// with ISAC, TRPN, HF, HFM, DUTTA and PASSINI defined, OHaraRudyParameters.h:20-36): Passini
// steady states and Dutta time constants for the I_Na gates, troponin buffering of Land et
// al., a stretch-activated current, the Gomez heart-failure factors. The reference evaluates
// every gate from its closed form each step (no lookup tables), so this does too.
//
// One template serves both precisions. R = double is the FP64 form (the reference's
// arithmetic; differences to it are a few ulp: parameter-only constants taken once on the
// host, divisions by literals as multiplications by their reciprocals, cubes and squares as
// products instead of pow, the currents summed in running totals). R = float is the mixed
// form: FP32 gates and currents on the SFU, and the six concentrations whose per-step
// increments are below FP32 resolution kept in compensated accumulators by the state store.
#pragma once

#include "cm_common.cuh"

namespace cm {

template <typename R>
struct ORDHet_ {
  R INaF, INaL, Ito, IKr, IKs, IK1;
};

// FP32 exp and reciprocal straight on the SFU (MUFU.EX2 / MUFU.RCP) with flush-to-zero, so
// each costs one FMUL plus one MUFU and no denormal fix-up: exp(x) = 2^(x log2 e), relative
// error about 1e-7 (1 + |x|); a / b = a * (1/b). Results that would be denormal are 0, which
// no quantity of this model needs.
CM_HD double o_exp(double x) { return exp(x); }
CM_HD float o_exp(float x) {
#ifdef __CUDA_ARCH__
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x * 1.44269504088896341f));
  return y;
#else
  return expf(x);
#endif
}
CM_HD double o_log(double x) { return log(x); }
CM_HD float o_log(float x) { return flog(x); }
CM_HD double o_div(double a, double b) { return a / b; }
CM_HD float o_div(float a, float b) {
#ifdef __CUDA_ARCH__
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
  return a * r;
#else
  return a / b;
#endif
}
// Division by a literal written as multiplication by its reciprocal, folded at compile time
// (one rounding more than the reference's division; a few ulp at most in FP64).
template <typename R>
CM_HD constexpr R rc(double c) {
  return R(1.0 / c);
}
CM_HD double o_pow(double a, double b) { return pow(a, b); }
CM_HD float o_pow(float a, float b) { return a > 0.f ? o_exp(b * flog(a)) : (b == 0.f ? 1.f : 0.f); }
// exp(z) - 1: in FP32 a short Taylor polynomial where exp(z) - 1 would cancel (|z| < 1e-2,
// truncation below 4e-9 relative), so the GHK flux terms stay accurate as Vm crosses 0.
CM_HD double o_expm1(double z) { return exp(z) - 1.0; }
CM_HD float o_expm1(float z) {
  return fabsf(z) < 1e-2f ? z * (1.f + z * (0.5f + z * (1.f / 6.f + z * (1.f / 24.f)))) : o_exp(z) - 1.f;
}

// Gate update of the reference: x = x_inf - (x_inf - x) exp(-tinc / tau). In FP32 the same
// update is taken as x - (x_inf - x) expm1(-tinc / tau): for the slow gates (tau up to 1 s,
// exp(-tinc/tau) = 0.99999) the rounding of exp near 1 would otherwise bias every step's
// increment by ~1 %, which accumulates over a beat.
CM_HD double o_gate(double inf, double x, double tinc, double tau) { return inf - (inf - x) * exp(-tinc / tau); }
CM_HD float o_gate(float inf, float x, float tinc, float tau) { return x - (inf - x) * o_expm1(o_div(-tinc, tau)); }

template <typename R>
CM_HD R o_sig(R z) {  // 1 / (1 + exp(z))
  return o_div(R(1), R(1) + o_exp(z));
}

// One Calc of one cell. The state store S is the cell's view of its batch:
//   void fetch(int part)       part 1: the store may read its remaining inputs now (before I_CaL)
//   R get(int k)               state k (ORDState order) as this step reads it
//   void set(int k, R v)       new value of a plain state, stored as soon as it is final
//   void add(int k, R x, R d)  x + d for Na_i, Na_ss, K_i, K_ss, Ca_nsr, Ca_jsr (x = get(k))
//   void cur(int k, R v)       current k of the reference block (diagnostics; may do nothing)
// Writing each state back as soon as it is final and summing the currents as they appear keeps
// the live set small. Returns dV [V]; V [V]; stretch as the reference's Calc argument.
template <typename R, typename S>
CM_HD R ord_calc(const ORDConsts<R> &C, S &x, const ORDHet_<R> &g, R V, R i_external, R stretch) {
  const R tinc = C.dt_ms;
  const R V_m = V * R(1000);
  const R Na_i = x.get(SO_Na_i), K_i = x.get(SO_K_i), Ca_ss = x.get(SO_Ca_ss);
  R I_sum = i_external;  // all currents + i_external (525-532)
  R s_Nai, s_Ki;         // cur_Nai (595), cur_Ki (601) without i_external

  // CaMK (115-131): the old trapped fraction sets this step's activity
  const R CaMK_trap = x.get(SO_CaMK_trap);
  const R CaMK_bound = R(0.05) * o_div(R(1) - CaMK_trap, R(1) + o_div(R(0.0015), Ca_ss));
  x.set(SO_CaMK_trap,
        CaMK_trap + tinc * (R(0.05) * CaMK_bound * (CaMK_bound + CaMK_trap) - R(0.00068) * CaMK_trap));
  const R phi = o_div(R(1), R(1) + o_div(R(0.15), (CaMK_bound + CaMK_trap) * C.HF1));

  // reversal potentials (133-138)
  const R E_Na = C.RToverF * o_log(o_div(C.Na_o, Na_i));
  const R E_K = C.RToverF * o_log(o_div(C.K_o, K_i));
  const R VFoverRT = V_m * C.FoRT;
  const R VFFoverRT = V_m * C.FFoRT;

  // I_Na (146-202)
  const R tau_m = o_div(R(1), R(6.765) * o_exp((V_m + R(11.64)) * rc<R>(34.77)) +
                                   R(8.552) * o_exp(-(V_m + R(77.42)) * rc<R>(5.955)));
  {
    const R m = o_gate(o_sig(-(V_m + R(39.57)) * rc<R>(9.871)), x.get(SO_m), tinc, tau_m);
    x.set(SO_m, m);
    const R h_inf = o_sig((V_m + R(78.5)) * rc<R>(6.22));
    const R tau_h_fast = o_div(R(1), R(3.686e-6) * o_exp(-(V_m + R(3.8875)) * rc<R>(7.8579)) +
                                          R(16.0) * o_exp((V_m - R(0.4963)) * rc<R>(9.1843)));
    const R tau_h_slow = o_div(R(1), R(0.009794) * o_exp(-(V_m + R(17.95)) * rc<R>(28.05)) +
                                          R(0.3343) * o_exp((V_m + R(5.730)) * rc<R>(56.66)));
    const R h_fast = o_gate(h_inf, x.get(SO_h_fast), tinc, tau_h_fast);
    x.set(SO_h_fast, h_fast);
    const R h_slow = o_gate(h_inf, x.get(SO_h_slow), tinc, tau_h_slow);
    x.set(SO_h_slow, h_slow);
    const R tau_j = R(4.8590) + o_div(R(1), R(0.8628) * o_exp(-(V_m + R(116.7258)) * rc<R>(7.6005)) +
                                                 R(1.1096) * o_exp((V_m + R(6.2719)) * rc<R>(9.0358)));
    const R j = o_gate(h_inf, x.get(SO_j), tinc, tau_j);
    x.set(SO_j, j);
    const R h_CaMK_slow =
        o_gate(o_sig((V_m + R(84.7)) * rc<R>(6.22)), x.get(SO_h_CaMK_slow), tinc, R(3) * tau_h_slow);
    x.set(SO_h_CaMK_slow, h_CaMK_slow);
    const R j_CaMK = o_gate(h_inf, x.get(SO_j_CaMK), tinc, R(1.46) * tau_j);
    x.set(SO_j_CaMK, j_CaMK);
    const R h = C.A_h_fast * h_fast + C.A_h_slow * h_slow;
    const R h_CaMK = C.A_h_fast * h_fast + C.A_h_slow * h_CaMK_slow;
    const R I_Na_fast =
        g.INaF * R(75.0) * (V_m - E_Na) * m * m * m * ((R(1) - phi) * h * j + phi * h_CaMK * j_CaMK);
    x.cur(0, I_Na_fast);
    I_sum += I_Na_fast;
    s_Nai = I_Na_fast;
  }

  // I_NaL (204-224)
  {
    const R m_L = o_gate(o_sig(-(V_m + R(42.85)) * rc<R>(5.264)), x.get(SO_m_L), tinc, tau_m);
    x.set(SO_m_L, m_L);
    const R h_L = o_gate(o_sig((V_m + R(87.61)) * rc<R>(7.488)), x.get(SO_h_L), tinc, C.tau_h_L_mod);
    x.set(SO_h_L, h_L);
    const R h_L_CaMK = o_gate(o_sig((V_m + R(93.81)) * rc<R>(7.488)), x.get(SO_h_L_CaMK), tinc, C.tau_h_L_CaMK);
    x.set(SO_h_L_CaMK, h_L_CaMK);
    const R I_Na_late = g.INaL * C.HF3 * R(0.0075) * (V_m - E_Na) * m_L * ((R(1) - phi) * h_L + phi * h_L_CaMK);
    x.cur(1, I_Na_late);
    I_sum += I_Na_late;
    s_Nai += I_Na_late;
  }

  // I_to (226-262); delta_epi only for epicardial cells
  {
    const R tau_a =
        o_div(R(1.0515), o_div(R(1), R(1.2089) * (R(1) + o_exp(-(V_m - R(18.4099)) * rc<R>(29.3814)))) +
                             o_div(R(3.5), R(1) + o_exp((V_m + R(100.0)) * rc<R>(29.3814))));
    const R a = o_gate(o_sig(-(V_m - R(14.34)) * rc<R>(14.82)), x.get(SO_a), tinc, tau_a);
    x.set(SO_a, a);
    const R a_CaMK = o_gate(o_sig(-(V_m - R(24.34)) * rc<R>(14.82)), x.get(SO_a_CaMK), tinc, tau_a);
    x.set(SO_a_CaMK, a_CaMK);
    const R i_inf = o_sig((V_m + R(43.94)) * rc<R>(5.711));
    const R delta_epi = C.epi != R(0) ? R(1) - R(0.95) * o_sig((V_m + R(70.0)) * rc<R>(5.0)) : R(1);
    const R tau_i_fast = (R(4.562) + o_div(R(1), R(0.3933) * o_exp(-(V_m + R(100.0)) * rc<R>(100.0)) +
                                                   R(0.08004) * o_exp((V_m + R(50.0)) * rc<R>(16.59)))) *
                         delta_epi;
    const R tau_i_slow = (R(23.62) + o_div(R(1), R(0.001416) * o_exp(-(V_m + R(96.52)) * rc<R>(59.05)) +
                                                   R(1.7808e-08) * o_exp((V_m + R(114.1)) * rc<R>(8.079)))) *
                         delta_epi;
    const R i_fast = o_gate(i_inf, x.get(SO_i_fast), tinc, tau_i_fast);
    x.set(SO_i_fast, i_fast);
    const R i_slow = o_gate(i_inf, x.get(SO_i_slow), tinc, tau_i_slow);
    x.set(SO_i_slow, i_slow);
    const R dev =
        R(1.354) + o_div(R(1.0e-04), o_exp((V_m - R(167.4)) * rc<R>(15.89)) + o_exp(-(V_m - R(12.23)) * rc<R>(0.2154)));
    const R rec = R(1) - R(0.5) * o_sig((V_m + R(70.0)) * rc<R>(20.0));
    const R i_CaMK_fast = o_gate(i_inf, x.get(SO_i_CaMK_fast), tinc, tau_i_fast * dev * rec);
    x.set(SO_i_CaMK_fast, i_CaMK_fast);
    const R i_CaMK_slow = o_gate(i_inf, x.get(SO_i_CaMK_slow), tinc, tau_i_slow * dev * rec);
    x.set(SO_i_CaMK_slow, i_CaMK_slow);
    const R A_i_fast = o_sig((V_m - R(213.6)) * rc<R>(151.2));
    const R A_i_slow = R(1) - A_i_fast;
    const R i = A_i_fast * i_fast + A_i_slow * i_slow;
    const R i_CaMK = A_i_fast * i_CaMK_fast + A_i_slow * i_CaMK_slow;
    const R I_to = g.Ito * C.HF4 * R(0.02) * (V_m - E_K) * ((R(1) - phi) * a * i + phi * a_CaMK * i_CaMK);
    x.cur(2, I_to);
    I_sum += I_to;
    s_Ki = I_to;
  }

  // I_CaL, I_CaNa, I_CaK (264-329)
  x.fetch(1);
  const R em1_Ca = o_expm1(R(2) * VFoverRT), em1_1 = o_expm1(VFoverRT);
  const R exp_z_Ca = em1_Ca + R(1), exp_z_1 = em1_1 + R(1);
  R I_CaL, s_Nass, s_Kss;
  {
    const R tau_d = R(0.6) + o_div(R(1), o_exp(R(-0.05) * (V_m + R(6.0))) + o_exp(R(0.09) * (V_m + R(14.0))));
    const R d = o_gate(o_sig(-(V_m + R(3.940)) * rc<R>(4.230)), x.get(SO_d), tinc, tau_d);
    x.set(SO_d, d);
    const R f_inf = o_sig((V_m + R(19.58)) * rc<R>(3.696));
    const R tau_f_fast = R(7.0) + o_div(R(1), R(0.0045) * o_exp(-(V_m + R(20.0)) * rc<R>(10.0)) +
                                                 R(0.0045) * o_exp((V_m + R(20.0)) * rc<R>(10.0)));
    const R tau_f_slow = R(1000.0) + o_div(R(1), R(3.5e-05) * o_exp(-(V_m + R(5.0)) * rc<R>(4.0)) +
                                                    R(3.5e-05) * o_exp((V_m + R(5.0)) * rc<R>(6.0)));
    const R f_fast = o_gate(f_inf, x.get(SO_f_fast), tinc, tau_f_fast);
    x.set(SO_f_fast, f_fast);
    const R f_slow = o_gate(f_inf, x.get(SO_f_slow), tinc, tau_f_slow);
    x.set(SO_f_slow, f_slow);
    const R tau_f_Ca_fast = R(7.0) + o_div(R(1), R(0.04) * o_exp(-(V_m - R(4.0)) * rc<R>(7.0)) +
                                                    R(0.04) * o_exp((V_m - R(4.0)) * rc<R>(7.0)));
    const R tau_f_Ca_slow =
        R(100.0) + o_div(R(1), R(0.00012) * o_exp(-V_m * rc<R>(3.0)) + R(0.00012) * o_exp(V_m * rc<R>(7.0)));
    const R f_Ca_fast = o_gate(f_inf, x.get(SO_f_Ca_fast), tinc, tau_f_Ca_fast);
    x.set(SO_f_Ca_fast, f_Ca_fast);
    const R f_Ca_slow = o_gate(f_inf, x.get(SO_f_Ca_slow), tinc, tau_f_Ca_slow);
    x.set(SO_f_Ca_slow, f_Ca_slow);
    const R j_Ca = o_gate(f_inf, x.get(SO_j_Ca), tinc, R(75.0));
    x.set(SO_j_Ca, j_Ca);
    const R f_CaMK_fast = o_gate(f_inf, x.get(SO_f_CaMK_fast), tinc, R(2.5) * tau_f_fast);
    x.set(SO_f_CaMK_fast, f_CaMK_fast);
    const R f_Ca_CaMK_fast = o_gate(f_inf, x.get(SO_f_Ca_CaMK_fast), tinc, R(2.5) * tau_f_Ca_fast);
    x.set(SO_f_Ca_CaMK_fast, f_Ca_CaMK_fast);
    const R A_f_Ca_fast = R(0.3) + R(0.6) * o_sig((V_m - R(10.0)) * rc<R>(10.0));
    const R A_f_Ca_slow = R(1) - A_f_Ca_fast;
    const R f = C.A_f_fast * f_fast + C.A_f_slow * f_slow;
    const R f_Ca = A_f_Ca_fast * f_Ca_fast + A_f_Ca_slow * f_Ca_slow;
    const R f_CaMK = C.A_f_fast * f_CaMK_fast + C.A_f_slow * f_slow;
    const R f_Ca_CaMK = A_f_Ca_fast * f_Ca_CaMK_fast + A_f_Ca_slow * f_Ca_slow;
    // n: the reference's alpha_n (k2n / k_m2_n) - (alpha_n (k2n / k_m2_n) - n) exp(-k_m2_n tinc),
    // k_m2_n = j_Ca, with alpha_n (k2n / k_m2_n) taken as one quotient
    const R k2n_km2n = o_div(R(1000.0), j_Ca);
    const R q = R(1) + o_div(R(0.002), Ca_ss);
    const R n_inf = o_div(k2n_km2n, k2n_km2n + (q * q) * (q * q));
    const R n = n_inf - (n_inf - x.get(SO_n)) * o_exp(-j_Ca * tinc);
    x.set(SO_n, n);
    const R Psi_Ca = R(4) * VFFoverRT * o_div(Ca_ss * exp_z_Ca - R(0.341) * C.Ca_o, em1_Ca);
    const R Psi_CaNa = VFFoverRT * o_div(R(0.75) * x.get(SO_Na_ss) * exp_z_1 - R(0.75) * C.Na_o, em1_1);
    const R Psi_CaK = VFFoverRT * o_div(R(0.75) * x.get(SO_K_ss) * exp_z_1 - R(0.75) * C.K_o, em1_1);
    const R gate_np = d * (R(1) - phi) * (f * (R(1) - n) + f_Ca * n * j_Ca);
    const R gate_camk = d * phi * (f_CaMK * (R(1) - n) + f_Ca_CaMK * n * j_Ca);
    I_CaL = C.P_Ca * Psi_Ca * gate_np + C.P_Ca_CaMK * Psi_Ca * gate_camk;
    const R I_CaNa = C.P_CaNa * Psi_CaNa * gate_np + C.P_CaNa_CaMK * Psi_CaNa * gate_camk;
    const R I_CaK = C.P_CaK * Psi_CaK * gate_np + C.P_CaK_CaMK * Psi_CaK * gate_camk;
    x.cur(3, I_CaL);
    x.cur(4, I_CaNa);
    x.cur(5, I_CaK);
    I_sum += I_CaL + I_CaNa + I_CaK;
    s_Nass = I_CaNa;
    s_Kss = I_CaK;
  }

  // I_Kr, I_Ks, I_K1 (331-367)
  {
    const R x_r_inf = o_sig(-(V_m + R(8.337)) * rc<R>(6.789));
    const R tau_x_r_fast = R(12.98) + o_div(R(1), R(0.3652) * o_exp((V_m - R(31.66)) * rc<R>(3.869)) +
                                                      R(4.123e-05) * o_exp(-(V_m - R(47.78)) * rc<R>(20.38)));
    const R tau_x_r_slow = R(1.865) + o_div(R(1), R(0.06629) * o_exp((V_m - R(34.7)) * rc<R>(7.355)) +
                                                      R(1.128e-05) * o_exp(-(V_m - R(29.74)) * rc<R>(25.94)));
    const R x_r_fast = o_gate(x_r_inf, x.get(SO_x_r_fast), tinc, tau_x_r_fast);
    x.set(SO_x_r_fast, x_r_fast);
    const R x_r_slow = o_gate(x_r_inf, x.get(SO_x_r_slow), tinc, tau_x_r_slow);
    x.set(SO_x_r_slow, x_r_slow);
    const R A_x_r_fast = o_sig((V_m + R(54.81)) * rc<R>(38.21));
    const R x_r = A_x_r_fast * x_r_fast + (R(1) - A_x_r_fast) * x_r_slow;
    const R R_Kr =
        o_div(R(1), (R(1) + o_exp((V_m + R(55.0)) * rc<R>(75.0))) * (R(1) + o_exp((V_m - R(10.0)) * rc<R>(30.0))));
    const R I_Kr = g.IKr * R(0.046) * C.sqrtKo54 * x_r * (V_m - E_K) * R_Kr;
    x.cur(6, I_Kr);

    const R x_s1_inf = o_sig(-(V_m + R(11.6)) * rc<R>(8.932));
    const R tau_x_s1 = R(817.3) + o_div(R(1), R(2.326e-04) * o_exp((V_m + R(48.28)) * rc<R>(17.80)) +
                                                  R(0.001292) * o_exp(-(V_m + R(210.0)) * rc<R>(230.0)));
    const R x_s1 = o_gate(x_s1_inf, x.get(SO_x_s1), tinc, tau_x_s1);
    x.set(SO_x_s1, x_s1);
    const R tau_x_s2 = o_div(R(1), R(0.01) * o_exp((V_m - R(50.0)) * rc<R>(20.0)) +
                                        R(0.0193) * o_exp(-(V_m + R(66.54)) * rc<R>(31.0)));
    const R x_s2 = o_gate(x_s1_inf, x.get(SO_x_s2), tinc, tau_x_s2);
    x.set(SO_x_s2, x_s2);
    const R E_Ks = C.RToverF * o_log(o_div(C.EKs_num, K_i + R(0.01833) * Na_i));
    const R Ca_i = x.get(SO_Ca_i);
    const R I_Ks = g.IKs * R(0.0034) * (R(1) + o_div(R(0.6), R(1) + o_pow(o_div(R(3.8e-05), Ca_i), R(1.4)))) *
                   x_s1 * x_s2 * (V_m - E_Ks);
    x.cur(7, I_Ks);

    const R x_K1_inf = o_sig(o_div(-(V_m + C.xK1_shift), C.xK1_slope));
    const R tau_x_K1 =
        o_div(R(122.2), o_exp(-(V_m + R(127.2)) * rc<R>(20.36)) + o_exp((V_m + R(236.8)) * rc<R>(69.33)));
    const R x_K1 = o_gate(x_K1_inf, x.get(SO_x_K1), tinc, tau_x_K1);
    x.set(SO_x_K1, x_K1);
    const R R_K1 = o_sig((V_m + C.RK1_shift) * rc<R>(9.493));
    const R I_K1 = g.IK1 * C.HF5 * R(0.1908) * C.sqrtKo * x_K1 * (V_m - E_K) * R_K1;
    x.cur(8, I_K1);
    I_sum += I_Kr + I_Ks + I_K1;
    s_Ki += I_Kr + I_Ks + I_K1;
  }

  // I_NaCa_i and I_NaCa_ss (369-443): the exchanger cycle's four-state steady state on the
  // myoplasm (s = 0) and subspace (s = 1) sides
  R I_NaCa_i, I_NaCa_ss;
  {
    const R kna3 = R(88.12), wna = R(6.0e4), wca = R(6.0e4), wnaca = R(5.0e3);
    const R h_Ca = o_exp(R(0.1670) * VFoverRT);
    const R h_Na = o_exp(R(0.5224) * VFoverRT);
    const R h_7 = R(1) + C.Na_o * (R(1) + o_div(R(1), h_Na)) * rc<R>(88.12);
    const R h_8 = o_div(C.Na_o, kna3 * h_Na * h_7);
    const R k_3_dd = h_8 * wnaca;
    const R k_3 = o_div(wca, h_7) + k_3_dd;
    const R k_8 = h_8 * C.h_11 * wna;
    const R k_1 = C.k_1, k_2 = C.k_2, k_5 = C.k_5;
    R I_NaCa[2];
#pragma unroll
    for (int s = 0; s < 2; s++) {
      const R na = s == 0 ? Na_i : x.get(SO_Na_ss);
      const R ca = s == 0 ? x.get(SO_Ca_i) : Ca_ss;
      const R h_1 = R(1) + na * (R(1) + h_Na) * rc<R>(88.12);
      const R h_2 = o_div(na * h_Na, kna3 * h_1);
      const R h_4 = R(1) + na * (R(1) + o_div(na, C.k_Na2)) * o_div(R(1), C.k_Na1);
      const R h_5 = o_div(na * na, h_4 * C.k_Na1 * C.k_Na2);
      const R k_4_dd = h_2 * wnaca;
      const R k_4 = o_div(wca, h_1 * h_Ca) + k_4_dd;
      const R k_6 = o_div(ca * C.k_Ca_on, h_4);
      const R k_7 = h_5 * h_2 * wna;
      const R x_1 = k_2 * k_4 * (k_7 + k_6) + k_5 * k_7 * (k_2 + k_3);
      const R x_2 = k_1 * k_7 * (k_4 + k_5) + k_4 * k_6 * (k_1 + k_8);
      const R x_3 = k_1 * k_3 * (k_7 + k_6) + k_8 * k_6 * (k_2 + k_3);
      const R x_4 = k_2 * k_8 * (k_4 + k_5) + k_3 * k_5 * (k_1 + k_8);
      const R inv = o_div(R(1), x_1 + x_2 + x_3 + x_4);
      const R J_Na = (R(3) * (x_4 * k_7 - x_1 * k_8) + x_3 * k_4_dd - x_2 * k_3_dd) * inv;
      const R J_Ca = (x_2 * k_2 - x_1 * k_1) * inv;
      const R ka = o_div(R(150.0e-6), ca);
      // G_NaCa 0.0008 x 0.8 (myoplasm) or x 0.2 (subspace), allosteric Ca activation
      I_NaCa[s] = C.INaCa_HF6 * (s == 0 ? R(0.0008 * 0.8) : R(0.0008 * 0.2)) * o_div(R(1), R(1) + ka * ka) *
                  (J_Na + R(2) * J_Ca);
    }
    I_NaCa_i = I_NaCa[0];
    I_NaCa_ss = I_NaCa[1];
    x.cur(9, I_NaCa_i);
    x.cur(10, I_NaCa_ss);
    I_sum += I_NaCa_i + I_NaCa_ss;
    s_Nai += R(3) * I_NaCa_i;
    s_Nass += R(3) * I_NaCa_ss;
  }

  // I_NaK (445-498): the pump cycle's four-state steady state
  {
    const R K_Nai = R(9.073) * o_exp(R(-0.1550) * VFoverRT * rc<R>(3));
    const R K_Nao = R(27.78) * o_exp(R(1.1550) * VFoverRT * rc<R>(3));
    const R Pnak = o_div(R(4.2), R(1) + R(1.0e-7 / 1.698e-7) + Na_i * rc<R>(224.0) + K_i * rc<R>(292.0));
    const R ni = o_div(Na_i, K_Nai), no = o_div(C.Na_o, K_Nao), ki = K_i * R(2), ko = C.K_o * rc<R>(0.3582);
    const R den_i = (R(1) + ni) * (R(1) + ni) * (R(1) + ni) + (R(1) + ki) * (R(1) + ki) - R(1);
    const R den_o = (R(1) + no) * (R(1) + no) * (R(1) + no) + (R(1) + ko) * (R(1) + ko) - R(1);
    const R rdi = o_div(R(1), den_i), rdo = o_div(R(1), den_o);
    const R alpha_1 = R(949.5) * ni * ni * ni * rdi;
    const R beta_2 = R(39.4) * no * no * no * rdo;
    const R alpha_3 = R(1899.0) * ko * ko * rdo;
    const R beta_3 = o_div(R(79300.0) * Pnak * R(1.0e-7), C.MgATP1);
    const R beta_4 = R(40.0) * ki * ki * rdi;
    const R al2 = C.alpha_2, al4 = C.alpha_4, be1 = C.beta_1;
    const R x_1 = al4 * alpha_1 * al2 + beta_2 * beta_4 * beta_3 + al2 * beta_4 * beta_3 + beta_3 * alpha_1 * al2;
    const R x_2 = beta_2 * be1 * beta_4 + alpha_1 * al2 * alpha_3 + alpha_3 * be1 * beta_4 + al2 * alpha_3 * beta_4;
    const R x_3 = al2 * alpha_3 * al4 + beta_3 * beta_2 * be1 + beta_2 * be1 * al4 + alpha_3 * al4 * be1;
    const R x_4 = beta_4 * beta_3 * beta_2 + alpha_3 * al4 * alpha_1 + beta_2 * al4 * alpha_1 + beta_3 * beta_2 * alpha_1;
    const R inv = o_div(R(1), x_1 + x_2 + x_3 + x_4);
    const R J_NaK_Na = R(3) * (x_1 * alpha_3 - x_2 * beta_3) * inv;
    const R J_NaK_K = R(2) * (x_4 * be1 - x_3 * alpha_1) * inv;
    const R I_NaK = C.INaK_HF7 * R(30.0) * (J_NaK_Na + J_NaK_K);
    x.cur(11, I_NaK);
    I_sum += I_NaK;
    s_Nai += R(3) * I_NaK;
    s_Ki -= R(2) * I_NaK;
  }

  // background currents, I_pCa, I_SAC (500-523)
  const R Ca_i = x.get(SO_Ca_i);
  R s_Cai;
  {
    const R I_Nab = C.INab * R(3.75e-10) * VFFoverRT * o_div(Na_i * exp_z_1 - C.Na_o, em1_1);
    const R I_Cab = C.ICab * R(2.5e-8) * R(4) * VFFoverRT * o_div(Ca_i * exp_z_Ca - R(0.341) * C.Ca_o, em1_Ca);
    const R I_Kb = C.IKb * R(0.003) * o_sig(-(V_m - R(14.48)) * rc<R>(18.34)) * (V_m - E_K);
    const R I_pCa = C.IpCa * R(0.0005) * o_div(Ca_i, R(0.0005) + Ca_i);
    const R I_SAC =
        C.ISAC_SWITCH * o_div(C.G_sac * (V_m - C.E_sac), R(1) + C.K_sac * o_exp(-C.alpha_sac * (stretch - R(1))));
    x.cur(12, I_Nab);
    x.cur(13, I_Cab);
    x.cur(14, I_Kb);
    x.cur(15, I_pCa);
    x.cur(16, I_SAC);
    I_sum += I_Nab + I_Cab + I_Kb + I_pCa + I_SAC;
    s_Nai += I_Nab;
    s_Ki += I_Kb + i_external;
    s_Cai = I_pCa + I_Cab - R(2) * I_NaCa_i;
  }

  // SR release and uptake (535-592); M cells release 1.7x, epicardial cells take up 1.3x
  const R Na_ss = x.get(SO_Na_ss), K_ss = x.get(SO_K_ss), Ca_nsr = x.get(SO_Ca_nsr), Ca_jsr = x.get(SO_Ca_jsr);
  const R cj = C.HF8x15 * o_div(R(1), Ca_jsr), cj2 = cj * cj, cj4 = cj2 * cj2;
  const R rel_inf = o_div(-I_CaL * C.rel_scale, R(1) + cj4 * cj4);
  const R tau_rel_b = o_div(R(1), R(1) + R(0.0123) * o_div(R(1), Ca_jsr));
  const R tau_NP = C.beta_tau * tau_rel_b, tau_CaMK = C.beta_tau_CaMK * tau_rel_b;
  const R J_rel_NP =
      o_gate(C.alpha_rel * rel_inf, x.get(SO_J_rel_NP), tinc, tau_NP < R(0.001) ? R(0.001) : tau_NP);
  x.set(SO_J_rel_NP, J_rel_NP);
  const R J_rel_CaMK =
      o_gate(C.alpha_rel_CaMK * rel_inf, x.get(SO_J_rel_CaMK), tinc, tau_CaMK < R(0.001) ? R(0.001) : tau_CaMK);
  x.set(SO_J_rel_CaMK, J_rel_CaMK);
  const R J_rel = (R(1) - phi) * J_rel_NP + phi * J_rel_CaMK;
  const R J_up_NP = o_div(R(0.004375) * Ca_i, R(0.00092) + Ca_i) * C.up_scale;
  const R J_up_CaMK = o_div(R(2.75) * (R(0.004375) * Ca_i), R(0.00092) - R(0.00017) + Ca_i) * C.up_scale;
  const R J_leak = C.HF9 * (R(0.0039375) * Ca_nsr) * rc<R>(15.0);
  const R J_up = C.HF0 * ((R(1) - phi) * J_up_NP + phi * J_up_CaMK - J_leak);
  const R J_tr = (Ca_nsr - Ca_jsr) * R(0.01);
  const R J_diff_Na = (Na_ss - Na_i) * R(0.5);
  const R J_diff_Ca = (Ca_ss - Ca_i) * R(5);
  const R J_diff_K = (K_ss - K_i) * R(0.5);

  // concentrations (594-660)
  x.add(SO_Na_i, Na_i, tinc * (-s_Nai * C.util_1 + J_diff_Na * C.util_2));
  x.add(SO_Na_ss, Na_ss, tinc * (-s_Nass * C.util_3 - J_diff_Na));
  x.add(SO_K_i, K_i, tinc * (-s_Ki * C.util_1 + J_diff_K * C.util_2));
  x.add(SO_K_ss, K_ss, tinc * (-(s_Kss * C.util_3) - J_diff_K));
  const R Ca_T50 = (C.Ca_T50 + C.beta1 * ((stretch < R(1.2) ? stretch : R(1.2)) - R(1))) * C.HFM;
  const R Ca_TRPN = x.get(SO_Ca_TRPN);
  const R y = o_div(R(1000) * Ca_i, Ca_T50);
  const R dCaTRPN = C.k_TRPN * ((C.n_TRPN == R(2) ? y * y : o_pow(y, C.n_TRPN)) * (R(1) - Ca_TRPN) - Ca_TRPN);
  x.set(SO_Ca_TRPN, Ca_TRPN + tinc * dCaTRPN);
  const R cb = R(0.00238) + Ca_i;
  const R beta_Cai = o_div(R(1), R(1) + o_div(C.cmdnmax * R(0.00238), cb * cb));
  x.set(SO_Ca_i, Ca_i + tinc * (beta_Cai * (-s_Cai * R(0.5) * C.util_1 - J_up * C.vnsr_vmyo + J_diff_Ca * C.util_2 -
                                             R(0.07) * dCaTRPN)));
  const R sb = R(0.00087) + Ca_ss, sl = R(0.0087) + Ca_ss;
  const R beta_Cass = o_div(R(1), R(1) + o_div(R(0.047 * 0.00087), sb * sb) + o_div(R(1.124 * 0.0087), sl * sl));
  x.set(SO_Ca_ss, Ca_ss + tinc * (beta_Cass * (-(I_CaL - R(2) * I_NaCa_ss) * R(0.5) * C.util_3 +
                                               J_rel * C.vjsr_vss - J_diff_Ca)));
  x.add(SO_Ca_nsr, Ca_nsr, tinc * (J_up - J_tr * C.vjsr_vnsr));
  const R jb = R(0.8) + Ca_jsr;
  x.add(SO_Ca_jsr, Ca_jsr, tinc * (o_div(R(1), R(1) + o_div(R(10.0 * 0.8), jb * jb)) * (J_tr - J_rel)));
  return R(0.001) * tinc * -I_sum;
}

}  // namespace cm
