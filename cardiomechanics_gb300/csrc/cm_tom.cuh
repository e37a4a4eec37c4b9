// Tomek 2019 human ventricular model (ToR-ORd) as the reference compiles it (Tomek.cpp:110-656
// with ISAC and TRPN defined, TomekParameters.h:18-23): ten Tusscher-style I_Na gates with a
// CaMK-phosphorylated pair, I_CaL split 80/20 between subspace and myoplasm with activity
// coefficients from the local ionic strength, a five-state I_Kr Markov chain, instantaneous
// I_K1, Ca-activated and background Cl- currents, troponin buffering and a stretch-activated
// current. Every gate from its closed form (no lookup tables), as the reference.
//
// The same template serves FP64 and the mixed form, with the helpers and state-store
// interface of the O'Hara-Rudy model (cm_ord.cuh).
#pragma once

#include "cm_ord.cuh"

namespace cm {

CM_HD double o_sqrt(double x) { return sqrt(x); }
CM_HD float o_sqrt(float x) { return fsqrt(x); }

// exp(-constA z^2 (sqrt(I)/(1+sqrt(I)) - 0.3 I)): the activity coefficient of Tomek::Calc
// (lines 272-279) at ionic strength I [M].
template <typename R>
CM_HD R t_gamma(R constA_z2, R I) {
  const R sI = o_sqrt(I);
  return o_exp(-constA_z2 * (o_div(sI, R(1) + sI) - R(0.3) * I));
}

// One Calc of one cell; the store interface of ord_calc (fetch, get, set, add, cur). cur
// indices 0..35 are the block's stored values in order (I_Na ... I_SAC), 36..39 the rates A_h,
// B_h, A_j, B_j. Returns dV [V].
template <typename R, typename S>
CM_HD R tom_calc(const TOMConsts<R> &C, S &x, const ORDHet_<R> &g, R V, R i_external, R stretch) {
  const R tinc = C.dt_ms;
  const R V_m = V * R(1000);
  const R Na_i = x.get(SM_Na_i), K_i = x.get(SM_K_i), Ca_ss = x.get(SM_Ca_ss), Cl_i = x.get(SM_Cl_i);
  R I_sum = i_external;
  R s_Nai, s_Ki;

  // CaMK (127-132)
  const R CaMK_trap = x.get(SM_CaMK_trap);
  const R CaMK_bound = o_div(R(0.05) * (R(1) - CaMK_trap), R(1) + o_div(R(0.0015), Ca_ss));
  const R CaMK_active = CaMK_bound + CaMK_trap;
  x.set(SM_CaMK_trap,
        CaMK_trap + tinc * (R(0.05) * CaMK_bound * (CaMK_bound + CaMK_trap) - R(0.00068) * CaMK_trap));
  const R phi = o_div(R(1), R(1) + o_div(R(0.15), CaMK_active));

  // reversal potentials (135-140)
  const R E_Na = C.RToverF * o_log(o_div(C.Na_o, Na_i));
  const R E_K = C.RToverF * o_log(o_div(C.K_o, K_i));
  const R E_Cl = C.RToF * o_log(o_div(Cl_i, C.Cl_o));
  const R VFoverRT = V_m * C.FoRT;
  const R VFFoverRT = V_m * C.FFoRT;

  // I_Na (150-182)
  const R tau_m = [&] {
    const R u = (V_m + R(45.79)) * rc<R>(15.54), w = (V_m - R(4.823)) * rc<R>(51.12);
    return R(0.1292) * o_exp(-(u * u)) + R(0.06487) * o_exp(-(w * w));
  }();
  {
    const R em = R(1) + o_exp(-(V_m + R(56.86)) * rc<R>(9.03));
    const R m = o_gate(o_div(R(1), em * em), x.get(SM_m), tinc, tau_m);
    x.set(SM_m, m);
    R A_h, B_h, A_j, B_j;
    if (V_m < R(-40.0)) {
      A_h = R(0.057) * o_exp(-(V_m + R(80.0)) * rc<R>(6.8));
      B_h = R(2.7) * o_exp(R(0.079) * V_m) + R(3.1e5) * o_exp(R(0.3485) * V_m);
      A_j = o_div((R(-2.5428e4) * o_exp(R(0.2444) * V_m) - R(6.948e-6) * o_exp(R(-0.04391) * V_m)) * (V_m + R(37.78)),
                  R(1) + o_exp(R(0.311) * (V_m + R(79.23))));
      B_j = o_div(R(0.02424) * o_exp(R(-0.01052) * V_m), R(1) + o_exp(R(-0.1378) * (V_m + R(40.14))));
    } else {
      A_h = R(0);
      B_h = o_div(R(0.77), R(0.13) * (R(1) + o_exp(-(V_m + R(10.66)) * rc<R>(11.1))));
      A_j = R(0);
      B_j = o_div(R(0.6) * o_exp(R(0.057) * V_m), R(1) + o_exp(R(-0.1) * (V_m + R(32.0))));
    }
    x.cur(36, A_h);
    x.cur(37, B_h);
    x.cur(38, A_j);
    x.cur(39, B_j);
    const R tau_h = o_div(R(1), A_h + B_h);
    const R eh = R(1) + o_exp((V_m + R(71.55)) * rc<R>(7.43));
    const R h_inf = o_div(R(1), eh * eh);
    const R h = o_gate(h_inf, x.get(SM_h), tinc, tau_h);
    x.set(SM_h, h);
    const R tau_j = o_div(R(1), A_j + B_j);
    const R j = o_gate(h_inf, x.get(SM_j), tinc, tau_j);
    x.set(SM_j, j);
    const R ehp = R(1) + o_exp((V_m + R(77.55)) * rc<R>(7.43));
    const R h_p = o_gate(o_div(R(1), ehp * ehp), x.get(SM_h_p), tinc, tau_h);
    x.set(SM_h_p, h_p);
    const R j_p = o_gate(h_inf, x.get(SM_j_p), tinc, R(1.46) * tau_j);
    x.set(SM_j_p, j_p);
    const R I_Na = g.INaF * R(11.7802) * (V_m - E_Na) * m * m * m * ((R(1) - phi) * h * j + phi * h_p * j_p);
    x.cur(0, I_Na);
    I_sum += I_Na;
    s_Nai = I_Na;
  }

  // I_NaL (186-198)
  {
    const R m_L = o_gate(o_sig(-(V_m + R(42.85)) * rc<R>(5.264)), x.get(SM_m_L), tinc, tau_m);
    x.set(SM_m_L, m_L);
    const R h_L = o_gate(o_sig((V_m + R(87.61)) * rc<R>(7.488)), x.get(SM_h_L), tinc, C.tau_h_L);
    x.set(SM_h_L, h_L);
    const R h_L_CaMK = o_gate(o_sig((V_m + R(93.81)) * rc<R>(7.488)), x.get(SM_h_L_CaMK), tinc, C.tau_h_L_CaMK);
    x.set(SM_h_L_CaMK, h_L_CaMK);
    const R I_Na_late = g.INaL * R(0.0279) * (V_m - E_Na) * m_L * ((R(1) - phi) * h_L + phi * h_L_CaMK);
    x.cur(1, I_Na_late);
    I_sum += I_Na_late;
    s_Nai += I_Na_late;
  }

  // I_to (200-231)
  {
    const R tau_a =
        o_div(R(1.0515), o_div(R(1), R(1.2089) * (R(1) + o_exp(-(V_m - R(18.4099)) * rc<R>(29.3814)))) +
                             o_div(R(3.5), R(1) + o_exp((V_m + R(100.0)) * rc<R>(29.3814))));
    const R a = o_gate(o_sig(-(V_m - R(14.34)) * rc<R>(14.82)), x.get(SM_a), tinc, tau_a);
    x.set(SM_a, a);
    const R a_CaMK = o_gate(o_sig(-(V_m - R(24.34)) * rc<R>(14.82)), x.get(SM_a_CaMK), tinc, tau_a);
    x.set(SM_a_CaMK, a_CaMK);
    const R i_inf = o_sig((V_m + R(43.94)) * rc<R>(5.711));
    const R delta_epi = C.epi != R(0) ? R(1) - R(0.95) * o_sig((V_m + R(70.0)) * rc<R>(5.0)) : R(1);
    const R tau_i_fast = (R(4.562) + o_div(R(1), R(0.3933) * o_exp(-(V_m + R(100.0)) * rc<R>(100.0)) +
                                                   R(0.08004) * o_exp((V_m + R(50.0)) * rc<R>(16.59)))) *
                         delta_epi;
    const R tau_i_slow = (R(23.62) + o_div(R(1), R(0.001416) * o_exp(-(V_m + R(96.52)) * rc<R>(59.05)) +
                                                   R(1.780e-08) * o_exp((V_m + R(114.1)) * rc<R>(8.079)))) *
                         delta_epi;
    const R i_fast = o_gate(i_inf, x.get(SM_i_fast), tinc, tau_i_fast);
    x.set(SM_i_fast, i_fast);
    const R i_slow = o_gate(i_inf, x.get(SM_i_slow), tinc, tau_i_slow);
    x.set(SM_i_slow, i_slow);
    const R dev =
        R(1.354) + o_div(R(1.0e-04), o_exp((V_m - R(167.4)) * rc<R>(15.89)) + o_exp(-(V_m - R(12.23)) * rc<R>(0.2154)));
    const R rec = R(1) - R(0.5) * o_sig((V_m + R(70.0)) * rc<R>(20.0));
    const R i_CaMK_fast = o_gate(i_inf, x.get(SM_i_CaMK_fast), tinc, tau_i_fast * dev * rec);
    x.set(SM_i_CaMK_fast, i_CaMK_fast);
    const R i_CaMK_slow = o_gate(i_inf, x.get(SM_i_CaMK_slow), tinc, tau_i_slow * dev * rec);
    x.set(SM_i_CaMK_slow, i_CaMK_slow);
    const R A_i_fast = o_sig((V_m - R(213.6)) * rc<R>(151.2));
    const R A_i_slow = R(1) - A_i_fast;
    const R i = A_i_fast * i_fast + A_i_slow * i_slow;
    const R i_CaMK = A_i_fast * i_CaMK_fast + A_i_slow * i_CaMK_slow;
    const R I_to = g.Ito * R(0.16) * (V_m - E_K) * ((R(1) - phi) * a * i + phi * a_CaMK * i_CaMK);
    x.cur(2, I_to);
    I_sum += I_to;
    s_Ki = I_to;
  }

  // I_CaL, I_CaNa, I_CaK (233-327)
  x.fetch(1);
  const R Na_ss = x.get(SM_Na_ss), K_ss = x.get(SM_K_ss), Ca_i = x.get(SM_Ca_i);
  const R em1_Ca = o_expm1(R(2) * VFoverRT), em1_1 = o_expm1(VFoverRT);
  const R exp_z_Ca = em1_Ca + R(1), exp_z_1 = em1_1 + R(1);
  R I_CaL_ss, I_CaL_i, s_Nass, s_Kss;
  {
    const R d_inf = V_m > R(31.4978) ? R(1) : R(1.0763) * o_exp(R(-1.007) * o_exp(R(-0.0829) * V_m));
    const R tau_d = R(0.6) + o_div(R(1), o_exp(R(-0.05) * (V_m + R(6.0))) + o_exp(R(0.09) * (V_m + R(14.0))));
    const R d = o_gate(d_inf, x.get(SM_d), tinc, tau_d);
    x.set(SM_d, d);
    const R f_inf = o_sig((V_m + R(19.58)) * rc<R>(3.696));
    const R tau_f_fast = R(7.0) + o_div(R(1), R(0.0045) * o_exp(-(V_m + R(20.0)) * rc<R>(10.0)) +
                                                 R(0.0045) * o_exp((V_m + R(20.0)) * rc<R>(10.0)));
    const R tau_f_slow = R(1000.0) + o_div(R(1), R(3.5e-05) * o_exp(-(V_m + R(5.0)) * rc<R>(4.0)) +
                                                    R(3.5e-05) * o_exp((V_m + R(5.0)) * rc<R>(6.0)));
    const R A_f_Ca_fast = R(0.3) + R(0.6) * o_sig((V_m - R(10.0)) * rc<R>(10.0));
    const R A_f_Ca_slow = R(1) - A_f_Ca_fast;
    const R f_fast = o_gate(f_inf, x.get(SM_f_fast), tinc, tau_f_fast);
    x.set(SM_f_fast, f_fast);
    const R f_slow = o_gate(f_inf, x.get(SM_f_slow), tinc, tau_f_slow);
    x.set(SM_f_slow, f_slow);
    const R tau_f_Ca_fast = R(7.0) + o_div(R(1), R(0.04) * o_exp(-(V_m - R(4.0)) * rc<R>(7.0)) +
                                                    R(0.04) * o_exp((V_m - R(4.0)) * rc<R>(7.0)));
    const R tau_f_Ca_slow =
        R(100.0) + o_div(R(1), R(0.00012) * o_exp(-V_m * rc<R>(3.0)) + R(0.00012) * o_exp(V_m * rc<R>(7.0)));
    const R f_Ca_fast = o_gate(f_inf, x.get(SM_f_Ca_fast), tinc, tau_f_Ca_fast);
    x.set(SM_f_Ca_fast, f_Ca_fast);
    const R f_Ca_slow = o_gate(f_inf, x.get(SM_f_Ca_slow), tinc, tau_f_Ca_slow);
    x.set(SM_f_Ca_slow, f_Ca_slow);
    const R j_Ca = o_gate(o_sig((V_m + R(18.08)) * rc<R>(2.7916)), x.get(SM_j_Ca), tinc, R(75.0));
    x.set(SM_j_Ca, j_Ca);
    const R f_CaMK_fast = o_gate(f_inf, x.get(SM_f_CaMK_fast), tinc, R(2.5) * tau_f_fast);
    x.set(SM_f_CaMK_fast, f_CaMK_fast);
    const R f_Ca_CaMK_fast = o_gate(f_inf, x.get(SM_f_Ca_CaMK_fast), tinc, R(2.5) * tau_f_Ca_fast);
    x.set(SM_f_Ca_CaMK_fast, f_Ca_CaMK_fast);
    const R f = C.A_f_fast * f_fast + C.A_f_slow * f_slow;
    const R f_Ca = A_f_Ca_fast * f_Ca_fast + A_f_Ca_slow * f_Ca_slow;
    const R f_CaMK = C.A_f_fast * f_CaMK_fast + C.A_f_slow * f_slow;
    const R f_Ca_CaMK = A_f_Ca_fast * f_Ca_CaMK_fast + A_f_Ca_slow * f_Ca_slow;
    // the two n gates: alpha_n (k2n / k_m2_n) as one quotient, k2n = 500, k_m2_n = j_Ca
    const R k2n_km2n = o_div(R(500.0), j_Ca);
    const R decay = o_exp(-j_Ca * tinc);
    const R qs = R(1) + o_div(R(0.002), Ca_ss), qi = R(1) + o_div(R(0.002), Ca_i);
    const R ns_inf = o_div(k2n_km2n, k2n_km2n + (qs * qs) * (qs * qs));
    const R ni_inf = o_div(k2n_km2n, k2n_km2n + (qi * qi) * (qi * qi));
    const R n_ss = ns_inf - (ns_inf - x.get(SM_n_ss)) * decay;
    x.set(SM_n_ss, n_ss);
    const R n_i = ni_inf - (ni_inf - x.get(SM_n_i)) * decay;
    x.set(SM_n_i, n_i);
    // permeation: activity coefficients at the subspace and myoplasm ionic strengths [M]
    const R I_ss = R(0.5e-3) * (Na_ss + K_ss + Cl_i + R(4) * Ca_ss);
    const R I_i = R(0.5e-3) * (Na_i + K_i + Cl_i + R(4) * Ca_i);
    const R gCa_ss = t_gamma(R(4) * C.constA, I_ss), g1_ss = t_gamma(C.constA, I_ss);
    const R gCa_i = t_gamma(R(4) * C.constA, I_i), g1_i = t_gamma(C.constA, I_i);
    const R Psi_Ca_ss = R(4) * VFFoverRT * o_div(gCa_ss * Ca_ss * exp_z_Ca - C.gamma_Ca_o * C.Ca_o, em1_Ca);
    const R Psi_CaNa_ss = VFFoverRT * o_div(g1_ss * Na_ss * exp_z_1 - C.gamma_Na_o * C.Na_o, em1_1);
    const R Psi_CaK_ss = VFFoverRT * o_div(g1_ss * K_ss * exp_z_1 - C.gamma_K_o * C.K_o, em1_1);
    const R Psi_Ca_i = R(4) * VFFoverRT * o_div(gCa_i * Ca_i * exp_z_Ca - C.gamma_Ca_o * C.Ca_o, em1_Ca);
    const R Psi_CaNa_i = VFFoverRT * o_div(g1_i * Na_i * exp_z_1 - C.gamma_Na_o * C.Na_o, em1_1);
    const R Psi_CaK_i = VFFoverRT * o_div(g1_i * K_i * exp_z_1 - C.gamma_K_o * C.K_o, em1_1);
    // gates of the non-phosphorylated and phosphorylated channels, subspace (0.8) and myoplasm (0.2)
    const R g_np_ss = R(0.8) * (R(1) - phi) * d * (f * (R(1) - n_ss) + j_Ca * f_Ca * n_ss);
    const R g_p_ss = R(0.8) * phi * R(1.1) * d * (f_CaMK * (R(1) - n_ss) + j_Ca * f_Ca_CaMK * n_ss);
    const R g_np_i = R(0.2) * (R(1) - phi) * d * (f * (R(1) - n_i) + j_Ca * f_Ca * n_i);
    const R g_p_i = R(0.2) * phi * R(1.1) * d * (f_CaMK * (R(1) - n_i) + j_Ca * f_Ca_CaMK * n_i);
    const R PCa = C.PCa;
    I_CaL_ss = PCa * Psi_Ca_ss * (g_np_ss + g_p_ss);
    const R I_CaNa_ss = R(0.00125) * PCa * Psi_CaNa_ss * (g_np_ss + g_p_ss);
    const R I_CaK_ss = R(3.574e-4) * PCa * Psi_CaK_ss * (g_np_ss + g_p_ss);
    I_CaL_i = PCa * Psi_Ca_i * (g_np_i + g_p_i);
    const R I_CaNa_i = R(0.00125) * PCa * Psi_CaNa_i * (g_np_i + g_p_i);
    const R I_CaK_i = R(3.574e-4) * PCa * Psi_CaK_i * (g_np_i + g_p_i);
    x.cur(3, I_CaL_ss + I_CaL_i);
    x.cur(4, I_CaNa_ss + I_CaNa_i);
    x.cur(5, I_CaK_ss + I_CaK_i);
    x.cur(6, I_CaL_i);
    x.cur(7, I_CaL_ss);
    x.cur(8, I_CaNa_i);
    x.cur(9, I_CaNa_ss);
    x.cur(10, I_CaK_i);
    x.cur(11, I_CaK_ss);
    I_sum += (I_CaL_ss + I_CaL_i) + (I_CaNa_ss + I_CaNa_i) + (I_CaK_ss + I_CaK_i);
    s_Nai += I_CaNa_i;
    s_Ki += I_CaK_i;
    s_Nass = I_CaNa_ss;
    s_Kss = I_CaK_ss;
  }

  // I_Kr (329-351): five-state Markov chain, explicit Euler in the reference's order
  {
    const R alpha_Kr = R(0.1161) * o_exp(R(0.299) * VFoverRT);
    const R beta_Kr = R(0.2442) * o_exp(R(-1.604) * VFoverRT);
    const R alpha_Kr_1 = R(1.25 * 0.1235), beta_Kr_1 = R(0.1911);
    const R alpha_Kr_2 = R(0.0578) * o_exp(R(0.971) * VFoverRT);
    const R beta_Kr_2 = R(0.349e-3) * o_exp(R(-1.062) * VFoverRT);
    const R alpha_Kr_i = R(0.2533) * o_exp(R(0.5953) * VFoverRT);
    const R beta_Kr_i = R(0.06525) * o_exp(R(-0.8209) * VFoverRT);
    const R alpha_C2_to_I = R(0.52e-4) * o_exp(R(1.525) * VFoverRT);
    const R beta_I_to_C2 = o_div(beta_Kr_2 * beta_Kr_i * alpha_C2_to_I, alpha_Kr_2 * alpha_Kr_i);
    R C_0 = x.get(SM_C_0), C_1 = x.get(SM_C_1), C_2 = x.get(SM_C_2), O = x.get(SM_O), I = x.get(SM_I);
    C_0 += tinc * (C_1 * beta_Kr - C_0 * alpha_Kr);
    C_1 += tinc * (C_0 * alpha_Kr + C_2 * beta_Kr_1 - C_1 * (beta_Kr + alpha_Kr_1));
    C_2 += tinc * (C_1 * alpha_Kr_1 + O * beta_Kr_2 + I * beta_I_to_C2 - C_2 * (beta_Kr_1 + alpha_Kr_2 + alpha_C2_to_I));
    O += tinc * ((alpha_Kr_2 * C_2 + beta_Kr_i * I) - (beta_Kr_2 + alpha_Kr_i) * O);
    I += tinc * ((alpha_C2_to_I * C_2 + alpha_Kr_i * O) - (beta_I_to_C2 + beta_Kr_i) * I);
    x.set(SM_C_0, C_0);
    x.set(SM_C_1, C_1);
    x.set(SM_C_2, C_2);
    x.set(SM_O, O);
    x.set(SM_I, I);
    const R I_Kr = g.IKr * R(0.0321) * C.sqrtKo5 * O * (V_m - E_K);
    x.cur(12, I_Kr);

    // I_Ks (355-363)
    const R x_s1_inf = o_sig(-(V_m + R(11.6)) * rc<R>(8.932));
    const R tau_x_s1 = R(817.3) + o_div(R(1), R(2.326e-04) * o_exp((V_m + R(48.28)) * rc<R>(17.80)) +
                                                  R(0.001292) * o_exp(-(V_m + R(210.0)) * rc<R>(230.0)));
    const R x_s1 = o_gate(x_s1_inf, x.get(SM_x_s1), tinc, tau_x_s1);
    x.set(SM_x_s1, x_s1);
    const R tau_x_s2 = o_div(R(1), R(0.01) * o_exp((V_m - R(50.0)) * rc<R>(20.0)) +
                                        R(0.0193) * o_exp(-(V_m + R(66.54)) * rc<R>(31.0)));
    const R x_s2 = o_gate(x_s1_inf, x.get(SM_x_s2), tinc, tau_x_s2);
    x.set(SM_x_s2, x_s2);
    const R E_Ks = C.RToverF * o_log(o_div(C.EKs_num, K_i + R(0.01833) * Na_i));
    const R I_Ks = g.IKs * R(0.0011) * (R(1) + o_div(R(0.6), R(1) + o_pow(o_div(R(3.8e-05), Ca_i), R(1.4)))) *
                   x_s1 * x_s2 * (V_m - E_Ks);
    x.cur(13, I_Ks);

    // I_K1 (365-370): instantaneous rectification
    const R dK = V_m - E_K;
    const R a_K1 = o_div(R(4.094), R(1) + o_exp(R(0.1217) * (dK - R(49.934))));
    const R b_K1 = o_div(R(15.72) * o_exp(R(0.0674) * (dK - R(3.257))) + o_exp(R(0.0618) * (dK - R(594.31))),
                         R(1) + o_exp(R(-0.1629) * (dK + R(14.207))));
    const R I_K1 = g.IK1 * R(0.6992) * C.sqrtKo5 * o_div(a_K1, a_K1 + b_K1) * dK;
    x.cur(14, I_K1);
    I_sum += I_Kr + I_Ks + I_K1;
    s_Ki += I_Kr + I_Ks + I_K1;
  }

  // I_NaCa_i and I_NaCa_ss (373-451): O'Hara-Rudy's exchanger, G 0.0034 x 0.65 | 0.35
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
      const R na = s == 0 ? Na_i : Na_ss;
      const R ca = s == 0 ? Ca_i : Ca_ss;
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
      I_NaCa[s] = C.INaCa * (s == 0 ? R(0.0034 * 0.65) : R(0.0034 * 0.35)) * o_div(R(1), R(1) + ka * ka) *
                  (J_Na + R(2) * J_Ca);
    }
    I_NaCa_i = I_NaCa[0];
    I_NaCa_ss = I_NaCa[1];
    x.cur(15, I_NaCa_i);
    x.cur(16, I_NaCa_ss);
    I_sum += I_NaCa_i + I_NaCa_ss;
    s_Nai += R(3) * I_NaCa_i;
    s_Nass += R(3) * I_NaCa_ss;
  }

  // I_NaK (453-503), P_NaK 15.4509
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
    const R I_NaK = C.INaK * R(15.4509) * (R(3) * (x_1 * alpha_3 - x_2 * beta_3) * inv +
                                          R(2) * (x_4 * be1 - x_3 * alpha_1) * inv);
    x.cur(17, I_NaK);
    I_sum += I_NaK;
    s_Nai += R(3) * I_NaK;
    s_Ki -= R(2) * I_NaK;
  }

  // I_CaCl, background currents, I_pCa, I_SAC (505-538)
  R s_Cai;
  {
    const R I_CaCl_junc = o_div(R(0.2843) * (V_m - E_Cl), R(1) + o_div(R(0.1), Ca_ss));
    const R I_CaCl_sl = R(0);  // the reference's sarcolemmal part is multiplied by 0
    const R I_Kb = C.IKb * R(0.0189) * o_sig(-(V_m - R(10.8968)) * rc<R>(23.9871)) * (V_m - E_K);
    const R I_Nab = C.INab * R(1.9239e-9) * VFFoverRT * o_div(Na_i * exp_z_1 - C.Na_o, em1_1);
    const R gCa_i = t_gamma(R(4) * C.constA, R(0.5e-3) * (Na_i + K_i + Cl_i + R(4) * Ca_i));
    const R I_Cab = C.ICab * R(5.9194e-8) * R(4) * VFFoverRT * o_div(gCa_i * Ca_i * exp_z_Ca - C.gamma_Ca_o * C.Ca_o, em1_Ca);
    const R I_Clb = R(1.98e-3) * (V_m - E_Cl);
    const R I_pCa = C.IpCa * o_div(R(0.0005) * Ca_i, R(0.0005) + Ca_i);
    const R I_SAC =
        C.ISAC_SWITCH * o_div(C.G_sac * (V_m - C.E_sac), R(1) + C.K_sac * o_exp(-C.alpha_sac * (stretch - R(1))));
    x.cur(18, I_CaCl_junc);
    x.cur(19, I_CaCl_sl);
    x.cur(20, I_CaCl_junc + I_CaCl_sl);
    x.cur(21, I_Nab);
    x.cur(22, I_Cab);
    x.cur(23, I_Kb);
    x.cur(24, I_Clb);
    x.cur(25, I_pCa);
    x.cur(35, I_SAC);
    I_sum += I_Nab + I_Cab + I_Kb + I_pCa + I_Clb + (I_CaCl_junc + I_CaCl_sl) + I_SAC;
    s_Nai += I_Nab;
    s_Ki += I_Kb + i_external;
    s_Cai = I_CaL_i + I_pCa + I_Cab - R(2) * I_NaCa_i;
  }

  // SR release and uptake (550-590)
  const R Ca_nsr = x.get(SM_Ca_nsr), Ca_jsr = x.get(SM_Ca_jsr);
  const R cj = R(1.7) * o_div(R(1), Ca_jsr), cj2 = cj * cj, cj4 = cj2 * cj2;
  const R I_CaL = I_CaL_ss + I_CaL_i;
  const R rel_inf = o_div(-I_CaL * C.rel_scale, R(1) + cj4 * cj4);
  const R tau_rel_b = o_div(R(1), R(1) + R(0.0123) * o_div(R(1), Ca_jsr));
  const R tau_NP = C.beta_tau * tau_rel_b, tau_CaMK = C.beta_tau_CaMK * tau_rel_b;
  const R J_rel_NP = o_gate(C.alpha_rel * rel_inf, x.get(SM_J_rel_NP), tinc, tau_NP < R(0.001) ? R(0.001) : tau_NP);
  x.set(SM_J_rel_NP, J_rel_NP);
  const R J_rel_CaMK =
      o_gate(C.alpha_rel_CaMK * rel_inf, x.get(SM_J_rel_CaMK), tinc, tau_CaMK < R(0.001) ? R(0.001) : tau_CaMK);
  x.set(SM_J_rel_CaMK, J_rel_CaMK);
  const R J_rel = R(1.5378) * (R(1) - phi) * J_rel_NP + phi * J_rel_CaMK;
  const R J_up_NP = o_div(R(0.005425) * Ca_i, R(0.00092) + Ca_i) * C.up_scale;
  const R J_up_CaMK = o_div(R(2.75 * 0.005425) * Ca_i, R(0.00092) - R(0.00017) + Ca_i) * C.up_scale;
  const R J_leak = R(0.0048825) * Ca_nsr * rc<R>(15.0);
  const R J_up = (R(1) - phi) * J_up_NP + phi * J_up_CaMK - J_leak;
  const R J_tr = (Ca_nsr - Ca_jsr) * rc<R>(60.0);
  const R J_diff_Na = (Na_ss - Na_i) * R(0.5);
  const R J_diff_Ca = (Ca_ss - Ca_i) * R(5);
  const R J_diff_K = (K_ss - K_i) * R(0.5);
  x.cur(26, J_diff_Na);
  x.cur(27, J_diff_Ca);
  x.cur(28, J_diff_K);
  x.cur(29, J_leak);
  x.cur(30, J_rel);
  x.cur(31, J_tr);
  x.cur(32, J_up);
  x.cur(33, I_sum);
  x.cur(34, -I_sum);

  // concentrations (592-654)
  x.add(SM_Na_i, Na_i, tinc * (-s_Nai * C.util_1 + J_diff_Na * C.util_2));
  x.add(SM_Na_ss, Na_ss, tinc * (-s_Nass * C.util_3 - J_diff_Na));
  x.add(SM_K_i, K_i, tinc * (-s_Ki * C.util_1 + J_diff_K * C.util_2));
  x.add(SM_K_ss, K_ss, tinc * (-(s_Kss * C.util_3) - J_diff_K));
  const R Ca_T50 = C.Ca_T50 + C.beta1 * ((stretch < R(1.2) ? stretch : R(1.2)) - R(1));
  const R Ca_TRPN = x.get(SM_Ca_TRPN);
  const R y = o_div(R(1000) * Ca_i, Ca_T50);
  const R dCaTRPN = C.k_TRPN * ((C.n_TRPN == R(2) ? y * y : o_pow(y, C.n_TRPN)) * (R(1) - Ca_TRPN) - Ca_TRPN);
  x.set(SM_Ca_TRPN, Ca_TRPN + tinc * dCaTRPN);
  const R cb = R(0.00238) + Ca_i;
  const R beta_Cai = o_div(R(1), R(1) + o_div(C.cmdnmax * R(0.00238), cb * cb));
  x.set(SM_Ca_i, Ca_i + tinc * (beta_Cai * (-s_Cai * R(0.5) * C.util_1 - J_up * C.vnsr_vmyo + J_diff_Ca * C.util_2 -
                                             R(0.07) * dCaTRPN)));
  const R sb = R(0.00087) + Ca_ss, sl = R(0.0087) + Ca_ss;
  const R beta_Cass = o_div(R(1), R(1) + o_div(R(0.047 * 0.00087), sb * sb) + o_div(R(1.124 * 0.0087), sl * sl));
  x.set(SM_Ca_ss, Ca_ss + tinc * (beta_Cass * (-(I_CaL_ss - R(2) * I_NaCa_ss) * R(0.5) * C.util_3 +
                                               J_rel * C.vjsr_vss - J_diff_Ca)));
  x.add(SM_Ca_nsr, Ca_nsr, tinc * (J_up - J_tr * C.vjsr_vnsr));
  const R jb = R(0.8) + Ca_jsr;
  x.add(SM_Ca_jsr, Ca_jsr, tinc * (o_div(R(1), R(1) + o_div(R(10.0 * 0.8), jb * jb)) * (J_tr - J_rel)));
  return R(0.001) * tinc * -I_sum;
}

}  // namespace cm
