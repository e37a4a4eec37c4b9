// Courtemanche 1998 atrial model (reference Courtemanche::Calc, CourtemancheEtAl.cpp:85-187,
// compiled there with ISAC and TRPN, CourtemancheParameters.h:20,23) as per-cell functions.
#pragma once

#include "cm_common.cuh"
#include "cm_fp64_math.cuh"

namespace cm {

template <typename R>
struct CRNCell {
  R h, j, oi, ui, Xr, Xs, u, v, w, m, oa, ua, d, f, f_Ca;  // gates
  R Ca_i, Ca_TRPN;
};

template <typename R>
struct CRNHet_ {
  R g_Na, g_to, g_Ks, g_CaL, g_bNa, g_bCa;
};

template <typename R>
CM_HD R clamp01(R x) {
  return x < R(0) ? R(0) : (x > R(1) ? R(1) : x);
}

// One reference Calc in FP64 (same update order as the reference: gates first from the old
// Vm row, f_Ca and w included; currents; SAC; troponin; SR and ion Euler updates; Ca_i with
// the old-Ca_i buffer factor; u/v from Fn). Returns dV [V]; dt in seconds (C.dt_ms = dt*1000).
CM_HD double crn_calc_fp64(const CRNConsts<double> &C, const double *__restrict__ row, CRNCell<double> &c,
                           double &Ca_up, double &Ca_rel, double &Na_i, double &K_i, const CRNHet_<double> &g,
                           double V, double i_external, double stretch, double &I_SAC_out, uint32_t &audit) {
  using fp64::ddiv;  // the FP64 exp, log and division of cm_fp64_math.cuh (within 1 ulp)
  using fp64::dexp;
  using fp64::dlog;
  const double tinc = C.dt_ms;
  const double V_int = V * 1000.0;
  const double dNa_i = ddiv(1.0, Na_i);
  const double VmE_Na = V_int - (C.RTdF * dlog(C.Na_o * dNa_i));
  const double VmE_K = V_int - (C.RTdF * dlog(ddiv(C.K_o, K_i)));
  const double VmE_Ca = V_int - (C.RTd2F * dlog(ddiv(C.Ca_o, c.Ca_i)));
  c.m = clamp01(row[CR_m_m] + (c.m - row[CR_m_m]) * row[CR_exptau_m]);
  c.h = row[CR_m_h] + (c.h - row[CR_m_h]) * row[CR_exptau_h];
  c.j = row[CR_m_j] + (c.j - row[CR_m_j]) * row[CR_exptau_j];
  c.oa = row[CR_m_oa] + (c.oa - row[CR_m_oa]) * row[CR_exptau_oa];
  c.oi = row[CR_m_oi] + (c.oi - row[CR_m_oi]) * row[CR_exptau_oi];
  c.ua = row[CR_m_ua] + (c.ua - row[CR_m_ua]) * row[CR_exptau_ua];
  c.ui = row[CR_m_ui] + (c.ui - row[CR_m_ui]) * row[CR_exptau_ui];
  c.Xr = row[CR_m_Xr] + (c.Xr - row[CR_m_Xr]) * row[CR_exptau_Xr];
  c.Xs = row[CR_m_Xs] + (c.Xs - row[CR_m_Xs]) * row[CR_exptau_Xs];
  c.d = row[CR_m_d] + (c.d - row[CR_m_d]) * row[CR_exptau_d];
  c.f = row[CR_m_f] + (c.f - row[CR_m_f]) * row[CR_exptau_f];
  c.f_Ca += (ddiv(1.0, 1.0 + c.Ca_i * 2857.1429) - c.f_Ca) * 0.5 * tinc;
  c.w = row[CR_m_w] + (c.w - row[CR_m_w]) * row[CR_exptau_w];

  const double I_Na = g.g_Na * c.m * c.m * c.m * c.h * c.j * VmE_Na;
  const double I_to = g.g_to * c.oa * c.oa * c.oa * c.oi * VmE_K;
  const double I_Kur = row[CR_g_Kur] * c.ua * c.ua * c.ua * c.ui * VmE_K;
  const double I_Kr = row[CR_CKr] * c.Xr * VmE_K;
  const double I_Ks = g.g_Ks * c.Xs * c.Xs * VmE_K;
  const double I_CaL = g.g_CaL * c.d * c.f * c.f_Ca * (V_int - C.E_rL);
  const double I_K1 = row[CR_CK1] * VmE_K;
  const double I_bNa = g.g_bNa * VmE_Na;
  const double I_bCa = g.g_bCa * VmE_Ca;
  const double temp = C.k_mNai * dNa_i;
  const double I_NaK = ddiv(row[CR_CNaK], 1.0 + temp * sqrt(temp));
  const double I_pCa = ddiv(C.I_pCamax * c.Ca_i, c.Ca_i + C.k_mpCa);
  const double I_NaCa = row[CR_CNaCa] * ((Na_i * Na_i * Na_i * C.Ca_o) - row[CR_expVm] * c.Ca_i);
  const double I_rel = C.k_rel * c.u * c.u * c.v * c.w * (Ca_rel - c.Ca_i);
  const double I_up = ddiv(C.I_upmax * c.Ca_i, c.Ca_i + C.k_up);
  const double I_upleak = C.kupleak * Ca_up;
  const double I_tr = (Ca_up - Ca_rel) * C.dt_tr;
  double I_SAC = ddiv(C.G_sac * (V_int - C.E_sac), 1. + C.K_sac * dexp(-C.alpha * (stretch - 1.)));
  I_SAC *= C.ISAC_SWITCH;
  const double Ca_T50 = C.Ca_T50 + C.beta1 * ((stretch < 1.2 ? stretch : 1.2) - 1.);
  const double x = ddiv(1000 * c.Ca_i, Ca_T50);
  const double px = C.n_TRPN == 2.0 ? x * x : pow(x, C.n_TRPN);
  const double dCaTRPN = C.k_TRPN * (px * (1. - c.Ca_TRPN) - c.Ca_TRPN);
  c.Ca_TRPN += tinc * dCaTRPN;
  Ca_up += tinc * (I_up - I_tr * C.VreldVup - I_upleak);
  Ca_rel += tinc * ddiv(I_tr - I_rel, 1.0 + ddiv(C.csqnkm, Ca_rel * Ca_rel + Ca_rel * C.kmcsqnm2 + C.kkmcsqn));
  Na_i += tinc * (-3.0 * I_NaK - 3.0 * I_NaCa - I_bNa - I_Na) * C.CmdFvi;
  K_i += tinc * (2.0 * I_NaK - I_K1 - I_to - I_Kur - I_Kr - I_Ks) * C.CmdFvi;
  double B1 = ((2.0 * I_NaCa - I_pCa - I_CaL - I_bCa) * .5 * C.CmdFvi) + ((I_upleak - I_up) * C.VupdVi + I_rel * C.VreldVi);
  B1 -= C.TRPNmax * dCaTRPN;
  const double B2 = 1.0 + ddiv(C.cmdnkm, (c.Ca_i * c.Ca_i) + (c.Ca_i * C.kmcmdnm2) + C.kkmcmdn);
  const double dCa_i = ddiv(B1, B2);
  c.Ca_i += tinc * dCa_i;
  const double Fn = dexp(-(C.Vrel * I_rel - (0.5 * I_CaL - 0.2 * I_NaCa) * C.Cmd2F) * 731.5289);
  const double m_u = ddiv(1.0, 1.0 + Fn * C.exp250);
  c.u += (m_u - c.u) * 0.125 * tinc;
  const double m_v = 1.0 - ddiv(1.0, 1.0 + Fn * C.exp50);
  const double t_v = 1.91 + 2.09 * m_u;
  c.v += ddiv((m_v - c.v) * tinc, t_v);
  const double I_tot =
      I_Na + I_CaL + I_pCa + I_K1 + I_to + I_Kur + I_Kr + I_Ks + I_bNa + I_bCa + I_NaK + I_NaCa + I_SAC - i_external;
  I_SAC_out = I_SAC;
  (void)audit;
  return -.001 * I_tot * tinc;
}

// Mixed form: gates, currents, Ca_i and Ca_TRPN in FP32; Na_i, K_i, Ca_up, Ca_rel in compensated
// FP32 accumulators (Acc). exp(250) and exp(169.5) exceed FP32, so Fn * exp(c) is evaluated as exp(arg + c).
CM_HD float crn_calc_mixed(const CRNConsts<float> &C, const float *__restrict__ row, CRNCell<float> &c,
                           Acc &Ca_up_a, Acc &Ca_rel_a, Acc &Na_a, Acc &K_a, const CRNHet_<float> &g,
                           float V, float i_external, float stretch, uint32_t &audit) {
  const float tinc = C.dt_ms;
  const float V_int = V * 1000.f;
  const float Na_i = Na_a.hi, K_i = K_a.hi, Ca_up = Ca_up_a.hi, Ca_rel = Ca_rel_a.hi;
  const float dNa_i = fdiv(1.f, Na_i);
  const float VmE_Na = V_int - C.RTdF * (C.logNao - flog(Na_i));
  const float VmE_K = V_int - C.RTdF * (C.logKo - flog(K_i));
  const float VmE_Ca = V_int - C.RTd2F * (C.logCao - flog(c.Ca_i));
  c.m = clamp01(row[CR_m_m] + (c.m - row[CR_m_m]) * row[CR_exptau_m]);
  c.h = row[CR_m_h] + (c.h - row[CR_m_h]) * row[CR_exptau_h];
  c.j = row[CR_m_j] + (c.j - row[CR_m_j]) * row[CR_exptau_j];
  c.oa = row[CR_m_oa] + (c.oa - row[CR_m_oa]) * row[CR_exptau_oa];
  c.oi = row[CR_m_oi] + (c.oi - row[CR_m_oi]) * row[CR_exptau_oi];
  c.ua = row[CR_m_ua] + (c.ua - row[CR_m_ua]) * row[CR_exptau_ua];
  c.ui = row[CR_m_ui] + (c.ui - row[CR_m_ui]) * row[CR_exptau_ui];
  c.Xr = row[CR_m_Xr] + (c.Xr - row[CR_m_Xr]) * row[CR_exptau_Xr];
  c.Xs = row[CR_m_Xs] + (c.Xs - row[CR_m_Xs]) * row[CR_exptau_Xs];
  c.d = row[CR_m_d] + (c.d - row[CR_m_d]) * row[CR_exptau_d];
  c.f = row[CR_m_f] + (c.f - row[CR_m_f]) * row[CR_exptau_f];
  c.f_Ca += (fdiv(1.f, 1.f + c.Ca_i * 2857.1429f) - c.f_Ca) * 0.5f * tinc;
  c.w = row[CR_m_w] + (c.w - row[CR_m_w]) * row[CR_exptau_w];

  const float I_Na = g.g_Na * c.m * c.m * c.m * c.h * c.j * VmE_Na;
  const float I_to = g.g_to * c.oa * c.oa * c.oa * c.oi * VmE_K;
  const float I_Kur = row[CR_g_Kur] * c.ua * c.ua * c.ua * c.ui * VmE_K;
  const float I_Kr = row[CR_CKr] * c.Xr * VmE_K;
  const float I_Ks = g.g_Ks * c.Xs * c.Xs * VmE_K;
  const float I_CaL = g.g_CaL * c.d * c.f * c.f_Ca * (V_int - C.E_rL);
  const float I_K1 = row[CR_CK1] * VmE_K;
  const float I_bNa = g.g_bNa * VmE_Na;
  const float I_bCa = g.g_bCa * VmE_Ca;
  const float temp = C.k_mNai * dNa_i;
  const float I_NaK = fdiv(row[CR_CNaK], 1.f + temp * fsqrt(temp));
  const float I_pCa = fdiv(C.I_pCamax * c.Ca_i, c.Ca_i + C.k_mpCa);
  const float I_NaCa = row[CR_CNaCa] * ((Na_i * Na_i * Na_i * C.Ca_o) - row[CR_expVm] * c.Ca_i);
  const float I_rel = C.k_rel * c.u * c.u * c.v * c.w * (Ca_rel - c.Ca_i);
  const float I_up = fdiv(C.I_upmax * c.Ca_i, c.Ca_i + C.k_up);
  const float I_upleak = C.kupleak * Ca_up;
  const float I_tr = (Ca_up - Ca_rel) * C.dt_tr;
  const float I_SAC = C.ISAC_SWITCH * fdiv(C.G_sac * (V_int - C.E_sac), 1.f + C.K_sac * fexp(-C.alpha * (stretch - 1.f)));
  const float Ca_T50 = C.Ca_T50 + C.beta1 * ((stretch < 1.2f ? stretch : 1.2f) - 1.f);
  const float x = fdiv(1000.f * c.Ca_i, Ca_T50);
  const float px = C.n_TRPN == 2.f ? x * x : powf(x, C.n_TRPN);
  const float dCaTRPN = C.k_TRPN * (px * (1.f - c.Ca_TRPN) - c.Ca_TRPN);
  c.Ca_TRPN += tinc * dCaTRPN;
  acc_add(Ca_up_a, tinc * (I_up - I_tr * C.VreldVup - I_upleak));
  acc_add(Ca_rel_a, tinc * fdiv((I_tr - I_rel) * (Ca_rel * Ca_rel + Ca_rel * C.kmcsqnm2 + C.kkmcsqn), Ca_rel * Ca_rel + Ca_rel * C.kmcsqnm2 + C.kkmcsqn + C.csqnkm));
  acc_add(Na_a, tinc * (-3.f * I_NaK - 3.f * I_NaCa - I_bNa - I_Na) * C.CmdFvi);
  acc_add(K_a, tinc * (2.f * I_NaK - I_K1 - I_to - I_Kur - I_Kr - I_Ks) * C.CmdFvi);
  float B1 = ((2.f * I_NaCa - I_pCa - I_CaL - I_bCa) * .5f * C.CmdFvi) + ((I_upleak - I_up) * C.VupdVi + I_rel * C.VreldVi);
  B1 -= C.TRPNmax * dCaTRPN;
  const float q = (c.Ca_i * c.Ca_i) + (c.Ca_i * C.kmcmdnm2) + C.kkmcmdn;
  c.Ca_i += tinc * fdiv(B1 * q, q + C.cmdnkm);  // B1 / (1 + cmdnkm/q)
  const float arg = -(C.Vrel * I_rel - (0.5f * I_CaL - 0.2f * I_NaCa) * C.Cmd2F) * 731.5289f;
  const float m_u = fdiv(1.f, 1.f + fexp(arg + 250.f));
  c.u += (m_u - c.u) * 0.125f * tinc;
  const float m_v = 1.f - fdiv(1.f, 1.f + fexp(arg + 169.5f));
  const float t_v = 1.91f + 2.09f * m_u;
  c.v += fdiv((m_v - c.v) * tinc, t_v);
  const float I_tot =
      I_Na + I_CaL + I_pCa + I_K1 + I_to + I_Kur + I_Kr + I_Ks + I_bNa + I_bCa + I_NaK + I_NaCa + I_SAC - i_external;
  (void)audit;
  return -.001f * I_tot * tinc;
}

}  // namespace cm
