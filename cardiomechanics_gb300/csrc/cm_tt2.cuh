// ten Tusscher-Panfilov 2006 (reference TenTusscherEtAl2::Calc, TenTusscher2.cpp:615-906)
// as per-cell functions shared by the FP64 and mixed-precision kernels.
#pragma once

#include "cm_common.cuh"
#include "cm_fp64_math.cuh"

namespace cm {

template <typename R>
struct TT2Cell {
  R m, h, j, xr1, xr2, xs, r, s, d, f, f2, fCa, Rq;  // gates (Rq: RyR recovery)
  R Ca_i, CaSS;                                      // buffered fast Ca pools
};

// Per-cell conductances (hetero overrides already applied).
template <typename R>
struct TT2Het_ {
  R g_Na, g_Kr, g_K1, g_Ks, g_to, g_CaL;
};

// Diagnostic currents (reference Array[0..16], TenTusscher2.cpp:883-899).
template <typename R>
struct TT2Diag {
  R v[17];
};

// One reference Calc in FP64. Update order as in the reference: currents from the old
// state; Rq forward Euler first and O from the new Rq (807-809); release/leak/transfer from
// the old CaSR/CaSS/Ca_i (810-812); the three buffered quadratics (814-836); Na_i/K_i Euler
// (838-852); fCa from the new CaSS (853-855, 880); the other gates Rush-Larsen from the
// table row of the old voltage (857-879). Returns dV = -dt * I_tot [V].
template <bool kDiag>
CM_HD double tt2_calc_fp64(const TT2Consts<double> &C, const double *__restrict__ row,
                           const double *__restrict__ eca, TT2Cell<double> &c, double &CaSR, double &Na_i,
                           double &K_i, const TT2Het_<double> &g, double V, double i_external, uint32_t &audit,
                           TT2Diag<double> *diag) {
  const double svolt = V * 1000;
  i_external = i_external * C.inv_stim_unit;
  int Caitab = (int)(C.CaiTabConst2 * c.Ca_i + C.CaiTabConst1);
  if (Caitab < 0 || Caitab >= kRows) {  // reference reads out of bounds here (line 641)
    audit |= 4u;
    Caitab = Caitab < 0 ? 0 : kRows - 1;
  }
  // E_X = RT/F ln(X_o / X_i) as RT/F (ln X_o - ln X_i), ln X_o precomputed; AK1 / (AK1 + BK1)
  // over one denominator. The FP64 exp, log and division are the table-driven / Newton forms of
  // cm_fp64_math.cuh (within 1 ulp of the library's): on GB300 this step is bound by its count of
  // FP64-pipe instructions.
  using fp64::ddiv;
  using fp64::dexp;
  using fp64::dlog;
  const double EK = C.RTONF * (C.logKo - dlog(K_i));
  const double VminEK = svolt - EK;
  const double ENa = C.RTONF * (C.logNao - dlog(Na_i));
  const double VminENa = svolt - ENa;
  const double EKs = C.RTONF * (C.logKoNao - dlog(K_i + C.pKNa * Na_i));
  // rec_iK1 = AK1/(AK1+BK1), AK1 = 0.1/(1+e1), BK1 = (3 e2 + e3)/(1+e4)
  const double e1 = dexp(0.06 * (VminEK - 200)), e2 = dexp(0.0002 * (VminEK + 100));
  const double e3 = dexp(0.1 * (VminEK - 10)), e4 = dexp(-0.5 * (VminEK));
  const double a1 = 0.1 * (1. + e4);
  const double rec_iK1 = ddiv(a1, a1 + (3. * e2 + e3) * (1. + e1));
  const double I_pCa = ddiv(C.g_pCa * c.Ca_i, C.KpCa + c.Ca_i);
  const double I_pK = row[T2_rec_ipK] * VminEK;
  const double I_to = g.g_to * c.r * c.s * VminEK;
  const double I_Kr = g.g_Kr * C.sqrtKo54 * c.xr1 * c.xr2 * VminEK;
  const double I_Ks = g.g_Ks * c.xs * c.xs * (svolt - EKs);
  const double I_K = I_Kr + I_Ks;
  const double I_K1 = g.g_K1 * C.sqrtKo54 * rec_iK1 * VminEK;
  const double I_bNa = C.g_bNa * VminENa;
  const double I_bCa = C.g_bCa * (svolt - eca[Caitab]);
  const double I_Na = g.g_Na * c.m * c.m * c.m * c.h * c.j * VminENa;
  const double I_CaL = g.g_CaL * c.d * c.f * c.f2 * c.fCa * ((row[T2_CaL_P1] * c.CaSS) - row[T2_CaL_P2]);
  const double I_NaCa = C.kNaCa * row[T2_NaCa_P1] * Na_i * Na_i * Na_i - C.kNaCa * row[T2_NaCa_P2] * c.Ca_i;
  const double I_NaK = C.knak * C.KoKmK * ddiv(Na_i, Na_i + C.KmNa) * row[T2_NaK_P1];
  const double I_tot = I_K + I_K1 + I_to + I_Na + I_bNa + I_CaL + I_bCa + I_NaK + I_NaCa + I_pCa + I_pK - i_external;

  const double Caisquare = c.Ca_i * c.Ca_i;
  const double CaSSsquare = c.CaSS * c.CaSS;
  // kCaSR = max_sr - (max_sr - min_sr)/(1 + (EC/CaSR)^2) over one denominator
  const double CaSR2 = CaSR * CaSR;
  const double kCaSR = C.max_sr - ddiv((C.max_sr - C.min_sr) * CaSR2, CaSR2 + C.EC * C.EC);
  const double k2 = C.ks2 * kCaSR;
  const double dRq = 1000.0 * ((-k2 * c.CaSS * c.Rq) + (C.k4 * (1.0 - c.Rq)));
  c.Rq += C.dt * dRq;
  // O = k1 CaSS^2 Rq / (k3 + k1 CaSS^2) with k1 = ks1 / kCaSR, over one denominator
  const double k1C2 = C.ks1 * CaSSsquare;
  const double O = ddiv(k1C2 * c.Rq, C.k3 * kCaSR + k1C2);
  const double I_rel = C.Vrel * O * (CaSR - c.CaSS);
  const double I_leak = 0.00036 * (CaSR - c.Ca_i);
  const double I_xfer = C.Vxfer * (c.CaSS - c.Ca_i);
  const double SERCA = ddiv(C.Vmaxup * Caisquare, Caisquare + C.Kupsquare);
  const double dCaSR = C.dt1000 * (SERCA - I_rel - I_leak);
  const double CaCSQN = ddiv(C.Bufsr * CaSR, CaSR + C.Kbufsr);
  const double bjsr = C.Bufsr - CaCSQN - dCaSR - CaSR + C.Kbufsr;
  const double cjsr = C.Kbufsr * (CaCSQN + dCaSR + CaSR);
  CaSR = (sqrt(bjsr * bjsr + 4 * cjsr) - bjsr) * 0.5;
  const double CaSSBuf = ddiv(C.Bufss * c.CaSS, c.CaSS + C.Kbufss);
  const double dCaSS = C.dt1000 * (-I_xfer * C.VcVss + I_rel * C.VsrVss + (-I_CaL * C.inversevssF2 * C.Cm));
  const double bjss = C.Bufss - CaSSBuf - dCaSS - c.CaSS + C.Kbufss;
  const double cjss = C.Kbufss * (CaSSBuf + dCaSS + c.CaSS);
  c.CaSS = (sqrt(bjss * bjss + 4. * cjss) - bjss) * 0.5;
  const double CaBuf = ddiv(C.Bufc * c.Ca_i, c.Ca_i + C.Kbufc);
  const double dCai =
      C.dt1000 * ((-(I_bCa + I_pCa - 2 * I_NaCa) * C.inverseviF2 * C.Cm) - (SERCA - I_leak) * C.invVcdVsr + I_xfer);
  const double bc = C.BufcPKbufc - CaBuf - dCai - c.Ca_i;
  const double cc = C.Kbufc * (CaBuf + dCai + c.Ca_i);
  c.Ca_i = (sqrt(bc * bc + 4 * cc) - bc) * 0.5;
  const double dNai = -(I_Na + I_bNa + 3 * I_NaK + 3 * I_NaCa) * C.inverseviF * C.Cm;
  Na_i += C.dt * dNai * 1000;
  const double dKi = -(-i_external + I_K1 + I_to + I_K - 2 * I_NaK + I_pK) * C.inverseviF * C.Cm;
  K_i += C.dt * dKi * 1000.0;
  const double CaSS005 = c.CaSS * 20.0;
  const double den = ddiv(1.0, 1.0 + CaSS005 * CaSS005);
  const double FCa_INF = 0.6 * den + 0.4;
  const double taufca = 0.080 * den + 0.002;

  c.m = row[T2_m_inf] - (row[T2_m_inf] - c.m) * row[T2_exptau_m];
  c.h = row[T2_h_inf] - (row[T2_h_inf] - c.h) * row[T2_exptau_h];
  c.j = row[T2_j_inf] - (row[T2_j_inf] - c.j) * row[T2_exptau_j];
  c.xr1 = row[T2_Xr1_inf] - (row[T2_Xr1_inf] - c.xr1) * row[T2_exptau_Xr1];
  c.xr2 = row[T2_Xr2_inf] - (row[T2_Xr2_inf] - c.xr2) * row[T2_exptau_Xr2];
  c.xs = row[T2_Xs_inf] - (row[T2_Xs_inf] - c.xs) * row[T2_exptau_Xs];
  c.s = row[T2_s_inf] - (row[T2_s_inf] - c.s) * row[T2_exptau_s];
  c.r = row[T2_r_inf] - (row[T2_r_inf] - c.r) * row[T2_exptau_r];
  c.d = row[T2_d_inf] - (row[T2_d_inf] - c.d) * row[T2_exptau_d];
  c.f = row[T2_f_inf] - (row[T2_f_inf] - c.f) * row[T2_exptau_f];
  c.f2 = row[T2_f2_inf] - (row[T2_f2_inf] - c.f2) * row[T2_exptau_f2];
  c.fCa = FCa_INF - (FCa_INF - c.fCa) * dexp(-ddiv(C.dt, taufca));
  if (kDiag) {
    double *a = diag->v;
    a[0] = I_Na; a[1] = I_CaL; a[2] = I_bCa; a[3] = I_pCa; a[4] = I_to; a[5] = I_Ks; a[6] = I_Kr;
    a[7] = I_K1; a[8] = I_pK; a[9] = I_bNa; a[10] = I_NaK; a[11] = I_NaCa; a[12] = I_rel; a[13] = I_leak;
    a[14] = I_xfer; a[15] = SERCA; a[16] = I_tot;
  }
  return C.dt * (-I_tot);
}

// Mixed form: the same update with gates, currents and the fast Ca pools in FP32. Vm, Na_i,
// K_i and CaSR are compensated FP32 accumulators (Acc; their per-step increments are
// 1e-7..1e-9 of their values and vanish in plain FP32); the three buffered-Ca updates use buffered_increment, which is
// the reference's quadratic rewritten without cancellation. Reversal potentials use
// log(a/b) = log a - log b with the constant logs precomputed; fractions that share a
// denominator are combined. row/eca are the FP32 copies of the FP64 tables.
CM_HD float tt2_calc_mixed(const TT2Consts<float> &C, const float *__restrict__ row, const float *__restrict__ eca,
                           TT2Cell<float> &c, Acc &CaSR_a, Acc &Na_a, Acc &K_a, const TT2Het_<float> &g,
                           float V, float i_external, uint32_t &audit) {
  const float svolt = V * 1000.f;
  i_external = i_external * C.inv_stim_unit;
  int Caitab = (int)(C.CaiTabConst2 * c.Ca_i + C.CaiTabConst1);
  if (Caitab < 0 || Caitab >= kRows) {
    audit |= 4u;
    Caitab = Caitab < 0 ? 0 : kRows - 1;
  }
  const float Na_i = Na_a.hi, K_i = K_a.hi, CaSR = CaSR_a.hi;
  const float logKi = flog(K_i);
  const float VminEK = svolt - C.RTONF * (C.logKo - logKi);
  const float VminENa = svolt - C.RTONF * (C.logNao - flog(Na_i));
  const float EKs = C.RTONF * (C.logKoNao - flog(K_i + C.pKNa * Na_i));
  const float e1 = fexp(0.06f * (VminEK - 200.f));
  const float e2 = fexp(0.0002f * (VminEK + 100.f));
  const float e3 = fexp(0.1f * (VminEK - 10.f));
  const float e4 = fexp(-0.5f * VminEK);
  // rec_iK1 = AK1/(AK1+BK1) with AK1 = 0.1/(1+e1), BK1 = (3 e2 + e3)/(1+e4), one division
  const float a1 = 0.1f * (1.f + e4);
  const float rec_iK1 = fdiv(a1, a1 + (3.f * e2 + e3) * (1.f + e1));
  const float I_pCa = fdiv(C.g_pCa * c.Ca_i, C.KpCa + c.Ca_i);
  const float I_pK = row[T2_rec_ipK] * VminEK;
  const float I_to = g.g_to * c.r * c.s * VminEK;
  const float I_Kr = g.g_Kr * C.sqrtKo54 * c.xr1 * c.xr2 * VminEK;
  const float I_Ks = g.g_Ks * c.xs * c.xs * (svolt - EKs);
  const float I_K = I_Kr + I_Ks;
  const float I_K1 = g.g_K1 * C.sqrtKo54 * rec_iK1 * VminEK;
  const float I_bNa = C.g_bNa * VminENa;
  const float I_bCa = C.g_bCa * (svolt - eca[Caitab]);
  const float I_Na = g.g_Na * c.m * c.m * c.m * c.h * c.j * VminENa;
  const float I_CaL = g.g_CaL * c.d * c.f * c.f2 * c.fCa * ((row[T2_CaL_P1] * c.CaSS) - row[T2_CaL_P2]);
  const float I_NaCa = C.kNaCa * (row[T2_NaCa_P1] * Na_i * Na_i * Na_i - row[T2_NaCa_P2] * c.Ca_i);
  const float I_NaK = C.knak * C.KoKmK * fdiv(Na_i, Na_i + C.KmNa) * row[T2_NaK_P1];
  const float I_tot = I_K + I_K1 + I_to + I_Na + I_bNa + I_CaL + I_bCa + I_NaK + I_NaCa + I_pCa + I_pK - i_external;

  const float Caisquare = c.Ca_i * c.Ca_i;
  const float CaSSsquare = c.CaSS * c.CaSS;
  const float CaSR2 = CaSR * CaSR;
  // kCaSR = max_sr - (max_sr - min_sr) / (1 + (EC/CaSR)^2)
  const float kCaSR = C.max_sr - fdiv((C.max_sr - C.min_sr) * CaSR2, CaSR2 + C.EC * C.EC);
  const float k2 = C.ks2 * kCaSR;
  const float k1 = fdiv(C.ks1, kCaSR);
  const float dRq = 1000.f * ((-k2 * c.CaSS * c.Rq) + (C.k4 * (1.f - c.Rq)));
  c.Rq += C.dt * dRq;
  const float k1C2 = k1 * CaSSsquare;
  const float O = fdiv(k1C2 * c.Rq, C.k3 + k1C2);
  const float I_rel = C.Vrel * O * (CaSR - c.CaSS);
  const float I_leak = 0.00036f * (CaSR - c.Ca_i);
  const float I_xfer = C.Vxfer * (c.CaSS - c.Ca_i);
  const float SERCA = fdiv(C.Vmaxup * Caisquare, Caisquare + C.Kupsquare);
  const float dCaSR = C.dt1000 * (SERCA - I_rel - I_leak);
  acc_add(CaSR_a, buffered_increment(CaSR, dCaSR, C.Bufsr, C.Kbufsr));
  const float dCaSS = C.dt1000 * (-I_xfer * C.VcVss + I_rel * C.VsrVss + (-I_CaL * C.inversevssF2 * C.Cm));
  c.CaSS += buffered_increment(c.CaSS, dCaSS, C.Bufss, C.Kbufss);
  const float dCai =
      C.dt1000 * ((-(I_bCa + I_pCa - 2.f * I_NaCa) * C.inverseviF2 * C.Cm) - (SERCA - I_leak) * C.invVcdVsr + I_xfer);
  c.Ca_i += buffered_increment(c.Ca_i, dCai, C.Bufc, C.Kbufc);
  const float dNai = -(I_Na + I_bNa + 3.f * I_NaK + 3.f * I_NaCa) * C.inverseviF * C.Cm;
  acc_add(Na_a, C.dt1000 * dNai);
  const float dKi = -(-i_external + I_K1 + I_to + I_K - 2.f * I_NaK + I_pK) * C.inverseviF * C.Cm;
  acc_add(K_a, C.dt1000 * dKi);
  const float CaSS005 = c.CaSS * 20.f;
  const float den = fdiv(1.f, 1.f + CaSS005 * CaSS005);
  const float FCa_INF = 0.6f * den + 0.4f;
  const float taufca = 0.080f * den + 0.002f;

  c.m = row[T2_m_inf] - (row[T2_m_inf] - c.m) * row[T2_exptau_m];
  c.h = row[T2_h_inf] - (row[T2_h_inf] - c.h) * row[T2_exptau_h];
  c.j = row[T2_j_inf] - (row[T2_j_inf] - c.j) * row[T2_exptau_j];
  c.xr1 = row[T2_Xr1_inf] - (row[T2_Xr1_inf] - c.xr1) * row[T2_exptau_Xr1];
  c.xr2 = row[T2_Xr2_inf] - (row[T2_Xr2_inf] - c.xr2) * row[T2_exptau_Xr2];
  c.xs = row[T2_Xs_inf] - (row[T2_Xs_inf] - c.xs) * row[T2_exptau_Xs];
  c.s = row[T2_s_inf] - (row[T2_s_inf] - c.s) * row[T2_exptau_s];
  c.r = row[T2_r_inf] - (row[T2_r_inf] - c.r) * row[T2_exptau_r];
  c.d = row[T2_d_inf] - (row[T2_d_inf] - c.d) * row[T2_exptau_d];
  c.f = row[T2_f_inf] - (row[T2_f_inf] - c.f) * row[T2_exptau_f];
  c.f2 = row[T2_f2_inf] - (row[T2_f2_inf] - c.f2) * row[T2_exptau_f2];
  c.fCa = FCa_INF - (FCa_INF - c.fCa) * fexp(-fdiv(C.dt, taufca));
  return C.dt * (-I_tot);
}

}  // namespace cm
