/* Test infrastructure only (the oracle). Plain-C FP64 restatement of the reference
 * cell-model update, written from KIT-IBT/CardioMechanics
 *   electrophysiology/src/CellModel/TenTusscher2.cpp            (Init 250-271, Calc 615-906)
 *   electrophysiology/src/CellModel/TenTusscher2Parameters.cpp  (Calculate 313-382, InitTable 384-524)
 *   electrophysiology/src/CellModel/CourtemancheEtAl.cpp        (Init 56-83, Calc 85-187)
 *   electrophysiology/src/CellModel/CourtemancheParameters.cpp  (Init 246-247, Calculate 252-280,
 *                                                                InitTable 282-395)
 *   electrophysiology/src/CellModel/OHaraRudy.cpp               (Init 54-102, Calc 105-663)
 *   electrophysiology/src/CellModel/OHaraRudyParameters.cpp     (Calculate 246-316; no tables)
 *   electrophysiology/src/CellModel/Tomek.cpp                   (Init 55-107, Calc 110-656)
 *   electrophysiology/src/CellModel/TomekParameters.cpp         (Calculate 233-302; no tables)
 *   electrophysiology/src/CellModel/CellModel.h:405-420         (driver stimulus + Vm update)
 * Expressions keep the reference's evaluation order so that, compiled without FP
 * contraction against the same libm, results match the reference bit for bit; the
 * tests pin that against oracle/_ref (the reference compiled from its own sources) and
 * against the committed golden vectors. Used only by tests/, bench.py's CPU baseline and
 * __graft_entry__.smoke() as the checker; never by the product.
 */
#define _POSIX_C_SOURCE 200809L /* pthread barriers under -std=c11 */
#include "cm_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ElphyModelBasis.h:46-56 table geometry. */
#define RANGE_TAB_HALF 200
#define DIVISION_TAB 10
#define D_DIVISION_TAB (1.0 / DIVISION_TAB)

/* ---------------------------------------------------------------- parameter lists */
/* Base parameters (read from the .ev file) followed by derived ones (Calculate()). */
#define TT2_PARAMS(X)                                                                               \
  X(R) X(Tx) X(F) X(init_m) X(init_h) X(init_j) X(init_Xr1) X(init_Xr2) X(init_Xs) X(init_r)       \
  X(init_s) X(init_d) X(init_f) X(init_f2) X(init_fCa) X(init_Rq) X(K_o) X(Ca_o) X(Na_o) X(Vc)      \
  X(Vsr) X(Vss) X(Vrel) X(ks1) X(ks2) X(k3) X(k4) X(EC) X(max_sr) X(min_sr) X(Vxfer) X(Bufc)        \
  X(Kbufc) X(Bufsr) X(Kbufsr) X(Bufss) X(Kbufss) X(Vmaxup) X(Kup) X(C) X(g_Kr) X(pKNa) X(g_Ks)      \
  X(g_K1) X(g_to) X(g_Na) X(g_bNa) X(KmK) X(KmNa) X(knak) X(g_CaL) X(g_bCa) X(kNaCa) X(KmNai)       \
  X(KmCa) X(ksat) X(n) X(g_pCa) X(KpCa) X(g_pK) X(init_V_m) X(init_Cai) X(init_CaSR) X(init_CaSS)  \
  X(init_Nai) X(init_Ki) X(CaiMin) X(CaiMax) X(s_inf_vHalf) X(tau_s_f1) X(tau_s_slope1)            \
  X(tau_s_vHalf1) X(tau_s_enable) X(tau_s_add) X(m_Xr1_1) X(m_Xr1_2) X(a_Xr1_1) X(a_Xr1_2)         \
  X(b_Xr1_1) X(b_Xr1_2) X(K_Q10Xr1) X(m_Xr2_1) X(m_Xr2_2) X(a_Xr2_1) X(a_Xr2_2) X(b_Xr2_1)         \
  X(b_Xr2_2) X(K_Q10Xr2) X(m_Xs_1) X(m_Xs_2) X(a_Xs_1) X(a_Xs_2) X(b_Xs_1) X(b_Xs_2)               \
  X(tau_Xs_add) X(K_Q10Xs) X(stim_duration) X(Amp) X(Vcell)                                        \
  X(RTONF) X(inverseRTONF) X(vi) X(inverseviF) X(inverseviF2) X(inversevssF2) X(VcdVsr)            \
  X(Kupsquare) X(BufcPKbufc) X(KmNai3) X(Nao3) X(StepCai)

#define CRN_PARAMS(X)                                                                               \
  X(R) X(Tx) X(F) X(C_m) X(Vcell) X(Vcell_outside) X(part_i) X(part_up) X(part_rel) X(Tfac) X(K_o)  \
  X(Na_o) X(Ca_o) X(g_Na) X(g_to) X(g_Kr) X(g_Ks) X(g_CaL) X(g_K1) X(g_bNa) X(g_bCa) X(I_NaKmax)    \
  X(k_mNai) X(k_mKo) X(I_pCamax) X(k_mpCa) X(k_NaCa) X(k_mNa) X(k_mCa) X(k_sat) X(gamm)             \
  X(CMDNmax) X(TRPNmax) X(CSQNmax) X(K_mcmdn) X(K_mtrpn) X(K_mcsqn) X(k_rel) X(k_up) X(I_upmax)     \
  X(Ca_upmax) X(t_tr) X(shiftm) X(shifth) X(shiftj) X(shiftoa) X(C_oa_1) X(C_oa_2) X(C_oa_3)        \
  X(C_oa_4) X(C_oa_5) X(C_oa_6) X(CaL_fT_1) X(Init_Na_i) X(Init_K_i) X(Init_m) X(Init_oa)           \
  X(Init_ua) X(Init_d) X(Init_f_Ca) X(Init_Ca_i) X(Init_Ca_up) X(Init_Ca_rel) X(Init_h) X(Init_j)   \
  X(Init_oi) X(Init_ui) X(Init_Xr) X(Init_Xs) X(Init_f) X(Init_u) X(Init_v) X(Init_w) X(Init_Vm)    \
  X(ua_a1) X(ua_a2) X(ua_a3) X(ua_a4) X(ua_a5) X(ua_b1) X(ua_b2) X(ua_b3) X(ua_m1) X(ua_m2)         \
  X(ua_KQ10) X(ui_a1) X(ui_a2) X(ui_a3) X(ui_a4) X(ui_b1) X(ui_b2) X(ui_m1) X(ui_m2) X(ui_KQ10)     \
  X(g_Kur1) X(g_Kur2) X(g_Kur3) X(g_Kur4) X(g_K1_1) X(g_K1_2) X(Xr_a1) X(Xr_a2) X(Xr_a3) X(Xr_b1)   \
  X(Xr_b2) X(Xr_KQ10) X(Xr_m1) X(Xr_m2) X(g_Kr1) X(g_Kr2) X(Xs_a1) X(Xs_a2) X(Xs_a3) X(Xs_b1)       \
  X(Xs_b2) X(Xs_KQ10) X(Xs_m1) X(Xs_m2) X(m_a1) X(m_a2) X(m_b1) X(m_b2) X(h_a1) X(h_a2) X(h_b1)     \
  X(h_b2) X(h_b3) X(h_b4) X(h_b5) X(h_b6) X(j_a1) X(j_a2) X(j_a3) X(j_a4) X(j_a5) X(j_b1) X(j_b2)   \
  X(j_b3) X(j_b4) X(j_b5) X(j_b6) X(tau_j_mult) X(tau_f_mult) X(E_rL) X(ISAC_SWITCH) X(alpha)       \
  X(G_sac) X(K_sac) X(E_sac) X(Init_Ca_TRPN) X(beta1) X(Ca_T50) X(k_TRPN) X(n_TRPN)                 \
  X(RTdF) X(FdRT) X(RTd2F) X(Vi) X(Vup) X(Vrel) X(VupdVi) X(VreldVi) X(VreldVup) X(CmdFvi)          \
  X(Cmd2F) X(csqnkm) X(kmcsqnm2) X(kkmcsqn) X(cmdnkm) X(kmcmdnm2) X(kkmcmdn) X(kupleak) X(dt_tr)

/* O'Hara-Rudy 2011 as compiled in the reference (ISAC, TRPN, HF, HFM, DUTTA and PASSINI all
 * defined, OHaraRudyParameters.h:20-36): the .ev parameters in the order of
 * NS_OHaraRudyParameters::varType (OHaraRudyParameters.h:40-180), then the values
 * OHaraRudyParameters::Calculate derives (246-316). */
#define ORD_PARAMS(X)                                                                               \
  X(amplitude) X(duration) X(celltype) X(Na_o) X(Ca_o) X(K_o) X(INaF_Multiplier) X(INaL_Multiplier) \
  X(Ito_Multiplier) X(PCa_Multiplier) X(IKr_Multiplier) X(IKs_Multiplier) X(IK1_Multiplier)         \
  X(INaCa_Multiplier) X(INaK_Multiplier) X(IKb_Multiplier) X(INab_Multiplier) X(ICab_Multiplier)    \
  X(IpCa_Multiplier) X(Init_Vm) X(Init_Na_i) X(Init_Na_ss) X(Init_K_i) X(Init_K_ss) X(Init_Ca_i)    \
  X(Init_Ca_ss) X(Init_Ca_nsr) X(Init_Ca_jsr) X(Init_m) X(Init_h_fast) X(Init_h_slow) X(Init_j)      \
  X(Init_h_CaMK_slow) X(Init_j_CaMK) X(Init_m_L) X(Init_h_L) X(Init_h_L_CaMK) X(Init_a)             \
  X(Init_i_fast) X(Init_i_slow) X(Init_a_CaMK) X(Init_i_CaMK_fast) X(Init_i_CaMK_slow) X(Init_d)    \
  X(Init_f_fast) X(Init_f_slow) X(Init_f_Ca_fast) X(Init_f_Ca_slow) X(Init_j_Ca) X(Init_n)          \
  X(Init_f_CaMK_fast) X(Init_f_Ca_CaMK_fast) X(Init_x_r_fast) X(Init_x_r_slow) X(Init_x_s1)         \
  X(Init_x_s2) X(Init_x_K1) X(Init_J_rel_NP) X(Init_J_rel_CaMK) X(Init_CaMK_trap) X(ISAC_SWITCH)    \
  X(alpha) X(G_sac) X(K_sac) X(E_sac) X(Init_Ca_TRPN) X(beta1) X(Ca_T50) X(k_TRPN) X(n_TRPN)        \
  X(HFM_Multiplier) X(HF_Gomez_1) X(HF_Gomez_2) X(HF_Gomez_3) X(HF_Gomez_4) X(HF_Gomez_5)           \
  X(HF_Gomez_6) X(HF_Gomez_7) X(HF_Gomez_8) X(HF_Gomez_9) X(HF_Gomez_0)                             \
  X(R) X(T) X(F) X(L) X(r) X(tau_h_L) X(A_h_fast) X(A_h_slow) X(v_cell) X(A_geo) X(A_cap) X(v_myo)  \
  X(v_nsr) X(v_jsr) X(v_ss) X(P_CaNa) X(P_CaK) X(P_Ca_CaMK) X(P_CaNa_CaMK) X(P_CaK_CaMK)            \
  X(A_f_fast) X(A_f_slow) X(k_Na1) X(k_Na2) X(k_asymm) X(k_Ca_on) X(k_Ca_off) X(k_m_1) X(k_p_2)     \
  X(k_p_4) X(MgADP) X(MgATP) X(K_MgATP) X(beta_tau) X(P_Ca) X(h_10) X(h_11) X(h_12) X(k_1) X(k_2)   \
  X(k_5) X(beta_1) X(alpha_2) X(alpha_4) X(alpha_rel) X(beta_tau_CaMK) X(alpha_rel_CaMK)            \
  X(tau_h_LCaMK) X(RToverF)

/* Tomek 2019 (ToR-ORd) as compiled in the reference (ISAC and TRPN defined,
 * TomekParameters.h:18-23): NS_TomekParameters::varType order (TomekParameters.h:28-165), the
 * values TomekParameters::Calculate derives (233-302) in the middle of the list as there. */
#define TOM_PARAMS(X)                                                                               \
  X(amplitude) X(duration) X(celltype) X(Na_o) X(Ca_o) X(K_o) X(Cl_o) X(INaF_Multiplier)            \
  X(INaL_Multiplier) X(Ito_Multiplier) X(PCa_Multiplier) X(IKr_Multiplier) X(IKs_Multiplier)        \
  X(IK1_Multiplier) X(INaCa_Multiplier) X(INaK_Multiplier) X(IKb_Multiplier) X(INab_Multiplier)     \
  X(ICab_Multiplier) X(IpCa_Multiplier) X(Init_Vm) X(Init_Na_i) X(Init_Na_ss) X(Init_K_i)           \
  X(Init_K_ss) X(Init_Ca_i) X(Init_Ca_ss) X(Init_Ca_nsr) X(Init_Ca_jsr) X(Init_Cl_i) X(Init_m)      \
  X(Init_A_h) X(Init_B_h) X(Init_h) X(Init_A_j) X(Init_B_j) X(Init_j) X(Init_h_p) X(Init_j_p)       \
  X(Init_m_L) X(Init_h_L) X(Init_h_L_CaMK) X(Init_a) X(Init_i_fast) X(Init_i_slow) X(Init_a_CaMK)   \
  X(Init_i_CaMK_fast) X(Init_i_CaMK_slow) X(Init_d) X(Init_f_fast) X(Init_f_slow) X(Init_f_Ca_fast) \
  X(Init_f_Ca_slow) X(Init_j_Ca) X(Init_n_ss) X(Init_n_i) X(Init_f_CaMK_fast)                       \
  X(Init_f_Ca_CaMK_fast) X(Init_C_0) X(Init_C_1) X(Init_C_2) X(Init_O) X(Init_I) X(Init_x_s1)       \
  X(Init_x_s2) X(Init_J_rel_NP) X(Init_J_rel_CaMK) X(Init_CaMK_trap)                                \
  X(R) X(T) X(F) X(L) X(r) X(tau_h_L) X(A_h) X(v_cell) X(A_geo) X(A_cap) X(v_myo) X(v_nsr) X(v_jsr) \
  X(v_ss) X(P_CaNa) X(P_CaK) X(P_Ca_CaMK) X(P_CaNa_CaMK) X(P_CaK_CaMK) X(A_f_fast) X(A_f_slow)      \
  X(k_Na1) X(k_Na2) X(k_asymm) X(k_Ca_on) X(k_Ca_off) X(k_m_1) X(k_p_2) X(k_p_4) X(MgADP) X(MgATP)  \
  X(K_MgATP) X(beta_tau) X(P_Ca) X(h_10) X(h_11) X(h_12) X(k_1) X(k_2) X(k_5) X(beta_1) X(alpha_2)  \
  X(alpha_4) X(alpha_rel) X(beta_tau_CaMK) X(alpha_rel_CaMK) X(tau_h_LCaMK) X(RToverF)              \
  X(ISAC_SWITCH) X(alpha) X(G_sac) X(K_sac) X(E_sac) X(Init_Ca_TRPN) X(beta1) X(Ca_T50) X(k_TRPN)   \
  X(n_TRPN)

#define ENUM_TT2(x) T_##x,
#define ENUM_CRN(x) C_##x,
#define ENUM_ORD(x) O_##x,
#define ENUM_TOM(x) M_##x,
#define NAME(x) #x,
enum { TT2_PARAMS(ENUM_TT2) T_LAST };
enum { CRN_PARAMS(ENUM_CRN) C_LAST };
enum { ORD_PARAMS(ENUM_ORD) O_LAST };
enum { TOM_PARAMS(ENUM_TOM) M_LAST };
static const char *tt2_names[] = {TT2_PARAMS(NAME)};
static const char *crn_names[] = {CRN_PARAMS(NAME)};
static const char *ord_names[] = {ORD_PARAMS(NAME)};
static const char *tom_names[] = {TOM_PARAMS(NAME)};

/* The reference backup block of Tomek (GetBase() = &m, Tomek.h:33-52): 48 states (A_h, B_h, A_j,
 * B_j are rates Calc recomputes; Cl_i never changes), then the 36 values Calc stores. */
enum {
  MB_m, MB_A_h, MB_B_h, MB_h, MB_A_j, MB_B_j, MB_j, MB_h_p, MB_j_p, MB_m_L, MB_h_L, MB_h_L_CaMK, MB_a,
  MB_i_fast, MB_i_slow, MB_a_CaMK, MB_i_CaMK_fast, MB_i_CaMK_slow, MB_d, MB_f_fast, MB_f_slow, MB_f_Ca_fast,
  MB_f_Ca_slow, MB_j_Ca, MB_f_CaMK_fast, MB_f_Ca_CaMK_fast, MB_n_ss, MB_n_i, MB_C_0, MB_C_1, MB_C_2, MB_O, MB_I,
  MB_x_s1, MB_x_s2, MB_Na_i, MB_Na_ss, MB_K_i, MB_K_ss, MB_Ca_i, MB_Ca_ss, MB_Ca_nsr, MB_Ca_jsr, MB_Cl_i,
  MB_CaMK_trap, MB_J_rel_NP, MB_J_rel_CaMK, MB_Ca_TRPN,
  MB_I_Na, MB_I_Na_late, MB_I_to, MB_I_CaL, MB_I_CaNa, MB_I_CaK, MB_I_CaL_i, MB_I_CaL_ss, MB_I_CaNa_i,
  MB_I_CaNa_ss, MB_I_CaK_i, MB_I_CaK_ss, MB_I_Kr, MB_I_Ks, MB_I_K1, MB_I_NaCa_i, MB_I_NaCa_ss, MB_I_NaK,
  MB_I_CaCl_junc, MB_I_CaCl_sl, MB_I_CaCl, MB_I_Nab, MB_I_Cab, MB_I_Kb, MB_I_Clb, MB_I_pCa, MB_J_diff_Na,
  MB_J_diff_Ca, MB_J_diff_K, MB_J_leak, MB_J_rel, MB_J_tr, MB_J_up, MB_cur_I_tot, MB_I_tot, MB_I_SAC,
  TOM_BLOCK
};

/* The reference backup block of OHaraRudy (GetBase() = &m, OHaraRudy.h:31-52): 42 states,
 * h_CaMK_fast included although Calc never touches it, then the 17 currents it stores. */
enum {
  OB_m, OB_h_fast, OB_h_slow, OB_j, OB_h_CaMK_fast, OB_h_CaMK_slow, OB_j_CaMK, OB_m_L, OB_h_L, OB_h_L_CaMK,
  OB_a, OB_i_fast, OB_i_slow, OB_a_CaMK, OB_i_CaMK_fast, OB_i_CaMK_slow, OB_d, OB_f_fast, OB_f_slow,
  OB_f_Ca_fast, OB_f_Ca_slow, OB_j_Ca, OB_n, OB_f_CaMK_fast, OB_f_Ca_CaMK_fast, OB_x_r_fast, OB_x_r_slow,
  OB_x_s1, OB_x_s2, OB_x_K1, OB_Na_i, OB_Na_ss, OB_K_i, OB_K_ss, OB_Ca_i, OB_Ca_ss, OB_Ca_nsr, OB_Ca_jsr,
  OB_CaMK_trap, OB_J_rel_NP, OB_J_rel_CaMK, OB_Ca_TRPN,
  OB_I_Na_fast, OB_I_Na_late, OB_I_to, OB_I_CaL, OB_I_CaNa, OB_I_CaK, OB_I_Kr, OB_I_Ks, OB_I_K1,
  OB_I_NaCa_i, OB_I_NaCa_ss, OB_I_NaK, OB_I_Nab, OB_I_Cab, OB_I_Kb, OB_I_pCa, OB_I_SAC,
  ORD_BLOCK
};

/* Lookup tables, in this file's order. */
#define TT2_TABLES(X)                                                                               \
  X(m_inf) X(h_inf) X(j_inf) X(Xr1_inf) X(Xr2_inf) X(Xs_inf) X(s_inf) X(r_inf) X(d_inf) X(f_inf)    \
  X(f2_inf) X(exptau_m) X(exptau_h) X(exptau_j) X(exptau_Xr1) X(exptau_Xr2) X(exptau_Xs)            \
  X(exptau_s) X(exptau_r) X(exptau_d) X(exptau_f) X(exptau_f2) X(NaK_P1) X(rec_ipK) X(NaCa_P1)      \
  X(NaCa_P2) X(CaL_P1) X(CaL_P2) X(ECA)
#define CRN_TABLES(X)                                                                               \
  X(m_m) X(exptau_m) X(m_h) X(exptau_h) X(m_j) X(exptau_j) X(m_oa) X(exptau_oa) X(m_oi)             \
  X(exptau_oi) X(m_ua) X(exptau_ua) X(m_ui) X(exptau_ui) X(m_Xr) X(exptau_Xr) X(m_Xs) X(exptau_Xs)  \
  X(m_d) X(exptau_d) X(m_f) X(exptau_f) X(m_w) X(exptau_w) X(expVm) X(CK1) X(g_Kur) X(CKr) X(CNaK)  \
  X(CNaCa) X(exp250_exp50)
#define TENUM_TT2(x) TT_##x,
#define TENUM_CRN(x) TC_##x,
enum { TT2_TABLES(TENUM_TT2) TT_LAST };
enum { CRN_TABLES(TENUM_CRN) TC_LAST };
static const char *tt2_tnames[] = {TT2_TABLES(NAME)};
static const char *crn_tnames[] = {CRN_TABLES(NAME)};

int cmo_n_params(int model) {
  return model == CMO_TT2 ? T_LAST
                          : (model == CMO_CRN ? C_LAST : (model == CMO_ORD ? O_LAST : (model == CMO_TOM ? M_LAST : -1)));
}
const char *cmo_param_name(int model, int i) {
  if (i < 0 || i >= cmo_n_params(model)) return 0;
  return model == CMO_TT2 ? tt2_names[i]
                          : (model == CMO_CRN ? crn_names[i] : (model == CMO_ORD ? ord_names[i] : tom_names[i]));
}
int cmo_param_index(int model, const char *name) {
  int n = cmo_n_params(model);
  for (int i = 0; i < n; i++)
    if (!strcmp(cmo_param_name(model, i), name)) return i;
  return -1;
}
int cmo_state_doubles(int model) {
  return model == CMO_TT2 ? 36
                          : (model == CMO_CRN ? 22 : (model == CMO_ORD ? ORD_BLOCK : (model == CMO_TOM ? TOM_BLOCK : -1)));
}
/* O'Hara-Rudy evaluates every gate directly (its InitTable loop body is empty,
 * OHaraRudyParameters.cpp:318-441): no tables. */
int cmo_n_tables(int model) {
  return model == CMO_TT2 ? TT_LAST : (model == CMO_CRN ? TC_LAST : (model == CMO_ORD || model == CMO_TOM ? 0 : -1));
}
const char *cmo_table_name(int model, int k) {
  if (k < 0 || k >= cmo_n_tables(model)) return 0;
  return model == CMO_TT2 ? tt2_tnames[k] : crn_tnames[k];
}

/* ---------------------------------------------------------------- TT2 */
#define P_(x) P[T_##x]
#define TB(x) (tables + (size_t)TT_##x * CMO_RTDT)

/* TenTusscher2Parameters::Calculate (313-338): derived quantities. */
static void tt2_derive(double *P) {
  P_(RTONF) = P_(R) * P_(Tx) / P_(F);
  P_(inverseRTONF) = 1 / P_(RTONF);
  P_(vi) = 0.016404; /* overwritten constant, TenTusscher2Parameters.cpp:322 */
  P_(inverseviF) = 1 / (P_(vi) * P_(F));
  P_(inverseviF2) = 1. / (2 * P_(vi) * P_(F));
  P_(inversevssF2) = 1 / (2 * (P_(vi) / 300.) * P_(F));
  P_(VcdVsr) = P_(Vc) / P_(Vsr);
  P_(Kupsquare) = P_(Kup) * P_(Kup);
  P_(BufcPKbufc) = P_(Bufc) + P_(Kbufc);
  P_(KmNai3) = P_(KmNai) * P_(KmNai) * P_(KmNai);
  P_(Nao3) = P_(Na_o) * P_(Na_o) * P_(Na_o);
  P_(StepCai) = (P_(CaiMax) - P_(CaiMin)) / CMO_RTDT;
}

/* TenTusscher2Parameters::InitTable (384-485). */
static void tt2_tables(const double *P, double tinc, double *tables) {
  for (double V = -RANGE_TAB_HALF + .0001; V < RANGE_TAB_HALF; V += D_DIVISION_TAB) {
    int Vi = (int)(DIVISION_TAB * (RANGE_TAB_HALF + V) + .5);
    if (Vi < 0 || Vi >= CMO_RTDT) continue;
    const double rec_iNaK =
        (1. / (1. + 0.1245 * exp(-0.1 * V * (P_(inverseRTONF))) + 0.0353 * exp(-V * (P_(inverseRTONF)))));
    TB(NaK_P1)[Vi] = rec_iNaK;
    TB(rec_ipK)[Vi] = P_(g_pK) / (1. + exp((25. - V) / 5.98));
    const double a_m = 1. / (1. + exp((-60. - V) / 5.));
    const double b_m = 0.1 / (1. + exp((V + 35.) / 5.)) + 0.10 / (1. + exp((V - 50.) / 200.));
    const double tau_m = a_m * b_m;
    TB(m_inf)[Vi] = 1. / ((1. + exp((-56.86 - V) / 9.03)) * (1. + exp((-56.86 - V) / 9.03)));
    double tau_h, tau_j;
    if (V >= -40.) {
      const double AH_1 = 0.;
      const double BH_1 = (0.77 / (0.13 * (1. + exp(-(V + 10.66) / 11.1))));
      tau_h = 1.0 / (AH_1 + BH_1);
    } else {
      const double AH_2 = (0.057 * exp(-(V + 80.) / 6.8));
      const double BH_2 = (2.7 * exp(0.079 * V) + (3.1e5) * exp(0.3485 * V));
      tau_h = 1.0 / (AH_2 + BH_2);
    }
    TB(h_inf)[Vi] = 1. / ((1. + exp((V + 71.55) / 7.43)) * (1. + exp((V + 71.55) / 7.43)));
    if (V >= -40.) {
      const double AJ_1 = 0.;
      const double BJ_1 = (0.6 * exp((0.057) * V) / (1. + exp(-0.1 * (V + 32.))));
      tau_j = 1.0 / (AJ_1 + BJ_1);
    } else {
      const double AJ_2 = (((-2.5428e4) * exp(0.2444 * V) - (6.948e-6) * exp(-0.04391 * V)) * (V + 37.78) /
                           (1. + exp(0.311 * (V + 79.23))));
      const double BJ_2 = (0.02424 * exp(-0.01052 * V) / (1. + exp(-0.1378 * (V + 40.14))));
      tau_j = 1.0 / (AJ_2 + BJ_2);
    }
    TB(j_inf)[Vi] = TB(h_inf)[Vi];
    TB(Xr1_inf)[Vi] = 1. / (1. + exp((P_(m_Xr1_1) - V) / (P_(m_Xr1_2))));
    const double a_Xr1 = 450. / (1. + exp((P_(a_Xr1_1) - V) / (P_(a_Xr1_2))));
    const double b_Xr1 = 6. / (1. + exp((V - (P_(b_Xr1_1))) / (P_(b_Xr1_2))));
    const double tau_Xr1 = a_Xr1 * b_Xr1 * fabs(P_(K_Q10Xr1));
    TB(Xr2_inf)[Vi] = 1. / (1. + exp((V - (P_(m_Xr2_1))) / (P_(m_Xr2_2))));
    const double a_Xr2 = 3. / (1. + exp((P_(a_Xr2_1) - V) / (P_(a_Xr2_2))));
    const double b_Xr2 = 1.12 / (1. + exp((V - (P_(b_Xr2_1))) / (P_(b_Xr2_2))));
    const double tau_Xr2 = a_Xr2 * b_Xr2 * fabs(P_(K_Q10Xr2));
    TB(Xs_inf)[Vi] = 1. / (1. + exp((P_(m_Xs_1) - V) / P_(m_Xs_2)));
    const double a_Xs = (1400. / (sqrt(1. + exp((P_(a_Xs_1) - V) / P_(a_Xs_2)))));
    const double b_Xs = (1. / (1. + exp((V - P_(b_Xs_1)) / P_(b_Xs_2))));
    const double tau_Xs = (a_Xs * b_Xs + P_(tau_Xs_add)) * fabs(P_(K_Q10Xs));
    TB(r_inf)[Vi] = 1. / (1. + exp((20 - V) / 6.));
    TB(s_inf)[Vi] = 1. / (1. + exp((V + (P_(s_inf_vHalf))) / 5.));
    const double tau_r = 9.5 * exp(-(V + 40.) * (V + 40.) / 1800.) + 0.8;
    const double tau_s =
        P_(tau_s_f1) * exp(-(V + (P_(tau_s_vHalf1))) * (V + (P_(tau_s_vHalf1))) / P_(tau_s_slope1)) +
        P_(tau_s_enable) * 5. / (1. + exp((V - 20.) / 5.)) + P_(tau_s_add);
    TB(d_inf)[Vi] = 1. / (1. + exp((-8. - V) / 7.5));
    const double a_d = 1.4 / (1. + exp((-35 - V) / 13)) + 0.25;
    const double b_d = 1.4 / (1. + exp((V + 5) / 5));
    const double c_d = 1. / (1. + exp((50 - V) / 20));
    const double tau_d = a_d * b_d + c_d;
    TB(f_inf)[Vi] = 1. / (1. + exp((V + 20) / 7));
    const double V27square = (V + 27) * (V + 27);
    const double exsquare = V27square / (15 * 15);
    const double a_f = 1102.5 * exp(-exsquare);
    const double b_f = 200. / (1. + exp((13 - V) / 10.));
    const double g_f = (180. / (1. + exp((V + 30) / 10.))) + 20.;
    const double tau_f = a_f + b_f + g_f;
    TB(f2_inf)[Vi] = (.67 / (1. + exp((V + 35.) / 7.))) + .33;
    const double a_f2 = 600. * exp(-(V + 25) * (V + 25) / 170.);
    const double b_f2 = 31. / (1. + exp((25 - V) / 10.));
    const double c_f2 = 16. / (1. + exp((V + 30) / 10.));
    const double tau_f2 = a_f2 + b_f2 + c_f2;
    TB(NaCa_P1)[Vi] = ((1. / ((P_(KmNai3)) + (P_(Nao3)))) * (1. / ((P_(KmCa)) + (P_(Ca_o)))) *
                       (1. / (1. + (P_(ksat)) * exp(((P_(n)) - 1.) * V * (P_(inverseRTONF)))))) *
                      (exp((P_(n)) * V * (P_(inverseRTONF))) * (P_(Ca_o)));
    TB(NaCa_P2)[Vi] = ((1. / ((P_(KmNai3)) + (P_(Nao3)))) * (1. / ((P_(KmCa)) + (P_(Ca_o)))) *
                       (1. / (1. + (P_(ksat)) * exp(((P_(n)) - 1.) * V * (P_(inverseRTONF)))))) *
                      (exp(((P_(n)) - 1) * V / (P_(RTONF))) * (P_(Na_o)) * (P_(Na_o)) * (P_(Na_o)) * 2.5);
    TB(CaL_P1)[Vi] = 4 * (V - 15.) * (P_(F)) / (P_(RTONF)) * (0.25 * exp(2 * (V - 15.) / (P_(RTONF)))) /
                     (exp(2 * (V - 15.) / (P_(RTONF))) - 1.);
    TB(CaL_P2)[Vi] = 4 * (V - 15.) * ((P_(F)) / (P_(RTONF))) * (1 * (P_(Ca_o))) /
                     (exp(2 * (V - 15.) / (P_(RTONF))) - 1.);
    const double HT = tinc * 1000;
    TB(exptau_m)[Vi] = exp(-HT / tau_m);
    TB(exptau_h)[Vi] = exp(-HT / tau_h);
    TB(exptau_j)[Vi] = exp(-HT / tau_j);
    TB(exptau_Xr1)[Vi] = exp(-HT / tau_Xr1);
    TB(exptau_Xr2)[Vi] = exp(-HT / tau_Xr2);
    TB(exptau_Xs)[Vi] = exp(-HT / tau_Xs);
    TB(exptau_s)[Vi] = exp(-HT / tau_s);
    TB(exptau_r)[Vi] = exp(-HT / tau_r);
    TB(exptau_d)[Vi] = exp(-HT / tau_d);
    TB(exptau_f)[Vi] = exp(-HT / tau_f);
    TB(exptau_f2)[Vi] = exp(-HT / tau_f2);
    const double Cai = Vi * (P_(StepCai));
    TB(ECA)[Vi] = ((P_(RTONF)) * 0.5) * (log(((P_(Ca_o)) / Cai)));
  }
}

/* Block offsets (TenTusscher2.h:77-123). */
enum { S_Cai = 0, S_CaSR, S_CaSS, S_Nai, S_Ki, S_Array, S_m = 23, S_h, S_j, S_xr1, S_xr2, S_xs, S_r, S_s,
       S_d, S_f, S_f2, S_fCa, S_Rq };

/* TenTusscherEtAl2::Init (250-271). */
static void tt2_init(const double *P, double *b) {
  memset(b, 0, 36 * sizeof(double));
  b[S_m] = P_(init_m); b[S_h] = P_(init_h); b[S_j] = P_(init_j); b[S_xr1] = P_(init_Xr1);
  b[S_xr2] = P_(init_Xr2); b[S_xs] = P_(init_Xs); b[S_r] = P_(init_r); b[S_s] = P_(init_s);
  b[S_d] = P_(init_d); b[S_f] = P_(init_f); b[S_f2] = P_(init_f2); b[S_fCa] = P_(init_fCa);
  b[S_Rq] = P_(init_Rq); b[S_Cai] = P_(init_Cai); b[S_CaSR] = P_(init_CaSR); b[S_CaSS] = P_(init_CaSS);
  b[S_Nai] = P_(init_Nai); b[S_Ki] = P_(init_Ki);
}

/* TenTusscherEtAl2::Calc (615-906), useCaTab on, no ischemia/Markov/SAC. */
static double tt2_calc(const double *P, const double *tables, double *b, double tinc, double V,
                       double i_external) {
  double Ca_i = b[S_Cai], CaSR = b[S_CaSR], CaSS = b[S_CaSS], Na_i = b[S_Nai], K_i = b[S_Ki];
  double m = b[S_m], h = b[S_h], j = b[S_j], xr1 = b[S_xr1], xr2 = b[S_xr2], xs = b[S_xs];
  double r = b[S_r], s = b[S_s], d = b[S_d], f = b[S_f], f2 = b[S_f2], fCa = b[S_fCa], Rq = b[S_Rq];
  const double svolt = V * 1000;
  const int Vi = (int)(DIVISION_TAB * (RANGE_TAB_HALF + svolt) + .5);
  i_external = i_external / 2.29656e-2;
  /* function-level statics in the reference (638-640); one parameter set here */
  const double CaiTabConst1 = -P_(CaiMin) / P_(StepCai) + 0.5;
  const double CaiTabConst2 = 1. / P_(StepCai);
  const int Caitab = (int)(CaiTabConst2 * Ca_i + CaiTabConst1);
  const double K_o_int = P_(K_o);
  const double RTONF = P_(RTONF);
  const double EK = RTONF * (log((K_o_int / K_i)));
  const double VminEK = svolt - EK;
  const double ENa = RTONF * (log((P_(Na_o) / Na_i)));
  const double VminENa = svolt - ENa;
  const double EKs = RTONF * (log((K_o_int + P_(pKNa) * P_(Na_o)) / (K_i + P_(pKNa) * Na_i)));
  const double AK1 = 0.1 / (1. + exp(0.06 * (VminEK - 200)));
  const double BK1 = (3. * exp(0.0002 * (VminEK + 100)) + exp(0.1 * (VminEK - 10))) / (1. + exp(-0.5 * (VminEK)));
  const double rec_iK1 = AK1 / (AK1 + BK1);
  const double I_pCa = P_(g_pCa) * Ca_i / (P_(KpCa) + Ca_i);
  const double I_pK = TB(rec_ipK)[Vi] * VminEK;
  const double I_to = P_(g_to) * r * s * VminEK;
  const double I_Kr = P_(g_Kr) * sqrt(K_o_int / 5.4) * xr1 * xr2 * VminEK;
  const double I_Ks = P_(g_Ks) * xs * xs * (svolt - EKs);
  const double I_K = I_Kr + I_Ks;
  const double I_K1 = P_(g_K1) * sqrt(K_o_int / 5.4) * rec_iK1 * VminEK;
  const double I_bNa = P_(g_bNa) * VminENa;
  const double I_bCa = P_(g_bCa) * (svolt - (TB(ECA)[Caitab]));
  const double I_Na = P_(g_Na) * m * m * m * h * j * VminENa;
  const double I_CaL = P_(g_CaL) * d * f * f2 * fCa * (((TB(CaL_P1)[Vi]) * CaSS) - (TB(CaL_P2)[Vi]));
  const double I_NaCa = P_(kNaCa) * (TB(NaCa_P1)[Vi]) * Na_i * Na_i * Na_i - P_(kNaCa) * (TB(NaCa_P2)[Vi]) * Ca_i;
  const double I_NaK =
      P_(knak) * (K_o_int / (K_o_int + P_(KmK))) * (Na_i / (Na_i + P_(KmNa))) * (TB(NaK_P1)[Vi]);
  const double I_tot = I_K + I_K1 + I_to + I_Na + I_bNa + I_CaL + I_bCa + I_NaK + I_NaCa + I_pCa + I_pK - i_external;

  const double Vss = P_(Vss), Cm = P_(C), max_sr = P_(max_sr), Bufsr = P_(Bufsr), EC = P_(EC);
  const double Kbufsr = P_(Kbufsr), Bufss = P_(Bufss), Kbufss = P_(Kbufss), Kbufc = P_(Kbufc);
  const double inverseviF = P_(inverseviF);
  const double Caisquare = Ca_i * Ca_i;
  const double CaSSsquare = CaSS * CaSS;
  const double kCaSR = max_sr - ((max_sr - P_(min_sr)) / (1 + (EC / CaSR) * (EC / CaSR)));
  const double k2 = P_(ks2) * kCaSR;
  const double k1 = P_(ks1) / kCaSR;
  const double dRq = 1000.0 * ((-k2 * CaSS * Rq) + (P_(k4) * (1.0 - Rq)));
  Rq += tinc * dRq;
  const double O = k1 * CaSSsquare * Rq / (P_(k3) + k1 * CaSSsquare);
  const double I_rel = P_(Vrel) * O * (CaSR - CaSS);
  const double I_leak = 0.00036 * (CaSR - Ca_i);
  const double I_xfer = P_(Vxfer) * (CaSS - Ca_i);
  const double SERCA = P_(Vmaxup) / (1. + (P_(Kupsquare) / Caisquare));
  const double dCaSR = tinc * 1000.0 * (SERCA - I_rel - I_leak);
  const double CaCSQN = Bufsr * CaSR / (CaSR + Kbufsr);
  const double bjsr = Bufsr - CaCSQN - dCaSR - CaSR + Kbufsr;
  const double cjsr = Kbufsr * (CaCSQN + dCaSR + CaSR);
  CaSR = (sqrt(bjsr * bjsr + 4 * cjsr) - bjsr) / 2.;
  const double CaSSBuf = Bufss * CaSS / (CaSS + Kbufss);
  const double dCaSS =
      tinc * 1000.0 * (-I_xfer * (P_(Vc) / Vss) + I_rel * (P_(Vsr) / Vss) + (-I_CaL * P_(inversevssF2) * Cm));
  const double bjss = Bufss - CaSSBuf - dCaSS - CaSS + Kbufss;
  const double cjss = Kbufss * (CaSSBuf + dCaSS + CaSS);
  CaSS = (sqrt(bjss * bjss + 4. * cjss) - bjss) / 2.;
  const double CaBuf = P_(Bufc) * Ca_i / (Ca_i + Kbufc);
  const double dCai =
      tinc * 1000.0 * ((-(I_bCa + I_pCa - 2 * I_NaCa) * P_(inverseviF2) * Cm) - (SERCA - I_leak) * (1.0 / P_(VcdVsr)) + I_xfer);
  const double bc = P_(BufcPKbufc) - CaBuf - dCai - Ca_i;
  const double cc = Kbufc * (CaBuf + dCai + Ca_i);
  Ca_i = (sqrt(bc * bc + 4 * cc) - bc) / 2.;
  const double dNai = -(I_Na + I_bNa + 3 * I_NaK + 3 * I_NaCa) * inverseviF * Cm;
  Na_i += tinc * dNai * 1000;
  const double dKi = -(-i_external + I_K1 + I_to + I_K - 2 * I_NaK + I_pK) * inverseviF * Cm;
  K_i += tinc * dKi * 1000.0;
  const double CaSS005 = (CaSS / 0.05);
  const double FCa_INF = 0.6 / (1.0 + CaSS005 * CaSS005) + 0.4;
  const double taufca = 0.080 / (1.0 + CaSS005 * CaSS005) + 0.002;

  const double M_INF = TB(m_inf)[Vi], H_INF = TB(h_inf)[Vi], J_INF = TB(j_inf)[Vi];
  const double Xr1_INF = TB(Xr1_inf)[Vi], Xr2_INF = TB(Xr2_inf)[Vi], Xs_INF = TB(Xs_inf)[Vi];
  const double S_INF = TB(s_inf)[Vi], R_INF = TB(r_inf)[Vi], D_INF = TB(d_inf)[Vi];
  const double F_INF = TB(f_inf)[Vi], F2_INF = TB(f2_inf)[Vi];
  m = M_INF - (M_INF - m) * TB(exptau_m)[Vi];
  h = H_INF - (H_INF - h) * TB(exptau_h)[Vi];
  j = J_INF - (J_INF - j) * TB(exptau_j)[Vi];
  xr1 = Xr1_INF - (Xr1_INF - xr1) * TB(exptau_Xr1)[Vi];
  xr2 = Xr2_INF - (Xr2_INF - xr2) * TB(exptau_Xr2)[Vi];
  xs = Xs_INF - (Xs_INF - xs) * TB(exptau_Xs)[Vi];
  s = S_INF - (S_INF - s) * TB(exptau_s)[Vi];
  r = R_INF - (R_INF - r) * TB(exptau_r)[Vi];
  d = D_INF - (D_INF - d) * TB(exptau_d)[Vi];
  f = F_INF - (F_INF - f) * TB(exptau_f)[Vi];
  f2 = F2_INF - (F2_INF - f2) * TB(exptau_f2)[Vi];
  fCa = FCa_INF - (FCa_INF - fCa) * exp(-tinc / taufca);

  double *A = b + S_Array; /* diagnostic currents (883-899) */
  A[0] = I_Na; A[1] = I_CaL; A[2] = I_bCa; A[3] = I_pCa; A[4] = I_to; A[5] = I_Ks; A[6] = I_Kr;
  A[7] = I_K1; A[8] = I_pK; A[9] = I_bNa; A[10] = I_NaK; A[11] = I_NaCa; A[12] = I_rel; A[13] = I_leak;
  A[14] = I_xfer; A[15] = SERCA; A[16] = I_tot;
  b[S_Cai] = Ca_i; b[S_CaSR] = CaSR; b[S_CaSS] = CaSS; b[S_Nai] = Na_i; b[S_Ki] = K_i;
  b[S_m] = m; b[S_h] = h; b[S_j] = j; b[S_xr1] = xr1; b[S_xr2] = xr2; b[S_xs] = xs; b[S_r] = r;
  b[S_s] = s; b[S_d] = d; b[S_f] = f; b[S_f2] = f2; b[S_fCa] = fCa; b[S_Rq] = Rq;
  return tinc * (-I_tot);
}
#undef P_
#undef TB

/* ---------------------------------------------------------------- Courtemanche */
#define P_(x) P[C_##x]
#define TB(x) (tables + (size_t)TC_##x * CMO_RTDT)

/* CourtemancheParameters::Calculate (252-280). */
static void crn_derive(double *P) {
  P_(RTdF) = P_(R) * (P_(Tx)) / (P_(F));
  P_(FdRT) = 1.0 / (P_(RTdF));
  P_(RTd2F) = P_(RTdF) * .5;
  P_(Vi) = P_(Vcell) * (P_(part_i));
  P_(Vup) = P_(Vcell) * (P_(part_up));
  P_(Vrel) = P_(Vcell) * (P_(part_rel));
  P_(VupdVi) = P_(Vup) / (P_(Vi));
  P_(VreldVi) = P_(Vrel) / (P_(Vi));
  P_(VreldVup) = P_(Vrel) / (P_(Vup));
  P_(CmdFvi) = P_(C_m) / (P_(F) * (P_(Vi)));
  P_(Cmd2F) = P_(C_m) / (P_(F) * 2.0);
  P_(csqnkm) = P_(CSQNmax) * P_(K_mcsqn);
  P_(kmcsqnm2) = P_(K_mcsqn) * 2.0;
  P_(kkmcsqn) = P_(K_mcsqn) * P_(K_mcsqn);
  P_(cmdnkm) = P_(CMDNmax) * P_(K_mcmdn);
  P_(kmcmdnm2) = P_(K_mcmdn) * 2.0;
  P_(kkmcmdn) = P_(K_mcmdn) * P_(K_mcmdn);
  P_(kupleak) = P_(I_upmax) / (P_(Ca_upmax));
  P_(dt_tr) = 1.0 / (P_(t_tr));
}

/* CourtemancheParameters::InitTable (282-395) plus exp250/exp50 (Init 246-247), which are
 * stored in the first two entries of the last table. */
static void crn_tables(const double *P, double tinc, double *tables) {
  tinc *= 1000;
  const double sigma = (exp(P_(Na_o) / 67.3) - 1.0) / 7.0;
  for (double V = -RANGE_TAB_HALF + .0001; V < RANGE_TAB_HALF; V += D_DIVISION_TAB) {
    int Vi = (int)(DIVISION_TAB * (RANGE_TAB_HALF + V) + .5);
    if (Vi < 0 || Vi >= CMO_RTDT) continue;
    double a = ((fabs(V + 47.13 - P_(shiftm)) < 1e-10
                     ? 3.2
                     : P_(m_a1) * (V + 47.13 - P_(shiftm)) / (1.0 - exp(-(V + 47.13 - P_(shiftm)) * P_(m_a2)))));
    double b = P_(m_b1) * exp(-(V - P_(shiftm)) / P_(m_b2));
    TB(exptau_m)[Vi] = exp(-tinc * (a + b));
    TB(m_m)[Vi] = a / (a + b);

    if (V >= -40.0 + P_(shifth)) {
      a = .0;
      b = 1.0 / (P_(h_b5) * (1.0 + exp(-(V + 10.66 - P_(shifth)) / P_(h_b6))));
    } else {
      a = P_(h_a1) * exp(-(V + 80.0 - P_(shifth)) / P_(h_a2));
      b = P_(h_b1) * exp(P_(h_b2) * (V - P_(shifth))) + P_(h_b3) * exp(P_(h_b4) * (V - P_(shifth)));
    }
    TB(exptau_h)[Vi] = exp(-tinc * (a + b));
    TB(m_h)[Vi] = a / (a + b);

    if (V >= -40.0 + P_(shiftj)) {
      a = .0;
      b = P_(j_b4) * exp(P_(j_b5) * (V - P_(shiftj))) / (1.0 + exp(P_(j_b6) * (V + 32.0 - P_(shiftj))));
    } else {
      a = (P_(j_a1) * exp(P_(j_a2) * (V - P_(shiftj))) - (P_(j_a3)) * exp(P_(j_a4) * (V - P_(shiftj)))) *
          (V + 37.78 - P_(shiftj)) / (1.0 + exp(P_(j_a5) * (V + 79.23 - P_(shiftj))));
      b = P_(j_b1) * exp(P_(j_b2) * (V - P_(shiftj))) / (1.0 + exp(P_(j_b3) * (V + 40.14 - P_(shiftj))));
    }
    TB(exptau_j)[Vi] = exp(-tinc * (a + b) / P_(tau_j_mult));
    TB(m_j)[Vi] = a / (a + b);

    a = P_(C_oa_1) / ((exp(-(V - P_(shiftoa) + 10.0) / (P_(C_oa_2)))) + (exp(-(V - P_(shiftoa) - 30.0) / (P_(C_oa_3)))));
    b = P_(C_oa_1) / (2.5 + exp((V - P_(shiftoa) + 82.0) / (P_(C_oa_4))));
    TB(m_oa)[Vi] = 1.0 / (1.0 + exp(-(V - P_(shiftoa) + P_(C_oa_6)) / (P_(C_oa_5))));
    TB(exptau_oa)[Vi] = exp(-tinc * ((a + b) * P_(Tfac)));

    a = 1.0 / (18.53 + exp((V + 113.7) / 10.95));
    b = 1.0 / (35.56 + exp(-(V + 1.26) / 7.44));
    TB(m_oi)[Vi] = 1.0 / (1.0 + exp((V + 43.1) / 5.3));
    TB(exptau_oi)[Vi] = exp(-tinc * ((a + b) * P_(Tfac)));

    a = P_(ua_a1) / ((exp((V + P_(ua_a2)) / (P_(ua_a3)))) + (exp((V + P_(ua_a4)) / (P_(ua_a5)))));
    b = .65 / (P_(ua_b1) + exp((V + P_(ua_b2)) / (P_(ua_b3))));
    TB(m_ua)[Vi] = 1.0 / (1.0 + exp((V + P_(ua_m1)) / (P_(ua_m2))));
    TB(exptau_ua)[Vi] = exp(-tinc * ((a + b) * P_(ua_KQ10)));

    a = P_(ui_a1) / (P_(ui_a2) + exp((V + P_(ui_a3)) / (P_(ui_a4))));
    b = 1.0 / exp((V + P_(ui_b1)) / (P_(ui_b2)));
    TB(m_ui)[Vi] = 1.0 / (1.0 + exp((V + P_(ui_m1)) / (P_(ui_m2))));
    TB(exptau_ui)[Vi] = exp(-tinc * ((a + b) * P_(ui_KQ10)));

    a = (fabs(V + P_(Xr_a2)) < 1e-10 ? 0.0015
                                      : P_(Xr_a1) * (V + P_(Xr_a2)) / (1.0 - exp((V + P_(Xr_a2)) / (P_(Xr_a3)))));
    b = (fabs(V - P_(Xr_b1)) < 1e-10 ? 3.7836118e-4
                                      : 7.3898e-5 * (V + P_(Xr_b1)) / (exp((V + P_(Xr_b1)) / (P_(Xr_b2))) - 1.0));
    TB(m_Xr)[Vi] = 1.0 / (1.0 + exp((V + P_(Xr_m1)) / (P_(Xr_m2))));
    TB(exptau_Xr)[Vi] = exp(-tinc * (P_(Xr_KQ10) * (a + b)));

    a = (fabs(V + P_(Xs_a2)) < 1e-10 ? 0.00068
                                      : P_(Xs_a1) * (V + P_(Xs_a2)) / (1.0 - exp((V + P_(Xs_a2)) / (P_(Xs_a3)))));
    b = (fabs(V + P_(Xs_b1)) < 1e-10 ? 0.000315
                                      : (3.5e-5) * (V + P_(Xs_b1)) / (exp((V + P_(Xs_b1)) / (P_(Xs_b2))) - 1.0));
    TB(exptau_Xs)[Vi] = exp(-tinc * (P_(Xs_KQ10) * (a + b)));
    TB(m_Xs)[Vi] = 1.0 / sqrt(1.0 + exp((V + P_(Xs_m1)) / (P_(Xs_m2))));

    a = 1.0 / (1.0 + exp(-(V + 10.0) / 6.24));
    TB(exptau_d)[Vi] = exp(-tinc * (fabs(V + 10.0) < 1e-10 ? 1.0 / (a * 4.579)
                                                            : 1.0 / (a * (1.0 - exp(-(V + 10.0) / 6.24)) / (0.035 * (V + 10.0)))));
    TB(m_d)[Vi] = 1.0 / (1.0 + exp(-(V + 10.0) / 8));
    if (V > 0) {
      TB(exptau_f)[Vi] = exp(-tinc * (1.0 / (P_(CaL_fT_1) / (0.0197 * exp(-0.0337 * 0.0337 * (V + 10.0) * (V + 10.0)) + 0.02) *
                                             P_(tau_f_mult))));
    } else {
      TB(exptau_f)[Vi] = exp(-tinc * (1.0 / (P_(CaL_fT_1) / (0.0197 * exp(-0.0337 * 0.0337 * (V + 10.0) * (V + 10.0)) + 0.02))));
    }
    TB(m_f)[Vi] = exp(-(V + 28.0) / 6.9) / (1.0 + exp(-(V + 28.0) / 6.9));

    TB(exptau_w)[Vi] =
        exp(-tinc * (fabs(V - 7.9) < 1e-10 ? 1.0 / (6.0 * 0.2 / 1.3)
                                            : 1.0 / (6.0 * (1.0 - exp(-(V - 7.9) / 5.0)) / (1.0 + 0.3 * exp(-(V - 7.9) / 5.0)) / (V - 7.9))));
    TB(m_w)[Vi] = 1.0 - 1.0 / (1.0 + exp(-(V - 40.0) / 17.0));

    const double VFdRT = V * P_(FdRT);
    TB(expVm)[Vi] = exp(-VFdRT) * P_(Na_o) * P_(Na_o) * P_(Na_o);
    TB(g_Kur)[Vi] = P_(g_Kur1) + P_(g_Kur2) / (1.0 + exp((V + P_(g_Kur3)) / (P_(g_Kur4))));
    TB(CKr)[Vi] = P_(g_Kr) / (1.0 + exp((V + P_(g_Kr1)) / (P_(g_Kr2))));
    TB(CK1)[Vi] = P_(g_K1) / (1.0 + exp((V + P_(g_K1_1)) * P_(g_K1_2)));
    TB(CNaK)[Vi] = P_(I_NaKmax) / (1.0 + .1245 * exp(-.1 * VFdRT) + .0365 * sigma * exp(-VFdRT)) * P_(K_o) /
                   (P_(K_o) + P_(k_mKo));
    TB(CNaCa)[Vi] = P_(k_NaCa) * exp(P_(gamm) * VFdRT) /
                    ((P_(k_mNa) * P_(k_mNa) * P_(k_mNa) + P_(Na_o) * P_(Na_o) * P_(Na_o)) * (P_(k_mCa) + P_(Ca_o)) *
                     (1.0 + P_(k_sat) * exp((P_(gamm) - 1.0) * VFdRT)));
  }
  memset(TB(exp250_exp50), 0, CMO_RTDT * sizeof(double));
  TB(exp250_exp50)[0] = exp(250.0);
  TB(exp250_exp50)[1] = exp(169.5);
}

enum { K_Cai = 0, K_Caup, K_Carel, K_h, K_j, K_oi, K_ui, K_Xr, K_Xs, K_u, K_v, K_w, K_Nai, K_Ki, K_m, K_oa,
       K_ua, K_d, K_f, K_fCa, K_ISAC, K_CaTRPN };

/* Courtemanche::Init (56-83). I_SAC is not set by Init; it starts at 0 here. */
static void crn_init(const double *P, double *b) {
  memset(b, 0, 22 * sizeof(double));
  b[K_Nai] = P_(Init_Na_i); b[K_Ki] = P_(Init_K_i); b[K_m] = P_(Init_m); b[K_oa] = P_(Init_oa);
  b[K_ua] = P_(Init_ua); b[K_d] = P_(Init_d); b[K_fCa] = P_(Init_f_Ca); b[K_Cai] = P_(Init_Ca_i);
  b[K_Caup] = P_(Init_Ca_up); b[K_Carel] = P_(Init_Ca_rel); b[K_h] = P_(Init_h); b[K_j] = P_(Init_j);
  b[K_oi] = P_(Init_oi); b[K_ui] = P_(Init_ui); b[K_Xr] = P_(Init_Xr); b[K_Xs] = P_(Init_Xs);
  b[K_f] = P_(Init_f); b[K_u] = P_(Init_u); b[K_v] = P_(Init_v); b[K_w] = P_(Init_w);
  b[K_CaTRPN] = P_(Init_Ca_TRPN) / P_(TRPNmax);
}

static inline double clamp01(double x) { return x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x); }

/* Courtemanche::Calc (85-187), ISAC and TRPN compiled in (CourtemancheParameters.h:20,23). */
static double crn_calc(const double *P, const double *tables, double *bk, double tinc, double V,
                       double i_external, double stretch) {
  double Ca_i = bk[K_Cai], Ca_up = bk[K_Caup], Ca_rel = bk[K_Carel], h = bk[K_h], j = bk[K_j];
  double oi = bk[K_oi], ui = bk[K_ui], Xr = bk[K_Xr], Xs = bk[K_Xs], u = bk[K_u], v = bk[K_v];
  double w = bk[K_w], Na_i = bk[K_Nai], K_i = bk[K_Ki], m = bk[K_m], oa = bk[K_oa], ua = bk[K_ua];
  double d = bk[K_d], f = bk[K_f], f_Ca = bk[K_fCa], Ca_TRPN = bk[K_CaTRPN];
  tinc *= 1000.0;
  const double V_int = V * 1000.0;
  const int Vi = (int)(DIVISION_TAB * (RANGE_TAB_HALF + V_int) + .5);
  const double dNa_i = 1.0 / Na_i;
  const double VmE_Na = V_int - ((P_(RTdF)) * log((P_(Na_o)) * dNa_i));
  const double VmE_K = V_int - ((P_(RTdF)) * log((P_(K_o)) / K_i));
  const double VmE_Ca = V_int - ((P_(RTd2F)) * log((P_(Ca_o)) / (double)Ca_i));
  const double m_m = TB(m_m)[Vi];
  m = m_m + (m - m_m) * TB(exptau_m)[Vi];
  m = clamp01(m);
  const double m_h = TB(m_h)[Vi];
  h = m_h + (h - m_h) * TB(exptau_h)[Vi];
  const double m_j = TB(m_j)[Vi];
  j = m_j + (j - m_j) * TB(exptau_j)[Vi];
  const double m_oa = TB(m_oa)[Vi];
  oa = m_oa + (oa - m_oa) * TB(exptau_oa)[Vi];
  const double m_oi = TB(m_oi)[Vi];
  oi = m_oi + (oi - m_oi) * TB(exptau_oi)[Vi];
  const double m_ua = TB(m_ua)[Vi];
  ua = m_ua + (ua - m_ua) * TB(exptau_ua)[Vi];
  const double m_ui = TB(m_ui)[Vi];
  ui = m_ui + (ui - m_ui) * TB(exptau_ui)[Vi];
  const double m_Xr = TB(m_Xr)[Vi];
  Xr = m_Xr + (Xr - m_Xr) * TB(exptau_Xr)[Vi];
  const double m_Xs = TB(m_Xs)[Vi];
  Xs = m_Xs + (Xs - m_Xs) * TB(exptau_Xs)[Vi];
  const double m_d = TB(m_d)[Vi];
  d = m_d + (d - m_d) * TB(exptau_d)[Vi];
  const double m_f = TB(m_f)[Vi];
  f = m_f + (f - m_f) * TB(exptau_f)[Vi];
  f_Ca += (1.0 / (1.0 + Ca_i * 2857.1429) - f_Ca) * 0.5 * tinc;
  const double m_w = TB(m_w)[Vi];
  w = m_w + (w - m_w) * TB(exptau_w)[Vi];

  const double I_Na = (P_(g_Na)) * m * m * m * h * j * VmE_Na;
  const double I_to = (P_(g_to)) * oa * oa * oa * oi * VmE_K;
  const double I_Kur = TB(g_Kur)[Vi] * ua * ua * ua * ui * VmE_K;
  const double I_Kr = TB(CKr)[Vi] * Xr * VmE_K;
  const double I_Ks = (P_(g_Ks)) * Xs * Xs * VmE_K;
  const double I_CaL = (P_(g_CaL)) * d * f * f_Ca * (V_int - (P_(E_rL)));
  const double I_K1 = TB(CK1)[Vi] * VmE_K;
  const double I_bNa = (P_(g_bNa)) * VmE_Na;
  const double I_bCa = (P_(g_bCa)) * VmE_Ca;
  const double temp = (P_(k_mNai)) * dNa_i;
  const double I_NaK = TB(CNaK)[Vi] / (1.0 + temp * sqrt(temp));
  const double I_pCa = (P_(I_pCamax)) * Ca_i / (Ca_i + (P_(k_mpCa)));
  const double I_NaCa = TB(CNaCa)[Vi] * ((Na_i * Na_i * Na_i * (P_(Ca_o))) - TB(expVm)[Vi] * Ca_i);
  const double I_rel = (P_(k_rel)) * u * u * v * w * (Ca_rel - Ca_i);
  const double I_up = (P_(I_upmax)) * Ca_i / (Ca_i + (P_(k_up)));
  const double I_upleak = (P_(kupleak)) * Ca_up;
  const double I_tr = (Ca_up - Ca_rel) * (P_(dt_tr));
  double I_SAC = P_(G_sac) * (V_int - P_(E_sac)) / (1. + P_(K_sac) * exp(-P_(alpha) * (stretch - 1.)));
  I_SAC *= P_(ISAC_SWITCH);
  const double Ca_T50 = P_(Ca_T50) + P_(beta1) * ((stretch < 1.2 ? stretch : 1.2) - 1.);
  const double dCaTRPN = P_(k_TRPN) * (pow(1000 * Ca_i / Ca_T50, P_(n_TRPN)) * (1. - Ca_TRPN) - Ca_TRPN);
  Ca_TRPN += tinc * dCaTRPN;
  Ca_up += tinc * (I_up - I_tr * (P_(VreldVup)) - I_upleak);
  Ca_rel += tinc * ((I_tr - I_rel) / (1.0 + (P_(csqnkm)) / (Ca_rel * Ca_rel + Ca_rel * (P_(kmcsqnm2)) + (P_(kkmcsqn)))));
  Na_i += tinc * (-3.0 * I_NaK - 3.0 * I_NaCa - I_bNa - I_Na) * (P_(CmdFvi));
  K_i += tinc * (2.0 * I_NaK - I_K1 - I_to - I_Kur - I_Kr - I_Ks) * (P_(CmdFvi));
  double B1 = ((2.0 * I_NaCa - I_pCa - I_CaL - I_bCa) * .5 * (P_(CmdFvi))) +
              ((I_upleak - I_up) * (P_(VupdVi)) + I_rel * (P_(VreldVi)));
  B1 -= P_(TRPNmax) * dCaTRPN;
  const double B2 = 1.0 + ((P_(cmdnkm)) / ((Ca_i * Ca_i) + (Ca_i * (P_(kmcmdnm2))) + (P_(kkmcmdn))));
  const double dCa_i = B1 / B2;
  Ca_i += tinc * dCa_i;
  const double Fn = exp(-((P_(Vrel)) * I_rel - (0.5 * I_CaL - 0.2 * I_NaCa) * (P_(Cmd2F))) * 731.5289);
  const double m_u = 1.0 / (1.0 + Fn * TB(exp250_exp50)[0]);
  u += (m_u - u) * 0.125 * tinc;
  const double m_v = 1.0 - 1.0 / (1.0 + Fn * TB(exp250_exp50)[1]);
  const double t_v = 1.91 + 2.09 * m_u;
  v += (m_v - v) * tinc / t_v;
  const double I_tot = I_Na + I_CaL + I_pCa + I_K1 + I_to + I_Kur + I_Kr + I_Ks + I_bNa + I_bCa + I_NaK + I_NaCa +
                       I_SAC - i_external;
  bk[K_Cai] = Ca_i; bk[K_Caup] = Ca_up; bk[K_Carel] = Ca_rel; bk[K_h] = h; bk[K_j] = j; bk[K_oi] = oi;
  bk[K_ui] = ui; bk[K_Xr] = Xr; bk[K_Xs] = Xs; bk[K_u] = u; bk[K_v] = v; bk[K_w] = w; bk[K_Nai] = Na_i;
  bk[K_Ki] = K_i; bk[K_m] = m; bk[K_oa] = oa; bk[K_ua] = ua; bk[K_d] = d; bk[K_f] = f; bk[K_fCa] = f_Ca;
  bk[K_ISAC] = I_SAC; bk[K_CaTRPN] = Ca_TRPN;
  return -.001 * I_tot * tinc;
}
#undef P_
#undef TB

/* ---------------------------------------------------------------- O'Hara-Rudy */
#define P_(x) P[O_##x]

/* OHaraRudyParameters::Calculate (246-316). */
static void ord_derive(double *P) {
  P_(R) = 8314.0;
  P_(T) = 310.0;
  P_(F) = 96485.0;
  P_(L) = 0.01;
  P_(r) = 0.0011;
  P_(tau_h_L) = 200.0;
  P_(A_h_fast) = 0.99;
  P_(A_h_slow) = 0.01;
  P_(A_f_fast) = 0.6;
  P_(k_Na1) = 15.0;
  P_(k_Na2) = 5.0;
  P_(k_asymm) = 12.5;
  P_(k_Ca_on) = 1.5e6;
  P_(k_Ca_off) = 5.0e3;
  P_(k_m_1) = 182.4;
  P_(k_p_2) = 687.2;
  P_(k_p_4) = 639.0;
  P_(MgADP) = 0.05;
  P_(MgATP) = 9.8;
  P_(K_MgATP) = 1.698e-7;
  P_(beta_tau) = 4.75;
  P_(P_Ca) = P_(PCa_Multiplier) * 0.0001;
  /* geometry (275-282): the reference takes pi as 3.14 */
  P_(v_cell) = 1000.0 * 3.14 * P_(r) * P_(r) * P_(L);
  P_(A_geo) = 2.0 * 3.14 * P_(r) * P_(r) + 2.0 * 3.14 * P_(r) * P_(L);
  P_(A_cap) = 2.0 * P_(A_geo);
  P_(v_myo) = 0.68 * P_(v_cell);
  P_(v_nsr) = 0.0552 * P_(v_cell);
  P_(v_jsr) = 0.0048 * P_(v_cell);
  P_(v_ss) = 0.02 * P_(v_cell);
  /* permeabilities (285-289); the CaMK-phosphorylated P_CaK uses 3.5743e-4, the other 3.574e-4 */
  P_(P_CaNa) = 0.00125 * P_(P_Ca);
  P_(P_CaK) = 3.574e-04 * P_(P_Ca);
  P_(P_Ca_CaMK) = 1.1 * P_(P_Ca);
  P_(P_CaNa_CaMK) = 0.00125 * P_(P_Ca_CaMK);
  P_(P_CaK_CaMK) = 3.5743e-04 * P_(P_Ca_CaMK);
  P_(A_f_slow) = 1.0 - P_(A_f_fast);
  /* Na/Ca exchanger and Na/K pump rate constants (295-310) */
  P_(h_10) = P_(k_asymm) + 1.0 + (P_(Na_o) * (1.0 + P_(Na_o) / P_(k_Na2))) / P_(k_Na1);
  P_(h_11) = (P_(Na_o) * P_(Na_o)) / (P_(h_10) * P_(k_Na1) * P_(k_Na2));
  P_(h_12) = 1.0 / P_(h_10);
  P_(k_1) = P_(h_12) * P_(Ca_o) * P_(k_Ca_on);
  P_(k_2) = P_(k_Ca_off);
  P_(k_5) = P_(k_Ca_off);
  P_(beta_1) = P_(k_m_1) * P_(MgADP);
  P_(alpha_2) = P_(k_p_2);
  P_(alpha_4) = (P_(k_p_4) * (P_(MgATP) / P_(K_MgATP))) / (1.0 + (P_(MgATP) / P_(K_MgATP)));
  P_(alpha_rel) = 0.5 * P_(beta_tau);
  P_(beta_tau_CaMK) = 1.25 * P_(beta_tau);
  P_(alpha_rel_CaMK) = 0.5 * P_(beta_tau_CaMK);
  P_(tau_h_LCaMK) = 3.0 * P_(tau_h_L);
  P_(RToverF) = (P_(R) * P_(T)) / P_(F);
}

/* OHaraRudy::Init (54-102). h_CaMK_fast is never initialised nor read by the reference;
 * it is 0 here. Ca_TRPN is kept as a fraction of its maximum (Init_Ca_TRPN / 0.07). */
static void ord_init(const double *P, double *b) {
  memset(b, 0, ORD_BLOCK * sizeof(double));
  b[OB_m] = P_(Init_m); b[OB_h_fast] = P_(Init_h_fast); b[OB_h_slow] = P_(Init_h_slow); b[OB_j] = P_(Init_j);
  b[OB_h_CaMK_slow] = P_(Init_h_CaMK_slow); b[OB_j_CaMK] = P_(Init_j_CaMK); b[OB_m_L] = P_(Init_m_L);
  b[OB_h_L] = P_(Init_h_L); b[OB_h_L_CaMK] = P_(Init_h_L_CaMK); b[OB_a] = P_(Init_a);
  b[OB_i_fast] = P_(Init_i_fast); b[OB_i_slow] = P_(Init_i_slow); b[OB_a_CaMK] = P_(Init_a_CaMK);
  b[OB_i_CaMK_fast] = P_(Init_i_CaMK_fast); b[OB_i_CaMK_slow] = P_(Init_i_CaMK_slow); b[OB_d] = P_(Init_d);
  b[OB_f_fast] = P_(Init_f_fast); b[OB_f_slow] = P_(Init_f_slow); b[OB_f_Ca_fast] = P_(Init_f_Ca_fast);
  b[OB_f_Ca_slow] = P_(Init_f_Ca_slow); b[OB_j_Ca] = P_(Init_j_Ca); b[OB_n] = P_(Init_n);
  b[OB_f_CaMK_fast] = P_(Init_f_CaMK_fast); b[OB_f_Ca_CaMK_fast] = P_(Init_f_Ca_CaMK_fast);
  b[OB_x_r_fast] = P_(Init_x_r_fast); b[OB_x_r_slow] = P_(Init_x_r_slow); b[OB_x_s1] = P_(Init_x_s1);
  b[OB_x_s2] = P_(Init_x_s2); b[OB_x_K1] = P_(Init_x_K1); b[OB_Na_i] = P_(Init_Na_i); b[OB_Na_ss] = P_(Init_Na_ss);
  b[OB_K_i] = P_(Init_K_i); b[OB_K_ss] = P_(Init_K_ss); b[OB_Ca_i] = P_(Init_Ca_i); b[OB_Ca_ss] = P_(Init_Ca_ss);
  b[OB_Ca_nsr] = P_(Init_Ca_nsr); b[OB_Ca_jsr] = P_(Init_Ca_jsr); b[OB_CaMK_trap] = P_(Init_CaMK_trap);
  b[OB_J_rel_NP] = P_(Init_J_rel_NP); b[OB_J_rel_CaMK] = P_(Init_J_rel_CaMK);
  b[OB_Ca_TRPN] = P_(Init_Ca_TRPN) / 0.07;
}

/* Gate update of the reference: x = x_inf - (x_inf - x) * exp(-tinc / tau). */
static inline double ord_gate(double inf, double x, double tinc, double tau) {
  return inf - (inf - x) * exp(-tinc / tau);
}

/* OHaraRudy::Calc (105-663), every expression in the reference's evaluation order. The
 * block is the reference backup block (states then the currents it stores). */
static double ord_calc(const double *P, double *b, double tinc, double V, double i_external, double stretch) {
  tinc *= 1000.0;
  const double V_m = V * 1000.0;
  const double lambda_m = 1.2 < stretch ? 1.2 : stretch; /* std::min(1.2, stretch) (109) */
  /* CaMK (115-131) */
  const double KmCaMK = 0.15, aCaMK = 0.05, bCaMK = 0.00068, CaMKo = 0.05, KmCaM = 0.0015;
  double CaMK_trap = b[OB_CaMK_trap];
  const double Ca_ss = b[OB_Ca_ss], Ca_i = b[OB_Ca_i], Na_i = b[OB_Na_i], Na_ss = b[OB_Na_ss];
  const double K_i = b[OB_K_i], K_ss = b[OB_K_ss], Ca_nsr = b[OB_Ca_nsr], Ca_jsr = b[OB_Ca_jsr];
  const double CaMK_bound = CaMKo * ((1.0 - CaMK_trap) / (1.0 + (KmCaM / Ca_ss)));
  const double CaMK_active = (CaMK_bound + CaMK_trap) * P_(HF_Gomez_1);
  const double dCaMK_trap = aCaMK * CaMK_bound * (CaMK_bound + CaMK_trap) - (bCaMK * CaMK_trap);
  CaMK_trap += tinc * dCaMK_trap;
  b[OB_CaMK_trap] = CaMK_trap;
  /* reversal potentials (133-138) */
  const double E_Na = P_(RToverF) * log(P_(Na_o) / Na_i);
  const double E_K = P_(RToverF) * log(P_(K_o) / K_i);
  const double PKNa = 0.01833;
  const double E_Ks = P_(RToverF) * log((P_(K_o) + PKNa * P_(Na_o)) / (K_i + PKNa * Na_i));
  const double VFFoverRT = (V_m * P_(F) * P_(F)) / (P_(R) * P_(T));
  const double VFoverRT = (V_m * P_(F)) / (P_(R) * P_(T));
  const double util_1 = P_(A_cap) / (P_(F) * P_(v_myo));
  const double util_2 = P_(v_ss) / P_(v_myo);
  const double util_3 = P_(A_cap) / (P_(F) * P_(v_ss));

  /* I_Na (146-202): Passini h_inf / h_CaMK_inf, Dutta tau_h_fast / tau_j */
  const double m_inf = 1.0 / (1.0 + exp(-(V_m + 39.57) / 9.871));
  const double tau_m = 1.0 / (6.765 * exp((V_m + 11.64) / 34.77) + 8.552 * exp(-(V_m + 77.42) / 5.955));
  b[OB_m] = ord_gate(m_inf, b[OB_m], tinc, tau_m);
  const double h_inf = 1.0 / (1.0 + exp((V_m + 78.5) / 6.22));
  const double tau_h_fast = 1.0 / (3.686e-6 * exp(-(V_m + 3.8875) / 7.8579) + 16.0 * exp((V_m - 0.4963) / 9.1843));
  const double tau_h_slow = 1.0 / (0.009794 * exp(-(V_m + 17.95) / 28.05) + 0.3343 * exp((V_m + 5.730) / 56.66));
  b[OB_h_fast] = ord_gate(h_inf, b[OB_h_fast], tinc, tau_h_fast);
  b[OB_h_slow] = ord_gate(h_inf, b[OB_h_slow], tinc, tau_h_slow);
  const double h = P_(A_h_fast) * b[OB_h_fast] + P_(A_h_slow) * b[OB_h_slow];
  const double j_inf = h_inf;
  const double tau_j = 4.8590 + 1.0 / (0.8628 * exp(-(V_m + 116.7258) / 7.6005) + 1.1096 * exp((V_m + 6.2719) / 9.0358));
  b[OB_j] = ord_gate(j_inf, b[OB_j], tinc, tau_j);
  const double h_CaMK_inf = 1.0 / (1.0 + exp((V_m + 84.7) / 6.22));
  const double tau_h_CaMK_slow = 3.0 * tau_h_slow;
  b[OB_h_CaMK_slow] = ord_gate(h_CaMK_inf, b[OB_h_CaMK_slow], tinc, tau_h_CaMK_slow);
  const double h_CaMK = P_(A_h_fast) * b[OB_h_fast] + P_(A_h_slow) * b[OB_h_CaMK_slow];
  const double tau_j_CaMK = 1.46 * tau_j;
  b[OB_j_CaMK] = ord_gate(j_inf, b[OB_j_CaMK], tinc, tau_j_CaMK);
  const double phi_INa_CaMK = 1.0 / (1.0 + KmCaMK / CaMK_active);
  const double G_Na_fast = 75.0;
  const double m = b[OB_m];
  const double I_Na_fast = P_(INaF_Multiplier) * G_Na_fast * (V_m - E_Na) * m * m * m *
                           ((1.0 - phi_INa_CaMK) * h * b[OB_j] + phi_INa_CaMK * h_CaMK * b[OB_j_CaMK]);

  /* I_NaL (204-224) */
  double thL_mod = 1.0;
  thL_mod *= P_(HF_Gomez_2);
  const double m_L_inf = 1.0 / (1.0 + exp(-(V_m + 42.85) / 5.264));
  b[OB_m_L] = ord_gate(m_L_inf, b[OB_m_L], tinc, tau_m);
  const double h_L_inf = 1.0 / (1.0 + exp((V_m + 87.61) / 7.488));
  b[OB_h_L] = ord_gate(h_L_inf, b[OB_h_L], tinc, thL_mod * P_(tau_h_L));
  const double h_L_CaMK_inf = 1.0 / (1.0 + exp((V_m + 93.81) / 7.488));
  const double tau_h_L_CaMK = 3.0 * P_(tau_h_L) * thL_mod;
  b[OB_h_L_CaMK] = ord_gate(h_L_CaMK_inf, b[OB_h_L_CaMK], tinc, tau_h_L_CaMK);
  const double G_Na_L = 0.0075;
  const double I_Na_late = P_(INaL_Multiplier) * P_(HF_Gomez_3) * G_Na_L * (V_m - E_Na) * b[OB_m_L] *
                           ((1.0 - phi_INa_CaMK) * b[OB_h_L] + phi_INa_CaMK * b[OB_h_L_CaMK]);

  /* I_to (226-262) */
  const double a_inf = 1.0 / (1.0 + exp(-(V_m - 14.34) / 14.82));
  const double tau_a =
      1.0515 / (1.0 / (1.2089 * (1.0 + exp(-(V_m - 18.4099) / 29.3814))) + 3.5 / (1.0 + exp((V_m + 100.0) / 29.3814)));
  b[OB_a] = ord_gate(a_inf, b[OB_a], tinc, tau_a);
  const double i_inf = 1.0 / (1.0 + exp((V_m + 43.94) / 5.711));
  const double delta_epi = P_(celltype) == 1.0 ? (1.0 - 0.95 / (1.0 + exp((V_m + 70.0) / 5.0))) : 1.0;
  const double tau_i_fast_base = 4.562 + 1.0 / (0.3933 * exp(-(V_m + 100.0) / 100.0) + 0.08004 * exp((V_m + 50.0) / 16.59));
  const double tau_i_slow_base =
      23.62 + 1.0 / (0.001416 * exp(-(V_m + 96.52) / 59.05) + 1.7808e-08 * exp((V_m + 114.1) / 8.079));
  const double tau_i_fast = tau_i_fast_base * delta_epi;
  const double tau_i_slow = tau_i_slow_base * delta_epi;
  b[OB_i_fast] = ord_gate(i_inf, b[OB_i_fast], tinc, tau_i_fast);
  b[OB_i_slow] = ord_gate(i_inf, b[OB_i_slow], tinc, tau_i_slow);
  const double A_i_fast = 1.0 / (1.0 + exp((V_m - 213.6) / 151.2));
  const double A_i_slow = 1.0 - A_i_fast;
  const double i = A_i_fast * b[OB_i_fast] + A_i_slow * b[OB_i_slow];
  const double a_CaMK_inf = 1.0 / (1.0 + exp(-(V_m - 24.34) / 14.82));
  b[OB_a_CaMK] = ord_gate(a_CaMK_inf, b[OB_a_CaMK], tinc, tau_a);
  const double delta_CaMK_develop = 1.354 + 1.0e-04 / (exp((V_m - 167.4) / 15.89) + exp(-(V_m - 12.23) / 0.2154));
  const double delta_CaMK_recover = 1.0 - 0.5 / (1.0 + exp((V_m + 70.0) / 20.0));
  const double tau_i_CaMK_fast = tau_i_fast * delta_CaMK_develop * delta_CaMK_recover;
  const double tau_i_CaMK_slow = tau_i_slow * delta_CaMK_develop * delta_CaMK_recover;
  b[OB_i_CaMK_fast] = ord_gate(i_inf, b[OB_i_CaMK_fast], tinc, tau_i_CaMK_fast);
  b[OB_i_CaMK_slow] = ord_gate(i_inf, b[OB_i_CaMK_slow], tinc, tau_i_CaMK_slow);
  const double i_CaMK = A_i_fast * b[OB_i_CaMK_fast] + A_i_slow * b[OB_i_CaMK_slow];
  const double G_to = 0.02;
  const double I_to = P_(Ito_Multiplier) * P_(HF_Gomez_4) * G_to * (V_m - E_K) *
                      ((1.0 - phi_INa_CaMK) * b[OB_a] * i + phi_INa_CaMK * b[OB_a_CaMK] * i_CaMK);

  /* I_CaL, I_CaNa, I_CaK (264-329) */
  const double d_inf = 1.0 / (1.0 + exp(-(V_m + 3.940) / 4.230));
  const double tau_d = 0.6 + 1.0 / (exp(-0.05 * (V_m + 6.0)) + exp(0.09 * (V_m + 14.0)));
  b[OB_d] = ord_gate(d_inf, b[OB_d], tinc, tau_d);
  const double f_inf = 1.0 / (1.0 + exp((V_m + 19.58) / 3.696));
  const double tau_f_fast = 7.0 + 1.0 / (0.0045 * exp(-(V_m + 20.0) / 10.0) + 0.0045 * exp((V_m + 20.0) / 10.0));
  const double tau_f_slow = 1000.0 + 1.0 / (3.5e-05 * exp(-(V_m + 5.0) / 4.0) + 3.5e-05 * exp((V_m + 5.0) / 6.0));
  b[OB_f_fast] = ord_gate(f_inf, b[OB_f_fast], tinc, tau_f_fast);
  b[OB_f_slow] = ord_gate(f_inf, b[OB_f_slow], tinc, tau_f_slow);
  const double f = P_(A_f_fast) * b[OB_f_fast] + P_(A_f_slow) * b[OB_f_slow];
  const double tau_f_Ca_fast = 7.0 + 1.0 / (0.04 * exp(-(V_m - 4.0) / 7.0) + 0.04 * exp((V_m - 4.0) / 7.0));
  const double tau_f_Ca_slow = 100.0 + 1.0 / (0.00012 * exp(-V_m / 3.0) + 0.00012 * exp(V_m / 7.0));
  b[OB_f_Ca_fast] = ord_gate(f_inf, b[OB_f_Ca_fast], tinc, tau_f_Ca_fast);
  b[OB_f_Ca_slow] = ord_gate(f_inf, b[OB_f_Ca_slow], tinc, tau_f_Ca_slow);
  const double A_f_Ca_fast = 0.3 + 0.6 / (1.0 + exp((V_m - 10.0) / 10.0));
  const double A_f_Ca_slow = 1.0 - A_f_Ca_fast;
  const double f_Ca = A_f_Ca_fast * b[OB_f_Ca_fast] + A_f_Ca_slow * b[OB_f_Ca_slow];
  const double tau_j_Ca = 75.0;
  b[OB_j_Ca] = ord_gate(f_inf, b[OB_j_Ca], tinc, tau_j_Ca);
  const double tau_f_CaMK_fast = 2.5 * tau_f_fast;
  b[OB_f_CaMK_fast] = ord_gate(f_inf, b[OB_f_CaMK_fast], tinc, tau_f_CaMK_fast);
  const double f_CaMK = P_(A_f_fast) * b[OB_f_CaMK_fast] + P_(A_f_slow) * b[OB_f_slow];
  const double tau_f_Ca_CaMK_fast = 2.5 * tau_f_Ca_fast;
  b[OB_f_Ca_CaMK_fast] = ord_gate(f_inf, b[OB_f_Ca_CaMK_fast], tinc, tau_f_Ca_CaMK_fast);
  const double f_Ca_CaMK = A_f_Ca_fast * b[OB_f_Ca_CaMK_fast] + A_f_Ca_slow * b[OB_f_Ca_slow];
  const double j_Ca = b[OB_j_Ca];
  const double k_m2_n = j_Ca * 1.0;
  const double Kmn = 0.002, k2n = 1000.0;
  const double alpha_n = 1.0 / ((k2n / k_m2_n) + pow((1.0 + (Kmn / Ca_ss)), 4.0));
  b[OB_n] = alpha_n * (k2n / k_m2_n) - (alpha_n * (k2n / k_m2_n) - b[OB_n]) * exp(-k_m2_n * tinc);
  const double n = b[OB_n];
  const double z_Ca = 2.0, z_Na = 1.0, z_K = 1.0;
  const double exp_z_Ca = exp(z_Ca * VFoverRT);
  const double exp_z_Na = exp(z_Na * VFoverRT);
  const double exp_z_K = exp(z_K * VFoverRT);
  const double gamma_Cai = 1.0, gamma_Cao = 0.341, gamma_Nai = 0.75, gamma_Nao = 0.75, gamma_Ki = 0.75,
               gamma_Ko = 0.75;
  const double Psi_Ca =
      z_Ca * z_Ca * VFFoverRT * (gamma_Cai * Ca_ss * exp_z_Ca - gamma_Cao * P_(Ca_o)) / (exp_z_Ca - 1.0);
  const double Psi_CaNa =
      z_Na * z_Na * VFFoverRT * (gamma_Nai * Na_ss * exp_z_Na - gamma_Nao * P_(Na_o)) / (exp_z_Na - 1.0);
  const double Psi_CaK = z_K * z_K * VFFoverRT * (gamma_Ki * K_ss * exp_z_K - gamma_Ko * P_(K_o)) / (exp_z_K - 1.0);
  const double I_CaL_b = P_(P_Ca) * Psi_Ca;
  const double I_CaNa_b = P_(P_CaNa) * Psi_CaNa;
  const double I_CaK_b = P_(P_CaK) * Psi_CaK;
  const double I_CaL_CaMK = P_(P_Ca_CaMK) * Psi_Ca;
  const double I_CaNa_CaMK = P_(P_CaNa_CaMK) * Psi_CaNa;
  const double I_CaK_CaMK = P_(P_CaK_CaMK) * Psi_CaK;
  const double d = b[OB_d], phi = phi_INa_CaMK;
  const double I_CaL = I_CaL_b * d * (1.0 - phi) * (f * (1.0 - n) + f_Ca * n * j_Ca) +
                       I_CaL_CaMK * d * phi * (f_CaMK * (1.0 - n) + f_Ca_CaMK * n * j_Ca);
  const double I_CaNa = I_CaNa_b * d * (1.0 - phi) * (f * (1.0 - n) + f_Ca * n * j_Ca) +
                        I_CaNa_CaMK * d * phi * (f_CaMK * (1.0 - n) + f_Ca_CaMK * n * j_Ca);
  const double I_CaK = I_CaK_b * d * (1.0 - phi) * (f * (1.0 - n) + f_Ca * n * j_Ca) +
                       I_CaK_CaMK * d * phi * (f_CaMK * (1.0 - n) + f_Ca_CaMK * n * j_Ca);

  /* I_Kr (331-344) */
  const double x_r_inf = 1.0 / (1.0 + exp((-(V_m + 8.337)) / 6.789));
  const double tau_x_r_fast =
      12.98 + 1.0 / (0.3652 * exp((V_m - 31.66) / 3.869) + 4.123e-05 * exp((-(V_m - 47.78)) / 20.38));
  const double tau_x_r_slow =
      1.865 + 1.0 / (0.06629 * exp((V_m - 34.7) / 7.355) + 1.128e-05 * exp((-(V_m - 29.74)) / 25.94));
  const double A_x_r_fast = 1.0 / (1.0 + exp((V_m + 54.81) / 38.21));
  const double A_x_r_slow = 1.0 - A_x_r_fast;
  b[OB_x_r_fast] = ord_gate(x_r_inf, b[OB_x_r_fast], tinc, tau_x_r_fast);
  b[OB_x_r_slow] = ord_gate(x_r_inf, b[OB_x_r_slow], tinc, tau_x_r_slow);
  const double x_r = A_x_r_fast * b[OB_x_r_fast] + A_x_r_slow * b[OB_x_r_slow];
  const double R_Kr = 1.0 / ((1.0 + exp((V_m + 55.0) / 75.0)) * (1.0 + exp((V_m - 10.0) / 30.0)));
  const double G_Kr = 0.046;
  const double I_Kr = P_(IKr_Multiplier) * G_Kr * sqrt(P_(K_o) / 5.4) * x_r * (V_m - E_K) * R_Kr;

  /* I_Ks (346-355) */
  const double x_s1_inf = 1.0 / (1.0 + exp(-(V_m + 11.6) / 8.932));
  const double tau_x_s1 = 817.3 + 1.0 / (2.326e-04 * exp((V_m + 48.28) / 17.80) + 0.001292 * exp(-(V_m + 210.0) / 230.0));
  b[OB_x_s1] = ord_gate(x_s1_inf, b[OB_x_s1], tinc, tau_x_s1);
  const double tau_x_s2 = 1.0 / (0.01 * exp((V_m - 50.0) / 20.0) + 0.0193 * exp(-(V_m + 66.54) / 31.0));
  b[OB_x_s2] = ord_gate(x_s1_inf, b[OB_x_s2], tinc, tau_x_s2);
  const double G_Ks = 0.0034;
  const double I_Ks = P_(IKs_Multiplier) * G_Ks * (1.0 + 0.6 / (1.0 + pow((3.8e-05 / Ca_i), 1.4))) * b[OB_x_s1] *
                      b[OB_x_s2] * (V_m - E_Ks);

  /* I_K1 (357-367) */
  const double x_K1_inf = 1.0 / (1.0 + exp(-(V_m + 2.5538 * P_(K_o) + 144.59) / (1.5692 * P_(K_o) + 3.8115)));
  const double tau_x_K1 = 122.2 / (exp(-(V_m + 127.2) / 20.36) + exp((V_m + 236.8) / 69.33));
  b[OB_x_K1] = ord_gate(x_K1_inf, b[OB_x_K1], tinc, tau_x_K1);
  const double R_K1 = 1.0 / (1.0 + exp((V_m + 105.8 - 2.6 * P_(K_o)) / 9.493));
  const double G_K1 = 0.1908;
  const double I_K1 = P_(IK1_Multiplier) * P_(HF_Gomez_5) * G_K1 * sqrt(P_(K_o)) * b[OB_x_K1] * (V_m - E_K) * R_K1;

  /* I_NaCa_i (369-413) */
  const double kna3 = 88.12, wna = 6.0e4, wca = 6.0e4, wnaca = 5.0e3, qna = 0.5224, qca = 0.1670;
  const double h_Ca = exp(qca * VFoverRT);
  const double h_Na = exp(qna * VFoverRT);
  const double h_1_i = 1.0 + (Na_i * (1.0 + h_Na)) / kna3;
  const double h_2_i = (Na_i * h_Na) / (kna3 * h_1_i);
  const double h_3_i = 1.0 / h_1_i;
  const double h_4_i = 1.0 + (Na_i * (1.0 + Na_i / P_(k_Na2))) / P_(k_Na1);
  const double h_5_i = (Na_i * Na_i) / (h_4_i * P_(k_Na1) * P_(k_Na2));
  const double h_6_i = 1.0 / h_4_i;
  const double h_7 = 1.0 + (P_(Na_o) * (1.0 + 1.0 / h_Na)) / kna3;
  const double h_8 = P_(Na_o) / (kna3 * h_Na * h_7);
  const double h_9 = 1.0 / h_7;
  const double k_3_d = h_9 * wca;
  const double k_3_dd = h_8 * wnaca;
  const double k_3 = k_3_d + k_3_dd;
  const double k_4_d_i = (h_3_i * wca) / h_Ca;
  const double k_4_dd_i = h_2_i * wnaca;
  const double k_4_i = k_4_d_i + k_4_dd_i;
  const double k_6_i = h_6_i * Ca_i * P_(k_Ca_on);
  const double k_7_i = h_5_i * h_2_i * wna;
  const double k_8 = h_8 * P_(h_11) * wna;
  const double k_1 = P_(k_1), k_2 = P_(k_2), k_5 = P_(k_5);
  const double x_1_i = k_2 * k_4_i * (k_7_i + k_6_i) + k_5 * k_7_i * (k_2 + k_3);
  const double x_2_i = k_1 * k_7_i * (k_4_i + k_5) + k_4_i * k_6_i * (k_1 + k_8);
  const double x_3_i = k_1 * k_3 * (k_7_i + k_6_i) + k_8 * k_6_i * (k_2 + k_3);
  const double x_4_i = k_2 * k_8 * (k_4_i + k_5) + k_3 * k_5 * (k_1 + k_8);
  const double E_1_i = x_1_i / (x_1_i + x_2_i + x_3_i + x_4_i);
  const double E_2_i = x_2_i / (x_1_i + x_2_i + x_3_i + x_4_i);
  const double E_3_i = x_3_i / (x_1_i + x_2_i + x_3_i + x_4_i);
  const double E_4_i = x_4_i / (x_1_i + x_2_i + x_3_i + x_4_i);
  const double KmCaAct = 150.0e-6;
  const double allo_i = 1.0 / (1.0 + (KmCaAct / Ca_i) * (KmCaAct / Ca_i));
  const double J_NaCa_Na_i = 3.0 * (E_4_i * k_7_i - E_1_i * k_8) + E_3_i * k_4_dd_i - E_2_i * k_3_dd;
  const double J_NaCa_Ca_i = E_2_i * k_2 - E_1_i * k_1;
  const double G_NaCa = 0.0008;
  const double I_NaCa_i = P_(INaCa_Multiplier) * P_(HF_Gomez_6) * G_NaCa * 0.8 * allo_i *
                          (z_Na * J_NaCa_Na_i + z_Ca * J_NaCa_Ca_i);

  /* I_NaCa_ss (415-443) */
  const double h_1_ss = 1.0 + (Na_ss * (1.0 + h_Na)) / kna3;
  const double h_2_ss = (Na_ss * h_Na) / (kna3 * h_1_ss);
  const double h_3_ss = 1.0 / h_1_ss;
  const double h_4_ss = 1.0 + (Na_ss * (1.0 + Na_ss / P_(k_Na2))) / P_(k_Na1);
  const double h_5_ss = (Na_ss * Na_ss) / (h_4_ss * P_(k_Na1) * P_(k_Na2));
  const double h_6_ss = 1.0 / h_4_ss;
  const double k_4_d_ss = (h_3_ss * wca) / h_Ca;
  const double k_4_dd_ss = h_2_ss * wnaca;
  const double k_4_ss = k_4_d_ss + k_4_dd_ss;
  const double k_6_ss = h_6_ss * Ca_ss * P_(k_Ca_on);
  const double k_7_ss = h_5_ss * h_2_ss * wna;
  const double x_1_ss = k_2 * k_4_ss * (k_7_ss + k_6_ss) + k_5 * k_7_ss * (k_2 + k_3);
  const double x_2_ss = k_1 * k_7_ss * (k_4_ss + k_5) + k_4_ss * k_6_ss * (k_1 + k_8);
  const double x_3_ss = k_1 * k_3 * (k_7_ss + k_6_ss) + k_8 * k_6_ss * (k_2 + k_3);
  const double x_4_ss = k_2 * k_8 * (k_4_ss + k_5) + k_3 * k_5 * (k_1 + k_8);
  const double E_1_ss = x_1_ss / (x_1_ss + x_2_ss + x_3_ss + x_4_ss);
  const double E_2_ss = x_2_ss / (x_1_ss + x_2_ss + x_3_ss + x_4_ss);
  const double E_3_ss = x_3_ss / (x_1_ss + x_2_ss + x_3_ss + x_4_ss);
  const double E_4_ss = x_4_ss / (x_1_ss + x_2_ss + x_3_ss + x_4_ss);
  const double allo_ss = 1.0 / (1.0 + (KmCaAct / Ca_ss) * (KmCaAct / Ca_ss));
  const double J_NaCa_Na_ss = 3.0 * (E_4_ss * k_7_ss - E_1_ss * k_8) + E_3_ss * k_4_dd_ss - E_2_ss * k_3_dd;
  const double J_NaCa_Ca_ss = E_2_ss * k_2 - E_1_ss * k_1;
  const double I_NaCa_ss = P_(INaCa_Multiplier) * P_(HF_Gomez_6) * G_NaCa * 0.2 * allo_ss *
                           (z_Na * J_NaCa_Na_ss + z_Ca * J_NaCa_Ca_ss);

  /* I_NaK (445-498) */
  const double k1p = 949.5, k2m = 39.4, k3p = 1899.0, k3m = 79300.0, k4m = 40.0, Knai0 = 9.073, Knao0 = 27.78,
               delta = -0.1550;
  const double K_Nai = Knai0 * exp(delta * VFoverRT * 1 / 3);
  const double K_Nao = Knao0 * exp((1.0 - delta) * VFoverRT * 1 / 3);
  const double Kki = 0.5, Kko = 0.3582, H = 1.0e-7, eP = 4.2, Khp = 1.698e-7, Knap = 224.0, Kxkur = 292.0;
  const double Pnak = eP / (1.0 + H / Khp + Na_i / Knap + K_i / Kxkur);
  const double alpha_1 = (k1p * pow((Na_i / K_Nai), 3.0)) /
                         (pow((1.0 + Na_i / K_Nai), 3.0) + pow((1.0 + K_i / Kki), 2.0) - 1.0);
  const double beta_2 = (k2m * pow((P_(Na_o) / K_Nao), 3.0)) /
                        (pow((1.0 + P_(Na_o) / K_Nao), 3.0) + pow((1.0 + P_(K_o) / Kko), 2.0) - 1.0);
  const double alpha_3 = (k3p * pow((P_(K_o) / Kko), 2.0)) /
                         (pow((1.0 + P_(Na_o) / K_Nao), 3.0) + pow((1.0 + P_(K_o) / Kko), 2.0) - 1.0);
  const double beta_3 = (k3m * Pnak * H) / (1.0 + P_(MgATP));
  const double beta_4 = (k4m * pow((K_i / Kki), 2.0)) /
                        (pow((1.0 + Na_i / K_Nai), 3.0) + pow((1.0 + K_i / Kki), 2.0) - 1.0);
  const double al2 = P_(alpha_2), al4 = P_(alpha_4), be1 = P_(beta_1);
  const double x_1 = al4 * alpha_1 * al2 + beta_2 * beta_4 * beta_3 + al2 * beta_4 * beta_3 + beta_3 * alpha_1 * al2;
  const double x_2 = beta_2 * be1 * beta_4 + alpha_1 * al2 * alpha_3 + alpha_3 * be1 * beta_4 + al2 * alpha_3 * beta_4;
  const double x_3 = al2 * alpha_3 * al4 + beta_3 * beta_2 * be1 + beta_2 * be1 * al4 + alpha_3 * al4 * be1;
  const double x_4 = beta_4 * beta_3 * beta_2 + alpha_3 * al4 * alpha_1 + beta_2 * al4 * alpha_1 + beta_3 * beta_2 * alpha_1;
  const double E_1 = x_1 / (x_1 + x_2 + x_3 + x_4);
  const double E_2 = x_2 / (x_1 + x_2 + x_3 + x_4);
  const double E_3 = x_3 / (x_1 + x_2 + x_3 + x_4);
  const double E_4 = x_4 / (x_1 + x_2 + x_3 + x_4);
  const double J_NaK_Na = 3.0 * (E_1 * alpha_3 - E_2 * beta_3);
  const double J_NaK_K = 2.0 * (E_4 * be1 - E_3 * alpha_1);
  const double P_NaK = 30.0;
  const double I_NaK = P_(INaK_Multiplier) * P_(HF_Gomez_7) * P_NaK * (z_Na * J_NaK_Na + z_K * J_NaK_K);

  /* background currents, I_pCa (500-517) */
  const double x_Kb = 1.0 / (1.0 + exp(-(V_m - 14.48) / (18.34)));
  const double G_Kb = 0.003;
  const double I_Kb = P_(IKb_Multiplier) * G_Kb * x_Kb * (V_m - E_K);
  const double P_Nab = 3.75e-10;
  const double I_Nab =
      P_(INab_Multiplier) * P_Nab * z_Na * z_Na * VFFoverRT * ((Na_i * exp_z_Na - P_(Na_o)) / (exp_z_Na - 1.0));
  const double P_Cab = 2.5e-8;
  const double I_Cab = P_(ICab_Multiplier) * P_Cab * z_Ca * z_Ca * VFFoverRT *
                       ((gamma_Cai * Ca_i * exp_z_Ca - gamma_Cao * P_(Ca_o)) / (exp_z_Ca - 1.0));
  const double G_pCa = 0.0005;
  const double I_pCa = P_(IpCa_Multiplier) * G_pCa * (Ca_i / (0.0005 + Ca_i));

  /* stretch-activated current (519-523) */
  double I_SAC = P_(G_sac) * (V_m - P_(E_sac)) / (1. + P_(K_sac) * exp(-P_(alpha) * (stretch - 1.)));
  I_SAC *= P_(ISAC_SWITCH);

  /* total current (525-533) */
  const double cur_I_tot = I_Na_fast + I_Na_late + I_to + I_CaL + I_CaNa + I_CaK + I_Kr + I_Ks + I_K1 + I_NaCa_i +
                           I_NaCa_ss + I_NaK + I_Nab + I_Cab + I_Kb + I_pCa + I_SAC + i_external;
  const double I_tot = -cur_I_tot;

  /* diffusion fluxes (535-541) */
  const double J_diff_Na = (Na_ss - Na_i) / 2.0;
  const double J_diff_Ca = (Ca_ss - Ca_i) / 0.2;
  const double J_diff_K = (K_ss - K_i) / 2.0;

  /* SR release (543-565); celltype 2 (M cells) scales the steady state by 1.7 */
  double J_rel_NP_inf = (P_(alpha_rel) * (-I_CaL)) / (1.0 + pow((1.5 * P_(HF_Gomez_8) / Ca_jsr), 8.0));
  double J_rel_CaMK_inf = (P_(alpha_rel_CaMK) * (-I_CaL)) / (1.0 + pow((1.5 * P_(HF_Gomez_8) / Ca_jsr), 8.0));
  if (P_(celltype) == 2.0) {
    J_rel_NP_inf *= 1.7;
    J_rel_CaMK_inf *= 1.7;
  }
  const double tau_rel_NP_b = P_(beta_tau) / (1.0 + (0.0123 / Ca_jsr));
  const double tau_rel_NP = tau_rel_NP_b < 0.001 ? 0.001 : tau_rel_NP_b;
  b[OB_J_rel_NP] = ord_gate(J_rel_NP_inf, b[OB_J_rel_NP], tinc, tau_rel_NP);
  const double tau_rel_CaMK_b = P_(beta_tau_CaMK) / (1.0 + (0.0123 / Ca_jsr));
  const double tau_rel_CaMK = tau_rel_CaMK_b < 0.001 ? 0.001 : tau_rel_CaMK_b;
  b[OB_J_rel_CaMK] = ord_gate(J_rel_CaMK_inf, b[OB_J_rel_CaMK], tinc, tau_rel_CaMK);
  const double J_rel = (1.0 - phi) * b[OB_J_rel_NP] + phi * b[OB_J_rel_CaMK];

  /* SERCA uptake and leak (567-588); celltype 1 (epicardial) scales uptake by 1.3 */
  double J_up_NP = (0.004375 * Ca_i) / (0.00092 + Ca_i);
  const double DJ_up_CaMK = 1.75, DK_m_PLB = 0.00017;
  double J_up_CaMK = (1.0 + DJ_up_CaMK) * (0.004375 * Ca_i) / (0.00092 - DK_m_PLB + Ca_i);
  if (P_(celltype) == 1.0) {
    J_up_NP *= 1.3;
    J_up_CaMK *= 1.3;
  }
  const double J_leak = P_(HF_Gomez_9) * (0.0039375 * Ca_nsr) / 15.0;
  const double J_up = P_(HF_Gomez_0) * ((1.0 - phi) * J_up_NP + phi * J_up_CaMK - J_leak);
  const double J_tr = (Ca_nsr - Ca_jsr) / 100.0;

  /* concentrations (594-605) */
  const double cur_Nai = I_Na_fast + I_Na_late + 3.0 * I_NaCa_i + 3.0 * I_NaK + I_Nab;
  const double dNa_i = -(cur_Nai)*util_1 + J_diff_Na * util_2;
  b[OB_Na_i] = Na_i + tinc * dNa_i;
  const double dNa_ss = -(I_CaNa + 3.0 * I_NaCa_ss) * util_3 - J_diff_Na;
  b[OB_Na_ss] = Na_ss + tinc * dNa_ss;
  const double cur_Ki = I_to + I_Kr + I_Ks + I_K1 + I_Kb + i_external - 2.0 * I_NaK;
  const double dK_i = -(cur_Ki)*util_1 + J_diff_K * util_2;
  b[OB_K_i] = K_i + tinc * dK_i;
  const double dK_ss = -(I_CaK * util_3) - J_diff_K;
  b[OB_K_ss] = K_ss + tinc * dK_ss;

  /* calcium buffering, troponin and the calcium compartments (607-660) */
  double cmdnmax = 0.05;
  if (P_(celltype) == 1) cmdnmax *= 1.3;
  const double kmcmdn = 0.00238, trpnmax = 0.07, BSRmax = 0.047, KmBSR = 0.00087, BSLmax = 1.124, KmBSL = 0.0087,
               csqnmax = 10.0, kmcsqn = 0.8;
  const double Ca_T50 = (P_(Ca_T50) + P_(beta1) * (lambda_m - 1.0)) * P_(HFM_Multiplier);
  const double Ca_TRPN = b[OB_Ca_TRPN];
  const double dCaTRPN = P_(k_TRPN) * (pow(1000 * Ca_i / Ca_T50, P_(n_TRPN)) * (1. - Ca_TRPN) - Ca_TRPN);
  b[OB_Ca_TRPN] = Ca_TRPN + tinc * dCaTRPN;
  const double I_Trpn = trpnmax * dCaTRPN;
  const double beta_Cai = 1.0 / (1.0 + ((cmdnmax * kmcmdn) / pow((kmcmdn + Ca_i), 2.0)));
  const double cur_Cai = I_pCa + I_Cab - 2.0 * I_NaCa_i;
  const double dCa_i =
      beta_Cai * (-(cur_Cai)*0.5 * util_1 - J_up * (P_(v_nsr) / P_(v_myo)) + J_diff_Ca * util_2 - I_Trpn);
  b[OB_Ca_i] = Ca_i + tinc * dCa_i;
  const double beta_Cass =
      1.0 / (1.0 + ((BSRmax * KmBSR) / pow((KmBSR + Ca_ss), 2.0)) + ((BSLmax * KmBSL) / pow((KmBSL + Ca_ss), 2.0)));
  const double dCa_ss =
      beta_Cass * (-(I_CaL - 2.0 * I_NaCa_ss) * 0.5 * util_3 + J_rel * (P_(v_jsr) / P_(v_ss)) - J_diff_Ca);
  b[OB_Ca_ss] = Ca_ss + tinc * dCa_ss;
  const double dCa_nsr = J_up - (J_tr * (P_(v_jsr) / P_(v_nsr)));
  b[OB_Ca_nsr] = Ca_nsr + tinc * dCa_nsr;
  const double beta_Cajsr = 1.0 / (1.0 + ((csqnmax * kmcsqn) / pow((kmcsqn + Ca_jsr), 2.0)));
  const double dCa_jsr = beta_Cajsr * (J_tr - J_rel);
  b[OB_Ca_jsr] = Ca_jsr + tinc * dCa_jsr;

  /* the currents the reference keeps in its block (OHaraRudy.h:48-52) */
  b[OB_I_Na_fast] = I_Na_fast; b[OB_I_Na_late] = I_Na_late; b[OB_I_to] = I_to; b[OB_I_CaL] = I_CaL;
  b[OB_I_CaNa] = I_CaNa; b[OB_I_CaK] = I_CaK; b[OB_I_Kr] = I_Kr; b[OB_I_Ks] = I_Ks; b[OB_I_K1] = I_K1;
  b[OB_I_NaCa_i] = I_NaCa_i; b[OB_I_NaCa_ss] = I_NaCa_ss; b[OB_I_NaK] = I_NaK; b[OB_I_Nab] = I_Nab;
  b[OB_I_Cab] = I_Cab; b[OB_I_Kb] = I_Kb; b[OB_I_pCa] = I_pCa; b[OB_I_SAC] = I_SAC;
  return 0.001 * tinc * I_tot;
}
#undef P_

/* ---------------------------------------------------------------- Tomek */
#define P_(x) P[M_##x]

/* TomekParameters::Calculate (233-302): as O'Hara-Rudy's, with one A_h. */
static void tom_derive(double *P) {
  P_(R) = 8314.0;
  P_(T) = 310.0;
  P_(F) = 96485.0;
  P_(L) = 0.01;
  P_(r) = 0.0011;
  P_(tau_h_L) = 200.0;
  P_(A_h) = 0.99;
  P_(A_f_fast) = 0.6;
  P_(k_Na1) = 15.0;
  P_(k_Na2) = 5.0;
  P_(k_asymm) = 12.5;
  P_(k_Ca_on) = 1.5e6;
  P_(k_Ca_off) = 5.0e3;
  P_(k_m_1) = 182.4;
  P_(k_p_2) = 687.2;
  P_(k_p_4) = 639.0;
  P_(MgADP) = 0.05;
  P_(MgATP) = 9.8;
  P_(K_MgATP) = 1.698e-7;
  P_(beta_tau) = 4.75;
  P_(P_Ca) = P_(PCa_Multiplier) * 0.0001;
  P_(v_cell) = 1000.0 * 3.14 * P_(r) * P_(r) * P_(L);
  P_(A_geo) = 2.0 * 3.14 * P_(r) * P_(r) + 2.0 * 3.14 * P_(r) * P_(L);
  P_(A_cap) = 2.0 * P_(A_geo);
  P_(v_myo) = 0.68 * P_(v_cell);
  P_(v_nsr) = 0.0552 * P_(v_cell);
  P_(v_jsr) = 0.0048 * P_(v_cell);
  P_(v_ss) = 0.02 * P_(v_cell);
  P_(P_CaNa) = 0.00125 * P_(P_Ca);
  P_(P_CaK) = 3.574e-04 * P_(P_Ca);
  P_(P_Ca_CaMK) = 1.1 * P_(P_Ca);
  P_(P_CaNa_CaMK) = 0.00125 * P_(P_Ca_CaMK);
  P_(P_CaK_CaMK) = 3.5743e-04 * P_(P_Ca_CaMK);
  P_(A_f_slow) = 1.0 - P_(A_f_fast);
  P_(h_10) = P_(k_asymm) + 1.0 + (P_(Na_o) * (1.0 + P_(Na_o) / P_(k_Na2))) / P_(k_Na1);
  P_(h_11) = (P_(Na_o) * P_(Na_o)) / (P_(h_10) * P_(k_Na1) * P_(k_Na2));
  P_(h_12) = 1.0 / P_(h_10);
  P_(k_1) = P_(h_12) * P_(Ca_o) * P_(k_Ca_on);
  P_(k_2) = P_(k_Ca_off);
  P_(k_5) = P_(k_Ca_off);
  P_(beta_1) = P_(k_m_1) * P_(MgADP);
  P_(alpha_2) = P_(k_p_2);
  P_(alpha_4) = (P_(k_p_4) * (P_(MgATP) / P_(K_MgATP))) / (1.0 + (P_(MgATP) / P_(K_MgATP)));
  P_(alpha_rel) = 0.5 * P_(beta_tau);
  P_(beta_tau_CaMK) = 1.25 * P_(beta_tau);
  P_(alpha_rel_CaMK) = 0.5 * P_(beta_tau_CaMK);
  P_(tau_h_LCaMK) = 3.0 * P_(tau_h_L);
  P_(RToverF) = (P_(R) * P_(T)) / P_(F);
}

/* Tomek::Init (55-107): A_j and B_j are not set there (Calc sets them before use); 0 here. */
static void tom_init(const double *P, double *b) {
  memset(b, 0, TOM_BLOCK * sizeof(double));
  b[MB_m] = P_(Init_m); b[MB_A_h] = P_(Init_A_h); b[MB_B_h] = P_(Init_B_h); b[MB_h] = P_(Init_h);
  b[MB_j] = P_(Init_j); b[MB_h_p] = P_(Init_h_p); b[MB_j_p] = P_(Init_j_p); b[MB_m_L] = P_(Init_m_L);
  b[MB_h_L] = P_(Init_h_L); b[MB_h_L_CaMK] = P_(Init_h_L_CaMK); b[MB_a] = P_(Init_a);
  b[MB_i_fast] = P_(Init_i_fast); b[MB_i_slow] = P_(Init_i_slow); b[MB_a_CaMK] = P_(Init_a_CaMK);
  b[MB_i_CaMK_fast] = P_(Init_i_CaMK_fast); b[MB_i_CaMK_slow] = P_(Init_i_CaMK_slow); b[MB_d] = P_(Init_d);
  b[MB_f_fast] = P_(Init_f_fast); b[MB_f_slow] = P_(Init_f_slow); b[MB_f_Ca_fast] = P_(Init_f_Ca_fast);
  b[MB_f_Ca_slow] = P_(Init_f_Ca_slow); b[MB_j_Ca] = P_(Init_j_Ca); b[MB_n_ss] = P_(Init_n_ss);
  b[MB_n_i] = P_(Init_n_i); b[MB_f_CaMK_fast] = P_(Init_f_CaMK_fast); b[MB_f_Ca_CaMK_fast] = P_(Init_f_Ca_CaMK_fast);
  b[MB_C_0] = P_(Init_C_0); b[MB_C_1] = P_(Init_C_1); b[MB_C_2] = P_(Init_C_2); b[MB_O] = P_(Init_O);
  b[MB_I] = P_(Init_I); b[MB_x_s1] = P_(Init_x_s1); b[MB_x_s2] = P_(Init_x_s2); b[MB_Na_i] = P_(Init_Na_i);
  b[MB_Na_ss] = P_(Init_Na_ss); b[MB_K_i] = P_(Init_K_i); b[MB_K_ss] = P_(Init_K_ss); b[MB_Ca_i] = P_(Init_Ca_i);
  b[MB_Ca_ss] = P_(Init_Ca_ss); b[MB_Ca_nsr] = P_(Init_Ca_nsr); b[MB_Ca_jsr] = P_(Init_Ca_jsr);
  b[MB_Cl_i] = P_(Init_Cl_i); b[MB_CaMK_trap] = P_(Init_CaMK_trap); b[MB_J_rel_NP] = P_(Init_J_rel_NP);
  b[MB_J_rel_CaMK] = P_(Init_J_rel_CaMK); b[MB_Ca_TRPN] = P_(Init_Ca_TRPN) / 0.07;
}

/* Ionic-strength activity coefficient of Tomek::Calc (272-279): exp(-constA z^2 (sqrt(I)/(1+sqrt(I)) - 0.3 I)). */
static inline double tom_gamma(double constA, double z2, double I) {
  return exp((-constA * z2 * ((sqrt(I) / (1. + sqrt(I))) - (0.3 * I))));
}

/* Tomek::Calc (110-656), the reference's evaluation order. */
static double tom_calc(const double *P, double *b, double tinc, double V, double i_external, double stretch) {
  tinc *= 1000.0;
  const double V_m = V * 1000.0;
  const double lambda_m = 1.2 < stretch ? 1.2 : stretch;
  const double KmCaMK = 0.15, aCaMK = 0.05, bCaMK = 0.00068, CaMKo = 0.05, KmCaM = 0.0015;
  const double Na_i = b[MB_Na_i], Na_ss = b[MB_Na_ss], K_i = b[MB_K_i], K_ss = b[MB_K_ss], Ca_i = b[MB_Ca_i],
               Ca_ss = b[MB_Ca_ss], Ca_nsr = b[MB_Ca_nsr], Ca_jsr = b[MB_Ca_jsr], Cl_i = b[MB_Cl_i];
  double CaMK_trap = b[MB_CaMK_trap];
  /* CaMK (127-132) */
  const double CaMK_bound = ((CaMKo * (1.0 - CaMK_trap)) / (1.0 + (KmCaM / Ca_ss)));
  const double CaMK_active = (CaMK_bound + CaMK_trap);
  const double dCaMK_trap = ((aCaMK * CaMK_bound * (CaMK_bound + CaMK_trap)) - (bCaMK * CaMK_trap));
  CaMK_trap += tinc * dCaMK_trap;
  b[MB_CaMK_trap] = CaMK_trap;
  /* reversal potentials (135-140) */
  const double E_Na = P_(RToverF) * log(P_(Na_o) / Na_i);
  const double E_K = P_(RToverF) * log(P_(K_o) / K_i);
  const double PKNa = 0.01833;
  const double E_Ks = P_(RToverF) * log((P_(K_o) + PKNa * P_(Na_o)) / (K_i + PKNa * Na_i));
  const double zcl = 1.0;
  const double E_Cl = ((P_(R) * P_(T)) / (zcl * P_(F))) * log((Cl_i / P_(Cl_o)));
  const double VFFoverRT = (V_m * P_(F) * P_(F)) / (P_(R) * P_(T));
  const double VFoverRT = (V_m * P_(F)) / (P_(R) * P_(T));
  const double util_1 = P_(A_cap) / (P_(F) * P_(v_myo));
  const double util_2 = P_(v_ss) / P_(v_myo);
  const double util_3 = P_(A_cap) / (P_(F) * P_(v_ss));

  /* I_Na (150-182): ten Tusscher gates with a CaMK-phosphorylated pair (h_p, j_p) */
  const double m_inf = 1.0 / ((1.0 + exp(-(V_m + 56.86) / 9.03)) * (1.0 + exp(-(V_m + 56.86) / 9.03)));
  const double tau_m = 0.1292 * exp(-(((V_m + 45.79) / 15.54) * ((V_m + 45.79) / 15.54))) +
                       0.06487 * exp(-(((V_m - 4.823) / 51.12) * ((V_m - 4.823) / 51.12)));
  b[MB_m] = m_inf - (m_inf - b[MB_m]) * exp(-tinc / tau_m);
  double A_h, B_h, A_j, B_j;
  if (V_m < -40.0) {
    A_h = (0.057 * exp((-(V_m + 80.0) / 6.8)));
    B_h = ((2.7 * exp((0.079 * V_m))) + (3.1e5 * exp((0.3485 * V_m))));
    A_j = ((((-2.5428e4 * exp((0.2444 * V_m))) - (6.948e-6 * exp((-0.04391 * V_m)))) * (V_m + 37.78)) /
           (1.0 + exp((0.311 * (V_m + 79.23)))));
    B_j = ((0.02424 * exp((-0.01052 * V_m))) / (1.0 + exp((-0.1378 * (V_m + 40.14)))));
  } else {
    A_h = 0.0;
    B_h = (0.77 / (0.13 * (1. + exp((-(V_m + 10.66) / 11.1)))));
    A_j = 0.0;
    B_j = ((0.6 * exp((0.057 * V_m))) / (1.0 + exp((-0.1 * (V_m + 32.0)))));
  }
  b[MB_A_h] = A_h; b[MB_B_h] = B_h; b[MB_A_j] = A_j; b[MB_B_j] = B_j;
  const double tau_h = 1.0 / (A_h + B_h);
  const double h_inf = (1.0 / ((1.0 + exp(((V_m + 71.55) / 7.43))) * (1.0 + exp(((V_m + 71.55) / 7.43)))));
  b[MB_h] = h_inf - (h_inf - b[MB_h]) * exp(-tinc / tau_h);
  const double tau_j = 1.0 / (A_j + B_j);
  const double j_inf = (1.0 / ((1.0 + exp(((V_m + 71.55) / 7.43))) * (1.0 + exp(((V_m + 71.55) / 7.43)))));
  b[MB_j] = j_inf - (j_inf - b[MB_j]) * exp(-tinc / tau_j);
  const double h_p_inf = (1.0 / ((1.0 + exp(((V_m + 77.55) / 7.43))) * (1.0 + exp(((V_m + 77.55) / 7.43)))));
  b[MB_h_p] = h_p_inf - (h_p_inf - b[MB_h_p]) * exp(-tinc / tau_h);
  const double tau_j_p = 1.46 * tau_j;
  b[MB_j_p] = j_inf - (j_inf - b[MB_j_p]) * exp(-tinc / tau_j_p);
  const double phi_INa_CaMK = 1.0 / (1.0 + KmCaMK / CaMK_active);
  const double G_Na = 11.7802;
  const double m = b[MB_m];
  const double I_Na = P_(INaF_Multiplier) * G_Na * (V_m - E_Na) * m * m * m *
                      ((1.0 - phi_INa_CaMK) * b[MB_h] * b[MB_j] + (phi_INa_CaMK * b[MB_h_p] * b[MB_j_p]));

  /* I_NaL (186-198) */
  const double thL_mod = 1.0;
  const double m_L_inf = 1.0 / (1.0 + exp(-(V_m + 42.85) / 5.264));
  b[MB_m_L] = m_L_inf - (m_L_inf - b[MB_m_L]) * exp(-tinc / tau_m);
  const double h_L_inf = 1.0 / (1.0 + exp((V_m + 87.61) / 7.488));
  b[MB_h_L] = h_L_inf - (h_L_inf - b[MB_h_L]) * exp(-tinc / (thL_mod * P_(tau_h_L)));
  const double h_L_CaMK_inf = 1.0 / (1.0 + exp((V_m + 93.81) / 7.488));
  const double tau_h_L_CaMK = 3.0 * P_(tau_h_L) * thL_mod;
  b[MB_h_L_CaMK] = h_L_CaMK_inf - (h_L_CaMK_inf - b[MB_h_L_CaMK]) * exp(-tinc / tau_h_L_CaMK);
  const double G_Na_L = 0.0279;
  const double I_Na_late = P_(INaL_Multiplier) * G_Na_L * (V_m - E_Na) * b[MB_m_L] *
                           ((1.0 - phi_INa_CaMK) * b[MB_h_L] + phi_INa_CaMK * b[MB_h_L_CaMK]);

  /* I_to (200-231) */
  const double a_inf = 1.0 / (1.0 + exp(-(V_m - 14.34) / 14.82));
  const double tau_a =
      1.0515 / (1.0 / (1.2089 * (1.0 + exp(-(V_m - 18.4099) / 29.3814))) + 3.5 / (1.0 + exp((V_m + 100.0) / 29.3814)));
  b[MB_a] = a_inf - (a_inf - b[MB_a]) * exp(-tinc / tau_a);
  const double i_inf = 1.0 / (1.0 + exp((V_m + 43.94) / 5.711));
  const double delta_epi = P_(celltype) == 1.0 ? (1.0 - 0.95 / (1.0 + exp((V_m + 70.0) / 5.0))) : 1.0;
  const double tau_i_fast_base = 4.562 + 1.0 / (0.3933 * exp(-(V_m + 100.0) / 100.0) + 0.08004 * exp((V_m + 50.0) / 16.59));
  const double tau_i_slow_base =
      23.62 + 1.0 / (0.001416 * exp(-(V_m + 96.52) / 59.05) + 1.780e-08 * exp((V_m + 114.1) / 8.079));
  const double tau_i_fast = tau_i_fast_base * delta_epi;
  const double tau_i_slow = tau_i_slow_base * delta_epi;
  b[MB_i_fast] = i_inf - (i_inf - b[MB_i_fast]) * exp(-tinc / tau_i_fast);
  b[MB_i_slow] = i_inf - (i_inf - b[MB_i_slow]) * exp(-tinc / tau_i_slow);
  const double A_i_fast = 1.0 / (1.0 + exp((V_m - 213.6) / 151.2));
  const double A_i_slow = 1.0 - A_i_fast;
  const double i = A_i_fast * b[MB_i_fast] + A_i_slow * b[MB_i_slow];
  const double a_CaMK_inf = 1.0 / (1.0 + exp(-(V_m - 24.34) / 14.82));
  b[MB_a_CaMK] = a_CaMK_inf - (a_CaMK_inf - b[MB_a_CaMK]) * exp(-tinc / tau_a);
  const double delta_CaMK_develop = 1.354 + 1.0e-04 / (exp((V_m - 167.4) / 15.89) + exp(-(V_m - 12.23) / 0.2154));
  const double delta_CaMK_recover = 1.0 - 0.5 / (1.0 + exp((V_m + 70.0) / 20.0));
  const double tau_i_CaMK_fast = tau_i_fast * delta_CaMK_develop * delta_CaMK_recover;
  const double tau_i_CaMK_slow = tau_i_slow * delta_CaMK_develop * delta_CaMK_recover;
  b[MB_i_CaMK_fast] = i_inf - (i_inf - b[MB_i_CaMK_fast]) * exp(-tinc / tau_i_CaMK_fast);
  b[MB_i_CaMK_slow] = i_inf - (i_inf - b[MB_i_CaMK_slow]) * exp(-tinc / tau_i_CaMK_slow);
  const double i_CaMK = A_i_fast * b[MB_i_CaMK_fast] + A_i_slow * b[MB_i_CaMK_slow];
  const double G_to = 0.16;
  const double I_to = P_(Ito_Multiplier) * G_to * (V_m - E_K) *
                      ((1.0 - phi_INa_CaMK) * b[MB_a] * i + phi_INa_CaMK * b[MB_a_CaMK] * i_CaMK);

  /* I_CaL, I_CaNa, I_CaK (233-327): subspace (80 %) and myoplasm (20 %) parts, each with its own
   * n gate and activity coefficients from the local ionic strength */
  double d_inf = 1.0763 * exp((-1.007 * exp((-0.0829 * V_m))));
  if (V_m > 31.4978) d_inf = 1.0;
  const double tau_d = 0.6 + 1.0 / (exp(-0.05 * (V_m + 6.0)) + exp(0.09 * (V_m + 14.0)));
  b[MB_d] = d_inf - (d_inf - b[MB_d]) * exp(-tinc / tau_d);
  const double f_inf = 1.0 / (1.0 + exp((V_m + 19.58) / 3.696));
  const double tau_f_fast = 7.0 + 1.0 / (0.0045 * exp(-(V_m + 20.0) / 10.0) + 0.0045 * exp((V_m + 20.0) / 10.0));
  const double tau_f_slow = 1000.0 + 1.0 / (3.5e-05 * exp(-(V_m + 5.0) / 4.0) + 3.5e-05 * exp((V_m + 5.0) / 6.0));
  const double A_f_Ca_fast = 0.3 + 0.6 / (1.0 + exp((V_m - 10.0) / 10.0));
  const double A_f_Ca_slow = 1.0 - A_f_Ca_fast;
  b[MB_f_fast] = f_inf - (f_inf - b[MB_f_fast]) * exp(-tinc / tau_f_fast);
  b[MB_f_slow] = f_inf - (f_inf - b[MB_f_slow]) * exp(-tinc / tau_f_slow);
  const double f = P_(A_f_fast) * b[MB_f_fast] + P_(A_f_slow) * b[MB_f_slow];
  const double tau_f_Ca_fast = 7.0 + 1.0 / (0.04 * exp(-(V_m - 4.0) / 7.0) + 0.04 * exp((V_m - 4.0) / 7.0));
  const double tau_f_Ca_slow = 100.0 + 1.0 / (0.00012 * exp(-V_m / 3.0) + 0.00012 * exp(V_m / 7.0));
  b[MB_f_Ca_fast] = f_inf - (f_inf - b[MB_f_Ca_fast]) * exp(-tinc / tau_f_Ca_fast);
  b[MB_f_Ca_slow] = f_inf - (f_inf - b[MB_f_Ca_slow]) * exp(-tinc / tau_f_Ca_slow);
  const double f_Ca = A_f_Ca_fast * b[MB_f_Ca_fast] + A_f_Ca_slow * b[MB_f_Ca_slow];
  const double j_Ca_inf = 1. / (1 + exp((V_m + 18.08) / (2.7916)));
  const double tau_j_Ca = 75.0;
  b[MB_j_Ca] = j_Ca_inf - (j_Ca_inf - b[MB_j_Ca]) * exp(-tinc / tau_j_Ca);
  const double tau_f_CaMK_fast = 2.5 * tau_f_fast;
  b[MB_f_CaMK_fast] = f_inf - (f_inf - b[MB_f_CaMK_fast]) * exp(-tinc / tau_f_CaMK_fast);
  const double f_CaMK = P_(A_f_fast) * b[MB_f_CaMK_fast] + P_(A_f_slow) * b[MB_f_slow];
  const double tau_f_Ca_CaMK_fast = 2.5 * tau_f_Ca_fast;
  b[MB_f_Ca_CaMK_fast] = f_inf - (f_inf - b[MB_f_Ca_CaMK_fast]) * exp(-tinc / tau_f_Ca_CaMK_fast);
  const double f_Ca_CaMK = A_f_Ca_fast * b[MB_f_Ca_CaMK_fast] + A_f_Ca_slow * b[MB_f_Ca_slow];
  const double j_Ca = b[MB_j_Ca];
  const double k_m2_n = j_Ca * 1.0;
  const double Kmn = 0.002, k2n = 500.0;
  const double alpha_n_Ca_ss = 1.0 / ((k2n / k_m2_n) + pow((1.0 + (Kmn / Ca_ss)), 4.0));
  b[MB_n_ss] = alpha_n_Ca_ss * (k2n / k_m2_n) - (alpha_n_Ca_ss * (k2n / k_m2_n) - b[MB_n_ss]) * exp(-k_m2_n * tinc);
  const double I_o = (0.5 * (P_(Na_o) + P_(K_o) + P_(Cl_o) + (4. * P_(Ca_o))) / 1000.);
  const double I_ss = ((0.5 * (Na_ss + K_ss + Cl_i + (4. * Ca_ss))) / 1000.);
  const double constA = (1.82e6 * pow((74. * 310.), -1.5));
  const double gamma_Ca_ss = tom_gamma(constA, 4., I_ss);
  const double gamma_Ca_o = tom_gamma(constA, 4., I_o);
  const double gamma_Na_ss = tom_gamma(constA, 1., I_ss);
  const double gamma_Na_o = tom_gamma(constA, 1., I_o);
  const double gamma_K_ss = tom_gamma(constA, 1., I_ss);
  const double gamma_K_o = tom_gamma(constA, 1., I_o);
  const double Psi_Ca_ss = ((4. * VFFoverRT * ((gamma_Ca_ss * Ca_ss * exp((2. * VFoverRT))) - (gamma_Ca_o * P_(Ca_o)))) /
                            (exp((2. * VFoverRT)) - 1.));
  const double Psi_CaNa_ss = ((1. * VFFoverRT * ((gamma_Na_ss * Na_ss * exp((1. * VFoverRT))) - (gamma_Na_o)*P_(Na_o))) /
                              (exp((1. * VFoverRT)) - 1.));
  const double Psi_CaK_ss = ((1. * VFFoverRT * ((gamma_K_ss * K_ss * exp((1. * VFoverRT))) - (gamma_K_o * P_(K_o)))) /
                             (exp((1. * VFoverRT)) - 1.));
  /* the reference scales the L-type permeability by IpCa_Multiplier (line 290) */
  const double PCa_b = 8.3757e-05;
  const double PCa = P_(IpCa_Multiplier) * PCa_b;
  const double PCaNa = (0.00125 * PCa), PCaK = (3.574e-4 * PCa), PCap = (1.1 * PCa), PCaNap = (0.00125 * PCap),
               PCaKp = (3.574e-4 * PCap);
  const double ICaL_fractionSS = 0.8;
  const double phi = 1.0 / (1.0 + KmCaMK / CaMK_active);
  const double d = b[MB_d], n_ss = b[MB_n_ss];
  const double I_CaL_ss = (ICaL_fractionSS * (((1. - phi) * PCa * Psi_Ca_ss * d * ((f * (1. - n_ss)) + (j_Ca * f_Ca * n_ss))) +
                                             (phi * PCap * Psi_Ca_ss * d * ((f_CaMK * (1. - n_ss)) + (j_Ca * f_Ca_CaMK * n_ss)))));
  const double I_CaNa_ss =
      (ICaL_fractionSS * (((1. - phi) * PCaNa * Psi_CaNa_ss * d * ((f * (1. - n_ss)) + (j_Ca * f_Ca * n_ss))) +
                          (phi * PCaNap * Psi_CaNa_ss * d * ((f_CaMK * (1. - n_ss)) + (j_Ca * f_Ca_CaMK * n_ss)))));
  const double I_CaK_ss = (ICaL_fractionSS * (((1. - phi) * PCaK * Psi_CaK_ss * d * ((f * (1. - n_ss)) + (j_Ca * f_Ca * n_ss))) +
                                             (phi * PCaKp * Psi_CaK_ss * d * ((f_CaMK * (1. - n_ss)) + (j_Ca * f_Ca_CaMK * n_ss)))));
  const double alpha_n_Ca_i =
      1.0 / ((k2n / k_m2_n) + ((1. + (Kmn / Ca_i)) * (1. + (Kmn / Ca_i)) * (1. + (Kmn / Ca_i)) * (1. + (Kmn / Ca_i))));
  b[MB_n_i] = alpha_n_Ca_i * (k2n / k_m2_n) - (alpha_n_Ca_i * (k2n / k_m2_n) - b[MB_n_i]) * exp(-k_m2_n * tinc);
  const double n_i = b[MB_n_i];
  const double I_i = ((0.5 * (Na_i + K_i + Cl_i + (4. * Ca_i))) / 1000.);
  const double gamma_Ca_i = tom_gamma(constA, 4., I_i);
  const double gamma_Na_i = tom_gamma(constA, 1., I_i);
  const double gamma_K_i = tom_gamma(constA, 1., I_i);
  const double Psi_Ca_i = ((4. * VFFoverRT * ((gamma_Ca_i * Ca_i * exp((2. * VFoverRT))) - (gamma_Ca_o * P_(Ca_o)))) /
                           (exp((2. * VFoverRT)) - 1.));
  const double Psi_CaNa_i = (1. * VFFoverRT * ((gamma_Na_i * Na_i * exp((1. * VFoverRT))) - (gamma_Na_o * P_(Na_o))) /
                             (exp((1. * VFoverRT)) - 1.));
  const double Psi_CaK_i = ((1. * VFFoverRT * ((gamma_K_i * K_i * exp((1. * VFoverRT))) - (gamma_K_o * P_(K_o)))) /
                            (exp((1. * VFoverRT)) - 1.));
  const double I_CaL_i = ((1. - ICaL_fractionSS) * (((1. - phi) * PCa * Psi_Ca_i * d * ((f * (1. - n_i)) + (j_Ca * f_Ca * n_i))) +
                                                   (phi * PCap * Psi_Ca_i * d * ((f_CaMK * (1. - n_i)) + (j_Ca * f_Ca_CaMK * n_i)))));
  const double I_CaNa_i =
      ((1. - ICaL_fractionSS) * (((1. - phi) * PCaNa * Psi_CaNa_i * d * ((f * (1. - n_i)) + (j_Ca * f_Ca * n_i))) +
                                 (phi * PCaNap * Psi_CaNa_i * d * ((f_CaMK * (1. - n_i)) + (j_Ca * f_Ca_CaMK * n_i)))));
  const double I_CaK_i =
      ((1. - ICaL_fractionSS) * (((1. - phi) * PCaK * Psi_CaK_i * d * ((f * (1. - n_i)) + (j_Ca * f_Ca * n_i))) +
                                 (phi * PCaKp * Psi_CaK_i * d * ((f_CaMK * (1. - n_i)) + (j_Ca * f_Ca_CaMK * n_i)))));
  const double I_CaL = I_CaL_ss + I_CaL_i;
  const double I_CaNa = I_CaNa_ss + I_CaNa_i;
  const double I_CaK = I_CaK_ss + I_CaK_i;

  /* I_Kr (329-351): five-state Markov chain, explicit Euler in the reference's order */
  const double alpha_Kr = 0.1161 * exp(0.299 * VFoverRT);
  const double beta_Kr = 0.2442 * exp(-1.604 * VFoverRT);
  const double alpha_Kr_1 = 1.25 * 0.1235, beta_Kr_1 = 0.1911;
  const double alpha_Kr_2 = 0.0578 * exp(0.971 * VFoverRT);
  const double beta_Kr_2 = 0.349e-3 * exp(-1.062 * VFoverRT);
  const double alpha_Kr_i = 0.2533 * exp(0.5953 * VFoverRT);
  const double beta_Kr_i = 0.06525 * exp(-0.8209 * VFoverRT);
  const double alpha_C2_to_I = 0.52e-4 * exp(1.525 * VFoverRT);
  const double beta_I_to_C2 = (beta_Kr_2 * beta_Kr_i * alpha_C2_to_I) / (alpha_Kr_2 * alpha_Kr_i);
  const double dC_0 = b[MB_C_1] * beta_Kr - b[MB_C_0] * alpha_Kr;
  b[MB_C_0] += tinc * dC_0;
  const double dC_1 = b[MB_C_0] * alpha_Kr + b[MB_C_2] * beta_Kr_1 - b[MB_C_1] * (beta_Kr + alpha_Kr_1);
  b[MB_C_1] += tinc * dC_1;
  const double dC_2 = b[MB_C_1] * alpha_Kr_1 + b[MB_O] * beta_Kr_2 + b[MB_I] * beta_I_to_C2 -
                      b[MB_C_2] * (beta_Kr_1 + alpha_Kr_2 + alpha_C2_to_I);
  b[MB_C_2] += tinc * dC_2;
  const double dO = (((alpha_Kr_2 * b[MB_C_2]) + (beta_Kr_i * b[MB_I])) - ((beta_Kr_2 + alpha_Kr_i) * b[MB_O]));
  b[MB_O] += tinc * dO;
  const double dI = (((alpha_C2_to_I * b[MB_C_2]) + (alpha_Kr_i * b[MB_O])) - ((beta_I_to_C2 + beta_Kr_i) * b[MB_I]));
  b[MB_I] += tinc * dI;
  const double G_Kr = 0.0321;
  const double I_Kr = P_(IKr_Multiplier) * G_Kr * sqrt(P_(K_o) / 5.0) * b[MB_O] * (V_m - E_K);

  /* I_Ks (355-363) */
  const double x_s1_inf = 1.0 / (1.0 + exp(-(V_m + 11.6) / 8.932));
  const double tau_x_s1 = 817.3 + 1.0 / (2.326e-04 * exp((V_m + 48.28) / 17.80) + 0.001292 * exp(-(V_m + 210.0) / 230.0));
  b[MB_x_s1] = x_s1_inf - (x_s1_inf - b[MB_x_s1]) * exp(-tinc / tau_x_s1);
  const double tau_x_s2 = 1.0 / (0.01 * exp((V_m - 50.0) / 20.0) + 0.0193 * exp(-(V_m + 66.54) / 31.0));
  b[MB_x_s2] = x_s1_inf - (x_s1_inf - b[MB_x_s2]) * exp(-tinc / tau_x_s2);
  const double G_Ks = 0.0011;
  const double I_Ks = P_(IKs_Multiplier) * G_Ks * (1.0 + (0.6 / (1.0 + pow((3.8e-05 / (Ca_i)), 1.4)))) * b[MB_x_s1] *
                      b[MB_x_s2] * (V_m - E_Ks);

  /* I_K1 (365-370): instantaneous rectification */
  const double a_K1 = 4.094 / (1.0 + exp(0.1217 * (V_m - E_K - 49.934)));
  const double b_K1 = (15.72 * exp(0.0674 * (V_m - E_K - 3.257)) + exp(0.0618 * (V_m - E_K - 594.31))) /
                      (1.0 + exp(-0.1629 * (V_m - E_K + 14.207)));
  const double K1_SS = (a_K1) / (a_K1 + b_K1);
  const double G_K1 = 0.6992;
  const double I_K1 = P_(IK1_Multiplier) * G_K1 * sqrt(P_(K_o) / 5.0) * K1_SS * (V_m - E_K);

  /* I_NaCa_i, I_NaCa_ss (373-451): O'Hara-Rudy's exchanger with 0.0034 x (0.65 | 0.35) */
  const double kna3 = 88.12, wna = 6.0e4, wca = 6.0e4, wnaca = 5.0e3, qna = 0.5224, qca = 0.1670;
  const double z_Ca = 2.0, z_Na = 1.0, z_K = 1.0;
  const double exp_z_Ca = exp(z_Ca * VFoverRT);
  const double exp_z_Na = exp(z_Na * VFoverRT);
  const double h_Ca = exp(qca * VFoverRT);
  const double h_Na = exp(qna * VFoverRT);
  const double h_1_i = 1.0 + (Na_i * (1.0 + h_Na)) / kna3;
  const double h_2_i = (Na_i * h_Na) / (kna3 * h_1_i);
  const double h_3_i = 1.0 / h_1_i;
  const double h_4_i = 1.0 + (Na_i * (1.0 + Na_i / P_(k_Na2))) / P_(k_Na1);
  const double h_5_i = (Na_i * Na_i) / (h_4_i * P_(k_Na1) * P_(k_Na2));
  const double h_6_i = 1.0 / h_4_i;
  const double h_7 = 1.0 + (P_(Na_o) * (1.0 + 1.0 / h_Na)) / kna3;
  const double h_8 = P_(Na_o) / (kna3 * h_Na * h_7);
  const double h_9 = 1.0 / h_7;
  const double k_3_d = h_9 * wca;
  const double k_3_dd = h_8 * wnaca;
  const double k_3 = k_3_d + k_3_dd;
  const double k_4_d_i = (h_3_i * wca) / h_Ca;
  const double k_4_dd_i = h_2_i * wnaca;
  const double k_4_i = k_4_d_i + k_4_dd_i;
  const double k_6_i = h_6_i * Ca_i * P_(k_Ca_on);
  const double k_7_i = h_5_i * h_2_i * wna;
  const double k_8 = h_8 * P_(h_11) * wna;
  const double k_1 = P_(k_1), k_2 = P_(k_2), k_5 = P_(k_5);
  const double x_1_i = k_2 * k_4_i * (k_7_i + k_6_i) + k_5 * k_7_i * (k_2 + k_3);
  const double x_2_i = k_1 * k_7_i * (k_4_i + k_5) + k_4_i * k_6_i * (k_1 + k_8);
  const double x_3_i = k_1 * k_3 * (k_7_i + k_6_i) + k_8 * k_6_i * (k_2 + k_3);
  const double x_4_i = k_2 * k_8 * (k_4_i + k_5) + k_3 * k_5 * (k_1 + k_8);
  const double E_1_i = x_1_i / (x_1_i + x_2_i + x_3_i + x_4_i);
  const double E_2_i = x_2_i / (x_1_i + x_2_i + x_3_i + x_4_i);
  const double E_3_i = x_3_i / (x_1_i + x_2_i + x_3_i + x_4_i);
  const double E_4_i = x_4_i / (x_1_i + x_2_i + x_3_i + x_4_i);
  const double KmCaAct = 150.0e-6;
  const double allo_i = 1.0 / (1.0 + ((KmCaAct / Ca_i) * (KmCaAct / Ca_i)));
  const double J_NaCa_Na_i = 3.0 * (E_4_i * k_7_i - E_1_i * k_8) + E_3_i * k_4_dd_i - E_2_i * k_3_dd;
  const double J_NaCa_Ca_i = E_2_i * k_2 - E_1_i * k_1;
  const double G_NaCa = 0.0034;
  const double I_NaCa_i = P_(INaCa_Multiplier) * G_NaCa * 0.65 * allo_i * (z_Na * J_NaCa_Na_i + z_Ca * J_NaCa_Ca_i);
  const double h_1_ss = 1.0 + (Na_ss * (1.0 + h_Na)) / kna3;
  const double h_2_ss = (Na_ss * h_Na) / (kna3 * h_1_ss);
  const double h_3_ss = 1.0 / h_1_ss;
  const double h_4_ss = 1.0 + (Na_ss * (1.0 + Na_ss / P_(k_Na2))) / P_(k_Na1);
  const double h_5_ss = (Na_ss * Na_ss) / (h_4_ss * P_(k_Na1) * P_(k_Na2));
  const double h_6_ss = 1.0 / h_4_ss;
  const double k_4_d_ss = (h_3_ss * wca) / h_Ca;
  const double k_4_dd_ss = h_2_ss * wnaca;
  const double k_4_ss = k_4_d_ss + k_4_dd_ss;
  const double k_6_ss = h_6_ss * Ca_ss * P_(k_Ca_on);
  const double k_7_ss = h_5_ss * h_2_ss * wna;
  const double x_1_ss = k_2 * k_4_ss * (k_7_ss + k_6_ss) + k_5 * k_7_ss * (k_2 + k_3);
  const double x_2_ss = k_1 * k_7_ss * (k_4_ss + k_5) + k_4_ss * k_6_ss * (k_1 + k_8);
  const double x_3_ss = k_1 * k_3 * (k_7_ss + k_6_ss) + k_8 * k_6_ss * (k_2 + k_3);
  const double x_4_ss = k_2 * k_8 * (k_4_ss + k_5) + k_3 * k_5 * (k_1 + k_8);
  const double E_1_ss = x_1_ss / (x_1_ss + x_2_ss + x_3_ss + x_4_ss);
  const double E_2_ss = x_2_ss / (x_1_ss + x_2_ss + x_3_ss + x_4_ss);
  const double E_3_ss = x_3_ss / (x_1_ss + x_2_ss + x_3_ss + x_4_ss);
  const double E_4_ss = x_4_ss / (x_1_ss + x_2_ss + x_3_ss + x_4_ss);
  const double allo_ss = 1.0 / (1.0 + (KmCaAct / Ca_ss) * (KmCaAct / Ca_ss));
  const double J_NaCa_Na_ss = 3.0 * (E_4_ss * k_7_ss - E_1_ss * k_8) + E_3_ss * k_4_dd_ss - E_2_ss * k_3_dd;
  const double J_NaCa_Ca_ss = E_2_ss * k_2 - E_1_ss * k_1;
  const double I_NaCa_ss =
      P_(INaCa_Multiplier) * G_NaCa * 0.35 * allo_ss * (z_Na * J_NaCa_Na_ss + z_Ca * J_NaCa_Ca_ss);

  /* I_NaK (453-503) */
  const double k1p = 949.5, k2m = 39.4, k3p = 1899.0, k3m = 79300.0, k4m = 40.0, Knai0 = 9.073, Knao0 = 27.78,
               delta = -0.1550;
  const double K_Nai = Knai0 * exp(delta * VFoverRT * 1 / 3);
  const double K_Nao = Knao0 * exp((1.0 - delta) * VFoverRT * 1 / 3);
  const double Kki = 0.5, Kko = 0.3582, H = 1.0e-7, eP = 4.2, Khp = 1.698e-7, Knap = 224.0, Kxkur = 292.0;
  const double Pnak = eP / (1.0 + H / Khp + Na_i / Knap + K_i / Kxkur);
  const double alpha_1 = (k1p * pow((Na_i / K_Nai), 3.0)) /
                         (pow((1.0 + Na_i / K_Nai), 3.0) + pow((1.0 + K_i / Kki), 2.0) - 1.0);
  const double beta_2 = (k2m * pow((P_(Na_o) / K_Nao), 3.0)) /
                        (pow((1.0 + P_(Na_o) / K_Nao), 3.0) + pow((1.0 + P_(K_o) / Kko), 2.0) - 1.0);
  const double alpha_3 = (k3p * pow((P_(K_o) / Kko), 2.0)) /
                         (pow((1.0 + P_(Na_o) / K_Nao), 3.0) + pow((1.0 + P_(K_o) / Kko), 2.0) - 1.0);
  const double beta_3 = (k3m * Pnak * H) / (1.0 + P_(MgATP));
  const double beta_4 = (k4m * pow((K_i / Kki), 2.0)) /
                        (pow((1.0 + Na_i / K_Nai), 3.0) + pow((1.0 + K_i / Kki), 2.0) - 1.0);
  const double al2 = P_(alpha_2), al4 = P_(alpha_4), be1 = P_(beta_1);
  const double x_1 = al4 * alpha_1 * al2 + beta_2 * beta_4 * beta_3 + al2 * beta_4 * beta_3 + beta_3 * alpha_1 * al2;
  const double x_2 = beta_2 * be1 * beta_4 + alpha_1 * al2 * alpha_3 + alpha_3 * be1 * beta_4 + al2 * alpha_3 * beta_4;
  const double x_3 = al2 * alpha_3 * al4 + beta_3 * beta_2 * be1 + beta_2 * be1 * al4 + alpha_3 * al4 * be1;
  const double x_4 = beta_4 * beta_3 * beta_2 + alpha_3 * al4 * alpha_1 + beta_2 * al4 * alpha_1 + beta_3 * beta_2 * alpha_1;
  const double E_1 = x_1 / (x_1 + x_2 + x_3 + x_4);
  const double E_2 = x_2 / (x_1 + x_2 + x_3 + x_4);
  const double E_3 = x_3 / (x_1 + x_2 + x_3 + x_4);
  const double E_4 = x_4 / (x_1 + x_2 + x_3 + x_4);
  const double J_NaK_Na = 3.0 * (E_1 * alpha_3 - E_2 * beta_3);
  const double J_NaK_K = 2.0 * (E_4 * be1 - E_3 * alpha_1);
  const double P_NaK = 15.4509;
  const double I_NaK = P_(INaK_Multiplier) * P_NaK * (z_Na * J_NaK_Na + z_K * J_NaK_K);

  /* I_CaCl, background currents, I_pCa, I_SAC (505-538) */
  const double I_CaCl_junc = (0.2843 * (V_m - E_Cl)) / (1. + (0.1 / Ca_ss));
  const double I_CaCl_sl = (0 * 0.2843 * (V_m - E_Cl)) / (1. + (0.1 / Ca_i));
  const double I_CaCl = I_CaCl_junc + I_CaCl_sl;
  const double x_Kb = 1.0 / (1.0 + exp(-(V_m - 10.8968) / (23.9871)));
  const double G_Kb = 0.0189;
  const double I_Kb = P_(IKb_Multiplier) * G_Kb * x_Kb * (V_m - E_K);
  const double P_Nab = 1.9239e-9;
  const double I_Nab =
      P_(INab_Multiplier) * P_Nab * z_Na * z_Na * VFFoverRT * ((Na_i * exp_z_Na - P_(Na_o)) / (exp_z_Na - 1.0));
  const double P_Cab = 5.9194e-8;
  const double I_Cab = P_(ICab_Multiplier) * P_Cab * z_Ca * z_Ca * VFFoverRT *
                       ((gamma_Ca_i * Ca_i * exp_z_Ca - gamma_Ca_o * P_(Ca_o)) / (exp_z_Ca - 1.0));
  const double P_Clb = 1.98e-3;
  const double I_Clb = P_Clb * (V_m - E_Cl);
  const double G_pCa = 0.0005;
  const double I_pCa = P_(IpCa_Multiplier) * ((G_pCa * Ca_i) / (0.0005 + Ca_i));
  double I_SAC = P_(G_sac) * (V_m - P_(E_sac)) / (1. + P_(K_sac) * exp(-P_(alpha) * (stretch - 1.)));
  I_SAC *= P_(ISAC_SWITCH);

  /* total current (540-548) */
  const double cur_I_tot = I_Na + I_Na_late + I_to + I_CaL + I_CaNa + I_CaK + I_Kr + I_Ks + I_K1 + I_NaCa_i + I_NaCa_ss +
                           I_NaK + I_Nab + I_Cab + I_Kb + I_pCa + I_Clb + I_CaCl + I_SAC + i_external;
  const double I_tot = -cur_I_tot;

  /* fluxes (550-590) */
  const double J_diff_Na = (Na_ss - Na_i) / 2.0;
  const double J_diff_Ca = (Ca_ss - Ca_i) / 0.2;
  const double J_diff_K = (K_ss - K_i) / 2.0;
  const double K_inf_rel = 1.7;
  double J_rel_NP_inf = (P_(alpha_rel) * (-I_CaL)) / (1.0 + pow((K_inf_rel / Ca_jsr), 8.0));
  double J_rel_CaMK_inf = (P_(alpha_rel_CaMK) * (-I_CaL)) / (1.0 + pow((K_inf_rel / Ca_jsr), 8.0));
  if (P_(celltype) == 2.0) {
    J_rel_NP_inf *= 1.7;
    J_rel_CaMK_inf *= 1.7;
  }
  const double tau_rel_NP_b = P_(beta_tau) / (1.0 + (0.0123 / Ca_jsr));
  const double tau_rel_NP = tau_rel_NP_b < 0.001 ? 0.001 : tau_rel_NP_b;
  b[MB_J_rel_NP] = J_rel_NP_inf - (J_rel_NP_inf - b[MB_J_rel_NP]) * exp(-tinc / tau_rel_NP);
  const double tau_rel_CaMK_b = P_(beta_tau_CaMK) / (1.0 + (0.0123 / Ca_jsr));
  const double tau_rel_CaMK = tau_rel_CaMK_b < 0.001 ? 0.001 : tau_rel_CaMK_b;
  b[MB_J_rel_CaMK] = J_rel_CaMK_inf - (J_rel_CaMK_inf - b[MB_J_rel_CaMK]) * exp(-tinc / tau_rel_CaMK);
  const double J_rel = 1.5378 * (1.0 - phi) * b[MB_J_rel_NP] + phi * b[MB_J_rel_CaMK];
  double J_up_NP = (0.005425 * Ca_i) / (0.00092 + Ca_i);
  double J_up_CaMK = (2.75 * 0.005425 * Ca_i) / (0.00092 - 0.00017 + Ca_i);
  if (P_(celltype) == 1.0) {
    J_up_NP *= 1.3;
    J_up_CaMK *= 1.3;
  }
  const double J_leak = (0.0048825 * Ca_nsr) / 15.0;
  const double J_up = ((1.0 - phi) * J_up_NP + (phi * J_up_CaMK) - J_leak);
  const double J_tr = (Ca_nsr - Ca_jsr) / 60.0;

  /* concentrations (592-654) */
  const double cur_Nai = I_Na + I_Na_late + 3.0 * I_NaCa_i + I_CaNa_i + 3.0 * I_NaK + I_Nab;
  const double dNa_i = -(cur_Nai)*util_1 + J_diff_Na * util_2;
  b[MB_Na_i] = Na_i + tinc * dNa_i;
  const double dNa_ss = -(I_CaNa_ss + 3.0 * I_NaCa_ss) * util_3 - J_diff_Na;
  b[MB_Na_ss] = Na_ss + tinc * dNa_ss;
  const double cur_Ki = I_to + I_Kr + I_Ks + I_K1 + I_Kb + i_external - 2.0 * I_NaK + I_CaK_i;
  const double dK_i = -(cur_Ki)*util_1 + J_diff_K * util_2;
  b[MB_K_i] = K_i + tinc * dK_i;
  const double dK_ss = -(I_CaK_ss)*util_3 - J_diff_K;
  b[MB_K_ss] = K_ss + tinc * dK_ss;
  double cmdnmax = 0.05;
  if (P_(celltype) == 1) cmdnmax *= 1.3;
  const double kmcmdn = 0.00238, trpnmax = 0.07, BSRmax = 0.047, KmBSR = 0.00087, BSLmax = 1.124, KmBSL = 0.0087,
               csqnmax = 10.0, kmcsqn = 0.8;
  const double Ca_T50 = (P_(Ca_T50) + P_(beta1) * (lambda_m - 1.0));
  const double Ca_TRPN = b[MB_Ca_TRPN];
  const double dCaTRPN = P_(k_TRPN) * (pow(1000 * Ca_i / Ca_T50, P_(n_TRPN)) * (1. - Ca_TRPN) - Ca_TRPN);
  b[MB_Ca_TRPN] = Ca_TRPN + tinc * dCaTRPN;
  const double I_Trpn = trpnmax * dCaTRPN;
  const double beta_Cai = 1.0 / (1.0 + ((cmdnmax * kmcmdn) / pow((kmcmdn + Ca_i), 2.0)));
  const double cur_Cai = I_CaL_i + I_pCa + I_Cab - 2.0 * I_NaCa_i;
  const double dCa_i =
      beta_Cai * (-(cur_Cai)*0.5 * util_1 - J_up * (P_(v_nsr) / P_(v_myo)) + J_diff_Ca * util_2 - I_Trpn);
  b[MB_Ca_i] = Ca_i + tinc * dCa_i;
  const double beta_Cass =
      1.0 / (1.0 + ((BSRmax * KmBSR) / pow((KmBSR + Ca_ss), 2.0)) + ((BSLmax * KmBSL) / pow((KmBSL + Ca_ss), 2.0)));
  const double dCa_ss =
      beta_Cass * (-(I_CaL_ss - 2.0 * I_NaCa_ss) * 0.5 * util_3 + J_rel * (P_(v_jsr) / P_(v_ss)) - J_diff_Ca);
  b[MB_Ca_ss] = Ca_ss + tinc * dCa_ss;
  const double dCa_nsr = J_up - ((J_tr * P_(v_jsr)) / P_(v_nsr));
  b[MB_Ca_nsr] = Ca_nsr + tinc * dCa_nsr;
  const double beta_Cajsr = 1.0 / (1.0 + ((csqnmax * kmcsqn) / pow((kmcsqn + Ca_jsr), 2.0)));
  const double dCa_jsr = beta_Cajsr * (J_tr - J_rel);
  b[MB_Ca_jsr] = Ca_jsr + tinc * dCa_jsr;

  /* the values the reference keeps in its block (Tomek.h:47-52) */
  b[MB_I_Na] = I_Na; b[MB_I_Na_late] = I_Na_late; b[MB_I_to] = I_to; b[MB_I_CaL] = I_CaL; b[MB_I_CaNa] = I_CaNa;
  b[MB_I_CaK] = I_CaK; b[MB_I_CaL_i] = I_CaL_i; b[MB_I_CaL_ss] = I_CaL_ss; b[MB_I_CaNa_i] = I_CaNa_i;
  b[MB_I_CaNa_ss] = I_CaNa_ss; b[MB_I_CaK_i] = I_CaK_i; b[MB_I_CaK_ss] = I_CaK_ss; b[MB_I_Kr] = I_Kr;
  b[MB_I_Ks] = I_Ks; b[MB_I_K1] = I_K1; b[MB_I_NaCa_i] = I_NaCa_i; b[MB_I_NaCa_ss] = I_NaCa_ss; b[MB_I_NaK] = I_NaK;
  b[MB_I_CaCl_junc] = I_CaCl_junc; b[MB_I_CaCl_sl] = I_CaCl_sl; b[MB_I_CaCl] = I_CaCl; b[MB_I_Nab] = I_Nab;
  b[MB_I_Cab] = I_Cab; b[MB_I_Kb] = I_Kb; b[MB_I_Clb] = I_Clb; b[MB_I_pCa] = I_pCa; b[MB_J_diff_Na] = J_diff_Na;
  b[MB_J_diff_Ca] = J_diff_Ca; b[MB_J_diff_K] = J_diff_K; b[MB_J_leak] = J_leak; b[MB_J_rel] = J_rel;
  b[MB_J_tr] = J_tr; b[MB_J_up] = J_up; b[MB_cur_I_tot] = cur_I_tot; b[MB_I_tot] = I_tot; b[MB_I_SAC] = I_SAC;
  return 0.001 * tinc * I_tot;
}
#undef P_

/* ---------------------------------------------------------------- public entry points */
static void derive(int model, double *P) {
  if (model == CMO_TT2) tt2_derive(P);
  else if (model == CMO_CRN) crn_derive(P);
  else if (model == CMO_ORD) ord_derive(P);
  else tom_derive(P);
}

int cmo_build_tables(int model, const double *P_in, double dt, double *tables) {
  int np = cmo_n_params(model);
  if (np < 0) return -1;
  double *P = (double *)malloc(np * sizeof(double));
  memcpy(P, P_in, np * sizeof(double));
  derive(model, P);
  if (cmo_n_tables(model) > 0) memset(tables, 0, (size_t)cmo_n_tables(model) * CMO_RTDT * sizeof(double));
  if (model == CMO_TT2) tt2_tables(P, dt, tables);
  else if (model == CMO_CRN) crn_tables(P, dt, tables);
  free(P);
  return 0;
}

void cmo_init_state(int model, const double *P, double *block) {
  if (model == CMO_TT2) tt2_init(P, block);
  else if (model == CMO_CRN) crn_init(P, block);
  else if (model == CMO_ORD) ord_init(P, block);
  else tom_init(P, block);
}

double cmo_init_vm(int model, const double *P) {
  return model == CMO_TT2 ? P[T_init_V_m]
                          : (model == CMO_CRN ? P[C_Init_Vm] : (model == CMO_ORD ? P[O_Init_Vm] : P[M_Init_Vm]));
}

double cmo_calc(int model, const double *P_in, const double *tables, double *block, double dt, double V,
                double i_ext, double stretch) {
  /* P_in holds base and derived values (the caller derives once via cmo_derive). */
  if (model == CMO_TT2) return tt2_calc(P_in, tables, block, dt, V, i_ext);
  if (model == CMO_CRN) return crn_calc(P_in, tables, block, dt, V, i_ext, stretch);
  if (model == CMO_ORD) return ord_calc(P_in, block, dt, V, i_ext, stretch);
  return tom_calc(P_in, block, dt, V, i_ext, stretch);
}

/* Fills the derived slots of P in place (Calculate()). */
void cmo_derive(int model, double *P) { derive(model, P); }

typedef struct {
  int model;
  const double *P;
  const double *tables;
  long lo, hi, n_cells;
  double *blocks, *Vm;
  int n_het;
  const int *het_idx;
  const double *het_vals;
  long n_steps;
  double dt, t0, textbegin;
  const double *tb_cell;
  double textlen, bcl, amp;
  long rec_every;
  double *trace;
  int bad;
} run_args;

static void *run_range(void *argp) {
  run_args *a = (run_args *)argp;
  const int np = cmo_n_params(a->model), ns = cmo_state_doubles(a->model);
  double *Pc = (double *)malloc(np * sizeof(double));
  const long n_rec = a->rec_every > 0 ? (a->n_steps + a->rec_every - 1) / a->rec_every : 0;
  for (long c = a->lo; c < a->hi; c++) {
    memcpy(Pc, a->P, np * sizeof(double));
    for (int k = 0; k < a->n_het; k++) Pc[a->het_idx[k]] = a->het_vals[(size_t)k * a->n_cells + c];
    double *blk = a->blocks + (size_t)c * ns;
    double t = a->t0, tb = a->tb_cell ? a->tb_cell[c] : a->textbegin, v = a->Vm[c];
    for (long s = 0; s < a->n_steps; s++) {
      if (a->trace && a->rec_every > 0 && s % a->rec_every == 0) a->trace[c * n_rec + s / a->rec_every] = v;
      /* CellModel.h:405-419 with textend = thresVm = freq = HUGE */
      double i_ext = 0.0;
      if (t >= tb) {
        i_ext = a->amp;
        if (t >= tb + a->textlen) tb += a->bcl;
      }
      if (a->model == CMO_TT2) v += tt2_calc(Pc, a->tables, blk, a->dt, v, i_ext);
      else if (a->model == CMO_CRN) v += crn_calc(Pc, a->tables, blk, a->dt, v, i_ext, 1.0);
      else if (a->model == CMO_ORD) v += ord_calc(Pc, blk, a->dt, v, i_ext, 1.0);
      else v += tom_calc(Pc, blk, a->dt, v, i_ext, 1.0);
      t += a->dt;
    }
    if (isnan(v)) a->bad = 1;
    a->Vm[c] = v;
  }
  free(Pc);
  return 0;
}

int cmo_run(int model, const double *P, const double *tables, long n_cells, double *blocks, double *Vm,
            int n_het, const int *het_idx, const double *het_vals, long n_steps, double dt, double t0,
            double textbegin, const double *textbegin_per_cell, double textlen, double bcl, double amp,
            long rec_every, double *trace, int n_threads) {
  if (cmo_n_params(model) < 0) return -1;
  if (n_threads < 1) n_threads = 1;
  if (n_threads > n_cells) n_threads = (int)(n_cells > 0 ? n_cells : 1);
  run_args *args = (run_args *)calloc(n_threads, sizeof(run_args));
  pthread_t *th = (pthread_t *)calloc(n_threads, sizeof(pthread_t));
  for (int k = 0; k < n_threads; k++) {
    run_args *a = &args[k];
    a->model = model; a->P = P; a->tables = tables; a->n_cells = n_cells;
    a->lo = n_cells * k / n_threads; a->hi = n_cells * (k + 1) / n_threads;
    a->blocks = blocks; a->Vm = Vm; a->n_het = n_het; a->het_idx = het_idx; a->het_vals = het_vals;
    a->n_steps = n_steps; a->dt = dt; a->t0 = t0; a->textbegin = textbegin; a->tb_cell = textbegin_per_cell;
    a->textlen = textlen; a->bcl = bcl; a->amp = amp; a->rec_every = rec_every; a->trace = trace;
  }
  if (n_threads == 1) {
    run_range(&args[0]);
  } else {
    for (int k = 0; k < n_threads; k++) pthread_create(&th[k], 0, run_range, &args[k]);
    for (int k = 0; k < n_threads; k++) pthread_join(th[k], 0);
  }
  int bad = 0;
  for (int k = 0; k < n_threads; k++) bad |= args[k].bad;
  free(args);
  free(th);
  return bad ? -3 : 0;
}

/* ---------------------------------------------------------------- monodomain coupling */
/* The explicit monodomain step of acCELLerate::IntraStep (acCELLerate.cpp:1839-2005; no mass
 * matrix, no Gauss points, no implicit smoothing, Godunov current scheme):
 *   B = A * Vm                           MatMult (1849), row entries summed in CSR order
 *   i_ext = B * scale + stimulus         nA/cell conversion (1880-1887), conditions (1892)
 *   dVm = Calc(dt, Vm, i_ext, 1, 1)      CalcCellModels (1757-1770)
 *   Vm += dVm, NaN / range check         (1930-1949)
 *   act = t where act == -1 and Vm >= threshold   (1997-2005)
 * The stimulus follows the driver rule (CellModel.h:405-419) with per-cell first times. */
typedef struct {
  int model;
  const double *P, *tables;
  long n_cells, lo, hi;
  double *blocks, *v_old, *v_new, *B;
  int n_het;
  const int *het_idx;
  const double *het_vals;
  const long *rowptr;
  const int *col;
  const double *val, *scale;
  double uniform_scale;
  long n_steps;
  double dt, t0, textlen, bcl, amp, act_threshold, vm_range;
  double *tb, *act;
  long rec_every;
  double *trace;
  pthread_barrier_t *bar;
  int bad;
} mono_args;

static void *mono_range(void *argp) {
  mono_args *a = (mono_args *)argp;
  const int np = cmo_n_params(a->model), ns = cmo_state_doubles(a->model);
  double *Pc = (double *)malloc(np * sizeof(double));
  const long n_rec = a->rec_every > 0 ? (a->n_steps + a->rec_every - 1) / a->rec_every : 0;
  double *vo = a->v_old, *vn = a->v_new;
  double t = a->t0;
  for (long s = 0; s < a->n_steps; s++) {
    for (long i = a->lo; i < a->hi; i++) {
      double b = 0.0;
      for (long e = a->rowptr[i]; e < a->rowptr[i + 1]; e++) b += a->val[e] * vo[a->col[e]];
      a->B[i] = b;
      if (a->trace && a->rec_every > 0 && s % a->rec_every == 0) a->trace[i * n_rec + s / a->rec_every] = vo[i];
    }
    pthread_barrier_wait(a->bar);
    for (long c = a->lo; c < a->hi; c++) {
      memcpy(Pc, a->P, np * sizeof(double));
      for (int k = 0; k < a->n_het; k++) Pc[a->het_idx[k]] = a->het_vals[(size_t)k * a->n_cells + c];
      double stim = 0.0;
      if (t >= a->tb[c]) {
        stim = a->amp;
        if (t >= a->tb[c] + a->textlen) a->tb[c] += a->bcl;
      }
      const double i_ext = a->B[c] * (a->scale ? a->scale[c] : a->uniform_scale) + stim;
      double *blk = a->blocks + (size_t)c * ns;
      double dv;
      if (a->model == CMO_TT2) dv = tt2_calc(Pc, a->tables, blk, a->dt, vo[c], i_ext);
      else if (a->model == CMO_CRN) dv = crn_calc(Pc, a->tables, blk, a->dt, vo[c], i_ext, 1.0);
      else if (a->model == CMO_ORD) dv = ord_calc(Pc, blk, a->dt, vo[c], i_ext, 1.0);
      else dv = tom_calc(Pc, blk, a->dt, vo[c], i_ext, 1.0);
      const double v = vo[c] + dv;
      vn[c] = v;
      if (isnan(v) || (a->vm_range > 0.0 && (v > a->vm_range || v < -a->vm_range))) a->bad = 1;
      if (a->act && a->act[c] == -1.0 && v >= a->act_threshold) a->act[c] = t;
    }
    pthread_barrier_wait(a->bar);
    double *tmp = vo;
    vo = vn;
    vn = tmp;
    t += a->dt;
  }
  free(Pc);
  return 0;
}

int cmo_mono_run(int model, const double *P, const double *tables, long n_cells, double *blocks, double *Vm,
                 int n_het, const int *het_idx, const double *het_vals, const long *rowptr, const int *col,
                 const double *val, const double *scale, double uniform_scale, long n_steps, double dt, double t0,
                 double textbegin, const double *textbegin_per_cell, double textlen, double bcl, double amp,
                 double *act, double act_threshold, double vm_range, long rec_every, double *trace, int n_threads) {
  if (cmo_n_params(model) < 0 || n_cells <= 0) return -1;
  if (n_threads < 1) n_threads = 1;
  if (n_threads > n_cells) n_threads = (int)n_cells;
  double *v2 = (double *)malloc(n_cells * sizeof(double));
  double *B = (double *)malloc(n_cells * sizeof(double));
  double *tb = (double *)malloc(n_cells * sizeof(double));
  for (long c = 0; c < n_cells; c++) tb[c] = textbegin_per_cell ? textbegin_per_cell[c] : textbegin;
  mono_args *args = (mono_args *)calloc(n_threads, sizeof(mono_args));
  pthread_t *th = (pthread_t *)calloc(n_threads, sizeof(pthread_t));
  pthread_barrier_t bar;
  pthread_barrier_init(&bar, 0, n_threads);
  for (int k = 0; k < n_threads; k++) {
    mono_args *a = &args[k];
    a->model = model; a->P = P; a->tables = tables; a->n_cells = n_cells;
    a->lo = n_cells * k / n_threads; a->hi = n_cells * (k + 1) / n_threads;
    a->blocks = blocks; a->v_old = Vm; a->v_new = v2; a->B = B;
    a->n_het = n_het; a->het_idx = het_idx; a->het_vals = het_vals;
    a->rowptr = rowptr; a->col = col; a->val = val; a->scale = scale; a->uniform_scale = uniform_scale;
    a->n_steps = n_steps; a->dt = dt; a->t0 = t0; a->textlen = textlen; a->bcl = bcl; a->amp = amp;
    a->act_threshold = act_threshold; a->vm_range = vm_range; a->tb = tb; a->act = act;
    a->rec_every = rec_every; a->trace = trace; a->bar = &bar;
  }
  if (n_threads == 1) {
    mono_range(&args[0]);
  } else {
    for (int k = 0; k < n_threads; k++) pthread_create(&th[k], 0, mono_range, &args[k]);
    for (int k = 0; k < n_threads; k++) pthread_join(th[k], 0);
  }
  if (n_steps % 2) memcpy(Vm, v2, n_cells * sizeof(double)); /* the last step wrote the second buffer */
  int bad = 0;
  for (int k = 0; k < n_threads; k++) bad |= args[k].bad;
  pthread_barrier_destroy(&bar);
  free(args);
  free(th);
  free(v2);
  free(B);
  free(tb);
  return bad ? -3 : 0;
}
