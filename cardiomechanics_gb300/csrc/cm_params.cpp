// Parameter sets of the models: built-in defaults, .ev loading, derived values and the
// FP64 voltage lookup tables. The arithmetic of derive() and build_tables() follows the
// reference expression by expression (TenTusscher2Parameters.cpp:313-485,
// CourtemancheParameters.cpp:246-395, OHaraRudyParameters.cpp:246-316) so that, against the
// same libm, derived values and tables agree with the reference bit for bit; the kernels
// then only read them. O'Hara-Rudy has no tables: its Calc evaluates every gate directly.
#include "cm_params.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "../../include/cardiomech_gb300.h"

namespace cm {
namespace {

// ----------------------------------------------------------------- TenTusscher2
// Defaults: the values of the reference's TenTusscher2_original_Epi.ev.
const ParamDef kTT2Base[] = {
    {"R", 8314.472}, {"Tx", 310.0}, {"F", 96485.3415}, {"init_m", 0.0},
    {"init_h", 0.75}, {"init_j", 0.75}, {"init_Xr1", 0.0}, {"init_Xr2", 1.0},
    {"init_Xs", 0.0}, {"init_r", 0.0}, {"init_s", 1.0}, {"init_d", 0.0},
    {"init_f", 1.0}, {"init_f2", 1.0}, {"init_fCa", 1.0}, {"init_Rq", 1.0},
    {"K_o", 5.4}, {"Ca_o", 2.0}, {"Na_o", 140.0}, {"Vc", 0.016404},
    {"Vsr", 0.001094}, {"Vss", 5.468e-05}, {"Vrel", 0.102}, {"ks1", 0.15},
    {"ks2", 0.045}, {"k3", 0.06}, {"k4", 0.005}, {"EC", 1.5},
    {"max_sr", 2.5}, {"min_sr", 1.0}, {"Vxfer", 0.0038}, {"Bufc", 0.2},
    {"Kbufc", 0.001}, {"Bufsr", 10.0}, {"Kbufsr", 0.3}, {"Bufss", 0.4},
    {"Kbufss", 0.00025}, {"Vmaxup", 0.006375}, {"Kup", 0.00025}, {"C", 0.185},
    {"g_Kr", 0.153}, {"pKNa", 0.03}, {"g_Ks", 0.392}, {"g_K1", 5.405},
    {"g_to", 0.294}, {"g_Na", 14.838}, {"g_bNa", 0.00029}, {"KmK", 1.0},
    {"KmNa", 40.0}, {"knak", 2.724}, {"g_CaL", 3.98e-05}, {"g_bCa", 0.000592},
    {"kNaCa", 1000.0}, {"KmNai", 87.5}, {"KmCa", 1.38}, {"ksat", 0.1},
    {"n", 0.35}, {"g_pCa", 0.1238}, {"KpCa", 0.0005}, {"g_pK", 0.0146},
    {"init_V_m", -0.0862}, {"init_Cai", 7e-05}, {"init_CaSR", 1.3}, {"init_CaSS", 7e-05},
    {"init_Nai", 7.67}, {"init_Ki", 138.3}, {"CaiMin", 0.0}, {"CaiMax", 0.012},
    {"s_inf_vHalf", 20.0}, {"tau_s_f1", 85.0}, {"tau_s_slope1", 320.0}, {"tau_s_vHalf1", 45.0},
    {"tau_s_enable", 1.0}, {"tau_s_add", 3.0}, {"m_Xr1_1", -26.0}, {"m_Xr1_2", 7.0},
    {"a_Xr1_1", -45.0}, {"a_Xr1_2", 10.0}, {"b_Xr1_1", -30.0}, {"b_Xr1_2", 11.5},
    {"K_Q10Xr1", 1.0}, {"m_Xr2_1", -88.0}, {"m_Xr2_2", 24.0}, {"a_Xr2_1", -60.0},
    {"a_Xr2_2", 20.0}, {"b_Xr2_1", 60.0}, {"b_Xr2_2", 20.0}, {"K_Q10Xr2", 1.0},
    {"m_Xs_1", -5.0}, {"m_Xs_2", 14.0}, {"a_Xs_1", 5.0}, {"a_Xs_2", 6.0},
    {"b_Xs_1", 35.0}, {"b_Xs_2", 15.0}, {"tau_Xs_add", 80.0}, {"K_Q10Xs", 1.0},
    {"stim_duration", 0.001}, {"Amp", 2.0}, {"Vcell", 1.6404e-14},
};
const char *const kTT2Derived[] = {"RTONF", "inverseRTONF", "vi", "inverseviF", "inverseviF2", "inversevssF2",
                                   "VcdVsr", "Kupsquare", "BufcPKbufc", "KmNai3", "Nao3", "StepCai"};
const char *const kTT2Tables[] = {"m_inf", "h_inf", "j_inf", "Xr1_inf", "Xr2_inf", "Xs_inf", "s_inf", "r_inf",
                                  "d_inf", "f_inf", "f2_inf", "exptau_m", "exptau_h", "exptau_j", "exptau_Xr1",
                                  "exptau_Xr2", "exptau_Xs", "exptau_s", "exptau_r", "exptau_d", "exptau_f",
                                  "exptau_f2", "NaK_P1", "rec_ipK", "NaCa_P1", "NaCa_P2", "CaL_P1", "CaL_P2", "ECA"};
const char *const kTT2State[] = {"Ca_i", "CaSR", "CaSS", "Na_i", "K_i", "m", "h", "j", "xr1",
                                 "xr2", "xs", "r", "s", "d", "f", "f2", "fCa", "Rq"};
const char *const kTT2Het[] = {"g_Na", "g_Kr", "g_K1", "g_Ks", "g_to", "g_CaL"};

// ----------------------------------------------------------------- Courtemanche
// Defaults: the values of the reference's CourtemancheEtAl.ev.
const ParamDef kCRNBase[] = {
    {"R", 8.3143}, {"Tx", 310.0}, {"F", 96.4867}, {"C_m", 100.0},
    {"Vcell", 20100.0}, {"Vcell_outside", 2895291.79}, {"part_i", 0.68}, {"part_up", 0.0552},
    {"part_rel", 0.0048}, {"Tfac", 3.0}, {"K_o", 5.4}, {"Na_o", 140.0},
    {"Ca_o", 1.8}, {"g_Na", 7.8}, {"g_to", 0.1652}, {"g_Kr", 0.029411765},
    {"g_Ks", 0.12941176}, {"g_CaL", 0.12375}, {"g_K1", 0.09}, {"g_bNa", 0.0006744375},
    {"g_bCa", 0.001131}, {"I_NaKmax", 0.59933874}, {"k_mNai", 10.0}, {"k_mKo", 1.5},
    {"I_pCamax", 0.275}, {"k_mpCa", 0.0005}, {"k_NaCa", 1600.0}, {"k_mNa", 87.5},
    {"k_mCa", 1.38}, {"k_sat", 0.1}, {"gamm", 0.35}, {"CMDNmax", 0.05},
    {"TRPNmax", 0.07}, {"CSQNmax", 10.0}, {"K_mcmdn", 0.00238}, {"K_mtrpn", 0.0005},
    {"K_mcsqn", 0.8}, {"k_rel", 30.0}, {"k_up", 0.00092}, {"I_upmax", 0.005},
    {"Ca_upmax", 15.0}, {"t_tr", 180.0}, {"shiftm", 0.0}, {"shifth", 0.0},
    {"shiftj", 0.0}, {"shiftoa", 0.0}, {"C_oa_1", 0.65}, {"C_oa_2", 8.5},
    {"C_oa_3", 59.0}, {"C_oa_4", 17.0}, {"C_oa_5", 17.54}, {"C_oa_6", 20.47},
    {"CaL_fT_1", 9.0}, {"Init_Na_i", 13.485}, {"Init_K_i", 127.4718}, {"Init_m", 0.003473},
    {"Init_oa", 0.032306}, {"Init_ua", 0.005555}, {"Init_d", 0.000156}, {"Init_f_Ca", 0.746737},
    {"Init_Ca_i", 0.000119}, {"Init_Ca_up", 1.57562}, {"Init_Ca_rel", 0.921569}, {"Init_h", 0.955651},
    {"Init_j", 0.970611}, {"Init_oi", 0.999071}, {"Init_ui", 0.991169}, {"Init_Xr", 0.002347},
    {"Init_Xs", 0.02107}, {"Init_f", 0.926327}, {"Init_u", 0.0}, {"Init_v", 1.0},
    {"Init_w", 0.999146}, {"Init_Vm", -0.080124}, {"ua_a1", 0.65}, {"ua_a2", 10.0},
    {"ua_a3", -8.5}, {"ua_a4", -30.0}, {"ua_a5", -59.0}, {"ua_b1", 2.5},
    {"ua_b2", 82.0}, {"ua_b3", 17.0}, {"ua_m1", 30.3}, {"ua_m2", -9.6},
    {"ua_KQ10", 3.0}, {"ui_a1", 1.0}, {"ui_a2", 21.0}, {"ui_a3", -185.0},
    {"ui_a4", -28.0}, {"ui_b1", -158.0}, {"ui_b2", -16.0}, {"ui_m1", -99.45},
    {"ui_m2", 27.48}, {"ui_KQ10", 3.0}, {"g_Kur1", 0.005}, {"g_Kur2", 0.05},
    {"g_Kur3", -15.0}, {"g_Kur4", -13.0}, {"g_K1_1", 80.0}, {"g_K1_2", 0.07},
    {"Xr_a1", 0.0003}, {"Xr_a2", 14.1}, {"Xr_a3", -5.0}, {"Xr_b1", -3.3328},
    {"Xr_b2", 5.1237}, {"Xr_KQ10", 1.0}, {"Xr_m1", 14.1}, {"Xr_m2", -6.5},
    {"g_Kr1", 15.0}, {"g_Kr2", 22.4}, {"Xs_a1", 4e-05}, {"Xs_a2", -19.9},
    {"Xs_a3", -17.0}, {"Xs_b1", -19.9}, {"Xs_b2", 9.0}, {"Xs_KQ10", 2.0},
    {"Xs_m1", -19.9}, {"Xs_m2", -12.7}, {"m_a1", 0.32}, {"m_a2", 0.1},
    {"m_b1", 0.08}, {"m_b2", 11.0}, {"h_a1", 0.135}, {"h_a2", 6.8},
    {"h_b1", 3.56}, {"h_b2", 0.079}, {"h_b3", 310000.0}, {"h_b4", 0.35},
    {"h_b5", 0.13}, {"h_b6", 11.1}, {"j_a1", -127140.0}, {"j_a2", 0.2444},
    {"j_a3", 3.474e-05}, {"j_a4", -0.04391}, {"j_a5", 0.311}, {"j_b1", 0.1212},
    {"j_b2", -0.01052}, {"j_b3", -0.1378}, {"j_b4", 0.3}, {"j_b5", -2.535e-07},
    {"j_b6", -0.1}, {"tau_j_mult", 1.0}, {"tau_f_mult", 1.0}, {"E_rL", 65.0},
    {"ISAC_SWITCH", 0.0}, {"alpha", 3.0}, {"G_sac", 0.27}, {"K_sac", 100.0},
    {"E_sac", 0.0}, {"Init_Ca_TRPN", 0.001315}, {"beta1", -1.2}, {"Ca_T50", 0.86},
    {"k_TRPN", 0.1}, {"n_TRPN", 2.0},
};
const char *const kCRNDerived[] = {"RTdF", "FdRT", "RTd2F", "Vi", "Vup", "Vrel", "VupdVi", "VreldVi",
                                   "VreldVup", "CmdFvi", "Cmd2F", "csqnkm", "kmcsqnm2", "kkmcsqn", "cmdnkm",
                                   "kmcmdnm2", "kkmcmdn", "kupleak", "dt_tr"};
const char *const kCRNTables[] = {"m_m", "exptau_m", "m_h", "exptau_h", "m_j", "exptau_j", "m_oa", "exptau_oa",
                                  "m_oi", "exptau_oi", "m_ua", "exptau_ua", "m_ui", "exptau_ui", "m_Xr",
                                  "exptau_Xr", "m_Xs", "exptau_Xs", "m_d", "exptau_d", "m_f", "exptau_f",
                                  "m_w", "exptau_w", "expVm", "CK1", "g_Kur", "CKr", "CNaK", "CNaCa"};
const char *const kCRNState[] = {"Ca_i", "Ca_up", "Ca_rel", "h", "j", "oi", "ui", "Xr", "Xs", "u", "v",
                                 "w", "Na_i", "K_i", "m", "oa", "ua", "d", "f", "f_Ca", "Ca_TRPN"};
const char *const kCRNHet[] = {"g_Na", "g_to", "g_Ks", "g_CaL", "g_bNa", "g_bCa"};


// ----------------------------------------------------------------- O'Hara-Rudy
// Defaults: the values of the reference's OHaraRudy.ev (= OHaraRudy_endo.ev, celltype 0);
// OHaraRudy_epi.ev (celltype 1) and OHaraRudy_mid.ev (celltype 2) load through .ev files.
// Order: NS_OHaraRudyParameters::varType (OHaraRudyParameters.h:40-180).
const ParamDef kORDBase[] = {
    {"amplitude", -50.0}, {"duration", 0.001}, {"celltype", 0.0}, {"Na_o", 140.0}, {"Ca_o", 1.8}, {"K_o", 5.4},
    {"INaF_Multiplier", 1.0}, {"INaL_Multiplier", 1.0}, {"Ito_Multiplier", 1.0}, {"PCa_Multiplier", 1.0},
    {"IKr_Multiplier", 1.0}, {"IKs_Multiplier", 1.0}, {"IK1_Multiplier", 1.0}, {"INaCa_Multiplier", 1.0},
    {"INaK_Multiplier", 1.0}, {"IKb_Multiplier", 1.0}, {"INab_Multiplier", 1.0}, {"ICab_Multiplier", 1.0},
    {"IpCa_Multiplier", 1.0}, {"Init_Vm", -0.087962}, {"Init_Na_i", 7.440001}, {"Init_Na_ss", 7.440078},
    {"Init_K_i", 144.078}, {"Init_K_ss", 144.078}, {"Init_Ca_i", 7.8e-05}, {"Init_Ca_ss", 7.7e-05},
    {"Init_Ca_nsr", 1.698587}, {"Init_Ca_jsr", 1.605945}, {"Init_m", 0.007374}, {"Init_h_fast", 0.820716},
    {"Init_h_slow", 0.820717}, {"Init_j", 0.820534}, {"Init_h_CaMK_slow", 0.628164}, {"Init_j_CaMK", 0.819121},
    {"Init_m_L", 0.00019}, {"Init_h_L", 0.48385}, {"Init_h_L_CaMK", 0.249012}, {"Init_a", 0.001004},
    {"Init_i_fast", 0.999551}, {"Init_i_slow", 0.487698}, {"Init_a_CaMK", 0.000511},
    {"Init_i_CaMK_fast", 0.999551}, {"Init_i_CaMK_slow", 0.538887}, {"Init_d", 0.0}, {"Init_f_fast", 1.0},
    {"Init_f_slow", 0.88001}, {"Init_f_Ca_fast", 1.0}, {"Init_f_Ca_slow", 0.99884}, {"Init_j_Ca", 0.999717},
    {"Init_n", 0.001876}, {"Init_f_CaMK_fast", 1.0}, {"Init_f_Ca_CaMK_fast", 1.0}, {"Init_x_r_fast", 1.2e-05},
    {"Init_x_r_slow", 0.551134}, {"Init_x_s1", 0.322839}, {"Init_x_s2", 0.000194}, {"Init_x_K1", 0.99677},
    {"Init_J_rel_NP", 0.0}, {"Init_J_rel_CaMK", 0.0}, {"Init_CaMK_trap", 0.01941}, {"ISAC_SWITCH", 0.0},
    {"alpha", 3.0}, {"G_sac", 0.27}, {"K_sac", 100.0}, {"E_sac", 0.0}, {"Init_Ca_TRPN", 0.000654},
    {"beta1", -1.2}, {"Ca_T50", 0.805}, {"k_TRPN", 0.1}, {"n_TRPN", 2.0}, {"HFM_Multiplier", 1.0},
    {"HF_Gomez_1", 1.0}, {"HF_Gomez_2", 1.0}, {"HF_Gomez_3", 1.0}, {"HF_Gomez_4", 1.0}, {"HF_Gomez_5", 1.0},
    {"HF_Gomez_6", 1.0}, {"HF_Gomez_7", 1.0}, {"HF_Gomez_8", 1.0}, {"HF_Gomez_9", 1.0}, {"HF_Gomez_0", 1.0},
};
const char *const kORDDerived[] = {
    "R", "T", "F", "L", "r", "tau_h_L", "A_h_fast", "A_h_slow", "v_cell", "A_geo", "A_cap", "v_myo", "v_nsr",
    "v_jsr", "v_ss", "P_CaNa", "P_CaK", "P_Ca_CaMK", "P_CaNa_CaMK", "P_CaK_CaMK", "A_f_fast", "A_f_slow",
    "k_Na1", "k_Na2", "k_asymm", "k_Ca_on", "k_Ca_off", "k_m_1", "k_p_2", "k_p_4", "MgADP", "MgATP", "K_MgATP",
    "beta_tau", "P_Ca", "h_10", "h_11", "h_12", "k_1", "k_2", "k_5", "beta_1", "alpha_2", "alpha_4", "alpha_rel",
    "beta_tau_CaMK", "alpha_rel_CaMK", "tau_h_LCaMK", "RToverF"};
const char *const kORDState[] = {
    "m", "h_fast", "h_slow", "j", "h_CaMK_slow", "j_CaMK", "m_L", "h_L", "h_L_CaMK", "a", "i_fast", "i_slow",
    "a_CaMK", "i_CaMK_fast", "i_CaMK_slow", "d", "f_fast", "f_slow", "f_Ca_fast", "f_Ca_slow", "j_Ca", "n",
    "f_CaMK_fast", "f_Ca_CaMK_fast", "x_r_fast", "x_r_slow", "x_s1", "x_s2", "x_K1", "Na_i", "Na_ss", "K_i",
    "K_ss", "Ca_i", "Ca_ss", "Ca_nsr", "Ca_jsr", "CaMK_trap", "J_rel_NP", "J_rel_CaMK", "Ca_TRPN"};
const char *const kORDHet[] = {"INaF_Multiplier", "INaL_Multiplier", "Ito_Multiplier",
                               "IKr_Multiplier",  "IKs_Multiplier",  "IK1_Multiplier"};

// ----------------------------------------------------------------- Tomek
// Defaults: the values of the reference's Tomek.ev (= Tomek_endo.ev, celltype 0); Tomek_epi.ev
// (celltype 1) and Tomek_mid.ev (celltype 2) load through .ev files.
// Order: NS_TomekParameters::varType (TomekParameters.h:28-164), the derived values apart.
const ParamDef kTOMBase[] = {
    {"amplitude", -53.0}, {"duration", 0.001}, {"celltype", 0.0}, {"Na_o", 140.0}, {"Ca_o", 1.8}, {"K_o", 5.0},
    {"Cl_o", 150.0}, {"INaF_Multiplier", 1.0}, {"INaL_Multiplier", 1.0}, {"Ito_Multiplier", 1.0},
    {"PCa_Multiplier", 1.0}, {"IKr_Multiplier", 1.0}, {"IKs_Multiplier", 1.0}, {"IK1_Multiplier", 1.0},
    {"INaCa_Multiplier", 1.0}, {"INaK_Multiplier", 1.0}, {"IKb_Multiplier", 1.0}, {"INab_Multiplier", 1.0},
    {"ICab_Multiplier", 1.0}, {"IpCa_Multiplier", 1.0}, {"Init_Vm", -0.08908318}, {"Init_Na_i", 12.04906},
    {"Init_Na_ss", 12.04937}, {"Init_K_i", 143.6267}, {"Init_K_ss", 143.6266}, {"Init_Ca_i", 7.217757e-05},
    {"Init_Ca_ss", 6.296698e-05}, {"Init_Ca_nsr", 1.521204}, {"Init_Ca_jsr", 1.522335}, {"Init_Cl_i", 24.0},
    {"Init_m", 0.0007521806}, {"Init_A_h", 0.2167647}, {"Init_B_h", 0.002371305}, {"Init_h", 0.8348669},
    {"Init_A_j", 0.01745803}, {"Init_B_j", 7.277467e-05}, {"Init_j", 0.8349011}, {"Init_h_p", 0.6810231},
    {"Init_j_p", 0.8347477}, {"Init_m_L", 0.0001533095}, {"Init_h_L", 0.5375133}, {"Init_h_L_CaMK", 0.2980653},
    {"Init_a", 0.0009307173}, {"Init_i_fast", 0.9996311}, {"Init_i_slow", 0.5974533},
    {"Init_a_CaMK", 0.0004742092}, {"Init_i_CaMK_fast", 0.9996311}, {"Init_i_CaMK_slow", 0.660594},
    {"Init_d", 0.0}, {"Init_f_fast", 1.0}, {"Init_f_slow", 0.9405982}, {"Init_f_Ca_fast", 1.0},
    {"Init_f_Ca_slow", 0.9999026}, {"Init_j_Ca", 0.9999791}, {"Init_n_ss", 0.0004337198},
    {"Init_n_i", 0.0007353402}, {"Init_f_CaMK_fast", 1.0}, {"Init_f_Ca_CaMK_fast", 1.0},
    {"Init_C_0", 1.024884}, {"Init_C_1", 0.0008543031}, {"Init_C_2", 0.000704028}, {"Init_O", 0.0003399541},
    {"Init_I", 1.181451e-05}, {"Init_x_s1", 0.2385143}, {"Init_x_s2", 0.0001707914},
    {"Init_J_rel_NP", 6.426104e-77}, {"Init_J_rel_CaMK", 2.843667e-62}, {"Init_CaMK_trap", 0.01118689},
    {"ISAC_SWITCH", 0.0}, {"alpha", 3.0}, {"G_sac", 0.27}, {"K_sac", 100.0}, {"E_sac", 0.0},
    {"Init_Ca_TRPN", 0.0005577823}, {"beta1", -2.4}, {"Ca_T50", 0.805}, {"k_TRPN", 0.1}, {"n_TRPN", 2.0},
};
const char *const kTOMDerived[] = {
    "R", "T", "F", "L", "r", "tau_h_L", "A_h", "v_cell", "A_geo", "A_cap", "v_myo", "v_nsr", "v_jsr", "v_ss",
    "P_CaNa", "P_CaK", "P_Ca_CaMK", "P_CaNa_CaMK", "P_CaK_CaMK", "A_f_fast", "A_f_slow", "k_Na1", "k_Na2",
    "k_asymm", "k_Ca_on", "k_Ca_off", "k_m_1", "k_p_2", "k_p_4", "MgADP", "MgATP", "K_MgATP", "beta_tau",
    "P_Ca", "h_10", "h_11", "h_12", "k_1", "k_2", "k_5", "beta_1", "alpha_2", "alpha_4", "alpha_rel",
    "beta_tau_CaMK", "alpha_rel_CaMK", "tau_h_LCaMK", "RToverF"};
const char *const kTOMState[] = {
    "m", "h", "j", "h_p", "j_p", "m_L", "h_L", "h_L_CaMK", "a", "i_fast", "i_slow", "a_CaMK", "i_CaMK_fast",
    "i_CaMK_slow", "d", "f_fast", "f_slow", "f_Ca_fast", "f_Ca_slow", "j_Ca", "f_CaMK_fast", "f_Ca_CaMK_fast",
    "n_ss", "n_i", "C_0", "C_1", "C_2", "O", "I", "x_s1", "x_s2", "Na_i", "Na_ss", "K_i", "K_ss", "Ca_i",
    "Ca_ss", "Ca_nsr", "Ca_jsr", "Cl_i", "CaMK_trap", "J_rel_NP", "J_rel_CaMK", "Ca_TRPN"};

#define COUNT(a) (int)(sizeof(a) / sizeof(a[0]))
const ModelSpec kSpecs[] = {
    {kTenTusscher2, "TenTusscher2", kTT2Base, COUNT(kTT2Base), kTT2Derived, COUNT(kTT2Derived), kTT2Tables,
     COUNT(kTT2Tables), kTT2State, COUNT(kTT2State), 36, kTT2Het, COUNT(kTT2Het), 0, 0},
    {kCourtemanche, "CourtemancheEtAl", kCRNBase, COUNT(kCRNBase), kCRNDerived, COUNT(kCRNDerived), kCRNTables,
     COUNT(kCRNTables), kCRNState, COUNT(kCRNState), 22, kCRNHet, COUNT(kCRNHet), 20.0, 0.002},
    // block: 42 states (h_CaMK_fast included) and 17 currents (OHaraRudy.h:31-52)
    {kOHaraRudy, "OHaraRudy", kORDBase, COUNT(kORDBase), kORDDerived, COUNT(kORDDerived), nullptr, 0, kORDState,
     COUNT(kORDState), 59, kORDHet, COUNT(kORDHet), 0, 0},
    // block: 48 states (the rates A_h, B_h, A_j, B_j included) and 36 stored values (Tomek.h:33-52)
    {kTomek, "Tomek", kTOMBase, COUNT(kTOMBase), kTOMDerived, COUNT(kTOMDerived), nullptr, 0, kTOMState,
     COUNT(kTOMState), 84, kORDHet, COUNT(kORDHet), 0, 0},
};

// ----------------------------------------------------------------- .ev files
// Format of CellModelValues.h:153-243: the first three non-comment lines carry the magic
// "CELLMODEL*IBT*KA", the model name and the entry count (0..256); then `count` entries of
// "name value", '#' lines and blank lines skipped.
int load_ev(const char *path, const char *model_name, std::vector<std::pair<std::string, double>> &out,
            std::string &err) {
  std::ifstream f(path);
  if (!f) {
    err = std::string("cannot open parameter file ") + path;
    return CM_ERR_FILE;
  }
  std::string line, header;
  int got = 0;
  auto content = [](const std::string &s) {
    size_t p = s.find_first_not_of(" \t\r");
    return p != std::string::npos && s[p] != '#';
  };
  while (got < 3 && std::getline(f, line))
    if (content(line)) {
      header += line + " ";
      ++got;
    }
  std::istringstream hs(header);
  std::string magic, name;
  int count = -1;
  hs >> magic >> name >> count;
  if (magic.compare(0, 16, "CELLMODEL*IBT*KA") != 0 || magic.size() >= 32) {
    err = std::string("bad header in ") + path;
    return CM_ERR_FILE;
  }
  if (name != model_name) {
    err = std::string("model type mismatch in ") + path + ": " + name + " != " + model_name;
    return CM_ERR_FILE;
  }
  if (count < 0 || count > 256) {
    err = std::string("entry count out of range in ") + path;
    return CM_ERR_FILE;
  }
  while ((int)out.size() < count && std::getline(f, line)) {
    if (!content(line)) continue;
    std::istringstream ls(line);
    std::string n;
    double v;
    if (!(ls >> n >> v)) {
      err = std::string("malformed entry '") + line + "' in " + path;
      return CM_ERR_FILE;
    }
    out.emplace_back(n, v);
  }
  if ((int)out.size() < count) {
    err = std::string("file ends before ") + std::to_string(count) + " entries: " + path;
    return CM_ERR_FILE;
  }
  return CM_OK;
}

}  // namespace

const ModelSpec *find_model(int model) {
  for (const auto &s : kSpecs)
    if (s.model == model) return &s;
  return nullptr;
}

int model_from_name(const char *name) {
  if (!name) return -1;
  for (const auto &s : kSpecs)
    if (!strcmp(s.name, name)) return s.model;
  return -1;
}

int ParamSet::index(const char *name) const {
  if (!name) return -1;
  for (int i = 0; i < spec->n_base; i++)
    if (!strcmp(spec->base[i].name, name)) return i;
  for (int i = 0; i < spec->n_derived; i++)
    if (!strcmp(spec->derived[i], name)) return spec->n_base + i;
  return -1;
}

double ParamSet::get(const char *name) const {
  int i = index(name);
  return i < 0 ? NAN : vals[i];
}

int ParamSet::init(int model, const char *ev_path, double dt_, std::string &err) {
  spec = find_model(model);
  if (!spec) {
    err = "model not implemented: " + std::to_string(model);
    return CM_ERR_MODEL;
  }
  if (!(dt_ > 0) || !std::isfinite(dt_)) {
    err = "dt must be positive and finite";
    return CM_ERR_ARG;
  }
  dt = dt_;
  vals.assign(spec->n_base + spec->n_derived, 0.0);
  for (int i = 0; i < spec->n_base; i++) vals[i] = spec->base[i].value;
  if (ev_path) {
    std::vector<std::pair<std::string, double>> entries;
    int rc = load_ev(ev_path, spec->name, entries, err);
    if (rc) return rc;
    // ParameterLoader::getParameterValue (ParameterLoader.cpp:41-59): first entry of the
    // given name wins; a needed name missing from the file is an error here.
    for (int i = 0; i < spec->n_base; i++) {
      bool found = false;
      for (auto &e : entries)
        if (e.first == spec->base[i].name) {
          vals[i] = e.second;
          found = true;
          break;
        }
      if (!found) {
        err = std::string("parameter '") + spec->base[i].name + "' not found in " + ev_path;
        return CM_ERR_PARAM;
      }
    }
  }
  rebuild();
  return CM_OK;
}

void ParamSet::rebuild() {
  derive();
  build_tables();
}

#define PV(x) vals[index(#x)]

void ParamSet::derive() {
  if (spec->model == kTenTusscher2) {
    // TenTusscher2Parameters::Calculate (313-338)
    PV(RTONF) = PV(R) * PV(Tx) / PV(F);
    PV(inverseRTONF) = 1 / PV(RTONF);
    PV(vi) = 0.016404;  // the reference overwrites 0.49*vol with this constant (322)
    PV(inverseviF) = 1 / (PV(vi) * PV(F));
    PV(inverseviF2) = 1. / (2 * PV(vi) * PV(F));
    PV(inversevssF2) = 1 / (2 * (PV(vi) / 300.) * PV(F));
    PV(VcdVsr) = PV(Vc) / PV(Vsr);
    PV(Kupsquare) = PV(Kup) * PV(Kup);
    PV(BufcPKbufc) = PV(Bufc) + PV(Kbufc);
    PV(KmNai3) = PV(KmNai) * PV(KmNai) * PV(KmNai);
    PV(Nao3) = PV(Na_o) * PV(Na_o) * PV(Na_o);
    PV(StepCai) = (PV(CaiMax) - PV(CaiMin)) / kRows;
  } else if (spec->model == kOHaraRudy) {
    derive_ord();
  } else if (spec->model == kTomek) {
    derive_tom();
  } else {
    // CourtemancheParameters::Calculate (252-280)
    PV(RTdF) = PV(R) * PV(Tx) / PV(F);
    PV(FdRT) = 1.0 / PV(RTdF);
    PV(RTd2F) = PV(RTdF) * .5;
    PV(Vi) = PV(Vcell) * PV(part_i);
    PV(Vup) = PV(Vcell) * PV(part_up);
    PV(Vrel) = PV(Vcell) * PV(part_rel);
    PV(VupdVi) = PV(Vup) / PV(Vi);
    PV(VreldVi) = PV(Vrel) / PV(Vi);
    PV(VreldVup) = PV(Vrel) / PV(Vup);
    PV(CmdFvi) = PV(C_m) / (PV(F) * PV(Vi));
    PV(Cmd2F) = PV(C_m) / (PV(F) * 2.0);
    PV(csqnkm) = PV(CSQNmax) * PV(K_mcsqn);
    PV(kmcsqnm2) = PV(K_mcsqn) * 2.0;
    PV(kkmcsqn) = PV(K_mcsqn) * PV(K_mcsqn);
    PV(cmdnkm) = PV(CMDNmax) * PV(K_mcmdn);
    PV(kmcmdnm2) = PV(K_mcmdn) * 2.0;
    PV(kkmcmdn) = PV(K_mcmdn) * PV(K_mcmdn);
    PV(kupleak) = PV(I_upmax) / PV(Ca_upmax);
    PV(dt_tr) = 1.0 / PV(t_tr);
  }
}

// OHaraRudyParameters::Calculate (246-316), value by value in the reference's order.
void ParamSet::derive_ord() {
  PV(R) = 8314.0;
  PV(T) = 310.0;
  PV(F) = 96485.0;
  PV(L) = 0.01;
  PV(r) = 0.0011;
  PV(tau_h_L) = 200.0;
  PV(A_h_fast) = 0.99;
  PV(A_h_slow) = 0.01;
  PV(A_f_fast) = 0.6;
  PV(k_Na1) = 15.0;
  PV(k_Na2) = 5.0;
  PV(k_asymm) = 12.5;
  PV(k_Ca_on) = 1.5e6;
  PV(k_Ca_off) = 5.0e3;
  PV(k_m_1) = 182.4;
  PV(k_p_2) = 687.2;
  PV(k_p_4) = 639.0;
  PV(MgADP) = 0.05;
  PV(MgATP) = 9.8;
  PV(K_MgATP) = 1.698e-7;
  PV(beta_tau) = 4.75;
  PV(P_Ca) = PV(PCa_Multiplier) * 0.0001;
  PV(v_cell) = 1000.0 * 3.14 * PV(r) * PV(r) * PV(L);  // the reference's pi is 3.14
  PV(A_geo) = 2.0 * 3.14 * PV(r) * PV(r) + 2.0 * 3.14 * PV(r) * PV(L);
  PV(A_cap) = 2.0 * PV(A_geo);
  PV(v_myo) = 0.68 * PV(v_cell);
  PV(v_nsr) = 0.0552 * PV(v_cell);
  PV(v_jsr) = 0.0048 * PV(v_cell);
  PV(v_ss) = 0.02 * PV(v_cell);
  PV(P_CaNa) = 0.00125 * PV(P_Ca);
  PV(P_CaK) = 3.574e-04 * PV(P_Ca);
  PV(P_Ca_CaMK) = 1.1 * PV(P_Ca);
  PV(P_CaNa_CaMK) = 0.00125 * PV(P_Ca_CaMK);
  PV(P_CaK_CaMK) = 3.5743e-04 * PV(P_Ca_CaMK);
  PV(A_f_slow) = 1.0 - PV(A_f_fast);
  PV(h_10) = PV(k_asymm) + 1.0 + (PV(Na_o) * (1.0 + PV(Na_o) / PV(k_Na2))) / PV(k_Na1);
  PV(h_11) = (PV(Na_o) * PV(Na_o)) / (PV(h_10) * PV(k_Na1) * PV(k_Na2));
  PV(h_12) = 1.0 / PV(h_10);
  PV(k_1) = PV(h_12) * PV(Ca_o) * PV(k_Ca_on);
  PV(k_2) = PV(k_Ca_off);
  PV(k_5) = PV(k_Ca_off);
  PV(beta_1) = PV(k_m_1) * PV(MgADP);
  PV(alpha_2) = PV(k_p_2);
  PV(alpha_4) = (PV(k_p_4) * (PV(MgATP) / PV(K_MgATP))) / (1.0 + (PV(MgATP) / PV(K_MgATP)));
  PV(alpha_rel) = 0.5 * PV(beta_tau);
  PV(beta_tau_CaMK) = 1.25 * PV(beta_tau);
  PV(alpha_rel_CaMK) = 0.5 * PV(beta_tau_CaMK);
  PV(tau_h_LCaMK) = 3.0 * PV(tau_h_L);
  PV(RToverF) = (PV(R) * PV(T)) / PV(F);
}

// TomekParameters::Calculate (233-302): O'Hara-Rudy's derivation with one A_h.
void ParamSet::derive_tom() {
  PV(R) = 8314.0;
  PV(T) = 310.0;
  PV(F) = 96485.0;
  PV(L) = 0.01;
  PV(r) = 0.0011;
  PV(tau_h_L) = 200.0;
  PV(A_h) = 0.99;
  PV(A_f_fast) = 0.6;
  PV(k_Na1) = 15.0;
  PV(k_Na2) = 5.0;
  PV(k_asymm) = 12.5;
  PV(k_Ca_on) = 1.5e6;
  PV(k_Ca_off) = 5.0e3;
  PV(k_m_1) = 182.4;
  PV(k_p_2) = 687.2;
  PV(k_p_4) = 639.0;
  PV(MgADP) = 0.05;
  PV(MgATP) = 9.8;
  PV(K_MgATP) = 1.698e-7;
  PV(beta_tau) = 4.75;
  PV(P_Ca) = PV(PCa_Multiplier) * 0.0001;
  PV(v_cell) = 1000.0 * 3.14 * PV(r) * PV(r) * PV(L);  // the reference's pi is 3.14
  PV(A_geo) = 2.0 * 3.14 * PV(r) * PV(r) + 2.0 * 3.14 * PV(r) * PV(L);
  PV(A_cap) = 2.0 * PV(A_geo);
  PV(v_myo) = 0.68 * PV(v_cell);
  PV(v_nsr) = 0.0552 * PV(v_cell);
  PV(v_jsr) = 0.0048 * PV(v_cell);
  PV(v_ss) = 0.02 * PV(v_cell);
  PV(P_CaNa) = 0.00125 * PV(P_Ca);
  PV(P_CaK) = 3.574e-04 * PV(P_Ca);
  PV(P_Ca_CaMK) = 1.1 * PV(P_Ca);
  PV(P_CaNa_CaMK) = 0.00125 * PV(P_Ca_CaMK);
  PV(P_CaK_CaMK) = 3.5743e-04 * PV(P_Ca_CaMK);
  PV(A_f_slow) = 1.0 - PV(A_f_fast);
  PV(h_10) = PV(k_asymm) + 1.0 + (PV(Na_o) * (1.0 + PV(Na_o) / PV(k_Na2))) / PV(k_Na1);
  PV(h_11) = (PV(Na_o) * PV(Na_o)) / (PV(h_10) * PV(k_Na1) * PV(k_Na2));
  PV(h_12) = 1.0 / PV(h_10);
  PV(k_1) = PV(h_12) * PV(Ca_o) * PV(k_Ca_on);
  PV(k_2) = PV(k_Ca_off);
  PV(k_5) = PV(k_Ca_off);
  PV(beta_1) = PV(k_m_1) * PV(MgADP);
  PV(alpha_2) = PV(k_p_2);
  PV(alpha_4) = (PV(k_p_4) * (PV(MgATP) / PV(K_MgATP))) / (1.0 + (PV(MgATP) / PV(K_MgATP)));
  PV(alpha_rel) = 0.5 * PV(beta_tau);
  PV(beta_tau_CaMK) = 1.25 * PV(beta_tau);
  PV(alpha_rel_CaMK) = 0.5 * PV(beta_tau_CaMK);
  PV(tau_h_LCaMK) = 3.0 * PV(tau_h_L);
  PV(RToverF) = (PV(R) * PV(T)) / PV(F);
}

void ParamSet::build_tables() {
  tables.assign(spec->n_tables, std::vector<double>(kRows, 0.0));
  if (spec->n_tables == 0) return;  // O'Hara-Rudy: closed forms only (its InitTable loop is empty)
  auto T = [&](const char *n) -> std::vector<double> & {
    for (int k = 0; k < spec->n_tables; k++)
      if (!strcmp(spec->table_names[k], n)) return tables[k];
    return tables[0];  // unreachable: names below are the spec's
  };
  // The voltage grid of both InitTable loops: V from -199.9999 mV in accumulated steps of 0.1.
  if (spec->model == kTenTusscher2) {
    const double iRTONF = PV(inverseRTONF), RTONF = PV(RTONF), F = PV(F), Ca_o = PV(Ca_o), Na_o = PV(Na_o);
    const double HT = dt * 1000;
    auto &NaK_P1 = T("NaK_P1"), &rec_ipK = T("rec_ipK"), &m_inf = T("m_inf"), &h_inf = T("h_inf"),
         &j_inf = T("j_inf"), &Xr1_inf = T("Xr1_inf"), &Xr2_inf = T("Xr2_inf"), &Xs_inf = T("Xs_inf"),
         &r_inf = T("r_inf"), &s_inf = T("s_inf"), &d_inf = T("d_inf"), &f_inf = T("f_inf"),
         &f2_inf = T("f2_inf"), &NaCa_P1 = T("NaCa_P1"), &NaCa_P2 = T("NaCa_P2"), &CaL_P1 = T("CaL_P1"),
         &CaL_P2 = T("CaL_P2"), &e_m = T("exptau_m"), &e_h = T("exptau_h"), &e_j = T("exptau_j"),
         &e_Xr1 = T("exptau_Xr1"), &e_Xr2 = T("exptau_Xr2"), &e_Xs = T("exptau_Xs"), &e_s = T("exptau_s"),
         &e_r = T("exptau_r"), &e_d = T("exptau_d"), &e_f = T("exptau_f"), &e_f2 = T("exptau_f2"),
         &ECA = T("ECA");
    for (double V = -kRangeHalf + .0001; V < kRangeHalf; V += 1.0 / kDivision) {
      const int i = (int)(kDivision * (kRangeHalf + V) + .5);
      if (i < 0 || i >= kRows) continue;
      NaK_P1[i] = (1. / (1. + 0.1245 * exp(-0.1 * V * iRTONF) + 0.0353 * exp(-V * iRTONF)));
      rec_ipK[i] = PV(g_pK) / (1. + exp((25. - V) / 5.98));
      const double tau_m = (1. / (1. + exp((-60. - V) / 5.))) *
                           (0.1 / (1. + exp((V + 35.) / 5.)) + 0.10 / (1. + exp((V - 50.) / 200.)));
      m_inf[i] = 1. / ((1. + exp((-56.86 - V) / 9.03)) * (1. + exp((-56.86 - V) / 9.03)));
      double tau_h, tau_j;
      if (V >= -40.) {
        tau_h = 1.0 / (0. + (0.77 / (0.13 * (1. + exp(-(V + 10.66) / 11.1)))));
        tau_j = 1.0 / (0. + (0.6 * exp((0.057) * V) / (1. + exp(-0.1 * (V + 32.)))));
      } else {
        tau_h = 1.0 / ((0.057 * exp(-(V + 80.) / 6.8)) + (2.7 * exp(0.079 * V) + (3.1e5) * exp(0.3485 * V)));
        const double aj = (((-2.5428e4) * exp(0.2444 * V) - (6.948e-6) * exp(-0.04391 * V)) * (V + 37.78) /
                           (1. + exp(0.311 * (V + 79.23))));
        const double bj = (0.02424 * exp(-0.01052 * V) / (1. + exp(-0.1378 * (V + 40.14))));
        tau_j = 1.0 / (aj + bj);
      }
      h_inf[i] = 1. / ((1. + exp((V + 71.55) / 7.43)) * (1. + exp((V + 71.55) / 7.43)));
      j_inf[i] = h_inf[i];
      Xr1_inf[i] = 1. / (1. + exp((PV(m_Xr1_1) - V) / PV(m_Xr1_2)));
      const double tau_Xr1 = (450. / (1. + exp((PV(a_Xr1_1) - V) / PV(a_Xr1_2)))) *
                             (6. / (1. + exp((V - PV(b_Xr1_1)) / PV(b_Xr1_2)))) * fabs(PV(K_Q10Xr1));
      Xr2_inf[i] = 1. / (1. + exp((V - PV(m_Xr2_1)) / PV(m_Xr2_2)));
      const double tau_Xr2 = (3. / (1. + exp((PV(a_Xr2_1) - V) / PV(a_Xr2_2)))) *
                             (1.12 / (1. + exp((V - PV(b_Xr2_1)) / PV(b_Xr2_2)))) * fabs(PV(K_Q10Xr2));
      Xs_inf[i] = 1. / (1. + exp((PV(m_Xs_1) - V) / PV(m_Xs_2)));
      const double tau_Xs = ((1400. / (sqrt(1. + exp((PV(a_Xs_1) - V) / PV(a_Xs_2))))) *
                                 (1. / (1. + exp((V - PV(b_Xs_1)) / PV(b_Xs_2)))) +
                             PV(tau_Xs_add)) *
                            fabs(PV(K_Q10Xs));
      r_inf[i] = 1. / (1. + exp((20 - V) / 6.));
      s_inf[i] = 1. / (1. + exp((V + PV(s_inf_vHalf)) / 5.));
      const double tau_r = 9.5 * exp(-(V + 40.) * (V + 40.) / 1800.) + 0.8;
      const double tau_s =
          PV(tau_s_f1) * exp(-(V + PV(tau_s_vHalf1)) * (V + PV(tau_s_vHalf1)) / PV(tau_s_slope1)) +
          PV(tau_s_enable) * 5. / (1. + exp((V - 20.) / 5.)) + PV(tau_s_add);
      d_inf[i] = 1. / (1. + exp((-8. - V) / 7.5));
      const double tau_d = (1.4 / (1. + exp((-35 - V) / 13)) + 0.25) * (1.4 / (1. + exp((V + 5) / 5))) +
                           (1. / (1. + exp((50 - V) / 20)));
      f_inf[i] = 1. / (1. + exp((V + 20) / 7));
      const double tau_f = 1102.5 * exp(-((V + 27) * (V + 27)) / (15 * 15)) + 200. / (1. + exp((13 - V) / 10.)) +
                           ((180. / (1. + exp((V + 30) / 10.))) + 20.);
      f2_inf[i] = (.67 / (1. + exp((V + 35.) / 7.))) + .33;
      const double tau_f2 = 600. * exp(-(V + 25) * (V + 25) / 170.) + 31. / (1. + exp((25 - V) / 10.)) +
                            16. / (1. + exp((V + 30) / 10.));
      const double ncx = (1. / (PV(KmNai3) + PV(Nao3))) * (1. / (PV(KmCa) + Ca_o)) *
                         (1. / (1. + PV(ksat) * exp((PV(n) - 1.) * V * iRTONF)));
      NaCa_P1[i] = ncx * (exp(PV(n) * V * iRTONF) * Ca_o);
      NaCa_P2[i] = ncx * (exp((PV(n) - 1) * V / RTONF) * Na_o * Na_o * Na_o * 2.5);
      CaL_P1[i] = 4 * (V - 15.) * F / RTONF * (0.25 * exp(2 * (V - 15.) / RTONF)) / (exp(2 * (V - 15.) / RTONF) - 1.);
      CaL_P2[i] = 4 * (V - 15.) * (F / RTONF) * (1 * Ca_o) / (exp(2 * (V - 15.) / RTONF) - 1.);
      e_m[i] = exp(-HT / tau_m);
      e_h[i] = exp(-HT / tau_h);
      e_j[i] = exp(-HT / tau_j);
      e_Xr1[i] = exp(-HT / tau_Xr1);
      e_Xr2[i] = exp(-HT / tau_Xr2);
      e_Xs[i] = exp(-HT / tau_Xs);
      e_s[i] = exp(-HT / tau_s);
      e_r[i] = exp(-HT / tau_r);
      e_d[i] = exp(-HT / tau_d);
      e_f[i] = exp(-HT / tau_f);
      e_f2[i] = exp(-HT / tau_f2);
      // ECa on the Ca grid Cai = i * StepCai (483-484); row 0 is +inf as in the reference.
      ECA[i] = (RTONF * 0.5) * log(Ca_o / (i * PV(StepCai)));
    }
  } else {
    const double tinc = dt * 1000;
    const double sigma = (exp(PV(Na_o) / 67.3) - 1.0) / 7.0;
    auto RL = [&](const char *gate, const char *tau, int i, double a, double b, double rate) {
      T(tau)[i] = exp(-tinc * rate);
      if (gate) T(gate)[i] = a / (a + b);
    };
    for (double V = -kRangeHalf + .0001; V < kRangeHalf; V += 1.0 / kDivision) {
      const int i = (int)(kDivision * (kRangeHalf + V) + .5);
      if (i < 0 || i >= kRows) continue;
      const double sm = V + 47.13 - PV(shiftm);
      double a = (fabs(sm) < 1e-10 ? 3.2 : PV(m_a1) * sm / (1.0 - exp(-sm * PV(m_a2))));
      double b = PV(m_b1) * exp(-(V - PV(shiftm)) / PV(m_b2));
      RL("m_m", "exptau_m", i, a, b, a + b);
      if (V >= -40.0 + PV(shifth)) {
        a = .0;
        b = 1.0 / (PV(h_b5) * (1.0 + exp(-(V + 10.66 - PV(shifth)) / PV(h_b6))));
      } else {
        a = PV(h_a1) * exp(-(V + 80.0 - PV(shifth)) / PV(h_a2));
        b = PV(h_b1) * exp(PV(h_b2) * (V - PV(shifth))) + PV(h_b3) * exp(PV(h_b4) * (V - PV(shifth)));
      }
      RL("m_h", "exptau_h", i, a, b, a + b);
      if (V >= -40.0 + PV(shiftj)) {
        a = .0;
        b = PV(j_b4) * exp(PV(j_b5) * (V - PV(shiftj))) / (1.0 + exp(PV(j_b6) * (V + 32.0 - PV(shiftj))));
      } else {
        a = (PV(j_a1) * exp(PV(j_a2) * (V - PV(shiftj))) - PV(j_a3) * exp(PV(j_a4) * (V - PV(shiftj)))) *
            (V + 37.78 - PV(shiftj)) / (1.0 + exp(PV(j_a5) * (V + 79.23 - PV(shiftj))));
        b = PV(j_b1) * exp(PV(j_b2) * (V - PV(shiftj))) / (1.0 + exp(PV(j_b3) * (V + 40.14 - PV(shiftj))));
      }
      T("exptau_j")[i] = exp(-tinc * (a + b) / PV(tau_j_mult));
      T("m_j")[i] = a / (a + b);
      const double Vo = V - PV(shiftoa);
      a = PV(C_oa_1) / ((exp(-(Vo + 10.0) / PV(C_oa_2))) + (exp(-(Vo - 30.0) / PV(C_oa_3))));
      b = PV(C_oa_1) / (2.5 + exp((Vo + 82.0) / PV(C_oa_4)));
      T("m_oa")[i] = 1.0 / (1.0 + exp(-(Vo + PV(C_oa_6)) / PV(C_oa_5)));
      RL(nullptr, "exptau_oa", i, a, b, (a + b) * PV(Tfac));
      a = 1.0 / (18.53 + exp((V + 113.7) / 10.95));
      b = 1.0 / (35.56 + exp(-(V + 1.26) / 7.44));
      T("m_oi")[i] = 1.0 / (1.0 + exp((V + 43.1) / 5.3));
      RL(nullptr, "exptau_oi", i, a, b, (a + b) * PV(Tfac));
      a = PV(ua_a1) / ((exp((V + PV(ua_a2)) / PV(ua_a3))) + (exp((V + PV(ua_a4)) / PV(ua_a5))));
      b = .65 / (PV(ua_b1) + exp((V + PV(ua_b2)) / PV(ua_b3)));
      T("m_ua")[i] = 1.0 / (1.0 + exp((V + PV(ua_m1)) / PV(ua_m2)));
      RL(nullptr, "exptau_ua", i, a, b, (a + b) * PV(ua_KQ10));
      a = PV(ui_a1) / (PV(ui_a2) + exp((V + PV(ui_a3)) / PV(ui_a4)));
      b = 1.0 / exp((V + PV(ui_b1)) / PV(ui_b2));
      T("m_ui")[i] = 1.0 / (1.0 + exp((V + PV(ui_m1)) / PV(ui_m2)));
      RL(nullptr, "exptau_ui", i, a, b, (a + b) * PV(ui_KQ10));
      a = (fabs(V + PV(Xr_a2)) < 1e-10 ? 0.0015
                                        : PV(Xr_a1) * (V + PV(Xr_a2)) / (1.0 - exp((V + PV(Xr_a2)) / PV(Xr_a3))));
      b = (fabs(V - PV(Xr_b1)) < 1e-10 ? 3.7836118e-4
                                        : 7.3898e-5 * (V + PV(Xr_b1)) / (exp((V + PV(Xr_b1)) / PV(Xr_b2)) - 1.0));
      T("m_Xr")[i] = 1.0 / (1.0 + exp((V + PV(Xr_m1)) / PV(Xr_m2)));
      RL(nullptr, "exptau_Xr", i, a, b, PV(Xr_KQ10) * (a + b));
      a = (fabs(V + PV(Xs_a2)) < 1e-10 ? 0.00068
                                        : PV(Xs_a1) * (V + PV(Xs_a2)) / (1.0 - exp((V + PV(Xs_a2)) / PV(Xs_a3))));
      b = (fabs(V + PV(Xs_b1)) < 1e-10 ? 0.000315
                                        : (3.5e-5) * (V + PV(Xs_b1)) / (exp((V + PV(Xs_b1)) / PV(Xs_b2)) - 1.0));
      RL(nullptr, "exptau_Xs", i, a, b, PV(Xs_KQ10) * (a + b));
      T("m_Xs")[i] = 1.0 / sqrt(1.0 + exp((V + PV(Xs_m1)) / PV(Xs_m2)));
      a = 1.0 / (1.0 + exp(-(V + 10.0) / 6.24));
      T("exptau_d")[i] = exp(-tinc * (fabs(V + 10.0) < 1e-10
                                          ? 1.0 / (a * 4.579)
                                          : 1.0 / (a * (1.0 - exp(-(V + 10.0) / 6.24)) / (0.035 * (V + 10.0)))));
      T("m_d")[i] = 1.0 / (1.0 + exp(-(V + 10.0) / 8));
      const double gf = PV(CaL_fT_1) / (0.0197 * exp(-0.0337 * 0.0337 * (V + 10.0) * (V + 10.0)) + 0.02);
      T("exptau_f")[i] = V > 0 ? exp(-tinc * (1.0 / (gf * PV(tau_f_mult)))) : exp(-tinc * (1.0 / gf));
      T("m_f")[i] = exp(-(V + 28.0) / 6.9) / (1.0 + exp(-(V + 28.0) / 6.9));
      T("exptau_w")[i] =
          exp(-tinc * (fabs(V - 7.9) < 1e-10
                           ? 1.0 / (6.0 * 0.2 / 1.3)
                           : 1.0 / (6.0 * (1.0 - exp(-(V - 7.9) / 5.0)) / (1.0 + 0.3 * exp(-(V - 7.9) / 5.0)) / (V - 7.9))));
      T("m_w")[i] = 1.0 - 1.0 / (1.0 + exp(-(V - 40.0) / 17.0));
      const double VFdRT = V * PV(FdRT);
      const double Na3 = PV(Na_o) * PV(Na_o) * PV(Na_o);
      T("expVm")[i] = exp(-VFdRT) * PV(Na_o) * PV(Na_o) * PV(Na_o);
      T("g_Kur")[i] = PV(g_Kur1) + PV(g_Kur2) / (1.0 + exp((V + PV(g_Kur3)) / PV(g_Kur4)));
      T("CKr")[i] = PV(g_Kr) / (1.0 + exp((V + PV(g_Kr1)) / PV(g_Kr2)));
      T("CK1")[i] = PV(g_K1) / (1.0 + exp((V + PV(g_K1_1)) * PV(g_K1_2)));
      T("CNaK")[i] = PV(I_NaKmax) / (1.0 + .1245 * exp(-.1 * VFdRT) + .0365 * sigma * exp(-VFdRT)) * PV(K_o) /
                     (PV(K_o) + PV(k_mKo));
      T("CNaCa")[i] = PV(k_NaCa) * exp(PV(gamm) * VFdRT) /
                      ((PV(k_mNa) * PV(k_mNa) * PV(k_mNa) + Na3) * (PV(k_mCa) + PV(Ca_o)) *
                       (1.0 + PV(k_sat) * exp((PV(gamm) - 1.0) * VFdRT)));
    }
    exp250 = exp(250.0);
    exp50 = exp(169.5);
  }
}

double ParamSet::init_vm() const {
  return spec->model == kTenTusscher2 ? vals[index("init_V_m")] : vals[index("Init_Vm")];
}
// GetAmplitude() / GetStimTime(): TT2, O'Hara-Rudy and Tomek read parameters (OHaraRudy.h:84-86,
// Tomek.h:100-102),
// Courtemanche returns constants.
double ParamSet::amplitude() const {
  if (spec->model == kOHaraRudy || spec->model == kTomek) return vals[index("amplitude")];
  return spec->model == kTenTusscher2 ? vals[index("Amp")] : spec->default_amplitude;
}
double ParamSet::stim_time() const {
  if (spec->model == kOHaraRudy || spec->model == kTomek) return vals[index("duration")];
  return spec->model == kTenTusscher2 ? vals[index("stim_duration")] : spec->default_stim_time;
}

void ParamSet::init_state(std::vector<double> &s) const {
  s.assign(spec->n_state, 0.0);
  if (spec->model == kTenTusscher2) {
    // TenTusscherEtAl2::Init (250-271)
    const char *init[] = {"init_Cai", "init_CaSR", "init_CaSS", "init_Nai", "init_Ki", "init_m",
                          "init_h", "init_j", "init_Xr1", "init_Xr2", "init_Xs", "init_r",
                          "init_s", "init_d", "init_f", "init_f2", "init_fCa", "init_Rq"};
    for (int k = 0; k < S2_N; k++) s[k] = vals[index(init[k])];
  } else if (spec->model == kOHaraRudy) {
    // OHaraRudy::Init (54-102): Init_<name> for every state; troponin as a fraction of trpnmax
    for (int k = 0; k < SO_Ca_TRPN; k++) s[k] = vals[index((std::string("Init_") + spec->state_names[k]).c_str())];
    s[SO_Ca_TRPN] = vals[index("Init_Ca_TRPN")] / 0.07;
  } else if (spec->model == kTomek) {
    // Tomek::Init (55-107): the same rule
    for (int k = 0; k < SM_Ca_TRPN; k++) s[k] = vals[index((std::string("Init_") + spec->state_names[k]).c_str())];
    s[SM_Ca_TRPN] = vals[index("Init_Ca_TRPN")] / 0.07;
  } else {
    // Courtemanche::Init (56-83)
    const char *init[] = {"Init_Ca_i", "Init_Ca_up", "Init_Ca_rel", "Init_h", "Init_j", "Init_oi",
                          "Init_ui", "Init_Xr", "Init_Xs", "Init_u", "Init_v", "Init_w",
                          "Init_Na_i", "Init_K_i", "Init_m", "Init_oa", "Init_ua", "Init_d",
                          "Init_f", "Init_f_Ca"};
    for (int k = 0; k < SC_CaTRPN; k++) s[k] = vals[index(init[k])];
    s[SC_CaTRPN] = vals[index("Init_Ca_TRPN")] / vals[index("TRPNmax")];
  }
}

void ParamSet::tt2_consts(TT2Consts<double> &d, TT2Consts<float> &f) const {
  d.RTONF = PV(RTONF);
  d.K_o = PV(K_o);
  d.Na_o = PV(Na_o);
  d.pKNa = PV(pKNa);
  d.pKNaNao = PV(pKNa) * PV(Na_o);
  d.sqrtKo54 = sqrt(PV(K_o) / 5.4);
  d.KoKmK = PV(K_o) / (PV(K_o) + PV(KmK));
  d.KmNa = PV(KmNa);
  d.g_pCa = PV(g_pCa);
  d.KpCa = PV(KpCa);
  d.g_to = PV(g_to);
  d.g_Kr = PV(g_Kr);
  d.g_Ks = PV(g_Ks);
  d.g_K1 = PV(g_K1);
  d.g_bNa = PV(g_bNa);
  d.g_bCa = PV(g_bCa);
  d.g_Na = PV(g_Na);
  d.g_CaL = PV(g_CaL);
  d.kNaCa = PV(kNaCa);
  d.knak = PV(knak);
  // function-level statics of the reference Calc (TenTusscher2.cpp:639-640)
  d.CaiTabConst1 = -PV(CaiMin) / PV(StepCai) + 0.5;
  d.CaiTabConst2 = 1. / PV(StepCai);
  d.Cm = PV(C);
  d.max_sr = PV(max_sr);
  d.min_sr = PV(min_sr);
  d.EC = PV(EC);
  d.ks1 = PV(ks1);
  d.ks2 = PV(ks2);
  d.k3 = PV(k3);
  d.k4 = PV(k4);
  d.Vrel = PV(Vrel);
  d.Vxfer = PV(Vxfer);
  d.Vmaxup = PV(Vmaxup);
  d.Kupsquare = PV(Kupsquare);
  d.Bufsr = PV(Bufsr);
  d.Kbufsr = PV(Kbufsr);
  d.Bufss = PV(Bufss);
  d.Kbufss = PV(Kbufss);
  d.Bufc = PV(Bufc);
  d.Kbufc = PV(Kbufc);
  d.BufcPKbufc = PV(BufcPKbufc);
  d.VcVss = PV(Vc) / PV(Vss);
  d.VsrVss = PV(Vsr) / PV(Vss);
  d.inversevssF2 = PV(inversevssF2);
  d.inverseviF = PV(inverseviF);
  d.inverseviF2 = PV(inverseviF2);
  d.invVcdVsr = 1.0 / PV(VcdVsr);
  d.dt = dt;
  d.dt1000 = dt * 1000.0;
  d.inv_stim_unit = 1.0 / 2.29656e-2;
  d.logKo = log(PV(K_o));
  d.logNao = log(PV(Na_o));
  d.logKoNao = log(PV(K_o) + PV(pKNa) * PV(Na_o));
  // FP32 copy, field by field
  const double *src = &d.RTONF;
  float *dst = &f.RTONF;
  const int nf = (int)(sizeof(TT2Consts<double>) / sizeof(double));
  for (int k = 0; k < nf; k++) dst[k] = (float)src[k];
}

void ParamSet::crn_consts(CRNConsts<double> &d, CRNConsts<float> &f) const {
  d.RTdF = PV(RTdF);
  d.RTd2F = PV(RTd2F);
  d.Na_o = PV(Na_o);
  d.K_o = PV(K_o);
  d.Ca_o = PV(Ca_o);
  d.g_Na = PV(g_Na);
  d.g_to = PV(g_to);
  d.g_Ks = PV(g_Ks);
  d.g_CaL = PV(g_CaL);
  d.E_rL = PV(E_rL);
  d.g_bNa = PV(g_bNa);
  d.g_bCa = PV(g_bCa);
  d.k_mNai = PV(k_mNai);
  d.I_pCamax = PV(I_pCamax);
  d.k_mpCa = PV(k_mpCa);
  d.k_rel = PV(k_rel);
  d.I_upmax = PV(I_upmax);
  d.k_up = PV(k_up);
  d.kupleak = PV(kupleak);
  d.dt_tr = PV(dt_tr);
  d.G_sac = PV(G_sac);
  d.E_sac = PV(E_sac);
  d.K_sac = PV(K_sac);
  d.alpha = PV(alpha);
  d.ISAC_SWITCH = PV(ISAC_SWITCH);
  d.Ca_T50 = PV(Ca_T50);
  d.beta1 = PV(beta1);
  d.k_TRPN = PV(k_TRPN);
  d.n_TRPN = PV(n_TRPN);
  d.VreldVup = PV(VreldVup);
  d.csqnkm = PV(csqnkm);
  d.kmcsqnm2 = PV(kmcsqnm2);
  d.kkmcsqn = PV(kkmcsqn);
  d.CmdFvi = PV(CmdFvi);
  d.VupdVi = PV(VupdVi);
  d.VreldVi = PV(VreldVi);
  d.TRPNmax = PV(TRPNmax);
  d.cmdnkm = PV(cmdnkm);
  d.kmcmdnm2 = PV(kmcmdnm2);
  d.kkmcmdn = PV(kkmcmdn);
  d.Vrel = PV(Vrel);
  d.Cmd2F = PV(Cmd2F);
  d.exp250 = exp250;
  d.exp50 = exp50;
  d.dt_ms = dt * 1000.0;
  d.logNao = log(PV(Na_o));
  d.logKo = log(PV(K_o));
  d.logCao = log(PV(Ca_o));
  const double *src = &d.RTdF;
  float *dst = &f.RTdF;
  const int nf = (int)(sizeof(CRNConsts<double>) / sizeof(double));
  for (int k = 0; k < nf; k++) dst[k] = (float)src[k];  // exp250/exp50 become inf; unused in FP32
}

void ParamSet::ord_consts(ORDConsts<double> &d, ORDConsts<float> &f) const {
  d.dt_ms = dt * 1000.0;
  d.RToverF = PV(RToverF);
  d.FoRT = PV(F) / (PV(R) * PV(T));
  d.FFoRT = PV(F) * PV(F) / (PV(R) * PV(T));
  d.Na_o = PV(Na_o);
  d.K_o = PV(K_o);
  d.Ca_o = PV(Ca_o);
  d.util_1 = PV(A_cap) / (PV(F) * PV(v_myo));
  d.util_2 = PV(v_ss) / PV(v_myo);
  d.util_3 = PV(A_cap) / (PV(F) * PV(v_ss));
  d.vnsr_vmyo = PV(v_nsr) / PV(v_myo);
  d.vjsr_vss = PV(v_jsr) / PV(v_ss);
  d.vjsr_vnsr = PV(v_jsr) / PV(v_nsr);
  d.A_h_fast = PV(A_h_fast);
  d.A_h_slow = PV(A_h_slow);
  d.A_f_fast = PV(A_f_fast);
  d.A_f_slow = PV(A_f_slow);
  d.tau_h_L_mod = PV(HF_Gomez_2) * PV(tau_h_L);               // (211, 215)
  d.tau_h_L_CaMK = 3.0 * PV(tau_h_L) * PV(HF_Gomez_2);       // (218)
  d.INaF = PV(INaF_Multiplier);
  d.INaL = PV(INaL_Multiplier);
  d.Ito = PV(Ito_Multiplier);
  d.IKr = PV(IKr_Multiplier);
  d.IKs = PV(IKs_Multiplier);
  d.IK1 = PV(IK1_Multiplier);
  d.HF1 = PV(HF_Gomez_1);
  d.HF3 = PV(HF_Gomez_3);
  d.HF4 = PV(HF_Gomez_4);
  d.HF5 = PV(HF_Gomez_5);
  d.INaCa_HF6 = PV(INaCa_Multiplier) * PV(HF_Gomez_6);
  d.INaK_HF7 = PV(INaK_Multiplier) * PV(HF_Gomez_7);
  d.IKb = PV(IKb_Multiplier);
  d.INab = PV(INab_Multiplier);
  d.ICab = PV(ICab_Multiplier);
  d.IpCa = PV(IpCa_Multiplier);
  d.P_Ca = PV(P_Ca);
  d.P_CaNa = PV(P_CaNa);
  d.P_CaK = PV(P_CaK);
  d.P_Ca_CaMK = PV(P_Ca_CaMK);
  d.P_CaNa_CaMK = PV(P_CaNa_CaMK);
  d.P_CaK_CaMK = PV(P_CaK_CaMK);
  d.k_Na1 = PV(k_Na1);
  d.k_Na2 = PV(k_Na2);
  d.k_Ca_on = PV(k_Ca_on);
  d.h_11 = PV(h_11);
  d.k_1 = PV(k_1);
  d.k_2 = PV(k_2);
  d.k_5 = PV(k_5);
  d.beta_1 = PV(beta_1);
  d.alpha_2 = PV(alpha_2);
  d.alpha_4 = PV(alpha_4);
  d.MgATP1 = 1.0 + PV(MgATP);
  d.alpha_rel = PV(alpha_rel);
  d.alpha_rel_CaMK = PV(alpha_rel_CaMK);
  d.beta_tau = PV(beta_tau);
  d.beta_tau_CaMK = PV(beta_tau_CaMK);
  // cell-type branches of Calc: M cells release 1.7x (557-560), epicardial cells take up 1.3x
  // (575-578), buffer 1.3x calmodulin (609-611) and inactivate I_to faster (delta_epi, 234)
  const double ct = PV(celltype);
  d.rel_scale = ct == 2.0 ? 1.7 : 1.0;
  d.HF8x15 = 1.5 * PV(HF_Gomez_8);
  d.up_scale = ct == 1.0 ? 1.3 : 1.0;
  d.HF9 = PV(HF_Gomez_9);
  d.HF0 = PV(HF_Gomez_0);
  d.cmdnmax = ct == 1.0 ? 0.05 * 1.3 : 0.05;
  d.epi = ct == 1.0 ? 1.0 : 0.0;
  d.sqrtKo54 = sqrt(PV(K_o) / 5.4);
  d.sqrtKo = sqrt(PV(K_o));
  d.EKs_num = PV(K_o) + 0.01833 * PV(Na_o);
  d.xK1_shift = 2.5538 * PV(K_o) + 144.59;
  d.xK1_slope = 1.5692 * PV(K_o) + 3.8115;
  d.RK1_shift = 105.8 - 2.6 * PV(K_o);
  d.G_sac = PV(G_sac);
  d.E_sac = PV(E_sac);
  d.K_sac = PV(K_sac);
  d.alpha_sac = PV(alpha);
  d.ISAC_SWITCH = PV(ISAC_SWITCH);
  d.Ca_T50 = PV(Ca_T50);
  d.beta1 = PV(beta1);
  d.HFM = PV(HFM_Multiplier);
  d.k_TRPN = PV(k_TRPN);
  d.n_TRPN = PV(n_TRPN);
  d.logNao = log(PV(Na_o));
  d.logKo = log(PV(K_o));
  d.logEKs_num = log(d.EKs_num);
  const double *src = &d.dt_ms;
  float *dst = &f.dt_ms;
  const int nf = (int)(sizeof(ORDConsts<double>) / sizeof(double));
  for (int k = 0; k < nf; k++) dst[k] = (float)src[k];
}

void ParamSet::tom_consts(TOMConsts<double> &d, TOMConsts<float> &f) const {
  d.dt_ms = dt * 1000.0;
  d.RToverF = PV(RToverF);
  d.FoRT = PV(F) / (PV(R) * PV(T));
  d.FFoRT = PV(F) * PV(F) / (PV(R) * PV(T));
  d.RToF = (PV(R) * PV(T)) / PV(F);  // E_Cl's factor, z_Cl = 1 (Tomek.cpp:139-140)
  d.Na_o = PV(Na_o);
  d.K_o = PV(K_o);
  d.Ca_o = PV(Ca_o);
  d.Cl_o = PV(Cl_o);
  d.util_1 = PV(A_cap) / (PV(F) * PV(v_myo));
  d.util_2 = PV(v_ss) / PV(v_myo);
  d.util_3 = PV(A_cap) / (PV(F) * PV(v_ss));
  d.vnsr_vmyo = PV(v_nsr) / PV(v_myo);
  d.vjsr_vss = PV(v_jsr) / PV(v_ss);
  d.vjsr_vnsr = PV(v_jsr) / PV(v_nsr);
  d.A_h = PV(A_h);
  d.A_f_fast = PV(A_f_fast);
  d.A_f_slow = PV(A_f_slow);
  d.tau_h_L = PV(tau_h_L);
  d.tau_h_L_CaMK = 3.0 * PV(tau_h_L);
  d.INaF = PV(INaF_Multiplier);
  d.INaL = PV(INaL_Multiplier);
  d.Ito = PV(Ito_Multiplier);
  d.IKr = PV(IKr_Multiplier);
  d.IKs = PV(IKs_Multiplier);
  d.IK1 = PV(IK1_Multiplier);
  d.INaCa = PV(INaCa_Multiplier);
  d.INaK = PV(INaK_Multiplier);
  d.IKb = PV(IKb_Multiplier);
  d.INab = PV(INab_Multiplier);
  d.ICab = PV(ICab_Multiplier);
  d.IpCa = PV(IpCa_Multiplier);
  // the reference scales the L-type permeability by IpCa_Multiplier, not PCa_Multiplier (292)
  d.PCa = PV(IpCa_Multiplier) * 8.3757e-05;
  d.k_Na1 = PV(k_Na1);
  d.k_Na2 = PV(k_Na2);
  d.k_Ca_on = PV(k_Ca_on);
  d.h_11 = PV(h_11);
  d.k_1 = PV(k_1);
  d.k_2 = PV(k_2);
  d.k_5 = PV(k_5);
  d.beta_1 = PV(beta_1);
  d.alpha_2 = PV(alpha_2);
  d.alpha_4 = PV(alpha_4);
  d.MgATP1 = 1.0 + PV(MgATP);
  d.alpha_rel = PV(alpha_rel);
  d.alpha_rel_CaMK = PV(alpha_rel_CaMK);
  d.beta_tau = PV(beta_tau);
  d.beta_tau_CaMK = PV(beta_tau_CaMK);
  // cell-type branches of Calc: M cells release 1.7x (558-561), epicardial cells take up 1.3x
  // (576-579), buffer 1.3x calmodulin (606-607) and inactivate I_to faster (delta_epi, 206)
  const double ct = PV(celltype);
  d.rel_scale = ct == 2.0 ? 1.7 : 1.0;
  d.up_scale = ct == 1.0 ? 1.3 : 1.0;
  d.cmdnmax = ct == 1.0 ? 0.05 * 1.3 : 0.05;
  d.epi = ct == 1.0 ? 1.0 : 0.0;
  d.sqrtKo5 = sqrt(PV(K_o) / 5.0);
  d.EKs_num = PV(K_o) + 0.01833 * PV(Na_o);
  // activity coefficients of the bath (271-279): ionic strength I_o [M], Davies' constant
  d.constA = 1.82e6 * pow(74. * 310., -1.5);
  const double I_o = 0.5 * (PV(Na_o) + PV(K_o) + PV(Cl_o) + 4. * PV(Ca_o)) / 1000.;
  auto gamma = [&](double z2) { return exp(-d.constA * z2 * (sqrt(I_o) / (1. + sqrt(I_o)) - 0.3 * I_o)); };
  d.gamma_Ca_o = gamma(4.);
  d.gamma_Na_o = gamma(1.);
  d.gamma_K_o = gamma(1.);
  d.G_sac = PV(G_sac);
  d.E_sac = PV(E_sac);
  d.K_sac = PV(K_sac);
  d.alpha_sac = PV(alpha);
  d.ISAC_SWITCH = PV(ISAC_SWITCH);
  d.Ca_T50 = PV(Ca_T50);
  d.beta1 = PV(beta1);
  d.k_TRPN = PV(k_TRPN);
  d.n_TRPN = PV(n_TRPN);
  const double *src = &d.dt_ms;
  float *dst = &f.dt_ms;
  const int nf = (int)(sizeof(TOMConsts<double>) / sizeof(double));
  for (int k = 0; k < nf; k++) dst[k] = (float)src[k];
}

void ParamSet::rows_fp64(std::vector<double> &rows, std::vector<double> &eca) const {
  if (spec->model == kOHaraRudy || spec->model == kTomek) {  // no voltage tables
    rows.clear();
    eca.clear();
    return;
  }
  if (spec->model == kTenTusscher2) {
    // column -> reference table name
    const char *col[T2_COLS] = {"m_inf", "exptau_m", "h_inf", "exptau_h", "j_inf", "exptau_j", "Xr1_inf",
                                "exptau_Xr1", "Xr2_inf", "exptau_Xr2", "Xs_inf", "exptau_Xs", "r_inf",
                                "exptau_r", "s_inf", "exptau_s", "d_inf", "exptau_d", "f_inf", "exptau_f",
                                "f2_inf", "exptau_f2", "rec_ipK", "CaL_P1", "CaL_P2", "NaCa_P1", "NaCa_P2",
                                "NaK_P1"};
    rows.assign((size_t)kRows * T2_COLS, 0.0);
    for (int c = 0; c < T2_COLS; c++) {
      int k = 0;
      while (strcmp(spec->table_names[k], col[c])) k++;
      for (int i = 0; i < kRows; i++) rows[(size_t)i * T2_COLS + c] = tables[k][i];
    }
    int ke = 0;
    while (strcmp(spec->table_names[ke], "ECA")) ke++;
    eca = tables[ke];
  } else {
    rows.assign((size_t)kRows * CR_COLS, 0.0);
    for (int c = 0; c < CR_COLS; c++)  // spec order is the column order for Courtemanche
      for (int i = 0; i < kRows; i++) rows[(size_t)i * CR_COLS + c] = tables[c][i];
    eca.clear();
  }
}

void ParamSet::rows_fp32(std::vector<float> &rows, std::vector<float> &eca) const {
  std::vector<double> r, e;
  rows_fp64(r, e);
  rows.assign(r.begin(), r.end());
  eca.assign(e.begin(), e.end());
}

#undef PV

}  // namespace cm
