// Per-cell output columns of vbElphyModel::Print / LongPrint for a cell of a batch, in the
// reference's column order, so that per-node code reading them (acCELLerate's sensor output,
// EMCoupling::GetResPara / GetResVal, acltCellModel.h:92-133) sees the same columns.
//
//   TenTusscher2: Print TenTusscher2.cpp:908-930 (states, O from the new Rq and CaSS);
//                 LongPrint 932-957 (the 17 stored currents Array[0..16]);
//                 names GetParameterNames 959-979, GetLongParameterNames 981-999.
//   Courtemanche: Print CourtemancheEtAl.cpp:189-198 (states, TRPNmax * Ca_TRPN: TRPN is defined,
//                 CourtemancheParameters.h:23); LongPrint 200-239 (currents from the state and the
//                 tables at the voltage row; I_SAC stored: ISAC is defined, :20); names 241-265.
//   O'Hara-Rudy:  Print OHaraRudy.cpp:665-679 (states, 0.07 * Ca_TRPN), LongPrint 681-691 (the
//                 17 stored currents, OHaraRudy.h:49-52, block slots 42-58); names 693-740.
//   Tomek:        Print Tomek.cpp:658-672 (states and the stored I_Na rates A_h, B_h, A_j, B_j,
//                 block slots 1, 2, 4, 5; 0.07 * Ca_TRPN), LongPrint 674-684 (stored currents and
//                 fluxes in print order, Tomek.h:43-47); names 686-733.
#include <cmath>
#include <cstring>
#include <vector>

#include "cm_handles.h"

extern "C" int cm_batch_get_cell(cm_batch_t b, int64_t cell, int layout, double *out);

namespace {

const char *const kTT2Print[] = {"m",   "h",   "j",  "d",  "f",   "f2",   "fCa",  "Rq",  "O",  "Xr1",
                                 "Xr2", "Xs",  "r",  "s",  "Cai", "CaSR", "CaSS", "Nai", "Ki"};
const char *const kTT2Long[] = {"I_Na", "I_CaL", "I_bCa",  "I_pCa",  "I_to",   "I_Ks",  "I_Kr",  "I_K1", "I_pK",
                                "I_bNa", "I_NaK", "I_NaCa", "I_rel", "I_leak", "I_xfer", "SERCA", "I_tot"};
const char *const kCRNPrint[] = {"m", "h", "j",   "oa", "oi",   "ua",   "ui",   "x_r",   "x_s",    "d",     "f",
                                 "fCa", "u", "v", "w",  "Na_i", "Ca_i", "K_i",  "Ca_up", "Ca_rel", "Ca_TRPN"};
const char *const kCRNLong[] = {"I_Na",  "I_K1",  "I_to",  "I_Kur", "I_Kr", "I_Ks", "I_CaL",
                                "I_pCa", "I_NaK", "I_NaCa", "I_bNa", "I_bCa", "I_ion", "Fn",
                                "I_rel", "I_tr",  "I_up",  "I_upLeak", "I_SAC"};
const char *const kORDPrint[] = {
    "m",          "h_fast",      "h_slow",    "j",         "h_CaMK_slow", "j_CaMK",    "m_L",         "h_L",
    "h_L_CaMK",   "a",           "i_fast",    "i_slow",    "a_CaMK",      "i_CaMK_fast", "i_CaMK_slow", "d",
    "f_fast",     "f_slow",      "f_Ca_fast", "f_Ca_slow", "j_Ca",        "f_CaMK_fast", "f_Ca_CaMK_fast", "n",
    "x_r_fast",   "x_r_slow",    "x_s1",      "x_s2",      "x_K1",        "Na_i",      "Na_ss",       "K_i",
    "K_ss",       "Ca_i",        "Ca_ss",     "Ca_nsr",    "Ca_jsr",      "CaMK_trap", "J_rel_NP",    "J_rel_CaMK",
    "Ca_TRPN"};
const char *const kORDLong[] = {"I_Na_fast", "I_Na_late", "I_to",  "I_CaL", "I_CaNa", "I_CaK",
                                "I_Kr",      "I_Ks",      "I_K1",  "I_NaCa_i", "I_NaCa_ss", "I_NaK",
                                "I_Nab",     "I_Cab",     "I_Kb",  "I_pCa", "I_SAC"};
const char *const kTOMPrint[] = {
    "m",        "A_h",       "B_h",       "h",         "A_j",         "B_j",         "j",           "h_p",
    "j_p",      "m_L",       "h_L",       "h_L_CaMK",  "a",           "i_fast",      "i_slow",      "a_CaMK",
    "i_CaMK_fast", "i_CaMK_slow", "d",    "f_fast",    "f_slow",      "f_Ca_fast",   "f_Ca_slow",   "j_Ca",
    "f_CaMK_fast", "f_Ca_CaMK_fast", "n_ss", "n_i",    "C_0",         "C_1",         "C_2",         "O",
    "I",        "x_s1",      "x_s2",      "Na_i",      "Na_ss",       "K_i",         "K_ss",        "Ca_i",
    "Ca_ss",    "Ca_nsr",    "Ca_jsr",    "Cl_i",      "CaMK_trap",   "J_rel_NP",    "J_rel_CaMK",  "Ca_TRPN"};
const char *const kTOMLong[] = {"I_Na",     "I_Na_late", "I_to",     "I_CaL_i",   "I_CaL_ss", "I_CaNa_i", "I_CaNa_ss",
                                "I_CaK_i",  "I_CaK_ss",  "I_CaL",    "I_CaNa",    "I_CaK",    "I_Kr",     "I_Ks",
                                "I_K1",     "I_NaCa_i",  "I_NaCa_ss", "I_NaK",    "I_CaCl",   "I_Nab",    "I_Cab",
                                "I_Kb",     "I_Clb",     "I_pCa",    "J_diff_Na", "J_diff_Ca", "J_diff_K", "J_leak",
                                "J_rel",    "J_tr",      "J_up",     "cur_I_tot", "I_SAC"};
// block slots of Tomek's LongPrint columns (member order of Tomek.h:43-47 from slot 48)
const int kTOMLongSlot[] = {48, 49, 50, 54, 55, 56, 57, 58, 59, 51, 52, 53, 60, 61, 62, 63, 64,
                            65, 68, 69, 70, 71, 72, 73, 74, 75, 76, 77, 78, 79, 80, 81, 83};
constexpr int kN_TT2P = sizeof(kTT2Print) / sizeof(kTT2Print[0]);
constexpr int kN_ORDP = sizeof(kORDPrint) / sizeof(kORDPrint[0]);
constexpr int kN_ORDL = sizeof(kORDLong) / sizeof(kORDLong[0]);
constexpr int kN_TOMP = sizeof(kTOMPrint) / sizeof(kTOMPrint[0]);
constexpr int kN_TOML = sizeof(kTOMLong) / sizeof(kTOMLong[0]);
static_assert(sizeof(kTOMLongSlot) / sizeof(kTOMLongSlot[0]) == kN_TOML, "one slot per Tomek column");
constexpr int kN_TT2L = sizeof(kTT2Long) / sizeof(kTT2Long[0]);
constexpr int kN_CRNP = sizeof(kCRNPrint) / sizeof(kCRNPrint[0]);
constexpr int kN_CRNL = sizeof(kCRNLong) / sizeof(kCRNLong[0]);

// Column count, or -1 where this build has no per-cell print columns for the model.
int n_columns(int model, bool long_form) {
  if (model == cm::kTenTusscher2) return kN_TT2P + (long_form ? kN_TT2L : 0);
  if (model == cm::kCourtemanche) return kN_CRNP + (long_form ? kN_CRNL : 0);
  if (model == cm::kOHaraRudy) return kN_ORDP + (long_form ? kN_ORDL : 0);
  if (model == cm::kTomek) return kN_TOMP + (long_form ? kN_TOML : 0);
  return -1;
}

double soa_value(const cm::ModelSpec *spec, const std::vector<double> &soa, const char *name) {
  for (int k = 0; k < spec->n_state; k++)
    if (!strcmp(spec->state_names[k], name)) return soa[k];
  return NAN;
}

const double *table(const cm::ParamSet &ps, const char *name) {
  for (int k = 0; k < ps.spec->n_tables; k++)
    if (!strcmp(ps.spec->table_names[k], name)) return ps.tables[k].data();
  return nullptr;
}

}  // namespace

extern "C" {

int cm_model_print_names(int model, int long_form, const char **names, int cap) {
  const int n = n_columns(model, long_form != 0);
  if (n < 0) return cm::fail(CM_ERR_UNSUPPORTED, "no per-cell print columns for this model");
  if (names && cap < n) return cm::fail(CM_ERR_ARG, "names: room for " + std::to_string(n) + " entries needed");
  if (!names) return n;
  const char *const *p = kCRNPrint, *const *l = kCRNLong;
  int np = kN_CRNP;
  if (model == cm::kTenTusscher2) p = kTT2Print, l = kTT2Long, np = kN_TT2P;
  if (model == cm::kOHaraRudy) p = kORDPrint, l = kORDLong, np = kN_ORDP;
  if (model == cm::kTomek) p = kTOMPrint, l = kTOMLong, np = kN_TOMP;
  for (int k = 0; k < n; k++) names[k] = k < np ? p[k] : l[k - np];
  return n;
}

int cm_batch_print_values(cm_batch_t b, int64_t cell, double V, int long_form, double *values, int cap) {
  if (!b || !values) return cm::fail(CM_ERR_ARG, "NULL argument");
  const cm::ParamSet &ps = b->ps;
  const int model = ps.spec->model;
  const int n = n_columns(model, long_form != 0);
  if (n < 0) return cm::fail(CM_ERR_UNSUPPORTED, "no per-cell print columns for this model");
  if (cap < n) return cm::fail(CM_ERR_ARG, "values: room for " + std::to_string(n) + " entries needed");
  std::vector<double> soa(ps.spec->n_state), blk(ps.spec->ref_block_doubles);
  int rc = cm_batch_get_cell(b, cell, CM_LAYOUT_SOA, soa.data());
  if (rc) return rc;
  if ((long_form || model == cm::kTomek) && (rc = cm_batch_get_cell(b, cell, CM_LAYOUT_REF_BLOCK, blk.data())))
    return rc;
  auto S = [&](const char *nm) { return soa_value(ps.spec, soa, nm); };
  auto P = [&](const char *nm) { return ps.get(nm); };
  int k = 0;
  if (model == cm::kTenTusscher2) {
    const double CaSR = S("CaSR"), CaSS = S("CaSS"), Rq = S("Rq");
    const double max_sr = P("max_sr"), EC = P("EC");
    const double kCaSR = max_sr - ((max_sr - P("min_sr")) / (1 + (EC / CaSR) * (EC / CaSR)));
    const double k1 = P("ks1") / kCaSR, CaSS2 = CaSS * CaSS;
    const double O = k1 * CaSS2 * Rq / (P("k3") + k1 * CaSS2);
    const double cols[kN_TT2P] = {S("m"),   S("h"),   S("j"),  S("d"),  S("f"),    S("f2"), S("fCa"),
                                  Rq,       O,        S("xr1"), S("xr2"), S("xs"),  S("r"),  S("s"),
                                  S("Ca_i"), CaSR,    CaSS,     S("Na_i"), S("K_i")};
    for (double c : cols) values[k++] = c;
    // Array[0..16] follows Ca_i, CaSR, CaSS, Na_i, K_i in the block (TenTusscher2.h:77-78)
    if (long_form)
      for (int a = 0; a < kN_TT2L; a++) values[k++] = blk[5 + a];
    return k;
  }
  if (model == cm::kOHaraRudy || model == cm::kTomek) {
    const bool tom = model == cm::kTomek;
    const char *const *names = tom ? kTOMPrint : kORDPrint;
    const int np = tom ? kN_TOMP : kN_ORDP;
    for (int c = 0; c < np; c++) {
      const char *nm = names[c];
      if (!strcmp(nm, "Ca_TRPN")) {
        values[k++] = 0.07 * S(nm);  // exported in mM
      } else if (tom && (!strcmp(nm, "A_h") || !strcmp(nm, "B_h") || !strcmp(nm, "A_j") || !strcmp(nm, "B_j"))) {
        values[k++] = blk[!strcmp(nm, "A_h") ? 1 : (!strcmp(nm, "B_h") ? 2 : (!strcmp(nm, "A_j") ? 4 : 5))];
      } else {
        values[k++] = S(nm);
      }
    }
    if (long_form) {
      if (tom)
        for (int c = 0; c < kN_TOML; c++) values[k++] = blk[kTOMLongSlot[c]];
      else
        for (int c = 0; c < kN_ORDL; c++) values[k++] = blk[42 + c];
    }
    return k;
  }
  // Courtemanche
  const double m = S("m"), h = S("h"), j = S("j"), oa = S("oa"), oi = S("oi"), ua = S("ua"), ui = S("ui");
  const double Xr = S("Xr"), Xs = S("Xs"), d = S("d"), f = S("f"), f_Ca = S("f_Ca"), u = S("u"), v = S("v"),
               w = S("w");
  const double Na_i = S("Na_i"), Ca_i = S("Ca_i"), K_i = S("K_i"), Ca_up = S("Ca_up"), Ca_rel = S("Ca_rel");
  const double cols[kN_CRNP] = {m, h, j, oa, oi, ua, ui, Xr, Xs, d, f, f_Ca, u, v, w, Na_i, Ca_i, K_i, Ca_up, Ca_rel,
                                P("TRPNmax") * S("Ca_TRPN")};
  for (double c : cols) values[k++] = c;
  if (!long_form) return k;
  const double V_int = V * 1000.0;
  int Vi = (int)(10.0 * (200.0 + V_int) + .5);
  if (Vi < 0) Vi = 0;  // the reference reads its tables unchecked; the row is clamped here
  if (Vi > cm::kRows - 1) Vi = cm::kRows - 1;
  const double dNa_i = 1.0 / Na_i;
  const double VmE_Na = V_int - (P("RTdF") * log(P("Na_o") * dNa_i));
  const double VmE_K = V_int - (P("RTdF") * log(P("K_o") / K_i));
  const double VmE_Ca = V_int - (P("RTd2F") * log(P("Ca_o") / Ca_i));
  const double I_Na = P("g_Na") * m * m * m * h * j * VmE_Na;
  const double I_to = P("g_to") * oa * oa * oa * oi * VmE_K;
  const double I_Kur = table(ps, "g_Kur")[Vi] * ua * ua * ua * ui * VmE_K;
  const double I_Kr = table(ps, "CKr")[Vi] * Xr * VmE_K;
  const double I_Ks = P("g_Ks") * Xs * Xs * VmE_K;
  const double I_CaL = P("g_CaL") * d * f * f_Ca * (V_int - P("E_rL"));
  const double I_K1 = table(ps, "CK1")[Vi] * VmE_K;
  const double I_bNa = P("g_bNa") * VmE_Na;
  const double I_bCa = P("g_bCa") * VmE_Ca;
  const double tmp = P("k_mNai") * dNa_i;
  const double I_NaK = table(ps, "CNaK")[Vi] / (1.0 + tmp * sqrt(tmp));
  const double I_pCa = P("I_pCamax") * Ca_i / (Ca_i + P("k_mpCa"));
  const double I_NaCa = table(ps, "CNaCa")[Vi] * ((Na_i * Na_i * Na_i * P("Ca_o")) - table(ps, "expVm")[Vi] * Ca_i);
  const double I_rel = P("k_rel") * u * u * v * w * (Ca_rel - Ca_i);
  const double I_up = P("I_upmax") * Ca_i / (Ca_i + P("k_up"));
  const double I_upleak = P("kupleak") * Ca_up;
  const double I_tr = (Ca_up - Ca_rel) * P("dt_tr");
  const double Fn = 1e-12 * P("Vrel") * I_rel - 5e-13 * P("C_m") * (0.5 * I_CaL - 0.2 * I_NaCa) / P("F");
  // I_SAC: the stored value, slot 20 of the block (where cm_batch_get_cell puts it)
  const double I_SAC = blk[20];
  const double I_mem = I_Na + I_CaL + I_pCa + I_K1 + I_to + I_Kur + I_Kr + I_Ks + I_bNa + I_bCa + I_NaK + I_NaCa + I_SAC;
  const double lc[kN_CRNL] = {I_Na,  I_K1,  I_to,  I_Kur, I_Kr, I_Ks, I_CaL, I_pCa, I_NaK,   I_NaCa,
                              I_bNa, I_bCa, I_mem, Fn,    I_rel, I_tr, I_up, I_upleak, I_SAC};
  for (double c : lc) values[k++] = c;
  return k;
}

}  // extern "C"
