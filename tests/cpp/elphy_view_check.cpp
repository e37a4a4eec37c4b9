// A C++ caller of libcmgb300 written the way CardioMechanics code calls its cell models:
//  1. the acCELLerate patch sketched in INTEGRATION.md (parameter set, batch, per-node
//     heterogeneity, initial Vm, cm_batch_step and the fused Godunov update, backup blocks);
//  2. per-node vbElphyModel views (include/cardiomech_gb300_elphy.hpp) against the batch path:
//     Calc node by node equals cm_batch_step bit for bit, GetResPara / GetResVal read the
//     LongPrint columns, WriteStatus / ReadStatus round-trip a node, Init restores it.
// Built with the stand-in interface (or the reference's ElphyModelBasis.h where present) and
// run on the GPU; prints OK and exits 0 when every check holds.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include VB_ELPHY_HEADER
#include "cardiomech_gb300_elphy.hpp"

using View = cmgb::CellView<vbElphyModel<double>>;

static int failures = 0;
#define CHECK(cond, ...)                                     \
  do {                                                       \
    if (!(cond)) {                                           \
      std::fprintf(stderr, "FAIL %s:%d: ", __FILE__, __LINE__); \
      std::fprintf(stderr, __VA_ARGS__);                     \
      std::fprintf(stderr, "\n");                            \
      failures++;                                            \
    }                                                        \
  } while (0)

// acltCellModel.h:92-133 (EMCoupling::GetResPara / GetResVal), restated for the test: find a
// column by name after "t" and "V_m", then read that token of LongPrint's output.
static int res_pos(vbElphyModel<double> *pem, const std::string &name) {
  std::vector<std::string> names{"t", "V_m"};
  pem->GetLongParameterNames(names);
  for (size_t i = 0; i < names.size(); i++)
    if (names[i] == name) return (int)i;
  return -1;
}
static double res_val(vbElphyModel<double> *pem, int pos, double t, double Vm) {
  std::ostringstream os;
  pem->LongPrint(os, t, Vm);
  std::istringstream is(os.str());
  double v = 0;
  for (int k = 0; k <= pos; k++) is >> v;
  return v;
}

int main() {
  const double dt = 1e-5, amp = 52.0 * 2.29656e-2;
  const int n = 6;
  // ---- 1. the INTEGRATION.md sketch: one material, NoCoupling
  cm_params_t p;
  cm_batch_t b, ref;
  if (cm_params_create(&p, CM_MODEL_TENTUSSCHER2, nullptr, dt) || cm_batch_create(&b, p, n, CM_PREC_FP64, nullptr) ||
      cm_batch_create(&ref, p, n, CM_PREC_FP64, nullptr)) {
    std::fprintf(stderr, "libcmgb300: %s\n", cm_last_error());
    return 2;
  }
  double gkr = 0;
  cm_params_get(p, "g_Kr", &gkr);
  std::vector<double> g(n);
  for (int l = 0; l < n; l++) g[l] = gkr * (0.9 + 0.04 * l);
  CHECK(cm_batch_set_hetero(ref, "g_Kr", g.data()) == 0, "%s", cm_last_error());
  cm_batch_set_diagnostics(b, 1);
  cm_batch_set_diagnostics(ref, 1);
  std::vector<double> vm_ref(n), vm_view(n), iext(n), dvm(n);
  CHECK(cm_batch_init_vm(ref, vm_ref.data()) == 0, "%s", cm_last_error());

  // ---- 2. the same nodes through per-node views of batch b
  auto nodes = std::make_shared<cmgb::BatchNodes>(p, b);
  std::vector<std::unique_ptr<View>> pem;
  for (int l = 0; l < n; l++) pem.emplace_back(new View(nodes, l));
  for (int l = 0; l < n; l++) {
    CHECK(pem[l]->AddHeteroValue("g_Kr", g[l]), "AddHeteroValue");
    vm_view[l] = pem[l]->GetVm();
  }
  CHECK(!pem[0]->AddHeteroValue("no_such_parameter", 1.0), "unknown name accepted");
  CHECK(vm_view == vm_ref, "GetVm differs from cm_batch_init_vm");

  // 3000 steps (30 ms) through the stimulus and the upstroke: node-by-node Calc against one
  // cm_batch_step per step (the driver's Vm += dV, CellModel.h:420)
  int worst_step = -1;
  for (int s = 0; s < 3000; s++) {
    const double t = s * dt;
    for (int l = 0; l < n; l++) iext[l] = t < 1e-3 ? amp : 0.0;
    CHECK(cm_batch_step(ref, dt, vm_ref.data(), iext.data(), nullptr, dvm.data()) == 0, "%s", cm_last_error());
    for (int l = 0; l < n; l++) {
      const double dv = pem[l]->Calc(dt, vm_view[l], iext[l], 1.0, 1);
      if (dv != dvm[l] && worst_step < 0) worst_step = s;
      vm_view[l] += dv;
      vm_ref[l] += dvm[l];
    }
  }
  CHECK(worst_step < 0, "per-node Calc differs from cm_batch_step at step %d", worst_step);
  CHECK(vm_view == vm_ref, "Vm differs after 3000 steps");
  CHECK(vm_ref[0] > 0.0, "no action potential (Vm %g)", vm_ref[0]);

  // GetResPara / GetResVal on LongPrint: columns equal the library's values; I_tot is the last
  // step's total current, dV = -dt * I_tot (TenTusscher2.cpp:905)
  const int pos_cai = res_pos(pem[2].get(), "Cai"), pos_itot = res_pos(pem[2].get(), "I_tot");
  CHECK(pos_cai == 16 && pos_itot > pos_cai, "column positions %d %d", pos_cai, pos_itot);
  const double cai = res_val(pem[2].get(), pos_cai, 0.03, vm_view[2]);
  // Print writes with the stream's default precision (6 significant digits), as the reference's does
  CHECK(std::fabs(cai - pem[2]->GetCai()) <= 1e-5 * std::fabs(cai), "Cai column %g vs GetCai %g", cai,
        pem[2]->GetCai());
  const double itot = res_val(pem[2].get(), pos_itot, 0.03, vm_view[2]);
  const double dv_last = pem[2]->Calc(dt, vm_view[2], 0.0, 1.0, 1);
  vm_view[2] += dv_last;
  const double itot_now = res_val(pem[2].get(), pos_itot, 0.03, vm_view[2]);
  CHECK(std::fabs(-dt * itot_now - dv_last) <= 1e-5 * std::fabs(dv_last) + 1e-15, "I_tot %g vs dV %g", itot_now,
        dv_last);
  (void)itot;
  std::vector<std::string> short_names;
  pem[0]->GetParameterNames(short_names);
  CHECK(short_names.size() == 19 && short_names[8] == "O", "Print names");

  // WriteStatus / ReadStatus round trip of node 4, and Set between two views
  std::vector<double> before(nodes->block_doubles()), after(nodes->block_doubles());
  std::memcpy(before.data(), pem[4]->GetBase(), pem[4]->GetSize());
  FILE *f = std::tmpfile();
  pem[4]->WriteStatus(f);
  for (int s = 0; s < 50; s++) vm_view[4] += pem[4]->Calc(dt, vm_view[4], 0.0, 1.0, 1);
  std::rewind(f);
  pem[4]->ReadStatus(f);
  std::fclose(f);
  nodes->flush();
  CHECK(cm_batch_get_cell(b, 4, CM_LAYOUT_REF_BLOCK, after.data()) == 0, "%s", cm_last_error());
  bool same = true;
  for (int k = 0; k < 5; k++) same = same && before[k] == after[k];   // Ca_i .. K_i
  for (int k = 23; k < 36; k++) same = same && before[k] == after[k]; // the gates
  CHECK(same, "ReadStatus did not restore node 4");
  pem[5]->Set(*pem[4]);
  nodes->flush();
  std::vector<double> b5(nodes->block_doubles());
  cm_batch_get_cell(b, 5, CM_LAYOUT_REF_BLOCK, b5.data());
  CHECK(b5[0] == after[0] && b5[35] == after[35], "Set did not copy node 4 to node 5");

  // Init: the node back to the initial block of a fresh batch
  pem[1]->Init();
  std::vector<double> fresh(nodes->block_doubles()), b1(nodes->block_doubles());
  cm_batch_t one;
  cm_batch_create(&one, p, 1, CM_PREC_FP64, nullptr);
  cm_batch_get_cell(one, 0, CM_LAYOUT_REF_BLOCK, fresh.data());
  cm_batch_destroy(one);
  cm_batch_get_cell(b, 1, CM_LAYOUT_REF_BLOCK, b1.data());
  CHECK(fresh[0] == b1[0] && fresh[35] == b1[35], "Init");
  CHECK(pem[0]->GetSize() == 288 && std::fabs(pem[0]->GetAmplitude()) > 0 && pem[0]->Volume() > 0, "getters");

  // the sketch's fused Godunov step and backup blocks
  CHECK(cm_batch_step_update(ref, dt, vm_ref.data(), iext.data(), nullptr, 0.2) == 0, "%s", cm_last_error());
  std::vector<double> blk((size_t)36 * n);
  CHECK(cm_batch_get_state(ref, CM_LAYOUT_REF_BLOCK, blk.data()) == 0, "%s", cm_last_error());
  CHECK(cm_batch_calc_cell(b, n, dt, -0.08, 0, 1, dvm.data()) == CM_ERR_ARG, "out-of-range cell accepted");

  // Courtemanche: Print / LongPrint columns through a view
  cm_params_t pc;
  cm_batch_t bc;
  CHECK(cm_params_create(&pc, CM_MODEL_COURTEMANCHE, nullptr, dt) == 0 && cm_batch_create(&bc, pc, 2, CM_PREC_FP64,
                                                                                          nullptr) == 0,
        "%s", cm_last_error());
  auto cnodes = std::make_shared<cmgb::BatchNodes>(pc, bc);
  View crn(cnodes, 1);
  double v = crn.GetVm();
  for (int s = 0; s < 500; s++) v += crn.Calc(dt, v, s < 200 ? 20.0 : 0.0, 1.0, 1);
  std::vector<std::string> cn{"t", "V_m"};
  crn.GetLongParameterNames(cn);
  CHECK(cn.size() == 2 + 21 + 19 && cn[2] == "m" && cn.back() == "I_SAC", "Courtemanche names (%zu)", cn.size());
  std::ostringstream os;
  crn.LongPrint(os, 0.005, v);
  std::istringstream is(os.str());
  std::vector<double> col;
  double x;
  while (is >> x) col.push_back(x);
  CHECK(col.size() == cn.size(), "Courtemanche LongPrint columns %zu", col.size());
  if (col.size() == cn.size()) {
    double sum = 0, big = 1;  // I_ion is the sum of the twelve membrane currents before it and I_SAC
    for (int k = 23; k < 35; k++) sum += col[k], big = std::fmax(big, std::fabs(col[k]));
    sum += col.back();
    CHECK(std::fabs(sum - col[35]) <= 1e-4 * big, "I_ion %g vs sum %g", col[35], sum);
    CHECK(std::fabs(col[1] - v) <= 1e-5 * std::fabs(v) && col[0] == 0.005, "t and V columns");
  }
  cm_batch_destroy(bc);
  cm_params_destroy(pc);

  // O'Hara-Rudy (12) and Tomek (14), FP64 with the stored values on: LongPrint has the
  // reference's column count, the state columns read back as the view's getters, the stored
  // currents are those of the last Calc (non-zero after a stimulated step)
  const int models[2] = {12, 14};
  const size_t want[2] = {2 + 41 + 17, 2 + 48 + 33};
  for (int q = 0; q < 2; q++) {
    cm_params_t po;
    cm_batch_t bo;
    CHECK(cm_params_create(&po, models[q], nullptr, dt) == 0 && cm_batch_create(&bo, po, 1, CM_PREC_FP64, nullptr) == 0,
          "%s", cm_last_error());
    cm_batch_set_diagnostics(bo, 1);
    auto onodes = std::make_shared<cmgb::BatchNodes>(po, bo);
    View ov(onodes, 0);
    double vo = ov.GetVm();
    for (int st = 0; st < 200; st++) vo += ov.Calc(dt, vo, st < 100 ? -53.0 : 0.0, 1.0, 1);
    std::vector<std::string> on{"t", "V_m"};
    ov.GetLongParameterNames(on);
    CHECK(on.size() == want[q] && on[2] == "m" && on.back() == "I_SAC", "model %d names (%zu)", models[q], on.size());
    std::ostringstream oss;
    ov.LongPrint(oss, 0.002, vo);
    std::istringstream iss(oss.str());
    std::vector<double> oc;
    while (iss >> x) oc.push_back(x);
    CHECK(oc.size() == on.size(), "model %d LongPrint columns %zu", models[q], oc.size());
    if (oc.size() == on.size()) {
      int nai = -1;
      for (size_t k = 0; k < on.size(); k++)
        if (on[k] == "Na_i") nai = (int)k;
      CHECK(nai > 0 && std::fabs(oc[nai] - ov.GetNai()) <= 1e-5 * ov.GetNai(), "model %d Na_i column", models[q]);
      double stored = 0;
      for (size_t k = on.size() - 5; k < on.size(); k++) stored += std::fabs(oc[k]);
      CHECK(stored > 0, "model %d stored currents are zero", models[q]);
    }
    cm_batch_destroy(bo);
    cm_params_destroy(po);
  }
  cm_batch_destroy(b);
  cm_batch_destroy(ref);
  cm_params_destroy(p);
  if (failures) {
    std::fprintf(stderr, "%d check(s) failed\n", failures);
    return 1;
  }
  std::printf("OK\n");
  return 0;
}
