/* cardiomech_gb300_elphy.hpp -- a per-node vbElphyModel view of a libcmgb300 batch (C++).
 *
 * CardioMechanics code that holds one vbElphyModel<double>* per node (acCELLerate's pem[] array,
 * acCELLerate.cpp:725-752; the sensor output through EMCoupling::GetResPara / GetResVal,
 * acltCellModel.h:92-133; backups through GetBase/GetSize, WriteStatus/ReadStatus,
 * ElphyModelBasis.h:243-253) keeps working when the nodes' state lives in a batch on the GPU:
 * each node gets a CellView, which implements the interface of vbElphyModel
 * (ElphyModelBasis.h:184-323) on one cell of the batch through the C ABI.
 *
 * The view is the slow path: one Calc is one launch for one cell. Time loops call
 * cm_batch_step / cm_batch_step_update on the whole batch instead and use the views for output,
 * backups, heterogeneity and the odd single-node call.
 *
 * Usage (Base is the caller's vbElphyModel<double>, from the reference's ElphyModelBasis.h):
 *
 *   auto nodes = std::make_shared<cmgb::BatchNodes>(params, batch);
 *   for (l = 0; l < n; l++) pem[l] = new cmgb::CellView<vbElphyModel<double>>(nodes, l);
 *   ... pem[l]->AddHeteroValue("g_Kr", v) ...; nodes->flush();   // before the next batch step
 *   cm_batch_step(batch, dt, Vm, i_ext, stretch, dVm);           // the time step, all nodes
 *   EMCoupling::GetResVal(pem[l], pos, value, t, Vm[l]);          // unchanged
 *
 * Writes through a block GetBase() handed out (ReadStatus, Set) reach the device at the view's
 * next use or at BatchNodes::flush(), which a caller runs before the next whole-batch step;
 * a block that was not changed is never written back, so it cannot undo a later batch step.
 * Errors are thrown as cmgb::Error (a std::runtime_error carrying cm_last_error()); the
 * reference throws kaBaseException in the same places.
 */
#ifndef CARDIOMECH_GB300_ELPHY_HPP
#define CARDIOMECH_GB300_ELPHY_HPP

#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "cardiomech_gb300.h"

namespace cmgb {

class Error : public std::runtime_error {
 public:
  explicit Error(const std::string &what) : std::runtime_error("libcmgb300: " + what) {}
};

inline int check(int rc) {
  if (rc < 0) throw Error(cm_last_error());
  return rc;
}

/* Host-side companion of one batch, shared by the views of its cells: the handles (borrowed,
 * not destroyed here), the model's constants, the per-node heterogeneous values staged by
 * AddHeteroValue, and the blocks handed out by GetBase. */
class BatchNodes {
 public:
  BatchNodes(cm_params_t params, cm_batch_t batch) : p_(params), b_(batch) {
    check(cm_batch_info(b_, &info_, &n_, &precision_));
    names_long_ = names(1);
    names_short_ = names(0);
  }
  BatchNodes(const BatchNodes &) = delete;
  BatchNodes &operator=(const BatchNodes &) = delete;

  cm_params_t params() const { return p_; }
  cm_batch_t batch() const { return b_; }
  const cm_info &info() const { return info_; }
  int64_t size() const { return n_; }
  int block_doubles() const { return info_.ref_block_doubles; }
  double param(const char *name) const {
    double v = 0;
    check(cm_params_get(p_, name, &v));
    return v;
  }
  const std::vector<std::string> &print_names(bool long_form) const { return long_form ? names_long_ : names_short_; }

  /* AddHeteroValue for one node: the value is staged and reaches the batch at flush(). An
   * array starts from the parameter set's value for every node. */
  bool stage_hetero(int64_t cell, const std::string &name, double value) {
    double base = 0;
    if (cell < 0 || cell >= n_ || cm_params_get(p_, name.c_str(), &base) != CM_OK) return false;
    auto it = hetero_.find(name);
    if (it == hetero_.end()) it = hetero_.emplace(name, std::vector<double>((size_t)n_, base)).first;
    it->second[(size_t)cell] = value;
    hetero_dirty_[name] = true;
    return true;
  }

  /* The node's block as GetBase() hands it out: pulled from the device now (after pushing any
   * change made to the block handed out before). */
  double *pull_block(int64_t cell) {
    Slot &s = slots_[cell];
    push_block(cell);
    s.buf.resize((size_t)block_doubles());
    check(cm_batch_get_cell(b_, cell, CM_LAYOUT_REF_BLOCK, s.buf.data()));
    s.pulled = s.buf;
    return s.buf.data();
  }

  /* Writes the node's handed-out block back if the caller changed it. */
  void push_block(int64_t cell) {
    auto it = slots_.find(cell);
    if (it == slots_.end() || it->second.buf.empty()) return;
    Slot &s = it->second;
    if (std::memcmp(s.buf.data(), s.pulled.data(), s.buf.size() * sizeof(double)) != 0) {
      check(cm_batch_set_cell(b_, cell, CM_LAYOUT_REF_BLOCK, s.buf.data()));
      s.pulled = s.buf;
    }
  }

  void push_hetero() {
    for (auto &kv : hetero_dirty_) {
      if (!kv.second) continue;
      check(cm_batch_set_hetero(b_, kv.first.c_str(), hetero_[kv.first].data()));
      kv.second = false;
    }
  }

  /* Everything staged through the views reaches the device: run before a whole-batch step. */
  void flush() {
    push_hetero();
    for (auto &kv : slots_) push_block(kv.first);
  }

  /* The model's initial block (what Init() gives a fresh model), computed once. */
  const std::vector<double> &initial_block() {
    if (init_block_.empty()) {
      cm_batch_t one = nullptr;
      check(cm_batch_create(&one, p_, 1, precision_, nullptr));
      init_block_.resize((size_t)block_doubles());
      const int rc = cm_batch_get_cell(one, 0, CM_LAYOUT_REF_BLOCK, init_block_.data());
      cm_batch_destroy(one);
      check(rc);
    }
    return init_block_;
  }

 private:
  struct Slot {
    std::vector<double> buf, pulled;
  };
  std::vector<std::string> names(int long_form) const {
    std::vector<std::string> out;
    const int n = cm_model_print_names(info_.model, long_form, nullptr, 0);
    if (n < 0) return out;  // no print columns for this model: Print / LongPrint throw
    std::vector<const char *> v((size_t)n);
    check(cm_model_print_names(info_.model, long_form, v.data(), n));
    for (const char *s : v) out.emplace_back(s);
    return out;
  }

  cm_params_t p_;
  cm_batch_t b_;
  cm_info info_{};
  int64_t n_ = 0;
  int precision_ = 0;
  std::vector<std::string> names_long_, names_short_;
  std::map<std::string, std::vector<double>> hetero_;
  std::map<std::string, bool> hetero_dirty_;
  std::map<int64_t, Slot> slots_;
  std::vector<double> init_block_;
};

/* vbElphyModel<double> on node `cell` of a batch. Base: the caller's vbElphyModel<double>. */
template <class Base>
class CellView : public Base {
 public:
  CellView(std::shared_ptr<BatchNodes> nodes, int64_t cell) : nodes_(std::move(nodes)), cell_(cell) {
    if (cell_ < 0 || cell_ >= nodes_->size()) throw Error("CellView: cell index out of range");
  }

  int64_t cell() const { return cell_; }
  BatchNodes &nodes() const { return *nodes_; }

  /* Init (TenTusscher2.cpp:250-271, CourtemancheEtAl.cpp:56-83): the cell's state back to the
   * parameter set's initial values. */
  void Init() override {
    sync();
    check(cm_batch_set_cell(nodes_->batch(), cell_, CM_LAYOUT_REF_BLOCK, nodes_->initial_block().data()));
  }

  /* One step of this node (ElphyModelBasis.h:264); tinc must be the parameter set's dt. The
   * models here always take their Rush-Larsen / Euler step, the reference's euler = 1. */
  double Calc(double tinc, double V, double i_external = 0., double stretch = 1., int euler = 1) override {
    (void)euler;
    sync();
    double dV = 0;
    check(cm_batch_calc_cell(nodes_->batch(), cell_, tinc, V, i_external, stretch, &dV));
    return dV;
  }

  void Print(std::ostream &os, double t, double V) override { print(os, t, V, false); }
  void LongPrint(std::ostream &os, double t, double V) override { print(os, t, V, true); }
  void GetParameterNames(std::vector<std::string> &out) override { append(out, false); }
  void GetLongParameterNames(std::vector<std::string> &out) override { append(out, true); }

  double GetVm() override { return nodes_->info().init_vm; }
  double GetCai() override { return state("Ca_i"); }
  double GetNai() override { return state("Na_i"); }
  double GetKi() override { return state("K_i"); }
  double GetCao() override { return nodes_->param("Ca_o"); }
  double GetNao() override { return nodes_->param("Na_o"); }
  double GetKo() override { return nodes_->param("K_o"); }
  int GetSize() override { return nodes_->block_doubles() * (int)sizeof(double); }
  double *GetBase() override { return nodes_->pull_block(cell_); }
  /* Volume() as the models define it: TenTusscher2 Vcell (TenTusscher2.h:197), Courtemanche
   * Vcell_outside * 1e-18 (CourtemancheEtAl.h:50), O'Hara-Rudy and Tomek the constant of
   * OHaraRudy.h:65 and Tomek.h:66. */
  double Volume() override {
    const int m = nodes_->info().model;
    if (m == CM_MODEL_TENTUSSCHER2) return nodes_->param("Vcell");
    if (m == CM_MODEL_COURTEMANCHE) return nodes_->param("Vcell_outside") * 1e-18;
    return 1.15606568e-12;
  }
  double GetAmplitude() override { return nodes_->info().amplitude; }
  double GetStimTime() override { return nodes_->info().stim_time; }
  bool AddHeteroValue(std::string desc, double val) override { return nodes_->stage_hetero(cell_, desc, val); }

 private:
  void sync() {
    nodes_->push_hetero();
    nodes_->push_block(cell_);
  }
  double state(const char *name) {
    sync();
    const int ns = nodes_->info().n_state_vars;
    std::vector<double> soa((size_t)ns);
    check(cm_batch_get_cell(nodes_->batch(), cell_, CM_LAYOUT_SOA, soa.data()));
    for (int k = 0; k < ns; k++)
      if (!std::strcmp(cm_state_name(nodes_->info().model, k), name)) return soa[(size_t)k];
    throw Error(std::string("no state ") + name + " in this model");
  }
  void append(std::vector<std::string> &out, bool long_form) const {
    const auto &nm = nodes_->print_names(long_form);
    if (nm.empty()) throw Error("no print columns for this model");
    out.insert(out.end(), nm.begin(), nm.end());
  }
  /* t, V, then the columns, each followed by one blank, as the reference's Print writes them. */
  void print(std::ostream &os, double t, double V, bool long_form) {
    sync();
    const auto &nm = nodes_->print_names(long_form);
    if (nm.empty()) throw Error("no print columns for this model");
    std::vector<double> v(nm.size());
    check(cm_batch_print_values(nodes_->batch(), cell_, V, long_form ? 1 : 0, v.data(), (int)v.size()));
    os << t << ' ' << V << ' ';
    for (double x : v) os << x << ' ';
  }

  std::shared_ptr<BatchNodes> nodes_;
  int64_t cell_;
};

}  // namespace cmgb

#endif
