// Host-side parameter sets: model registry, .ev loading, derived values and FP64 lookup
// tables (the reference's vbElphyParameters / initElphyParameters side of the interface).
#pragma once

#include <string>
#include <vector>

#include "cm_common.cuh"

namespace cm {

// Reference ElphyModelType values (ElphyModelBasis.h:62-81).
enum ModelId { kCourtemanche = 2, kTenTusscher2 = 5, kOHaraRudy = 12, kTomek = 14 };

struct ParamDef {
  const char *name;
  double value;
};

struct ModelSpec {
  int model;
  const char *name;                // reference ElphyModelDescriptor
  const ParamDef *base;            // parameters read from the .ev file, with built-in defaults
  int n_base;
  const char *const *derived;      // names of the values Calculate() derives
  int n_derived;
  const char *const *table_names;  // reference table array names (none for O'Hara-Rudy, Tomek)
  int n_tables;
  const char *const *state_names;  // SOA state order
  int n_state;
  int ref_block_doubles;           // GetSize() / 8
  const char *const *het_names;    // per-cell parameter slots
  int n_het;
  double default_amplitude;        // GetAmplitude() fallback when not a parameter
  double default_stim_time;
};

const ModelSpec *find_model(int model);
int model_from_name(const char *name);

class ParamSet {
 public:
  const ModelSpec *spec = nullptr;
  double dt = 0;
  std::vector<double> vals;                 // base then derived, spec order
  std::vector<std::vector<double>> tables;  // reference table arrays, spec order
  double exp250 = 0, exp50 = 0;             // Courtemanche scalars (CourtemancheParameters.cpp:246-247)

  // Returns 0 or a cm_status; err receives a message.
  int init(int model, const char *ev_path, double dt_, std::string &err);
  int index(const char *name) const;  // -1 if unknown
  double get(const char *name) const;
  void rebuild();  // derive + tables

  double init_vm() const;
  double amplitude() const;
  double stim_time() const;

  // Device-ready forms.
  void tt2_consts(TT2Consts<double> &d, TT2Consts<float> &f) const;
  void crn_consts(CRNConsts<double> &d, CRNConsts<float> &f) const;
  void ord_consts(ORDConsts<double> &d, ORDConsts<float> &f) const;
  void tom_consts(TOMConsts<double> &d, TOMConsts<float> &f) const;
  // Row-major voltage tables (kRows x cols) and the TT2 ECa table.
  void rows_fp64(std::vector<double> &rows, std::vector<double> &eca) const;
  void rows_fp32(std::vector<float> &rows, std::vector<float> &eca) const;
  // Initial SOA state of one cell (spec->n_state doubles).
  void init_state(std::vector<double> &s) const;

 private:
  void derive();
  void derive_ord();
  void derive_tom();
  void build_tables();
};

}  // namespace cm
