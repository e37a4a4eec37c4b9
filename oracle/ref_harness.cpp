// Test infrastructure only: a C-ABI harness around the reference's own CellModel
// library (KIT-IBT/CardioMechanics, electrophysiology/src/CellModel), compiled
// from the reference sources by oracle/Makefile into oracle/_ref/libcmref.so.
//
// Nothing in the product links this file. It exists so that tests/golden/make_golden.py
// can run the unmodified reference Calc on seeded inputs and commit golden vectors,
// and so that the C restatement in oracle/cm_oracle.c can be pinned against it.
//
// The loop it drives mirrors the reference single-cell driver
// (CellModel/CellModel.h:356-423 `CellParameters::calculate`, time loop
// CellModel/CellModelTest.cpp:353 `for (t = tbegin; t < tend; t += tinc)`) and the
// tissue caller (acCELLerate/acCELLerate.cpp:1757-1770 `CalcCellModels`).
#include <CellModelLayer.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

// The drivers define this global (CellModel/CellModelTest.cpp:24); the library expects it.
PrintParameterModus PrintParameterMode = PrintParameterModeOff;

namespace {

struct RefHandle {
  ElphyModelType emt;
  vbElphyParameters<double> *pep = nullptr;
  std::vector<vbElphyModel<double> *> cells;
  std::string err;
};

thread_local std::string g_err;

// Stimulus state of one driver cell (CellModel.h:405-419 with thresVm = freq = HUGE,
// textend = HUGE, textdiv = 1).
inline double stim_current(double t, double &textbegin, double textlen, double bcl, double amp) {
  double i_ext = 0.0;
  if (t >= textbegin) {
    i_ext = amp;
    if (t >= textbegin + textlen) textbegin += bcl;
  }
  return i_ext;
}

}  // namespace

extern "C" {

const char *ref_last_error() { return g_err.c_str(); }

// model: reference ElphyModelType value (EMT_TenTusscher2 = 5, EMT_CourtemancheEtAl = 2,
// EMT_OHaraRudy = 12, EMT_Tomek = 14).
void *ref_create(int model, const char *ev_path, double dt, int n_cells) {
  try {
    if (!getenv("kaRootDir")) {
      g_err = "kaRootDir is not set";
      return nullptr;
    }
    auto *h = new RefHandle();
    h->emt = (ElphyModelType)model;
    initElphyParameters<double>(&h->pep, ev_path, h->emt, dt);
    h->cells.resize(n_cells, nullptr);
    for (int i = 0; i < n_cells; i++) initElphyModel<double>(&h->cells[i], h->pep, h->emt);
    return h;
  } catch (kaBaseException &e) {
    g_err = e.getText();
    return nullptr;
  } catch (...) {
    g_err = "unknown exception";
    return nullptr;
  }
}

void ref_destroy(void *hv) {
  auto *h = (RefHandle *)hv;
  if (!h) return;
  for (auto *c : h->cells) delete c;
  delete h->pep;
  delete h;
}

int ref_n_cells(void *hv) { return (int)((RefHandle *)hv)->cells.size(); }

// Per-cell parameter override by name (absolute value), ElphyModelBasis.h:319-322.
int ref_add_hetero(void *hv, const char *name, const double *values) {
  auto *h = (RefHandle *)hv;
  try {
    for (size_t i = 0; i < h->cells.size(); i++)
      if (!h->cells[i]->AddHeteroValue(name, values[i])) return -2;
  } catch (kaBaseException &e) {
    g_err = e.getText();
    return -1;
  }
  return 0;
}

int ref_state_doubles(void *hv) {
  auto *h = (RefHandle *)hv;
  return h->cells[0]->GetSize() / (int)sizeof(double);
}

void ref_get_state(void *hv, double *out) {
  auto *h = (RefHandle *)hv;
  int n = ref_state_doubles(hv);
  for (size_t i = 0; i < h->cells.size(); i++) memcpy(out + i * n, h->cells[i]->GetBase(), n * sizeof(double));
}

void ref_set_state(void *hv, const double *in) {
  auto *h = (RefHandle *)hv;
  int n = ref_state_doubles(hv);
  for (size_t i = 0; i < h->cells.size(); i++) memcpy(h->cells[i]->GetBase(), in + i * n, n * sizeof(double));
}

double ref_init_vm(void *hv) { return ((RefHandle *)hv)->cells[0]->GetVm(); }
double ref_amplitude(void *hv) { return ((RefHandle *)hv)->cells[0]->GetAmplitude(); }
double ref_stim_time(void *hv) { return ((RefHandle *)hv)->cells[0]->GetStimTime(); }

// One Calc per cell: dVm[i] = Calc(dt, Vm[i], i_ext[i], stretch, 1).
void ref_calc(void *hv, double dt, const double *Vm, const double *i_ext, double stretch, double *dVm) {
  auto *h = (RefHandle *)hv;
  for (size_t i = 0; i < h->cells.size(); i++) dVm[i] = h->cells[i]->Calc(dt, Vm[i], i_ext[i], stretch, 1);
}

// Driver loop: n_steps of `Vm += Calc(dt, Vm, i_ext(t), 1, 1)` for every cell, t starting
// at t0 and accumulated as t += dt. trace (optional) receives Vm before every
// rec_every-th step: trace[cell * n_rec + k], n_rec = ceil(n_steps / rec_every).
// n_threads > 1 splits the cells over std::threads (cells are independent).
int ref_run(void *hv, double *Vm, long n_steps, double dt, double t0, double textbegin, double textlen,
            double bcl, double amp, long rec_every, double *trace, int n_threads) {
  auto *h = (RefHandle *)hv;
  const long n = (long)h->cells.size();
  const long n_rec = rec_every > 0 ? (n_steps + rec_every - 1) / rec_every : 0;
  int bad = 0;
  auto work = [&](long lo, long hi) {
    for (long c = lo; c < hi; c++) {
      double t = t0, tb = textbegin, v = Vm[c];
      vbElphyModel<double> *pem = h->cells[c];
      for (long s = 0; s < n_steps; s++) {
        if (trace && rec_every > 0 && s % rec_every == 0) trace[c * n_rec + s / rec_every] = v;
        const double i_ext = stim_current(t, tb, textlen, bcl, amp);
        v += pem->Calc(dt, v, i_ext, 1.0, 1);
        t += dt;
      }
      if (std::isnan(v)) bad = 1;
      Vm[c] = v;
    }
  };
  if (n_threads <= 1) {
    work(0, n);
  } else {
    std::vector<std::thread> th;
    for (int k = 0; k < n_threads; k++) {
      long lo = n * k / n_threads, hi = n * (k + 1) / n_threads;
      th.emplace_back(work, lo, hi);
    }
    for (auto &x : th) x.join();
  }
  return bad ? -3 : 0;
}

// Parameter dump (after Init + Calculate): names and values of P[0 .. vtLast).
int ref_n_params(void *hv) {
  auto *h = (RefHandle *)hv;
  auto *p = dynamic_cast<vbNewElphyParameters *>(h->pep);
  if (!p) return -1;
  int n = 0;
  // vtLast is model specific; walk until an empty name.
  switch (h->emt) {
    case EMT_TenTusscher2: n = NS_TenTusscher2Parameters::vtLast; break;
    case EMT_CourtemancheEtAl: n = NS_CourtemancheParameters::vtLast; break;
    case EMT_OHaraRudy: n = NS_OHaraRudyParameters::vtLast; break;
    case EMT_Tomek: n = NS_TomekParameters::vtLast; break;
    default: return -1;
  }
  return n;
}

const char *ref_param_name(void *hv, int i) {
  auto *p = dynamic_cast<vbNewElphyParameters *>(((RefHandle *)hv)->pep);
  return p->P[i].name.c_str();
}

double ref_param_value(void *hv, int i) {
  auto *p = dynamic_cast<vbNewElphyParameters *>(((RefHandle *)hv)->pep);
  return p->P[i].value;
}

// Copy one named lookup table (RTDT entries) out of the parameter object.
int ref_table(void *hv, const char *name, double *out) {
  auto *h = (RefHandle *)hv;
  const double *src = nullptr;
  std::string n(name);
  if (h->emt == EMT_TenTusscher2) {
    auto *p = (TenTusscher2Parameters *)h->pep;
#define T2(x) if (n == #x) src = p->x;
    T2(rec_ipK) T2(d_inf) T2(f_inf) T2(f2_inf) T2(m_inf) T2(h_inf) T2(j_inf) T2(Xr1_inf) T2(Xr2_inf)
    T2(Xs_inf) T2(r_inf) T2(s_inf) T2(NaCa_P1) T2(NaCa_P2) T2(NaK_P1) T2(CaL_P1) T2(CaL_P2)
    T2(exptau_m) T2(exptau_h) T2(exptau_j) T2(exptau_Xr1) T2(exptau_Xr2) T2(exptau_Xs) T2(exptau_s)
    T2(exptau_r) T2(exptau_d) T2(exptau_f) T2(exptau_f2) T2(ECA)
#undef T2
  } else if (h->emt == EMT_CourtemancheEtAl) {
    auto *p = (CourtemancheParameters *)h->pep;
#define T3(x) if (n == #x) src = p->x;
    T3(m_m) T3(exptau_m) T3(m_h) T3(exptau_h) T3(m_j) T3(exptau_j) T3(m_oa) T3(exptau_oa) T3(m_oi)
    T3(exptau_oi) T3(m_ua) T3(exptau_ua) T3(m_ui) T3(exptau_ui) T3(m_Xr) T3(exptau_Xr) T3(m_Xs)
    T3(exptau_Xs) T3(m_d) T3(exptau_d) T3(m_f) T3(exptau_f) T3(m_w) T3(exptau_w) T3(expVm) T3(CK1)
    T3(g_Kur) T3(CKr) T3(CNaK) T3(CNaCa)
#undef T3
    if (n == "exp250") { out[0] = p->exp250; return 1; }
    if (n == "exp50") { out[0] = p->exp50; return 1; }
  }
  if (!src) return -1;
  memcpy(out, src, RTDT * sizeof(double));
  return RTDT;
}

}  // extern "C"
