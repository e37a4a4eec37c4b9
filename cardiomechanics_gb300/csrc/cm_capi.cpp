// C ABI of libcmgb300.so (declared in include/cardiomech_gb300.h): handles, argument
// checking, host/device staging and dispatch to the kernels. No exception leaves this file.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "cm_handles.h"
#include "cm_multi.h"

using namespace cm;

std::string &cm::last_error() {
  thread_local std::string e;
  return e;
}

namespace {

int64_t round_ld(int64_t n) { return ((n + 255) / 256) * 256; }  // whole staged tiles

// SOA index (model order) -> plane of the mixed layout; `pair` variables are compensated
// accumulators stored as hi (plane slot) and lo (plane slot + 1).
void mixed_slot(int model, int k, bool &pair, int &slot) {
  if (model == kOHaraRudy) {
    slot = ord_mixed_plane(k, pair);
  } else if (model == kTomek) {
    slot = tom_mixed_plane(k, pair);
  } else if (model == kTenTusscher2) {
    // SOA: Ca_i CaSR CaSS Na_i K_i m h j xr1 xr2 xs r s d f f2 fCa Rq
    static const int map[] = {13, 15, 14, 17, 19, 0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12};
    slot = map[k];
    pair = k == 1 || k == 3 || k == 4;
  } else {
    // SOA: Ca_i Ca_up Ca_rel h j oi ui Xr Xs u v w Na_i K_i m oa ua d f f_Ca Ca_TRPN
    static const int map[] = {15, 17, 19, 0, 1, 2, 3, 4, 5, 6, 7, 8, 21, 23, 9, 10, 11, 12, 13, 14, 16};
    slot = map[k];
    pair = k == 1 || k == 2 || k == 12 || k == 13;
  }
}

// Reference backup block index of SOA variable k (TenTusscher2.h:77-123, CourtemancheEtAl.h:32-42,
// OHaraRudy.h:31-43: slot 4 is h_CaMK_fast, which the SOA layout leaves out; Tomek.h:33-44:
// slots 1, 2, 4, 5 are the rates A_h, B_h, A_j, B_j).
int ref_block_index(int model, int k) {
  if (model == kTenTusscher2) return k < 5 ? k : k + 18;
  if (model == kOHaraRudy) return k < 4 ? k : k + 1;
  if (model == kTomek) return k == 0 ? 0 : (k == 1 ? 3 : (k == 2 ? 6 : k + 4));
  return k < 20 ? k : 21;
}

// Device view of a caller array: the pointer itself if on the device, else a staged copy.
int stage_in(cm_batch_s *b, const double *p, int slot, const double **out) {
  if (!p) {
    *out = nullptr;
    return CM_OK;
  }
  if (is_device_ptr(p)) {
    *out = p;
    return CM_OK;
  }
  int rc = ensure_stage(b, b->d.n);
  if (rc) return rc;
  CK(cudaMemcpyAsync(b->stage[slot], p, b->d.n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  *out = b->stage[slot];
  return CM_OK;
}

int upload_tables(cm_batch_s *b) {
  if (b->table_mem) cudaFree(b->table_mem);
  b->table_mem = nullptr;
  if (b->d.precision == CM_PREC_FP64) {
    std::vector<double> rows, eca;
    b->ps.rows_fp64(rows, eca);
    size_t nb = (rows.size() + eca.size()) * sizeof(double);
    CK(cudaMalloc(&b->table_mem, std::max<size_t>(nb, 16)));
    double *dst = (double *)b->table_mem;
    if (!rows.empty()) CK(cudaMemcpy(dst, rows.data(), rows.size() * sizeof(double), cudaMemcpyHostToDevice));
    if (!eca.empty()) CK(cudaMemcpy(dst + rows.size(), eca.data(), eca.size() * sizeof(double), cudaMemcpyHostToDevice));
    b->d.rows64 = dst;
    b->d.eca64 = eca.empty() ? nullptr : dst + rows.size();
  } else {
    std::vector<float> rows, eca;
    b->ps.rows_fp32(rows, eca);
    size_t nb = (rows.size() + eca.size()) * sizeof(float);
    CK(cudaMalloc(&b->table_mem, std::max<size_t>(nb, 16)));
    float *dst = (float *)b->table_mem;
    if (!rows.empty()) CK(cudaMemcpy(dst, rows.data(), rows.size() * sizeof(float), cudaMemcpyHostToDevice));
    if (!eca.empty()) CK(cudaMemcpy(dst + rows.size(), eca.data(), eca.size() * sizeof(float), cudaMemcpyHostToDevice));
    b->d.rows32 = dst;
    b->d.eca32 = eca.empty() ? nullptr : dst + rows.size();
  }
  if (b->ps.spec->model == kTenTusscher2) b->ps.tt2_consts(b->d.tt2_64, b->d.tt2_32);
  else if (b->ps.spec->model == kOHaraRudy) b->ps.ord_consts(b->d.ord_64, b->d.ord_32);
  else if (b->ps.spec->model == kTomek) b->ps.tom_consts(b->d.tom_64, b->d.tom_32);
  else b->ps.crn_consts(b->d.crn_64, b->d.crn_32);
  return CM_OK;
}

// Diagnostic values an FP64 batch can record per cell, and where value k sits in the reference
// block: TT2 Array[0..16], CRN I_SAC, ORd its 17 stored currents, Tomek its 36 stored values
// (slots 48..83) and the four I_Na rates (slots 1, 2, 4, 5).
int diag_count(int model) { return model == kCourtemanche ? 1 : (model == kTomek ? kTOMDiag : 17); }
int diag_block_pos(int model, int k) {
  if (model == kTomek) {
    static const int rates[4] = {1, 2, 4, 5};
    return k < kTOMStored ? 48 + k : rates[k - kTOMStored];
  }
  return (model == kTenTusscher2 ? 5 : (model == kOHaraRudy ? 42 : 20)) + k;
}

// Host SOA (n_state x n, model order) <-> device layout.
int soa_to_device(cm_batch_s *b, const std::vector<double> &soa) {
  const int64_t n = b->d.n, ld = b->d.ld;
  const int ns = b->ps.spec->n_state;
  if (b->d.precision == CM_PREC_FP64) {
    for (int k = 0; k < ns; k++)
      CK(cudaMemcpyAsync(b->d.s64 + k * ld, soa.data() + (size_t)k * n, n * sizeof(double), cudaMemcpyHostToDevice,
                         b->stream));
    CK(cudaStreamSynchronize(b->stream));
    return CM_OK;
  }
  std::vector<float> f(n), g(n);
  for (int k = 0; k < ns; k++) {
    bool pair;
    int slot;
    mixed_slot(b->d.model, k, pair, slot);
    for (int64_t c = 0; c < n; c++) {
      const Acc a = acc_from_double(soa[(size_t)k * n + c]);
      f[c] = pair ? a.hi : (float)soa[(size_t)k * n + c];
      g[c] = a.lo;
    }
    CK(cudaMemcpy(b->d.s32 + slot * ld, f.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    if (pair) CK(cudaMemcpy(b->d.s32 + (slot + 1) * ld, g.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  }
  return CM_OK;
}

int device_to_soa(cm_batch_s *b, std::vector<double> &soa) {
  const int64_t n = b->d.n, ld = b->d.ld;
  const int ns = b->ps.spec->n_state;
  soa.assign((size_t)ns * n, 0.0);
  CK(cudaStreamSynchronize(b->stream));
  if (b->d.precision == CM_PREC_FP64) {
    for (int k = 0; k < ns; k++)
      CK(cudaMemcpy(soa.data() + (size_t)k * n, b->d.s64 + k * ld, n * sizeof(double), cudaMemcpyDeviceToHost));
    return CM_OK;
  }
  std::vector<float> f(n), g(n);
  for (int k = 0; k < ns; k++) {
    bool pair;
    int slot;
    mixed_slot(b->d.model, k, pair, slot);
    CK(cudaMemcpy(f.data(), b->d.s32 + slot * ld, n * sizeof(float), cudaMemcpyDeviceToHost));
    if (pair) CK(cudaMemcpy(g.data(), b->d.s32 + (slot + 1) * ld, n * sizeof(float), cudaMemcpyDeviceToHost));
    for (int64_t c = 0; c < n; c++) soa[(size_t)k * n + c] = pair ? acc_to_double(Acc{f[c], g[c]}) : (double)f[c];
  }
  return CM_OK;
}

void fill_info(const ParamSet &ps, cm_info *info) {
  info->model = ps.spec->model;
  info->n_state_vars = ps.spec->n_state;
  info->ref_block_doubles = ps.spec->ref_block_doubles;
  info->n_tables = ps.spec->n_tables;
  info->table_rows = kRows;
  info->dt = ps.dt;
  info->init_vm = ps.init_vm();
  info->amplitude = ps.amplitude();
  info->stim_time = ps.stim_time();
}

}  // namespace

extern "C" {

int cm_abi_version(void) { return CM_ABI_VERSION; }

const char *cm_last_error(void) { return cm::last_error().c_str(); }

int cm_model_from_name(const char *name) { return model_from_name(name); }

int cm_model_info(int model, cm_info *info) {
  const ModelSpec *s = find_model(model);
  if (!s) return fail(CM_ERR_MODEL, "model not implemented: " + std::to_string(model));
  if (!info) return fail(CM_ERR_ARG, "info is NULL");
  memset(info, 0, sizeof(*info));
  info->model = model;
  info->n_state_vars = s->n_state;
  info->ref_block_doubles = s->ref_block_doubles;
  info->n_tables = s->n_tables;
  info->table_rows = kRows;
  return CM_OK;
}

const char *cm_state_name(int model, int k) {
  const ModelSpec *s = find_model(model);
  if (!s || k < 0 || k >= s->n_state) return nullptr;
  return s->state_names[k];
}

int cm_params_create(cm_params_t *out, int model, const char *ev_path, double dt) {
  if (!out) return fail(CM_ERR_ARG, "out is NULL");
  *out = nullptr;
  auto *p = new (std::nothrow) cm_params_s();
  if (!p) return fail(CM_ERR_NOMEM, "host allocation failed");
  std::string err;
  int rc = p->ps.init(model, ev_path, dt, err);
  if (rc) {
    delete p;
    return fail(rc, err);
  }
  *out = p;
  return CM_OK;
}

int cm_params_destroy(cm_params_t p) {
  delete p;
  return CM_OK;
}

int cm_params_info(cm_params_t p, cm_info *info) {
  if (!p || !info) return fail(CM_ERR_ARG, "NULL argument");
  fill_info(p->ps, info);
  return CM_OK;
}

int cm_params_get(cm_params_t p, const char *name, double *value) {
  if (!p || !name || !value) return fail(CM_ERR_ARG, "NULL argument");
  int i = p->ps.index(name);
  if (i < 0) return fail(CM_ERR_PARAM, std::string("unknown parameter ") + name);
  *value = p->ps.vals[i];
  return CM_OK;
}

int cm_params_set(cm_params_t p, const char *name, double value) {
  if (!p || !name) return fail(CM_ERR_ARG, "NULL argument");
  int i = p->ps.index(name);
  if (i < 0) return fail(CM_ERR_PARAM, std::string("unknown parameter ") + name);
  if (i >= p->ps.spec->n_base) return fail(CM_ERR_PARAM, std::string(name) + " is derived; set its inputs");
  p->ps.vals[i] = value;
  p->ps.rebuild();
  return CM_OK;
}

int cm_params_table(cm_params_t p, const char *name, double *out) {
  if (!p || !name || !out) return fail(CM_ERR_ARG, "NULL argument");
  for (int k = 0; k < p->ps.spec->n_tables; k++)
    if (!strcmp(p->ps.spec->table_names[k], name)) {
      memcpy(out, p->ps.tables[k].data(), kRows * sizeof(double));
      return CM_OK;
    }
  if (p->ps.spec->model == kCourtemanche && (!strcmp(name, "exp250") || !strcmp(name, "exp50"))) {
    out[0] = !strcmp(name, "exp250") ? p->ps.exp250 : p->ps.exp50;
    return CM_OK;
  }
  return fail(CM_ERR_PARAM, std::string("unknown table ") + name);
}

int cm_batch_destroy(cm_batch_t b);

int cm_batch_create(cm_batch_t *out, cm_params_t p, int64_t n_cells, int precision, void *stream) {
  if (!out || !p) return fail(CM_ERR_ARG, "NULL argument");
  *out = nullptr;
  if (n_cells < 0) return fail(CM_ERR_ARG, "n_cells < 0");
  if (precision != CM_PREC_FP64 && precision != CM_PREC_MIXED) return fail(CM_ERR_ARG, "unknown precision");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(CM_ERR_CUDA, "no CUDA device: this library has no CPU path");
  }
  auto *b = new (std::nothrow) cm_batch_s();
  if (!b) return fail(CM_ERR_NOMEM, "host allocation failed");
  b->ps = p->ps;
  b->stream = (cudaStream_t)stream;
  b->d.model = p->ps.spec->model;
  b->d.precision = precision;
  b->d.n = n_cells;
  b->d.ld = round_ld(n_cells);
  const int64_t ld = b->d.ld;
  const size_t n64 = (size_t)n_fp64_vars(b->d.model, precision) * ld;
  const size_t n32 = precision == CM_PREC_MIXED ? (size_t)n_fp32_vars(b->d.model) * ld : 0;
  int rc = CM_OK;
  cudaError_t e = cudaMalloc(&b->state_mem, std::max<size_t>(1, n64 * sizeof(double) + n32 * sizeof(float)));
  if (e != cudaSuccess) rc = cuda_fail(e, "cudaMalloc(state)");
  if (!rc) {
    b->d.s64 = (double *)b->state_mem;
    b->d.s32 = precision == CM_PREC_MIXED ? (float *)(b->d.s64 + n64) : nullptr;
    e = cudaMalloc(&b->audit_cell, std::max<int64_t>(1, n_cells) * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->audit_or, sizeof(unsigned int));
    if (e != cudaSuccess) rc = cuda_fail(e, "cudaMalloc(audit)");
  }
  if (!rc) {
    b->d.audit_cell = b->audit_cell;
    b->d.audit_or = b->audit_or;
    rc = upload_tables(b);
  }
  if (!rc) rc = cm_batch_reset(b);
  if (rc) {
    std::string keep = cm::last_error();
    cm_batch_destroy(b);
    cm::last_error() = keep;
    return rc;
  }
  *out = b;
  return CM_OK;
}

int cm_batch_destroy(cm_batch_t b) {
  if (!b) return CM_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  else cudaDeviceSynchronize();
  cudaFree(b->state_mem);
  cudaFree(b->table_mem);
  for (auto p : b->het_mem) cudaFree(p);
  cudaFree(b->audit_cell);
  cudaFree(b->audit_or);
  cudaFree(b->diag);
  for (auto p : b->stage) cudaFree(p);
  cudaFree(b->tb_cell);
  cudaFree(b->vm_planes);
  cudaFree(b->vm_planes2);
  cudaFree(b->probe_idx);
  cudaFree(b->probe_out);
  delete b;
  return CM_OK;
}

int cm_batch_info(cm_batch_t b, cm_info *info, int64_t *n_cells, int *precision) {
  if (!b) return fail(CM_ERR_ARG, "NULL batch");
  if (info) fill_info(b->ps, info);
  if (n_cells) *n_cells = b->d.n;
  if (precision) *precision = b->d.precision;
  return CM_OK;
}

int cm_batch_reset(cm_batch_t b) {
  if (!b) return fail(CM_ERR_ARG, "NULL batch");
  std::vector<double> one;
  b->ps.init_state(one);
  const int64_t n = b->d.n;
  std::vector<double> soa((size_t)one.size() * n);
  for (size_t k = 0; k < one.size(); k++) std::fill(soa.begin() + k * n, soa.begin() + (k + 1) * n, one[k]);
  int rc = soa_to_device(b, soa);
  if (rc) return rc;
  CK(cudaMemsetAsync(b->audit_cell, 0, std::max<int64_t>(1, n) * sizeof(uint32_t), b->stream));
  CK(cudaMemsetAsync(b->audit_or, 0, sizeof(unsigned int), b->stream));
  if (b->diag) {
    const int nd = diag_count(b->d.model);
    CK(cudaMemsetAsync(b->diag, 0, (size_t)nd * b->d.ld * sizeof(double), b->stream));
  }
  CK(cudaStreamSynchronize(b->stream));
  return CM_OK;
}

int cm_batch_set_diagnostics(cm_batch_t b, int on) {
  if (!b) return fail(CM_ERR_ARG, "NULL batch");
  if (on && b->d.precision != CM_PREC_FP64) return fail(CM_ERR_UNSUPPORTED, "diagnostic currents need an FP64 batch");
  if (on && !b->diag) {
    const int nd = diag_count(b->d.model);
    CK(cudaMalloc(&b->diag, (size_t)nd * b->d.ld * sizeof(double)));
    CK(cudaMemset(b->diag, 0, (size_t)nd * b->d.ld * sizeof(double)));
  }
  b->diag_on = on != 0;
  b->d.diag = b->diag_on ? b->diag : nullptr;
  return CM_OK;
}

int cm_batch_set_hetero(cm_batch_t b, const char *name, const double *values) {
  if (!b || !name) return fail(CM_ERR_ARG, "NULL argument");
  int slot = -1;
  for (int k = 0; k < b->ps.spec->n_het; k++)
    if (!strcmp(b->ps.spec->het_names[k], name)) slot = k;
  if (slot < 0) {
    if (b->ps.index(name) < 0) return fail(CM_ERR_PARAM, std::string("unknown parameter ") + name);
    return fail(CM_ERR_UNSUPPORTED, std::string("per-cell values of ") + name + " are not supported");
  }
  if (!values) {
    cudaFree(b->het_mem[slot]);
    b->het_mem[slot] = nullptr;
    b->d.het[slot] = nullptr;
    return CM_OK;
  }
  const int64_t n = b->d.n;
  std::vector<double> host(n);
  if (is_device_ptr(values)) CK(cudaMemcpy(host.data(), values, n * sizeof(double), cudaMemcpyDeviceToHost));
  else memcpy(host.data(), values, n * sizeof(double));
  const size_t es = b->d.precision == CM_PREC_FP64 ? sizeof(double) : sizeof(float);
  if (!b->het_mem[slot]) {  // padded to ld: staged kernels copy whole tiles
    CK(cudaMalloc(&b->het_mem[slot], std::max<int64_t>(1, b->d.ld) * es));
    CK(cudaMemset(b->het_mem[slot], 0, std::max<int64_t>(1, b->d.ld) * es));
  }
  if (b->d.precision == CM_PREC_FP64) {
    CK(cudaMemcpy(b->het_mem[slot], host.data(), n * sizeof(double), cudaMemcpyHostToDevice));
  } else {
    std::vector<float> f(host.begin(), host.end());
    CK(cudaMemcpy(b->het_mem[slot], f.data(), n * sizeof(float), cudaMemcpyHostToDevice));
  }
  b->d.het[slot] = b->het_mem[slot];
  return CM_OK;
}

int cm_batch_init_vm(cm_batch_t b, double *Vm) {
  if (!b || !Vm) return fail(CM_ERR_ARG, "NULL argument");
  std::vector<double> v(b->d.n, b->ps.init_vm());
  if (is_device_ptr(Vm)) CK(cudaMemcpy(Vm, v.data(), b->d.n * sizeof(double), cudaMemcpyHostToDevice));
  else memcpy(Vm, v.data(), b->d.n * sizeof(double));
  return CM_OK;
}

int cm_batch_get_state(cm_batch_t b, int layout, double *buf) {
  if (!b || !buf) return fail(CM_ERR_ARG, "NULL argument");
  if (layout != CM_LAYOUT_SOA && layout != CM_LAYOUT_REF_BLOCK) return fail(CM_ERR_ARG, "unknown layout");
  std::vector<double> soa;
  int rc = device_to_soa(b, soa);
  if (rc) return rc;
  const int64_t n = b->d.n;
  const int ns = b->ps.spec->n_state, nb = b->ps.spec->ref_block_doubles;
  std::vector<double> out;
  if (layout == CM_LAYOUT_SOA) {
    out.swap(soa);
  } else {
    out.assign((size_t)nb * n, 0.0);
    for (int k = 0; k < ns; k++) {
      const int pos = ref_block_index(b->d.model, k);
      for (int64_t c = 0; c < n; c++) out[(size_t)c * nb + pos] = soa[(size_t)k * n + c];
    }
    if (b->diag) {  // diagnostic slots: TT2 Array[0..16], CRN I_SAC
      const int nd = diag_count(b->d.model);
      std::vector<double> dg((size_t)nd * n);
      for (int k = 0; k < nd; k++)
        CK(cudaMemcpy(dg.data() + (size_t)k * n, b->diag + k * b->d.ld, n * sizeof(double), cudaMemcpyDeviceToHost));
      for (int k = 0; k < nd; k++) {
        const int pos = diag_block_pos(b->d.model, k);
        for (int64_t c = 0; c < n; c++) out[(size_t)c * nb + pos] = dg[(size_t)k * n + c];
      }
    }
  }
  if (is_device_ptr(buf)) CK(cudaMemcpy(buf, out.data(), out.size() * sizeof(double), cudaMemcpyHostToDevice));
  else memcpy(buf, out.data(), out.size() * sizeof(double));
  return CM_OK;
}

int cm_batch_set_state(cm_batch_t b, int layout, const double *buf) {
  if (!b || !buf) return fail(CM_ERR_ARG, "NULL argument");
  if (layout != CM_LAYOUT_SOA && layout != CM_LAYOUT_REF_BLOCK) return fail(CM_ERR_ARG, "unknown layout");
  const int64_t n = b->d.n;
  const int ns = b->ps.spec->n_state, nb = b->ps.spec->ref_block_doubles;
  const size_t count = (size_t)(layout == CM_LAYOUT_SOA ? ns : nb) * n;
  std::vector<double> in(count);
  if (is_device_ptr(buf)) CK(cudaMemcpy(in.data(), buf, count * sizeof(double), cudaMemcpyDeviceToHost));
  else memcpy(in.data(), buf, count * sizeof(double));
  std::vector<double> soa;
  if (layout == CM_LAYOUT_SOA) {
    soa.swap(in);
  } else {
    soa.assign((size_t)ns * n, 0.0);
    for (int k = 0; k < ns; k++) {
      const int pos = ref_block_index(b->d.model, k);
      for (int64_t c = 0; c < n; c++) soa[(size_t)k * n + c] = in[(size_t)c * nb + pos];
    }
  }
  return soa_to_device(b, soa);
}

int cm_diag_batch_wait_check(void *batch, int64_t skip_tile, uint32_t spin_limit) {
  cm_batch_t b = (cm_batch_t)batch;
  if (!b) return fail(CM_ERR_ARG, "NULL batch");
  if (skip_tile < -1) return fail(CM_ERR_ARG, "skip_tile: a tile index or -1");
  b->d.fault_skip_tile = skip_tile;
  b->d.spin_limit = spin_limit ? spin_limit : (1u << 26);
  return CM_OK;
}

int cm_batch_get_cell(cm_batch_t b, int64_t cell, int layout, double *out) {
  if (!b || !out) return fail(CM_ERR_ARG, "NULL argument");
  if (layout != CM_LAYOUT_SOA && layout != CM_LAYOUT_REF_BLOCK) return fail(CM_ERR_ARG, "unknown layout");
  if (cell < 0 || cell >= b->d.n) return fail(CM_ERR_ARG, "cell index out of range");
  const int ns = b->ps.spec->n_state, nb = b->ps.spec->ref_block_doubles;
  const int64_t ld = b->d.ld;
  CK(cudaStreamSynchronize(b->stream));
  // the cell's column of every state plane in one strided copy
  std::vector<double> soa(ns);
  if (b->d.precision == CM_PREC_FP64) {
    CK(cudaMemcpy2D(soa.data(), sizeof(double), b->d.s64 + cell, ld * sizeof(double), sizeof(double), ns,
                    cudaMemcpyDeviceToHost));
  } else {
    const int nw = n_fp32_vars(b->d.model);
    std::vector<float> w(nw);
    CK(cudaMemcpy2D(w.data(), sizeof(float), b->d.s32 + cell, ld * sizeof(float), sizeof(float), nw,
                    cudaMemcpyDeviceToHost));
    for (int k = 0; k < ns; k++) {
      bool pair;
      int slot;
      mixed_slot(b->d.model, k, pair, slot);
      soa[k] = pair ? acc_to_double(Acc{w[slot], w[slot + 1]}) : (double)w[slot];
    }
  }
  if (layout == CM_LAYOUT_SOA) {
    memcpy(out, soa.data(), ns * sizeof(double));
    return CM_OK;
  }
  std::fill(out, out + nb, 0.0);
  for (int k = 0; k < ns; k++) out[ref_block_index(b->d.model, k)] = soa[k];
  if (b->diag) {
    const int nd = diag_count(b->d.model);
    std::vector<double> dg(nd);
    CK(cudaMemcpy2D(dg.data(), sizeof(double), b->diag + cell, ld * sizeof(double), sizeof(double), nd,
                    cudaMemcpyDeviceToHost));
    for (int k = 0; k < nd; k++) out[diag_block_pos(b->d.model, k)] = dg[k];
  }
  return CM_OK;
}

int cm_batch_set_cell(cm_batch_t b, int64_t cell, int layout, const double *in) {
  if (!b || !in) return fail(CM_ERR_ARG, "NULL argument");
  if (layout != CM_LAYOUT_SOA && layout != CM_LAYOUT_REF_BLOCK) return fail(CM_ERR_ARG, "unknown layout");
  if (cell < 0 || cell >= b->d.n) return fail(CM_ERR_ARG, "cell index out of range");
  const int ns = b->ps.spec->n_state;
  const int64_t ld = b->d.ld;
  std::vector<double> soa(ns);
  for (int k = 0; k < ns; k++) soa[k] = layout == CM_LAYOUT_SOA ? in[k] : in[ref_block_index(b->d.model, k)];
  CK(cudaStreamSynchronize(b->stream));
  if (b->d.precision == CM_PREC_FP64) {
    CK(cudaMemcpy2D(b->d.s64 + cell, ld * sizeof(double), soa.data(), sizeof(double), sizeof(double), ns,
                    cudaMemcpyHostToDevice));
    return CM_OK;
  }
  const int nw = n_fp32_vars(b->d.model);
  std::vector<float> w(nw, 0.f);
  for (int k = 0; k < ns; k++) {
    bool pair;
    int slot;
    mixed_slot(b->d.model, k, pair, slot);
    const Acc a = acc_from_double(soa[k]);
    w[slot] = pair ? a.hi : (float)soa[k];
    if (pair) w[slot + 1] = a.lo;
  }
  CK(cudaMemcpy2D(b->d.s32 + cell, ld * sizeof(float), w.data(), sizeof(float), sizeof(float), nw,
                  cudaMemcpyHostToDevice));
  return CM_OK;
}

int cm_batch_calc_cell(cm_batch_t b, int64_t cell, double dt, double V, double i_ext, double stretch, double *dV) {
  if (!b || !dV) return fail(CM_ERR_ARG, "NULL argument");
  if (cell < 0 || cell >= b->d.n) return fail(CM_ERR_ARG, "cell index out of range");
  if (dt != b->ps.dt)
    return fail(CM_ERR_ARG, "dt differs from the parameter set's dt (" + std::to_string(b->ps.dt) +
                                "): the lookup tables depend on dt; create a parameter set for this dt");
  int rc;
  if ((rc = ensure_stage(b, 4))) return rc;
  // the batch seen from this cell: every per-cell plane starts at the cell, one cell long
  DevBatch d = b->d;
  d.n = 1;
  const size_t het_word = d.precision == CM_PREC_FP64 ? sizeof(double) : sizeof(float);
  if (d.s64) d.s64 += cell;
  if (d.s32) d.s32 += cell;
  for (auto &h : d.het)
    if (h) h = (const char *)h + cell * het_word;
  if (d.audit_cell) d.audit_cell += cell;
  if (d.diag) d.diag += cell;
  const double io_in[3] = {V, i_ext, stretch};
  CK(cudaMemcpyAsync(b->stage[0], io_in, sizeof(io_in), cudaMemcpyHostToDevice, b->stream));
  StepIO io;
  io.vm = b->stage[0];
  io.iext = b->stage[0] + 1;
  io.stretch = b->stage[0] + 2;
  io.dvm = b->stage[0] + 3;
  CK(launch_step(d, io, 0, 0, b->stream));
  CK(cudaMemcpyAsync(dV, b->stage[0] + 3, sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  return CM_OK;
}

int cm_batch_step(cm_batch_t b, double dt, const double *Vm, const double *i_ext, const double *stretch, double *dVm) {
  if (!b || !Vm || !dVm) return fail(CM_ERR_ARG, "NULL argument");
  if (dt != b->ps.dt)
    return fail(CM_ERR_ARG, "dt differs from the parameter set's dt (" + std::to_string(b->ps.dt) +
                                "): the lookup tables depend on dt; create a parameter set for this dt");
  if (b->d.n == 0) return CM_OK;
  StepIO io;
  int rc;
  if ((rc = stage_in(b, Vm, 0, &io.vm))) return rc;
  if ((rc = stage_in(b, i_ext, 1, &io.iext))) return rc;
  if ((rc = stage_in(b, stretch, 2, &io.stretch))) return rc;
  const bool host_out = !is_device_ptr(dVm);
  if (host_out) {
    if ((rc = ensure_stage(b, b->d.n))) return rc;
    io.dvm = b->stage[3];
  } else {
    io.dvm = dVm;
  }
  CK(launch_step(b->d, io, b->d.variant, b->d.grid_mode, b->stream));
  if (host_out) {
    CK(cudaMemcpyAsync(dVm, io.dvm, b->d.n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
  }
  return CM_OK;
}

int cm_batch_step_update(cm_batch_t b, double dt, double *Vm, const double *i_ext, const double *stretch,
                         double vm_range) {
  return cm_batch_step_update_act(b, dt, Vm, i_ext, stretch, vm_range, nullptr, 0.0, 0.0);
}

int cm_batch_step_update_act(cm_batch_t b, double dt, double *Vm, const double *i_ext, const double *stretch,
                             double vm_range, double *act_time, double t, double act_threshold) {
  if (!b || !Vm) return fail(CM_ERR_ARG, "NULL argument");
  if (dt != b->ps.dt)
    return fail(CM_ERR_ARG, "dt differs from the parameter set's dt (" + std::to_string(b->ps.dt) +
                                "): the lookup tables depend on dt; create a parameter set for this dt");
  if (b->d.n == 0) return CM_OK;
  StepIO io;
  int rc;
  const bool host_vm = !is_device_ptr(Vm);
  const double *vin;
  if ((rc = stage_in(b, Vm, 0, &vin))) return rc;
  io.vm = vin;
  io.vm_out = const_cast<double *>(vin);
  io.vm_range = vm_range;
  if ((rc = stage_in(b, i_ext, 1, &io.iext))) return rc;
  if ((rc = stage_in(b, stretch, 2, &io.stretch))) return rc;
  const bool host_act = act_time && !is_device_ptr(act_time);
  if (act_time) {
    const double *ain;
    if ((rc = stage_in(b, act_time, 3, &ain))) return rc;
    io.act = const_cast<double *>(ain);
    io.act_time = t;
    io.act_threshold = act_threshold;
  }
  CK(launch_step(b->d, io, b->d.variant, b->d.grid_mode, b->stream));
  if (host_vm) CK(cudaMemcpyAsync(Vm, io.vm_out, b->d.n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  if (host_act) CK(cudaMemcpyAsync(act_time, io.act, b->d.n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  unsigned int mask = 0;
  CK(cudaMemcpyAsync(&mask, b->audit_or, sizeof(unsigned int), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  if (mask & (CM_AUDIT_NAN | CM_AUDIT_VMRANGE))
    return fail(CM_ERR_NUMERIC, "Vm is NaN, infinite or outside the allowed range in at least one cell");
  return CM_OK;
}

int cm_batch_run(cm_batch_t b, double *Vm, int64_t n_steps, const cm_stimulus *stim, const int64_t *probe_cells,
                 int64_t n_probe, int64_t probe_every, double *probe_vm) {
  if (!b || !Vm) return fail(CM_ERR_ARG, "NULL argument");
  if (n_steps < 0) return fail(CM_ERR_ARG, "n_steps < 0");
  if (n_probe > 0 && (!probe_cells || !probe_vm || probe_every <= 0))
    return fail(CM_ERR_ARG, "probes need probe_cells, probe_vm and probe_every > 0");
  const int64_t n = b->d.n;
  if (n == 0 || n_steps == 0) return CM_OK;
  int rc;
  const bool host_vm = !is_device_ptr(Vm);
  double *dvm = Vm;
  if (host_vm) {
    if ((rc = ensure_stage(b, n))) return rc;
    dvm = b->stage[0];
    CK(cudaMemcpyAsync(dvm, Vm, n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  }
  cm_stimulus st = {};
  if (stim) st = *stim;
  const bool per_cell = stim && stim->textbegin_per_cell;
  double *tb_cell = nullptr;
  if (per_cell && (rc = per_cell_times(b, stim->textbegin_per_cell, b->stream, &tb_cell))) return rc;
  const int64_t n_rec = n_probe > 0 ? (n_steps + probe_every - 1) / probe_every : 0;
  if (n_probe > 0) {
    for (int64_t i = 0; i < n_probe; i++)
      if (probe_cells[i] < 0 || probe_cells[i] >= n) return fail(CM_ERR_ARG, "probe cell index out of range");
    if (b->probe_cap < n_probe) {
      cudaFree(b->probe_idx);
      b->probe_idx = nullptr;
      b->probe_cap = 0;
      CK(cudaMalloc(&b->probe_idx, n_probe * sizeof(int64_t)));
      b->probe_cap = n_probe;
    }
    if (b->probe_out_cap < n_probe * n_rec) {
      cudaFree(b->probe_out);
      b->probe_out = nullptr;
      b->probe_out_cap = 0;
      CK(cudaMalloc(&b->probe_out, n_probe * n_rec * sizeof(double)));
      b->probe_out_cap = n_probe * n_rec;
    }
    CK(cudaMemcpyAsync(b->probe_idx, probe_cells, n_probe * sizeof(int64_t), cudaMemcpyHostToDevice, b->stream));
  }
  StepIO io;
  io.vm = dvm;
  io.vm_out = dvm;
  const bool planes = b->d.precision == CM_PREC_MIXED;
  if (planes) {
    if (!b->vm_planes) CK(cudaMalloc(&b->vm_planes, std::max<int64_t>(1, 2 * b->d.ld) * sizeof(float)));
    io.vm_hi = b->vm_planes;
    io.vm_lo = b->vm_planes + b->d.ld;
    io.vm = nullptr;
    io.vm_out = nullptr;
    CK(launch_vm_split(dvm, io.vm_hi, io.vm_lo, n, b->stream));
  }
  io.textlen = st.textlen;
  io.bcl = st.bcl;
  io.amp = st.amplitude;
  io.tb_cell = tb_cell;
  // The reference driver accumulates t += dt and advances textbegin on the host side of
  // each cell; with one protocol for all cells the same arithmetic runs here once per step.
  double t = st.t0, tb = st.textbegin;
  for (int64_t s = 0; s < n_steps; s++) {
    if (n_probe > 0 && s % probe_every == 0)
      CK(launch_probe(planes ? nullptr : dvm, io.vm_hi, io.vm_lo, b->probe_idx, n_probe, b->probe_out, n_rec,
                      s / probe_every, b->stream));
    io.t = t;
    if (!per_cell) {
      double i_ext = 0.0;
      if (stim && t >= tb) {
        i_ext = st.amplitude;
        if (t >= tb + st.textlen) tb += st.bcl;
      }
      io.iext_uniform = i_ext;
    }
    CK(launch_step(b->d, io, b->d.variant, b->d.grid_mode, b->stream));
    t += b->ps.dt;
  }
  if (planes) CK(launch_vm_join(io.vm_hi, io.vm_lo, dvm, n, b->stream));
  if (host_vm) CK(cudaMemcpyAsync(Vm, dvm, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  if (n_probe > 0) {
    const bool host_probe = !is_device_ptr(probe_vm);
    CK(cudaMemcpyAsync(probe_vm, b->probe_out, n_probe * n_rec * sizeof(double),
                       host_probe ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, b->stream));
  }
  unsigned int mask = 0;
  CK(cudaMemcpyAsync(&mask, b->audit_or, sizeof(unsigned int), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  if (mask & CM_AUDIT_NAN) return fail(CM_ERR_NUMERIC, "Vm is NaN or infinite in at least one cell");
  return CM_OK;
}

int cm_batch_set_launch(cm_batch_t b, int variant, int grid_mode) {
  if (!b) return fail(CM_ERR_ARG, "NULL batch");
  if (variant < 0 || variant >= n_shape_variants() || grid_mode < 0 || grid_mode > 64)
    return fail(CM_ERR_ARG, "launch shape out of range");
  b->d.variant = variant;
  b->d.grid_mode = grid_mode;
  return CM_OK;
}

int cm_batch_autotune(cm_batch_t b, int n_trial_steps, int *variant, double *ms_per_step) {
  if (!b) return fail(CM_ERR_ARG, "NULL batch");
  if (n_trial_steps < 1) n_trial_steps = 1;
  const int64_t n = b->d.n;
  if (n == 0 || b->d.precision == CM_PREC_FP64) {
    if (variant) *variant = 0;
    if (ms_per_step) *ms_per_step = 0;
    return CM_OK;
  }
  const size_t n64 = (size_t)n_fp64_vars(b->d.model, b->d.precision) * b->d.ld;
  const size_t n32 = (size_t)n_fp32_vars(b->d.model) * b->d.ld;
  const size_t bytes = n64 * sizeof(double) + n32 * sizeof(float);
  void *saved = nullptr;
  double *vm = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = CM_OK;
  float best = 1e30f;
  int best_v = 0, best_g = 0;
  unsigned int audit_saved = 0;
  // trial Vm: compensated planes (hi, lo) of the rest potential, 2 x n floats in n doubles
  const Acc a0 = acc_from_double(b->ps.init_vm());
  const int64_t ld = b->d.ld;
  std::vector<float> v0(2 * ld, a0.hi);
  std::fill(v0.begin() + ld, v0.end(), a0.lo);
  cudaError_t e = cudaMalloc(&saved, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&vm, 2 * ld * sizeof(float));
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaMemcpyAsync(saved, b->state_mem, bytes, cudaMemcpyDeviceToDevice, b->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&audit_saved, b->audit_or, sizeof(unsigned int), cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(vm, v0.data(), 2 * ld * sizeof(float), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  const int grid_modes[] = {0, 2, 4, 8};
  for (int v = 0; e == cudaSuccess && v < n_shape_variants(); v++) {
    for (int g : grid_modes) {
      DevBatch d = b->d;
      d.variant = v;
      d.grid_mode = g;
      StepIO io;
      io.vm_hi = (float *)vm;  // the trial Vm as compensated planes
      io.vm_lo = (float *)vm + ld;
      // the variants past the register shapes are the staged kernels; a batch they do not cover
      // would time shape 0
      if (v >= n_register_shapes() && !staged_supported(d, io)) continue;
      for (int k = 0; k < 2 && e == cudaSuccess; k++) e = launch_step(d, io, v, g, b->stream);
      if (e == cudaSuccess) e = cudaEventRecord(e0, b->stream);
      for (int k = 0; k < n_trial_steps && e == cudaSuccess; k++) e = launch_step(d, io, v, g, b->stream);
      if (e == cudaSuccess) e = cudaEventRecord(e1, b->stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e == cudaSuccess && ms < best) {
        best = ms;
        best_v = v;
        best_g = g;
      }
    }
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(b->state_mem, saved, bytes, cudaMemcpyDeviceToDevice, b->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->audit_or, &audit_saved, sizeof(unsigned int), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) rc = cuda_fail(e, "autotune");
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(saved);
  cudaFree(vm);
  if (rc) return rc;
  b->d.variant = best_v;
  b->d.grid_mode = best_g;
  if (variant) *variant = best_v * 100 + best_g;
  if (ms_per_step) *ms_per_step = best / n_trial_steps;
  return CM_OK;
}

int cm_batch_audit(cm_batch_t b, uint32_t *mask, uint32_t *per_cell) {
  if (!b) return fail(CM_ERR_ARG, "NULL batch");
  unsigned int m = 0;
  CK(cudaMemcpyAsync(&m, b->audit_or, sizeof(unsigned int), cudaMemcpyDeviceToHost, b->stream));
  if (per_cell && b->d.n > 0) {
    const bool dev = is_device_ptr(per_cell);
    CK(cudaMemcpyAsync(per_cell, b->audit_cell, b->d.n * sizeof(uint32_t),
                       dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, b->stream));
  }
  CK(cudaStreamSynchronize(b->stream));
  CK(cudaMemsetAsync(b->audit_cell, 0, std::max<int64_t>(1, b->d.n) * sizeof(uint32_t), b->stream));
  CK(cudaMemsetAsync(b->audit_or, 0, sizeof(unsigned int), b->stream));
  CK(cudaStreamSynchronize(b->stream));
  if (mask) *mask = m;
  return CM_OK;
}

// ------------------------------------------------------------------ batched form

}  // extern "C"

struct cm_multi_s {
  std::vector<cm_batch_t> batches;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  MultiInst *d_insts = nullptr;
  MultiTile *d_tiles = nullptr;
  MultiClock *d_clk = nullptr;
  unsigned int *d_counters = nullptr;
  std::vector<double *> vm_stage;   // host Vm staged as doubles
  std::vector<float *> vm_planes;   // every instance's Vm as hi/lo planes during a run
  std::vector<double *> vm_dev;     // device doubles of the current run (caller's or staged)
  int n_tiles = 0, tile_cells = 4096, shape = 0, blocks_per_sm = 2;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 32;
};

namespace {

void multi_drop_graph(cm_multi_s *m) {
  if (m->graph) cudaGraphExecDestroy(m->graph);
  m->graph = nullptr;
}

int multi_build_tiles(cm_multi_s *m, int tile_cells) {
  if (tile_cells < 32 || tile_cells > (1 << 24)) return fail(CM_ERR_ARG, "tile_cells out of range");
  std::vector<MultiTile> tiles;
  for (int i = 0; i < (int)m->batches.size(); i++) {
    const int64_t n = m->batches[i]->d.n;
    for (int64_t st = 0; st < n; st += tile_cells)
      tiles.push_back({i, (int)st, (int)std::min<int64_t>(tile_cells, n - st), 0});
  }
  cudaFree(m->d_tiles);
  m->d_tiles = nullptr;
  CK(cudaMalloc(&m->d_tiles, std::max<size_t>(1, tiles.size()) * sizeof(MultiTile)));
  if (!tiles.empty())
    CK(cudaMemcpy(m->d_tiles, tiles.data(), tiles.size() * sizeof(MultiTile), cudaMemcpyHostToDevice));
  m->n_tiles = (int)tiles.size();
  m->tile_cells = tile_cells;
  multi_drop_graph(m);
  return CM_OK;
}

MultiLaunch multi_launch_desc(const cm_multi_s *m) {
  MultiLaunch L;
  L.insts = m->d_insts;
  L.tiles = m->d_tiles;
  L.n_tiles = m->n_tiles;
  L.n_inst = (int)m->batches.size();
  L.clk = m->d_clk;
  L.counters = m->d_counters;
  L.shape = m->shape;
  L.grid = std::max(1, sm_count() * m->blocks_per_sm);
  L.tile_cells = m->tile_cells;
  return L;
}

// Uploads the instance table (Vm pointers, protocols) and the initial clocks.
int multi_prepare(cm_multi_s *m, double *const *Vm, const cm_stimulus *stims, std::vector<bool> &host_vm) {
  const int n = (int)m->batches.size();
  std::vector<MultiInst> insts(n);
  std::vector<MultiClock> clk(n);
  host_vm.assign(n, false);
  if ((int)m->vm_stage.size() < n) m->vm_stage.resize(n, nullptr);
  if ((int)m->vm_planes.size() < n) m->vm_planes.resize(n, nullptr);
  m->vm_dev.assign(n, nullptr);
  for (int i = 0; i < n; i++) {
    cm_batch_s *b = m->batches[i];
    insts[i].d = b->d;
    double *v = Vm[i];
    if (!v && b->d.n > 0) return fail(CM_ERR_ARG, "Vm[" + std::to_string(i) + "] is NULL");
    if (v && !is_device_ptr(v)) {
      host_vm[i] = true;
      if (!m->vm_stage[i]) CK(cudaMalloc(&m->vm_stage[i], std::max<int64_t>(1, b->d.n) * sizeof(double)));
      CK(cudaMemcpyAsync(m->vm_stage[i], v, b->d.n * sizeof(double), cudaMemcpyHostToDevice, m->stream));
      v = m->vm_stage[i];
    }
    if (!m->vm_planes[i]) CK(cudaMalloc(&m->vm_planes[i], std::max<int64_t>(1, 2 * b->d.ld) * sizeof(float)));
    insts[i].vm_hi = m->vm_planes[i];
    insts[i].vm_lo = m->vm_planes[i] + b->d.ld;
    m->vm_dev[i] = v;
    if (v) CK(launch_vm_split(v, insts[i].vm_hi, insts[i].vm_lo, b->d.n, m->stream));
    const cm_stimulus st = stims ? stims[i] : cm_stimulus{0, 0, nullptr, 0, 0, 0};
    if (st.textbegin_per_cell) return fail(CM_ERR_UNSUPPORTED, "per-cell stimulus times are not supported in a multi");
    insts[i].textlen = st.textlen;
    insts[i].bcl = st.bcl;
    insts[i].amp = stims ? st.amplitude : 0.0;
    insts[i].dt = b->ps.dt;
    clk[i].t = st.t0;
    clk[i].tb = stims ? st.textbegin : 1e300;
  }
  CK(cudaMemcpyAsync(m->d_insts, insts.data(), n * sizeof(MultiInst), cudaMemcpyHostToDevice, m->stream));
  CK(cudaMemcpyAsync(m->d_clk, clk.data(), n * sizeof(MultiClock), cudaMemcpyHostToDevice, m->stream));
  CK(cudaMemsetAsync(m->d_counters, 0, 2 * sizeof(unsigned int), m->stream));
  return CM_OK;
}

int multi_steps(cm_multi_s *m, int64_t n_steps, bool use_graph) {
  const MultiLaunch L = multi_launch_desc(m);
  int64_t s = 0;
  if (use_graph && n_steps >= m->graph_steps) {
    if (!m->graph) {
      cudaGraph_t g;
      CK(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
      for (int k = 0; k < m->graph_steps; k++) {
        cudaError_t e = launch_multi(L, k & 1, m->stream);
        if (e != cudaSuccess) {
          cudaStreamEndCapture(m->stream, &g);
          return cuda_fail(e, "launch_multi (capture)");
        }
      }
      CK(cudaStreamEndCapture(m->stream, &g));
      cudaError_t e = cudaGraphInstantiate(&m->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    }
    for (; s + m->graph_steps <= n_steps; s += m->graph_steps) CK(cudaGraphLaunch(m->graph, m->stream));
  }
  for (; s < n_steps; s++) CK(launch_multi(L, (int)(s & 1), m->stream));
  return CM_OK;
}

}  // namespace

extern "C" {

int cm_multi_destroy(cm_multi_t m) {
  if (!m) return CM_OK;
  cudaStreamSynchronize(m->stream);
  multi_drop_graph(m);
  cudaFree(m->d_insts);
  cudaFree(m->d_tiles);
  cudaFree(m->d_clk);
  cudaFree(m->d_counters);
  for (auto p : m->vm_stage) cudaFree(p);
  for (auto p : m->vm_planes) cudaFree(p);
  if (m->own_stream) cudaStreamDestroy(m->stream);
  delete m;
  return CM_OK;
}

int cm_multi_create(cm_multi_t *out, const cm_batch_t *batches, int n_batches, void *stream) {
  if (!out || !batches || n_batches <= 0) return fail(CM_ERR_ARG, "need at least one batch");
  *out = nullptr;
  for (int i = 0; i < n_batches; i++) {
    if (!batches[i]) return fail(CM_ERR_ARG, "NULL batch");
    if (batches[i]->d.precision != CM_PREC_MIXED)
      return fail(CM_ERR_UNSUPPORTED, "the batched form runs CM_PREC_MIXED batches");
    if (batches[i]->d.model == kOHaraRudy || batches[i]->d.model == kTomek)
      return fail(CM_ERR_UNSUPPORTED, "the batched form covers TenTusscher2 and CourtemancheEtAl batches");
    if (batches[i]->d.ld * 24 >= (int64_t)2147483647) return fail(CM_ERR_ARG, "instance too large for a multi");
  }
  auto *m = new (std::nothrow) cm_multi_s();
  if (!m) return fail(CM_ERR_NOMEM, "host allocation failed");
  m->batches.assign(batches, batches + n_batches);
  int rc = CM_OK;
  cudaError_t e = cudaSuccess;
  if (stream) {
    m->stream = (cudaStream_t)stream;
  } else {
    e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);  // capturable
    m->own_stream = e == cudaSuccess;
  }
  if (e == cudaSuccess) e = cudaMalloc(&m->d_insts, n_batches * sizeof(MultiInst));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_clk, 2 * n_batches * sizeof(MultiClock));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_counters, 2 * sizeof(unsigned int));
  if (e != cudaSuccess) rc = cuda_fail(e, "cm_multi_create");
  if (!rc) rc = multi_build_tiles(m, m->tile_cells);
  if (rc) {
    std::string keep = cm::last_error();
    cm_multi_destroy(m);
    cm::last_error() = keep;
    return rc;
  }
  *out = m;
  return CM_OK;
}

int cm_multi_set_launch(cm_multi_t m, int tile_cells, int shape, int blocks_per_sm) {
  if (!m) return fail(CM_ERR_ARG, "NULL multi");
  if (shape < 0 || shape >= n_multi_shapes() || blocks_per_sm < 1 || blocks_per_sm > 32)
    return fail(CM_ERR_ARG, "launch shape out of range");
  if (tile_cells != m->tile_cells) {
    int rc = multi_build_tiles(m, tile_cells);
    if (rc) return rc;
  }
  if (shape != m->shape || blocks_per_sm != m->blocks_per_sm) multi_drop_graph(m);
  m->shape = shape;
  m->blocks_per_sm = blocks_per_sm;
  return CM_OK;
}

int cm_multi_run(cm_multi_t m, double *const *Vm, int64_t n_steps, const cm_stimulus *stims) {
  if (!m || !Vm) return fail(CM_ERR_ARG, "NULL argument");
  if (n_steps < 0) return fail(CM_ERR_ARG, "n_steps < 0");
  std::vector<bool> host_vm;
  int rc = multi_prepare(m, Vm, stims, host_vm);
  if (rc) return rc;
  if ((rc = multi_steps(m, n_steps, true))) return rc;
  unsigned int mask = 0;
  std::vector<unsigned int> masks(m->batches.size(), 0);
  for (size_t i = 0; i < m->batches.size(); i++) {
    const int64_t ni = m->batches[i]->d.n;
    CK(launch_vm_join(m->vm_planes[i], m->vm_planes[i] + m->batches[i]->d.ld, m->vm_dev[i], ni, m->stream));
    if (host_vm[i])
      CK(cudaMemcpyAsync(Vm[i], m->vm_stage[i], m->batches[i]->d.n * sizeof(double), cudaMemcpyDeviceToHost,
                         m->stream));
    CK(cudaMemcpyAsync(&masks[i], m->batches[i]->audit_or, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                       m->stream));
  }
  CK(cudaStreamSynchronize(m->stream));
  for (auto x : masks) mask |= x;
  if (mask & CM_AUDIT_NAN) return fail(CM_ERR_NUMERIC, "Vm is NaN or infinite in at least one cell");
  return CM_OK;
}

int cm_multi_autotune(cm_multi_t m, int n_trial_steps, int *tile_cells, int *shape, int *blocks_per_sm,
                      double *ms_per_step) {
  if (!m) return fail(CM_ERR_ARG, "NULL multi");
  if (n_trial_steps < 1) n_trial_steps = 1;
  const int n = (int)m->batches.size();
  // save every instance's state and audit word; trial Vm starts from each model's rest value
  std::vector<void *> saved(n, nullptr);
  std::vector<size_t> bytes(n, 0);
  std::vector<unsigned int> audit(n, 0);
  std::vector<double *> vms(n, nullptr);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (int i = 0; i < n && e == cudaSuccess; i++) {
    cm_batch_s *b = m->batches[i];
    bytes[i] = (size_t)n_fp64_vars(b->d.model, b->d.precision) * b->d.ld * sizeof(double) +
               (size_t)n_fp32_vars(b->d.model) * b->d.ld * sizeof(float);
    e = cudaMalloc(&saved[i], bytes[i]);
    if (e == cudaSuccess) e = cudaMemcpyAsync(saved[i], b->state_mem, bytes[i], cudaMemcpyDeviceToDevice, m->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&audit[i], b->audit_or, sizeof(unsigned int), cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaMalloc(&vms[i], std::max<int64_t>(1, b->d.n) * sizeof(double));
    if (e == cudaSuccess) {
      std::vector<double> v0(b->d.n, b->ps.init_vm());
      e = cudaMemcpy(vms[i], v0.data(), b->d.n * sizeof(double), cudaMemcpyHostToDevice);
    }
  }
  const int old_tile = m->tile_cells, old_shape = m->shape, old_bps = m->blocks_per_sm;
  float best = 1e30f;
  int bt = old_tile, bs = old_shape, bb = old_bps;
  int rc = CM_OK;
  if (e != cudaSuccess) rc = cuda_fail(e, "multi autotune setup");
  std::vector<bool> host_vm;
  const int tiles[] = {1024, 2048, 4096, 8192, 16384};
  const int bpss[] = {1, 2, 4, 8};
  for (int t : tiles) {
    if (rc) break;
    if ((rc = multi_build_tiles(m, t))) break;
    for (int sh = 0; sh < n_multi_shapes() && !rc; sh++) {
      for (int bps : bpss) {
        if (multi_block(sh) * bps > 2048) continue;
        m->shape = sh;
        m->blocks_per_sm = bps;
        if ((rc = multi_prepare(m, vms.data(), nullptr, host_vm))) break;
        if ((rc = multi_steps(m, 2, false))) break;
        cudaEventRecord(e0, m->stream);
        if ((rc = multi_steps(m, n_trial_steps, false))) break;
        cudaEventRecord(e1, m->stream);
        e = cudaEventSynchronize(e1);
        float ms = 0;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e != cudaSuccess) {
          rc = cuda_fail(e, "multi autotune");
          break;
        }
        if (ms < best) {
          best = ms;
          bt = t;
          bs = sh;
          bb = bps;
        }
      }
    }
  }
  for (int i = 0; i < n; i++) {
    if (saved[i]) {
      cudaMemcpyAsync(m->batches[i]->state_mem, saved[i], bytes[i], cudaMemcpyDeviceToDevice, m->stream);
      cudaMemcpyAsync(m->batches[i]->audit_or, &audit[i], sizeof(unsigned int), cudaMemcpyHostToDevice, m->stream);
    }
  }
  cudaStreamSynchronize(m->stream);
  for (int i = 0; i < n; i++) {
    cudaFree(saved[i]);
    cudaFree(vms[i]);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (!rc) rc = multi_build_tiles(m, bt);
  if (rc) return rc;
  m->shape = bs;
  m->blocks_per_sm = bb;
  multi_drop_graph(m);
  if (tile_cells) *tile_cells = bt;
  if (shape) *shape = bs;
  if (blocks_per_sm) *blocks_per_sm = bb;
  if (ms_per_step) *ms_per_step = best / n_trial_steps;
  return CM_OK;
}

}  // extern "C"
