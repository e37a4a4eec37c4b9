// C ABI of the learned macro step: the MLP handle and the surrogate (training-data generation
// with the plain integrator, fitting, surrogate runs). See cm_surrogate.h for the method.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "cm_handles.h"
#include "cm_mlp.h"
#include "cm_noalloc.h"
#include "cm_surrogate.h"

using namespace cm;

struct cm_mlp_s {
  Mlp m;
  int device = -1;  // the device the network's memory lives on (current at creation)
};

struct cm_surrogate_s {
  ParamSet fine, coarse_ps;
  int substeps = 10;
  cudaStream_t stream = nullptr;
  TT2Consts<float> coarse{};
  float *rows_coarse = nullptr, *eca = nullptr;
  // FP64 constants and tables of the fine step (the audit sample integrated in FP64)
  TT2Consts<double> fine64{};
  double *rows_fine64 = nullptr, *eca_fine64 = nullptr;
  cm_mlp_s net;
  SurNorm norm{};
  bool fitted = false;
  // dataset (raw and normalised)
  float *dX = nullptr, *dT = nullptr, *nX = nullptr, *nT = nullptr;
  int64_t cap = 0;
  unsigned long long *d_count = nullptr;
  // generation scratch
  float *gX = nullptr, *gC = nullptr, *gOld = nullptr, *gT = nullptr;
  uint8_t *gkeep = nullptr;
  int64_t *gchunk = nullptr;  // per-chunk counts, then offsets, of the ordered append
  int64_t gcap = 0;
  // run scratch
  int *fallback = nullptr;
  int64_t rcap = 0;
  // audit: two snapshot buffers (even / odd macro steps) and their counters; the macro step k
  // writes buffer k % 2 and audits buffer (k - 1) % 2
  float *snap = nullptr;
  unsigned int *n_snap = nullptr;
  int64_t snap_cap = 0;
  int pending = -1;  // buffer holding the last macro step's sample, not audited yet (-1: none)
  // FP32 constants and tables of the fine step (the mixed-form audit)
  TT2Consts<float> fine32{};
  float *rows_fine32 = nullptr, *eca_fine32 = nullptr;
  // the run's counters in one 32-byte device block (one memset clears them, one copy reads them):
  // totals = n_sur, n_fallback_total, n_audit; then the largest audit error and the macro step's
  // fallback count (the fallback kernel's list length)
  unsigned long long *totals = nullptr;
  float *audit_err = nullptr;          // in the block, after totals
  unsigned int *n_fallback = nullptr;  // in the block, after audit_err
  bool counters_zeroed = false;        // the block was cleared at the end of the last run
  unsigned long long *host_res = nullptr;  // page-locked: the block and the batch's audit mask
  float *bias_block = nullptr;  // b1 | b2 | b3 of the network, contiguous (the inference kernel's layout)
  uint64_t bias_version = ~0ull;  // the network's weight version bias_block was copied from
  std::vector<cudaEvent_t> ev;  // 3 per macro step of a chunk: kernel timing of runs
};

namespace {

constexpr size_t kCounterBytes = 4 * sizeof(unsigned long long);

// unpadded <-> padded parameter blocks of an Mlp
void unpadded_sizes(const Mlp &m, size_t sz[6]) {
  sz[0] = (size_t)m.H * m.n_in;
  sz[1] = m.H;
  sz[2] = (size_t)m.H * m.H;
  sz[3] = m.H;
  sz[4] = (size_t)m.n_out * m.H;
  sz[5] = m.n_out;
}

int64_t n_unpadded(const Mlp &m) {
  size_t sz[6];
  unpadded_sizes(m, sz);
  int64_t n = 0;
  for (size_t x : sz) n += (int64_t)x;
  return n;
}

// copies between the unpadded host layout and the padded device block (FP32)
int mlp_copy(Mlp &m, float *dev_block, float *host, bool to_host) {
  std::vector<float> pad(m.n_params, 0.f);
  if (!to_host) {
    CK(cudaMemcpy(pad.data(), dev_block, m.n_params * sizeof(float), cudaMemcpyDeviceToHost));  // keep padding
  } else {
    CK(cudaStreamSynchronize(m.stream));
    CK(cudaMemcpy(pad.data(), dev_block, m.n_params * sizeof(float), cudaMemcpyDeviceToHost));
  }
  size_t k = 0;
  auto blk = [&](int b, int rows, int cols, int ldp) {
    for (int r = 0; r < rows; r++)
      for (int c = 0; c < cols; c++, k++) {
        float &p = pad[m.off[b] + (size_t)r * ldp + c];
        if (to_host) host[k] = p;
        else p = host[k];
      }
  };
  blk(0, m.H, m.n_in, m.in_pad);
  blk(1, 1, m.H, m.H);
  blk(2, m.H, m.H, m.H);
  blk(3, 1, m.H, m.H);
  blk(4, m.n_out, m.H, m.H);
  blk(5, 1, m.n_out, m.out_pad);
  if (!to_host) CK(cudaMemcpy(dev_block, pad.data(), m.n_params * sizeof(float), cudaMemcpyHostToDevice));
  return CM_OK;
}

// host view of an array that may live on the device
int fetch(const float *p, size_t n, std::vector<float> &out) {
  out.resize(n);
  if (is_device_ptr(p)) CK(cudaMemcpy(out.data(), p, n * sizeof(float), cudaMemcpyDeviceToHost));
  else memcpy(out.data(), p, n * sizeof(float));
  return CM_OK;
}

// device copy of a caller array (returns the caller's pointer if already on the device)
int to_device(const float *p, size_t n, const float **dev, float **owned) {
  *owned = nullptr;
  if (is_device_ptr(p)) {
    *dev = p;
    return CM_OK;
  }
  CK(cudaMalloc(owned, std::max<size_t>(1, n) * sizeof(float)));
  CK(cudaMemcpy(*owned, p, n * sizeof(float), cudaMemcpyHostToDevice));
  *dev = *owned;
  return CM_OK;
}

// The reference driver's stimulus for `steps` fine steps from (t, tb), advancing them.
bool protocol_steps(const cm_stimulus *st, int steps, double dt, double &t, double &tb, float *iext) {
  bool on = false;
  for (int k = 0; k < steps; k++) {
    double i = 0.0;
    if (st && t >= tb) {
      i = st->amplitude;
      if (t >= tb + st->textlen) tb += st->bcl;
    }
    iext[k] = (float)i;
    on = on || i != 0.0;
    t += dt;
  }
  return on;
}

int check_batch(cm_batch_s *b) {
  if (!b) return fail(CM_ERR_ARG, "NULL batch");
  if (b->d.model != kTenTusscher2 || b->d.precision != CM_PREC_MIXED)
    return fail(CM_ERR_UNSUPPORTED, "the surrogate runs MIXED TenTusscher2 batches");
  if (b->d.n >= ((int64_t)1 << 31) / 24) return fail(CM_ERR_ARG, "batch too large for the surrogate");
  return CM_OK;
}

// Vm planes of a batch for a run: split from the caller's doubles. Page-locked host memory is
// read (and later written) by the split/join kernels themselves over the host link; other host
// memory goes through a staging copy.
int planes_in(cm_batch_s *b, double *Vm, double **dvm, bool &host_vm, cudaStream_t s) {
  const int64_t n = b->d.n;
  host_vm = !is_device_ptr(Vm);
  *dvm = Vm;
  double *mapped = host_vm ? mapped_host_ptr(Vm) : nullptr;
  if (mapped) {
    host_vm = false;  // the kernels reach it: no copy back either
    *dvm = mapped;
  } else if (host_vm) {
    if (b->stage_n < n) {
      for (auto &p : b->stage) {
        cudaFree(p);
        p = nullptr;
      }
      b->stage_n = 0;
      for (auto &p : b->stage) CK(cudaMalloc(&p, std::max<int64_t>(1, n) * sizeof(double)));
      b->stage_n = n;
    }
    *dvm = b->stage[0];
    CK(cudaMemcpyAsync(*dvm, Vm, n * sizeof(double), cudaMemcpyHostToDevice, s));
  }
  if (!b->vm_planes) CK(cudaMalloc(&b->vm_planes, std::max<int64_t>(1, 2 * b->d.ld) * sizeof(float)));
  CK(launch_vm_split(*dvm, b->vm_planes, b->vm_planes + b->d.ld, n, s));
  return CM_OK;
}

int planes_out(cm_batch_s *b, double *Vm, double *dvm, bool host_vm, cudaStream_t s) {
  const int64_t n = b->d.n;
  CK(launch_vm_join(b->vm_planes, b->vm_planes + b->d.ld, dvm, n, s));
  if (host_vm) CK(cudaMemcpyAsync(Vm, dvm, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  return CM_OK;
}

// The caller's Vm as the macro-step kernels take it: page-locked host memory directly (the
// kernels read and write each cell's FP64 Vm once per macro step over the host link: no split and
// join kernel per call); device memory, and other host memory through a staging copy, as the
// device planes of the compensated pair (split once per call, joined by vm_out).
int vm_in(cm_batch_s *b, double *Vm, double **direct, double **dvm, bool &host_vm, cudaStream_t s) {
  *direct = nullptr;
  if (!is_device_ptr(Vm)) {
    if (double *mapped = mapped_host_ptr(Vm)) {
      *direct = mapped;
      *dvm = mapped;
      host_vm = false;
      return CM_OK;
    }
  }
  return planes_in(b, Vm, dvm, host_vm, s);
}

int vm_out(cm_batch_s *b, double *Vm, double *dvm, const double *direct, bool host_vm, cudaStream_t s) {
  if (direct) return CM_OK;
  return planes_out(b, Vm, dvm, host_vm, s);
}

// The audit of one snapshot buffer (its entries, FP64 or mixed), as the kernels take it.
SurAuditArgs audit_args(const cm_surrogate_s *s, int buf, bool fp64) {
  SurAuditArgs aa{};
  aa.snap = s->snap + (size_t)buf * kSnapPlanes * s->snap_cap;
  aa.n_snap = s->n_snap + buf;
  aa.snap_cap = (int)s->snap_cap;
  aa.substeps = s->substeps;
  aa.fp64 = fp64 ? 1 : 0;
  aa.c64 = s->fine64;
  aa.rows64 = s->rows_fine64;
  aa.eca64 = s->eca_fine64;
  aa.c32 = s->fine32;
  aa.rows32 = s->rows_fine32;
  aa.eca32 = s->eca_fine32;
  aa.audit_err = s->audit_err;
  aa.n_audit = s->totals + 2;
  return aa;
}

// Audits the pending sample on its own (a kernel of its own) and clears it.
int flush_pending(cm_surrogate_s *s, bool fp64, cudaStream_t st) {
  if (s->pending < 0) return CM_OK;
  CK(launch_sur_audit(audit_args(s, s->pending, fp64), st));
  CK(cudaMemsetAsync(s->n_snap + s->pending, 0, sizeof(unsigned int), st));
  s->pending = -1;
  return CM_OK;
}

}  // namespace

extern "C" {

// ------------------------------------------------------------------ MLP

int cm_mlp_create(cm_mlp_t *out, int n_in, int n_hidden, int n_out, uint64_t seed, void *stream) {
  if (!out || n_in < 1 || n_in > 256 || n_hidden < 64 || n_hidden % 64 || n_out < 1 || n_out > 256)
    return fail(CM_ERR_ARG, "MLP sizes: n_in, n_out in [1, 256], n_hidden a positive multiple of 64");
  *out = nullptr;
  auto *m = new (std::nothrow) cm_mlp_s();
  if (!m) return fail(CM_ERR_NOMEM, "host allocation failed");
  cudaError_t e = cudaGetDevice(&m->device);
  if (e == cudaSuccess) e = m->m.init(n_in, n_hidden, n_out, seed, (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) {
    m->m.release();
    delete m;
    return cuda_fail(e, "cm_mlp_create");
  }
  *out = m;
  return CM_OK;
}

int cm_mlp_destroy(cm_mlp_t m) {
  if (!m) return CM_OK;
  cudaStreamSynchronize(m->m.stream);
  m->m.release();
  delete m;
  return CM_OK;
}

int64_t cm_mlp_n_params(cm_mlp_t m) { return m ? n_unpadded(m->m) : -1; }

int cm_mlp_get_params(cm_mlp_t m, float *params) {
  if (!m || !params) return fail(CM_ERR_ARG, "NULL argument");
  std::vector<float> h(n_unpadded(m->m));
  int rc = mlp_copy(m->m, m->m.w, h.data(), true);
  if (rc) return rc;
  if (is_device_ptr(params)) CK(cudaMemcpy(params, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
  else memcpy(params, h.data(), h.size() * sizeof(float));
  return CM_OK;
}

int cm_mlp_set_params(cm_mlp_t m, const float *params) {
  if (!m || !params) return fail(CM_ERR_ARG, "NULL argument");
  std::vector<float> h;
  int rc = fetch(params, n_unpadded(m->m), h);
  if (rc) return rc;
  CK(cudaStreamSynchronize(m->m.stream));
  if ((rc = mlp_copy(m->m, m->m.w, h.data(), false))) return rc;
  CK(m->m.sync_bf16());
  CK(cudaStreamSynchronize(m->m.stream));
  return CM_OK;
}

int cm_mlp_get_grads(cm_mlp_t m, float *grads) {
  if (!m || !grads) return fail(CM_ERR_ARG, "NULL argument");
  std::vector<float> h(n_unpadded(m->m));
  int rc = mlp_copy(m->m, m->m.g, h.data(), true);
  if (rc) return rc;
  if (is_device_ptr(grads)) CK(cudaMemcpy(grads, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
  else memcpy(grads, h.data(), h.size() * sizeof(float));
  return CM_OK;
}

int cm_mlp_forward(cm_mlp_t m, const float *X, int64_t n, float *Y) {
  if (!m || !X || !Y || n < 0) return fail(CM_ERR_ARG, "bad argument");
  if (n == 0) return CM_OK;
  const float *dX;
  float *own = nullptr, *dY = Y;
  int rc = to_device(X, (size_t)n * m->m.n_in, &dX, &own);
  if (rc) return rc;
  const bool host_y = !is_device_ptr(Y);
  if (host_y) CK(cudaMalloc(&dY, (size_t)n * m->m.n_out * sizeof(float)));
  cudaError_t e = m->m.forward(dX, n, dY);
  if (e == cudaSuccess && host_y)
    e = cudaMemcpyAsync(Y, dY, (size_t)n * m->m.n_out * sizeof(float), cudaMemcpyDeviceToHost, m->m.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->m.stream);
  cudaFree(own);
  if (host_y) cudaFree(dY);
  return e == cudaSuccess ? CM_OK : cuda_fail(e, "cm_mlp_forward");
}

int cm_mlp_loss_grad(cm_mlp_t m, const float *X, const float *T, int64_t n, float *loss) {
  if (!m || !X || !T || n <= 0) return fail(CM_ERR_ARG, "bad argument");
  const float *dX, *dT;
  float *o1 = nullptr, *o2 = nullptr;
  int rc = to_device(X, (size_t)n * m->m.n_in, &dX, &o1);
  if (!rc) rc = to_device(T, (size_t)n * m->m.n_out, &dT, &o2);
  if (rc) {
    cudaFree(o1);
    return rc;
  }
  cudaError_t e = m->m.loss_grad(dX, dT, n);
  float l = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&l, m->m.loss, sizeof(float), cudaMemcpyDeviceToHost, m->m.stream);
  if (e == cudaSuccess) e = m->m.check_tc();
  cudaFree(o1);
  cudaFree(o2);
  if (e != cudaSuccess) return cuda_fail(e, "cm_mlp_loss_grad");
  if (loss) *loss = l;
  return CM_OK;
}

int cm_mlp_adam_step(cm_mlp_t m, float lr, float beta1, float beta2, float eps) {
  if (!m) return fail(CM_ERR_ARG, "NULL MLP");
  CK(m->m.adam_step(lr, beta1, beta2, eps));
  CK(cudaStreamSynchronize(m->m.stream));
  return CM_OK;
}

// ------------------------------------------------------------------ surrogate

int cm_surrogate_destroy(cm_surrogate_t s) {
  if (!s) return CM_OK;
  cudaStreamSynchronize(s->stream);
  for (cudaEvent_t e : s->ev) cudaEventDestroy(e);
  if (s->host_res) cudaFreeHost(s->host_res);
  s->net.m.release();
  for (void *p : {(void *)s->rows_coarse, (void *)s->eca, (void *)s->dX, (void *)s->dT, (void *)s->nX,
                  (void *)s->nT, (void *)s->d_count, (void *)s->gX, (void *)s->gC, (void *)s->gOld, (void *)s->gT,
                  (void *)s->gkeep, (void *)s->gchunk, (void *)s->fallback, (void *)s->snap, (void *)s->n_snap,
                  (void *)s->totals, (void *)s->rows_fine64, (void *)s->eca_fine64, (void *)s->bias_block,
                  (void *)s->rows_fine32, (void *)s->eca_fine32})
    cudaFree(p);
  delete s;
  return CM_OK;
}

int cm_surrogate_create(cm_surrogate_t *out, cm_params_t p, int substeps, uint64_t seed, void *stream) {
  if (!out || !p) return fail(CM_ERR_ARG, "NULL argument");
  *out = nullptr;
  if (p->ps.spec->model != kTenTusscher2) return fail(CM_ERR_UNSUPPORTED, "the surrogate covers TenTusscher2");
  if (substeps < 1 || substeps > 64) return fail(CM_ERR_ARG, "substeps in [1, 64]");
  auto *s = new (std::nothrow) cm_surrogate_s();
  if (!s) return fail(CM_ERR_NOMEM, "host allocation failed");
  s->fine = p->ps;
  s->coarse_ps = p->ps;
  s->substeps = substeps;
  s->stream = (cudaStream_t)stream;
  s->coarse_ps.dt = p->ps.dt * substeps;
  s->coarse_ps.rebuild();  // tables for the macro step
  TT2Consts<double> cd;
  s->coarse_ps.tt2_consts(cd, s->coarse);
  std::vector<float> rows, eca;
  s->coarse_ps.rows_fp32(rows, eca);
  int rc = CM_OK;
  cudaError_t e = cudaMalloc(&s->rows_coarse, rows.size() * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&s->eca, eca.size() * sizeof(float));
  if (e == cudaSuccess) e = cudaMemcpy(s->rows_coarse, rows.data(), rows.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(s->eca, eca.data(), eca.size() * sizeof(float), cudaMemcpyHostToDevice);
  {
    s->fine.tt2_consts(s->fine64, s->fine32);
    std::vector<float> r32, e32;
    s->fine.rows_fp32(r32, e32);
    if (e == cudaSuccess) e = cudaMalloc(&s->rows_fine32, r32.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&s->eca_fine32, e32.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(s->rows_fine32, r32.data(), r32.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(s->eca_fine32, e32.data(), e32.size() * sizeof(float), cudaMemcpyHostToDevice);
    std::vector<double> r64, e64;
    s->fine.rows_fp64(r64, e64);
    if (e == cudaSuccess) e = cudaMalloc(&s->rows_fine64, r64.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&s->eca_fine64, e64.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(s->rows_fine64, r64.data(), r64.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(s->eca_fine64, e64.data(), e64.size() * sizeof(double), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMalloc(&s->d_count, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(s->d_count, 0, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&s->totals, kCounterBytes);
  if (e == cudaSuccess) {
    s->audit_err = reinterpret_cast<float *>(s->totals + 3);
    s->n_fallback = reinterpret_cast<unsigned int *>(s->totals + 3) + 1;
    e = cudaMallocHost(&s->host_res, kCounterBytes + 16);
  }
  if (e == cudaSuccess) e = cudaMalloc(&s->bias_block, 288 * sizeof(float));
  if (e == cudaSuccess) e = cudaGetDevice(&s->net.device);
  if (e == cudaSuccess) e = s->net.m.init(kSurIn, kSurH, kSurOut, seed, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) rc = cuda_fail(e, "cm_surrogate_create");
  for (int k = 0; k < kSurIn; k++) s->norm.inv_sd_x[k] = 1.f;
  for (int k = 0; k < kSurOut; k++) s->norm.sd_y[k] = s->norm.apply_y[k] = 1.f;
  if (rc) {
    std::string keep = last_error();
    cm_surrogate_destroy(s);
    last_error() = keep;
    return rc;
  }
  *out = s;
  return CM_OK;
}

int cm_surrogate_reset_network(cm_surrogate_t s, uint64_t seed) {
  if (!s) return fail(CM_ERR_ARG, "NULL surrogate");
  CK(s->net.m.reset(seed));
  CK(cudaStreamSynchronize(s->stream));
  s->fitted = false;
  return CM_OK;
}

int cm_surrogate_mlp(cm_surrogate_t s, cm_mlp_t *mlp) {
  if (!s || !mlp) return fail(CM_ERR_ARG, "NULL argument");
  *mlp = &s->net;
  return CM_OK;
}

int cm_surrogate_generate(cm_surrogate_t s, cm_batch_t b, double *Vm, int64_t n_macro, const cm_stimulus *stim,
                          int64_t cell_stride, int64_t max_pairs, int64_t *n_pairs) {
  if (!s || !Vm || n_macro < 0 || cell_stride < 1 || max_pairs < 0) return fail(CM_ERR_ARG, "bad argument");
  if (stim && stim->textbegin_per_cell)
    return fail(CM_ERR_UNSUPPORTED, "training-data generation takes one stimulus protocol for all cells");
  int rc = check_batch(b);
  if (rc) return rc;
  if (b->ps.dt != s->fine.dt) return fail(CM_ERR_ARG, "batch dt differs from the surrogate's fine dt");
  const int64_t n = b->d.n;
  if (n > 0x7fffffff) return fail(CM_ERR_ARG, "training-data generation takes at most 2^31 - 1 cells");
  const int64_t n_sample = (n + cell_stride - 1) / cell_stride;
  cudaStream_t st = b->stream;
  // dataset capacity (grows, keeping what is there)
  if (max_pairs > s->cap) {
    float *nx = nullptr, *nt = nullptr;
    CK(cudaMalloc(&nx, std::max<int64_t>(1, max_pairs) * kSurIn * sizeof(float)));
    CK(cudaMalloc(&nt, std::max<int64_t>(1, max_pairs) * kSurOut * sizeof(float)));
    unsigned long long have = 0;
    CK(cudaMemcpy(&have, s->d_count, sizeof(have), cudaMemcpyDeviceToHost));
    have = std::min<unsigned long long>(have, (unsigned long long)s->cap);
    if (have) {
      CK(cudaMemcpy(nx, s->dX, have * kSurIn * sizeof(float), cudaMemcpyDeviceToDevice));
      CK(cudaMemcpy(nt, s->dT, have * kSurOut * sizeof(float), cudaMemcpyDeviceToDevice));
    }
    cudaFree(s->dX);
    cudaFree(s->dT);
    s->dX = nx;
    s->dT = nt;
    s->cap = max_pairs;
  }
  if (n_sample > s->gcap) {
    for (void *p : {(void *)s->gX, (void *)s->gC, (void *)s->gOld, (void *)s->gT, (void *)s->gkeep, (void *)s->gchunk})
      cudaFree(p);
    CK(cudaMalloc(&s->gX, n_sample * kSurIn * sizeof(float)));
    CK(cudaMalloc(&s->gC, n_sample * kSurOut * sizeof(float)));
    CK(cudaMalloc(&s->gOld, n_sample * 8 * sizeof(float)));
    CK(cudaMalloc(&s->gT, n_sample * kSurOut * sizeof(float)));
    CK(cudaMalloc(&s->gkeep, n_sample));
    CK(cudaMalloc(&s->gchunk, sur_append_scratch_words(n_sample) * sizeof(int64_t)));
    s->gcap = n_sample;
  }
  double *dvm;
  bool host_vm;
  if ((rc = planes_in(b, Vm, &dvm, host_vm, st))) return rc;
  float *hi = b->vm_planes, *lo = b->vm_planes + b->d.ld;
  const cm_stimulus stv = stim ? *stim : cm_stimulus{0, 1e300, nullptr, 0, 0, 0};
  double t = stv.t0, tb = stv.textbegin;
  const float inv_g0_Na = (float)(1.0 / s->fine.get("g_Na")), inv_g0_Kr = (float)(1.0 / s->fine.get("g_Kr")),
              inv_g0_K1 = (float)(1.0 / s->fine.get("g_K1"));
  float iext[64];
  for (int64_t mstep = 0; mstep < n_macro; mstep++) {
    SurGenArgs ga{};
    ga.fine = b->d;
    ga.coarse = s->coarse;
    ga.rows_coarse = s->rows_coarse;
    ga.eca = s->eca;
    ga.vm_hi = hi;
    ga.vm_lo = lo;
    ga.stride = cell_stride;
    ga.offset = 0;
    ga.n_sample = n_sample;
    ga.X = s->gX;
    ga.C = s->gC;
    ga.Old = s->gOld;
    ga.inv_g0_Na = inv_g0_Na;
    ga.inv_g0_Kr = inv_g0_Kr;
    ga.inv_g0_K1 = inv_g0_K1;
    CK(launch_sur_gen(ga, st));
    const bool on = protocol_steps(stim ? &stv : nullptr, s->substeps, s->fine.dt, t, tb, iext);
    // the macro step's fine steps of every cell in one launch (Vm in registers between them; the
    // same per-step update as the batch's step kernel)
    SurPlainArgs fa{};
    fa.fine = b->d;
    fa.vm_hi = hi;
    fa.vm_lo = lo;
    fa.list = nullptr;
    fa.n_all = (int)n;
    fa.substeps = s->substeps;
    for (int k = 0; k < s->substeps; k++) fa.iext[k] = iext[k];
    CK(launch_sur_plain(fa, (int)n, st));
    SurPostArgs pa{};
    pa.fine = b->d;
    pa.vm_hi = hi;
    pa.vm_lo = lo;
    pa.stride = cell_stride;
    pa.offset = 0;
    pa.n_sample = n_sample;
    pa.C = s->gC;
    pa.Old = s->gOld;
    pa.T = s->gT;
    pa.keep = s->gkeep;
    pa.gate_mv_per_ms = 5.f;
    pa.macro_ms = (float)(s->coarse_ps.dt * 1000.0);
    pa.stim_on = on ? 1 : 0;
    CK(launch_sur_post(pa, st));
    CK(launch_sur_append(s->gX, s->gT, s->gkeep, n_sample, s->dX, s->dT, s->d_count, s->cap, s->gchunk, st));
  }
  if ((rc = planes_out(b, Vm, dvm, host_vm, st))) return rc;
  unsigned long long have = 0;
  CK(cudaMemcpyAsync(&have, s->d_count, sizeof(have), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (n_pairs) *n_pairs = (int64_t)std::min<unsigned long long>(have, (unsigned long long)s->cap);
  return CM_OK;
}

int cm_surrogate_dataset(cm_surrogate_t s, int64_t *n_pairs, float *X, float *T) {
  if (!s) return fail(CM_ERR_ARG, "NULL surrogate");
  unsigned long long have = 0;
  CK(cudaMemcpy(&have, s->d_count, sizeof(have), cudaMemcpyDeviceToHost));
  const int64_t n = (int64_t)std::min<unsigned long long>(have, (unsigned long long)s->cap);
  if (n_pairs) *n_pairs = n;
  if (X && n) CK(cudaMemcpy(X, s->dX, n * kSurIn * sizeof(float), cudaMemcpyDefault));
  if (T && n) CK(cudaMemcpy(T, s->dT, n * kSurOut * sizeof(float), cudaMemcpyDefault));
  return CM_OK;
}

int cm_surrogate_fit(cm_surrogate_t s, int batch, int steps, float lr, uint64_t seed, float *final_loss) {
  if (!s || batch < 64 || steps < 0 || !(lr > 0)) return fail(CM_ERR_ARG, "bad argument");
  int64_t n = 0;
  int rc = cm_surrogate_dataset(s, &n, nullptr, nullptr);
  if (rc) return rc;
  if (n < batch) return fail(CM_ERR_ARG, "fewer training pairs than one minibatch");
  // normalisation from a strided subsample of at most 2^18 rows
  const int64_t m = std::min<int64_t>(n, (int64_t)1 << 18), stride = n / m;
  std::vector<float> hx((size_t)n * kSurIn), ht((size_t)n * kSurOut);
  CK(cudaMemcpy(hx.data(), s->dX, hx.size() * sizeof(float), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(ht.data(), s->dT, ht.size() * sizeof(float), cudaMemcpyDeviceToHost));
  for (int k = 0; k < kSurIn; k++) {
    double sum = 0, sq = 0;
    for (int64_t r = 0; r < m; r++) {
      const double v = hx[(size_t)(r * stride) * kSurIn + k];
      sum += v;
      sq += v * v;
    }
    const double mu = sum / m, var = std::max(0.0, sq / m - mu * mu);
    s->norm.mu_x[k] = (float)mu;
    s->norm.inv_sd_x[k] = (float)(1.0 / std::max(std::sqrt(var), 1e-6 * std::max(1.0, std::fabs(mu))));
  }
  for (int k = 0; k < kSurOut; k++) {
    double sq = 0;
    for (int64_t r = 0; r < m; r++) {
      const double v = ht[(size_t)(r * stride) * kSurOut + k];
      sq += v * v;
    }
    s->norm.sd_y[k] = (float)std::max(std::sqrt(sq / m), 1e-12);
  }
  cudaFree(s->nX);
  cudaFree(s->nT);
  s->nX = s->nT = nullptr;
  CK(cudaMalloc(&s->nX, (size_t)n * kSurIn * sizeof(float)));
  CK(cudaMalloc(&s->nT, (size_t)n * kSurOut * sizeof(float)));
  CK(launch_sur_normalize(s->dX, s->dT, n, s->norm, s->nX, s->nT, s->stream));
  float loss = 0;
  CK(s->net.m.train(s->nX, s->nT, n, batch, steps, lr, seed, &loss));
  CK(cudaStreamSynchronize(s->stream));
  // R^2 of every output on a strided subsample: which corrections the network predicts
  {
    const int64_t mv = std::min<int64_t>(n, (int64_t)1 << 16), sv = n / mv;
    std::vector<float> xs((size_t)mv * kSurIn), ys((size_t)mv * kSurOut);
    for (int64_t r = 0; r < mv; r++)
      for (int k = 0; k < kSurIn; k++)
        xs[(size_t)r * kSurIn + k] = (hx[(size_t)(r * sv) * kSurIn + k] - s->norm.mu_x[k]) * s->norm.inv_sd_x[k];
    float *dx = nullptr, *dy = nullptr;
    cudaError_t e = cudaMalloc(&dx, xs.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&dy, ys.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(dx, xs.data(), xs.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = s->net.m.forward(dx, mv, dy);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMemcpy(ys.data(), dy, ys.size() * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    if (e != cudaSuccess) return cuda_fail(e, "cm_surrogate_fit");
    for (int k = 0; k < kSurOut; k++) {
      double mt = 0;
      for (int64_t r = 0; r < mv; r++) mt += ht[(size_t)(r * sv) * kSurOut + k] / s->norm.sd_y[k];
      mt /= mv;
      double res = 0, tot = 0;
      for (int64_t r = 0; r < mv; r++) {
        const double tn = ht[(size_t)(r * sv) * kSurOut + k] / s->norm.sd_y[k];
        const double d = ys[(size_t)r * kSurOut + k] - tn;
        res += d * d;
        tot += (tn - mt) * (tn - mt);
      }
      s->norm.r2[k] = tot > 0 ? (float)(1.0 - res / tot) : 0.f;
      s->norm.apply_y[k] = s->norm.r2[k] >= kSurMinR2 ? s->norm.sd_y[k] : 0.f;
    }
  }
  s->fitted = true;
  if (final_loss) *final_loss = loss;
  return CM_OK;
}

int64_t cm_surrogate_blob_size(cm_surrogate_t s) {
  return s ? (int64_t)(sizeof(SurNorm) / sizeof(float)) + n_unpadded(s->net.m) : -1;
}

int cm_surrogate_get_blob(cm_surrogate_t s, float *blob) {
  if (!s || !blob) return fail(CM_ERR_ARG, "NULL argument");
  const int64_t nn = sizeof(SurNorm) / sizeof(float);
  std::vector<float> h(cm_surrogate_blob_size(s));
  memcpy(h.data(), &s->norm, sizeof(SurNorm));
  int rc = mlp_copy(s->net.m, s->net.m.w, h.data() + nn, true);
  if (rc) return rc;
  if (is_device_ptr(blob)) CK(cudaMemcpy(blob, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
  else memcpy(blob, h.data(), h.size() * sizeof(float));
  return CM_OK;
}

int cm_surrogate_set_blob(cm_surrogate_t s, const float *blob) {
  if (!s || !blob) return fail(CM_ERR_ARG, "NULL argument");
  const int64_t nn = sizeof(SurNorm) / sizeof(float);
  std::vector<float> h;
  int rc = fetch(blob, cm_surrogate_blob_size(s), h);
  if (rc) return rc;
  memcpy(&s->norm, h.data(), sizeof(SurNorm));
  CK(cudaStreamSynchronize(s->stream));
  if ((rc = mlp_copy(s->net.m, s->net.m.w, h.data() + nn, false))) return rc;
  CK(s->net.m.sync_bf16());
  CK(cudaStreamSynchronize(s->stream));
  s->fitted = true;
  return CM_OK;
}

int cm_batch_run_surrogate(cm_batch_t b, cm_surrogate_t s, double *Vm, int64_t n_macro, const cm_stimulus *stim,
                           int mode, int audit_mod, cm_surrogate_stats *stats) {
  if (!s || !Vm || n_macro < 0 || audit_mod < 0 || (mode & ~(CM_SUR_COARSE_ONLY | CM_SUR_AUDIT_FP64)))
    return fail(CM_ERR_ARG, "bad argument");
  int rc = check_batch(b);
  if (rc) return rc;
  if (b->ps.dt != s->fine.dt) return fail(CM_ERR_ARG, "batch dt differs from the surrogate's fine dt");
  const int64_t n = b->d.n;
  cudaStream_t st = b->stream;
  if (n > s->rcap) {
    cudaFree(s->fallback);
    s->fallback = nullptr;
    CK(cudaMalloc(&s->fallback, std::max<int64_t>(1, n) * sizeof(int)));
    s->rcap = n;
  }
  // the counters: cleared at the end of the last run (behind its result copy), else here
  if (!s->counters_zeroed) CK(cudaMemsetAsync(s->totals, 0, kCounterBytes, st));
  s->counters_zeroed = false;
  const bool audit_fp64 = (mode & CM_SUR_AUDIT_FP64) != 0;
  const int64_t snap_need = audit_mod > 0 ? (n + audit_mod - 1) / audit_mod + 32 : 32;
  if (snap_need > s->snap_cap || audit_mod == 0) {
    if ((rc = flush_pending(s, audit_fp64, st))) return rc;  // before its buffer goes or no audit follows
  }
  if (snap_need > s->snap_cap) {
    CK(cudaStreamSynchronize(st));
    cudaFree(s->snap);
    s->snap = nullptr;
    s->snap_cap = 0;
    CK(cudaMalloc(&s->snap, 2 * (size_t)kSnapPlanes * snap_need * sizeof(float)));
    s->snap_cap = snap_need;
  }
  if (!s->n_snap) {
    CK(cudaMalloc(&s->n_snap, 2 * sizeof(unsigned int)));
    CK(cudaMemsetAsync(s->n_snap, 0, 2 * sizeof(unsigned int), st));
  }
  // the first macro step writes the buffer that holds no pending sample and audits the other
  // (the pending sample of the previous call, or nothing: its counter is zero)
  int wbuf = s->pending >= 0 ? (s->pending ^ 1) : 0;
  if (s->pending < 0) CK(cudaMemsetAsync(s->n_snap, 0, 2 * sizeof(unsigned int), st));
  double *dvm, *direct;
  bool host_vm = false;
  if ((rc = vm_in(b, Vm, &direct, &dvm, host_vm, st))) return rc;
  float *hi = direct ? nullptr : b->vm_planes, *lo = direct ? nullptr : b->vm_planes + b->d.ld;
  const cm_stimulus stv = stim ? *stim : cm_stimulus{0, 1e300, nullptr, 0, 0, 0};
  double t = stv.t0, tb = stv.textbegin;
  SurKernelArgs ka{};
  ka.fine = b->d;
  ka.coarse = s->coarse;
  ka.rows_coarse = s->rows_coarse;
  ka.eca = s->eca;
  ka.vm = direct;
  ka.vm_hi = direct ? nullptr : hi;
  ka.vm_lo = direct ? nullptr : lo;
  ka.norm = s->norm;
  ka.w1 = s->net.m.wb + s->net.m.off[0];
  ka.w2 = s->net.m.wb + s->net.m.off[2];
  ka.w3 = s->net.m.wb + s->net.m.off[4];
  ka.bias = nullptr;
  ka.mode = mode & CM_SUR_COARSE_ONLY;
  ka.gate_mv_per_ms = 5.f;
  ka.audit_mod = audit_mod;
  ka.fallback = s->fallback;
  ka.n_fallback = s->n_fallback;
  ka.n_fallback_total = s->totals + 1;
  ka.snap_cap = (int)s->snap_cap;
  ka.n_sur = s->totals;
  ka.inv_g0_Na = (float)(1.0 / s->fine.get("g_Na"));
  ka.inv_g0_Kr = (float)(1.0 / s->fine.get("g_Kr"));
  ka.inv_g0_K1 = (float)(1.0 / s->fine.get("g_K1"));
  // biases as one contiguous FP32 block b1 | b2 | b3 (the kernel's layout), copied again only
  // when the network's weights have changed since
  float *bias = s->bias_block;
  if (s->bias_version != s->net.m.version) {
    CK(cudaMemcpyAsync(bias, s->net.m.w + s->net.m.off[1], 128 * sizeof(float), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(bias + 128, s->net.m.w + s->net.m.off[3], 128 * sizeof(float), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(bias + 256, s->net.m.w + s->net.m.off[5], 32 * sizeof(float), cudaMemcpyDeviceToDevice, st));
    s->bias_version = s->net.m.version;
  }
  ka.bias = bias;
  SurPlainArgs pa{};
  pa.fine = b->d;
  pa.vm = direct;
  pa.vm_hi = ka.vm_hi;
  pa.vm_lo = ka.vm_lo;
  pa.list = s->fallback;
  pa.n_list = s->n_fallback;
  pa.substeps = s->substeps;
  cudaError_t e = cudaSuccess;
  const bool per_cell = stim && stim->textbegin_per_cell;
  if (per_cell) {  // the reference driver's per-cell textbegin, advanced on the device
    double *tbc = nullptr;
    if ((rc = per_cell_times(b, stim->textbegin_per_cell, st, &tbc))) return rc;
    ka.tb_cell = tbc;
    pa.tb_cell = tbc;
    pa.textlen = stv.textlen;
    pa.bcl = stv.bcl;
    pa.amp = stv.amplitude;
  }
  constexpr int kEvChunk = 256;
  while (s->ev.size() < 3 * (size_t)kEvChunk) {
    cudaEvent_t ev;
    CK(cudaEventCreate(&ev));
    s->ev.push_back(ev);
  }
  double ms_step = 0, ms_plain = 0;
  for (int64_t mstep = 0; mstep < n_macro && e == cudaSuccess; mstep++) {
    bool on = false;
    if (per_cell) {
      for (int k = 0; k < s->substeps; k++) {
        pa.tk[k] = t;
        if (k + 1 < s->substeps) t += s->fine.dt;
      }
      ka.t_last = t;
      t += s->fine.dt;
    } else {
      on = protocol_steps(stim ? &stv : nullptr, s->substeps, s->fine.dt, t, tb, pa.iext);
    }
    ka.stim_on = on ? 1 : 0;
    ka.audit_phase = audit_mod > 0 ? (int)(mstep % audit_mod) : 0;
    const int buf = wbuf;
    wbuf ^= 1;
    ka.snap = s->snap + (size_t)buf * kSnapPlanes * s->snap_cap;
    ka.n_snap = s->n_snap + buf;
    const SurAuditArgs aa = audit_args(s, buf ^ 1, audit_fp64);  // the previous step's sample
    if (mstep > 0) e = cudaMemsetAsync(s->n_fallback, 0, sizeof(unsigned int), st);  // step 0: cleared above
    // the two kernels bracketed by events; every kEvChunk steps the chunk's times are summed
    // (the last chunk's after the final synchronisation below)
    const int j = (int)(mstep % kEvChunk);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev[3 * j], st);
    if (e == cudaSuccess) e = launch_sur_step(ka, audit_mod > 0 ? &aa : nullptr, n, st);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev[3 * j + 1], st);
    // the previous step's sample is audited: the next step writes its buffer from zero
    if (e == cudaSuccess && audit_mod > 0) e = cudaMemsetAsync(s->n_snap + (buf ^ 1), 0, sizeof(unsigned int), st);
    if (e == cudaSuccess) e = launch_sur_plain(pa, (int)n, st);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev[3 * j + 2], st);
    if (e == cudaSuccess && j == kEvChunk - 1 && mstep != n_macro - 1) {
      e = cudaEventSynchronize(s->ev[3 * j + 2]);
      for (int i = 0; i <= j && e == cudaSuccess; i++) {
        float a = 0.f, b2 = 0.f;
        e = cudaEventElapsedTime(&a, s->ev[3 * i], s->ev[3 * i + 1]);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&b2, s->ev[3 * i + 1], s->ev[3 * i + 2]);
        ms_step += a;
        ms_plain += b2;
      }
    }
  }
  if (e != cudaSuccess) return cuda_fail(e, "surrogate run");
  // the last step's sample is audited by the next run's first macro step, or by
  // cm_surrogate_flush_audit
  if (audit_mod > 0 && n_macro > 0) s->pending = wbuf ^ 1;
  rc = vm_out(b, Vm, dvm, direct, host_vm, st);
  // the counters and the audit mask into page-locked memory, then the counters cleared for the
  // next run, all behind the last kernels: one synchronisation ends the call
  unsigned long long *res = s->host_res;
  if (!rc) {
    e = cudaMemcpyAsync(res, s->totals, kCounterBytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(res + 4, b->audit_or, sizeof(unsigned int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->totals, 0, kCounterBytes, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) s->counters_zeroed = true;
    if (e == cudaSuccess && n_macro > 0) {  // the last chunk's kernel times
      const int jl = (int)((n_macro - 1) % kEvChunk);
      for (int i = 0; i <= jl && e == cudaSuccess; i++) {
        float a = 0.f, b2 = 0.f;
        e = cudaEventElapsedTime(&a, s->ev[3 * i], s->ev[3 * i + 1]);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&b2, s->ev[3 * i + 1], s->ev[3 * i + 2]);
        ms_step += a;
        ms_plain += b2;
      }
    }
    if (e != cudaSuccess) rc = cuda_fail(e, "surrogate run");
  }
  if (rc) return rc;
  unsigned long long tot[3] = {res[0], res[1], res[2]};
  float aerr;
  unsigned int mask;
  std::memcpy(&aerr, res + 3, sizeof(float));
  std::memcpy(&mask, res + 4, sizeof(unsigned int));
  if (stats) {
    stats->cell_macro_steps = n * n_macro;
    stats->surrogate = (int64_t)tot[0];
    stats->fallback = (int64_t)tot[1];
    stats->audited = (int64_t)tot[2];
    stats->max_audit_err_mv = aerr;
    stats->ms_step_kernel = ms_step;
    stats->ms_plain_kernel = ms_plain;
  }
  if (mask & CM_AUDIT_NAN) return fail(CM_ERR_NUMERIC, "Vm is NaN or infinite in at least one cell");
  return CM_OK;
}

int cm_surrogate_flush_audit(cm_surrogate_t s, int mode, cm_surrogate_stats *stats) {
  if (!s) return fail(CM_ERR_ARG, "NULL surrogate");
  if (stats) *stats = cm_surrogate_stats{};
  if (s->pending < 0) return CM_OK;
  cudaStream_t st = s->stream;
  s->counters_zeroed = false;
  CK(cudaMemsetAsync(s->totals, 0, kCounterBytes, st));
  int rc = flush_pending(s, (mode & CM_SUR_AUDIT_FP64) != 0, st);
  if (rc) return rc;
  unsigned long long tot[3] = {0, 0, 0};
  float aerr = 0.f;
  CK(cudaMemcpyAsync(tot, s->totals, sizeof(tot), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&aerr, s->audit_err, sizeof(float), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (stats) {
    stats->audited = (int64_t)tot[2];
    stats->max_audit_err_mv = aerr;
  }
  return CM_OK;
}

int cm_mlp_forward_static(cm_mlp_t m, const float *X, int64_t n, float *Y) {
  if (!m || !X || !Y || n < 0) return fail(CM_ERR_ARG, "bad argument");
  if (n == 0) return CM_OK;
  if (!is_device_ptr(X) || !is_device_ptr(Y))
    return fail(CM_ERR_ARG, "cm_mlp_forward_static takes device arrays only (staging host arrays would allocate)");
  // the scratch address is looked up for the current device: it must be the network's
  int dev = -1;
  CK(cudaGetDevice(&dev));
  if (dev != m->device)
    return fail(CM_ERR_ARG, "cm_mlp_forward_static: the current device (" + std::to_string(dev) +
                                ") is not the one the network was created on (" + std::to_string(m->device) + ")");
  void *scratch = nullptr;
  size_t bytes = 0;
  CK(static_scratch(&scratch, &bytes));
  const int64_t max_rows = (int64_t)(bytes / m->m.forward_scratch_bytes_per_row()) / 64 * 64;
  if (n > max_rows)
    return fail(CM_ERR_ARG, "cm_mlp_forward_static: n = " + std::to_string(n) + " rows exceeds the static scratch (" +
                                std::to_string(bytes) + " bytes: at most " + std::to_string(max_rows) +
                                " rows for this network)");
  CK(m->m.forward_in_scratch(scratch, X, n, Y));
  CK(cudaStreamSynchronize(m->m.stream));
  return CM_OK;
}

int cm_diag_mlp_workspace_rows(void *m, int64_t *rows) {
  if (!m || !rows) return fail(CM_ERR_ARG, "NULL argument");
  *rows = ((cm_mlp_s *)m)->m.ws_rows;
  return CM_OK;
}

}  // extern "C"
