// The implicit finite-element monodomain step (include/cardiomech_gb300.h, "implicit step"):
// the theta-scheme solve of acCELLerate::IntraStep (acCELLerate.cpp:1951-1993) on the device,
// alone (cm_theta_solve) or with the cell update, Godunov step, range check and activation times
// of the same step (cm_batch_run_theta, acCELLerate.cpp:1839-2005 with IntraRHS set).
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <string>

#include "cm_handles.h"

using namespace cm;

struct cm_theta_s {
  cm_diffusion_s *lhs = nullptr, *rhs = nullptr;  // borrowed: A and R
  int64_t n = 0;
  double *vec = nullptr;  // dinv, r, z, p, q (n each)
  double *part = nullptr;  // bb, pq (G each), rz, zz (2 G each)
  ThetaStat *st = nullptr;
  ThetaStat *st_host = nullptr;  // pinned
  int *bad = nullptr;
  ThetaCfg cfg;
  int max_iter = 1000;
  int last_iters = 7;  // iterations of the last solve (the fallback's first chunk)
  cudaGraphExec_t loop = nullptr;  // the iterations as a conditional while node, for x == loop_x
  double *loop_x = nullptr;
  bool no_graph = false;           // the conditional node could not be built: chunks of launches
  ThetaStat *ring = nullptr;       // pinned outcome records of cm_batch_run_theta
  double *xbuf = nullptr;          // cm_theta_solve's device copy of a host x (one address: one graph)
  int G = 0;
  ThetaOp op(const cm_diffusion_s *d) const {
    ThetaOp o;
    o.ptr = d->sl_ptr;
    o.col = d->sl_col;
    o.val = d->val64;
    o.n = d->n;
    return o;
  }
  ThetaVecs vecs(double *x) const {
    ThetaVecs v;
    v.x = x;
    v.dinv = vec;
    v.r = vec + n;
    v.z = vec + 2 * n;
    v.p = vec + 3 * n;
    v.q = vec + 4 * n;
    return v;
  }
  ThetaPart parts() const {
    ThetaPart P;
    P.G = G;
    P.bb = part;
    P.pq = part + G;
    P.rz = part + 2 * G;
    P.zz = part + 4 * G;
    return P;
  }
};

namespace {

constexpr int kRing = 64;  // solves between two reads of their outcomes in cm_batch_run_theta

void free_theta(cm_theta_s *t) {
  if (t->loop) cudaGraphExecDestroy(t->loop);
  cudaFree(t->vec);
  cudaFree(t->part);
  cudaFree(t->st);
  cudaFree(t->bad);
  cudaFreeHost(t->st_host);
  cudaFreeHost(t->ring);
  cudaFree(t->xbuf);
  delete t;
}

// Enqueues one solve on stream s (x on the device): the setup kernels, then the iterations as
// one launch of the conditional-loop graph. Returns with the outcome still on the device (t->st)
// unless the graph could not be built, in which case chunks of iterations are launched with a
// read of the outcome after each (*synced = true, outcome in *t->st_host).
int theta_enqueue(cm_theta_s *t, double *x, cudaStream_t s, bool *synced) {
  const ThetaOp A = t->op(t->lhs), R = t->op(t->rhs);
  const ThetaVecs v = t->vecs(x);
  const ThetaPart P = t->parts();
  *synced = false;
  CK(launch_theta_init(A, R, v, P, t->cfg, t->st, s));
  if (!t->no_graph && (t->loop == nullptr || t->loop_x != x)) {
    if (t->loop) {
      CK(cudaStreamSynchronize(s));
      cudaGraphExecDestroy(t->loop);
      t->loop = nullptr;
    }
    cudaError_t e = build_theta_graph(A, v, P, t->cfg, t->st, t->max_iter, &t->loop);
    if (e != cudaSuccess) {
      cudaGetLastError();
      t->loop = nullptr;
      t->no_graph = true;
    } else {
      t->loop_x = x;
    }
  }
  if (t->loop) {
    CK(cudaGraphLaunch(t->loop, s));
    return CM_OK;
  }
  int k = 0;
  int c = std::max(1, std::min(t->last_iters + 1, 32));
  do {
    c = std::min(c, t->max_iter - k);
    CK(launch_theta_iters(A, v, P, t->cfg, t->st, t->max_iter, c, s));
    k += c;
    c = 4;
    CK(cudaMemcpyAsync(t->st_host, t->st, sizeof(ThetaStat), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  } while (!t->st_host->done && k < t->max_iter);
  t->last_iters = t->st_host->iters;
  *synced = true;
  return CM_OK;
}

void account(cm_theta_stats *stats, const ThetaStat &o) {
  if (!stats) return;
  stats->solves++;
  stats->iterations += o.iters;
  stats->max_iterations = std::max<int64_t>(stats->max_iterations, o.iters);
  if (o.done != 1) stats->not_converged++;
  stats->last_norm = o.znorm;
}

}  // namespace

extern "C" {

int cm_theta_create(cm_theta_t *out, cm_diffusion_t lhs, cm_diffusion_t rhs, double rtol, double atol, int max_iter) {
  if (!out || !lhs || !rhs) return fail(CM_ERR_ARG, "NULL argument");
  *out = nullptr;
  if (lhs->n != rhs->n) return fail(CM_ERR_ARG, "the two operators differ in size");
  if (!(rtol > 0.0) || !(atol >= 0.0) || max_iter < 1) return fail(CM_ERR_ARG, "need rtol > 0, atol >= 0, max_iter >= 1");
  auto *t = new (std::nothrow) cm_theta_s();
  if (!t) return fail(CM_ERR_NOMEM, "host allocation failed");
  t->lhs = lhs;
  t->rhs = rhs;
  t->n = lhs->n;
  t->cfg.rtol = rtol;
  t->cfg.atol = atol;
  t->max_iter = max_iter;
  t->G = theta_grid();
  cudaError_t e = cudaMalloc(&t->vec, std::max<int64_t>(1, 5 * t->n) * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&t->part, (size_t)6 * t->G * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&t->st, sizeof(ThetaStat));
  if (e == cudaSuccess) e = cudaMalloc(&t->bad, sizeof(int));
  if (e == cudaSuccess) e = cudaMallocHost(&t->st_host, sizeof(ThetaStat));
  if (e == cudaSuccess) e = cudaMemset(t->bad, 0, sizeof(int));
  if (e == cudaSuccess) e = launch_theta_dinv(t->op(lhs), t->vec, t->bad, nullptr);
  int bad = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&bad, t->bad, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    free_theta(t);
    return cuda_fail(e, "cm_theta_create");
  }
  if (bad) {
    free_theta(t);
    return fail(CM_ERR_ARG, "the left-hand operator has a row without a positive diagonal entry");
  }
  *out = t;
  return CM_OK;
}

int cm_theta_destroy(cm_theta_t t) {
  if (!t) return CM_OK;
  cudaDeviceSynchronize();
  free_theta(t);
  return CM_OK;
}

int cm_theta_solve(cm_theta_t t, double *x, cm_theta_stats *stats) {
  if (!t || !x) return fail(CM_ERR_ARG, "NULL argument");
  const int64_t n = t->n;
  if (n == 0) return CM_OK;
  const bool host = !is_device_ptr(x);
  double *dx = x;
  if (host) {
    if (!t->xbuf) CK(cudaMalloc(&t->xbuf, n * sizeof(double)));
    dx = t->xbuf;
    CK(cudaMemcpy(dx, x, n * sizeof(double), cudaMemcpyHostToDevice));
  }
  ThetaStat o{};
  bool synced = false;
  int rc = theta_enqueue(t, dx, nullptr, &synced);
  if (!rc && !synced) {
    cudaError_t e = cudaMemcpy(t->st_host, t->st, sizeof(ThetaStat), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = cuda_fail(e, "cm_theta_solve");
  }
  if (!rc) o = *t->st_host;
  if (!rc && host) {
    cudaError_t e = cudaMemcpy(x, dx, n * sizeof(double), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = cuda_fail(e, "cm_theta_solve");
  }
  if (rc) return rc;
  account(stats, o);
  if (o.done == 2 || o.done == 3)
    return fail(CM_ERR_NUMERIC, o.done == 2 ? "the solve diverged" : "the solve broke down (non-finite values)");
  return CM_OK;
}

int cm_batch_run_theta(cm_batch_t b, cm_theta_t t, double *Vm, int64_t n_steps, const cm_stimulus *stim,
                       double vm_range, double *act, double act_threshold, cm_theta_stats *stats) {
  if (!b || !t || !Vm) return fail(CM_ERR_ARG, "NULL argument");
  if (t->n != b->d.n) return fail(CM_ERR_ARG, "the operators' rows differ from the batch's cells");
  if (n_steps < 0) return fail(CM_ERR_ARG, "n_steps < 0");
  const int64_t n = b->d.n;
  if (n == 0 || n_steps == 0) return CM_OK;
  int rc;
  if ((rc = ensure_stage(b, n))) return rc;
  const bool host_vm = !is_device_ptr(Vm);
  double *x = host_vm ? b->stage[0] : Vm;
  if (host_vm) CK(cudaMemcpyAsync(x, Vm, n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  double *dact = nullptr;
  const bool host_act = act && !is_device_ptr(act);
  if (act) {
    dact = host_act ? b->stage[2] : act;
    if (host_act) CK(cudaMemcpyAsync(dact, act, n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  }
  cm_stimulus st = {};
  if (stim) st = *stim;
  const bool per_cell = stim && stim->textbegin_per_cell;
  double *tb_cell = nullptr;
  if (per_cell && (rc = per_cell_times(b, stim->textbegin_per_cell, b->stream, &tb_cell))) return rc;
  // the cell update and Godunov step in place (acCELLerate.cpp:1904-1949): no coupling current
  // (B = 0 on the implicit path, 1860-1862), the stimulus as the conditions give it
  if (!t->ring) CK(cudaMallocHost(&t->ring, kRing * sizeof(ThetaStat)));
  ThetaStat *ring = t->ring;
  StepIO io;
  io.vm = x;
  io.vm_out = x;
  io.vm_range = vm_range;
  io.textlen = st.textlen;
  io.bcl = st.bcl;
  io.amp = st.amplitude;
  io.tb_cell = tb_cell;
  double t_now = st.t0, tb = st.textbegin;
  for (int64_t s = 0; s < n_steps; s++) {
    io.t = t_now;
    if (!per_cell) {
      double i_ext = 0.0;
      if (stim && t_now >= tb) {
        i_ext = st.amplitude;
        if (t_now >= tb + st.textlen) tb += st.bcl;
      }
      io.iext_uniform = i_ext;
    }
    CK(launch_step(b->d, io, b->d.variant, b->d.grid_mode, b->stream));
    bool synced = false;
    if ((rc = theta_enqueue(t, x, b->stream, &synced))) return rc;
    // the outcomes go to a ring of pinned records, read every kRing steps (no read per step)
    const int slot = (int)(s % kRing);
    CK(cudaMemcpyAsync(ring + slot, t->st, sizeof(ThetaStat), cudaMemcpyDeviceToHost, b->stream));
    if (dact) CK(launch_theta_act(x, dact, n, act_threshold, t_now, b->stream));
    t_now += b->ps.dt;
    if (slot == kRing - 1 || s == n_steps - 1) {
      CK(cudaStreamSynchronize(b->stream));
      for (int j = 0; j <= slot; j++) {
        account(stats, ring[j]);
        if (ring[j].done == 2 || ring[j].done == 3)
          return fail(CM_ERR_NUMERIC, std::string(ring[j].done == 2 ? "the solve diverged" : "the solve broke down") +
                                          " at step " + std::to_string(s - slot + j));
      }
    }
  }
  if (host_vm) CK(cudaMemcpyAsync(Vm, x, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  if (host_act) CK(cudaMemcpyAsync(act, dact, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  unsigned int mask = 0;
  CK(cudaMemcpyAsync(&mask, b->audit_or, sizeof(unsigned int), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  if (mask & (CM_AUDIT_NAN | CM_AUDIT_VMRANGE))
    return fail(CM_ERR_NUMERIC, "Vm is NaN, infinite or outside the allowed range in at least one cell");
  return CM_OK;
}

}  // extern "C"
