// Monodomain coupling (include/cardiomech_gb300.h, "monodomain coupling"): the intra matrix of
// acCELLerate::IntraStep in 32-row slices on the device, its product, and the fused
// product + cell update + Godunov step + checks + activation times (acCELLerate.cpp:1839-2005).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "cm_handles.h"

using namespace cm;


namespace {

void free_diffusion(cm_diffusion_s *d) {
  cudaFree(d->sl_ptr);
  cudaFree(d->sl_col);
  cudaFree(d->val64);
  cudaFree(d->val32);
  cudaFree(d->rowsum32);
  cudaFree(d->scale64);
  cudaFree(d->scale32);
  delete d;
}

template <typename T>
int upload(T **dst, const std::vector<T> &src) {
  CK(cudaMalloc(dst, std::max<size_t>(1, src.size()) * sizeof(T)));
  if (!src.empty()) CK(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  return CM_OK;
}

}  // namespace

extern "C" {

int cm_diffusion_create(cm_diffusion_t *out, int64_t n, const int64_t *rowptr, const int32_t *col,
                        const double *val, const double *scale, double uniform_scale) {
  if (!out) return fail(CM_ERR_ARG, "NULL argument");
  *out = nullptr;
  if (n < 0) return fail(CM_ERR_ARG, "n < 0");
  if (n > 0 && (!rowptr || !col || !val)) return fail(CM_ERR_ARG, "NULL CSR array");
  if (n > ((int64_t)1 << 31) - 64) return fail(CM_ERR_ARG, "more rows than 32-bit column indices address");
  // the CSR must be well formed before anything reaches the device: every column is read by
  // the kernels as an index into Vm
  if (n > 0 && rowptr[0] != 0) return fail(CM_ERR_ARG, "rowptr[0] != 0");
  for (int64_t r = 0; r < n; r++)
    if (rowptr[r + 1] < rowptr[r]) return fail(CM_ERR_ARG, "rowptr decreases at row " + std::to_string(r));
  const int64_t nnz = n > 0 ? rowptr[n] : 0;
  for (int64_t e = 0; e < nnz; e++)
    if (col[e] < 0 || (int64_t)col[e] >= n)
      return fail(CM_ERR_ARG, "column index out of range at entry " + std::to_string(e));
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(CM_ERR_CUDA, "no CUDA device: this library has no CPU path");
  }
  // 32-row slices, entry k of row 32 s + r at ptr[s] + 32 k + r; a slice is as wide as its
  // longest row; padding entries: value 0, the row's own column
  const int64_t ns = (n + 31) / 32;
  std::vector<int64_t> ptr(ns + 1, 0);
  for (int64_t s = 0; s < ns; s++) {
    int64_t w = 0;
    for (int64_t r = 32 * s; r < std::min(n, 32 * s + 32); r++) w = std::max(w, rowptr[r + 1] - rowptr[r]);
    ptr[s + 1] = ptr[s] + 32 * w;
  }
  const int64_t ent = ptr[ns];
  int64_t wmax = 0;
  for (int64_t s = 0; s < ns; s++) wmax = std::max(wmax, (ptr[s + 1] - ptr[s]) / 32);
  // per-node planes padded to whole 256-cell tiles (the staged kernel copies whole tiles)
  const int64_t npad = ((n + 255) / 256) * 256;
  std::vector<int32_t> c32(ent);
  std::vector<double> v64(ent, 0.0);
  std::vector<float> v32(ent, 0.f), rs(npad, 0.f), sc32;
  for (int64_t s = 0; s < ns; s++) {
    const int64_t w = (ptr[s + 1] - ptr[s]) / 32;
    for (int64_t r = 0; r < 32; r++) {
      const int64_t row = 32 * s + r;
      const int64_t len = row < n ? rowptr[row + 1] - rowptr[row] : 0;
      double sum = 0.0;
      for (int64_t k = 0; k < w; k++) {
        const int64_t e = ptr[s] + 32 * k + r;
        if (k < len) {
          const int64_t src = rowptr[row] + k;
          c32[e] = col[src];
          v64[e] = val[src];
          v32[e] = col[src] == row ? 0.f : (float)val[src];
          sum += val[src];
        } else {
          c32[e] = (int32_t)(row < n ? row : 0);
        }
      }
      if (row < n) rs[row] = (float)sum;
    }
  }
  auto *d = new (std::nothrow) cm_diffusion_s();
  if (!d) return fail(CM_ERR_NOMEM, "host allocation failed");
  d->n = n;
  d->n_slices = ns;
  d->entries = ent;
  d->wmax = (int)std::min<int64_t>(wmax, 1 << 20);
  d->uniform = uniform_scale;
  int rc = upload(&d->sl_ptr, ptr);
  if (!rc) rc = upload(&d->sl_col, c32);
  if (!rc) rc = upload(&d->val64, v64);
  if (!rc) rc = upload(&d->val32, v32);
  if (!rc) rc = upload(&d->rowsum32, rs);
  if (!rc && scale) {
    std::vector<double> s64(scale, scale + n);
    sc32.assign(npad, 0.f);
    std::copy(scale, scale + n, sc32.begin());
    rc = upload(&d->scale64, s64);
    if (!rc) rc = upload(&d->scale32, sc32);
  }
  if (rc) {
    std::string keep = last_error();
    free_diffusion(d);
    last_error() = keep;
    return rc;
  }
  *out = d;
  return CM_OK;
}

int cm_diffusion_destroy(cm_diffusion_t d) {
  if (!d) return CM_OK;
  cudaDeviceSynchronize();
  free_diffusion(d);
  return CM_OK;
}

int cm_diffusion_apply(cm_diffusion_t d, const double *x, double *y) {
  if (!d || !x || !y) return fail(CM_ERR_ARG, "NULL argument");
  if (x == y) return fail(CM_ERR_ARG, "x and y alias");
  const int64_t n = d->n;
  if (n == 0) return CM_OK;
  const bool hx = !is_device_ptr(x), hy = !is_device_ptr(y);
  double *dx = const_cast<double *>(x), *dy = y;
  if (hx) CK(cudaMalloc(&dx, n * sizeof(double)));
  if (hy) CK(cudaMalloc(&dy, n * sizeof(double)));
  cudaError_t e = cudaSuccess;
  if (hx) e = cudaMemcpy(dx, x, n * sizeof(double), cudaMemcpyHostToDevice);
  StepIO io;
  d->fill(io, false);
  if (e == cudaSuccess) e = launch_diffusion_apply(io, dx, dy, n, nullptr);
  if (e == cudaSuccess && hy) e = cudaMemcpy(y, dy, n * sizeof(double), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (hx) cudaFree(dx);
  if (hy) cudaFree(dy);
  if (e != cudaSuccess) return cuda_fail(e, "cm_diffusion_apply");
  return CM_OK;
}

int cm_batch_run_diffuse(cm_batch_t b, cm_diffusion_t d, double *Vm, int64_t n_steps, const cm_stimulus *stim,
                         double vm_range, double *act, double act_threshold) {
  if (!b || !d || !Vm) return fail(CM_ERR_ARG, "NULL argument");
  if (d->n != b->d.n) return fail(CM_ERR_ARG, "the operator's rows differ from the batch's cells");
  if (n_steps < 0) return fail(CM_ERR_ARG, "n_steps < 0");
  const int64_t n = b->d.n, ld = b->d.ld;
  if (n == 0 || n_steps == 0) return CM_OK;
  int rc;
  // Vm on the device (the caller's array, or stage 0) and a second buffer for the new values
  if ((rc = ensure_stage(b, n))) return rc;
  const bool host_vm = !is_device_ptr(Vm);
  double *v0 = host_vm ? b->stage[0] : Vm, *v1 = b->stage[1];
  if (host_vm) CK(cudaMemcpyAsync(v0, Vm, n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
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
  const bool mixed = b->d.precision == CM_PREC_MIXED;
  float *planes[2] = {nullptr, nullptr};
  if (mixed) {
    if (!b->vm_planes) CK(cudaMalloc(&b->vm_planes, std::max<int64_t>(1, 2 * ld) * sizeof(float)));
    if (!b->vm_planes2) CK(cudaMalloc(&b->vm_planes2, std::max<int64_t>(1, 2 * ld) * sizeof(float)));
    planes[0] = b->vm_planes;
    planes[1] = b->vm_planes2;
    CK(launch_vm_split(v0, planes[0], planes[0] + ld, n, b->stream));
  }
  StepIO io;
  d->fill(io, mixed);
  io.vm_range = vm_range;
  io.act = dact;
  io.act_threshold = act_threshold;
  io.textlen = st.textlen;
  io.bcl = st.bcl;
  io.amp = st.amplitude;
  io.tb_cell = tb_cell;
  double t = st.t0, tb = st.textbegin;
  int cur = 0;
  for (int64_t s = 0; s < n_steps; s++) {
    io.t = t;
    io.act_time = t;  // IntraStep stamps activation with the step's own time (acCELLerate.cpp:2002)
    if (!per_cell) {
      double i_ext = 0.0;
      if (stim && t >= tb) {
        i_ext = st.amplitude;
        if (t >= tb + st.textlen) tb += st.bcl;
      }
      io.iext_uniform = i_ext;
    }
    if (mixed) {
      io.vm_hi = planes[cur];
      io.vm_lo = planes[cur] + ld;
      io.vm_hi_out = planes[cur ^ 1];
      io.vm_lo_out = planes[cur ^ 1] + ld;
    } else {
      io.vm = cur ? v1 : v0;
      io.vm_out = cur ? v0 : v1;
    }
    CK(launch_step(b->d, io, b->d.variant, b->d.grid_mode, b->stream));
    cur ^= 1;
    t += b->ps.dt;
  }
  if (mixed) {
    CK(launch_vm_join(planes[cur], planes[cur] + ld, v0, n, b->stream));
  } else if (cur) {
    CK(cudaMemcpyAsync(v0, v1, n * sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  }
  if (host_vm) CK(cudaMemcpyAsync(Vm, v0, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  if (host_act) CK(cudaMemcpyAsync(act, dact, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  unsigned int mask = 0;
  CK(cudaMemcpyAsync(&mask, b->audit_or, sizeof(unsigned int), cudaMemcpyDeviceToHost, b->stream));
  CK(cudaStreamSynchronize(b->stream));
  if (mask & (CM_AUDIT_NAN | CM_AUDIT_VMRANGE))
    return fail(CM_ERR_NUMERIC, "Vm is NaN, infinite or outside the allowed range in at least one cell");
  return CM_OK;
}

}  // extern "C"
