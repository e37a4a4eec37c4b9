"""GB300-native cell-model update for KIT-IBT/CardioMechanics' electrophysiology reaction step.

The compute lives in libcmgb300.so (hand-written sm_103a CUDA + a C ABI, declared in
include/cardiomech_gb300.h). This module is a thin ctypes view of that ABI whose names
follow the reference's cell-model interface:

    reference (CellModel/)                          here
    initElphyParameters(&pep, ev, emt, tinc)        Params(model, ev_path, dt)
    initElphyModel(&pem, pep, emt) x N + Init()     Batch(params, n_cells, precision)
    pem->AddHeteroValue(name, v)                    batch.add_hetero_value(name, values)
    pem->Calc(tinc, Vm, i_ext, stretch, 1)          batch.calc(dt, Vm, i_ext, stretch) -> dVm
    Vm += Calc(...) driver loop (CellModel.h:420)   batch.run(Vm, n_steps, stimulus)
    GetBase()/GetSize(), Read/WriteStatus           batch.get_state(layout) / set_state
    GetVm(), GetAmplitude(), GetStimTime()          batch.init_vm(), params.info

There is no CPU path: without the library or without a GPU the calls raise.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libcmgb300.so"

TENTUSSCHER2 = 5
COURTEMANCHE = 2
OHARARUDY = 12
TOMEK = 14
FP64, MIXED = 0, 1
LAYOUT_REF_BLOCK, LAYOUT_SOA = 0, 1
AUDIT_NAN, AUDIT_VRANGE, AUDIT_CARANGE, AUDIT_GATE, AUDIT_SURROGATE, AUDIT_VMRANGE = 1, 2, 4, 8, 16, 32

_STATUS = {0: "CM_OK", -1: "CM_ERR_ARG", -2: "CM_ERR_MODEL", -3: "CM_ERR_FILE", -4: "CM_ERR_PARAM",
           -5: "CM_ERR_CUDA", -6: "CM_ERR_NOMEM", -7: "CM_ERR_UNSUPPORTED", -8: "CM_ERR_NUMERIC"}

# Exported symbols of the C ABI (include/cardiomech_gb300.h).
# cm_batch_run_surrogate mode bits
SUR_COARSE_ONLY = 1
SUR_AUDIT_FP64 = 2

ABI_SYMBOLS = (
    "cm_abi_version", "cm_last_error", "cm_model_from_name", "cm_model_info", "cm_state_name",
    "cm_params_create", "cm_params_destroy", "cm_params_info", "cm_params_get", "cm_params_set",
    "cm_params_table", "cm_batch_create", "cm_batch_destroy", "cm_batch_info", "cm_batch_reset",
    "cm_batch_set_hetero", "cm_batch_set_diagnostics", "cm_batch_init_vm", "cm_batch_get_state",
    "cm_batch_step_update_act",
    "cm_batch_set_state", "cm_batch_step", "cm_batch_step_update", "cm_batch_run", "cm_batch_audit",
    "cm_batch_autotune", "cm_batch_set_launch", "cm_diag_fma_peak", "cm_diag_umma_tile",
    "cm_diag_mlp_workspace_rows", "cm_diag_batch_wait_check", "cm_diag_fp64_math", "cm_diag_pair_convert", "cm_model_print_names", "cm_batch_print_values",
    "cm_batch_get_cell", "cm_batch_set_cell", "cm_batch_calc_cell",
    "cm_multi_create", "cm_multi_destroy", "cm_multi_run", "cm_multi_autotune", "cm_multi_set_launch",
    "cm_mlp_create", "cm_mlp_destroy", "cm_mlp_n_params", "cm_mlp_get_params", "cm_mlp_set_params",
    "cm_mlp_get_grads", "cm_mlp_forward", "cm_mlp_loss_grad", "cm_mlp_adam_step", "cm_surrogate_create",
    "cm_surrogate_destroy", "cm_surrogate_mlp", "cm_surrogate_generate", "cm_surrogate_dataset",
    "cm_surrogate_fit", "cm_surrogate_blob_size", "cm_surrogate_get_blob", "cm_surrogate_set_blob",
    "cm_batch_run_surrogate", "cm_mlp_forward_static", "cm_surrogate_flush_audit",
    "cm_diffusion_create", "cm_diffusion_destroy", "cm_diffusion_apply", "cm_batch_run_diffuse",
    "cm_backup_write", "cm_backup_read", "cm_theta_create", "cm_theta_destroy", "cm_theta_solve",
    "cm_batch_run_theta", "cm_surrogate_reset_network",
)


class CMError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_STATUS.get(code, code)}: {msg}")
        self.code = code


class Info(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int), ("n_state_vars", ctypes.c_int), ("ref_block_doubles", ctypes.c_int),
                ("n_tables", ctypes.c_int), ("table_rows", ctypes.c_int), ("dt", ctypes.c_double),
                ("init_vm", ctypes.c_double), ("amplitude", ctypes.c_double), ("stim_time", ctypes.c_double)]


class Stimulus(ctypes.Structure):
    _fields_ = [("t0", ctypes.c_double), ("textbegin", ctypes.c_double),
                ("textbegin_per_cell", ctypes.POINTER(ctypes.c_double)), ("textlen", ctypes.c_double),
                ("bcl", ctypes.c_double), ("amplitude", ctypes.c_double)]


class ThetaStats(ctypes.Structure):
    _fields_ = [("solves", ctypes.c_int64), ("iterations", ctypes.c_int64), ("max_iterations", ctypes.c_int64),
                ("not_converged", ctypes.c_int64), ("last_norm", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SurrogateStats(ctypes.Structure):
    _fields_ = [("cell_macro_steps", ctypes.c_int64), ("surrogate", ctypes.c_int64), ("fallback", ctypes.c_int64),
                ("audited", ctypes.c_int64), ("max_audit_err_mv", ctypes.c_double),
                ("ms_step_kernel", ctypes.c_double), ("ms_plain_kernel", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded C-ABI library. Raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m cardiomechanics_gb300.build`")
    L = ctypes.CDLL(str(LIB_PATH))
    vp, dp, i64 = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int64
    L.cm_last_error.restype = ctypes.c_char_p
    L.cm_state_name.restype = ctypes.c_char_p
    L.cm_model_from_name.argtypes = [ctypes.c_char_p]
    L.cm_model_info.argtypes = [ctypes.c_int, ctypes.POINTER(Info)]
    L.cm_params_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_char_p, ctypes.c_double]
    L.cm_params_destroy.argtypes = [vp]
    L.cm_params_info.argtypes = [vp, ctypes.POINTER(Info)]
    L.cm_params_get.argtypes = [vp, ctypes.c_char_p, dp]
    L.cm_params_set.argtypes = [vp, ctypes.c_char_p, ctypes.c_double]
    L.cm_params_table.argtypes = [vp, ctypes.c_char_p, dp]
    L.cm_batch_create.argtypes = [ctypes.POINTER(vp), vp, i64, ctypes.c_int, vp]
    L.cm_batch_destroy.argtypes = [vp]
    L.cm_batch_info.argtypes = [vp, ctypes.POINTER(Info), ctypes.POINTER(i64), ctypes.POINTER(ctypes.c_int)]
    L.cm_batch_reset.argtypes = [vp]
    L.cm_batch_set_hetero.argtypes = [vp, ctypes.c_char_p, vp]
    L.cm_batch_set_diagnostics.argtypes = [vp, ctypes.c_int]
    L.cm_batch_init_vm.argtypes = [vp, vp]
    L.cm_batch_get_state.argtypes = [vp, ctypes.c_int, vp]
    L.cm_batch_set_state.argtypes = [vp, ctypes.c_int, vp]
    L.cm_batch_step.argtypes = [vp, ctypes.c_double, vp, vp, vp, vp]
    L.cm_batch_step_update.argtypes = [vp, ctypes.c_double, vp, vp, vp, ctypes.c_double]
    L.cm_batch_step_update_act.argtypes = [vp, ctypes.c_double, vp, vp, vp, ctypes.c_double, vp, ctypes.c_double,
                                           ctypes.c_double]
    L.cm_batch_run.argtypes = [vp, vp, i64, ctypes.POINTER(Stimulus), vp, i64, i64, vp]
    L.cm_diffusion_create.argtypes = [ctypes.POINTER(vp), i64, vp, vp, vp, vp, ctypes.c_double]
    L.cm_diffusion_destroy.argtypes = [vp]
    L.cm_diffusion_apply.argtypes = [vp, vp, vp]
    L.cm_batch_run_diffuse.argtypes = [vp, vp, vp, i64, ctypes.POINTER(Stimulus), ctypes.c_double, vp,
                                       ctypes.c_double]
    L.cm_batch_audit.argtypes = [vp, ctypes.POINTER(ctypes.c_uint32), vp]
    L.cm_batch_autotune.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
    L.cm_batch_set_launch.argtypes = [vp, ctypes.c_int, ctypes.c_int]
    L.cm_multi_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.c_int, vp]
    L.cm_multi_destroy.argtypes = [vp]
    L.cm_multi_run.argtypes = [vp, ctypes.POINTER(vp), i64, ctypes.POINTER(Stimulus)]
    L.cm_multi_autotune.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                    ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
    L.cm_multi_set_launch.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.cm_theta_create.argtypes = [ctypes.POINTER(vp), vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_int]
    L.cm_theta_destroy.argtypes = [vp]
    L.cm_theta_solve.argtypes = [vp, vp, ctypes.POINTER(ThetaStats)]
    L.cm_batch_run_theta.argtypes = [vp, vp, vp, i64, ctypes.POINTER(Stimulus), ctypes.c_double, vp, ctypes.c_double,
                                     ctypes.POINTER(ThetaStats)]
    L.cm_backup_write.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(vp),
                                  ctypes.POINTER(vp), ctypes.POINTER(vp)]
    L.cm_backup_read.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(vp), ctypes.POINTER(vp),
                                 ctypes.POINTER(vp), ctypes.c_char_p, ctypes.c_size_t]
    fp = ctypes.POINTER(ctypes.c_float)
    L.cm_mlp_create.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, vp]
    L.cm_mlp_destroy.argtypes = [vp]
    L.cm_mlp_n_params.argtypes = [vp]
    L.cm_mlp_n_params.restype = ctypes.c_int64
    for f in ("cm_mlp_get_params", "cm_mlp_set_params", "cm_mlp_get_grads"):
        getattr(L, f).argtypes = [vp, vp]
    L.cm_mlp_forward.argtypes = [vp, vp, i64, vp]
    L.cm_mlp_forward_static.argtypes = [vp, vp, i64, vp]
    L.cm_surrogate_flush_audit.argtypes = [vp, ctypes.c_int, vp]
    L.cm_mlp_loss_grad.argtypes = [vp, vp, vp, i64, fp]
    L.cm_mlp_adam_step.argtypes = [vp, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float]
    L.cm_surrogate_create.argtypes = [ctypes.POINTER(vp), vp, ctypes.c_int, ctypes.c_uint64, vp]
    L.cm_surrogate_destroy.argtypes = [vp]
    L.cm_surrogate_mlp.argtypes = [vp, ctypes.POINTER(vp)]
    L.cm_surrogate_generate.argtypes = [vp, vp, vp, i64, ctypes.POINTER(Stimulus), i64, i64, ctypes.POINTER(i64)]
    L.cm_surrogate_dataset.argtypes = [vp, ctypes.POINTER(i64), vp, vp]
    L.cm_surrogate_fit.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_uint64, fp]
    L.cm_surrogate_reset_network.argtypes = [vp, ctypes.c_uint64]
    L.cm_surrogate_blob_size.argtypes = [vp]
    L.cm_surrogate_blob_size.restype = ctypes.c_int64
    L.cm_surrogate_get_blob.argtypes = [vp, vp]
    L.cm_surrogate_set_blob.argtypes = [vp, vp]
    L.cm_batch_run_surrogate.argtypes = [vp, vp, vp, i64, ctypes.POINTER(Stimulus), ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(SurrogateStats)]
    L.cm_diag_fma_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double), vp]
    L.cm_diag_umma_tile.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, vp, vp]
    L.cm_diag_mlp_workspace_rows.argtypes = [vp, ctypes.POINTER(i64)]
    L.cm_diag_batch_wait_check.argtypes = [vp, i64, ctypes.c_uint32]
    L.cm_diag_fp64_math.argtypes = [vp, vp, i64, vp, vp]
    L.cm_diag_pair_convert.argtypes = [vp, i64, vp, vp, vp, vp, vp]
    L.cm_model_print_names.argtypes = [ctypes.c_int, ctypes.c_int, vp, ctypes.c_int]
    L.cm_batch_print_values.argtypes = [vp, i64, ctypes.c_double, ctypes.c_int, dp, ctypes.c_int]
    L.cm_batch_get_cell.argtypes = [vp, i64, ctypes.c_int, dp]
    L.cm_batch_set_cell.argtypes = [vp, i64, ctypes.c_int, dp]
    L.cm_batch_calc_cell.argtypes = [vp, i64, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp]
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise CMError(rc, lib().cm_last_error().decode())


def _ptr(a):
    """Raw address of a numpy array, a torch tensor (host or device) or None."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


def _f64(a, n, name):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != n:
            raise ValueError(f"{name}: need a contiguous float64 array of {n} elements")
        return a
    import torch  # device tensors are plumbing only
    if a.dtype != torch.float64 or not a.is_contiguous() or a.numel() != n:
        raise ValueError(f"{name}: need a contiguous float64 tensor of {n} elements")
    return a


def _per_cell_times(a, n):
    """Per-cell first stimulus times: None, a float64 numpy array or tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray) or not hasattr(a, "data_ptr"):
        return _f64(np.ascontiguousarray(a, np.float64), n, "textbegin_per_cell")
    return _f64(a, n, "textbegin_per_cell")


def fma_peak_tflops(fp64: bool, stream=None) -> float:
    """Measured dense FMA rate of the current GPU (TFLOP/s), FP64 or FP32."""
    v = ctypes.c_double()
    _check(lib().cm_diag_fma_peak(int(fp64), ctypes.byref(v), None if stream is None else ctypes.c_void_p(int(stream))))
    return v.value


def fp64_math(x, y):
    """The FP64 cell-model steps' exp(x), log(y) and x / y beside the CUDA library's, for float64
    CUDA tensors x, y of one length: returns a (6, n) float64 numpy array, rows exp64, log64,
    div64, exp, log, division."""
    if x.shape != y.shape or str(x.dtype) != "torch.float64" or str(y.dtype) != "torch.float64" \
            or not x.is_cuda or not y.is_cuda:
        raise ValueError("fp64_math: x and y must be float64 CUDA tensors of one shape")
    x, y = x.contiguous(), y.contiguous()
    out = x.new_empty((x.numel(), 6))
    _check(lib().cm_diag_fp64_math(_ptr(x), _ptr(y), x.numel(), _ptr(out), None))
    return out.cpu().numpy().T.copy()


def pair_convert(x):
    """The mixed kernels' double <-> (hi, lo) FP32 pair conversions on a float64 CUDA tensor x:
    returns numpy arrays hi, lo (float32), back = hi + lo and widened = (double)(float)x (float64)."""
    import torch
    if str(x.dtype) != "torch.float64" or not x.is_cuda:
        raise ValueError("pair_convert: x must be a float64 CUDA tensor")
    x = x.contiguous()
    n = x.numel()
    hi = torch.empty(n, dtype=torch.float32, device=x.device)
    lo = torch.empty_like(hi)
    back = torch.empty(n, dtype=torch.float64, device=x.device)
    wid = torch.empty_like(back)
    _check(lib().cm_diag_pair_convert(_ptr(x), n, _ptr(hi), _ptr(lo), _ptr(back), _ptr(wid), None))
    return hi.cpu().numpy(), lo.cpu().numpy(), back.cpu().numpy(), wid.cpu().numpy()


def model_info(model: int) -> Info:
    info = Info()
    _check(lib().cm_model_info(model, ctypes.byref(info)))
    return info


def state_names(model: int) -> list[str]:
    return [lib().cm_state_name(model, k).decode() for k in range(model_info(model).n_state_vars)]


class Params:
    """Parameter set + lookup tables for one (model, .ev file, dt): initElphyParameters."""

    def __init__(self, model: int | str, ev_path: str | None = None, dt: float = 1e-5):
        if isinstance(model, str):
            m = lib().cm_model_from_name(model.encode())
            if m < 0:
                raise CMError(-2, f"unknown model {model}")
            model = m
        h = ctypes.c_void_p()
        _check(lib().cm_params_create(ctypes.byref(h), model, ev_path.encode() if ev_path else None, dt))
        self._h = h
        self.model = model

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.cm_params_destroy(self._h)
            self._h = None

    @property
    def info(self) -> Info:
        info = Info()
        _check(lib().cm_params_info(self._h, ctypes.byref(info)))
        return info

    def get(self, name: str) -> float:
        v = ctypes.c_double()
        _check(lib().cm_params_get(self._h, name.encode(), ctypes.byref(v)))
        return v.value

    def set(self, name: str, value: float) -> None:
        _check(lib().cm_params_set(self._h, name.encode(), value))

    def table(self, name: str) -> np.ndarray:
        out = np.zeros(self.info.table_rows)
        _check(lib().cm_params_table(self._h, name.encode(), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out


class Batch:
    """n_cells cells of one model on the GPU: initElphyModel x n + Init()."""

    def __init__(self, params: Params, n_cells: int, precision: int = FP64, stream=None):
        h = ctypes.c_void_p()
        s = None if stream is None else ctypes.c_void_p(int(stream))
        _check(lib().cm_batch_create(ctypes.byref(h), params._h, int(n_cells), precision, s))
        self._h = h
        self.n = int(n_cells)
        self.model = params.model
        self.precision = precision
        self.info = params.info

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.cm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def reset(self):
        _check(lib().cm_batch_reset(self._h))

    def add_hetero_value(self, name: str, values) -> None:
        v = None if values is None else _f64(np.ascontiguousarray(values, np.float64)
                                             if not hasattr(values, "data_ptr") else values, self.n, name)
        _check(lib().cm_batch_set_hetero(self._h, name.encode(), _ptr(v)))

    def set_diagnostics(self, on: bool) -> None:
        _check(lib().cm_batch_set_diagnostics(self._h, int(on)))

    def init_vm(self) -> np.ndarray:
        out = np.zeros(self.n)
        _check(lib().cm_batch_init_vm(self._h, _ptr(out)))
        return out

    def get_state(self, layout: int = LAYOUT_SOA) -> np.ndarray:
        k = self.info.n_state_vars if layout == LAYOUT_SOA else self.info.ref_block_doubles
        out = np.zeros(k * self.n)
        _check(lib().cm_batch_get_state(self._h, layout, _ptr(out)))
        return out.reshape((k, self.n) if layout == LAYOUT_SOA else (self.n, k))

    def set_state(self, buf, layout: int = LAYOUT_SOA) -> None:
        b = np.ascontiguousarray(buf, np.float64)
        _check(lib().cm_batch_set_state(self._h, layout, _ptr(b)))

    def calc(self, dt, Vm, i_ext=None, stretch=None, dVm=None):
        """One reference Calc per cell; returns dVm (host numpy unless device dVm given)."""
        Vm = _f64(Vm, self.n, "Vm")
        i_ext = _f64(i_ext, self.n, "i_ext")
        stretch = _f64(stretch, self.n, "stretch")
        if dVm is None:
            dVm = np.zeros(self.n)
        _check(lib().cm_batch_step(self._h, dt, _ptr(Vm), _ptr(i_ext), _ptr(stretch), _ptr(dVm)))
        return dVm

    def calc_update(self, dt, Vm, i_ext=None, stretch=None, vm_range=0.0):
        """One Calc per cell fused with Vm += dVm and the NaN/range check; Vm updated in place."""
        Vm = _f64(Vm, self.n, "Vm")
        i_ext = _f64(i_ext, self.n, "i_ext")
        stretch = _f64(stretch, self.n, "stretch")
        _check(lib().cm_batch_step_update(self._h, dt, _ptr(Vm), _ptr(i_ext), _ptr(stretch), vm_range))

    def calc_update_act(self, dt, Vm, act_time, t, threshold, i_ext=None, stretch=None, vm_range=0.0):
        """calc_update plus activation times: act_time (float64, -1 = not yet activated) gets t
        for every cell whose new Vm reaches threshold; updated in place."""
        Vm = _f64(Vm, self.n, "Vm")
        act_time = _f64(act_time, self.n, "act_time")
        i_ext = _f64(i_ext, self.n, "i_ext")
        stretch = _f64(stretch, self.n, "stretch")
        _check(lib().cm_batch_step_update_act(self._h, dt, _ptr(Vm), _ptr(i_ext), _ptr(stretch), vm_range,
                                              _ptr(act_time), t, threshold))

    def run(self, Vm, n_steps, *, textbegin=0.0, textlen=1e-3, bcl=1.0, amplitude=0.0, t0=0.0,
            textbegin_per_cell=None, probe_cells=None, probe_every=0):
        """Fused driver loop; Vm (host numpy or device tensor) updated in place. Returns the
        probe traces (n_probe, n_rec) when probe_cells is given."""
        Vm = _f64(Vm, self.n, "Vm")
        tbc = _per_cell_times(textbegin_per_cell, self.n)
        st = Stimulus(t0, textbegin, None if tbc is None else ctypes.cast(_ptr(tbc), ctypes.POINTER(ctypes.c_double)),
                      textlen, bcl, amplitude)
        pc = None
        n_probe = 0
        trace = None
        if probe_cells is not None:
            pc = np.ascontiguousarray(probe_cells, np.int64)
            n_probe = pc.size
            n_rec = (n_steps + probe_every - 1) // probe_every
            trace = np.zeros((n_probe, n_rec))
        _check(lib().cm_batch_run(self._h, _ptr(Vm), int(n_steps), ctypes.byref(st), _ptr(pc), n_probe,
                                  int(probe_every), _ptr(trace)))
        return trace

    def autotune(self, n_trial_steps: int = 20):
        """Pick the fastest launch shape on this batch; returns (variant*100 + grid_mode, ms/step)."""
        v = ctypes.c_int()
        ms = ctypes.c_double()
        _check(lib().cm_batch_autotune(self._h, n_trial_steps, ctypes.byref(v), ctypes.byref(ms)))
        return v.value, ms.value

    def set_launch(self, variant: int, grid_mode: int = 0) -> None:
        _check(lib().cm_batch_set_launch(self._h, variant, grid_mode))

    def run_surrogate(self, surrogate, Vm, n_macro, *, textbegin=0.0, textlen=1e-3, bcl=1.0, amplitude=0.0,
                      t0=0.0, mode=0, audit_mod=100, textbegin_per_cell=None):
        """n_macro learned macro steps (surrogate.substeps fine steps each); Vm updated in place.
        mode 0: coarse step + network, SUR_COARSE_ONLY: coarse step alone; | SUR_AUDIT_FP64: the
        audit sample is integrated in FP64. Returns the run statistics."""
        Vm = _f64(Vm, self.n, "Vm")
        tbc = _per_cell_times(textbegin_per_cell, self.n)
        st = Stimulus(t0, textbegin, None if tbc is None else ctypes.cast(_ptr(tbc), ctypes.POINTER(ctypes.c_double)),
                      textlen, bcl, amplitude)
        stats = SurrogateStats()
        _check(lib().cm_batch_run_surrogate(self._h, surrogate._h, _ptr(Vm), int(n_macro), ctypes.byref(st), mode,
                                            audit_mod, ctypes.byref(stats)))
        return stats.as_dict()

    def run_diffuse(self, diffusion, Vm, n_steps, *, textbegin=0.0, textlen=1e-3, bcl=1.0, amplitude=0.0,
                    t0=0.0, textbegin_per_cell=None, vm_range=0.0, act=None, act_threshold=-0.02):
        """n_steps monodomain steps coupled by `diffusion` (acCELLerate::IntraStep's explicit
        path): i_ext = scale * (A Vm) + stimulus, Vm += Calc(...), range check, activation
        times in `act` (float64, -1 = not yet). Vm and act updated in place."""
        Vm = _f64(Vm, self.n, "Vm")
        act = _f64(act, self.n, "act")
        tbc = _per_cell_times(textbegin_per_cell, self.n)
        st = Stimulus(t0, textbegin, None if tbc is None else ctypes.cast(_ptr(tbc), ctypes.POINTER(ctypes.c_double)),
                      textlen, bcl, amplitude)
        _check(lib().cm_batch_run_diffuse(self._h, diffusion._h, _ptr(Vm), int(n_steps), ctypes.byref(st),
                                          vm_range, _ptr(act), act_threshold))

    def run_theta(self, theta, Vm, n_steps, *, textbegin=0.0, textlen=1e-3, bcl=1.0, amplitude=0.0, t0=0.0,
                  textbegin_per_cell=None, vm_range=0.0, act=None, act_threshold=-0.02):
        """n_steps implicit finite-element monodomain steps (acCELLerate::IntraStep with IntraRHS):
        cell update with the stimulus, Vm += dVm, range check, the solve of `theta`, activation
        times. Vm and act updated in place; returns the solves' statistics."""
        Vm = _f64(Vm, self.n, "Vm")
        act = _f64(act, self.n, "act")
        tbc = _per_cell_times(textbegin_per_cell, self.n)
        st = Stimulus(t0, textbegin, None if tbc is None else ctypes.cast(_ptr(tbc), ctypes.POINTER(ctypes.c_double)),
                      textlen, bcl, amplitude)
        stats = ThetaStats()
        _check(lib().cm_batch_run_theta(self._h, theta._h, _ptr(Vm), int(n_steps), ctypes.byref(st), vm_range,
                                        _ptr(act), act_threshold, ctypes.byref(stats)))
        return stats.as_dict()

    def audit(self, per_cell: bool = False):
        m = ctypes.c_uint32()
        pc = np.zeros(self.n, np.uint32) if per_cell else None
        _check(lib().cm_batch_audit(self._h, ctypes.byref(m), _ptr(pc)))
        return (m.value, pc) if per_cell else m.value


class Diffusion:
    """The monodomain coupling operator: Intra.A (CSR) and the per-node conversion of A*Vm to
    the cell model's i_external (the reference's -Volume()/volume_local*1e9)."""

    def __init__(self, rowptr, col, val, scale=None, uniform_scale=1.0):
        rowptr = np.ascontiguousarray(rowptr, np.int64)
        col = np.ascontiguousarray(col, np.int32)
        val = np.ascontiguousarray(val, np.float64)
        n = rowptr.size - 1
        sc = None if scale is None else np.ascontiguousarray(scale, np.float64)
        if sc is not None and sc.size != n:
            raise ValueError("scale: need one value per row")
        if col.size != val.size or (n >= 0 and col.size < (rowptr[-1] if n > 0 else 0)):
            raise ValueError("col/val shorter than rowptr[-1]")
        h = ctypes.c_void_p()
        _check(lib().cm_diffusion_create(ctypes.byref(h), n, _ptr(rowptr), _ptr(col), _ptr(val), _ptr(sc),
                                         float(uniform_scale)))
        self._h = h
        self.n = n

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.cm_diffusion_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def apply(self, x, y=None):
        """y = scale * (A x) in FP64 on the GPU."""
        x = _f64(x if hasattr(x, "data_ptr") else np.ascontiguousarray(x, np.float64), self.n, "x")
        if y is None:
            y = np.zeros(self.n)
        _check(lib().cm_diffusion_apply(self._h, _ptr(x), _ptr(y)))
        return y


class Theta:
    """The implicit finite-element step's solve (acCELLerate::IntraStep with IntraRHS): x <- A^-1 (R x)
    by Jacobi-preconditioned conjugate gradients in FP64. lhs, rhs: Diffusion operators of A and R
    built with uniform_scale 1 (kept alive by this object)."""

    def __init__(self, lhs, rhs, rtol=1e-6, atol=1e-6, max_iter=1000):
        self.lhs, self.rhs = lhs, rhs
        h = ctypes.c_void_p()
        _check(lib().cm_theta_create(ctypes.byref(h), lhs._h, rhs._h, float(rtol), float(atol), int(max_iter)))
        self._h = h
        self.n = lhs.n

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.cm_theta_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def solve(self, x):
        """x <- A^-1 (R x) in place (float64 array or tensor); returns the solve's statistics."""
        x = _f64(x, self.n, "x")
        stats = ThetaStats()
        _check(lib().cm_theta_solve(self._h, _ptr(x), ctypes.byref(stats)))
        return stats.as_dict()


class Multi:
    """Batched form: several MIXED batches (any sizes; TenTusscher2 and Courtemanche) advanced in lock step by one
    persistent launch per time step, replayed from a CUDA graph."""

    def __init__(self, batches, stream=None):
        self.batches = list(batches)
        arr = (ctypes.c_void_p * len(self.batches))(*[b._h.value for b in self.batches])
        h = ctypes.c_void_p()
        s = None if stream is None else ctypes.c_void_p(int(stream))
        _check(lib().cm_multi_create(ctypes.byref(h), arr, len(self.batches), s))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.cm_multi_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def run(self, vms, n_steps, stims):
        """vms: one float64 array/tensor per instance (updated in place); stims: one dict per
        instance with keys textbegin, textlen, bcl, amplitude (optional t0)."""
        vs = [_f64(v, b.n, "Vm") for v, b in zip(vms, self.batches)]
        ptrs = (ctypes.c_void_p * len(vs))(*[_ptr(v) for v in vs])
        st = (Stimulus * len(vs))(*[Stimulus(d.get("t0", 0.0), d.get("textbegin", 0.0), None, d.get("textlen", 1e-3),
                                             d.get("bcl", 1.0), d.get("amplitude", 0.0)) for d in stims])
        _check(lib().cm_multi_run(self._h, ptrs, int(n_steps), st))

    def autotune(self, n_trial_steps=5):
        t, sh, bps, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _check(lib().cm_multi_autotune(self._h, n_trial_steps, ctypes.byref(t), ctypes.byref(sh), ctypes.byref(bps),
                                       ctypes.byref(ms)))
        return {"tile_cells": t.value, "shape": sh.value, "blocks_per_sm": bps.value, "ms_per_step": ms.value}

    def set_launch(self, tile_cells, shape=0, blocks_per_sm=2):
        _check(lib().cm_multi_set_launch(self._h, tile_cells, shape, blocks_per_sm))


def _backup_args(batches, vms, node_ids):
    batches = list(batches)
    parts = (ctypes.c_void_p * len(batches))(*[b._h.value for b in batches])
    vs = [_f64(v, b.n, "Vm") for v, b in zip(vms, batches)]
    vptr = (ctypes.c_void_p * len(vs))(*[_ptr(v) for v in vs])
    ids = None
    if node_ids is not None:
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.int64) for a in node_ids]
        for a, b in zip(arrs, batches):
            if a is not None and a.size != b.n:
                raise ValueError("node_ids: one index per cell of its part")
        ids = (ctypes.c_void_p * len(arrs))(*[None if a is None else a.ctypes.data for a in arrs])
        ids._keep = arrs
    return batches, parts, vptr, ids


def backup_write(path, time_str, batches, vms, node_ids=None):
    """acCELLerate backup file (acCELLerate.cpp:1616-1661) of the parts' nodes: header lines, then
    per node its Vm and its cell model's reference block. node_ids: per part the global index of
    each of its cells, or None for consecutive parts."""
    batches, parts, vptr, ids = _backup_args(batches, vms, node_ids)
    _check(lib().cm_backup_write(str(path).encode(), str(time_str).encode(), len(batches), parts, ids, vptr))


def backup_read(path, batches, vms, node_ids=None) -> str:
    """Reads an acCELLerate backup file (acCELLerate.cpp:1511-1614) into the parts' states and Vm
    arrays; returns its time string."""
    batches, parts, vptr, ids = _backup_args(batches, vms, node_ids)
    buf = ctypes.create_string_buffer(64)
    _check(lib().cm_backup_read(str(path).encode(), len(batches), parts, ids, vptr, buf, 64))
    return buf.value.decode()


def _f32(a, n, name):
    if isinstance(a, np.ndarray):
        if a.dtype != np.float32 or not a.flags.c_contiguous or a.size != n:
            raise ValueError(f"{name}: need a contiguous float32 array of {n} elements")
        return a
    if a.numel() != n or not a.is_contiguous():
        raise ValueError(f"{name}: need a contiguous float32 tensor of {n} elements")
    return a


class Mlp:
    """The surrogate's network: n_in -> H -> H -> n_out, tanh, BF16 tensor-core GEMMs, FP32 Adam."""

    def __init__(self, n_in=22, n_hidden=128, n_out=19, seed=1, stream=None, _borrow=None):
        self.n_in, self.n_hidden, self.n_out = n_in, n_hidden, n_out
        if _borrow is not None:
            self._h, self._owned = _borrow, False
        else:
            h = ctypes.c_void_p()
            s = None if stream is None else ctypes.c_void_p(int(stream))
            _check(lib().cm_mlp_create(ctypes.byref(h), n_in, n_hidden, n_out, seed, s))
            self._h, self._owned = h, True
        self.n_params = int(lib().cm_mlp_n_params(self._h))

    def __del__(self):
        if getattr(self, "_owned", False) and getattr(self, "_h", None) and _lib is not None:
            _lib.cm_mlp_destroy(self._h)
            self._h = None

    def shapes(self):
        H = self.n_hidden
        return [(H, self.n_in), (H,), (H, H), (H,), (self.n_out, H), (self.n_out,)]

    def _split(self, flat):
        out, k = [], 0
        for shp in self.shapes():
            n = int(np.prod(shp))
            out.append(flat[k:k + n].reshape(shp))
            k += n
        return out

    def get_params(self):
        out = np.zeros(self.n_params, np.float32)
        _check(lib().cm_mlp_get_params(self._h, out.ctypes.data))
        return self._split(out)

    def set_params(self, params):
        flat = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float32).ravel() for p in params]))
        _check(lib().cm_mlp_set_params(self._h, flat.ctypes.data))

    def get_grads(self):
        out = np.zeros(self.n_params, np.float32)
        _check(lib().cm_mlp_get_grads(self._h, out.ctypes.data))
        return self._split(out)

    def forward(self, X):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros((X.shape[0], self.n_out), np.float32)
        _check(lib().cm_mlp_forward(self._h, X.ctypes.data, X.shape[0], Y.ctypes.data))
        return Y

    def loss_grad(self, X, T):
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        loss = ctypes.c_float()
        _check(lib().cm_mlp_loss_grad(self._h, X.ctypes.data, T.ctypes.data, X.shape[0], ctypes.byref(loss)))
        return loss.value

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        _check(lib().cm_mlp_adam_step(self._h, lr, beta1, beta2, eps))


class Surrogate:
    """Learned macro step for TenTusscher2 (coarse physics step of substeps*dt + MLP residual)."""

    def __init__(self, params: Params, substeps=10, seed=1, stream=None):
        h = ctypes.c_void_p()
        s = None if stream is None else ctypes.c_void_p(int(stream))
        _check(lib().cm_surrogate_create(ctypes.byref(h), params._h, substeps, seed, s))
        self._h = h
        self.substeps = substeps
        m = ctypes.c_void_p()
        _check(lib().cm_surrogate_mlp(self._h, ctypes.byref(m)))
        self.mlp = Mlp(_borrow=m)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            self.mlp = None
            _lib.cm_surrogate_destroy(self._h)
            self._h = None

    def generate(self, batch, Vm, n_macro, *, textbegin=0.0, textlen=1e-3, bcl=1.0, amplitude=0.0, t0=0.0,
                 cell_stride=1, max_pairs=10_000_000):
        Vm = _f64(Vm, batch.n, "Vm")
        st = Stimulus(t0, textbegin, None, textlen, bcl, amplitude)
        n = ctypes.c_int64()
        _check(lib().cm_surrogate_generate(self._h, batch._h, _ptr(Vm), int(n_macro), ctypes.byref(st),
                                           int(cell_stride), int(max_pairs), ctypes.byref(n)))
        return n.value

    def dataset(self):
        n = ctypes.c_int64()
        _check(lib().cm_surrogate_dataset(self._h, ctypes.byref(n), None, None))
        X = np.zeros((n.value, 22), np.float32)
        T = np.zeros((n.value, 19), np.float32)
        _check(lib().cm_surrogate_dataset(self._h, ctypes.byref(n), X.ctypes.data, T.ctypes.data))
        return X, T

    def fit(self, batch=4096, steps=2000, lr=1e-3, seed=1):
        loss = ctypes.c_float()
        _check(lib().cm_surrogate_fit(self._h, batch, steps, lr, seed, ctypes.byref(loss)))
        return loss.value

    def reset_network(self, seed):
        """Fresh network weights from seed, optimiser state cleared; the dataset is kept."""
        _check(lib().cm_surrogate_reset_network(self._h, int(seed)))

    def flush_audit(self, mode=0):
        """Audit the last run's pending sample now; returns its statistics."""
        st = SurrogateStats()
        _check(lib().cm_surrogate_flush_audit(self._h, int(mode), ctypes.byref(st)))
        return st.as_dict()

    def get_blob(self):
        out = np.zeros(int(lib().cm_surrogate_blob_size(self._h)), np.float32)
        _check(lib().cm_surrogate_get_blob(self._h, out.ctypes.data))
        return out

    def set_blob(self, blob):
        b = np.ascontiguousarray(blob, np.float32)
        _check(lib().cm_surrogate_set_blob(self._h, b.ctypes.data))
