"""Test infrastructure: the CPU checkers for the cell-model update.

Two implementations, both FP64 on the CPU:

* ``Port``  -- oracle/cm_oracle.c, a plain-C restatement of the reference's
  TenTusscher2 / Courtemanche / OHaraRudy / Tomek Calc and InitTable (see that file for file:line
  citations). Builds anywhere with gcc; it is the checker on machines without the
  reference tree and the timed CPU baseline.
* ``Ref``   -- oracle/_ref/libcmref.so, the reference's own CellModel library compiled
  from its sources (oracle/Makefile target ``ref``) behind oracle/ref_harness.cpp.
  Only available where the reference tree exists; used to pin ``Port`` and to
  generate the golden vectors under tests/golden/.

Only tests/, bench.py's CPU-baseline leg and __graft_entry__.smoke() import this
package, and only as the checker.
"""
from __future__ import annotations

import ctypes
import json
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_SO = HERE / "_build" / "libcmoracle.so"
REF_SO = HERE / "_ref" / "libcmref.so"
REF_TREE = Path(os.environ.get("CM_REFERENCE_TREE", "/root/reference"))
GOLDEN = HERE.parent / "tests" / "golden"

TT2, CRN, ORD, TOM = 0, 1, 2, 3
MODEL_NAMES = {TT2: "TenTusscher2", CRN: "CourtemancheEtAl", ORD: "OHaraRudy", TOM: "Tomek"}
# Reference ElphyModelType values (ElphyModelBasis.h:62-81).
REF_EMT = {TT2: 5, CRN: 2, ORD: 12, TOM: 14}
# O'Hara-Rudy and Tomek cell types of the reference's parameter files (celltype 0 / 1 / 2).
ORD_VARIANTS = ("endo", "epi", "mid")
TOM_VARIANTS = ORD_VARIANTS
RTDT = 4000

_dp = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_dp)


def build_port() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "port"], check=True)
    return PORT_SO


def build_ref() -> Path | None:
    """Compile the reference CellModel library; None where the reference tree is absent."""
    if not (REF_TREE / "electrophysiology" / "src" / "CellModel").is_dir():
        return None
    subprocess.run(["make", "-s", "-j8", "-C", str(HERE), "ref", f"REF={REF_TREE}"], check=True)
    return REF_SO


def load_params(model: int, variant: str = "epi") -> dict:
    """Resolved reference parameter set (names -> FP64 values) from the golden fixture.
    For O'Hara-Rudy, variant is the cell type (endo, epi, mid); the other models have one set."""
    if model in (ORD, TOM):
        name = f"params_{'ord' if model == ORD else 'tom'}_{variant}.json"
    else:
        name = "params_tt2_epi.json" if model == TT2 else "params_crn.json"
    with open(GOLDEN / name) as f:
        return json.load(f)["params"]


class Port:
    """ctypes view of oracle/cm_oracle.c."""

    def __init__(self):
        if not PORT_SO.exists():
            build_port()
        L = ctypes.CDLL(str(PORT_SO))
        L.cmo_param_name.restype = ctypes.c_char_p
        L.cmo_table_name.restype = ctypes.c_char_p
        L.cmo_param_index.argtypes = [ctypes.c_int, ctypes.c_char_p]
        L.cmo_derive.argtypes = [ctypes.c_int, _dp]
        L.cmo_build_tables.argtypes = [ctypes.c_int, _dp, ctypes.c_double, _dp]
        L.cmo_init_state.argtypes = [ctypes.c_int, _dp, _dp]
        L.cmo_init_vm.argtypes = [ctypes.c_int, _dp]
        L.cmo_init_vm.restype = ctypes.c_double
        L.cmo_calc.argtypes = [ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, ctypes.c_double,
                               ctypes.c_double, ctypes.c_double]
        L.cmo_calc.restype = ctypes.c_double
        _lp = ctypes.POINTER(ctypes.c_long)
        _ip = ctypes.POINTER(ctypes.c_int)
        L.cmo_mono_run.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_long, _dp, _dp, ctypes.c_int, _ip, _dp, _lp,
                                   _ip, _dp, _dp, ctypes.c_double, ctypes.c_long, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, _dp, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_long, _dp,
                                   ctypes.c_int]
        L.cmo_run.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_long, _dp, _dp, ctypes.c_int,
                              ctypes.POINTER(ctypes.c_int), _dp, ctypes.c_long, ctypes.c_double,
                              ctypes.c_double, ctypes.c_double, _dp, ctypes.c_double, ctypes.c_double,
                              ctypes.c_double, ctypes.c_long, _dp, ctypes.c_int]
        self.L = L

    def param_names(self, model):
        return [self.L.cmo_param_name(model, i).decode() for i in range(self.L.cmo_n_params(model))]

    def table_names(self, model):
        return [self.L.cmo_table_name(model, k).decode() for k in range(self.L.cmo_n_tables(model))]

    def state_doubles(self, model):
        return self.L.cmo_state_doubles(model)

    def param_vector(self, model, values: dict) -> np.ndarray:
        """Base values by name (missing base names are an error), derived slots recomputed."""
        names = self.param_names(model)
        P = np.zeros(len(names))
        for i, n in enumerate(names):
            if n in values:
                P[i] = values[n]
        self.L.cmo_derive(model, _ptr(P))
        return P

    def tables(self, model, P, dt) -> np.ndarray:
        T = np.zeros((self.L.cmo_n_tables(model), RTDT))
        rc = self.L.cmo_build_tables(model, _ptr(P), dt, _ptr(T))
        assert rc == 0
        return T

    def init_state(self, model, P, n_cells) -> np.ndarray:
        ns = self.state_doubles(model)
        B = np.zeros((n_cells, ns))
        one = np.zeros(ns)
        self.L.cmo_init_state(model, _ptr(P), _ptr(one))
        B[:] = one
        return B

    def init_vm(self, model, P) -> float:
        return self.L.cmo_init_vm(model, _ptr(P))

    def calc(self, model, P, T, blocks, dt, Vm, i_ext, stretch=1.0, het=None):
        """One Calc per cell; blocks updated in place; returns dVm."""
        n = blocks.shape[0]
        dV = np.zeros(n)
        for c in range(n):
            Pc = P
            if het:
                Pc = P.copy()
                for name, vals in het.items():
                    Pc[self.L.cmo_param_index(model, name.encode())] = vals[c]
            row = np.ascontiguousarray(blocks[c])
            dV[c] = self.L.cmo_calc(model, _ptr(Pc), _ptr(T), _ptr(row), dt, float(Vm[c]),
                                    float(i_ext[c]), stretch)
            blocks[c] = row
        return dV

    def run(self, model, P, T, blocks, Vm, n_steps, dt, *, t0=0.0, textbegin=0.0, textlen=1e-3,
            bcl=1.0, amp=0.0, het=None, textbegin_per_cell=None, rec_every=0, n_threads=1):
        """Driver loop (CellModel.h:405-420) over all cells; blocks and Vm updated in place.
        Returns the Vm trace (n_cells, n_rec) when rec_every > 0."""
        n = blocks.shape[0]
        assert blocks.flags.c_contiguous and Vm.flags.c_contiguous
        het = het or {}
        idx = (ctypes.c_int * max(1, len(het)))(*[self.L.cmo_param_index(model, k.encode()) for k in het])
        assert all(i >= 0 for i in list(idx)[:len(het)]), "unknown hetero parameter"
        hv = np.ascontiguousarray(np.stack([np.asarray(v, np.float64) for v in het.values()])) if het else None
        n_rec = (n_steps + rec_every - 1) // rec_every if rec_every > 0 else 0
        trace = np.zeros((n, n_rec)) if n_rec else None
        tbc = None if textbegin_per_cell is None else np.ascontiguousarray(textbegin_per_cell, np.float64)
        rc = self.L.cmo_run(model, _ptr(P), _ptr(T), n, _ptr(blocks), _ptr(Vm), len(het), idx, _ptr(hv),
                            n_steps, dt, t0, textbegin, _ptr(tbc), textlen, bcl, amp, rec_every,
                            _ptr(trace), n_threads)
        if rc != 0:
            raise FloatingPointError(f"oracle run failed rc={rc}")
        return trace


    def mono_run(self, model, P, T, blocks, Vm, n_steps, dt, rowptr, col, val, *, scale=None,
                 uniform_scale=1.0, t0=0.0, textbegin=0.0, textbegin_per_cell=None, textlen=1e-3, bcl=1.0,
                 amp=0.0, het=None, act=None, act_threshold=-0.02, vm_range=0.0, rec_every=0, n_threads=1):
        """Explicit monodomain steps (acCELLerate::IntraStep, Godunov): B = A Vm in CSR order,
        i_ext = B * scale + stimulus, Vm += Calc. blocks, Vm and act updated in place; returns
        the Vm trace (n_cells, n_rec) when rec_every > 0."""
        n = blocks.shape[0]
        assert blocks.flags.c_contiguous and Vm.flags.c_contiguous
        het = het or {}
        idx = (ctypes.c_int * max(1, len(het)))(*[self.L.cmo_param_index(model, k.encode()) for k in het])
        assert all(i >= 0 for i in list(idx)[:len(het)]), "unknown hetero parameter"
        hv = np.ascontiguousarray(np.stack([np.asarray(v, np.float64) for v in het.values()])) if het else None
        rp = np.ascontiguousarray(rowptr, np.int64).astype(np.dtype("l"))
        cl = np.ascontiguousarray(col, np.int32).astype(np.intc)
        vl = np.ascontiguousarray(val, np.float64)
        sc = None if scale is None else np.ascontiguousarray(scale, np.float64)
        tbc = None if textbegin_per_cell is None else np.ascontiguousarray(textbegin_per_cell, np.float64)
        n_rec = (n_steps + rec_every - 1) // rec_every if rec_every > 0 else 0
        trace = np.zeros((n, n_rec)) if n_rec else None
        if act is not None:
            assert act.dtype == np.float64 and act.flags.c_contiguous and act.size == n
        rc = self.L.cmo_mono_run(model, _ptr(P), _ptr(T), n, _ptr(blocks), _ptr(Vm), len(het), idx, _ptr(hv),
                                 rp.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                                 cl.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _ptr(vl), _ptr(sc),
                                 uniform_scale, n_steps, dt, t0, textbegin, _ptr(tbc), textlen, bcl, amp, _ptr(act),
                                 act_threshold, vm_range, rec_every, _ptr(trace), n_threads)
        if rc != 0:
            raise FloatingPointError(f"oracle monodomain run failed rc={rc}")
        return trace


class Ref:
    """ctypes view of the reference library (oracle/_ref/libcmref.so)."""

    def __init__(self):
        if not REF_SO.exists():
            if build_ref() is None:
                raise FileNotFoundError("reference tree not present; oracle/_ref cannot be built")
        os.environ.setdefault("kaRootDir", str(REF_TREE))
        L = ctypes.CDLL(str(REF_SO))
        L.ref_create.restype = ctypes.c_void_p
        L.ref_create.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_double, ctypes.c_int]
        L.ref_last_error.restype = ctypes.c_char_p
        for f in ("ref_init_vm", "ref_amplitude", "ref_stim_time"):
            getattr(L, f).restype = ctypes.c_double
            getattr(L, f).argtypes = [ctypes.c_void_p]
        L.ref_destroy.argtypes = [ctypes.c_void_p]
        L.ref_add_hetero.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _dp]
        L.ref_state_doubles.argtypes = [ctypes.c_void_p]
        L.ref_get_state.argtypes = [ctypes.c_void_p, _dp]
        L.ref_set_state.argtypes = [ctypes.c_void_p, _dp]
        L.ref_calc.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp, _dp, ctypes.c_double, _dp]
        L.ref_run.argtypes = [ctypes.c_void_p, _dp, ctypes.c_long, ctypes.c_double, ctypes.c_double,
                              ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                              ctypes.c_long, _dp, ctypes.c_int]
        L.ref_n_params.argtypes = [ctypes.c_void_p]
        L.ref_param_name.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ref_param_name.restype = ctypes.c_char_p
        L.ref_param_value.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ref_param_value.restype = ctypes.c_double
        L.ref_table.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _dp]
        self.L = L

    @staticmethod
    def ev_path(model, variant="epi"):
        d = REF_TREE / "electrophysiology" / "data"
        if model in (ORD, TOM):
            return str(d / f"{MODEL_NAMES[model]}_{variant}.ev")
        return str(d / ("TenTusscher2_original_Epi.ev" if model == TT2 else "CourtemancheEtAl.ev"))

    def create(self, model, dt, n_cells, ev=None):
        return RefCells(self, model, ev or self.ev_path(model), dt, n_cells)


class RefCells:
    def __init__(self, ref: Ref, model, ev, dt, n_cells):
        self.ref, self.L, self.model, self.n = ref, ref.L, model, n_cells
        self.h = self.L.ref_create(REF_EMT[model], ev.encode(), dt, n_cells)
        if not self.h:
            raise RuntimeError(self.L.ref_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            self.L.ref_destroy(self.h)
            self.h = None

    def params(self) -> dict:
        return {self.L.ref_param_name(self.h, i).decode(): self.L.ref_param_value(self.h, i)
                for i in range(self.L.ref_n_params(self.h))}

    def table(self, name) -> np.ndarray:
        out = np.zeros(RTDT)
        rc = self.L.ref_table(self.h, name.encode(), _ptr(out))
        if rc < 0:
            raise KeyError(name)
        return out[:rc]

    def init_vm(self):
        return self.L.ref_init_vm(self.h)

    def add_hetero(self, name, values):
        v = np.ascontiguousarray(values, np.float64)
        rc = self.L.ref_add_hetero(self.h, name.encode(), _ptr(v))
        if rc != 0:
            raise ValueError(f"AddHeteroValue({name}) failed rc={rc}")

    def get_state(self):
        ns = self.L.ref_state_doubles(self.h)
        out = np.zeros((self.n, ns))
        self.L.ref_get_state(self.h, _ptr(out))
        return out

    def set_state(self, blocks):
        b = np.ascontiguousarray(blocks, np.float64)
        self.L.ref_set_state(self.h, _ptr(b))

    def calc(self, dt, Vm, i_ext, stretch=1.0):
        Vm = np.ascontiguousarray(Vm, np.float64)
        ie = np.ascontiguousarray(i_ext, np.float64)
        dV = np.zeros(self.n)
        self.L.ref_calc(self.h, dt, _ptr(Vm), _ptr(ie), stretch, _ptr(dV))
        return dV

    def run(self, Vm, n_steps, dt, *, t0=0.0, textbegin=0.0, textlen=1e-3, bcl=1.0, amp=0.0,
            rec_every=0, n_threads=1):
        n_rec = (n_steps + rec_every - 1) // rec_every if rec_every > 0 else 0
        trace = np.zeros((self.n, n_rec)) if n_rec else None
        rc = self.L.ref_run(self.h, _ptr(Vm), n_steps, dt, t0, textbegin, textlen, bcl, amp, rec_every,
                            _ptr(trace), n_threads)
        if rc != 0:
            raise FloatingPointError(f"reference run failed rc={rc}")
        return trace
