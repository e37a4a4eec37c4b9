"""GPU parity of the Tomek model (model 14) through the C ABI against the oracle and the golden
vectors of the reference's own Tomek class, for its three cell types.

Tolerances:
  FP64 batches  one Calc: rtol 1e-10 (CUDA's exp/log/pow differ from glibc by a few ulp, the
                kernel fuses multiply-adds and takes parameter-only products once on the host);
                two beats: |dVm| <= 1e-5 mV, APD90 and upstroke within 1e-3 ms of the oracle.
  mixed batches APD90 within 1 ms, upstroke within 0.1 ms, RMS Vm error <= 0.5 mV per cell.
"""
import json
import os

import numpy as np
import pytest

import oracle as O
from cardiomechanics_gb300 import analysis as A
from cardiomechanics_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOM = 14
DT = 1e-5
VARIANTS = list(O.TOM_VARIANTS)
SOA_BLOCK = [0, 3, 6] + list(range(7, 48))  # block slot of each SOA state (Tomek.h:33-44)


def tom_params(cm, variant, dt=DT):
    """The reference's Tomek_<variant>.ev: built-in endo values with the cell type's base values
    set by name (derived values recompute)."""
    p = cm.Params(TOM, None, dt)
    if variant != "endo":
        for name, v in O.load_params(O.TOM, variant).items():
            try:
                p.set(name, v)
            except cm.CMError:
                pass  # a derived value
    return p


@pytest.mark.parametrize("variant", VARIANTS)
def test_one_step_known_answers_fp64(gpu, variant):
    cm = gpu
    g = np.load(O.GOLDEN / f"step_tom_{variant}.npz")
    dt = float(g["dt"])
    p = tom_params(cm, variant, dt)
    n = g["state_in"].shape[0]
    b = cm.Batch(p, n, cm.FP64)
    b.set_diagnostics(True)
    b.set_state(g["state_in"], cm.LAYOUT_REF_BLOCK)
    for k, name in enumerate(g["hetero_names"]):
        b.add_hetero_value(str(name), p.get(str(name)) * g["hetero_scale"][k])
    dV = b.calc(dt, np.ascontiguousarray(g["vm"]), np.ascontiguousarray(g["i_ext"]))
    S = b.get_state(cm.LAYOUT_REF_BLOCK)
    ref = g["state_out"]
    # the 48 states and rates, then the 36 stored values
    np.testing.assert_allclose(S[:, :48], ref[:, :48], rtol=1e-10, atol=1e-250)
    scale = np.abs(ref[:, 48:]).max(axis=0)
    np.testing.assert_allclose(S[:, 48:], ref[:, 48:], rtol=1e-9, atol=1e-12 * scale.max())
    np.testing.assert_allclose(dV, g["dvm"], rtol=1e-9, atol=1e-16)
    assert b.audit() == 0


def run_pair(cm, port, variant, precision, n, steps, bcl, lo, hi, seed=1, rec=10):
    p = tom_params(cm, variant)
    b = cm.Batch(p, n, precision)
    sc = W.conductance_scales(seed, n, len(W.ORD_INSTANCE_G), lo, hi)
    names = port.param_names(O.TOM)
    P = port.param_vector(O.TOM, O.load_params(O.TOM, variant))
    het = {}
    for k, name in enumerate(W.ORD_INSTANCE_G):
        het[name] = P[names.index(name)] * sc[k]
        b.add_hetero_value(name, het[name])
    vm = b.init_vm()
    tr = b.run(vm, steps, textbegin=0.0, textlen=1e-3, bcl=bcl, amplitude=W.TOM_STIM, probe_cells=np.arange(n),
               probe_every=rec)
    B = port.init_state(O.TOM, P, n)
    vo = np.full(n, port.init_vm(O.TOM, P))
    tro = port.run(O.TOM, P, np.zeros((0, O.RTDT)), B, vo, steps, DT, textbegin=0.0, textlen=1e-3, bcl=bcl,
                   amp=W.TOM_STIM, het=het, rec_every=rec, n_threads=8)
    beats = [k * bcl for k in range(int(round(steps * DT / bcl)))]
    u, a = A.beat_markers(tr, rec * DT, beats)
    uo, ao = A.beat_markers(tro, rec * DT, beats)
    return b, vm, vo, tr, tro, u, a, uo, ao, B


@pytest.mark.parametrize("variant", VARIANTS)
def test_trace_fp64(gpu, port, variant):
    """Two beats at BCL 500 ms, conductance multipliers +-5 %, 64 cells."""
    b, vm, vo, tr, tro, u, a, uo, ao, B = run_pair(gpu, port, variant, gpu.FP64, 64, 100000, 0.5, 0.95, 1.05)
    assert np.all(np.isfinite(ao)) and np.all(ao > 0.15)
    assert np.abs(tr - tro).max() <= 1e-8
    assert np.abs(vm - vo).max() <= 1e-8
    assert np.nanmax(np.abs(a - ao)) <= 1e-6
    assert np.nanmax(np.abs(u - uo)) <= 1e-6
    S = b.get_state(gpu.LAYOUT_SOA)
    np.testing.assert_allclose(S, B[:, SOA_BLOCK].T, rtol=1e-6, atol=1e-12)


@pytest.mark.parametrize("variant", VARIANTS)
def test_trace_mixed(gpu, port, variant):
    """Precision form: per-quantity error vs the FP64 oracle, 3 beats at BCL 800 ms, +-10 %."""
    b, vm, vo, tr, tro, u, a, uo, ao, B = run_pair(gpu, port, variant, gpu.MIXED, 32, 240000, 0.8, 0.9, 1.1)
    assert np.all(np.isfinite(ao))
    rms = np.sqrt(((tr - tro) ** 2).mean(axis=1))
    S = b.get_state(gpu.LAYOUT_SOA)
    ref_soa = B[:, SOA_BLOCK].T
    names = gpu.state_names(TOM)
    conc = {"Na_i", "Na_ss", "K_i", "K_ss", "Ca_i", "Ca_ss", "Ca_nsr", "Ca_jsr", "Cl_i", "CaMK_trap", "Ca_TRPN",
            "J_rel_NP", "J_rel_CaMK"}
    report = {"model": "Tomek", "celltype": variant, "cells": int(S.shape[1]), "beats": 3, "bcl_ms": 800,
              "conductance_jitter": 0.1, "vm_rms_mv_max": float(rms.max() * 1e3),
              "vm_max_abs_mv": float(np.abs(tr - tro).max() * 1e3),
              "apd90_max_abs_ms": float(np.nanmax(np.abs(a - ao)) * 1e3),
              "upstroke_max_abs_ms": float(np.nanmax(np.abs(u - uo)) * 1e3), "states": {}}
    errs = {}
    for k, name in enumerate(names):
        d = np.abs(S[k] - ref_soa[k]).max()
        if name in conc:
            errs[name] = float(d / max(np.abs(ref_soa[k]).max(), 1e-30))
            report["states"][name] = {"max_rel_err": errs[name]}
        else:
            errs[name] = float(d)
            report["states"][name] = {"max_abs_err": errs[name]}
    out = os.environ.get("CM_REPORT_DIR")
    if out:
        with open(os.path.join(out, f"accuracy_mixed_tom_{variant}.json"), "w") as f:
            json.dump(report, f, indent=1)
    assert np.nanmax(np.abs(a - ao)) <= 1e-3      # APD90 within 1 ms
    assert np.nanmax(np.abs(u - uo)) <= 1e-4      # upstroke within 0.1 ms
    assert rms.max() <= 0.5e-3                    # RMS Vm error within 0.5 mV
    for name, e in errs.items():
        # gates (in [0, 1]) and Markov occupancies absolute, concentrations and release fluxes
        # relative to their range
        assert e < (5e-3 if name in conc else 2e-3), (name, e)


def test_stretch_and_sac(gpu, port):
    """Stretch reaches Calc per cell (troponin Ca50, capped at 1.2) and, with ISAC_SWITCH = 1,
    the stretch-activated current; one FP64 Calc against the oracle's."""
    cm = gpu
    g = np.load(O.GOLDEN / "step_tom_endo.npz")
    n = 64
    S0 = np.ascontiguousarray(g["state_in"][100:100 + n])
    vm = np.ascontiguousarray(g["vm"][100:100 + n])
    stretch = np.linspace(0.85, 1.35, n)
    p = tom_params(cm, "endo")
    p.set("ISAC_SWITCH", 1.0)
    b = cm.Batch(p, n, cm.FP64)
    b.set_state(S0, cm.LAYOUT_REF_BLOCK)
    dV = b.calc(DT, vm, np.zeros(n), stretch)
    P = port.param_vector(O.TOM, O.load_params(O.TOM, "endo"))
    P[port.param_names(O.TOM).index("ISAC_SWITCH")] = 1.0
    B = S0.copy()
    dVo = np.array([port.L.cmo_calc(O.TOM, O._ptr(P), None, B[c].ctypes.data_as(O._dp), DT, float(vm[c]), 0.0,
                                    float(stretch[c])) for c in range(n)])
    np.testing.assert_allclose(dV, dVo, rtol=1e-9, atol=1e-16)
    S = b.get_state(cm.LAYOUT_SOA)
    np.testing.assert_allclose(S, B[:, SOA_BLOCK].T, rtol=1e-10, atol=1e-250)


def test_fp64_step_equals_run_and_state_roundtrip(gpu):
    """calc_update repeated equals the fused run loop bit for bit; SOA and reference-block
    states round-trip; the mixed form's accumulators survive a set/get."""
    cm = gpu
    p = tom_params(cm, "mid")
    n = 300
    out = []
    for mode in ("step", "run"):
        b = cm.Batch(p, n, cm.FP64)
        vm = b.init_vm()
        if mode == "run":
            b.run(vm, 500, textbegin=0.0, textlen=1e-3, bcl=1.0, amplitude=W.TOM_STIM)
        else:  # the driver's stimulus rule (CellModel.h:405-419) on the caller's side
            t, tb = 0.0, 0.0
            for s in range(500):
                i = 0.0
                if t >= tb:
                    i = W.TOM_STIM
                    if t >= tb + 1e-3:
                        tb += 1.0
                b.calc_update(DT, vm, np.full(n, i))
                t += DT
        out.append((vm.copy(), b.get_state()))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    b = cm.Batch(p, n, cm.MIXED)
    blk = b.get_state(cm.LAYOUT_REF_BLOCK)
    assert blk.shape == (n, 84)
    soa = b.get_state()
    k = cm.state_names(TOM).index("Na_i")
    soa[k] += 1e-9  # below FP32 resolution, kept by the compensated pair
    b.set_state(soa)
    assert np.abs(b.get_state()[k] - soa[k]).max() < 1e-13

