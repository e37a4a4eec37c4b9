"""GPU parity: the CUDA kernels through the C ABI against the oracle and the golden vectors.

Tolerances:
  FP64 batches  one Calc: states rtol 1e-11 (the kernel's exp, log and division are within 1 ulp
                of glibc's, some quotients are taken over one denominator and multiply-adds are
                fused); dV and the diagnostic currents rtol 1e-10 (I_tot is a sum of currents
                that cancel to ~1e-6 of their size); 1000 ms traces: |dVm| <= 1e-5 mV, APD90 and
                upstroke within 1e-3 ms of the oracle.
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

TAG = {5: "tt2", 2: "crn"}
OM = {5: O.TT2, 2: O.CRN}
HET = {5: W.TT2_HETERO, 2: W.CRN_HETERO, 12: W.ORD_HETERO, 14: W.TOM_HETERO}
AMP = {5: W.TT2_STIM_NA, 2: W.CRN_STIM_PAPF, 12: W.ORD_STIM, 14: W.TOM_STIM}
TLEN = {5: 1e-3, 2: 2e-3, 12: 1e-3, 14: 1e-3}


# the diagnostic currents of the reference block: TT2 Array[0..16] (I_Na ... I_tot) at slots 5..21
DIAG_COLS = {5: tuple(range(5, 22))}


def ref_block_cols(model):
    # TT2 Array[17] is never written by the reference
    return [c for c in range(36) if c != 22] if model == 5 else list(range(22))


@pytest.mark.parametrize("model", [5, 2])
def test_one_step_known_answers_fp64(gpu, model):
    cm = gpu
    g = np.load(O.GOLDEN / f"step_{TAG[model]}.npz")
    dt = float(g["dt"])
    p = cm.Params(model, None, dt)
    n = g["state_in"].shape[0]
    b = cm.Batch(p, n, cm.FP64)
    b.set_diagnostics(True)
    b.set_state(g["state_in"], cm.LAYOUT_REF_BLOCK)
    for k, name in enumerate(g["hetero_names"]):
        b.add_hetero_value(str(name), p.get(str(name)) * g["hetero_scale"][k])
    dV = b.calc(dt, np.ascontiguousarray(g["vm"]), np.ascontiguousarray(g["i_ext"]))
    S = b.get_state(cm.LAYOUT_REF_BLOCK)
    cols = ref_block_cols(model)
    cur = [c for c in cols if c in DIAG_COLS.get(model, ())]
    st = [c for c in cols if c not in cur]
    np.testing.assert_allclose(S[:, st], g["state_out"][:, st], rtol=1e-11, atol=1e-250)
    np.testing.assert_allclose(S[:, cur], g["state_out"][:, cur], rtol=1e-10, atol=1e-250)
    np.testing.assert_allclose(dV, g["dvm"], rtol=1e-10, atol=1e-16)
    # rows at the table edges stay in bounds; out-of-table voltages raise the audit bit
    assert b.audit() & cm.AUDIT_VRANGE == 0
    b.calc(dt, np.full(n, 0.25), None)
    assert b.audit() & cm.AUDIT_VRANGE


def run_pair(cm, port, model, precision, n, steps, bcl, lo, hi, seed=1, rec=10):
    dt = 1e-5
    p = cm.Params(model, None, dt)
    b = cm.Batch(p, n, precision)
    sc = W.conductance_scales(seed, n, 3, lo, hi)
    names = port.param_names(OM[model])
    P = port.param_vector(OM[model], O.load_params(OM[model]))
    het = {}
    for k, name in enumerate(HET[model]):
        het[name] = P[names.index(name)] * sc[k]
        b.add_hetero_value(name, het[name])
    vm = b.init_vm()
    probes = np.arange(n)
    tr = b.run(vm, steps, textbegin=0.0, textlen=TLEN[model], bcl=bcl, amplitude=AMP[model],
               probe_cells=probes, probe_every=rec)
    T = port.tables(OM[model], P, dt)
    B = port.init_state(OM[model], P, n)
    vo = np.full(n, port.init_vm(OM[model], P))
    tro = port.run(OM[model], P, T, B, vo, steps, dt, textbegin=0.0, textlen=TLEN[model], bcl=bcl,
                   amp=AMP[model], het=het, rec_every=rec, n_threads=8)
    beats = [k * bcl for k in range(int(round(steps * dt / bcl)))]
    u, a = A.beat_markers(tr, rec * dt, beats)
    uo, ao = A.beat_markers(tro, rec * dt, beats)
    return b, vm, vo, tr, tro, u, a, uo, ao, B


@pytest.mark.parametrize("model", [5, 2])
def test_trace_fp64(gpu, port, model):
    b, vm, vo, tr, tro, u, a, uo, ao, B = run_pair(gpu, port, model, gpu.FP64, 64, 100000, 1.0, 0.95, 1.05)
    assert np.all(np.isfinite(ao)) and np.all(ao > 0.15)
    assert np.abs(tr - tro).max() <= 1e-8
    assert np.abs(vm - vo).max() <= 1e-8
    assert np.nanmax(np.abs(a - ao)) <= 1e-6
    assert np.nanmax(np.abs(u - uo)) <= 1e-6
    S = b.get_state(gpu.LAYOUT_REF_BLOCK)
    cols = [c for c in ref_block_cols(model) if not (model == 5 and 5 <= c < 23) and not (model == 2 and c == 20)]
    np.testing.assert_allclose(S[:, cols], B[:, cols], rtol=1e-6, atol=1e-12)


@pytest.mark.parametrize("model", [5, 2])
def test_trace_mixed(gpu, port, model):
    """Precision form: per-quantity error vs the FP64 oracle, 3 beats at BCL 800 ms, +-10%."""
    b, vm, vo, tr, tro, u, a, uo, ao, B = run_pair(gpu, port, model, gpu.MIXED, 32, 240000, 0.8, 0.9, 1.1)
    assert np.all(np.isfinite(ao))
    assert np.nanmax(np.abs(a - ao)) <= 1e-3      # APD90 within 1 ms
    assert np.nanmax(np.abs(u - uo)) <= 1e-4      # upstroke within 0.1 ms
    rms = np.sqrt(((tr - tro) ** 2).mean(axis=1))
    assert rms.max() <= 0.5e-3                    # RMS Vm error within 0.5 mV
    S = b.get_state(gpu.LAYOUT_SOA)
    ref_soa = B[:, [c for c in range(B.shape[1]) if (c < 5 or c >= 23)]].T if model == 5 else \
        B[:, [c for c in range(22) if c != 20]].T
    # per-quantity error after 3 beats: gates (in [0, 1]) absolute, concentrations relative
    names = gpu.state_names(model)
    conc = {"Ca_i", "CaSR", "CaSS", "Na_i", "K_i", "Ca_up", "Ca_rel", "Ca_TRPN"}
    report = {"model": "TenTusscher2" if model == 5 else "CourtemancheEtAl", "cells": int(S.shape[1]),
              "beats": 3, "bcl_ms": 800, "conductance_jitter": 0.1,
              "vm_rms_mv_max": float(rms.max() * 1e3), "vm_max_abs_mv": float(np.abs(tr - tro).max() * 1e3),
              "apd90_max_abs_ms": float(np.nanmax(np.abs(a - ao)) * 1e3),
              "upstroke_max_abs_ms": float(np.nanmax(np.abs(u - uo)) * 1e3), "states": {}}
    for k, name in enumerate(names):
        d = np.abs(S[k] - ref_soa[k]).max()
        if name in conc:
            rel = float(d / np.abs(ref_soa[k]).max())
            report["states"][name] = {"max_rel_err": rel}
            assert rel < 5e-3, (name, rel)
        else:
            report["states"][name] = {"max_abs_err": float(d)}
            assert d < 2e-3, (name, d)
    out = os.environ.get("CM_REPORT_DIR")
    if out:
        with open(os.path.join(out, f"accuracy_mixed_{TAG[model]}.json"), "w") as f:
            json.dump(report, f, indent=1)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_per_cell_stimulus_times(gpu, port, precision):
    """The driver protocol with a first stimulus time per cell, against the oracle's loop; a
    device array of times is advanced in place (a second run continues from it), a host array
    is left as it was."""
    import torch
    cm = gpu
    n, dt, bcl, steps = 96, 1e-5, 0.3, 20000
    prec = cm.FP64 if precision == "fp64" else cm.MIXED
    tbc0 = np.linspace(0.0, 0.25, n)
    p = cm.Params(5, None, dt)
    b = cm.Batch(p, n, prec)
    vm = b.init_vm()
    tb_host = tbc0.copy()
    b.run(vm, steps // 2, textlen=1e-3, bcl=bcl, amplitude=AMP[5], textbegin_per_cell=tb_host)
    assert np.array_equal(tb_host, tbc0)
    # the same first half with the times on the device, then the second half continuing from them
    b2 = cm.Batch(p, n, prec)
    vm2 = b2.init_vm()
    tb_dev = torch.tensor(tbc0, device="cuda")
    b2.run(vm2, steps // 2, textlen=1e-3, bcl=bcl, amplitude=AMP[5], textbegin_per_cell=tb_dev)
    np.testing.assert_array_equal(vm2, vm)
    t_half = 0.0
    for _ in range(steps // 2):
        t_half += dt
    b2.run(vm2, steps - steps // 2, t0=t_half, textlen=1e-3, bcl=bcl, amplitude=AMP[5], textbegin_per_cell=tb_dev)
    P = port.param_vector(O.TT2, O.load_params(O.TT2))
    B = port.init_state(O.TT2, P, n)
    vo = np.full(n, port.init_vm(O.TT2, P))
    port.run(O.TT2, P, port.tables(O.TT2, P, dt), B, vo, steps, dt, textlen=1e-3, bcl=bcl, amp=AMP[5],
             textbegin_per_cell=tbc0, n_threads=8)
    t_end = 2 * t_half
    if precision == "fp64":
        assert np.abs(vm2 - vo).max() <= 1e-8, np.abs(vm2 - vo).max()
    else:  # within 0.5 mV, away from the upstrokes in progress at the end (a 1 us shift is mV there)
        calm = ~((tbc0 > t_end - 5e-3) & (tbc0 <= t_end))
        assert np.abs(vm2 - vo)[calm].max() <= 5e-4, np.abs(vm2 - vo)[calm].max()
    # the times advanced as the driver advances textbegin: past every stimulus that has ended
    tb_end = tb_dev.cpu().numpy()
    assert np.all(tb_end >= tbc0) and np.any(tb_end > tbc0)
    assert np.all(tb_end + 1e-3 + 2 * dt >= t_end)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_step_update_activation_times(gpu, precision):
    """The fused Godunov update with activation times (acCELLerate.cpp:1997-2005): every cell's
    entry becomes the time of the first step whose new Vm reaches the threshold, as a host loop
    over the returned Vm finds it; entries already set stay."""
    cm = gpu
    n, dt, thr = 64, 1e-5, -0.04
    b = cm.Batch(cm.Params(5, None, dt), n, cm.FP64 if precision == "fp64" else cm.MIXED)
    vm = b.init_vm()
    act = np.full(n, -1.0)
    act[5] = 123.0  # already activated: must stay
    first = act.copy()
    onset = 3 * np.arange(n)
    t = 0.0
    for k in range(420):
        iext = np.where((k >= onset) & (k < onset + 100), AMP[5], 0.0)
        b.calc_update_act(dt, vm, act, t, thr, i_ext=iext, vm_range=0.2)
        newly = (first == -1.0) & (vm >= thr)
        first[newly] = t
        t += dt
    np.testing.assert_array_equal(act, first)
    assert act[5] == 123.0 and (act > 0).sum() == n


def test_device_pointers_and_step_equals_run(gpu):
    import torch
    cm = gpu
    p = cm.Params(5, None, 1e-5)
    n = 1000
    b1 = cm.Batch(p, n, cm.FP64)
    b2 = cm.Batch(p, n, cm.FP64)
    vm_host = b1.init_vm()
    vm_dev = torch.tensor(vm_host, device="cuda")
    b1.run(vm_host, 500, textbegin=0.0, textlen=1e-3, bcl=1.0, amplitude=AMP[5])
    # the same 500 steps through per-step Calc with caller-side stimulus and Vm update
    t, tb = 0.0, 0.0
    dv = torch.empty_like(vm_dev)
    for s in range(500):
        i = 0.0
        if t >= tb:
            i = AMP[5]
            if t >= tb + 1e-3:
                tb += 1.0
        ie = torch.full_like(vm_dev, i)
        b2.calc(1e-5, vm_dev, ie, None, dVm=dv)
        vm_dev += dv
        t += 1e-5
    torch.cuda.synchronize()
    assert np.array_equal(vm_dev.cpu().numpy(), vm_host)
    assert np.array_equal(b1.get_state(), b2.get_state())


def test_state_roundtrip_and_reset(gpu):
    cm = gpu
    for model in (5, 2):
        p = cm.Params(model, None, 1e-5)
        for prec in (cm.FP64, cm.MIXED):
            b = cm.Batch(p, 300, prec)
            s0 = b.get_state(cm.LAYOUT_REF_BLOCK)
            vm = b.init_vm()
            b.run(vm, 200, amplitude=AMP[model], textlen=TLEN[model])
            s1 = b.get_state(cm.LAYOUT_REF_BLOCK)
            assert not np.array_equal(s0, s1)
            b.set_state(s0, cm.LAYOUT_REF_BLOCK)
            if prec == cm.FP64:
                assert np.array_equal(b.get_state(cm.LAYOUT_REF_BLOCK), s0)
            b.set_state(s1, cm.LAYOUT_REF_BLOCK)
            b.reset()
            np.testing.assert_allclose(b.get_state(cm.LAYOUT_REF_BLOCK), s0, rtol=1e-7)


def test_errors_and_audit(gpu):
    cm = gpu
    p = cm.Params(5, None, 1e-5)
    b = cm.Batch(p, 64, cm.FP64)
    vm = b.init_vm()
    with pytest.raises(cm.CMError) as e:
        b.calc(2e-5, vm)
    assert e.value.code == -1
    with pytest.raises(cm.CMError) as e:
        b.add_hetero_value("g_pK", np.ones(64))
    assert e.value.code == -7
    with pytest.raises(cm.CMError) as e:
        b.add_hetero_value("nonsense", np.ones(64))
    assert e.value.code == -4
    # NaN injected into one cell's state on the host: the fused run reports it, per cell
    s = b.get_state()
    s[3, 17] = np.nan  # K_i of cell 17
    b.set_state(s)
    with pytest.raises(cm.CMError) as e:
        b.run(vm, 10, amplitude=AMP[5])
    assert e.value.code == -8
    m, per = b.audit(per_cell=True)
    assert m & cm.AUDIT_NAN and per[17] & cm.AUDIT_NAN and per[16] == 0
    assert b.audit() == 0


def test_full_size_determinism_mixed(gpu):
    """4,194,304 cells (2048 x 2048 sheet), 200 steps twice from reset: bitwise identical,
    finite, and cells with equal conductances end equal (a size-independent property)."""
    import torch
    cm = gpu
    n = 2048 * 2048
    p = cm.Params(5, None, 1e-5)
    b = cm.Batch(p, n, cm.MIXED)
    sc = W.conductance_scales(2, n, 3, 0.9, 1.1)
    sc[:, 1::2] = 1.0
    for k, name in enumerate(W.TT2_HETERO):
        b.add_hetero_value(name, p.get(name) * sc[k])
    outs = []
    for rep in range(2):
        b.reset()
        vm = torch.tensor(b.init_vm(), device="cuda")
        b.run(vm, 200, textlen=1e-3, amplitude=AMP[5])
        outs.append(vm.cpu().numpy())
    assert np.array_equal(outs[0], outs[1])
    assert np.all(np.isfinite(outs[0]))
    odd = outs[0][1::2]
    assert np.all(odd == odd[0])
    assert b.audit() == 0


@pytest.mark.parametrize("model", [5, 2, 12, 14])
def test_launch_shapes_agree(gpu, model):
    """Every launch shape of the mixed kernel (register budgets, grid modes, the
    shared-memory-staged bulk-copy kernels and their producer/consumer pipelines) integrates the
    same cells to the same result, up to FP32 rounding differences between instruction
    schedules."""
    cm = gpu
    n = 3 * 256 + 77  # partial last tile
    p = cm.Params(model, None, 1e-5)
    out = []
    for variant, grid_mode in [(0, 0), (1, 2), (3, 4), (5, 2), (6, 1), (5, 4), (7, 2), (8, 1), (7, 4)]:
        b = cm.Batch(p, n, cm.MIXED)
        sc = W.conductance_scales(4, n, 3, 0.9, 1.1)
        for k, name in enumerate(HET[model]):
            b.add_hetero_value(name, p.get(name) * sc[k])
        b.set_launch(variant, grid_mode)
        vm = b.init_vm()
        b.run(vm, 2000, textlen=TLEN[model], amplitude=AMP[model], bcl=1.0)
        assert b.audit() == 0
        out.append((vm, b.get_state()))
    for vm, st in out[1:]:
        assert np.abs(vm - out[0][0]).max() <= 1e-6
        np.testing.assert_allclose(st, out[0][1], rtol=1e-4, atol=1e-7)
