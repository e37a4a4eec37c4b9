"""Learned macro step, end to end on the GPU: training pairs from the plain integrator, networks
fitted on the tensor cores for three seeds, the candidate with the smallest trace error on
selection cells kept (`learned.train_and_select`), then held-out cells with per-cell stimulus
phases run with the surrogate against the FP64 oracle.

Bars (the benchmark spec): APD90 within 1 ms and RMS Vm within 0.5 mV of the FP64 oracle. The gain is
shown on whole traces: the same held-out cells run with the coarse step alone (the method
without the network) are less accurate than with the selected network."""
import hashlib
import os

import numpy as np
import pytest

import oracle as O
from cardiomechanics_gb300 import analysis as A
from cardiomechanics_gb300 import learned as L
from cardiomechanics_gb300 import workloads as W

pytestmark = pytest.mark.gpu

DT, S = 1e-5, 10
AMP = W.TT2_STIM_NA


def population(cm, p, n, seed, lo=0.85, hi=1.15):
    b = cm.Batch(p, n, cm.MIXED)
    sc = W.conductance_scales(seed, n, 3, lo, hi)
    for k, name in enumerate(W.TT2_HETERO):
        b.add_hetero_value(name, p.get(name) * sc[k])
    return b, sc


def continued(t, tb, steps, bcl, textlen=1e-3):
    for _ in range(steps):
        if t >= tb and t >= tb + textlen:
            tb += bcl
        t += DT
    return t, tb


def sha(blob):
    return hashlib.sha256(np.ascontiguousarray(blob, np.float32).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def trained(gpu):
    cm = gpu
    p = cm.Params(cm.TENTUSSCHER2, None, DT)
    sur = cm.Surrogate(p, substeps=S, seed=1)
    rep = L.train_and_select(cm, p, sur, seeds=(1, 2, 3))
    assert rep["pairs"] > 10_000_000
    print("selected", rep["selected"], "coarse only", rep["coarse_only"])
    return cm, p, sur, rep


def run_traces(cm, b, sur, vm, n_macro, bcl, mode):
    """Macro steps one at a time; Vm after each (0.1 ms resolution)."""
    tr = np.zeros((b.n, n_macro + 1))
    tr[:, 0] = vm
    t, tb = 0.0, 0.0
    stats = []
    for k in range(n_macro):
        st = b.run_surrogate(sur, vm, 1, t0=t, textbegin=tb, textlen=1e-3, bcl=bcl, amplitude=AMP, mode=mode,
                             audit_mod=100)
        stats.append(st)
        t, tb = continued(t, tb, S, bcl)
        tr[:, k + 1] = vm
    return tr, stats


def test_training_is_deterministic(trained):
    """The same seed gives the same network: two fits on the dataset of this surrogate, and a fit
    on a dataset generated again by another surrogate, give blobs with one sha256."""
    cm, p, sur, rep = trained
    selected = sur.get_blob()
    seed = rep["selected"]["seed"]
    L.fit(sur, seed)
    a = sha(sur.get_blob())
    L.fit(sur, seed)
    b = sha(sur.get_blob())
    other = cm.Surrogate(p, substeps=S, seed=1)
    assert L.generate(cm, p, other) == rep["pairs"]
    L.fit(other, seed)
    c = sha(other.get_blob())
    sur.set_blob(selected)
    assert a == b == c


def test_surrogate_accuracy_and_gain(trained, port):
    """Held-out cells (their own conductances and per-cell stimulus phases in [0, BCL)), five
    beats at BCL 500 ms from the initial state, FP64 audit on: the selected network meets both
    bars against the FP64 oracle, and its largest APD90 and RMS Vm errors are below those of the
    coarse step alone on the same cells; every one of the three seeds' best candidates beats the
    coarse step alone on the selection cells too."""
    cm, p, sur, rep = trained
    n, beats, t_end = 256, 5, 3.0
    het_seed = 99
    ph = W.uniform(98, np.arange(n, dtype=np.uint64)) * L.BCL
    names = port.param_names(O.TT2)
    P = port.param_vector(O.TT2, O.load_params(O.TT2))
    sc = W.conductance_scales(het_seed, n, 3, 0.85, 1.15)
    het = {k: P[names.index(k)] * sc[i] for i, k in enumerate(W.TT2_HETERO)}
    B = port.init_state(O.TT2, P, n)
    vo = np.full(n, port.init_vm(O.TT2, P))
    tro = port.run(O.TT2, P, port.tables(O.TT2, P, DT), B, vo, int(round(t_end / DT)) + 1, DT, textlen=1e-3,
                   bcl=L.BCL, amp=AMP, het=het, textbegin_per_cell=ph, rec_every=S, n_threads=os.cpu_count() or 8)
    res = {}
    for name, mode in (("learned", cm.SUR_AUDIT_FP64), ("coarse", cm.SUR_COARSE_ONLY | cm.SUR_AUDIT_FP64)):
        tr, st = L.surrogate_traces(cm, p, sur, n, het_seed, ph, t_end, 1, mode)
        res[name] = dict(L.trace_errors(tr, tro, ph, S * DT, beats), **st)
    print("held out", res)
    lrn, crs = res["learned"], res["coarse"]
    assert lrn["surrogate"] > 0.9 * lrn["cell_macro_steps"]  # most cell-macro-steps take the learned step
    assert lrn["fallback"] <= 1.5 * crs["fallback"]          # its steps pass the range audit
    assert lrn["max_audit_err_mv"] < 1.0
    # spec bars against the FP64 oracle
    assert lrn["missing_beats"] == 0 and lrn["apd90_max_ms"] <= 1.0 and lrn["rms_vm_mv_max"] <= 0.5, res
    # what the network buys over the coarse step alone, on whole traces
    assert lrn["apd90_max_ms"] < crs["apd90_max_ms"] and lrn["rms_vm_mv_max"] < crs["rms_vm_mv_max"], res
    # and not by luck of one seed: on the selection cells, every seed's best candidate beats the
    # coarse step alone on both bars' errors
    for seed in sorted({c["seed"] for c in rep["candidates"]}):
        best = min((c for c in rep["candidates"] if c["seed"] == seed), key=lambda c: c["score"])
        assert best["apd90_max_ms"] < rep["coarse_only"]["apd90_max_ms"], (seed, best, rep["coarse_only"])
        assert best["rms_vm_mv_max"] < rep["coarse_only"]["rms_vm_mv_max"], (seed, best, rep["coarse_only"])


def test_surrogate_blob_roundtrip(trained):
    cm, p, sur, _ = trained
    blob = sur.get_blob()
    other = cm.Surrogate(p, substeps=S, seed=7)
    other.set_blob(blob)
    np.testing.assert_array_equal(other.get_blob(), blob)


def test_surrogate_fp64_audit(trained, port):
    """The audit sample integrated in FP64 (the reference arithmetic) instead of the mixed step:
    the run stays within the bars and the audit compares the network with FP64 steps."""
    cm, p, sur, _ = trained
    n, bcl = 128, 0.5
    n_macro = int(round(bcl / (S * DT)))
    b, sc = population(cm, p, n, seed=98)
    names = port.param_names(O.TT2)
    P = port.param_vector(O.TT2, O.load_params(O.TT2))
    het = {k: P[names.index(k)] * sc[i] for i, k in enumerate(W.TT2_HETERO)}
    B = port.init_state(O.TT2, P, n)
    vo = np.full(n, port.init_vm(O.TT2, P))
    tro = port.run(O.TT2, P, port.tables(O.TT2, P, DT), B, vo, n_macro * S, DT, textlen=1e-3, bcl=bcl, amp=AMP,
                   het=het, rec_every=S, n_threads=8)
    tro = np.concatenate([tro, vo[:, None]], axis=1)
    vm = b.init_vm()
    tr, stats = run_traces(cm, b, sur, vm, n_macro, bcl, cm.SUR_AUDIT_FP64)
    u, a = A.beat_markers(tr, S * DT, [0.0])
    uo, ao = A.beat_markers(tro, S * DT, [0.0])
    rms = (np.sqrt(((tr - tro) ** 2).mean(axis=1)) * 1e3).max()
    audited = sum(s["audited"] for s in stats)
    err = max(s["max_audit_err_mv"] for s in stats)
    print("fp64 audit", dict(apd=np.nanmax(np.abs(a - ao)) * 1e3, rms=rms, audited=audited, err=err))
    assert audited > 0 and np.isfinite(err) and err < 1.0
    assert np.nanmax(np.abs(a - ao)) * 1e3 <= 1.0 and rms <= 0.5
    # the last macro step's sample waits for the next run; flushing audits it now, once
    fl = sur.flush_audit(cm.SUR_AUDIT_FP64)
    assert fl["audited"] > 0 and fl["max_audit_err_mv"] < 1.0
    assert sur.flush_audit(cm.SUR_AUDIT_FP64)["audited"] == 0


def test_inference_kernel_matches_network(trained):
    """The tensor-core inference inside the macro step gives the network's output: for every one
    of the 19 outputs, the state after one macro step with the network minus the state after the
    coarse step alone (same initial state) equals sd_y * net(features), the network evaluated by
    the training GEMMs, cell by cell. BF16 operands on both sides, but the two sum in different
    orders (the kernel adds the hidden biases inside the tensor core's FP32 accumulation, the
    GEMMs after it) and the features differ in their last FP32 bits, so a hidden pre-activation
    can round to the neighbouring BF16 value on one side only; the tolerance is 10 % of the
    output's scale plus 8 units in the last place of the state's FP32 value."""
    cm, p, sur, _ = trained
    selected = sur.get_blob()
    every = selected.copy()
    every[L.APPLIED] = every[44:63]  # every output's correction applied, at its target scale
    sur.set_blob(every)
    try:
        _inference_check(cm, p, sur)
    finally:
        sur.set_blob(selected)


def _inference_check(cm, p, sur):
    n = 1000
    b, sc = population(cm, p, n, seed=97)
    vm = b.init_vm()
    b.run(vm, 3000, textbegin=0.0, textlen=1e-3, bcl=0.8, amplitude=AMP)  # 30 ms: plateau
    s0, v0 = b.get_state(), vm.copy()
    kw = dict(t0=3000 * DT, textbegin=0.8, textlen=1e-3, bcl=0.8, amplitude=AMP, audit_mod=0)
    va = v0.copy()
    st0 = b.run_surrogate(sur, va, 1, mode=0, **kw)
    sa = b.get_state()
    b.set_state(s0)
    vb = v0.copy()
    st1 = b.run_surrogate(sur, vb, 1, mode=cm.SUR_COARSE_ONLY, **kw)
    sb = b.get_state()
    assert st0["surrogate"] == n and st1["surrogate"] == n, (st0, st1)
    names = cm.state_names(cm.TENTUSSCHER2)
    idx = {k: i for i, k in enumerate(names)}
    gates = ["m", "h", "j", "xr1", "xr2", "xs", "r", "s", "d", "f", "f2", "fCa", "Rq"]
    outs = gates + ["Ca_i", "CaSS", "CaSR", "Na_i", "K_i"]
    S0 = {k: s0[idx[k]] for k in names}
    F = np.stack([v0 * 1e3] + [S0[k] for k in gates] +
                 [np.log(np.maximum(S0["Ca_i"], 1e-12)), np.log(np.maximum(S0["CaSS"], 1e-12)), S0["CaSR"],
                  S0["Na_i"], S0["K_i"], np.log(sc[0]), np.log(sc[1]), np.log(sc[2])], axis=1)
    blob = sur.get_blob()
    mu, inv_sd, sd_y, apply_y = blob[:22], blob[22:44], blob[44:63], blob[63:82]
    assert np.all(apply_y > 0)
    Y = sur.mlp.forward(((F - mu) * inv_sd).astype(np.float32)).astype(np.float64)
    got = [(va - vb) * 1e3] + [sa[idx[k]] - sb[idx[k]] for k in outs]
    scale = [np.abs(v0 * 1e3)] + [np.abs(sb[idx[k]]) for k in outs]
    worst = 0.0
    for k in range(19):
        want = apply_y[k] * Y[:, k]
        tol = 0.1 * sd_y[k] * np.maximum(1.0, np.abs(Y[:, k])) + 8 * np.spacing(scale[k].astype(np.float32))
        err = np.abs(got[k] - want)
        worst = max(worst, float((err / tol).max()))
        assert np.all(err <= tol), (k, float(err.max()), float(tol.min()), int((err > tol).sum()))
    print("inference: worst error / tolerance", worst)


def test_surrogate_per_cell_stimulus(trained):
    """Per-cell first stimulus times (the reference driver's textbegin per cell): one batch with
    two stimulus phases equals two batches with one phase each, cell by cell."""
    cm, p, sur, _ = trained
    n, bcl, n_macro = 256, 0.5, 2500
    phases = (0.0, 0.2)
    kw = dict(textlen=1e-3, bcl=bcl, amplitude=AMP, audit_mod=0)
    sep = []
    for k, ph in enumerate(phases):
        b, _ = population(cm, p, n, seed=60 + k)
        v = b.init_vm()
        b.run_surrogate(sur, v, n_macro, textbegin=ph, **kw)
        sep.append(v)
    both = cm.Batch(p, 2 * n, cm.MIXED)
    scs = [W.conductance_scales(60 + k, n, 3, 0.85, 1.15) for k in range(2)]
    for j, name in enumerate(W.TT2_HETERO):
        both.add_hetero_value(name, p.get(name) * np.concatenate([scs[0][j], scs[1][j]]))
    v = both.init_vm()
    tbc = np.repeat(np.array(phases), n)
    st = both.run_surrogate(sur, v, n_macro, textbegin_per_cell=tbc, **kw)
    assert st["surrogate"] > 0.9 * 2 * n * n_macro
    np.testing.assert_allclose(v, np.concatenate(sep), rtol=0, atol=1e-9)


def test_surrogate_host_vm_forms(trained):
    """Vm in page-locked host memory (read and written as FP64 by the macro-step kernels over the
    host link, once per macro step), in pageable host memory (staged) and on the device (kept as
    the compensated FP32 pair through a call): device and pageable give the same cells bit for
    bit; page-locked host memory too when every call advances one macro step (the acCELLerate
    pattern), and within 1 uV over calls of many macro steps, where the pair is rounded to FP64
    after every step instead of once per call."""
    import torch
    cm, p, sur, _ = trained
    n = 1000
    kw = dict(textbegin=0.0, textlen=1e-3, bcl=0.5, amplitude=AMP, audit_mod=0)
    for n_macro, calls in ((1, 40), (300, 3)):
        out = []
        for form in ("device", "pinned", "pageable"):
            b, _ = population(cm, p, n, seed=70)
            v0 = b.init_vm()
            if form == "device":
                v = torch.tensor(v0, device="cuda")
            elif form == "pinned":
                v = torch.tensor(v0).pin_memory()
            else:
                v = v0
            for k in range(calls):  # several calls: the host copy must be current after each
                t0 = k * n_macro * S * DT
                b.run_surrogate(sur, v, n_macro, t0=t0, **kw)
            out.append(v.cpu().numpy() if hasattr(v, "cpu") else v.copy())
        assert np.array_equal(out[0], out[2]), n_macro
        if n_macro == 1:
            assert np.array_equal(out[0], out[1])
        else:
            np.testing.assert_allclose(out[1], out[0], rtol=0, atol=1e-6 * 1e-3)
