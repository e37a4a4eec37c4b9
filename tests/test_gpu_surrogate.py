"""Learned macro step, end to end on the GPU: training pairs from the plain integrator, fit on
the tensor cores, then a held-out population run with the surrogate against the FP64 oracle.

Bars (the benchmark spec): APD90 within 1 ms and RMS Vm within 0.5 mV of the FP64 oracle. The
ablation shows what the network adds: the same run with the coarse step alone (the method
without the network) must be less accurate."""
import numpy as np
import pytest

import oracle as O
from cardiomechanics_gb300 import analysis as A
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


@pytest.fixture(scope="module")
def trained(gpu):
    cm = gpu
    p = cm.Params(cm.TENTUSSCHER2, None, DT)
    sur = cm.Surrogate(p, substeps=S, seed=1)
    b, _ = population(cm, p, 2048, seed=11)
    vm = b.init_vm()
    # 4 beats at BCL 500 ms: 20,000 macro steps, every 4th cell sampled
    n = sur.generate(b, vm, 20000, textlen=1e-3, bcl=0.5, amplitude=AMP, cell_stride=4, max_pairs=12_000_000)
    assert n > 5_000_000
    l1 = sur.fit(batch=4096, steps=4000, lr=1e-3, seed=1)
    l2 = sur.fit(batch=8192, steps=2000, lr=2e-4, seed=2)
    return cm, p, sur, (l1, l2)


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


def test_surrogate_accuracy_and_gain(trained, port):
    cm, p, sur, losses = trained
    assert losses[1] < 0.05, losses  # normalised MSE
    n, bcl, beats = 128, 0.8, 2
    n_macro = int(round(beats * bcl / (S * DT)))
    # held-out population (other seed)
    b0, sc = population(cm, p, n, seed=99)
    names = port.param_names(O.TT2)
    P = port.param_vector(O.TT2, O.load_params(O.TT2))
    het = {k: P[names.index(k)] * sc[i] for i, k in enumerate(W.TT2_HETERO)}
    T = port.tables(O.TT2, P, DT)
    B = port.init_state(O.TT2, P, n)
    vo = np.full(n, port.init_vm(O.TT2, P))
    tro = port.run(O.TT2, P, T, B, vo, n_macro * S, DT, textlen=1e-3, bcl=bcl, amp=AMP, het=het, rec_every=S,
                   n_threads=8)
    tro = np.concatenate([tro, vo[:, None]], axis=1)
    res = {}
    for mode in (0, 1):
        b, _ = population(cm, p, n, seed=99)
        vm = b.init_vm()
        tr, stats = run_traces(cm, b, sur, vm, n_macro, bcl, mode)
        u, a = A.beat_markers(tr, S * DT, [k * bcl for k in range(beats)])
        uo, ao = A.beat_markers(tro, S * DT, [k * bcl for k in range(beats)])
        rms = np.sqrt(((tr - tro) ** 2).mean(axis=1)) * 1e3
        res[mode] = dict(apd=np.nanmax(np.abs(a - ao)) * 1e3, rms=rms.max(), up=np.nanmax(np.abs(u - uo)) * 1e3,
                         sur=sum(s["surrogate"] for s in stats), fb=sum(s["fallback"] for s in stats),
                         audit=max(s["max_audit_err_mv"] for s in stats))
        assert np.all(np.isfinite(a)), mode
    print("surrogate", res)
    assert res[0]["sur"] > 0.9 * n * n_macro  # most cell-macro-steps use the learned step
    assert res[0]["apd"] <= 1.0 and res[0]["rms"] <= 0.5, res
    assert res[0]["rms"] < res[1]["rms"] and res[0]["apd"] <= res[1]["apd"] + 1e-3, res


def test_surrogate_blob_roundtrip(trained):
    cm, p, sur, _ = trained
    blob = sur.get_blob()
    other = cm.Surrogate(p, substeps=S, seed=7)
    other.set_blob(blob)
    np.testing.assert_array_equal(other.get_blob(), blob)
