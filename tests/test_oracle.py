"""The oracle (oracle/cm_oracle.c) pinned against the reference: golden vectors generated by
running the reference's own CellModel library (tests/golden/make_golden.py), and, where the
reference tree is present, against that library directly."""
import hashlib
import json

import numpy as np
import pytest

import oracle as O
from cardiomechanics_gb300 import workloads as W

MODELS = [O.TT2, O.CRN]
TAG = {O.TT2: "tt2", O.CRN: "crn"}


def params(port, model):
    return port.param_vector(model, O.load_params(model))


@pytest.mark.parametrize("model", MODELS)
def test_derived_parameters_match_reference(port, model):
    ref = O.load_params(model)
    P = params(port, model)
    for i, name in enumerate(port.param_names(model)):
        if name in ref:
            assert P[i] == ref[name], name


@pytest.mark.parametrize("model", MODELS)
def test_tables_match_reference(port, model):
    g = np.load(O.GOLDEN / f"tables_{TAG[model]}.npz")
    T = port.tables(model, params(port, model), float(g["dt"]))
    names = port.table_names(model)
    assert list(map(str, g["names"])) == names
    for k, name in enumerate(names):
        if hashlib.sha256(T[k].tobytes()).hexdigest() == g["sha256"][k]:
            continue
        # another libm (e.g. aarch64 glibc) may differ in the last bit of exp/log
        np.testing.assert_allclose(T[k][::50], g["rows"][k], rtol=4e-16 * 8, atol=0, err_msg=name)


@pytest.mark.parametrize("model", MODELS)
def test_one_step_known_answers(port, model):
    g = np.load(O.GOLDEN / f"step_{TAG[model]}.npz")
    P = params(port, model)
    dt = float(g["dt"])
    T = port.tables(model, P, dt)
    S = g["state_in"].copy()
    names = port.param_names(model)
    het = {str(n): P[names.index(str(n))] * g["hetero_scale"][k] for k, n in enumerate(g["hetero_names"])}
    dV = port.calc(model, P, T, S, dt, g["vm"], g["i_ext"], het=het)
    ns = S.shape[1]
    # TT2 Array[17] is never written by the reference (uninitialised); compare the rest
    cols = [c for c in range(ns) if not (model == O.TT2 and c == 22)]
    np.testing.assert_allclose(S[:, cols], g["state_out"][:, cols], rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(dV, g["dvm"], rtol=1e-12, atol=1e-18)


@pytest.mark.parametrize("model", MODELS)
def test_driver_trace(port, model):
    g = np.load(O.GOLDEN / f"trace_{TAG[model]}.npz")
    P = params(port, model)
    dt = float(g["dt"])
    T = port.tables(model, P, dt)
    n = g["hetero_scale"].shape[1]
    names = port.param_names(model)
    het = {str(nm): P[names.index(str(nm))] * g["hetero_scale"][k] for k, nm in enumerate(g["hetero_names"])}
    B = port.init_state(model, P, n)
    Vm = np.full(n, port.init_vm(model, P))
    tr = port.run(model, P, T, B, Vm, int(g["n_steps"]), dt, textlen=float(g["textlen"]), bcl=float(g["bcl"]),
                  amp=float(g["amp"]), het=het, rec_every=int(g["rec_every"]))
    np.testing.assert_allclose(tr, g["trace"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(Vm, g["final_vm"], rtol=0, atol=1e-9)
    cols = [c for c in range(B.shape[1]) if c < 5 or c >= 23] if model == O.TT2 else list(range(B.shape[1]))
    np.testing.assert_allclose(B[:, cols], g["final_state"][:, cols], rtol=1e-8, atol=1e-12)
    # an action potential happened in every beat
    assert tr.max() > 0.0


def test_threads_do_not_change_results(port):
    P = params(port, O.TT2)
    T = port.tables(O.TT2, P, 1e-5)
    out = []
    for nt in (1, 3):
        B = port.init_state(O.TT2, P, 6)
        Vm = np.full(6, port.init_vm(O.TT2, P))
        port.run(O.TT2, P, T, B, Vm, 3000, 1e-5, amp=W.TT2_STIM_NA, n_threads=nt)
        out.append((B.copy(), Vm.copy()))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.fixture(scope="module")
def ref():
    try:
        return O.Ref()
    except FileNotFoundError:
        pytest.skip("reference tree not present")


@pytest.mark.parametrize("model", MODELS)
def test_port_is_bitwise_reference(port, ref, model):
    """Fresh seeded case, not in the golden set: port and compiled reference agree bit for bit."""
    n, dt = 5, 2e-5
    cells = ref.create(model, dt, n)
    rp = cells.params()
    P = port.param_vector(model, rp)
    T = port.tables(model, P, dt)
    hn = W.TT2_HETERO if model == O.TT2 else W.CRN_HETERO
    sc = W.conductance_scales(99, n, len(hn), 0.7, 1.3)
    het = {}
    for k, name in enumerate(hn):
        het[name] = rp[name] * sc[k]
        cells.add_hetero(name, het[name])
    amp = W.TT2_STIM_NA if model == O.TT2 else W.CRN_STIM_PAPF
    tl = 1e-3 if model == O.TT2 else 2e-3
    vr = np.full(n, cells.init_vm())
    tr_r = cells.run(vr, 20000, dt, textbegin=0.01, textlen=tl, bcl=0.3, amp=amp, rec_every=7)
    B = port.init_state(model, P, n)
    vp = np.full(n, port.init_vm(model, P))
    tr_p = port.run(model, P, T, B, vp, 20000, dt, textbegin=0.01, textlen=tl, bcl=0.3, amp=amp, het=het,
                    rec_every=7)
    assert np.array_equal(tr_p, tr_r)
    Sr = cells.get_state()
    cols = [c for c in range(B.shape[1]) if not (model == O.TT2 and c == 22)]
    assert np.array_equal(B[:, cols], Sr[:, cols])


def test_backup_fixture_layout():
    """The backup-file fixture (tests/golden/make_golden.py backup) is laid out as
    acCELLerate::WriteBackup writes (acCELLerate.cpp:1616-1661): two header lines, then per node
    Vm and the model's block, nodes in global order."""
    data = (O.GOLDEN / "backup_mixed.abp").read_bytes()
    g = np.load(O.GOLDEN / "backup_mixed.npz")
    head = b"acCELLerateBackupVersion1.0\n0.05 7\n"
    assert data.startswith(head)
    nodes = {}
    for key in ("tt2", "crn", "ord_endo"):
        for k, gid in enumerate(g[f"ids_{key}"]):
            nodes[int(gid)] = np.concatenate([[g[f"vm_{key}"][k]], g[f"blocks_{key}"][k]])
    body = np.frombuffer(data[len(head):], "<f8")
    expect = np.concatenate([nodes[i] for i in range(7)])
    assert np.array_equal(body, expect)
    assert [nodes[i].size - 1 for i in range(3)] == [36, 22, 59]  # TT2, Courtemanche, O'Hara-Rudy blocks
