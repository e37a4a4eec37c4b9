"""The O'Hara-Rudy restatement in the oracle (oracle/cm_oracle.c, ord_*) pinned against the
reference: golden vectors generated by the reference's own OHaraRudy class
(tests/golden/make_golden.py ord) for its three cell types, and, where the reference tree is
present, against the compiled reference directly (bit for bit)."""
import numpy as np
import pytest

import oracle as O
from cardiomechanics_gb300 import workloads as W

VARIANTS = list(O.ORD_VARIANTS)


def params(port, variant):
    return port.param_vector(O.ORD, O.load_params(O.ORD, variant))


def het_of(port, P, g):
    names = port.param_names(O.ORD)
    return {str(n): P[names.index(str(n))] * g["hetero_scale"][k] for k, n in enumerate(g["hetero_names"])}


@pytest.mark.parametrize("variant", VARIANTS)
def test_derived_parameters_match_reference(port, variant):
    ref = O.load_params(O.ORD, variant)
    P = params(port, variant)
    names = port.param_names(O.ORD)
    assert set(names) == set(ref), "parameter lists differ"
    for i, name in enumerate(names):
        assert P[i] == ref[name], name
    assert port.L.cmo_n_tables(O.ORD) == 0 and port.state_doubles(O.ORD) == 59


@pytest.mark.parametrize("variant", VARIANTS)
def test_one_step_known_answers(port, variant):
    """One Calc on states along paced trajectories, extreme voltages, with and without
    stimulus; celltype 1 and 2 take the epicardial / M-cell branches of Calc."""
    g = np.load(O.GOLDEN / f"step_ord_{variant}.npz")
    P = params(port, variant)
    dt = float(g["dt"])
    S = g["state_in"].copy()
    dV = port.calc(O.ORD, P, np.zeros((0, O.RTDT)), S, dt, g["vm"], g["i_ext"], het=het_of(port, P, g))
    np.testing.assert_allclose(S, g["state_out"], rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(dV, g["dvm"], rtol=1e-12, atol=1e-18)


@pytest.mark.parametrize("variant", VARIANTS)
def test_driver_trace(port, variant):
    g = np.load(O.GOLDEN / f"trace_ord_{variant}.npz")
    P = params(port, variant)
    dt = float(g["dt"])
    n = g["hetero_scale"].shape[1]
    B = port.init_state(O.ORD, P, n)
    Vm = np.full(n, port.init_vm(O.ORD, P))
    tr = port.run(O.ORD, P, np.zeros((0, O.RTDT)), B, Vm, int(g["n_steps"]), dt, textlen=float(g["textlen"]),
                  bcl=float(g["bcl"]), amp=float(g["amp"]), het=het_of(port, P, g), rec_every=int(g["rec_every"]))
    np.testing.assert_allclose(tr, g["trace"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(Vm, g["final_vm"], rtol=0, atol=1e-9)
    cols = [c for c in range(B.shape[1]) if c != 4]  # h_CaMK_fast: uninitialised in the reference
    np.testing.assert_allclose(B[:, cols], g["final_state"][:, cols], rtol=1e-8, atol=1e-12)
    assert tr.max() > 0.02  # an action potential in both beats


def test_celltypes_differ(port):
    """The three parameter files give three different action potentials (the celltype
    branches and multipliers are exercised)."""
    peaks = [np.load(O.GOLDEN / f"trace_ord_{v}.npz")["trace"].max() for v in VARIANTS]
    assert len(set(np.round(peaks, 6))) == 3


@pytest.fixture(scope="module")
def ref():
    try:
        return O.Ref()
    except FileNotFoundError:
        pytest.skip("reference tree not present")


@pytest.mark.parametrize("variant", ["endo", "mid"])
def test_port_is_bitwise_reference(port, ref, variant):
    """Fresh seeded case, not in the golden set: port and compiled reference agree bit for bit."""
    n, dt = 5, 2e-5
    cells = ref.create(O.ORD, dt, n, ev=O.Ref.ev_path(O.ORD, variant))
    rp = cells.params()
    P = port.param_vector(O.ORD, rp)
    hn = W.ORD_INSTANCE_G
    sc = W.conductance_scales(99, n, len(hn), 0.7, 1.3)
    het = {}
    for k, name in enumerate(hn):
        het[name] = rp[name] * sc[k]
        cells.add_hetero(name, het[name])
    vr = np.full(n, cells.init_vm())
    S0 = cells.get_state()
    S0[:, 4] = 0.0
    cells.set_state(S0)
    tr_r = cells.run(vr, 20000, dt, textbegin=0.01, textlen=1e-3, bcl=0.3, amp=W.ORD_STIM, rec_every=7)
    B = port.init_state(O.ORD, P, n)
    vp = np.full(n, port.init_vm(O.ORD, P))
    tr_p = port.run(O.ORD, P, np.zeros((0, O.RTDT)), B, vp, 20000, dt, textbegin=0.01, textlen=1e-3, bcl=0.3,
                    amp=W.ORD_STIM, het=het, rec_every=7)
    assert np.array_equal(tr_p, tr_r)
    assert np.array_equal(B, cells.get_state())


def test_stretch_and_sac_bitwise_reference(port, ref):
    """Stretch enters through the troponin Ca50 (lambda capped at 1.2) and, with ISAC_SWITCH on,
    through I_SAC; one Calc per cell at several stretches, port against reference."""
    n, dt = 6, 1e-5
    cells = ref.create(O.ORD, dt, n, ev=O.Ref.ev_path(O.ORD, "endo"))
    rp = cells.params()
    cells.add_hetero("ISAC_SWITCH", np.ones(n))
    P = port.param_vector(O.ORD, rp)
    g = np.load(O.GOLDEN / "step_ord_endo.npz")
    S = np.ascontiguousarray(g["state_in"][100:100 + n])
    vm = g["vm"][100:100 + n]
    for stretch in (0.9, 1.0, 1.1, 1.3):
        cells.set_state(S)
        dv_r = cells.calc(dt, vm, np.zeros(n), stretch)
        B = S.copy()
        Pc = P.copy()
        Pc[port.param_names(O.ORD).index("ISAC_SWITCH")] = 1.0
        dv_p = np.array([port.L.cmo_calc(O.ORD, O._ptr(Pc), None, B[c].ctypes.data_as(O._dp), dt, float(vm[c]), 0.0,
                                         stretch) for c in range(n)])
        assert np.array_equal(dv_p, dv_r), stretch
        assert np.array_equal(B, cells.get_state()), stretch
