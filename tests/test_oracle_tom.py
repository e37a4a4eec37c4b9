"""The Tomek (ToR-ORd) restatement in the oracle (oracle/cm_oracle.c, tom_*) pinned against the
reference: golden vectors generated by the reference's own Tomek class
(tests/golden/make_golden.py tom) for its three cell types, and, where the reference tree is
present, against the compiled reference directly (bit for bit)."""
import numpy as np
import pytest

import oracle as O
from cardiomechanics_gb300 import workloads as W

VARIANTS = list(O.TOM_VARIANTS)
NONE = np.zeros((0, O.RTDT))


def params(port, variant):
    return port.param_vector(O.TOM, O.load_params(O.TOM, variant))


def het_of(port, P, g):
    names = port.param_names(O.TOM)
    return {str(n): P[names.index(str(n))] * g["hetero_scale"][k] for k, n in enumerate(g["hetero_names"])}


@pytest.mark.parametrize("variant", VARIANTS)
def test_derived_parameters_match_reference(port, variant):
    ref = O.load_params(O.TOM, variant)
    P = params(port, variant)
    names = port.param_names(O.TOM)
    assert set(names) == set(ref)
    for i, name in enumerate(names):
        assert P[i] == ref[name], name
    assert port.L.cmo_n_tables(O.TOM) == 0 and port.state_doubles(O.TOM) == 84


@pytest.mark.parametrize("variant", VARIANTS)
def test_one_step_known_answers(port, variant):
    g = np.load(O.GOLDEN / f"step_tom_{variant}.npz")
    P = params(port, variant)
    dt = float(g["dt"])
    S = g["state_in"].copy()
    dV = port.calc(O.TOM, P, NONE, S, dt, g["vm"], g["i_ext"], het=het_of(port, P, g))
    np.testing.assert_allclose(S, g["state_out"], rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(dV, g["dvm"], rtol=1e-12, atol=1e-18)


@pytest.mark.parametrize("variant", VARIANTS)
def test_driver_trace(port, variant):
    g = np.load(O.GOLDEN / f"trace_tom_{variant}.npz")
    P = params(port, variant)
    dt = float(g["dt"])
    n = g["hetero_scale"].shape[1]
    B = port.init_state(O.TOM, P, n)
    Vm = np.full(n, port.init_vm(O.TOM, P))
    tr = port.run(O.TOM, P, NONE, B, Vm, int(g["n_steps"]), dt, textlen=float(g["textlen"]), bcl=float(g["bcl"]),
                  amp=float(g["amp"]), het=het_of(port, P, g), rec_every=int(g["rec_every"]))
    np.testing.assert_allclose(tr, g["trace"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(Vm, g["final_vm"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(B, g["final_state"], rtol=1e-8, atol=1e-12)
    assert tr.max() > 0.02


@pytest.fixture(scope="module")
def ref():
    try:
        return O.Ref()
    except FileNotFoundError:
        pytest.skip("reference tree not present")


@pytest.mark.parametrize("variant", ["endo", "mid"])
def test_port_is_bitwise_reference(port, ref, variant):
    """Fresh seeded case, per-cell multipliers and stretch with I_SAC on, not in the golden set."""
    n, dt = 5, 2e-5
    cells = ref.create(O.TOM, dt, n, ev=O.Ref.ev_path(O.TOM, variant))
    rp = cells.params()
    P = port.param_vector(O.TOM, rp)
    hn = ("INaF_Multiplier", "INaL_Multiplier", "Ito_Multiplier", "IKr_Multiplier", "IKs_Multiplier",
          "IK1_Multiplier")
    sc = W.conductance_scales(99, n, len(hn), 0.7, 1.3)
    het = {}
    for k, name in enumerate(hn):
        het[name] = rp[name] * sc[k]
        cells.add_hetero(name, het[name])
    vr = np.full(n, cells.init_vm())
    S0 = cells.get_state()
    S0[:, 4:6] = 0.0
    S0[:, 48:] = 0.0
    cells.set_state(S0)
    tr_r = cells.run(vr, 20000, dt, textbegin=0.01, textlen=1e-3, bcl=0.3, amp=W.TOM_STIM, rec_every=7)
    B = port.init_state(O.TOM, P, n)
    vp = np.full(n, port.init_vm(O.TOM, P))
    tr_p = port.run(O.TOM, P, NONE, B, vp, 20000, dt, textbegin=0.01, textlen=1e-3, bcl=0.3, amp=W.TOM_STIM, het=het,
                    rec_every=7)
    assert np.array_equal(tr_p, tr_r)
    assert np.array_equal(B, cells.get_state())
    # stretch and the stretch-activated current: one Calc per cell
    cells.add_hetero("ISAC_SWITCH", np.ones(n))
    names = port.param_names(O.TOM)
    Pcell = []
    for c in range(n):
        Pc = P.copy()
        Pc[names.index("ISAC_SWITCH")] = 1.0
        for name, vals in het.items():
            Pc[names.index(name)] = vals[c]
        Pcell.append(Pc)
    for stretch in (0.9, 1.1, 1.3):
        dv_r = cells.calc(dt, vr, np.zeros(n), stretch)
        dv_p = np.array([port.L.cmo_calc(O.TOM, O._ptr(Pcell[c]), None, B[c].ctypes.data_as(O._dp), dt,
                                         float(vp[c]), 0.0, stretch) for c in range(n)])
        assert np.array_equal(dv_p, dv_r), stretch
        assert np.array_equal(B, cells.get_state()), stretch
