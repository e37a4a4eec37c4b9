"""The oracle's explicit monodomain loop (oracle/cm_oracle.c, cmo_mono_run) against its pieces:
the CSR product summed row by row in order, the per-node scale and stimulus, and the oracle's
own single-cell Calc, composed step by step here in Python (bit for bit); plus a propagating
wave on a cable. The cell-model Calc itself is pinned to the reference by test_oracle*.py; the
PETSc tissue host (acCELLerate) does not build here, so the composition is checked against its
definition (acCELLerate.cpp:1839-2005), not against a run of acCELLerate."""
import numpy as np
import pytest

import oracle as O
from cardiomechanics_gb300 import workloads as W

EMT = {O.TT2: 5, O.CRN: 2, O.ORD: 12}
AMP = {O.TT2: W.TT2_STIM_NA, O.CRN: W.CRN_STIM_PAPF, O.ORD: W.ORD_STIM}


def setup(port, model, n):
    P = port.param_vector(model, O.load_params(model, "endo" if model == O.ORD else "epi"))
    T = port.tables(model, P, 1e-5) if model != O.ORD else np.zeros((0, O.RTDT))
    return P, T, port.init_state(model, P, n), np.full(n, port.init_vm(model, P))


@pytest.mark.parametrize("model", [O.TT2, O.CRN, O.ORD])
def test_mono_run_is_its_composition(port, model):
    nx, ny, steps, dt = 5, 4, 40, 1e-5
    n = nx * ny
    rp, col, val = W.grid_laplacian(nx, ny)
    P, T, B, vm = setup(port, model, n)
    vm[:3] += 0.03  # a perturbed corner drives currents through the operator
    scale = W.COUPLING_SCALE[EMT[model]] * np.linspace(0.9, 1.1, n)
    tb = np.where(np.arange(n) % 7 == 0, 0.0, 1e9)  # a few stimulated cells
    act = np.full(n, -1.0)
    B1, v1, a1 = B.copy(), vm.copy(), act.copy()
    port.mono_run(model, P, T, B1, v1, steps, dt, rp, col, val, scale=scale, textbegin_per_cell=tb,
                  textlen=1e-4, bcl=1.0, amp=AMP[model], act=a1, act_threshold=-0.06, n_threads=3)
    # the same steps composed here: product (CSR order), conversion, stimulus, Calc, update
    B2, v2, a2, tb2 = B.copy(), vm.copy(), act.copy(), tb.copy()
    t = 0.0
    for s in range(steps):
        prod = np.zeros(n)
        for i in range(n):
            acc = 0.0
            for e in range(rp[i], rp[i + 1]):
                acc += float(val[e]) * float(v2[col[e]])
            prod[i] = acc
        iext = np.zeros(n)
        for c in range(n):
            st = 0.0
            if t >= tb2[c]:
                st = AMP[model]
                if t >= tb2[c] + 1e-4:
                    tb2[c] += 1.0
            iext[c] = prod[c] * scale[c] + st
        dv = port.calc(model, P, T, B2, dt, v2, iext)
        v2 = v2 + dv
        hit = (a2 == -1.0) & (v2 >= -0.06)
        a2[hit] = t
        t += dt
    assert np.array_equal(v1, v2)
    assert np.array_equal(B1, B2)
    assert np.array_equal(a1, a2)


def test_wave_on_a_cable(port):
    """A 0.1 mm-spaced TT2 cable stimulated at one end: every cell activates, in order, at a
    conduction velocity in the physiological range (D = 0.1 mm^2/ms)."""
    n, steps, dt = 40, 6000, 1e-5
    rp, col, val = W.grid_laplacian(n, 1)
    P, T, B, vm = setup(port, O.TT2, n)
    tb = np.where(np.arange(n) < 3, 0.0, 1e9)
    act = np.full(n, -1.0)
    port.mono_run(O.TT2, P, T, B, vm, steps, dt, rp, col, val, uniform_scale=W.COUPLING_SCALE[5],
                  textbegin_per_cell=tb, textlen=1e-3, bcl=1.0, amp=2 * W.TT2_STIM_NA, act=act,
                  act_threshold=-0.02)
    assert np.all(act >= 0)
    assert np.all(np.diff(act[5:-5]) > 0)
    cv = (30 * 1e-4) / (act[35] - act[5])  # m/s
    assert 0.1 < cv < 1.5, cv


def test_range_check(port):
    n = 6
    rp, col, val = W.grid_laplacian(n, 1)
    P, T, B, vm = setup(port, O.TT2, n)
    with pytest.raises(FloatingPointError):
        port.mono_run(O.TT2, P, T, B, vm, 200, 1e-5, rp, col, val, uniform_scale=W.COUPLING_SCALE[5],
                      amp=2 * W.TT2_STIM_NA, textlen=2e-3, vm_range=0.01)
