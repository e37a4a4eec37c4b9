"""Edge cases on the GPU: empty and single-cell batches through every entry point, and ragged
sizes (partial 128-cell tiles, fewer cells than one tile) through the learned macro step."""
import numpy as np
import pytest

import oracle as O
from cardiomechanics_gb300 import workloads as W

pytestmark = pytest.mark.gpu

DT = 1e-5
AMP = W.TT2_STIM_NA


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_empty_batch(gpu, precision):
    cm = gpu
    p = cm.Params(5, None, DT)
    b = cm.Batch(p, 0, cm.FP64 if precision == "fp64" else cm.MIXED)
    vm = np.zeros(0)
    assert b.calc(DT, vm).size == 0
    b.calc_update(DT, vm)
    b.run(vm, 100, amplitude=AMP)
    assert b.get_state().size == 0
    assert b.audit() == 0
    if precision == "mixed":
        sur = cm.Surrogate(p, substeps=10, seed=1)
        st = b.run_surrogate(sur, vm, 5, amplitude=AMP)
        assert st["cell_macro_steps"] == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_single_cell_against_oracle(gpu, port, precision):
    """One cell, one stimulated beat and its return to rest (500 ms), the fused driver loop against
    the oracle's."""
    cm = gpu
    p = cm.Params(5, None, DT)
    b = cm.Batch(p, 1, cm.FP64 if precision == "fp64" else cm.MIXED)
    vm = b.init_vm()
    b.run(vm, 50000, textlen=1e-3, bcl=1.0, amplitude=AMP)
    P = port.param_vector(O.TT2, O.load_params(O.TT2))
    B = port.init_state(O.TT2, P, 1)
    vo = np.full(1, port.init_vm(O.TT2, P))
    port.run(O.TT2, P, port.tables(O.TT2, P, DT), B, vo, 50000, DT, textlen=1e-3, bcl=1.0, amp=AMP)
    tol = 1e-8 if precision == "fp64" else 1e-4
    assert abs(vm[0] - vo[0]) <= tol, (vm[0], vo[0])
    assert b.audit() == 0


@pytest.mark.parametrize("n", [1, 127, 129, 385])
def test_macro_step_ragged_sizes(gpu, n):
    """Fewer cells than one tile, and partial last tiles: macro steps with a network whose output
    layer is zero (corrections 0) equal the coarse step alone, bit for bit, with the FP64 audit
    on; the audit sample is taken and checked."""
    cm = gpu
    p = cm.Params(5, None, DT)
    sur = cm.Surrogate(p, substeps=10, seed=2)
    prm = sur.mlp.get_params()
    prm[4][:] = 0.0
    prm[5][:] = 0.0
    sur.mlp.set_params(prm)
    sc = W.conductance_scales(8, n, 3, 0.9, 1.1)
    out, stats = [], []
    for mode in (cm.SUR_AUDIT_FP64, cm.SUR_COARSE_ONLY):
        b = cm.Batch(p, n, cm.MIXED)
        for k, name in enumerate(W.TT2_HETERO):
            b.add_hetero_value(name, p.get(name) * sc[k])
        vm = b.init_vm()
        stats.append(b.run_surrogate(sur, vm, 400, textlen=1e-3, bcl=1.0, amplitude=AMP, mode=mode, audit_mod=7))
        out.append((vm, b.get_state()))
        assert b.audit() == 0
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert np.all(np.isfinite(out[0][0]))
    st = stats[0]
    assert st["surrogate"] + st["fallback"] == n * 400
    assert st["audited"] > 0 and st["max_audit_err_mv"] < 5.0  # the coarse step vs 10 FP64 steps
