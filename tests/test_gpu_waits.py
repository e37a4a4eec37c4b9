"""Bounded device waits run out and report, without a fault or a hang.

Every mbarrier wait of the bulk-copy kernels has a poll limit; when it runs out the kernel sets
CM_AUDIT_TIMEOUT (64) in the batch's audit mask, waits (bounded) for the copies it did issue,
frees its tensor memory and returns (the reference's analogue is the fatal NaN / range check
after the cell update, acCELLerate.cpp:1936-1946). The test hook cm_diag_batch_wait_check makes
the kernel issue no copy for one tile -- nothing is in flight for it -- with a short poll limit,
so the wait for that tile's data runs out; the cells of the tiles left undone keep their state,
every other cell matches an undisturbed run, and the batch works normally afterwards."""
import numpy as np
import pytest

from cardiomechanics_gb300 import workloads as W

pytestmark = pytest.mark.gpu

AUDIT_TIMEOUT = 64
SHORT = 1 << 16  # polls: a few milliseconds, far above a copy's latency


def _batches(cm, p, n, k=2):
    out = []
    for _ in range(k):
        b = cm.Batch(p, n, cm.MIXED)
        sc = W.conductance_scales(3, n, 3, 0.9, 1.1)
        for j, name in enumerate(W.TT2_HETERO):
            b.add_hetero_value(name, p.get(name) * sc[j])
        out.append(b)
    return out


def test_pipeline_wait_runs_out(gpu):
    import torch
    cm = gpu
    L = cm.lib()
    p = cm.Params(cm.TENTUSSCHER2, None, 1e-5)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    grid = 2 * sms                      # launch shape 7 = mixed_pipe_kernel<TT2, 256, 2>, 2 blocks per SM
    n = 256 * grid * 3                  # three tiles per block
    ref, b = _batches(cm, p, n)
    for x in (ref, b):
        x.set_launch(7, 2)
    v_ref, v = ref.init_vm(), b.init_vm()
    v0 = v.copy()
    skip = 5                            # block 5's first tile: that block leaves all its tiles undone
    assert L.cm_diag_batch_wait_check(b._h, skip, SHORT) == 0
    kw = dict(textbegin=0.0, textlen=1e-3, bcl=1.0, amplitude=W.TT2_STIM_NA)
    ref.run(v_ref, 1, **kw)
    b.run(v, 1, **kw)
    assert ref.audit() == 0
    assert b.audit() & AUDIT_TIMEOUT
    undone = np.zeros(n, bool)
    for t in range(skip, n // 256, grid):
        undone[t * 256:(t + 1) * 256] = True
    # (Vm goes through its FP32 hi/lo pair and back: equal to the pair's precision)
    np.testing.assert_allclose(v[undone], v0[undone], rtol=0, atol=1e-12)
    np.testing.assert_array_equal(v[~undone], v_ref[~undone])
    # the batch stays usable: the hook off, a fresh state, one step equals the undisturbed run
    assert L.cm_diag_batch_wait_check(b._h, -1, 0) == 0
    b.reset()
    v = b.init_vm()
    b.run(v, 1, **kw)
    assert b.audit() == 0
    np.testing.assert_array_equal(v, v_ref)


def test_macro_step_wait_runs_out(gpu):
    import torch
    cm = gpu
    L = cm.lib()
    p = cm.Params(cm.TENTUSSCHER2, None, 1e-5)
    sur = cm.Surrogate(p, substeps=10, seed=1)
    prm = sur.mlp.get_params()          # a network whose output layer is zero: the tensor-core path
    prm[4][:] = 0.0                     # runs (tensor memory allocated, three MMAs per tile) and the
    prm[5][:] = 0.0                     # step equals the coarse step
    sur.mlp.set_params(prm)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    n = 512 * sms * 2                   # 128-cell tiles, four per block and round
    ref, b = _batches(cm, p, n)
    v_ref, v = ref.init_vm(), b.init_vm()
    v0 = v.copy()
    skip = 7
    assert L.cm_diag_batch_wait_check(b._h, skip, SHORT) == 0
    rest = dict(textbegin=10.0, mode=0, audit_mod=0)  # no stimulus: every cell takes the learned step
    st_ref = ref.run_surrogate(sur, v_ref, 1, **rest)
    st = b.run_surrogate(sur, v, 1, **rest)
    assert ref.audit() == 0
    assert b.audit() & AUDIT_TIMEOUT
    tile = np.zeros(n, bool)
    tile[skip * 128:(skip + 1) * 128] = True
    # the tile whose copy never came is undone (Vm through its FP32 hi/lo pair and back)
    np.testing.assert_allclose(v[tile], v0[tile], rtol=0, atol=1e-12)
    moved = np.abs(v - v0) > 1e-12
    np.testing.assert_array_equal(v[moved], v_ref[moved])  # every cell advanced advanced correctly
    assert moved.sum() >= n - 4 * 128 * 2 and st["surrogate"] <= st_ref["surrogate"]
    # usable afterwards
    assert L.cm_diag_batch_wait_check(b._h, -1, 0) == 0
    b.reset()
    v = b.init_vm()
    b.run_surrogate(sur, v, 1, **rest)
    assert b.audit() == 0
    np.testing.assert_array_equal(v, v_ref)
