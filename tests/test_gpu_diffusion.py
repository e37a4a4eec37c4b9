"""GPU parity of the monodomain coupling (cm_diffusion_*, cm_batch_run_diffuse) against the
oracle's explicit monodomain loop (cmo_mono_run) on tissue sheets, for the four models.

Tolerances:
  product alone (FP64)   rtol 1e-13 against the CSR sum in order (the kernel fuses multiply-adds)
  fused run, FP64        |dVm| <= 1e-8 V after the run; activation times within one step
  fused run, mixed       activation times within 0.1 ms, RMS Vm error <= 0.5 mV per cell
  fused run vs apply + step_update_act (FP64): bit for bit (same product, same cell update)
"""
import numpy as np
import pytest

import oracle as O
from cardiomechanics_gb300 import workloads as W

pytestmark = pytest.mark.gpu

DT = 1e-5
OM = {5: O.TT2, 2: O.CRN, 12: O.ORD, 14: O.TOM}
AMP = {5: 2 * W.TT2_STIM_NA, 2: 2 * W.CRN_STIM_PAPF, 12: 2 * W.ORD_STIM, 14: 2 * W.TOM_STIM}
HET = {5: W.TT2_HETERO, 2: W.CRN_HETERO, 12: W.ORD_HETERO, 14: W.TOM_HETERO}
TLEN = {5: 1e-3, 2: 2e-3, 12: 1e-3, 14: 1e-3}  # Courtemanche: its own 2 ms stimulus (CourtemancheEtAl.h:54)


def csr_random(n, seed=3):
    """An irregular CSR matrix: row lengths 1..40 (slices of different widths), unsorted columns."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(1, 41, n)
    rowptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    col = rng.integers(0, n, rowptr[-1]).astype(np.int32)
    val = rng.standard_normal(rowptr[-1])
    return rowptr, col, val


def csr_mul(rowptr, col, val, x):
    y = np.zeros(rowptr.size - 1)
    for i in range(y.size):
        s = 0.0
        for e in range(rowptr[i], rowptr[i + 1]):
            s += val[e] * x[col[e]]
        y[i] = s
    return y


def test_apply_matches_csr(gpu):
    import torch
    cm = gpu
    n = 1000
    rp, col, val = csr_random(n)
    scale = np.linspace(-2.0, 3.0, n)
    x = np.random.default_rng(4).standard_normal(n)
    d = cm.Diffusion(rp, col, val, scale=scale)
    ref = csr_mul(rp, col, val, x) * scale
    np.testing.assert_allclose(d.apply(x), ref, rtol=1e-13, atol=1e-12)
    xd = torch.tensor(x, device="cuda")
    yd = torch.zeros(n, dtype=torch.float64, device="cuda")
    d.apply(xd, yd)
    torch.cuda.synchronize()
    np.testing.assert_allclose(yd.cpu().numpy(), ref, rtol=1e-13, atol=1e-12)
    du = cm.Diffusion(rp, col, val, uniform_scale=0.5)
    np.testing.assert_allclose(du.apply(x), 0.5 * csr_mul(rp, col, val, x), rtol=1e-13, atol=1e-12)


def sheet(cm, port, model, precision, nx, ny, steps, *, seed=1):
    """An nx x ny sheet (0.1 mm grid, D = 0.1 mm^2/ms), the left three columns stimulated at
    t = 0, conductances +-5 %; GPU run and oracle run. Returns both Vm, both act, both traces."""
    n = nx * ny
    rp, col, val = W.grid_laplacian(nx, ny)
    p = cm.Params(model, None, DT)
    P = port.param_vector(OM[model], O.load_params(OM[model], "endo" if model in (12, 14) else "epi"))
    names = port.param_names(OM[model])
    sc = W.conductance_scales(seed, n, 3, 0.95, 1.05)
    het = {k: P[names.index(k)] * sc[i] for i, k in enumerate(HET[model])}
    tb = np.where(np.arange(n) % nx < 3, 0.0, 1e9)
    b = cm.Batch(p, n, precision)
    for k, v in het.items():
        b.add_hetero_value(k, v)
    d = cm.Diffusion(rp, col, val, uniform_scale=W.COUPLING_SCALE[model])
    vm = b.init_vm()
    act = np.full(n, -1.0)
    b.run_diffuse(d, vm, steps, textbegin_per_cell=tb, textlen=TLEN[model], bcl=1.0, amplitude=AMP[model], act=act,
                  act_threshold=-0.02, vm_range=0.2)
    T = port.tables(OM[model], P, DT) if model not in (12, 14) else np.zeros((0, O.RTDT))
    B = port.init_state(OM[model], P, n)
    vo = np.full(n, port.init_vm(OM[model], P))
    ao = np.full(n, -1.0)
    port.mono_run(OM[model], P, T, B, vo, steps, DT, rp, col, val, uniform_scale=W.COUPLING_SCALE[model],
                  textbegin_per_cell=tb, textlen=TLEN[model], bcl=1.0, amp=AMP[model], het=het, act=ao,
                  act_threshold=-0.02, n_threads=8)
    return b, vm, vo, act, ao


@pytest.mark.parametrize("model,nx,ny,steps", [(5, 48, 16, 2500), (2, 40, 12, 2500), (12, 32, 10, 2000), (14, 32, 10, 2000)])
def test_sheet_fp64(gpu, port, model, nx, ny, steps):
    b, vm, vo, act, ao = sheet(gpu, port, model, gpu.FP64, nx, ny, steps)
    assert np.sum(ao >= 0) > nx * ny // 3          # the wave crossed a good part of the sheet
    assert np.abs(vm - vo).max() <= 1e-8
    assert np.array_equal(act >= 0, ao >= 0)
    assert np.abs(act - ao)[ao >= 0].max() <= DT * 1.0001
    assert b.audit() == 0


@pytest.mark.parametrize("model,nx,ny,steps", [(5, 48, 16, 2500), (2, 40, 12, 2500), (12, 32, 10, 2000), (14, 32, 10, 2000)])
def test_sheet_mixed(gpu, port, model, nx, ny, steps):
    b, vm, vo, act, ao = sheet(gpu, port, model, gpu.MIXED, nx, ny, steps)
    hit = ao >= 0
    assert hit.sum() > nx * ny // 3
    # cells at the edge of the front may cross the threshold one run and not the other
    both = hit & (act >= 0)
    assert both.sum() >= hit.sum() - ny
    assert np.abs(act - ao)[both].max() <= 1e-4    # activation within 0.1 ms
    assert np.sqrt(np.mean((vm - vo) ** 2)) <= 0.5e-3


def test_fused_equals_apply_plus_update(gpu):
    """The fused run against the same steps taken as cm_diffusion_apply + cm_batch_step_update_act
    (FP64): the same product and the same cell update, so bit for bit."""
    cm = gpu
    nx, ny, steps = 24, 8, 300
    n = nx * ny
    rp, col, val = W.grid_laplacian(nx, ny)
    p = cm.Params(5, None, DT)
    d = cm.Diffusion(rp, col, val, uniform_scale=W.COUPLING_SCALE[5])
    out = []
    for mode in ("fused", "split"):
        b = cm.Batch(p, n, cm.FP64)
        vm = b.init_vm()
        vm[: 3 * nx] += 0.06  # an initial depolarised strip instead of a stimulus
        act = np.full(n, -1.0)
        if mode == "fused":
            b.run_diffuse(d, vm, steps, act=act, act_threshold=-0.02)
        else:
            t = 0.0
            for s in range(steps):
                iext = d.apply(vm)
                b.calc_update_act(DT, vm, act, t, -0.02, i_ext=iext)
                t += DT
        out.append((vm.copy(), b.get_state(), act.copy()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2])
    assert np.sum(out[0][2] >= 0) > 3 * nx


def test_errors_and_range(gpu):
    cm = gpu
    p = cm.Params(5, None, DT)
    rp, col, val = W.grid_laplacian(8, 8)
    d = cm.Diffusion(rp, col, val, uniform_scale=W.COUPLING_SCALE[5])
    b = cm.Batch(p, 63, cm.FP64)
    with pytest.raises(cm.CMError) as e:
        b.run_diffuse(d, b.init_vm(), 10)
    assert e.value.code == -1
    b = cm.Batch(p, 64, cm.MIXED)
    vm = b.init_vm()
    with pytest.raises(cm.CMError) as e:  # a strong stimulus drives Vm past a 10 mV range
        b.run_diffuse(d, vm, 400, amplitude=5 * W.TT2_STIM_NA, textlen=4e-3, vm_range=0.01)
    assert e.value.code == -8
    assert b.audit() & cm.AUDIT_VMRANGE
