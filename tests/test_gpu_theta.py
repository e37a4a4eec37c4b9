"""The implicit finite-element monodomain step (cm_theta_*, cm_batch_run_theta; acCELLerate::
IntraStep with IntraRHS, acCELLerate.cpp:1839-2005) against a direct solve and an oracle loop:
the oracle's cell update (the reference's Calc restated, bit-exact to it) with the driver's
stimulus rule and Godunov step, then b = R x and a sparse LU solve of A x = b (scipy).

Tolerances: the solve with rtol 1e-12 against the LU solution: 1e-10 relative; the coupled run
(rtol 1e-12): |dVm| <= 1e-7 V after 20 ms, activation times within one step; with the reference's
rtol = atol = 1e-6: activation times within one step."""
import numpy as np
import pytest

import oracle as O
from cardiomechanics_gb300 import workloads as W

pytestmark = pytest.mark.gpu
spla = pytest.importorskip("scipy.sparse.linalg")

DT = 1e-5


def operators(cm, nx, ny, nz=1, dt=DT):
    M, K = W.fe_q1_grid(nx, ny, nz)
    A, R = W.theta_operators(M, K, dt)
    return A, R, cm.Diffusion(*W.csr_arrays(A)), cm.Diffusion(*W.csr_arrays(R))


def test_solve_matches_direct(gpu):
    cm = gpu
    A, R, dA, dR = operators(cm, 40, 30)
    x = np.random.default_rng(2).normal(-0.08, 0.02, A.shape[0])
    ref = spla.spsolve(A.tocsc(), R @ x)
    th = cm.Theta(dA, dR, rtol=1e-12, atol=0.0, max_iter=500)
    st = th.solve(x)
    assert st["solves"] == 1 and st["not_converged"] == 0 and 0 < st["iterations"] < 500
    np.testing.assert_allclose(x, ref, rtol=1e-10, atol=1e-12)


def test_solve_meets_reference_test(gpu):
    """rtol = atol = 1e-6 (acCELLerate.cpp:21-22): the preconditioned residual meets PETSc's
    default test, max(rtol ||D^-1 b||, atol)."""
    cm = gpu
    A, R, dA, dR = operators(cm, 24, 20, 6)
    x0 = np.random.default_rng(3).normal(-0.08, 0.02, A.shape[0])
    b = R @ x0
    x = x0.copy()
    st = cm.Theta(dA, dR).solve(x)
    dinv = 1.0 / A.diagonal()
    z = dinv * (b - A @ x)
    assert np.linalg.norm(z) < max(1e-6 * np.linalg.norm(dinv * b), 1e-6)
    assert st["not_converged"] == 0


def oracle_run(port, A, R, n, nx, steps, tb0, amp, tlen, thr=-0.02):
    P = port.param_vector(O.TT2, O.load_params(O.TT2))
    T = port.tables(O.TT2, P, DT)
    B = port.init_state(O.TT2, P, n)
    vm = np.full(n, port.init_vm(O.TT2, P))
    act = np.full(n, -1.0)
    tb = tb0.copy()
    lu = spla.factorized(A.tocsc())
    t = 0.0
    for s in range(steps):
        port.run(O.TT2, P, T, B, vm, 1, DT, t0=t, textbegin_per_cell=tb.copy(), textlen=tlen, bcl=1e9, amp=amp)
        adv = (t >= tb) & (t >= tb + tlen)
        tb[adv] += 1e9
        vm[:] = lu(R @ vm)
        hit = (act == -1.0) & (vm >= thr)
        act[hit] = t
        t += DT
    return vm, act


@pytest.mark.parametrize("prec", [0, 1])
def test_sheet_against_oracle(gpu, port, prec):
    """A 48 x 16 TT2 sheet, left three columns stimulated, 20 ms."""
    cm = gpu
    nx, ny, steps = 48, 16, 2000
    n = nx * ny
    A, R, dA, dR = operators(cm, nx, ny)
    tb = np.where(np.arange(n) % nx < 3, 0.0, 1e9)
    amp = 2 * W.TT2_STIM_NA
    vo, ao = oracle_run(port, A, R, n, nx, steps, tb, amp, 1e-3)
    assert (ao >= 0).sum() > n // 3
    b = cm.Batch(cm.Params(cm.TENTUSSCHER2, None, DT), n, prec)
    th = cm.Theta(dA, dR, rtol=1e-12, atol=0.0)
    vm = b.init_vm()
    act = np.full(n, -1.0)
    st = b.run_theta(th, vm, steps, textbegin_per_cell=tb, textlen=1e-3, bcl=1e9, amplitude=amp, vm_range=0.2,
                     act=act)
    assert st["solves"] == steps and st["not_converged"] == 0
    hit = ao >= 0
    if prec == cm.FP64:
        assert np.abs(vm - vo).max() <= 1e-7
        assert np.array_equal(act >= 0, hit)
        assert np.abs(act - ao)[hit].max() <= DT * 1.0001
    else:  # the mixed cell update: activation within 0.1 ms, RMS Vm within 0.5 mV
        both = hit & (act >= 0)
        assert both.sum() >= hit.sum() - ny
        assert np.abs(act - ao)[both].max() <= 1e-4
        assert np.sqrt(np.mean((vm - vo) ** 2)) <= 0.5e-3
    # the reference's tolerances: the same activation map
    b2 = cm.Batch(cm.Params(cm.TENTUSSCHER2, None, DT), n, cm.FP64)
    vm2 = b2.init_vm()
    act2 = np.full(n, -1.0)
    st2 = b2.run_theta(cm.Theta(dA, dR), vm2, steps, textbegin_per_cell=tb, textlen=1e-3, bcl=1e9, amplitude=amp,
                       act=act2)
    assert st2["iterations"] < st["iterations"]
    assert np.array_equal(act2 >= 0, hit) and np.abs(act2 - ao)[hit].max() <= DT * 1.0001


def test_errors(gpu):
    cm = gpu
    A, R, dA, dR = operators(cm, 8, 8)
    neg = A.copy()
    neg.setdiag(-neg.diagonal())
    with pytest.raises(cm.CMError) as e:
        cm.Theta(cm.Diffusion(*W.csr_arrays(neg.tocsr())), dR)
    assert e.value.code == -1
    _, _, dA2, _ = operators(cm, 8, 9)
    with pytest.raises(cm.CMError):
        cm.Theta(dA2, dR)
    th = cm.Theta(dA, dR, rtol=1e-14, atol=0.0, max_iter=2)
    x = np.random.default_rng(0).normal(size=64)
    st = th.solve(x)  # out of iterations: a warning in the reference, a count here
    assert st["not_converged"] == 1 and st["iterations"] == 2
