"""The finite-element operators of the implicit step's workloads and tests
(workloads.fe_q1_grid, theta_operators; the reference's setup at acCELLerate.cpp:541-653):
trilinear / bilinear elements on a structured grid, checked against their defining properties."""
import numpy as np
import pytest

from cardiomechanics_gb300 import workloads as W

sp = pytest.importorskip("scipy.sparse")


@pytest.mark.parametrize("dims", [(5, 4, 1), (4, 3, 3)])
def test_mass_and_stiffness(dims):
    nx, ny, nz = dims
    h, sigma = 1e-4, 0.1
    M, K = W.fe_q1_grid(nx, ny, nz, h=h, sigma=sigma)
    n = nx * ny * nz
    d = 2 if nz == 1 else 3
    vol = ((nx - 1) * h) * ((ny - 1) * h) * (((nz - 1) * h) if d == 3 else 1.0)
    one = np.ones(n)
    assert abs(one @ M @ one - vol) < 1e-12 * vol          # the mass integrates 1 to the volume
    assert np.abs(K @ one).max() < 1e-9 * np.abs(K).max()   # constants are in the stiffness kernel
    assert abs(M - M.T).max() == 0 and abs(K - K.T).max() == 0
    x = np.arange(nx, dtype=float) * h                      # a linear field in x: its energy
    f = np.tile(x, n // nx)
    assert abs(f @ K @ f - sigma * vol) < 1e-9 * sigma * vol
    # an interior row couples to 3^d nodes; on cubes the trilinear stiffness's six face couplings
    # vanish exactly (-16 h/36 + 2 x 8 h/36), leaving 21
    l = 1 + nx * (1 + (ny if d == 3 else 0))
    assert M[l].nnz == 3 ** d and K[l].nnz == (9 if d == 2 else 21)


def test_theta_operators():
    M, K = W.fe_q1_grid(6, 5, 1)
    dt, cmb, th = 1e-5, 1400.0, 0.5
    A, R = W.theta_operators(M, K, dt, cm_beta=cmb, theta=th)
    assert abs(A - (cmb / dt * M + th * K)).max() == 0
    assert abs(R - (cmb / dt * M - (1 - th) * K)).max() == 0
    assert np.linalg.eigvalsh(A.toarray()).min() > 0        # symmetric positive definite
    rp, col, val = W.csr_arrays(A)
    assert rp.dtype == np.int64 and col.dtype == np.int32 and val.dtype == np.float64
    assert all(np.all(np.diff(col[rp[i]:rp[i + 1]]) > 0) for i in range(A.shape[0]))  # sorted columns
