"""Seeded synthetic workloads for the cell-model update.

Counter-based generator: value k of stream `seed` is splitmix64(seed * 2**32 + k), mapped to
a double in [0, 1) from its top 53 bits. Stateless, so any subset of cells can be
regenerated without generating the rest, identically in numpy and in C.

Conductance jitter follows the order "one draw per cell per parameter in the listed
order": draw index = cell * n_params + p.
"""
from __future__ import annotations

import numpy as np

_M1 = np.uint64(0x9E3779B97F4A7C15)
_M2 = np.uint64(0xBF58476D1CE4E5B9)
_M3 = np.uint64(0x94D049BB133111EB)


def splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = np.asarray(x, np.uint64) + _M1
        z = (z ^ (z >> np.uint64(30))) * _M2
        z = (z ^ (z >> np.uint64(27))) * _M3
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, idx: np.ndarray) -> np.ndarray:
    """U[0,1) doubles for draw indices idx of stream seed."""
    with np.errstate(over="ignore"):
        base = np.uint64(seed) << np.uint64(32)
        z = splitmix64(np.asarray(idx, np.uint64) + base)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def conductance_scales(seed: int, n_cells: int, n_params: int, lo: float, hi: float,
                       cells: np.ndarray | None = None) -> np.ndarray:
    """(n_params, len(cells)) scale factors U[lo, hi]; cells defaults to range(n_cells)."""
    c = np.arange(n_cells, dtype=np.uint64) if cells is None else np.asarray(cells, np.uint64)
    out = np.empty((n_params, c.size))
    for p in range(n_params):
        out[p] = lo + (hi - lo) * uniform(seed, c * np.uint64(n_params) + np.uint64(p))
    return out


# Stimulus: the ten Tusscher convention "-52 pA/pF" is the reference's i_external in nA per
# cell, which TenTusscher2.cpp:630 divides by 2.29656e-2 to get pA/pF.
TT2_STIM_NA = 52.0 * 2.29656e-2
# Courtemanche takes i_external in pA/pF directly (CourtemancheEtAl.h:52 default 20).
CRN_STIM_PAPF = 20.0
# O'Hara-Rudy adds i_external to its total current in uA/uF; its parameter files give
# amplitude -50 for 1 ms (OHaraRudy_*.ev, GetAmplitude() = amplitude, OHaraRudy.h:84).
ORD_STIM = -50.0
# Tomek: the same convention, amplitude -53 for 1 ms (Tomek_*.ev).
TOM_STIM = -53.0

# Per-cell heterogeneous conductances used by the workloads, by model.
TT2_HETERO = ("g_Na", "g_Kr", "g_K1")
CRN_HETERO = ("g_Na", "g_to", "g_CaL")
ORD_HETERO = ("INaF_Multiplier", "IKr_Multiplier", "IK1_Multiplier")
TOM_HETERO = ORD_HETERO

# Conductances a per-instance parameter set scales in the batched form, by model (the
# heterogeneity slots of each model).
TT2_INSTANCE_G = ("g_Na", "g_Kr", "g_K1", "g_Ks", "g_to", "g_CaL")
CRN_INSTANCE_G = ("g_Na", "g_to", "g_Ks", "g_CaL", "g_bNa", "g_bCa")
ORD_INSTANCE_G = ("INaF_Multiplier", "INaL_Multiplier", "Ito_Multiplier", "IKr_Multiplier", "IKs_Multiplier",
                  "IK1_Multiplier")


def batched_instances(seed: int, n_inst: int = 256, lo: int = 1_000, hi: int = 1_000_000,
                      g_lo: float = 0.8, g_hi: float = 1.2) -> list[dict]:
    """Instances of the batched form: size log-uniform in [lo, hi] cells, model ten Tusscher 2006
    or Courtemanche 1998 with equal probability, each of the model's six instance conductances
    scaled by U[g_lo, g_hi], stimulus phase U[0, 1) of the cycle length. Draw index of instance
    i, field k (0 size, 1 model, 2 phase, 3..8 conductances) = i * 9 + k."""
    out = []
    for i in range(n_inst):
        u = uniform(seed, np.arange(i * 9, i * 9 + 9, dtype=np.uint64))
        n = int(round(np.exp(np.log(lo) + (np.log(hi) - np.log(lo)) * u[0])))
        model = "TenTusscher2" if u[1] < 0.5 else "CourtemancheEtAl"
        names = TT2_INSTANCE_G if model == "TenTusscher2" else CRN_INSTANCE_G
        out.append({"n": n, "model": model, "phase": float(u[2]),
                    "scales": {nm: g_lo + (g_hi - g_lo) * float(u[3 + k]) for k, nm in enumerate(names)}})
    return out


def full_form_instances(seed: int, n_inst: int = 64, total: int = 1 << 24, align: int = 256) -> list[dict]:
    """Instances of the full chosen form: n_inst sizes with log-uniform weights over a factor of
    64, scaled to `total` cells and rounded to multiples of `align` (the last instance takes the
    remainder), and a stimulus phase U[0, 1) of the cycle length each. Draw index of instance i,
    field k (0 size, 1 phase) = i * 2 + k."""
    u = uniform(seed, np.arange(2 * n_inst, dtype=np.uint64)).reshape(n_inst, 2)
    w = np.exp(np.log(64.0) * u[:, 0])
    sizes = np.maximum(align, np.floor(w / w.sum() * total / align).astype(np.int64) * align)
    sizes[-1] += total - sizes.sum()
    return [{"n": int(sizes[i]), "phase": float(u[i, 1])} for i in range(n_inst)]


# Monodomain coupling: i_external per unit of A*Vm when A is a stiffness-type operator in 1/s
# (A*Vm in V/s, the local diffusion term being -A*Vm): TT2 takes nA per cell and converts with
# 2.29656e-2 nA per pA/pF (TenTusscher2.cpp:630), Courtemanche pA/pF, O'Hara-Rudy uA/uF with the
# sign of an outward current (OHaraRudy.cpp:525-533).
COUPLING_SCALE = {5: -2.29656e-2, 2: -1.0, 12: 1.0, 14: 1.0}


def grid_laplacian(nx: int, ny: int, nz: int = 1, d_over_h2: float = 1.0e4):
    """Finite-difference operator K of D * Laplacian on an nx x ny x nz grid with no-flux edges,
    in CSR (rowptr int64, col int32, val float64), node l = x + nx (y + ny z), columns sorted:
    K_ll = d_over_h2 * (number of neighbours), K_lm = -d_over_h2 for each neighbour m. The
    default 1e4 / s is D = 0.1 mm^2/ms on a 0.1 mm grid."""
    n = nx * ny * nz
    idx = np.arange(n, dtype=np.int64)
    x, y, z = idx % nx, (idx // nx) % ny, idx // (nx * ny)
    cols, vals = [], []
    nb = np.zeros(n, np.int64)
    offs = []
    for d, ok in ((-nx * ny, z > 0), (-nx, y > 0), (-1, x > 0), (1, x < nx - 1), (nx, y < ny - 1),
                  (nx * ny, z < nz - 1)):
        offs.append((d, ok))
        nb += ok
    entries = []
    for d, ok in offs[:3]:
        entries.append((np.where(ok, idx + d, -1), np.where(ok, -d_over_h2, 0.0)))
    entries.append((idx, nb * d_over_h2))
    for d, ok in offs[3:]:
        entries.append((np.where(ok, idx + d, -1), np.where(ok, -d_over_h2, 0.0)))
    C = np.stack([e[0] for e in entries], axis=1)
    V = np.stack([e[1] for e in entries], axis=1)
    keep = C >= 0
    rowptr = np.concatenate([[0], np.cumsum(keep.sum(axis=1))]).astype(np.int64)
    return rowptr, C[keep].astype(np.int32), V[keep].astype(np.float64)


def fe_q1_grid(nx: int, ny: int, nz: int = 1, h: float = 1.0e-4, sigma: float = 0.1):
    """Mass M and stiffness K (conductivity sigma [S/m]) of bilinear (nz = 1) or trilinear
    finite elements on a structured grid of nx x ny (x nz) nodes with spacing h [m], node
    l = x + nx (y + ny z), assembled as Kronecker products of the 1-D linear-element matrices
    (exact for tensor-product Q1 elements). Returns scipy CSR matrices (M, K)."""
    import scipy.sparse as sp

    def one_d(m):
        e = np.ones(m)
        mass = sp.diags([e[:-1], 4 * e, e[:-1]], [-1, 0, 1]).tolil() * (h / 6.0)
        mass[0, 0] = mass[m - 1, m - 1] = 2 * h / 6.0
        stiff = sp.diags([-e[:-1], 2 * e, -e[:-1]], [-1, 0, 1]).tolil() / h
        stiff[0, 0] = stiff[m - 1, m - 1] = 1.0 / h
        return mass.tocsr(), stiff.tocsr()

    dims = [nx, ny] + ([nz] if nz > 1 else [])
    mk = [one_d(m) for m in dims]
    M = mk[-1][0]
    for m, _ in reversed(mk[:-1]):
        M = sp.kron(M, m, format="csr")
    K = None
    for d in range(len(dims)):
        term = None
        for k in reversed(range(len(dims))):
            f = mk[k][1] if k == d else mk[k][0]
            term = f if term is None else sp.kron(term, f, format="csr")
        K = term if K is None else K + term
    K = (sigma * K).tocsr()
    M.sort_indices()
    K.sort_indices()
    return M.tocsr(), K


def theta_operators(M, K, dt: float, cm_beta: float = 0.01 * 1.4e5, theta: float = 0.5):
    """The reference's theta-scheme operators (acCELLerate.cpp:541-653): A = C_m beta/dt M + theta K
    (Intra.A) and R = C_m beta/dt M - (1 - theta) K (IntraRHS), both on the union of M's and K's
    patterns, in CSR with sorted columns. Default C_m beta: 1 uF/cm^2 x 1400/cm."""
    a = cm_beta / dt
    A = (a * M + theta * K).tocsr()
    R = (a * M - (1.0 - theta) * K).tocsr()
    A.sort_indices()
    R.sort_indices()
    return A, R


def csr_arrays(S):
    """(rowptr int64, col int32, val float64) of a scipy CSR matrix."""
    return S.indptr.astype(np.int64), S.indices.astype(np.int32), S.data.astype(np.float64)
