"""The FP64 exp, log and division of the FP64 cell-model steps (csrc/cm_fp64_math.cuh) against
the CUDA library's and against extended-precision host values.

The plain FP64 ten Tusscher step (reference TenTusscher2.cpp:615-906) evaluates 5 exponentials,
3 logarithms and 11 divisions per cell and step; on GB300 the step is bound by its FP64-pipe
instruction count, so it uses table-driven exp/log and a Newton division instead of the library
forms. These must stay within 1 ulp of the correctly rounded value over the argument ranges the
cell models produce and beyond."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ulps(a, b):
    """|a - b| in units in the last place: the difference of the float64 bit patterns, taken in
    int64 (same-sign values)."""
    return np.abs(a.view(np.int64) - b.view(np.int64))


def _cases(n, seed):
    rng = np.random.default_rng(seed)
    x = np.concatenate([
        rng.uniform(-60.0, 60.0, n),              # the cell models' exponents (scaled mV, tau ratios)
        rng.uniform(-699.0, 699.0, n // 4),       # the whole fast range
        np.array([0.0, -0.0, 1e-300, -1e-300, 1e-17, 0.5, -0.5, 700.0, -700.0, 709.0, -745.0]),
    ])
    y = np.concatenate([
        np.exp(rng.uniform(-12.0, 12.0, n)),      # concentrations, sums of rates
        np.exp(rng.uniform(-690.0, 690.0, n // 4)),
        np.array([1.0, 2.0, 0.5, 1.0 + 2.0**-52, 1.0 - 2.0**-53, 138.0, 8.0, 5.4, 1e-300, 3.0, 7.0]),
    ])
    return x, y


def test_fp64_math_against_library_and_extended(gpu):
    import torch
    cm = gpu
    x, y = _cases(1 << 17, 11)
    r = cm.fp64_math(torch.tensor(x, device="cuda"), torch.tensor(y, device="cuda"))
    exp64, log64, div64, exp_lib, log_lib, div_lib = r
    # the library's and ours: within 1 ulp of each other
    assert _ulps(exp64, exp_lib).max() <= 1
    assert _ulps(log64, log_lib).max() <= 1
    # division: the IEEE quotient (the device's and numpy's are both correctly rounded)
    assert np.array_equal(div_lib, x / y)
    assert _ulps(div64, div_lib).max() <= 1
    assert np.mean(div64 == div_lib) > 0.999
    # against extended precision, rounded to float64: at most 1 ulp
    ld = np.longdouble
    ref_exp = np.exp(x.astype(ld)).astype(np.float64)
    ref_log = np.log(y.astype(ld)).astype(np.float64)
    assert _ulps(exp64, ref_exp).max() <= 1
    assert _ulps(log64, ref_log).max() <= 1
    assert np.mean(exp64 == ref_exp) > 0.99
    assert np.mean(log64 == ref_log) > 0.99


def test_pair_conversions(gpu):
    """The mixed kernels' FP64 <-> compensated FP32 pair conversions, done on the bit patterns with
    integer instructions: the pair of the FP64-instruction form (hi = x rounded to FP32, lo = the
    rounded remainder), exact widening of every FP32 value, and the documented edge cases."""
    import torch
    cm = gpu
    rng = np.random.default_rng(5)
    normal = np.concatenate([
        rng.uniform(-0.1, 0.06, 1 << 16),                       # Vm [V]
        rng.choice([-1.0, 1.0], 1 << 15) * np.exp(rng.uniform(np.log(2.0**-73), np.log(2.0**127), 1 << 15)),
    ])
    ties = np.array([1.0 + 2.0**-24, -(1.0 + 2.0**-24), 3.0 * 2.0**-25 + 2.0**-1])  # remainder exactly half an ulp
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-40, -1e-40, 2.0**-100, 3e38, -3.4e38, 1e39, -1e300,
                        1.5e-45, 2.0**-127])
    x = np.concatenate([normal, ties, special])
    hi, lo, back, wid = cm.pair_convert(torch.tensor(x, device="cuda"))
    n = normal.size
    h32 = normal.astype(np.float32)
    assert np.array_equal(hi[:n], h32)
    assert np.array_equal(lo[:n], (normal - h32.astype(np.float64)).astype(np.float32))
    assert np.array_equal(back[:n], hi[:n].astype(np.float64) + lo[:n].astype(np.float64))
    assert np.all(np.abs(back[:n] - normal) <= np.abs(normal) * 2.0**-48)
    # ties: hi rounded away from zero, the pair still exact
    t = slice(n, n + ties.size)
    assert np.all(np.abs(hi[t]) >= np.abs(ties.astype(np.float32)))
    assert np.array_equal(hi[t].astype(np.float64) + lo[t].astype(np.float64), ties)
    # edge cases
    s = slice(n + ties.size, None)
    hs, ls = hi[s], lo[s]
    assert hs[0] == 0 and not np.signbit(hs[0]) and hs[1] == 0 and np.signbit(hs[1]) and ls[0] == 0 and ls[1] == 0
    assert hs[2] == np.inf and hs[3] == -np.inf and ls[2] == 0 and ls[3] == 0
    assert np.isnan(hs[4])
    assert hs[5] == 0 and not np.signbit(hs[5]) and hs[6] == 0 and np.signbit(hs[6])   # |x| < 2^-126: signed zero
    assert hs[7] == np.float32(2.0**-100) and ls[7] == 0                              # |x| < 2^-74: lo = 0
    assert hs[8] == np.float32(3e38) and np.isfinite(hs[8])
    assert hs[9] == np.float32(-3.4e38)
    assert hs[10] == np.inf and hs[11] == -np.inf and ls[10] == 0 and ls[11] == 0
    # widening: exact for every FP32 value, subnormal, zero, inf and NaN included
    with np.errstate(over="ignore"):  # 1e39 and -1e300 become infinite in FP32, as intended
        f = x.astype(np.float32)
    ok = ~np.isnan(f)
    assert np.array_equal(wid[ok], f[ok].astype(np.float64))
    assert np.array_equal(np.signbit(wid[ok]), np.signbit(f[ok]))
    assert np.all(np.isnan(wid[~ok]))
