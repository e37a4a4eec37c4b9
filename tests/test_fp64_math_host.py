"""The FP64 exp, log and division of the FP64 cell-model steps (csrc/cm_fp64_math.cuh) and the
compensated-pair conversions of the mixed kernels (csrc/cm_common.cuh), checked on the host: the
committed tables equal their generator's output, and the device algorithms, emulated operation by
operation (every fused multiply-add rounded once, exactly as the device rounds it; the pair
conversion's integer steps on the bit patterns), stay within 1 ulp of the correctly rounded value
and give the FP64-instruction form's pair. The GPU tests (tests/test_gpu_fp64_math.py) run the
compiled functions themselves."""
import io
import math
import random
import re
import struct
from contextlib import redirect_stdout
from fractions import Fraction
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "cardiomechanics_gb300" / "csrc"
HEADER = (CSRC / "cm_fp64_tables.h").read_text()


def _const(name):
    return float.fromhex(re.search(name + r" = (\S+);", HEADER).group(1))


def _table(name):
    body = re.search(name + r"\[\d+\] = \{(.*?)\};", HEADER, re.S).group(1)
    return [float.fromhex(v.strip()) for v in body.split(",") if v.strip()]


LN2_HI, LN2_LO = _const("kLn2Hi"), _const("kLn2Lo")
L64_HI, L64_LO, INV64 = _const("kLn2By64Hi"), _const("kLn2By64Lo"), _const("k64ByLn2")
INV_F, LOGF_HI, LOGF_LO = _table("kLogInvF"), _table("kLogFHi"), _table("kLogFLo")
EXP_HI, EXP_LO = _table("kExp2Hi"), _table("kExp2Lo")
SHIFT = float.fromhex("0x1.8p52")


def fma(a, b, c):
    return float(Fraction(a) * Fraction(b) + Fraction(c))  # one rounding, as the device's fma


def bits(x):
    return struct.unpack("<q", struct.pack("<d", x))[0]


def from_bits(i):
    return struct.unpack("<d", struct.pack("<q", i))[0]


def ulps(a, b):
    return abs(bits(a) - bits(b))


def exp64(x):
    """cm::fp64::exp64 for |x| < 700, step by step."""
    t = fma(x, INV64, SHIFT)
    k = bits(t) & 0xFFFFFFFF
    k = k - (1 << 32) if k >= 1 << 31 else k
    kd = t - SHIFT
    r = fma(-kd, L64_HI, x)
    r = fma(-kd, L64_LO, r)
    j, m = k & 63, k >> 6
    q = fma(r, 1.0 / 720, 1.0 / 120)
    q = fma(q, r, 1.0 / 24)
    q = fma(q, r, 1.0 / 6)
    q = fma(q, r, 0.5)
    p = fma(q, r * r, r)
    y = EXP_HI[j] + fma(EXP_HI[j], p, EXP_LO[j])
    yb = bits(y)
    return from_bits((((yb >> 32) + (m << 20)) << 32) | (yb & 0xFFFFFFFF))


def log64(x):
    """cm::fp64::log64 for positive normal x, step by step."""
    b = bits(x)
    hx, lo = b >> 32, b & 0xFFFFFFFF
    m = (hx >> 20) - 1023
    fr = hx & 0xFFFFF
    j = ((fr >> 12) + 1) >> 1
    y = from_bits(((fr | 0x3FF00000) << 32) | lo)
    f_j = from_bits((0x3FF00000 + (j << 13)) << 32)
    u = (y - f_j) * INV_F[j]
    q = fma(u, 1.0 / 7, -1.0 / 6)
    q = fma(q, u, 0.2)
    q = fma(q, u, -0.25)
    q = fma(q, u, 1.0 / 3)
    q = fma(q, u, -0.5)
    p = fma(q, u * u, u)
    a = fma(float(m), LN2_HI, LOGF_HI[j])
    bb = fma(float(m), LN2_LO, LOGF_LO[j]) + p
    return a + bb


def div64(a, b, r0):
    """cm::fp64::div64 from a given approximate reciprocal r0 of b."""
    e = fma(-b, r0, 1.0)
    r1 = fma(fma(e, e, e), r0, r0)
    q1 = a * r1
    return fma(fma(-b, q1, a), r1, q1)


def test_tables_are_the_generators():
    pytest.importorskip("mpmath")
    import importlib.util
    spec = importlib.util.spec_from_file_location("gen_fp64_tables", CSRC / "gen_fp64_tables.py")
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    out = io.StringIO()
    with redirect_stdout(out):
        gen.main()
    assert out.getvalue() == HEADER


def test_log_heads_sum_exactly():
    # m kLn2Hi + kLogFHi[j] is exact for |m| <= 1023: both on the 2^-42 grid
    for v in [LN2_HI, *LOGF_HI]:
        assert Fraction(v) * 2**42 == int(Fraction(v) * 2**42)


def test_exp_log_within_one_ulp():
    rng = random.Random(7)
    xs = [rng.uniform(-60.0, 60.0) for _ in range(600)] + [rng.uniform(-699.0, 699.0) for _ in range(300)]
    xs += [0.0, 1e-300, -1e-17, 0.5, -0.5, 699.9, -699.9]
    for x in xs:
        assert ulps(exp64(x), math.exp(x)) <= 1, x
    ys = [math.exp(rng.uniform(-12.0, 12.0)) for _ in range(600)] + [math.exp(rng.uniform(-700.0, 700.0)) for _ in range(300)]
    ys += [1.0, 2.0, 0.5, 1.0 + 2.0**-52, 1.0 - 2.0**-53, 138.0, 8.0, 5.4, 3.0]
    for y in ys:
        assert ulps(log64(y), math.log(y)) <= 1, y


def test_division_from_any_reciprocal_within_2_to_minus_20():
    rng = random.Random(11)
    for _ in range(2000):
        a = rng.uniform(-1e3, 1e3) * 10.0 ** rng.randint(-30, 30)
        b = rng.uniform(0.01, 1e3) * 10.0 ** rng.randint(-30, 30)
        r0 = (1.0 / b) * (1.0 + rng.uniform(-1.0, 1.0) * 2.0**-20)
        q = div64(a, b, r0)
        assert ulps(q, a / b) <= 1, (a, b)


# ---- the compensated-pair conversions of csrc/cm_common.cuh (device integer forms), emulated

def _f32_bits(u):
    return struct.unpack("<f", struct.pack("<I", u & 0xFFFFFFFF))[0]


def _to_f32(x):
    return struct.unpack("<f", struct.pack("<f", x))[0]


def acc_from_double(x):
    """cm::acc_from_double's device form, step by step (integer arithmetic on the bit pattern)."""
    b = bits(x) & 0xFFFFFFFFFFFFFFFF
    hw, lw = b >> 32, b & 0xFFFFFFFF
    s = hw & 0x80000000
    e = (hw >> 20) & 0x7FF
    lr = (lw + 0x10000000) & 0xFFFFFFFF
    hr = (hw + (1 if lr < lw else 0)) & 0xFFFFFFFF
    er = (hr >> 20) & 0x7FF
    hi = (s | (((er - 896) & 0xFFFFFFFF) << 23) | ((hr & 0xFFFFF) << 3) | (lr >> 29)) & 0xFFFFFFFF
    rem = ((lw & 0x1FFFFFFF) << 3) & 0xFFFFFFFF
    rem = (rem - (1 << 32) if rem >= 1 << 31 else rem) >> 3
    rem = -rem if s else rem
    lo = 0.0
    if 949 <= e and er <= 1150:
        lo = _to_f32(_to_f32(float(rem)) * 2.0 ** (e - 1075))  # I2F rounds once; the scale is exact
    inf_or_nan = e == 0x7FF
    nan = inf_or_nan and ((hw & 0xFFFFF) | lw) != 0
    if e < 897:
        hi = s
    if er > 1150 or inf_or_nan:
        hi = s | 0x7F800000
    if nan:
        hi = s | 0x7FC00000
    return _f32_bits(hi), lo


def test_pair_conversion_emulated():
    rng = random.Random(13)
    xs = [rng.uniform(-0.1, 0.06) for _ in range(3000)]
    xs += [rng.choice([-1.0, 1.0]) * math.exp(rng.uniform(math.log(2.0**-73), math.log(2.0**127))) for _ in range(3000)]
    for x in xs:
        hi, lo = acc_from_double(x)
        h32 = _to_f32(x)
        ulp32 = math.ldexp(1.0, math.frexp(h32)[1] - 24)  # FP32 spacing at h32
        if abs(Fraction(x) - Fraction(h32)) * 2 == Fraction(ulp32):
            continue  # exact ties round away from zero here, to even in FP32: checked below
        assert hi == h32, x
        assert lo == _to_f32(x - h32), x
    # ties keep the pair exact
    for x in (1.0 + 2.0**-24, -(1.0 + 2.0**-24), 0.5 + 3.0 * 2.0**-25):
        hi, lo = acc_from_double(x)
        assert Fraction(hi) + Fraction(lo) == Fraction(x) and abs(hi) >= abs(_to_f32(x))
    # edge cases
    assert acc_from_double(0.0) == (0.0, 0.0) and math.copysign(1.0, acc_from_double(-0.0)[0]) == -1.0
    assert acc_from_double(1e-40)[0] == 0.0 and acc_from_double(2.0**-100) == (2.0**-100, 0.0)
    assert acc_from_double(1e39)[0] == math.inf and acc_from_double(-1e300)[0] == -math.inf
    assert math.isnan(acc_from_double(math.nan)[0]) and acc_from_double(math.inf)[0] == math.inf
