"""Writes cm_fp64_tables.h: the constants and tables of the table-driven FP64 exp and log in
cm_fp64_math.cuh, rounded from 200-bit values (mpmath). Run once after changing a table's size:
    python gen_fp64_tables.py > cm_fp64_tables.h
The values are plain mathematics: ln 2 split for exact products, 1/F_j and ln F_j for
F_j = 1 + j/128 (j = 0..128), and 2^(j/64) (j = 0..63) as head + tail pairs."""
import mpmath as mp

mp.mp.prec = 200


def head_bits(x, bits):
    """x truncated to its leading `bits` significant bits (so that small multiples are exact)."""
    m, e = mp.frexp(x)
    return float(mp.floor(m * 2**bits) / 2**bits * mp.mpf(2) ** e)


def array(name, vals, comment):
    out = [f"// {comment}", f"__device__ const double {name}[{len(vals)}] = {{"]
    for i in range(0, len(vals), 3):
        out.append("    " + ", ".join(float(v).hex() for v in vals[i:i + 3]) + ",")
    out.append("};")
    return "\n".join(out)


def main():
    ln2 = mp.log(2)
    ln2_hi = head_bits(ln2, 42)
    l64_hi = head_bits(ln2 / 64, 36)
    lines = [
        "// Generated by gen_fp64_tables.py (mpmath, 200-bit arithmetic); do not edit.",
        "#pragma once",
        "",
        "namespace cm {",
        "namespace fp64 {",
        "",
        f"constexpr double kLn2Hi = {ln2_hi.hex()};       // ln 2, leading 42 bits (m * kLn2Hi exact, |m| < 2^11)",
        f"constexpr double kLn2Lo = {float(ln2 - ln2_hi).hex()};       // ln 2 - kLn2Hi",
        f"constexpr double kLn2By64Hi = {l64_hi.hex()};   // ln 2 / 64, leading 36 bits (k * it exact, |k| < 2^17)",
        f"constexpr double kLn2By64Lo = {float(ln2 / 64 - l64_hi).hex()};   // ln 2 / 64 - kLn2By64Hi",
        f"constexpr double k64ByLn2 = {float(64 / ln2).hex()};     // 64 / ln 2",
        "",
    ]
    F = [1 + mp.mpf(j) / 128 for j in range(129)]
    # ln F_j's head on the grid of kLn2Hi (multiples of 2^-42), so that m kLn2Hi + kLogFHi[j] is
    # exact for |m| < 2^10: the logarithm's only large rounding is its last addition
    lh = [float(mp.nint(mp.log(f) * 2**42) / 2**42) for f in F]
    lines.append(array("kLogInvF", [1 / f for f in F], "1 / F_j, F_j = 1 + j/128"))
    lines.append(array("kLogFHi", lh, "ln F_j rounded to a multiple of 2^-42"))
    lines.append(array("kLogFLo", [mp.log(f) - mp.mpf(h) for f, h in zip(F, lh)], "ln F_j - kLogFHi[j]"))
    T = [mp.mpf(2) ** (mp.mpf(j) / 64) for j in range(64)]
    th = [float(t) for t in T]
    lines.append(array("kExp2Hi", th, "2^(j/64), rounded"))
    lines.append(array("kExp2Lo", [t - mp.mpf(h) for t, h in zip(T, th)], "2^(j/64) - kExp2Hi[j]"))
    lines += ["", "}  // namespace fp64", "}  // namespace cm", ""]
    print("\n".join(lines))


if __name__ == "__main__":
    main()
