"""Generate gx_log_table.cuh: the constants of the table-driven FP64 logarithm
in gx_fast64.cuh (Tang's method: x = 2^k c_j (1 + r), c_j = 1 + j/64).

For j = 0..64 the table holds 1/c_j rounded to double, and ln(c_j) split as
hi + lo (hi rounded to double, lo = ln(c_j) - hi rounded to double), both from
60-digit arithmetic; ln 2 is split the same way with hi rounded to 32
significant bits so that k * hi is exact for |k| < 2^11.  Run:
    python gen_log_table.py > gx_log_table.cuh
"""
import mpmath

mpmath.mp.dps = 60


def split(x):
    hi = float(x)  # mpf -> nearest double
    lo = float(x - mpmath.mpf(hi))
    return hi, lo


def main():
    out = ["// gx_log_table.cuh -- generated by gen_log_table.py; do not edit.",
           "// Constants of the table-driven FP64 logarithm (log_f in gx_fast64.cuh):",
           "// for c_j = 1 + j/64, j = 0..64: {1 / c_j, ln(c_j) high part, ln(c_j) low part}.",
           "#pragma once", "", "namespace gx {", "namespace fast {", "",
           "static __device__ const double LOG_TAB[65][3] = {"]
    for j in range(65):
        c = mpmath.mpf(1) + mpmath.mpf(j) / 64
        inv = float(1 / c)
        hi, lo = split(mpmath.log(c))
        out.append(f"    {{{inv.hex()}, {hi.hex()}, {lo.hex()}}},  // j = {j}")
    out.append("};")
    ln2 = mpmath.log(2)
    # hi: ln 2 rounded to 32 significant bits
    m, e = mpmath.frexp(ln2)
    hi = float(mpmath.nint(m * 2 ** 32) * mpmath.mpf(2) ** (e - 32))
    lo = float(ln2 - mpmath.mpf(hi))
    out += ["", f"constexpr double LN2_HI = {hi.hex()};  // 32 significant bits",
            f"constexpr double LN2_LO = {lo.hex()};", "", "}  // namespace fast", "}  // namespace gx", ""]
    print("\n".join(out))


if __name__ == "__main__":
    main()
