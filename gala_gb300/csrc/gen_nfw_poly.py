"""Generate gx_nfw_poly.cuh: the two polynomials of the FP32 NFW radial factor
F(u) = f(u) / u^3, f(u) = ln(1 + u) - u / (1 + u) (nfw_factor in gx_fp32.cuh).

  inside  (u < 1):  F = H(u) / (2 u),       H(u) = 2 f(u) / u^2
  outside (u >= 1): F = (ln u + K(w)) w^3,  K(w) = ln(1 + w) - 1 / (1 + w),  w = 1 / u

H and K are analytic on [0, 1] (their nearest singularity is at -1), so each is
a degree-10 polynomial in x = 2u - 1 (resp. 2w - 1) on [-1, 1]: the Chebyshev
approximation of mpmath.chebyfit from 50-digit values of H and K, written in
monomial form and rounded to float.  The script prints the approximation error
of each (before rounding) and the largest relative error of the float
coefficients evaluated in double, both on a dense grid.  Run:
    python gen_nfw_poly.py > gx_nfw_poly.cuh
"""
import sys

import mpmath
import numpy as np

mpmath.mp.dps = 50
DEG = 10


def H(x):
    u = (mpmath.mpf(x) + 1) / 2
    if u == 0:
        return mpmath.mpf(1)
    return 2 * (mpmath.log1p(u) - u / (1 + u)) / u ** 2


def K(y):
    w = (mpmath.mpf(y) + 1) / 2
    return mpmath.log1p(w) - 1 / (1 + w)


def fit(fn, name):
    poly, err = mpmath.chebyfit(fn, [-1, 1], DEG + 1, error=True)
    coef = [float(c) for c in reversed(poly)]  # c0 .. c10
    c32 = np.array(coef, dtype=np.float32).astype(np.float64)
    xs = np.linspace(-1.0, 1.0, 4001)
    exact = np.array([float(fn(x)) for x in xs])
    approx = np.polynomial.polynomial.polyval(xs, c32)
    scale = np.maximum(np.abs(exact), 0.19)  # f >= 0.19 where K is used, H >= 0.38
    rel = float(np.max(np.abs(approx - exact) / scale))
    print(f"{name}: approximation error {float(err):.2e}, float coefficients {rel:.2e}", file=sys.stderr)
    return coef


def main():
    h = fit(H, "H")
    k = fit(K, "K")
    out = ["// gx_nfw_poly.cuh -- generated by gen_nfw_poly.py; do not edit.",
           "// Degree-10 Chebyshev approximations on [-1, 1] (monomial coefficients c0..c10) of",
           "//   H(x) = 2 f(u) / u^2,           u = (x + 1) / 2   (NFW factor inside r_s)",
           "//   K(y) = ln(1 + w) - 1 / (1 + w), w = (y + 1) / 2   (NFW factor outside r_s)",
           "// with f(u) = ln(1 + u) - u / (1 + u), evaluated in Estrin's scheme (depth 4 after x).",
           "#pragma once", "", "namespace gx {", "",
           "__device__ __forceinline__ float estrin10(float x, float c0, float c1, float c2, float c3, float c4, float c5,",
           "                                          float c6, float c7, float c8, float c9, float c10) {",
           "    const float x2 = x * x, x4 = x2 * x2, x8 = x4 * x4;",
           "    const float b0 = fmaf(fmaf(c3, x, c2), x2, fmaf(c1, x, c0));",
           "    const float b1 = fmaf(fmaf(c7, x, c6), x2, fmaf(c5, x, c4));",
           "    const float b2 = fmaf(c10, x2, fmaf(c9, x, c8));",
           "    return fmaf(b2, x8, fmaf(b1, x4, b0));",
           "}", ""]
    for name, c in (("nfw_poly_h", h), ("nfw_poly_k", k)):
        vals = ", ".join(f"{float(np.float32(v))!r}f" for v in c)
        out.append(f"__device__ __forceinline__ float {name}(float x) {{")
        out.append(f"    return estrin10(x, {vals});")
        out.append("}")
        out.append("")
    out += ["}  // namespace gx", ""]
    print("\n".join(out))

if __name__ == "__main__":
    main()
