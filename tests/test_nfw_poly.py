"""The FP32 NFW radial factor of the compensated integrators (nfw_fac in
gala_gb300/csrc/gx_fp32.cuh, polynomials in gx_nfw_poly.cuh made by
gen_nfw_poly.py), restated here in float32 arithmetic (each fmaf a single
rounding, via float64 products of float32 operands) and checked against
f(u)/u^3, f(u) = ln(1 + u) - u / (1 + u), in 50-digit arithmetic over
u in [1e-3, 1e3]; the header's coefficients are the generator's."""
import re
import sys
from pathlib import Path

import numpy as np
import pytest

mpmath = pytest.importorskip("mpmath")

CSRC = Path(__file__).resolve().parents[1] / "gala_gb300" / "csrc"
f32 = np.float32


def _coefficients():
    text = (CSRC / "gx_nfw_poly.cuh").read_text()
    polys = {}
    for name in ("nfw_poly_h", "nfw_poly_k"):
        body = text[text.index(f"float {name}(float x)"):]
        args = body[body.index("estrin10(x, ") + len("estrin10(x, "):body.index(");")]
        polys[name] = [f32(float(v.rstrip("f"))) for v in args.split(",")]
    return polys


def _fma(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def _estrin10(x, c):
    x2 = f32(x * x)
    x4 = f32(x2 * x2)
    x8 = f32(x4 * x4)
    b0 = _fma(_fma(c[3], x, c[2]), x2, _fma(c[1], x, c[0]))
    b1 = _fma(_fma(c[7], x, c[6]), x2, _fma(c[5], x, c[4]))
    b2 = _fma(c[10], x2, _fma(c[9], x, c[8]))
    return _fma(b2, x8, _fma(b1, x4, b0))


def _nfw_fac(s2, si, irs, rs, polys):
    """nfw_fac with p0 = 1, exact log2 and 1/sqrt (the MUFU forms add their
    own ~1e-7)."""
    x = _fma(s2, f32(si * f32(f32(2.0) * irs)), f32(-1.0))
    y = _fma(si, f32(f32(2.0) * rs), f32(-1.0))
    lg = f32(np.log2(np.float64(f32(s2 * f32(irs * irs)))))
    w = f32(si * rs)
    inner = f32(_estrin10(x, polys["nfw_poly_h"]) * f32(si * f32(f32(0.5) * rs)))
    outer = f32(_fma(lg, f32(0.34657359027997264), _estrin10(y, polys["nfw_poly_k"])) * f32(w * f32(w * w)))
    return inner if x < 1.0 else outer


def test_nfw_factor_against_50_digits():
    mpmath.mp.dps = 50
    polys = _coefficients()
    rs = f32(15.6)
    irs = f32(1.0 / 15.6)
    worst = 0.0
    for u in np.geomspace(1e-3, 1e3, 3001):
        r = f32(u * 15.6)
        s2 = f32(r * r)
        si = f32(1.0 / np.sqrt(np.float64(s2)))
        got = _nfw_fac(s2, si, irs, rs, polys)
        # the exact factor at the radius and scale the float arithmetic carries
        uu = mpmath.sqrt(mpmath.mpf(float(s2))) * mpmath.mpf(float(irs))
        exact = (mpmath.log1p(uu) - uu / (1 + uu)) / uu ** 3
        worst = max(worst, abs(float(got) / float(exact) - 1.0))
    assert worst < 1e-6, worst


def test_header_is_the_generators_output(capsys):
    sys.path.insert(0, str(CSRC))
    try:
        import gen_nfw_poly
    finally:
        sys.path.pop(0)
    gen_nfw_poly.main()
    out = capsys.readouterr().out
    assert out.strip() == (CSRC / "gx_nfw_poly.cuh").read_text().strip()
    assert re.search(r"float nfw_poly_h\(float x\)", out)
