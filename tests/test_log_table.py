"""The constants of the DOP853 kernel's table-driven logarithm
(gala_gb300/csrc/gx_log_table.cuh, made by gen_log_table.py) checked against
60-digit values: 1/c_j is the double nearest 1/(1 + j/64); ln(c_j) high + low
carries ln(c_j) to ~2^-100 relative; ln 2 high is rounded to 32 significant
bits (its low 21 mantissa bits clear, so k ln 2 high is exact for |k| < 2^11)
and high + low carries ln 2 to ~2^-84 relative."""
import re
from pathlib import Path

import pytest

mpmath = pytest.importorskip("mpmath")

HEADER = Path(__file__).resolve().parents[1] / "gala_gb300" / "csrc" / "gx_log_table.cuh"
HEX = r"(-?0x[0-9a-fA-F.]+p[-+]?\d+)"


def _table():
    text = HEADER.read_text()
    rows = [tuple(float.fromhex(x) for x in m.groups())
            for m in re.finditer(r"\{" + HEX + r", " + HEX + r", " + HEX + r"\}", text)]
    consts = {name: float.fromhex(v) for name, v in re.findall(r"(LN2_HI|LN2_LO) = " + HEX, text)}
    return rows, consts


def test_log_table_against_60_digits():
    mpmath.mp.dps = 60
    rows, consts = _table()
    assert len(rows) == 65 and set(consts) == {"LN2_HI", "LN2_LO"}
    for j, (rc, hi, lo) in enumerate(rows):
        c = mpmath.mpf(1) + mpmath.mpf(j) / 64
        assert rc == float(1 / c), j                      # correctly rounded reciprocal
        err = abs(mpmath.mpf(hi) + mpmath.mpf(lo) - mpmath.log(c))
        assert err <= mpmath.mpf(2) ** -100 * max(abs(mpmath.log(c)), mpmath.mpf(2) ** -60), j
        assert abs(lo) <= abs(hi) * 2.0 ** -52 or hi == 0.0, j
    ln2 = mpmath.log(2)
    assert abs(mpmath.mpf(consts["LN2_HI"]) + mpmath.mpf(consts["LN2_LO"]) - ln2) <= ln2 * mpmath.mpf(2) ** -84
    mant = int(consts["LN2_HI"].hex().split(".")[1].split("p")[0], 16)
    assert mant & ((1 << 21) - 1) == 0
    for k in (-1074, -1023, -1, 1, 1023, 2047):   # every exponent log_f meets, and beyond
        assert mpmath.mpf(k * consts["LN2_HI"]) == k * mpmath.mpf(consts["LN2_HI"])
