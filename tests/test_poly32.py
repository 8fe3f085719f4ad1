"""The FP32 Green function's polynomial coefficients (green.cuh, BEM_P32_*) are the
Liang-Wu-Noblesse polynomials of the reference (Kernels.cpp:120-256, BEM_POLY_TABLE)
and the StruveH1 constants (Kernels.cpp:76-116) re-expanded as the FP32 forms need
them, rounded to float: recomputed here with exact rational arithmetic (2/pi to 70
digits) and compared bit for bit.  Host only."""
import os
import re
from fractions import Fraction as Fr
from math import comb

import numpy as np

GREEN = os.path.join(os.path.dirname(__file__), "..", "bemuse_gb300", "csrc", "green.cuh")
TWO_OVER_PI = Fr("0.6366197723675813430755350534900574481378385829618257949906693762355871905")


def _src():
    return open(GREEN).read()


def _list(src, name):
    return [x.strip() for x in re.search(r"#define %s (.*)" % name, src).group(1).split(",")]


def _f32(x):
    return np.float32(float(x))  # Fraction -> double is correctly rounded, then to float


def _shift(c, x0):
    """Coefficients of p(x0 + u) in ascending powers of u from those of p(x)."""
    n = len(c)
    return [sum(c[i] * comb(i, j) * x0 ** (i - j) for i in range(j, n)) for j in range(n)]


def test_shifted_lwn_polynomials_match_the_reference_table():
    src = _src()
    tab = {m.group(1): [Fr(v.strip()) for v in m.group(3).split(",")]
           for m in re.finditer(r"X\((\w+), (\d+), ([^)]*)\)", src)}
    assert sorted(tab) == sorted(["A", "B", "C", "D", "dA", "dB", "dC"])
    for name, c in tab.items():
        want = [_f32(v) for v in _shift(c, Fr(1, 2))]
        got = [np.float32(v.rstrip("f")) for v in _list(src, "BEM_P32_" + name)]
        assert got == want, name


def test_h1_gap_coefficients_match_the_struve_constants():
    src = _src()
    hs = [Fr(v) for v in _list(src, "BEM_H1_SMALL")]
    c1 = [Fr(v) for v in _list(src, "BEM_H1_C1")]
    c2 = [Fr(v) for v in _list(src, "BEM_H1_C2")]
    q = _shift([TWO_OVER_PI] + [-h for h in hs], Fr(1, 2))
    want_s = [_f32(q[j] / Fr(9) ** j) for j in range(7)]
    want_d = [_f32(2 * (c2[i] - c1[i])) for i in range(4)]
    assert [np.float32(v.rstrip("f")) for v in _list(src, "BEM_P32_h1s")] == want_s
    assert [np.float32(v.rstrip("f")) for v in _list(src, "BEM_P32_h1d")] == want_d


def test_shifted_polynomial_is_the_same_polynomial():
    # the re-expansion is exact: both forms agree in FP64 to rounding on rho in [0, 1]
    src = _src()
    m = re.search(r"X\(A, 10, ([^)]*)\)", src)
    c = [float(v) for v in m.group(1).split(",")]
    s = [float(v) for v in _shift([Fr(v) for v in m.group(1).split(",")], Fr(1, 2))]
    rho = np.linspace(0.0, 1.0, 101)
    mono = sum(ci * rho ** i for i, ci in enumerate(c))
    shifted = sum(si * (rho - 0.5) ** i for i, si in enumerate(s))
    assert np.max(np.abs(mono - shifted)) < 1e-9 * np.max(np.abs(mono)) * 1e3
