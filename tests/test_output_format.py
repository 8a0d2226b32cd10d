"""The CPU restatement of MCF's E16.8 particle-file text (oracle/mcf_format.py)
pinned to the Fortran E edit descriptor's form (0P scale factor:
[-]0.dddddddd, E+ee or +eee above 99, right-justified in 16) on hand-checked
values, including decimal ties (resolved to even) and carries into the
exponent.  The device formatter is checked against it in test_gpu_output.py."""
import numpy as np
import pytest

from oracle.mcf_format import e16_8, particle_rows, restart_text

CASES = [
    (1.0, "  0.10000000E+01"),
    (-1.5e-3, " -0.15000000E-02"),
    (0.0, "  0.00000000E+00"),
    (-0.0, " -0.00000000E+00"),
    (12.0, "  0.12000000E+02"),
    (1e100, "  0.10000000+101"),
    (1e-100, "  0.10000000E-99"),
    (1e-101, "  0.10000000-100"),
    (123456785.0, "  0.12345678E+09"),   # exact tie: to even
    (123456795.0, "  0.12345680E+09"),   # exact tie: to even (carry)
    (0.999999999, "  0.10000000E+01"),   # rounds up into the next decade
    (99999999.5, "  0.10000000E+09"),    # tie, 99999999 odd -> up, carry
    (3.14159265358979, "  0.31415927E+01"),
    (-2.5e-310, " -0.25000000-309"),
    (float("nan"), "             NaN"),
    (float("-inf"), "       -Infinity"),
]


@pytest.mark.parametrize("x,s", CASES)
def test_e16_8_known_values(x, s):
    assert e16_8(x) == s
    assert len(e16_8(x)) == 16


def test_rows_and_restart_layout():
    x = np.array([[1.0, 2.0, 3.0]])
    v = np.array([[0.5, -0.5, 0.0]])
    rows = particle_rows(x, v, [1.25], [1.0], np.array([[7, -3]]))
    assert rows.count("\n") == 1 and len(rows) == 10 * 16 + 1
    assert rows.split("\n")[0][-32:] == "  0.70000000E+01 -0.30000000E+01"
    assert restart_text(x, v, [1.25], [1.0], np.array([[7, -3]])).startswith("           1\n")
