"""The CPU restatement of MCF's E16.8 particle-file text (oracle/mcf_format.py)
pinned to the Fortran E edit descriptor's form (0P scale factor:
[-]0.dddddddd, E+ee or +eee above 99, right-justified in 16) on hand-checked
values, including decimal ties (resolved to even) and carries into the
exponent; the statistic line's (I9,<n>E16.8) layout.  The device formatter is checked against it in test_gpu_output.py."""
import numpy as np
import pytest

from oracle.mcf_format import e16_8, i9, particle_rows, restart_text, statistic_line

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


def test_statistic_line_layout():
    assert i9(120) == "      120"
    assert i9(-99999999) == "-99999999"
    assert i9(1_000_000_000) == "*********"
    line = statistic_line(20, 0.002, 1.5, [0.25, -0.0, 0.0])
    assert line == ("       20  0.20000000E-02  0.15000000E+01  0.25000000E+00"
                    " -0.00000000E+00  0.00000000E+00\n")
    # stress_tensor on: s(2), s(3) of the column-major d*d sum
    line = statistic_line(3, 1.0, 2.0, [1.0, 2.0], stress=[9.0, 0.5, -0.125, 9.0])
    assert line.endswith("  0.50000000E+00 -0.12500000E+00\n")
    assert len(line) == 9 + 16 * 6 + 1
