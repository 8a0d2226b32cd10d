"""CPU restatement of MCF's particle-file and statistic-line text.  TEST INFRASTRUCTURE ONLY:
the tests compare the device formatter (mcfg_write_particles) with it; the product
never imports it.

MCF writes its particle output (io_write_particles.F90:225-403) and restart
files (io_write_restart_particles.F90:100-215) with ppm_io in ASCII mode:
WRITE(unit, '(<ncol>E16.8)') of the (ncol, N) array, one record per
particle; the restart file first writes the particle count list-directed
(ppm_io_write_ascii.F90: WRITE(unit, *)).  The statistic file gets one
line per write, (I9,<n>E16.8) of step, time, kinetic energy, momentum and
the stress sums s(2) s(3), trailing blanks trimmed
(io_write_statistic.F90:131-257).  E16.8 with the default scale
factor prints [-]0.d1...d8 followed by E+ee, or +eee when the exponent
exceeds 99, right-justified in 16 columns; the eight digits here are
Python's correctly rounded ones (ties to even), the C library's %.7E.
"""
from __future__ import annotations

import math

import numpy as np


def e16_8(x: float) -> str:
    x = float(x)
    if math.isnan(x):
        return "NaN".rjust(16)
    if math.isinf(x):
        return ("-Infinity" if x < 0 else "Infinity").rjust(16)
    neg = math.copysign(1.0, x) < 0
    ax = abs(x)
    if ax == 0.0:
        digits, e = "00000000", 0
    else:
        mant, ex = f"{ax:.7e}".split("e")
        digits = mant.replace(".", "")
        e = int(ex) + 1
    body = ("-" if neg else "") + "0." + digits
    if abs(e) <= 99:
        body += "E" + ("-" if e < 0 else "+") + f"{abs(e):02d}"
    else:
        body += ("-" if e < 0 else "+") + f"{abs(e):03d}"
    return body.rjust(16)


def particle_rows(x, v, rho, m, ids, s=None) -> str:
    """x(d) v(d) rho m pid sid [s(2) s(3)] per particle, (ncol E16.8)."""
    cols = [np.asarray(x, float), np.asarray(v, float), np.asarray(rho, float)[:, None],
            np.asarray(m, float)[:, None], np.asarray(ids, float)]
    if s is not None:
        cols.append(np.asarray(s, float)[:, 1:3])
    table = np.concatenate(cols, axis=1)
    return "".join("".join(e16_8(val) for val in row) + "\n" for row in table)


def restart_text(x, v, rho, m, ids) -> str:
    return f"{x.shape[0]:12d}\n" + particle_rows(x, v, rho, m, ids)


def i9(step: int) -> str:
    """Fortran I9: right-justified in 9 columns, asterisks when it does not fit."""
    t = str(int(step))
    return t.rjust(9) if len(t) <= 9 else "*" * 9


def statistic_line(step, time, k_energy, momentum, stress=None) -> str:
    """io_write_statistic.F90:131-257 without the optional flow_v_fixed,
    dynamic_density_ref and p_energy columns; stress is the d*d sum
    (column-major) when stress_tensor is on."""
    vals = [time, k_energy, *list(momentum)]
    if stress is not None:
        vals += [stress[1], stress[2]]
    return (i9(step) + "".join(e16_8(v) for v in vals)).rstrip() + "\n"
