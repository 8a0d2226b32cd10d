"""Analytic reference of the transient plane Poiseuille flow.  TEST
INFRASTRUCTURE ONLY: the tests compare the oracle's and the device path's
velocity profiles with it; the product never imports it.

Fluid at rest between no-slip planes y = 0 and y = L, driven from t = 0 by a
uniform body force F along x: the Fourier series of Morris, Fox and Zhu
(J. Comput. Phys. 136, 1997, eq. 21), the formula MCF's post-processing
script evaluates (mcf/scripts/poiseuille_theoretical_2d.perl:20-37, which
prints the profile with the opposite sign):

  u(y, t) = F/(2 nu) y (L - y)
            - sum_n 4 F L^2 / (nu pi^3 (2n+1)^3) sin((2n+1) pi y / L)
                    exp(-(2n+1)^2 pi^2 nu t / L^2)
"""
from __future__ import annotations

import math

import numpy as np


def poiseuille_transient(y, t: float, F: float, nu: float, L: float, tol: float = 1e-18):
    y = np.asarray(y, dtype=np.float64)
    u = F / (2.0 * nu) * y * (L - y)
    n = 0
    while True:
        k = 2 * n + 1
        term = (4.0 * F * L * L / (nu * math.pi ** 3 * k ** 3)
                * np.sin(math.pi * y / L * k) * math.exp(-k * k * math.pi ** 2 * nu * t / (L * L)))
        u = u - term
        n += 1
        if np.max(np.abs(term), initial=0.0) < tol or n > 100000:
            return u
