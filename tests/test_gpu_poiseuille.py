"""Transient plane Poiseuille flow through the C-ABI against its analytic
series (Morris, Fox and Zhu 1997; the formula of MCF's
poiseuille_theoretical_2d.perl) and against the CPU oracle: the whole step
-- solid walls with Morris no-slip, body force, velocity Verlet -- over
thousands of steps.

Bars: from t = 0.07 L^2/nu on, the fluid velocity within 5% of u_max of the
series with the no-slip planes at the domain faces, and within 0.3% with the
planes 0.2 dx outside them (the discretisation's uniform slip, the same for
the oracle); looser at t = 0.017 L^2/nu, while the profile is steep; FP64
within 1e-7 of u_max of the oracle's trajectory (2D, 4000 steps)."""
import numpy as np
import pytest

from mcf_gb300 import SDPD, configs
from mcf_gb300.params import PRECISION_FP32_MIXED, PRECISION_FP64
from oracle.analytic import poiseuille_transient
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

F, NU = 0.01, 1.0


def profile_errors(w, d, t, L):
    fl = w.id[:, 1] == 0
    y, vx = d["x"][fl, 1], d["v"][fl, 0]
    ua = poiseuille_transient(y, t, F, NU, L)
    ub = poiseuille_transient(y + 0.2, t, F, NU, L + 0.4)
    return np.max(np.abs(vx - ua)) / ua.max(), np.max(np.abs(vx - ub)) / ub.max()


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_FP32_MIXED])
def test_channel_3d_against_series(gpu_lib, precision):
    L = 24
    w = configs.poiseuille_channel(dim=3, n_side=L, force=F, precision=precision)
    g = SDPD(w.params)
    g.upload(w.x, w.v, w.m, w.id)
    g.marching_init_force(0)
    s = 0
    # (time, bar with the planes at the faces, bar with the 0.2 dx slip):
    # the early profile is steep at the walls, where the slip model is coarse
    for t, b_face, b_slip in ((10.0, 0.08, 0.012), (40.0, 0.05, 3e-3), (100.0, 0.05, 3e-3)):
        n = int(round(t / w.dt)) - s
        g.run_vv(s, n, w.dt)
        s += n
        e_face, e_slip = profile_errors(w, g.download("x", "v"), s * w.dt, float(L))
        assert e_face < b_face, (t, e_face)
        assert e_slip < b_slip, (t, e_slip)


def test_channel_2d_fp64_against_oracle(gpu_lib):
    w = configs.poiseuille_channel(dim=2, n_side=20, force=F)
    g = SDPD(w.params)
    g.upload(w.x, w.v, w.m, w.id)
    o = Oracle(w.params)
    o.upload(w.x, w.v, w.m, w.id)
    g.marching_init_force(0)
    o.marching_init_force(0)
    g.run_vv(0, 4000, w.dt)
    o.run_vv(0, 4000, w.dt)
    a = g.download("x", "v")
    b = o.download("x", "v")
    umax = np.abs(b["v"][:, 0]).max()
    assert np.abs(a["v"] - b["v"]).max() <= 1e-7 * umax
    assert np.abs(a["x"] - b["x"]).max() <= 1e-9 * 20.0
    e_face, e_slip = profile_errors(w, a, 4000 * w.dt, 20.0)
    assert e_face < 0.05 and e_slip < 3e-3
