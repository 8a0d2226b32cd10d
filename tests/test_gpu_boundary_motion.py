"""GPU tests of the moving boundaries through the C-ABI against the CPU
oracle: Lees-Edwards y faces (sheared images, crossing with shifted x and
velocity) and moving / oscillating solid walls.

With the candidate list kept across steps (list reuse) the same bars hold
against the oracle over 300 steps with rebuilds in between.  Bars as for
the fixed boundaries: FP64 density within 1e-12 relative and
acceleration within 1e-12 of the per-particle scale S_i = sum_j |a_ij| at a
shear offset that is not a whole number of cells; kT = 0 trajectories of
100 steps within 1e-9 of the box (positions) and 1e-7 of the velocity
scale; the FP32-mixed path within 1e-4 of S_i.  Physics: under steady
simple shear the x-momentum flux across y planes per volume is -eta *
shear rate (the SDPD shear viscosity recovers its input, within the
kernel's discretisation error: 10% bound).
"""
import math

import numpy as np
import pytest

from mcf_gb300 import SDPD, configs
from mcf_gb300.params import PRECISION_FP32_MIXED, PRECISION_FP64
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def pair(w, time=0.0, shear_type=(0,) * 6, freq=(0.0,) * 6, **over):
    p = w.params.copy()
    for k, v in over.items():
        setattr(p, k, v)
    g = SDPD(p)
    g.set_boundary_motion(shear_type, freq, time)
    g.upload(w.x, w.v, w.m, w.id)
    o = Oracle(p)
    o.set_boundary_motion(shear_type, freq, time)
    o.upload(w.x, w.v, w.m, w.id)
    return g, o


def sheared(dim, n_side, rate=0.3, seed=41, amp=0.4):
    w = configs.lees_edwards(dim=dim, n_side=n_side, shear_rate=rate)
    rng = np.random.default_rng(seed)
    w.x = np.mod(w.x + rng.uniform(-amp, amp, w.x.shape), float(n_side))
    return w


@pytest.mark.parametrize("time", [7.3, 1234.567])
@pytest.mark.parametrize("dim", [2, 3])
def test_le_fp64_density_force(gpu_lib, dim, time):
    w = sheared(dim, 16 if dim == 3 else 24)
    g, o = pair(w, time)
    g.marching_init_force(0)
    o.marching_init_force(0)
    a = g.download("rho", "f")
    b = o.download("rho", "f")
    assert np.max(np.abs(a["rho"] - b["rho"]) / b["rho"]) <= 1e-12
    scale = o.force_scale()[:, None] + np.abs(b["f"])
    assert np.max(np.abs(a["f"] - b["f"]) / scale) <= 1e-12
    assert abs(g.info()["shear_length"] - 0.3 * w.params.max_phys[0] * time) <= 1e-9 * time


@pytest.mark.parametrize("dim", [2, 3])
def test_le_fp64_trajectory(gpu_lib, dim):
    w = sheared(dim, 14 if dim == 3 else 20, rate=0.5)
    g, o = pair(w, 3.7)
    g.marching_init_force(0)
    o.marching_init_force(0)
    for s in range(1, 101):
        g.marching_integrate_VV(s, w.dt)
        o.marching_integrate_VV(s, w.dt)
    a = g.download("x", "v", "rho")
    b = o.download("x", "v", "rho")
    L = float(w.params.max_phys[0])
    d = np.abs(a["x"] - b["x"])
    d = np.minimum(d, L - d)
    assert d.max() <= 1e-9 * L
    assert np.abs(a["v"] - b["v"]).max() <= 1e-7 * np.abs(b["v"]).max()
    assert np.max(np.abs(a["rho"] - b["rho"]) / b["rho"]) <= 1e-10
    assert g.info()["time_current"] == o.time


@pytest.mark.parametrize("dim", [2, 3])
def test_le_fp32_mixed_force(gpu_lib, dim):
    w = sheared(dim, 16 if dim == 3 else 24, amp=0.05)
    g, o = pair(w, 7.3, precision=PRECISION_FP32_MIXED)
    g.marching_init_force(0)
    o.marching_init_force(0)
    a = g.download("rho", "f")
    b = o.download("rho", "f")
    assert np.max(np.abs(a["rho"] - b["rho"]) / b["rho"]) < 2e-6
    scale = o.force_scale()[:, None]
    assert np.max(np.abs(a["f"] - b["f"]) / scale) < 1e-4


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("osc", [False, True])
def test_moving_walls_fp64_trajectory(gpu_lib, dim, osc):
    w = configs.couette_walls(dim=dim, n_side=16 if dim == 3 else 24, v_top=0.2)
    freq = 2 * math.pi / 0.04
    st = (0, 0, 0, 2 if osc else 0, 0, 0)
    fr = (0, 0, 0, freq, 0, 0)
    g, o = pair(w, 0.0, st, fr)
    g.marching_init_force(0)
    o.marching_init_force(0)
    for s in range(1, 101):
        g.marching_integrate_VV(s, w.dt)
        o.marching_integrate_VV(s, w.dt)
    a = g.download("x", "v")
    b = o.download("x", "v")
    L = float(w.params.max_phys[0])
    d = np.abs(a["x"] - b["x"])
    d = np.minimum(d, L - d)
    assert d.max() <= 1e-9 * L
    assert np.abs(a["v"] - b["v"]).max() <= 1e-7 * np.abs(b["v"]).max()
    top = w.id[:, 1] == -4
    assert np.all(a["v"][top] == b["v"][top])


def test_le_and_walls_fp32_run_vv_equals_step_vv(gpu_lib):
    for w, t in ((sheared(3, 14), 2.5), (configs.couette_walls(dim=3, n_side=12), 0.0)):
        outs = []
        for mode in ("step", "run"):
            p = w.params.copy()
            p.precision = PRECISION_FP32_MIXED
            g = SDPD(p)
            g.set_boundary_motion((0,) * 6, (0.0,) * 6, t)
            g.upload(w.x, w.v, w.m, w.id)
            g.marching_init_force(0)
            if mode == "step":
                for s in range(1, 11):
                    g.marching_integrate_VV(s, w.dt)
            else:
                g.run_vv(0, 10, w.dt)
            outs.append(g.download("x", "v"))
        for k in ("x", "v"):
            assert np.array_equal(outs[0][k], outs[1][k])


@pytest.mark.parametrize("reuse", [0, 1])
@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_FP32_MIXED])
def test_le_shear_viscosity(gpu_lib, precision, reuse):
    # steady simple shear on the linear profile: the flux of x momentum
    # across y planes, sum_pairs r_y f_x / V -> -eta * rate (m = 1), averaged
    # over 400 steps.  (SDPD's viscous pair force is along v_ij, not r_ij,
    # so the pair virial is not symmetric: its r_x f_y part carries no
    # viscous stress.)
    rate = 0.05
    w = configs.lees_edwards(dim=3, n_side=16, shear_rate=rate, precision=precision)
    p = w.params
    p.stress_tensor = 1
    p.reserved[1] = reuse
    g = SDPD(p)
    g.set_boundary_motion((0,) * 6, (0.0,) * 6, 0.0)
    g.upload(w.x, w.v, w.m, w.id)
    g.marching_init_force(0)
    g.run_vv(0, 200, w.dt)
    acc, nsamp = 0.0, 0
    for s in range(200, 600, 20):
        g.run_vv(s, 20, w.dt)
        _, _, st = g.statistic_compute_statistic()
        acc += st[1]  # component (y, x): r_y f_x
        nsamp += 1
    V = 16.0 ** 3
    eta_eff = -(acc / nsamp) / V / rate
    assert abs(eta_eff / p.eta - 1.0) < 0.1, eta_eff
    # the profile stays linear: mean v_x per y slab against rate (y - L/2)
    r = g.download("x", "v")
    bins = np.floor(r["x"][:, 1] / 2.0).astype(int)
    prof = np.array([r["v"][bins == b, 0].mean() for b in range(8)])
    ref = rate * (2.0 * np.arange(8) + 1.0 - 8.0)
    assert np.max(np.abs(prof - ref)) < 0.1 * rate * 8.0


@pytest.mark.parametrize("dim", [2, 3])
def test_le_list_reuse_fp64_trajectory(gpu_lib, dim):
    # candidate list kept across steps: the crossing rows keep the cells of
    # the rebuild's shift while the images move (0.007-0.01 a step, past a
    # whole cell between rebuilds), rebuilds come from displacements off the
    # imposed shear and from particles re-entering through a y face (y
    # velocities of 0.2 carry dozens of them across)
    w = sheared(dim, 14 if dim == 3 else 20, rate=0.5)
    w.v[:, 1] += np.random.default_rng(5).normal(0.0, 0.2, w.v.shape[0])
    g, o = pair(w, 3.7)
    p = w.params.copy()
    p.reserved[1] = 1
    g = SDPD(p)
    g.set_boundary_motion((0,) * 6, (0.0,) * 6, 3.7)
    g.upload(w.x, w.v, w.m, w.id)
    g.marching_init_force(0)
    o.marching_init_force(0)
    for s in range(1, 301):
        g.marching_integrate_VV(s, w.dt)
        o.marching_integrate_VV(s, w.dt)
    info = g.info()
    assert info["skin"] > 0.3 and 3 <= info["list_rebuilds"] <= 150
    a = g.download("x", "v", "rho")
    b = o.download("x", "v", "rho")
    L = float(w.params.max_phys[0])
    d = np.abs(a["x"] - b["x"])
    d = np.minimum(d, L - d)
    assert d.max() <= 1e-9 * L
    assert np.abs(a["v"] - b["v"]).max() <= 1e-7 * np.abs(b["v"]).max()
    assert np.max(np.abs(a["rho"] - b["rho"]) / b["rho"]) <= 1e-10
    assert np.all((a["x"] >= 0.0) & (a["x"] < L))


def test_le_list_reuse_fp32_matches_rebuild_every_step(gpu_lib):
    w = sheared(3, 14, rate=0.5)
    w.v[:, 1] += np.random.default_rng(6).normal(0.0, 0.2, w.v.shape[0])
    outs = []
    for reuse in (0, 1):
        p = w.params.copy()
        p.precision = PRECISION_FP32_MIXED
        p.reserved[1] = reuse
        g = SDPD(p)
        g.set_boundary_motion((0,) * 6, (0.0,) * 6, 2.5)
        g.upload(w.x, w.v, w.m, w.id)
        g.marching_init_force(0)
        g.run_vv(0, 200, w.dt)
        outs.append((g.download("x", "v"), g.info()))
    assert outs[1][1]["list_rebuilds"] >= 2
    L = float(w.params.max_phys[0])
    d = np.abs(outs[0][0]["x"] - outs[1][0]["x"])
    d = np.minimum(d, L - d)
    assert d.max() <= 1e-6 * L
    vs = np.abs(outs[0][0]["v"]).max()
    assert np.abs(outs[0][0]["v"] - outs[1][0]["v"]).max() <= 1e-5 * vs


def test_le_rejects_what_it_does_not_support(gpu_lib):
    w = configs.lees_edwards(dim=3, n_side=14)
    p = w.params.copy()
    p.wall_v[3][2] = 0.1  # sliding along z
    with pytest.raises(Exception, match="only along x"):
        SDPD(p)
    small = configs.lees_edwards(dim=3, n_side=12)  # 3 x-cells of 3.0003
    with pytest.raises(Exception, match="4 cells along x"):
        SDPD(small.params)
    p = w.params.copy()
    p.stress_tensor = 1
    g = SDPD(p)
    g.upload(w.x, w.v, w.m, w.id)
    with pytest.raises(RuntimeError, match="periodic"):
        g.adjoint_run(0, 2, w.dt, [0.0] * 9)
