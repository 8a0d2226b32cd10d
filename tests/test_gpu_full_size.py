"""FP64 GPU path against the oracle at the sizes of the five workloads.

The other parity tests run on 12^3-24^3 boxes; these run the workloads at
their own sizes through the C-ABI, with the oracle's threaded loops (MCF's
symmetric loop mode, symmetry = T, x-slabs of cells over all host cores)
as the checker:

  - C2, 64^3 = 262,144 particles, jittered lattice: cell lists bit-exact,
    one right-hand side at 1e-12 (density relative; acceleration of the
    per-particle scale sum_j |a_ij| + |a_i|, floored at 1e-6 of its median,
    since a pressure near zero has no relative accuracy), one with the
    random force at 1e-5 of
    the scale (FP32 Box-Muller normals, as in the small-box tests), then 10
    kT = 0 steps: positions within 1e-9 of the box, velocities within 1e-7
    of the velocity scale (the bars of the 100-step C1 trajectory);
  - C3, 100^3 fluid + 80,000 wall particles: cell lists bit-exact, one
    right-hand side at 1e-12, 5 kT = 0 steps at the trajectory bars;
  - C4, 96^3 lattice with 200 rigid spheres (moving, turning): one
    right-hand side at 1e-12, the boundary particles' rigid velocities, and
    drag and torque of every colloid within 1e-10 of the largest
    (particles_compute_interaction.F90:609-900,
    particles_collect_colloid_interaction.F90:93-136);
  - C4 with the colloids integrated on the device (Adams-Bashforth order 3,
    marching_integrate_VV.F90:455-765): 3 steps, colloid centres within
    1e-11 of the box, velocities and angular velocities within 1e-9 of their
    scale, particle positions and velocities at the trajectory bars;
  - C5, 128^2 Oldroyd-B: 10 kT = 0 steps, positions, velocities and the
    conformation tensor at the bars of the small Oldroyd-B test;
  - the FP32-mixed path at C3's and C4's sizes at the bars of the small
    FP32-mixed tests (density 2e-6 relative, acceleration 1e-4 of the
    per-particle scale, the random force with the same Philox draws; the
    colloids' boundary particles, drag and torque 1e-3), and with list
    reuse (the candidate list, the compact pair list, the sweep over it)
    5 kT = 0 steps: positions within 1e-9 of the box, velocities within
    the acceleration bar accumulated over the steps; C2's right-hand side
    with the random force; C5's conformation tensor after 10 steps within
    1e-3 of its change.
"""
import os

import numpy as np
import pytest

from mcf_gb300 import SDPD, configs
from mcf_gb300.params import PRECISION_FP32_MIXED
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

THREADS = max(1, os.cpu_count() or 1)


def pair(w, **over):
    p = w.params.copy()
    for k, v in over.items():
        setattr(p, k, v)
    g = SDPD(p)
    g.upload(w.x, w.v, w.m, w.id)
    o = Oracle(p, threads=THREADS)
    o.upload(w.x, w.v, w.m, w.id)
    return g, o


def lists_equal(g, o):
    g.particles_adjust_particles()
    o.particles_adjust_particles()
    ga = g.technique_build_list()
    oa = o.technique_build_list()
    for a, b in zip(ga, oa):
        assert np.array_equal(a, b)


def worst(err, scale, sid, a, b, k=4):
    """the particles furthest past the bar, for the failure message"""
    ratio = np.where(scale > 0, err / np.where(scale > 0, scale, 1.0), np.where(err > 0, np.inf, 0))
    r = ratio.max(1)
    idx = np.argsort(-r)[:k]
    return [(int(i), int(sid[i]), float(r[i]), a[i].tolist(), b[i].tolist()) for i in idx]


def rhs_close(g, o, step=0, tol=1e-12):
    g.marching_init_force(step)
    o.marching_init_force(step)
    a = g.download("rho", "f")
    b = o.download("rho", "f")
    assert np.all(np.abs(a["rho"] - b["rho"]) <= 1e-12 * np.abs(b["rho"]))
    # per-particle scale sum_j |a_ij| + |a_i|, with a floor of 1e-6 of its
    # median: the pressure c^2 (rho - rho_ref) carries an absolute error of
    # c^2 rho eps whatever its size, so the pressure force of a particle whose
    # partners all sit within ~1e-4 of rho_ref (a million-particle box has
    # some, most of them wall particles with few fluid partners near the
    # cut-off) has no relative accuracy in either implementation
    fs = o.force_scale()
    scale = fs[:, None] + np.abs(b["f"]) + 1e-6 * np.median(fs)
    err = np.abs(a["f"] - b["f"])
    ok = err <= tol * scale
    assert np.all(ok), worst(err, tol * scale, o.sid, a["f"], b["f"])
    return a, b


def trajectory_close(g, o, nsteps, dt, box, tol_x=1e-9, tol_v=1e-7, extra=()):
    g.run_vv(0, nsteps, dt)
    o.run_vv(0, nsteps, dt)
    a = g.download("x", "v", *extra)
    b = o.download("x", "v", *extra)
    assert np.max(np.abs(a["x"] - b["x"])) <= tol_x * box
    vs = np.abs(b["v"]).max()
    assert vs > 0
    assert np.max(np.abs(a["v"] - b["v"])) <= tol_v * vs
    return a, b


def c2_case():
    w = configs.c2_fluctuating_3d()  # lattice with 0.05 dx uniform jitter
    rng = np.random.default_rng(64)
    w.v = rng.normal(0.0, 1e-3, w.v.shape)
    return w


def test_c2_64cubed_lists_rhs_and_10_steps(gpu_lib):
    w = c2_case()
    g, o = pair(w, Brownian=0, kt=0.0)
    lists_equal(g, o)
    rhs_close(g, o)
    trajectory_close(g, o, 10, w.dt, 64.0)


def test_c2_64cubed_rhs_with_random_force(gpu_lib):
    w = c2_case()
    g, o = pair(w)  # kT = 1e-3, Hu-Adams noise
    assert w.params.Brownian == 1 and w.params.kt > 0
    rhs_close(g, o, step=11, tol=1e-5)


def test_c3_100cubed_walls_lists_rhs_and_5_steps(gpu_lib):
    w = configs.c3_poiseuille_3d()
    assert w.n == 1_080_000 and w.n_fluid == 1_000_000
    rng = np.random.default_rng(100)
    fl = w.id[:, 1] == 0
    w.x[fl] += rng.uniform(-0.05, 0.05, (int(fl.sum()), 3))
    w.v[fl] = rng.normal(0.0, 1e-3, (int(fl.sum()), 3))
    g, o = pair(w, Brownian=0, kt=0.0)
    lists_equal(g, o)
    rhs_close(g, o)
    trajectory_close(g, o, 5, w.dt, 100.0)


def test_c4_96cubed_200_colloids_rhs_drag_torque(gpu_lib):
    w, cs = configs.c4_colloids(v_scale=0.05, omega_scale=0.02)
    assert cs.x.shape[0] == 200
    rng = np.random.default_rng(96)
    fl = w.id[:, 1] == 0
    w.x[fl] += rng.uniform(-0.05, 0.05, (int(fl.sum()), 3))
    w.v[fl] = rng.normal(0.0, 1e-3, (int(fl.sum()), 3))
    g, o = pair(w, Brownian=0, kt=0.0)
    for h in (g, o):
        h.set_colloids(cs.params, cs.x, cs.v, cs.omega, cs.radius)
    rhs_close(g, o)
    bp = w.id[:, 1] > 0
    va = g.download("v")["v"]
    vb = o.download("v")["v"]
    assert np.allclose(va[bp], vb[bp], rtol=0, atol=1e-14)
    da, ta = g.colloid_drag()
    db, tb = o.colloid_drag()
    scale = np.abs(db).max() + np.abs(tb).max()
    assert scale > 0
    assert np.max(np.abs(da - db)) <= 1e-10 * scale
    assert np.max(np.abs(ta - tb)) <= 1e-10 * scale


def test_c4_96cubed_200_colloids_device_dynamics_3_steps(gpu_lib):
    import math

    from mcf_gb300.params import ColloidDynamics

    w, cs = configs.c4_colloids(v_scale=0.05, omega_scale=0.02)
    rng = np.random.default_rng(97)
    fl = w.id[:, 1] == 0
    w.v[fl] = rng.normal(0.0, 1e-3, (int(fl.sum()), 3))
    cd = ColloidDynamics()
    cd.integrate_AB = 3
    cd.sub_time_step = 1
    cd.body_force_type = 1
    cd.body_force[0] = 0.05
    m = 4.0 / 3.0 * math.pi * cs.radius ** 3.0
    mmi = np.repeat((0.4 * m * cs.radius ** 2)[:, None], 3, 1)
    g, o = pair(w, Brownian=0, kt=0.0)
    for h in (g, o):
        h.set_colloids(cs.params, cs.x, cs.v, cs.omega, cs.radius)
        h.set_colloid_dynamics(cd, m, mmi)
        h.marching_init_force(0)
    dt = 10 * w.dt
    g.run_vv(0, 3, dt)
    o.run_vv(0, 3, dt)
    a, b = g.colloid_state(), o.colloid_state()
    assert np.max(np.abs(a["x"] - b["x"])) <= 1e-11 * 96.0
    for k in ("v", "omega"):
        assert np.max(np.abs(a[k] - b[k])) <= 1e-9 * np.abs(b[k]).max(), k
    pa, pb = g.download("x", "v"), o.download("x", "v")
    assert np.max(np.abs(pa["x"] - pb["x"])) <= 1e-9 * 96.0
    assert np.max(np.abs(pa["v"] - pb["v"])) <= 1e-7 * np.abs(pb["v"]).max()


def test_c5_128squared_oldroyd_b_10_steps(gpu_lib):
    w = configs.c5_oldroyd_b_2d()
    assert w.n == 16384
    rng = np.random.default_rng(128)
    w.x = w.x + rng.uniform(-0.05, 0.05, w.x.shape)
    g, o = pair(w, Brownian=0, kt=0.0)
    ct0 = np.tile(np.array([1.0, 0.0, 0.0, 1.0]), (w.n, 1))
    for h in (g, o):
        h.upload(w.x, w.v, w.m, w.id, ct0)
    rhs_close(g, o)
    a, b = trajectory_close(g, o, 10, w.dt, 128.0, tol_x=1e-12, tol_v=1e-10, extra=("ct",))
    assert np.max(np.abs(a["ct"] - b["ct"])) <= 1e-12
    assert np.max(np.abs(b["ct"] - ct0)) > 1e-8  # the tensor has moved


def fp32_rhs_close(g, o, step=0, tol_boundary=1e-4):
    """the FP32-mixed path's bars: density 2e-6 relative, acceleration 1e-4
    of the per-particle scale (floored at 1e-6 of its median, as above);
    colloid boundary particles at tol_boundary"""
    g.marching_init_force(step)
    o.marching_init_force(step)
    a = g.download("rho", "f")
    b = o.download("rho", "f")
    assert np.max(np.abs(a["rho"] - b["rho"]) / b["rho"]) < 2e-6
    fs = o.force_scale()
    tol = np.where(o.sid > 0, tol_boundary, 1e-4)[:, None]
    scale = tol * (fs[:, None] + 1e-6 * np.median(fs))
    err = np.abs(a["f"] - b["f"])
    assert np.all(err <= scale), worst(err, scale, o.sid, a["f"], b["f"])


def c3_case():
    w = configs.c3_poiseuille_3d()
    rng = np.random.default_rng(100)
    fl = w.id[:, 1] == 0
    w.x[fl] += rng.uniform(-0.05, 0.05, (int(fl.sum()), 3))
    w.v[fl] = rng.normal(0.0, 1e-3, (int(fl.sum()), 3))
    return w


def test_c3_100cubed_fp32_mixed_rhs(gpu_lib):
    w = c3_case()
    g, o = pair(w, Brownian=0, kt=0.0, precision=PRECISION_FP32_MIXED)
    fp32_rhs_close(g, o)
    g, o = pair(w, precision=PRECISION_FP32_MIXED)  # kT = 1e-4, Hu-Adams noise
    fp32_rhs_close(g, o, step=7)


def test_c3_100cubed_fp32_mixed_list_reuse_5_steps(gpu_lib):
    # the headline path: candidate list, compact pair list, force sweep over it
    w = c3_case()
    p = w.params.copy()
    p.Brownian, p.kt, p.precision = 0, 0.0, PRECISION_FP32_MIXED
    p.reserved[1] = 1
    g = SDPD(p)
    g.upload(w.x, w.v, w.m, w.id)
    o = Oracle(p, threads=THREADS)
    o.upload(w.x, w.v, w.m, w.id)
    g.marching_init_force(0)
    o.marching_init_force(0)
    g.run_vv(0, 5, w.dt)
    o.run_vv(0, 5, w.dt)
    a = g.download("x", "v")
    b = o.download("x", "v")
    assert np.max(np.abs(a["x"] - b["x"])) <= 1e-9 * 100.0
    # the acceleration bar (1e-4 of the largest per-particle scale)
    # accumulated over the 5 steps
    assert np.max(np.abs(a["v"] - b["v"])) <= 1e-4 * o.force_scale().max() * 5 * w.dt
    assert g.info()["num_pairs"] > 100 * w.n


def test_c4_96cubed_200_colloids_fp32_mixed_rhs(gpu_lib):
    w, cs = configs.c4_colloids(v_scale=0.05, omega_scale=0.02)
    rng = np.random.default_rng(96)
    fl = w.id[:, 1] == 0
    w.x[fl] += rng.uniform(-0.05, 0.05, (int(fl.sum()), 3))
    w.v[fl] = rng.normal(0.0, 1e-3, (int(fl.sum()), 3))
    g, o = pair(w, Brownian=0, kt=0.0, precision=PRECISION_FP32_MIXED)
    for h in (g, o):
        h.set_colloids(cs.params, cs.x, cs.v, cs.omega, cs.radius)
    # the boundary particles carry the FP32 no-slip term (their offsets to
    # the centre and the clamped distance ratio in FP32): 1e-3 of their
    # scale, and so drag and torque
    fp32_rhs_close(g, o, tol_boundary=1e-3)
    da, ta = g.colloid_drag()
    db, tb = o.colloid_drag()
    scale = np.abs(db).max() + np.abs(tb).max()
    assert np.max(np.abs(da - db)) <= 1e-3 * scale
    assert np.max(np.abs(ta - tb)) <= 1e-3 * scale


def test_c2_64cubed_fp32_mixed_rhs_with_random_force(gpu_lib):
    w = c2_case()
    g, o = pair(w, precision=PRECISION_FP32_MIXED)  # kT = 1e-3, Hu-Adams noise
    fp32_rhs_close(g, o, step=11)


def test_c5_128squared_oldroyd_b_fp32_mixed_10_steps(gpu_lib):
    # the conformation tensor stays FP64; its change over the steps within
    # 1e-3 of the FP64 oracle's (the small Oldroyd-B FP32 bar)
    w = configs.c5_oldroyd_b_2d()
    rng = np.random.default_rng(128)
    w.x = w.x + rng.uniform(-0.05, 0.05, w.x.shape)
    g, o = pair(w, Brownian=0, kt=0.0, precision=PRECISION_FP32_MIXED)
    ct0 = np.tile(np.array([1.0, 0.0, 0.0, 1.0]), (w.n, 1))
    for h in (g, o):
        h.upload(w.x, w.v, w.m, w.id, ct0)
        h.marching_init_force(0)
        h.run_vv(0, 10, w.dt)
    a = g.download("ct", "x")
    b = o.download("ct", "x")
    dev = np.abs(b["ct"] - ct0)
    assert dev.max() > 1e-8
    assert np.max(np.abs(a["ct"] - b["ct"])) <= 1e-3 * dev.max() + 1e-9
    assert np.max(np.abs(a["x"] - b["x"])) <= 1e-9 * 128.0
