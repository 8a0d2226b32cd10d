"""Rigid-body dynamics of the colloids on the GPU against the oracle.

With mcfg_set_colloid_dynamics every VV step integrates the colloids on the
device (marching_integrate_VV.F90:455-765): fluid drag and torque from the
boundary particles, Adams-Bashforth rotation, translation and velocity
updates, colloid-colloid repulsion, body force, accelerations, wrap, and the
boundary particles moved with their colloid.  Bars (FP64 path against the
oracle, the sums differ only in order):
  - colloid centres within 1e-11 of the box, velocities, angular
    velocities and their histories within 1e-9 of their scale, the
    accumulated orientation within 1e-11;
  - particle positions within 1e-9 of the box, velocities within 1e-7 of
    the velocity scale (the trajectory bars of the other parity tests).
The FP32-mixed path with list reuse and graph replay follows the FP64 path
within a stated error, and replays bit-identically to per-step launches.
"""
import math

import numpy as np
import pytest

from mcf_gb300 import SDPD, configs
from mcf_gb300.params import PRECISION_FP32_MIXED, ColloidDynamics
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def case(ab=3, nsub=2, n_side=24, n_colloid=4, radius=3.0, seed=13):
    w, cs = configs.c4_colloids(n_side=n_side, n_colloid=n_colloid, radius=radius,
                                v_scale=0.05, omega_scale=0.02)
    rng = np.random.default_rng(seed)
    fl = w.id[:, 1] == 0
    w.v[fl] = rng.normal(0, 1e-2, (int(fl.sum()), 3))
    w.x[fl] += rng.uniform(-0.1, 0.1, (int(fl.sum()), 3))
    cd = ColloidDynamics()
    cd.integrate_AB = ab
    cd.sub_time_step = nsub
    cd.step_start = 0
    cd.body_force_type = 1
    cd.body_force[0] = 0.05
    m = 4.0 / 3.0 * math.pi * cs.radius ** 3.0  # particles_compute_mass.F90, rho 1
    mmi = np.repeat((0.4 * m * cs.radius ** 2)[:, None], 3, 1)
    return w, cs, cd, m, mmi


def start(h, w, cs, cd, m, mmi):
    h.upload(w.x, w.v, w.m, w.id)
    h.set_colloids(cs.params, cs.x, cs.v, cs.omega, cs.radius)
    h.set_colloid_dynamics(cd, m, mmi)
    h.marching_init_force(0)


def pair(w, cs, cd, m, mmi, **over):
    p = w.params.copy()
    p.Brownian = 0
    p.kt = 0.0
    for k, v in over.items():
        setattr(p, k, v)
    g = SDPD(p)
    o = Oracle(p)
    for h in (g, o):
        start(h, w, cs, cd, m, mmi)
    return g, o


def states_close(a, b, L):
    assert np.max(np.abs(a["x"] - b["x"])) <= 1e-11 * L
    for k in ("v", "omega", "f", "alpha"):
        sc = np.abs(b[k]).max() + 1e-30
        assert np.max(np.abs(a[k] - b[k])) <= 1e-9 * sc, k
    assert np.max(np.abs(a["acc"] - b["acc"])) <= 1e-11
    assert np.max(np.abs(a["theta"] - b["theta"])) <= 1e-11 * (np.abs(b["theta"]).max() + 1e-30)


@pytest.mark.parametrize("ab,nsub", [(1, 1), (3, 2), (5, 1)])
def test_colloid_dynamics_fp64_matches_oracle(gpu_lib, ab, nsub):
    w, cs, cd, m, mmi = case(ab, nsub)
    g, o = pair(w, cs, cd, m, mmi)
    a, b = g.colloid_state(), o.colloid_state()
    states_close(a, b, 24.0)  # the initial accelerations
    nsteps = 12
    for s in range(1, nsteps + 1):
        g.marching_integrate_VV(s, w.dt * 40)
        o.marching_integrate_VV(s, w.dt * 40)
    a, b = g.colloid_state(), o.colloid_state()
    states_close(a, b, 24.0)
    assert np.max(np.abs(b["v"][0] - cs.v)) > 1e-6  # the colloids did accelerate
    pa, pb = g.download("x", "v"), o.download("x", "v")
    assert np.max(np.abs(pa["x"] - pb["x"])) <= 1e-9 * 24.0
    assert np.max(np.abs(pa["v"] - pb["v"])) <= 1e-7 * np.abs(pb["v"]).max()


def test_colloid_integrate_stage_entry(gpu_lib):
    w, cs, cd, m, mmi = case(ab=2, nsub=1)
    g, o = pair(w, cs, cd, m, mmi)
    g.colloid_integrate(1, 2e-3)
    o.colloid_integrate(1, 2e-3)
    states_close(g.colloid_state(), o.colloid_state(), 24.0)
    bp = w.id[:, 1] > 0
    xa, xb = g.download("x")["x"], o.download("x")["x"]
    d = (xa - xb)[bp]
    d -= 24.0 * np.round(d / 24.0)  # the device keeps each particle's periodic image
    assert np.max(np.abs(d)) <= 1e-11 * 24.0


def test_colloid_dynamics_reuse_graph_and_fp32(gpu_lib):
    w, cs, cd, m, mmi = case(ab=3, nsub=1)
    dt = w.dt * 20
    runs = {}
    for name, prec, reuse in (("fp64", 0, 0), ("fp64_reuse", 0, 1), ("fp32_reuse", 1, 1)):
        p = w.params.copy()
        p.Brownian = 0
        p.kt = 0.0
        p.precision = PRECISION_FP32_MIXED if prec else 0
        p.reserved[1] = reuse
        hs = []
        for mode in ("step", "run"):
            h = SDPD(p)
            start(h, w, cs, cd, m, mmi)
            if mode == "step":
                for s in range(1, 31):
                    h.marching_integrate_VV(s, dt)
            else:
                h.run_vv(0, 30, dt)
            hs.append((h.colloid_state(), h.download("x", "v")))
        # graph replay (run_vv) and per-step launches give the same bits
        for k in ("x", "v", "omega"):
            assert np.array_equal(hs[0][0][k], hs[1][0][k]), (name, k)
        assert np.array_equal(hs[0][1]["x"], hs[1][1]["x"]), name
        runs[name] = hs[0]
    a, b = runs["fp64_reuse"], runs["fp64"]
    states_close(a[0], b[0], 24.0)
    assert np.max(np.abs(a[1]["x"] - b[1]["x"])) <= 1e-9 * 24.0
    # FP32-mixed pair arithmetic: colloid velocities and angular velocities
    c32, c64 = runs["fp32_reuse"][0], runs["fp64"][0]
    ev = np.max(np.abs(c32["v"][0] - c64["v"][0])) / np.abs(c64["v"][0]).max()
    ew = np.max(np.abs(c32["omega"][0] - c64["omega"][0])) / np.abs(c64["omega"][0]).max()
    assert ev < 1e-4 and ew < 1e-3, (ev, ew)


def test_colloid_state_between_graph_replays(gpu_lib):
    # run, read the colloids, run again, read again: every read after graph
    # replays (run_vv's two-step graph, the host-array step's graph) returns
    # the device's current state, as per-step launches do
    w, cs, cd, m, mmi = case(ab=2, nsub=1)
    dt = w.dt * 20
    p = w.params.copy()
    p.Brownian = 0
    p.kt = 0.0
    p.reserved[1] = 1
    p.precision = PRECISION_FP32_MIXED
    ref = SDPD(p)
    start(ref, w, cs, cd, m, mmi)
    ref_states = []
    for s in range(1, 21):
        ref.marching_integrate_VV(s, dt)
        if s in (8, 20):
            ref_states.append(ref.colloid_state())
    g = SDPD(p)
    start(g, w, cs, cd, m, mmi)
    g.run_vv(0, 8, dt)
    a8 = g.colloid_state()
    g.run_vv(8, 12, dt)
    a20 = g.colloid_state()
    for got, want in ((a8, ref_states[0]), (a20, ref_states[1])):
        for k in ("x", "v", "omega"):
            assert np.array_equal(got[k], want[k]), k
    # the host-array step: registered arrays replay its graph, plain arrays
    # take per-step launches; the reads between the steps agree
    runs = []
    for reg in (False, True):
        h = SDPD(p)
        start(h, w, cs, cd, m, mmi)
        st = h.download("x", "v")
        x, v = np.ascontiguousarray(st["x"]), np.ascontiguousarray(st["v"])
        if reg:
            h.host_register(x)
            h.host_register(v)
        try:
            for s in range(1, 9):
                h.step_vv_host(s, dt, x, v)
            b8 = h.colloid_state()
            for s in range(9, 21):
                h.step_vv_host(s, dt, x, v)
            b20 = h.colloid_state()
        finally:
            if reg:
                h.host_unregister(x)
                h.host_unregister(v)
        runs.append((b8, b20))
    for got, want in zip(runs[1], runs[0]):
        for k in ("x", "v", "omega"):
            assert np.array_equal(got[k], want[k]), k
    assert not np.array_equal(runs[1][0]["x"], runs[1][1]["x"])  # the colloids moved


def test_move_colloids_refused_while_integrating_on_device(gpu_lib):
    from mcf_gb300.mcfg import MCFGError

    w, cs, cd, m, mmi = case(ab=1, nsub=1)
    g, _ = pair(w, cs, cd, m, mmi)
    with pytest.raises(MCFGError):
        g.move_colloids(cs.x, None, cs.v, cs.omega)
