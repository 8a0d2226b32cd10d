"""The oracle's rigid-body dynamics of the colloids (CPU, no GPU needed).

MCF integrates its colloids with explicit Adams-Bashforth steps inside the VV
step (marching_integrate_VV.F90:455-765).  These tests pin the oracle's
restatement of that update on systems of boundary particles alone (no
fluid, so the fluid drag is zero):

  - a constant body force: the centre and velocity follow an independent
    numpy restatement of the Fortran recursion bit for bit, orders 1-5
    (colloid_integrate_translate_position.F90 / _velocity.F90,
    colloid_compute_translate_acceleration.F90, the order ramping up from
    the first step after step_start, sub-steps);
  - a free rotation: the angular velocity stays constant, theta(3)
    accumulates |omega| dt per step, and the boundary particles turn
    rigidly about the centre (colloid_compute_rotation_vector.F90,
    tool_rotation_matrix.F90, particles_compute_colloid_relative/
    _absolute_position.F90);
  - two colloids pushing each other apart (DLVO repulsion): total momentum
    stays zero (colloid_compute_repulsion_cc.F90 summed per colloid).
"""
import math

import numpy as np
import pytest

from mcf_gb300 import configs
from mcf_gb300.params import ColloidDynamics, ColloidParams
from oracle.oracle import Oracle

# Fortran's expression order of the Adams-Bashforth increments
AB_COEF = {1: ([1.0], 1.0), 2: ([3.0, -1.0], 2.0), 3: ([23.0, -16.0, 5.0], 12.0),
           4: ([55.0, -59.0, 37.0, -9.0], 24.0),
           5: ([1901.0, -2774.0, 2616.0, -1274.0, 251.0], 720.0)}


def ab_incr(order, hist, dt):
    """( c1 h1 - c2 h2 + ... ) * dt / div, left to right, numpy float64"""
    if order == 1:
        return hist[0] * dt
    cs, div = AB_COEF[order]
    s = cs[0] * hist[0]
    for c, h in zip(cs[1:], hist[1:]):
        s = s + c * h if c > 0 else s - (-c) * h
    return s * dt / div


def sphere_shell(centre, radius, dx=1.0):
    """lattice sites within 1.05 * 3 dx inside a sphere's surface"""
    r = int(math.ceil(radius)) + 1
    g = np.arange(-r, r + 1, dtype=np.float64) * dx
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    d = np.sqrt((pts ** 2).sum(1))
    keep = (d <= radius) & (d > radius - 3.15)
    return pts[keep] + np.asarray(centre)


def colloids_only(centres, radius=3.0, L=24.0, omega=None, v=None, translate=1, rotate=0,
                  repul=0):
    """boundary particles of colloids in an otherwise empty periodic box"""
    xs, sids = [], []
    for c, ctr in enumerate(centres):
        p = sphere_shell(ctr, radius)
        xs.append(p)
        sids.append(np.full(len(p), c + 1, np.int32))
    x = np.concatenate(xs) % L
    sid = np.concatenate(sids)
    n = x.shape[0]
    w = configs.c4_colloids(n_side=int(L), n_colloid=1, radius=radius)[0]
    p = w.params.copy()
    p.Brownian = 0
    p.kt = 0.0
    p.body_force_type = 0
    ids = np.stack([np.arange(1, n + 1, dtype=np.int32), sid], 1)
    nc = len(centres)
    cp = ColloidParams()
    cp.num_colloid = nc
    cp.noslip_type = 2
    cp.translate = translate
    cp.rotate = rotate
    cp.cc_repul_type = repul
    cp.cc_repul_F0 = 10.0
    cp.cc_repul_cut_off = 0.1 * radius
    cp.cc_repul_cut_on = 0.01 * radius
    cp.dout = 0.05
    cx = np.asarray(centres, np.float64)
    cv = np.zeros((nc, 3)) if v is None else np.asarray(v, np.float64)
    om = np.zeros((nc, 3)) if omega is None else np.asarray(omega, np.float64)
    m = np.full(nc, 4.0 / 3.0 * math.pi * radius ** 3.0)
    mmi = np.repeat((0.4 * m * radius ** 2)[:, None], 3, 1)
    return p, x, np.zeros((n, 3)), np.ones(n), ids, cp, cx, cv, om, np.full(nc, radius), m, mmi


def dyn(ab=3, nsub=1, step_start=0, g=(0.0, 0.0, 0.0)):
    cd = ColloidDynamics()
    cd.integrate_AB = ab
    cd.sub_time_step = nsub
    cd.step_start = step_start
    cd.body_force_type = 1 if any(g) else 0
    for a in range(3):
        cd.body_force[a] = g[a]
    return cd


def make_oracle(case, cd):
    p, x, v, m, ids, cp, cx, cv, om, rad, cm, mmi = case
    o = Oracle(p)
    o.upload(x, v, m, ids)
    o.set_colloids(cp, cx, cv, om, rad)
    o.set_colloid_dynamics(cd, cm, mmi)
    o.marching_init_force(0)
    return o


@pytest.mark.parametrize("ab,nsub,step_start", [(1, 1, 0), (2, 1, 0), (3, 2, 0), (4, 1, 7),
                                                (5, 3, 0)])
def test_body_force_follows_the_fortran_recursion(ab, nsub, step_start):
    g = (0.013, -0.004, 0.0021)
    case = colloids_only([[6.0, 7.0, 8.0]])
    o = make_oracle(case, dyn(ab, nsub, step_start, g))
    dt = 0.05
    m = case[10][0]
    # restatement: f = (0 + g m) / m after init, then per sub-step
    x = np.array([6.0, 7.0, 8.0])
    vh = [np.zeros(3) for _ in range(ab)]
    fh = [np.zeros(3) for _ in range(ab)]
    fh = [(np.zeros(3) + np.array(g) * m) / m] + fh[:-1]
    dts = dt / nsub
    nsteps = 9
    for step in range(step_start + 1, step_start + 1 + nsteps):
        for i in range(1, nsub + 1):
            order = min(step - 1 + i - step_start, ab)
            x = x + ab_incr(order, vh, dts)
            vnew = vh[0] + ab_incr(order, fh, dts)
            vh = [vnew] + vh[:-1]
            fh = [(np.zeros(3) + np.array(g) * m) / m] + fh[:-1]
            x = np.where(x >= 24.0, x - 24.0, x)
        o.marching_integrate_VV(step, dt)
    st = o.colloid_state()
    assert np.array_equal(st["x"][0], x)
    assert np.array_equal(st["v"][:, 0, :], np.array(vh))
    assert np.array_equal(st["f"][:, 0, :], np.array(fh))
    # constant acceleration: every order integrates the velocity exactly
    t = nsteps * dt
    assert np.allclose(vh[0], np.array(g) * t, rtol=1e-12, atol=0)


def test_free_rotation_is_rigid():
    w0 = np.array([0.02, -0.03, 0.05])
    case = colloids_only([[12.0, 12.0, 12.0]], omega=[w0], translate=0, rotate=1)
    o = make_oracle(case, dyn(ab=4))
    x0 = o.download("x")["x"] - 12.0
    dt = 0.1
    nsteps = 30
    o.run_vv(0, nsteps, dt)
    st = o.colloid_state()
    assert np.allclose(st["omega"][0, 0], w0, rtol=0, atol=1e-15)
    phi = np.linalg.norm(w0) * dt
    assert st["theta"][0, 2] == pytest.approx(nsteps * phi, rel=1e-13)
    x1 = o.download("x")["x"] - 12.0
    # distances to the centre kept, the shell turned by |w| t about w
    assert np.allclose(np.linalg.norm(x1, axis=1), np.linalg.norm(x0, axis=1), atol=1e-11)
    ax = w0 / np.linalg.norm(w0)
    ang = nsteps * phi
    K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
    R = np.eye(3) + math.sin(ang) * K + (1 - math.cos(ang)) * K @ K
    assert np.allclose(x1, x0 @ R.T, atol=1e-10)
    # the accumulated orientation is the same rotation
    acc = st["acc"][0].reshape(3, 3, order="F")
    assert np.allclose(acc, R, atol=1e-12)


def test_repulsion_conserves_momentum():
    # two spheres of radius 3 with a gap of 0.5 (< 5 hn = 1.5): DLVO pushes
    # them apart along x
    case = colloids_only([[6.0, 12.0, 12.0], [12.5, 12.0, 12.0]], repul=2)
    o = make_oracle(case, dyn(ab=2))
    o.run_vv(0, 20, 0.02)
    st = o.colloid_state()
    m = case[10]
    p = (m[:, None] * st["v"][0]).sum(0)
    assert np.max(np.abs(p)) <= 1e-13 * np.max(np.abs(m[:, None] * st["v"][0]))
    assert st["v"][0, 0, 0] < 0 < st["v"][0, 1, 0]
    assert st["x"][1, 0] - st["x"][0, 0] > 6.5
