"""Moving boundaries in the CPU oracle (what the CUDA path is compared with):

  - Lees-Edwards y faces: images above the y+ face at x + shear_length
    modulo L_x (ppm_bcdef_le_y.inc), their velocity + the face velocity
    difference (particles_set_boundary_ghost_velocity.F90), particles
    crossing a face re-entering with shifted x and velocity
    (particles_adjust_particles.F90:228-257, 352-381), shear_length from
    boundary_update_boundary.F90:102-122;
  - moving and oscillating solid walls: wall particles drift with their
    velocity and take the face velocity at the end of a step
    (particles_integrate_boundary_position.F90, particles_set_boundary_
    velocity.F90, marching_integrate_VV.F90:783-806, 1650-1675).

The oracle's Lees-Edwards pair set is checked against a brute-force
restatement of the sheared-image geometry, independent of its cell list and
ghosts.
"""
import math

import numpy as np
import pytest

from mcf_gb300 import configs
from mcf_gb300.params import BC_PERIODIC
from oracle.oracle import Oracle


def le_oracle(w, time):
    o = Oracle(w.params)
    o.set_boundary_motion([0] * 6, [0.0] * 6, time)
    o.upload(w.x, w.v, w.m, w.id)
    return o


def brute_density(o, x, L, S, rc, dim):
    """sum_j W(r_ij) with the Lees-Edwards geometry: a pair more than L/2
    apart in y is a pair across the face, the lower particle's image at
    (x + S, y + L); x and z minimum image."""
    n = x.shape[0]
    rho = np.zeros(n)
    kern = np.vectorize(lambda r: o.kernel(r)[0])
    for i in range(n):
        d = x[i] - x
        up = d[:, 1] > 0.5 * L    # i above, j below: j's image above
        dn = d[:, 1] < -0.5 * L   # i below, j above: j's image below
        d[up, 1] -= L
        d[up, 0] -= S
        d[dn, 1] += L
        d[dn, 0] += S
        d[:, 0] -= L * np.round(d[:, 0] / L)
        if dim == 3:
            d[:, 2] -= L * np.round(d[:, 2] / L)
        r = np.sqrt((d * d).sum(1))
        r[i] = np.inf
        sel = r < rc
        rho[i] = kern(r[sel]).sum()
    return rho


@pytest.mark.parametrize("dim", [2, 3])
def test_le_pair_set_matches_brute_force(dim):
    n_side = 12 if dim == 3 else 16
    w = configs.lees_edwards(dim=dim, n_side=n_side, shear_rate=0.3)
    rng = np.random.default_rng(31)
    w.x = np.mod(w.x + rng.uniform(-0.4, 0.4, w.x.shape), float(n_side))
    time = 7.3
    o = le_oracle(w, time)
    o.marching_init_force(0)
    rho = o.download("rho")["rho"]
    L = float(n_side)
    S = 0.3 * L * time  # (v0(y+) - v0(y-)) * time
    w0 = o.kernel(0.0)[0]
    ref = brute_density(o, w.x, L, S, 3.0, dim) + w0
    assert np.max(np.abs(rho - ref) / ref) < 1e-12


def test_le_zero_shear_equals_periodic():
    w = configs.lees_edwards(dim=3, n_side=12, shear_rate=0.0)
    p = w.params.copy()
    p.bcdef[2] = p.bcdef[3] = BC_PERIODIC
    a = le_oracle(w, 0.0)
    b = Oracle(p)
    b.upload(w.x, w.v, w.m, w.id)
    for o in (a, b):
        o.marching_init_force(0)
        o.run_vv(0, 5, w.dt)
    ra, rb = a.download("x", "v", "rho", "f"), b.download("x", "v", "rho", "f")
    for k in ("x", "v", "rho"):
        assert np.max(np.abs(ra[k] - rb[k])) <= 1e-12 * np.max(np.abs(rb[k])), k
    assert np.max(np.abs(ra["f"] - rb["f"])) <= 1e-10 * np.max(np.abs(rb["f"]))


def test_le_internal_forces_cancel():
    w = configs.lees_edwards(dim=3, n_side=12, shear_rate=0.2)
    o = le_oracle(w, 3.1)
    o.marching_init_force(0)
    f = o.download("f")["f"]
    tot = (w.m[:, None] * f).sum(0)
    assert np.all(np.abs(tot) <= 1e-12 * (w.m[:, None] * np.abs(f)).sum(0))


def test_le_crossing_shifts_position_and_velocity():
    w = configs.lees_edwards(dim=3, n_side=12, shear_rate=0.3)
    L = 12.0
    x = w.x.copy()
    v = w.v.copy()
    x[0] = [1.0, -0.1, 5.0]
    v[0] = [0.1, 0.0, 0.0]
    x[1] = [11.5, 12.05, 3.0]
    v[1] = [0.2, 0.0, 0.0]
    w.x, w.v = x, v
    o = le_oracle(w, 2.0)   # S = 0.3 * 12 * 2 = 7.2, dv = 3.6
    o.particles_adjust_particles()
    r = o.download("x", "v")
    S, dv = 0.3 * L * 2.0, 0.3 * L
    np.testing.assert_allclose(r["x"][0], [np.mod(1.0 + S, L), -0.1 + L, 5.0], rtol=0, atol=1e-12)
    np.testing.assert_allclose(r["v"][0], [0.1 + dv, 0.0, 0.0], rtol=0, atol=1e-12)
    np.testing.assert_allclose(r["x"][1], [np.mod(11.5 - S, L), 12.05 - L, 3.0], rtol=0, atol=1e-12)
    np.testing.assert_allclose(r["v"][1], [0.2 - dv, 0.0, 0.0], rtol=0, atol=1e-12)


def test_time_advances_like_mcf():
    w = configs.lees_edwards(dim=2, n_side=16, shear_rate=0.1)
    o = le_oracle(w, 0.25)
    o.marching_init_force(0)
    o.run_vv(0, 7, w.dt)
    t = 0.25
    for _ in range(7):
        t = t + w.dt
    assert o.time == t


def test_walls_drift_and_take_the_face_velocity():
    w = configs.couette_walls(dim=2, n_side=16, v_top=0.05)
    o = Oracle(w.params)
    o.upload(w.x, w.v, w.m, w.id)
    o.marching_init_force(0)
    o.run_vv(0, 10, w.dt)
    r = o.download("x", "v")
    top = w.id[:, 1] == -4
    bot = w.id[:, 1] == -3
    L = 16.0
    moved = np.mod(r["x"][top, 0] - w.x[top, 0] + 0.5 * L, L) - 0.5 * L
    np.testing.assert_allclose(moved, 10 * 0.05 * w.dt, rtol=1e-9)
    assert np.array_equal(r["x"][bot], w.x[bot])
    assert np.all(r["v"][top, 0] == 0.05) and np.all(r["v"][top, 1] == 0.0)
    assert np.all(r["v"][bot] == 0.0)


def test_oscillating_wall_velocity_follows_mcf_time():
    w = configs.couette_walls(dim=2, n_side=16, v_top=0.05)
    freq = 2 * np.pi / 0.05
    o = Oracle(w.params)
    o.set_boundary_motion([0, 0, 0, 2, 0, 0], [0, 0, 0, freq, 0, 0], 0.0)
    o.upload(w.x, w.v, w.m, w.id)
    o.marching_init_force(0)
    t = 0.0
    for s in range(1, 8):
        o.marching_integrate_VV(s, w.dt)
        t = t + w.dt
        v = o.download("v")["v"]
        top = w.id[:, 1] == -4
        # end of step: shear_v at time_current + dt (marching_integrate_VV.F90:1657)
        assert np.all(v[top, 0] == 0.05 * math.cos(freq * (t + w.dt)))
