"""GPU parity tests: the CUDA path through the C-ABI against the CPU oracle.

Bars of the plain FP64 path:
  - cell lists bit-exact (per real cell, sorted host indices, PPM order);
  - per-step density within 1e-12 relative;
  - per-step acceleration within 1e-12 of the per-particle scale
    S_i = sum_j |a_ij| (net forces on near-lattice states are sums of large
    cancelling pair terms, so |a_i| itself is no scale);
  - with the random force on, the pair normals are FP32 Box-Muller values
    (hardware log2/sine/cosine on the GPU, within ~5e-6 of the exact values
    the CPU draws with libm): tolerance 1e-5 * S_i;
  - kT=0 trajectories over 100 steps: positions within 1e-9 of the box
    length, velocities within 1e-7 of the velocity scale.
"""
import numpy as np
import pytest

from mcf_gb300 import SDPD, configs
from mcf_gb300.params import PRECISION_FP32_MIXED, PRECISION_FP64
from oracle.oracle import Oracle
from tests.golden import make_golden

pytestmark = pytest.mark.gpu


def both(w, **over):
    p = w.params.copy()
    for k, v in over.items():
        setattr(p, k, v)
    g = SDPD(p)
    g.upload(w.x, w.v, w.m, w.id)
    o = Oracle(p)
    o.upload(w.x, w.v, w.m, w.id)
    return g, o


def jittered_2d(n_side=32, amp=0.3, seed=5):
    w = configs.c1_poiseuille_2d(n_side=n_side)
    rng = np.random.default_rng(seed)
    w.x = w.x + rng.uniform(-amp, amp, w.x.shape) / n_side
    w.v = rng.normal(0, 1e-2, w.v.shape)
    return w


def jittered_3d(n_side=12, amp=0.3, seed=6, **kw):
    w = configs.c2_fluctuating_3d(n_side=n_side, **kw)
    rng = np.random.default_rng(seed)
    w.x = w.x + rng.uniform(-amp, amp, w.x.shape)
    w.v = rng.normal(0, 1e-2, w.v.shape)
    return w


def compare_lists(g, o):
    ga = g.technique_build_list()
    oa = o.technique_build_list()
    assert np.array_equal(ga[0], oa[0])
    assert np.array_equal(ga[1], oa[1])
    assert np.array_equal(ga[2], oa[2])


# ---------------------------------------------------------------- cell list
@pytest.mark.parametrize("maker", ["c1", "jit2d", "jit3d", "walls"])
def test_cell_list_bit_exact(gpu_lib, maker):
    w = {"c1": lambda: configs.c1_poiseuille_2d(),
         "jit2d": jittered_2d,
         "jit3d": jittered_3d,
         "walls": lambda: make_golden.workload("walls_small")}[maker]()
    g, o = both(w)
    g.particles_adjust_particles()
    o.particles_adjust_particles()
    compare_lists(g, o)


def test_cell_list_boundary_positions(gpu_lib):
    # positions on cell faces, on the domain faces and one ulp inside them
    w = configs.c2_fluctuating_3d(n_side=12)
    p = w.params
    n = w.n
    rng = np.random.default_rng(3)
    cs = (p.max_phys_t[0] - p.min_phys_t[0]) / int((12.0) / (3.0 * 1.0001))
    faces = np.array([0.0, cs, 2 * cs, 12.0 - 1e-15, np.nextafter(12.0, 0), np.nextafter(cs, 0),
                      np.nextafter(cs, 13)])
    x = w.x.copy()
    x[: n // 2] = rng.choice(faces, size=(n // 2, 3))
    w.x = x
    g, o = both(w)
    g.particles_adjust_particles()
    o.particles_adjust_particles()
    compare_lists(g, o)


# ------------------------------------------------------- density and force
def check_rhs(g, o, noise=False, step=0):
    g.marching_init_force(step)
    o.marching_init_force(step)
    a = g.download("rho", "p", "f")
    b = o.download("rho", "p", "f")
    assert np.all(np.abs(a["rho"] - b["rho"]) <= 1e-12 * np.abs(b["rho"]))
    scale = o.force_scale()[:, None] + np.abs(b["f"])
    tol = 1e-5 if noise else 1e-12
    err = np.abs(a["f"] - b["f"])
    assert np.all(err <= tol * scale), float(np.max(err / scale))
    return a, b


@pytest.mark.parametrize("ftype", [1, 2, 3, 4])
@pytest.mark.parametrize("dim", [2, 3])
def test_fp64_density_force(gpu_lib, ftype, dim):
    w = jittered_2d() if dim == 2 else jittered_3d()
    over = dict(rhs_force_type=ftype, Brownian=0, kt=0.0)
    if ftype == 1:
        over["rhs_density_type"] = 1
    g, o = both(w, **over)
    check_rhs(g, o)


@pytest.mark.parametrize("ktype,eos", [(2, 1), (1, 2)])
def test_fp64_kernel_and_eos_variants(gpu_lib, ktype, eos):
    w = jittered_3d()
    g, o = both(w, kernel_type=ktype, stateEquation_type=eos, gamma=7.0 if eos == 2 else 1.0,
                rho_ref=1.0, Brownian=0, kt=0.0)
    check_rhs(g, o)


@pytest.mark.parametrize("ftype", [2, 3, 4])
def test_fp64_random_force(gpu_lib, ftype):
    w = jittered_3d()
    g, o = both(w, rhs_force_type=ftype, Brownian=1, kt=1e-3)
    a, b = check_rhs(g, o, noise=True, step=17)
    # the random term is on: the force differs from the deterministic one
    g2, o2 = both(w, rhs_force_type=ftype, Brownian=0, kt=0.0)
    g2.marching_init_force(17)
    c = g2.download("f")["f"]
    assert np.max(np.abs(a["f"] - c)) > 1e-6


def test_fp64_walls(gpu_lib):
    w = make_golden.workload("walls_small")
    g, o = both(w, Brownian=0, kt=0.0)
    check_rhs(g, o)


def test_fp64_golden_fixtures(gpu_lib):
    for name, fx in make_golden.load_all().items():
        w = make_golden.workload(name)
        g = SDPD(w.params)
        if make_golden.motion(name):
            g.set_boundary_motion(*make_golden.motion(name))
        g.upload(w.x, w.v, w.m, w.id)
        g.marching_init_force(0)
        d = g.download("rho", "f")
        assert np.all(np.abs(d["rho"] - fx["rho0"]) <= 1e-12 * np.abs(fx["rho0"]))
        noise = bool(w.params.Brownian and w.params.kt > 0)
        tol = 1e-5 if noise else 1e-9
        assert np.all(np.abs(d["f"] - fx["f0"]) <= tol * (np.abs(fx["f0"]).max() + 1.0))
        # the dumped steps (1, 5, 10, 100 for C1 and C2; 5 for the others).
        # With the random force the GPU's FP32 normals differ from the
        # CPU's in the last bits: measured 5e-7 of the velocity scale and
        # 8e-12 of the box after 100 C2 steps, against 7e-15 and 1e-16
        # without it (C1)
        L = np.asarray(w.params.max_phys_t)[: w.params.num_dim] - \
            np.asarray(w.params.min_phys_t)[: w.params.num_dim]
        bx, bv, br, bf = (1e-9, 1e-5, 1e-9, 1e-5) if noise else (1e-10, 1e-8, 1e-12, 1e-10)
        done = 0
        for t in make_golden.STEPS.get(name, (5,)):
            g.run_vv(done, t - done, w.dt)
            done = t
            dt_ = g.download("x", "v", "rho", "f")
            dx = np.abs(dt_["x"] - fx[f"x{t}"])
            dx = np.minimum(dx, L - dx)
            assert dx.max() <= bx * L.max(), (name, t)
            assert np.abs(dt_["v"] - fx[f"v{t}"]).max() <= \
                bv * (np.abs(fx[f"v{t}"]).max() + 1e-3), (name, t)
            assert np.max(np.abs(dt_["rho"] - fx[f"rho{t}"]) / fx[f"rho{t}"]) <= br, (name, t)
            assert np.abs(dt_["f"] - fx[f"f{t}"]).max() <= \
                bf * (np.abs(fx[f"f{t}"]).max() + 1.0), (name, t)


def test_stress_tensor_and_statistics(gpu_lib):
    w = jittered_3d()
    g, o = both(w, stress_tensor=1, Brownian=0, kt=0.0)
    g.marching_init_force(0)
    o.marching_init_force(0)
    a = g.download("s")["s"]
    b = o.download("s")["s"]
    assert np.max(np.abs(a - b)) <= 1e-10 * (np.abs(b).max() + 1e-30)
    ke_g, mom_g, st_g = g.statistic_compute_statistic()
    ke_o, mom_o, st_o = o.statistic_compute_statistic()
    assert abs(ke_g - ke_o) <= 1e-12 * ke_o
    assert np.allclose(mom_g, mom_o, rtol=1e-12, atol=1e-15)
    assert np.allclose(st_g, st_o, rtol=1e-10, atol=1e-12 * np.abs(st_o).max())


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_FP32_MIXED])
@pytest.mark.parametrize("maker", ["jit3d", "walls", "jit2d"])
def test_symmetric_sweep_matches_gather_sweep(gpu_lib, precision, maker):
    # the stress tensor selects the two-sided gather sweep, without it the
    # FP64 path runs the symmetric (each pair once) sweep: same accelerations
    w = {"jit3d": jittered_3d, "walls": lambda: make_golden.workload("walls_small"),
         "jit2d": jittered_2d}[maker]()
    res = []
    for stress in (0, 1):
        p = w.params.copy()
        p.precision = precision
        p.stress_tensor = stress
        p.Brownian = 1
        p.kt = 1e-3
        g = SDPD(p)
        g.upload(w.x, w.v, w.m, w.id)
        g.marching_init_force(3)
        res.append(g.download("f")["f"])
    scale = np.abs(res[1]).max()
    tol = 1e-13 if precision == PRECISION_FP64 else 2e-5
    assert np.max(np.abs(res[0] - res[1])) <= tol * scale


# ------------------------------------------------------------- trajectories
def test_fp64_trajectory_100_steps_kt0(gpu_lib):
    w = configs.c1_poiseuille_2d()
    g, o = both(w)
    g.marching_init_force(0)
    o.marching_init_force(0)
    for s in range(1, 101):
        g.marching_integrate_VV(s, w.dt)
        o.marching_integrate_VV(s, w.dt)
    a = g.download("x", "v", "rho")
    b = o.download("x", "v", "rho")
    dx = np.abs(a["x"] - b["x"])
    dx = np.minimum(dx, 1.0 - dx)  # periodic images
    assert dx.max() <= 1e-9
    vs = np.abs(b["v"]).max()
    assert np.abs(a["v"] - b["v"]).max() <= 1e-7 * vs
    assert np.all(np.abs(a["rho"] - b["rho"]) <= 1e-10 * b["rho"])


def test_run_vv_equals_step_vv_and_is_deterministic(gpu_lib):
    w = jittered_3d()
    outs = []
    for mode in ("step", "run", "run"):
        g = SDPD(w.params)
        g.upload(w.x, w.v, w.m, w.id)
        g.marching_init_force(0)
        if mode == "step":
            for s in range(1, 6):
                g.marching_integrate_VV(s, w.dt)
        else:
            g.run_vv(0, 5, w.dt)
        outs.append(g.download("x", "v", "f"))
    for k in ("x", "v", "f"):
        assert np.array_equal(outs[0][k], outs[1][k])
        assert np.array_equal(outs[1][k], outs[2][k])


# --------------------------------------------------------- FP32-mixed path
def test_fp32_mixed_error_vs_fp64(gpu_lib):
    w = jittered_3d(amp=0.05)
    g32, o = both(w, precision=PRECISION_FP32_MIXED, Brownian=0, kt=0.0)
    g32.marching_init_force(0)
    o.marching_init_force(0)
    a = g32.download("rho", "f")
    b = o.download("rho", "f")
    rel_rho = np.abs(a["rho"] - b["rho"]) / b["rho"]
    assert rel_rho.max() < 2e-6
    scale = o.force_scale()[:, None]
    assert np.max(np.abs(a["f"] - b["f"]) / scale) < 1e-4


@pytest.mark.parametrize("ftype,ktype,eos", [(1, 1, 1), (2, 1, 1), (4, 1, 1), (3, 2, 1),
                                             (3, 1, 2), (4, 2, 2)])
@pytest.mark.parametrize("dim", [2, 3])
def test_fp32_mixed_force_forms_kernels_eos(gpu_lib, ftype, ktype, eos, dim):
    # every pair form, the Lucy kernel and the Batchelor equation of state
    # in the FP32-mixed path: density within 2e-6, acceleration within 1e-4
    # of the per-particle scale
    w = jittered_2d(amp=0.05) if dim == 2 else jittered_3d(amp=0.05)
    over = dict(precision=PRECISION_FP32_MIXED, rhs_force_type=ftype, kernel_type=ktype,
                stateEquation_type=eos, gamma=7.0 if eos == 2 else 1.0, rho_ref=1.0,
                Brownian=0, kt=0.0)
    if ftype == 1:
        over["rhs_density_type"] = 1
    g, o = both(w, **over)
    g.marching_init_force(0)
    o.marching_init_force(0)
    a = g.download("rho", "f")
    b = o.download("rho", "f")
    assert np.max(np.abs(a["rho"] - b["rho"]) / b["rho"]) < 2e-6
    scale = o.force_scale()[:, None]
    assert np.max(np.abs(a["f"] - b["f"]) / scale) < 1e-4


@pytest.mark.parametrize("ftype", [2, 3, 4])
def test_fp32_mixed_random_force(gpu_lib, ftype):
    # the same Philox draws in the FP32-mixed path: within 1e-4 of the scale
    w = jittered_3d(amp=0.05)
    g, o = both(w, precision=PRECISION_FP32_MIXED, rhs_force_type=ftype, Brownian=1, kt=1e-3)
    g.marching_init_force(23)
    o.marching_init_force(23)
    a = g.download("f")["f"]
    b = o.download("f")["f"]
    assert np.max(np.abs(a - b) / o.force_scale()[:, None]) < 1e-4


# ----------------------------------------------------------- error handling
def test_neighbour_overflow_is_reported(gpu_lib):
    from mcf_gb300 import MCFGError
    from mcf_gb300.params import MCFG_EOVERFLOW

    w = jittered_3d()
    p = w.params.copy()
    p.reserved[0] = 8  # far below the ~92 neighbours per particle
    g = SDPD(p)
    g.upload(w.x, w.v, w.m, w.id)
    with pytest.raises(MCFGError) as ei:
        g.marching_init_force(0)
    assert ei.value.code == MCFG_EOVERFLOW
    # the handle stays usable
    g.upload(w.x, w.v, w.m, w.id)
    g.technique_build_list()


# ------------------------------------------------------------ Oldroyd-B model
def oldroyd_case(n_side=24, seed=8):
    w = configs.c5_oldroyd_b_2d(n_side=n_side)
    rng = np.random.default_rng(seed)
    w.x = w.x + rng.uniform(-0.2, 0.2, w.x.shape)
    w.v = rng.normal(0, 1e-2, w.v.shape)
    return w


@pytest.mark.parametrize("noise", [0, 1])
def test_oldroyd_b_fp64_steps(gpu_lib, noise):
    w = oldroyd_case()
    g, o = both(w, Brownian=noise, kt=1e-4 if noise else 0.0)
    g.marching_init_force(0)
    o.marching_init_force(0)
    a = g.download("f")["f"]
    b = o.download("f")["f"]
    scale = o.force_scale()[:, None] + np.abs(b)
    assert np.all(np.abs(a - b) <= (1e-5 if noise else 1e-12) * scale)
    for s in range(1, 6):
        g.marching_integrate_VV(s, w.dt)
        o.marching_integrate_VV(s, w.dt)
    a = g.download("x", "v", "ct")
    b = o.download("x", "v", "ct")
    tol_x, tol_v, tol_c = (1e-9, 1e-6, 1e-9) if noise else (1e-12, 1e-10, 1e-12)
    assert np.max(np.abs(a["x"] - b["x"])) <= tol_x * 24
    assert np.max(np.abs(a["v"] - b["v"])) <= tol_v * (np.abs(b["v"]).max() + 1e-30)
    assert np.max(np.abs(a["ct"] - b["ct"])) <= tol_c


def test_oldroyd_b_fp32_mixed_ct_error(gpu_lib):
    w = oldroyd_case()
    g, o = both(w, precision=PRECISION_FP32_MIXED, Brownian=0, kt=0.0)
    g.marching_init_force(0)
    o.marching_init_force(0)
    g.run_vv(0, 5, w.dt)
    o.run_vv(0, 5, w.dt)
    a = g.download("ct")["ct"]
    b = o.download("ct")["ct"]
    dev = np.abs(b - np.array([1.0, 0, 0, 1.0]))
    assert np.max(np.abs(a - b)) <= 1e-3 * dev.max() + 1e-9


# ------------------------------------------------------------------ colloids
def colloid_case(precision=PRECISION_FP64, noslip=2):
    w, cs = configs.c4_colloids(n_side=24, n_colloid=4, radius=3.0, precision=precision,
                                v_scale=0.05, omega_scale=0.02)
    rng = np.random.default_rng(13)
    fl = w.id[:, 1] == 0
    w.v[fl] = rng.normal(0, 1e-2, (int(fl.sum()), 3))
    w.x[fl] += rng.uniform(-0.1, 0.1, (int(fl.sum()), 3))
    cs.params.noslip_type = noslip
    return w, cs


@pytest.mark.parametrize("noslip", [1, 2])
def test_colloid_pair_terms_fp64(gpu_lib, noslip):
    w, cs = colloid_case(noslip=noslip)
    assert (w.id[:, 1] > 0).sum() > 100
    g, o = both(w, Brownian=0, kt=0.0)
    for h in (g, o):
        h.set_colloids(cs.params, cs.x, cs.v, cs.omega, cs.radius)
    a, b = check_rhs(g, o)
    va = g.download("v")["v"]
    vb = o.download("v")["v"]
    bp = w.id[:, 1] > 0
    assert np.allclose(va[bp], vb[bp], rtol=0, atol=1e-14)  # rigid boundary velocities
    da, ta = g.colloid_drag()
    db, tb = o.colloid_drag()
    scale = np.abs(db).max() + np.abs(tb).max()
    assert np.max(np.abs(da - db)) <= 1e-10 * scale
    assert np.max(np.abs(ta - tb)) <= 1e-10 * scale
    assert np.allclose(g.colloid_repulsion(), o.colloid_repulsion(), rtol=1e-12, atol=1e-14)


def test_colloid_steps_fp64_and_fp32(gpu_lib):
    w, cs = colloid_case()
    g, o = both(w, Brownian=0, kt=0.0)
    p32 = w.params.copy()
    p32.precision = PRECISION_FP32_MIXED
    p32.Brownian = 0
    p32.kt = 0.0
    g32 = SDPD(p32)
    g32.upload(w.x, w.v, w.m, w.id)
    for h in (g, o, g32):
        h.set_colloids(cs.params, cs.x, cs.v, cs.omega, cs.radius)
        h.marching_init_force(0)
        h.run_vv(0, 5, w.dt)
    a, b, c32 = (h.download("x", "v") for h in (g, o, g32))
    assert np.max(np.abs(a["x"] - b["x"])) <= 1e-11
    vs = np.abs(b["v"]).max()
    assert np.max(np.abs(a["v"] - b["v"])) <= 1e-9 * vs
    assert np.max(np.abs(c32["v"] - b["v"])) <= 2e-4 * vs


# ------------------------------------------------------- neighbour-list reuse
def _reuse_pair(w, nsteps, dt, **over):
    """the same run with and without list reuse: (standard, reuse) handles"""
    out = []
    for reuse in (0, 1):
        p = w.params.copy()
        p.reserved[1] = reuse
        for k, v in over.items():
            setattr(p, k, v)
        h = SDPD(p)
        h.upload(w.x, w.v, w.m, w.id)
        h.marching_init_force(0)
        h.run_vv(0, nsteps, dt)
        out.append(h)
    return out


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_FP32_MIXED])
def test_list_reuse_matches_rebuild_every_step(gpu_lib, precision):
    # 16^3 jittered: cells of 3.2 for rc = 3, skin 0.198
    w = jittered_3d(n_side=16, precision=precision)
    a, b = _reuse_pair(w, 50, w.dt, Brownian=0, kt=0.0)
    info = b.info()
    assert info["skin"] > 0.19 and info["list_rebuilds"] >= 1
    da, db = a.download("x", "v"), b.download("x", "v")
    L = 16.0
    assert np.all((db["x"] >= 0.0) & (db["x"] < L))  # downloaded wrapped
    dx = da["x"] - db["x"]
    dx -= L * np.round(dx / L)
    tol = 1e-10 if precision == PRECISION_FP64 else 1e-5
    assert np.max(np.abs(dx)) <= tol
    assert np.max(np.abs(da["v"] - db["v"])) <= tol * np.max(np.abs(da["v"]))


def test_list_reuse_rebuilds_on_displacement(gpu_lib):
    # fast particles (|v| ~ 0.3, dt = 1e-2: ~3e-3 per step against half a
    # skin of 0.1): the device rebuilds many times; the trajectory is the
    # one without reuse and the oracle's
    w = jittered_3d(n_side=16)
    rng = np.random.default_rng(9)
    w.v = rng.normal(0, 0.3, w.v.shape)
    a, b = _reuse_pair(w, 100, 1e-2, Brownian=0, kt=0.0)
    assert b.info()["list_rebuilds"] >= 5
    da, db = a.download("x", "v", "rho", "f"), b.download("x", "v", "rho", "f")
    L = 16.0
    dx = da["x"] - db["x"]
    dx -= L * np.round(dx / L)
    assert np.max(np.abs(dx)) <= 1e-9
    assert np.max(np.abs(da["v"] - db["v"])) <= 1e-8 * np.max(np.abs(da["v"]))
    assert np.max(np.abs(da["rho"] - db["rho"]) / da["rho"]) <= 1e-10


def test_list_reuse_walls_oldroyd_and_noise(gpu_lib):
    # walls: per-step pair terms with Morris no-slip; Oldroyd-B: ct travels
    # with the rebuild permutation; noise: same keys, same draws
    w = make_golden.workload("walls_small")
    a, b = _reuse_pair(w, 30, w.dt)
    da, db = a.download("x", "v", "f"), b.download("x", "v", "f")
    assert np.max(np.abs(da["x"] - db["x"])) <= 1e-10
    assert np.max(np.abs(da["v"] - db["v"])) <= 1e-8 * np.max(np.abs(da["v"]))
    w = oldroyd_case()
    a, b = _reuse_pair(w, 20, w.dt)
    da, db = a.download("x", "v", "ct"), b.download("x", "v", "ct")
    L = w.params.max_phys[0] - w.params.min_phys[0]
    dx = da["x"] - db["x"]
    dx -= L * np.round(dx / L)
    assert np.max(np.abs(dx)) <= 1e-10
    assert np.max(np.abs(da["ct"] - db["ct"])) <= 1e-10


def test_update_state_keeps_order_and_reuse(gpu_lib):
    # MCF's per-step drop-in: download, (modify), hand the arrays back
    w = jittered_3d(n_side=16)
    p = w.params.copy()
    p.reserved[1] = 1
    p.Brownian = 0
    p.kt = 0.0
    ref = SDPD(p)
    ref.upload(w.x, w.v, w.m, w.id)
    ref.marching_init_force(0)
    ref.run_vv(0, 30, w.dt)
    h = SDPD(p)
    h.upload(w.x, w.v, w.m, w.id)
    h.marching_init_force(0)
    for s in range(30):
        st = h.download("x", "v", "f")
        h.update_state(st["x"], st["v"], st["f"])
        h.marching_integrate_VV(s + 1, w.dt)
    assert h.info()["list_rebuilds"] == ref.info()["list_rebuilds"] == 1
    a, b = ref.download("x", "v"), h.download("x", "v")
    assert np.max(np.abs(a["x"] - b["x"])) <= 1e-12 * 16
    assert np.max(np.abs(a["v"] - b["v"])) <= 1e-10 * np.max(np.abs(a["v"]))
    # a changed state: the same as uploading it afresh
    st = h.download("x", "v", "f")
    st["v"] *= 0.5
    h.update_state(st["x"], st["v"], st["f"])
    g = SDPD(p)
    g.upload(st["x"], st["v"], w.m, w.id)
    g.upload_force(st["f"])
    h.run_vv(30, 10, w.dt)
    g.run_vv(30, 10, w.dt)
    a, b = g.download("x", "v"), h.download("x", "v")
    assert np.max(np.abs(a["x"] - b["x"])) <= 1e-10
    assert np.max(np.abs(a["v"] - b["v"])) <= 1e-8 * np.max(np.abs(a["v"]))


def _rotation(axis, angle):
    a = np.asarray(axis, float) / np.linalg.norm(axis)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K


def test_colloid_move_then_steps(gpu_lib):
    # MCF's Colloid object integrates the rigid bodies on the host; the
    # boundary particles follow on the device (relative position, rotation,
    # new centre), then the steps continue with the moved colloids
    w, cs = colloid_case()
    g, o = both(w, Brownian=0, kt=0.0)
    for h in (g, o):
        h.set_colloids(cs.params, cs.x, cs.v, cs.omega, cs.radius)
        h.marching_init_force(0)
        h.run_vv(0, 3, w.dt)
    rng = np.random.default_rng(31)
    nc = cs.x.shape[0]
    x_new = cs.x + rng.uniform(-0.05, 0.05, cs.x.shape)
    rot = np.stack([_rotation(rng.normal(size=3), 0.02) for _ in range(nc)])
    rot_f = np.ascontiguousarray(rot.transpose(0, 2, 1)).reshape(nc, 9)  # R(i,j) at i + 3j
    v_new = cs.v * 1.5
    om_new = cs.omega * 0.5
    for h in (g, o):
        h.move_colloids(x_new, rot_f, v_new, om_new)
    a, b = g.download("x"), o.download("x")
    L = 24.0
    dx = a["x"] - b["x"]
    dx -= L * np.round(dx / L)
    assert np.max(np.abs(dx)) <= 1e-12
    for h in (g, o):
        h.run_vv(3, 5, w.dt)
    a, b = g.download("x", "v"), o.download("x", "v")
    dx = a["x"] - b["x"]
    dx -= L * np.round(dx / L)
    assert np.max(np.abs(dx)) <= 1e-11
    assert np.max(np.abs(a["v"] - b["v"])) <= 1e-9 * np.abs(b["v"]).max()
    da, ta = g.colloid_drag()
    db, tb = o.colloid_drag()
    scale = np.abs(db).max() + np.abs(tb).max()
    assert np.max(np.abs(da - db)) <= 1e-9 * scale and np.max(np.abs(ta - tb)) <= 1e-9 * scale


def test_step_vv_host_equals_update_step_download(gpu_lib):
    # the fused host-array step (inputs over, step, positions back on a
    # second stream, velocities back) against the three calls it replaces,
    # with and without list reuse, over steps that rebuild the list
    for reuse in (0, 1):
        w = jittered_3d(n_side=14)
        w.params.reserved[1] = reuse
        outs = []
        for mode in ("fused", "calls"):
            g = SDPD(w.params)
            g.upload(w.x, w.v, w.m, w.id)
            g.marching_init_force(0)
            st = g.download("x", "v")
            x = np.ascontiguousarray(st["x"])
            v = np.ascontiguousarray(st["v"])
            for s in range(1, 8):
                if mode == "fused":
                    g.step_vv_host(s, w.dt, x, v)
                else:
                    g.update_state(x=x, v=v)
                    g.marching_integrate_VV(s, w.dt)
                    r = g.download("x", "v")
                    x, v = np.ascontiguousarray(r["x"]), np.ascontiguousarray(r["v"])
                v = v * 1.0  # the host owns its arrays between steps
            outs.append((x.copy(), v.copy()))
        assert np.array_equal(outs[0][0], outs[1][0])
        assert np.array_equal(outs[0][1], outs[1][1])


def test_host_registered_arrays_step_alike(gpu_lib):
    # MCF's ordinary host arrays page-locked with mcfg_host_register: with
    # list reuse the host step then replays a captured graph (inputs over,
    # the step, positions and velocities back); plain arrays take per-step
    # launches.  The same steps bit for bit, FP64 and FP32-mixed, across
    # device-side rebuilds; unregistering leaves the arrays usable
    # particles past skin/2 (0.495 in the 12^3 box) within a few steps
    fast = jittered_3d(n_side=12)
    fast.v = np.random.default_rng(9).normal(0, 2.0, fast.v.shape)
    cases = [(jittered_3d(n_side=14), None, 0), (make_golden.workload("walls_small"), None, 1),
             (fast, 1e-2, 1)]
    for w, dt, prec in cases:
        dt = dt or w.dt
        outs = []
        for reg in (False, True):
            p = w.params.copy()
            p.reserved[1] = 1
            p.precision = PRECISION_FP32_MIXED if prec else 0
            g = SDPD(p)
            g.upload(w.x, w.v, w.m, w.id)
            g.marching_init_force(0)
            st = g.download("x", "v")
            x = np.ascontiguousarray(st["x"])
            v = np.ascontiguousarray(st["v"])
            if reg:
                g.host_register(x)
                g.host_register(v)
            for s in range(1, 16):
                g.step_vv_host(s, dt, x, v)
            if reg:
                g.host_unregister(x)
                g.host_unregister(v)
            outs.append((x.copy(), v.copy(), g.download("f")["f"], g.info()))
        for q in range(3):
            assert np.array_equal(outs[0][q], outs[1][q]), q
        assert outs[0][3]["list_rebuilds"] == outs[1][3]["list_rebuilds"]
        assert outs[0][3]["time_current"] == outs[1][3]["time_current"]
        if w is fast:
            assert outs[1][3]["list_rebuilds"] > 1  # rebuilds inside the replays
    with pytest.raises(Exception):
        g.host_unregister(x)  # no longer registered
    g.step_vv_host(16, dt, x, v)  # the failed call leaves the handle usable


def test_host_step_graph_follows_a_new_particle_set(gpu_lib):
    # the captured host step bakes buffers and host arrays: a new upload
    # (another n, other registered arrays) must recapture, and the handle
    # then steps exactly as a fresh one does
    def registered_run(g, w, steps):
        st = g.download("x", "v")
        x, v = np.ascontiguousarray(st["x"]), np.ascontiguousarray(st["v"])
        g.host_register(x)
        g.host_register(v)
        try:
            for s in range(1, steps + 1):
                g.step_vv_host(s, w.dt, x, v)
        finally:
            g.host_unregister(x)
            g.host_unregister(v)
        return x, v

    w1, w2 = jittered_3d(n_side=12), jittered_3d(n_side=14)
    p = w1.params.copy()
    p.reserved[1] = 1
    p.precision = PRECISION_FP32_MIXED
    p2 = w2.params.copy()
    p2.reserved[1] = 1
    p2.precision = PRECISION_FP32_MIXED
    g = SDPD(p2)  # sized for the larger set, used for both
    g.upload(w1.x, w1.v, w1.m, w1.id)
    g.marching_init_force(0)
    registered_run(g, w1, 6)
    g.upload(w2.x, w2.v, w2.m, w2.id)
    g.marching_init_force(0)
    xa, va = registered_run(g, w2, 6)
    fresh = SDPD(p2)
    fresh.upload(w2.x, w2.v, w2.m, w2.id)
    fresh.marching_init_force(0)
    xb, vb = registered_run(fresh, w2, 6)
    assert xa.shape == xb.shape == (w2.n, 3)
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_run_vv_graph_replay_equals_step_vv(gpu_lib):
    # with list reuse mcfg_run_vv replays a captured pair of steps (the
    # Philox step from the device counter), mcfg_step_vv launches every
    # step: bit-identical, also across device-side rebuilds and odd counts
    fast = jittered_3d(n_side=12)
    fast.v = np.random.default_rng(9).normal(0, 0.3, fast.v.shape)
    cases = [(jittered_3d(n_side=12), 1e-4), (make_golden.workload("walls_small"), None),
             (fast, 1e-2)]
    for w, dt in cases:
        dt = dt or w.dt
        outs = []
        for mode in ("run", "step"):
            p = w.params.copy()
            p.reserved[1] = 1
            p.precision = PRECISION_FP32_MIXED
            p.Brownian, p.kt = 1, 1e-4
            g = SDPD(p)
            g.upload(w.x, w.v, w.m, w.id)
            g.marching_init_force(0)
            if mode == "run":
                g.run_vv(0, 9, dt)
                g.run_vv(9, 6, dt)
            else:
                for s in range(1, 16):
                    g.marching_integrate_VV(s, dt)
            outs.append((g.download("x", "v", "f"), g.info()))
        for k in ("x", "v", "f"):
            assert np.array_equal(outs[0][0][k], outs[1][0][k]), k
        assert outs[0][1]["list_rebuilds"] == outs[1][1]["list_rebuilds"]
        assert outs[0][1]["time_current"] == outs[1][1]["time_current"]
