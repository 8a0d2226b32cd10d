"""Synthetic SDPD workloads (MCF input decks restated as parameter blocks
and seeded initial particles).

Particles are placed like particles_init_global_inter_cubic/_square
(lattice at min + dx/2 + k*dx over the total domain, repeated addition),
solid-wall particles are the lattice sites outside the fluid domain along a
wall axis (boundary_check_wall_solid_particle.F90: sid = 1-2i below, -2i
above), masses are rho0 * prod(dx) (particles_compute_mass.F90:363-450) and
pids run 1..N.  Perturbations MCF itself does not generate (jitter, initial
velocity noise) are seeded numpy draws, fed the way MCF's read_external
input would feed them.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .params import (BC_LE, BC_PERIODIC, BC_WALL_SOLID, PRECISION_FP64, ColloidParams,
                     SDPDParams, make_params)

BASE_SEED = 20261203


@dataclass
class Workload:
    name: str
    params: SDPDParams
    x: np.ndarray
    v: np.ndarray
    m: np.ndarray
    id: np.ndarray
    dt: float
    steps: int

    @property
    def n(self) -> int:
        return int(self.m.shape[0])

    @property
    def n_fluid(self) -> int:
        return int((self.id[:, 1] == 0).sum())


def lattice(dim: int, min_t, max_t, dx) -> np.ndarray:
    """particles_init_global_inter_cubic/_square: sx = min + dx/2, sx += dx
    while sx < max (x fastest), exactly as the repeated addition rounds."""
    axes = []
    for a in range(dim):
        vals = []
        s = min_t[a] + 0.5 * dx[a]
        while s < max_t[a]:
            vals.append(s)
            s = s + dx[a]
        axes.append(np.array(vals))
    if dim == 2:
        yy, xx = np.meshgrid(axes[1], axes[0], indexing="ij")
        return np.stack([xx.ravel(), yy.ravel()], axis=1)
    zz, yy, xx = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    return np.stack([xx.ravel(), yy.ravel(), zz.ravel()], axis=1)


def wall_sid(x: np.ndarray, params: SDPDParams) -> np.ndarray:
    dim = params.num_dim
    sid = np.zeros(x.shape[0], np.int32)
    for i in range(dim):
        if params.bcdef[2 * i] == BC_WALL_SOLID:
            lo = (x[:, i] <= params.min_phys[i]) & (x[:, i] >= params.min_phys_t[i]) & (sid == 0)
            sid[lo] = 1 - 2 * (i + 1)
        if params.bcdef[2 * i + 1] == BC_WALL_SOLID:
            hi = (x[:, i] >= params.max_phys[i]) & (x[:, i] < params.max_phys_t[i]) & (sid == 0)
            sid[hi] = -2 * (i + 1)
    return sid


def _finish(name, p, dx, jitter, vstd, seed, dt, steps, rho0=1.0) -> Workload:
    dim = p.num_dim
    x = lattice(dim, list(p.min_phys_t)[:dim], list(p.max_phys_t)[:dim], dx)
    sid = wall_sid(x, p)
    rng = np.random.default_rng(seed)
    if jitter:
        fl = sid == 0
        x[fl] += rng.uniform(-jitter, jitter, size=(int(fl.sum()), dim)) * np.asarray(dx)
    n = x.shape[0]
    v = np.zeros((n, dim))
    if vstd:
        fl = sid == 0
        v[fl] = rng.normal(0.0, vstd, size=(int(fl.sum()), dim))
    m = np.full(n, rho0 * float(np.prod(dx)))
    ids = np.stack([np.arange(1, n + 1, dtype=np.int32), sid], axis=1).astype(np.int32)
    return Workload(name, p, x, v, m, ids, dt, steps)


def _box(dim, lo, hi, walls_axis=None, nwall_layers=0, dx=1.0):
    mn = [0.0] * 3
    mx = [0.0] * 3
    mn_t = [0.0] * 3
    mx_t = [0.0] * 3
    bc = [BC_PERIODIC] * 6
    for a in range(dim):
        mn[a], mx[a] = lo, hi
        mn_t[a], mx_t[a] = lo, hi
    if walls_axis is not None:
        a = walls_axis
        bc[2 * a] = bc[2 * a + 1] = BC_WALL_SOLID
        # physics_adjust_parameters.F90:229-273
        mn_t[a] = lo - nwall_layers * dx
        mx_t[a] = hi + nwall_layers * dx
    return dict(num_dim=dim, bcdef=bc, min_phys=mn, max_phys=mx, min_phys_t=mn_t, max_phys_t=mx_t)


def wall_layers(cut_off: float, dx: float, dynamic: bool = False) -> int:
    """CEILING((1 + 0.05) * cut_off [* 2 if dynamic] / dx),
    physics_adjust_parameters.F90:229-273 with mcf_wall_in_layer_coeff."""
    w = (1.0 + 0.05) * cut_off
    if dynamic:
        w *= 2.0
    return int(np.ceil(w / dx - 1e-12))


def c1_poiseuille_2d(n_side: int = 64, precision: int = PRECISION_FP64, seed: int = BASE_SEED + 1,
                     body_force_type: int = 2) -> Workload:
    """2D 64x64 periodic unit box, dx=1/64, rc=3dx, c=10, eta=1, g_x=1,
    kT=0, v0 ~ N(0, (1e-4)^2), dt=1e-4, 1000 steps.  Fully periodic with a
    constant g is uniform acceleration, so the profile uses MCF's periodic
    reverse-Poiseuille body force (body_force_type 2)."""
    dx = 1.0 / n_side
    p = make_params(**_box(2, 0.0, 1.0), cut_off=3 * dx, c=10.0, eta=1.0, kt=0.0, Brownian=0,
                    body_force_type=body_force_type, body_force=[1.0, 0.0, 0.0], dt=1e-4,
                    precision=precision, seed=seed)
    return _finish("C1 2D 64^2 Poiseuille FP64", p, [dx, dx], 0.0, 1e-4, seed, 1e-4, 1000)


def c2_fluctuating_3d(n_side: int = 64, precision: int = PRECISION_FP64,
                      seed: int = BASE_SEED + 2) -> Workload:
    """3D 64^3 periodic cube, dx=1, jitter U(-0.05,0.05)dx, rc=3, c=10,
    eta=1, kT=1e-3 (Brownian), no body force, dt=1e-4, 2000 steps."""
    L = float(n_side)
    p = make_params(**_box(3, 0.0, L), cut_off=3.0, c=10.0, eta=1.0, kt=1e-3, Brownian=1,
                    body_force_type=0, dt=1e-4, precision=precision, seed=seed)
    return _finish(f"C2 3D {n_side}^3 fluctuating", p, [1.0] * 3, 0.05, 0.0, seed, 1e-4, 2000)


def c3_poiseuille_3d(n_side: int = 100, precision: int = PRECISION_FP64, walls: bool = True,
                     seed: int = BASE_SEED + 3, n_yz: int | None = None) -> Workload:
    """3D 100^3, dx=1, rc=3, c=20, eta=0.5, g_x=0.1, kT=1e-4, dt=5e-5,
    5000 steps.  Poiseuille in y with solid walls in y (4 layers of
    constant-density wall particles per side, Morris no-slip) or, with
    walls=False, MCF's periodic reverse-Poiseuille force.  n_yz: a box of
    n_side sites along x and n_yz along y and z (a slice of the workload)."""
    L = float(n_side)
    if walls:
        nl = wall_layers(3.0, 1.0)
        box = _box(3, 0.0, L, walls_axis=1, nwall_layers=nl, dx=1.0)
        p = make_params(**box, cut_off=3.0, c=20.0, eta=0.5, kt=1e-4, Brownian=1,
                        body_force_type=1, body_force=[0.1, 0.0, 0.0], dt=5e-5,
                        wall_noslip_type=2, wall_rho_type=0, init_density=1.0,
                        precision=precision, seed=seed)
    else:
        p = make_params(**_box(3, 0.0, L), cut_off=3.0, c=20.0, eta=0.5, kt=1e-4, Brownian=1,
                        body_force_type=2, body_force=[0.1, 0.0, 0.0], dt=5e-5,
                        precision=precision, seed=seed)
    name = f"C3 3D {n_side}^3 Poiseuille"
    if n_yz is not None and n_yz != n_side:
        for a in (1, 2):
            off = p.min_phys[a] - p.min_phys_t[a]
            p.max_phys[a] = float(n_yz)
            p.max_phys_t[a] = float(n_yz) + off
        name = f"C3 3D {n_side}x{n_yz}x{n_yz} Poiseuille"
    return _finish(name, p, [1.0] * 3, 0.0, 0.0, seed, 5e-5, 5000)


def c5_oldroyd_b_2d(n_side: int = 128, precision: int = PRECISION_FP64, seed: int = BASE_SEED + 5,
                    amplitude: float = 0.01) -> Workload:
    """2D 128x128 periodic Oldroyd-B shear: dx = 1 (L = 128; with L = 1 the
    explicit scheme at dt = 1e-3 is 65x past MCF's viscous limit), solvent
    eta_s = 0.5, G = n_p kt_p = 0.5 and tau = 1 (eta_p = G tau = 0.5), c = 10,
    kT = 1e-4 with the Philox increments, body force g_x sin(2 pi y / L_y)
    (body_force_type 3; amplitude 0.01 keeps the Mach number small on the
    L = 128 box), dt = 1e-3, 200 steps; conformation tensor starts at I."""
    L = float(n_side)
    p = make_params(**_box(2, 0.0, L), cut_off=3.0, c=10.0, eta=0.5, kt=1e-4, Brownian=1,
                    Newtonian=0, tau=1.0, n_p=1.0, kt_p=0.5, body_force_type=3,
                    body_force=[amplitude, 0.0, 0.0], dt=1e-3, precision=precision, seed=seed)
    return _finish(f"C5 2D {n_side}^2 Oldroyd-B", p, [1.0, 1.0], 0.0, 0.0, seed, 1e-3, 200)


def lees_edwards(dim: int = 3, n_side: int = 24, shear_rate: float = 0.05,
                 precision: int = PRECISION_FP64, seed: int = BASE_SEED + 6,
                 kt: float = 0.0) -> Workload:
    """Simple shear through Lees-Edwards y faces (bcdef 10, the planes above
    and below slide along x at +-shear_rate L/2, boundary_update_boundary.F90
    and ppm_bcdef_le_y.inc), periodic x (and z), dx = 1, box starting at 0:
    C2's physics (quintic rc = 3, Hu-Adams, c = 10, eta = 1), dt = 1e-3,
    particles jittered by 0.05 dx, velocities on the linear profile
    v_x = shear_rate (y - L/2) plus N(0, 1e-4)."""
    L = float(n_side)
    box = _box(dim, 0.0, L)
    box["bcdef"][2] = box["bcdef"][3] = BC_LE
    wv = [[0.0] * 3 for _ in range(6)]
    wv[2][0] = -0.5 * shear_rate * L
    wv[3][0] = 0.5 * shear_rate * L
    p = make_params(**box, cut_off=3.0, c=10.0, eta=1.0, kt=kt, Brownian=1 if kt > 0 else 0,
                    body_force_type=0, dt=1e-3, precision=precision, seed=seed, wall_v=wv)
    w = _finish(f"Lees-Edwards {dim}D {n_side}^{dim} shear {shear_rate}", p, [1.0] * dim, 0.05,
                1e-4, seed, 1e-3, 1000)
    w.v[:, 0] += shear_rate * (w.x[:, 1] - 0.5 * L)
    return w


def couette_walls(dim: int = 2, n_side: int = 32, v_top: float = 0.05,
                  precision: int = PRECISION_FP64, seed: int = BASE_SEED + 7) -> Workload:
    """Couette / oscillating-wall flow between solid y walls (Morris no-slip,
    4 layers each side): the top wall moves along x at v_top (MCF's
    shear_v0 of face y+), the bottom one rests; wall particles start with
    their face velocity.  Periodic x (and z), dx = 1, C2's physics, dt = 1e-3.
    mcfg_set_boundary_motion with shear_type[3] = 2 turns the top wall into
    an oscillating one."""
    L = float(n_side)
    nl = wall_layers(3.0, 1.0)
    box = _box(dim, 0.0, L, walls_axis=1, nwall_layers=nl, dx=1.0)
    wv = [[0.0] * 3 for _ in range(6)]
    wv[3][0] = v_top
    p = make_params(**box, cut_off=3.0, c=10.0, eta=1.0, kt=0.0, Brownian=0,
                    wall_noslip_type=2, wall_rho_type=0, init_density=1.0, body_force_type=0,
                    dt=1e-3, precision=precision, seed=seed, wall_v=wv)
    w = _finish(f"Couette {dim}D {n_side}^{dim} v_top {v_top}", p, [1.0] * dim, 0.05, 1e-4, seed,
                1e-3, 1000)
    top = w.id[:, 1] == -4
    w.v[top, 0] = v_top
    return w


def poiseuille_channel(dim: int = 2, n_side: int = 20, force: float = 0.01,
                       precision: int = PRECISION_FP64, seed: int = BASE_SEED + 8) -> Workload:
    """Transient plane Poiseuille flow: fluid at rest on the dx = 1 lattice
    between solid y walls (Morris no-slip, 4 constant-density layers each
    side, the channel y in [0, n_side]), periodic x (and z), driven by a
    uniform body force g_x = force (body_force_type 1); c = 10, eta = 1
    (nu = 1 at rho = 1), kT = 0, dt = 0.01 (the viscous limit
    0.125 dx^2 / nu is 0.125)."""
    L = float(n_side)
    nl = wall_layers(3.0, 1.0)
    box = _box(dim, 0.0, L, walls_axis=1, nwall_layers=nl, dx=1.0)
    p = make_params(**box, cut_off=3.0, c=10.0, eta=1.0, kt=0.0, Brownian=0,
                    body_force_type=1, body_force=[force, 0.0, 0.0], dt=0.01,
                    wall_noslip_type=2, wall_rho_type=0, init_density=1.0,
                    precision=precision, seed=seed)
    w = _finish(f"Poiseuille channel {dim}D {n_side}^{dim} g {force}", p, [1.0] * dim, 0.0, 0.0,
                seed, 0.01, 10000)
    w.v[:] = 0.0
    return w


def write_mcf_scalability_deck(folder, n_side: int = 100, box: float | None = None):
    """Write, in MCF's deck format, the physics of MCF's 1M-particle
    scalability input (mcf_config_test_SupMuc/ctrl.mcf and
    physics_config.mcf): 3D periodic cube of n_side^3 lattice sites, dx =
    0.1 (box 10 at 100^3), cut-off 0.4 = 4 dx, quintic kernel, number
    density, Batchelor equation of state (c = 84.6, rho = 1, rho_ref = 0.9,
    gamma = 7), Hu-Adams angular force (rhs_force_type 4, eta = 8.46,
    eta_coef = 4), no noise, no body force, 2000 steps, dt from MCF's
    criteria (the viscous one, 2.63e-4).  Returns the folder."""
    from pathlib import Path
    f = Path(folder)
    f.mkdir(parents=True, exist_ok=True)
    L = box if box is not None else 0.1 * n_side
    ctrl = {"job_name": "ppm_mcf_scalability", "mcf_physics_config_file": "physics_config.mcf",
            "relax_run": "F", "read_external": "F", "kernel_type": 1, "symmetry": "T",
            "rhs_density_type": 2, "dynamic_density_ref": "F", "stateEquation_type": 2,
            "Newtonian": "T", "Brownian": "F", "random_seed": -1, "rhs_force_type": 4,
            "pp_interact_cc": "F", "p_energy": "F", "flow_v_fixed": "F", "integrate_type": 2,
            "adaptive_dt": 0}
    phys = {"num_species": 1, "num_dim": 3, "min_phys": "0.0, 0.0, 0.0",
            "max_phys": f"{L!r}, {L!r}, {L!r}", "lattice": 1,
            "num_part": f"{n_side}, {n_side}, {n_side}", "cut_off": 0.4, "dt": -1.0,
            "step_start": 0, "step_end": 2000, "rho": 1.0, "eta": 8.46, "eta_coef": 4.0,
            "kt": 0.0, "c": 84.6, "rho_ref": 0.9, "gamma": 7.0, "body_force_type": 0,
            "body_force": "0.0, 0.0, 0.0", "num_colloid": 0, "bcdef": "1,1,1,1,1,1",
            "shear_type": "1,1,1,1,1,1", "wall_rho_type": 0, "wall_noslip": 2}
    (f / "ctrl.mcf").write_text("".join(f"{k} = {v}\n" for k, v in ctrl.items()))
    (f / "physics_config.mcf").write_text("".join(f"{k} = {v}\n" for k, v in phys.items()))
    return f


@dataclass
class ColloidSet:
    params: ColloidParams
    x: np.ndarray
    v: np.ndarray
    omega: np.ndarray
    radius: np.ndarray


def c4_colloids(n_side: int = 96, n_colloid: int = 200, radius: float = 4.0,
                precision: int = PRECISION_FP64, seed: int = BASE_SEED + 4,
                min_gap: float = 1.0, v_scale: float = 0.0, omega_scale: float = 0.0):
    """3D colloidal suspension: periodic cube of n_side^3 lattice sites, dx = 1,
    n_colloid rigid spheres of the given radius at seeded non-overlapping
    centres.  Lattice sites inside a sphere within din = 1.05 rc of its
    surface are its boundary particles (sid = colloid number), deeper ones
    are dropped, the rest are solvent (colloid_check_boundary_particle.F90
    with coll_place lattice).  Morris no-slip, constant boundary density,
    eta = 1, c = 10, kT = 1e-3, g_x = 0.05, dt = 5e-5; colloid-colloid
    repulsion is MCF's DLVO form with hn = 0.1 a (the closest MCF has to
    F0 exp(-r / 0.1 a)), F0 = 10.  Returns (Workload, ColloidSet)."""
    L = float(n_side)
    rng = np.random.default_rng(seed)
    centres = []
    tries = 0
    while len(centres) < n_colloid and tries < 200000:
        tries += 1
        cand = rng.uniform(0.0, L, 3)
        ok = True
        for c in centres:
            dd = cand - c
            dd -= L * np.round(dd / L)
            if np.sqrt(dd @ dd) < 2 * radius + min_gap:
                ok = False
                break
        if ok:
            centres.append(cand)
    cx = np.array(centres).reshape(-1, 3)
    nc = cx.shape[0]
    p = make_params(**_box(3, 0.0, L), cut_off=3.0, c=10.0, eta=1.0, kt=1e-3, Brownian=1,
                    body_force_type=1, body_force=[0.05, 0.0, 0.0], dt=5e-5, precision=precision,
                    seed=seed, init_density=1.0)
    x = lattice(3, [0.0] * 3, [L] * 3, [1.0] * 3)
    din = 1.05 * 3.0
    sid = np.zeros(x.shape[0], np.int32)
    keep = np.ones(x.shape[0], bool)
    for ci in range(nc):
        dd = x - cx[ci]
        dd -= L * np.round(dd / L)
        dist = np.sqrt((dd * dd).sum(1))
        inside = dist <= radius
        sid[inside] = ci + 1
        keep[dist <= radius - din] = False
    x, sid = x[keep], sid[keep]
    n = x.shape[0]
    m = np.ones(n)
    ids = np.stack([np.arange(1, n + 1, dtype=np.int32), sid], axis=1).astype(np.int32)
    w = Workload(f"C4 3D {n_side}^3 + {nc} colloids", p, x, np.zeros((n, 3)), m, ids, 5e-5, 2000)
    cp = ColloidParams()
    cp.num_colloid = nc
    cp.noslip_type = 2
    cp.rho_type = 0
    cp.translate = 1
    cp.rotate = 1
    cp.pp_interact_cc = 0
    cp.cc_repul_type = 2
    cp.dout = 0.05 * 1.0  # mcf_colloid_out_layer_coeff * dx
    cp.cc_repul_F0 = 10.0
    cp.cc_repul_cut_off = 0.1 * radius
    cp.cc_repul_cut_on = 0.01 * radius
    cv = rng.normal(0.0, v_scale, (nc, 3)) if v_scale else np.zeros((nc, 3))
    om = rng.normal(0.0, omega_scale, (nc, 3)) if omega_scale else np.zeros((nc, 3))
    return w, ColloidSet(cp, cx, cv, om, np.full(nc, radius))


WORKLOADS = {"c1": c1_poiseuille_2d, "c2": c2_fluctuating_3d, "c3": c3_poiseuille_3d,
             "c4": c4_colloids, "c5": c5_oldroyd_b_2d}
