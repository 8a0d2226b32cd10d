"""MCF input decks (ctrl.mcf + physics_config.mcf) read into a run of this
library: parameter block, initial particles, colloids, boundary motion,
time step and step count.

A user of MCF keeps their decks: `load_mcf_deck("run_dir")` reads the
control file and the physics file it names the way MCF's readers do
(io_read_ctrl.F90, io_read_physics.F90: one `key = value` per line, `#`
comment lines, keys case-insensitive, values list-directed; colloid keys
repeat once per colloid), then sets the run up as MCF's initialisation
does:

- kernel smoothing length h = rc/3 (quintic) or rc (Lucy), kernel_new.F90:41-63;
- dx = (max_phys - min_phys) / num_part per axis, wall layers
  CEILING(1.05 rc [x 2 with dynamic wall density] / dx) outside every solid
  wall face, physics_adjust_parameters.F90:145-273;
- time step, when dt <= 0: the smallest of 0.25 h / c, 0.125 h^2 rho / eta
  and 0.25 sqrt(h / |g|), physics_initialize_dt.F90:60-140;
- particles on the square / cubic lattice over the total domain
  (particles_init_global_inter_square/_cubic.F90), solid-wall sids
  (boundary_check_wall_solid_particle.F90), colloid boundary particles
  (lattice sites inside a colloid within 1.05 rc of its surface; deeper
  ones dropped), masses rho * dx(1) * ... * dx(d) in that order
  (particles_compute_mass.F90:363-450), pids 1..N.

With read_external the particles come from the io deck's
read_particles_file instead (io_read_particles.F90; MCF's restart files
and those mcfg_write_particles writes).

What this path does not cover is rejected with the key that asks for it
(relaxation runs, other lattices, the
eigen-dynamics conformation model, adaptive time steps, dynamic reference
density, non-spherical colloids), and the decks' output settings
(io_config.mcf) are left to the caller.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .configs import Workload, lattice, wall_sid
from .params import (BC_LE, BC_PERIODIC, BC_WALL_SOLID, PRECISION_FP64, ColloidParams,
                     SDPDParams, make_params)


def parse_mcf_file(path) -> dict[str, list[str]]:
    """`key = value` lines of an MCF config file: upper-case keys, each with
    the list of its values in file order (repeated keys, e.g. per colloid)."""
    out: dict[str, list[str]] = {}
    for raw in Path(path).read_text().splitlines():
        line = raw.rstrip()
        if not line.strip() or line.lstrip().startswith("#"):
            continue
        if "=" not in line:
            continue
        k, v = line.split("=", 1)
        out.setdefault(k.strip().upper(), []).append(v.strip())
    return out


def _items(v: str) -> list[str]:
    return [t for t in re.split(r"[,\s]+", v.strip()) if t]


def _float(t: str) -> float:
    return float(t.replace("d", "e").replace("D", "e"))


def _floats(v: str, n: int | None = None) -> list[float]:
    vals = [_float(t) for t in _items(v)]
    return vals if n is None else vals[:n]


def _ints(v: str, n: int | None = None) -> list[int]:
    vals = [int(t) for t in _items(v)]
    return vals if n is None else vals[:n]


def _logical(v: str) -> bool:
    t = v.strip().lstrip(".").upper()
    if not t or t[0] not in "TF":
        raise ValueError(f"not a logical value: {v!r}")
    return t[0] == "T"


@dataclass
class McfDeck:
    """One MCF run set up for this library.  `workload` holds the particles
    (x, v, m, id in MCF's layout) with the parameter block; `colloids` the
    colloid parameters and per-colloid arrays (None without colloids);
    `shear_type` / `shear_freq` go to SDPD.set_boundary_motion."""
    name: str
    workload: Workload
    dt: float
    n_steps: int
    step_start: int
    h: float
    dx: list[float]
    colloids: dict | None = None
    shear_type: list[int] = field(default_factory=lambda: [0] * 6)
    shear_freq: list[float] = field(default_factory=lambda: [0.0] * 6)

    @property
    def params(self) -> SDPDParams:
        return self.workload.params


def _get(d, key, default=None):
    v = d.get(key)
    return v[0] if v else default


def _need(d, key, path):
    v = d.get(key)
    if not v:
        raise ValueError(f"{path}: {key} is required")
    return v[0]


def read_particles_file(path, dim: int):
    """MCF's particle input / restart file (io_read_particles.F90): the
    particle count list-directed, then per particle x(d) v(d) rho m pid sid
    list-directed (the restart file mcfg_write_particles writes with kind
    1).  Returns x, v, rho, m, id as MCF lays them out."""
    lines = Path(path).read_text().splitlines()
    head = [t for t in lines if t.strip()]
    n = int(_items(head[0])[0])
    rows = [[_float(t) for t in _items(line)] for line in head[1:1 + n]]
    if len(rows) != n or any(len(r) < 2 * dim + 4 for r in rows):
        raise ValueError(f"{path}: expected {n} records of {2 * dim + 4} values")
    a = np.array([r[:2 * dim + 4] for r in rows], dtype=np.float64).reshape(n, 2 * dim + 4)
    ids = np.rint(a[:, 2 * dim + 2:2 * dim + 4]).astype(np.int32)
    return a[:, :dim].copy(), a[:, dim:2 * dim].copy(), a[:, 2 * dim].copy(), \
        a[:, 2 * dim + 1].copy(), ids


def _unsupported(ctrl, phys):
    checks = [
        ("RELAX_RUN", ctrl, lambda v: _logical(v), "relaxation runs"),
        ("DYNAMIC_DENSITY_REF", ctrl, lambda v: _logical(v), "a dynamic reference density"),
        ("FLOW_V_FIXED", ctrl, lambda v: _logical(v), "a fixed mean flow velocity"),
        ("P_ENERGY", ctrl, lambda v: _logical(v), "the potential-energy statistic"),
        ("ADAPTIVE_DT", ctrl, lambda v: int(v) != 0, "adaptive time steps"),
        ("INTEGRATE_TYPE", ctrl, lambda v: int(v) != 2, "integrators other than velocity Verlet (2)"),
        ("EIGEN_DYNAMICS", phys, lambda v: _logical(v), "the eigen-dynamics conformation model"),
        ("LATTICE", phys, lambda v: int(v) != 1, "lattices other than square / cubic (1)"),
    ]
    for key, src, bad, what in checks:
        v = _get(src, key)
        if v is not None and bad(v):
            raise ValueError(f"{key} = {v}: {what} not supported on this path")


def load_mcf_deck(path, precision: int = PRECISION_FP64, list_reuse: bool = False,
                  seed: int | None = None) -> McfDeck:
    """Read MCF's control file (`path` itself, or `path`/ctrl.mcf) and the
    physics file it names (mcf_physics_config_file, relative to the
    control file's folder) and set the run up as MCF would."""
    p = Path(path)
    ctrl_path = p / "ctrl.mcf" if p.is_dir() else p
    ctrl = parse_mcf_file(ctrl_path)
    phys_name = _get(ctrl, "MCF_PHYSICS_CONFIG_FILE", "physics_config.mcf")
    phys = parse_mcf_file(ctrl_path.parent / phys_name)
    _unsupported(ctrl, phys)

    dim = int(_get(phys, "NUM_DIM", "2"))
    if dim not in (2, 3):
        raise ValueError(f"NUM_DIM = {dim}: this path runs 2D and 3D")
    nspec = int(_get(phys, "NUM_SPECIES", "1"))
    ncoll = int(_get(phys, "NUM_COLLOID", "0")) if nspec > 1 else 0
    phys_path = ctrl_path.parent / phys_name
    mn = _floats(_need(phys, "MIN_PHYS", phys_path), dim)
    mx = _floats(_need(phys, "MAX_PHYS", phys_path), dim)
    npart = _ints(_need(phys, "NUM_PART", phys_path), dim)
    rc = _float(_need(phys, "CUT_OFF", phys_path))
    if len(mn) < dim or len(mx) < dim or len(npart) < dim:
        raise ValueError(f"{phys_path}: MIN_PHYS, MAX_PHYS and NUM_PART need {dim} values")
    kernel_type = int(_get(ctrl, "KERNEL_TYPE", "1"))
    h = rc / 3.0 if kernel_type == 1 else rc  # kernel_new.F90:41-63
    dx = [(mx[a] - mn[a]) / npart[a] for a in range(dim)]
    bc = _ints(_get(phys, "BCDEF", ",".join(["1"] * (2 * dim))), 2 * dim)
    for f, b in enumerate(bc):
        if b not in (BC_PERIODIC, BC_WALL_SOLID, BC_LE):
            raise ValueError(f"BCDEF face {f + 1} = {b}: periodic (1), solid wall (9) and "
                             "Lees-Edwards (10) faces are supported")
    wall_rho_type = int(_get(phys, "WALL_RHO_TYPE", "0"))
    # physics_adjust_parameters.F90:229-273: wall layers outside each solid face
    mn_t, mx_t = list(mn), list(mx)
    for a in range(dim):
        w = (1.0 + 0.05) * rc * (2.0 if wall_rho_type == 1 else 1.0)
        if bc[2 * a] == BC_WALL_SOLID:
            mn_t[a] = mn[a] - math.ceil(w / dx[a]) * dx[a]
        if bc[2 * a + 1] == BC_WALL_SOLID:
            mx_t[a] = mx[a] + math.ceil(w / dx[a]) * dx[a]
    rho = _float(_get(phys, "RHO", "1.0"))
    eta = _float(_get(phys, "ETA", "0.0"))
    c = _float(_get(phys, "C", "0.0"))
    g = _floats(_get(phys, "BODY_FORCE", ",".join(["0.0"] * dim)), dim)
    # physics_initialize_dt.F90:60-140
    dt = _float(_get(phys, "DT", "-1.0"))
    if dt <= 0.0:
        fa = math.sqrt(sum(x * x for x in g))
        cands = []
        if c > 0:
            cands.append(0.25 * h / c)
        if eta > 0:
            cands.append(0.125 * h * h * rho / eta)
        if fa > 0:
            cands.append(0.25 * math.sqrt(h / fa))
        dt = min(cands) if cands else 1.0e6
    step_start = max(int(_get(phys, "STEP_START", "0")), 0)
    step_end = int(_get(phys, "STEP_END", "-1"))
    if step_end > 0:
        n_steps = step_end - step_start
    else:
        t0 = max(_float(_get(phys, "TIME_START", "0.0")), 0.0)
        t1 = _float(_get(phys, "TIME_END", "-1.0"))
        n_steps = int(math.ceil((t1 - t0) / dt - 1e-9)) if t1 > 0 else 0
    # shear_v(3, 6) of io_read_physics.F90:1378-1406 -> wall_v[face][axis]
    wv = [[0.0] * 3 for _ in range(6)]
    sv = _get(phys, "SHEAR_V")
    if sv is not None:
        vals = _floats(sv)
        order = ([(0, 1), (1, 1), (2, 0), (3, 0)] if dim == 2 else
                 [(0, 1), (0, 2), (1, 1), (1, 2), (2, 0), (2, 2), (3, 0), (3, 2),
                  (4, 0), (4, 1), (5, 0), (5, 1)])
        for (f, a), val in zip(order, vals):
            wv[f][a] = val
    shear_type = [0] * 6
    shear_freq = [0.0] * 6
    if _get(phys, "SHEAR_TYPE") is not None:
        for f, t in enumerate(_ints(_get(phys, "SHEAR_TYPE"), 2 * dim)):
            shear_type[f] = t
    if _get(phys, "SHEAR_FREQ") is not None:
        for f, t in enumerate(_floats(_get(phys, "SHEAR_FREQ"), 2 * dim)):
            shear_freq[f] = t
    rs = int(_get(ctrl, "RANDOM_SEED", "-1"))
    params = make_params(
        num_dim=dim, bcdef=bc + [BC_PERIODIC] * (6 - 2 * dim),
        min_phys=mn + [0.0] * (3 - dim), max_phys=mx + [0.0] * (3 - dim),
        min_phys_t=mn_t + [0.0] * (3 - dim), max_phys_t=mx_t + [0.0] * (3 - dim),
        cut_off=rc, kernel_type=kernel_type,
        rhs_density_type=int(_get(ctrl, "RHS_DENSITY_TYPE", "2")),
        rhs_force_type=int(_get(ctrl, "RHS_FORCE_TYPE", "3")),
        stateEquation_type=int(_get(ctrl, "STATEEQUATION_TYPE", "1")),
        c=c, rho=rho, rho_ref=_float(_get(phys, "RHO_REF", str(rho))),
        gamma=_float(_get(phys, "GAMMA", "1.0")), eta=eta,
        eta_coef=_float(_get(phys, "ETA_COEF", "0.0")),
        kt=_float(_get(phys, "KT", "0.0")), dt=dt,
        Brownian=1 if _logical(_get(ctrl, "BROWNIAN", "F")) else 0,
        symmetry=1 if _logical(_get(ctrl, "SYMMETRY", "T")) else 0,
        body_force_type=int(_get(phys, "BODY_FORCE_TYPE", "0")),
        body_force=g + [0.0] * (3 - dim),
        wall_rho_type=wall_rho_type, wall_noslip_type=int(_get(phys, "WALL_NOSLIP", "2")),
        stress_tensor=1 if _logical(_get(ctrl, "STRESS_TENSOR", "F")) else 0,
        wall_v=wv, init_density=rho,
        Newtonian=1 if _logical(_get(ctrl, "NEWTONIAN", "T")) else 0,
        tau=_float(_get(phys, "TAU", "1.0")), n_p=_float(_get(phys, "N_P", "0.0")),
        kt_p=_float(_get(phys, "KT_P", "0.0")), precision=precision,
        seed=seed if seed is not None else (rs if rs > 0 else 20261203))
    if list_reuse:
        params.reserved[1] = 1
    # neighbour capacity for the deck's cut-off (full lists: pi rc^2 or
    # 4/3 pi rc^3 lattice sites, with room for compression and disorder)
    vol = math.pi * rc * rc if dim == 2 else 4.0 / 3.0 * math.pi * rc ** 3
    est = vol / float(np.prod(dx))
    default_cap = 96 if dim == 2 else 256
    if 1.3 * est + 16 > default_cap:
        params.reserved[0] = int(math.ceil(1.3 * est + 16))

    # particles: lattice over the total domain, wall sids, colloids
    x = lattice(dim, mn_t, mx_t, dx)
    sid = wall_sid(x, params)
    keep = np.ones(x.shape[0], bool)
    colloids = None
    if ncoll > 0:
        def per(key, k, n, fill=0.0):
            vals = phys.get(key, [])
            if k < len(vals):
                v = _floats(vals[k])
                return (v + [fill] * n)[:n]
            return [fill] * n
        cx = np.array([per("COLL_X", k, 3) for k in range(ncoll)])
        cv = np.array([per("COLL_V", k, 3) for k in range(ncoll)])
        om = np.array([per("COLL_OMEGA", k, 3) for k in range(ncoll)])
        rad = np.array([per("COLL_RADIUS", k, 1)[0] for k in range(ncoll)])
        for k in range(ncoll):
            shape = int(_floats(phys["COLL_SHAPE"][k])[0]) if k < len(phys.get("COLL_SHAPE", [])) else 1
            if shape not in (1, 2):
                raise ValueError(f"COLL_SHAPE = {shape}: only circular / spherical colloids")
        din = 1.05 * rc
        L = np.array([mx_t[a] - mn_t[a] for a in range(dim)])
        per_ax = np.array([bc[2 * a] == BC_PERIODIC for a in range(dim)])
        for k in range(ncoll):
            dd = x - cx[k, :dim]
            dd[:, per_ax] -= L[per_ax] * np.round(dd[:, per_ax] / L[per_ax])
            dist = np.sqrt((dd * dd).sum(1))
            sid[(dist <= rad[k]) & (sid == 0)] = k + 1
            keep &= ~(dist <= rad[k] - din)
        cp = ColloidParams()
        cp.num_colloid = ncoll
        cp.noslip_type = int(_get(phys, "COLL_NOSLIP", "2"))
        cp.rho_type = int(_get(phys, "COLL_RHO_TYPE", "0"))
        cp.translate = 1 if _logical(_get(phys, "COLL_TRANSLATE", "F")) else 0
        cp.rotate = 1 if _logical(_get(phys, "COLL_ROTATE", "F")) else 0
        cp.pp_interact_cc = 1 if _logical(_get(ctrl, "PP_INTERACT_CC", "F")) else 0
        cp.cc_repul_type = int(_get(ctrl, "CC_REPUL_TYPE", "0"))
        cp.dout = 0.05 * dx[0]  # mcf_colloid_out_layer_coeff * dx(1)
        cp.cc_repul_F0 = _float(_get(phys, "CC_REPUL_F0", "0.0"))
        cp.cc_repul_cut_off = _float(_get(phys, "CC_REPUL_CUT_OFF", "0.0"))
        cp.cc_repul_cut_on = _float(_get(phys, "CC_REPUL_CUT_ON", "0.0"))
        colloids = {"params": cp, "x": cx, "v": cv, "omega": om, "radius": rad}
    x, sid = x[keep], sid[keep]
    n = x.shape[0]
    mass = rho
    for a in range(dim):
        mass = mass * dx[a]
    m = np.full(n, mass)
    ids = np.stack([np.arange(1, n + 1, dtype=np.int32), sid], axis=1).astype(np.int32)
    v = np.zeros((n, dim))
    if _logical(_get(ctrl, "READ_EXTERNAL", "F")):
        # mcf.F90:701-734: the particles come from read_particles_file of
        # the io deck (a restart file), the rest of the set-up stays
        io_name = _get(ctrl, "MCF_IO_CONFIG_FILE", "io_config.mcf")
        io_path = ctrl_path.parent / io_name
        io = parse_mcf_file(io_path) if io_path.exists() else {}
        fname = _get(io, "READ_PARTICLES_FILE", "mcf_restart_particles.dat")
        x, v, _, m, ids = read_particles_file(ctrl_path.parent / fname, dim)
        n = x.shape[0]
    name = _get(ctrl, "JOB_NAME", ctrl_path.parent.name)
    wl = Workload(f"MCF deck {name}", params, x, v, m, ids, dt, n_steps)
    return McfDeck(name=name, workload=wl, dt=dt, n_steps=n_steps, step_start=step_start, h=h,
                   dx=dx, colloids=colloids, shear_type=shear_type, shear_freq=shear_freq)
