"""MCF input decks run through the C-ABI against the CPU oracle: the
physics of MCF's 1M-particle scalability deck on a 20^3 box (cut-off 4 dx,
~270 neighbours a particle, Batchelor equation of state with gamma = 7,
Hu-Adams angular force), of its 2D flow-around-a-cylinder deck (one
fixed colloid, cut-off 4.8 dx, Batchelor, Hu-Adams) and of a channel with
solid walls and two moving spheres (wall, colloid and fluid pair terms in
one sweep), all read by mcf_config.load_mcf_deck from deck files written
here.

Bars as for the other workloads: FP64 density within 1e-12 relative and
acceleration within 1e-12 of the per-particle scale sum_j |a_ij|; kT = 0
trajectories within 1e-9 of the box and 1e-7 of the velocity scale;
colloid drag within 1e-10 relative; FP32-mixed acceleration within 1e-4
of the scale."""
import numpy as np
import pytest

from mcf_gb300 import SDPD
from mcf_gb300.configs import write_mcf_scalability_deck
from mcf_gb300.mcf_config import load_mcf_deck
from mcf_gb300.params import PRECISION_FP32_MIXED, PRECISION_FP64
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def cylinder_deck(folder):
    """The physics of MCF's 2D flow-around-a-cylinder deck: 0.1 x 0.1
    periodic box of 50 x 50 sites, rc = 9.6e-3, rho = 1000, eta = 0.1,
    c = 0.02, rho_ref = 900, gamma = 7 (Batchelor), g_x = 5e-5, one fixed
    cylinder of radius 0.02 at the centre with Morris no-slip."""
    folder.mkdir(parents=True, exist_ok=True)
    (folder / "ctrl.mcf").write_text(
        "job_name = flow_around_cylinder\nmcf_physics_config_file = physics_config.mcf\n"
        "relax_run = F\nread_external = F\nkernel_type = 1\nsymmetry = T\n"
        "rhs_density_type = 2\nstateEquation_type = 2\nNewtonian = T\nBrownian = F\n"
        "random_seed = -1\nrhs_force_type = 3\npp_interact_cc = F\nstress_tensor = F\n"
        "integrate_type = 2\n")
    (folder / "physics_config.mcf").write_text(
        "num_species = 2\nnum_dim = 2\nmin_phys = 0.0, 0.0\nmax_phys = 0.1, 0.1\n"
        "lattice = 1\nnum_part = 50, 50\ncut_off = 9.6e-3\ndt = -1.0\nstep_start = -1\n"
        "step_end = -1\ntime_start = 0.0\ntime_end = 1000.0\nrho = 1.0e+3\neta = 0.1\n"
        "eta_coef = 4.0\nkt = 0.0\nc = 2.0e-2\nrho_ref = 9.0e+2\ngamma = 7.0\n"
        "body_force_type = 1\nbody_force = 5.0e-5, 0.0\nnum_colloid = 1\ncoll_rho_type = 0\n"
        "coll_translate = F\ncoll_rotate = F\ncoll_place = 1\ncoll_noslip = 2\n"
        "coll_shape = 1\ncoll_radius = 0.02,0.0\ncoll_x = 0.05,0.05\ncoll_v = 0.0,0.0\n"
        "coll_omega = 0.0,0.0,0.0\nbcdef = 1,1,1,1\nwall_rho_type = 0\nwall_noslip = 2\n")
    return folder


def both(deck, precision=PRECISION_FP64):
    w = deck.workload
    p = w.params.copy()
    p.precision = precision
    g = SDPD(p)
    o = Oracle(w.params)
    for h in (g, o):
        h.upload(w.x, w.v, w.m, w.id)
        if deck.colloids is not None:
            c = deck.colloids
            h.set_colloids(c["params"], c["x"], c["v"], c["omega"], c["radius"])
        h.marching_init_force(0)
    return g, o


def check_rhs(g, o, tol=1e-12):
    a = g.download("rho", "f")
    b = o.download("rho", "f")
    assert np.max(np.abs(a["rho"] - b["rho"]) / b["rho"]) <= tol
    scale = o.force_scale()[:, None] + np.abs(b["f"])
    err = np.abs(a["f"] - b["f"])
    # particles without any force term (inside a colloid shell) agree exactly
    assert np.all(err[scale == 0] == 0)
    assert np.max(err[scale > 0] / scale[scale > 0]) <= tol


def check_trajectory(g, o, L):
    a = g.download("x", "v")
    b = o.download("x", "v")
    d = np.abs(a["x"] - b["x"])
    d = np.minimum(d, L - d)
    assert d.max() <= 1e-9 * L
    assert np.abs(a["v"] - b["v"]).max() <= 1e-7 * np.abs(b["v"]).max()


def test_scalability_deck_physics_fp64(gpu_lib, tmp_path):
    deck = load_mcf_deck(write_mcf_scalability_deck(tmp_path / "supermuc", n_side=20))
    assert deck.params.rhs_force_type == 4 and deck.params.reserved[0] >= 300
    w = deck.workload
    rng = np.random.default_rng(12)
    w.x = np.mod(w.x + rng.uniform(-0.02, 0.02, w.x.shape), 2.0)  # off the lattice
    w.v = rng.normal(0.0, 0.05, w.v.shape)
    g, o = both(deck)
    check_rhs(g, o)
    assert g.info()["max_neigh"] > 250
    for s in range(1, 31):
        g.marching_integrate_VV(s, deck.dt)
        o.marching_integrate_VV(s, deck.dt)
    check_trajectory(g, o, 2.0)


def test_default_capacity_fits_the_deck_cut_off(gpu_lib, tmp_path):
    # without an explicit capacity the library sizes the lists from the
    # upload's number density: rc = 4 dx in 3D needs ~270 entries
    deck = load_mcf_deck(write_mcf_scalability_deck(tmp_path / "cap", n_side=20))
    w = deck.workload
    rng = np.random.default_rng(14)  # off the lattice: some particles see > 256
    w.x = np.mod(w.x + rng.uniform(-0.02, 0.02, w.x.shape), 2.0)
    p = w.params.copy()
    p.reserved[0] = 0
    g = SDPD(p)
    g.upload(w.x, w.v, w.m, w.id)
    g.marching_init_force(0)
    g.run_vv(0, 3, deck.dt)
    info = g.info()
    assert info["neigh_capacity"] >= 300 and info["max_neigh"] > 256


def test_scalability_deck_physics_fp32(gpu_lib, tmp_path):
    deck = load_mcf_deck(write_mcf_scalability_deck(tmp_path / "supermuc32", n_side=20))
    w = deck.workload
    rng = np.random.default_rng(13)
    w.x = np.mod(w.x + rng.uniform(-0.02, 0.02, w.x.shape), 2.0)
    g, o = both(deck, PRECISION_FP32_MIXED)
    a = g.download("rho", "f")
    b = o.download("rho", "f")
    assert np.max(np.abs(a["rho"] - b["rho"]) / b["rho"]) < 2e-6
    assert np.max(np.abs(a["f"] - b["f"]) / o.force_scale()[:, None]) < 1e-4


def test_cylinder_deck_fp64(gpu_lib, tmp_path):
    deck = load_mcf_deck(cylinder_deck(tmp_path / "cyl"))
    assert deck.dt == pytest.approx(0.0128) and deck.colloids["params"].num_colloid == 1
    g, o = both(deck)
    check_rhs(g, o)
    for s in range(1, 21):
        g.marching_integrate_VV(s, deck.dt)
        o.marching_integrate_VV(s, deck.dt)
    check_trajectory(g, o, 0.1)
    da, ta = g.colloid_drag()
    db, tb = o.colloid_drag()
    assert np.max(np.abs(da - db)) <= 1e-10 * np.max(np.abs(db))


def test_walls_and_colloids_together_fp64(gpu_lib, tmp_path):
    # a deck with solid y walls and two translating, rotating spheres in the
    # channel: wall-fluid, colloid-fluid and colloid-wall pair terms in one
    # sweep, against the oracle
    folder = tmp_path / "wc"
    folder.mkdir()
    (folder / "ctrl.mcf").write_text(
        "mcf_physics_config_file = physics_config.mcf\nkernel_type = 1\nsymmetry = T\n"
        "rhs_density_type = 2\nstateEquation_type = 1\nNewtonian = T\nBrownian = F\n"
        "rhs_force_type = 3\nstress_tensor = F\nintegrate_type = 2\n")
    (folder / "physics_config.mcf").write_text(
        "num_species = 2\nnum_dim = 3\nmin_phys = 0, 0, 0\nmax_phys = 16, 16, 16\n"
        "lattice = 1\nnum_part = 16, 16, 16\ncut_off = 3.0\ndt = 1e-3\nstep_end = 20\n"
        "rho = 1.0\neta = 1.0\nc = 10.0\nrho_ref = 1.0\ngamma = 1.0\nkt = 0.0\n"
        "body_force_type = 1\nbody_force = 0.05, 0, 0\nbcdef = 1, 1, 9, 9, 1, 1\n"
        "wall_rho_type = 0\nwall_noslip = 2\nnum_colloid = 2\ncoll_translate = T\n"
        "coll_rotate = T\ncoll_noslip = 2\n"
        "coll_shape = 2\ncoll_radius = 3.2, 0\ncoll_x = 4.3, 5.1, 8.2\n"
        "coll_v = 0.01, 0, 0\ncoll_omega = 0, 0, 0.02\n"
        "coll_shape = 2\ncoll_radius = 2.6, 0\ncoll_x = 11.7, 10.4, 7.9\n"
        "coll_v = -0.01, 0.005, 0\ncoll_omega = 0.01, 0, 0\n")
    deck = load_mcf_deck(folder)
    sid = deck.workload.id[:, 1]
    assert (sid == 1).sum() > 0 and (sid == 2).sum() > 0 and (sid < 0).sum() == 16 * 16 * 8
    w = deck.workload
    w.v = np.random.default_rng(15).normal(0.0, 1e-2, w.v.shape) * (sid == 0)[:, None]
    g, o = both(deck)
    check_rhs(g, o)
    for s in range(1, 21):
        g.marching_integrate_VV(s, deck.dt)
        o.marching_integrate_VV(s, deck.dt)
    check_trajectory(g, o, 16.0)
    da, ta = g.colloid_drag()
    db, tb = o.colloid_drag()
    assert np.max(np.abs(da - db)) <= 1e-10 * np.max(np.abs(db))
    assert np.max(np.abs(ta - tb)) <= 1e-10 * np.max(np.abs(tb))
