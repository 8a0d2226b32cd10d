"""MCF input decks read into runs of this library (mcf_gb300/mcf_config.py):
the readers' rules (key = value lines, # comments, case-insensitive keys,
list-directed values, colloid keys once per colloid), MCF's set-up
arithmetic (dx, wall layers, time step, masses, shear velocities) on decks
written here, particles read from a restart file (read_external), and --
where the reference tree is present -- its two sample decks (the 2D flow
around a cylinder and the 1M-particle 3D scalability deck), read exactly as
MCF sets them up (MCF_REFERENCE_DIR names the reference's mcf/ folder;
those tests skip when it is unset)."""
import math
import os
from pathlib import Path

import numpy as np
import pytest

from mcf_gb300.mcf_config import load_mcf_deck, parse_mcf_file, read_particles_file
from mcf_gb300.params import BC_WALL_SOLID
from oracle.mcf_format import e16_8, restart_text

_REF_ENV = os.environ.get("MCF_REFERENCE_DIR", "")
REF = Path(_REF_ENV) if _REF_ENV else None


def write_deck(folder: Path, ctrl: dict, phys: dict, extra_phys: str = "") -> Path:
    folder.mkdir(parents=True, exist_ok=True)
    lines = ["# control deck written by the test", "mcf_physics_config_file = phys.mcf"]
    lines += [f"{k} = {v}" for k, v in ctrl.items()]
    (folder / "ctrl.mcf").write_text("\n".join(lines) + "\n")
    plines = ["#  physics deck", ""] + [f"{k} = {v}" for k, v in phys.items()]
    (folder / "phys.mcf").write_text("\n".join(plines) + "\n" + extra_phys)
    return folder


CTRL = {"kernel_type": 1, "symmetry": "T", "rhs_density_type": 2, "stateEquation_type": 1,
        "Newtonian": "T", "Brownian": "F", "random_seed": 77, "rhs_force_type": 3,
        "stress_tensor": "F", "integrate_type": 2, "relax_run": "F", "read_external": "F"}


def channel_phys(**over):
    d = {"num_species": 1, "num_dim": 2, "min_phys": "0.0, 0.0", "max_phys": "1.0, 1.0",
         "lattice": 1, "num_part": "20, 20", "cut_off": "0.15", "dt": -1.0,
         "step_start": 0, "step_end": -1, "time_start": 0.0, "time_end": 0.5,
         "rho": "1.0d0", "eta": 0.5, "c": 10.0, "rho_ref": 1.0, "gamma": 1.0,
         "body_force_type": 1, "body_force": "0.5, 0.0", "bcdef": "1, 1, 9, 9",
         "shear_type": "1, 1, 1, 2", "shear_v": "0.0, 0.0, 0.0, 0.25",
         "shear_freq": "0.0, 0.0, 0.0, 3.0", "wall_rho_type": 0, "wall_noslip": 2}
    d.update(over)
    return d


def test_reader_rules(tmp_path):
    f = tmp_path / "a.mcf"
    f.write_text("# comment = not a key\n\nNum_Dim = 3\ncoll_x = 1,2,3\ncoll_x = 4 5 6\n"
                 "no equals sign here\n  eta  =  8.46  \n")
    d = parse_mcf_file(f)
    assert d["NUM_DIM"] == ["3"] and d["ETA"] == ["8.46"]
    assert d["COLL_X"] == ["1,2,3", "4 5 6"] and "# COMMENT" not in d


def test_channel_deck_setup(tmp_path):
    deck = load_mcf_deck(write_deck(tmp_path / "run", CTRL, channel_phys()))
    p = deck.params
    dx = 1.0 / 20
    assert deck.dx == [dx, dx] and deck.h == pytest.approx(0.05)
    # wall layers CEILING(1.05 rc / dx) = 4 below and above along y
    assert p.min_phys_t[1] == pytest.approx(-4 * dx) and p.max_phys_t[1] == pytest.approx(1 + 4 * dx)
    assert list(p.bcdef)[:4] == [1, 1, BC_WALL_SOLID, BC_WALL_SOLID]
    # dt: min(0.25 h / c, 0.125 h^2 rho / eta, 0.25 sqrt(h / |g|))
    h = 0.15 / 3
    want = min(0.25 * h / 10.0, 0.125 * h * h / 0.5, 0.25 * math.sqrt(h / 0.5))
    assert deck.dt == want and deck.n_steps == math.ceil(0.5 / want - 1e-9)
    w = deck.workload
    sid = w.id[:, 1]
    assert w.n == 20 * 28 and (sid == -3).sum() == 80 and (sid == -4).sum() == 80
    assert np.all(w.m == (1.0 * dx) * dx)
    # shear_v (2D): v_y of the x faces, v_x of the y faces
    assert p.wall_v[3][0] == 0.25 and p.wall_v[2][0] == 0.0
    assert deck.shear_type[:4] == [1, 1, 1, 2] and deck.shear_freq[3] == 3.0
    assert p.seed == 77 and p.stateEquation_type == 1 and p.rhs_force_type == 3


def test_shear_v_3d_order(tmp_path):
    phys = channel_phys(num_dim=3, min_phys="0,0,0", max_phys="1,1,1", num_part="10,10,10",
                        body_force="0,0,0", bcdef="1,1,9,9,1,1",
                        shear_v="1,2,3,4,5,6,7,8,9,10,11,12", shear_type="1,1,1,1,1,1",
                        shear_freq="0,0,0,0,0,0")
    p = load_mcf_deck(write_deck(tmp_path / "r3", CTRL, phys)).params
    # io_read_physics.F90:1394-1403: (v_y, v_z) of x faces, (v_x, v_z) of y
    # faces, (v_x, v_y) of z faces
    got = [[p.wall_v[f][a] for a in range(3)] for f in range(6)]
    assert got == [[0, 1, 2], [0, 3, 4], [5, 0, 6], [7, 0, 8], [9, 10, 0], [11, 12, 0]]


@pytest.mark.parametrize("key,val", [("relax_run", ".true."), ("integrate_type", 1),
                                     ("adaptive_dt", 1)])
def test_unsupported_ctrl_keys_are_named(tmp_path, key, val):
    ctrl = dict(CTRL)
    ctrl[key] = val
    with pytest.raises(ValueError, match=key.upper()):
        load_mcf_deck(write_deck(tmp_path / key, ctrl, channel_phys()))


def test_colloid_keys_per_colloid(tmp_path):
    phys = channel_phys(num_species=2, bcdef="1,1,1,1", body_force="1e-3, 0")
    phys["num_colloid"] = 2
    extra = ("coll_shape = 1\ncoll_radius = 0.2, 0.0\ncoll_x = 0.3, 0.5\ncoll_v = 0.1, 0\n"
             "coll_shape = 1\ncoll_radius = 0.15, 0.0\ncoll_x = 0.75, 0.5\ncoll_v = -0.1, 0\n"
             "coll_translate = T\ncoll_rotate = F\ncoll_noslip = 2\n")
    deck = load_mcf_deck(write_deck(tmp_path / "c", CTRL, phys, extra))
    c = deck.colloids
    assert c["params"].num_colloid == 2 and c["params"].translate == 1
    assert np.allclose(c["x"][:, :2], [[0.3, 0.5], [0.75, 0.5]])
    assert np.allclose(c["radius"], [0.2, 0.15]) and np.allclose(c["v"][:, 0], [0.1, -0.1])
    sid = deck.workload.id[:, 1]
    x = deck.workload.x
    # boundary particles inside each disk, none deeper than 1.05 rc
    for k, (cx, r) in enumerate(zip(c["x"][:, :2], c["radius"])):
        dist = np.sqrt(((x - cx) ** 2).sum(1))
        assert np.all(dist[sid == k + 1] <= r)
        assert np.all(dist[sid == 0] > r) and not np.any(dist <= r - 1.05 * 0.15)


@pytest.mark.skipif(REF is None or not REF.exists(),
                    reason="MCF_REFERENCE_DIR unset or not a directory")
def test_reference_sample_decks():
    cyl = load_mcf_deck(REF / "mcf_config")
    p = cyl.params
    assert cyl.name == "flow_around_cylinder" and p.num_dim == 2
    assert cyl.dx == [0.002, 0.002] and cyl.h == pytest.approx(3.2e-3)
    # viscous limit 0.125 h^2 rho / eta = 0.0128 is the smallest
    assert cyl.dt == pytest.approx(0.0128) and cyl.n_steps == 78125
    assert p.stateEquation_type == 2 and p.gamma == 7.0 and p.rhs_force_type == 3
    assert cyl.colloids["params"].num_colloid == 1
    assert cyl.colloids["params"].translate == 0 and cyl.colloids["params"].rotate == 0
    assert cyl.workload.n + 80 == 2500 and (cyl.workload.id[:, 1] == 1).sum() == 236
    big = load_mcf_deck(REF / "mcf_config_test_SupMuc")
    q = big.params
    assert big.workload.n == 1_000_000 and big.n_steps == 2000 and big.colloids is None
    assert q.rhs_force_type == 4 and q.cut_off == 0.4 and q.c == 84.6 and q.eta == 8.46
    h = 0.4 / 3
    assert big.dt == 0.125 * h * h * 1.0 / 8.46
    assert q.reserved[0] >= 300  # rc = 4 dx: ~268 neighbours per particle


def test_read_external_restart_file(tmp_path):
    # a run's restart text (MCF's E16.8 records) read back as the particles
    # of a deck with read_external: the values of the text, the same ids
    first = load_mcf_deck(write_deck(tmp_path / "a", CTRL, channel_phys()))
    w = first.workload
    rng = np.random.default_rng(3)
    v = rng.normal(0.0, 1e-2, w.x.shape)
    rho = rng.uniform(0.9, 1.1, w.n) * 400.0
    folder = tmp_path / "b"
    ctrl = dict(CTRL, read_external="T", mcf_io_config_file="io.mcf")
    write_deck(folder, ctrl, channel_phys())
    (folder / "io.mcf").write_text("read_particles_file = restart_in.dat\n")
    (folder / "restart_in.dat").write_text(restart_text(w.x, v, rho, w.m, w.id))
    deck = load_mcf_deck(folder)
    r = deck.workload
    assert r.n == w.n and np.array_equal(r.id, w.id)
    as_text = np.vectorize(lambda q: float(e16_8(q)))
    assert np.array_equal(r.x, as_text(w.x)) and np.array_equal(r.v, as_text(v))
    assert np.array_equal(r.m, as_text(w.m))
    x2, v2, rho2, m2, id2 = read_particles_file(folder / "restart_in.dat", 2)
    assert np.array_equal(rho2, as_text(rho))


def test_missing_required_key_is_named(tmp_path):
    phys = channel_phys()
    del phys["cut_off"]
    with pytest.raises(ValueError, match="CUT_OFF is required"):
        load_mcf_deck(write_deck(tmp_path / "m", CTRL, phys))
