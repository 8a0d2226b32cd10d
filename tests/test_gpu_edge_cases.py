"""Edge cases through the C-ABI: an empty particle set (every entry point
returns cleanly with empty results and writes files with no records), a
single particle (its density is the self term W(0), its acceleration the
body force alone), two particles straddling a periodic face, and the
smallest periodic box the cell list allows (3 cells per axis: every
neighbour slot a distinct cell), each against the CPU oracle."""
import numpy as np
import pytest

from mcf_gb300 import SDPD, configs
from mcf_gb300.params import PRECISION_FP32_MIXED, PRECISION_FP64
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def test_empty_particle_set(gpu_lib, tmp_path):
    w = configs.c2_fluctuating_3d(n_side=12)
    g = SDPD(w.params)
    g.upload(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0), np.zeros((0, 2), np.int32))
    g.marching_init_force(0)
    g.run_vv(0, 3, w.dt)
    d = g.download("x", "v", "rho", "f")
    assert all(a.size == 0 for a in d.values())
    ke, mom, _ = g.statistic_compute_statistic()
    assert ke == 0.0 and not np.any(mom)
    g.write_particles(tmp_path / "empty.out")
    g.write_particles(tmp_path / "empty.dat", kind=1)
    assert (tmp_path / "empty.out").read_text() == ""
    assert (tmp_path / "empty.dat").read_text() == "           0\n"


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_FP32_MIXED])
def test_single_particle(gpu_lib, precision):
    w = configs.c1_poiseuille_2d(n_side=16, body_force_type=1)
    p = w.params.copy()
    p.precision = precision
    x = np.array([[0.3, 0.7]])
    v = np.array([[0.01, -0.02]])
    m = w.m[:1]
    ids = np.array([[1, 0]], np.int32)
    g = SDPD(p)
    g.upload(x, v, m, ids)
    g.marching_init_force(0)
    o = Oracle(p)
    o.upload(x, v, m, ids)
    o.marching_init_force(0)
    a = g.download("rho", "f")
    b = o.download("rho", "f")
    assert abs(a["rho"][0] - b["rho"][0]) <= 1e-12 * b["rho"][0]
    assert np.array_equal(a["f"], b["f"]) and np.allclose(a["f"], [[1.0, 0.0]])
    assert g.info()["num_pairs"] == 0
    g.run_vv(0, 10, w.dt)
    o.run_vv(0, 10, w.dt)
    assert np.allclose(g.download("x")["x"], o.download("x")["x"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("dim", [2, 3])
def test_pair_across_a_periodic_face(gpu_lib, dim):
    w = configs.c2_fluctuating_3d(n_side=12) if dim == 3 else configs.c5_oldroyd_b_2d(n_side=12)
    p = w.params.copy()
    p.Newtonian = 1
    p.Brownian = 0
    p.kt = 0.0
    p.body_force_type = 0
    L = 12.0
    x = np.full((2, dim), 6.0)
    x[0, 0], x[1, 0] = 0.4, L - 0.9  # 1.3 apart through the x face
    v = np.zeros((2, dim))
    v[0, 1] = 0.05
    ids = np.array([[1, 0], [2, 0]], np.int32)
    m = np.ones(2)
    g = SDPD(p)
    g.upload(x, v, m, ids)
    g.marching_init_force(0)
    o = Oracle(p)
    o.upload(x, v, m, ids)
    o.marching_init_force(0)
    a = g.download("rho", "f")
    b = o.download("rho", "f")
    assert np.allclose(a["rho"], b["rho"], rtol=1e-12, atol=0)
    assert np.allclose(a["f"], b["f"], rtol=1e-12, atol=1e-15 * np.abs(b["f"]).max())
    assert np.abs(b["f"]).max() > 0 and np.allclose(a["f"][0], -a["f"][1], rtol=1e-12)
    assert g.info()["num_pairs"] == 2


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_FP32_MIXED])
def test_smallest_periodic_box(gpu_lib, precision):
    # 9.5 / (3 * 1.0001) -> 3 cells a side of 3.17: each particle's
    # neighbourhood wraps onto the opposite faces in every direction
    w = configs.c2_fluctuating_3d(n_side=12)
    p = w.params.copy()
    p.precision = precision
    p.Brownian = 0
    p.kt = 0.0
    for a in range(3):
        p.max_phys[a] = p.max_phys_t[a] = 9.5
    rng = np.random.default_rng(21)
    n = 800
    x = rng.uniform(0.0, 9.5, (n, 3))
    v = rng.normal(0.0, 0.01, (n, 3))
    m = np.full(n, 9.5 ** 3 / n)
    ids = np.stack([np.arange(1, n + 1), np.zeros(n)], 1).astype(np.int32)
    g = SDPD(p)
    g.upload(x, v, m, ids)
    g.marching_init_force(0)
    o = Oracle(p)
    o.upload(x, v, m, ids)
    o.marching_init_force(0)
    assert tuple(g.info()["num_cell_dim"])[:3] == (3, 3, 3)
    a = g.download("rho", "f")
    b = o.download("rho", "f")
    scale = o.force_scale()[:, None] + np.abs(b["f"])
    if precision == PRECISION_FP64:
        assert np.max(np.abs(a["rho"] - b["rho"]) / b["rho"]) <= 1e-12
        assert np.max(np.abs(a["f"] - b["f"]) / scale) <= 1e-12
    else:
        assert np.max(np.abs(a["rho"] - b["rho"]) / b["rho"]) <= 2e-6
        assert np.max(np.abs(a["f"] - b["f"]) / scale) <= 1e-4
