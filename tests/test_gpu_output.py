"""MCF's particle files formatted on the device (mcfg_write_particles)
against the CPU restatement of the text (oracle/mcf_format.py), byte for
byte: the particle output with and without the stress columns and the
restart file of a stepped workload, and E16.8 of values chosen to be hard
(decimal ties, powers of ten and their neighbours, carries into the next
decade, signed zero, subnormals, exponents past 99, random magnitudes
1e-17 .. 1e29); the statistic line (mcfg_write_statistic) against the
restatement fed with the same global sums."""
import numpy as np
import pytest

from mcf_gb300 import SDPD, configs
from oracle.mcf_format import particle_rows, restart_text, statistic_line

pytestmark = pytest.mark.gpu


def hard_values(rng, n):
    vals = [1.0, -1.5e-3, 0.0, -0.0, 12.0, 123456785.0, 123456795.0, 0.999999999, 99999999.5,
            10000000.5, 12345678.5, 99999998.5, 3.14159265358979, 0.5, 0.25, 0.125, 1e-18,
            9.99999995e-5, 1e29, 5e-324, 2.5e-310, 1e-30, 1e35, 1e100, -1e-100, 1e-101,
            1.7976931348623157e308]
    for e in range(-20, 31):
        p = 10.0 ** e
        vals += [p, np.nextafter(p, 0.0), np.nextafter(p, np.inf), -p]
    # exact decimal ties at the ninth digit: k + 1/2 for 8-digit k, scaled by 2^j
    ks = rng.integers(10_000_000, 99_999_999, 200)
    vals += [float(k) + 0.5 for k in ks]
    vals += [(float(k) + 0.5) * 2.0 ** -20 for k in ks[:50]]
    rnd = 10.0 ** rng.uniform(-17, 29, n) * rng.choice([-1.0, 1.0], n)
    out = np.concatenate([np.array(vals), rnd])
    return out


def test_particle_file_of_a_stepped_workload(gpu_lib, tmp_path):
    w = configs.c3_poiseuille_3d(n_side=16)
    w.params.stress_tensor = 1
    g = SDPD(w.params)
    g.upload(w.x, w.v, w.m, w.id)
    g.marching_init_force(0)
    g.run_vv(0, 5, w.dt)
    d = g.download("x", "v", "rho", "s")
    g.write_particles(tmp_path / "mcf_particles00000005.out")
    assert (tmp_path / "mcf_particles00000005.out").read_text() == \
        particle_rows(d["x"], d["v"], d["rho"], w.m, w.id)
    g.write_particles(tmp_path / "with_stress.out", stress=True)
    assert (tmp_path / "with_stress.out").read_text() == \
        particle_rows(d["x"], d["v"], d["rho"], w.m, w.id, s=d["s"])
    g.write_particles(tmp_path / "mcf_restart_particles00000005.dat", kind=1)
    assert (tmp_path / "mcf_restart_particles00000005.dat").read_text() == \
        restart_text(d["x"], d["v"], d["rho"], w.m, w.id)


def test_hard_values_2d_and_3d(gpu_lib, tmp_path):
    rng = np.random.default_rng(77)
    for w in (configs.c2_fluctuating_3d(n_side=12), configs.c5_oldroyd_b_2d(n_side=40)):
        n, dim = w.x.shape
        vals = hard_values(rng, n * dim)
        w.v = vals[: n * dim].reshape(n, dim) if vals.size >= n * dim else \
            np.resize(vals, (n, dim))
        g = SDPD(w.params)
        g.upload(w.x, w.v, w.m, w.id)
        d = g.download("x", "v", "rho")
        path = tmp_path / f"hard_{dim}.out"
        g.write_particles(path)
        got = path.read_text().splitlines()
        ref = particle_rows(d["x"], d["v"], d["rho"], w.m, w.id).splitlines()
        assert len(got) == len(ref) == n
        bad = [(i, a, b) for i, (a, b) in enumerate(zip(got, ref)) if a != b]
        assert not bad, bad[:3]


@pytest.mark.parametrize("stress", [False, True])
def test_statistic_lines_appended(gpu_lib, tmp_path, stress):
    w = configs.c5_oldroyd_b_2d(n_side=40) if not stress else configs.c2_fluctuating_3d(n_side=12)
    w.params.stress_tensor = 1 if stress else 0
    g = SDPD(w.params)
    g.upload(w.x, w.v, w.m, w.id)
    g.marching_init_force(0)
    path = tmp_path / "mcf_statistic.dat"
    ref = ""
    for s0 in (0, 5, 10):
        if s0:
            g.run_vv(s0 - 5, 5, w.dt)
        ke, mom, st = g.statistic_compute_statistic()
        g.write_statistic(path, s0, s0 * w.dt)
        ref += statistic_line(s0, s0 * w.dt, ke, mom[: w.x.shape[1]], st if stress else None)
    assert path.read_text() == ref
    assert path.read_text().count("\n") == 3
