"""x-slab decomposition with GPU handles (mcf_gb300.decomp).

Two and three slabs of one box, each slab its own handle on the one GPU of
this run, halos exchanged through host copies in one process: the owned
particles follow the undivided GPU run to rounding (the bars of the CPU
decomposition tests: both draw the same FP32 normals), FP64, and the CPU
oracle's undivided run at the random-force bars of the parity tests (the
GPU's FP32 Box-Muller normals differ from the CPU's in the last bits:
positions 1e-9 of the box, velocities, accelerations 1e-5 of their scale,
densities 1e-9); the FP32-mixed slabs follow the undivided FP32-mixed run
within the FP32 trajectory bar.
"""
import numpy as np
import pytest

from mcf_gb300 import SDPD
from mcf_gb300.decomp import LocalExchange, SlabDecomposition
from mcf_gb300.params import PRECISION_FP32_MIXED
from tests.test_decomposition import (NSTEPS, by_pid, check, stats_close, undivided,
                                      workload)

pytestmark = pytest.mark.gpu


def gpu_undivided(w):
    g = SDPD(w.params)
    g.upload(w.x, w.v, w.m, w.id)
    g.marching_init_force(0)
    g.run_vv(0, NSTEPS, w.dt)
    return g.download("x", "v", "rho", "f")


@pytest.mark.parametrize("nslab", [2, 3])
def test_gpu_slabs_follow_the_undivided_box(gpu_lib, nslab):
    w = workload()
    dec = SlabDecomposition(w.params, nslab, factory=SDPD, exchange=LocalExchange())
    dec.upload(w.x, w.v, w.m, w.id)
    dec.init_force(0)
    dec.run_vv(0, NSTEPS, w.dt)
    got = by_pid(dec.owned_state(), w.n, 3)
    assert dec.migrated > 0
    check(w, got, gpu_undivided(w))
    check(w, got, undivided(w), bars=(1e-9, 1e-5, 1e-9, 1e-5))
    # the box's statistics from the slabs' own particles, all-reduced
    g = SDPD(w.params)
    g.upload(w.x, w.v, w.m, w.id)
    g.marching_init_force(0)
    g.run_vv(0, NSTEPS, w.dt)
    stats_close(dec.statistics(), g.statistic_compute_statistic())


def test_gpu_slabs_fp32_mixed(gpu_lib):
    w = workload()
    w.params.precision = PRECISION_FP32_MIXED
    dec = SlabDecomposition(w.params, 2, factory=SDPD, exchange=LocalExchange())
    dec.upload(w.x, w.v, w.m, w.id)
    dec.init_force(0)
    dec.run_vv(0, NSTEPS, w.dt)
    got = by_pid(dec.owned_state(), w.n, 3)
    ref = gpu_undivided(w)
    L = 18.0
    dx = got["x"] - ref["x"]
    dx -= L * np.round(dx / L)
    assert np.max(np.abs(dx)) <= 1e-6 * L
    assert np.max(np.abs(got["v"] - ref["v"])) <= 1e-4 * np.abs(ref["v"]).max()


def test_statistics_owned_contract(gpu_lib):
    # all particles: mcfg_statistics' sums; none: zeros; out of range: refused
    from mcf_gb300.mcfg import MCFGError

    w = workload()
    g = SDPD(w.params)
    g.upload(w.x, w.v, w.m, w.id)
    g.marching_init_force(0)
    g.run_vv(0, 2, w.dt)
    ke, mom, st = g.statistic_compute_statistic()
    ke_o, mom_o, st_o = g.statistic_compute_statistic(n_owned=w.n)
    assert ke_o == ke and np.array_equal(mom_o, mom) and np.array_equal(st_o, st)
    ke0, mom0, st0 = g.statistic_compute_statistic(n_owned=0)
    assert ke0 == 0.0 and not np.any(mom0) and not np.any(st0)
    # the first half in host order against the same sums on the host
    half = w.n // 2
    keh, momh, _ = g.statistic_compute_statistic(n_owned=half)
    d = g.download("v")["v"][:half]
    fl = w.id[:half, 1] == 0
    ref_ke = 0.5 * float(np.sum(w.m[:half][fl] * np.sum(d[fl] ** 2, axis=1)))
    assert abs(keh - ref_ke) <= 1e-12 * ref_ke
    assert np.allclose(momh, (w.m[:half][fl, None] * d[fl]).sum(0), rtol=1e-12, atol=1e-15)
    for bad in (-1, w.n + 1):
        with pytest.raises(MCFGError):
            g.statistic_compute_statistic(n_owned=bad)


def test_gpu_slab_without_particles(gpu_lib):
    # a void across one of four slabs: that handle holds halo particles
    # only (or none), the decomposed run still follows the undivided one
    w = workload()
    keep = ~((w.x[:, 0] >= 9.0) & (w.x[:, 0] < 13.5))
    w.x, w.v, w.m, w.id = w.x[keep], w.v[keep], w.m[keep], w.id[keep].copy()
    w.id[:, 0] = np.arange(1, w.n + 1, dtype=np.int32)
    w.v[w.id[:, 1] == 0, 0] -= 1.0
    dec = SlabDecomposition(w.params, 4, factory=SDPD, exchange=LocalExchange())
    dec.upload(w.x, w.v, w.m, w.id)
    assert dec.subs[2].n_own == 0
    dec.init_force(0)
    dec.run_vv(0, NSTEPS, w.dt)
    got = by_pid(dec.owned_state(), w.n, 3)
    check(w, got, gpu_undivided(w))
