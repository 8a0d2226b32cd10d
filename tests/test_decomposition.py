"""x-slab domain decomposition (mcf_gb300.decomp) on the CPU.

The decomposed run must follow the undivided box to rounding: the same
pairs, the same Wiener increments (keyed by the particle ids), summed in
another order.  The CPU oracle runs every slab:
  - slabs of one process exchanging in memory (1, 2 and 3 slabs; with one
    slab the halos are the box's own periodic images);
  - one slab per process, world_size 2 and 4, gloo point-to-point messages
    over 127.0.0.1 (migration and both ghost gets cross process borders).
Bars: positions within 1e-11 of the box, velocities within 1e-9 of the
velocity scale, densities within 1e-12 relative, accelerations within 1e-9
of their scale, after the initial right-hand side and 6 steps with the
random force on, particles migrating between slabs.  The box's statistics
(kinetic energy, momentum, stress), summed per slab over its own particles
and all-reduced over the slabs, within 1e-9 of the undivided box's.
"""
import os
import socket

import numpy as np
import pytest

from mcf_gb300 import configs
from mcf_gb300.decomp import LocalExchange, SlabDecomposition, TorchExchange
from oracle.oracle import Oracle

NSTEPS = 6


def workload():
    # 18 x 18 x 18 lattice between y walls, C3's physics with a faster flow
    # so that particles cross slab faces during the steps
    w = configs.c3_poiseuille_3d(n_side=18)
    rng = np.random.default_rng(18)
    fl = w.id[:, 1] == 0
    # lattice planes 0.01 below every integer x (slab faces at 6, 9, 12, 18):
    # particles cross them within the first steps
    w.x[fl, 0] += 0.49
    w.x[fl] += rng.uniform(-0.1, 0.1, (int(fl.sum()), 3))
    w.v[fl] = rng.normal(0.0, 0.3, (int(fl.sum()), 3))
    w.v[fl, 0] += 1.0
    p = w.params
    p.kt = 1e-3
    p.Brownian = 1
    p.stress_tensor = 1  # the statistics' stress sum
    w.dt = 2e-3
    p.dt = w.dt  # the random force's time step in the stage routines
    return w


def undivided(w, stats=False):
    o = Oracle(w.params)
    o.upload(w.x, w.v, w.m, w.id)
    o.marching_init_force(0)
    o.run_vv(0, NSTEPS, w.dt)
    out = o.download("x", "v", "rho", "f")
    return (out, o.statistic_compute_statistic()) if stats else out


def stats_close(got, ref, tol=1e-9):
    """kinetic energy relative; momentum and stress within tol of their scale"""
    assert abs(got[0] - ref[0]) <= tol * abs(ref[0])
    for q in (1, 2):
        scale = np.abs(ref[q]).max()
        assert scale > 0
        assert np.max(np.abs(got[q] - ref[q])) <= tol * scale


def by_pid(parts, n, d):
    out = {k: np.full((n, d) if k in ("x", "v", "f") else (n,), np.nan)
           for k in ("x", "v", "f", "rho")}
    seen = np.zeros(n, int)
    for part in parts:
        idx = part["id"][:, 0] - 1
        seen[idx] += 1
        for k in out:
            out[k][idx] = part[k]
    assert np.all(seen == 1)  # every particle owned by exactly one slab
    return out


def check(w, got, ref, bars=(1e-11, 1e-9, 1e-12, 1e-9)):
    """bars: positions (of the box), velocities (of their scale), densities
    (relative), accelerations (of their scale)"""
    bx, bv, br, bf = bars
    L = 18.0
    dx = got["x"] - ref["x"]
    dx -= L * np.round(dx / L)  # a slab may hold a particle in another image
    assert np.max(np.abs(dx)) <= bx * L
    assert np.max(np.abs(got["v"] - ref["v"])) <= bv * np.abs(ref["v"]).max()
    assert np.max(np.abs(got["rho"] - ref["rho"]) / ref["rho"]) <= br
    assert np.max(np.abs(got["f"] - ref["f"])) <= bf * np.abs(ref["f"]).max()


@pytest.mark.parametrize("nslab", [1, 2, 3])
def test_slabs_in_one_process_follow_the_undivided_box(nslab):
    w = workload()
    ref, ref_stats = undivided(w, stats=True)
    dec = SlabDecomposition(w.params, nslab, factory=Oracle, exchange=LocalExchange())
    dec.upload(w.x, w.v, w.m, w.id)
    dec.init_force(0)
    dec.run_vv(0, NSTEPS, w.dt)
    got = by_pid(dec.owned_state(), w.n, 3)
    check(w, got, ref)
    assert dec.migrated > 0  # particles crossed slab faces (or the periodic x face)
    stats_close(dec.statistics(), ref_stats)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = workload()
        dec = SlabDecomposition(w.params, world, factory=Oracle, exchange=TorchExchange(3),
                                mine=[rank])
        dec.upload(w.x, w.v, w.m, w.id)
        dec.init_force(0)
        dec.run_vv(0, NSTEPS, w.dt)
        parts = dec.owned_state()
        stats = dec.statistics()  # all-reduced over the ranks
        gathered = [None] * world if rank == 0 else None
        dist.gather_object((parts[0], stats), gathered, dst=0)
        if rank == 0:
            q.put(gathered)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 4])
def test_slabs_on_gloo_ranks_follow_the_undivided_box(world):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    w = workload()
    ref, ref_stats = undivided(w, stats=True)
    check(w, by_pid([g[0] for g in gathered], w.n, 3), ref)
    for _, stats in gathered:  # every rank holds the box's sums
        stats_close(stats, ref_stats)


def test_a_slab_without_particles():
    # a void across one of four slabs: that slab owns nothing (it still
    # receives halo particles and returns no densities of its own); the
    # others follow the undivided box as before
    w = workload()
    keep = ~((w.x[:, 0] >= 9.0) & (w.x[:, 0] < 13.5))  # slab 2 of 4 spans [9, 13.5)
    w.x, w.v, w.m, w.id = w.x[keep], w.v[keep], w.m[keep], w.id[keep].copy()
    w.id[:, 0] = np.arange(1, w.n + 1, dtype=np.int32)
    w.v[w.id[:, 1] == 0, 0] -= 1.0  # no mean drift into the void during the steps
    ref = undivided(w)
    dec = SlabDecomposition(w.params, 4, factory=Oracle, exchange=LocalExchange())
    dec.upload(w.x, w.v, w.m, w.id)
    assert dec.subs[2].n_own == 0
    dec.init_force(0)
    dec.run_vv(0, NSTEPS, w.dt)
    got = by_pid(dec.owned_state(), w.n, 3)
    check(w, got, ref)


def test_decomposition_refuses_what_it_does_not_cover():
    from mcf_gb300.params import BC_WALL_SOLID

    w = workload()
    p = w.params.copy()
    p.bcdef[0] = p.bcdef[1] = BC_WALL_SOLID
    with pytest.raises(ValueError, match="periodic along x"):
        SlabDecomposition(p, 2, factory=Oracle)
    with pytest.raises(ValueError, match="narrower than the halo"):
        SlabDecomposition(w.params, 7, factory=Oracle)  # 18/7 < 3.0003
    p = w.params.copy()
    p.Newtonian = 0
    with pytest.raises(ValueError, match="Newtonian"):
        SlabDecomposition(p, 2, factory=Oracle)
    dec = SlabDecomposition(w.params, 2, factory=Oracle, exchange=LocalExchange())
    dec.upload(w.x, w.v, w.m, w.id)
    dec.init_force(0)
    with pytest.raises(ValueError, match="params.dt"):
        dec.step_vv(1, 2.0 * w.params.dt)
