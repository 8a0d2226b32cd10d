"""Fluctuating SDPD checked statistically (kT > 0, Philox Wiener increments).

Equipartition.  The kinetic temperature <m v_a^2> is compared with what the
reference's random force implies:
  - Espanol-Revenga (rhs_force_type 2, rhs_force_ff_Newtonian_Espanol.F90:
    130-247) satisfies the fluctuation-dissipation balance: T_kin = kT;
  - Hu-Adams (type 3, rhs_force_ff_Newtonian_HuAdams.F90:176-239) draws
    We = dW e with dW symmetric and traceless, whose component along e has
    variance 1 - 1/d and across e 1/2, with f_r^2 = -4 kT f_d.  Across e that
    is the balanced amount, along e 2(1 - 1/d) times it, so
    T_kin / kT = (d - 1 + 2(1 - 1/d)) / d: 10/9 in 3D, exactly 1 in 2D.
Each is asserted to 1% after equilibration.

FP32-mixed against FP64 with independent noise streams (another seed):
velocity autocorrelation and shear-stress fluctuation variance agree within
their statistical errors.  Against the CPU oracle with the same keys: the
kinetic energy and shear stress of every step of a fluctuating trajectory
agree to 3e-5 relative (the GPU's FP32 normals are within ~5e-6 of the
oracle's exact Box-Muller values).

Workload: periodic cubes (squares) at dx = 1 with C2's physics (quintic
rc = 3, c = 10, eta = 1, kT = 1e-3), velocities from Maxwell-Boltzmann,
dt = 1e-3 to equilibrate (about 10 time units; the start from a lattice
relaxes slowly through its sound modes) and for sampling.

At C2's own size (64^3 = 262,144 particles) and time step (1e-4, 2000
steps after the equilibration) the same comparisons run with an ensemble:
the shear stress of 512 sub-boxes of 8^3 lattice sites (each a nearly
independent sample, 200 snapshots) gives the stress-fluctuation variance to
about 1.5%, so FP32-mixed and FP64 (independent streams) must agree within
5%; equipartition within 1% in both; the velocity autocorrelation of 20,000
particles within 0.01.
"""
import numpy as np
import pytest

from mcf_gb300 import SDPD, configs
from mcf_gb300.params import PRECISION_FP32_MIXED, PRECISION_FP64
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

KT = 1e-3
DT = 1e-3


def fluct_workload(dim=3, n_side=32, precision=PRECISION_FP32_MIXED, ftype=3,
                   seed=20261203 + 2, vseed=7):
    if dim == 3:
        w = configs.c2_fluctuating_3d(n_side=n_side, precision=precision)
    else:
        w = configs.c5_oldroyd_b_2d(n_side=n_side, precision=precision)
        w.params.Newtonian = 1
        w.params.body_force_type = 0
        w.params.eta = 1.0
    p = w.params
    p.stress_tensor = 1
    p.seed = seed
    p.kt = KT
    p.rhs_force_type = ftype
    w.dt = DT
    rng = np.random.default_rng(vseed)
    w.v = rng.normal(0.0, np.sqrt(KT / w.m[0]), w.v.shape)
    w.v -= w.v.mean(0)
    return w


def equilibrated(w, nsteps):
    sd = SDPD(w.params)
    sd.upload(w.x, w.v, w.m, w.id)
    sd.marching_init_force(0)
    sd.run_vv(0, nsteps, w.dt)
    return sd


def sample(sd, w, step0, nsteps, every, keep_v=False):
    ke, sxy, vs = [], [], []
    d = w.params.num_dim
    for s in range(step0, step0 + nsteps, every):
        sd.run_vv(s, every, w.dt)
        k, _, st = sd.statistic_compute_statistic()
        ke.append(k)
        sxy.append(0.5 * (st[1] + st[d]))
        if keep_v:
            vs.append(sd.download("v")["v"].copy())
    return np.array(ke), np.array(sxy), (np.array(vs) if keep_v else None)


def t_kin(ke, w):
    d = w.params.num_dim
    return 2.0 * ke.mean() / ((w.n - 1) * d) / KT


def expected_ratio(d, ftype):
    return 1.0 if ftype == 2 else (d - 1 + 2.0 * (1.0 - 1.0 / d)) / d


@pytest.mark.parametrize("dim,n_side,ftype", [(3, 32, 2), (3, 32, 3), (2, 128, 3)])
def test_equipartition(gpu_lib, dim, n_side, ftype):
    w = fluct_workload(dim=dim, n_side=n_side, ftype=ftype)
    sd = equilibrated(w, 10000)
    ke, _, _ = sample(sd, w, 10000, 10000, 100)
    ratio = t_kin(ke, w) / expected_ratio(dim, ftype)
    assert abs(ratio - 1.0) < 0.01, ratio


def test_equipartition_fp64_from_equilibrium(gpu_lib):
    w = fluct_workload()
    eq = equilibrated(w, 10000).download("x", "v")
    w64 = fluct_workload(precision=PRECISION_FP64)
    w64.x, w64.v = eq["x"], eq["v"]
    sd = equilibrated(w64, 0)
    ke, _, _ = sample(sd, w64, 0, 3000, 50)
    ratio = t_kin(ke, w64) / expected_ratio(3, 3)
    assert abs(ratio - 1.0) < 0.01, ratio


def vacf(vs, max_lag):
    c0 = np.mean(np.sum(vs * vs, axis=2))
    return np.array([np.mean(np.sum(vs[: len(vs) - lag] * vs[lag:], axis=2)) / c0
                     for lag in range(max_lag + 1)])


def test_vacf_and_stress_variance_fp32_vs_fp64(gpu_lib):
    w = fluct_workload()
    eq = equilibrated(w, 10000).download("x", "v")
    series = []
    for prec, seed in ((PRECISION_FP64, 11), (PRECISION_FP32_MIXED, 12)):
        wp = fluct_workload(precision=prec, seed=seed)
        wp.x, wp.v = eq["x"], eq["v"]
        sd = equilibrated(wp, 0)
        series.append(sample(sd, wp, 0, 2000, 10, keep_v=True))
    (_, s_a, v_a), (_, s_b, v_b) = series
    ca, cb = vacf(v_a, 40), vacf(v_b, 40)
    assert ca[40] < 0.6 and cb[40] < 0.6  # it decays over the window
    assert np.max(np.abs(ca - cb)) < 0.03, np.max(np.abs(ca - cb))
    # 200 shear-stress samples a few steps correlated: ~15-25% sampling error
    ratio = np.var(s_a) / np.var(s_b)
    assert abs(ratio - 1.0) < 0.35, ratio


def test_c2_64cubed_ensemble_statistics_fp32_vs_fp64(gpu_lib):
    w = fluct_workload(n_side=64)
    eq = equilibrated(w, 10000).download("x", "v")
    rng = np.random.default_rng(64)
    pick = rng.choice(w.n, 20000, replace=False)
    nsub = 8  # sub-boxes per axis
    out = []
    for prec, seed in ((PRECISION_FP64, 11), (PRECISION_FP32_MIXED, 12)):
        wp = fluct_workload(n_side=64, precision=prec, seed=seed)
        wp.x, wp.v = eq["x"], eq["v"]
        wp.dt = 1e-4  # C2's time step
        sd = equilibrated(wp, 0)
        ke, subs, vs = [], [], []
        for s0 in range(0, 2000, 10):
            sd.run_vv(s0, 10, wp.dt)
            st = sd.download("x", "v", "s")
            ke.append(0.5 * float((wp.m[:, None] * st["v"] ** 2).sum()))
            cell = np.floor(np.mod(st["x"], 64.0) / (64.0 / nsub)).astype(int)
            key = cell[:, 0] + nsub * (cell[:, 1] + nsub * cell[:, 2])
            sxy = 0.5 * (st["s"][:, 1] + st["s"][:, 3])
            subs.append(np.bincount(key, weights=sxy, minlength=nsub ** 3))
            vs.append(st["v"][pick].copy())
        out.append((np.array(ke), np.array(subs), np.array(vs), wp))
    (ke_a, sub_a, v_a, w_a), (ke_b, sub_b, v_b, w_b) = out
    for ke, wp in ((ke_a, w_a), (ke_b, w_b)):
        ratio = t_kin(ke, wp) / expected_ratio(3, 3)
        assert abs(ratio - 1.0) < 0.01, ratio
    ca, cb = vacf(v_a, 100), vacf(v_b, 100)
    assert np.max(np.abs(ca - cb)) < 0.01, np.max(np.abs(ca - cb))
    # variance of the sub-box shear stress about its own mean
    va = np.var(sub_a - sub_a.mean(0))
    vb = np.var(sub_b - sub_b.mean(0))
    assert abs(va / vb - 1.0) < 0.05, va / vb


def test_fluctuating_trajectory_matches_oracle(gpu_lib):
    w = fluct_workload(n_side=10, precision=PRECISION_FP64)
    T = 200
    sd = equilibrated(w, 0)
    ke_g, s_g, _ = sample(sd, w, 0, T, 1)
    o = Oracle(w.params)
    o.upload(w.x, w.v, w.m, w.id)
    o.marching_init_force(0)
    ke_o, s_o = [], []
    for t in range(1, T + 1):
        o.marching_integrate_VV(t, w.dt)
        k, _, st = o.statistic_compute_statistic()
        ke_o.append(k)
        s_o.append(0.5 * (st[1] + st[3]))
    ke_o, s_o = np.array(ke_o), np.array(s_o)
    # the GPU's normals are within ~5e-6 of the exact Box-Muller values the
    # oracle draws (hardware log2 / sine / cosine), so the series agree to a
    # few 1e-6 over these 200 steps
    assert np.max(np.abs(ke_g - ke_o) / ke_o) < 3e-5, np.max(np.abs(ke_g - ke_o) / ke_o)
    assert np.max(np.abs(s_g - s_o)) < 3e-5 * np.max(np.abs(s_o))
