"""The FP64 reference gradient (torch autograd of a dense restatement) pinned
to the CPU oracle: same trajectory and time-averaged stress, and its
gradient against central finite differences of the oracle itself.  These
run on the CPU; the CUDA adjoint is checked against this reference in
test_gpu_adjoint.py."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from mcf_gb300 import configs  # noqa: E402
from oracle.adjoint_ref import RefTrajectory, reference_gradient  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402

W_XY_2D = [0.0, 0.5, 0.5, 0.0]   # symmetric shear stress (S_xy + S_yx)/2
W_XY_3D = [0.0, 0.5, 0.0, 0.5, 0.0, 0.0, 0.0, 0.0, 0.0]


def oldroyd_small(n_side=12, noise=True, seed=21):
    w = configs.c5_oldroyd_b_2d(n_side=n_side, amplitude=0.05)
    rng = np.random.default_rng(seed)
    w.x = w.x + rng.uniform(-0.2, 0.2, w.x.shape)
    w.v = rng.normal(0, 2e-2, w.v.shape)
    p = w.params
    p.stress_tensor = 1
    if not noise:
        p.Brownian = 0
        p.kt = 0.0
    ct = np.tile(np.eye(2).reshape(1, 4), (w.n, 1)) + rng.normal(0, 0.02, (w.n, 4))
    ct[:, 2] = ct[:, 1]
    return w, ct


def newtonian_small_3d(n_side=10, noise=True, seed=22):
    w = configs.c2_fluctuating_3d(n_side=n_side)
    rng = np.random.default_rng(seed)
    w.x = w.x + rng.uniform(-0.2, 0.2, w.x.shape)
    w.v = rng.normal(0, 2e-2, w.v.shape)
    p = w.params
    p.stress_tensor = 1
    p.body_force_type = 1
    p.body_force[0] = 0.05
    if not noise:
        p.Brownian = 0
        p.kt = 0.0
    return w, None


def oracle_J(w, ct, nsteps, wts, **over):
    p = w.params.copy()
    for k, v in over.items():
        setattr(p, k, v)
    o = Oracle(p)
    o.upload(w.x, w.v, w.m, w.id, ct=ct)
    o.marching_init_force(0)
    acc = 0.0
    d = w.params.num_dim
    for t in range(1, nsteps + 1):
        o.marching_integrate_VV(t, w.dt)
        _, _, st = o.statistic_compute_statistic()
        acc += float(np.dot(wts, st[: d * d]))
    return acc / nsteps, o


@pytest.mark.parametrize("maker", ["oldroyd", "newtonian3d"])
def test_reference_trajectory_matches_oracle(maker):
    w, ct = oldroyd_small() if maker == "oldroyd" else newtonian_small_3d()
    wts = W_XY_2D if maker == "oldroyd" else W_XY_3D
    T = 6
    J_o, o = oracle_J(w, ct, T, wts)
    tr = RefTrajectory(w.params, w.x, w.v, w.m, w.id[:, 0], ct)
    p = w.params
    J_r = tr.run(0, T, w.dt, wts, torch.tensor(p.eta, dtype=torch.float64),
                 torch.tensor(p.tau if p.tau > 0 else 1.0, dtype=torch.float64),
                 torch.tensor(p.c, dtype=torch.float64))
    assert abs(float(J_r) - J_o) <= 1e-10 * abs(J_o) + 1e-15
    fin = o.download("x", "v")
    x, v, c = (t.detach().numpy() for t in tr.final)
    L = p.max_phys_t[0] - p.min_phys_t[0]
    dx = x - fin["x"]
    dx -= L * np.round(dx / L)
    assert np.max(np.abs(dx)) <= 1e-12
    assert np.max(np.abs(v - fin["v"])) <= 1e-10 * np.max(np.abs(fin["v"]))
    if not p.Newtonian:
        cto = o.download("ct")["ct"]
        assert np.max(np.abs(c.transpose(0, 2, 1).reshape(-1, 4) - cto)) <= 1e-12


@pytest.mark.parametrize("maker", ["oldroyd", "newtonian3d"])
def test_reference_gradient_matches_oracle_fd(maker):
    # autograd of the restatement against central differences of the
    # oracle (relative step 1e-5), for eta, tau (Oldroyd-B) and c; the
    # bound allows the differences' rounding, a few ulps of J over the step
    w, ct = oldroyd_small() if maker == "oldroyd" else newtonian_small_3d()
    wts = W_XY_2D if maker == "oldroyd" else W_XY_3D
    T = 4
    J, g = reference_gradient(w.params, w.x, w.v, w.m, w.id[:, 0], ct, 0, T, w.dt, wts)
    names = ["eta", "tau", "c"]
    for k, name in enumerate(names):
        if name == "tau" and w.params.Newtonian:
            assert g[k] == 0.0
            continue
        th = getattr(w.params, name)
        hstep = 1e-5 * abs(th)
        jp, _ = oracle_J(w, ct, T, wts, **{name: th + hstep})
        jm, _ = oracle_J(w, ct, T, wts, **{name: th - hstep})
        fd = (jp - jm) / (2 * hstep)
        tol = 1e-6 * max(abs(fd), abs(g[k])) + 8 * np.finfo(float).eps * abs(J) / hstep
        assert abs(fd - g[k]) <= tol, (name, fd, g[k])
