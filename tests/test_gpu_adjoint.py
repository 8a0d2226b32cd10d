"""GPU tests of the hand-written adjoint (mcfg_adjoint_run) of the
time-averaged stress J = mean_t sum_q w[q] S_t[q].

References:
  - the FP64 reference gradient: torch autograd of the dense restatement in
    oracle/adjoint_ref.py, itself pinned to the CPU oracle (trajectory and
    central differences, test_adjoint_ref.py);
  - central finite differences of the GPU's own J on the full 2D 128^2
    Oldroyd-B workload, 200 steps, checkpoints every 20: step 1e-6 (eta, c)
    and Richardson-extrapolated steps 1e-2 / 2e-2 (eta, tau, c), see the test.
Tolerances: without noise the adjoint matches the reference gradient to
1e-8 relative; with the random term on, the GPU's FP32 Box-Muller normals
(hardware log2 / sine / cosine) are within ~6e-6 of the exact ones the CPU
reference draws, and the trajectories they drive differ accordingly, so the
bound is 5e-5 of the largest gradient entry; against finite differences of
the GPU's own J the bound is 1e-4.
The torch.autograd.Function wrapper below is test-harness only.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from mcf_gb300 import SDPD, configs  # noqa: E402
from oracle.adjoint_ref import reference_gradient  # noqa: E402
from tests.test_adjoint_ref import W_XY_2D, W_XY_3D, newtonian_small_3d, oldroyd_small  # noqa: E402

pytestmark = pytest.mark.gpu


def gpu_adjoint(w, ct, T, wts, K=20, state_grads=False, **over):
    p = w.params.copy()
    for k, v in over.items():
        setattr(p, k, v)
    g = SDPD(p)
    g.upload(w.x, w.v, w.m, w.id, ct=ct)
    return g, g.adjoint_run(0, T, w.dt, wts, checkpoint_every=K, state_grads=state_grads)


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("noise", [False, True])
@pytest.mark.parametrize("maker", ["oldroyd", "newtonian3d"])
def test_adjoint_matches_reference_gradient(gpu_lib, maker, noise):
    w, ct = oldroyd_small(noise=noise) if maker == "oldroyd" else newtonian_small_3d(noise=noise)
    wts = W_XY_2D if maker == "oldroyd" else W_XY_3D
    T = 8
    _, (J, g, st) = gpu_adjoint(w, ct, T, wts, K=3, state_grads=True)
    Jr, gr, sr = reference_gradient(w.params, w.x, w.v, w.m, w.id[:, 0], ct, 0, T, w.dt, wts,
                                    state_grads=True)
    tol = 5e-5 if noise else 1e-8
    assert abs(J - Jr) <= tol * abs(Jr)
    scale = np.abs(gr).max()
    assert np.max(np.abs(g - gr)) <= tol * scale, (g, gr)
    for key in st:
        assert rel_err(st[key], sr[key]) <= tol, key


def test_adjoint_checkpoint_interval_does_not_change_the_result(gpu_lib):
    w, ct = oldroyd_small()
    res = [gpu_adjoint(w, ct, 7, W_XY_2D, K=K, state_grads=True)[1] for K in (1, 3, 7, 50)]
    for J, g, st in res[1:]:
        assert J == res[0][0]
        assert np.array_equal(g, res[0][1])
        for key in st:
            assert np.array_equal(st[key], res[0][2][key])


def test_adjoint_forward_equals_run_vv(gpu_lib):
    # the adjoint's forward pass is the VV trajectory of mcfg_run_vv: the
    # state it leaves is bit-identical, and J is the mean of the statistics
    w, ct = oldroyd_small()
    T = 6
    g, (J, _) = gpu_adjoint(w, ct, T, W_XY_2D)
    a = g.download("x", "v", "ct")
    h = SDPD(w.params.copy())
    h.upload(w.x, w.v, w.m, w.id, ct=ct)
    h.marching_init_force(0)
    acc = 0.0
    for t in range(1, T + 1):
        h.marching_integrate_VV(t, w.dt)
        _, _, st = h.statistic_compute_statistic()
        acc += float(np.dot(W_XY_2D, st[:4]))
    b = h.download("x", "v", "ct")
    for key in a:
        assert np.array_equal(a[key], b[key]), key
    assert abs(J - acc / T) <= 1e-13 * abs(acc / T)


def test_adjoint_rejects_unsupported_configurations(gpu_lib):
    w, ct = oldroyd_small()
    p = w.params.copy()
    p.precision = 1
    g = SDPD(p)
    g.upload(w.x, w.v, w.m, w.id, ct=ct)
    with pytest.raises(RuntimeError, match="FP64"):
        g.adjoint_run(0, 2, w.dt, W_XY_2D)
    walls = configs.c3_poiseuille_3d(n_side=12)
    walls.params.stress_tensor = 1
    g = SDPD(walls.params)
    g.upload(walls.x, walls.v, walls.m, walls.id)
    with pytest.raises(RuntimeError, match="periodic"):
        g.adjoint_run(0, 2, walls.dt, W_XY_3D)


class StressAdjoint(torch.autograd.Function):
    """J(eta, tau, c) of a fixed initial state, with the backward from the
    CUDA adjoint (test harness only)."""

    @staticmethod
    def forward(ctx, theta, w_, T, K):
        p = w_.params.copy()
        p.eta, p.tau, p.c = (float(t) for t in theta)
        g = SDPD(p)
        g.upload(w_.x, w_.v, w_.m, w_.id)
        J, grad = g.adjoint_run(0, T, w_.dt, W_XY_2D, checkpoint_every=K)
        ctx.save_for_backward(torch.as_tensor(grad))
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gout):
        (grad,) = ctx.saved_tensors
        return gout * grad, None, None, None


def test_c5_gradient_against_finite_differences(gpu_lib):
    # full 2D 128^2 Oldroyd-B workload: 200 steps, checkpoints every 20, kT =
    # 1e-4 with the Philox increments; a small seeded velocity perturbation
    # gives the shear stress a signal from step one.
    # (1) central differences with step 1e-6 (relative) for eta and c,
    #     within 1e-4 plus the rounding floor of the quotient: J sums ~3e6
    #     stress terms over the trajectory and carries ~1e-13 of rounding
    #     (measured up to 3e-13 here), so the floor is 1e-12 / h;
    # (2) Richardson-extrapolated central differences (steps 1e-2, 2e-2)
    #     for all three, within 1e-4: rounding and truncation both far below.
    #     dJ/dtau is five orders below J/tau here (the conformation tensor
    #     starts at I and moves by O(L t)), so at step 1e-6 its quotient
    #     would be mostly rounding; tau is checked by (2) only.
    w = configs.c5_oldroyd_b_2d()
    w.params.stress_tensor = 1
    rng = np.random.default_rng(55)
    w.v = rng.normal(0, 1e-3, w.v.shape)
    theta = torch.tensor([w.params.eta, w.params.tau, w.params.c], dtype=torch.float64,
                         requires_grad=True)
    J = StressAdjoint.apply(theta, w, 200, 20)
    J.backward()
    g = theta.grad.numpy()
    th0 = theta.detach().clone()

    def J_at(k, h):
        t = th0.clone()
        t[k] += h
        return float(StressAdjoint.apply(t, w, 200, 20))

    for k in range(3):
        th = float(th0[k])
        if k != 1:
            h = 1e-6 * abs(th)
            fd = (J_at(k, h) - J_at(k, -h)) / (2 * h)
            floor = 1e-12 / h
            assert abs(fd - g[k]) <= 1e-4 * max(abs(fd), abs(g[k])) + floor, (k, fd, g[k])
        h1 = 1e-2 * abs(th)
        d1 = (J_at(k, h1) - J_at(k, -h1)) / (2 * h1)
        d2 = (J_at(k, 2 * h1) - J_at(k, -2 * h1)) / (4 * h1)
        fdr = (4 * d1 - d2) / 3
        assert abs(fdr - g[k]) <= 1e-4 * abs(g[k]), (k, fdr, g[k])
