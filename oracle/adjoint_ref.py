"""FP64 reference gradient of the time-averaged stress -- TEST INFRASTRUCTURE.

A differentiable restatement, in torch float64 on the CPU, of the SDPD
velocity-Verlet trajectory that the CPU oracle (oracle/mcf_oracle.c)
computes for fully periodic, all-fluid boxes.  torch.autograd
differentiates it, giving the reference gradient that the hand-written
CUDA adjoint (mcfg_adjoint_run) is checked against.  Nothing here is used by
the library: only tests import this module.

Physics restated (reference files of MCF):
  - quintic spline / Lucy kernel: kernel_kernel_quintic_spline.F90:69-99,
    177-215, kernel_kernel_Lucy.F90:68-78,155-168, constants kernel_new.F90:
    47-63 (3D quintic coefficient 3/(359 pi h^3));
  - number density n_i = W(0) + sum_j W(r_ij): particles_compute_density.F90:
    369,578-867, rhs_density.F90:95-96;
  - equation of state, vector forms: stateEquation_compute_pressure.F90:
    147-180, p0 of stateEquation_new.F90:102-103;
  - Hu-Adams pair force with the Wiener term: rhs_force_ff_Newtonian_HuAdams.
    F90:124-239 (We = dW e drawn from its law given e, as the oracle's
    pair_we); non-Newtonian form with the pressure tensor:
    rhs_force_ff_non_Newtonian_HuAdams.F90:95-201,
    particles_compute_pressure_tensor.F90:88-133;
  - velocity gradient pp_vgt_ip.inc:12-24, act particles_compute_act.F90:
    112-156, ct half steps particles_integrate_ct.F90:66-68;
  - stress s_i += r_ij (x) a_ij / 2: pp_interaction_ff.inc:83-93, summed as in
    statistic_compute_statistic.F90:230-303;
  - body force particles_apply_body_force.F90:96-353;
  - VV order marching_integrate_VV.F90:303-1620.
Pairs are found by minimum image (the box is at least twice the cut-off);
the random term uses the oracle's Philox/Box-Muller normals of each pid
pair (orc_pair_normals) the same way, so the noise is the oracle's.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .oracle import pair_normals_batch

torch_dtype = torch.float64


class RefTrajectory:
    def __init__(self, params, x, v, m, pid, ct=None):
        p = params
        self.p = p
        self.d = int(p.num_dim)
        d = self.d
        self.xmin = torch.tensor([p.min_phys_t[a] for a in range(d)], dtype=torch_dtype)
        self.xmax = torch.tensor([p.max_phys_t[a] for a in range(d)], dtype=torch_dtype)
        self.L = self.xmax - self.xmin
        self.x0 = torch.as_tensor(np.asarray(x, np.float64)[:, :d]).clone()
        self.v0 = torch.as_tensor(np.asarray(v, np.float64)[:, :d]).clone()
        self.m = torch.as_tensor(np.asarray(m, np.float64)).clone()
        self.pid = np.asarray(pid, np.int32)
        n = self.x0.shape[0]
        self.newtonian = bool(p.Newtonian)
        if ct is None:
            ct = np.tile(np.eye(d).reshape(1, d * d), (n, 1))
        # ct[i, a + d*b] = c(a, b)
        self.ct0 = torch.as_tensor(np.asarray(ct, np.float64)).reshape(n, d, d).transpose(1, 2).clone()
        rc = p.cut_off
        self.rc = rc
        if p.kernel_type == 1:
            h = rc / 3.0
            coef = 7.0 / (478.0 * math.pi * h * h) if d == 2 else 3.0 / (359.0 * math.pi * h ** 3)
        else:
            h = rc
            coef = 5.0 / (math.pi * h * h) if d == 2 else 105.0 / (16.0 * math.pi * h ** 3)
        self.h, self.coef = h, coef
        self.w0 = coef * (243.0 - 6.0 * 32.0 + 15.0) if p.kernel_type == 1 else coef
        self.G = 0.0 if self.newtonian else p.n_p * p.kt_p
        self.noise = bool(p.Brownian) and p.kt > 1e-14

    # -- kernel -----------------------------------------------------------
    def kernel(self, r):
        s = r / self.h
        if self.p.kernel_type == 1:
            s3 = torch.clamp(3.0 - s, min=0.0)
            s2 = torch.clamp(2.0 - s, min=0.0)
            s1 = torch.clamp(1.0 - s, min=0.0)
            w = s3 ** 5 - 6.0 * s2 ** 5 + 15.0 * s1 ** 5
            g = 5.0 * s3 ** 4 - 30.0 * s2 ** 4 + 75.0 * s1 ** 4
            return self.coef * w, -self.coef / self.h * g
        om = torch.clamp(1.0 - s, min=0.0)
        return self.coef * (1.0 + 3.0 * s) * om ** 3, -self.coef / self.h * 12.0 * s * om ** 2

    # -- pieces of the right-hand side ------------------------------------
    def pairs(self, x):
        with torch.no_grad():
            r = x[:, None, :] - x[None, :, :]
            r = r - self.L * torch.round(r / self.L)
            d2 = (r * r).sum(-1)
            n = x.shape[0]
            mask = (d2 < self.rc * self.rc) & ~torch.eye(n, dtype=torch.bool)
            I, J = torch.nonzero(mask, as_tuple=True)
        return I, J

    def pressure(self, nd, c):
        p = self.p
        r_eos = nd * self.m
        if p.stateEquation_type == 1:
            rg = r_eos if p.gamma == 1.0 else r_eos ** p.gamma
            return c * c * (rg - p.rho_ref)
        p0 = c * c * p.rho * (p.rho_ref / p.rho) ** p.gamma / p.gamma
        q = r_eos / p.rho_ref
        return p0 * ((q if p.gamma == 1.0 else q ** p.gamma) - 1.0)

    def rhs(self, x, v, ct, step, dt, eta, c):
        d = self.d
        n = x.shape[0]
        I, J = self.pairs(x)
        r = x[I] - x[J]
        r = r - self.L * torch.round(r / self.L).detach()
        dist = torch.sqrt((r * r).sum(-1))
        W, gw = self.kernel(dist)
        nd = self.w0 + torch.zeros(n, dtype=torch_dtype).index_add(0, I, W)
        p = self.pressure(nd, c)
        B = 1.0 / (nd * nd)
        A = (p + self.G) * B
        u = 1.0 / dist
        e = r * u[:, None]
        vij = v[I] - v[J]
        f_c = (A[I] + A[J]) * gw
        f_d = eta * (B[I] + B[J]) * gw * u
        g = f_d[:, None] * vij - f_c[:, None] * e
        if not self.newtonian:
            Q = self.G * ct * B[:, None, None]
            P = Q[I] + Q[J]
            g = g + (gw * u)[:, None] * torch.einsum("kab,ka->kb", P, r)
        if self.noise:
            # We = s (ca (e.g) e + cb (g - (e.g) e)) with the pair's first d
            # normals g and s = +1 if pid_i < pid_j (the oracle's pair_we)
            pi_, pj_ = self.pid[I.numpy()], self.pid[J.numpy()]
            z = pair_normals_batch(self.p.seed, step, pi_, pj_, d)
            gz = torch.as_tensor(z[:, :d].astype(np.float64))
            sg = torch.as_tensor(np.where(pi_ < pj_, 1.0, -1.0))
            cb = 0.70710678118654752440
            ca = 0.81649658092772603273 if d == 3 else cb
            eg = (e * gz).sum(-1)
            We = sg[:, None] * ((ca - cb) * eg[:, None] * e + cb * gz)
            f_r = torch.sqrt(-4.0 * self.p.kt * f_d) / math.sqrt(dt)
            g = g + f_r[:, None] * We
        a = torch.zeros(n, d, dtype=torch_dtype).index_add(0, I, g / self.m[I][:, None])
        # stress S[b, a] = sum over ordered pairs r_a g_b / (2 m_i)
        S = torch.einsum("ka,kb->ba", r, g / (2.0 * self.m[I])[:, None])
        # body force
        bf = self.p.body_force
        t = self.p.body_force_type
        if t == 1:
            add = torch.tensor([bf[q] if abs(bf[q]) > 1e-14 else 0.0 for q in range(d)],
                               dtype=torch_dtype)
            a = a + add
        elif t == 2 and abs(bf[0]) > 1e-14:
            half = self.p.max_phys[d - 1] * 0.5
            y = x[:, d - 1].detach()
            sgn = torch.where(y < half, 1.0, torch.where(y > half, -1.0, 0.0)).to(torch_dtype)
            a = a + torch.stack([sgn * bf[0]] + [torch.zeros(n, dtype=torch_dtype)] * (d - 1), 1)
        elif t == 3 and abs(bf[0]) > 1e-14:
            kw = 2.0 * math.pi / (self.p.max_phys[1] - self.p.min_phys[1])
            gx = bf[0] * torch.sin(kw * x[:, 1])
            a = a + torch.stack([gx] + [torch.zeros(n, dtype=torch_dtype)] * (d - 1), 1)
        L = None
        if not self.newtonian:
            fac = gw * u / nd[I]
            L = torch.zeros(n, d, d, dtype=torch_dtype).index_add(
                0, I, torch.einsum("ka,kb->kab", -vij, r) * fac[:, None, None])
        return a, L, S, nd, p

    def act(self, ct, L, tau):
        eye = torch.eye(self.d, dtype=torch_dtype)
        return ct @ L.transpose(1, 2) + L @ ct - (ct - eye) / tau

    def wrap(self, x):
        x = torch.where(x >= self.xmax, x - self.L, x)
        return torch.where(x < self.xmin, x + self.L, x)

    # -- trajectory ----------------------------------------------------------
    def run(self, step0, nsteps, dt, w, eta, tau, c, x0=None, v0=None, ct0=None):
        """J = mean_{t=1..T} sum_q w[q] S_t[q] (q = b*d + a as the stress layout)."""
        d = self.d
        x = self.wrap(self.x0 if x0 is None else x0)
        v = self.v0 if v0 is None else v0
        ct = self.ct0 if ct0 is None else ct0
        wt = torch.as_tensor(np.asarray(w, np.float64)[: d * d]).reshape(d, d)  # [b, a]
        a, L, S, _, _ = self.rhs(x, v, ct, step0, dt, eta, c)
        act = self.act(ct, L, tau) if not self.newtonian else None
        J = torch.zeros((), dtype=torch_dtype)
        for t in range(1, nsteps + 1):
            vh = v + 0.5 * dt * a
            x = self.wrap(x + dt * vh)
            if act is not None:
                ct = ct + 0.5 * dt * act
            a, L, S, _, _ = self.rhs(x, vh, ct, step0 + t, dt, eta, c)
            J = J + (wt * S).sum()
            if not self.newtonian:
                act = self.act(ct, L, tau)
                ct = ct + 0.5 * dt * act
            v = vh + 0.5 * dt * a
        self.final = (x, v, ct)
        return J / nsteps


def reference_gradient(params, x, v, m, pid, ct, step0, nsteps, dt, w, state_grads=False):
    """(J, dJ/d(eta, tau, c)[, dict of dJ/dx0, dJ/dv0, dJ/dct0]) by autograd."""
    tr = RefTrajectory(params, x, v, m, pid, ct)
    eta = torch.tensor(params.eta, dtype=torch_dtype, requires_grad=True)
    tau = torch.tensor(params.tau if params.tau > 0 else 1.0, dtype=torch_dtype,
                       requires_grad=True)
    c = torch.tensor(params.c, dtype=torch_dtype, requires_grad=True)
    x0 = tr.x0.clone().requires_grad_(state_grads)
    v0 = tr.v0.clone().requires_grad_(state_grads)
    ct0 = tr.ct0.clone().requires_grad_(state_grads and not tr.newtonian)
    J = tr.run(step0, nsteps, dt, w, eta, tau, c, x0, v0, ct0)
    inputs = [eta, tau, c]
    if state_grads:
        inputs += [x0, v0] + ([ct0] if not tr.newtonian else [])
    grads = torch.autograd.grad(J, inputs, allow_unused=True)
    g = np.array([0.0 if q is None else float(q) for q in grads[:3]])
    if params.Newtonian:
        g[1] = 0.0
    if not state_grads:
        return float(J.detach()), g
    out = {"x": grads[3].numpy(), "v": grads[4].numpy()}
    if not tr.newtonian:
        d = tr.d
        out["ct"] = grads[5].transpose(1, 2).reshape(-1, d * d).numpy()
    return float(J.detach()), g, out
