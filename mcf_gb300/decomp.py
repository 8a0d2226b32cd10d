"""x-slab domain decomposition of one SDPD box over several subdomains.

MCF decomposes space over its MPI ranks with PPM: every step it migrates
the particles that left a processor's subdomain
(particles_decompose_partial.F90:216-334, called at
marching_integrate_VV.F90:849-856) and fetches ghost copies of the
neighbours' particles within the cut-off (particles_map_ghost_get.F90:
310-524; with symmetry = T it also puts the ghosts' partial sums back,
particles_map_ghost_put.F90:274-330).  Here the subdomains are slabs along
x of a box that is periodic along x; each slab runs its own handle (an
SDPD object on its own GPU, or any object with MCF's routine names, such
as the CPU oracle) on the slab widened by a halo of one cell side on both
x faces, which are freespace faces (no images, no wall particles).  The
GPU sweeps gather every pair from both of its particles (MCF's
symmetry = F), so a subdomain computes its own particles' densities and
forces and needs two ghost gets a step and no ghost put:

  1. half kick and drift (particles_integrate_velocity / _position);
  2. migration: owned particles that left the slab go to the neighbour that
     owns them now (positions wrapped across the periodic x face);
  3. ghost get 1: owned particles within the halo width of a slab face go,
     with x v m id, to the neighbour across that face (shifted by L_x
     across the periodic face); every subdomain then holds owned + ghost
     particles (mcfg_upload);
  4. cell list and density (ghost densities are incomplete);
  5. ghost get 2: the halo particles' densities from their owners
     (mcfg_update_density), in the order of ghost get 1;
  6. pressure, pair force, body force, half kick.

Statistics (kinetic energy, momentum, stress) are summed per subdomain over
its own particles (mcfg_statistics_owned) and all-reduced over the
subdomains, as MCF sums per rank and calls MPI_ALLREDUCE.

Owned particles' densities and forces are sums over the same partners as
in the undivided box (to summation order); the Wiener increments are keyed
by the particle ids, so the decomposed run follows the undivided one to
rounding.  The transport moves host arrays: torch.distributed point-to-point
messages between processes (gloo on CPU; NCCL where the halos stay on the
GPU would replace it), or in-process exchange between subdomains of one
process.  No TMA or multicast of peer memory is involved.

Limits: slabs along x only (the box must be periodic along x; y and z may
have solid walls), the fixed time step params.dt (which the stage routines
give the random force), no colloids, no Lees-Edwards faces, no moving
walls, no Oldroyd-B model.
"""
from __future__ import annotations

import numpy as np

from .params import BC_FREESPACE, BC_PERIODIC, SDPDParams


class LocalExchange:
    """Message passing between the subdomains of one process."""

    def exchange(self, outbox):
        """outbox[r] = {'left': dict, 'right': dict}: messages of subdomain r
        for its left and right neighbours.  Returns inbox[r] = {'left': the
        message from the left neighbour, 'right': from the right}."""
        n = len(outbox)
        return [{"left": outbox[(r - 1) % n]["right"], "right": outbox[(r + 1) % n]["left"]}
                for r in range(n)]

    def allreduce(self, vec):
        """sum over all subdomains: they are all in this process already"""
        return np.asarray(vec, np.float64)


class TorchExchange:
    """Point-to-point messages between processes with torch.distributed
    (one subdomain per rank, neighbours rank-1 and rank+1 around the ring):
    the per-key counts travel first, then the arrays as tensors."""

    KEYS = ("x", "v", "m", "id", "rho")

    def __init__(self, dim: int):
        import torch.distributed as dist

        self.dist = dist
        self.dim = dim
        self.rank = dist.get_rank()
        self.size = dist.get_world_size()

    def _shape(self, key, count):
        if key in ("x", "v"):
            return (count, self.dim)
        if key == "id":
            return (count, 2)
        return (count,)

    def _send_recv(self, out, to, frm):
        import torch

        dist = self.dist
        hdr = torch.tensor([out[k].shape[0] if k in out else -1 for k in self.KEYS],
                           dtype=torch.int64)
        hin = torch.empty_like(hdr)
        for r in (dist.isend(hdr, to), dist.irecv(hin, frm)):
            r.wait()
        send = [torch.from_numpy(np.ascontiguousarray(out[k])) for k in self.KEYS if k in out]
        recv = {}
        for q, k in enumerate(self.KEYS):
            c = int(hin[q])
            if c >= 0:
                recv[k] = torch.empty(self._shape(k, c),
                                      dtype=torch.int32 if k == "id" else torch.float64)
        reqs = [dist.isend(t, to) for t in send] + [dist.irecv(t, frm) for t in recv.values()]
        for r in reqs:
            r.wait()
        return {k: t.numpy() for k, t in recv.items()}

    def exchange(self, outbox):
        (box,) = outbox
        left, right = (self.rank - 1) % self.size, (self.rank + 1) % self.size
        # to the right neighbour / from the left one, then the other way
        from_left = self._send_recv(box["right"], right, left)
        from_right = self._send_recv(box["left"], left, right)
        return [{"left": from_left, "right": from_right}]

    def allreduce(self, vec):
        """sum of the ranks' FP64 vectors (MCF's MPI_ALLREDUCE of the
        statistic sums, statistic_compute_statistic.F90:348-403)"""
        import torch

        t = torch.from_numpy(np.array(vec, np.float64))
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return t.numpy()


class Subdomain:
    """One slab [x_lo, x_hi) and its handle."""

    def __init__(self, factory, params: SDPDParams, index: int, x_lo: float, x_hi: float,
                 halo: float):
        self.index = index
        self.x_lo, self.x_hi, self.halo = x_lo, x_hi, halo
        p = params.copy()
        p.min_phys_t[0] = p.min_phys[0] = x_lo - halo
        p.max_phys_t[0] = p.max_phys[0] = x_hi + halo
        p.bcdef[0] = p.bcdef[1] = BC_FREESPACE
        self.params = p
        self.h = factory(p)
        self.d = int(p.num_dim)
        # owned particles (host copies between the phases of a step)
        self.x = self.v = self.m = self.id = None
        self.n_own = 0
        self.sent = {}

    def owned(self, x, v, m, id_):
        self.x, self.v, self.m, self.id = x, v, m, id_
        self.n_own = int(m.shape[0])


class SlabDecomposition:
    """An SDPD box decomposed into slabs along x.

    factory(params) -> handle with MCF's routine names (mcf_gb300.SDPD or
    oracle.Oracle).  nslab slabs in all; this process runs the slabs in
    `mine` (all of them with LocalExchange, its own rank with
    TorchExchange)."""

    def __init__(self, params: SDPDParams, nslab: int, factory, exchange=None, mine=None):
        d = int(params.num_dim)
        if params.bcdef[0] != BC_PERIODIC or params.bcdef[1] != BC_PERIODIC:
            raise ValueError("slab decomposition: the box must be periodic along x")
        if params.bcdef[2] == 10 or params.Newtonian == 0:
            raise ValueError("slab decomposition: no Lees-Edwards faces, Newtonian fluid only")
        self.params = params.copy()
        self.d = d
        self.nslab = nslab
        lo, hi = params.min_phys_t[0], params.max_phys_t[0]
        self.L = hi - lo
        self.bounds = [lo + self.L * r / nslab for r in range(nslab + 1)]
        cf = params.cell_factor if params.cell_factor > 0 else 1.0001
        self.halo = params.cut_off * cf
        if min(b - a for a, b in zip(self.bounds, self.bounds[1:])) < self.halo:
            raise ValueError("slab decomposition: a slab is narrower than the halo")
        self.exchange = exchange or LocalExchange()
        self.mine = list(range(nslab)) if mine is None else list(mine)
        self.subs = [Subdomain(factory, params, r, self.bounds[r], self.bounds[r + 1], self.halo)
                     for r in self.mine]
        self.step_count = 0
        self.migrated = 0  # particles handed to a neighbour so far (this process)

    # -- set-up ----------------------------------------------------------------
    def upload(self, x, v, m, id_):
        """global arrays (host order); every slab keeps the particles it owns"""
        x = np.asarray(x, np.float64).reshape(-1, self.d)
        v = np.asarray(v, np.float64).reshape(-1, self.d)
        m = np.asarray(m, np.float64)
        id_ = np.asarray(id_, np.int32).reshape(-1, 2)
        xs = self.params.min_phys_t[0] + np.mod(x[:, 0] - self.params.min_phys_t[0], self.L)
        x = x.copy()
        x[:, 0] = xs
        for s in self.subs:
            sel = (xs >= s.x_lo) & (xs < s.x_hi)
            s.owned(x[sel].copy(), v[sel].copy(), m[sel].copy(), id_[sel].copy())

    # -- the two ghost gets ------------------------------------------------------
    def _band(self, s, side):
        """owned particles within the halo width of face `side` of slab s"""
        if side == "left":
            return np.nonzero(s.x[:, 0] < s.x_lo + s.halo)[0]
        return np.nonzero(s.x[:, 0] >= s.x_hi - s.halo)[0]

    def _shift(self, s, side):
        """x shift of a message crossing face `side` of slab s (periodic)"""
        r = s.index
        if side == "left" and r == 0:
            return self.L
        if side == "right" and r == self.nslab - 1:
            return -self.L
        return 0.0

    def _ghost_get_1(self):
        outbox = []
        for s in self.subs:
            box = {}
            for side in ("left", "right"):
                idx = self._band(s, side)
                s.sent[side] = idx
                xg = s.x[idx].copy()
                xg[:, 0] += self._shift(s, side)
                box[side] = {"x": xg, "v": s.v[idx], "m": s.m[idx], "id": s.id[idx]}
            outbox.append(box)
        return self.exchange.exchange(outbox)

    def _migrate(self):
        outbox = []
        for s in self.subs:
            box = {}
            xs = s.x[:, 0]
            for side, sel in (("left", xs < s.x_lo), ("right", xs >= s.x_hi)):
                xm = s.x[sel].copy()
                xm[:, 0] += self._shift(s, side)
                box[side] = {"x": xm, "v": s.v[sel], "m": s.m[sel], "id": s.id[sel]}
            keep = (xs >= s.x_lo) & (xs < s.x_hi)
            self.migrated += int((~keep).sum())
            s.owned(s.x[keep], s.v[keep], s.m[keep], s.id[keep])
            outbox.append(box)
        inbox = self.exchange.exchange(outbox)
        for s, ib in zip(self.subs, inbox):
            parts = [(s.x, s.v, s.m, s.id)] + [(ib[k]["x"], ib[k]["v"], ib[k]["m"], ib[k]["id"])
                                              for k in ("left", "right")]
            s.owned(*[np.concatenate([p[q] for p in parts]) for q in range(4)])

    # -- the step ----------------------------------------------------------------
    def _rhs(self, step):
        """ghost get 1, upload, list, density, ghost get 2, pressure, force"""
        inbox = self._ghost_get_1()
        for s, ib in zip(self.subs, inbox):
            g = [ib[k] for k in ("left", "right")]
            s.n_ghost = [int(q["m"].shape[0]) for q in g]
            xa = np.concatenate([s.x] + [q["x"] for q in g])
            va = np.concatenate([s.v] + [q["v"] for q in g])
            ma = np.concatenate([s.m] + [q["m"] for q in g])
            ia = np.concatenate([s.id] + [q["id"] for q in g])
            s.h.upload(xa, va, ma, ia)
            s.h.particles_adjust_particles()  # periodic wrap along y, z
            s.h.technique_build_list(want_lists=False)
            s.h.particles_compute_density()
            s.rho = s.h.download("rho")["rho"]
        outbox = [{side: {"rho": s.rho[:s.n_own][s.sent[side]]} for side in ("left", "right")}
                  for s in self.subs]
        inbox = self.exchange.exchange(outbox)
        for s, ib in zip(self.subs, inbox):
            rho = s.rho.copy()
            a = s.n_own
            rho[a:a + s.n_ghost[0]] = ib["left"]["rho"]
            rho[a + s.n_ghost[0]:] = ib["right"]["rho"]
            s.h.update_density(rho)
            s.h.particles_compute_pressure()
            s.h.particles_compute_interaction(step)
            s.h.particles_apply_body_force()

    def init_force(self, step=0):
        """the right-hand side before the first step (marching_marching.F90)"""
        self._rhs(step)

    def step_vv(self, step, dt):
        """one VV step of every slab of this process; dt must be params.dt,
        the time step the stage routines give the random force"""
        if dt != self.params.dt:
            raise ValueError("slab decomposition: dt must equal params.dt (the random force's)")
        for s in self.subs:
            s.h.particles_integrate_velocity(dt, 0.5)
            s.h.particles_integrate_position(dt)
            st = s.h.download("x", "v")
            s.owned(st["x"][:s.n_own].copy(), st["v"][:s.n_own].copy(), s.m, s.id)
        self._migrate()
        self._rhs(step)
        for s in self.subs:
            s.h.particles_integrate_velocity(dt, 0.5)
            st = s.h.download("x", "v")
            s.owned(st["x"][:s.n_own].copy(), st["v"][:s.n_own].copy(), s.m, s.id)
        self.step_count += 1

    def run_vv(self, step0, nsteps, dt):
        for k in range(1, nsteps + 1):
            self.step_vv(step0 + k, dt)

    def statistics(self):
        """kinetic energy, momentum[3] and stress[9] of the whole box
        (statistic_compute_statistic.F90:230-303): every subdomain sums its
        own particles (its ghosts left out), then the sums are all-reduced
        over the subdomains (:348-403)."""
        loc = np.zeros(13)
        for s in self.subs:
            ke, mom, st = s.h.statistic_compute_statistic(n_owned=s.n_own)
            loc += np.concatenate([[ke], mom, st])
        tot = self.exchange.allreduce(loc)
        return float(tot[0]), tot[1:4].copy(), tot[4:13].copy()

    # -- results -----------------------------------------------------------------
    def owned_state(self, fields=("x", "v", "rho", "f")):
        """per local slab: ids and the owned particles' fields"""
        out = []
        for s in self.subs:
            st = s.h.download(*fields)
            out.append({"id": s.id.copy(), **{k: st[k][:s.n_own].copy() for k in fields}})
        return out
