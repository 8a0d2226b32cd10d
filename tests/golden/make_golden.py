"""Generate / load the regression fixtures of the oracle (tests/golden/*.npz).

Run `python -m tests.golden.make_golden` to regenerate.  The reference (MCF)
ships no golden vectors and cannot be built here, so these fixtures pin the
oracle against its own past outputs; the analytic checks in
tests/test_oracle.py pin it against MCF's formulas.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from mcf_gb300 import configs  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402

CASES = ("c1_small", "c2_small", "walls_small", "le_small", "couette_osc_small")

# steps after which a case's state is dumped
STEPS = {"c1_small": (1, 5, 10, 100), "c2_small": (1, 5, 10, 100)}

# boundary motion of a case: (shear_type[6], shear_freq[6], time_current)
MOTION = {
    "le_small": ((0,) * 6, (0.0,) * 6, 2.7),
    "couette_osc_small": ((0, 0, 0, 2, 0, 0), (0.0, 0.0, 0.0, 2 * np.pi / 0.02, 0.0, 0.0), 0.013),
}


def motion(name: str):
    return MOTION.get(name)


def workload(name: str) -> configs.Workload:
    if name == "c1_small":
        w = configs.c1_poiseuille_2d(n_side=16)
        rng = np.random.default_rng(11)
        w.x = w.x + rng.uniform(-0.05, 0.05, w.x.shape) / 16
        w.v = rng.normal(0, 1e-3, w.v.shape)
        return w
    if name == "c2_small":
        return configs.c2_fluctuating_3d(n_side=10)
    if name == "walls_small":
        w = configs.c3_poiseuille_3d(n_side=10)
        rng = np.random.default_rng(12)
        fl = w.id[:, 1] == 0
        w.v[fl] = rng.normal(0, 1e-2, (int(fl.sum()), 3))
        return w
    if name == "le_small":
        w = configs.lees_edwards(dim=3, n_side=14, shear_rate=0.3)
        rng = np.random.default_rng(13)
        w.x = np.mod(w.x + rng.uniform(-0.3, 0.3, w.x.shape), 14.0)
        return w
    if name == "couette_osc_small":
        w = configs.couette_walls(dim=2, n_side=16, v_top=0.1)
        rng = np.random.default_rng(14)
        fl = w.id[:, 1] == 0
        w.v[fl] = rng.normal(0, 1e-2, (int(fl.sum()), 2))
        return w
    raise KeyError(name)


def compute(name: str) -> dict:
    w = workload(name)
    o = Oracle(w.params)
    if motion(name):
        o.set_boundary_motion(*motion(name))
    o.upload(w.x, w.v, w.m, w.id)
    o.marching_init_force(0)
    ncd, cs, lp = o.technique_build_list()
    out = {"num_cell_dim": ncd, "cell_start": cs, "lpdx": lp}
    d0 = o.download("rho", "p", "f")
    out.update({"rho0": d0["rho"], "p0": d0["p"], "f0": d0["f"]})
    # per-stage dumps after steps 1, 5, 10 and 100 for the two base
    # workloads (C1, C2), after step 5 for the others
    marks = STEPS.get(name, (5,))
    done = 0
    for t in marks:
        o.run_vv(done, t - done, w.dt)
        done = t
        d1 = o.download("x", "v", "rho", "f")
        out.update({f"x{t}": d1["x"], f"v{t}": d1["v"], f"rho{t}": d1["rho"], f"f{t}": d1["f"]})
    return out


def load_all() -> dict:
    res = {}
    for name in CASES:
        with np.load(HERE / f"{name}.npz") as z:
            res[name] = {k: z[k] for k in z.files}
    return res


if __name__ == "__main__":
    for name in CASES:
        np.savez_compressed(HERE / f"{name}.npz", **compute(name))
        print("wrote", name)
