"""ctypes wrapper of the CPU oracle (oracle/_lib/liborc.so).

TEST INFRASTRUCTURE ONLY.  The oracle restates MCF's Fortran SDPD step in C
(see mcf_oracle.c for the per-routine citations).  Only tests/, the smoke
check of __graft_entry__ and the CPU-baseline leg of bench.py use it; the
product path (mcf_gb300) never imports this module.

Parity status: parity unpinned against outputs of the reference itself (MCF
cannot be built here and ships no golden vectors); pinned by analytic checks
and committed fixtures instead (tests/golden).
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

from mcf_gb300.params import ColloidDynamics, ColloidParams, SDPDParams  # noqa: E402  (layouts only)

from . import build as _build  # noqa: E402

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_h = C.c_void_p
_LIB = None


def load(rebuild: bool = True) -> C.CDLL:
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.build() if rebuild else _build.OUT
    lib = C.CDLL(str(path))
    sig = {
        "orc_create": (_h, [C.POINTER(SDPDParams), C.c_char_p, C.c_int]),
        "orc_destroy": (None, [_h]),
        "orc_last_error": (C.c_char_p, [_h]),
        "orc_set_threads": (C.c_int, [_h, C.c_int]),
        "orc_upload": (C.c_int, [_h, C.c_int64, _dp, _dp, _dp, _ip, _dp]),
        "orc_adjust_particles": (C.c_int, [_h]),
        "orc_build_list": (C.c_int, [_h]),
        "orc_export_lists": (C.c_int, [_h, _ip, _ip, _ip]),
        "orc_compute_density": (C.c_int, [_h]),
        "orc_compute_pressure": (C.c_int, [_h]),
        "orc_update_density": (C.c_int, [_h, _dp]),
        "orc_compute_interaction": (C.c_int, [_h, C.c_int64]),
        "orc_apply_body_force": (C.c_int, [_h]),
        "orc_integrate_velocity": (C.c_int, [_h, C.c_double, C.c_double]),
        "orc_integrate_position": (C.c_int, [_h, C.c_double]),
        "orc_init_force": (C.c_int, [_h, C.c_int64]),
        "orc_step_vv": (C.c_int, [_h, C.c_int64, C.c_double]),
        "orc_run_vv": (C.c_int, [_h, C.c_int64, C.c_int32, C.c_double]),
        "orc_set_boundary_motion": (C.c_int, [_h, C.POINTER(C.c_int32), _dp, C.c_double]),
        "orc_time": (C.c_double, [_h]),
        "orc_download": (C.c_int, [_h, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
        "orc_statistics": (C.c_int, [_h, _dp, _dp, _dp]),
        "orc_statistics_owned": (C.c_int, [_h, C.c_int64, _dp, _dp, _dp]),
        "orc_counts": (C.c_int, [_h, C.POINTER(C.c_int64)]),
        "orc_force_scale": (C.c_int, [_h, _dp]),
        "orc_timers": (C.c_int, [_h, _dp]),
        "orc_lattice": (C.c_int64, [C.c_int, _dp, _dp, _dp, _dp, C.c_int64]),
        "orc_philox4x32_10": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                     C.POINTER(C.c_uint32)]),
        "orc_pair_normals": (None, [C.c_uint64, C.c_int64, C.c_int32, C.c_int32, C.c_int,
                                    C.POINTER(C.c_float)]),
        "orc_pair_normals_batch": (None, [C.c_uint64, C.c_int64, C.c_int64,
                                          C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int,
                                          C.POINTER(C.c_float)]),
        "orc_kernel": (C.c_int, [_h, C.c_double, _dp, _dp]),
        "orc_pair_we": (C.c_int, [_h, C.c_int64, C.c_int32, C.c_int32, _dp, _dp]),
        "orc_set_colloids": (C.c_int, [_h, C.POINTER(ColloidParams), _dp, _dp, _dp, _dp]),
        "orc_colloid_drag": (C.c_int, [_h, _dp, _dp]),
        "orc_move_colloids": (C.c_int, [_h, _dp, _dp, _dp, _dp]),
        "orc_colloid_repulsion": (C.c_int, [_h, _dp]),
        "orc_set_colloid_dynamics": (C.c_int, [_h, C.POINTER(ColloidDynamics), _dp, _dp, _dp, _dp,
                                               _dp, _dp, _dp, _dp]),
        "orc_colloid_integrate": (C.c_int, [_h, C.c_int64, C.c_double]),
        "orc_get_colloid_state": (C.c_int, [_h, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                            _dp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


class OracleError(RuntimeError):
    pass


class Oracle:
    """CPU FP64 restatement with the same routine names as mcf_gb300.SDPD."""

    def __init__(self, params: SDPDParams, threads: int = 1):
        self.lib = load()
        self.params = params.copy()
        self.dim = int(params.num_dim)
        err = C.create_string_buffer(256)
        h = self.lib.orc_create(C.byref(self.params), err, 256)
        if not h:
            raise OracleError(err.value.decode())
        self._h = h
        self.n = 0
        self.lib.orc_set_threads(h, int(threads))

    def _check(self, name, rc):
        if rc != 0:
            raise OracleError(f"{name}: {self.lib.orc_last_error(self._h).decode()}")

    def close(self):
        if getattr(self, "_h", None):
            self.lib.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def sid(self) -> np.ndarray:
        """species id of each uploaded particle (host order)"""
        return self._id[:, 1]

    def set_threads(self, n: int):
        self.lib.orc_set_threads(self._h, int(n))

    def upload(self, x, v, m, id_, ct=None):
        n = int(np.asarray(m).shape[0])
        d = self.dim
        self._x = np.ascontiguousarray(x, np.float64).reshape(n, d)
        self._v = np.ascontiguousarray(v, np.float64).reshape(n, d)
        self._m = np.ascontiguousarray(m, np.float64).reshape(n)
        self._id = np.ascontiguousarray(id_, np.int32).reshape(n, 2)
        ctp = None if ct is None else np.ascontiguousarray(ct, np.float64)
        self._check("orc_upload", self.lib.orc_upload(self._h, n, _ptr(self._x, C.c_double),
                                                      _ptr(self._v, C.c_double),
                                                      _ptr(self._m, C.c_double),
                                                      _ptr(self._id, C.c_int32),
                                                      _ptr(ctp, C.c_double)))
        self.n = n

    def download(self, *fields):
        n, d = self.n, self.dim
        shapes = {"x": (n, d), "v": (n, d), "rho": (n,), "p": (n,), "f": (n, d), "s": (n, d * d),
                  "ct": (n, d * d)}
        out = {k: np.empty(shapes[k], np.float64) for k in fields}
        g = lambda k: _ptr(out.get(k), C.c_double)  # noqa: E731
        self._check("orc_download",
                    self.lib.orc_download(self._h, g("x"), g("v"), g("rho"), g("p"), g("f"),
                                          g("ct"), g("s")))
        return out

    def particles_adjust_particles(self):
        self._check("adjust", self.lib.orc_adjust_particles(self._h))

    def technique_build_list(self, want_lists: bool = True):
        self._check("build_list", self.lib.orc_build_list(self._h))
        if not want_lists:
            return None
        ncd = np.zeros(3, np.int32)
        self._check("export", self.lib.orc_export_lists(self._h, _ptr(ncd, C.c_int32), None, None))
        ncell = int(np.prod(ncd))
        cs = np.empty(ncell + 1, np.int32)
        lp = np.empty(max(self.n, 1), np.int32)
        self._check("export", self.lib.orc_export_lists(self._h, _ptr(ncd, C.c_int32),
                                                        _ptr(cs, C.c_int32), _ptr(lp, C.c_int32)))
        return ncd, cs, lp[: int(cs[-1])]

    def particles_compute_density(self):
        self._check("density", self.lib.orc_compute_density(self._h))

    def update_density(self, rho):
        r = np.ascontiguousarray(rho, np.float64).reshape(self.n)
        self._check("update_density", self.lib.orc_update_density(self._h, _ptr(r, C.c_double)))

    def particles_compute_pressure(self):
        self._check("pressure", self.lib.orc_compute_pressure(self._h))

    def particles_compute_interaction(self, step: int = 0):
        self._check("interaction", self.lib.orc_compute_interaction(self._h, int(step)))

    def particles_apply_body_force(self):
        self._check("body_force", self.lib.orc_apply_body_force(self._h))

    def particles_integrate_velocity(self, dt, lam):
        self._check("integrate_velocity", self.lib.orc_integrate_velocity(self._h, dt, lam))

    def particles_integrate_position(self, dt):
        self._check("integrate_position", self.lib.orc_integrate_position(self._h, dt))

    def marching_init_force(self, step: int = 0):
        self._check("init_force", self.lib.orc_init_force(self._h, int(step)))

    def marching_integrate_VV(self, step, dt):
        self._check("step_vv", self.lib.orc_step_vv(self._h, int(step), float(dt)))

    def run_vv(self, step0, nsteps, dt):
        self._check("run_vv", self.lib.orc_run_vv(self._h, int(step0), int(nsteps), float(dt)))

    def set_boundary_motion(self, shear_type, shear_freq, time: float = 0.0):
        st = np.ascontiguousarray(shear_type, dtype=np.int32).reshape(6)
        sf = np.ascontiguousarray(shear_freq, dtype=np.float64).reshape(6)
        self._check("orc_set_boundary_motion",
                    self.lib.orc_set_boundary_motion(self._h, _ptr(st, C.c_int32),
                                                     _ptr(sf, C.c_double), float(time)))

    @property
    def time(self) -> float:
        return float(self.lib.orc_time(self._h))

    def statistic_compute_statistic(self, n_owned=None):
        """kinetic energy, momentum[3], stress[9]; with n_owned, over the first
        n_owned particles only (a subdomain's own, its ghosts left out)"""
        ke = C.c_double()
        mom = np.zeros(3)
        st = np.zeros(9)
        if n_owned is None:
            rc = self.lib.orc_statistics(self._h, C.byref(ke), _ptr(mom, C.c_double),
                                         _ptr(st, C.c_double))
        else:
            rc = self.lib.orc_statistics_owned(self._h, int(n_owned), C.byref(ke),
                                               _ptr(mom, C.c_double), _ptr(st, C.c_double))
        self._check("statistics", rc)
        return ke.value, mom, st

    def force_scale(self) -> np.ndarray:
        out = np.empty(self.n)
        self.lib.orc_force_scale(self._h, _ptr(out, C.c_double))
        return out

    def set_colloids(self, cp, x, v, omega, radius):
        self._cp = cp
        self._cx = np.ascontiguousarray(x, np.float64)
        self._cv = np.ascontiguousarray(v, np.float64)
        self._com = np.ascontiguousarray(omega, np.float64)
        self._crad = np.ascontiguousarray(radius, np.float64)
        self._check("set_colloids", self.lib.orc_set_colloids(
            self._h, C.byref(cp), _ptr(self._cx, C.c_double), _ptr(self._cv, C.c_double),
            _ptr(self._com, C.c_double), _ptr(self._crad, C.c_double)))

    def move_colloids(self, x_new, rot, v, omega):
        self._cx = np.ascontiguousarray(x_new, np.float64)
        self._cv = np.ascontiguousarray(v, np.float64)
        self._com = np.ascontiguousarray(omega, np.float64)
        r = None if rot is None else np.ascontiguousarray(rot, np.float64)
        self._check("move_colloids", self.lib.orc_move_colloids(
            self._h, _ptr(self._cx, C.c_double), _ptr(r, C.c_double),
            _ptr(self._cv, C.c_double), _ptr(self._com, C.c_double)))

    def colloid_drag(self):
        nc = self._cp.num_colloid
        drag = np.zeros((nc, self.dim))
        torque = np.zeros((nc, 3))
        self._check("colloid_drag", self.lib.orc_colloid_drag(self._h, _ptr(drag, C.c_double),
                                                               _ptr(torque, C.c_double)))
        return drag, torque

    def colloid_repulsion(self):
        out = np.zeros((self._cp.num_colloid, self.dim))
        self._check("colloid_repulsion", self.lib.orc_colloid_repulsion(self._h,
                                                                         _ptr(out, C.c_double)))
        return out

    def set_colloid_dynamics(self, cd, mass, mmi, v_hist=None, omega_hist=None, f_hist=None,
                             alpha_hist=None, acc_matrix=None, theta=None):
        self._cd = cd
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64)
                for a in (mass, mmi, v_hist, omega_hist, f_hist, alpha_hist, acc_matrix, theta)]
        self._check("set_colloid_dynamics", self.lib.orc_set_colloid_dynamics(
            self._h, C.byref(cd), *[_ptr(a, C.c_double) for a in arrs]))

    def colloid_integrate(self, step, dt):
        self._check("colloid_integrate", self.lib.orc_colloid_integrate(self._h, int(step),
                                                                         float(dt)))

    def colloid_state(self):
        """x, v, omega, f, alpha histories (level-major), drag, torque,
        rot_matrix, acc_matrix, theta"""
        nc, d, ab = self._cp.num_colloid, self.dim, self._cd.integrate_AB
        out = {"x": np.zeros((nc, d)), "v": np.zeros((ab, nc, d)), "omega": np.zeros((ab, nc, 3)),
               "f": np.zeros((ab, nc, d)), "alpha": np.zeros((ab, nc, 3)),
               "drag": np.zeros((nc, d)), "torque": np.zeros((nc, 3)),
               "rot": np.zeros((nc, 9)), "acc": np.zeros((nc, 9)), "theta": np.zeros((nc, 3))}
        keys = ["x", "v", "omega", "f", "alpha", "drag", "torque", "rot", "acc", "theta"]
        self._check("get_colloid_state", self.lib.orc_get_colloid_state(
            self._h, *[_ptr(out[k], C.c_double) for k in keys]))
        return out

    def pair_we(self, step, pidi, pidj, e):
        e = np.ascontiguousarray(e, np.float64)
        out = np.zeros(3)
        self.lib.orc_pair_we(self._h, int(step), int(pidi), int(pidj), _ptr(e, C.c_double),
                             _ptr(out, C.c_double))
        return out[: self.dim]

    def counts(self):
        c = (C.c_int64 * 3)()
        self.lib.orc_counts(self._h, c)
        return {"real": c[0], "ghost": c[1], "pairs": c[2]}

    def timers(self):
        t = np.zeros(4)
        self.lib.orc_timers(self._h, _ptr(t, C.c_double))
        return {"list": t[0], "density": t[1], "force": t[2], "update": t[3]}

    def kernel(self, r: float):
        w = C.c_double()
        g = C.c_double()
        self.lib.orc_kernel(self._h, float(r), C.byref(w), C.byref(g))
        return w.value, g.value


def pair_normals(seed: int, step: int, pa: int, pb: int, dim: int) -> np.ndarray:
    z = (C.c_float * 6)()
    load().orc_pair_normals(seed, step, pa, pb, dim, z)
    return np.array(z[: (6 if dim == 3 else 3)], dtype=np.float32)


def pair_normals_batch(seed: int, step: int, pa, pb, dim: int) -> np.ndarray:
    """normals of the pairs (pa[k], pb[k]): float32 [npairs, 6]"""
    pa = np.ascontiguousarray(pa, np.int32)
    pb = np.ascontiguousarray(pb, np.int32)
    z = np.zeros((pa.size, 6), np.float32)
    load().orc_pair_normals_batch(seed, step, pa.size, _ptr(pa, C.c_int32), _ptr(pb, C.c_int32),
                                  dim, _ptr(z, C.c_float))
    return z


def philox(ctr, key) -> list[int]:
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    load().orc_philox4x32_10(c, k, o)
    return list(o)
