"""Host-side mirror of MCF's per-step particle interface over libmcfg.so.

The methods carry the names of the Fortran routines they replace
(technique_build_list, particles_compute_density, ...), take MCF's array
layout (x(d,N) stored as an (N, d) C-contiguous array, id(2,N) as (N, 2)
int32) and report failures the way MCF's `stat_info` does, as an exception
naming the routine.  There is no CPU fallback: if libmcfg.so cannot be
loaded or no GPU is present, construction fails.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .params import STATUS_NAMES, ColloidDynamics, ColloidParams, SDPDInfo, SDPDParams

_LIB = None
LIB_PATH = Path(__file__).resolve().parent / "libmcfg.so"

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_h = C.c_void_p


class MCFGError(RuntimeError):
    """A libmcfg call returned a non-zero status."""

    def __init__(self, routine: str, code: int, message: str):
        self.routine = routine
        self.code = code
        super().__init__(f"{routine} : {message} ({STATUS_NAMES.get(code, code)})")


def load_library(path: Path | str | None = None) -> C.CDLL:
    """Load libmcfg.so and declare the C-ABI prototypes (include/mcfg.h)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} not found: build it with `python -m mcf_gb300.build`")
    lib = C.CDLL(str(p))
    sig = {
        "mcfg_sizeof_params": (C.c_int64, []),
        "mcfg_create": (C.c_int, [C.POINTER(SDPDParams), C.POINTER(_h)]),
        "mcfg_destroy": (C.c_int, [_h]),
        "mcfg_last_error": (C.c_char_p, [_h]),
        "mcfg_create_error": (C.c_char_p, []),
        "mcfg_get_info": (C.c_int, [_h, C.POINTER(SDPDInfo)]),
        "mcfg_upload": (C.c_int, [_h, C.c_int64, _dp, _dp, _dp, _ip, _dp]),
        "mcfg_adjust_particles": (C.c_int, [_h]),
        "mcfg_build_list": (C.c_int, [_h, _ip, _ip, _ip]),
        "mcfg_compute_density": (C.c_int, [_h]),
        "mcfg_compute_pressure": (C.c_int, [_h]),
        "mcfg_update_density": (C.c_int, [_h, _dp]),
        "mcfg_compute_interaction": (C.c_int, [_h, C.c_int64]),
        "mcfg_apply_body_force": (C.c_int, [_h]),
        "mcfg_integrate_velocity": (C.c_int, [_h, C.c_double, C.c_double]),
        "mcfg_integrate_position": (C.c_int, [_h, C.c_double]),
        "mcfg_init_force": (C.c_int, [_h, C.c_int64]),
        "mcfg_step_vv": (C.c_int, [_h, C.c_int64, C.c_double]),
        "mcfg_run_vv": (C.c_int, [_h, C.c_int64, C.c_int32, C.c_double]),
        "mcfg_step_vv_host": (C.c_int, [_h, C.c_int64, C.c_double, _dp, _dp]),
        "mcfg_update_state": (C.c_int, [_h, _dp, _dp, _dp]),
        "mcfg_adjoint_run": (C.c_int, [_h, C.c_int64, C.c_int32, C.c_double, C.c_int32, _dp, _dp,
                                       _dp, _dp, _dp, _dp]),
        "mcfg_download": (C.c_int, [_h, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
        "mcfg_statistics": (C.c_int, [_h, _dp, _dp, _dp]),
        "mcfg_statistics_owned": (C.c_int, [_h, C.c_int64, _dp, _dp, _dp]),
        "mcfg_synchronize": (C.c_int, [_h]),
        "mcfg_upload_force": (C.c_int, [_h, _dp]),
        "mcfg_get_stream": (C.c_void_p, [_h]),
        "mcfg_set_profiling": (C.c_int, [_h, C.c_int]),
        "mcfg_get_phase_times": (C.c_int, [_h, _dp, C.POINTER(C.c_int64)]),
        "mcfg_density_noalloc": (C.c_int, [C.POINTER(SDPDParams), C.c_int32, C.c_int32,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p]),
        "mcfg_noalloc_status": (C.c_int, [C.c_int32, C.c_void_p, C.POINTER(C.c_int32)]),
        "mcfg_noalloc_error": (C.c_char_p, []),
        "mcfg_set_colloids": (C.c_int, [_h, C.POINTER(ColloidParams), _dp, _dp, _dp, _dp]),
        "mcfg_colloid_drag": (C.c_int, [_h, _dp, _dp]),
        "mcfg_move_colloids": (C.c_int, [_h, _dp, _dp, _dp, _dp]),
        "mcfg_colloid_repulsion": (C.c_int, [_h, _dp]),
        "mcfg_set_colloid_dynamics": (C.c_int, [_h, C.POINTER(ColloidDynamics), _dp, _dp, _dp,
                                                _dp, _dp, _dp, _dp, _dp]),
        "mcfg_colloid_integrate": (C.c_int, [_h, C.c_int64, C.c_double]),
        "mcfg_get_colloid_state": (C.c_int, [_h, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                             _dp, _dp]),
        "mcfg_set_boundary_motion": (C.c_int, [_h, C.POINTER(C.c_int32), _dp, C.c_double]),
        "mcfg_write_particles": (C.c_int, [_h, C.c_char_p, C.c_int32, C.c_int32]),
        "mcfg_write_statistic": (C.c_int, [_h, C.c_char_p, C.c_int64, C.c_double]),
        "mcfg_host_register": (C.c_int, [_h, C.c_void_p, C.c_int64]),
        "mcfg_host_unregister": (C.c_int, [_h, C.c_void_p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.mcfg_sizeof_params() != C.sizeof(SDPDParams):
        raise ImportError("mcfg_params layout mismatch between libmcfg.so and params.py")
    if path is None:
        _LIB = lib
    return lib


def _ptr(a: np.ndarray | None, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def _as(a, dtype, shape=None) -> np.ndarray:
    out = np.ascontiguousarray(a, dtype=dtype)
    if shape is not None and out.shape != shape:
        out = out.reshape(shape)
    return out


class SDPD:
    """One GPU-resident particle system (an MCF Particles object's hot path)."""

    def __init__(self, params: SDPDParams, lib: C.CDLL | None = None):
        self.lib = lib or load_library()
        self.params = params.copy()
        self.dim = int(params.num_dim)
        h = _h()
        rc = self.lib.mcfg_create(C.byref(self.params), C.byref(h))
        if rc != 0:
            raise MCFGError("mcfg_create", rc, self.lib.mcfg_create_error().decode())
        self._h = h
        self.n = 0

    # -- bookkeeping -------------------------------------------------------
    def _check(self, routine: str, rc: int) -> None:
        if rc != 0:
            raise MCFGError(routine, rc, self.lib.mcfg_last_error(self._h).decode())

    def close(self) -> None:
        if getattr(self, "_h", None):
            self.lib.mcfg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def info(self) -> dict:
        inf = SDPDInfo()
        self._check("mcfg_get_info", self.lib.mcfg_get_info(self._h, C.byref(inf)))
        return {
            "num_part": inf.num_part,
            "num_cell_dim": tuple(inf.num_cell_dim),
            "num_cell": inf.num_cell,
            "num_outside": inf.num_outside,
            "num_pairs": inf.num_pairs,
            "max_neigh": inf.max_neigh,
            "neigh_capacity": inf.neigh_capacity,
            "kernel_launches": inf.kernel_launches,
            "device_bytes": inf.device_bytes,
            "list_rebuilds": inf.list_rebuilds,
            "skin": inf.skin,
            "time_current": inf.time_current,
            "shear_length": inf.shear_length,
        }

    def write_particles(self, path, kind: int = 0, stress: bool = False) -> None:
        """MCF's particle output (kind 0, io_write_particles) or restart
        (kind 1, io_write_restart_particles) file, formatted on the device
        (mcfg_write_particles)."""
        self._check("mcfg_write_particles",
                    self.lib.mcfg_write_particles(self._h, str(path).encode(), int(kind),
                                                  1 if stress else 0))

    def host_register(self, a: np.ndarray) -> None:
        """Page-lock a C-contiguous host array for full-speed copies
        (mcfg_host_register); unregister it before it is freed."""
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("host_register needs a C-contiguous array")
        self._check("mcfg_host_register",
                    self.lib.mcfg_host_register(self._h, a.ctypes.data, a.nbytes))

    def host_unregister(self, a: np.ndarray) -> None:
        self._check("mcfg_host_unregister", self.lib.mcfg_host_unregister(self._h, a.ctypes.data))

    def write_statistic(self, path, step: int, time: float) -> None:
        """Append one line of MCF's statistic file (io_write_statistic):
        step, time, kinetic energy, momentum and, with stress_tensor, the
        stress sums s(2) s(3) (mcfg_write_statistic)."""
        self._check("mcfg_write_statistic",
                    self.lib.mcfg_write_statistic(self._h, str(path).encode(), int(step),
                                                  float(time)))

    def set_boundary_motion(self, shear_type, shear_freq, time: float = 0.0) -> None:
        """MCF's Boundary shear_type / shear_freq per face (2 = oscillating
        solid wall) and time_current (mcfg_set_boundary_motion)."""
        st = np.ascontiguousarray(shear_type, dtype=np.int32).reshape(6)
        sf = np.ascontiguousarray(shear_freq, dtype=np.float64).reshape(6)
        self._check("mcfg_set_boundary_motion",
                    self.lib.mcfg_set_boundary_motion(self._h, st.ctypes.data_as(C.POINTER(C.c_int32)),
                                                      _ptr(sf, C.c_double), float(time)))

    # -- data --------------------------------------------------------------
    def upload(self, x, v, m, id_, ct=None) -> None:
        n = int(np.asarray(m).shape[0])
        d = self.dim
        self._x = _as(x, np.float64, (n, d))
        self._v = _as(v, np.float64, (n, d))
        self._m = _as(m, np.float64, (n,))
        self._id = _as(id_, np.int32, (n, 2))
        ctp = None if ct is None else _as(ct, np.float64, (n, d * d))
        rc = self.lib.mcfg_upload(self._h, n, _ptr(self._x, C.c_double), _ptr(self._v, C.c_double),
                                  _ptr(self._m, C.c_double), _ptr(self._id, C.c_int32),
                                  _ptr(ctp, C.c_double))
        self._check("mcfg_upload", rc)
        self.n = n

    def download(self, *fields: str) -> dict:
        """fields among x, v, rho, p, f, s, ct; arrays in host particle order."""
        n, d = self.n, self.dim
        shapes = {"x": (n, d), "v": (n, d), "rho": (n,), "p": (n,), "f": (n, d), "s": (n, d * d),
                  "ct": (n, d * d)}
        out = {k: np.empty(shapes[k], np.float64) for k in fields}
        g = lambda k: _ptr(out.get(k), C.c_double)  # noqa: E731
        rc = self.lib.mcfg_download(self._h, g("x"), g("v"), g("rho"), g("p"), g("f"), g("ct"),
                                    g("s"))
        self._check("mcfg_download", rc)
        return out

    # -- MCF routines ------------------------------------------------------
    def particles_adjust_particles(self) -> None:
        self._check("particles_adjust_particles", self.lib.mcfg_adjust_particles(self._h))

    def technique_build_list(self, want_lists: bool = True):
        """Cell list of the current positions.  Returns (num_cell_dim,
        cell_start[num_cell+1], lpdx[n]) with 0-based host indices, or None."""
        if not want_lists:
            self._check("technique_build_list", self.lib.mcfg_build_list(self._h, None, None, None))
            return None
        ncell = self.info()["num_cell"]
        ncd = np.zeros(3, np.int32)
        cs = np.empty(ncell + 1, np.int32)
        lp = np.empty(max(self.n, 1), np.int32)
        self._check("technique_build_list",
                    self.lib.mcfg_build_list(self._h, _ptr(ncd, C.c_int32), _ptr(cs, C.c_int32),
                                             _ptr(lp, C.c_int32)))
        return ncd, cs, lp[: self.n]

    def particles_compute_density(self) -> None:
        self._check("particles_compute_density", self.lib.mcfg_compute_density(self._h))

    def update_density(self, rho) -> None:
        """mcfg_update_density: densities (host order) from the caller, e.g. a
        subdomain's halo particles' densities from their owners"""
        r = _as(rho, np.float64, (self.n,))
        self._check("mcfg_update_density", self.lib.mcfg_update_density(self._h,
                                                                         _ptr(r, C.c_double)))

    def particles_compute_pressure(self) -> None:
        self._check("particles_compute_pressure", self.lib.mcfg_compute_pressure(self._h))

    def particles_compute_interaction(self, step: int = 0) -> None:
        self._check("particles_compute_interaction",
                    self.lib.mcfg_compute_interaction(self._h, int(step)))

    def particles_apply_body_force(self) -> None:
        self._check("particles_apply_body_force", self.lib.mcfg_apply_body_force(self._h))

    def particles_integrate_velocity(self, dt: float, lam: float) -> None:
        self._check("particles_integrate_velocity",
                    self.lib.mcfg_integrate_velocity(self._h, float(dt), float(lam)))

    def particles_integrate_position(self, dt: float) -> None:
        self._check("particles_integrate_position",
                    self.lib.mcfg_integrate_position(self._h, float(dt)))

    def marching_init_force(self, step: int = 0) -> None:
        self._check("marching_init_force", self.lib.mcfg_init_force(self._h, int(step)))

    def marching_integrate_VV(self, step: int, dt: float) -> None:
        self._check("marching_integrate_VV", self.lib.mcfg_step_vv(self._h, int(step), float(dt)))

    def step_vv_host(self, step: int, dt: float, x: np.ndarray, v: np.ndarray) -> None:
        """mcfg_step_vv_host: x, v (float64, C-contiguous [n, d]) in, the new
        state written back into them."""
        for a in (x, v):
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.shape != (self.n, self.dim):
                raise ValueError("x, v must be C-contiguous float64 [n, d]")
        self._check("mcfg_step_vv_host",
                    self.lib.mcfg_step_vv_host(self._h, int(step), float(dt),
                                               _ptr(x, C.c_double), _ptr(v, C.c_double)))

    def run_vv(self, step0: int, nsteps: int, dt: float) -> None:
        self._check("marching_marching", self.lib.mcfg_run_vv(self._h, int(step0), int(nsteps), float(dt)))

    def adjoint_run(self, step0: int, nsteps: int, dt: float, w, checkpoint_every: int = 20,
                    state_grads: bool = False):
        """Time-averaged stress J = mean_t sum_q w[q] S_t[q] over nsteps VV steps from
        the uploaded state, and its gradient by the hand-written adjoint.
        Returns (J, dJ/d(eta, tau, c)) or, with state_grads, also a dict of
        dJ/dx0, dJ/dv0 (and dJ/dct0 for Oldroyd-B) in host order."""
        d = self.dim
        wv = np.zeros(9)
        wv[: d * d] = np.asarray(w, np.float64).reshape(-1)[: d * d]
        J = C.c_double()
        g = np.zeros(3)
        out = {}
        if state_grads:
            out["x"] = np.zeros((self.n, d))
            out["v"] = np.zeros((self.n, d))
            if not self.params.Newtonian:
                out["ct"] = np.zeros((self.n, d * d))
        self._check("mcfg_adjoint_run", self.lib.mcfg_adjoint_run(
            self._h, int(step0), int(nsteps), float(dt), int(checkpoint_every),
            _ptr(wv, C.c_double), C.byref(J), _ptr(g, C.c_double),
            _ptr(out.get("x"), C.c_double), _ptr(out.get("v"), C.c_double),
            _ptr(out.get("ct"), C.c_double)))
        return (J.value, g, out) if state_grads else (J.value, g)

    def statistic_compute_statistic(self, n_owned=None):
        """kinetic energy, momentum[3], stress[9]; with n_owned, over the first
        n_owned particles of the last upload only (a subdomain's own)"""
        ke = C.c_double()
        mom = np.zeros(3)
        st = np.zeros(9)
        if n_owned is None:
            rc = self.lib.mcfg_statistics(self._h, C.byref(ke), _ptr(mom, C.c_double),
                                          _ptr(st, C.c_double))
        else:
            rc = self.lib.mcfg_statistics_owned(self._h, int(n_owned), C.byref(ke),
                                                _ptr(mom, C.c_double), _ptr(st, C.c_double))
        self._check("statistic_compute_statistic", rc)
        return ke.value, mom, st

    # -- colloids (Class_Colloid) -------------------------------------------
    def set_colloids(self, cp: ColloidParams, x, v, omega, radius) -> None:
        self._cp = cp
        self._cx = _as(x, np.float64)
        self._cv = _as(v, np.float64)
        self._com = _as(omega, np.float64)
        self._crad = _as(radius, np.float64)
        self._check("mcfg_set_colloids", self.lib.mcfg_set_colloids(
            self._h, C.byref(cp), _ptr(self._cx, C.c_double), _ptr(self._cv, C.c_double),
            _ptr(self._com, C.c_double), _ptr(self._crad, C.c_double)))

    def move_colloids(self, x_new, rot, v, omega) -> None:
        """mcfg_move_colloids: boundary particles follow their colloids"""
        self._cx = _as(x_new, np.float64)
        self._cv = _as(v, np.float64)
        self._com = _as(omega, np.float64)
        r = None if rot is None else _as(rot, np.float64)
        self._check("mcfg_move_colloids", self.lib.mcfg_move_colloids(
            self._h, _ptr(self._cx, C.c_double), _ptr(r, C.c_double),
            _ptr(self._cv, C.c_double), _ptr(self._com, C.c_double)))

    def colloid_drag(self):
        """particles_collect_colloid_interaction: (drag[nc, d], torque[nc, 3])"""
        nc = self._cp.num_colloid
        drag = np.zeros((nc, self.dim))
        torque = np.zeros((nc, 3))
        self._check("particles_collect_colloid_interaction",
                    self.lib.mcfg_colloid_drag(self._h, _ptr(drag, C.c_double),
                                               _ptr(torque, C.c_double)))
        return drag, torque

    def colloid_repulsion(self):
        """colloid_compute_repulsion_cc summed per colloid: force[nc, d]"""
        out = np.zeros((self._cp.num_colloid, self.dim))
        self._check("colloid_compute_repulsion_cc",
                    self.lib.mcfg_colloid_repulsion(self._h, _ptr(out, C.c_double)))
        return out

    def set_colloid_dynamics(self, cd: ColloidDynamics, mass, mmi, v_hist=None, omega_hist=None,
                             f_hist=None, alpha_hist=None, acc_matrix=None, theta=None) -> None:
        """mcfg_set_colloid_dynamics: integrate the colloids on the device"""
        self._cd = cd
        self._cdyn = [None if a is None else _as(a, np.float64)
                      for a in (mass, mmi, v_hist, omega_hist, f_hist, alpha_hist, acc_matrix,
                                theta)]
        self._check("mcfg_set_colloid_dynamics", self.lib.mcfg_set_colloid_dynamics(
            self._h, C.byref(cd), *[_ptr(a, C.c_double) for a in self._cdyn]))

    def colloid_integrate(self, step: int, dt: float) -> None:
        """mcfg_colloid_integrate: the colloid part of one VV step"""
        self._check("mcfg_colloid_integrate",
                    self.lib.mcfg_colloid_integrate(self._h, int(step), float(dt)))

    def colloid_state(self) -> dict:
        """mcfg_get_colloid_state: x[nc, d], histories [AB, nc, d|3], drag, torque,
        rot / acc matrices [nc, 9] (column-major), acc_vector [nc, 4], theta"""
        nc, d, ab = self._cp.num_colloid, self.dim, self._cd.integrate_AB
        out = {"x": np.zeros((nc, d)), "v": np.zeros((ab, nc, d)), "omega": np.zeros((ab, nc, 3)),
               "f": np.zeros((ab, nc, d)), "alpha": np.zeros((ab, nc, 3)),
               "drag": np.zeros((nc, d)), "torque": np.zeros((nc, 3)),
               "rot": np.zeros((nc, 9)), "acc": np.zeros((nc, 9)),
               "acc_vector": np.zeros((nc, 4)), "theta": np.zeros((nc, 3))}
        keys = ["x", "v", "omega", "f", "alpha", "drag", "torque", "rot", "acc", "acc_vector",
                "theta"]
        self._check("mcfg_get_colloid_state", self.lib.mcfg_get_colloid_state(
            self._h, *[_ptr(out[k], C.c_double) for k in keys]))
        return out

    def update_state(self, x=None, v=None, f=None) -> None:
        """mcfg_update_state: new x / v / f for the uploaded particles, host order"""
        n, d = self.n, self.dim
        arrs = [None if a is None else _as(a, np.float64, (n, d)) for a in (x, v, f)]
        self._check("mcfg_update_state", self.lib.mcfg_update_state(
            self._h, *(_ptr(a, C.c_double) for a in arrs)))

    def upload_force(self, f) -> None:
        self._f = _as(f, np.float64, (self.n, self.dim))
        self._check("mcfg_upload_force", self.lib.mcfg_upload_force(self._h, _ptr(self._f, C.c_double)))

    def stream(self) -> int:
        """cudaStream_t of the handle as an integer (for torch.cuda.ExternalStream)."""
        return int(self.lib.mcfg_get_stream(self._h) or 0)

    def set_profiling(self, mode: int) -> None:
        self._check("mcfg_set_profiling", self.lib.mcfg_set_profiling(self._h, int(mode)))

    def phase_times(self) -> dict:
        ms = np.zeros(5)
        cnt = np.zeros(5, np.int64)
        self._check("mcfg_get_phase_times",
                    self.lib.mcfg_get_phase_times(self._h, _ptr(ms, C.c_double),
                                                  cnt.ctypes.data_as(C.POINTER(C.c_int64))))
        names = ("list", "density", "force", "update", "other")
        return {n: (float(ms[i]), int(cnt[i])) for i, n in enumerate(names)}

    def synchronize(self) -> None:
        self._check("mcfg_synchronize", self.lib.mcfg_synchronize(self._h))
