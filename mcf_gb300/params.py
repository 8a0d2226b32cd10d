"""ctypes mirrors of the C-ABI structs in include/mcfg.h.

`SDPDParams` is `mcfg_params`; the field names are MCF's configuration keys
(mcf_config/ctrl.mcf, mcf_config/physics_config.mcf) so a parameter set reads
like an MCF input deck.
"""
from __future__ import annotations

import ctypes as C

MCFG_OK = 0
MCFG_EINVAL = -1
MCFG_ECUDA = -2
MCFG_ENOMEM = -3
MCFG_ESTATE = -4
MCFG_EOVERFLOW = -5
MCFG_EPHYS = -6
MCFG_ENODEV = -7
MCFG_ETIMEOUT = -8
MCFG_ENOTSUP = -9

STATUS_NAMES = {
    MCFG_OK: "MCFG_OK",
    MCFG_EINVAL: "MCFG_EINVAL",
    MCFG_ECUDA: "MCFG_ECUDA",
    MCFG_ENOMEM: "MCFG_ENOMEM",
    MCFG_ESTATE: "MCFG_ESTATE",
    MCFG_EOVERFLOW: "MCFG_EOVERFLOW",
    MCFG_EPHYS: "MCFG_EPHYS",
    MCFG_ENODEV: "MCFG_ENODEV",
    MCFG_ETIMEOUT: "MCFG_ETIMEOUT",
    MCFG_ENOTSUP: "MCFG_ENOTSUP",
}

BC_PERIODIC = 1
BC_FREESPACE = 2  # no images, no wall particles (a subdomain's cut faces)
BC_WALL_SOLID = 9
BC_LE = 10  # Lees-Edwards (y faces, sliding along x)
PRECISION_FP64 = 0
PRECISION_FP32_MIXED = 1


class SDPDParams(C.Structure):
    _fields_ = [
        ("num_dim", C.c_int32),
        ("bcdef", C.c_int32 * 6),
        ("min_phys", C.c_double * 3),
        ("max_phys", C.c_double * 3),
        ("min_phys_t", C.c_double * 3),
        ("max_phys_t", C.c_double * 3),
        ("cut_off", C.c_double),
        ("cell_factor", C.c_double),
        ("kernel_type", C.c_int32),
        ("rhs_density_type", C.c_int32),
        ("rhs_force_type", C.c_int32),
        ("stateEquation_type", C.c_int32),
        ("c", C.c_double),
        ("rho", C.c_double),
        ("rho_ref", C.c_double),
        ("gamma", C.c_double),
        ("eta", C.c_double),
        ("eta_coef", C.c_double),
        ("kt", C.c_double),
        ("dt", C.c_double),
        ("Brownian", C.c_int32),
        ("symmetry", C.c_int32),
        ("body_force_type", C.c_int32),
        ("wall_rho_type", C.c_int32),
        ("body_force", C.c_double * 3),
        ("wall_noslip_type", C.c_int32),
        ("stress_tensor", C.c_int32),
        ("wall_v", (C.c_double * 3) * 6),
        ("init_density", C.c_double),
        ("Newtonian", C.c_int32),
        ("precision", C.c_int32),
        ("tau", C.c_double),
        ("n_p", C.c_double),
        ("kt_p", C.c_double),
        ("seed", C.c_uint64),
        ("device", C.c_int32),
        ("reserved", C.c_int32 * 7),
    ]

    def copy(self) -> "SDPDParams":
        out = SDPDParams()
        C.memmove(C.byref(out), C.byref(self), C.sizeof(SDPDParams))
        return out


class ColloidParams(C.Structure):
    """mcfg_colloid_params: the Colloid object's pair-term parameters."""

    _fields_ = [
        ("num_colloid", C.c_int32),
        ("noslip_type", C.c_int32),
        ("rho_type", C.c_int32),
        ("translate", C.c_int32),
        ("rotate", C.c_int32),
        ("pp_interact_cc", C.c_int32),
        ("cc_repul_type", C.c_int32),
        ("reserved0", C.c_int32),
        ("dout", C.c_double),
        ("cc_repul_F0", C.c_double),
        ("cc_repul_cut_off", C.c_double),
        ("cc_repul_cut_on", C.c_double),
    ]


class ColloidDynamics(C.Structure):
    """mcfg_colloid_dynamics: the Colloid object's rigid-body integration
    settings (Adams-Bashforth order, sub-steps, step_start, body force)."""

    _fields_ = [
        ("integrate_AB", C.c_int32),
        ("sub_time_step", C.c_int32),
        ("step_start", C.c_int64),
        ("body_force_type", C.c_int32),
        ("reserved0", C.c_int32),
        ("body_force", C.c_double * 3),
    ]


class SDPDInfo(C.Structure):
    _fields_ = [
        ("num_part", C.c_int64),
        ("num_cell_dim", C.c_int32 * 3),
        ("num_cell", C.c_int32),
        ("num_outside", C.c_int64),
        ("num_pairs", C.c_int64),
        ("max_neigh", C.c_int32),
        ("neigh_capacity", C.c_int32),
        ("kernel_launches", C.c_int64),
        ("device_bytes", C.c_int64),
        ("list_rebuilds", C.c_int64),
        ("skin", C.c_double),
        ("time_current", C.c_double),
        ("shear_length", C.c_double),
    ]


def make_params(**kw) -> SDPDParams:
    """Parameter block with MCF's defaults for the SDPD path; keyword names
    are the struct fields (array fields accept sequences)."""
    p = SDPDParams()
    p.num_dim = 3
    for i in range(6):
        p.bcdef[i] = BC_PERIODIC
    p.cell_factor = 1.0001
    p.kernel_type = 1
    p.rhs_density_type = 2
    p.rhs_force_type = 3
    p.stateEquation_type = 1
    p.c = 10.0
    p.rho = 1.0
    p.rho_ref = 1.0
    p.gamma = 1.0
    p.eta = 1.0
    p.eta_coef = 1.0
    p.symmetry = 1
    p.wall_rho_type = 0
    p.wall_noslip_type = 2
    p.init_density = 1.0
    p.Newtonian = 1
    p.precision = PRECISION_FP64
    p.seed = 20261203
    for k, v in kw.items():
        cur = getattr(p, k)
        if isinstance(cur, C.Array):
            if k == "wall_v":
                for f, row in enumerate(v):
                    for a, val in enumerate(row):
                        cur[f][a] = val
            else:
                for i, val in enumerate(v):
                    cur[i] = val
        else:
            setattr(p, k, v)
    return p
