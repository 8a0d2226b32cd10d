"""GB300-native SDPD right-hand side and velocity-Verlet step for MCF.

The compute path is libmcfg.so (hand-written CUDA for sm_103a) behind the
C-ABI of include/mcfg.h; `SDPD` is its host-side mirror of MCF's particle
routines.
"""
from .params import (BC_LE, BC_PERIODIC, BC_WALL_SOLID, PRECISION_FP32_MIXED, PRECISION_FP64, SDPDInfo,
                     SDPDParams, make_params)
from .mcfg import MCFGError, SDPD, load_library

__all__ = ["SDPD", "SDPDParams", "SDPDInfo", "MCFGError", "make_params", "load_library",
           "BC_PERIODIC", "BC_WALL_SOLID", "BC_LE", "PRECISION_FP64", "PRECISION_FP32_MIXED"]
