"""CPU tests of the C-ABI boundary: libmcfg.so loads, exports every entry
point include/mcfg.h declares, agrees on the parameter layout, and rejects
bad parameter blocks with MCFG_EINVAL and a message before touching a GPU."""
import ctypes as C
import re
from pathlib import Path

import pytest

from mcf_gb300.params import MCFG_EINVAL, SDPDParams, make_params

HEADER = Path(__file__).resolve().parent.parent / "include" / "mcfg.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mcfg_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("mcfg_create", "mcfg_upload", "mcfg_build_list", "mcfg_compute_density",
                 "mcfg_compute_interaction", "mcfg_step_vv", "mcfg_download", "mcfg_destroy"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_params_layout(lib):
    assert lib.mcfg_sizeof_params() == C.sizeof(SDPDParams)


@pytest.mark.parametrize("field,value,msg", [
    ("num_dim", 4, "num_dim"),
    ("cut_off", 0.0, "cut_off"),
    ("kernel_type", 3, "kernel_type"),
    ("rhs_force_type", 7, "rhs_force_type"),
    ("body_force_type", 9, "body_force_type"),
    ("precision", 5, "precision"),
])
def test_create_rejects_bad_params(lib, field, value, msg):
    p = make_params(min_phys=[0, 0, 0], max_phys=[12, 12, 12], min_phys_t=[0, 0, 0],
                    max_phys_t=[12, 12, 12], cut_off=3.0)
    setattr(p, field, value)
    h = C.c_void_p()
    rc = lib.mcfg_create(C.byref(p), C.byref(h))
    assert rc == MCFG_EINVAL
    assert msg in lib.mcfg_create_error().decode()
    assert not h.value


def test_create_rejects_open_periodic_axis(lib):
    p = make_params(min_phys=[0, 0, 0], max_phys=[12, 12, 12], min_phys_t=[0, 0, 0],
                    max_phys_t=[12, 12, 12], cut_off=3.0)
    p.bcdef[0] = 9  # wall below, periodic above
    h = C.c_void_p()
    assert lib.mcfg_create(C.byref(p), C.byref(h)) == MCFG_EINVAL
    assert "periodic" in lib.mcfg_create_error().decode()


def test_null_handle_calls_fail_cleanly(lib):
    assert lib.mcfg_compute_density(None) == MCFG_EINVAL
    assert lib.mcfg_step_vv(None, 1, 1e-3) == MCFG_EINVAL
    assert lib.mcfg_destroy(None) == 0
    assert lib.mcfg_last_error(None) == b"null handle"
