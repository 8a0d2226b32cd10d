import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libmcfg.so)")


@pytest.fixture(scope="session")
def lib():
    """The product library, built in-tree if stale."""
    from mcf_gb300 import build
    from mcf_gb300.mcfg import load_library

    build.build()
    return load_library()


@pytest.fixture(scope="session")
def gpu_lib(lib):
    import ctypes as C

    from mcf_gb300.params import make_params

    # a GPU test must run on the GPU: fail loudly if no device is usable
    h = C.c_void_p()
    p = make_params(num_dim=3, min_phys=[0, 0, 0], max_phys=[12, 12, 12],
                    min_phys_t=[0, 0, 0], max_phys_t=[12, 12, 12], cut_off=3.0)
    rc = lib.mcfg_create(C.byref(p), C.byref(h))
    if rc != 0:
        pytest.fail(f"no usable GPU for a gpu-marked test: {lib.mcfg_create_error().decode()}")
    lib.mcfg_destroy(h)
    return lib
