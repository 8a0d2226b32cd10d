"""The allocation-free density entry point (mcfg_density_noalloc).

It serves callers that cannot allocate device memory: the caller owns every
device buffer and the library keeps its cell list in a fixed array of its
own.  Checked through the C-ABI against the handle-based
mcfg_compute_density on two calls in a row (the second call must not see the
first call's counters), with the FP64 density tolerance of the parity tests
(1e-12 relative).  Collected last so that a run stopping at the first failure
has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from mcf_gb300 import SDPD, configs
from tests.golden import make_golden

pytestmark = pytest.mark.gpu


def _case(name):
    if name == "jit3d":
        w = configs.c2_fluctuating_3d(n_side=12)
        rng = np.random.default_rng(21)
        w.x = w.x + rng.uniform(-0.3, 0.3, w.x.shape)
        return w
    return make_golden.workload("walls_small")


def _reference_density(w):
    g = SDPD(w.params)
    g.upload(w.x, w.v, w.m, w.id)
    g.technique_build_list(want_lists=False)
    g.particles_compute_density()
    return g.download("rho")["rho"]


def _noalloc_density(lib, torch, w):
    dev = torch.device("cuda", 0)
    x = torch.as_tensor(np.ascontiguousarray(w.x), device=dev)
    m = torch.as_tensor(np.ascontiguousarray(w.m), device=dev)
    ids = torch.as_tensor(np.ascontiguousarray(w.id, dtype=np.int32), device=dev)
    rho = torch.full((w.n,), float("nan"), dtype=torch.float64, device=dev)
    p = w.params.copy()
    stream = torch.cuda.current_stream(dev)
    rc = lib.mcfg_density_noalloc(C.byref(p), w.n, x.data_ptr(), m.data_ptr(), ids.data_ptr(),
                                  rho.data_ptr(), C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.mcfg_noalloc_error().decode()
    torch.cuda.synchronize(dev)
    return rho.cpu().numpy()


def test_noalloc_density_matches_handle_density_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    for name in ("jit3d", "walls"):  # two calls in a row, different inputs
        w = _case(name)
        ref = _reference_density(w)
        got = _noalloc_density(gpu_lib, torch, w)
        assert np.all(np.isfinite(got))
        assert np.all(np.abs(got - ref) <= 1e-12 * np.abs(ref)), name


def test_noalloc_rejects_oversize(gpu_lib):
    w = _case("jit3d")
    p = w.params.copy()
    rc = gpu_lib.mcfg_density_noalloc(C.byref(p), 70000, None, None, None, None, None)
    assert rc != 0
    assert b"65,536" in gpu_lib.mcfg_noalloc_error() or b"65536" in gpu_lib.mcfg_noalloc_error()
