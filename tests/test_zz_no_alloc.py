"""The allocation-free density entry point (mcfg_density_noalloc).

It serves callers that cannot allocate device memory (code running while a
caching allocator holds its lock, hosts that hand over only buffers they
registered themselves, fixed device-memory budgets): the caller owns every
device buffer and the library keeps its cell list in a fixed array of its
own.  Checked through the C-ABI against the handle-based
mcfg_compute_density on two calls in a row (the second call must not see the
first call's counters), with the FP64 density tolerance of the parity tests
(1e-12 relative); colloid boundary particles with a dynamic density follow
the same rule as the handle path; a repeated call gives identical bits; a
zero density raises the status flag.  Collected last so that a run stopping
at the first failure has run every other test.
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
        return w, None
    if name == "colloids":
        w, cs = configs.c4_colloids(n_side=24, n_colloid=4, radius=3.0, v_scale=0.05,
                                    omega_scale=0.02)
        rng = np.random.default_rng(13)
        fl = w.id[:, 1] == 0
        w.x[fl] += rng.uniform(-0.1, 0.1, (int(fl.sum()), 3))
        cs.params.rho_type = 1  # boundary particles sum their density
        return w, cs
    return make_golden.workload("walls_small"), None


def _reference_density(w, cs):
    g = SDPD(w.params)
    g.upload(w.x, w.v, w.m, w.id)
    if cs is not None:
        g.set_colloids(cs.params, cs.x, cs.v, cs.omega, cs.radius)
    g.technique_build_list(want_lists=False)
    g.particles_compute_density()
    return g.download("rho")["rho"]


def _noalloc_density(lib, torch, w, coll_rho_type=0, params=None):
    dev = torch.device("cuda", 0)
    x = torch.as_tensor(np.ascontiguousarray(w.x), device=dev)
    m = torch.as_tensor(np.ascontiguousarray(w.m), device=dev)
    ids = torch.as_tensor(np.ascontiguousarray(w.id, dtype=np.int32), device=dev)
    rho = torch.full((w.n,), float("nan"), dtype=torch.float64, device=dev)
    p = (params if params is not None else w.params).copy()
    stream = torch.cuda.current_stream(dev)
    rc = lib.mcfg_density_noalloc(C.byref(p), coll_rho_type, w.n, x.data_ptr(), m.data_ptr(),
                                  ids.data_ptr(), rho.data_ptr(), C.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.mcfg_noalloc_error().decode()
    flags = C.c_int32(-1)
    rc = lib.mcfg_noalloc_status(0, C.c_void_p(stream.cuda_stream), C.byref(flags))
    assert rc == 0, lib.mcfg_noalloc_error().decode()
    torch.cuda.synchronize(dev)
    return rho.cpu().numpy(), flags.value


def test_noalloc_density_matches_handle_density_twice(gpu_lib):
    torch = pytest.importorskip("torch")
    for name in ("jit3d", "walls"):  # two calls in a row, different inputs
        w, _ = _case(name)
        ref = _reference_density(w, None)
        got, flags = _noalloc_density(gpu_lib, torch, w)
        assert flags == 0
        assert np.all(np.isfinite(got))
        assert np.all(np.abs(got - ref) <= 1e-12 * np.abs(ref)), name


def test_noalloc_colloid_density_rule_and_repeat(gpu_lib):
    torch = pytest.importorskip("torch")
    w, cs = _case("colloids")
    bp = w.id[:, 1] > 0
    assert bp.sum() > 100
    ref = _reference_density(w, cs)
    got, flags = _noalloc_density(gpu_lib, torch, w, coll_rho_type=1)
    assert flags == 0
    assert np.all(np.abs(got - ref) <= 1e-12 * np.abs(ref))
    # the boundary particles did sum over their pairs (not init_density/m)
    assert np.ptp(got[bp]) > 1e-6
    again, _ = _noalloc_density(gpu_lib, torch, w, coll_rho_type=1)
    assert np.array_equal(got, again)  # fixed summation order
    const, _ = _noalloc_density(gpu_lib, torch, w, coll_rho_type=0)
    assert np.allclose(const[bp], w.params.init_density / w.m[bp], rtol=0, atol=0)


def test_noalloc_zero_density_flag_and_device_kept(gpu_lib):
    torch = pytest.importorskip("torch")
    w, _ = _case("walls")
    p = w.params.copy()
    p.init_density = 0.0  # constant-density walls come out at 0
    torch.cuda.set_device(0)
    got, flags = _noalloc_density(gpu_lib, torch, w, params=p)
    assert flags == 1
    assert np.all(got[w.id[:, 1] < 0] == 0.0)
    assert torch.cuda.current_device() == 0
    ok, flags = _noalloc_density(gpu_lib, torch, w)  # the next call starts clean
    assert flags == 0


def test_noalloc_rejects_oversize(gpu_lib):
    w, _ = _case("jit3d")
    p = w.params.copy()
    rc = gpu_lib.mcfg_density_noalloc(C.byref(p), 0, 70000, None, None, None, None, None)
    assert rc != 0
    assert b"65,536" in gpu_lib.mcfg_noalloc_error() or b"65536" in gpu_lib.mcfg_noalloc_error()
