"""The C-ABI from a plain C99 caller (tests/c_caller/mcfg_c_caller.c).

MCF would bind include/mcfg.h through iso_c_binding; the Python mirror binds
it through ctypes.  Here a C program includes the header, links
libmcfg.so and drives a step loop with every status checked:
  - CPU: it compiles with -std=c99 -Wall -Wextra -Werror (the header is
    valid C, the struct layout agrees with the library's), and without a
    GPU its mcfg_create fails cleanly: exit status 2 and the library's
    message, no crash;
  - GPU: its x, v, kinetic energy and momentum after the steps equal, bit
    for bit, those of the same inputs stepped through the ctypes mirror
    (FP64 and FP32-mixed with list reuse).
"""
import os
import shutil
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "c_caller" / "mcfg_c_caller.c"


@pytest.fixture(scope="module")
def c_caller(lib, tmp_path_factory):
    cc = os.environ.get("CC") or shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from mcf_gb300 import build

    libdir = build.LIB.parent
    exe = tmp_path_factory.mktemp("c_caller") / "mcfg_c_caller"
    cmd = [cc, "-std=c99", "-O2", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
           str(SRC), "-o", str(exe), "-L", str(libdir), "-lmcfg", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def _has_gpu(lib):
    import ctypes as C

    from mcf_gb300.params import make_params

    h = C.c_void_p()
    p = make_params(num_dim=3, min_phys=[0, 0, 0], max_phys=[12, 12, 12],
                    min_phys_t=[0, 0, 0], max_phys_t=[12, 12, 12], cut_off=3.0)
    if lib.mcfg_create(C.byref(p), C.byref(h)) != 0:
        return False
    lib.mcfg_destroy(h)
    return True


def test_c_caller_builds_and_fails_cleanly_without_a_gpu(lib, c_caller, tmp_path):
    r = subprocess.run([str(c_caller), str(tmp_path / "out.bin"), "12", "2", "0", "0"],
                       capture_output=True, text=True, timeout=300)
    if _has_gpu(lib):
        assert r.returncode == 0, r.stderr
        return
    assert r.returncode == 2, (r.returncode, r.stdout, r.stderr)
    assert r.stderr.startswith("mcfg error: mcfg_create: ")
    assert len(r.stderr.strip()) > len("mcfg error: mcfg_create: ")


def _lcg_inputs(ns, seed=20261203):
    """the C program's lattice: the same LCG, the same order of draws"""
    mask = (1 << 64) - 1
    state = seed

    def uniform():
        nonlocal state
        state = (state * 6364136223846793005 + 1442695040888963407) & mask
        return (state >> 11) * (1.0 / 9007199254740992.0)

    n = ns ** 3
    x = np.empty((n, 3))
    v = np.empty((n, 3))
    q = 0
    for i in range(ns):
        for j in range(ns):
            for k in range(ns):
                c = (i + 0.5, j + 0.5, k + 0.5)
                for a in range(3):
                    x[q, a] = c[a] + 0.1 * (uniform() - 0.5)
                    v[q, a] = 0.02 * (uniform() - 0.5)
                q += 1
    ids = np.stack([np.arange(1, n + 1), np.zeros(n, int)], 1).astype(np.int32)
    return x, v, np.ones(n), ids


def _python_run(ns, steps, precision, reuse):
    from mcf_gb300 import SDPD
    from mcf_gb300.params import make_params

    L = float(ns)
    p = make_params(num_dim=3, min_phys=[0, 0, 0], max_phys=[L, L, L], min_phys_t=[0, 0, 0],
                    max_phys_t=[L, L, L], cut_off=3.0, cell_factor=1.0001, kernel_type=1,
                    rhs_density_type=2, rhs_force_type=3, stateEquation_type=1, c=10.0,
                    rho=1.0, rho_ref=1.0, gamma=1.0, eta=1.0, kt=1e-3, dt=1e-3, Brownian=1,
                    symmetry=1, wall_noslip_type=2, init_density=1.0, Newtonian=1,
                    precision=precision, seed=42, device=0)
    p.reserved[1] = reuse
    x, v, m, ids = _lcg_inputs(ns)
    g = SDPD(p)
    g.upload(x, v, m, ids)
    g.marching_init_force(0)
    x, v = np.ascontiguousarray(x), np.ascontiguousarray(v)
    for s in range(1, steps + 1):
        g.step_vv_host(s, 1e-3, x, v)
    ke, mom, _ = g.statistic_compute_statistic()
    return x, v, ke, mom


@pytest.mark.gpu
@pytest.mark.parametrize("precision,reuse", [(0, 0), (1, 1)])
def test_c_caller_matches_the_ctypes_path(gpu_lib, c_caller, tmp_path, precision, reuse):
    ns, steps = 12, 8
    out = tmp_path / "out.bin"
    r = subprocess.run([str(c_caller), str(out), str(ns), str(steps), str(precision), str(reuse)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    raw = out.read_bytes()
    (n,) = struct.unpack_from("<q", raw, 0)
    assert n == ns ** 3
    arr = np.frombuffer(raw, dtype=np.float64, offset=8)
    cx, cv = arr[:3 * n].reshape(n, 3), arr[3 * n:6 * n].reshape(n, 3)
    cke, cmom = arr[6 * n], arr[6 * n + 1:6 * n + 4]
    px, pv, pke, pmom = _python_run(ns, steps, precision, reuse)
    assert np.array_equal(cx, px) and np.array_equal(cv, pv)
    assert cke == pke and np.array_equal(cmom, pmom)
    assert np.max(np.abs(pv)) > 0
