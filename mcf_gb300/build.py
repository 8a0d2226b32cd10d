"""Build libmcfg.so (CUDA, sm_103a) in-tree with nvcc.

Each translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a`` and linked into
``mcf_gb300/libmcfg.so``.  No cmake, no torch extension machinery: the
library exposes a plain C ABI (include/mcfg.h).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libmcfg.so"
SOURCES = ["mcfg_api.cu", "cell_list.cu", "pair_kernels.cu", "update.cu", "noalloc.cu", "adjoint.cu",
           "output.cu", "colloid.cu", "sweep32.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _flags() -> list[str]:
    return [
        "-O3",
        "-std=c++17",
        "-lineinfo",
        *ARCH,
        "-Xcompiler",
        "-fPIC",
        # host arithmetic (boundary updates, constants) rounded as written on
        # both x86-64 and aarch64 hosts, like the oracle
        "-Xcompiler",
        "-ffp-contract=off",
        "-Xptxas",
        "-warn-spills",
        "-I",
        str(ROOT / "include"),
    ]


# Per-file flags.  The pair sweeps run their FP32 path with flush-to-zero and
# approximate FP32 division / square root (MUFU based, no slow-path calls);
# these flags do not touch FP64 arithmetic, so the FP64 path is unchanged.
# The adjoint replays the pair normals (FP32 Box-Muller), so it is compiled
# with the same flags to draw the same bits.
_PAIR_FLAGS = ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"]
EXTRA = {"pair_kernels.cu": _PAIR_FLAGS, "adjoint.cu": _PAIR_FLAGS, "sweep32.cu": _PAIR_FLAGS}


def _compile(src: str, verbose: bool) -> Path:
    obj = BUILD / (Path(src).stem + ".o")
    cmd = [nvcc_path(), *_flags(), *EXTRA.get(src, []), "-c", str(CSRC / src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)
    return obj


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [ROOT / "include" / "mcfg.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile the CUDA library if any source is newer than it."""
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc_path(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    print(LIB)
