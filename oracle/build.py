"""Compile the CPU oracle (mcf_oracle.c) into oracle/_lib/liborc.so.

Test infrastructure: the oracle is the parity checker of the CUDA path and
the timed CPU baseline; the product library never links it.  Portable C
(no x86 intrinsics, no -march=native) so it builds the same on x86-64 and
aarch64; -ffp-contract=off keeps every FP64 expression rounded as written.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "mcf_oracle.c"
OUT = HERE / "_lib" / "liborc.so"


def build(verbose: bool = False, force: bool = False) -> Path:
    deps = [SRC, HERE / "mcf_oracle.h", HERE.parent / "include" / "mcfg.h", Path(__file__)]
    if not force and OUT.exists() and all(OUT.stat().st_mtime >= p.stat().st_mtime for p in deps):
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [cc, "-O2", "-std=c11", "-D_POSIX_C_SOURCE=200809L", "-fPIC", "-shared",
           "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-Wall", "-o", str(tmp), str(SRC),
           "-lm"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr)
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
