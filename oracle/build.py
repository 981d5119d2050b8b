"""Builds the CPU oracle (TEST INFRASTRUCTURE ONLY) into oracle/_build/libblz_oracle.so.

The oracle is compiled with -ffp-contract=off and without fast-math so every FP32 operation rounds
exactly as written (see blz_oracle.h). The product library never links it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libblz_oracle.so"
SOURCES = [HERE / "blz_oracle.c"]
FLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-fno-fast-math",
         "-fno-strict-aliasing", "-Wall", "-Wno-unused-function"]


def build(force: bool = False) -> Path:
    if not force and LIB.exists():
        t = LIB.stat().st_mtime
        deps = SOURCES + [HERE / "blz_oracle.h", HERE.parent / "include" / "blz_types.h",
                          HERE.parent / "include" / "blz_cull.h", Path(__file__)]
        if all(p.stat().st_mtime <= t for p in deps):
            return LIB
    BUILD.mkdir(exist_ok=True)
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the oracle")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, *FLAGS, "-o", str(tmp), *map(str, SOURCES), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
