"""Builds libblz_cull.so in-tree with nvcc for sm_103a.

Every translation unit is compiled in parallel into blitzen_gb300/_build/ and linked into
blitzen_gb300/_lib/libblz_cull.so. Host code is compiled with -ffp-contract=off so the view
constants and every host-side FP32 expression round exactly as written.
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
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libblz_cull.so"

SOURCES = [
    "api.cu",
    "batch.cu",
    "cull_objects.cu",
    "cull_instanced.cu",
    "cull_clusters.cu",
    "pyramid.cu",
    "scene_kernels.cu",
    "serve.cpp",
    "view.cpp",
    "noalloc.cu",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-Xcompiler", "-fPIC",
    "-Xcompiler", "-ffp-contract=off",
    "-Xcompiler", "-fno-fast-math",
    "-I", str(ROOT / "include"),
]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(path).exists():
        raise RuntimeError("nvcc not found")
    return path


def _compile(src: str, extra: list[str]) -> Path:
    out = BUILD / (Path(src).stem + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", str(CSRC / src), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return out


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.iterdir()) + list((ROOT / "include").iterdir()) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.is_file())


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compiles and links the library if any source is newer than it; returns the .so path."""
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", str(tmp), *map(str, objs), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def ptxas_report() -> str:
    """Register / spill / shared-memory report of every kernel (nvcc -Xptxas -v)."""
    lines = []
    for src in SOURCES:
        if not src.endswith(".cu"):
            continue
        cmd = [nvcc(), *ARCH, *COMMON, "-Xptxas", "-v", "-c", str(CSRC / src), "-o", os.devnull]
        r = subprocess.run(cmd, capture_output=True, text=True)
        lines.append(f"== {src}\n{r.stderr}")
    return "\n".join(lines)


if __name__ == "__main__":
    if "--ptxas" in sys.argv:
        print(ptxas_report())
    else:
        build(force="--force" in sys.argv, verbose=True)
