"""Builds the reference's own code for this path into oracle/_ref/ (TEST INFRASTRUCTURE ONLY).

Two pieces of the reference compile on the CPU from their own sources under the reference tree:

  libref_camera.so  the camera code that produces the cull uniform (src/Game/blitzenCamera.cpp with
                    the BlitML headers), wrapped by oracle/ref_camera.cpp;
  libref_hlsl.so    the D3D12 cull and pyramid compute shaders (src/Renderer/HlslShaders/CS/*.hlsl
                    and Headers/*.hlsl) compiled as C++ against oracle/ref_hlsl/hlsl_shim.h and run
                    by oracle/ref_hlsl/ref_hlsl_runner.cpp.

The shader text needs a few mechanical edits that only the D3D compiler understands: register
bindings and system-value semantics are dropped, the [numthreads] attribute is dropped, a cbuffer's
members become plain globals, and `out T name` parameters become `T& name`. The edited files are
written to the git-ignored oracle/_ref/hlsl/ and nothing from the reference enters the repository.
The Vulkan GLSL shaders are not built this way: their buffer-block syntax has no C++ counterpart,
and their cull arithmetic is the same functions as the HLSL ones.

Returns None (and builds nothing) when the reference tree is absent, as on the GPU machine.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
REFERENCE = Path(os.environ.get("BLZ_REFERENCE_TREE", "/root/reference"))
HLSL_DIR = REFERENCE / "src" / "Renderer" / "HlslShaders"
HLSL_FILES = [
    "Headers/sharedBuffers.hlsl", "Headers/cullBuffers.hlsl", "Headers/hlslMath.hlsl",
    "CS/drawCull.cs.hlsl", "CS/drawOccFirst.cs.hlsl", "CS/drawOccLate.cs.hlsl", "CS/drawOccTemporal.hlsl",
    "CS/drawCountReset.cs.hlsl", "CS/drawInstCountReset.cs.hlsl", "CS/drawInstCull.cs.hlsl",
    "CS/drawInstCmd.cs.hlsl", "CS/depthPyramid.cs.hlsl",
]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-w"]


def available() -> bool:
    return (REFERENCE / "src" / "Game" / "blitzenCamera.cpp").exists() and HLSL_DIR.exists()


def hlsl_to_cpp(text: str) -> str:
    """The mechanical edits listed in the module docstring."""
    text = re.sub(r"\s*:\s*register\s*\(\s*\w+\s*\)", "", text)
    text = re.sub(r"\s*:\s*SV_\w+", "", text)
    text = re.sub(r"^\s*\[numthreads\([^\]]*\)\]\s*$", "", text, flags=re.M)
    text = re.sub(r"cbuffer\s+\w+\s*\{(.*?)\}\s*;?", r"\1", text, flags=re.S)
    text = re.sub(r"\bout\s+(\w+)\s+(\w+)", r"\1& \2", text)
    return text


def _cxx() -> str:
    c = shutil.which("g++") or shutil.which("c++")
    if not c:
        raise RuntimeError("no C++ compiler")
    return c


def _newer(target: Path, deps: list[Path]) -> bool:
    return target.exists() and all(d.stat().st_mtime <= target.stat().st_mtime for d in deps if d.exists())


def build_camera() -> Path | None:
    if not available():
        return None
    OUT.mkdir(exist_ok=True)
    lib = OUT / "libref_camera.so"
    src = [HERE / "ref_camera.cpp", REFERENCE / "src" / "Game" / "blitzenCamera.cpp"]
    if _newer(lib, src + [Path(__file__)]):
        return lib
    cmd = [_cxx(), *CXX_FLAGS, "-fpermissive", "-DBLIT_DYNAMIC_OBJECT_TEST", "-include", "cstring",
           "-I", str(REFERENCE / "src"), "-o", str(lib), *map(str, src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference camera build failed:\n{' '.join(cmd)}\n{r.stderr[-4000:]}")
    return lib


def build_hlsl() -> Path | None:
    if not available():
        return None
    gen = OUT / "hlsl"
    for rel in HLSL_FILES:
        dst = gen / rel
        dst.parent.mkdir(parents=True, exist_ok=True)
        dst.write_text(hlsl_to_cpp((HLSL_DIR / rel).read_text()))
    lib = OUT / "libref_hlsl.so"
    runner = HERE / "ref_hlsl" / "ref_hlsl_runner.cpp"
    cmd = [_cxx(), *CXX_FLAGS, "-I", str(HERE / "ref_hlsl"), "-I", str(gen), "-o", str(lib), str(runner)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference HLSL build failed:\n{' '.join(cmd)}\n{r.stderr[-6000:]}")
    return lib


def build() -> dict[str, Path | None]:
    return {"camera": build_camera(), "hlsl": build_hlsl()}


if __name__ == "__main__":
    print(build())
