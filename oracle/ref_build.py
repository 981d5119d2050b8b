"""Builds the reference's own code for this path into oracle/_ref/ (TEST INFRASTRUCTURE ONLY).

Two pieces of the reference compile on the CPU from their own sources under the reference tree:

  libref_camera.so  the camera code that produces the cull uniform (src/Game/blitzenCamera.cpp with
                    the BlitML headers), wrapped by oracle/ref_camera.cpp;
  libref_hlsl.so    the D3D12 cull and pyramid compute shaders (src/Renderer/HlslShaders/CS/*.hlsl
                    and Headers/*.hlsl) compiled as C++ against oracle/ref_hlsl/hlsl_shim.h and run
                    by oracle/ref_hlsl/ref_hlsl_runner.cpp;
  libref_glsl.so    the Vulkan cull, depth-pyramid and cluster compute shaders
                    (src/Renderer/VulkanShaders/*.comp.glsl and VulkanShaderHeaders/*.glsl) compiled
                    as C++ against oracle/ref_glsl/glsl_shim.h and run by
                    oracle/ref_glsl/ref_glsl_runner.cpp.

The shader text needs a few mechanical edits that only the shader compilers understand. HLSL:
register bindings and system-value semantics are dropped, the [numthreads] attribute is dropped, a
cbuffer's members become plain globals, and `out T name` parameters become `T& name`. GLSL:
#version/#extension lines and the local-size layout are dropped, a layout-qualified buffer,
uniform or push-constant block becomes a struct (its unsized arrays pointers; a buffer_reference
block a struct type; an anonymous block plain globals), a sampler or image uniform a plain global,
`out T name` parameters `T& name`, a multi-component swizzle (`.xyz`) a call (`.xyz()`), and a
struct with a vec3/vec4/mat4 member gets the 16-byte alignment std430 gives it. The
edited files are written to the git-ignored oracle/_ref/ and nothing from the reference enters the
repository.

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
GLSL_DIR = REFERENCE / "src" / "Renderer"
GLSL_FILES = [
    "VulkanShaderHeaders/ShaderBuffers.glsl", "VulkanShaderHeaders/CullingShaderData.glsl",
    "VulkanShaders/TransparentDrawCull.comp.glsl", "VulkanShaders/InitialDrawCull.comp.glsl",
    "VulkanShaders/LateDrawCull.comp.glsl", "VulkanShaders/DepthPyramidGeneration.comp.glsl",
    "VulkanShaders/PreClusterDrawCull.comp.glsl", "VulkanShaders/InitialClusterCull.comp.glsl",
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


def _glsl_block(m: re.Match) -> str:
    """One layout-qualified buffer / uniform block as C++ (see the module docstring)."""
    layout, name, body, inst = m.group(1), m.group(3), m.group(4), m.group(5)
    body = re.sub(r"(\w+)\s+(\w+)\s*\[\s*\]\s*;", r"\1* \2;", body)
    if inst:
        return f"struct {name} {{{body}}} {inst};"
    if "buffer_reference" in layout:
        return f"struct {name} {{{body}}};"
    return body


def glsl_to_cpp(text: str) -> str:
    """The mechanical GLSL edits listed in the module docstring."""
    text = re.sub(r"^\s*#\s*(version|extension)\b.*$", "", text, flags=re.M)
    text = re.sub(r"layout\s*\([^)]*\)\s*in\s*;", "", text)
    text = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+(?:(?:readonly|writeonly)\s+)?(sampler2D|image2D)\s+(\w+)\s*;",
                  r"\1 \2;", text)
    text = re.sub(r"layout\s*\(([^)]*)\)\s*((?:readonly|writeonly|coherent|restrict)\s+)*(?:buffer|uniform)\s+(\w+)"
                  r"\s*\{(.*?)\}\s*(\w*)\s*;", _glsl_block, text, flags=re.S)
    text = re.sub(r"\bout\s+(\w+)\s+(\w+)", r"\1& \2", text)
    text = re.sub(r"\.([xyzw]{2,4})\b(?!\s*\()", r".\1()", text)
    # std430 / std140: a struct with a vec3, vec4 or mat4 member is 16-byte aligned (its array stride
    # a multiple of 16), while a vec3 itself takes 12 bytes and lets a scalar follow in its fourth slot
    text = re.sub(r"\bstruct\s+(\w+)\s*\{([^{}]*?\b(?:vec3|vec4|mat4)\b[^{}]*?)\}",
                  r"struct alignas(16) \1 {\2}", text)
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


def build_glsl() -> Path | None:
    if not available():
        return None
    gen = OUT / "glsl"
    for rel in GLSL_FILES:
        dst = gen / rel
        dst.parent.mkdir(parents=True, exist_ok=True)
        dst.write_text(glsl_to_cpp((GLSL_DIR / rel).read_text()))
    lib = OUT / "libref_glsl.so"
    runner = HERE / "ref_glsl" / "ref_glsl_runner.cpp"
    cmd = [_cxx(), *CXX_FLAGS, "-I", str(HERE / "ref_glsl"), "-I", str(gen), "-o", str(lib), str(runner)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference GLSL build failed:\n{' '.join(cmd)}\n{r.stderr[-6000:]}")
    return lib


def build() -> dict[str, Path | None]:
    return {"camera": build_camera(), "hlsl": build_hlsl(), "glsl": build_glsl()}


if __name__ == "__main__":
    print(build())
