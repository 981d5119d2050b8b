"""The C ABI without a GPU: the library loads, exports every function include/*.h declares, its
structs have the sizes and offsets the ctypes and numpy mirrors assume, and its host-only calls
and argument checks behave as documented. No compute call is made here."""
import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from blitzen_gb300 import abi
from oracle import oracle as O

ROOT = Path(__file__).resolve().parent.parent
INCLUDE = ROOT / "include"
DECL = re.compile(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(blz_\w+)\s*\(", re.M)


def declared_functions() -> list[str]:
    names = []
    for h in sorted(INCLUDE.glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        text = re.sub(r"#define[^\n]*", "", text)
        names += DECL.findall(text)
    return sorted(set(names))


def test_every_declared_function_is_exported_and_bound(lib):
    names = declared_functions()
    assert len(names) >= 40, names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"
    unbound = sorted(set(names) - set(abi.exported_names()))
    assert not unbound, f"declared but without a ctypes prototype: {unbound}"
    extra = sorted(set(abi.exported_names()) - set(names))
    assert not extra, f"ctypes prototypes of undeclared functions: {extra}"


PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include "blz_cull.h"
#define S(T) printf(#T " %zu\n", sizeof(T));
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  S(BlzRenderObject) S(BlzMeshTransform) S(BlzPrimitiveSurface) S(BlzLodData) S(BlzLodInstanceCounter)
  S(BlzCluster) S(BlzIndirectDraw) S(BlzDrawCmd) S(BlzClusterDispatchData) S(BlzCameraViewData)
  S(BlzSceneDesc) S(BlzPyramid) S(BlzRenderList) S(BlzCullTarget) S(BlzBatchView) S(BlzLaunchShape)
  S(BlzServeConfig) S(BlzServeRequest) S(BlzServeResult) S(BlzServeStats) S(BlzTaskTarget)
  S(BlzIndirectTask) S(BlzMeshTaskPayload)
  O(BlzCameraViewData, lodTarget) O(BlzCameraViewData, zNear) O(BlzCameraViewData, pyramidWidth)
  O(BlzBatchView, mode) O(BlzBatchView, visibility) O(BlzBatchView, pyramid) O(BlzBatchView, target)
  O(BlzBatchView, dynamicTransforms) O(BlzServeRequest, rotateAxes) O(BlzPyramid, mipOffset)
  O(BlzCluster, coneAxisX) O(BlzCluster, dataOffset) O(BlzLodData, error) O(BlzTaskTarget, taskCount)
  O(BlzTaskTarget, payloadCapacity)
  return 0;
}
"""


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory) -> dict[str, int]:
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("probe")
    (d / "probe.c").write_text(PROBE)
    exe = d / "probe"
    subprocess.run([cc, "-std=c11", "-I", str(INCLUDE), str(d / "probe.c"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (line.split() for line in out.splitlines())}


def test_struct_sizes_match_c(c_layout):
    for name, n in abi.C_SIZES.items():
        assert c_layout[name] == n, (name, c_layout[name], n)
    for name, cls in abi.CTYPES_OF.items():
        assert C.sizeof(cls) == c_layout[name], name
    for dt, name in ((abi.RENDER_OBJECT, "BlzRenderObject"), (abi.MESH_TRANSFORM, "BlzMeshTransform"),
                     (abi.PRIMITIVE_SURFACE, "BlzPrimitiveSurface"), (abi.LOD_DATA, "BlzLodData"),
                     (abi.LOD_INSTANCE_COUNTER, "BlzLodInstanceCounter"), (abi.CLUSTER, "BlzCluster"),
                     (abi.INDIRECT_TASK, "BlzIndirectTask"), (abi.MESH_TASK_PAYLOAD, "BlzMeshTaskPayload")):
        assert dt.itemsize == c_layout[name], name
    assert c_layout["BlzIndirectDraw"] == abi.STRIDE_VULKAN and c_layout["BlzDrawCmd"] == abi.STRIDE_D3D12


def test_field_offsets_match_c(c_layout):
    for key, n in c_layout.items():
        if "." not in key:
            continue
        struct, field = key.split(".")
        if struct in abi.CTYPES_OF:
            assert getattr(abi.CTYPES_OF[struct], field).offset == n, key
        elif struct == "BlzCluster":
            assert abi.CLUSTER.fields["coneAxis" if field == "coneAxisX" else field][1] == n, key
        elif struct == "BlzLodData":
            assert abi.LOD_DATA.fields[field][1] == n, key
    assert c_layout["BlzCameraViewData.lodTarget"] == 180


def test_version_and_host_calls(lib):
    assert b"sm_103a" in lib.blz_version()
    for w, h in ((1920, 1080), (1, 1), (333, 199), (4096, 17)):
        for mode in (abi.HIZ_D3D12, abi.HIZ_VULKAN):
            p, nbytes = abi.pyramid_layout(w, h, mode)
            q = O.HostPyramid(w, h, mode)
            assert (p.width, p.height, p.mipCount) == (q.desc.width, q.desc.height, q.desc.mipCount)
            assert list(p.mipOffset) == list(q.desc.mipOffset)
            assert nbytes == q.data.nbytes
    p, _ = abi.pyramid_layout(1920, 1080, abi.HIZ_D3D12)
    assert (p.width, p.height, p.mipCount) == (960, 540, 9)  # GetDepthPyramidMipLevels (blitML.h:95-107)
    p, _ = abi.pyramid_layout(1920, 1080, abi.HIZ_VULKAN)
    assert (p.width, p.height) == (1024, 1024)
    assert lib.blz_pyramid_layout(0, 1080, abi.HIZ_D3D12, None) == 0


def test_argument_errors_need_no_device(lib):
    v = abi.view_setup(1.2, 1920.0, 1080.0, 0.1, 1e4)
    t = abi.CullTarget(None, 24, 0, None)
    rc = lib.blz_cull_frustum(None, C.byref(v), abi.RenderList(None, 0), C.byref(t), None)
    assert rc == 1 and b"NULL" in lib.blz_last_error()
    rc = lib.blz_cull_frustum_noalloc(None, C.byref(v), abi.RenderList(None, 0), C.byref(t), None)
    assert rc == 1
    rc = lib.blz_cull_batch(None, None, 0, None)
    assert rc == 1
    s = abi.ServeConfig(1 << 20, 1, 1, 0, 24)
    out = C.c_void_p()
    assert lib.blz_serve_create(None, C.byref(s), C.byref(out)) == 1
    assert lib.blz_view_setup(None, 1.0, 1.0, 1.0, 0.1, 1.0, None, 0.0, 0.0, 0.0, 0.0) == 1


def test_context_creation_without_a_device_fails_cleanly(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    h = C.c_void_p()
    rc = lib.blz_ctx_create(0, C.byref(h))
    assert rc != 0 and not h.value
    assert len(lib.blz_last_error()) > 0


def test_headers_compile_as_cpp_for_a_cpp_caller():
    """The C++ caller (tests/cpp/abi_smoke.cpp, the reference renderer's language) compiles against
    include/*.h: syntax only, nothing is linked or run here."""
    cxx = shutil.which("g++") or shutil.which("c++")
    cuda_inc = Path("/usr/local/cuda/include")
    if not cxx or not (cuda_inc / "cuda_runtime.h").exists():
        pytest.skip("no C++ compiler or CUDA headers")
    subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", "-I", str(INCLUDE), "-I", str(cuda_inc),
                    str(ROOT / "tests" / "cpp" / "abi_smoke.cpp")], check=True)
