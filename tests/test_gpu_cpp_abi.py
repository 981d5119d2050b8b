"""The C ABI from a C++ caller with no Python in its process (tests/cpp/abi_smoke.cpp): the program's
draw counts and record checksums must equal the oracle's for the same scene, built here with the
same generator, including a cull over dynamic rows bound from pinned host memory."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from blitzen_gb300 import abi
from blitzen_gb300 import scenes as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
CUDA = Path("/usr/local/cuda")


def _fnv(data: bytes) -> int:
    h = 1469598103934665603
    for b in data:
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


class _Lcg:
    def __init__(self, seed):
        self.s = seed

    def next(self) -> int:
        self.s = (self.s * 1664525 + 1013904223) & 0xFFFFFFFF
        return self.s

    def unit(self) -> np.float32:
        return np.float32(self.next() >> 8) * np.float32(1.0 / 16777216.0)


def _scene():
    N, M, L = 50000, 8, 4
    r = _Lcg(12345)
    surf = np.zeros(M, abi.PRIMITIVE_SURFACE)
    lods = np.zeros(M * L, abi.LOD_DATA)
    for m in range(M):
        surf[m]["center"] = [r.unit() - np.float32(0.5), r.unit() - np.float32(0.5), r.unit() - np.float32(0.5)]
        surf[m]["radius"] = np.float32(0.5) + np.float32(2.0) * r.unit()
        surf[m]["lodOffset"], surf[m]["lodCount"] = m * L, L
        for l in range(L):
            d = lods[m * L + l]
            d["indexCount"], d["firstIndex"] = 30000 >> l, 1000 * (m * L + l)
            d["error"] = 0.0 if l == 0 else np.float32(0.01) * np.float32(1 << (2 * (l - 1)))
            lods[m * L + l] = d
    tr = np.zeros(N, abi.MESH_TRANSFORM)
    objs = np.zeros(N, abi.RENDER_OBJECT)
    for i in range(N):
        x = np.float32(2000.0) * r.unit() - np.float32(1000.0)
        y = np.float32(2000.0) * r.unit() - np.float32(1000.0)
        z = np.float32(2000.0) * r.unit() - np.float32(1000.0)
        tr[i]["pos"] = [x, y, z]
        tr[i]["scale"] = np.float32(0.5) + np.float32(1.5) * r.unit()
        tr[i]["orientation"] = [0.0, 0.0, 0.0, 1.0]
        objs[i]["transformId"] = i
        objs[i]["surfaceId"] = r.next() % M
    return S.Scene(objs, tr, surf, lods)


@pytest.fixture(scope="module")
def program(lib, tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx or not (CUDA / "include" / "cuda_runtime.h").exists():
        pytest.skip("no C++ compiler or CUDA headers")
    out = tmp_path_factory.mktemp("cpp") / "abi_smoke"
    libdir = ROOT / "blitzen_gb300" / "_lib"
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", str(ROOT / "include"), "-I", str(CUDA / "include"),
           str(ROOT / "tests" / "cpp" / "abi_smoke.cpp"), "-o", str(out), "-L", str(libdir), "-lblz_cull",
           "-L", str(CUDA / "lib64"), "-lcudart", f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{CUDA / 'lib64'}"]
    subprocess.run(cmd, check=True)
    return out


def test_cpp_caller_matches_oracle(program):
    line = subprocess.run([str(program)], check=True, capture_output=True, text=True, timeout=300).stdout.split()
    got = dict(frustum=int(line[1]), hf=int(line[2], 16), first=int(line[4]), late=int(line[6]), hl=int(line[7], 16),
               hv=int(line[9], 16), bound=int(line[11]), hb=int(line[12], 16))
    sc = _scene()
    v = O.view_setup(float(np.float32(1.2217305)), 1920.0, 1080.0, 0.1, 1e4, (0.0, 0.0, 0.0), 0.3, 0.1, 960.0, 540.0)
    n, recs, _ = O.cull(0, v, sc)
    assert got["frustum"] == n
    assert got["hf"] == _fnv(recs[:, :6].astype(np.uint32).tobytes())
    vis = (np.arange(sc.count) & 1).astype(np.uint32)
    n1, _, _ = O.cull(1, v, sc, vis=vis)
    assert got["first"] == n1
    depth = np.zeros((1080, 1920), np.float32)
    depth[:, :960] = np.float32(0.001)
    pyr = O.pyramid_build(depth)
    n2, recs2, _ = O.cull(2, v, sc, vis=vis, pyramid=pyr)
    assert got["late"] == n2
    assert got["hl"] == _fnv(recs2[:, :6].astype(np.uint32).tobytes())
    assert got["hv"] == _fnv(vis.tobytes())
    # transforms [0, 4096) read from bound pinned rows, moved 150 units along x
    moved = S.Scene(sc.objects, sc.transforms.copy(), sc.surfaces, sc.lods)
    moved.transforms["pos"][:4096, 0] += np.float32(150.0)
    nb, recsb, _ = O.cull(0, v, moved)
    assert got["bound"] == nb and nb != n
    assert got["hb"] == _fnv(recsb[:, :6].astype(np.uint32).tobytes())
