"""Writes the golden fixtures of tests/golden/ from the reference's own code (run in a tree that has
the reference checkout; the fixtures then travel without it).

The outputs come from the reference, compiled on the CPU by oracle/ref_build.py:
  * CameraViewData from its camera code (SetupCamera / UpdateProjection, blitzenCamera.cpp:7-126);
  * cull records, counters and visibility from its D3D12 compute shaders compiled as C++
    (drawCull.cs.hlsl, drawOccFirst.cs.hlsl, drawOccLate.cs.hlsl, drawOccTemporal.hlsl,
    drawInstCountReset/drawInstCull/drawInstCmd.cs.hlsl, depthPyramid.cs.hlsl) dispatched in the
    order of src/Renderer/BlitzenDX12/dx12Draw.cpp.
The oracle is used only to choose inputs: the boundary cases (spheres one ulp either side of each
frustum plane, of the near plane in projectSphere, of a Hi-Z mip-level change, and LOD errors equal
to the LOD threshold) are found by bisection on its predicates, and the reference then says what
the answer at each of them is.

Files (numpy .npz, compressed):
  camera.npz     256 camera parameter sets and the 256-byte view the reference makes from each
  pyramid.npz    depth buffers of several extents and the reference's D3D12 pyramid of each
  cull.npz       a 3,000-object random scene, a rasterised depth and its pyramid, 4 cameras x 4
                 cull kinds: draw count, 32-byte records, visibility after the pass
  kat.npz        the boundary-case scene with a constant-per-mip pyramid, 4 cull kinds
  instanced.npz  the random scene's instanced cull: counters, instance ids, records
  vkpyramid.npz  depth buffers and the reference's Vulkan pyramid of each (DepthPyramidGeneration
                 .comp.glsl dispatched per level as vulkanDraw.cpp:554-622 does)
  vkcull.npz     the random scene, 4 cameras x 3 Vulkan culls (TransparentDrawCull, InitialDrawCull,
                 LateDrawCull against the Vulkan pyramid): draw count, 24-byte records, visibility
  vkkat.npz      spheres one ulp either side of every Hi-Z level change of the Vulkan form, against
                 constant-per-mip pyramids (LateDrawCull), with visibility
  vkclusters.npz a cluster scene through PreClusterDrawCull + InitialClusterCull: dispatch entries and
                 records (the reference runs no per-cluster test: its cone test is commented out)
The Vulkan outputs come from the reference's GLSL compiled as C++ (oracle/ref_glsl/); the sampler's
MIN-footprint is the one definition there that is not the reference's text (glsl_shim.h).

Usage: python tests/golden/make_golden.py   (rebuilds oracle/_ref from the reference first)
"""
from __future__ import annotations

import ctypes as C
import math
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from blitzen_gb300 import abi, scenes as S  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import ref_build  # noqa: E402

P, U = C.c_void_p, C.c_uint32
W, H = 1920, 1080


def ref_libs():
    libs = ref_build.build()
    if not libs["camera"] or not libs["hlsl"]:
        raise SystemExit("the reference tree is not available: nothing to generate from")
    cam = C.CDLL(str(libs["camera"]))
    cam.ref_view_setup.argtypes = [P, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, P, C.c_float,
                                   C.c_float, C.c_float, C.c_float]
    hl = C.CDLL(str(libs["hlsl"]))
    hl.ref_hlsl_cull.argtypes = [C.c_int, P, P, P, U, P, P, P, U]
    hl.ref_hlsl_cull.restype = U
    hl.ref_hlsl_pyramid.argtypes = [P, U, U, P]
    hl.ref_hlsl_instanced.argtypes = [P, P, P, U, P, P, U, P, U]
    hl.ref_hlsl_instanced.restype = U
    return cam, hl


def glsl_lib():
    lib = ref_build.build_glsl()
    if not lib:
        raise SystemExit("the reference tree is not available: nothing to generate from")
    gl = C.CDLL(str(lib))
    gl.ref_glsl_cull.argtypes = [C.c_int, P, P, P, U, P, P, P]
    gl.ref_glsl_cull.restype = U
    gl.ref_glsl_pyramid.argtypes = [P, U, U, P]
    gl.ref_glsl_clusters.argtypes = [P, P, P, U, P, P, P]
    gl.ref_glsl_clusters.restype = U
    return gl


def ref_view(cam, fov, w, h, zn, zf, pos, yaw, pitch, pw, ph) -> abi.CameraViewData:
    v = abi.CameraViewData()
    p = (C.c_float * 3)(*pos)
    cam.ref_view_setup(C.byref(v), fov, w, h, zn, zf, C.byref(p), yaw, pitch, pw, ph)
    return v


def vbytes(v) -> np.ndarray:
    return np.frombuffer(bytes(v), np.uint8).copy()


# ------------------------------------------------------------------ camera


def make_camera(cam) -> dict:
    rng = np.random.default_rng(101)
    rows = []
    fov = S.fov_radians()
    fixed = [
        (fov, 1920.0, 1080.0, 0.1, 650.0, (0.0, 0.0, 0.0), 0.0, 0.0, 960.0, 540.0),
        (fov, 1920.0, 1080.0, 0.1, 1e30, (0.0, 0.0, 0.0), 0.0, 0.0, 960.0, 540.0),
        (fov, 1280.0, 720.0, 1.0, 1e4, (10.0, -5.0, 3.0), 3.14159265, 0.0, 640.0, 360.0),
        (S.fov_radians(45.0), 800.0, 800.0, 0.01, 100.0, (-1.0, 2.0, 3.0), -1.5, 1.5, 400.0, 400.0),
        (S.fov_radians(110.0), 3840.0, 2160.0, 0.5, 5e5, (1e4, 1e4, -1e4), 0.7, -1.2, 1920.0, 1080.0),
    ]
    rows.extend(fixed)
    while len(rows) < 256:
        rows.append((S.fov_radians(float(rng.uniform(30, 120))), float(rng.choice([640, 1280, 1920, 2560, 3840])),
                     float(rng.choice([360, 720, 1080, 1440, 2160])), float(rng.choice([0.01, 0.1, 1.0])),
                     float(rng.choice([100.0, 650.0, 1e4, 1e30])),
                     tuple(float(x) for x in rng.uniform(-5000, 5000, 3).astype(np.float32)),
                     float(np.float32(rng.uniform(-6.3, 6.3))), float(np.float32(rng.uniform(-1.55, 1.55))),
                     float(rng.choice([480.0, 960.0, 1024.0])), float(rng.choice([270.0, 540.0, 1024.0]))))
    params = np.array([[r[0], r[1], r[2], r[3], r[4], *r[5], r[6], r[7], r[8], r[9]] for r in rows], np.float32)
    views = np.stack([vbytes(ref_view(cam, *(float(x) for x in p[:5]), tuple(float(x) for x in p[5:8]),
                                      *(float(x) for x in p[8:12]))) for p in params])
    return {"params": params, "views": views}


# ------------------------------------------------------------------ pyramid


def ref_pyramid(hl, depth: np.ndarray) -> O.HostPyramid:
    h, w = depth.shape
    p = O.HostPyramid(w, h, abi.HIZ_D3D12)
    hl.ref_hlsl_pyramid(np.ascontiguousarray(depth, np.float32).ctypes.data, w, h, C.byref(p.desc))
    return p


def make_pyramid(hl) -> dict:
    rng = np.random.default_rng(202)
    out = {}
    shapes = [(1, 3), (2, 2), (5, 7), (48, 64), (199, 333)]
    for i, (h, w) in enumerate(shapes):
        d = rng.random((h, w), dtype=np.float32)
        d[rng.random((h, w)) < 0.3] = 0.0  # cleared depth
        p = ref_pyramid(hl, d)
        out[f"depth{i}"] = d
        out[f"pyr{i}"] = p.data.copy()
        out[f"mips{i}"] = np.array([p.desc.mipCount, p.desc.width, p.desc.height], np.uint32)
    out["count"] = np.array([len(shapes)], np.uint32)
    return out


# ------------------------------------------------------------------ culls


def run_ref_cull(hl, kind: int, view, scene, vis: np.ndarray | None, pyr) -> tuple[int, np.ndarray, np.ndarray | None]:
    d, keep = O.scene_desc(scene)
    n = scene.count
    cmds = np.zeros((max(n, 1), 8), np.uint32)
    v = None if vis is None else np.ascontiguousarray(vis.copy(), np.uint32)
    cnt = hl.ref_hlsl_cull(kind, C.byref(view), C.byref(d), keep[0].ctypes.data, n,
                           None if v is None else v.ctypes.data, C.byref(pyr.desc) if pyr else None,
                           cmds.ctypes.data, n)
    return int(cnt), cmds[:cnt].copy(), v


def scene_arrays(prefix: str, sc) -> dict:
    return {f"{prefix}objects": sc.objects, f"{prefix}transforms": sc.transforms, f"{prefix}surfaces": sc.surfaces,
            f"{prefix}lods": sc.lods}


def make_cull(cam, hl) -> dict:
    sc = S.stress_scene(3000, seed=303, n_meshes=24, extent=300.0, n_boxes=200)
    # a few degenerate transforms the generators of the reference also produce: zero scale and a
    # non-unit quaternion
    sc.transforms["scale"][5] = 0.0
    sc.transforms["orientation"][6] = np.array([0.5, 0.5, 0.5, 0.9], np.float32)
    fov = S.fov_radians()
    views = [ref_view(cam, fov, 1920.0, 1080.0, 0.1, 1e4, (0.0, 0.0, 0.0), 0.0, 0.0, 160.0, 90.0),
             ref_view(cam, fov, 1920.0, 1080.0, 0.1, 650.0, (20.0, -10.0, -300.0), 0.3, 0.1, 160.0, 90.0),
             ref_view(cam, fov, 1920.0, 1080.0, 0.1, 1e30, (0.0, 50.0, 0.0), 2.0, -0.4, 160.0, 90.0),
             ref_view(cam, fov, 1920.0, 1080.0, 0.1, 1e4, (0.0, 0.0, 0.0), 3.14159265, 0.0, 160.0, 90.0)]
    out = scene_arrays("", sc)
    out["visibility"] = sc.visibility
    out["views"] = np.stack([vbytes(v) for v in views])
    for c, v in enumerate(views):
        depth = O.depth_raster(v, sc.boxes, 320, 180)
        pyr = ref_pyramid(hl, depth)
        out[f"depth{c}"] = depth
        out[f"pyr{c}"] = pyr.data.copy()
        for kind in range(4):
            vis = sc.visibility if kind in (1, 2) else None
            cnt, cmds, vis_out = run_ref_cull(hl, kind, v, sc, vis, pyr if kind in (2, 3) else None)
            out[f"count{c}_{kind}"] = np.array([cnt], np.uint32)
            out[f"cmds{c}_{kind}"] = cmds
            if vis_out is not None:
                out[f"vis{c}_{kind}"] = vis_out
    return out


def make_instanced(cam, hl) -> dict:
    sc = S.stress_scene(3000, seed=303, n_meshes=24, extent=300.0, n_boxes=200)
    v = ref_view(cam, S.fov_radians(), 1920.0, 1080.0, 0.1, 1e4, (0.0, 0.0, -100.0), 0.2, 0.0, 160.0, 90.0)
    slots = sc.count
    ctr = O.new_counters(sc, slots)
    inst = np.full(len(sc.lods) * slots, 0xFFFFFFFF, np.uint32)
    cmds = np.zeros((len(sc.lods), 8), np.uint32)
    d, keep = O.scene_desc(sc)
    cnt = hl.ref_hlsl_instanced(C.byref(v), C.byref(d), keep[0].ctypes.data, sc.count, ctr.ctypes.data,
                                inst.ctypes.data, len(inst), cmds.ctypes.data, len(sc.lods))
    out = scene_arrays("", sc)
    out.update({"view": vbytes(v), "slots": np.array([slots], np.uint32), "count": np.array([cnt], np.uint32),
                "cmds": cmds[:cnt].copy(), "counters": ctr, "instances": inst})
    return out


# ------------------------------------------------------------------ boundary cases


def _key(x) -> int:
    """Integer key in the order of the floats (-0 and +0 share 0)."""
    b = int(np.array([x], np.float32).view(np.uint32)[0])
    return b if b < 0x80000000 else -(b & 0x7FFFFFFF)


def _val(k: int) -> float:
    b = k if k >= 0 else (0x80000000 | -k)
    return float(np.array([b], np.uint32).view(np.float32)[0])


def bisect(pred, lo: float, hi: float) -> int:
    """With pred(lo) != pred(hi): the key of the first float above lo where pred takes pred(hi)'s value."""
    a, b = _key(lo), _key(hi)
    pa = pred(_val(a))
    assert pred(_val(b)) != pa, (lo, hi)
    while b - a > 1:
        m = (a + b) // 2
        if pred(_val(m)) == pa:
            a = m
        else:
            b = m
    return b


class KatScene:
    """Objects with identity orientation and unit scale unless stated, one surface each (centre 0)."""

    def __init__(self):
        self.tr, self.surf, self.lods = [], [], []
        self.std_lod = self.add_lods([0.0, 0.01, 0.04, 0.16])

    def add_lods(self, errors) -> int:
        off = len(self.lods)
        for i, e in enumerate(errors):
            self.lods.append((30000 >> i, 1000 * off + i, float(e)))
        return off

    def add(self, pos, radius, scale=1.0, quat=(0.0, 0.0, 0.0, 1.0), lod=None, lod_count=4) -> int:
        self.tr.append((tuple(float(c) for c in pos), float(scale), quat))
        self.surf.append((float(radius), self.std_lod if lod is None else lod, lod_count))
        return len(self.tr) - 1

    def _scene(self, tr_list, surf_list) -> S.Scene:
        n = len(tr_list)
        tr = np.zeros(n, abi.MESH_TRANSFORM)
        tr["pos"] = [t[0] for t in tr_list]
        tr["scale"] = [t[1] for t in tr_list]
        tr["orientation"] = [t[2] for t in tr_list]
        surf = np.zeros(n, abi.PRIMITIVE_SURFACE)
        surf["radius"] = [s[0] for s in surf_list]
        surf["lodOffset"] = [s[1] for s in surf_list]
        surf["lodCount"] = [s[2] for s in surf_list]
        lods = np.zeros(len(self.lods), abi.LOD_DATA)
        lods["indexCount"] = [x[0] for x in self.lods]
        lods["firstIndex"] = [x[1] for x in self.lods]
        lods["error"] = [x[2] for x in self.lods]
        objs = np.zeros(n, abi.RENDER_OBJECT)
        objs["transformId"] = np.arange(n)
        objs["surfaceId"] = np.arange(n)
        return S.Scene(objs, tr, surf, lods)

    def scene(self) -> S.Scene:
        return self._scene(self.tr, self.surf)

    def probe(self, view, mode, pyr, **obj):
        """Oracle decision (visible, LOD) for one candidate object on its own."""
        saved = (self.tr, self.surf)
        self.tr, self.surf = [], []
        self.add(**obj)
        sc = self._scene(self.tr, self.surf)
        self.tr, self.surf = saved
        return O.object_test(mode, view, sc, 0, pyr)


def constant_pyramid(width, height, values) -> O.HostPyramid:
    p = O.HostPyramid(width, height, abi.HIZ_D3D12)
    for lvl in range(p.desc.mipCount):
        p.mip(lvl)[:] = values[lvl % len(values)]
    return p


def make_kat(cam):
    zfar = 1000.0
    znear = 0.1
    view = ref_view(cam, S.fov_radians(), 1920.0, 1080.0, znear, zfar, (0.0, 0.0, 0.0), 0.0, 0.0, 960.0, 540.0)
    pyr_alt = constant_pyramid(1920, 1080, [0.0, 1.0])   # even mips pass, odd mips occlude
    pyr_all = constant_pyramid(1920, 1080, [1.0])        # everything projected and in range is occluded
    k = KatScene()
    ulps = (-2, -1, 0, 1, 2)

    def in_frustum(**obj):
        return k.probe(view, 0, None, **obj)[0] > 0

    # left/right and top/bottom planes: x (or y) one ulp either side of the boundary, both signs
    for z in (5.0, 50.0, 500.0):
        for r in (0.5, 2.0):
            for axis in (0, 1):
                def pos(x, z=z, axis=axis):
                    p = [0.0, 0.0, z]
                    p[axis] = x
                    return p
                b = bisect(lambda x, r=r, pos=pos: in_frustum(pos=pos(x), radius=r), 0.0, 4.0 * z + 10.0 * r)
                for u in ulps:
                    for sign in (1.0, -1.0):
                        k.add(pos=pos(sign * _val(b + u)), radius=r)
    # near (z + r > zNear) and far (z - r < zFar) along the view axis
    for r in (0.05, 1.0, 3.0):
        b = bisect(lambda z, r=r: in_frustum(pos=(0.0, 0.0, z), radius=r), -2.0 * r, 1.0)
        for u in ulps:
            k.add(pos=(0.0, 0.0, _val(b + u)), radius=r)
        b = bisect(lambda z, r=r: in_frustum(pos=(0.0, 0.0, z), radius=r), zfar - 10.0, zfar + 10.0)
        for u in ulps:
            k.add(pos=(0.0, 0.0, _val(b + u)), radius=r)
    # projectSphere's near guard (c.z < r + zNear): unprojected spheres are visible, projected ones
    # meet the all-occluding pyramid (small radii keep the footprint inside the mip chain)
    for r in (0.02, 0.05):
        b = bisect(lambda z, r=r: k.probe(view, 3, pyr_all, pos=(0.0, 0.0, z), radius=r)[0] > 0, znear, r + 1.0)
        assert abs(_val(b) - (r + znear)) < 1e-5, (r, _val(b))
        for u in ulps:
            k.add(pos=(0.0, 0.0, _val(b + u)), radius=r)
    # Hi-Z mip-level changes: radius sweeps at several places against the alternating pyramid
    for z, x in ((100.0, 0.0), (37.5, 11.0), (400.0, -60.0)):
        def vis(r, z=z, x=x):
            return k.probe(view, 3, pyr_alt, pos=(x, 0.0, z), radius=r)[0] > 0
        rs = np.geomspace(0.01, z * 0.5, 1500).astype(np.float32)
        vals = [vis(float(r)) for r in rs]
        for i in range(1, len(rs)):
            if vals[i] != vals[i - 1]:
                b = bisect(vis, float(rs[i - 1]), float(rs[i]))
                for u in ulps:
                    k.add(pos=(x, 0.0, z), radius=_val(b + u))
    # LOD ties: an error equal to the threshold is not below it (cullBuffers.hlsl:42-55)
    rng = np.random.default_rng(404)
    for j in range(24):
        z = float(np.float32(rng.uniform(5.0, 900.0)))
        x = float(np.float32(rng.uniform(-0.2, 0.2) * z))
        scale = float(np.float32(rng.choice([0.5, 1.0, 1.7, 3.0])))
        r = float(np.float32(rng.uniform(0.2, 3.0)))
        off = k.add_lods([0.0, 1.0, 1e30, 1e30])

        def picks_lod1(e, off=off, x=x, z=z, r=r, scale=scale):
            k.lods[off + 1] = (15000, 1000 * off + 1, float(e))
            return k.probe(view, 0, None, pos=(x, 0.0, z), radius=r, scale=scale, lod=off)[1] == off + 1

        b = bisect(picks_lod1, 1e-12, 1e6)  # the smallest error that is not below the threshold
        k.lods[off + 1] = (15000, 1000 * off + 1, 1.0)
        for u in (-1, 0, 1):
            o2 = k.add_lods([0.0, _val(b + u), _val(b + u), 1e30])
            k.add(pos=(x, 0.0, z), radius=r, scale=scale, lod=o2)
    # camera inside the sphere (distance clamps to 0), single-LOD and two-LOD chains
    k.add(pos=(0.0, 0.0, 1.0), radius=5.0)
    one = k.add_lods([0.0])
    k.add(pos=(0.0, 0.0, 50.0), radius=1.0, lod=one, lod_count=1)
    two = k.add_lods([0.0, 0.0])
    k.add(pos=(0.0, 0.0, 50.0), radius=1.0, lod=two, lod_count=2)
    sc = k.scene()
    vis = (np.arange(sc.count) % 2).astype(np.uint32)
    out = scene_arrays("", sc)
    out["visibility"] = vis
    out["view"] = vbytes(view)
    out["pyr_alt"] = pyr_alt.data.copy()
    out["pyr_all"] = pyr_all.data.copy()
    return out, sc, view, vis, {"alt": pyr_alt, "all": pyr_all}


def kat_outputs(hl, out, sc, view, vis, pyrs) -> None:
    for pname, pyr in pyrs.items():
        for kind in range(4):
            v = vis if kind in (1, 2) else None
            cnt, cmds, vis_out = run_ref_cull(hl, kind, view, sc, v, pyr if kind in (2, 3) else None)
            out[f"count_{pname}_{kind}"] = np.array([cnt], np.uint32)
            out[f"cmds_{pname}_{kind}"] = cmds
            if vis_out is not None:
                out[f"vis_{pname}_{kind}"] = vis_out


# ------------------------------------------------------------------ Vulkan form (GLSL)


def vk_ref_pyramid(gl, depth: np.ndarray) -> O.HostPyramid:
    h, w = depth.shape
    p = O.HostPyramid(w, h, abi.HIZ_VULKAN)
    gl.ref_glsl_pyramid(np.ascontiguousarray(depth, np.float32).ctypes.data, w, h, C.byref(p.desc))
    return p


def make_vk_pyramid(gl) -> dict:
    rng = np.random.default_rng(505)
    out = {}
    shapes = [(1, 3), (2, 2), (5, 7), (48, 64), (199, 333), (37, 1000)]
    depths = []
    for h, w in shapes:
        d = rng.random((h, w), dtype=np.float32)
        d[rng.random((h, w)) < 0.3] = 0.0  # cleared depth
        depths.append(d)
    # an occluder raster of the stress camera at 640 x 360 (mip 0 512 x 256)
    v = abi.view_setup(S.fov_radians(), 640.0, 360.0, S.ZNEAR, 1e4, (0.0, 0.0, 0.0), 0.0, 0.0, 512.0, 256.0)
    depths.append(O.depth_raster(v, S.make_occluders(np.random.default_rng(506), 300), 640, 360))
    for i, d in enumerate(depths):
        p = vk_ref_pyramid(gl, d)
        out[f"depth{i}"] = d
        out[f"pyr{i}"] = p.data.copy()
        out[f"mips{i}"] = np.array([p.desc.mipCount, p.desc.width, p.desc.height], np.uint32)
    out["count"] = np.array([len(depths)], np.uint32)
    return out


def run_vk_cull(gl, kind: int, view, scene, vis, pyr) -> tuple[int, np.ndarray, np.ndarray | None]:
    d, keep = O.scene_desc(scene)
    n = scene.count
    cmds = np.zeros((max(n, 1), 6), np.uint32)
    v = None if vis is None else np.ascontiguousarray(vis.copy(), np.uint32)
    cnt = gl.ref_glsl_cull(kind, C.byref(view), C.byref(d), keep[0].ctypes.data, n,
                           None if v is None else v.ctypes.data, C.byref(pyr.desc) if pyr else None, cmds.ctypes.data)
    return int(cnt), cmds[:cnt].copy(), v


def make_vk_cull(cam, gl) -> dict:
    sc = S.stress_scene(3000, seed=303, n_meshes=24, extent=300.0, n_boxes=200)
    sc.transforms["scale"][5] = 0.0
    sc.transforms["orientation"][6] = np.array([0.5, 0.5, 0.5, 0.9], np.float32)
    fov = S.fov_radians()
    pw, ph = 256.0, 128.0  # the Vulkan pyramid of a 320 x 180 depth buffer
    views = [ref_view(cam, fov, 1920.0, 1080.0, 0.1, 1e4, (0.0, 0.0, 0.0), 0.0, 0.0, pw, ph),
             ref_view(cam, fov, 1920.0, 1080.0, 0.1, 650.0, (20.0, -10.0, -300.0), 0.3, 0.1, pw, ph),
             ref_view(cam, fov, 1920.0, 1080.0, 0.1, 1e30, (0.0, 50.0, 0.0), 2.0, -0.4, pw, ph),
             ref_view(cam, fov, 1920.0, 1080.0, 0.1, 1e4, (0.0, 0.0, 0.0), 3.14159265, 0.0, pw, ph)]
    out = scene_arrays("", sc)
    out["visibility"] = sc.visibility
    out["views"] = np.stack([vbytes(v) for v in views])
    for c, v in enumerate(views):
        depth = O.depth_raster(v, sc.boxes, 320, 180)
        pyr = vk_ref_pyramid(gl, depth)
        out[f"depth{c}"] = depth
        out[f"pyr{c}"] = pyr.data.copy()
        for kind in range(3):
            vis = sc.visibility if kind in (1, 2) else None
            cnt, cmds, vis_out = run_vk_cull(gl, kind, v, sc, vis, pyr if kind == 2 else None)
            out[f"count{c}_{kind}"] = np.array([cnt], np.uint32)
            out[f"cmds{c}_{kind}"] = cmds
            if vis_out is not None:
                out[f"vis{c}_{kind}"] = vis_out
    return out


def vk_constant_pyramid(width, height, values) -> O.HostPyramid:
    p = O.HostPyramid(width, height, abi.HIZ_VULKAN)
    for lvl in range(p.desc.mipCount):
        p.mip(lvl)[:] = values[lvl % len(values)]
    return p


def make_vk_kat(cam, gl) -> dict:
    """Spheres at every Hi-Z level change of the Vulkan form: level = floor(log2(max extent)) in
    pyramid texels, clamped to [0, 16] by the sampler and to the last mip by the image. With
    constant-per-mip pyramids the footprint does not matter, so the reference's own level choice and
    clamping decide every answer."""
    znear = 0.1
    pw, ph = 1024.0, 1024.0  # the Vulkan pyramid of a 1920 x 1080 depth buffer
    view = ref_view(cam, S.fov_radians(), 1920.0, 1080.0, znear, 1e4, (0.0, 0.0, 0.0), 0.0, 0.0, pw, ph)
    pyr_alt = vk_constant_pyramid(1920, 1080, [0.0, 1.0])   # even mips pass, odd mips occlude
    pyr_top = vk_constant_pyramid(1920, 1080, [0.0] * 9 + [1.0])  # only the last mip (9) occludes
    k = KatScene()
    ulps = (-2, -1, 0, 1, 2)
    for pyr in (pyr_alt, pyr_top):
        for z, x in ((100.0, 0.0), (37.5, 11.0), (400.0, -60.0), (12.0, 2.0)):
            def vis(r, z=z, x=x, pyr=pyr):
                return k.probe(view, 3, pyr, pos=(x, 0.0, z), radius=r)[0] > 0
            rs = np.geomspace(0.001, z * 0.9, 2000).astype(np.float32)
            vals = [vis(float(r)) for r in rs]
            for i in range(1, len(rs)):
                if vals[i] != vals[i - 1]:
                    b = bisect(vis, float(rs[i - 1]), float(rs[i]))
                    for u in ulps:
                        k.add(pos=(x, 0.0, z), radius=_val(b + u))
    # spheres whose projection spans the whole screen (level past the chain) and ones right at zNear
    for r in (5.0, 50.0, 400.0):
        k.add(pos=(0.0, 0.0, r + 0.5), radius=r)
    sc = k.scene()
    vis0 = np.zeros(sc.count, np.uint32)  # nothing visible last frame: every visible object is emitted
    out = scene_arrays("", sc)
    out["view"] = vbytes(view)
    for name, pyr in (("alt", pyr_alt), ("top", pyr_top)):
        cnt, cmds, vis_out = run_vk_cull(gl, 2, view, sc, vis0, pyr)
        out[f"pyr_{name}"] = pyr.data.copy()
        out[f"count_{name}"] = np.array([cnt], np.uint32)
        out[f"cmds_{name}"] = cmds
        out[f"vis_{name}"] = vis_out
    return out, sc.count


def make_vk_clusters(cam, gl) -> dict:
    """A cluster scene whose clusters every per-cluster test of the library lets through (cluster
    spheres of radius 1e6, a zero cone axis with cutoff 127): the library's cluster cull then emits
    what the reference's object stage expands, and both are compared with these records."""
    sc = S.cluster_scene(600, seed=606, n_meshes=8, clusters_per_mesh=24, extent=200.0)
    sc.clusters["radius"] = np.float32(1e6)
    sc.clusters["coneAxis"] = 0
    sc.clusters["coneCutoff"] = 127
    v = ref_view(cam, S.fov_radians(), 1920.0, 1080.0, 0.1, 1e4, (0.0, 0.0, -50.0), 0.2, 0.05, 960.0, 540.0)
    d, keep = O.scene_desc(sc)
    cap = int(sc.lods["clusterCount"].max()) * sc.count
    dispatch = np.zeros((cap, 3), np.uint32)
    cmds = np.zeros((cap, 6), np.uint32)
    entries = C.c_uint32(0)
    cnt = gl.ref_glsl_clusters(C.byref(v), C.byref(d), keep[0].ctypes.data, sc.count, dispatch.ctypes.data,
                               C.byref(entries), cmds.ctypes.data)
    out = scene_arrays("", sc)
    out["clusters"] = sc.clusters
    out["view"] = vbytes(v)
    out["count"] = np.array([cnt], np.uint32)
    out["cmds"] = cmds[:cnt].copy()
    out["dispatch"] = dispatch[:entries.value].copy()
    return out


def main():
    cam, hl = ref_libs()
    np.savez_compressed(HERE / "camera.npz", **make_camera(cam))
    np.savez_compressed(HERE / "pyramid.npz", **make_pyramid(hl))
    np.savez_compressed(HERE / "cull.npz", **make_cull(cam, hl))
    np.savez_compressed(HERE / "instanced.npz", **make_instanced(cam, hl))
    out, sc, view, vis, pyrs = make_kat(cam)
    kat_outputs(hl, out, sc, view, vis, pyrs)
    np.savez_compressed(HERE / "kat.npz", **out)
    gl = glsl_lib()
    np.savez_compressed(HERE / "vkpyramid.npz", **make_vk_pyramid(gl))
    np.savez_compressed(HERE / "vkcull.npz", **make_vk_cull(cam, gl))
    vk_out, vk_n = make_vk_kat(cam, gl)
    np.savez_compressed(HERE / "vkkat.npz", **vk_out)
    np.savez_compressed(HERE / "vkclusters.npz", **make_vk_clusters(cam, gl))
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)
    print("kat objects", sc.count, "vulkan kat objects", vk_n)


if __name__ == "__main__":
    main()
