"""ctypes wrapper of the CPU oracle. TEST INFRASTRUCTURE ONLY (tests, smoke check, CPU baseline).

Takes and returns numpy arrays in the reference layouts; see blz_oracle.h for the arithmetic
conventions it fixes.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from blitzen_gb300.abi import LOD_INSTANCE_COUNTER, MESH_TRANSFORM, CameraViewData, Pyramid, SceneDesc

from .build import build

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        P, U = C.c_void_p, C.c_uint32
        _lib.bo_view_setup.argtypes = [P, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, P, C.c_float,
                                       C.c_float, C.c_float, C.c_float]
        _lib.bo_pyramid_layout.argtypes = [U, U, U, P]
        _lib.bo_pyramid_layout.restype = C.c_uint64
        _lib.bo_pyramid_build.argtypes = [P, P]
        _lib.bo_cull.argtypes = [C.c_int, P, P, P, U, P, P, P, U, U, P, C.c_int]
        _lib.bo_cull.restype = U
        _lib.bo_cull_instanced.argtypes = [P, P, P, U, P, P, U, U, P, U, U, P, C.c_int]
        _lib.bo_cull_instanced.restype = U
        _lib.bo_cull_clusters.argtypes = [P, P, P, U, P, P, U, U, P, P, C.c_int]
        _lib.bo_cull_clusters.restype = U
        _lib.bo_transforms_update.argtypes = [P, U, P, P, U, P]
        _lib.bo_transforms_rotate.argtypes = [P, U, P, P, C.c_float, U, P, P]
        _lib.bo_depth_raster_boxes.argtypes = [P, P, U, P, U, U]
        _lib.bo_ftou.argtypes = [C.c_float]
        _lib.bo_ftou.restype = U
        _lib.bo_floor_log2_u.argtypes = [C.c_float]
        _lib.bo_floor_log2_u.restype = U
        _lib.bo_object_test.argtypes = [C.c_int, P, P, _RenderObject, P, C.POINTER(U)]
        _lib.bo_object_test.restype = C.c_int
    return _lib


class _RenderObject(C.Structure):
    _fields_ = [("transformId", C.c_uint32), ("surfaceId", C.c_uint32)]


def _ptr(a: np.ndarray | None):
    return None if a is None else C.c_void_p(a.ctypes.data)


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


def view_setup(fov, width, height, znear, zfar, position=(0.0, 0.0, 0.0), yaw=0.0, pitch=0.0, pw=0.0, ph=0.0) -> CameraViewData:
    v = CameraViewData()
    pos = (C.c_float * 3)(*position)
    lib().bo_view_setup(C.byref(v), fov, width, height, znear, zfar, C.byref(pos), yaw, pitch, pw, ph)
    return v


def scene_desc(scene) -> tuple[SceneDesc, list]:
    keep = [np.ascontiguousarray(a) for a in (scene.objects, scene.transforms, scene.surfaces, scene.lods, scene.clusters)]
    d = SceneDesc(keep[0].ctypes.data, len(keep[0]), keep[1].ctypes.data, len(keep[1]), keep[2].ctypes.data,
                  len(keep[2]), keep[3].ctypes.data, len(keep[3]), keep[4].ctypes.data if len(keep[4]) else None,
                  len(keep[4]))
    return d, keep


class HostPyramid:
    """A pyramid in host memory: the ctypes descriptor plus the numpy storage it points to."""

    def __init__(self, depth_w: int, depth_h: int, mode: int = 0):
        self.desc = Pyramid()
        nbytes = lib().bo_pyramid_layout(depth_w, depth_h, mode, C.byref(self.desc))
        if nbytes == 0:
            raise ValueError("bad pyramid extent")
        self.data = np.zeros(nbytes // 4, np.float32)
        self.desc.data = self.data.ctypes.data

    def mip(self, level: int) -> np.ndarray:
        h, w = self.desc.mip_shape(level)
        off = self.desc.mipOffset[level]
        return self.data[off:off + w * h].reshape(h, w)


def pyramid_build(depth: np.ndarray, mode: int = 0, into: HostPyramid | None = None) -> HostPyramid:
    """Builds the pyramid of `depth` (into a caller's HostPyramid of the same extent and mode, or a new one)."""
    depth = np.ascontiguousarray(depth, dtype=np.float32)
    p = into if into is not None else HostPyramid(depth.shape[1], depth.shape[0], mode)
    lib().bo_pyramid_build(C.byref(p.desc), _ptr(depth))
    return p


def cull(mode: int, view: CameraViewData, scene, objects: np.ndarray | None = None, vis: np.ndarray | None = None,
         pyramid: HostPyramid | None = None, stride: int = 24, capacity: int | None = None, threads: int = 1,
         out: np.ndarray | None = None, desc=None):
    """Returns (count, records[min(count,capacity), stride/4] uint32, flags). vis (LATE) is updated in place.

    `out` is an optional caller buffer of at least max(capacity, 1) records of stride/4 words, and
    `desc` an optional (SceneDesc, arrays) pair from scene_desc(scene): with both, the call
    allocates nothing on the Python side."""
    d, keep = desc if desc is not None else scene_desc(scene)
    objs = keep[0] if objects is None else np.ascontiguousarray(objects)
    n = len(objs)
    cap = n if capacity is None else capacity
    if out is None:
        out = np.zeros((max(cap, 1), stride // 4), np.uint32)
    elif out.dtype != np.uint32 or out.ndim != 2 or out.shape[1] != stride // 4 or out.shape[0] < max(cap, 1) \
            or not out.flags.c_contiguous:
        raise ValueError("out must be C-contiguous uint32 [>= capacity, stride/4]")
    flags = C.c_uint32(0)
    cnt = lib().bo_cull(mode, C.byref(view), C.byref(d), _ptr(objs), n, _ptr(vis),
                        C.byref(pyramid.desc) if pyramid else None, _ptr(out), stride, cap, C.byref(flags), threads)
    return int(cnt), out[:min(cnt, cap)], int(flags.value)


def cull_instanced(view, scene, counters: np.ndarray, instance_capacity: int, slots_per_lod: int, stride: int = 24,
                   capacity: int | None = None, objects=None, threads: int = 1):
    d, keep = scene_desc(scene)
    objs = keep[0] if objects is None else np.ascontiguousarray(objects)
    cap = len(scene.lods) if capacity is None else capacity
    out = np.zeros((max(cap, 1), stride // 4), np.uint32)
    inst = np.full(max(instance_capacity, 1), 0xFFFFFFFF, np.uint32)
    ctr = np.ascontiguousarray(counters.copy())
    flags = C.c_uint32(0)
    cnt = lib().bo_cull_instanced(C.byref(view), C.byref(d), _ptr(objs), len(objs), _ptr(ctr), _ptr(inst),
                                  instance_capacity, slots_per_lod, _ptr(out), stride, cap, C.byref(flags), threads)
    return int(cnt), out[:min(cnt, cap)], ctr, inst[:instance_capacity], int(flags.value)


def cull_clusters(view, scene, pyramid: HostPyramid | None = None, stride: int = 24, capacity: int | None = None,
                  objects=None, threads: int = 1):
    d, keep = scene_desc(scene)
    objs = keep[0] if objects is None else np.ascontiguousarray(objects)
    cap = len(scene.clusters) * 0 + (capacity if capacity is not None else int(_cluster_upper_bound(scene, objs)))
    out = np.zeros((max(cap, 1), stride // 4), np.uint32)
    ids = np.zeros(max(cap, 1), np.uint32)
    flags = C.c_uint32(0)
    cnt = lib().bo_cull_clusters(C.byref(view), C.byref(d), _ptr(objs), len(objs),
                                 C.byref(pyramid.desc) if pyramid else None, _ptr(out), stride, cap, _ptr(ids),
                                 C.byref(flags), threads)
    return int(cnt), out[:min(cnt, cap)], ids[:min(cnt, cap)], int(flags.value)


def cluster_tasks(view, scene, pyramid: HostPyramid | None = None, objects=None, threads: int = 1):
    """The cluster cull in mesh-shader form, restated from the cluster records: every object with s
    surviving clusters gets one IndirectTask {first payload, ceil(s/32), 1, 1}
    (VulkanShaderHeaders/ShaderBuffers.glsl:86-92) and ceil(s/32) MeshTaskPayloads {drawId,
    meshletIndices[32]} (ShaderBuffers.glsl:203-206) holding its surviving cluster ids in order,
    0xFFFFFFFF past the last. Objects in ascending render-list order. Returns (tasks[n, 4],
    payloads[m, 33]) as uint32."""
    cap = _cluster_upper_bound(scene, _objects_of(scene, objects))
    n, recs, ids, _ = cull_clusters(view, scene, pyramid=pyramid, capacity=cap, objects=objects, threads=threads)
    obj = recs[:, 0].astype(np.int64)
    if n == 0:
        return np.zeros((0, 4), np.uint32), np.zeros((0, 33), np.uint32)
    starts = np.flatnonzero(np.r_[True, obj[1:] != obj[:-1]])
    sizes = np.diff(np.r_[starts, n])
    k = (sizes + 31) // 32
    first = np.r_[0, np.cumsum(k)[:-1]]
    tasks = np.stack([first, k, np.ones_like(k), np.ones_like(k)], axis=1).astype(np.uint32)
    payloads = np.full((int(k.sum()), 33), 0xFFFFFFFF, np.uint32)
    # survivor j of its object's run lands in payload first + j // 32, slot j % 32
    run_of = np.repeat(np.arange(len(starts)), sizes)
    j = np.arange(n) - starts[run_of]
    pi = first[run_of] + j // 32
    payloads[pi, 1 + j % 32] = ids
    payloads[:, 0] = np.repeat(obj[starts], k)
    return tasks, payloads


def _objects_of(scene, objects):
    return scene.objects if objects is None else np.ascontiguousarray(objects)


def _cluster_upper_bound(scene, objs) -> int:
    per_surface = np.zeros(len(scene.surfaces), np.int64)
    for s in range(len(scene.surfaces)):
        off, cnt = int(scene.surfaces[s]["lodOffset"]), int(scene.surfaces[s]["lodCount"])
        if cnt:
            per_surface[s] = int(scene.lods[off:off + cnt]["clusterCount"].max())
    return int(per_surface[objs["surfaceId"]].sum())


def depth_raster(view, boxes: np.ndarray, width: int, height: int) -> np.ndarray:
    boxes = np.ascontiguousarray(boxes, dtype=np.float32)
    depth = np.zeros((height, width), np.float32)
    lib().bo_depth_raster_boxes(C.byref(view), _ptr(boxes), len(boxes), _ptr(depth), width, height)
    return depth


def transforms_rotate(transforms: np.ndarray, ids: np.ndarray, axes: np.ndarray, angle: float) -> np.ndarray:
    ids = np.ascontiguousarray(ids, np.uint32)
    axes = np.ascontiguousarray(axes, np.float32)
    dst = np.zeros(len(ids), MESH_TRANSFORM)
    flags = C.c_uint32(0)
    lib().bo_transforms_rotate(_ptr(transforms), len(transforms), _ptr(ids), _ptr(axes), angle, len(ids), _ptr(dst),
                               C.byref(flags))
    return dst


def new_counters(scene, slots_per_lod: int = 100_000) -> np.ndarray:
    """LodInstanceCounter table with instanceOffset = lodIndex * slots (blitzenMeshes.cpp:160)."""
    c = np.zeros(len(scene.lods), LOD_INSTANCE_COUNTER)
    c["instanceOffset"] = np.arange(len(scene.lods), dtype=np.uint64) * slots_per_lod
    return c


def ftou(x: float) -> int:
    return int(lib().bo_ftou(x))


def floor_log2_u(x: float) -> int:
    return int(lib().bo_floor_log2_u(x))


def object_test(mode: int, view: CameraViewData, scene, obj_index: int, pyramid: HostPyramid | None = None):
    """One object's decision: (visible 0/1 or -1 on a bad index, chosen global LOD index or None)."""
    d, keep = scene_desc(scene)
    o = keep[0][obj_index]
    lod = C.c_uint32(0xFFFFFFFF)
    v = lib().bo_object_test(mode, C.byref(view), C.byref(d), _RenderObject(int(o["transformId"]), int(o["surfaceId"])),
                             C.byref(pyramid.desc) if pyramid else None, C.byref(lod))
    return int(v), (int(lod.value) if v > 0 else None)
