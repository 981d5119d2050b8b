"""ctypes bindings of libblz_cull.so (include/blz_cull.h) and numpy mirrors of the buffer layouts.

The numpy dtypes have the byte layout of the reference structs (include/blz_types.h), so arrays
built here can be handed to the library (and to the reference's own CPU code) unchanged.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_lib" / "libblz_cull.so"

# ----------------------------------------------------------------------------- numpy layouts

RENDER_OBJECT = np.dtype([("transformId", "<u4"), ("surfaceId", "<u4")])
MESH_TRANSFORM = np.dtype([("pos", "<f4", 3), ("scale", "<f4"), ("orientation", "<f4", 4)])
PRIMITIVE_SURFACE = np.dtype([("center", "<f4", 3), ("radius", "<f4"), ("materialId", "<u4"),
                              ("lodOffset", "<u4"), ("lodCount", "<u4"), ("vertexOffset", "<u4")])
LOD_DATA = np.dtype([("indexCount", "<u4"), ("firstIndex", "<u4"), ("clusterOffset", "<u4"),
                     ("clusterCount", "<u4"), ("error", "<f4"), ("padding", "<u4", 3)])
LOD_INSTANCE_COUNTER = np.dtype([("instanceOffset", "<u4"), ("instanceCount", "<u4")])
CLUSTER = np.dtype({
    "names": ["center", "radius", "coneAxis", "coneCutoff", "dataOffset", "vertexCount", "triangleCount"],
    "formats": [("<f4", 3), "<f4", ("i1", 3), "i1", "<u4", "u1", "u1"],
    "offsets": [0, 12, 16, 19, 20, 24, 25],
    "itemsize": 32,
})
INDIRECT_TASK = np.dtype([("taskId", "<u4"), ("groupCountX", "<u4"), ("groupCountY", "<u4"), ("groupCountZ", "<u4")])
MESH_TASK_PAYLOAD = np.dtype([("drawId", "<u4"), ("meshletIndices", "<u4", 32)])
for _dt, _n in ((RENDER_OBJECT, 8), (MESH_TRANSFORM, 32), (PRIMITIVE_SURFACE, 32), (LOD_DATA, 32),
                (LOD_INSTANCE_COUNTER, 8), (CLUSTER, 32), (INDIRECT_TASK, 16), (MESH_TASK_PAYLOAD, 132)):
    assert _dt.itemsize == _n

STRIDE_VULKAN = 24
STRIDE_D3D12 = 32
HIZ_D3D12 = 0
HIZ_VULKAN = 1
MODE_FRUSTUM, MODE_FIRST, MODE_LATE, MODE_TEMPORAL = 0, 1, 2, 3
SCENE_COPY_FROM_HOST, SCENE_BORROW_DEVICE = 0, 1
NOALLOC_MAX_OBJECTS = 1 << 20
NO_MESHLET = 0xFFFFFFFF

FLAG_COMMAND_OVERFLOW = 1
FLAG_INSTANCE_OVERFLOW = 2
FLAG_BAD_INDEX = 4
FLAG_TIMEOUT = 8

STATUS = {0: "OK", 1: "INVALID_ARGUMENT", 2: "CAPACITY", 3: "OUT_OF_MEMORY", 4: "TIMEOUT", 5: "CUDA",
          6: "BAD_INDEX", 7: "NOT_READY", 8: "NO_SCENE"}

# ----------------------------------------------------------------------------- ctypes structs


class CameraViewData(C.Structure):
    _fields_ = [("viewMatrix", C.c_float * 16), ("projectionViewMatrix", C.c_float * 16),
                ("position", C.c_float * 3), ("frustumRight", C.c_float), ("frustumLeft", C.c_float),
                ("frustumTop", C.c_float), ("frustumBottom", C.c_float), ("proj0", C.c_float),
                ("proj5", C.c_float), ("zNear", C.c_float), ("zFar", C.c_float),
                ("pyramidWidth", C.c_float), ("pyramidHeight", C.c_float), ("lodTarget", C.c_float),
                ("_pad", C.c_uint8 * 72)]

    def to_bytes(self) -> bytes:
        return bytes(memoryview(self))

    @classmethod
    def from_bytes(cls, b: bytes) -> "CameraViewData":
        v = cls()
        C.memmove(C.addressof(v), b, 256)
        return v


assert C.sizeof(CameraViewData) == 256


class SceneDesc(C.Structure):
    _fields_ = [("renderObjects", C.c_void_p), ("renderObjectCount", C.c_uint32),
                ("transforms", C.c_void_p), ("transformCount", C.c_uint32),
                ("surfaces", C.c_void_p), ("surfaceCount", C.c_uint32),
                ("lods", C.c_void_p), ("lodCount", C.c_uint32),
                ("clusters", C.c_void_p), ("clusterCount", C.c_uint32)]


class Pyramid(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32),
                ("mipCount", C.c_uint32), ("mode", C.c_uint32), ("depthWidth", C.c_uint32),
                ("depthHeight", C.c_uint32), ("mipOffset", C.c_uint32 * 16)]

    def mip_shape(self, level: int) -> tuple[int, int]:
        return max(1, self.height >> level), max(1, self.width >> level)


class RenderList(C.Structure):
    _fields_ = [("objects", C.c_void_p), ("count", C.c_uint32)]


class CullTarget(C.Structure):
    _fields_ = [("commands", C.c_void_p), ("stride", C.c_uint32), ("capacity", C.c_uint32),
                ("drawCount", C.c_void_p)]


class TaskTarget(C.Structure):
    _fields_ = [("tasks", C.c_void_p), ("payloads", C.c_void_p), ("taskCapacity", C.c_uint32),
                ("payloadCapacity", C.c_uint32), ("taskCount", C.c_void_p), ("payloadCount", C.c_void_p)]


class BatchView(C.Structure):
    _fields_ = [("view", CameraViewData), ("list", RenderList), ("mode", C.c_uint32),
                ("reserved0", C.c_uint32), ("visibility", C.c_void_p), ("pyramid", C.POINTER(Pyramid)),
                ("target", CullTarget), ("dynamicTransforms", C.c_void_p), ("dynamicCount", C.c_uint32),
                ("reserved1", C.c_uint32), ("_tail", C.c_uint8 * 176)]  # C pads to the view's 256-byte alignment


class LaunchShape(C.Structure):
    _fields_ = [("threadsPerBlock", C.c_uint32), ("objectsPerThread", C.c_uint32),
                ("blocksPerSm", C.c_uint32), ("chunkObjects", C.c_uint32)]


class ServeConfig(C.Structure):
    _fields_ = [("outputPoolBytes", C.c_uint64), ("maxInFlight", C.c_uint32), ("maxBatchViews", C.c_uint32),
                ("dynamicCount", C.c_uint32), ("stride", C.c_uint32)]


class ServeRequest(C.Structure):
    _fields_ = [("view", CameraViewData), ("list", RenderList), ("mode", C.c_uint32),
                ("rotateCount", C.c_uint32), ("pyramid", C.POINTER(Pyramid)), ("rotateAxes", C.c_void_p),
                ("rotateAngle", C.c_float), ("copyToHost", C.c_uint32), ("_tail", C.c_uint8 * 208)]


class ServeResult(C.Structure):
    _fields_ = [("status", C.c_uint32), ("drawCount", C.c_uint32), ("deviceRecords", C.c_void_p),
                ("hostRecords", C.c_void_p), ("arrivalSeconds", C.c_double), ("completeSeconds", C.c_double)]


class ServeStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("batches", C.c_uint64),
                ("objects", C.c_uint64), ("p50Ms", C.c_double), ("p99Ms", C.c_double), ("meanMs", C.c_double),
                ("maxMs", C.c_double), ("peakOutputBytes", C.c_uint64), ("maxConcurrentBatches", C.c_uint32),
                ("maxBatchSize", C.c_uint32)]


# Sizes of the C structs (checked against a compiled probe in the tests).
C_SIZES = {"BlzBatchView": 512, "BlzServeRequest": 512, "BlzServeResult": 40, "BlzServeStats": 80,
           "BlzServeConfig": 24, "BlzPyramid": 96, "BlzSceneDesc": 80, "BlzCullTarget": 24, "BlzRenderList": 16,
           "BlzLaunchShape": 16, "BlzCameraViewData": 256, "BlzTaskTarget": 40}
CTYPES_OF = {"BlzBatchView": BatchView, "BlzServeRequest": ServeRequest, "BlzServeResult": ServeResult,
             "BlzServeStats": ServeStats, "BlzServeConfig": ServeConfig, "BlzPyramid": Pyramid,
             "BlzSceneDesc": SceneDesc, "BlzCullTarget": CullTarget, "BlzRenderList": RenderList,
             "BlzLaunchShape": LaunchShape, "BlzCameraViewData": CameraViewData, "BlzTaskTarget": TaskTarget}
for _name, _cls in CTYPES_OF.items():
    assert C.sizeof(_cls) == C_SIZES[_name], (_name, C.sizeof(_cls))

# ----------------------------------------------------------------------------- function table

_P = C.c_void_p
_U32 = C.c_uint32
_I = C.c_int
_PROTOS = {
    "blz_ctx_create": (_I, [_I, C.POINTER(_P)]),
    "blz_ctx_destroy": (_I, [_P]),
    "blz_last_error": (C.c_char_p, []),
    "blz_version": (C.c_char_p, []),
    "blz_ctx_check": (_I, [_P, _P, C.POINTER(_U32)]),
    "blz_ctx_set_wait_limit": (_I, [_P, _U32]),
    "blz_ctx_debug_advance_ticket": (_I, [_P, _U32, _P]),
    "blz_ctx_debug_skip_frame_tiles": (_I, [_P, _U32, _P]),
    "blz_ctx_launch_count": (C.c_uint64, [_P]),
    "blz_scene_upload": (_I, [_P, C.POINTER(SceneDesc), _U32, _P]),
    "blz_scene_device_tables": (_I, [_P, C.POINTER(SceneDesc)]),
    "blz_transforms_update": (_I, [_P, _P, _P, _U32, _P]),
    "blz_transforms_update_device": (_I, [_P, _P, _P, _U32, _P]),
    "blz_transforms_rotate": (_I, [_P, _P, _P, C.c_float, _U32, _P, _P]),
    "blz_scene_bind_dynamic": (_I, [_P, _P, _U32]),
    "blz_pyramid_layout": (C.c_uint64, [_U32, _U32, _U32, C.POINTER(Pyramid)]),
    "blz_pyramid_build": (_I, [_P, C.POINTER(Pyramid), _P, _P]),
    "blz_depth_raster_boxes": (_I, [_P, C.POINTER(CameraViewData), _P, _U32, _P, _U32, _U32, _P]),
    "blz_cull_frustum": (_I, [_P, C.POINTER(CameraViewData), RenderList, C.POINTER(CullTarget), _P]),
    "blz_cull_frustum_noalloc": (_I, [_P, C.POINTER(CameraViewData), RenderList, C.POINTER(CullTarget), _P]),
    "blz_cull_first": (_I, [_P, C.POINTER(CameraViewData), RenderList, _P, C.POINTER(CullTarget), _P]),
    "blz_cull_late": (_I, [_P, C.POINTER(CameraViewData), RenderList, _P, C.POINTER(Pyramid), C.POINTER(CullTarget), _P]),
    "blz_frame_first": (_I, [_P, C.POINTER(CameraViewData), RenderList, _P, C.POINTER(CullTarget), _P]),
    "blz_frame_late": (_I, [_P, C.POINTER(Pyramid), C.POINTER(CullTarget), _P]),
    "blz_cull_frame": (_I, [_P, C.POINTER(CameraViewData), RenderList, _P, _P, C.POINTER(Pyramid), C.POINTER(CullTarget),
                            C.POINTER(CullTarget), _P]),
    "blz_cull_temporal": (_I, [_P, C.POINTER(CameraViewData), RenderList, C.POINTER(Pyramid), C.POINTER(CullTarget), _P]),
    "blz_cull_instanced": (_I, [_P, C.POINTER(CameraViewData), RenderList, _P, _P, _U32, _U32, C.POINTER(CullTarget), _P]),
    "blz_cull_clusters": (_I, [_P, C.POINTER(CameraViewData), RenderList, C.POINTER(Pyramid), C.POINTER(CullTarget), _P, _P]),
    "blz_cull_cluster_tasks": (_I, [_P, C.POINTER(CameraViewData), RenderList, C.POINTER(Pyramid), C.POINTER(TaskTarget), _P]),
    "blz_cull_batch": (_I, [_P, C.POINTER(BatchView), _U32, _P]),
    "blz_cull_batch_per_view": (_I, [_P, C.POINTER(BatchView), _U32, _P]),
    "blz_batch_graph_create": (_I, [_P, C.POINTER(BatchView), _U32, _P, C.POINTER(_P)]),
    "blz_batch_graph_set_view": (_I, [_P, _U32, C.POINTER(CameraViewData)]),
    "blz_batch_graph_launch": (_I, [_P, _P]),
    "blz_batch_graph_destroy": (_I, [_P]),
    "blz_get_launch_shape": (_I, [_P, C.POINTER(LaunchShape)]),
    "blz_set_launch_shape": (_I, [_P, C.POINTER(LaunchShape)]),
    "blz_autotune_batch": (_I, [_P, C.POINTER(BatchView), _U32, _U32, _P, C.POINTER(LaunchShape), C.POINTER(C.c_float)]),
    "blz_autotune_single": (_I, [_P, C.POINTER(CameraViewData), RenderList, _U32, _P, C.POINTER(Pyramid),
                                 C.POINTER(CullTarget), _U32, _P, C.POINTER(LaunchShape), C.POINTER(C.c_float)]),
    "blz_capture_begin": (_I, [_P, _P]),
    "blz_capture_end": (_I, [_P, _P, C.POINTER(_P), C.POINTER(_U32)]),
    "blz_graph_launch": (_I, [_P, _P]),
    "blz_graph_destroy": (_I, [_P]),
    "blz_serve_create": (_I, [_P, C.POINTER(ServeConfig), C.POINTER(_P)]),
    "blz_serve_submit": (_I, [_P, C.POINTER(ServeRequest), C.POINTER(C.c_uint64)]),
    "blz_serve_wait": (_I, [_P, C.c_uint64, _U32, C.POINTER(ServeResult)]),
    "blz_serve_release": (_I, [_P, C.c_uint64]),
    "blz_serve_stats": (_I, [_P, C.POINTER(ServeStats)]),
    "blz_serve_destroy": (_I, [_P]),
    "blz_view_setup": (_I, [C.POINTER(CameraViewData), C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                            C.POINTER(C.c_float * 3), C.c_float, C.c_float, C.c_float, C.c_float]),
}


class BlzError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: {STATUS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads the in-tree library (raises if it has not been built: there is no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: build it with `python -m blitzen_gb300.build` or __graft_entry__.build()")
    lib = C.CDLL(str(p))
    for name, (res, args) in _PROTOS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def exported_names() -> list[str]:
    return list(_PROTOS)


def check(rc: int, where: str) -> None:
    if rc != 0:
        msg = load().blz_last_error().decode(errors="replace")
        raise BlzError(rc, where, msg)


def view_setup(fov: float, width: float, height: float, znear: float, zfar: float, position=(0.0, 0.0, 0.0),
               yaw: float = 0.0, pitch: float = 0.0, pyramid_width: float = 0.0,
               pyramid_height: float = 0.0) -> CameraViewData:
    """The cull uniform of a camera, built by the library (host code, no GPU needed)."""
    v = CameraViewData()
    pos = (C.c_float * 3)(*position)
    check(load().blz_view_setup(C.byref(v), fov, width, height, znear, zfar, C.byref(pos), yaw, pitch,
                                pyramid_width, pyramid_height), "blz_view_setup")
    return v


def pyramid_layout(depth_w: int, depth_h: int, mode: int = HIZ_D3D12) -> tuple[Pyramid, int]:
    p = Pyramid()
    nbytes = load().blz_pyramid_layout(depth_w, depth_h, mode, C.byref(p))
    if nbytes == 0:
        raise BlzError(1, "blz_pyramid_layout", f"bad extent {depth_w}x{depth_h} mode {mode}")
    return p, int(nbytes)
