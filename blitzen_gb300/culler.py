"""Host-side mirror of the reference renderer's cull interface, over libblz_cull.so.

The reference reaches its cull through renderer members (SetupForRendering, UpdateObjectTransform,
DrawFrame; src/Renderer/BlitzenVulkan/vulkanRenderer.h:20-40, src/Renderer/BlitzenDX12/dx12Renderer.h:22-43)
and static dispatch helpers (DrawCullFirstPass, GenerateDepthPyramid, DrawCullOcclusionPass,
DrawInstanceCullPass, PreClusterDrawCull/ClusterCull; vulkanDraw.cpp:107-622, dx12Draw.cpp:114-415).
`Culler` offers those operations by the same names, with device buffers held in torch tensors
(torch is only the allocator and the stream here; every pass is a libblz_cull kernel).

Errors: the reference returns 0 and logs; here every failing call raises `BlzError` with the
library's message. There is no CPU fallback: a missing library is an error.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import abi
from .abi import BlzError, CameraViewData, CullTarget, Pyramid, RenderList, SceneDesc, check
from .scenes import Scene


def _stream_ptr(stream: torch.cuda.Stream | None) -> C.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _dev_u32(n: int, device) -> torch.Tensor:
    return torch.zeros(max(int(n), 1), dtype=torch.int32, device=device)


def to_device(a: np.ndarray, device) -> torch.Tensor:
    """A numpy array's bytes in a device tensor (int32 words when the size allows, else bytes)."""
    raw = np.ascontiguousarray(a).view(np.uint8).reshape(-1)
    if raw.nbytes % 4 == 0:
        return torch.from_numpy(raw.view(np.int32).copy()).to(device)
    return torch.from_numpy(raw.copy()).to(device)


@dataclass
class Target:
    """Indirect-command output (binding 7 / u0) and its draw count (binding 9 / u1)."""
    commands: torch.Tensor
    count: torch.Tensor
    stride: int
    capacity: int

    @classmethod
    def alloc(cls, capacity: int, stride: int = abi.STRIDE_VULKAN, device="cuda") -> "Target":
        words = max(int(capacity), 1) * stride // 4
        return cls(torch.zeros(words, dtype=torch.int32, device=device), _dev_u32(1, device), stride, int(capacity))

    def ctype(self) -> CullTarget:
        return CullTarget(self.commands.data_ptr(), self.stride, self.capacity, self.count.data_ptr())

    def read(self) -> tuple[int, np.ndarray]:
        """(drawCount, records[min(count, capacity), stride/4] as uint32)."""
        n = int(self.count.cpu().numpy().view(np.uint32)[0])
        m = min(n, self.capacity)
        recs = self.commands[: m * self.stride // 4].cpu().numpy().view(np.uint32).reshape(m, self.stride // 4)
        return n, recs


@dataclass
class TaskTarget:
    """Mesh-shader output of the cluster cull: IndirectTask records (ShaderBuffers.glsl:86-92), their
    MeshTaskPayloads (ShaderBuffers.glsl:203-206) and the two counts."""
    tasks: torch.Tensor
    payloads: torch.Tensor
    counts: torch.Tensor  # [taskCount, payloadCount]
    task_capacity: int
    payload_capacity: int

    @classmethod
    def alloc(cls, task_capacity: int, payload_capacity: int, device="cuda") -> "TaskTarget":
        return cls(torch.zeros(max(int(task_capacity), 1) * 4, dtype=torch.int32, device=device),
                   torch.zeros(max(int(payload_capacity), 1) * 33, dtype=torch.int32, device=device),
                   _dev_u32(2, device), int(task_capacity), int(payload_capacity))

    def ctype(self) -> abi.TaskTarget:
        return abi.TaskTarget(self.tasks.data_ptr(), self.payloads.data_ptr(), self.task_capacity,
                              self.payload_capacity, self.counts.data_ptr(), self.counts.data_ptr() + 4)

    def read(self) -> tuple[int, int, np.ndarray, np.ndarray]:
        """(taskCount, payloadCount, tasks[n, 4], payloads[m, 33]) as uint32, cut to the capacities."""
        nt, np_ = (int(x) for x in self.counts.cpu().numpy().view(np.uint32)[:2])
        mt, mp = min(nt, self.task_capacity), min(np_, self.payload_capacity)
        tasks = self.tasks[: mt * 4].cpu().numpy().view(np.uint32).reshape(mt, 4)
        payloads = self.payloads[: mp * 33].cpu().numpy().view(np.uint32).reshape(mp, 33)
        return nt, np_, tasks, payloads


class DevicePyramid:
    """A Hi-Z pyramid in device memory with its descriptor (BlzPyramid)."""

    def __init__(self, depth_w: int, depth_h: int, mode: int = abi.HIZ_D3D12, device="cuda"):
        self.desc, nbytes = abi.pyramid_layout(depth_w, depth_h, mode)
        self.storage = torch.zeros(nbytes // 4, dtype=torch.float32, device=device)
        self.desc.data = self.storage.data_ptr()

    @property
    def extent(self) -> tuple[int, int]:
        return self.desc.width, self.desc.height

    def mip(self, level: int) -> np.ndarray:
        h, w = self.desc.mip_shape(level)
        off = self.desc.mipOffset[level]
        return self.storage[off: off + w * h].cpu().numpy().reshape(h, w)


class Graph:
    """A recorded sequence of library calls (blz_capture_begin / blz_capture_end)."""

    def __init__(self, lib, handle, kernels: int):
        self.lib, self.handle, self.kernels = lib, handle, kernels

    def launch(self, stream=None) -> None:
        check(self.lib.blz_graph_launch(self.handle, _stream_ptr(stream)), "blz_graph_launch")

    def close(self) -> None:
        if self.handle:
            self.lib.blz_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Culler:
    """One library context: resident scene tables, scratch and status word for one stream."""

    def __init__(self, device: int = 0):
        if not torch.cuda.is_available():
            raise RuntimeError("libblz_cull needs a CUDA device")
        self.lib = abi.load()
        self.device = torch.device("cuda", device)
        torch.cuda.set_device(self.device)
        h = C.c_void_p()
        check(self.lib.blz_ctx_create(device, C.byref(h)), "blz_ctx_create")
        self.ctx = h
        self._keep: list[torch.Tensor] = []
        self.scene_count = 0

    def close(self) -> None:
        if self.ctx:
            self.lib.blz_ctx_destroy(self.ctx)
            self.ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ scene

    def setup_for_rendering(self, scene: Scene, stream=None) -> None:
        """Makes the scene's tables resident (SetupForRendering / StaticBuffersInit)."""
        tens = [to_device(a, self.device) if len(a) else None for a in
                (scene.objects, scene.transforms, scene.surfaces, scene.lods, scene.clusters)]
        self._keep = [t for t in tens if t is not None]
        ptr = [t.data_ptr() if t is not None else None for t in tens]
        desc = SceneDesc(ptr[0], scene.count, ptr[1], len(scene.transforms), ptr[2], len(scene.surfaces),
                         ptr[3], len(scene.lods), ptr[4], len(scene.clusters))
        torch.cuda.synchronize(self.device)
        check(self.lib.blz_scene_upload(self.ctx, C.byref(desc), abi.SCENE_BORROW_DEVICE, _stream_ptr(stream)),
              "blz_scene_upload")
        self.scene_count = scene.count
        self.scene_tensors = tens

    def update_object_transform(self, ids: np.ndarray, transforms: np.ndarray, stream=None) -> None:
        """UpdateObjectTransform for many ids (host arrays, staged through pinned memory)."""
        ids = np.ascontiguousarray(ids, np.uint32)
        tr = np.ascontiguousarray(transforms)
        check(self.lib.blz_transforms_update(self.ctx, ids.ctypes.data, tr.ctypes.data, len(ids), _stream_ptr(stream)),
              "blz_transforms_update")

    def update_object_transform_device(self, ids: torch.Tensor, transforms: torch.Tensor, stream=None) -> None:
        """UpdateObjectTransform from device-accessible buffers (device memory, or pinned host memory
        the kernel reads directly); recordable in a graph."""
        check(self.lib.blz_transforms_update_device(self.ctx, ids.data_ptr(), transforms.data_ptr(),
                                                    ids.numel(), _stream_ptr(stream)), "blz_transforms_update_device")

    def bind_dynamic_transforms(self, rows: torch.Tensor | None) -> None:
        """Transforms [0, n) read from `rows` (n MeshTransform rows in device or pinned host memory)
        by every later cull; None unbinds. The reference's dynamic objects are transforms [0, 1000)
        rewritten each frame through a mapped staging buffer (blitRender.h:10, vulkanDraw.cpp:46-60)."""
        if rows is None:
            check(self.lib.blz_scene_bind_dynamic(self.ctx, None, 0), "blz_scene_bind_dynamic")
        else:
            check(self.lib.blz_scene_bind_dynamic(self.ctx, rows.data_ptr(), rows.numel() * rows.element_size() // 32),
                  "blz_scene_bind_dynamic")

    def rotate_transforms(self, ids: torch.Tensor, axes: torch.Tensor, angle: float, dst: torch.Tensor, stream=None):
        check(self.lib.blz_transforms_rotate(self.ctx, ids.data_ptr(), axes.data_ptr(), angle, ids.numel(),
                                             dst.data_ptr(), _stream_ptr(stream)), "blz_transforms_rotate")

    # ------------------------------------------------------------------ passes

    @staticmethod
    def _list(objects: torch.Tensor | None, count: int | None) -> RenderList:
        if objects is None:
            return RenderList(None, count or 0)
        return RenderList(objects.data_ptr(), count if count is not None else objects.numel() * 4 // 8)

    def draw_cull(self, view: CameraViewData, target: Target, objects=None, count=None, stream=None) -> None:
        """Frustum + LOD (TransparentDrawCull / drawCull.cs.hlsl)."""
        t = target.ctype()
        check(self.lib.blz_cull_frustum(self.ctx, C.byref(view), self._list(objects, count), C.byref(t),
                                        _stream_ptr(stream)), "blz_cull_frustum")

    def draw_cull_first_pass(self, view, visibility: torch.Tensor, target: Target, objects=None, count=None, stream=None):
        """Occlusion pass 1 (InitialDrawCull / drawOccFirst)."""
        t = target.ctype()
        check(self.lib.blz_cull_first(self.ctx, C.byref(view), self._list(objects, count), visibility.data_ptr(),
                                      C.byref(t), _stream_ptr(stream)), "blz_cull_first")

    def generate_depth_pyramid(self, pyramid: DevicePyramid, depth: torch.Tensor, stream=None) -> None:
        check(self.lib.blz_pyramid_build(self.ctx, C.byref(pyramid.desc), depth.data_ptr(), _stream_ptr(stream)),
              "blz_pyramid_build")

    def draw_cull_occlusion_pass(self, view, visibility: torch.Tensor, pyramid: DevicePyramid, target: Target,
                                 objects=None, count=None, stream=None):
        """Occlusion pass 2 (LateDrawCull / drawOccLate)."""
        t = target.ctype()
        check(self.lib.blz_cull_late(self.ctx, C.byref(view), self._list(objects, count), visibility.data_ptr(),
                                     C.byref(pyramid.desc), C.byref(t), _stream_ptr(stream)), "blz_cull_late")

    def frame_first_pass(self, view, visibility: torch.Tensor, target: Target, objects=None, count=None, stream=None):
        """Pass 1 of a kept frame (blz_frame_first): pass 1's records, and the frustum survivors kept
        for frame_occlusion_pass."""
        t = target.ctype()
        check(self.lib.blz_frame_first(self.ctx, C.byref(view), self._list(objects, count), visibility.data_ptr(),
                                       C.byref(t), _stream_ptr(stream)), "blz_frame_first")

    def frame_occlusion_pass(self, pyramid: DevicePyramid, target: Target, stream=None):
        """Pass 2 of the kept frame (blz_frame_late): the kept survivors against the pyramid."""
        t = target.ctype()
        check(self.lib.blz_frame_late(self.ctx, C.byref(pyramid.desc), C.byref(t), _stream_ptr(stream)),
              "blz_frame_late")

    def cull_frame(self, view, visibility: torch.Tensor, depth: torch.Tensor | None, pyramid: DevicePyramid,
                   target1: Target, target2: Target, objects=None, count=None, stream=None):
        """Both occlusion passes and the pyramid of one frame in one call (blz_cull_frame). depth None
        uses the pyramid as it stands instead of building it."""
        a, b = target1.ctype(), target2.ctype()
        check(self.lib.blz_cull_frame(self.ctx, C.byref(view), self._list(objects, count), visibility.data_ptr(),
                                      depth.data_ptr() if depth is not None else None, C.byref(pyramid.desc),
                                      C.byref(a), C.byref(b), _stream_ptr(stream)), "blz_cull_frame")

    def draw_cull_temporal(self, view, pyramid: DevicePyramid, target: Target, objects=None, count=None, stream=None):
        t = target.ctype()
        check(self.lib.blz_cull_temporal(self.ctx, C.byref(view), self._list(objects, count), C.byref(pyramid.desc),
                                         C.byref(t), _stream_ptr(stream)), "blz_cull_temporal")

    def draw_instance_cull_pass(self, view, counters: torch.Tensor, instances: torch.Tensor, slots_per_lod: int,
                                target: Target, objects=None, count=None, stream=None):
        t = target.ctype()
        check(self.lib.blz_cull_instanced(self.ctx, C.byref(view), self._list(objects, count), counters.data_ptr(),
                                          instances.data_ptr(), instances.numel(), slots_per_lod, C.byref(t),
                                          _stream_ptr(stream)), "blz_cull_instanced")

    def cluster_cull(self, view, target: Target, pyramid: DevicePyramid | None = None,
                     cluster_ids: torch.Tensor | None = None, objects=None, count=None, stream=None):
        t = target.ctype()
        check(self.lib.blz_cull_clusters(self.ctx, C.byref(view), self._list(objects, count),
                                         C.byref(pyramid.desc) if pyramid else None, C.byref(t),
                                         cluster_ids.data_ptr() if cluster_ids is not None else None,
                                         _stream_ptr(stream)), "blz_cull_clusters")

    def cluster_task_cull(self, view, target: TaskTarget, pyramid: DevicePyramid | None = None, objects=None,
                          count=None, stream=None):
        """The cluster cull in mesh-shader form (the reference's disabled OpaqueMeshShader path,
        vulkanDraw.cpp:425-436, fed by culled meshlets)."""
        t = target.ctype()
        check(self.lib.blz_cull_cluster_tasks(self.ctx, C.byref(view), self._list(objects, count),
                                              C.byref(pyramid.desc) if pyramid else None, C.byref(t),
                                              _stream_ptr(stream)), "blz_cull_cluster_tasks")

    def raster_boxes(self, view, boxes: torch.Tensor, depth: torch.Tensor, width: int, height: int, stream=None):
        check(self.lib.blz_depth_raster_boxes(self.ctx, C.byref(view), boxes.data_ptr(), boxes.numel() // 6,
                                              depth.data_ptr(), width, height, _stream_ptr(stream)),
              "blz_depth_raster_boxes")

    # ------------------------------------------------------------------ recorded frames

    def capture_begin(self, stream=None) -> None:
        """Starts recording this context's calls on `stream` (a non-default stream) into a graph."""
        check(self.lib.blz_capture_begin(self.ctx, _stream_ptr(stream)), "blz_capture_begin")

    def capture_end(self, stream=None) -> "Graph":
        g, k = C.c_void_p(), C.c_uint32(0)
        check(self.lib.blz_capture_end(self.ctx, _stream_ptr(stream), C.byref(g), C.byref(k)), "blz_capture_end")
        return Graph(self.lib, g, int(k.value))

    # ------------------------------------------------------------------ launch shape

    def set_launch_shape(self, threads: int, objects_per_thread: int, blocks_per_sm: int = 0,
                         chunk_objects: int = 0) -> None:
        """The batch launch shape (and the single-view one where it has that shape); forgets the
        autotuners' cached choices (blz_set_launch_shape)."""
        check(self.lib.blz_set_launch_shape(self.ctx, C.byref(abi.LaunchShape(threads, objects_per_thread,
                                                                              blocks_per_sm, chunk_objects))),
              "blz_set_launch_shape")

    def launch_shape(self) -> dict:
        s = abi.LaunchShape()
        check(self.lib.blz_get_launch_shape(self.ctx, C.byref(s)), "blz_get_launch_shape")
        return {"threads": s.threadsPerBlock, "objects_per_thread": s.objectsPerThread, "blocks_per_sm": s.blocksPerSm,
                "chunk_objects": s.chunkObjects or 512}

    def autotune_single(self, view, mode: int, target: Target, visibility: torch.Tensor | None = None,
                        pyramid: DevicePyramid | None = None, objects=None, count=None, repeats: int = 3,
                        stream=None) -> tuple[dict, float]:
        """Times every single-view shape on this pass and caches the fastest for the list's size and the
        pass (blz_autotune_single); returns (shape, microseconds). The visibility is left as it was."""
        t = target.ctype()
        best, us = abi.LaunchShape(), C.c_float(0)
        check(self.lib.blz_autotune_single(self.ctx, C.byref(view), self._list(objects, count), mode,
                                           visibility.data_ptr() if visibility is not None else None,
                                           C.byref(pyramid.desc) if pyramid else None, C.byref(t), repeats,
                                           _stream_ptr(stream), C.byref(best), C.byref(us)), "blz_autotune_single")
        return ({"threads": best.threadsPerBlock, "objects_per_thread": best.objectsPerThread,
                 "chunk_objects": best.chunkObjects}, float(us.value))

    # ------------------------------------------------------------------ status

    def check(self, stream=None) -> int:
        """Synchronises and returns the device status flags (raises on overflow / bad index / timeout)."""
        f = C.c_uint32(0)
        rc = self.lib.blz_ctx_check(self.ctx, _stream_ptr(stream), C.byref(f))
        if rc != 0:
            raise BlzError(rc, "blz_ctx_check", self.lib.blz_last_error().decode())
        return int(f.value)

    def flags(self, stream=None) -> int:
        """Like check(), but returns the flags instead of raising."""
        f = C.c_uint32(0)
        self.lib.blz_ctx_check(self.ctx, _stream_ptr(stream), C.byref(f))
        return int(f.value)

    def set_wait_limit(self, polls: int) -> None:
        """Polls of one state before a device-side wait gives up (0: the default)."""
        check(self.lib.blz_ctx_set_wait_limit(self.ctx, polls), "blz_ctx_set_wait_limit")

    def debug_advance_ticket(self, n: int, stream=None) -> None:
        """Test hook: the next ticket-taking launch starts past n places, so its waits run out."""
        check(self.lib.blz_ctx_debug_advance_ticket(self.ctx, n, _stream_ptr(stream)), "blz_ctx_debug_advance_ticket")

    def debug_skip_frame_tiles(self, n: int, stream=None) -> None:
        """Test hook: the next cull_frame with a depth buffer skips the pyramid's first n tiles, so its
        warps time out waiting for the pyramid (blz_ctx_debug_skip_frame_tiles)."""
        check(self.lib.blz_ctx_debug_skip_frame_tiles(self.ctx, n, _stream_ptr(stream)), "blz_ctx_debug_skip_frame_tiles")

    @property
    def launches(self) -> int:
        return int(self.lib.blz_ctx_launch_count(self.ctx))
