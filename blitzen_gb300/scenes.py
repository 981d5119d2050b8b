"""Seeded synthetic scenes in the reference's buffer layouts.

The reference builds its stress scenes from OBJ meshes with random transforms
(src/Renderer/Resources/RenderObject/blitzenRender.cpp:108-166); the culling path only ever sees
the resulting tables. These generators produce the same tables directly, with the distributions
of the benchmark configurations:

  frustum_lod_scene   100k objects in [-1000,1000]^3, 16 meshes x 4 LODs           (config 1)
  stress_scene        4M objects in [-5000,5000]^3, 64 meshes x 4 LODs, occluders  (config 2)
  cluster_scene       50k objects, 32 meshes of ~200 clusters                      (config 3)
  multiview_batch     64 views over the stress scene, log-uniform sizes            (config 4)

Everything is generated with numpy's PCG64 from a seed, in float64 and rounded once to float32,
so a seed always yields the same bytes.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .abi import CLUSTER, LOD_DATA, MESH_TRANSFORM, PRIMITIVE_SURFACE, RENDER_OBJECT

LOD_INDEX_COUNTS = (30000, 15000, 7500, 3750)
LOD_ERRORS = (0.0, 0.01, 0.04, 0.16)
FOV_DEGREES = 70.0
WINDOW = (1920.0, 1080.0)
ZNEAR = 0.1


@dataclass
class Scene:
    objects: np.ndarray                       # RENDER_OBJECT
    transforms: np.ndarray                    # MESH_TRANSFORM
    surfaces: np.ndarray                      # PRIMITIVE_SURFACE
    lods: np.ndarray                          # LOD_DATA
    clusters: np.ndarray = field(default_factory=lambda: np.zeros(0, CLUSTER))
    boxes: np.ndarray = field(default_factory=lambda: np.zeros((0, 6), np.float32))  # occluders
    visibility: np.ndarray | None = None      # uint32 "visible last frame"

    @property
    def count(self) -> int:
        return int(self.objects.shape[0])

    def table_bytes(self) -> int:
        return sum(a.nbytes for a in (self.objects, self.transforms, self.surfaces, self.lods, self.clusters))


def fov_radians(degrees: float = FOV_DEGREES) -> float:
    """Radians as the reference computes them: degrees * (pi / 180) in float32 (blitML.h:30,613)."""
    pi = np.float32(3.14159265358979323846)
    return float(np.float32(degrees) * (pi / np.float32(180.0)))


def random_unit_quaternions(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform rotations (Shoemake's subgroup algorithm), x, y, z, w."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    q = np.stack([a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2), b * np.sin(2 * np.pi * u3),
                  b * np.cos(2 * np.pi * u3)], axis=1)
    return q.astype(np.float32)


def make_meshes(rng: np.random.Generator, n_meshes: int, lod_counts=LOD_INDEX_COUNTS, lod_errors=LOD_ERRORS,
                clusters_per_mesh: int = 0) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Surfaces (bounding sphere centre U[-1,1]^3, radius U[0.5,3]), their LOD chains, and clusters.

    With clusters_per_mesh > 0 every mesh gets one LOD whose cluster range covers its clusters
    (about clusters_per_mesh each, U[0.8, 1.2] of it)."""
    surfaces = np.zeros(n_meshes, PRIMITIVE_SURFACE)
    surfaces["center"] = rng.uniform(-1.0, 1.0, (n_meshes, 3)).astype(np.float32)
    surfaces["radius"] = rng.uniform(0.5, 3.0, n_meshes).astype(np.float32)
    nl = 1 if clusters_per_mesh else len(lod_counts)
    surfaces["lodOffset"] = np.arange(n_meshes, dtype=np.uint32) * nl
    surfaces["lodCount"] = nl
    lods = np.zeros(n_meshes * nl, LOD_DATA)
    if clusters_per_mesh:
        counts = rng.integers(int(clusters_per_mesh * 0.8), int(clusters_per_mesh * 1.2) + 1, n_meshes)
        offsets = np.concatenate([[0], np.cumsum(counts)[:-1]])
        lods["clusterOffset"] = offsets
        lods["clusterCount"] = counts
        lods["indexCount"] = counts * 124 * 3
        lods["firstIndex"] = offsets * 124 * 3
        total = int(counts.sum())
        cl = np.zeros(total, CLUSTER)
        mesh_of = np.repeat(np.arange(n_meshes), counts)
        rad = surfaces["radius"][mesh_of].astype(np.float64)
        # cluster spheres inside the mesh sphere: centre within the mesh radius, radius U[0.05, 0.5] of it
        dirs = rng.normal(size=(total, 3))
        dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
        cl["center"] = (surfaces["center"][mesh_of] + dirs * (rad * rng.uniform(0, 1, total))[:, None]).astype(np.float32)
        cl["radius"] = (rad * rng.uniform(0.05, 0.5, total)).astype(np.float32)
        axes = rng.normal(size=(total, 3))
        axes /= np.linalg.norm(axes, axis=1, keepdims=True)
        cl["coneAxis"] = np.clip(np.round(axes * 127.0), -127, 127).astype(np.int8)
        cl["coneCutoff"] = np.clip(np.round(rng.uniform(-1.0, 1.0, total) * 127.0), -127, 127).astype(np.int8)
        cl["triangleCount"] = rng.integers(64, 125, total).astype(np.uint8)
        cl["vertexCount"] = rng.integers(32, 65, total).astype(np.uint8)
        cl["dataOffset"] = (np.arange(total, dtype=np.uint64) * 124 * 3).astype(np.uint32)
        return surfaces, lods, cl
    first = 0
    for m in range(n_meshes):
        for i, (ic, err) in enumerate(zip(lod_counts, lod_errors)):
            lods[m * nl + i]["indexCount"] = ic
            lods[m * nl + i]["firstIndex"] = first
            lods[m * nl + i]["error"] = np.float32(err)
            first += ic
    return surfaces, lods, np.zeros(0, CLUSTER)


def make_objects(rng: np.random.Generator, n: int, extent: float, n_meshes: int) -> tuple[np.ndarray, np.ndarray]:
    """n objects, one transform each: position U[-extent, extent]^3, scale U[0.5, 2], unit quaternion."""
    tr = np.zeros(n, MESH_TRANSFORM)
    tr["pos"] = rng.uniform(-extent, extent, (n, 3)).astype(np.float32)
    tr["scale"] = rng.uniform(0.5, 2.0, n).astype(np.float32)
    tr["orientation"] = random_unit_quaternions(rng, n)
    objs = np.zeros(n, RENDER_OBJECT)
    objs["transformId"] = np.arange(n, dtype=np.uint32)
    objs["surfaceId"] = rng.integers(0, n_meshes, n).astype(np.uint32)
    return objs, tr


def make_occluders(rng: np.random.Generator, n: int, zmin: float = 1500.0, zmax: float = 8000.0,
                   size=(10.0, 200.0), half_fov_tan=(1.25, 0.70)) -> np.ndarray:
    """Axis-aligned occluder boxes (min xyz, max xyz) in front of a camera at the origin looking +Z.

    The default depth range hides about half of the frustum-visible objects of the stress scene
    behind the boxes (nearer boxes cover the whole screen, farther ones hide almost nothing)."""
    z = rng.uniform(zmin, zmax, n)
    x = rng.uniform(-1, 1, n) * z * half_fov_tan[0]
    y = rng.uniform(-1, 1, n) * z * half_fov_tan[1]
    ext = rng.uniform(size[0], size[1], (n, 3))
    c = np.stack([x, y, z], axis=1)
    return np.concatenate([c - ext / 2, c + ext / 2], axis=1).astype(np.float32)


def frustum_lod_scene(n: int = 100_000, seed: int = 0, n_meshes: int = 16, extent: float = 1000.0) -> Scene:
    rng = np.random.default_rng(seed)
    surfaces, lods, _ = make_meshes(rng, n_meshes)
    objs, tr = make_objects(rng, n, extent, n_meshes)
    return Scene(objs, tr, surfaces, lods)


def stress_scene(n: int = 4_000_000, seed: int = 0, n_meshes: int = 64, extent: float = 5000.0,
                 n_boxes: int = 2000, visible_fraction: float = 0.5) -> Scene:
    rng = np.random.default_rng(seed)
    surfaces, lods, _ = make_meshes(rng, n_meshes)
    objs, tr = make_objects(rng, n, extent, n_meshes)
    boxes = make_occluders(rng, n_boxes)
    vis = (rng.random(n) < visible_fraction).astype(np.uint32)
    return Scene(objs, tr, surfaces, lods, boxes=boxes, visibility=vis)


STRESS_DEPTH = (1920, 1080)  # the stress frame's depth buffer (width, height)
STRESS_ZFAR = 1e4


def stress_view():
    """The stress frame's camera: the origin looking +Z, 70 degree vertical field of view at
    1920x1080, zNear 0.1, zFar 1e4, and the D3D12 pyramid extent (half the depth buffer)."""
    from . import abi
    w, h = STRESS_DEPTH
    return abi.view_setup(fov_radians(), float(w), float(h), ZNEAR, STRESS_ZFAR, (0.0, 0.0, 0.0), 0.0, 0.0,
                          w / 2, h / 2)


def cluster_scene(n: int = 50_000, seed: int = 0, n_meshes: int = 32, clusters_per_mesh: int = 200,
                  extent: float = 1000.0) -> Scene:
    rng = np.random.default_rng(seed)
    surfaces, lods, clusters = make_meshes(rng, n_meshes, clusters_per_mesh=clusters_per_mesh)
    objs, tr = make_objects(rng, n, extent, n_meshes)
    boxes = make_occluders(rng, 500, zmin=150.0, zmax=1200.0)
    return Scene(objs, tr, surfaces, lods, clusters=clusters, boxes=boxes)


@dataclass
class ViewSpec:
    position: tuple[float, float, float]
    yaw: float
    pitch: float
    subset: np.ndarray          # sorted render-object indices of the view


def multiview_specs(scene_count: int, n_views: int = 64, seed: int = 0, lo: int = 1000, hi: int = 2_000_000,
                    extent: float = 5000.0) -> list[ViewSpec]:
    """Views with a random position in the scene, random yaw/pitch and a log-uniform object subset."""
    rng = np.random.default_rng(seed + 1000)
    specs = []
    for _ in range(n_views):
        size = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        size = min(size, scene_count)
        subset = np.sort(rng.choice(scene_count, size=size, replace=False)).astype(np.uint32)
        pos = tuple(float(v) for v in rng.uniform(-extent, extent, 3).astype(np.float32))
        yaw = float(np.float32(rng.uniform(-math.pi, math.pi)))
        pitch = float(np.float32(rng.uniform(-0.5, 0.5)))
        specs.append(ViewSpec(pos, yaw, pitch, subset))
    return specs


def subset_objects(scene: Scene, subset: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(scene.objects[subset])


def views_boxes(rng_seed: int, n_views: int, n_boxes: int = 2000) -> list[np.ndarray]:
    """Occluders for each view, in that view's camera frame (placed in front of it); the caller maps
    them to world space with the view's inverse rotation when needed."""
    rng = np.random.default_rng(rng_seed + 2000)
    return [make_occluders(rng, n_boxes) for _ in range(n_views)]
