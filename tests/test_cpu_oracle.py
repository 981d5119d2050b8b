"""Known-answer tests of the oracle's explicit definitions, and (where the reference checkout is
present) the oracle against the reference's own code compiled on the CPU on fresh random inputs.
No GPU."""
import ctypes as C
import math
from pathlib import Path

import numpy as np
import pytest

from blitzen_gb300 import abi
from blitzen_gb300 import scenes as S
from oracle import oracle as O

ROOT = Path(__file__).resolve().parent.parent
REF = ROOT / "oracle" / "_ref"


def f32(x):
    return float(np.float32(x))


def test_ftou_follows_d3d_conversion():
    # NaN and non-positive values give 0, values past the range saturate, the rest truncate
    assert O.ftou(float("nan")) == 0
    assert O.ftou(-1.5) == 0 and O.ftou(-0.0) == 0 and O.ftou(0.0) == 0
    assert O.ftou(0.999) == 0 and O.ftou(1.0) == 1 and O.ftou(7.99) == 7
    assert O.ftou(4294967040.0) == 4294967040
    assert O.ftou(4294967296.0) == 0xFFFFFFFF and O.ftou(float("inf")) == 0xFFFFFFFF


def test_floor_log2_from_the_exponent():
    for k in range(-20, 30):
        p = math.ldexp(1.0, k)
        below = float(np.nextafter(np.float32(p), np.float32(0)))
        above = float(np.nextafter(np.float32(p), np.float32(np.inf)))
        want = max(k, 0)
        assert O.floor_log2_u(p) == want, p
        assert O.floor_log2_u(above) == want, above
        assert O.floor_log2_u(below) == max(k - 1, 0), below
    assert O.floor_log2_u(0.0) == 0 and O.floor_log2_u(-3.0) == 0 and O.floor_log2_u(float("nan")) == 0


def test_view_constants_of_the_default_camera():
    v = O.view_setup(S.fov_radians(), 1920.0, 1080.0, 0.1, 1e4, pw=960.0, ph=540.0)
    # the values the reference's camera code produces for this camera (70 degrees, 1920x1080)
    got = {k: f32(getattr(v, k)) for k in ("frustumRight", "frustumLeft", "frustumTop", "frustumBottom",
                                          "proj0", "proj5", "lodTarget")}
    want = {"frustumRight": 0.626278281, "frustumLeft": 0.779599547, "frustumTop": 0.819152057,
            "frustumBottom": 0.57357645, "proj0": 0.803333282, "proj5": 1.42814803, "lodTarget": 0.00129668054}
    for k, w in want.items():
        assert got[k] == f32(w), (k, got[k], w)


def test_empty_all_in_all_out():
    sc = S.frustum_lod_scene(2000, seed=9, extent=50.0)
    v_in = O.view_setup(S.fov_radians(), 1920.0, 1080.0, 0.1, 1e30, position=(0.0, 0.0, -1e6))
    n, recs, _ = O.cull(0, v_in, sc)
    assert n == sc.count and np.array_equal(recs[:, 0], np.arange(sc.count))  # stable order
    v_out = O.view_setup(S.fov_radians(), 1920.0, 1080.0, 0.1, 1e30, position=(0.0, 0.0, -1e6), yaw=math.pi)
    assert O.cull(0, v_out, sc)[0] == 0
    assert O.cull(0, v_in, sc, objects=sc.objects[:0])[0] == 0


def test_bad_indices_are_flagged_and_skipped():
    sc = S.frustum_lod_scene(100, seed=1, extent=20.0)
    objs = sc.objects.copy()
    objs[3]["transformId"] = 10**6
    objs[7]["surfaceId"] = 10**6
    v = O.view_setup(S.fov_radians(), 1920.0, 1080.0, 0.1, 1e30, position=(0.0, 0.0, -1e3))
    n, recs, flags = O.cull(0, v, sc, objects=objs)
    assert flags & abi.FLAG_BAD_INDEX
    assert 3 not in recs[:, 0] and 7 not in recs[:, 0]


def _ref_hlsl():
    lib = REF / "libref_hlsl.so"
    if not lib.exists():
        pytest.skip("the reference's shaders are not built here (no reference checkout)")
    r = C.CDLL(str(lib))
    P, U = C.c_void_p, C.c_uint32
    r.ref_hlsl_cull.argtypes = [C.c_int, P, P, P, U, P, P, P, U]
    r.ref_hlsl_cull.restype = U
    r.ref_hlsl_pyramid.argtypes = [P, U, U, P]
    return r


@pytest.mark.parametrize("seed", [1, 2])
def test_oracle_against_reference_shaders_live(seed):
    r = _ref_hlsl()
    sc = S.stress_scene(40_000, seed=seed, n_meshes=32, extent=800.0, n_boxes=300)
    rng = np.random.default_rng(seed)
    v = abi.view_setup(S.fov_radians(), 1920.0, 1080.0, 0.1, 1e4, tuple(float(x) for x in rng.uniform(-50, 50, 3)),
                       float(rng.uniform(-3, 3)), float(rng.uniform(-0.5, 0.5)), 480.0, 270.0)
    depth = O.depth_raster(v, sc.boxes, 960, 540)
    p_or = O.pyramid_build(depth)
    p_ref = O.HostPyramid(960, 540)
    r.ref_hlsl_pyramid(depth.ctypes.data, 960, 540, C.byref(p_ref.desc))
    assert np.array_equal(p_or.data.view(np.uint32), p_ref.data.view(np.uint32))
    d, keep = O.scene_desc(sc)
    for kind in range(4):
        vis_o = sc.visibility.copy() if kind in (1, 2) else None
        vis_r = sc.visibility.copy() if kind in (1, 2) else None
        n, recs, _ = O.cull(kind, v, sc, vis=vis_o, pyramid=p_or if kind in (2, 3) else None, stride=32, threads=4)
        out = np.zeros((sc.count, 8), np.uint32)
        m = r.ref_hlsl_cull(kind, C.byref(v), C.byref(d), keep[0].ctypes.data, sc.count,
                            None if vis_r is None else vis_r.ctypes.data,
                            C.byref(p_ref.desc) if kind in (2, 3) else None, out.ctypes.data, sc.count)
        assert n == m, (kind, n, m)
        assert np.array_equal(recs, out[:m]), kind
        if vis_o is not None:
            assert np.array_equal(vis_o, vis_r), kind


def test_cluster_task_form_groups_the_cluster_records():
    """The oracle's mesh-shader form against a direct loop over the per-cluster records: one task
    per object with survivors, payloads of 32 in order, 0xFFFFFFFF past the last survivor."""
    sc = S.cluster_scene(400, seed=3, clusters_per_mesh=120)
    v = O.view_setup(S.fov_radians(), 1920.0, 1080.0, 0.1, 1e4, position=(0.0, 0.0, -50.0))
    tasks, payloads = O.cluster_tasks(v, sc)
    n, recs, ids, _ = O.cull_clusters(v, sc, capacity=O._cluster_upper_bound(sc, sc.objects))
    runs: dict[int, list[int]] = {}
    for obj, cid in zip(recs[:, 0].tolist(), ids.tolist()):
        runs.setdefault(obj, []).append(cid)
    want_t, want_p = [], []
    for obj in sorted(runs):
        cl = runs[obj]
        want_t.append([len(want_p), (len(cl) + 31) // 32, 1, 1])
        for g in range(0, len(cl), 32):
            part = cl[g:g + 32]
            want_p.append([obj] + part + [abi.NO_MESHLET] * (32 - len(part)))
    assert n > 0 and any(len(cl) > 32 for cl in runs.values())
    assert np.array_equal(tasks, np.array(want_t, np.uint32).reshape(-1, 4))
    assert np.array_equal(payloads, np.array(want_p, np.uint32).reshape(-1, 33))
    # no survivors: empty arrays
    t0, p0 = O.cluster_tasks(v, sc, objects=sc.objects[:0])
    assert t0.shape == (0, 4) and p0.shape == (0, 33)
