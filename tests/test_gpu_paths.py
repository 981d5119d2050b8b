"""Parity of the instanced, cluster, raster, transform, batched and serving paths with the oracle."""
import ctypes as C

import numpy as np
import pytest
import torch

from blitzen_gb300 import abi
from blitzen_gb300 import scenes as S
from blitzen_gb300.abi import BatchView, RenderList
from blitzen_gb300.culler import Culler, DevicePyramid, Target, TaskTarget, to_device
from oracle import oracle as O
from tests.helpers import H, W, assert_records_equal, view_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def stress_ctx(lib):
    c = Culler(0)
    sc = S.stress_scene(300_000, seed=11, extent=3000.0)
    c.setup_for_rendering(sc)
    yield c, sc
    c.close()


# ----------------------------------------------------------------------------- instanced

@pytest.mark.parametrize("slots", [100_000, 50])
def test_instanced_matches_oracle(stress_ctx, slots):
    c, sc = stress_ctx
    v = view_for(zfar=1e4)
    ctr = O.new_counters(sc, slots)
    cap = len(sc.lods) * slots
    dctr = torch.from_numpy(ctr.view(np.int32).reshape(-1).copy()).cuda()
    dinst = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
    t = Target.alloc(len(sc.lods), abi.STRIDE_D3D12)
    c.draw_instance_cull_pass(v, dctr, dinst, slots, t)
    flags = c.flags()
    n, cmds, octr, oinst, oflags = O.cull_instanced(v, sc, ctr, cap, slots, stride=abi.STRIDE_D3D12)
    assert flags == oflags
    if slots == 50:
        assert flags & abi.FLAG_INSTANCE_OVERFLOW
    assert_records_equal(t.read(), (n, cmds), "instanced commands")
    assert np.array_equal(dctr.cpu().numpy().view(np.uint32), octr.view(np.uint32).reshape(-1))
    assert np.array_equal(dinst.cpu().numpy().view(np.uint32), oinst)


def test_instanced_long_chunks_matches_oracle(lib):
    """1M objects, every one in view: single-view chunks of 256 objects emit more records than the
    place kernel's first batch holds (160), so this takes the path that ranks a chunk's records slice
    by slice, beside the one that keeps the first batch's ranks."""
    sc = S.stress_scene(1_000_000, seed=1)
    c = Culler(0)
    try:
        c.setup_for_rendering(sc)
        v = view_for(zfar=1e30, position=(0.0, 0.0, -20000.0))
        slots = 100_000
        ctr = O.new_counters(sc, slots)
        cap = len(sc.lods) * slots
        dctr = torch.from_numpy(ctr.view(np.int32).reshape(-1).copy()).cuda()
        dinst = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
        t = Target.alloc(len(sc.lods), abi.STRIDE_D3D12)
        c.draw_instance_cull_pass(v, dctr, dinst, slots, t)
        flags = c.flags()
        n, cmds, octr, oinst, oflags = O.cull_instanced(v, sc, ctr, cap, slots, stride=abi.STRIDE_D3D12)
        visible = int(octr.view(np.uint32).reshape(-1, 2)[:, 1].sum())
        assert visible > 0.9 * sc.count, visible
        assert flags == oflags == 0
        assert_records_equal(t.read(), (n, cmds), "instanced commands")
        assert np.array_equal(dctr.cpu().numpy().view(np.uint32), octr.view(np.uint32).reshape(-1))
        assert np.array_equal(dinst.cpu().numpy().view(np.uint32), oinst)
    finally:
        c.close()


def test_instanced_empty_view(stress_ctx):
    c, sc = stress_ctx
    v = view_for(zfar=1e4, position=(0.0, 0.0, 1e7))  # every object behind the camera
    ctr = O.new_counters(sc, 1000)
    dctr = torch.from_numpy(ctr.view(np.int32).reshape(-1).copy()).cuda()
    dinst = torch.zeros(len(sc.lods) * 1000, dtype=torch.int32, device="cuda")
    t = Target.alloc(len(sc.lods))
    t.count.fill_(77)
    c.draw_instance_cull_pass(v, dctr, dinst, 1000, t)
    assert c.check() == 0
    assert t.read()[0] == 0
    assert (dctr.cpu().numpy().view(np.uint32).reshape(-1, 2)[:, 1] == 0).all()


@pytest.mark.parametrize("slots", [5_000, 7])
def test_instanced_many_lods_matches_oracle(lib, slots):
    """More LODs than the staged path keeps in shared memory (1,200): the single-kernel form runs."""
    c = Culler(0)
    try:
        sc = S.frustum_lod_scene(60_000, seed=5, n_meshes=300, extent=800.0)
        assert len(sc.lods) > 1024
        c.setup_for_rendering(sc)
        v = view_for(zfar=1e4)
        ctr = O.new_counters(sc, slots)
        cap = len(sc.lods) * slots
        dctr = torch.from_numpy(ctr.view(np.int32).reshape(-1).copy()).cuda()
        dinst = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
        t = Target.alloc(len(sc.lods), abi.STRIDE_D3D12)
        c.draw_instance_cull_pass(v, dctr, dinst, slots, t)
        flags = c.flags()
        n, cmds, octr, oinst, oflags = O.cull_instanced(v, sc, ctr, cap, slots, stride=abi.STRIDE_D3D12)
        assert flags == oflags
        assert_records_equal(t.read(), (n, cmds), "instanced commands, 1,200 LODs")
        assert np.array_equal(dctr.cpu().numpy().view(np.uint32), octr.view(np.uint32).reshape(-1))
        assert np.array_equal(dinst.cpu().numpy().view(np.uint32), oinst)
    finally:
        c.close()


# ----------------------------------------------------------------------------- raster + transforms

def test_depth_raster_matches_oracle(stress_ctx):
    c, sc = stress_ctx
    for k, (pos, yaw) in enumerate([((0.0, 0.0, 0.0), 0.0), ((100.0, -50.0, 200.0), 0.4)]):
        v = view_for(position=pos, yaw=yaw)
        depth = torch.full((W * H,), 5.0, dtype=torch.float32, device="cuda")
        c.raster_boxes(v, torch.from_numpy(sc.boxes.reshape(-1)).cuda(), depth, W, H)
        assert c.check() == 0
        ref = O.depth_raster(v, sc.boxes, W, H)
        assert np.array_equal(depth.cpu().numpy().reshape(H, W), ref), k


def test_transforms_update_and_rotate(stress_ctx):
    c, sc = stress_ctx
    rng = np.random.default_rng(3)
    ids = rng.choice(sc.count, 500, replace=False).astype(np.uint32)
    axes = rng.normal(size=(500, 3))
    axes = (axes / np.linalg.norm(axes, axis=1, keepdims=True)).astype(np.float32)
    dst = torch.zeros(500 * 8, dtype=torch.float32, device="cuda")
    c.rotate_transforms(torch.from_numpy(ids.view(np.int32).copy()).cuda(), torch.from_numpy(axes.reshape(-1)).cuda(),
                        0.01, dst)
    assert c.check() == 0
    ref = O.transforms_rotate(sc.transforms, ids, axes, 0.01)
    assert np.array_equal(dst.cpu().numpy().view(np.uint32), ref.view(np.uint32).reshape(-1))
    # scatter them back through the host-array entry point and cull: same as the oracle on the edited scene
    c.update_object_transform(ids, ref)
    edited = S.Scene(sc.objects, sc.transforms.copy(), sc.surfaces, sc.lods)
    edited.transforms[ids] = ref
    v = view_for(zfar=1e4)
    t = Target.alloc(sc.count)
    c.draw_cull(v, t)
    assert c.check() == 0
    n, recs, _ = O.cull(0, v, edited)
    assert_records_equal(t.read(), (n, recs), "after transform update")
    c.update_object_transform(ids, sc.transforms[ids])  # restore the resident scene


# ----------------------------------------------------------------------------- clusters

@pytest.fixture(scope="module")
def cluster_ctx(lib):
    c = Culler(0)
    sc = S.cluster_scene(20_000, seed=2, clusters_per_mesh=200)
    c.setup_for_rendering(sc)
    yield c, sc
    c.close()


@pytest.mark.parametrize("with_hiz", [False, True])
def test_clusters_match_oracle(cluster_ctx, with_hiz):
    c, sc = cluster_ctx
    v = view_for(zfar=1e4, position=(0.0, 0.0, -50.0))
    pyr = opyr = None
    if with_hiz:
        depth = O.depth_raster(v, sc.boxes, W, H)
        pyr = DevicePyramid(W, H)
        c.generate_depth_pyramid(pyr, torch.from_numpy(depth).cuda())
        opyr = O.pyramid_build(depth)
    cap = O._cluster_upper_bound(sc, sc.objects)
    t = Target.alloc(cap)
    ids = torch.zeros(cap, dtype=torch.int32, device="cuda")
    c.cluster_cull(v, t, pyramid=pyr, cluster_ids=ids)
    assert c.check() == 0
    n, recs, oids, _ = O.cull_clusters(v, sc, pyramid=opyr, capacity=cap)
    assert n > 0
    assert_records_equal(t.read(), (n, recs), "clusters")
    assert np.array_equal(ids[:n].cpu().numpy().view(np.uint32), oids)


def test_clusters_repeated_calls_of_changing_size(cluster_ctx):
    """The test launch's finished-block counts (per tile and over the tiles) are rewound by the
    blocks that finish them: calls of different list sizes in a row, with and without Hi-Z, each
    match the oracle."""
    c, sc = cluster_ctx
    v = view_for(zfar=1e4, position=(0.0, 0.0, -50.0))
    pyr, opyr = _cluster_pyramid(c, sc, v)
    rng = np.random.default_rng(8)
    for k, size in enumerate([sc.count, 33, 5_000, 1, sc.count, 2_017]):
        objs = sc.objects if size == sc.count else sc.objects[rng.permutation(sc.count)[:size]]
        dobjs = to_device(objs, "cuda")
        with_hiz = k % 2 == 1
        cap = max(O._cluster_upper_bound(sc, objs), 1)
        t = Target.alloc(cap)
        c.cluster_cull(v, t, pyramid=pyr if with_hiz else None, objects=dobjs, count=len(objs))
        assert c.check() == 0
        n, recs, _, _ = O.cull_clusters(v, sc, pyramid=opyr if with_hiz else None, capacity=cap, objects=objs)
        assert_records_equal(t.read(), (n, recs), f"call {k} ({size} objects)")


def test_cluster_cone_test_culls_something(cluster_ctx):
    c, sc = cluster_ctx
    v = view_for(zfar=1e4, position=(0.0, 0.0, -50.0))
    cap = O._cluster_upper_bound(sc, sc.objects)
    n, _, _, _ = O.cull_clusters(v, sc, capacity=cap)
    # all clusters of frustum-visible objects, no cone test: an upper bound the cone test must undercut
    open_cones = S.Scene(sc.objects, sc.transforms, sc.surfaces, sc.lods, clusters=sc.clusters.copy())
    open_cones.clusters["coneCutoff"] = 127
    n_open, _, _, _ = O.cull_clusters(v, open_cones, capacity=cap)
    assert n < n_open


def _cluster_pyramid(c, sc, v):
    depth = O.depth_raster(v, sc.boxes, W, H)
    pyr = DevicePyramid(W, H)
    c.generate_depth_pyramid(pyr, torch.from_numpy(depth).cuda())
    return pyr, O.pyramid_build(depth)


@pytest.mark.parametrize("with_hiz", [False, True])
def test_cluster_tasks_match_oracle(cluster_ctx, with_hiz):
    """Mesh-shader form: IndirectTask + MeshTaskPayload records equal the oracle's, word for word
    (unused payload slots included), and carry the same clusters as the per-cluster records."""
    c, sc = cluster_ctx
    v = view_for(zfar=1e4, position=(0.0, 0.0, -50.0))
    pyr, opyr = _cluster_pyramid(c, sc, v) if with_hiz else (None, None)
    tasks, payloads = O.cluster_tasks(v, sc, pyramid=opyr)
    assert len(tasks) > 50 and len(payloads) > len(tasks)  # objects with more than 32 survivors occur
    t = TaskTarget.alloc(sc.count, len(payloads) + 7)
    t.payloads.fill_(0x5A5A5A5A)  # every word of a written payload must be overwritten
    c.cluster_task_cull(v, t, pyramid=pyr)
    assert c.check() == 0
    nt, np_, gt, gp = t.read()
    assert (nt, np_) == (len(tasks), len(payloads))
    assert np.array_equal(gt, tasks)
    assert np.array_equal(gp, payloads)
    # the payloads list exactly the clusters the per-cluster records name
    cap = O._cluster_upper_bound(sc, sc.objects)
    n, _, oids, _ = O.cull_clusters(v, sc, pyramid=opyr, capacity=cap)
    flat = gp[:, 1:].reshape(-1)
    assert np.array_equal(flat[flat != abi.NO_MESHLET], oids)


def test_cluster_tasks_subset_and_empty(cluster_ctx):
    c, sc = cluster_ctx
    v = view_for(zfar=1e4, position=(0.0, 0.0, -50.0))
    objs = sc.objects[np.random.default_rng(5).permutation(sc.count)[:777]]
    dobjs = to_device(objs, "cuda")
    tasks, payloads = O.cluster_tasks(v, sc, objects=objs)
    t = TaskTarget.alloc(len(objs), max(len(payloads), 1))
    c.cluster_task_cull(v, t, objects=dobjs, count=len(objs))
    assert c.check() == 0
    nt, np_, gt, gp = t.read()
    assert (nt, np_) == (len(tasks), len(payloads))
    assert np.array_equal(gt, tasks) and np.array_equal(gp, payloads)
    # an empty list writes zero counts
    t.counts.fill_(-1)
    c.cluster_task_cull(v, t, objects=dobjs, count=0)
    assert c.check() == 0
    assert t.read()[:2] == (0, 0)


def test_cluster_tasks_overflow_keeps_prefix(cluster_ctx):
    c, sc = cluster_ctx
    v = view_for(zfar=1e4, position=(0.0, 0.0, -50.0))
    tasks, payloads = O.cluster_tasks(v, sc)
    nt_cap, np_cap = len(tasks) // 3, len(payloads) // 2
    t = TaskTarget.alloc(nt_cap, np_cap)
    c.cluster_task_cull(v, t)
    flags = c.flags()
    nt, np_, gt, gp = t.read()
    assert (nt, np_) == (len(tasks), len(payloads))
    assert np.array_equal(gt, tasks[:nt_cap])
    # payloads that were written completely match (a payload whose object's tail lies past the
    # capacity is still complete: each payload is written only by its own object)
    assert np.array_equal(gp, payloads[:np_cap])
    assert flags & abi.FLAG_COMMAND_OVERFLOW


# ----------------------------------------------------------------------------- batch

def _batch(c, sc, n_views=12, seed=4, mode=abi.MODE_TEMPORAL):
    specs = S.multiview_specs(sc.count, n_views, seed=seed, lo=100, hi=sc.count, extent=1000.0)
    keep, views, ref = [], (BatchView * n_views)(), []
    rng = np.random.default_rng(seed)
    for i, sp in enumerate(specs):
        v = view_for(zfar=1e4, position=sp.position, yaw=sp.yaw, pitch=sp.pitch)
        objs = S.subset_objects(sc, sp.subset)
        dobjs = to_device(objs, "cuda")
        boxes = S.make_occluders(rng, 300, zmin=50.0, zmax=2000.0)
        depth = O.depth_raster(view_for(), boxes, W, H)  # any depth image works for parity
        pyr = DevicePyramid(W, H)
        c.generate_depth_pyramid(pyr, torch.from_numpy(depth).cuda())
        t = Target.alloc(len(objs))
        keep += [dobjs, pyr, t]
        views[i].view = v
        views[i].list = RenderList(dobjs.data_ptr(), len(objs))
        views[i].mode = mode
        views[i].pyramid = C.pointer(pyr.desc)
        views[i].target = t.ctype()
        ref.append((v, objs, O.pyramid_build(depth), t))
    return views, keep, ref


def test_batch_of_mixed_modes_matches_oracle(stress_ctx):
    """One batch holding frustum, pass-1, pass-2 and temporal views (the mode is read per view)."""
    c, sc = stress_ctx
    views, keep, ref = _batch(c, sc, n_views=8, seed=13)
    modes = [abi.MODE_FRUSTUM, abi.MODE_FIRST, abi.MODE_LATE, abi.MODE_TEMPORAL] * 2
    vis_host = []
    for i, m in enumerate(modes):
        views[i].mode = m
        if m in (abi.MODE_FIRST, abi.MODE_LATE):
            vh = (np.random.default_rng(i).random(ref[i][1].shape[0]) < 0.5).astype(np.uint32)
            vd = torch.from_numpy(vh.view(np.int32).copy()).cuda()
            keep.append(vd)
            views[i].visibility = vd.data_ptr()
            vis_host.append((vh, vd))
        else:
            vis_host.append(None)
    lib = abi.load()
    abi.check(lib.blz_cull_batch(c.ctx, views, len(ref), None), "blz_cull_batch")
    assert c.check() == 0
    for i, (v, objs, opyr, t) in enumerate(ref):
        m = modes[i]
        ovis = vis_host[i][0].copy() if vis_host[i] is not None else None
        n, recs, _ = O.cull(m, v, sc, objects=objs, vis=ovis,
                            pyramid=opyr if m in (abi.MODE_LATE, abi.MODE_TEMPORAL) else None)
        assert_records_equal(t.read(), (n, recs), f"view {i} mode {m}")
        if m == abi.MODE_LATE:
            assert np.array_equal(vis_host[i][1].cpu().numpy().view(np.uint32), ovis), f"view {i} visibility"


@pytest.mark.parametrize("shape", [(256, 4, 0), (128, 1, 1), (512, 2, 0), (128, 8, 0), (256, 2, 2)])
def test_batch_matches_per_view_and_oracle(stress_ctx, shape):
    c, sc = stress_ctx
    views, keep, ref = _batch(c, sc)
    lib = abi.load()
    abi.check(lib.blz_set_launch_shape(c.ctx, C.byref(abi.LaunchShape(shape[0], shape[1], shape[2], 0))), "shape")
    abi.check(lib.blz_cull_batch(c.ctx, views, len(ref), None), "blz_cull_batch")
    assert c.check() == 0
    batched = [r[3].read() for r in ref]
    for r in ref:
        r[3].count.fill_(0)
        r[3].commands.zero_()
    abi.check(lib.blz_cull_batch_per_view(c.ctx, views, len(ref), None), "per view")
    assert c.check() == 0
    for i, (v, objs, opyr, t) in enumerate(ref):
        per = t.read()
        assert_records_equal(batched[i], per, f"view {i} batched vs per-view")
        n, recs, _ = O.cull(3, v, sc, objects=objs, pyramid=opyr)
        assert_records_equal(batched[i], (n, recs), f"view {i} vs oracle")


def test_batch_graph_replay(stress_ctx):
    c, sc = stress_ctx
    views, keep, ref = _batch(c, sc, n_views=8, seed=9)
    lib = abi.load()
    g = C.c_void_p()
    abi.check(lib.blz_batch_graph_create(c.ctx, views, len(ref), None, C.byref(g)), "graph create")
    try:
        for rep in range(3):
            for r in ref:
                r[3].count.fill_(0)
            abi.check(lib.blz_batch_graph_launch(g, None), "graph launch")
            assert c.check() == 0
            for i, (v, objs, opyr, t) in enumerate(ref):
                n, recs, _ = O.cull(3, v, sc, objects=objs, pyramid=opyr)
                assert_records_equal(t.read(), (n, recs), f"replay {rep} view {i}")
        # a new camera for view 0 between replays
        nv = view_for(zfar=1e4, yaw=1.0)
        abi.check(lib.blz_batch_graph_set_view(g, 0, C.byref(nv)), "set view")
        abi.check(lib.blz_batch_graph_launch(g, None), "graph launch")
        assert c.check() == 0
        n, recs, _ = O.cull(3, nv, sc, objects=ref[0][1], pyramid=ref[0][2])
        assert_records_equal(ref[0][3].read(), (n, recs), "view 0 after set_view")
    finally:
        lib.blz_batch_graph_destroy(g)


def test_autotune_picks_a_supported_shape(stress_ctx):
    """blz_autotune_batch picks a shape and a chunk size, caches them for the batch's size (a second
    call returns the same choice untimed), batches of that size use them and still match the oracle,
    and an explicit shape forgets the cache."""
    c, sc = stress_ctx
    views, keep, ref = _batch(c, sc, n_views=4, seed=21)
    lib = abi.load()
    best, us = abi.LaunchShape(), C.c_float(0)
    abi.check(lib.blz_autotune_batch(c.ctx, views, len(ref), 2, None, C.byref(best), C.byref(us)), "autotune")
    assert best.threadsPerBlock in (128, 256, 512) and best.objectsPerThread in (1, 2, 4, 8)
    assert best.chunkObjects in (256, 512, 1024)
    assert us.value > 0
    again, us2 = abi.LaunchShape(), C.c_float(0)
    abi.check(lib.blz_autotune_batch(c.ctx, views, len(ref), 2, None, C.byref(again), C.byref(us2)), "autotune")
    assert (again.threadsPerBlock, again.objectsPerThread, again.blocksPerSm, again.chunkObjects) == \
        (best.threadsPerBlock, best.objectsPerThread, best.blocksPerSm, best.chunkObjects)
    assert us2.value == us.value  # the cached choice, not a new measurement
    # an explicit shape forgets the cache; the next call measures again and caches anew
    c.set_launch_shape(128, 1, 4, 1024)
    abi.check(lib.blz_autotune_batch(c.ctx, views, len(ref), 1, None, C.byref(again), C.byref(us2)), "autotune")
    assert again.chunkObjects in (256, 512, 1024)
    # batches of that size run with the tuned shape and still match the oracle
    for _, _, _, t in ref:
        t.count.fill_(0)
    abi.check(lib.blz_cull_batch(c.ctx, views, len(ref), None), "batch")
    assert c.check() == 0
    for i, (v, objs, hp, t) in enumerate(ref):
        n, recs, _ = O.cull(3, v, sc, objects=objs, pyramid=hp)
        assert_records_equal(t.read(), (n, recs), f"view {i} under the tuned shape {c.launch_shape()}")
    c.set_launch_shape(256, 2)


def test_autotune_single_caches_and_keeps_visibility(stress_ctx):
    """blz_autotune_single times the single-view shapes on pass 2 without changing the visibility,
    caches the fastest for (list size, pass), and pass 2 under it matches the oracle."""
    c, sc = stress_ctx
    v = view_for(zfar=1e4)
    depth = O.depth_raster(v, S.make_occluders(np.random.default_rng(8), 300), W, H)
    pyr = DevicePyramid(W, H)
    c.generate_depth_pyramid(pyr, torch.from_numpy(depth).cuda())
    vis0 = (np.random.default_rng(9).random(sc.count) < 0.5).astype(np.uint32)
    vis = torch.from_numpy(vis0.view(np.int32).copy()).cuda()
    t = Target.alloc(sc.count)
    shape, us = c.autotune_single(v, abi.MODE_LATE, t, visibility=vis, pyramid=pyr, repeats=2)
    assert (shape["threads"], shape["objects_per_thread"]) in SINGLE_SHAPES
    assert shape["chunk_objects"] % 32 == 0 and shape["chunk_objects"] > 0
    assert us > 0
    assert np.array_equal(vis.cpu().numpy().view(np.uint32), vis0)  # the tuner worked on a copy
    again, us2 = c.autotune_single(v, abi.MODE_LATE, t, visibility=vis, pyramid=pyr, repeats=2)
    assert again == shape and us2 == us  # cached
    t.count.fill_(0)
    c.draw_cull_occlusion_pass(v, vis, pyr, t)
    assert c.check() == 0
    ovis = vis0.copy()
    n, recs, _ = O.cull(2, v, sc, vis=ovis, pyramid=O.pyramid_build(depth))
    assert_records_equal(t.read(), (n, recs), f"pass 2 under the tuned shape {shape}")
    assert np.array_equal(vis.cpu().numpy().view(np.uint32), ovis)
    c.set_launch_shape(256, 2)  # forgets the cached choice


SINGLE_SHAPES = [(256, 1), (256, 2), (256, 4), (128, 2), (128, 4), (512, 1)]


# ----------------------------------------------------------------------------- serving

def _serve_requests(sc, n, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(n):
        count = int(np.exp(rng.uniform(np.log(1000), np.log(sc.count // 2))))
        start = int(rng.integers(0, sc.count - count))
        axes = rng.normal(size=(1000, 3))
        axes = (axes / np.linalg.norm(axes, axis=1, keepdims=True)).astype(np.float32)
        pos = tuple(float(x) for x in rng.uniform(-500, 500, 3).astype(np.float32))
        reqs.append((start, count, axes, view_for(zfar=1e4, position=pos, yaw=float(rng.uniform(-3, 3)))))
    return reqs


def _submit(lib, server, c, reqs):
    objs_dev = c.scene_tensors[0]
    tickets = []
    for start, count, axes, v in reqs:
        r = abi.ServeRequest()
        r.view = v
        r.list = RenderList(objs_dev.data_ptr() + start * 8, count)
        r.mode = abi.MODE_FRUSTUM
        r.rotateCount = 1000
        r.rotateAxes = axes.ctypes.data
        r.rotateAngle = 0.01
        r.copyToHost = 1
        t = C.c_uint64()
        abi.check(lib.blz_serve_submit(server, C.byref(r), C.byref(t)), "submit")
        tickets.append(t.value)
    return tickets


def _collect(lib, server, tickets):
    out = []
    for t in tickets:
        res = abi.ServeResult()
        abi.check(lib.blz_serve_wait(server, t, 20_000, C.byref(res)), "wait")
        n = res.drawCount
        recs = np.ctypeslib.as_array(C.cast(res.hostRecords, C.POINTER(C.c_uint32)), shape=(n * 6,)).copy() if n else np.zeros(0, np.uint32)
        out.append((res.status, n, recs))
        abi.check(lib.blz_serve_release(server, t), "release")
    return out


def test_serving_results_same_alone_and_in_the_mix(stress_ctx):
    c, sc = stress_ctx
    lib = abi.load()
    cfg = abi.ServeConfig(256 << 20, 4, 16, 1000, abi.STRIDE_VULKAN)
    server = C.c_void_p()
    abi.check(lib.blz_serve_create(c.ctx, C.byref(cfg), C.byref(server)), "serve create")
    try:
        reqs = _serve_requests(sc, 24, seed=1)
        alone = []
        for rq in reqs:
            alone += _collect(lib, server, _submit(lib, server, c, [rq]))
        mixed = _collect(lib, server, _submit(lib, server, c, reqs))
        stats = abi.ServeStats()
        lib.blz_serve_stats(server, C.byref(stats))
        assert stats.completed == 48
        assert stats.maxBatchSize > 1  # the mix was batched
        for k, (a, m) in enumerate(zip(alone, mixed)):
            assert a[0] == 0 and m[0] == 0
            assert a[1] == m[1] and np.array_equal(a[2], m[2]), f"request {k} differs alone vs mixed"
        # one request against the oracle with its rotated dynamic objects applied
        start, count, axes, v = reqs[3]
        rot = O.transforms_rotate(sc.transforms, np.arange(1000, dtype=np.uint32), axes, 0.01)
        edited = S.Scene(sc.objects, sc.transforms.copy(), sc.surfaces, sc.lods)
        edited.transforms[:1000] = rot
        n, recs, _ = O.cull(0, v, edited, objects=sc.objects[start:start + count])
        assert alone[3][1] == n
        assert np.array_equal(alone[3][2].reshape(-1, 6), recs[:, :6])
    finally:
        lib.blz_serve_destroy(server)


def test_serving_admission_waits_for_memory(stress_ctx):
    c, sc = stress_ctx
    lib = abi.load()
    # a pool that holds about one large request at a time
    cfg = abi.ServeConfig(8 << 20, 4, 16, 1000, abi.STRIDE_VULKAN)
    server = C.c_void_p()
    abi.check(lib.blz_serve_create(c.ctx, C.byref(cfg), C.byref(server)), "serve create")
    try:
        reqs = [(0, 250_000, np.tile(np.float32([0, 0, 1]), (1000, 1)), view_for(zfar=1e4))] * 6
        res = _collect(lib, server, _submit(lib, server, c, reqs))
        assert all(r[0] == 0 for r in res)
        assert len({r[1] for r in res}) == 1
        stats = abi.ServeStats()
        lib.blz_serve_stats(server, C.byref(stats))
        assert stats.peakOutputBytes <= 8 << 20
    finally:
        lib.blz_serve_destroy(server)


# ----------------------------------------------------------------------------- bound dynamic rows

def _moved_rows(sc, n, seed):
    rng = np.random.default_rng(seed)
    rows = sc.transforms[:n].copy()
    rows["pos"] += rng.uniform(-400.0, 400.0, size=(n, 3)).astype(np.float32)
    rows["orientation"] = S.random_unit_quaternions(rng, n)
    return rows


@pytest.mark.parametrize("where", ["pinned", "device"])
def test_bound_dynamic_rows_match_edited_scene(stress_ctx, where):
    """Transforms [0, n) read from bound rows (pinned host or device memory) give the oracle's
    results on a scene whose table holds those rows; unbinding restores the resident table."""
    c, sc = stress_ctx
    n = 1000
    rows = _moved_rows(sc, n, 21)
    host = torch.from_numpy(rows.view(np.float32).reshape(-1).copy())
    bound = host.pin_memory() if where == "pinned" else host.cuda()
    edited = S.Scene(sc.objects, sc.transforms.copy(), sc.surfaces, sc.lods)
    edited.transforms[:n] = rows
    v = view_for(zfar=1e4)
    depth = O.depth_raster(v, sc.boxes, W, H)
    pyr = DevicePyramid(W, H)
    c.generate_depth_pyramid(pyr, torch.from_numpy(depth).cuda())
    opyr = O.pyramid_build(depth)
    c.bind_dynamic_transforms(bound)
    try:
        t = Target.alloc(sc.count)
        c.draw_cull(v, t)
        assert c.check() == 0
        assert_records_equal(t.read(), O.cull(0, v, edited)[:2], "frustum, bound rows")
        vis0 = sc.visibility.copy()
        dvis = torch.from_numpy(vis0.view(np.int32).copy()).cuda()
        c.draw_cull_first_pass(v, dvis, t)
        assert c.check() == 0
        assert_records_equal(t.read(), O.cull(1, v, edited, vis=vis0.copy())[:2], "pass 1, bound rows")
        c.draw_cull_occlusion_pass(v, dvis, pyr, t)
        assert c.check() == 0
        ovis = vis0.copy()
        n2, recs2, _ = O.cull(2, v, edited, vis=ovis, pyramid=opyr)
        assert_records_equal(t.read(), (n2, recs2), "pass 2, bound rows")
        assert np.array_equal(dvis.cpu().numpy().view(np.uint32), ovis)
    finally:
        c.bind_dynamic_transforms(None)
    t = Target.alloc(sc.count)
    c.draw_cull(v, t)
    assert c.check() == 0
    assert_records_equal(t.read(), O.cull(0, v, sc)[:2], "frustum after unbinding")


def test_bound_dynamic_rows_in_batch_rotate_and_clusters(stress_ctx, cluster_ctx):
    c, sc = stress_ctx
    n = 700
    rows = _moved_rows(sc, n, 22)
    bound = torch.from_numpy(rows.view(np.float32).reshape(-1).copy()).pin_memory()
    edited = S.Scene(sc.objects, sc.transforms.copy(), sc.surfaces, sc.lods)
    edited.transforms[:n] = rows
    c.bind_dynamic_transforms(bound)
    try:
        # a batch of frustum views reads the bound rows too
        views, keep, ref = _batch(c, sc, n_views=4, seed=23, mode=abi.MODE_FRUSTUM)
        abi.check(abi.load().blz_cull_batch(c.ctx, views, len(ref), None), "blz_cull_batch")
        assert c.check() == 0
        for i, (v, objs, _, t) in enumerate(ref):
            assert_records_equal(t.read(), O.cull(0, v, edited, objects=objs)[:2], f"batch view {i}, bound rows")
        # rotation starts from the bound row for ids below the bound count
        ids = np.array([3, 650, 699, 5000], np.uint32)
        axes = np.tile(np.array([[0.0, 0.0, 1.0]], np.float32), (4, 1))
        dst = torch.zeros(4 * 8, dtype=torch.float32, device="cuda")
        c.rotate_transforms(torch.from_numpy(ids.view(np.int32).copy()).cuda(), torch.from_numpy(axes.reshape(-1)).cuda(),
                            0.25, dst)
        assert c.check() == 0
        want = O.transforms_rotate(edited.transforms, ids, axes, 0.25)
        assert np.array_equal(dst.cpu().numpy().view(np.uint32), want.view(np.uint32).reshape(-1))
    finally:
        c.bind_dynamic_transforms(None)
    # the cluster cull of another context
    cc, csc = cluster_ctx
    crows = _moved_rows(csc, 300, 24)
    cedit = S.Scene(csc.objects, csc.transforms.copy(), csc.surfaces, csc.lods, clusters=csc.clusters)
    cedit.transforms[:300] = crows
    cb = torch.from_numpy(crows.view(np.float32).reshape(-1).copy()).pin_memory()
    v = view_for(zfar=1e4, position=(0.0, 0.0, -50.0))
    cap = O._cluster_upper_bound(csc, csc.objects)
    cc.bind_dynamic_transforms(cb)
    try:
        t = Target.alloc(cap)
        cc.cluster_cull(v, t)
        assert cc.check() == 0
        n, recs, _, _ = O.cull_clusters(v, cedit, capacity=cap)
        assert_records_equal(t.read(), (n, recs), "clusters, bound rows")
    finally:
        cc.bind_dynamic_transforms(None)


def test_bind_dynamic_argument_checks(stress_ctx):
    c, sc = stress_ctx
    rows = torch.zeros((len(sc.transforms) + 1) * 8, dtype=torch.float32, device="cuda")
    with pytest.raises(abi.BlzError):
        c.bind_dynamic_transforms(rows)  # more rows than the scene has transforms
    with pytest.raises(abi.BlzError):
        c.bind_dynamic_transforms(rows[4:12])  # not 32-byte aligned
    c.bind_dynamic_transforms(None)


def test_cluster_object_stage_matches_the_pinned_frustum_lod_path(lib):
    """With every cluster test made to pass (huge cluster spheres, open cones, no pyramid), the
    cluster cull emits exactly the chosen LOD's cluster range of every object the frustum + LOD cull
    emits: the cluster path's object stage agrees with the path pinned to the reference shaders."""
    sc = S.cluster_scene(6000, seed=7, clusters_per_mesh=60)
    sc.clusters["radius"] = 1e6
    sc.clusters["coneAxis"] = 0       # a zero axis never passes the cutoff (an int8 axis can be
    sc.clusters["coneCutoff"] = 127   # a little longer than 1, so cutoff 1.0 alone does not open it)
    c = Culler(0)
    try:
        c.setup_for_rendering(sc)
        v = view_for(zfar=1e4, position=(0.0, 0.0, -50.0))
        t = Target.alloc(sc.count)
        c.draw_cull(v, t)
        assert c.check() == 0
        n, recs = t.read()
        assert n > 100
        want_obj, want_ids = [], []
        for rec in recs:
            s = sc.surfaces[sc.objects[rec[0]]["surfaceId"]]
            lods = sc.lods[int(s["lodOffset"]):int(s["lodOffset"]) + int(s["lodCount"])]
            k = int(np.flatnonzero((lods["firstIndex"] == rec[3]) & (lods["indexCount"] == rec[1]))[0])
            off, cnt = int(lods[k]["clusterOffset"]), int(lods[k]["clusterCount"])
            want_obj += [int(rec[0])] * cnt
            want_ids += list(range(off, off + cnt))
        cap = len(want_ids) + 10
        ct = Target.alloc(cap)
        ids = torch.zeros(cap, dtype=torch.int32, device="cuda")
        c.cluster_cull(v, ct, cluster_ids=ids)
        assert c.check() == 0
        m, crecs = ct.read()
        assert m == len(want_ids)
        assert np.array_equal(crecs[:, 0], np.array(want_obj, np.uint32))
        assert np.array_equal(ids[:m].cpu().numpy().view(np.uint32), np.array(want_ids, np.uint32))
    finally:
        c.close()


def test_cluster_tasks_with_vulkan_hiz(cluster_ctx):
    """The task form against a Vulkan-form pyramid (PreviousPow2 mip 0, MIN-sampler footprint)."""
    c, sc = cluster_ctx
    pl, _ = abi.pyramid_layout(W, H, abi.HIZ_VULKAN)
    v = view_for(zfar=1e4, position=(0.0, 0.0, -50.0), pw=float(pl.width), ph=float(pl.height))
    depth = O.depth_raster(v, sc.boxes, W, H)
    pyr = DevicePyramid(W, H, abi.HIZ_VULKAN)
    c.generate_depth_pyramid(pyr, torch.from_numpy(depth).cuda())
    tasks, payloads = O.cluster_tasks(v, sc, pyramid=O.pyramid_build(depth, abi.HIZ_VULKAN))
    assert len(tasks) > 20
    t = TaskTarget.alloc(sc.count, len(payloads) + 3)
    c.cluster_task_cull(v, t, pyramid=pyr)
    assert c.check() == 0
    nt, np_, gt, gp = t.read()
    assert (nt, np_) == (len(tasks), len(payloads))
    assert np.array_equal(gt, tasks) and np.array_equal(gp, payloads)


def test_instanced_with_bound_dynamic_rows(stress_ctx):
    c, sc = stress_ctx
    n, slots = 2000, 100_000
    rows = _moved_rows(sc, n, 31)
    bound = torch.from_numpy(rows.view(np.float32).reshape(-1).copy()).pin_memory()
    edited = S.Scene(sc.objects, sc.transforms.copy(), sc.surfaces, sc.lods)
    edited.transforms[:n] = rows
    v = view_for(zfar=1e4)
    ctr = O.new_counters(sc, slots)
    cap = len(sc.lods) * slots
    dctr = torch.from_numpy(ctr.view(np.int32).reshape(-1).copy()).cuda()
    dinst = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
    t = Target.alloc(len(sc.lods), abi.STRIDE_D3D12)
    c.bind_dynamic_transforms(bound)
    try:
        c.draw_instance_cull_pass(v, dctr, dinst, slots, t)
        assert c.check() == 0
    finally:
        c.bind_dynamic_transforms(None)
    m, cmds, octr, oinst, _ = O.cull_instanced(v, edited, ctr, cap, slots, stride=abi.STRIDE_D3D12)
    assert_records_equal(t.read(), (m, cmds), "instanced commands, bound rows")
    assert np.array_equal(dctr.cpu().numpy().view(np.uint32), octr.view(np.uint32).reshape(-1))
    assert np.array_equal(dinst.cpu().numpy().view(np.uint32), oinst)
