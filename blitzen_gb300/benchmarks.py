"""Secondary measurements reported next to the headline frame.

batched_views  64 views over the resident stress scene, each with its own camera (random position in
               the scene, random yaw and pitch), its own log-uniform object subset (1k..2M) and its own
               pyramid from a 1920x1080 depth of occluders in front of it; frustum + Hi-Z + LOD per
               view (the temporal pass). One persistent graph-replayed launch versus one launch per
               view, after the autotuner picked the launch shape. Every batched result is compared
               with the per-view result (bit-exact) before anything is timed.
serving        the request loop over the resident scene: Poisson arrivals at 2,000 requests/s, each a
               camera over a window of 1k..1M objects with the 1,000 dynamic objects rotated by
               0.01 rad about random axes; p50/p99 latency from arrival to result and objects/s.
instanced      the instanced cull over the resident scene (256 LODs x 100k instance slots).
clusters       the cluster cull over 50k objects of ~200 clusters each, with Hi-Z and cone test.
"""
from __future__ import annotations

import ctypes as C
import math
import sys
import threading
import time

import numpy as np
import torch

from . import abi
from . import scenes as S
from .abi import BatchView, RenderList
from .culler import DevicePyramid, Target, TaskTarget, to_device

W, H = 1920, 1080


def _camera_to_world(view: abi.CameraViewData, p: np.ndarray, position) -> np.ndarray:
    """World coordinates of camera-frame points: the view rotation transposed, plus the position."""
    m = np.frombuffer(bytes(view.viewMatrix), np.float32).reshape(4, 4)  # m[c, r] = element (r, c)
    # the view rotation is R^T with element (r, c) = m[c, r], so R[i][j] = m[i, j]; p_world = R p + position
    rot = m[:3, :3].astype(np.float64)
    return (p.astype(np.float64) @ rot.T + np.asarray(position, np.float64)).astype(np.float32)


def build_views(culler, scene, device, n_views=64, seed=0, lo=1000, hi=2_000_000, boxes_out=None):
    """The batched-views workload: per view a camera, a render list (a subset of the scene), an
    occluder depth rasterised on the GPU and its pyramid, and an output. `boxes_out`, when a list,
    receives each view's occluder boxes (world space), so that a check can rebuild the depth."""
    specs = S.multiview_specs(scene.count, n_views, seed=seed, lo=lo, hi=hi)
    rng = np.random.default_rng(seed + 7)
    views = (BatchView * n_views)()
    keep = []
    total = 0
    for i, sp in enumerate(specs):
        v = abi.view_setup(S.fov_radians(), float(W), float(H), S.ZNEAR, 1e4, sp.position, sp.yaw, sp.pitch,
                           W / 2, H / 2)
        objs = to_device(S.subset_objects(scene, sp.subset), device)
        boxes_cam = S.make_occluders(rng, 2000)
        lo_w = _camera_to_world(v, boxes_cam[:, :3], sp.position)
        hi_w = _camera_to_world(v, boxes_cam[:, 3:], sp.position)
        boxes = np.concatenate([np.minimum(lo_w, hi_w), np.maximum(lo_w, hi_w)], axis=1).astype(np.float32)
        if boxes_out is not None:
            boxes_out.append(boxes)
        depth = torch.zeros(W * H, dtype=torch.float32, device=device)
        culler.raster_boxes(v, torch.from_numpy(boxes.reshape(-1)).to(device), depth, W, H)
        pyr = DevicePyramid(W, H, abi.HIZ_D3D12, device)
        culler.generate_depth_pyramid(pyr, depth)
        t = Target.alloc(len(sp.subset), abi.STRIDE_VULKAN, device)
        views[i].view = v
        views[i].list = RenderList(objs.data_ptr(), len(sp.subset))
        views[i].mode = abi.MODE_TEMPORAL
        views[i].pyramid = C.pointer(pyr.desc)
        views[i].target = t.ctype()
        keep.append((objs, pyr, t))
        total += len(sp.subset)
    torch.cuda.synchronize(device)
    return views, keep, total


def _time(fn, reps, stream):
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = []
    for _ in range(reps):
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        out.append(a.elapsed_time(b))
    return float(np.median(out))


def batched_views(culler, scene, device, n_views=64, reps=20, shape=None) -> dict:
    """64 views of log-uniform size over the resident scene: one batched launch (and its graph)
    against one launch per view. shape = (threads, objects per thread, blocks per SM[, objects per
    chunk]) fixes the launch shape; by default the autotuner picks it and its chunk size."""
    lib = abi.load()
    views, keep, total = build_views(culler, scene, device, n_views)
    stream = torch.cuda.current_stream(device)
    sp = C.c_void_p(stream.cuda_stream)

    # the per-view arm first, with the context's own single-view launch shape (setting a batch
    # shape below can change that one too)
    abi.check(lib.blz_cull_batch_per_view(culler.ctx, views, n_views, sp), "per view")
    per_view = [k[2].read() for k in keep]
    for _ in range(3):
        lib.blz_cull_batch_per_view(culler.ctx, views, n_views, sp)
    t_per = _time(lambda: lib.blz_cull_batch_per_view(culler.ctx, views, n_views, sp), reps, stream)

    best, us = abi.LaunchShape(), C.c_float(0)
    if shape is None:  # autotuned launch shape for this batch
        abi.check(lib.blz_autotune_batch(culler.ctx, views, n_views, 3, sp, C.byref(best), C.byref(us)), "autotune")
    else:
        best = abi.LaunchShape(shape[0], shape[1], shape[2], shape[3] if len(shape) > 3 else 0)
        abi.check(lib.blz_set_launch_shape(culler.ctx, C.byref(best)), "launch shape")

    # parity: batched == per-view, record by record, before timing the batch
    abi.check(lib.blz_cull_batch(culler.ctx, views, n_views, sp), "batch")
    batched = [k[2].read() for k in keep]
    culler.check(stream)
    identical = all(a[0] == b[0] and np.array_equal(a[1], b[1]) for a, b in zip(batched, per_view))

    g = C.c_void_p()
    abi.check(lib.blz_batch_graph_create(culler.ctx, views, n_views, sp, C.byref(g)), "graph")
    try:
        for _ in range(3):
            lib.blz_batch_graph_launch(g, sp)
        t_graph = _time(lambda: lib.blz_batch_graph_launch(g, sp), reps, stream)
        t_batch = _time(lambda: lib.blz_cull_batch(culler.ctx, views, n_views, sp), reps, stream)
    finally:
        lib.blz_batch_graph_destroy(g)
    culler.check(stream)
    return {
        "views": n_views, "objects": total, "identical_to_per_view": identical,
        "launch_shape": {"threads": best.threadsPerBlock, "objects_per_thread": best.objectsPerThread,
                         "blocks_per_sm": best.blocksPerSm, "chunk_objects": best.chunkObjects or 512,
                         "autotune_us": float(us.value) if shape is None else None},
        "batched_graph_ms": t_graph, "batched_ms": t_batch, "per_view_ms": t_per,
        "batched_objects_per_s": total / (t_graph * 1e-3), "per_view_objects_per_s": total / (t_per * 1e-3),
        "speedup": t_per / t_graph,
        "draws": int(sum(b[0] for b in batched)),
    }


def _serve_run(culler, scene, n_req, seed, arrivals=None, max_outstanding=None) -> dict:
    """One run of the request loop over the resident scene: n_req cull requests (view windows of
    log-uniform 1k-1M objects, 1,000 dynamic rotations each), submitted at the given arrival times
    (open loop) or whenever fewer than max_outstanding are unfinished (closed loop). A fresh server
    per run, so its latency statistics are the run's own."""
    lib = abi.load()
    cfg = abi.ServeConfig(2 << 30, 4, 64, 1000, abi.STRIDE_VULKAN)
    server = C.c_void_p()
    abi.check(lib.blz_serve_create(culler.ctx, C.byref(cfg), C.byref(server)), "serve create")
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(math.log(1000), math.log(1_000_000), n_req)).astype(np.int64)
    starts = np.array([rng.integers(0, scene.count - c) for c in counts])
    axes = rng.normal(size=(64, 1000, 3))
    axes = (axes / np.linalg.norm(axes, axis=2, keepdims=True)).astype(np.float32)
    objs_dev = culler.scene_tensors[0]
    views = []
    for k in range(64):
        pos = tuple(float(x) for x in rng.uniform(-4000, 4000, 3).astype(np.float32))
        views.append(abi.view_setup(S.fov_radians(), float(W), float(H), S.ZNEAR, 1e4, pos,
                                    float(rng.uniform(-3, 3)), float(rng.uniform(-0.5, 0.5)), W / 2, H / 2))
    tickets = []
    lock = threading.Lock()
    done = threading.Event()
    released = []

    def consumer():
        i = 0
        while True:
            with lock:
                ready = i < len(tickets)
                t = tickets[i] if ready else None
            if not ready:
                if done.is_set():
                    with lock:
                        if i >= len(tickets):
                            return
                    continue
                time.sleep(20e-6)
                continue
            res = abi.ServeResult()
            lib.blz_serve_wait(server, t, 60_000, C.byref(res))
            lib.blz_serve_release(server, t)
            released.append(res.status)
            i += 1

    th = threading.Thread(target=consumer, daemon=True)
    old_switch = sys.getswitchinterval()
    sys.setswitchinterval(2e-5)  # the consumer thread must get the GIL between arrivals
    th.start()
    late = 0.0  # how far behind its schedule the open-loop submission ran, at most
    t0 = time.perf_counter()
    req = abi.ServeRequest()
    for k in range(n_req):
        if arrivals is not None:
            while True:  # sleep through the gap (releasing the GIL), spin only its last 100 us
                left = arrivals[k] - (time.perf_counter() - t0)
                if left <= 0:
                    late = max(late, -left)
                    break
                if left > 150e-6:
                    time.sleep(left - 100e-6)
        else:
            while k - len(released) >= max_outstanding:
                time.sleep(10e-6)
        req.view = views[k % 64]
        req.list = RenderList(objs_dev.data_ptr() + int(starts[k]) * 8, int(counts[k]))
        req.mode = abi.MODE_FRUSTUM
        req.rotateCount = 1000
        req.rotateAxes = axes[k % 64].ctypes.data
        req.rotateAngle = 0.01
        req.copyToHost = 0
        t = C.c_uint64()
        abi.check(lib.blz_serve_submit(server, C.byref(req), C.byref(t)), "submit")
        with lock:
            tickets.append(t.value)
    done.set()
    th.join()
    sys.setswitchinterval(old_switch)
    elapsed = time.perf_counter() - t0
    st = abi.ServeStats()
    lib.blz_serve_stats(server, C.byref(st))
    lib.blz_serve_destroy(server)
    return {"requests": n_req, "elapsed_s": elapsed, "achieved_rate_per_s": n_req / elapsed,
            "p50_ms": st.p50Ms, "p99_ms": st.p99Ms, "mean_ms": st.meanMs, "max_ms": st.maxMs,
            "batches": st.batches, "max_batch": st.maxBatchSize, "max_concurrent_batches": st.maxConcurrentBatches,
            "objects_per_s": float(counts.sum()) / elapsed, "errors": int(sum(1 for s in released if s)),
            "submit_late_ms": late * 1e3}


def serving(culler, scene, device, seconds=2.0, rates=(2000.0, 8000.0, 20000.0, 50000.0), p99_bound_ms=1.0,
            seed=0) -> dict:
    """The serving loop at Poisson arrival rates (open loop, `seconds` each) and closed loop with 64
    requests outstanding (its saturation throughput). Latency runs from a request's submission to
    its completion event; `submit_late_ms` says how far the submitting thread fell behind the
    schedule, so a point whose submissions could not keep up is visible as such.
    `max_rate_p99_under_bound` is the highest offered rate whose p99 stayed under p99_bound_ms and
    whose requests were all served at that rate."""
    curve = []
    for i, rate in enumerate(rates):
        rng = np.random.default_rng(seed + 17 * i)
        n_req = int(seconds * rate)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
        pt = _serve_run(culler, scene, n_req, seed + i, arrivals=arrivals)
        pt["offered_rate_per_s"] = rate
        curve.append(pt)
    closed = _serve_run(culler, scene, 40_000, seed + 99, max_outstanding=64)
    ok = [p["offered_rate_per_s"] for p in curve
          if p["p99_ms"] < p99_bound_ms and p["errors"] == 0 and p["achieved_rate_per_s"] >= 0.95 * p["offered_rate_per_s"]]
    first = curve[0]
    return {"offered_rate_per_s": first["offered_rate_per_s"], "p50_ms": first["p50_ms"], "p99_ms": first["p99_ms"],
            "objects_per_s": first["objects_per_s"], "curve": curve, "p99_bound_ms": p99_bound_ms,
            "max_rate_p99_under_bound": max(ok) if ok else None,
            "saturation": {"outstanding": 64, "requests_per_s": closed["achieved_rate_per_s"],
                           "objects_per_s": closed["objects_per_s"], "p50_ms": closed["p50_ms"],
                           "p99_ms": closed["p99_ms"], "max_batch": closed["max_batch"], "errors": closed["errors"]}}


def _replay_ms(culler, fn, reps, flush, stream) -> float:
    """Mean CUDA-event time of `fn` recorded once and replayed as a graph, L2 flushed before each.
    The mean, not the median: the event timer advances in steps of about 2 us on these GPUs, so a
    median snaps to one of those steps while the mean of many replays resolves finer."""
    with torch.cuda.stream(stream):
        fn()
        culler.capture_begin()
        fn()
        g = culler.capture_end()
        for _ in range(3):
            g.launch()
        times = []
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(reps):
            flush.sum(dtype=torch.int64)
            a.record()
            g.launch()
            b.record()
            b.synchronize()
            times.append(a.elapsed_time(b))
        g.close()
    return float(np.mean(times))


def instanced(culler, scene, device, reps=30, slots=100_000) -> dict:
    """The instanced cull (drawInstCull) over the resident stress scene, 256 LODs x 100k slots."""
    v = abi.view_setup(S.fov_radians(), float(W), float(H), S.ZNEAR, 1e4, (0, 0, 0), 0, 0, W / 2, H / 2)
    n_lods = len(scene.lods)
    ctr = np.zeros(n_lods, abi.LOD_INSTANCE_COUNTER)
    ctr["instanceOffset"] = np.arange(n_lods, dtype=np.uint64) * slots
    dctr = to_device(ctr, device)
    inst = torch.empty(n_lods * slots, dtype=torch.int32, device=device)
    t = Target.alloc(n_lods, abi.STRIDE_VULKAN, device)
    flush = torch.ones(128 << 20, dtype=torch.int32, device=device)
    side = torch.cuda.Stream(device)
    ms = _replay_ms(culler, lambda: culler.draw_instance_cull_pass(v, dctr, inst, slots, t), reps, flush, side)
    culler.check(side)
    counts = dctr.cpu().numpy().view(np.uint32).reshape(-1, 2)[:, 1]
    visible = int(counts.sum())
    n_cmd = int(t.read()[0])
    nbytes = scene.count * (8 + 32) + 4 * visible + 8 * n_lods * 2 + n_cmd * abi.STRIDE_VULKAN
    return {"objects": scene.count, "visible_instances": visible, "commands": n_cmd, "ms": ms,
            "objects_per_s": scene.count / (ms * 1e-3), "algorithmic_bytes": nbytes,
            "GB/s": nbytes / (ms * 1e-3) / 1e9}


def clusters(device, reps=30) -> dict:
    """The cluster cull over the cluster configuration: 50k objects, 32 meshes of ~200 clusters,
    frustum + LOD per object, then sphere frustum + Hi-Z + normal cone per cluster.

    The rate reported is cluster tests per second: the clusters actually tested (the chosen LOD's
    clusters of every object inside the frustum) over the time. That count is measured on the GPU by
    the same cull over a copy of the scene whose clusters pass every test (radius 1e6, a zero cone
    axis with cutoff 127, no pyramid), which emits exactly its candidates."""
    from .culler import Culler
    sc = S.cluster_scene(50_000, seed=0)
    c = Culler(device.index if device.index is not None else 0)
    try:
        v = abi.view_setup(S.fov_radians(), float(W), float(H), S.ZNEAR, 1e4, (0.0, 0.0, -50.0), 0, 0, W / 2, H / 2)
        per_surface = np.array([int(sc.lods[int(s["lodOffset"]):int(s["lodOffset"]) + int(s["lodCount"])]["clusterCount"].max())
                                for s in sc.surfaces], np.int64)
        cap = int(per_surface[sc.objects["surfaceId"]].sum())
        t = Target.alloc(cap, abi.STRIDE_VULKAN, device)
        ids = torch.empty(cap, dtype=torch.int32, device=device)
        # the number of clusters tested: the same cull with every cluster test passing
        opened = S.Scene(sc.objects, sc.transforms, sc.surfaces, sc.lods, clusters=sc.clusters.copy())
        opened.clusters["radius"] = np.float32(1e6)
        opened.clusters["coneAxis"] = 0
        opened.clusters["coneCutoff"] = 127
        c.setup_for_rendering(opened)
        c.cluster_cull(v, t)
        c.check()
        tested = int(t.read()[0])
        c.setup_for_rendering(sc)
        depth = torch.zeros(W * H, dtype=torch.float32, device=device)
        c.raster_boxes(v, torch.from_numpy(sc.boxes.reshape(-1)).to(device), depth, W, H)
        pyr = DevicePyramid(W, H, abi.HIZ_D3D12, device)
        c.generate_depth_pyramid(pyr, depth)
        flush = torch.ones(128 << 20, dtype=torch.int32, device=device)
        side = torch.cuda.Stream(device)
        ms = _replay_ms(c, lambda: c.cluster_cull(v, t, pyramid=pyr, cluster_ids=ids), reps, flush, side)
        c.check(side)
        n = int(t.read()[0])
        nbytes = sc.count * (8 + 32) + sc.clusters.nbytes + n * (abi.STRIDE_VULKAN + 4)
        # the mesh-shader form of the same cull: one task per object, payloads of 32 meshlets
        tt = TaskTarget.alloc(sc.count, (cap + 31) // 32 + sc.count)
        ms_t = _replay_ms(c, lambda: c.cluster_task_cull(v, tt, pyramid=pyr), reps, flush, side)
        c.check(side)
        nt, npl = (int(x) for x in tt.read()[:2])
        tbytes = sc.count * (8 + 32) + sc.clusters.nbytes + nt * 16 + npl * 132
        return {"objects": sc.count, "clusters_in_scene": len(sc.clusters), "clusters_tested": tested,
                "cluster_capacity_bound": cap, "clusters_emitted": n, "ms": ms,
                "objects_per_s": sc.count / (ms * 1e-3), "cluster_tests_per_s": tested / (ms * 1e-3),
                "algorithmic_bytes": nbytes, "GB/s": nbytes / (ms * 1e-3) / 1e9,
                "task_form": {"ms": ms_t, "tasks": nt, "payloads": npl, "algorithmic_bytes": tbytes,
                              "cluster_tests_per_s": tested / (ms_t * 1e-3)}}
    finally:
        c.close()


def run_extras(culler, scene, device) -> dict:
    out = {}
    try:
        out["instanced"] = instanced(culler, scene, device)
    except Exception as ex:
        out["instanced"] = {"error": repr(ex)}
    try:
        out["clusters"] = clusters(device)
    except Exception as ex:
        out["clusters"] = {"error": repr(ex)}
    try:
        out["batched_views"] = batched_views(culler, scene, device)
    except Exception as ex:
        out["batched_views"] = {"error": repr(ex)}
    try:
        out["serving"] = serving(culler, scene, device)
    except Exception as ex:
        out["serving"] = {"error": repr(ex)}
    return out
