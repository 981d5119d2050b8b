"""Benchmark of the GPU-driven cull path (one JSON line on rank 0).

Workload (the stress configuration): 4,000,000 render objects in [-5000,5000]^3 over 64 meshes x 4
LODs; one step is one occlusion frame of the reference's path (VulkanRenderer::DrawFrame,
vulkanDraw.cpp:1015-1031; dx12Draw.cpp:590-641), the draws aside:
  pass 1   objects visible last frame (random 50% bitmask): frustum + LOD, pass-1 records
  pyramid  Hi-Z over a 1920x1080 fp32 reverse-Z depth buffer (2,000 occluder boxes)
  pass 2   every object: frustum + Hi-Z + LOD, pass-2 records, visibility rewritten
Inputs are resident in HBM when the timed region starts; before each step the visibility buffer is
restored to the 50% mask and L2 is flushed (a 512 MiB read), both outside the timed events.

value  = objects per second of the device-timed frames: each step replays blz_cull_frame (recorded
         once with blz_capture_begin/end) as one CUDA graph between two CUDA events. That frame is
         two launches: one building the pyramid's tiles and then deciding both passes for every
         object in one sweep, one writing both record lists. The frame's
         other forms (blz_frame_first + blz_pyramid_build + blz_frame_late; blz_cull_first +
         blz_pyramid_build + blz_cull_late) are timed the same way in `frame_forms`, and every part
         as its own graph in `roofline.others`. All three forms give the same records, counts,
         pyramid and visibility, checked against the oracle (`bit_exact`).
roofline = the headline frame's sweep (blz_cull_frame over the pyramid already built: the decide
         launch for both passes and the launch writing both record lists), algorithmic bytes over
         its CUDA-event time, against the measured copy bandwidth. `others.frame` is the whole
         frame against its bytes, pyramid included.
e2e    = the same frame through the C ABI with host buffers, all inside the timed region: the host
         writes the 1,000 dynamic transform rows into a pinned buffer and replays the recorded step
         (blz_graph_launch): the 8.3 MB depth upload and the pyramid run beside blz_frame_first,
         then blz_frame_late, and both draw counts land in pinned host memory, which the host reads.
--impl reference runs the CPU oracle (a port of the reference's shaders, all host threads) on the
same frames.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

W, H = 1920, 1080
DYNAMIC = 1000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--objects", type=int, default=4_000_000)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="bounded CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--shape", default="", help="launch shape THREADSxOBJECTS_PER_THREAD (default: library default)")
    ap.add_argument("--no-clock-hold", action="store_true",
                    help="do not extend the load to 1.5 s for the clock sampler (profiling runs)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(ms: float, world: int, device) -> float:
    """The slowest rank's step time (each rank culls its own frame; the job takes the longest)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    tt = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def job_throughput(objects_per_rank: int, world: int, ms: float) -> float:
    """Objects per second of the whole job: every rank's objects over the slowest rank's time."""
    return objects_per_rank * world / (ms * 1e-3)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows: list[list[str]] = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) >= 9:
                for k, name in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


# ----------------------------------------------------------------------------- reference arm

def oracle_frame(sc, v, depth, threads):
    """One stress frame of the oracle (the multithreaded C port of the reference's shaders) with every
    buffer allocated beforehand: frame() restores the visibility mask, then times bo_cull pass 1,
    bo_pyramid_build and bo_cull pass 2 alone, and returns (seconds, (n1, records1), (n2, records2),
    pyramid, visibility)."""
    from oracle import oracle as O
    desc = O.scene_desc(sc)
    out1 = np.zeros((sc.count, 6), np.uint32)
    out2 = np.zeros((sc.count, 6), np.uint32)
    pyr = O.HostPyramid(W, H, 0)
    vis = sc.visibility.copy()
    depth = np.ascontiguousarray(depth, dtype=np.float32)

    def frame():
        np.copyto(vis, sc.visibility)
        t0 = time.perf_counter()
        n1, r1, _ = O.cull(1, v, sc, vis=vis, threads=threads, out=out1, desc=desc)
        O.pyramid_build(depth, into=pyr)
        n2, r2, _ = O.cull(2, v, sc, vis=vis, pyramid=pyr, threads=threads, out=out2, desc=desc)
        return time.perf_counter() - t0, (n1, r1), (n2, r2), pyr, vis

    return frame


def time_oracle_frames(frame, min_frames: int, seconds: float) -> list[float]:
    """At least min_frames timed frames, more while the time budget lasts."""
    times = []
    t_end = time.perf_counter() + seconds
    while len(times) < min_frames or time.perf_counter() < t_end:
        times.append(frame()[0])
        if len(times) >= min_frames and time.perf_counter() > t_end:
            break
    return times


def run_reference(args, rank, world):
    """The CPU oracle on the full stress frame, every host thread; rank 0 only."""
    if rank != 0:
        return
    from blitzen_gb300 import scenes as S
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    sc = S.stress_scene(args.objects, seed=args.seed)
    v = O.view_setup(S.fov_radians(), float(W), float(H), S.ZNEAR, S.STRESS_ZFAR, (0, 0, 0), 0, 0, W / 2, H / 2)
    frame = oracle_frame(sc, v, O.depth_raster(v, sc.boxes, W, H), threads)
    for _ in range(max(1, min(args.warmup, 2))):
        frame()
    times = time_oracle_frames(frame, max(5, args.steps), 0.0)
    per = statistics.median(times)
    value = args.objects / per
    line = {
        "impl": "reference", "metric": "objects culled/s (4M-object two-pass occlusion frame)", "value": value,
        "unit": "objects/s", "n_gpus": world, "steps": len(times), "warmup": args.warmup,
        "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)", "config": workload_config(args),
        "cpu_baseline": {"value": value, "unit": "objects/s", "cores": threads, "kind": "port",
                         "sample": f"median of {len(times)} full {args.objects}-object frames (bo_cull pass 1 + "
                                   f"bo_pyramid_build + bo_cull pass 2; buffers preallocated, visibility "
                                   f"restored outside the clock)"},
        "e2e": {"value": value, "unit": "objects/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(args):
    return {"workload": "stress scene two-pass occlusion frame", "objects": args.objects, "meshes": 64, "lods": 256,
            "depth": f"{W}x{H} fp32 reverse-Z, 2000 occluder boxes", "pass1_visible_fraction": 0.5,
            "hiz": "d3d12", "record_stride": 24, "l2": "flushed between steps (512 MiB read)",
            "parallelism": "one frame per GPU (weak scaling, no collective)"}


# ----------------------------------------------------------------------------- our arm

def frame_matches(want, t1, t2, vis, pyr) -> bool:
    """Both draw counts, every word of every record, the visibility buffer and every pyramid texel
    equal the oracle's frame `want` = ((n1, records1), (n2, records2), pyramid words, visibility)."""
    (n1, r1), (n2, r2), pyr_words, ovis = want
    g1, g2 = t1.read(), t2.read()
    ok = g1[0] == n1 and np.array_equal(g1[1], r1) and g2[0] == n2 and np.array_equal(g2[1], r2)
    ok = ok and np.array_equal(vis.cpu().numpy().view(np.uint32), ovis)
    ok = ok and np.array_equal(pyr.storage.cpu().numpy().view(np.uint32), pyr_words.view(np.uint32))
    return bool(ok)


def recorded_traffic(kernels, objects: int):
    """DRAM bytes of one launch of each of `kernels`, summed, on the stress frame from the committed
    ncu figures, or None when a kernel is missing or was captured on another scene size."""
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as f:
            d = json.load(f)
        es = [d["kernels"][k] for k in kernels]
        if any(int(e["objects"]) != objects for e in es):
            return None
        return {"bytes_per_launch": sum(int(e["dram_bytes_per_launch"]) for e in es),
                "source": "; ".join(f"{k}: ncu capture at commit {e['commit']}: {e['command']}" for k, e in zip(kernels, es))}
    except Exception:
        return None


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    import torch.distributed as dist

    from blitzen_gb300 import abi
    from blitzen_gb300 import scenes as S
    from blitzen_gb300.culler import Culler, DevicePyramid, Target

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl")

    sc = S.stress_scene(args.objects, seed=args.seed + rank)
    N = sc.count
    c = Culler(local)
    if args.shape:
        t_, o_ = (int(x) for x in args.shape.lower().split("x"))
        c.set_launch_shape(t_, o_)
    c.setup_for_rendering(sc)
    v = S.stress_view()
    depth = torch.zeros(W * H, dtype=torch.float32, device=dev)
    c.raster_boxes(v, torch.from_numpy(sc.boxes.reshape(-1)).to(dev), depth, W, H)
    vis0 = torch.from_numpy(sc.visibility.view(np.int32).copy()).to(dev)
    vis = vis0.clone()
    t1, t2 = Target.alloc(N, abi.STRIDE_VULKAN, dev), Target.alloc(N, abi.STRIDE_VULKAN, dev)
    pyr = DevicePyramid(W, H, abi.HIZ_D3D12, dev)
    # L2 flush by reading 512 MiB (a read leaves clean lines, so the next kernel pays no write-back)
    flush = torch.ones(128 << 20, dtype=torch.int32, device=dev)

    def flush_l2():
        flush.sum(dtype=torch.int64)

    n_prev = int(sc.visibility.sum())

    side = torch.cuda.Stream(dev)  # graphs are captured from, and replayed on, a non-default stream

    # The frame in the library's three forms, each one step of the workload:
    #   one_call        blz_cull_frame: the pyramid's tiles, then one sweep deciding both passes for
    #                   every object (each warp waits for the finished pyramid before its first Hi-Z
    #                   test), then both record lists in one launch
    #   kept_frame      blz_frame_first, blz_pyramid_build, blz_frame_late (the renderer's order)
    #   separate_calls  blz_cull_first, blz_pyramid_build, blz_cull_late (each pass on its own)
    def frame_one_call():
        c.cull_frame(v, vis, depth, pyr, t1, t2)

    def frame_kept():
        c.frame_first_pass(v, vis, t1)
        c.generate_depth_pyramid(pyr, depth)
        c.frame_occlusion_pass(pyr, t2)

    def frame_calls():
        c.draw_cull_first_pass(v, vis, t1)
        c.generate_depth_pyramid(pyr, depth)
        c.draw_cull_occlusion_pass(v, vis, pyr, t2)

    forms = {"one_call": frame_one_call, "kept_frame": frame_kept, "separate_calls": frame_calls}

    # the oracle's answer for this frame (every host thread), the reference every check below uses
    threads = os.cpu_count() or 1
    hdepth_np = depth.cpu().numpy().reshape(H, W)
    _, o1, o2, opyr, ovis = oracle_frame(sc, v, hdepth_np, threads)()
    want = ((o1[0], o1[1].copy()), (o2[0], o2[1].copy()), opyr.data.copy(), ovis.copy())
    exact = {}

    def timed(g, n):
        """n replays of graph g, each after restoring the visibility mask and flushing L2 (both outside
        the events); the per-replay CUDA-event times in ms."""
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        for a, b in evs:
            vis.copy_(vis0)
            flush_l2()
            a.record()
            g.launch()
            b.record()
        side.synchronize()
        return [a.elapsed_time(b) for a, b in evs]

    with torch.cuda.stream(side):
        for name, fn in forms.items():
            for _ in range(max(args.warmup, 3)):
                vis.copy_(vis0)
                fn()
            side.synchronize()
            c.check()
            exact[name] = frame_matches(want, t1, t2, vis, pyr)
        V1, _ = t1.read()
        V2, _ = t2.read()
        graphs = {}
        for name, fn in forms.items():
            c.capture_begin()
            fn()
            graphs[name] = c.capture_end()
        kernels_per_step = graphs["one_call"].kernels
        # each part on its own, for the breakdown (frame_late reuses what the last pass 1 kept)
        parts = {}
        for name, fn in (("sweep", lambda: c.cull_frame(v, vis, None, pyr, t1, t2)),
                         ("frame_first", lambda: c.frame_first_pass(v, vis, t1)),
                         ("pyramid", lambda: c.generate_depth_pyramid(pyr, depth)),
                         ("frame_late", lambda: c.frame_occlusion_pass(pyr, t2)),
                         ("pass1", lambda: c.draw_cull_first_pass(v, vis, t1)),
                         ("pass2", lambda: c.draw_cull_occlusion_pass(v, vis, pyr, t2))):
            c.capture_begin()
            fn()
            parts[name] = c.capture_end()
        # the separate-calls frame without pass 2 (pass 2 inside that frame = the difference)
        c.capture_begin()
        c.draw_cull_first_pass(v, vis, t1)
        c.generate_depth_pyramid(pyr, depth)
        frame_ab = c.capture_end()
        head = graphs["one_call"]
        timed(head, max(args.warmup, 3))

        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        with ClockSampler(local) as clocks:
            wall0 = time.perf_counter()
            ms = timed(head, args.steps)
            wall = time.perf_counter() - wall0
            launches = kernels_per_step * args.steps
            # keep the same load on the GPU until the sampler has seen at least 1.5 s of it
            while not args.no_clock_hold and time.perf_counter() - wall0 < 1.5:
                timed(head, 20)
        # the state the last timed replay left: both record lists, the pyramid and the visibility
        exact["timed_frame"] = frame_matches(want, t1, t2, vis, pyr)
        t_form = {name: statistics.mean(timed(g, args.steps)) for name, g in graphs.items()}
        t_part = {name: statistics.mean(timed(g, args.steps)) for name, g in parts.items()}
        # the sweep over the pyramid the replays left: the same frame as the headline's
        vis.copy_(vis0)
        parts["sweep"].launch()
        side.synchronize()
        exact["sweep"] = frame_matches(want, t1, t2, vis, pyr)
        t_ab = statistics.mean(timed(frame_ab, args.steps))
    c.check()
    t_step = max_over_ranks(sum(ms) / len(ms), world, dev)
    if world > 1:
        dist.barrier()
    value = job_throughput(N, world, t_step)

    # roofline: the dominant work of the headline frame is its sweep, the two launches after the
    # pyramid (cull_decide_kernel<5> deciding both passes for every object, cull_scatter2_kernel
    # writing both record lists), timed as blz_cull_frame over the pyramid already built. Its
    # algorithmic bytes are what the reference's two passes must move: each object's render object
    # and transform read once, its visibility word read once and rewritten (pass 2 writes every
    # object's), both record lists and their counts
    stride = abi.STRIDE_VULKAN
    mip_bytes = pyr.storage.numel() * 4
    bytes_pyr = W * H * 4 + mip_bytes
    bytes_sweep = N * (8 + 32) + 4 * N + 4 * N + (V1 + V2) * stride + 8
    bytes_a = N * (8 + 32 + 4) + 4 * (n_prev - V1) + V1 * stride + 4
    bytes_frame = bytes_sweep + bytes_pyr
    bytes_late = N * (8 + 32) + 4 * N + 4 * N + V2 * stride + 4
    bytes_first = 4 * N + n_prev * (8 + 32) + V1 * stride + 4
    peak, peak_kind = peaks()
    t_sw = t_part["sweep"]
    ach = bytes_sweep / (t_sw * 1e-3) / 1e9

    def gbs(b, t):
        return b / (t * 1e-3) / 1e9

    roofline = {"bound": "hbm", "kernel": "one-call frame sweep: cull_decide_kernel<5> + cull_scatter2_kernel",
                "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "peak_source": peak_kind,
                "traffic": None, "algorithmic_bytes": bytes_sweep, "ms": t_sw,
                "ms_note": "blz_cull_frame with no depth (the pyramid already built) recorded as its own graph: "
                           "the headline frame without its pyramid tiles",
                "others": {
                    "frame": {"ms": t_step, "bytes": bytes_frame, "GB/s": gbs(bytes_frame, t_step),
                              "frac": gbs(bytes_frame, t_step) / peak,
                              "note": "blz_cull_frame (the timed step; the pyramid built inside its sweep launch); "
                                      "bytes: every object's tables and visibility read once, visibility written "
                                      "once, both record lists, the depth buffer read and the pyramid written"},
                    "frame_first": {"ms": t_part["frame_first"], "bytes": bytes_a,
                                    "GB/s": gbs(bytes_a, t_part["frame_first"]),
                                    "frac": gbs(bytes_a, t_part["frame_first"]) / peak,
                                    "note": "kept frame's pass 1 (cull_decide_kernel<4> + cull_scatter_kernel); "
                                            "bytes: tables + visibility read, the visibility words it settles, "
                                            "pass 1's records"},
                    "frame_late": {"ms": t_part["frame_late"], "note": "survivors' pyramid test + scatter"},
                    "pyramid": {"ms": t_part["pyramid"], "bytes": bytes_pyr, "GB/s": gbs(bytes_pyr, t_part["pyramid"])},
                    "pass1": {"ms": t_part["pass1"], "bytes": bytes_first, "GB/s": gbs(bytes_first, t_part["pass1"])},
                    "pass2": {"ms": t_part["pass2"], "bytes": bytes_late, "GB/s": gbs(bytes_late, t_part["pass2"]),
                              "ms_in_separate_frame": t_form["separate_calls"] - t_ab,
                              "frac_in_separate_frame": gbs(bytes_late, t_form["separate_calls"] - t_ab) / peak}}}
    frames = {name: {"ms": t, "objects_per_s": job_throughput(N, world, t)} for name, t in t_form.items()}
    # DRAM bytes per launch from an ncu capture (profiles/dram_traffic.json names the commit and the
    # command it was taken with); a capture, not a measurement of this run
    traffic = recorded_traffic(("cull_decide_kernel<5>", "cull_scatter2_kernel"), args.objects)
    if traffic:
        roofline["traffic"] = traffic["bytes_per_launch"]
        roofline["traffic_source"] = traffic["source"]
    frame_traffic = recorded_traffic(("cull_frame_kernel<0,256,2>", "cull_scatter2_kernel"), args.objects)
    if frame_traffic:
        roofline["others"]["frame"]["traffic"] = frame_traffic["bytes_per_launch"]
        roofline["others"]["frame"]["traffic_source"] = frame_traffic["source"]

    # ---------------- e2e through the C ABI with host buffers
    hdepth = torch.empty(W * H, dtype=torch.float32, pin_memory=True)
    hdepth.copy_(depth.cpu())
    rng = np.random.default_rng(args.seed + 99)
    dyn_ids = np.arange(DYNAMIC, dtype=np.uint32)
    dyn_tr = sc.transforms[:DYNAMIC].copy()
    hcounts = torch.empty(2, dtype=torch.int32, pin_memory=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def e2e_run(frame_call):
        out = []
        for k in range(args.warmup + args.steps):
            vis.copy_(vis0)
            flush_l2()
            dyn_tr["orientation"] = S.random_unit_quaternions(rng, DYNAMIC)
            torch.cuda.synchronize()
            with torch.cuda.stream(side):  # the step's work on a non-default stream
                e0.record()
                c.update_object_transform(dyn_ids, dyn_tr)  # blz_transforms_update: host rows via pinned staging
                depth.copy_(hdepth, non_blocking=True)
                frame_call()
                hcounts[0:1].copy_(t1.count, non_blocking=True)
                hcounts[1:2].copy_(t2.count, non_blocking=True)
                e1.record()
            e1.synchronize()
            if k >= args.warmup:
                out.append(e0.elapsed_time(e1))
        return max_over_ranks(sum(out) / len(out), world, dev)

    # the serial forms: update, upload, the recorded one-call frame (or direct calls), count copies
    t_e2e_copies = e2e_run(graphs["one_call"].launch)
    t_e2e_direct = e2e_run(frame_one_call)

    # The whole step as one recorded graph over fixed pinned host buffers. The host writes the
    # step's 1,000 dynamic transform rows into a pinned buffer bound as the scene's dynamic rows
    # (transforms [0, 1000), the reference's dynamic-object range) and launches the graph. In it:
    #  - the depth upload (a copy-engine node, ~46 us for 8.3 MB over the CPU-GPU link) and the
    #    pyramid build run on a second stream beside pass 1, which does not read the depth;
    #  - both passes read the dynamic rows straight from pinned memory;
    #  - the scatter kernels write both draw counts into pinned host memory, which the host reads.
    # Pass 1 is the kept frame's (blz_frame_first) and pass 2 tests its survivors (blz_frame_late);
    # the separate-calls form of the same step is timed beside it.
    hcounts0 = torch.zeros(2, dtype=torch.int32, pin_memory=True)
    t1h = Target(t1.commands, hcounts0[0:1], t1.stride, t1.capacity)
    t2h = Target(t2.commands, hcounts0[1:2], t2.stride, t2.capacity)
    h_tr = torch.empty(DYNAMIC * 8, dtype=torch.float32, pin_memory=True)
    h_tr_np = h_tr.numpy().view(dyn_tr.dtype)
    h_tr_np[:] = dyn_tr
    c.bind_dynamic_transforms(h_tr)
    fork, join = torch.cuda.Event(), torch.cuda.Event()
    side2 = torch.cuda.Stream(dev)

    def record_step(pass1, pass2):
        with torch.cuda.stream(side):
            c.capture_begin()
            fork.record(side)
            side2.wait_event(fork)
            with torch.cuda.stream(side2):
                depth.copy_(hdepth, non_blocking=True)
                c.generate_depth_pyramid(pyr, depth)
            join.record(side2)
            pass1()
            side.wait_event(join)
            pass2()
            return c.capture_end()

    step_graphs = {
        "kept_frame": record_step(lambda: c.frame_first_pass(v, vis, t1h), lambda: c.frame_occlusion_pass(pyr, t2h)),
        "separate_calls": record_step(lambda: c.draw_cull_first_pass(v, vis, t1h),
                                      lambda: c.draw_cull_occlusion_pass(v, vis, pyr, t2h)),
    }

    def zero_copy_run(g):
        # the step runs on a non-default stream, as a renderer submits its frame: a launch on the
        # legacy default stream costs the host about 5 us more on these boxes
        out = []
        for k in range(args.warmup + args.steps):
            vis.copy_(vis0)
            flush_l2()
            dyn_tr["orientation"] = S.random_unit_quaternions(rng, DYNAMIC)
            torch.cuda.synchronize()
            e0.record(side)
            h_tr_np[:] = dyn_tr  # the step's input rows, host side
            g.launch(side)
            e1.record(side)
            e1.synchronize()
            counts = hcounts0.numpy().copy()  # the step's result, already in host memory
            if k >= args.warmup:
                out.append(e0.elapsed_time(e1))
        return max_over_ranks(sum(out) / len(out), world, dev), counts

    t_e2e_sep, _ = zero_copy_run(step_graphs["separate_calls"])
    t_e2e, counts = zero_copy_run(step_graphs["kept_frame"])

    # the CPU-GPU link's host-to-device rate, measured here: the step's depth upload alone (pinned
    # host buffer, one copy-engine copy), median of 20; the e2e step cannot finish before this upload
    # and the work that needs the depth (pyramid, pass 2) are done
    link_ms = []
    for _ in range(23):
        torch.cuda.synchronize()
        e0.record()
        depth.copy_(hdepth, non_blocking=True)
        e1.record()
        e1.synchronize()
        link_ms.append(e0.elapsed_time(e1))
    link_ms = statistics.median(link_ms[3:])
    link = {"h2d_GBs": W * H * 4 / (link_ms * 1e-3) / 1e9, "depth_upload_ms": link_ms,
            "upload_share_of_step": link_ms / t_e2e,
            "note": "measured host-to-device rate of the CPU-GPU link (8.3 MB depth copy from pinned memory); "
                    "the step's critical path is the upload, then the pyramid and pass 2 (pass 1 runs beside it)"}
    # the last recorded step against the oracle on the scene as that step saw it (its dynamic rows)
    edited = S.Scene(sc.objects, sc.transforms.copy(), sc.surfaces, sc.lods, visibility=sc.visibility)
    edited.transforms[:DYNAMIC] = h_tr_np
    _, e1_, e2_, eyr, evis = oracle_frame(edited, v, hdepth_np, threads)()
    t1_host = Target(t1.commands, torch.from_numpy(counts[0:1].copy()), t1.stride, t1.capacity)
    t2_host = Target(t2.commands, torch.from_numpy(counts[1:2].copy()), t2.stride, t2.capacity)
    exact["e2e_step"] = frame_matches(((e1_[0], e1_[1]), (e2_[0], e2_[1]), eyr.data, evis), t1_host, t2_host, vis, pyr)
    del edited
    for g in step_graphs.values():
        g.close()
    c.bind_dynamic_transforms(None)
    c.update_object_transform(dyn_ids, dyn_tr)  # the resident table catches up with the last step's rows
    e2e = {"value": job_throughput(N, world, t_e2e), "unit": "objects/s", "ms_per_step": t_e2e,
           "h2d_bytes_per_step": W * H * 4 + 2 * DYNAMIC * 32, "d2h_bytes_per_step": 8,
           "path": "host writes the 1,000 dynamic transform rows to a pinned buffer bound as the scene's dynamic rows "
                   "(blz_scene_bind_dynamic); one blz_graph_launch of the recorded step: depth upload + pyramid beside "
                   "blz_frame_first, then blz_frame_late; both passes read the rows over the CPU-GPU link; draw "
                   "counts written to pinned memory",
           "link": link,
           "separate_calls": {"value": job_throughput(N, world, t_e2e_sep), "ms_per_step": t_e2e_sep,
                              "path": "the same step with blz_cull_first / blz_cull_late"},
           "with_copies": {"value": job_throughput(N, world, t_e2e_copies), "ms_per_step": t_e2e_copies,
                           "path": "blz_transforms_update + depth H2D copy + recorded blz_cull_frame + count D2H "
                                   "copies, serial"},
           "direct_calls": {"value": job_throughput(N, world, t_e2e_direct), "ms_per_step": t_e2e_direct,
                            "path": "with copies, and blz_cull_frame called directly"}}

    extras = {}
    if not args.no_extras and rank == 0:
        try:
            from blitzen_gb300 import benchmarks
            extras = benchmarks.run_extras(c, sc, dev)
        except Exception as ex:  # extras never hide the headline line
            extras = {"error": repr(ex)}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(sc, v, depth.cpu().numpy().reshape(H, W), args.cpu_seconds)

    if rank == 0:
        line = {
            "metric": "objects culled/s (4M-object two-pass occlusion frame)", "value": value, "unit": "objects/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "config": workload_config(args), "roofline": roofline,
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks.summary(),
            "wall_s_timed": wall, "draws": {"pass1": V1, "pass2": V2}, "launch_shape": c.launch_shape(),
            "frame_forms": frames,
            "bit_exact": all(exact.values()), "bit_exact_checks": exact,
            "extras": extras,
        }
        print(json.dumps(line), flush=True)
    c.close()
    if world > 1:
        dist.destroy_process_group()


def cpu_baseline(sc, v, depth, seconds):
    """The oracle on the same full frame as the reference arm: the median of as many frames as fit in
    `seconds` (at least 5), every host thread."""
    threads = os.cpu_count() or 1
    frame = oracle_frame(sc, v, depth, threads)
    frame()
    times = time_oracle_frames(frame, 5, seconds)
    per = statistics.median(times)
    return {"value": sc.count / per, "unit": "objects/s", "cores": threads, "kind": "port", "ms": per * 1e3,
            "sample": f"median of {len(times)} full {sc.count}-object frames (bo_cull pass 1 + bo_pyramid_build + "
                      f"bo_cull pass 2; buffers preallocated, visibility restored outside the clock)"}


if __name__ == "__main__":
    main()
