"""The benchmark's own frame, word for word against the oracle.

The stress configuration at full size, exactly as bench.py builds it: stress_scene(4,000,000,
seed 0), the stress camera, the 2,000-box occluder depth rasterised on the device, the seeded 50 %
"visible last frame" mask. One frame is pass 1 (drawOccFirst.cs.hlsl:13-58), the D3D12 pyramid
(depthPyramid.cs.hlsl:13-26) and pass 2 (drawOccLate.cs.hlsl:13-67), dispatched in the order of
dx12Draw.cpp:590-641. Checked: both draw counts, every word of every record in both record strides,
every pyramid texel and the rewritten visibility buffer — as direct calls and as the recorded
graph the bench replays. The oracle runs with every host thread.
"""
import os

import numpy as np
import pytest
import torch

from blitzen_gb300 import abi
from blitzen_gb300 import scenes as S
from blitzen_gb300.culler import DevicePyramid, Target
from oracle import oracle as O
from tests.helpers import assert_records_equal

pytestmark = pytest.mark.gpu

N = 4_000_000
W, H = S.STRESS_DEPTH


@pytest.fixture(scope="module")
def bench_frame(lib):
    from blitzen_gb300.culler import Culler
    sc = S.stress_scene(N, seed=0)
    v = S.stress_view()
    c = Culler(0)
    c.setup_for_rendering(sc)
    depth = torch.zeros(W * H, dtype=torch.float32, device="cuda")
    c.raster_boxes(v, torch.from_numpy(sc.boxes.reshape(-1)).cuda(), depth, W, H)
    threads = os.cpu_count() or 1
    odepth = O.depth_raster(v, sc.boxes, W, H)
    ovis = sc.visibility.copy()
    want = {}
    for stride in (abi.STRIDE_VULKAN, abi.STRIDE_D3D12):
        vis = sc.visibility.copy()
        n1, r1, f1 = O.cull(1, v, sc, vis=vis, stride=stride, threads=threads)
        opyr = O.pyramid_build(odepth)
        n2, r2, f2 = O.cull(2, v, sc, vis=vis, pyramid=opyr, stride=stride, threads=threads)
        assert f1 == 0 and f2 == 0
        want[stride] = ((n1, r1), (n2, r2))
        ovis = vis
    yield c, sc, v, depth, odepth, opyr, ovis, want
    c.close()


def _frame_buffers(sc, stride):
    vis = torch.from_numpy(sc.visibility.view(np.int32).copy()).cuda()
    return vis, Target.alloc(N, stride), Target.alloc(N, stride), DevicePyramid(W, H, abi.HIZ_D3D12)


def _check(bf, stride, vis, t1, t2, pyr, what):
    c, sc, v, depth, odepth, opyr, ovis, want = bf
    (n1, r1), (n2, r2) = want[stride]
    assert_records_equal(t1.read(), (n1, r1), f"{what}: pass 1, stride {stride}")
    assert_records_equal(t2.read(), (n2, r2), f"{what}: pass 2, stride {stride}")
    assert np.array_equal(pyr.storage.cpu().numpy().view(np.uint32), opyr.data.view(np.uint32)), f"{what}: pyramid"
    assert np.array_equal(vis.cpu().numpy().view(np.uint32), ovis), f"{what}: visibility"


def test_bench_depth_raster_matches_oracle(bench_frame):
    c, sc, v, depth, odepth = bench_frame[:5]
    assert np.array_equal(depth.cpu().numpy().reshape(H, W).view(np.uint32), odepth.view(np.uint32))


def test_bench_frame_counts_are_the_recorded_ones(bench_frame):
    """The frame's draw counts; a change here means the scene generator or the camera changed."""
    want = bench_frame[7][abi.STRIDE_VULKAN]
    assert (want[0][0], want[1][0]) == (275_128, 140_678)


@pytest.mark.parametrize("stride", [abi.STRIDE_VULKAN, abi.STRIDE_D3D12])
def test_bench_frame_direct_calls(bench_frame, stride):
    c, sc, v, depth = bench_frame[:4]
    vis, t1, t2, pyr = _frame_buffers(sc, stride)
    c.draw_cull_first_pass(v, vis, t1)
    c.generate_depth_pyramid(pyr, depth)
    c.draw_cull_occlusion_pass(v, vis, pyr, t2)
    assert c.check() == 0
    _check(bench_frame, stride, vis, t1, t2, pyr, "direct")


@pytest.mark.parametrize("stride", [abi.STRIDE_VULKAN, abi.STRIDE_D3D12])
def test_bench_frame_recorded_replays(bench_frame, stride):
    """The frame recorded once and replayed (the bench's timed form), three replays in a row."""
    c, sc, v, depth = bench_frame[:4]
    vis, t1, t2, pyr = _frame_buffers(sc, stride)
    vis0 = vis.clone()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        c.draw_cull_first_pass(v, vis, t1)  # grows the scratch outside the capture
        c.generate_depth_pyramid(pyr, depth)
        c.draw_cull_occlusion_pass(v, vis, pyr, t2)
        c.capture_begin()
        c.draw_cull_first_pass(v, vis, t1)
        c.generate_depth_pyramid(pyr, depth)
        c.draw_cull_occlusion_pass(v, vis, pyr, t2)
        g = c.capture_end()
        try:
            for rep in range(3):
                vis.copy_(vis0)
                t1.count.fill_(0)
                t2.count.fill_(0)
                pyr.storage.fill_(-1.0)
                g.launch()
                side.synchronize()
                _check(bench_frame, stride, vis, t1, t2, pyr, f"replay {rep}")
        finally:
            g.close()
    assert c.check(side) == 0


@pytest.mark.parametrize("stride", [abi.STRIDE_VULKAN, abi.STRIDE_D3D12])
def test_bench_frame_kept_frame(bench_frame, stride):
    """blz_frame_first, the pyramid, blz_frame_late: the renderer's frame order with pass 2 testing
    only what pass 1 kept."""
    c, sc, v, depth = bench_frame[:4]
    vis, t1, t2, pyr = _frame_buffers(sc, stride)
    c.frame_first_pass(v, vis, t1)
    c.generate_depth_pyramid(pyr, depth)
    c.frame_occlusion_pass(pyr, t2)
    assert c.check() == 0
    _check(bench_frame, stride, vis, t1, t2, pyr, "kept frame")


@pytest.mark.parametrize("stride", [abi.STRIDE_VULKAN, abi.STRIDE_D3D12])
def test_bench_frame_one_call_recorded(bench_frame, stride):
    """blz_cull_frame directly, then recorded once and replayed three times (the bench's headline form)."""
    c, sc, v, depth = bench_frame[:4]
    vis, t1, t2, pyr = _frame_buffers(sc, stride)
    vis0 = vis.clone()
    c.cull_frame(v, vis, depth, pyr, t1, t2)
    assert c.check() == 0
    _check(bench_frame, stride, vis, t1, t2, pyr, "one call")
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        c.capture_begin()
        c.cull_frame(v, vis, depth, pyr, t1, t2)
        g = c.capture_end()
        try:
            for rep in range(3):
                vis.copy_(vis0)
                t1.count.fill_(0)
                t2.count.fill_(0)
                t1.commands.fill_(0)
                t2.commands.fill_(0)
                pyr.storage.fill_(-1.0)
                g.launch()
                side.synchronize()
                _check(bench_frame, stride, vis, t1, t2, pyr, f"one call, replay {rep}")
        finally:
            g.close()
    assert c.check(side) == 0
