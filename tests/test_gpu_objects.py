"""Parity of the per-object culls (frustum, occlusion pass 1 / pass 2, temporal) with the oracle.

Bit-exact: draw counts, every record word, and the rewritten visibility buffer.
"""
import numpy as np
import pytest
import torch

from blitzen_gb300 import abi
from blitzen_gb300 import scenes as S
from blitzen_gb300.culler import DevicePyramid, Target, to_device
from oracle import oracle as O
from tests.helpers import H, W, assert_records_equal, view_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c1_ctx(lib):
    from blitzen_gb300.culler import Culler
    c = Culler(0)
    sc = S.frustum_lod_scene(100_000, seed=0)
    c.setup_for_rendering(sc)
    yield c, sc
    c.close()


@pytest.fixture
def culler(c1_ctx):
    return c1_ctx[0]


@pytest.fixture
def c1(c1_ctx):
    return c1_ctx[1]


@pytest.mark.parametrize("zfar", [650.0, 1e30])
@pytest.mark.parametrize("stride", [abi.STRIDE_VULKAN, abi.STRIDE_D3D12])
def test_frustum_lod_config1(culler, c1, zfar, stride):
    v = view_for(zfar=zfar)
    t = Target.alloc(c1.count, stride)
    culler.draw_cull(v, t)
    assert culler.check() == 0
    gpu = t.read()
    n, recs, flags = O.cull(0, v, c1, stride=stride)
    assert flags == 0
    assert n > 0
    assert_records_equal(gpu, (n, recs), f"frustum zfar={zfar} stride={stride}")


def test_frustum_random_cameras(culler, c1):
    rng = np.random.default_rng(5)
    for k in range(6):
        pos = tuple(float(x) for x in rng.uniform(-800, 800, 3).astype(np.float32))
        v = view_for(zfar=float(rng.uniform(100, 3000)), position=pos, yaw=float(rng.uniform(-3, 3)),
                     pitch=float(rng.uniform(-1, 1)))
        t = Target.alloc(c1.count)
        culler.draw_cull(v, t)
        n, recs, _ = O.cull(0, v, c1)
        assert_records_equal(t.read(), (n, recs), f"camera {k}")


def test_capacity_overflow_is_flagged_and_bounded(culler, c1):
    v = view_for(zfar=1e30)
    n, recs, _ = O.cull(0, v, c1)
    cap = n // 2
    t = Target.alloc(cap + 8)
    t.capacity = cap
    sentinel = t.commands.clone()
    culler.draw_cull(v, t)
    flags = culler.flags()
    assert flags & abi.FLAG_COMMAND_OVERFLOW
    gn, grecs = t.read()
    assert gn == n
    assert np.array_equal(grecs[:, :6], recs[:cap, :6])
    # nothing written past the capacity
    assert torch.equal(t.commands[cap * 6:], sentinel[cap * 6:])


def test_empty_list_writes_zero_count(culler, c1):
    v = view_for()
    t = Target.alloc(16)
    t.count.fill_(12345)
    culler.draw_cull(v, t, objects=torch.zeros(2, dtype=torch.int32, device="cuda"), count=0)
    assert culler.check() == 0
    assert t.read()[0] == 0


def test_custom_render_list_and_bad_index(culler, c1):
    objs = c1.objects[::3].copy()
    objs["surfaceId"][7] = 10_000          # out of range surface: skipped and flagged
    objs["transformId"][11] = 10_000_000   # out of range transform
    dev = to_device(objs, "cuda")
    v = view_for(zfar=1e30)
    t = Target.alloc(len(objs))
    culler.draw_cull(v, t, objects=dev, count=len(objs))
    flags = culler.flags()
    assert flags & abi.FLAG_BAD_INDEX
    n, recs, oflags = O.cull(0, v, c1, objects=objs)
    assert oflags & abi.FLAG_BAD_INDEX
    assert_records_equal(t.read(), (n, recs), "custom list")


@pytest.fixture(scope="module")
def stress_ctx(lib):
    from blitzen_gb300.culler import Culler
    c = Culler(0)
    sc = S.stress_scene(1_000_000, seed=1)
    c.setup_for_rendering(sc)
    v = view_for(zfar=1e4)
    depth = O.depth_raster(v, sc.boxes, W, H)
    yield c, (sc, v, depth)
    c.close()


@pytest.fixture
def stress(stress_ctx):
    return stress_ctx[1]


@pytest.fixture
def sculler(stress_ctx):
    return stress_ctx[0]


@pytest.mark.parametrize("mode", [abi.HIZ_D3D12, abi.HIZ_VULKAN])
def test_pyramid_matches_oracle(sculler, stress, mode):
    sc, v, depth = stress
    p = DevicePyramid(W, H, mode)
    sculler.generate_depth_pyramid(p, torch.from_numpy(depth).cuda())
    assert sculler.check() == 0
    ref = O.pyramid_build(depth, mode)
    got = p.storage.cpu().numpy()
    assert p.desc.mipCount == ref.desc.mipCount
    assert np.array_equal(got.view(np.uint32), ref.data.view(np.uint32))


@pytest.mark.parametrize("wh", [(1, 1), (1, 7), (2, 3), (7, 1), (65, 33), (129, 257), (1023, 577), (4097, 130)])
@pytest.mark.parametrize("mode", [abi.HIZ_D3D12, abi.HIZ_VULKAN])
def test_pyramid_odd_sizes(sculler, wh, mode):
    w, h = wh
    rng = np.random.default_rng(w * 131 + h)
    depth = rng.random((h, w), dtype=np.float32)
    depth[rng.random((h, w)) < 0.1] = 0.0
    p = DevicePyramid(w, h, mode)
    sculler.generate_depth_pyramid(p, torch.from_numpy(depth).cuda())
    assert sculler.check() == 0
    ref = O.pyramid_build(depth, mode)
    assert np.array_equal(p.storage.cpu().numpy().view(np.uint32), ref.data.view(np.uint32)), (w, h, mode)


def run_frame(c, form, v, vis, depth, pyr, t1, t2, objects=None, count=None):
    """One occlusion frame in one of the library's three forms: the separate calls (blz_cull_first,
    blz_pyramid_build, blz_cull_late), the kept frame (blz_frame_first, blz_pyramid_build,
    blz_frame_late), the one call (blz_cull_frame) or the one call over a pyramid built before it
    (blz_cull_frame with no depth)."""
    if form == "calls":
        c.draw_cull_first_pass(v, vis, t1, objects=objects, count=count)
        c.generate_depth_pyramid(pyr, depth)
        c.draw_cull_occlusion_pass(v, vis, pyr, t2, objects=objects, count=count)
    elif form == "kept":
        c.frame_first_pass(v, vis, t1, objects=objects, count=count)
        c.generate_depth_pyramid(pyr, depth)
        c.frame_occlusion_pass(pyr, t2)
    elif form == "prebuilt":
        c.generate_depth_pyramid(pyr, depth)
        c.cull_frame(v, vis, None, pyr, t1, t2, objects=objects, count=count)
    else:
        c.cull_frame(v, vis, depth, pyr, t1, t2, objects=objects, count=count)


FORMS = ["calls", "kept", "one_call", "prebuilt"]


@pytest.mark.parametrize("form", FORMS)
@pytest.mark.parametrize("hiz", [abi.HIZ_D3D12, abi.HIZ_VULKAN])
def test_two_pass_occlusion(sculler, stress, hiz, form):
    sc, v, depth = stress
    if hiz == abi.HIZ_VULKAN:
        pl, _ = abi.pyramid_layout(W, H, hiz)
        v = view_for(zfar=1e4, pw=float(pl.width), ph=float(pl.height))
    vis = torch.from_numpy(sc.visibility.view(np.int32).copy()).cuda()
    t1, t2 = Target.alloc(sc.count), Target.alloc(sc.count)
    p = DevicePyramid(W, H, hiz)
    run_frame(sculler, form, v, vis, torch.from_numpy(depth).cuda(), p, t1, t2)
    assert sculler.check() == 0

    ovis = sc.visibility.copy()
    n1, r1, _ = O.cull(O_FIRST, v, sc, vis=ovis)
    opyr = O.pyramid_build(depth, hiz)
    n2, r2, _ = O.cull(O_LATE, v, sc, vis=ovis, pyramid=opyr)
    assert_records_equal(t1.read(), (n1, r1), "first pass")
    assert_records_equal(t2.read(), (n2, r2), "late pass")
    assert np.array_equal(vis.cpu().numpy().view(np.uint32), ovis)
    assert n2 > 0 and n1 > 0


def test_temporal(sculler, stress):
    sc, v, depth = stress
    p = DevicePyramid(W, H)
    sculler.generate_depth_pyramid(p, torch.from_numpy(depth).cuda())
    t = Target.alloc(sc.count, abi.STRIDE_D3D12)
    sculler.draw_cull_temporal(v, p, t)
    assert sculler.check() == 0
    n, recs, _ = O.cull(O_TEMPORAL, v, sc, pyramid=O.pyramid_build(depth), stride=abi.STRIDE_D3D12)
    nf, _, _ = O.cull(0, v, sc)
    assert 0 < n < nf  # the occluders hide part of the frustum-visible set
    assert_records_equal(t.read(), (n, recs), "temporal")


def test_deterministic_rerun(sculler, stress):
    sc, v, depth = stress
    p = DevicePyramid(W, H)
    sculler.generate_depth_pyramid(p, torch.from_numpy(depth).cuda())
    outs = []
    for _ in range(3):
        t = Target.alloc(sc.count)
        sculler.draw_cull_temporal(v, p, t)
        outs.append(t.commands.clone())
    assert torch.equal(outs[0], outs[1]) and torch.equal(outs[1], outs[2])


O_FIRST, O_LATE, O_TEMPORAL = 1, 2, 3


def test_recorded_frame_replays_match_direct_calls(culler, c1):
    """A frame recorded with blz_capture_begin/end and replayed with blz_graph_launch gives the
    same records and visibility as the direct calls, replay after replay."""
    v = view_for(zfar=3000.0, yaw=0.4)
    depth = torch.from_numpy(O.depth_raster(v, S.make_occluders(np.random.default_rng(3), 300), W, H)).cuda()
    vis0 = (np.random.default_rng(4).random(c1.count) < 0.5).astype(np.uint32)
    vis = torch.from_numpy(vis0.view(np.int32).copy()).cuda()
    t1, t2 = Target.alloc(c1.count), Target.alloc(c1.count)
    pyr = DevicePyramid(W, H)
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        culler.draw_cull_first_pass(v, vis, t1)
        culler.generate_depth_pyramid(pyr, depth)
        culler.draw_cull_occlusion_pass(v, vis, pyr, t2)
        side.synchronize()
        want = (t1.read(), t2.read(), vis.cpu().numpy().copy())
        culler.capture_begin()
        culler.draw_cull_first_pass(v, vis, t1)
        culler.generate_depth_pyramid(pyr, depth)
        culler.draw_cull_occlusion_pass(v, vis, pyr, t2)
        g = culler.capture_end()
        try:
            assert g.kernels >= 3  # pass 1, pyramid, pass 2
            for rep in range(3):
                vis.copy_(torch.from_numpy(vis0.view(np.int32).copy()).cuda())
                t1.count.fill_(0)
                t2.count.fill_(0)
                g.launch()
                side.synchronize()
                assert_records_equal(t1.read(), want[0], f"replay {rep} pass 1")
                assert_records_equal(t2.read(), want[1], f"replay {rep} pass 2")
                assert np.array_equal(vis.cpu().numpy(), want[2])
        finally:
            g.close()
    assert culler.check(side) == 0


def test_capture_refuses_to_grow_scratch(culler, c1):
    """Scratch cannot be allocated inside a capture: a list longer than any run before is refused."""
    big = to_device(np.tile(c1.objects, 40), "cuda")  # more chunks than the context has seen
    t = Target.alloc(16)
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        culler.capture_begin()
        with pytest.raises(abi.BlzError) as ei:
            culler.draw_cull(view_for(), t, objects=big, count=c1.count * 40)
        g = culler.capture_end()
        g.close()
    assert ei.value.code == 2  # BLZ_ERR_CAPACITY


@pytest.mark.parametrize("form", ["kept", "one_call"])
def test_kept_frame_unusual_words_bad_ids_and_overflow(culler, c1, form):
    """The kept frame against the oracle where the forms could part: visibility words other than 0/1
    (any non-zero word is 'visible last frame', every word ends 0 or 1), out-of-range transform and
    surface ids in a custom render list, and both outputs smaller than their record counts."""
    v = view_for(zfar=1e4, yaw=0.3)
    depth = O.depth_raster(v, S.make_occluders(np.random.default_rng(21), 400), W, H)
    objs = c1.objects[::2].copy()
    objs["surfaceId"][5] = 10_000
    objs["transformId"][9] = 10_000_000
    words = np.array([0, 1, 2, 0x80000000, 0xFFFFFFFF], np.uint32)
    vis0 = words[np.random.default_rng(22).integers(0, len(words), len(objs))]
    ovis = vis0.copy()
    n1, r1, f1 = O.cull(1, v, c1, objects=objs, vis=ovis)
    n2, r2, f2 = O.cull(2, v, c1, objects=objs, vis=ovis, pyramid=O.pyramid_build(depth))
    assert (f1 | f2) & abi.FLAG_BAD_INDEX
    dev = to_device(objs, "cuda")
    for cap1, cap2 in ((len(objs), len(objs)), (n1 // 2, n2 // 3)):
        vis = torch.from_numpy(vis0.view(np.int32).copy()).cuda()
        t1, t2 = Target.alloc(cap1), Target.alloc(cap2)
        pyr = DevicePyramid(W, H)
        run_frame(culler, form, v, vis, torch.from_numpy(depth).cuda(), pyr, t1, t2, objects=dev, count=len(objs))
        flags = culler.flags()
        assert flags & abi.FLAG_BAD_INDEX
        assert bool(flags & abi.FLAG_COMMAND_OVERFLOW) == (cap1 < n1 or cap2 < n2)
        assert_records_equal(t1.read(), (n1, r1[:cap1]), f"{form} pass 1, capacity {cap1}")
        assert_records_equal(t2.read(), (n2, r2[:cap2]), f"{form} pass 2, capacity {cap2}")
        assert np.array_equal(vis.cpu().numpy().view(np.uint32), ovis)


def test_kept_frame_empty_list_and_missing_first(culler, c1):
    v = view_for()
    vis = torch.zeros(4, dtype=torch.int32, device="cuda")
    t1, t2 = Target.alloc(4), Target.alloc(4)
    t1.count.fill_(7)
    t2.count.fill_(7)
    pyr = DevicePyramid(W, H)
    depth = torch.zeros(W * H, dtype=torch.float32, device="cuda")
    culler.cull_frame(v, vis, depth, pyr, t1, t2, objects=torch.zeros(2, dtype=torch.int32, device="cuda"), count=0)
    assert culler.check() == 0
    assert t1.read()[0] == 0 and t2.read()[0] == 0
    from blitzen_gb300.culler import Culler
    fresh = Culler(0)
    try:
        fresh.setup_for_rendering(c1)
        with pytest.raises(abi.BlzError) as ei:
            fresh.frame_occlusion_pass(pyr, t2)
        assert ei.value.code == 1
    finally:
        fresh.close()


def test_late_pass_with_unusual_visibility_words(culler, c1):
    """Pass 2 treats any non-zero word as 'visible last frame' and rewrites every word to 0 or 1,
    as drawOccLate.cs.hlsl does, whatever the word held (0, 1, 2, 2^31, 2^32-1)."""
    v = view_for(zfar=1e4)
    depth = O.depth_raster(v, S.make_occluders(np.random.default_rng(8), 400), W, H)
    pyr = DevicePyramid(W, H)
    culler.generate_depth_pyramid(pyr, torch.from_numpy(depth).cuda())
    words = np.array([0, 1, 2, 0x80000000, 0xFFFFFFFF], np.uint32)
    vis0 = words[np.random.default_rng(9).integers(0, len(words), c1.count)]
    vis = torch.from_numpy(vis0.view(np.int32).copy()).cuda()
    t = Target.alloc(c1.count)
    culler.draw_cull_occlusion_pass(v, vis, pyr, t)
    assert culler.check() == 0
    ovis = vis0.copy()
    n, recs, _ = O.cull(2, v, c1, vis=ovis, pyramid=O.pyramid_build(depth))
    assert_records_equal(t.read(), (n, recs), "late, unusual words")
    assert np.array_equal(vis.cpu().numpy().view(np.uint32), ovis)
