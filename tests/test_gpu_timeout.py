"""The device-side waits run out and the context recovers, on the GPU, without any fault or hang.

The library's kernels wait in two places, each a bounded poll:
  - the per-LOD look-back of the single-kernel instanced cull (more than 1,024 LODs) polls a tile
    state that a tile which started earlier publishes. Here the context's ticket counter is
    advanced first (blz_ctx_debug_advance_ticket), so the next launch's tiles wait for places no
    tile holds;
  - the one-call frame given a depth buffer polls the pyramid-ready flag the launch's own blocks
    set. Here the frame's pyramid-tile ticket is advanced first (blz_ctx_debug_skip_frame_tiles),
    so the first tiles are never built and the flag is never set.
With a short wait limit (blz_ctx_set_wait_limit) each wait gives up, the launch raises
BLZ_FLAG_TIMEOUT, blz_ctx_check returns BLZ_ERR_TIMEOUT, and the next launch with the default limit
matches the oracle again. The reference's counterpart is the bounded fence wait of its frame loop
(vulkanData.h:196-197).
"""
import numpy as np
import pytest
import torch

from blitzen_gb300 import abi
from blitzen_gb300 import scenes as S
from blitzen_gb300.culler import Culler, DevicePyramid, Target
from oracle import oracle as O
from tests.helpers import H, W, assert_records_equal, view_for

pytestmark = pytest.mark.gpu

SHORT = 16  # polls before a wait gives up


def _expect_timeout(c):
    assert c.flags() & abi.FLAG_TIMEOUT  # taken and cleared here; blz_ctx_check reset the protocol
    c.set_wait_limit(0)


@pytest.fixture(scope="module")
def many_lods(lib):
    c = Culler(0)
    sc = S.frustum_lod_scene(60_000, seed=5, n_meshes=300, extent=800.0)
    assert len(sc.lods) > 1024
    c.setup_for_rendering(sc)
    yield c, sc
    c.close()


def _instanced(c, sc, v, ctr, slots):
    cap = len(sc.lods) * slots
    dctr = torch.from_numpy(ctr.view(np.int32).reshape(-1).copy()).cuda()
    dinst = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
    t = Target.alloc(len(sc.lods))
    c.draw_instance_cull_pass(v, dctr, dinst, slots, t)
    return dctr, dinst, t


@pytest.mark.parametrize("advance", [1, 4])
def test_instanced_lookback_runs_out_then_recovers(many_lods, advance):
    c, sc = many_lods
    v = view_for(zfar=1e4)
    slots = 5_000
    ctr = O.new_counters(sc, slots)
    c.set_wait_limit(SHORT)
    c.debug_advance_ticket(advance)
    _instanced(c, sc, v, ctr, slots)
    _expect_timeout(c)
    dctr, dinst, t = _instanced(c, sc, v, ctr, slots)
    assert c.check() == 0
    n, cmds, octr, oinst, _ = O.cull_instanced(v, sc, ctr, len(sc.lods) * slots, slots)
    assert_records_equal(t.read(), (n, cmds), "instanced after the timeout")
    assert np.array_equal(dctr.cpu().numpy().view(np.uint32), octr.view(np.uint32).reshape(-1))
    assert np.array_equal(dinst.cpu().numpy().view(np.uint32), oinst)


def test_check_reports_the_timeout(many_lods):
    c, sc = many_lods
    v = view_for(zfar=1e4)
    c.set_wait_limit(SHORT)
    c.debug_advance_ticket(2)
    _instanced(c, sc, v, O.new_counters(sc, 5_000), 5_000)
    with pytest.raises(abi.BlzError) as ei:
        c.check()
    assert ei.value.code == 4  # BLZ_ERR_TIMEOUT
    c.set_wait_limit(0)
    _instanced(c, sc, v, O.new_counters(sc, 5_000), 5_000)
    assert c.check() == 0


def test_wait_limit_and_ticket_arguments(many_lods):
    c, _ = many_lods
    with pytest.raises(abi.BlzError):
        c.debug_advance_ticket(0)
    with pytest.raises(abi.BlzError):
        c.debug_advance_ticket(5000)
    c.set_wait_limit(0)


@pytest.fixture(scope="module")
def frame_scene(lib):
    c = Culler(0)
    sc = S.stress_scene(300_000, seed=3)
    c.setup_for_rendering(sc)
    v = view_for(zfar=1e4)
    depth = O.depth_raster(v, sc.boxes, W, H)
    yield c, sc, v, depth
    c.close()


@pytest.mark.parametrize("skip", [1, 37])
def test_frame_pyramid_wait_runs_out_then_recovers(frame_scene, skip):
    c, sc, v, depth = frame_scene
    ddepth = torch.from_numpy(depth.reshape(-1)).cuda()
    vis0 = torch.from_numpy(sc.visibility.view(np.int32).copy()).cuda()
    vis = vis0.clone()
    t1, t2 = Target.alloc(sc.count), Target.alloc(sc.count)
    pyr = DevicePyramid(W, H)
    c.set_wait_limit(SHORT)
    c.debug_skip_frame_tiles(skip)
    c.cull_frame(v, vis, ddepth, pyr, t1, t2)
    _expect_timeout(c)
    # the frame after it is whole: records, visibility and pyramid as the oracle's
    vis.copy_(vis0)
    c.cull_frame(v, vis, ddepth, pyr, t1, t2)
    assert c.check() == 0
    ovis = sc.visibility.copy()
    n1, r1, _ = O.cull(1, v, sc, vis=ovis)
    opyr = O.pyramid_build(depth)
    n2, r2, _ = O.cull(2, v, sc, vis=ovis, pyramid=opyr)
    assert_records_equal(t1.read(), (n1, r1), "pass 1 after the timeout")
    assert_records_equal(t2.read(), (n2, r2), "pass 2 after the timeout")
    assert np.array_equal(vis.cpu().numpy().view(np.uint32), ovis)
    assert np.array_equal(pyr.storage.cpu().numpy().view(np.uint32), opyr.data.view(np.uint32))


def test_frame_tile_skip_arguments(frame_scene):
    c = frame_scene[0]
    with pytest.raises(abi.BlzError):
        c.debug_skip_frame_tiles(0)
    with pytest.raises(abi.BlzError):
        c.debug_skip_frame_tiles(2000)
