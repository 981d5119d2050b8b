"""blz_cull_frustum_noalloc, the frustum + LOD cull whose staging is a fixed array inside the
library, against blz_cull_frustum on the same inputs, two calls in a row, through the C ABI.

Collected last so that it also runs after every other test has used the context paths; it
creates its own context and scene, so it passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from blitzen_gb300 import abi
from blitzen_gb300 import scenes as S
from blitzen_gb300.abi import RenderList
from blitzen_gb300.culler import Target, to_device
from oracle import oracle as O
from tests.helpers import assert_records_equal, view_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene_ctx(lib):
    from blitzen_gb300.culler import Culler
    c = Culler(0)
    sc = S.frustum_lod_scene(200_000, seed=11)
    c.setup_for_rendering(sc)
    yield c, sc
    c.close()


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _noalloc(c, view, target, objects=None, count=0):
    lst = RenderList(objects.data_ptr() if objects is not None else None, int(count))
    return c.lib.blz_cull_frustum_noalloc(c.ctx, C.byref(view), lst, C.byref(target.ctype()), _stream())


def _existing(c, view, target, objects=None, count=0):
    lst = RenderList(objects.data_ptr() if objects is not None else None, int(count))
    return c.lib.blz_cull_frustum(c.ctx, C.byref(view), lst, C.byref(target.ctype()), _stream())


def test_noalloc_equals_existing_two_calls_in_a_row(scene_ctx):
    c, sc = scene_ctx
    views = [view_for(zfar=3000.0), view_for(zfar=1e30, position=(40.0, -25.0, 60.0), yaw=1.1, pitch=-0.3)]
    for k, v in enumerate(views):
        for stride in (abi.STRIDE_VULKAN, abi.STRIDE_D3D12):
            a = Target.alloc(sc.count, stride)
            b = Target.alloc(sc.count, stride)
            assert _noalloc(c, v, a) == 0, abi.load().blz_last_error()
            assert _existing(c, v, b) == 0, abi.load().blz_last_error()
            assert c.check() == 0
            ga, gb = a.read(), b.read()
            assert ga[0] > 0
            assert_records_equal(ga, gb, f"call {k} stride {stride}")
    # and the first view once more against the oracle
    t = Target.alloc(sc.count)
    assert _noalloc(c, views[0], t) == 0
    n, recs, _ = O.cull(0, views[0], sc)
    assert_records_equal(t.read(), (n, recs), "oracle")


# every single-view launch shape blz_ctx_set_launch_shape accepts (threads, objects per thread)
SHAPES = [(256, 1), (256, 2), (256, 4), (128, 2), (128, 4), (512, 1)]


@pytest.mark.parametrize("shape", SHAPES)
def test_noalloc_equals_existing_under_every_launch_shape(scene_ctx, shape):
    """The fixed 512-object chunks of the no-alloc entry point under each launch shape, two calls in
    a row, against blz_cull_frustum under the same shape."""
    c, sc = scene_ctx
    c.set_launch_shape(*shape)
    try:
        for k, v in enumerate([view_for(zfar=2500.0, yaw=0.7), view_for(zfar=1e30, position=(-30.0, 10.0, 5.0))]):
            a, b = Target.alloc(sc.count), Target.alloc(sc.count)
            assert _noalloc(c, v, a) == 0, abi.load().blz_last_error()
            assert _existing(c, v, b) == 0, abi.load().blz_last_error()
            assert c.check() == 0
            assert_records_equal(a.read(), b.read(), f"shape {shape} call {k}")
    finally:
        c.set_launch_shape(256, 2)


def test_noalloc_at_the_object_bound_and_after_a_short_list(scene_ctx):
    c, sc = scene_ctx
    reps = -(-abi.NOALLOC_MAX_OBJECTS // sc.count)
    full = np.tile(sc.objects, reps)[: abi.NOALLOC_MAX_OBJECTS]
    objs = to_device(full, c.device)
    v = view_for(zfar=1e30)
    for count in (abi.NOALLOC_MAX_OBJECTS, 777, abi.NOALLOC_MAX_OBJECTS):
        a = Target.alloc(count)
        b = Target.alloc(count)
        assert _noalloc(c, v, a, objs, count) == 0, abi.load().blz_last_error()
        assert _existing(c, v, b, objs, count) == 0, abi.load().blz_last_error()
        assert c.check() == 0
        assert_records_equal(a.read(), b.read(), f"count {count}")


def test_noalloc_empty_list_and_overflow(scene_ctx):
    c, sc = scene_ctx
    v = view_for(zfar=1e30)
    t = Target.alloc(4)
    t.count.fill_(123)
    objs = to_device(sc.objects[:1], c.device)
    assert _noalloc(c, v, t, objs, 0) == 0
    assert c.check() == 0
    assert t.read()[0] == 0
    # a capacity below the visible count: same count, same stored prefix, flag raised
    n, recs, _ = O.cull(0, v, sc)
    a = Target.alloc(n // 3 + 1)
    a.capacity = n // 3
    assert _noalloc(c, v, a) == 0
    assert c.flags() & abi.FLAG_COMMAND_OVERFLOW
    gn, grecs = a.read()
    assert gn == n
    assert np.array_equal(grecs[:, :6], recs[: n // 3, :6])


def test_noalloc_rejects_lists_past_the_bound(scene_ctx):
    c, _ = scene_ctx
    too_long = torch.zeros((abi.NOALLOC_MAX_OBJECTS + 1) * 2, dtype=torch.int32, device=c.device)
    t = Target.alloc(16)
    before = c.launches
    rc = _noalloc(c, view_for(), t, too_long, abi.NOALLOC_MAX_OBJECTS + 1)
    assert rc == 2  # BLZ_ERR_CAPACITY
    assert b"at most" in abi.load().blz_last_error()
    assert c.launches == before
