"""The device-side wait runs out and the context recovers, on the GPU, without any fault or hang.

The one wait of the library's kernels is the per-LOD look-back of the single-kernel instanced cull
(more than 1,024 LODs): a bounded poll of a tile state that a tile which started earlier publishes.
Here the context's ticket counter is advanced first (blz_ctx_debug_advance_ticket), so the next
launch's tiles wait for places no tile holds; with a short wait limit (blz_ctx_set_wait_limit) each
gives up, the launch raises BLZ_FLAG_TIMEOUT, blz_ctx_check returns BLZ_ERR_TIMEOUT, and the next
launch with the default limit matches the oracle again. The reference's counterpart is the bounded
fence wait of its frame loop (vulkanData.h:196-197).
"""
import numpy as np
import pytest
import torch

from blitzen_gb300 import abi
from blitzen_gb300 import scenes as S
from blitzen_gb300.culler import Culler, Target
from oracle import oracle as O
from tests.helpers import assert_records_equal, view_for

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
