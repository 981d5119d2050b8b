"""The CUDA path against the golden fixtures made from the reference's own shaders, bit-exact:
cull records (32-byte D3D12 layout and 24-byte Vulkan layout), draw counts, visibility, pyramids
and the instanced cull, on the random scene and on the boundary-case scene."""
import numpy as np
import pytest
import torch

from blitzen_gb300 import abi
from blitzen_gb300.culler import Culler, DevicePyramid, Target, to_device
from tests.golden import fixtures as G

pytestmark = pytest.mark.gpu


def _ctx(lib, d):
    c = Culler(0)
    c.setup_for_rendering(G.scene(d))
    return c


def _device_pyramid(data: np.ndarray, depth_w: int, depth_h: int) -> DevicePyramid:
    p = DevicePyramid(depth_w, depth_h, abi.HIZ_D3D12)
    assert p.storage.numel() == data.size
    p.storage.copy_(torch.from_numpy(data.copy()))
    return p


def _run(c, kind, v, vis, pyr, t):
    if kind == 0:
        c.draw_cull(v, t)
    elif kind == 1:
        c.draw_cull_first_pass(v, vis, t)
    elif kind == 2:
        c.draw_cull_occlusion_pass(v, vis, pyr, t)
    else:
        c.draw_cull_temporal(v, pyr, t)


def _check(t, vis, d, count_key, cmds_key, vis_key, what):
    n, recs = t.read()
    ref_n = int(d[count_key][0])
    ref = d[cmds_key]
    assert n == ref_n, f"{what}: count {n} != reference {ref_n}"
    words = t.stride // 4
    bad = np.nonzero((recs[:, :6] != ref[:, :6]).any(axis=1))[0]
    assert bad.size == 0, f"{what}: {bad.size} records differ, first {bad[0]}: {recs[bad[0]]} vs {ref[bad[0]]}"
    if words == 8:
        assert np.array_equal(recs, ref), f"{what}: pad words"
    if vis is not None and vis_key in d.files:
        assert np.array_equal(vis.cpu().numpy().view(np.uint32), d[vis_key]), f"{what}: visibility"


@pytest.mark.parametrize("stride", [abi.STRIDE_D3D12, abi.STRIDE_VULKAN])
def test_random_scene_matches_reference(lib, stride):
    d = G.load("cull")
    c = _ctx(lib, d)
    try:
        n = len(d["objects"])
        for cam in range(len(d["views"])):
            v = G.view(d["views"][cam])
            pyr = _device_pyramid(d[f"pyr{cam}"], 320, 180)
            for kind in range(4):
                vis = torch.from_numpy(d["visibility"].view(np.int32).copy()).cuda()
                t = Target.alloc(n, stride)
                _run(c, kind, v, vis, pyr, t)
                assert c.check() == 0
                _check(t, vis if kind in (1, 2) else None, d, f"count{cam}_{kind}", f"cmds{cam}_{kind}",
                       f"vis{cam}_{kind}", f"camera {cam} kind {kind} stride {stride}")
    finally:
        c.close()


@pytest.mark.parametrize("pyr_name", ["alt", "all"])
def test_boundary_cases_match_reference(lib, pyr_name):
    d = G.load("kat")
    c = _ctx(lib, d)
    try:
        n = len(d["objects"])
        v = G.view(d["view"])
        pyr = _device_pyramid(d[f"pyr_{pyr_name}"], 1920, 1080)
        for kind in range(4):
            vis = torch.from_numpy(d["visibility"].view(np.int32).copy()).cuda()
            t = Target.alloc(n, abi.STRIDE_D3D12)
            _run(c, kind, v, vis, pyr, t)
            assert c.check() == 0
            _check(t, vis if kind in (1, 2) else None, d, f"count_{pyr_name}_{kind}", f"cmds_{pyr_name}_{kind}",
                   f"vis_{pyr_name}_{kind}", f"boundary {pyr_name} kind {kind}")
    finally:
        c.close()


def test_pyramids_match_reference(culler):
    d = G.load("pyramid")
    for i in range(int(d["count"][0])):
        depth = d[f"depth{i}"]
        h, w = depth.shape
        p = DevicePyramid(w, h, abi.HIZ_D3D12)
        culler.generate_depth_pyramid(p, torch.from_numpy(depth.reshape(-1).copy()).cuda())
        culler.check()
        got = p.storage.cpu().numpy()
        assert [p.desc.mipCount, p.desc.width, p.desc.height] == list(d[f"mips{i}"])
        assert np.array_equal(got.view(np.uint32), d[f"pyr{i}"].view(np.uint32)), f"pyramid {w}x{h}"


def test_instanced_matches_reference(lib):
    d = G.load("instanced")
    c = _ctx(lib, d)
    try:
        v = G.view(d["view"])
        slots = int(d["slots"][0])
        nl = len(d["lods"])
        ctr = np.zeros(nl, abi.LOD_INSTANCE_COUNTER)
        ctr["instanceOffset"] = np.arange(nl) * slots
        ctr_d = to_device(ctr, "cuda")
        inst = torch.full((nl * slots,), -1, dtype=torch.int32, device="cuda")
        t = Target.alloc(nl, abi.STRIDE_D3D12)
        c.draw_instance_cull_pass(v, ctr_d, inst, slots, t)
        assert c.check() == 0
        n, recs = t.read()
        assert n == int(d["count"][0])
        assert np.array_equal(recs, d["cmds"])
        assert np.array_equal(ctr_d.cpu().numpy().view(np.uint32), d["counters"].view(np.uint32).reshape(-1))
        assert np.array_equal(inst.cpu().numpy().view(np.uint32), d["instances"])
    finally:
        c.close()


# ----------------------------------------------------------------------------- Vulkan form (GLSL)
# Fixtures from the reference's GLSL shaders compiled as C++: the Vulkan pyramid (PreviousPow2,
# MIN sampler), the three Vulkan culls with the Vulkan Hi-Z, the level-change boundary scene and
# the cluster path's records.


def _vk_device_pyramid(data: np.ndarray, depth_w: int, depth_h: int) -> DevicePyramid:
    p = DevicePyramid(depth_w, depth_h, abi.HIZ_VULKAN)
    assert p.storage.numel() == data.size
    p.storage.copy_(torch.from_numpy(data.copy()))
    return p


def test_vulkan_pyramids_match_reference(culler):
    d = G.load("vkpyramid")
    for i in range(int(d["count"][0])):
        depth = d[f"depth{i}"]
        h, w = depth.shape
        p = DevicePyramid(w, h, abi.HIZ_VULKAN)
        culler.generate_depth_pyramid(p, torch.from_numpy(depth.reshape(-1).copy()).cuda())
        culler.check()
        assert [p.desc.mipCount, p.desc.width, p.desc.height] == list(d[f"mips{i}"])
        assert np.array_equal(p.storage.cpu().numpy().view(np.uint32), d[f"pyr{i}"].view(np.uint32)), f"{w}x{h}"


@pytest.mark.parametrize("stride", [abi.STRIDE_VULKAN, abi.STRIDE_D3D12])
def test_vulkan_culls_match_reference(lib, stride):
    d = G.load("vkcull")
    c = _ctx(lib, d)
    try:
        n = len(d["objects"])
        for cam in range(len(d["views"])):
            v = G.view(d["views"][cam])
            pyr = _vk_device_pyramid(d[f"pyr{cam}"], 320, 180)
            for kind in range(3):
                vis = torch.from_numpy(d["visibility"].view(np.int32).copy()).cuda()
                t = Target.alloc(n, stride)
                _run(c, kind, v, vis, pyr, t)
                assert c.check() == 0
                n_, recs = t.read()
                ref = d[f"cmds{cam}_{kind}"]
                assert n_ == int(d[f"count{cam}_{kind}"][0]), f"camera {cam} kind {kind}"
                assert np.array_equal(recs[:, :6], ref), f"camera {cam} kind {kind} stride {stride}"
                if kind in (1, 2):
                    assert np.array_equal(vis.cpu().numpy().view(np.uint32), d[f"vis{cam}_{kind}"])
    finally:
        c.close()


@pytest.mark.parametrize("form", ["kept", "one_call"])
def test_vulkan_frame_forms_match_reference(lib, form):
    """The kept frame and the one-call frame with the Vulkan Hi-Z: pass 1's records are the
    InitialDrawCull fixture, pass 2's and the visibility the LateDrawCull one (pass 1 leaves the
    visibility as it found it), the pyramid the DepthPyramidGeneration one."""
    d = G.load("vkcull")
    c = _ctx(lib, d)
    try:
        n = len(d["objects"])
        for cam in range(len(d["views"])):
            v = G.view(d["views"][cam])
            depth = torch.from_numpy(d[f"depth{cam}"].reshape(-1).copy()).cuda()
            vis = torch.from_numpy(d["visibility"].view(np.int32).copy()).cuda()
            t1, t2 = Target.alloc(n), Target.alloc(n)
            pyr = DevicePyramid(320, 180, abi.HIZ_VULKAN)
            if form == "kept":
                c.frame_first_pass(v, vis, t1)
                c.generate_depth_pyramid(pyr, depth)
                c.frame_occlusion_pass(pyr, t2)
            else:
                c.cull_frame(v, vis, depth, pyr, t1, t2)
            assert c.check() == 0
            assert np.array_equal(pyr.storage.cpu().numpy().view(np.uint32), d[f"pyr{cam}"].view(np.uint32))
            for t, kind in ((t1, 1), (t2, 2)):
                n_, recs = t.read()
                assert n_ == int(d[f"count{cam}_{kind}"][0]) and np.array_equal(recs, d[f"cmds{cam}_{kind}"]), \
                    f"{form} camera {cam} pass {kind}"
            assert np.array_equal(vis.cpu().numpy().view(np.uint32), d[f"vis{cam}_2"])
    finally:
        c.close()


@pytest.mark.parametrize("pyr_name", ["alt", "top"])
def test_vulkan_boundary_cases_match_reference(lib, pyr_name):
    d = G.load("vkkat")
    c = _ctx(lib, d)
    try:
        n = len(d["objects"])
        v = G.view(d["view"])
        pyr = _vk_device_pyramid(d[f"pyr_{pyr_name}"], 1920, 1080)
        vis = torch.zeros(n, dtype=torch.int32, device="cuda")
        t = Target.alloc(n)
        c.draw_cull_occlusion_pass(v, vis, pyr, t)
        assert c.check() == 0
        n_, recs = t.read()
        assert n_ == int(d[f"count_{pyr_name}"][0]) and np.array_equal(recs, d[f"cmds_{pyr_name}"])
        assert np.array_equal(vis.cpu().numpy().view(np.uint32), d[f"vis_{pyr_name}"])
    finally:
        c.close()


@pytest.mark.parametrize("stride", [abi.STRIDE_VULKAN, abi.STRIDE_D3D12])
def test_cluster_records_match_reference(lib, stride):
    """blz_cull_clusters on a scene whose clusters pass every per-cluster test: the records and
    cluster ids of PreClusterDrawCull + InitialClusterCull."""
    d = G.load("vkclusters")
    sc = G.scene(d)
    sc.clusters = d["clusters"]
    c = Culler(0)
    try:
        c.setup_for_rendering(sc)
        v = G.view(d["view"])
        cap = len(d["dispatch"]) + 16
        t = Target.alloc(cap, stride)
        ids = torch.zeros(cap, dtype=torch.int32, device="cuda")
        c.cluster_cull(v, t, cluster_ids=ids)
        assert c.check() == 0
        n, recs = t.read()
        assert n == int(d["count"][0])
        assert np.array_equal(recs[:, :6], d["cmds"])
        assert np.array_equal(ids.cpu().numpy().view(np.uint32)[:n], d["dispatch"][:, 2])
    finally:
        c.close()
