"""The oracle and the library's host code against the golden fixtures made from the reference's
own camera code and D3D12 compute shaders (tests/golden/make_golden.py). No GPU.

Bit-exact: every view byte, every pyramid texel, every record word, every visibility word.
"""
import numpy as np
import pytest

from blitzen_gb300 import abi
from oracle import oracle as O
from tests.golden import fixtures as G

KINDS = {0: "frustum (drawCull)", 1: "pass 1 (drawOccFirst)", 2: "pass 2 (drawOccLate)", 3: "temporal (drawOccTemporal)"}


def _host_pyramid(data: np.ndarray, depth_w: int, depth_h: int) -> O.HostPyramid:
    p = O.HostPyramid(depth_w, depth_h, abi.HIZ_D3D12)
    assert p.data.size == data.size
    p.data[:] = data
    return p


def _cmp(got: tuple[int, np.ndarray], cnt: int, cmds: np.ndarray, what: str):
    n, recs = got
    assert n == cnt, f"{what}: count {n} != reference {cnt}"
    assert recs.shape == cmds.shape, f"{what}: shape {recs.shape} != {cmds.shape}"
    bad = np.nonzero((recs != cmds).any(axis=1))[0]
    assert bad.size == 0, f"{what}: {bad.size} records differ, first {bad[0]}: {recs[bad[0]]} vs {cmds[bad[0]]}"


def test_camera_oracle_and_library_match_reference():
    d = G.load("camera")
    for i, p in enumerate(d["params"]):
        f = [float(x) for x in p]
        args = (f[0], f[1], f[2], f[3], f[4], (f[5], f[6], f[7]), f[8], f[9], f[10], f[11])
        ref = d["views"][i].tobytes()
        assert bytes(O.view_setup(*args)) == ref, f"oracle view {i} differs from the reference camera"
        assert bytes(abi.view_setup(*args)) == ref, f"library view {i} differs from the reference camera"


def test_pyramid_oracle_matches_reference():
    d = G.load("pyramid")
    for i in range(int(d["count"][0])):
        depth = d[f"depth{i}"]
        p = O.pyramid_build(depth, abi.HIZ_D3D12)
        assert [p.desc.mipCount, p.desc.width, p.desc.height] == list(d[f"mips{i}"])
        assert np.array_equal(p.data.view(np.uint32), d[f"pyr{i}"].view(np.uint32)), f"pyramid {depth.shape}"


@pytest.mark.parametrize("cam", range(4))
@pytest.mark.parametrize("kind", range(4))
def test_cull_oracle_matches_reference(cam, kind):
    d = G.load("cull")
    sc = G.scene(d)
    v = G.view(d["views"][cam])
    pyr = _host_pyramid(d[f"pyr{cam}"], 320, 180) if kind in (2, 3) else None
    vis = sc.visibility.copy() if kind in (1, 2) else None
    n, recs, flags = O.cull(kind, v, sc, vis=vis, pyramid=pyr, stride=32)
    assert flags == 0
    _cmp((n, recs), int(d[f"count{cam}_{kind}"][0]), d[f"cmds{cam}_{kind}"], f"camera {cam} {KINDS[kind]}")
    if kind in (1, 2):
        assert np.array_equal(vis, d[f"vis{cam}_{kind}"]), "visibility after the pass"


@pytest.mark.parametrize("pyr_name", ["alt", "all"])
@pytest.mark.parametrize("kind", range(4))
def test_boundary_cases_oracle_matches_reference(pyr_name, kind):
    d = G.load("kat")
    sc = G.scene(d)
    v = G.view(d["view"])
    pyr = _host_pyramid(d[f"pyr_{pyr_name}"], 1920, 1080) if kind in (2, 3) else None
    vis = sc.visibility.copy() if kind in (1, 2) else None
    n, recs, flags = O.cull(kind, v, sc, vis=vis, pyramid=pyr, stride=32)
    assert flags == 0
    _cmp((n, recs), int(d[f"count_{pyr_name}_{kind}"][0]), d[f"cmds_{pyr_name}_{kind}"], f"{pyr_name} {KINDS[kind]}")
    if kind in (1, 2):
        assert np.array_equal(vis, d[f"vis_{pyr_name}_{kind}"])


def test_boundary_cases_straddle():
    """The boundary scene really sits on the boundaries: both answers occur in every group."""
    d = G.load("kat")
    n = len(d["objects"])
    emitted = np.zeros(n, bool)
    emitted[d["cmds_all_0"][:, 0]] = True
    assert 0 < emitted.sum() < n
    # LOD ties: the chosen LOD differs between error = threshold - 1 ulp and error = threshold
    lod_of = dict(zip(d["cmds_all_0"][:, 0].tolist(), d["cmds_all_0"][:, 3].tolist()))
    assert len(set(lod_of.values())) > 4


def test_instanced_oracle_matches_reference():
    d = G.load("instanced")
    sc = G.scene(d)
    v = G.view(d["view"])
    slots = int(d["slots"][0])
    ctr = O.new_counters(sc, slots)
    n, recs, ctr_o, inst_o, flags = O.cull_instanced(v, sc, ctr, len(sc.lods) * slots, slots, stride=32)
    assert flags == 0
    _cmp((n, recs), int(d["count"][0]), d["cmds"], "instanced")
    assert np.array_equal(ctr_o.view(np.uint32), d["counters"].view(np.uint32))
    assert np.array_equal(inst_o, d["instances"])


def test_oracle_threads_do_not_change_results():
    d = G.load("cull")
    sc = G.scene(d)
    v = G.view(d["views"][0])
    pyr = _host_pyramid(d["pyr0"], 320, 180)
    one = O.cull(3, v, sc, pyramid=pyr, stride=24, threads=1)
    many = O.cull(3, v, sc, pyramid=pyr, stride=24, threads=7)
    assert one[0] == many[0] and np.array_equal(one[1], many[1])


# ----------------------------------------------------------------------------- Vulkan form (GLSL)
# Fixtures from the reference's GLSL shaders compiled as C++ (oracle/ref_glsl/): everything but the
# depth sampler's MIN footprint is the reference's own text there.

VK_KINDS = {0: "frustum (TransparentDrawCull)", 1: "pass 1 (InitialDrawCull)", 2: "pass 2 (LateDrawCull)"}


def _vk_host_pyramid(data: np.ndarray, depth_w: int, depth_h: int) -> O.HostPyramid:
    p = O.HostPyramid(depth_w, depth_h, abi.HIZ_VULKAN)
    assert p.data.size == data.size
    p.data[:] = data
    return p


def test_vulkan_pyramid_oracle_matches_reference():
    """DepthPyramidGeneration.comp.glsl dispatched per level (vulkanDraw.cpp:554-622): PreviousPow2
    extent, the MIN sampler at (pos + 0.5) / levelExtent."""
    d = G.load("vkpyramid")
    for i in range(int(d["count"][0])):
        depth = d[f"depth{i}"]
        p = O.pyramid_build(depth, abi.HIZ_VULKAN)
        assert [p.desc.mipCount, p.desc.width, p.desc.height] == list(d[f"mips{i}"])
        assert np.array_equal(p.data.view(np.uint32), d[f"pyr{i}"].view(np.uint32)), f"pyramid {depth.shape}"


@pytest.mark.parametrize("cam", range(4))
@pytest.mark.parametrize("kind", range(3))
def test_vulkan_cull_oracle_matches_reference(cam, kind):
    d = G.load("vkcull")
    sc = G.scene(d)
    v = G.view(d["views"][cam])
    pyr = _vk_host_pyramid(d[f"pyr{cam}"], 320, 180) if kind == 2 else None
    vis = sc.visibility.copy() if kind in (1, 2) else None
    n, recs, flags = O.cull(kind, v, sc, vis=vis, pyramid=pyr, stride=24)
    assert flags == 0
    _cmp((n, recs), int(d[f"count{cam}_{kind}"][0]), d[f"cmds{cam}_{kind}"], f"camera {cam} {VK_KINDS[kind]}")
    if kind in (1, 2):
        assert np.array_equal(vis, d[f"vis{cam}_{kind}"]), "visibility after the pass"


@pytest.mark.parametrize("pyr_name", ["alt", "top"])
def test_vulkan_boundary_cases_oracle_matches_reference(pyr_name):
    """Spheres one ulp either side of every level change of the Vulkan Hi-Z (LateDrawCull with the
    reference's level choice and LOD clamping), against constant-per-mip pyramids."""
    d = G.load("vkkat")
    sc = G.scene(d)
    v = G.view(d["view"])
    pyr = _vk_host_pyramid(d[f"pyr_{pyr_name}"], 1920, 1080)
    vis = np.zeros(len(sc.objects), np.uint32)
    n, recs, flags = O.cull(2, v, sc, vis=vis, pyramid=pyr, stride=24)
    assert flags == 0
    _cmp((n, recs), int(d[f"count_{pyr_name}"][0]), d[f"cmds_{pyr_name}"], f"vulkan boundary {pyr_name}")
    assert np.array_equal(vis, d[f"vis_{pyr_name}"])
    assert 0 < n < len(sc.objects)  # both answers occur


def test_vulkan_cluster_records_oracle_matches_reference():
    """PreClusterDrawCull + InitialClusterCull: the chosen LOD's clusters of every object inside the
    frustum, records {objectId, triangleCount * 3, 1, dataOffset, 0, 0} in dispatch order. The scene's
    clusters pass every per-cluster test of the oracle (the reference runs none)."""
    d = G.load("vkclusters")
    sc = G.scene(d)
    sc.clusters = d["clusters"]
    v = G.view(d["view"])
    n, recs, ids, flags = O.cull_clusters(v, sc, stride=24)
    assert flags == 0
    _cmp((n, recs), int(d["count"][0]), d["cmds"], "cluster records")
    assert np.array_equal(ids, d["dispatch"][:, 2]), "cluster ids"
    assert np.array_equal(recs[:, 0], d["dispatch"][:, 0]), "object ids"
