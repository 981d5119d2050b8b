"""The batched-views workload at full size (64 views over the 4M-object stress scene, log-uniform
1k..2M objects per view, each with its own rasterised depth and pyramid, frustum + Hi-Z + LOD),
batched in one launch, compared view by view with the oracle on the same inputs."""
import ctypes as C

import numpy as np
import pytest
import torch

from blitzen_gb300 import abi
from blitzen_gb300 import benchmarks as B
from blitzen_gb300 import scenes as S
from blitzen_gb300.culler import Culler
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def full(lib):
    c = Culler(0)
    sc = S.stress_scene(4_000_000, seed=0)
    c.setup_for_rendering(sc)
    yield c, sc
    c.close()


def test_batched_views_full_size_match_oracle(full):
    c, sc = full
    views, keep, total = B.build_views(c, sc, c.device, n_views=64)
    specs = S.multiview_specs(sc.count, 64, seed=0, lo=1000, hi=2_000_000)
    lib = abi.load()
    abi.check(lib.blz_cull_batch(c.ctx, views, 64, None), "blz_cull_batch")
    assert c.check() == 0
    threads = O.default_threads()
    for i, sp in enumerate(specs):
        objs, pyr, t = keep[i]
        hp = O.HostPyramid(B.W, B.H, abi.HIZ_D3D12)
        hp.data[:] = pyr.storage.cpu().numpy()
        n, recs, flags = O.cull(abi.MODE_TEMPORAL, views[i].view, sc, objects=S.subset_objects(sc, sp.subset),
                                pyramid=hp, stride=t.stride, threads=threads)
        gn, grecs = t.read()
        assert gn == n, f"view {i}: {gn} draws, oracle {n}"
        assert np.array_equal(grecs[:, :6], recs[:, :6]), f"view {i}: records differ"
