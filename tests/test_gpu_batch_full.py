"""The batched-views workload at full size (64 views over the 4M-object stress scene, log-uniform
1k..2M objects per view, each with its own rasterised depth and pyramid, frustum + Hi-Z + LOD),
batched in one launch under every supported launch shape and every chunk size, compared view by view
with the oracle. Each view's depth and pyramid are rebuilt by the oracle from the view's occluder
boxes; the GPU's pyramids must equal them and the oracle culls against its own."""
import numpy as np
import pytest

from blitzen_gb300 import abi
from blitzen_gb300 import benchmarks as B
from blitzen_gb300 import scenes as S
from blitzen_gb300.culler import Culler
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# (threads, objects per thread, blocks per SM, objects per chunk): every shape at the default chunk
# (512), and every chunk size the autotuner can pick (256, 512, 1024) under the extreme shapes
SHAPES = [(256, 2, 0, 0), (512, 2, 0, 0), (512, 1, 0, 0), (256, 1, 0, 0), (256, 4, 0, 0), (128, 1, 0, 0),
          (128, 2, 0, 0), (128, 4, 0, 0), (128, 8, 0, 0), (256, 2, 1, 0), (256, 2, 2, 0), (128, 2, 4, 0),
          (512, 2, 1, 0),
          (256, 2, 0, 256), (128, 8, 0, 256), (512, 1, 0, 256), (512, 2, 1, 256), (128, 1, 4, 256),
          (256, 2, 0, 1024), (128, 8, 0, 1024), (512, 1, 0, 1024), (512, 2, 1, 1024), (128, 1, 4, 1024)]


@pytest.fixture(scope="module")
def full(lib):
    c = Culler(0)
    sc = S.stress_scene(4_000_000, seed=0)
    c.setup_for_rendering(sc)
    boxes = []
    views, keep, _ = B.build_views(c, sc, c.device, n_views=64, boxes_out=boxes)
    specs = S.multiview_specs(sc.count, 64, seed=0, lo=1000, hi=2_000_000)
    threads = O.default_threads()
    ref = []
    for i, sp in enumerate(specs):
        objs, pyr, t = keep[i]
        # the view's occluder depth and pyramid rebuilt by the oracle, and the GPU's pyramid (rastered
        # and reduced on the GPU) checked against it texel for texel; the oracle culls against its own
        hp = O.pyramid_build(O.depth_raster(views[i].view, boxes[i], B.W, B.H))
        assert np.array_equal(pyr.storage.cpu().numpy().view(np.uint32), hp.data.view(np.uint32)), f"view {i}: pyramid"
        n, recs, _ = O.cull(abi.MODE_TEMPORAL, views[i].view, sc, objects=S.subset_objects(sc, sp.subset),
                            pyramid=hp, stride=t.stride, threads=threads)
        ref.append((n, recs))
    yield c, views, keep, ref
    c.close()


@pytest.mark.parametrize("shape", SHAPES)
def test_batched_views_full_size_match_oracle(full, shape):
    c, views, keep, ref = full
    lib = abi.load()
    for _, _, t in keep:
        t.count.fill_(0)
    c.set_launch_shape(*shape)
    abi.check(lib.blz_cull_batch(c.ctx, views, 64, None), "blz_cull_batch")
    assert c.check() == 0
    for i, (n, recs) in enumerate(ref):
        gn, grecs = keep[i][2].read()
        assert gn == n, f"shape {shape} view {i}: {gn} draws, oracle {n}"
        assert np.array_equal(grecs[:, :6], recs[:, :6]), f"shape {shape} view {i}: records differ"
