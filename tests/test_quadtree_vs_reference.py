"""The view-driven requests (tp_quadtree_requests) against the reference's own
quadtree, compiled here by oracle/ref_build.py: TerrainQuad's constructor, update
and subdivide (TerrainQuad.cpp:44-173) and TerrainNode's getCameraDist,
getSplitDistance and getLocalCamera (TerrainNode.cpp) as written, on a stand-in
node that sees every quad and no occluder.  The quads update visits, in its order
(parents first, the children near to far), are the product's requests: along the
streaming workload's camera path and for random roots, depths, split distances,
distance factors, cameras and ground heights.

Runs where the reference tree is present; skipped elsewhere."""
import ctypes as C

import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref(oracle_lib):
    L = oracle_lib.ref_lib()
    if L is None or not hasattr(L, "ref_quadtree"):
        pytest.skip("the reference sources are not on this machine")
    return L


def reference_quads(ref, root, max_level, split, dist_factor, cam, ground):
    buf = np.empty(3 * (1 << 18), np.int32)
    n = ref.ref_quadtree(root, max_level, split, dist_factor, cam[0], cam[1], cam[2], ground, buf.ctypes.data,
                         1 << 18)
    assert n <= 1 << 18
    return [tuple(int(v) for v in buf[3 * i:3 * i + 3]) for i in range(n)]


def test_streaming_camera_path(ref, product):
    from proland_gb300 import streaming as S
    for k, cam in enumerate(S.camera_path(frames=600)):
        if k % 15:
            continue
        want = reference_quads(ref, S.ROOT_SIZE, S.MAX_LEVEL, S.SPLIT_DIST, 1.0, cam, 0.0)
        assert S.quadtree_requests(cam) == want, k


@pytest.mark.parametrize("seed", range(4))
def test_random_views(ref, product, seed):
    from proland_gb300 import streaming as S
    rng = np.random.default_rng(seed)
    for _ in range(20):
        root = float(np.float32(rng.choice([S.ROOT_SIZE, 100000.0, 12.72e6, 6000.0])))
        max_level = int(rng.integers(3, 16))
        split = float(np.float32(rng.uniform(1.2, 8.0)))
        dist_factor = float(np.float32(rng.choice([0.5, 1.0, 2.0])))
        cam = (float(rng.uniform(-root / 2, root / 2)), float(rng.uniform(-root / 2, root / 2)),
               float(rng.uniform(5.0, root / 4)))
        ground = float(np.float32(rng.uniform(-400.0, 400.0)))   # groundHeightAtCamera is a float
        want = reference_quads(ref, root, max_level, split, dist_factor, cam, ground)
        got = S.quadtree_requests(cam, root=root, max_level=max_level, split=split, dist_factor=dist_factor,
                                  ground=ground, capacity=1 << 18)
        assert got == want
