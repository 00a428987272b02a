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


@pytest.mark.parametrize("capacity", [4500, 6000])
def test_sampler_over_a_camera_path(ref, product, capacity):
    """TileSampler::update as written (TileSampler.cpp: prefetch, putTiles, getTiles,
    needTile, the Tree; with the reference's defaults, a producer whose scheduler does
    not prefetch) over the reference's quadtree and TileCache, frame by frame along a
    camera path, beside the product's sampler (tp_sampler_update) fed the product's
    requests: after every frame the used and unused tile counts, the free slots and the
    cache's query and miss counters are the same -- the sampler releases and acquires
    tiles in the same walk order, so its cache evicts the same tiles once it is full of
    used and cached tiles."""
    from proland_gb300 import streaming as S
    max_level = 10
    ref.ref_sampler_create(S.ROOT_SIZE, max_level, S.SPLIT_DIST, capacity)
    storage = product.TileStorage(101, 1, capacity, on_device=product.TileStorage.BOOKKEEPING)
    cache = product.TileCache(storage, "residuals")
    sampler = product.TileSampler(product.ResidualProducer(cache))
    full = 0
    for k, cam in enumerate(S.camera_path(frames=240)):
        out = np.zeros(5, np.int32)
        ref.ref_sampler_frame(cam[0], cam[1], cam[2], out.ctypes.data)
        sampler.update(S.quadtree_requests(cam, max_level=max_level))
        mine = (cache.get_used_tiles(), cache.get_unused_tiles(), storage.get_free_slots()) + cache.stats()
        assert mine == tuple(int(v) for v in out), (k, mine, list(out))
        full += int(out[2] == 0)
    sampler.close()
    assert full > 20      # the cache evicted for many frames
