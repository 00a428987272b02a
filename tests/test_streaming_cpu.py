"""The streaming request generator (tp_quadtree_requests) against the oracle's
restatement of TerrainQuad's split rule, and the camera path's request counts."""
import numpy as np
import pytest

import oracle


@pytest.fixture(scope="module")
def S(product):
    from proland_gb300 import streaming
    return streaming


def test_requests_match_oracle(S):
    cams = S.camera_path(600)
    for f in (0, 37, 150, 333, 480, 599):
        got = S.quadtree_requests(cams[f])
        want = oracle.quadtree_requests(cams[f], S.ROOT_SIZE, S.MAX_LEVEL, S.SPLIT_DIST)
        assert got == want, f
    # off-centre camera near the terrain edge, and a non-flat ground under it
    for cam, ground in (((24000.0, -24999.0, 30.0), 0.0), ((-3.0, 7.0, 900.0), 120.0)):
        assert S.quadtree_requests(cam, ground=ground) == oracle.quadtree_requests(
            cam, S.ROOT_SIZE, S.MAX_LEVEL, S.SPLIT_DIST, ground=ground)


def test_parents_first_and_capacity(S, product):
    req = S.quadtree_requests((100.0, -200.0, 60.0))
    seen = set()
    for (l, x, y) in req:
        assert l == 0 or (l - 1, x // 2, y // 2) in seen
        seen.add((l, x, y))
    assert max(l for l, _, _ in req) >= 10
    with pytest.raises(product.TPError):
        S.quadtree_requests((100.0, -200.0, 60.0), capacity=10)


def test_camera_path_request_counts(S):
    cams = S.camera_path(600)
    prev, news, sizes = set(), [], []
    for f in range(0, 600, 3):
        cur = set(S.quadtree_requests(cams[f]))
        news.append(len(cur - prev))
        sizes.append(len(cur))
        prev = cur
    assert max(sizes) <= 8192          # a frame's quadtree fits the 8192-slot cache
    assert max(news[1:]) >= 1000 and np.mean(news[1:]) >= 200
