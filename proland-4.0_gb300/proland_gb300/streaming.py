"""View-driven streaming: a seeded camera path and the tiles its quadtree needs
per frame (tp_quadtree_requests), produced through the TileCache / producers with
tiles held while their quad exists and released when it disappears, as the
reference's TileSampler does (TileSampler.cpp:416-461).

Configuration of the benchmark's streaming case: root quad 50 km
(terrain1/helloworld.xml:51), levels 0-14, split distance 6 (TerrainNode.cpp:129:
splitFactor 2 x viewport 2048 / 1024 x tan 40 deg / tan(fov / 2) with a 58.4
degree field of view), 600 frames descending from 10 km to 50 m altitude while the
camera sweeps the terrain; the quadtrees then hold 0.9k-6.4k tiles and each frame
brings 0-2.3k new ones (about 560 on average).
"""
import ctypes as C

import numpy as np

from ._lib import check, lib

ROOT_SIZE = 50000.0
MAX_LEVEL = 14
SPLIT_DIST = 6.0


def camera_path(frames=600, seed=7, z0=10000.0, z1=50.0, root=ROOT_SIZE, speed=4.0):
    """(x, y, z) per frame: altitude falls geometrically from z0 to z1 while the
    camera sweeps a seeded smooth curve inside the terrain."""
    rng = np.random.default_rng(seed)
    t = np.linspace(0.0, 1.0, frames)
    z = z0 * (z1 / z0) ** t
    a = rng.uniform(0, 2 * np.pi, 4)
    w = 2 * np.pi * speed * t
    x = 0.3 * root * (np.sin(0.7 * w + a[0]) * 0.8 + 0.2 * np.sin(2.3 * w + a[1]))
    y = 0.3 * root * (np.cos(0.5 * w + a[2]) * 0.8 + 0.2 * np.sin(1.9 * w + a[3]))
    return np.stack([x, y, z], 1)


def quadtree_requests(cam, root=ROOT_SIZE, max_level=MAX_LEVEL, split=SPLIT_DIST, dist_factor=1.0, ground=0.0,
                      capacity=1 << 16):
    """[(level, tx, ty), ...] of the quadtree for camera position `cam`, parents first."""
    buf = (C.c_int32 * (3 * capacity))()
    n = C.c_int()
    check(lib().tp_quadtree_requests(root, max_level, split, dist_factor, float(cam[0]), float(cam[1]),
                                     float(cam[2]), ground, buf, capacity, C.byref(n)))
    a = np.frombuffer(buf, np.int32, 3 * n.value).reshape(-1, 3)
    return [tuple(int(v) for v in r) for r in a]


class Streamer:
    """Holds the tiles of the current frame's quadtree (one user each) and swaps
    them for the next frame's: new tiles are acquired (and produced by one
    scheduler run), tiles of vanished quads are released to the cache's LRU."""

    def __init__(self, producer):
        self.producer = producer
        self.held = {}

    def frame(self, requests, scheduler_run, stream=None):
        want = set(requests)
        # tiles of vanished quads go back to the cache's LRU first, so that their
        # slots can take this frame's new tiles
        for r in [r for r in self.held if r not in want]:
            self.producer.put_tile(self.held.pop(r))
        new = [r for r in requests if r not in self.held]
        for r in new:
            t = self.producer.get_tile(*r)
            if t is None:
                raise RuntimeError("tile cache full at %s" % (r,))
            self.held[r] = t
        scheduler_run([self.producer], stream)
        return new
