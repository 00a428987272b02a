"""Road meshes for elevation layers, as the graph layers build them on the host.

`road_strip` restates the undeformed branch of ElevationGraphLayer::drawCurveAltitude
(graph/.../dem/ElevationGraphLayer.cpp:247-310) for one polyline, with the widths and
tile transform of RoadElevationLayer::doCreateTile (RoadElevationLayer.cpp:409-433,
BASEWIDTH/TOTALWIDTH at :42-43).  The curve's altitude profile
(RoadElevationCurveData::getAltitude, which samples the CPU elevation tiles) is
replaced by the altitudes given at the polyline points, interpolated linearly along
the curve; caps are not drawn.  The meshes go to `elevation_layers` or to an
elevation producer's layer callback.
"""
import math

import numpy as np


def tile_transform(tile_origin, tile_size, W, border=2):
    """(centre x, centre y, factor): world point p -> clip (p - centre) * factor, and the
    texel scale of RoadElevationLayer.cpp:409-413."""
    ox, oy = tile_origin
    scale = 2.0 * (W - 1.0 - 2.0 * border) / tile_size
    return ox + tile_size / 2.0, oy + tile_size / 2.0, scale / W, scale


def road_strip(points, altitudes, width, tile_origin, tile_size, W, border=2):
    """Triangle-strip vertices [n, 4] float32 (x, y, altitude, u) of a road of the given
    width along `points` (world coordinates) on tile (origin, size)."""
    pts = np.asarray(points, np.float64)
    alt = np.asarray(altitudes, np.float64)
    cx, cy, factor, scale = tile_transform(tile_origin, tile_size, W, border)
    base = width + 2.0 * math.sqrt(2.0) / scale   # BASEWIDTH
    total = base * 3.0                            # TOTALWIDTH
    nwidth = total / base
    step = max(1.0, 1.0 / scale)
    w = total / 2.0
    n = len(pts)
    out = []

    def vert(x, y, z, u):
        out.append(((x - cx) * factor, (y - cy) * factor, z, u))

    for i in range(n):
        cur = pts[i]
        if i == 0:
            d = pts[1] - cur
            d = d / np.hypot(*d)
        elif i == n - 1:
            d = cur - pts[i - 1]
            d = d / np.hypot(*d)
        else:
            d = (cur - pts[i - 1]) / np.hypot(*(cur - pts[i - 1])) + (pts[i + 1] - cur) / np.hypot(*(pts[i + 1] - cur))
            l = (d[0] * d[0] + d[1] * d[1]) * 0.5
            d = d / l
        dx, dy = d[0] * w, d[1] * w
        vert(cur[0] - dy, cur[1] + dx, alt[i], -nwidth)
        vert(cur[0] + dy, cur[1] - dx, alt[i], nwidth)
        if i < n - 1:
            nxt = pts[i + 1]
            seg = np.hypot(*(nxt - cur))
            nx, ny = w * (nxt[0] - cur[0]) / seg, w * (nxt[1] - cur[1]) / seg
            for j in range(1, int(math.floor(seg / step))):
                c = j * step / seg
                x, y = cur[0] + c * (nxt[0] - cur[0]), cur[1] + c * (nxt[1] - cur[1])
                z = alt[i] + c * (alt[i + 1] - alt[i])
                vert(x - ny, y + nx, z, -nwidth)
                vert(x + ny, y - nx, z, nwidth)
    return np.asarray(out, np.float32)
