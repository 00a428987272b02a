"""Meshes of the road and water elevation layers, as the graph layers build them on
the host, for `elevation_layers` or an elevation producer's layer callback.

* `curve_altitude_meshes` restates the undeformed branch of
  ElevationGraphLayer::drawCurveAltitude (graph/.../dem/ElevationGraphLayer.cpp:250-370):
  a strip along a polyline with u = -nwidth / +nwidth on its two sides, subdivided
  every `step`, and the optional end caps.  The curve's altitude profile
  (ElevationCurveData::getAltitude, which samples the CPU elevation tiles) is
  replaced by the altitudes given at the polyline points, interpolated linearly along
  the curve.
* `road_strip` is that strip with the widths of RoadElevationLayer::doCreateTile
  (RoadElevationLayer.cpp:409-433, BASEWIDTH / TOTALWIDTH at :42-43), without caps.
* `curve_part_strip` restates the undeformed branch of GraphLayer::drawCurve with a
  `part` vector (graph/.../producer/GraphLayer.cpp:320-357), the water layer's area
  boundaries.
* `fill_triangles` covers area contours with triangles under the odd winding rule of
  the GLU tesselator that GraphLayer::drawArea feeds (GraphLayer.cpp:856-875,
  Tesselator.cpp): a slab decomposition, not the tesselator's own triangles (the fill
  pass writes one constant, so only the covered texels matter).
* `water_layer` gives the meshes, fragment programs and pass states of
  WaterElevationLayer::doCreateTile (WaterElevationLayer.cpp:240-350) for one tile.

Types follow the reference's: float where it computes in float (scale, widths,
drawCurve's directions), double elsewhere, vertices rounded to float.
"""
import math

import numpy as np

from . import (DEPTH_ALWAYS, DEPTH_LESS, DEPTH_NOTEQUAL, LAYER_FILL, LAYER_ROAD, LAYER_WATER_LARGE,
               LAYER_WATER_RIVER, NO_DEPTH_WRITE, NO_W_WRITE, NO_Z_WRITE, TRIANGLE_STRIP, TRIANGLES)

f32 = np.float32


def tile_transform(tile_origin, tile_size, W, border=2):
    """(centre x, centre y, factor, scale): world point p -> clip (p - centre) * factor,
    and the texel scale of RoadElevationLayer.cpp:413-414 / WaterElevationLayer.cpp:
    258-260 (float scale = 2 (W - 1 - 2 border) / size; factor = scale / W in float)."""
    ox, oy = tile_origin
    scale = f32(float(f32(2.0) * (f32(W) - f32(1.0) - f32(2.0) * f32(border))) / tile_size)
    return ox + tile_size / 2.0, oy + tile_size / 2.0, float(f32(scale / f32(W))), scale


def base_width(width, scale):
    """BASEWIDTH(width, scale) = width + 2 sqrt(2) / scale, in float."""
    return f32(f32(width) + f32(f32(2.0) * f32(math.sqrt(2.0))) / f32(scale))


def _length(v):
    """Length of a 2D vector as the reference's vec2d::length forms it: sqrt(x*x + y*y)
    in double (hypot can differ in the last bit)."""
    return math.sqrt(v[0] * v[0] + v[1] * v[1])


def _clip(transform, x, y):
    cx, cy, factor = transform[:3]
    return (x - cx) * factor, (y - cy) * factor


def curve_altitude_meshes(points, altitudes, width, nwidth, step, transform, start_cap=False, end_cap=False):
    """drawCurveAltitude's meshes for one polyline (world `points`, `altitudes` at the
    points): [start cap,] strip[, end cap] as (vertices [n, 4] float32 (x, y, z, u),
    indices or None, mode).  width, nwidth and step are the reference's float
    arguments; transform as tile_transform returns it."""
    pts = np.asarray(points, np.float64)
    alt = np.asarray(altitudes, np.float64)
    nwidth = float(f32(nwidth))
    step = float(f32(step))
    w = float(f32(f32(width) / f32(2.0)))
    n = len(pts)
    strip = []

    def vert(out, x, y, z, u):
        X, Y = _clip(transform, x, y)
        out.append((X, Y, z, u))

    def cap(cur, z, dx, dy, sign):
        v = []
        for px, py, u in ((cur[0] - dy, cur[1] + dx, nwidth), (cur[0] - dy / nwidth, cur[1] + dx / nwidth, 1.0),
                          (cur[0] + dy / nwidth, cur[1] - dx / nwidth, 1.0), (cur[0] + dy, cur[1] - dx, nwidth)):
            vert(v, px, py, z, u)
        idx_ = sign * dx * (nwidth - 1) / nwidth
        idy = sign * dy * (nwidth - 1) / nwidth
        for px, py in ((cur[0] - dy - idx_, cur[1] + dx - idy), (cur[0] - dy / nwidth - idx_, cur[1] + dx / nwidth - idy),
                       (cur[0] + dy / nwidth - idx_, cur[1] - dx / nwidth - idy), (cur[0] + dy - idx_, cur[1] - dx - idy)):
            vert(v, px, py, z, nwidth)
        ix = np.array([0, 1, 4, 4, 1, 5, 1, 2, 5, 5, 2, 6, 2, 3, 7, 7, 6, 2], np.uint32)
        return np.asarray(v, np.float32), ix, TRIANGLES

    out = []
    end = None
    for i in range(n):
        cur = pts[i]
        if i == 0:
            d = (pts[1] - cur) / _length(pts[1] - cur)
        elif i == n - 1:
            d = (cur - pts[i - 1]) / _length(cur - pts[i - 1])
        else:
            d = (cur - pts[i - 1]) / _length(cur - pts[i - 1]) + (pts[i + 1] - cur) / _length(pts[i + 1] - cur)
            l = (d[0] * d[0] + d[1] * d[1]) * 0.5
            d = d / l
        dx, dy = d[0] * w, d[1] * w
        if i == 0 and start_cap:
            out.append(cap(cur, alt[i], dx, dy, 1.0))
        vert(strip, cur[0] - dy, cur[1] + dx, alt[i], -nwidth)
        vert(strip, cur[0] + dy, cur[1] - dx, alt[i], nwidth)
        if i < n - 1:
            nxt = pts[i + 1]
            seg = _length(nxt - cur)
            nx, ny = w * (nxt[0] - cur[0]) / seg, w * (nxt[1] - cur[1]) / seg
            for j in range(1, int(math.floor(seg / step))):
                c = float(f32(f32(j) * f32(step))) / seg     # int * float is a float product
                x, y = cur[0] + c * (nxt[0] - cur[0]), cur[1] + c * (nxt[1] - cur[1])
                z = alt[i] + c * (alt[i + 1] - alt[i])
                vert(strip, x - ny, y + nx, z, -nwidth)
                vert(strip, x + ny, y - nx, z, nwidth)
        if i == n - 1 and end_cap:
            end = cap(cur, alt[i], dx, dy, -1.0)
    out.append((np.asarray(strip, np.float32), None, TRIANGLE_STRIP))
    if end is not None:
        out.append(end)
    return out


def road_strip(points, altitudes, width, tile_origin, tile_size, W, border=2):
    """Triangle-strip vertices [n, 4] float32 (x, y, altitude, u) of a road of the given
    width along `points` (world coordinates) on tile (origin, size): the road layer's
    TOTALWIDTH strip with u = -/+ TOTALWIDTH / BASEWIDTH at its sides."""
    tr = tile_transform(tile_origin, tile_size, W, border)
    scale = tr[3]
    base = base_width(width, scale)
    total = f32(base * f32(3.0))
    step = max(f32(1.0), f32(f32(1.0) / scale))
    return curve_altitude_meshes(points, altitudes, total, f32(total / base), step, tr)[0][0]


def road_layer(tile_origin, tile_size, W, roads=(), border=2):
    """The meshes RoadElevationLayer::doCreateTile (RoadElevationLayer.cpp:388-437) draws
    on one tile, in its order, as (vertices, indices or None, mode, program, state,
    fill_depth) for a producer's layer callback: for each road = (points, altitudes,
    width[, start_cap, end_cap]) whose width * scale > 1, its TOTALWIDTH(BASEWIDTH(width))
    altitude strip (nwidth TOTALWIDTH / BASEWIDTH, step max(1, 1 / scale)) with a cap at
    each end the graph marks as an extremity, road program, LESS with depth writes, z and
    w.  The graph filters (curve type ROAD, parents) are the caller's."""
    tr = tile_transform(tile_origin, tile_size, W, border)
    scale = tr[3]
    step = max(f32(1.0), f32(f32(1.0) / scale))
    out = []
    for r in roads:
        pts, alt, width = r[:3]
        caps = tuple(r[3:5]) if len(r) > 3 else (False, False)
        if f32(width) * scale <= 1.0:
            continue
        base = base_width(width, scale)
        total = f32(base * f32(3.0))
        for v, ix, mode in curve_altitude_meshes(pts, alt, total, f32(total / base), step, tr, *caps):
            out.append((v, ix, mode, LAYER_ROAD, DEPTH_LESS, 0.0))
    return out


def curve_part_strip(points, part, transform):
    """GraphLayer::drawCurve(tileCoords, p, part, ...)'s strip: vertices (x, y, 0, part.z)
    at the curve points offset by part.x along the float direction (dy, dx), and (x, y,
    0, part.w) offset by part.y along (dy, -dx); part is a vec4f, so the offsets
    dy * part.x ... are float products."""
    pts = np.asarray(points, np.float64)
    part = np.asarray(part, np.float32)
    n = len(pts)
    out = []
    prevl = f32(0.0)
    nextl = f32(_length(pts[1] - pts[0]))
    for i in range(n):
        cur = pts[i]
        if i == 0:
            dx = f32((pts[1][0] - cur[0]) / nextl)
            dy = f32((pts[1][1] - cur[1]) / nextl)
        elif i == n - 1:
            dx = f32((cur[0] - pts[i - 1][0]) / prevl)
            dy = f32((cur[1] - pts[i - 1][1]) / prevl)
        else:
            dx = f32((cur[0] - pts[i - 1][0]) / prevl)
            dy = f32((cur[1] - pts[i - 1][1]) / prevl)
            # float += double: the sum is formed in double and rounded once
            dx = f32(float(dx) + (pts[i + 1][0] - cur[0]) / float(nextl))
            dy = f32(float(dy) + (pts[i + 1][1] - cur[1]) / float(nextl))
            l = f32(f32(f32(dx * dx) + f32(dy * dy)) * f32(0.5))
            dx, dy = f32(dx / l), f32(dy / l)
        a = _clip(transform, cur[0] + float(f32(dy * part[0])), cur[1] + float(f32(dx * part[0])))
        b = _clip(transform, cur[0] + float(f32(dy * part[1])), cur[1] - float(f32(dx * part[1])))
        out.append((a[0], a[1], 0.0, float(part[2])))
        out.append((b[0], b[1], 0.0, float(part[3])))
        prevl = nextl
        if i < n - 2:
            nextl = f32(_length(pts[i + 2] - pts[i + 1]))
    return np.asarray(out, np.float32)


def fill_triangles(contours, transform, color_z=0.0, color_w=0.0):
    """Triangles [3k, 4] float32 (x, y, color_z, color_w) covering the contours (world
    points, each closed implicitly) under the odd winding rule: between consecutive
    vertex or crossing heights, the edges spanning the slab sorted by x, and the
    trapezoids between the 1st and 2nd, 3rd and 4th, ... of them."""
    edges = []
    for c in contours:
        c = np.asarray(c, np.float64)
        for k in range(len(c)):
            (xa, ya), (xb, yb) = _clip(transform, *c[k]), _clip(transform, *c[(k + 1) % len(c)])
            if ya != yb:
                edges.append((xa, ya, xb, yb) if ya < yb else (xb, yb, xa, ya))
    ys = {e[1] for e in edges} | {e[3] for e in edges}
    for i in range(len(edges)):  # heights where two edges cross
        x1, y1, x2, y2 = edges[i]
        for j in range(i + 1, len(edges)):
            x3, y3, x4, y4 = edges[j]
            den = (x2 - x1) * (y4 - y3) - (y2 - y1) * (x4 - x3)
            if den == 0.0:
                continue
            t = ((x3 - x1) * (y4 - y3) - (y3 - y1) * (x4 - x3)) / den
            s = ((x3 - x1) * (y2 - y1) - (y3 - y1) * (x2 - x1)) / den
            if 0.0 < t < 1.0 and 0.0 < s < 1.0:
                ys.add(y1 + t * (y2 - y1))
    ys = sorted(ys)

    def x_at(e, y):
        xa, ya, xb, yb = e
        return xa + (y - ya) * (xb - xa) / (yb - ya)

    out = []
    for y0, y1 in zip(ys[:-1], ys[1:]):
        ym = 0.5 * (y0 + y1)
        act = sorted((e for e in edges if e[1] < ym < e[3]), key=lambda e: x_at(e, ym))
        for k in range(0, len(act) - 1, 2):
            l, r = act[k], act[k + 1]
            l0, r0, r1, l1 = (x_at(l, y0), y0), (x_at(r, y0), y0), (x_at(r, y1), y1), (x_at(l, y1), y1)
            for tri in ((l0, r0, r1), (l0, r1, l1)):
                out.extend((p[0], p[1], color_z, color_w) for p in tri)
    return np.asarray(out, np.float32).reshape(-1, 4)


def water_layer(tile_origin, tile_size, W, areas=(), boundaries=(), curves=(), rivers=(), border=2):
    """The meshes WaterElevationLayer::doCreateTile (WaterElevationLayer.cpp:240-350)
    draws on one tile, in its order, as (vertices, indices or None, mode, program,
    state, fill_depth) for a producer's layer callback:

    * when there are areas: their contours filled with the fill program (colour 0,
      depth 0.02) under ALWAYS with depth writes, alpha (w) only; the area boundary
      curves, `boundaries` = (points, orientation) with the island orientation already
      flipped as the reference does, drawn with part (0, +-12, 1, 2) at river = 1 in
      the same state; then `curves` = (points, altitudes, width), the other curves,
      as altitude strips of their width (nwidth 1, no caps) at river = 2 under
      NOTEQUAL, no depth write, blue (z) only;
    * `rivers` = (points, altitudes, width[, start_cap, end_cap]) as altitude strips
      of TOTALWIDTH(BASEWIDTH(width)) at river = 1 under LESS with depth writes, z and w.

    Curves whose width * scale <= 1 are left out, as the reference does; the graph
    filters (curve types, parents, area membership) are the caller's.  areas: a list
    of contour lists (world points)."""
    tr = tile_transform(tile_origin, tile_size, W, border)
    scale = tr[3]
    step = max(f32(1.0), f32(f32(1.0) / scale))
    out = []
    if areas:
        fill = fill_triangles([c for a in areas for c in a], tr)
        area_state = DEPTH_ALWAYS | NO_Z_WRITE
        out.append((fill, None, TRIANGLES, LAYER_FILL, area_state, 0.02))
        for pts, orientation in boundaries:
            part = (0.0, 12.0, 1.0, 2.0) if orientation != 0 else (0.0, -12.0, 1.0, 2.0)
            out.append((curve_part_strip(pts, part, tr), None, TRIANGLE_STRIP, LAYER_WATER_RIVER, area_state, 0.0))
        for pts, alt, width in curves:
            if f32(width) * scale <= 1.0:
                continue
            for v, ix, mode in curve_altitude_meshes(pts, alt, width, 1.0, step, tr):
                out.append((v, ix, mode, LAYER_WATER_LARGE, DEPTH_NOTEQUAL | NO_DEPTH_WRITE | NO_W_WRITE, 0.0))
    for r in rivers:
        pts, alt, width = r[:3]
        caps = tuple(r[3:5]) if len(r) > 3 else (False, False)
        if f32(width) * scale <= 1.0:
            continue
        base = base_width(width, scale)
        total = f32(base * f32(3.0))
        for v, ix, mode in curve_altitude_meshes(pts, alt, total, f32(total / base), step, tr, *caps):
            out.append((v, ix, mode, LAYER_WATER_RIVER, DEPTH_LESS, 0.0))
    return out
