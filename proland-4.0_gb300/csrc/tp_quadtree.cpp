// The host request generator of view-driven streaming: the tiles a terrain's
// quadtree needs for one camera position, by TerrainQuad::update's split rule
// (TerrainQuad.cpp:80-105): a quad of size l at (ox, oy) is subdivided while
// dist < l * splitDist and its level is below maxLevel, with
// dist = TerrainNode::getCameraDist (TerrainNode.cpp:92-97) of the box
// [ox, ox + l] x [oy, oy + l] x [min(0, ground), max(0, ground)]:
//   max(|cz - zmax| / distFactor, max(min(|cx - xmin|, |cx - xmax|), min(|cy - ymin|, |cy - ymax|))).
// The root quad spans [-size/2, size/2]^2.  Every quad counts as visible (no GL
// frustum here).  Quads are listed parents first, children in the reference's
// near-to-far order (TerrainQuad.cpp:107-138).
#include <algorithm>
#include <cmath>

#include "tp_internal.h"

namespace {

struct Walk {
    double cx, cy, cz, zmin, zmax;
    float split, dist_factor;
    int max_level;
    tp_tile_req *out;
    int capacity, count;
};

void visit(Walk &w, int level, int tx, int ty, double ox, double oy, double l)
{
    if (w.count < w.capacity) w.out[w.count] = tp_tile_req{level, tx, ty};
    ++w.count;
    const float dist = (float)std::max(std::abs(w.cz - w.zmax) / w.dist_factor,
                                       std::max(std::min(std::abs(w.cx - ox), std::abs(w.cx - (ox + l))),
                                                std::min(std::abs(w.cy - oy), std::abs(w.cy - (oy + l)))));
    if (!((double)dist < l * (double)w.split && level < w.max_level)) return;
    static const int kOrder[4][4] = {{0, 1, 2, 3}, {1, 0, 3, 2}, {2, 0, 3, 1}, {3, 1, 2, 0}};
    const double mx = ox + l / 2.0, my = oy + l / 2.0;
    const int *order = kOrder[(w.cy < my ? 0 : 2) + (w.cx < mx ? 0 : 1)];
    for (int k = 0; k < 4; ++k) {
        const int c = order[k], i = c & 1, j = c >> 1;
        visit(w, level + 1, 2 * tx + i, 2 * ty + j, ox + i * l / 2.0, oy + j * l / 2.0, l / 2.0);
    }
}

}  // namespace

extern "C" int tp_quadtree_requests(double root_size, int max_level, float split_dist, float dist_factor, double cam_x,
                                    double cam_y, double cam_z, double ground, tp_tile_req *out, int capacity,
                                    int *count)
{
    if (!(root_size > 0.0) || max_level < 0 || max_level > 30 || !(split_dist > 1.0f) || !(dist_factor > 0.0f) ||
        capacity < 0 || (capacity > 0 && !out) || !count)
        return tp::fail(TP_E_BAD_ARG, "tp_quadtree_requests: bad arguments");
    Walk w{cam_x, cam_y, cam_z, std::min(0.0, ground), std::max(0.0, ground), split_dist, dist_factor, max_level, out,
           capacity, 0};
    visit(w, 0, 0, 0, -root_size / 2.0, -root_size / 2.0, root_size);
    *count = w.count;
    if (w.count > capacity) return tp::fail(TP_E_BAD_ARG, "tp_quadtree_requests: more quads than capacity");
    return TP_OK;
}
