"""Builds the residual-pyramid fixtures of the tests from the reference's DEM.dat
files (read from the reference checkout; run in a container that has it).

For each source file it writes a smaller, valid .dat pyramid holding the first
tiles (levels 0..3 and tile (4, 0, 0)): the original 7-word header and offset
table, with the offsets of the tiles left out set to an empty range, followed
by the original TIFF strips of the tiles kept, byte for byte.  The decoded
int16 samples of those tiles (decoded here with Python's zlib, independently
of the library's own inflate) and the header fields go to dem_golden.npz;
sources.txt records the source files' SHA-256.

The ortho fixture is cut the same way from the reference's RGB.dat (an
OrthoCPUProducer pyramid, 196-wide RGBA tiles): tiles (0, 0, 0) and (1, 1, 0)
kept in rgb_graph1_mini.dat, their decoded bytes in ortho_golden.npz.

    python tests/golden/make_golden.py <reference checkout>
"""
import hashlib
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle  # noqa: E402  (pure-Python .dat reader: DatFile)

SOURCES = {
    "terrain4": "src/terrain/examples/terrain4/DEM.dat",
    "edit3": "src/edit/examples/edit3/DEM.dat",
}
KEEP = [(0, 0, 0), (1, 0, 0), (2, 0, 0), (3, 0, 0), (4, 0, 0)]
ORTHO_SOURCE = ("graph1", "src/graph/examples/graph1/RGB.dat")
ORTHO_KEEP = [(0, 0, 0), (1, 1, 0)]


def mini_ortho_dat(d):
    offsets = np.zeros(2 * d.ntiles, np.int64)
    blob = b""
    for lvl, tx, ty in ORTHO_KEEP:
        tid = d.tile_id(lvl, tx, ty)
        strip = d.strip(lvl, tx, ty)
        offsets[2 * tid] = len(blob)
        blob += strip
        offsets[2 * tid + 1] = len(blob)
    head = struct.pack("<7i", d.max_level, d.tile_size, d.channels, d.root, d.root_tx, d.root_ty, d.flags)
    return head + offsets.tobytes() + blob


def mini_dat(d):
    ids = sorted({d.tile_id(*k) for k in KEEP})
    blob = b""
    offsets = np.zeros(2 * d.ntiles, np.uint32)
    for tid in ids:
        a, b = int(d.offsets[2 * tid]), int(d.offsets[2 * tid + 1])
        strip = d.data[d.header + a:d.header + b]
        offsets[2 * tid] = len(blob)
        blob += strip
        offsets[2 * tid + 1] = len(blob)
    head = struct.pack("<6if", d.min_level, d.max_level, d.tile_size, d.root_level, d.root_tx, d.root_ty, d.scale)
    return head + offsets.tobytes() + blob


def main(ref_root):
    arrays = {}
    lines = []
    for name, rel in SOURCES.items():
        path = os.path.join(ref_root, rel)
        data = open(path, "rb").read()
        lines.append("%s  %s  %d bytes  sha256 %s" % (name, rel, len(data), hashlib.sha256(data).hexdigest()))
        d = oracle.DatFile(data)
        with open(os.path.join(HERE, "dem_%s_mini.dat" % name), "wb") as f:
            f.write(mini_dat(d))
        arrays["%s_header" % name] = np.array([d.min_level, d.max_level, d.tile_size, d.root_level,
                                               d.root_tx, d.root_ty, d.ntiles], np.int32)
        arrays["%s_scale" % name] = np.array([d.scale], np.float32)
        for lvl, tx, ty in KEEP:
            arrays["%s_L%d_%d_%d" % (name, lvl, tx, ty)] = d.tile_int16(lvl, tx, ty).copy()
    np.savez_compressed(os.path.join(HERE, "dem_golden.npz"), **arrays)
    name, rel = ORTHO_SOURCE
    data = open(os.path.join(ref_root, rel), "rb").read()
    lines.append("%s  %s  %d bytes  sha256 %s" % (name, rel, len(data), hashlib.sha256(data).hexdigest()))
    od = oracle.OrthoDatFile(data)
    with open(os.path.join(HERE, "rgb_%s_mini.dat" % name), "wb") as f:
        f.write(mini_ortho_dat(od))
    oarr = {"header": np.array([od.max_level, od.tile_size, od.channels, od.root, od.root_tx, od.root_ty, od.flags,
                                od.ntiles], np.int32)}
    for lvl, tx, ty in ORTHO_KEEP:
        oarr["L%d_%d_%d" % (lvl, tx, ty)] = od.tile(lvl, tx, ty).copy()
    np.savez_compressed(os.path.join(HERE, "ortho_golden.npz"), **oarr)
    with open(os.path.join(HERE, "sources.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference checkout>")
    main(sys.argv[1])
