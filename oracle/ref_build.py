"""Builds oracle/_ref/libref.so from the reference's own C++ sources -- TEST
INFRASTRUCTURE ONLY: the oracle's restatement is checked against it
(tests/test_oracle_vs_reference.py); nothing of the product uses it.

The reference's hot-path files include its external engine headers (render,
task graph, resources), which are absent, so the files cannot be compiled
whole.  The pieces that carry the arithmetic are plain C++ and are compiled
as they are written, read from the reference tree at build time:

* ``core/sources/proland/math/noise.cpp`` whole (``lrandom``/``frandom`` of
  ``noise.h:50-68``, ``cnoise`` and its tables, ``noise.cpp:68-165``), with a
  stand-in for the missing ``pmath.h`` (``oracle/ref_stubs/pmath.h``);
* ``createDemNoise`` (``terrain/sources/proland/dem/ElevationProducer.cpp:50-133``),
  the function as written, against stand-in texture types that hand its float
  array back;
* the noise-layer choice of ``ElevationProducer::doCreateTile``
  (``ElevationProducer.cpp:345-376``, from ``int noiseL = 0;`` to
  ``noiseL = noiseLs[noiseL];``), wrapped in a function;
* the residual addressing and stencil loop of ``CPUElevationProducer::doCreateTile``
  (``CPUElevationProducer.cpp:178-245``, from ``int residualTileWidth`` to the
  end of the sample loop), wrapped in a function with stand-in slot, cache and
  producer types;
* ``HeightMipmap::computeResidual``, ``encodeResidual`` and ``computeApproxTile``
  (``terrain/sources/proland/preprocess/terrain/HeightMipmap.cpp:449-559``),
  the member functions as written, on a stand-in class holding ``tileSize`` and
  ``topLevelSize``.

The preprocess pyramid, in its own unit (``ref_mipmap.cpp``): ``HeightMipmap``'s
constructor, ``compute1``/``compute2``, ``readTile``, ``buildBaseLevelTiles``,
``buildMipmapLevel``, ``buildResiduals``, ``getTileHeight``, ``reset``, ``getTile``,
``getApproxTile``/``saveApproxTile``, the residual functions and the ``.dat`` writer
``generate``/``produceTile``/``produceTilesLebeguesOrder`` (``HeightMipmap.cpp``),
``AbstractTileCache``'s LRU ``getTile``, clamped ``getTileHeight`` and ``reset``
(``AbstractTileCache.cpp``) and ``rotation`` (``ColorMipmap.cpp``), on stand-in class
declarations and libtiff's writer over in-memory files (client-procedure files written
out as TIFF 6.0 with a zlib strip, for the ``.dat`` tiles through ``mfs.cpp``).

The GPU path, in a second unit (``ref_gpu.cpp``):

* ``ElevationProducer::doCreateTile`` (``ElevationProducer.cpp:280-405``, its layered
  branch included, the layers themselves given) and
  ``NormalProducer::doCreateTile`` (``NormalProducer.cpp:164-281``), the functions
  as written, with the uniform look-ups of their ``init`` functions, on stand-ins
  for the Ork engine types they call (``oracle/ref_stubs/ork_gl.h``: uniforms that
  write into the shader's variables, a framebuffer whose ``drawQuad`` runs the
  fragment shader at every pixel, slots backed by float arrays, Ork's vector and
  matrix arithmetic);
* ``OrthoProducer::doCreateTile`` (``ortho/OrthoProducer.cpp:273-385``) the same way,
  and ``createOrthoNoise`` (``:26-122``) in the first unit;
* ``WaterElevationLayer::doCreateTile`` with ``GraphLayer::drawArea``, over a stand-in
  graph, its draws recorded with the framebuffer state and uniforms at each;
* ``ElevationGraphLayer::drawCurveAltitude`` and ``GraphLayer::drawCurve`` of a part, and
  the lines of ``RoadElevationLayer::doCreateTile`` that place one road (its scale, tile
  offset, ``BASEWIDTH`` / ``TOTALWIDTH`` and the drawCurveAltitude call), on stand-in
  curves whose meshes the framebuffer stand-in records;
* in a third unit, ``ResidualProducer``'s ``init``, ``hasTile``, ``doCreateTile``,
  ``getTileSize``, ``getTileId``, ``readTile`` and ``upsample``, and
  ``OrthoCPUProducer``'s ``init``, ``hasTile``, ``doCreateTile`` and ``getTileId``, as written, with the
  reference's ``core/sources/proland/util/mfs.cpp`` and a libtiff stand-in
  (``oracle/ref_stubs/tiffio.h``, zlib), so that it reads the reference's own pyramids;
* in a fourth unit, ``TileCache``'s and ``TileStorage``'s functions
  (``core/sources/proland/producer/TileCache.cpp``, ``TileStorage.cpp``) as written, for a
  step-by-step comparison with the product's cache;
* in a fifth unit, ``TerrainQuad``'s ``update`` / ``subdivide`` and ``TerrainNode``'s
  ``getCameraDist`` (``core/sources/proland/terrain/``) as written, for the view-driven
  requests;
* in a sixth unit, ``TileSampler``'s ``update``, ``prefetch``, ``putTiles``, ``getTiles`` and
  ``needTile`` with ``TileProducer``'s cache calls, over the quadtree and cache functions
  above, for a frame-by-frame comparison with the product's sampler;
* the shaders those functions draw -- the upsample shaders of terrain1, terrain2,
  terrain4 (flipped diagonals) and the demo (modulated noise, with and without
  ``NO_CLAMP``), the normal shaders of terrain1, terrain2 (sphere) and the demo
  (coarse normals, four output formats), the blend shaders of graph1 and the demo,
  the ortho upsample shaders of terrain3 and the demo -- and the layers' fragment
  shaders (road, water, fill), rewritten mechanically into C++ by
  ``oracle/ref_glsl.py`` and compiled against ``oracle/ref_stubs/glsl.h``.

Texture sampling is the choice the oracle makes (nearest texel, clamped to the
edge; the noise array wraps), as the reference's GL filtering is not part of its
source.

Each piece is located by its text (a signature or the first and last
statements), so the recipe fails loudly if the reference differs.  The extracted
text goes to oracle/_ref/gen/ (git-ignored) and is compiled with
``-ffp-contract=off``: each float operation rounded on its own, as the C++
source writes it (a compiler that contracts a * b + c into one FMA -- the default
of gcc on aarch64 -- changes last bits; on x86-64 without FMA flags the two agree).

Usage: python oracle/ref_build.py [reference root]; the root defaults to
/root/reference, where this machine keeps the reference.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
GEN_DIR = os.path.join(OUT_DIR, "gen")
LIB = os.path.join(OUT_DIR, "libref.so")
DEFAULT_ROOT = "/root/reference"

NOISE_CPP = "src/core/sources/proland/math/noise.cpp"
NOISE_DIR = "src/core/sources"
ELEV_CPP = "src/terrain/sources/proland/dem/ElevationProducer.cpp"
CPU_ELEV_CPP = "src/terrain/sources/proland/dem/CPUElevationProducer.cpp"
MIPMAP_CPP = "src/terrain/sources/proland/preprocess/terrain/HeightMipmap.cpp"
ORTHO_CPP = "src/terrain/sources/proland/ortho/OrthoProducer.cpp"
GRAPH_LAYER_CPP = "src/graph/sources/proland/dem/ElevationGraphLayer.cpp"
ROAD_LAYER_CPP = "src/graph/sources/proland/dem/RoadElevationLayer.cpp"
GRAPH_PRODUCER_CPP = "src/graph/sources/proland/graph/producer/GraphLayer.cpp"
WATER_LAYER_CPP = "src/graph/sources/proland/dem/WaterElevationLayer.cpp"


def _read(root, rel):
    with open(os.path.join(root, rel)) as f:
        return f.read()


def _strip_comment(line):
    return line.split("//", 1)[0]


def extract_function(text, signature):
    """The function whose definition line matches the regex `signature`, from that
    line to its closing brace."""
    lines = text.splitlines()
    start = next((i for i, l in enumerate(lines) if re.search(signature, l)), None)
    if start is None:
        raise RuntimeError("reference function not found: %s" % signature)
    depth, seen = 0, False
    for k in range(start, len(lines)):
        code = _strip_comment(lines[k])
        depth += code.count("{") - code.count("}")
        seen = seen or "{" in code
        if seen and depth == 0:
            return "\n".join(lines[start:k + 1]) + "\n", start + 1
    raise RuntimeError("unbalanced braces after: %s" % signature)


def extract_block(text, first, last, after=None):
    """Lines from the one containing `first` to the one containing `last` (the first
    such lines after the line containing `after`, when given)."""
    lines = text.splitlines()
    base = 0
    if after is not None:
        base = next((i for i, l in enumerate(lines) if after in l), None)
        if base is None:
            raise RuntimeError("reference anchor not found: %s" % after)
    s = next((i for i in range(base, len(lines)) if first in lines[i]), None)
    if s is None:
        raise RuntimeError("reference statement not found: %s" % first)
    e = next((i for i in range(s, len(lines)) if last in lines[i]), None)
    if e is None:
        raise RuntimeError("reference statement not found: %s" % last)
    return "\n".join(lines[s:e + 1]) + "\n", s + 1


def extract_braced(text, first, after):
    """From the line containing `first` (after `after`) through its closing brace."""
    lines = text.splitlines()
    base = next((i for i, l in enumerate(lines) if after in l), None)
    if base is None:
        raise RuntimeError("reference anchor not found: %s" % after)
    s = next((i for i in range(base, len(lines)) if first in lines[i]), None)
    if s is None:
        raise RuntimeError("reference statement not found: %s" % first)
    depth = 0
    for k in range(s, len(lines)):
        code = _strip_comment(lines[k])
        depth += code.count("{") - code.count("}")
        if depth == 0:
            return "\n".join(lines[s:k + 1]) + "\n", s + 1
    raise RuntimeError("unbalanced braces after: %s" % first)


def extract_loop_to_end(text, first, after):
    """From the line containing `first` (after `after`) through the end of the first
    `for` loop that starts at or after it (brace matched)."""
    lines = text.splitlines()
    base = next((i for i, l in enumerate(lines) if after in l), None)
    if base is None:
        raise RuntimeError("reference anchor not found: %s" % after)
    s = next((i for i in range(base, len(lines)) if first in lines[i]), None)
    if s is None:
        raise RuntimeError("reference statement not found: %s" % first)
    f = next((i for i in range(s, len(lines)) if re.match(r"\s*for\s*\(", lines[i])), None)
    depth, seen = 0, False
    for k in range(f, len(lines)):
        code = _strip_comment(lines[k])
        depth += code.count("{") - code.count("}")
        seen = seen or "{" in code
        if seen and depth == 0:
            return "\n".join(lines[s:k + 1]) + "\n", s + 1
    raise RuntimeError("unbalanced braces after: %s" % first)


# Stand-in types the extracted pieces compile against (this project's own code).
_PRELUDE = r"""
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstring>
#include "proland/math/noise.h"
using namespace std;

namespace proland {
// createDemNoise builds a texture from its float array: these stand-ins copy the
// array out instead.
static void *g_captured = nullptr;
enum { R16F, RED, FLOAT, REPEAT, NEAREST, RGBA8, RGBA, UNSIGNED_BYTE };
struct CPUBuffer { const void *data; explicit CPUBuffer(const void *d) : data(d) {} };
struct Buffer { struct Parameters {}; };
struct Texture { struct Parameters {
    Parameters &wrapS(int) { return *this; } Parameters &wrapT(int) { return *this; }
    Parameters &min(int) { return *this; } Parameters &mag(int) { return *this; } }; };
struct Texture2DArray {
    Texture2DArray(int w, int h, int layers, int, int, int type, Texture::Parameters, Buffer::Parameters, CPUBuffer b) {
        const size_t texel = type == UNSIGNED_BYTE ? 4 : sizeof(float);   // RGBA bytes or one float
        if (g_captured) memcpy(g_captured, b.data, texel * (size_t)w * h * layers);
    }
};
template <class T> struct ptr {
    T *p;
    ptr(T *q) : p(q) {}
    ~ptr() { delete p; }
};
}  // namespace proland

// CPUElevationProducer::doCreateTile's slots, cache tiles and residual producer.
struct RefSlotBase { virtual ~RefSlotBase() {} };
template <class T> struct CPUTileStorage { struct CPUSlot : RefSlotBase { T *data = nullptr; }; };
struct TileCache { struct Tile { RefSlotBase *slot; RefSlotBase *getData() { return slot; } }; };
struct RefStorage { int w; int getTileSize() { return w; } };
struct RefCache { RefStorage s; RefStorage *getStorage() { return &s; } };
struct RefResidualProducer {
    RefCache c;
    int border = 2;
    bool has = false;
    TileCache::Tile tile{nullptr};
    int asked[3] = {-1, -1, -1};
    RefCache *getCache() { return &c; }
    int getBorder() { return border; }
    TileCache::Tile *findTile(int l, int x, int y) { asked[0] = l; asked[1] = x; asked[2] = y; return has ? &tile : nullptr; }
    bool hasTile(int, int, int) { return has; }
};

// HeightMipmap's residual members on a class holding the two sizes they read.
struct HeightMipmap {
    int tileSize, topLevelSize;
    void computeResidual(float *parentTile, float *tile, int level, int tx, int ty, float *residual, float &maxR, float &meanR);
    void encodeResidual(int level, float *residual, unsigned char *encoded);
    void computeApproxTile(float *parentTile, float *residual, int level, int tx, int ty, float *tile, float &maxErr);
};
"""


def generate(root):
    elev = _read(root, ELEV_CPP)
    cpu = _read(root, CPU_ELEV_CPP)
    mip = _read(root, MIPMAP_CPP)
    dem, dem_line = extract_function(elev, r"ptr<Texture2DArray>\s+createDemNoise\s*\(\s*int\s+tileWidth\s*\)")
    orn, orn_line = extract_function(_read(root, ORTHO_CPP),
                                     r"ptr<Texture2DArray>\s+createOrthoNoise\s*\(\s*int\s+tileWidth\s*\)")
    sel, sel_line = extract_block(elev, "int noiseL = 0;", "noiseL = noiseLs[noiseL];",
                                  after="bool ElevationProducer::doCreateTile(")
    loop, loop_line = extract_loop_to_end(cpu, "int residualTileWidth =", after="bool CPUElevationProducer::doCreateTile(")
    fns = []
    for name in ("computeResidual", "encodeResidual", "computeApproxTile"):
        body, line = extract_function(mip, r"void\s+HeightMipmap::%s\s*\(" % name)
        fns.append(("HeightMipmap.cpp:%d" % line, body))
    src = [_PRELUDE]
    src.append("namespace proland {\n// %s:%d\n%s}  // namespace proland\n" % (ELEV_CPP, dem_line, dem))
    src.append("namespace proland {\n// %s:%d\n%s}  // namespace proland\n" % (ORTHO_CPP, orn_line, orn))
    src.append(r"""
extern "C" long ref_lrandom(long *seed) { return proland::lrandom(seed); }
extern "C" float ref_frandom(long *seed) { return proland::frandom(seed); }
extern "C" float ref_cnoise2(float x, float y) { return proland::cnoise(x, y); }
extern "C" void ref_dem_noise(int W, float *out)
{
    proland::g_captured = out;
    proland::createDemNoise(W);
    proland::g_captured = nullptr;
}
extern "C" void ref_ortho_noise(int W, unsigned char *out)
{
    proland::g_captured = out;
    proland::createOrthoNoise(W);
    proland::g_captured = nullptr;
}
""")
    src.append("""
extern "C" void ref_noise_select(int face, int level, int tx, int ty, int *rot, int *layer)
{
    using namespace proland;
    // %s:%d
%s
    *rot = noiseR;
    *layer = noiseL;
}
""" % (ELEV_CPP, sel_line, sel))
    src.append("""
// residual: residual_width^2 floats or NULL (hasTile false); asked: the residual tile
// (level, tx, ty) the loop looked up
extern "C" void ref_cpu_elevation_tile(int tileWidth, int level, int tx, int ty, float *parent, int residual_width,
                                       float *residual, float *out, int *asked)
{
    const int tileSize = tileWidth - 5;
    CPUTileStorage<float>::CPUSlot parentSlot, outSlot, resSlot;
    parentSlot.data = parent;
    outSlot.data = out;
    resSlot.data = residual;
    CPUTileStorage<float>::CPUSlot *parentCpuData = level > 0 ? &parentSlot : NULL;
    CPUTileStorage<float>::CPUSlot *cpuData = &outSlot;
    RefResidualProducer producer;
    producer.c.s.w = residual_width;
    producer.has = residual != NULL;
    producer.tile.slot = &resSlot;
    RefResidualProducer *residualTiles = &producer;
    // %s:%d
%s
    asked[0] = producer.asked[0];
    asked[1] = producer.asked[1];
    asked[2] = producer.asked[2];
}
""" % (CPU_ELEV_CPP, loop_line, loop))
    for where, body in fns:
        src.append("// %s\n%s" % (where, body))
    src.append(r"""
extern "C" void ref_compute_residual(int tile_size, int top_level_size, float *parent, float *tile, int level, int tx,
                                     int ty, float *residual, float *max_r, float *mean_r)
{
    HeightMipmap h{tile_size, top_level_size};
    h.computeResidual(parent, tile, level, tx, ty, residual, *max_r, *mean_r);
}
extern "C" void ref_encode_residual(int tile_size, int top_level_size, int level, float *residual, unsigned char *encoded)
{
    HeightMipmap h{tile_size, top_level_size};
    h.encodeResidual(level, residual, encoded);
}
extern "C" void ref_compute_approx_tile(int tile_size, int top_level_size, float *parent, float *residual, int level,
                                        int tx, int ty, float *tile, float *max_err)
{
    HeightMipmap h{tile_size, top_level_size};
    h.computeApproxTile(parent, residual, level, tx, ty, tile, *max_err);
}
""")
    os.makedirs(GEN_DIR, exist_ok=True)
    path = os.path.join(GEN_DIR, "ref_pieces.cpp")
    with open(path, "w") as f:
        f.write("".join(src))
    return path


# ---- the preprocess pyramid: HeightMipmap's levels and residuals -----------------------
TILE_CACHE_CPP = "src/terrain/sources/proland/preprocess/terrain/AbstractTileCache.cpp"
COLOR_MIPMAP_CPP = "src/terrain/sources/proland/preprocess/terrain/ColorMipmap.cpp"
_MIPMAP_PRELUDE = r"""
#include <assert.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <zlib.h>

#include <algorithm>
#include <list>
#include <map>
#include <string>
#include <vector>

#include "proland/util/mfs.h"

#define printf(...) ((void)0)

namespace refmip {
using std::list;
using std::map;
using std::max;
using std::min;
using std::string;

// libtiff's writer and directory reader over files held in memory.  A file is its list of
// directories, a directory the one strip written into it: the pyramid's tiles are one
// Deflate strip each, and reading a lossless strip back gives the bytes written.  A file
// opened on client procedures (TIFFClientOpen, how HeightMipmap::produceTile writes the
// .dat tiles) is written out at TIFFClose as a little-endian TIFF 6.0 file: the header,
// the strip compressed by zlib at the default level (libtiff's Deflate), then one image
// directory with the fields set on it and the strip's offset, byte count and row count.
typedef int32_t tsize_t;
typedef uint32_t toff_t;
typedef void *thandle_t;
typedef tsize_t (*TIFFReadWriteProc)(thandle_t, void *, tsize_t);
typedef toff_t (*TIFFSeekProc)(thandle_t, toff_t, int);
typedef int (*TIFFCloseProc)(thandle_t);
typedef toff_t (*TIFFSizeProc)(thandle_t);
typedef int (*TIFFMapFileProc)(thandle_t, void **, toff_t *);
typedef void (*TIFFUnmapFileProc)(thandle_t, void *, toff_t);
enum {
    TIFFTAG_IMAGEWIDTH = 256, TIFFTAG_IMAGELENGTH = 257, TIFFTAG_BITSPERSAMPLE = 258, TIFFTAG_COMPRESSION = 259,
    TIFFTAG_PHOTOMETRIC = 262, TIFFTAG_ORIENTATION = 274, TIFFTAG_SAMPLESPERPIXEL = 277, TIFFTAG_PLANARCONFIG = 284,
    COMPRESSION_DEFLATE = 32946, ORIENTATION_BOTLEFT = 4, PLANARCONFIG_CONTIG = 1, PHOTOMETRIC_MINISBLACK = 1
};
typedef std::vector<std::vector<unsigned char>> MemTiff;
static map<string, MemTiff> g_tiff;
struct TIFF {
    string name;
    bool writing;
    MemTiff dirs;
    std::vector<unsigned char> strip;
    int dir;
    thandle_t handle = nullptr;  // client procedures, when opened on them
    TIFFReadWriteProc write = nullptr;
    TIFFSeekProc seek = nullptr;
    TIFFCloseProc close = nullptr;
    map<int, uint32_t> fields;
};
TIFF *TIFFOpen(const char *name, const char *mode)
{
    TIFF *f = new TIFF{name, mode[0] == 'w', MemTiff(), {}, 0};
    if (!f->writing) {
        auto i = g_tiff.find(name);
        if (i == g_tiff.end()) {
            delete f;
            return nullptr;
        }
        f->dirs = i->second;
    }
    return f;
}
TIFF *TIFFClientOpen(const char *name, const char *, thandle_t h, TIFFReadWriteProc, TIFFReadWriteProc wr,
                     TIFFSeekProc sk, TIFFCloseProc cl, TIFFSizeProc, TIFFMapFileProc, TIFFUnmapFileProc)
{
    TIFF *f = new TIFF{name, true, MemTiff(), {}, 0};
    f->handle = h;
    f->write = wr;
    f->seek = sk;
    f->close = cl;
    return f;
}
int TIFFSetField(TIFF *f, int tag, ...)
{
    va_list ap;
    va_start(ap, tag);
    f->fields[tag] = va_arg(ap, uint32_t);
    va_end(ap);
    return 1;
}
static void tiff_put(std::vector<unsigned char> &b, uint32_t v, int n)
{
    for (int k = 0; k < n; ++k) b.push_back((unsigned char)(v >> (8 * k)));
}
// the client file of TIFFClose: header, compressed strip, image directory
static void tiff_write_client(TIFF *f)
{
    const std::vector<unsigned char> &raw = f->dirs.empty() ? f->strip : f->dirs[0];
    uLongf zn = compressBound(raw.size());
    std::vector<unsigned char> z(zn);
    compress2(z.data(), &zn, raw.data(), raw.size(), Z_DEFAULT_COMPRESSION);
    z.resize(zn);
    std::vector<unsigned char> b = {'I', 'I'};
    tiff_put(b, 42, 2);
    tiff_put(b, 8 + (uint32_t)((z.size() + 1) & ~(size_t)1), 4);
    b.insert(b.end(), z.begin(), z.end());
    if (b.size() & 1) b.push_back(0);
    map<int, uint32_t> fl = f->fields;
    if (!fl.count(TIFFTAG_COMPRESSION)) fl[TIFFTAG_COMPRESSION] = 1;
    fl[273] = 8;                        // StripOffsets
    fl[278] = fl[TIFFTAG_IMAGELENGTH];  // RowsPerStrip
    fl[279] = (uint32_t)z.size();       // StripByteCounts
    const uint32_t spp = fl.count(TIFFTAG_SAMPLESPERPIXEL) ? fl[TIFFTAG_SAMPLESPERPIXEL] : 1;
    tiff_put(b, (uint32_t)fl.size(), 2);
    for (auto &e : fl) {
        const bool wide = e.first == 256 || e.first == 257 || e.first == 273 || e.first == 278 || e.first == 279;
        const uint32_t count = e.first == TIFFTAG_BITSPERSAMPLE ? spp : 1;
        tiff_put(b, e.first, 2);
        tiff_put(b, wide ? 4 : 3, 2);
        tiff_put(b, count, 4);
        if (wide) {
            tiff_put(b, e.second, 4);
        } else {
            // up to two SHORTs fit in the entry; the pyramid's tiles have at most two samples
            tiff_put(b, e.second, 2);
            tiff_put(b, count > 1 ? e.second : 0, 2);
        }
    }
    tiff_put(b, 0, 4);
    f->seek(f->handle, 0, SEEK_SET);
    f->write(f->handle, b.data(), (tsize_t)b.size());
    f->close(f->handle);
}
tsize_t TIFFWriteEncodedStrip(TIFF *f, int, void *data, tsize_t size)
{
    const unsigned char *p = (const unsigned char *)data;
    f->strip.assign(p, p + size);
    return size;
}
int TIFFWriteDirectory(TIFF *f)
{
    f->dirs.push_back(f->strip);
    f->strip.clear();
    return 1;
}
int TIFFSetDirectory(TIFF *f, int d)
{
    f->dir = d;
    return d < (int)f->dirs.size();
}
tsize_t TIFFReadEncodedStrip(TIFF *f, int, void *buf, tsize_t)
{
    if (f->dir >= (int)f->dirs.size()) return -1;
    const std::vector<unsigned char> &s = f->dirs[f->dir];
    memcpy(buf, s.data(), s.size());
    return (tsize_t)s.size();
}
void TIFFClose(TIFF *f)
{
    if (f->write) {
        tiff_write_client(f);
    } else if (f->writing) {
        g_tiff[f->name] = f->dirs;
    }
    delete f;
}
// Util.cpp's flog: whether a file is still to be made (its log-file restart is left out)
bool flog(const string &name) { return g_tiff.find(name) == g_tiff.end(); }
// Ork's fopen(FILE **, name, mode)
inline void fopen(FILE **f, const char *name, const char *mode) { *f = ::fopen(name, mode); }

// AbstractTileCache.h and HeightMipmap.h: the classes' members and virtual functions,
// all public so that the test driver can set the current level
struct vec4f {
    float x, y, z, w;
};
struct AbstractTileCache {
    struct Tile {
        int tx, ty;
        unsigned char *data;
        Tile(int tx, int ty, unsigned char *data = NULL) : tx(tx), ty(ty), data(data) {}
        ~Tile() { delete[] data; }
        int key(int width) { return tx + ty * width; }
    };
    AbstractTileCache(int width, int height, int tileSize, int channels, int capacity = 20)
        : width(width), height(height), tileSize(tileSize), channels(channels), capacity(capacity) {}
    virtual ~AbstractTileCache() { reset(0, 0, 0); }
    int getWidth() { return width; }
    int getHeight() { return height; }
    int getTileSize() { return tileSize; }
    unsigned char *getTile(int tx, int ty);
    virtual float getTileHeight(int x, int y);
    virtual void reset(int width, int height, int tileSize);
    virtual unsigned char *readTile(int tx, int ty) = 0;
    int width, height, tileSize, channels, capacity;
    typedef map<int, list<Tile *>::iterator> Cache;
    Cache tileCache;
    list<Tile *> tileCacheOrder;
};
struct HeightMipmap : AbstractTileCache {
    struct HeightFunction {
        virtual float getHeight(int x, int y) = 0;
    };
    HeightMipmap *left, *right, *bottom, *top;
    int leftr, rightr, bottomr, topr;
    HeightMipmap(HeightFunction *height, int topLevelSize, int baseLevelSize, int tileSize, float scale,
                 const string &cache);
    ~HeightMipmap();
    void compute1();
    bool compute2();
    virtual float getTileHeight(int x, int y);
    virtual void reset(int width, int height, int tileSize);
    virtual unsigned char *readTile(int tx, int ty);
    virtual void getTile(int level, int tx, int ty, float *tile);
    HeightFunction *height;
    int topLevelSize, baseLevelSize, tileSize;
    float scale;
    string cache;
    int minLevel, maxLevel, currentMipLevel;
    unsigned char *tile;
    int currentLevel, constantTile;
    void generate(int rootLevel, int rootTx, int rootTy, float scale, const string &file);
    void buildBaseLevelTiles();
    void buildBaseLevelTile(int tx, int ty, TIFF *f);
    void buildMipmapLevel(int level);
    void buildResiduals(int level);
    void getApproxTile(int level, int tx, int ty, float *tile);
    void saveApproxTile(int level, int tx, int ty, float *tile);
    void computeResidual(float *parentTile, float *tile, int level, int tx, int ty, float *residual, float &maxR,
                         float &meanR);
    void encodeResidual(int level, float *residual, unsigned char *encoded);
    void computeApproxTile(float *parentTile, float *residual, int level, int tx, int ty, float *tile, float &maxErr);
    void produceTile(int level, int tx, int ty, unsigned int *offset, unsigned int *offsets, FILE *f);
    void produceTilesLebeguesOrder(int l, int level, int tx, int ty, unsigned int *offset, unsigned int *offsets,
                                   FILE *f);
};
"""

_MIPMAP_DRIVER = r"""
// the input map: int16 samples on a (baseLevelSize + 1)^2 grid, read with clamped coordinates
struct GridHeights : HeightMipmap::HeightFunction {
    const int16_t *h = nullptr;
    int n = 0;
    float getHeight(int x, int y)
    {
        x = x < 0 ? 0 : (x > n - 1 ? n - 1 : x);
        y = y < 0 ? 0 : (y > n - 1 ? n - 1 : y);
        return h[(size_t)y * n + x];
    }
};
static HeightMipmap *g_mip = nullptr;
static GridHeights g_heights;
}  // namespace refmip

using namespace refmip;

// HeightMipmap's pyramid of `base` ((top << max_level) + 1 square, tiles of ts >= top
// intervals): compute1 (base-level tiles), compute2 until it is done (the levels below),
// then buildResiduals for levels 1..max_level, as HeightMipmap::generate runs them.  The
// approximation tiles go to files in `dir`.  Returns maxLevel.
extern "C" int ref_mipmap_build_sized(const int16_t *base, int top, int ts, int max_level, float scale,
                                      const char *dir)
{
    delete g_mip;
    g_tiff.clear();
    g_heights.h = base;
    g_heights.n = (top << max_level) + 1;
    g_mip = new HeightMipmap(&g_heights, top, top << max_level, ts, scale, dir);
    g_mip->compute1();
    while (g_mip->compute2()) {
    }
    for (int level = 1; level <= g_mip->maxLevel; ++level) g_mip->buildResiduals(level);
    g_heights.h = nullptr;
    return g_mip->maxLevel;
}
extern "C" int ref_mipmap_build(const int16_t *base, int ts, int max_level, float scale, const char *dir)
{
    return ref_mipmap_build_sized(base, ts, ts, max_level, scale, dir);
}

// HeightMipmap::generate after ref_mipmap_build_sized: the .dat pyramid file at `path`
// (its residual levels are built already, so generate only writes the file); minLevel
extern "C" int ref_mipmap_generate(int root_level, int root_tx, int root_ty, float scale, const char *path)
{
    g_mip->generate(root_level, root_tx, root_ty, scale, path);
    return g_mip->minLevel;
}

// HeightMipmap::getTile of (level, tx, ty), the cache set to that level as buildResiduals
// sets it: (ts + 5)^2 floats
extern "C" void ref_mipmap_level_tile(int level, int tx, int ty, float *out)
{
    HeightMipmap *m = g_mip;
    m->currentLevel = level;
    const int n = m->baseLevelSize >> (m->maxLevel - level);
    m->reset(n, n, min(m->topLevelSize << level, m->tileSize));
    m->getTile(level, tx, ty, out);
}

// the approximation tile of (level, tx, ty) (level < maxLevel): getApproxTile, (ts + 5)^2 floats
extern "C" void ref_mipmap_approx_tile(int level, int tx, int ty, float *out)
{
    g_mip->getApproxTile(level, tx, ty, out);
}

// the encoded residual of (level, tx, ty) from buildResiduals' files: its byte count, or -1
extern "C" int ref_mipmap_residual(int level, int tx, int ty, unsigned char *out, int cap)
{
    HeightMipmap *m = g_mip;
    const int nTiles = max(1, (m->baseLevelSize / m->tileSize) >> (m->maxLevel - level));
    const int per = min(nTiles, 16);
    char name[512];
    snprintf(name, sizeof(name), "%s/residual-%.2d-%.4d-%.4d.tiff", m->cache.c_str(), level, tx / per, ty / per);
    auto i = g_tiff.find(name);
    const int d = tx % per + (ty % per) * per;
    if (i == g_tiff.end() || d >= (int)i->second.size() || (int)i->second[d].size() > cap) return -1;
    memcpy(out, i->second[d].data(), i->second[d].size());
    return (int)i->second[d].size();
}

extern "C" void ref_mipmap_free()
{
    delete g_mip;
    g_mip = nullptr;
    g_tiff.clear();
}
"""


def generate_mipmap(root):
    """oracle/_ref/gen/ref_mipmap.cpp: HeightMipmap's pyramid build as written -- base-level
    tiles, decimated levels, the residual chain -- with AbstractTileCache's tile cache and
    clamped reads, against in-memory TIFF files."""
    mip = _read(root, MIPMAP_CPP)
    src = ["// generated by oracle/ref_build.py from the reference's sources\n", _MIPMAP_PRELUDE]
    tc = _read(root, TILE_CACHE_CPP)
    for sig in (r"unsigned char\s*\*\s*AbstractTileCache::getTile\s*\(", r"float\s+AbstractTileCache::getTileHeight\s*\(",
                r"void\s+AbstractTileCache::reset\s*\("):
        body, line = extract_function(tc, sig)
        src.append("// %s:%d\n%s" % (TILE_CACHE_CPP, line, body))
    body, line = extract_function(_read(root, COLOR_MIPMAP_CPP), r"void\s+rotation\s*\(\s*int\s+r\s*,.*\)\s*$")
    src.append("// %s:%d\n%s" % (COLOR_MIPMAP_CPP, line, body))
    for sig in (r"HeightMipmap::HeightMipmap\s*\(", r"HeightMipmap::~HeightMipmap\s*\(", r"void\s+HeightMipmap::compute1\s*\(",
                r"bool\s+HeightMipmap::compute2\s*\(", r"unsigned char\s*\*\s*HeightMipmap::readTile\s*\(",
                r"void\s+HeightMipmap::buildBaseLevelTiles\s*\(", r"void\s+HeightMipmap::buildBaseLevelTile\s*\(",
                r"void\s+HeightMipmap::buildMipmapLevel\s*\(", r"void\s+HeightMipmap::buildResiduals\s*\(",
                r"float\s+HeightMipmap::getTileHeight\s*\(", r"void\s+HeightMipmap::reset\s*\(",
                r"void\s+HeightMipmap::getTile\s*\(", r"void\s+HeightMipmap::getApproxTile\s*\(",
                r"void\s+HeightMipmap::saveApproxTile\s*\(", r"void\s+HeightMipmap::computeResidual\s*\(",
                r"void\s+HeightMipmap::encodeResidual\s*\(", r"void\s+HeightMipmap::computeApproxTile\s*\(",
                r"void\s+HeightMipmap::generate\s*\(", r"void\s+HeightMipmap::produceTile\s*\(",
                r"void\s+HeightMipmap::produceTilesLebeguesOrder\s*\("):
        body, line = extract_function(mip, sig)
        src.append("// %s:%d\n%s" % (MIPMAP_CPP, line, body))
    src.append(_MIPMAP_DRIVER)
    os.makedirs(GEN_DIR, exist_ok=True)
    path = os.path.join(GEN_DIR, "ref_mipmap.cpp")
    with open(path, "w") as f:
        f.write("".join(src))
    return path


# ---- the GPU path: producers' doCreateTile with the shaders they draw ------------------
NORMAL_CPP = "src/terrain/sources/proland/dem/NormalProducer.cpp"
# variant index -> (name, shader, extra defines); the indices are the first argument
# of ref_gl_elevation_tile / ref_gl_normal_tile
UPSAMPLE_SHADERS = [
    ("terrain1", "src/terrain/examples/terrain1/upsampleShader.glsl", ()),
    ("terrain2", "src/terrain/examples/terrain2/upsampleShader.glsl", ()),
    ("terrain4", "src/terrain/examples/terrain4/upsampleShader.glsl", ()),
    ("demo", "src/demo/shaders/elevation/upsampleShader.glsl", ()),
    ("demo_noclamp", "src/demo/shaders/elevation/upsampleShader.glsl", ("NO_CLAMP",)),
]
NORMAL_SHADERS = [
    ("terrain1", "src/terrain/examples/terrain1/normalShader.glsl", ()),
    ("terrain2", "src/terrain/examples/terrain2/normalShader.glsl", ()),
    ("demo", "src/demo/shaders/elevation/normalShader.glsl", ()),
]
# the blend programs ElevationProducer draws after the layers (index: ref_gl_elevation_tile_layers)
BLEND_SHADERS = [
    ("graph1", "src/graph/examples/graph1/blendShader.glsl", ()),
    ("demo", "src/demo/shaders/elevation/blendShader.glsl", ()),
]
# the ortho producer's upsample programs (index: ref_gl_ortho_tile)
ORTHO_SHADERS = [
    ("terrain3", "src/terrain/examples/terrain3/upsampleOrthoShader.glsl", ()),
    ("demo", "src/demo/shaders/ortho/upsampleOrthoShader.glsl", ()),
]
# the layers' fragment programs (index: ref_gl_layer_fragment)
LAYER_SHADERS = [
    ("road_graph1", "src/graph/examples/graph1/roadLayerElevationShader.glsl", ()),
    ("road_demo", "src/demo/shaders/elevation/roadLayerElevationShader.glsl", ()),
    ("water_river1", "src/river/examples/river1/waterLayerElevationShader.glsl", ()),
    ("water_demo", "src/demo/shaders/elevation/waterLayerElevationShader.glsl", ()),
    ("fill", "src/river/examples/river1/fillShader.glsl", ()),
]

_GPU_PRELUDE = r"""
namespace refgl {
Logger *Logger::DEBUG_LOGGER = nullptr;
Logger *Logger::ERROR_LOGGER = nullptr;
using proland::cnoise;
using std::abs;
using std::atan2;
using std::floor;
using std::max;

// The graph types drawCurveAltitude reads (graph/Curve.h, dem/ElevationCurveData.h):
// a polyline with its curvilinear coordinates and width; the altitude profile is
// the identity, getAltitude(s) = s, so that a vertex's altitude shows where on the
// curve it was sampled.
// A curve's type, parent and first area (WaterElevationLayer reads them; no parent:
// the curve is its own), and whether a cap is wanted at each end (GraphLayer::extremity).
struct Node {};
typedef ptr<Node> NodePtr;
struct Area;
struct Curve {
    vector<vec2d> points;
    vector<float> s;
    float width = 0.0f;
    int type = 0;
    Curve *parent = nullptr;
    Area *area1 = nullptr;
    bool cap_start = false, cap_end = false;
    Node start, end;
    int getSize() const { return (int)points.size(); }
    vec2d getXY(int i) const { return points[i]; }
    float getS(int i) const { return s[i]; }
    float getWidth() const { return width; }
    int getType() const { return type; }
    ptr<Curve> getParent() const { return ptr<Curve>(parent); }
    ptr<Area> getArea1() const { return ptr<Area>(area1); }
    ptr<Curve> getAncestor() const { return ptr<Curve>(const_cast<Curve *>(this)); }
    NodePtr getStart() const { return NodePtr(const_cast<Node *>(&start)); }
    NodePtr getEnd() const { return NodePtr(const_cast<Node *>(&end)); }
};
typedef ptr<Curve> CurvePtr;
struct CurveData {
    virtual ~CurveData() {}
};
struct ElevationCurveData : CurveData {
    float getAltitude(float s) { return s; }
};
// an area: its boundary curves with their orientations (graph/Area.h)
struct Area {
    vector<std::pair<Curve *, int> > curves;
    int getCurveCount() const { return (int)curves.size(); }
    CurvePtr getCurve(int j, int &orientation) const
    {
        orientation = curves[j].second;
        return CurvePtr(curves[j].first);
    }
};
typedef ptr<Area> AreaPtr;
// the tessellator records the contours it is given (GLU, which triangulates them, is
// not here)
struct Tesselator {
    vector<vector<vec2d> > contours;
    void beginPolygon(ptr<Mesh<vec2f, unsigned int> >) { contours.clear(); }
    void beginContour() { contours.emplace_back(); }
    void newVertex(double x, double y) { contours.back().push_back(vec2d(x, y)); }
    void endContour() {}
    void endPolygon() {}
};

// GraphLayer's members the drawing functions call: isDeformed, extremity (here
// whether the curve asks for a cap at that end), GraphLayer::drawCurve of a part and
// drawArea.
struct GraphLayer {
    bool deformed = false;
    bool isDeformed() const { return deformed; }
    bool extremity(CurvePtr c, NodePtr p) { return p.p == &c->start ? c->cap_start : c->cap_end; }
    void drawCurve(const vec3d &tileCoords, CurvePtr p, const vec4f &part, ptr<FrameBuffer> fb, ptr<Program> prog,
                   Mesh<vec4f, unsigned int> &mesh, vec2d *nx, vec2d *ny, vec2d *lx, vec2d *ly);
    void drawArea(const vec3d &tileCoords, AreaPtr a, Tesselator &tess);
};

struct ElevationGraphLayer : GraphLayer {
    void drawCurveAltitude(const vec3d &tileCoords, CurvePtr p, ElevationCurveData *data, float width, float nwidth,
                           float stepLength, bool caps, ptr<FrameBuffer> fb, ptr<Program> prog,
                           Mesh<vec4f, unsigned int> &mesh, vec2d *nx, vec2d *ny, vec2d *lx, vec2d *ly);
};

// WaterElevationLayer::doCreateTile's graph: curves and areas, in the order its
// iterators give them (graph/Graph.h), on an object slot of the graph producer's tile.
struct GraphObject {
    virtual ~GraphObject() {}
};
struct Graph : GraphObject {
    vector<Curve *> curves;
    vector<Area *> areas;
    struct AreaIterator {
        const Graph *g = nullptr;
        size_t k = 0;
        bool hasNext() { return k < g->areas.size(); }
        AreaPtr next() { return AreaPtr(g->areas[k++]); }
    };
    struct CurveIterator {
        const Graph *g = nullptr;
        size_t k = 0;
        bool hasNext() { return k < g->curves.size(); }
        CurvePtr next() { return CurvePtr(g->curves[k++]); }
    };
    AreaIterator area_it;
    CurveIterator curve_it;
    int getCurveCount() { return (int)curves.size(); }
    int getAreaCount() { return (int)areas.size(); }
    ptr<AreaIterator> getAreas()
    {
        area_it.g = this;
        area_it.k = 0;
        return ptr<AreaIterator>(&area_it);
    }
    ptr<CurveIterator> getCurves()
    {
        curve_it.g = this;
        curve_it.k = 0;
        return ptr<CurveIterator>(&curve_it);
    }
};
typedef ptr<Graph> GraphPtr;
struct ObjectTileStorage {
    struct ObjectSlot : TileStorage::Slot {
        ptr<GraphObject> data;
    };
};
struct SceneManager {
    static FrameBuffer *current;
    static ptr<FrameBuffer> getCurrentFrameBuffer() { return ptr<FrameBuffer>(current); }
};
struct WaterElevationCurveData {
    enum riverType { RIVER = 0, ISLAND = 1, LAKE = 2 };
};

// The members WaterElevationLayer::doCreateTile uses (WaterElevationLayer.h,
// GraphLayer / TileLayer): the tile's coordinates q, flat (no deformation).
struct WaterElevationLayer : ElevationGraphLayer {
    int displayLevel = 0;
    ptr<TileProducer> graphProducer;
    ptr<Program> layerProgram, fillProg;
    ptr<Mesh<vec2f, unsigned int> > mesh;
    ptr<Mesh<vec4f, unsigned int> > meshuv;
    ptr<Tesselator> tess;
    ptr<Uniform3f> tileOffsetU;
    ptr<Uniform1i> riverU;
    ptr<Uniform3f> fillOffsetU;
    ptr<Uniform1f> depthU;
    ptr<Uniform4f> colorU;
    vec3d q;
    int tileSize = 101, tileBorder = 2;
    std::map<Curve *, ElevationCurveData> curveData;
    vec3d getTileCoords(int, int, int) { return q; }
    void getDeformParameters(const vec3d &, vec2d &, vec2d &, vec2d &, vec2d &) {}
    int getTileSize() { return tileSize; }
    int getTileBorder() { return tileBorder; }
    CurveData *findCurveData(CurvePtr c) { return &curveData[c.p]; }
    int getProducerId() { return 0; }
    bool doCreateTile(int level, int tx, int ty, TileStorage::Slot *data);
};

struct RoadElevationCurveData {
    enum roadType { ROAD = 0, UNKNOWN = 1, BRIDGE = 2 };
};

// The members RoadElevationLayer::doCreateTile uses (RoadElevationLayer.h, GraphLayer /
// TileLayer), and draw_road: its lines that place one road on a tile.
struct RoadElevationLayer : ElevationGraphLayer {
    int tileSize = 101, tileBorder = 2;
    int displayLevel = 0;
    ptr<TileProducer> graphProducer;
    ptr<Program> layerProgram;
    Mesh<vec4f, unsigned int> *meshuv = nullptr;
    ptr<Uniform3f> tileOffsetU;
    vec3d q;
    std::map<Curve *, ElevationCurveData> curveData;
    int getTileSize() { return tileSize; }
    int getTileBorder() { return tileBorder; }
    vec3d getTileCoords(int, int, int) { return q; }
    void getDeformParameters(const vec3d &, vec2d &, vec2d &, vec2d &, vec2d &) {}
    CurveData *findCurveData(CurvePtr c) { return &curveData[c.p]; }
    int getProducerId() { return 0; }
    bool doCreateTile(int level, int tx, int ty, TileStorage::Slot *data);
    void draw_road(const vec3d &q, CurvePtr c, ElevationCurveData *cData, ptr<FrameBuffer> fb, float *scale_out);
};

// The members ElevationProducer::doCreateTile and its init's uniform look-ups use
// (ElevationProducer.h), on the stand-in producer.
struct ElevationProducer : TileProducer {
    ptr<FrameBuffer> frameBuffer;
    ptr<TileProducer> residualTiles;
    ptr<Texture2D> demTexture, layerTexture, residualTexture;
    ptr<Program> upsample, blend;
    ptr<Texture2DArray> noiseTexture;
    vector<float> noiseAmp;
    int gridMeshSize = 24;
    bool flipDiagonals = false;
    int face = 0;
    float *residualTile = nullptr;
    ptr<Uniform4f> tileWSDFU;
    ptr<UniformSampler> coarseLevelSamplerU;
    ptr<Uniform4f> coarseLevelOSLU;
    ptr<UniformSampler> residualSamplerU;
    ptr<Uniform4f> residualOSHU;
    ptr<UniformSampler> noiseSamplerU;
    ptr<Uniform4f> noiseUVLHU;
    ptr<UniformSampler> blendCoarseLevelSamplerU;
    ptr<Uniform1f> blendScaleU;
    void bind_uniforms();
    bool doCreateTile(int level, int tx, int ty, TileStorage::Slot *data);
};

// The members NormalProducer::doCreateTile and its init's look-ups use (NormalProducer.h).
struct NormalProducer : TileProducer {
    ptr<FrameBuffer> frameBuffer;
    ptr<TileProducer> elevationTiles;
    ptr<Program> normals;
    bool deform = false;
    int gridMeshSize = 24;
    ptr<Uniform3f> tileSDFU;
    ptr<UniformSampler> elevationSamplerU;
    ptr<Uniform4f> elevationOSLU;
    ptr<UniformSampler> normalSamplerU;
    ptr<Uniform4f> normalOSLU;
    ptr<UniformMatrix4f> patchCornersU;
    ptr<UniformMatrix4f> patchVerticalsU;
    ptr<Uniform4f> patchCornerNormsU;
    ptr<UniformMatrix3f> worldToTangentFrameU;
    ptr<UniformMatrix3f> parentToTangentFrameU;
    ptr<Uniform4f> deformU;
    void bind_uniforms();
    bool doCreateTile(int level, int tx, int ty, TileStorage::Slot *data);
};

// The members OrthoProducer::doCreateTile and its init's look-ups use (OrthoProducer.h).
struct OrthoProducer : TileProducer {
    ptr<FrameBuffer> frameBuffer;
    ptr<TileProducer> residualTiles;
    ptr<Texture2D> orthoTexture, residualTexture;
    int face = 0;
    ptr<Program> upsample;
    int channels = 4;
    int maxLevel = -1;
    ptr<Texture2DArray> noiseTexture;
    vec4f rootNoiseColor, noiseColor;
    vector<float> noiseAmp;
    bool noiseHsv = false;
    float scale = 1.0f;
    ptr<Uniform1f> tileWidthU;
    ptr<UniformSampler> coarseLevelSamplerU;
    ptr<Uniform4f> coarseLevelOSLU;
    ptr<UniformSampler> residualSamplerU;
    ptr<Uniform4f> residualOSHU;
    ptr<UniformSampler> noiseSamplerU;
    ptr<Uniform4i> noiseUVLHU;
    ptr<Uniform4f> noiseColorU;
    ptr<Uniform4f> rootNoiseColorU;
    void bind_uniforms();
    bool doCreateTile(int level, int tx, int ty, TileStorage::Slot *data);
};
}  // namespace refgl
"""

_GPU_DRIVERS = r"""
namespace {
// samplers a producer leaves unset read this texture (a single zero texel)
refgl::Texture g_zero_texture;

void reset_samplers(const refgl::UniformEntry *table)
{
    static const float zero[4] = {0, 0, 0, 0};
    g_zero_texture.view.data = zero;
    g_zero_texture.view.w = g_zero_texture.view.h = g_zero_texture.view.layers = 1;
    g_zero_texture.view.comps = 4;
    for (const refgl::UniformEntry *e = table; e->name; ++e) {
        if (e->kind == refgl::U_SAMPLER2D) ((glsl::sampler2D *)e->dst)->t = &g_zero_texture.view;
        if (e->kind == refgl::U_SAMPLER2DARRAY) ((glsl::sampler2DArray *)e->dst)->t = &g_zero_texture.view;
    }
}
}  // namespace

namespace {
struct LayerPlanes {
    refgl::FrameBuffer *fb;
    const float *z, *w;
};
// what the layers drew: z and w into the colour attachment being drawn (COLOR0)
void draw_layer_planes(void *arg)
{
    const LayerPlanes &L = *(const LayerPlanes *)arg;
    std::vector<float> &c = L.fb->color[L.fb->draw_buffer];
    for (int p = 0; p < L.fb->w * L.fb->h; ++p) {
        c[(size_t)p * 4 + 2] = L.z[p];
        c[(size_t)p * 4 + 3] = L.w[p];
    }
}

int elevation_tile(int variant, int W, int level, int tx, int ty, int face, const float *parent_rgba,
                   const float *residual, int residual_width, const float *noise, const float *noise_amp, int n_amp,
                   float root_quad_size, int grid_mesh_size, int flip, int blend_variant, const float *layer_z,
                   const float *layer_w, float *out_rgba)
{
    using namespace refgl;
    if (variant < 0 || variant >= (int)(sizeof(g_upsample) / sizeof(g_upsample[0]))) return 1;
    if (blend_variant >= (int)(sizeof(g_blend) / sizeof(g_blend[0]))) return 1;
    GPUTileStorage storage;
    storage.tileSize = W;
    TileCache cache;
    cache.storage = &storage;
    Texture2DArray parentTex, outTex, noiseTex;
    parentTex.alloc(W, W, 2, 4, false);
    outTex.alloc(W, W, 3, 4, false);
    noiseTex.alloc(W, W, 6, 1, true);
    std::memcpy(noiseTex.store.data(), noise, sizeof(float) * 6 * W * W);
    Texture2D residualTex, demTex;
    residualTex.alloc(W, W, 1, 1, false);
    demTex.alloc(W, W, 1, 4, false);
    FrameBuffer fb;
    fb.init(W);
    Program prog;
    prog.table = g_upsample[variant].table;
    prog.run = g_upsample[variant].run;
    reset_samplers(prog.table);

    ElevationProducer e;
    e.cache = &cache;
    e.rootQuadSize = root_quad_size;
    e.frameBuffer = &fb;
    e.upsample = &prog;
    e.noiseTexture = &noiseTex;
    e.residualTexture = &residualTex;
    e.demTexture = &demTex;
    e.noiseAmp.assign(noise_amp, noise_amp + n_amp);
    e.gridMeshSize = grid_mesh_size;
    e.flipDiagonals = flip != 0;
    e.face = face;
    std::vector<float> residualTile((size_t)W * W);
    e.residualTile = residualTile.data();

    GPUTileStorage::GPUSlot parentSlot, outSlot;
    parentSlot.owner = outSlot.owner = &storage;
    parentSlot.t = &parentTex;
    parentSlot.l = 1;
    outSlot.t = &outTex;
    outSlot.l = 2;
    if (level > 0) {
        std::memcpy(&parentTex.store[(size_t)W * W * 4], parent_rgba, sizeof(float) * W * W * 4);
        e.tiles[std::make_tuple(level - 1, tx / 2, ty / 2)].data = &parentSlot;
    }
    CPUTileStorage<float> rstorage;
    rstorage.tileSize = residual_width;
    TileCache rcache;
    rcache.storage = &rstorage;
    TileProducer rproducer;
    rproducer.cache = &rcache;
    CPUTileStorage<float>::CPUSlot rslot;
    rslot.owner = &rstorage;
    rslot.data = (float *)residual;
    if (residual_width > 0) {
        e.residualTiles = &rproducer;
        if (residual) {
            const int mod = (residual_width - 5) / (W - 5);
            rproducer.tiles[std::make_tuple(level, tx / mod, ty / mod)].data = &rslot;
        }
    }
    Program blendProg;
    LayerPlanes planes{&fb, layer_z, layer_w};
    if (blend_variant >= 0) {
        // the framebuffer's COLOR0 is demTexture, which the blend program reads
        demTex.view.data = fb.color[0].data();
        blendProg.table = g_blend[blend_variant].table;
        blendProg.run = g_blend[blend_variant].run;
        reset_samplers(blendProg.table);
        e.blend = &blendProg;
        e.layer_hook = draw_layer_planes;
        e.layer_arg = &planes;
    }
    e.bind_uniforms();
    if (!e.doCreateTile(level, tx, ty, &outSlot)) return 2;
    std::memcpy(out_rgba, &outTex.store[(size_t)2 * W * W * 4], sizeof(float) * W * W * 4);
    return 0;
}
}  // namespace

// One elevation tile through ElevationProducer::doCreateTile and the upsample shader
// `variant`: parent_rgba the parent slot's four channels (zf, zc, zm, 0; W*W*4, level > 0),
// residual the residual producer's tile (residual_width^2; NULL: the producer has no
// tile there; residual_width 0: no residual producer), noise the six noise layers
// (W*W each, as the R16F texture holds them), noise_amp the per-level amplitudes.
// out_rgba: the produced slot, W*W*4.  Returns 0.
extern "C" int ref_gl_elevation_tile(int variant, int W, int level, int tx, int ty, int face,
                                     const float *parent_rgba, const float *residual, int residual_width,
                                     const float *noise, const float *noise_amp, int n_amp, float root_quad_size,
                                     int grid_mesh_size, int flip, float *out_rgba)
{
    return elevation_tile(variant, W, level, tx, ty, face, parent_rgba, residual, residual_width, noise, noise_amp,
                          n_amp, root_quad_size, grid_mesh_size, flip, -1, nullptr, nullptr, out_rgba);
}

// The same tile by a producer with layers: the layers draw layer_z and layer_w (W*W
// each) into the z and w channels, then doCreateTile draws the blend program
// `blend_variant` into COLOR1 and copies that into the slot.
extern "C" int ref_gl_elevation_tile_layers(int variant, int blend_variant, int W, int level, int tx, int ty,
                                            int face, const float *parent_rgba, const float *residual,
                                            int residual_width, const float *noise, const float *noise_amp,
                                            int n_amp, float root_quad_size, int grid_mesh_size, int flip,
                                            const float *layer_z, const float *layer_w, float *out_rgba)
{
    if (blend_variant < 0) return 1;
    return elevation_tile(variant, W, level, tx, ty, face, parent_rgba, residual, residual_width, noise, noise_amp,
                          n_amp, root_quad_size, grid_mesh_size, flip, blend_variant, layer_z, layer_w, out_rgba);
}

// One ortho tile through OrthoProducer::doCreateTile and the upsample shader `variant`:
// parent the parent slot's RGBA8 texels (W*W*4 bytes; level > 0), residual the residual
// producer's RGBA8 tile (W*W*4 bytes; NULL: the producer has no tile there), noise
// createOrthoNoise's six RGBA8 layers, noise_amp the per-level amplitudes, the colours,
// the HSV flag and the residual scale as OrthoProducer::init takes them.  out: what the
// fragment shader writes (W*W*4 floats, result / 255), before the RGBA8 framebuffer
// rounds it.  Returns 0.
extern "C" int ref_gl_ortho_tile_channels(int variant, int W, int level, int tx, int ty, int face,
                                          const unsigned char *parent, const unsigned char *residual, int channels,
                                          const unsigned char *noise, const float *noise_amp, int n_amp,
                                          const float *root_color, const float *noise_color, int hsv, float scale,
                                          float *out);
extern "C" int ref_gl_ortho_tile(int variant, int W, int level, int tx, int ty, int face, const unsigned char *parent,
                                 const unsigned char *residual, const unsigned char *noise, const float *noise_amp,
                                 int n_amp, const float *root_color, const float *noise_color, int hsv, float scale,
                                 float *out)
{
    return ref_gl_ortho_tile_channels(variant, W, level, tx, ty, face, parent, residual, 4, noise, noise_amp, n_amp,
                                      root_color, noise_color, hsv, scale, out);
}

// The same with a residual producer of `channels` channels (residual: W*W*channels bytes),
// which doCreateTile uploads as RED, RG, RGB or RGBA.
extern "C" int ref_gl_ortho_tile_channels(int variant, int W, int level, int tx, int ty, int face,
                                          const unsigned char *parent, const unsigned char *residual, int channels,
                                          const unsigned char *noise, const float *noise_amp, int n_amp,
                                          const float *root_color, const float *noise_color, int hsv, float scale,
                                          float *out)
{
    using namespace refgl;
    if (variant < 0 || variant >= (int)(sizeof(g_ortho) / sizeof(g_ortho[0]))) return 1;
    GPUTileStorage storage;
    storage.tileSize = W;
    TileCache cache;
    cache.storage = &storage;
    Texture2DArray parentTex, outTex, noiseTex;
    parentTex.alloc(W, W, 2, 4, false);
    parentTex.format = RGBA8;
    outTex.alloc(W, W, 3, 4, false);   // float: the shader's output is returned unrounded
    noiseTex.alloc(W, W, 6, 4, true);
    noiseTex.format = RGBA8;
    for (size_t k = 0; k < (size_t)6 * W * W * 4; ++k) noiseTex.store[k] = (float)noise[k] / 255.0f;
    Texture2D residualTex, orthoTex;
    residualTex.alloc(W, W, 1, 4, false);
    residualTex.format = RGBA8;
    FrameBuffer fb;
    fb.init(W);
    Program prog;
    prog.table = g_ortho[variant].table;
    prog.run = g_ortho[variant].run;
    reset_samplers(prog.table);

    OrthoProducer o;
    o.cache = &cache;
    o.frameBuffer = &fb;
    o.upsample = &prog;
    o.noiseTexture = &noiseTex;
    o.residualTexture = &residualTex;
    o.orthoTexture = &orthoTex;
    o.rootNoiseColor = vec4f(root_color[0], root_color[1], root_color[2], root_color[3]);
    o.noiseColor = vec4f(noise_color[0], noise_color[1], noise_color[2], noise_color[3]);
    o.noiseAmp.assign(noise_amp, noise_amp + n_amp);
    o.noiseHsv = hsv != 0;
    o.scale = scale;
    o.face = face;
    o.channels = channels;
    GPUTileStorage::GPUSlot parentSlot, outSlot;
    parentSlot.owner = outSlot.owner = &storage;
    parentSlot.t = &parentTex;
    parentSlot.l = 1;
    outSlot.t = &outTex;
    outSlot.l = 2;
    if (level > 0) {
        for (size_t k = 0; k < (size_t)W * W * 4; ++k) parentTex.store[(size_t)W * W * 4 + k] = (float)parent[k] / 255.0f;
        o.tiles[std::make_tuple(level - 1, tx / 2, ty / 2)].data = &parentSlot;
    }
    CPUTileStorage<unsigned char> rstorage;
    rstorage.tileSize = W;
    TileCache rcache;
    rcache.storage = &rstorage;
    TileProducer rproducer;
    rproducer.cache = &rcache;
    CPUTileStorage<unsigned char>::CPUSlot rslot;
    rslot.owner = &rstorage;
    rslot.data = (unsigned char *)residual;
    if (residual) rproducer.tiles[std::make_tuple(level, tx, ty)].data = &rslot;
    o.residualTiles = &rproducer;
    o.bind_uniforms();
    if (!o.doCreateTile(level, tx, ty, &outSlot)) return 2;
    std::memcpy(out, &outTex.store[(size_t)2 * W * W * 4], sizeof(float) * W * W * 4);
    return 0;
}

// The uniforms NormalProducer::doCreateTile sets for a spherical tile (demo normal
// shader, RGBA32F storage), as the producer builds them (row-major): patchCorners[16],
// patchVerticals[16], patchCornerNorms[4], worldToTangentFrame[9],
// parentToTangentFrame[9] (level > 0), deform[4].  Returns 0.
extern "C" int ref_gl_normal_tile(int variant, int W, int level, int tx, int ty, const float *elev_rgba, int format,
                                  const float *parent, float root_quad_size, int grid_mesh_size, int deform,
                                  float *out);
extern "C" int ref_sphere_uniforms(int W, int level, int tx, int ty, float root_quad_size, float *out58)
{
    std::vector<float> elev((size_t)W * W * 4, 0.0f), parent((size_t)(W - 4) * (W - 4) * 4, 0.0f),
        out((size_t)(W - 4) * (W - 4) * 4);
    const int rc = ref_gl_normal_tile(2, W, level, tx, ty, elev.data(), 0, parent.data(), root_quad_size, 24, 1,
                                      out.data());
    if (rc) return rc;
    struct Want {
        const char *name;
        int rows, cols;
    };
    static const Want want[] = {{"patchCorners", 4, 4}, {"patchVerticals", 4, 4}, {"patchCornerNorms", 1, 4},
                                {"worldToTangentFrame", 3, 3}, {"parentToTangentFrame", 3, 3}, {"deform", 1, 4}};
    float *o = out58;
    for (const Want &w : want) {
        const refgl::UniformEntry *e = g_normal[2].table;
        while (e->name && std::string(e->name) != w.name) ++e;
        if (!e->name) return 3;
        const float *d = (const float *)e->dst;   // a matrix is column-major in the shader
        for (int r = 0; r < w.rows; ++r)
            for (int c = 0; c < w.cols; ++c) *o++ = w.rows == 1 ? d[c] : d[c * w.rows + r];
    }
    return 0;
}

namespace {
std::vector<refgl::FrameBuffer::Drawn> g_drawn;

// a curve of n points (xy: 2n doubles), their curvilinear coordinates (or 0) and width
refgl::Curve make_curve(const double *xy, const float *s, int n, float width)
{
    refgl::Curve c;
    for (int k = 0; k < n; ++k) {
        c.points.push_back(refgl::vec2d(xy[2 * k], xy[2 * k + 1]));
        c.s.push_back(s ? s[k] : 0.0f);
    }
    c.width = width;
    return c;
}
}  // namespace

// One road through the lines of RoadElevationLayer::doCreateTile that place it on tile
// q = (x, y, size) of a tileSize-wide storage with the given border (scale, tile
// offset, BASEWIDTH / TOTALWIDTH, the drawCurveAltitude call) and
// ElevationGraphLayer::drawCurveAltitude: the road's n points (xy, 2n doubles), their
// curvilinear coordinates s (the altitude profile is s itself), its width, caps at the
// start / end.  Returns the number of meshes drawn (ref_drawn_mesh reads them), or -1;
// scale_out: the layer's scale.
extern "C" int ref_road_meshes(double qx, double qy, double qz, int tile_size, int border, const double *xy,
                               const float *s, int n, float width, int cap_start, int cap_end, float *scale_out)
{
    using namespace refgl;
    if (n < 2) return -1;
    Curve c = make_curve(xy, s, n, width);
    ElevationCurveData data;
    FrameBuffer fb;
    Program prog;
    Mesh<vec4f, unsigned int> mesh;
    RoadElevationLayer layer;
    layer.tileSize = tile_size;
    layer.tileBorder = border;
    layer.layerProgram = &prog;
    layer.meshuv = &mesh;
    c.cap_start = cap_start != 0;
    c.cap_end = cap_end != 0;
    layer.draw_road(vec3d(qx, qy, qz), &c, &data, &fb, scale_out);
    g_drawn = fb.drawn;
    return (int)g_drawn.size();
}

// ElevationGraphLayer::drawCurveAltitude called directly (flat tile): tile coordinates
// (centre x, centre y, factor), the curve, and the function's width, nwidth,
// stepLength and caps arguments.  Returns the number of meshes drawn, or -1.
extern "C" int ref_curve_altitude(double cx, double cy, double factor, const double *xy, const float *s, int n,
                                  float width, float nwidth, float step, int cap_start, int cap_end)
{
    using namespace refgl;
    if (n < 2) return -1;
    Curve c = make_curve(xy, s, n, width);
    ElevationCurveData data;
    FrameBuffer fb;
    Program prog;
    Mesh<vec4f, unsigned int> mesh;
    ElevationGraphLayer layer;
    c.cap_start = cap_start != 0;
    c.cap_end = cap_end != 0;
    layer.drawCurveAltitude(vec3d(cx, cy, factor), &c, &data, width, nwidth, step, true, &fb, &prog, mesh, nullptr,
                            nullptr, nullptr, nullptr);
    g_drawn = fb.drawn;
    return (int)g_drawn.size();
}

// GraphLayer::drawCurve(tileCoords, p, part, ...) on a flat tile: the curve's points and
// width, part = (offset a, offset b, w at a, w at b).  Returns the number of meshes drawn.
extern "C" int ref_curve_part(double cx, double cy, double factor, const double *xy, int n, float width,
                              const float *part)
{
    using namespace refgl;
    if (n < 2) return -1;
    Curve c = make_curve(xy, nullptr, n, width);
    FrameBuffer fb;
    Program prog;
    Mesh<vec4f, unsigned int> mesh;
    GraphLayer layer;
    layer.drawCurve(vec3d(cx, cy, factor), &c, vec4f(part[0], part[1], part[2], part[3]), &fb, &prog, mesh, nullptr,
                    nullptr, nullptr, nullptr);
    g_drawn = fb.drawn;
    return (int)g_drawn.size();
}

namespace {
struct WaterDraws {
    int river = 0;
    float depth = 0.0f, color[4] = {0, 0, 0, 0}, offset[3] = {0, 0, 0}, fill_offset[3] = {0, 0, 0};
};
void water_snapshot(void *arg, refgl::FrameBuffer::Drawn &d)
{
    const WaterDraws &w = *(const WaterDraws *)arg;
    d.extra = {(float)w.river, w.depth, w.color[0], w.color[1], w.color[2], w.color[3]};
}
std::vector<std::vector<refgl::vec2d> > g_contours;
}  // namespace

// WaterElevationLayer::doCreateTile on tile q = (x, y, size) at `level` of a
// tile_size-wide storage, over a graph of n_curves curves -- curve k has info[6k..6k+5]
// = (points, type, parent: 1 itself / 0 none, area1: 1 set / 0 none, cap at start, cap
// at end), its points in xy (2 doubles each, curve after curve), their curvilinear
// coordinates in s, its width -- and n_areas areas, area a listing area_info (its curve
// count, then (curve index, orientation) pairs).  The draws are read by
// ref_drawn_mesh and ref_water_draw, the area contours by ref_water_contour.  Returns
// the number of draws, or -1.
extern "C" int ref_water_layer(double qx, double qy, double qz, int tile_size, int level, int n_curves,
                               const int *info, const double *xy, const float *s, const float *widths, int n_areas,
                               const int *area_info)
{
    using namespace refgl;
    std::vector<Curve> curves(n_curves);
    std::vector<Area> areas(n_areas);
    Graph g;
    for (int k = 0, at = 0; k < n_curves; ++k) {
        const int *c = info + 6 * k;
        for (int i = 0; i < c[0]; ++i, ++at) {
            curves[k].points.push_back(vec2d(xy[2 * at], xy[2 * at + 1]));
            curves[k].s.push_back(s[at]);
        }
        curves[k].type = c[1];
        curves[k].parent = c[2] ? &curves[k] : nullptr;
        curves[k].area1 = c[3] && n_areas ? &areas[0] : nullptr;
        curves[k].cap_start = c[4] != 0;
        curves[k].cap_end = c[5] != 0;
        curves[k].width = widths[k];
        g.curves.push_back(&curves[k]);
    }
    for (int a = 0, at = 0; a < n_areas; ++a) {
        const int n = area_info[at++];
        for (int j = 0; j < n; ++j, at += 2) {
            if (area_info[at] < 0 || area_info[at] >= n_curves) return -1;
            areas[a].curves.push_back(std::make_pair(&curves[area_info[at]], area_info[at + 1]));
        }
        g.areas.push_back(&areas[a]);
    }
    ObjectTileStorage::ObjectSlot graphSlot;
    graphSlot.data = ptr<GraphObject>(&g);
    TileProducer graphProducer;
    graphProducer.tiles[std::make_tuple(level, 0, 0)].data = &graphSlot;
    FrameBuffer fb;
    SceneManager::current = &fb;
    WaterDraws w;
    fb.on_draw = water_snapshot;
    fb.on_draw_arg = &w;
    Program layerProgram, fillProg;
    Mesh<vec2f, unsigned int> mesh;
    Mesh<vec4f, unsigned int> meshuv;
    Tesselator tess;
    Uniform tileOffsetU{U_VEC3, w.offset}, riverU{U_INT, &w.river}, fillOffsetU{U_VEC3, w.fill_offset},
        depthU{U_FLOAT, &w.depth}, colorU{U_VEC4, w.color};
    WaterElevationLayer layer;
    layer.graphProducer = &graphProducer;
    layer.layerProgram = &layerProgram;
    layer.fillProg = &fillProg;
    layer.mesh = &mesh;
    layer.meshuv = &meshuv;
    layer.tess = &tess;
    layer.tileOffsetU = &tileOffsetU;
    layer.riverU = &riverU;
    layer.fillOffsetU = &fillOffsetU;
    layer.depthU = &depthU;
    layer.colorU = &colorU;
    layer.q = vec3d(qx, qy, qz);
    layer.tileSize = tile_size;
    layer.doCreateTile(level, 0, 0, nullptr);
    SceneManager::current = nullptr;
    for (FrameBuffer::Drawn &d : fb.drawn) d.extra.push_back(d.program == &fillProg ? 0.0f : 1.0f);
    g_drawn = fb.drawn;
    g_contours = tess.contours;
    return (int)g_drawn.size();
}

namespace {
// a graph of curves (ref_water_layer's encoding) for the layers' harnesses
void build_graph(int n_curves, const int *info, const double *xy, const float *s, const float *widths,
                 std::vector<refgl::Curve> &curves, refgl::Graph &g)
{
    curves.assign(n_curves, refgl::Curve());
    for (int k = 0, at = 0; k < n_curves; ++k) {
        const int *c = info + 6 * k;
        for (int i = 0; i < c[0]; ++i, ++at) {
            curves[k].points.push_back(refgl::vec2d(xy[2 * at], xy[2 * at + 1]));
            curves[k].s.push_back(s[at]);
        }
        curves[k].type = c[1];
        curves[k].parent = c[2] ? &curves[k] : nullptr;
        curves[k].cap_start = c[4] != 0;
        curves[k].cap_end = c[5] != 0;
        curves[k].width = widths[k];
        g.curves.push_back(&curves[k]);
    }
}
}  // namespace

// RoadElevationLayer::doCreateTile on tile q = (x, y, size) at `level`, over a graph of
// curves encoded as for ref_water_layer (type 0 ROAD), after ElevationProducer's
// setDepthTest(true, LESS).  The draws are read by ref_drawn_mesh and ref_water_draw.
// Returns their number.
extern "C" int ref_road_layer(double qx, double qy, double qz, int tile_size, int level, int n_curves,
                              const int *info, const double *xy, const float *s, const float *widths)
{
    using namespace refgl;
    std::vector<Curve> curves;
    Graph g;
    build_graph(n_curves, info, xy, s, widths, curves, g);
    ObjectTileStorage::ObjectSlot graphSlot;
    graphSlot.data = ptr<GraphObject>(&g);
    TileProducer graphProducer;
    graphProducer.tiles[std::make_tuple(level, 0, 0)].data = &graphSlot;
    FrameBuffer fb;
    fb.setDepthTest(true, LESS);
    SceneManager::current = &fb;
    WaterDraws w;
    fb.on_draw = water_snapshot;
    fb.on_draw_arg = &w;
    Program layerProgram;
    Mesh<vec4f, unsigned int> meshuv;
    Uniform tileOffsetU{U_VEC3, w.offset};
    RoadElevationLayer layer;
    layer.graphProducer = &graphProducer;
    layer.layerProgram = &layerProgram;
    layer.meshuv = &meshuv;
    layer.tileOffsetU = &tileOffsetU;
    layer.q = vec3d(qx, qy, qz);
    layer.tileSize = tile_size;
    layer.doCreateTile(level, 0, 0, nullptr);
    SceneManager::current = nullptr;
    for (FrameBuffer::Drawn &d : fb.drawn) d.extra.push_back(1.0f);
    g_drawn = fb.drawn;
    return (int)g_drawn.size();
}

// Draw k of the last ref_water_layer: state[0..7] = program (0 fill, 1 layer), river,
// depth test on, depth function (0 LESS, 1 ALWAYS, 2 NOTEQUAL), depth mask, colour mask
// of z, colour mask of w, mode; uniforms[0..4] = fill depth and colour.
extern "C" int ref_water_draw(int k, int *state, float *uniforms)
{
    if (k < 0 || k >= (int)g_drawn.size()) return 1;
    const refgl::FrameBuffer::Drawn &d = g_drawn[k];
    state[0] = (int)d.extra[6];
    state[1] = (int)d.extra[0];
    state[2] = d.depth_test;
    state[3] = d.depth_func;
    state[4] = d.depth_mask;
    state[5] = d.color_mask[2];
    state[6] = d.color_mask[3];
    state[7] = d.mode;
    for (int i = 0; i < 5; ++i) uniforms[i] = d.extra[1 + i];
    return 0;
}

// contour k of the areas the last ref_water_layer filled, in clip coordinates: its
// vertex count, and its vertices (2 doubles each) when `out` is given
extern "C" int ref_water_contour(int k, double *out)
{
    if (k < 0 || k >= (int)g_contours.size()) return -1;
    if (out)
        for (size_t i = 0; i < g_contours[k].size(); ++i) {
            out[2 * i] = g_contours[k][i].x;
            out[2 * i + 1] = g_contours[k][i].y;
        }
    return (int)g_contours[k].size();
}

// Mesh k of the last ref_road_meshes / ref_curve_altitude / ref_curve_part: its mode (0 triangles, 1 strip), vertex and index
// counts, and (when the buffers are given) its (x, y, z, w) vertices and indices.
extern "C" int ref_drawn_mesh(int k, int *mode, int *n_vertices, int *n_indices, float *vertices, unsigned *indices)
{
    if (k < 0 || k >= (int)g_drawn.size()) return 1;
    const refgl::FrameBuffer::Drawn &d = g_drawn[k];
    *mode = d.mode;
    *n_vertices = (int)d.vertices.size() / 4;
    *n_indices = (int)d.indices.size();
    if (vertices) std::memcpy(vertices, d.vertices.data(), d.vertices.size() * sizeof(float));
    if (indices) std::memcpy(indices, d.indices.data(), d.indices.size() * sizeof(unsigned));
    return 0;
}

// One fragment of the layer program `shader` (LAYER_SHADERS order) at the interpolated
// varying st: uniforms river (water programs), depth and color (fill program); data
// (4 floats) and the fragment depth it writes.  Returns 0.
extern "C" int ref_gl_layer_fragment(int shader, int river, float depth, const float *color, float st_x, float st_y,
                                     float *data, float *frag_depth)
{
    if (shader < 0 || shader >= (int)(sizeof(g_layer) / sizeof(g_layer[0]))) return 1;
    for (const refgl::UniformEntry *e = g_layer[shader].table; e->name; ++e) {
        const std::string n = e->name;
        if (n == "river") *(int *)e->dst = river;
        if (n == "depth") *(float *)e->dst = depth;
        if (n == "color") std::memcpy(e->dst, color, 4 * sizeof(float));
        if (n == "tileOffset") {   // both layers set (0, 0, 1): vertices are in clip coordinates
            static const float identity[3] = {0.0f, 0.0f, 1.0f};
            std::memcpy(e->dst, identity, sizeof(identity));
        }
    }
    g_layer[shader].fragment(st_x, st_y, data, frag_depth);
    return 0;
}

// One normal tile through NormalProducer::doCreateTile and the normal shader `variant`:
// elev_rgba the elevation slot (W*W*4), format 0-3 the normal storage's (RGBA32F, RGBA8,
// RG32F, RG8), parent the parent normal slot (Wn*Wn*components, Wn = W - 4; level > 0;
// NULL: zeros), deform the spherical flag.  out: the produced slot, Wn*Wn*components.  Returns 0.
extern "C" int ref_gl_normal_tile(int variant, int W, int level, int tx, int ty, const float *elev_rgba, int format,
                                  const float *parent, float root_quad_size, int grid_mesh_size, int deform,
                                  float *out)
{
    using namespace refgl;
    if (variant < 0 || variant >= (int)(sizeof(g_normal) / sizeof(g_normal[0])) || format < 0 || format > 3) return 1;
    static const TextureInternalFormat formats[4] = {RGBA32F, RGBA8, RG32F, RG8};
    const int Wn = W - 4, comps = format < 2 ? 4 : 2;
    GPUTileStorage estorage, nstorage;
    estorage.tileSize = W;
    nstorage.tileSize = Wn;
    TileCache ecache, ncache;
    ecache.storage = &estorage;
    ncache.storage = &nstorage;
    Texture2DArray elevTex, normTex;
    elevTex.alloc(W, W, 2, 4, false);
    normTex.alloc(Wn, Wn, 2, comps, false);
    normTex.format = formats[format];
    nstorage.texture0 = &normTex;
    FrameBuffer fb;
    fb.init(Wn);
    Program prog;
    prog.table = g_normal[variant].table;
    prog.run = g_normal[variant].run;
    reset_samplers(prog.table);

    TileProducer elevations;
    elevations.cache = &ecache;
    elevations.border = 2;
    GPUTileStorage::GPUSlot eslot, pslot, oslot;
    eslot.owner = &estorage;
    eslot.t = &elevTex;
    eslot.l = 1;
    std::memcpy(&elevTex.store[(size_t)W * W * 4], elev_rgba, sizeof(float) * W * W * 4);
    elevations.tiles[std::make_tuple(level, tx, ty)].data = &eslot;

    NormalProducer n;
    n.cache = &ncache;
    n.rootQuadSize = root_quad_size;
    n.frameBuffer = &fb;
    n.elevationTiles = &elevations;
    n.normals = &prog;
    n.deform = deform != 0;
    n.gridMeshSize = grid_mesh_size;
    pslot.owner = oslot.owner = &nstorage;
    pslot.t = oslot.t = &normTex;
    pslot.l = 0;
    oslot.l = 1;
    if (level > 0) {  // doCreateTile asserts the parent normal tile is in the cache
        if (parent) std::memcpy(normTex.store.data(), parent, sizeof(float) * Wn * Wn * comps);
        n.tiles[std::make_tuple(level - 1, tx / 2, ty / 2)].data = &pslot;
    }
    n.bind_uniforms();
    if (!n.doCreateTile(level, tx, ty, &oslot)) return 2;
    std::memcpy(out, &normTex.store[(size_t)Wn * Wn * comps], sizeof(float) * Wn * Wn * comps);
    return 0;
}
"""


RESIDUAL_CPP = "src/terrain/sources/proland/dem/ResidualProducer.cpp"
ORTHO_CPU_CPP = "src/terrain/sources/proland/ortho/OrthoCPUProducer.cpp"
MFS_CPP = "src/core/sources/proland/util/mfs.cpp"

_RESIDUAL_PRELUDE = r"""
#include <pthread.h>
#include <sys/types.h>
#include <cstdio>
#include <string>
#include "ork_gl.h"
#include "tiffio.h"
#include "proland/util/mfs.h"

namespace refgl {
using namespace std;   // as ResidualProducer.cpp

// Ork's file helpers the functions call: fopen into a FILE **, a 64-bit fseek
inline void fopen(FILE **f, const char *name, const char *mode) { *f = std::fopen(name, mode); }
inline int fseek64(FILE *f, long long off, int whence) { return fseeko(f, (off_t)off, whence); }

// The members the extracted functions use (ResidualProducer.h).
struct ResidualProducer : TileProducer {
    std::string name;
    int tileSize = 0, rootLevel = 0, deltaLevel = 0, rootTx = 0, rootTy = 0, minLevel = 0, maxLevel = 0;
    float scale = 1.0f;
    unsigned int header = 0;
    unsigned int *offsets = nullptr;
    void *mutex = nullptr;
    FILE *tileFile = nullptr;
    std::vector<ptr<ResidualProducer> > producers;
    static void *key;
    ~ResidualProducer() { delete[] offsets; }
    void init(ptr<TileCache> cache, const char *name, int deltaLevel = 0, float zscale = 1.0);
    bool hasTile(int level, int tx, int ty);
    bool doCreateTile(int level, int tx, int ty, TileStorage::Slot *data);
    void upsample(int level, int tx, int ty, float *parentTile, float *result);
    int getTileSize(int level);
    int getTileId(int level, int tx, int ty);
    void readTile(int level, int tx, int ty, unsigned char *compressedData, unsigned char *uncompressedData,
                  float *tile, float *result);
};

// The members OrthoCPUProducer's extracted functions use (OrthoCPUProducer.h).
struct OrthoCPUProducer : TileProducer {
    std::string name;
    int maxLevel = 0, tileSize = 0, channels = 0, border = 2;
    bool dxt = false;
    long long header = 0;
    long long *offsets = nullptr;
    void *mutex = nullptr;
    FILE *tileFile = nullptr;
    static void *key;
    ~OrthoCPUProducer() { delete[] offsets; }
    void init(ptr<TileCache> cache, const char *name);
    bool hasTile(int level, int tx, int ty);
    bool doCreateTile(int level, int tx, int ty, TileStorage::Slot *data);
    int getTileId(int level, int tx, int ty);
};
"""

_RESIDUAL_DRIVER = r"""
}  // namespace refgl

// One residual tile through ResidualProducer::init (the .dat at `path`, deltaLevel,
// zscale), hasTile and doCreateTile, into a one-channel CPU slot of tile_width^2 floats
// (the tile written from its lower left corner at pitch tile_width).  has: hasTile.
// Returns 0, or 1 when the file does not open as a pyramid.
extern "C" int ref_residual_tile(const char *path, int delta, float zscale, int tile_width, int level, int tx, int ty,
                                 float *out, int *has)
{
    using namespace refgl;
    CPUTileStorage<float> storage;
    storage.tileSize = tile_width;
    TileCache cache;
    cache.storage = &storage;
    ResidualProducer r;
    r.init(&cache, path, delta, zscale);
    if (r.maxLevel < 0 || r.tileSize + 5 != tile_width) return 1;
    *has = r.hasTile(level, tx, ty) ? 1 : 0;
    CPUTileStorage<float>::CPUSlot slot;
    slot.owner = &storage;
    slot.data = out;
    r.doCreateTile(level, tx, ty, &slot);
    return 0;
}

// One tile of an ortho pyramid through OrthoCPUProducer::init, hasTile and doCreateTile
// into a CPU slot of width^2 * channels bytes (`capacity` at least that).  info: the
// pyramid's (maxLevel, tileSize, channels, border, width).  has: hasTile.  Returns 0,
// 1 when the file does not open, 2 when `out` is too small.
extern "C" int ref_ortho_dat_tile(const char *path, int level, int tx, int ty, unsigned char *out, int capacity,
                                  int *info, int *has)
{
    using namespace refgl;
    CPUTileStorage<unsigned char> storage;
    TileCache cache;
    cache.storage = &storage;
    OrthoCPUProducer o;
    o.init(&cache, path);
    if (o.maxLevel < 0) return 1;
    const int width = o.tileSize + 2 * o.border;
    info[0] = o.maxLevel;
    info[1] = o.tileSize;
    info[2] = o.channels;
    info[3] = o.border;
    info[4] = width;
    if (capacity < width * width * o.channels) return 2;
    storage.tileSize = width;
    storage.channels = o.channels;
    *has = o.hasTile(level, tx, ty) ? 1 : 0;
    CPUTileStorage<unsigned char>::CPUSlot slot;
    slot.owner = &storage;
    slot.data = out;
    slot.size = width * width * o.channels;
    if (*has) o.doCreateTile(level, tx, ty, &slot);
    return 0;
}
"""


def generate_residual(root):
    """oracle/_ref/gen/ref_residual.cpp: ResidualProducer's file reading, tile ids,
    delta chain and upsample as written (with mfs.cpp compiled beside it and the
    libtiff stand-in)."""
    res = _read(root, RESIDUAL_CPP)
    src = ["// generated by oracle/ref_build.py from the reference's sources\n", _RESIDUAL_PRELUDE]
    block, line = extract_block(res, "#define MAX_TILE_SIZE", "#define MAX_TILE_SIZE")
    src.append("// %s:%d\n%s" % (RESIDUAL_CPP, line, block))
    block, line = extract_block(res, "void *ResidualProducer::key = NULL;", "void *ResidualProducer::key = NULL;")
    src.append("// :%d\n%s" % (line, block))
    for sig in (r"void\s+residualDelete\s*\(", r"void\s+ResidualProducer::init\s*\(\s*ptr<TileCache>",
                r"bool\s+ResidualProducer::hasTile\s*\(", r"bool\s+ResidualProducer::doCreateTile\s*\(",
                r"int\s+ResidualProducer::getTileSize\s*\(", r"int\s+ResidualProducer::getTileId\s*\(",
                r"void\s+ResidualProducer::readTile\s*\(", r"void\s+ResidualProducer::upsample\s*\("):
        body, line = extract_function(res, sig)
        src.append("// :%d\n%s" % (line, body))
    ortho = _read(root, ORTHO_CPU_CPP)
    block, line = extract_block(ortho, "#define MAX_TILE_SIZE", "#define MAX_TILE_SIZE")
    src.append("#undef MAX_TILE_SIZE\n// %s:%d\n%s" % (ORTHO_CPU_CPP, line, block))
    block, line = extract_block(ortho, "void *OrthoCPUProducer::key = NULL;", "void *OrthoCPUProducer::key = NULL;")
    src.append("// :%d\n%s" % (line, block))
    for sig in (r"void\s+orthoCPUDelete\s*\(", r"void\s+OrthoCPUProducer::init\s*\(\s*ptr<TileCache>",
                r"bool\s+OrthoCPUProducer::hasTile\s*\(", r"bool\s+OrthoCPUProducer::doCreateTile\s*\(",
                r"int\s+OrthoCPUProducer::getTileId\s*\("):
        body, line = extract_function(ortho, sig)
        src.append("// :%d\n%s" % (line, body))
    src.append(_RESIDUAL_DRIVER)
    os.makedirs(GEN_DIR, exist_ok=True)
    path = os.path.join(GEN_DIR, "ref_residual.cpp")
    with open(path, "w") as f:
        f.write("".join(src))
    return path


CACHE_CPP = "src/core/sources/proland/producer/TileCache.cpp"
STORAGE_CPP = "src/core/sources/proland/producer/TileStorage.cpp"

STORAGE_SIGS = [r"^TileStorage::Slot::Slot\(", r"^TileStorage::Slot::~Slot\(",
                r"TileStorage \*TileStorage::Slot::getOwner\(", r"void TileStorage::Slot::lock\(",
                r"^TileStorage::TileStorage\(\)", r"void TileStorage::init\(", r"^TileStorage::~TileStorage\(",
                r"TileStorage::Slot \*TileStorage::newSlot\(", r"void TileStorage::deleteSlot\(",
                r"int TileStorage::getTileSize\(", r"int TileStorage::getCapacity\(",
                r"int TileStorage::getFreeSlots\("]
CACHE_SIGS = [r"^TileCache::Tile::Tile\(", r"^TileCache::Tile::~Tile\(",
              r"TileStorage::Slot \*TileCache::Tile::getData\(",
              r"TileCache::Tile::Id TileCache::Tile::getId\(\) const",
              r"TileCache::Tile::TId TileCache::Tile::getTId\(\) const",
              r"TileCache::Tile::Id TileCache::Tile::getId\(int", r"TileCache::Tile::TId TileCache::Tile::getTId\(int",
              r"^TileCache::TileCache\(\)", r"void TileCache::init\(", r"^TileCache::~TileCache\(",
              r"ptr<TileStorage> TileCache::getStorage\(", r"ptr<Scheduler> TileCache::getScheduler\(",
              r"int TileCache::getUsedTiles\(",
              r"int TileCache::getUnusedTiles\(", r"TileCache::Tile\* TileCache::findTile\(",
              r"TileCache::Tile\* TileCache::getTile\(", r"ptr<Task> TileCache::prefetchTile\(",
              r"int TileCache::putTile\(", r"void TileCache::invalidateTiles\(",
              r"void TileCache::invalidateTile\(", r"void TileCache::createTileTaskDeleted\("]

_DECL_STORAGE = r"""
// The declaration of TileStorage.h the extracted functions define.
struct TileStorage : Object {
    struct Slot {
        std::pair<int, std::pair<int, std::pair<int, int> > > id;
        void *producerTask;
        int index = -1;   // the harness's name for the slot
        Slot(TileStorage *owner);
        virtual ~Slot();
        TileStorage *getOwner();
        void lock(bool lock);
    private:
        TileStorage *owner;
        void *mutex;
    };
    TileStorage(int tileSize, int capacity);
    TileStorage();
    virtual ~TileStorage();
    Slot *newSlot();
    void deleteSlot(Slot *t);
    int getTileSize();
    int getCapacity();
    int getFreeSlots();
    void init(int tileSize, int capacity);
    int tileSize, capacity;
    std::list<Slot *> freeSlots;
};

"""

_DECL_CACHE = r"""
// The declaration of TileCache.h the extracted functions define.
struct TileCache : Object {
    class Tile {
    public:
        typedef std::pair<int, std::pair<int, int> > Id;
        typedef std::pair<int, Id> TId;
        const int producerId;
        const int level;
        const int tx;
        const int ty;
        const ptr<Task> task;
        Tile(int producerId, int level, int tx, int ty, ptr<Task> task, TileStorage::Slot *data);
        ~Tile();
        TileStorage::Slot *getData(bool check = true);
        Id getId() const;
        TId getTId() const;
        static Id getId(int level, int tx, int ty);
        static TId getTId(int producerId, int level, int tx, int ty);
        TileStorage::Slot *data;
        int users;
    };
    TileCache(ptr<TileStorage> storage, std::string name, ptr<Scheduler> scheduler = ptr<Scheduler>());
    TileCache();
    virtual ~TileCache();
    ptr<TileStorage> getStorage();
    ptr<Scheduler> getScheduler();
    int getUsedTiles();
    int getUnusedTiles();
    Tile *findTile(int producerId, int level, int tx, int ty, bool includeCache = false);
    Tile *getTile(int producerId, int level, int tx, int ty, unsigned int deadline, int *users = NULL);
    ptr<Task> prefetchTile(int producerId, int level, int tx, int ty);
    int putTile(Tile *t);
    void invalidateTiles(int producerId);
    void invalidateTile(int producerId, int level, int tx, int ty);
    void init(ptr<TileStorage> storage, std::string name, ptr<Scheduler> scheduler = ptr<Scheduler>());
    void createTileTaskDeleted(int producerId, int level, int tx, int ty);
    typedef std::map<Tile::TId, std::list<Tile *>::iterator> Cache;
    std::string name;
    int nextProducerId;
    std::map<int, TileProducer *> producers;
    ptr<TileStorage> storage;
    ptr<Scheduler> scheduler;
    std::map<Tile::TId, Tile *> usedTiles;
    Cache unusedTiles;
    std::list<Tile *> unusedTilesOrder;
    std::map<Tile::TId, Task *> deletedTiles;
    int queries;
    int misses;
    void *mutex;
};
"""

_CACHE_PRELUDE = r"""
#include <pthread.h>
#include <cassert>
#include <cstdarg>
#include <list>
#include <map>
#include <string>
#include <utility>
#include <vector>
#include "ork_gl.h"

namespace refcache {
using namespace std;   // as TileCache.cpp and TileStorage.cpp
using refgl::ptr;

// Ork stand-ins: Object, the debug logger, tasks with a done flag, a scheduler.
struct Object {
    explicit Object(const char *) {}
    virtual ~Object() {}
};
struct Logger {
    static Logger *DEBUG_LOGGER;
    void logf(const char *, const char *, ...) {}
};
Logger *Logger::DEBUG_LOGGER = nullptr;
struct Task {
    enum reason { DATA_NEEDED, DATA_CHANGED };
    bool done = false;
    bool isDone() { return done; }
    void setIsDone(bool d, unsigned int, reason) { done = d; }
};
struct Scheduler {
    void reschedule(ptr<Task> t, Task::reason r, unsigned int) { t->setIsDone(false, 0, r); }
};

""" + _DECL_STORAGE + r"""
// a producer whose createTile returns the task to reuse, or a new one not done
struct TileProducer {
    std::vector<Task *> tasks;
    ~TileProducer()
    {
        for (Task *t : tasks) delete t;
    }
    ptr<Task> createTile(int, int, int, TileStorage::Slot *, unsigned int, ptr<Task> task)
    {
        if (task.p) return task;
        tasks.push_back(new Task());
        return ptr<Task>(tasks.back());
    }
};

""" + _DECL_CACHE

_CACHE_DRIVER = r"""
}  // namespace refcache

namespace {
struct CacheHarness {
    refcache::TileStorage storage;
    refcache::TileCache cache;
    std::vector<refcache::TileProducer *> producers;
    ~CacheHarness()
    {
        // release every tile (the cache's destructor expects no used tile)
        for (auto &u : cache.usedTiles) u.second->users = 0;
        std::vector<refcache::TileCache::Tile *> used;
        for (auto &u : cache.usedTiles) used.push_back(u.second);
        for (refcache::TileCache::Tile *t : used) {
            t->users = 1;
            cache.putTile(t);
        }
        for (refcache::TileProducer *p : producers) delete p;
    }
};
CacheHarness *g_cache = nullptr;

int slot_of(refcache::TileCache::Tile *t) { return t ? t->data->index : -1; }
}  // namespace

// A TileCache over a storage of `capacity` slots (created in index order, as the
// storages' init functions do) shared by `nproducers` producers (ids 0, 1, ...).
extern "C" void ref_cache_create(int capacity, int nproducers)
{
    delete g_cache;
    g_cache = new CacheHarness();
    g_cache->storage.init(1, capacity);
    for (int k = 0; k < capacity; ++k) {
        refcache::TileStorage::Slot *s = new refcache::TileStorage::Slot(&g_cache->storage);
        s->index = k;
        g_cache->storage.freeSlots.push_back(s);
    }
    g_cache->cache.init(&g_cache->storage, "cache");
    for (int k = 0; k < nproducers; ++k) {
        g_cache->producers.push_back(new refcache::TileProducer());
        g_cache->cache.producers[k] = g_cache->producers.back();
    }
}

// getTile: the tile's slot or -1 (cache full); users_before: its users before the call
extern "C" int ref_cache_get(int producer, int level, int tx, int ty, int *users_before)
{
    int users = -1;
    refcache::TileCache::Tile *t = g_cache->cache.getTile(producer, level, tx, ty, 0, &users);
    *users_before = t ? users : -1;
    return slot_of(t);
}

// putTile of the used tile (producer, level, tx, ty): its users after, or -1 if not used
extern "C" int ref_cache_put(int producer, int level, int tx, int ty)
{
    refcache::TileCache::Tile *t = g_cache->cache.findTile(producer, level, tx, ty, false);
    return t ? g_cache->cache.putTile(t) : -1;
}

// findTile: the tile's slot or -1
extern "C" int ref_cache_find(int producer, int level, int tx, int ty, int include_cache)
{
    return slot_of(g_cache->cache.findTile(producer, level, tx, ty, include_cache != 0));
}

// prefetchTile: 1 when it created the tile (a task returned), else 0
extern "C" int ref_cache_prefetch(int producer, int level, int tx, int ty)
{
    return g_cache->cache.prefetchTile(producer, level, tx, ty).p != nullptr ? 1 : 0;
}

extern "C" void ref_cache_counts(int *used, int *unused, int *free_slots)
{
    *used = g_cache->cache.getUsedTiles();
    *unused = g_cache->cache.getUnusedTiles();
    *free_slots = g_cache->storage.getFreeSlots();
}

// whether the task of the tile (used or cached) is done; -1 without such a tile
extern "C" int ref_cache_done(int producer, int level, int tx, int ty)
{
    refcache::TileCache::Tile *t = g_cache->cache.findTile(producer, level, tx, ty, true);
    return t ? (t->task->isDone() ? 1 : 0) : -1;
}

// the tile's task runs: marks it done (what the scheduler does)
extern "C" void ref_cache_produce(int producer, int level, int tx, int ty)
{
    refcache::TileCache::Tile *t = g_cache->cache.findTile(producer, level, tx, ty, true);
    if (t) t->task->setIsDone(true, 0, refcache::Task::DATA_NEEDED);
}

extern "C" void ref_cache_invalidate(int producer) { g_cache->cache.invalidateTiles(producer); }
"""


def generate_cache(root):
    """oracle/_ref/gen/ref_cache.cpp: TileCache's and TileStorage's functions as written."""
    cache = _read(root, CACHE_CPP)
    storage = _read(root, STORAGE_CPP)
    src = ["// generated by oracle/ref_build.py from the reference's sources\n", _CACHE_PRELUDE]
    for text, rel, sigs in ((storage, STORAGE_CPP, STORAGE_SIGS), (cache, CACHE_CPP, CACHE_SIGS)):
        for sig in sigs:
            body, line = extract_function(text, sig)
            src.append("// %s:%d\n%s" % (rel, line, body))
    src.append(_CACHE_DRIVER)
    os.makedirs(GEN_DIR, exist_ok=True)
    path = os.path.join(GEN_DIR, "ref_cache.cpp")
    with open(path, "w") as f:
        f.write("".join(src))
    return path


QUAD_CPP = "src/core/sources/proland/terrain/TerrainQuad.cpp"
NODE_CPP = "src/core/sources/proland/terrain/TerrainNode.cpp"

QUAD_SIGS = [r"^TerrainQuad::TerrainQuad\(", r"bool TerrainQuad::isLeaf\(", r"void TerrainQuad::update\(",
             r"void TerrainQuad::subdivide\("]
NODE_SIGS = [r"float TerrainNode::getCameraDist\(", r"float TerrainNode::getSplitDistance\(",
             r"vec3d TerrainNode::getLocalCamera\("]

_DECL_QUAD = r"""
// The TerrainNode members TerrainQuad::update calls: every quad partially visible
// (the test has no view frustum), nothing occluded; getVisibility records the boxes
// in the order update meets them.
struct TerrainNode {
    bool splitInvisibleQuads = false;
    int maxLevel = 0;
    float splitDist = 2.0f, distFactor = 1.0f;
    vec3d localCameraPos{0, 0, 0};
    static float groundHeightAtCamera;
    std::vector<std::tuple<double, double, double> > visits;
    SceneManager::visibility getVisibility(const box3d &b)
    {
        visits.push_back(std::make_tuple(b.xmin, b.ymin, b.xmax - b.xmin));
        return SceneManager::PARTIALLY_VISIBLE;
    }
    bool isOccluded(const box3d &) { return false; }
    bool addOccluder(const box3d &) { return false; }
    float getCameraDist(const box3d &localBox) const;
    float getSplitDistance() const;
    vec3d getLocalCamera() const;
};
float TerrainNode::groundHeightAtCamera = 0.0f;

// The declaration of TerrainQuad.h the extracted functions define.
struct TerrainQuad : Object {
    const TerrainQuad *parent;
    const int level;
    const int tx;
    const int ty;
    const double ox;
    const double oy;
    const double l;
    float zmin;
    float zmax;
    ptr<TerrainQuad> children[4];
    SceneManager::visibility visible;
    bool occluded;
    bool drawable;
    TerrainQuad(TerrainNode *owner, const TerrainQuad *parent, int tx, int ty, double ox, double oy, double l,
                float zmin, float zmax);
    bool isLeaf() const;
    void update();
    TerrainNode *owner;
    void subdivide();
    TerrainNode *getOwner();
    int getDepth() const;
};
"""

_QUAD_PRELUDE = r"""
#include <algorithm>
#include <cassert>
#include <cmath>
#include <map>
#include <memory>
#include <tuple>
#include <vector>

namespace refquad {
using namespace std;   // as TerrainQuad.cpp and TerrainNode.cpp

// an owning pointer in the place of Ork's reference-counted ptr
template <class T> struct ptr {
    std::shared_ptr<T> s;
    ptr() {}
    ptr(T *q) : s(q) {}
    T *operator->() const { return s.get(); }
    bool operator==(const T *q) const { return s.get() == q; }
    bool operator!=(const T *q) const { return s.get() != q; }
};
struct Object {
    explicit Object(const char *) {}
    virtual ~Object() {}
};
inline bool isFinite(float x) { return std::isfinite(x); }
struct vec3d {
    double x, y, z;
};
struct box3d {
    double xmin, xmax, ymin, ymax, zmin, zmax;
    box3d(double a, double b, double c, double d, double e, double f)
        : xmin(a), xmax(b), ymin(c), ymax(d), zmin(e), zmax(f) {}
};
struct SceneManager {
    enum visibility { FULLY_VISIBLE, PARTIALLY_VISIBLE, INVISIBLE };
};

""" + _DECL_QUAD

_QUAD_DRIVER = r"""
void collect(const TerrainQuad *q, std::map<std::tuple<double, double, double>, const TerrainQuad *> &m)
{
    m[std::make_tuple(q->ox, q->oy, q->l)] = q;
    if (!q->isLeaf())
        for (int k = 0; k < 4; ++k) collect(q->children[k].s.get(), m);
}
}  // namespace refquad

// The quads of a terrain's quadtree after TerrainQuad::update of its root (the root
// quad of TerrainNode::init, [-size, size]^2 with size = root_size / 2) for a camera at
// (cx, cy, cz) and the ground height at the camera: (level, tx, ty) in the order
// update visits them (3 ints each, at most `capacity` quads).  Returns the count.
extern "C" int ref_quadtree(double root_size, int max_level, float split_dist, float dist_factor, double cx, double cy,
                            double cz, float ground, int *out, int capacity)
{
    using namespace refquad;
    TerrainNode node;
    node.maxLevel = max_level;
    node.splitDist = split_dist;
    node.distFactor = dist_factor;
    node.localCameraPos = vec3d{cx, cy, cz};
    TerrainNode::groundHeightAtCamera = ground;
    const float size = (float)(root_size / 2.0);
    TerrainQuad root(&node, NULL, 0, 0, -size, -size, 2.0 * size, 0.0f, 0.0f);
    root.update();
    std::map<std::tuple<double, double, double>, const TerrainQuad *> quads;
    collect(&root, quads);
    int n = 0;
    for (const auto &v : node.visits) {
        const TerrainQuad *q = quads.at(v);
        if (n < capacity) {
            out[3 * n] = q->level;
            out[3 * n + 1] = q->tx;
            out[3 * n + 2] = q->ty;
        }
        ++n;
    }
    return n;
}
"""


def generate_quadtree(root):
    """oracle/_ref/gen/ref_quadtree.cpp: TerrainQuad's update / subdivide and
    TerrainNode's distance functions as written."""
    quad = _read(root, QUAD_CPP)
    node = _read(root, NODE_CPP)
    src = ["// generated by oracle/ref_build.py from the reference's sources\n", _QUAD_PRELUDE]
    for text, rel, sigs in ((quad, QUAD_CPP, QUAD_SIGS), (node, NODE_CPP, NODE_SIGS)):
        for sig in sigs:
            body, line = extract_function(text, sig)
            src.append("// %s:%d\n%s" % (rel, line, body))
    src.append(_QUAD_DRIVER)
    os.makedirs(GEN_DIR, exist_ok=True)
    path = os.path.join(GEN_DIR, "ref_quadtree.cpp")
    with open(path, "w") as f:
        f.write("".join(src))
    return path


PRODUCER_CPP = "src/core/sources/proland/producer/TileProducer.cpp"
SAMPLER_CPP = "src/core/sources/proland/terrain/TileSampler.cpp"
PRODUCER_SIGS = [r"ptr<Task> TileProducer::startCreateTile\(", r"void TileProducer::stopCreateTile\(",
                 r"float TileProducer::getRootQuadSize\(", r"void TileProducer::setRootQuadSize\(",
                 r"int TileProducer::getId\(", r"ptr<TileCache> TileProducer::getCache\(",
                 r"bool TileProducer::isGpuProducer\(", r"int TileProducer::getBorder\(",
                 r"bool TileProducer::hasTile\(", r"bool TileProducer::hasChildren\(",
                 r"TileCache::Tile\* TileProducer::findTile\(", r"TileCache::Tile\* TileProducer::getTile\(",
                 r"bool TileProducer::prefetchTile\(", r"void TileProducer::putTile\(",
                 r"void TileProducer::update\(ptr<SceneManager>"]
SAMPLER_SIGS = [r"void TileSampler::init\(", r"ptr<Task> TileSampler::update\(", r"^TileSampler::Tree::Tree\(",
                r"^TileSampler::Tree::~Tree\(", r"void TileSampler::Tree::recursiveDelete\(",
                r"bool TileSampler::needTile\(", r"void TileSampler::putTiles\(", r"void TileSampler::getTiles\(",
                r"void TileSampler::prefetch\("]

_SAMPLER_PRELUDE = r"""
#include <pthread.h>
#include <algorithm>
#include <cassert>
#include <cmath>
#include <list>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

namespace refsampler {
using namespace std;   // as the extracted files

struct TerrainQuad;
// Ork's ptr: owning for terrain quads (their children are dropped by assignment),
// a plain reference to objects the harness owns otherwise.
template <class T> struct ptr {
    std::shared_ptr<T> s;
    ptr() {}
    ptr(T *q) : s(q, [](T *x) { if (std::is_same<T, TerrainQuad>::value) delete x; }) {}
    template <class U> ptr(const ptr<U> &o) : s(o.s, o.s.get()) {}
    T *operator->() const { return s.get(); }
    T *get() const { return s.get(); }
    template <class U> ptr<U> cast() const
    {
        ptr<U> r;
        r.s = std::shared_ptr<U>(s, dynamic_cast<U *>(s.get()));
        return r;
    }
    bool operator==(const T *q) const { return s.get() == q; }
    bool operator!=(const T *q) const { return s.get() != q; }
};

struct Object {
    explicit Object(const char *) {}
    virtual ~Object() {}
};
struct Logger {
    static Logger *DEBUG_LOGGER, *ERROR_LOGGER;
    void log(const string &, const string &) {}
    void logf(const char *, const char *, ...) {}
};
Logger *Logger::DEBUG_LOGGER = nullptr;
Logger *Logger::ERROR_LOGGER = nullptr;
inline bool isFinite(float x) { return std::isfinite(x); }
struct vec2f {
    float x, y;
    vec2f(float a, float b) : x(a), y(b) {}
};
struct vec3d {
    double x, y, z;
};
struct box3d {
    double xmin, xmax, ymin, ymax, zmin, zmax;
    box3d(double a, double b, double c, double d, double e, double f)
        : xmin(a), xmax(b), ymin(c), ymax(d), zmin(e), zmax(f) {}
};
struct SceneManager {
    enum visibility { FULLY_VISIBLE, PARTIALLY_VISIBLE, INVISIBLE };
};
struct Task {
    enum reason { DATA_NEEDED, DATA_CHANGED };
    bool done = false;
    Task() {}
    Task(const char *, bool, int) {}
    virtual ~Task() {}
    bool isDone() { return done; }
    void setIsDone(bool d, unsigned int, reason) { done = d; }
    virtual bool run() { return true; }
};
struct TaskGraph : Task {
    std::vector<Task *> tasks;
    void addTask(ptr<Task> t) { tasks.push_back(t.get()); }
    void addDependency(ptr<Task>, ptr<Task>) {}
    bool isEmpty() { return tasks.empty(); }
};
// the cache has no scheduler: prefetchTile creates nothing (a scheduler that does not
// prefetch for the producer)
struct Scheduler {
    bool supportsPrefetch(bool) { return false; }
    void schedule(ptr<Task>) {}
    void reschedule(ptr<Task> t, Task::reason r, unsigned int) { t->setIsDone(false, 0, r); }
};
"""

_SAMPLER_CLASSES = r"""
struct GPUTileStorage : TileStorage {
    void *getTileMap() { return nullptr; }   // no tile map: update's tile-map task never runs
};

struct TileLayer {
    void useTile(int, int, int, unsigned int) {}
    void unuseTile(int, int, int) {}
    void prefetchTile(int, int, int) {}
    void startCreateTile(int, int, int, unsigned int, ptr<Task>, ptr<TaskGraph>) {}
    void stopCreateTile(int, int, int) {}
    void setCache(ptr<TileCache>, int) {}
    void setTileSize(int, int, float) {}
};

// The TileProducer members the extracted functions use (TileProducer.h); createTile
// hands out a task, not done, or the one to reuse.
struct TileProducer {
    ptr<TileCache> cache;
    int id = 0;
    float rootQuadSize = 0.0f;
    bool gpuProducer = true;
    std::vector<ptr<TileLayer> > layers;
    std::vector<Task *> tasks;
    virtual ~TileProducer()
    {
        for (Task *t : tasks) delete t;
    }
    float getRootQuadSize();
    void setRootQuadSize(float size);
    int getId();
    ptr<TileCache> getCache();
    bool isGpuProducer();
    virtual int getBorder();
    virtual bool hasTile(int level, int tx, int ty);
    virtual bool hasChildren(int level, int tx, int ty);
    TileCache::Tile *findTile(int level, int tx, int ty, bool includeCache = false, bool done = false);
    TileCache::Tile *getTile(int level, int tx, int ty, unsigned int deadline);
    bool prefetchTile(int level, int tx, int ty);
    void putTile(TileCache::Tile *t);
    virtual void update(ptr<SceneManager> scene);
    bool updateTileMap(float, vec2f, int) { return false; }
    virtual ptr<Task> startCreateTile(int level, int tx, int ty, unsigned int deadline, ptr<Task> task,
                                      ptr<TaskGraph> owner);
    virtual void stopCreateTile(int level, int tx, int ty);
    // a task graph holding the tile's task (TileProducer::createTaskGraph makes a
    // CreateTileTaskGraph)
    ptr<TaskGraph> createTaskGraph(ptr<Task> task)
    {
        TaskGraph *g = new TaskGraph();
        tasks.push_back(g);
        g->addTask(task);
        return ptr<TaskGraph>(g);
    }
    // as TileProducer::createTile: a new task (or the one to reuse), made ready by
    // startCreateTile, which acquires the tiles the tile is made from
    ptr<Task> createTile(int level, int tx, int ty, TileStorage::Slot *, unsigned int deadline, ptr<Task> task)
    {
        if (task.get()) return task;
        tasks.push_back(new Task());
        return startCreateTile(level, tx, ty, deadline, ptr<Task>(tasks.back()), ptr<TaskGraph>());
    }
};

// The members ElevationProducer's and NormalProducer's start / stopCreateTile use.
struct ElevationProducer : TileProducer {
    ptr<TileProducer> residualTiles;
    ptr<Task> startCreateTile(int level, int tx, int ty, unsigned int deadline, ptr<Task> task,
                              ptr<TaskGraph> owner) override;
    void stopCreateTile(int level, int tx, int ty) override;
};
struct NormalProducer : TileProducer {
    ptr<TileProducer> elevationTiles;
    ptr<Task> startCreateTile(int level, int tx, int ty, unsigned int deadline, ptr<Task> task,
                              ptr<TaskGraph> owner) override;
    void stopCreateTile(int level, int tx, int ty) override;
};

struct TileFilter {
    virtual ~TileFilter() {}
    virtual bool storeTile(ptr<TerrainQuad> q) = 0;
};

// The declaration of TileSampler.h the extracted functions define.
struct TileSampler : Object {
    class Tree {
    public:
        bool newTree;
        bool needTile;
        Tree *parent;
        TileCache::Tile *t;
        Tree *children[4];
        Tree(Tree *parent);
        virtual ~Tree();
        virtual void recursiveDelete(TileSampler *owner);
    };
    TileSampler() : Object("TileSampler") {}
    void init(const string &name, ptr<TileProducer> producer);
    ptr<Task> update(ptr<SceneManager> scene, ptr<TerrainQuad> root);
    bool needTile(ptr<TerrainQuad> q);
    void putTiles(Tree **t, ptr<TerrainQuad> q);
    void getTiles(Tree *parent, Tree **t, ptr<TerrainQuad> q, ptr<TaskGraph> result);
    void prefetch(Tree *t, ptr<TerrainQuad> q, int &prefetchCount);
    string name;
    ptr<TileProducer> producer;
    std::vector<ptr<TerrainNode> > terrains;
    bool storeLeaf, storeParent, storeInvisible, async, mipmap;
    std::vector<TileFilter *> storeFilters;
    Tree *root;
    void *lastProgram;
};
"""

_SAMPLER_DRIVER = r"""
namespace {
struct SamplerHarness {
    GPUTileStorage storage;
    TileCache cache;
    TileProducer producer;
    TerrainNode node;
    TerrainQuad *root = nullptr;
    TileSampler sampler;
    ~SamplerHarness()
    {
        if (sampler.root) sampler.root->recursiveDelete(&sampler);
        sampler.root = nullptr;
        delete root;
    }
};
SamplerHarness *g_sampler = nullptr;
}  // namespace
}  // namespace refsampler

// A terrain (root quad of size root_size, as TerrainNode::init makes it), one producer on
// a cache of `capacity` slots and a TileSampler with the reference's defaults.
extern "C" void ref_sampler_create(double root_size, int max_level, float split_dist, int capacity)
{
    using namespace refsampler;
    delete g_sampler;
    g_sampler = new SamplerHarness();
    SamplerHarness &h = *g_sampler;
    h.storage.init(1, capacity);
    for (int k = 0; k < capacity; ++k) {
        TileStorage::Slot *s = new TileStorage::Slot(&h.storage);
        s->index = k;
        h.storage.freeSlots.push_back(s);
    }
    h.cache.init(&h.storage, "tiles");
    h.producer.cache = &h.cache;
    h.producer.id = h.cache.nextProducerId++;
    h.cache.producers[h.producer.id] = &h.producer;
    h.node.maxLevel = max_level;
    h.node.splitDist = split_dist;
    const float size = (float)(root_size / 2.0);
    h.root = new TerrainQuad(&h.node, NULL, 0, 0, -size, -size, 2.0 * size, 0.0f, 0.0f);
    h.sampler.init("elevation", &h.producer);
}

// One frame: the camera moves, the quadtree updates, TileSampler::update acquires and
// releases.  out: used tiles, unused tiles, free slots, the cache's queries and misses.
extern "C" void ref_sampler_frame(double cx, double cy, double cz, int *out5)
{
    using namespace refsampler;
    SamplerHarness &h = *g_sampler;
    h.node.localCameraPos = vec3d{cx, cy, cz};
    h.node.visits.clear();
    h.root->update();
    ptr<TerrainQuad> root;
    root.s = std::shared_ptr<TerrainQuad>(h.root, [](TerrainQuad *) {});   // the harness owns the root
    h.sampler.update(ptr<SceneManager>(), root);
    out5[0] = h.cache.getUsedTiles();
    out5[1] = h.cache.getUnusedTiles();
    out5[2] = h.storage.getFreeSlots();
    out5[3] = h.cache.queries;
    out5[4] = h.cache.misses;
}

namespace refsampler {
namespace {
// residual, elevation and normal producers on caches of their own (ElevationProducer /
// NormalProducer start and stop their tiles as written)
struct DepsHarness {
    GPUTileStorage storage[3];
    TileCache cache[3];
    TileProducer residuals;
    ElevationProducer elevations;
    NormalProducer normals;
    TileProducer *producer(int k) { return k == 0 ? &residuals : k == 1 ? (TileProducer *)&elevations : &normals; }
    ~DepsHarness()
    {
        // the caches' destructors expect every tile released
        for (int k = 2; k >= 0; --k) {
            std::vector<TileCache::Tile *> used;
            for (auto &u : cache[k].usedTiles) used.push_back(u.second);
            for (TileCache::Tile *t : used) {
                t->users = 1;
                cache[k].putTile(t);
            }
        }
    }
};
DepsHarness *g_deps = nullptr;
}  // namespace
}  // namespace refsampler

// tile widths: residuals rw, elevations w, normals w - 4; `capacity` slots each
extern "C" void ref_deps_create(int w, int rw, int capacity)
{
    using namespace refsampler;
    delete g_deps;
    g_deps = new DepsHarness();
    DepsHarness &h = *g_deps;
    const int widths[3] = {rw, w, w - 4};
    for (int k = 0; k < 3; ++k) {
        h.storage[k].init(widths[k], capacity);
        for (int s = 0; s < capacity; ++s) {
            TileStorage::Slot *slot = new TileStorage::Slot(&h.storage[k]);
            slot->index = s;
            h.storage[k].freeSlots.push_back(slot);
        }
        h.cache[k].init(&h.storage[k], "cache");
        TileProducer *p = h.producer(k);
        p->cache = &h.cache[k];
        p->id = h.cache[k].nextProducerId++;
        h.cache[k].producers[p->id] = p;
    }
    h.elevations.residualTiles = &h.residuals;
    h.normals.elevationTiles = &h.elevations;
}

// getTile on producer k (0 residuals, 1 elevations, 2 normals): 0, or -1 when the cache is full
extern "C" int ref_deps_get(int k, int level, int tx, int ty)
{
    return refsampler::g_deps->producer(k)->getTile(level, tx, ty, 0) ? 0 : -1;
}

// users of tile (level, tx, ty) of producer k (0: cached unused, -1: absent)
extern "C" int ref_deps_users(int k, int level, int tx, int ty)
{
    refsampler::TileCache::Tile *t = refsampler::g_deps->cache[k].findTile(0, level, tx, ty, true);
    return t ? t->users : -1;
}

extern "C" void ref_deps_counts(int k, int *used, int *unused)
{
    *used = refsampler::g_deps->cache[k].getUsedTiles();
    *unused = refsampler::g_deps->cache[k].getUnusedTiles();
}

// users of tile (level, tx, ty) in the cache (0: cached unused, -1: absent)
extern "C" int ref_sampler_users(int level, int tx, int ty)
{
    using namespace refsampler;
    TileCache::Tile *t = g_sampler->cache.findTile(0, level, tx, ty, true);
    return t ? t->users : -1;
}
"""


def generate_sampler(root):
    """oracle/_ref/gen/ref_sampler.cpp: the terrain quadtree, the tile cache, the
    producer's cache calls and TileSampler's update as written, in one namespace."""
    texts = {rel: _read(root, rel) for rel in (STORAGE_CPP, CACHE_CPP, QUAD_CPP, NODE_CPP, PRODUCER_CPP,
                                               SAMPLER_CPP, ELEV_CPP, NORMAL_CPP)}
    src = ["// generated by oracle/ref_build.py from the reference's sources\n", _SAMPLER_PRELUDE, _DECL_STORAGE,
           "struct TileProducer;\n", _DECL_CACHE, _DECL_QUAD, _SAMPLER_CLASSES]
    cls, line = extract_block(texts[SAMPLER_CPP], "class UpdateTileMapTask : public Task", "};")
    src.append("// %s:%d\n%s" % (SAMPLER_CPP, line, cls))
    extra = [(QUAD_CPP, [r"TerrainNode \*TerrainQuad::getOwner\(", r"int TerrainQuad::getDepth\("]),
             (ELEV_CPP, [r"ptr<Task> ElevationProducer::startCreateTile\(", r"void ElevationProducer::stopCreateTile\("]),
             (NORMAL_CPP, [r"ptr<Task> NormalProducer::startCreateTile\(", r"void NormalProducer::stopCreateTile\("])]
    for rel, sigs in [(STORAGE_CPP, STORAGE_SIGS), (CACHE_CPP, CACHE_SIGS), (QUAD_CPP, QUAD_SIGS),
                      (NODE_CPP, NODE_SIGS), (PRODUCER_CPP, PRODUCER_SIGS), (SAMPLER_CPP, SAMPLER_SIGS)] + extra:
        for sig in sigs:
            body, line = extract_function(texts[rel], sig)
            src.append("// %s:%d\n%s" % (rel, line, body))
    src.append(_SAMPLER_DRIVER)
    os.makedirs(GEN_DIR, exist_ok=True)
    path = os.path.join(GEN_DIR, "ref_sampler.cpp")
    with open(path, "w") as f:
        f.write("".join(src))
    return path


def _load_sibling(name):
    """oracle/<name>.py by path (this file also runs as a script and is loaded by path)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("oracle_" + name, os.path.join(HERE, name + ".py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def generate_gpu(root):
    """oracle/_ref/gen/ref_gpu.cpp: the shaders as C++, the producers' init look-ups and
    doCreateTile functions as written, the drivers."""
    ref_glsl = _load_sibling("ref_glsl")
    elev = _read(root, ELEV_CPP)
    norm = _read(root, NORMAL_CPP)
    src = ["// generated by oracle/ref_build.py from the reference's sources\n#include <cstring>\n#include <vector>\n"
           "#include \"ork_gl.h\"\n#include \"proland/math/noise.h\"\n"]
    shader_parts, tables = [], {"g_upsample": [], "g_normal": [], "g_blend": [], "g_ortho": []}
    # full-screen quads: st in pixels (upsample, normals) or in [0, 1] (blend), as
    # each program's vertex shader makes it
    for kind, shaders, unit in (("g_upsample", UPSAMPLE_SHADERS, False), ("g_normal", NORMAL_SHADERS, False),
                                ("g_blend", BLEND_SHADERS, True), ("g_ortho", ORTHO_SHADERS, False)):
        for name, rel, defines in shaders:
            ns = "%s_%s" % (kind[2:], name)
            body, uniforms, _ = ref_glsl.shader_to_cpp(_read(root, rel), ns, "_FRAGMENT_", defines)
            shader_parts.append("// %s\n%s%s%s" % (rel, body, ref_glsl.uniform_table(ns, uniforms),
                                                  ref_glsl.quad_runner(ns, unit)))
            tables[kind].append(ns)
    layers = []
    for name, rel, defines in LAYER_SHADERS:
        ns = "layer_%s" % name
        body, uniforms, others = ref_glsl.shader_to_cpp(_read(root, rel), ns, "_FRAGMENT_", defines)
        shader_parts.append("// %s\n%s%s%s" % (rel, body, ref_glsl.uniform_table(ns, uniforms),
                                              ref_glsl.fragment_call(ns, any(n == "st" for _, n in others))))
        layers.append(ns)
    src.extend(shader_parts)
    src.append(_GPU_PRELUDE)
    src.append("namespace {\nstruct ProgramSource { const refgl::UniformEntry *table; void (*run)(refgl::FrameBuffer &); };\n")
    for kind, names in tables.items():
        src.append("const ProgramSource %s[] = {%s};\n" % (kind, ", ".join("{%s_uniforms, %s_run}" % (n, n)
                                                                             for n in names)))
    src.append("struct FragmentSource { const refgl::UniformEntry *table; void (*fragment)(float, float, float *, "
               "float *); };\nconst FragmentSource g_layer[] = {%s};\n"
               % ", ".join("{%s_uniforms, %s_fragment}" % (n, n) for n in layers))
    src.append("}  // namespace\n")
    ups, ups_line = extract_block(elev, 'this->tileWSDFU = upsample->getUniform4f("tileWSDF");',
                                  'this->noiseUVLHU = upsample->getUniform4f("noiseUVLH");',
                                  after="void ElevationProducer::init(")
    bls, bls_line = extract_braced(elev, "if (this->blend != NULL) {", after="void ElevationProducer::init(")
    dct, dct_line = extract_function(elev, r"bool\s+ElevationProducer::doCreateTile\s*\(")
    nups, nups_line = extract_block(norm, 'this->tileSDFU = normals->getUniform3f("tileSDF");',
                                    'this->deformU = normals->getUniform4f("deform");',
                                    after="void NormalProducer::init(")
    ndct, ndct_line = extract_function(norm, r"bool\s+NormalProducer::doCreateTile\s*\(")
    ortho = _read(root, ORTHO_CPP)
    oups, oups_line = extract_block(ortho, 'tileWidthU = upsample->getUniform1f("tileWidth");',
                                    'rootNoiseColorU = upsample->getUniform4f("rootNoiseColor");',
                                    after="void OrthoProducer::init(")
    odct, odct_line = extract_function(ortho, r"bool\s+OrthoProducer::doCreateTile\s*\(")
    src.append("namespace refgl {\n")
    src.append("void ElevationProducer::bind_uniforms()\n{\n// %s:%d\n%s// %s:%d\n%s}\n"
               % (ELEV_CPP, ups_line, ups, ELEV_CPP, bls_line, bls))
    src.append("// %s:%d\n%s" % (ELEV_CPP, dct_line, dct))
    src.append("// %s:%d\nvoid NormalProducer::bind_uniforms()\n{\n%s}\n" % (NORMAL_CPP, nups_line, nups))
    src.append("// %s:%d\n%s" % (NORMAL_CPP, ndct_line, ndct))
    graph = _read(root, GRAPH_LAYER_CPP)
    road = _read(root, ROAD_LAYER_CPP)
    dca, dca_line = extract_function(graph, r"void\s+ElevationGraphLayer::drawCurveAltitude\s*\(")
    dcp, dcp_line = extract_function(_read(root, GRAPH_PRODUCER_CPP),
                                     r"void\s+GraphLayer::drawCurve\s*\(\s*const vec3d &tileCoords,\s*CurvePtr p,"
                                     r"\s*const vec4f &part")
    macros, macros_line = extract_block(road, "#define BASEWIDTH(", "#define TOTALWIDTH(")
    placing, placing_line = extract_block(road, "float scale = 2.0f * (getTileSize()", "vec3d tileOffset = vec3d(",
                                          after="bool RoadElevationLayer::doCreateTile(")
    cw, cw_line = extract_block(road, "float cwidth = c->getWidth();", "float cwidth = c->getWidth();",
                                after="bool RoadElevationLayer::doCreateTile(")
    widths, widths_line = extract_block(road, "float w = BASEWIDTH(cwidth, scale);", "float tw = TOTALWIDTH(w);",
                                        after="bool RoadElevationLayer::doCreateTile(")
    call, call_line = extract_block(road, "ElevationGraphLayer::drawCurveAltitude(tileOffset, c, cData,",
                                    "ElevationGraphLayer::drawCurveAltitude(tileOffset, c, cData,",
                                    after="bool RoadElevationLayer::doCreateTile(")
    src.append("// %s:%d\n%s" % (GRAPH_LAYER_CPP, dca_line, dca))
    src.append("// %s:%d\n%s" % (GRAPH_PRODUCER_CPP, dcp_line, dcp))
    dra, dra_line = extract_function(_read(root, GRAPH_PRODUCER_CPP), r"void\s+GraphLayer::drawArea\s*\(")
    src.append("// %s:%d\n%s" % (GRAPH_PRODUCER_CPP, dra_line, dra))
    water = _read(root, WATER_LAYER_CPP)
    wdct, wdct_line = extract_function(water, r"bool\s+WaterElevationLayer::doCreateTile\s*\(")
    wmac, wmac_line = extract_block(water, "#define BASEWIDTH(", "#define TOTALWIDTH(")
    src.append("}  // namespace refgl\n#undef BASEWIDTH\n#undef TOTALWIDTH\n// %s:%d\n%snamespace refgl {\n"
               "FrameBuffer *SceneManager::current = nullptr;\n// %s:%d\n%s"
               % (WATER_LAYER_CPP, wmac_line, wmac, WATER_LAYER_CPP, wdct_line, wdct))
    src.append("}  // namespace refgl\n// %s:%d\n%snamespace refgl {\n" % (ROAD_LAYER_CPP, macros_line, macros))
    src.append("void RoadElevationLayer::draw_road(const vec3d &q, CurvePtr c, ElevationCurveData *cData, "
               "ptr<FrameBuffer> fb, float *scale_out)\n{\n    vec2d nx, ny, lx, ly;\n"
               "    // %s:%d\n%s    // :%d\n%s    // :%d\n%s    // :%d\n%s    *scale_out = scale;\n}\n"
               % (ROAD_LAYER_CPP, placing_line, placing, cw_line, cw, widths_line, widths, call_line, call))
    rdct, rdct_line = extract_function(road, r"bool\s+RoadElevationLayer::doCreateTile\s*\(")
    src.append("// %s:%d\n%s" % (ROAD_LAYER_CPP, rdct_line, rdct))
    src.append("// %s:%d\nvoid OrthoProducer::bind_uniforms()\n{\n%s}\n" % (ORTHO_CPP, oups_line, oups))
    src.append("// %s:%d\n%s" % (ORTHO_CPP, odct_line, odct))
    src.append("}  // namespace refgl\n")
    src.append(_GPU_DRIVERS)
    os.makedirs(GEN_DIR, exist_ok=True)
    path = os.path.join(GEN_DIR, "ref_gpu.cpp")
    with open(path, "w") as f:
        f.write("".join(src))
    return path


def build(root=DEFAULT_ROOT, force=False):
    """Compiles libref.so when the reference tree is present; returns its path, or
    None without the reference (the GPU machine has none; the pin runs where it is)."""
    if not os.path.isdir(os.path.join(root, "src")):
        return LIB if os.path.exists(LIB) else None
    srcs = [os.path.join(root, p) for p in (NOISE_CPP, ELEV_CPP, CPU_ELEV_CPP, MIPMAP_CPP, NORMAL_CPP, ORTHO_CPP,
                                            GRAPH_LAYER_CPP, ROAD_LAYER_CPP, GRAPH_PRODUCER_CPP, WATER_LAYER_CPP,
                                            RESIDUAL_CPP,
                                            ORTHO_CPU_CPP, MFS_CPP, CACHE_CPP, STORAGE_CPP, QUAD_CPP, NODE_CPP,
                                            PRODUCER_CPP, SAMPLER_CPP, TILE_CACHE_CPP, COLOR_MIPMAP_CPP)]
    srcs += [os.path.join(root, rel) for _, rel, _ in UPSAMPLE_SHADERS + NORMAL_SHADERS + BLEND_SHADERS +
             LAYER_SHADERS + ORTHO_SHADERS]
    srcs += [os.path.abspath(__file__), os.path.join(HERE, "ref_glsl.py")]
    srcs += [os.path.join(HERE, "ref_stubs", h) for h in ("pmath.h", "glsl.h", "ork_gl.h", "tiffio.h")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in srcs):
        return LIB
    gen = generate(root)
    gen_gpu = generate_gpu(root)
    gen_res = generate_residual(root)
    gen_cache = generate_cache(root)
    gen_quad = generate_quadtree(root)
    gen_sampler = generate_sampler(root)
    gen_mip = generate_mipmap(root)
    tmp = LIB + ".tmp%d" % os.getpid()
    inc = ["-I", os.path.join(HERE, "ref_stubs"), "-I", os.path.join(root, NOISE_DIR),
           "-I", os.path.join(root, "src/core/sources/proland/math")]
    flags = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-w", "-DPROLAND_API="]
    units = [(gen, "c++14"), (gen_gpu, "c++17"), (gen_res, "c++17"), (gen_cache, "c++17"), (gen_quad, "c++17"),
             (gen_sampler, "c++17"), (gen_mip, "c++17"), (os.path.join(root, NOISE_CPP), "c++14"), (os.path.join(root, MFS_CPP), "c++14")]
    objs = [os.path.join(GEN_DIR, os.path.basename(unit) + ".o") for unit, _ in units]
    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        jobs = [ex.submit(subprocess.check_call, ["g++", "-c", "-std=" + std] + flags + inc + ["-o", obj, unit])
                for (unit, std), obj in zip(units, objs)]
        for j in jobs:
            j.result()
    subprocess.check_call(["g++", "-shared", "-o", tmp] + objs + ["-lz", "-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_ROOT, force=True))
