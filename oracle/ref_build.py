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
static float *g_captured = nullptr;
enum { R16F, RED, FLOAT, REPEAT, NEAREST };
struct CPUBuffer { const void *data; explicit CPUBuffer(const void *d) : data(d) {} };
struct Buffer { struct Parameters {}; };
struct Texture { struct Parameters {
    Parameters &wrapS(int) { return *this; } Parameters &wrapT(int) { return *this; }
    Parameters &min(int) { return *this; } Parameters &mag(int) { return *this; } }; };
struct Texture2DArray {
    Texture2DArray(int w, int h, int layers, int, int, int, Texture::Parameters, Buffer::Parameters, CPUBuffer b) {
        if (g_captured) memcpy(g_captured, b.data, sizeof(float) * (size_t)w * h * layers);
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
    sel, sel_line = extract_block(elev, "int noiseL = 0;", "noiseL = noiseLs[noiseL];",
                                  after="bool ElevationProducer::doCreateTile(")
    loop, loop_line = extract_loop_to_end(cpu, "int residualTileWidth =", after="bool CPUElevationProducer::doCreateTile(")
    fns = []
    for name in ("computeResidual", "encodeResidual", "computeApproxTile"):
        body, line = extract_function(mip, r"void\s+HeightMipmap::%s\s*\(" % name)
        fns.append(("HeightMipmap.cpp:%d" % line, body))
    src = [_PRELUDE]
    src.append("namespace proland {\n// %s:%d\n%s}  // namespace proland\n" % (ELEV_CPP, dem_line, dem))
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


def build(root=DEFAULT_ROOT, force=False):
    """Compiles libref.so when the reference tree is present; returns its path, or
    None without the reference (the GPU machine has none; the pin runs where it is)."""
    if not os.path.isdir(os.path.join(root, "src")):
        return LIB if os.path.exists(LIB) else None
    srcs = [os.path.join(root, NOISE_CPP), os.path.join(root, ELEV_CPP), os.path.join(root, CPU_ELEV_CPP),
            os.path.join(root, MIPMAP_CPP), os.path.abspath(__file__), os.path.join(HERE, "ref_stubs", "pmath.h")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in srcs):
        return LIB
    gen = generate(root)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-std=c++14", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-w",
           "-I", os.path.join(HERE, "ref_stubs"), "-I", os.path.join(root, NOISE_DIR),
           "-I", os.path.join(root, "src/core/sources/proland/math"),
           "-o", tmp, gen, os.path.join(root, NOISE_CPP)]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_ROOT, force=True))
