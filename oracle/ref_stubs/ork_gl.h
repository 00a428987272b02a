// Stand-ins for the parts of Ork (the engine the reference builds on, not part of
// the reference tree) that the extracted GPU producer code calls:
// ElevationProducer::doCreateTile, NormalProducer::doCreateTile and
// OrthoProducer::doCreateTile, and the uniform look-ups of their init functions.  TEST INFRASTRUCTURE ONLY
// (oracle/ref_build.py compiles them with the extracted code and the reference's
// shaders, rewritten as C++ against glsl.h).
//
// What they do:
// * Uniform*::set / setMatrix write the value into the shader's global variable
//   (a row-major Ork matrix is uploaded transposed, so that the shader's column
//   c is the matrix's column c, as glUniformMatrix*fv(..., GL_TRUE, ...) does);
//   a uniform the shader does not declare is NULL, as Program::getUniform* answers.
// * FrameBuffer::drawQuad(program) runs the program's fragment shader once per
//   pixel (i, j) of the viewport with the varying st = (i + 0.5, j + 0.5), the
//   pixel centre of the full-screen quad, and stores `data` into the colour
//   attachment; clear() fills it with the clear colour.
// * GPUSlot::copyPixels copies the read colour attachment into the slot's layer.
// * TileProducer::doCreateTile (drawing the layers) runs a hook the harness gives.
// * FrameBuffer::draw(program, mesh) records the mesh (mode, vertices, indices).
// * Texture2D::setSubImage copies float or byte pixels in.
// * vec3<T>, vec4<T>, mat3<T>, mat4<T>: component-wise arithmetic in T;
//   length = sqrt(x*x + y*y + z*z), normalize divides each component by it
//   (and reports it), crossProduct the determinant form, matrices row-major
//   (m[r][c]) with the usual product summed over k = 0, 1, 2 in order.
#pragma once

#include <cassert>
#include <cmath>
#include <cstring>
// The C++ <math.h> declares the float overloads of the math functions in the global
// namespace (sqrt(2.0f) is a float square root), as the reference's translation units
// see them through the engine headers: RoadElevationLayer.cpp's BASEWIDTH calls
// sqrt(2.0f) with no `using namespace std`.
#include <math.h>
#include <map>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "glsl.h"

namespace refgl {

using std::ostringstream;
using std::string;
using std::vector;
typedef float GLfloat;
typedef int GLint;

template <class T> struct ptr {  // non-owning: the harness owns every object
    T *p = nullptr;
    ptr() {}
    ptr(T *q) : p(q) {}
    template <class U> ptr(const ptr<U> &o) : p(o.p) {}
    T *operator->() const { return p; }
    T &operator*() const { return *p; }
    T *get() const { return p; }
    template <class U> ptr<U> cast() const { return ptr<U>(dynamic_cast<U *>(p)); }
    bool operator==(const T *q) const { return p == q; }
    bool operator!=(const T *q) const { return p != q; }
};

inline bool isFinite(float x) { return std::isfinite(x); }

// ---- Ork math ----------------------------------------------------------------------
template <class T> struct vec2 {
    T x, y;
    vec2() : x(0), y(0) {}
    vec2(T a, T b) : x(a), y(b) {}
    vec2 operator+(const vec2 &o) const { return vec2(x + o.x, y + o.y); }
    vec2 operator-(const vec2 &o) const { return vec2(x - o.x, y - o.y); }
    vec2 operator*(T s) const { return vec2(x * s, y * s); }
    T length() const { return std::sqrt(x * x + y * y); }
};

template <class T> struct vec3 {
    T x, y, z;
    vec3() : x(0), y(0), z(0) {}
    vec3(T a, T b, T c) : x(a), y(b), z(c) {}
    vec3 operator+(const vec3 &o) const { return vec3(x + o.x, y + o.y, z + o.z); }
    vec3 operator-(const vec3 &o) const { return vec3(x - o.x, y - o.y, z - o.z); }
    vec3 operator*(T s) const { return vec3(x * s, y * s, z * s); }
    T length() const { return std::sqrt(x * x + y * y + z * z); }
    vec3 normalize() const
    {
        T l = length();
        return vec3(x / l, y / l, z / l);
    }
    vec3 normalize(T *previousLength) const
    {
        *previousLength = length();
        return vec3(x / *previousLength, y / *previousLength, z / *previousLength);
    }
    vec3 crossProduct(const vec3 &v) const { return vec3(y * v.z - z * v.y, z * v.x - x * v.z, x * v.y - y * v.x); }
    vec2<T> xy() const { return vec2<T>(x, y); }
    template <class U> vec3<U> cast() const { return vec3<U>((U)x, (U)y, (U)z); }
    static const vec3 UNIT_Y;
};
template <class T> const vec3<T> vec3<T>::UNIT_Y(0, 1, 0);

template <class T> struct vec4 {
    T x, y, z, w;
    vec4() : x(0), y(0), z(0), w(0) {}
    vec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    vec4 operator*(const vec4 &o) const { return vec4(x * o.x, y * o.y, z * o.z, w * o.w); }
    vec4 operator*(T s) const { return vec4(x * s, y * s, z * s, w * s); }
    vec4 operator/(T s) const { return vec4(x / s, y / s, z / s, w / s); }
    template <class U> vec4<U> cast() const { return vec4<U>((U)x, (U)y, (U)z, (U)w); }
};

template <class T> struct mat3 {
    T m[3][3];
    mat3() { std::memset(m, 0, sizeof(m)); }
    mat3(T m00, T m01, T m02, T m10, T m11, T m12, T m20, T m21, T m22)
    {
        m[0][0] = m00; m[0][1] = m01; m[0][2] = m02;
        m[1][0] = m10; m[1][1] = m11; m[1][2] = m12;
        m[2][0] = m20; m[2][1] = m21; m[2][2] = m22;
    }
    mat3 operator*(const mat3 &b) const
    {
        mat3 r;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) r.m[i][j] = m[i][0] * b.m[0][j] + m[i][1] * b.m[1][j] + m[i][2] * b.m[2][j];
        return r;
    }
    template <class U> mat3<U> cast() const
    {
        mat3<U> r;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) r.m[i][j] = (U)m[i][j];
        return r;
    }
    static const mat3 IDENTITY;
};
template <class T> const mat3<T> mat3<T>::IDENTITY(1, 0, 0, 0, 1, 0, 0, 0, 1);

template <class T> struct mat4 {
    T m[4][4];
    mat4() { std::memset(m, 0, sizeof(m)); }
    mat4(T m00, T m01, T m02, T m03, T m10, T m11, T m12, T m13, T m20, T m21, T m22, T m23, T m30, T m31, T m32,
         T m33)
    {
        const T v[16] = {m00, m01, m02, m03, m10, m11, m12, m13, m20, m21, m22, m23, m30, m31, m32, m33};
        for (int k = 0; k < 16; ++k) m[k / 4][k % 4] = v[k];
    }
    template <class U> mat4<U> cast() const
    {
        mat4<U> r;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) r.m[i][j] = (U)m[i][j];
        return r;
    }
};

typedef vec2<double> vec2d;
typedef vec2<float> vec2f;
typedef vec3<float> vec3f;
typedef vec3<double> vec3d;
typedef vec4<float> vec4f;
typedef vec4<double> vec4d;
typedef vec4<int> vec4i;
typedef mat3<float> mat3f;
typedef mat3<double> mat3d;
typedef mat4<float> mat4f;
typedef mat4<double> mat4d;

// ---- logging ------------------------------------------------------------------------
struct Logger {
    static Logger *DEBUG_LOGGER;
    static Logger *ERROR_LOGGER;
    void log(const string &, const string &) {}
};

// ---- textures, buffers -----------------------------------------------------------------
enum TextureInternalFormat { R16F, R32F, RG8, RGBA8, RG32F, RGBA32F, RGB32F };
enum TextureFormat { RED, RG, RGB, RGBA };
enum PixelType { FLOAT, UNSIGNED_BYTE };
enum BufferId { COLOR0, COLOR1, DEPTH };
enum Function { LESS, ALWAYS, NOTEQUAL };

struct Buffer {
    struct Parameters {};
    virtual ~Buffer() {}
};
struct CPUBuffer : Buffer {
    const void *data;
    explicit CPUBuffer(const void *d) : data(d) {}
};

struct Texture {
    glsl::Texture view;
    vector<float> store;
    TextureInternalFormat format = RGBA32F;
    virtual ~Texture() {}
    void alloc(int w, int h, int layers, int comps, bool repeat)
    {
        store.assign((size_t)w * h * layers * comps, 0.0f);
        view.data = store.data();
        view.w = w;
        view.h = h;
        view.layers = layers;
        view.comps = comps;
        view.repeat = repeat;
    }
    TextureInternalFormat getInternalFormat() { return format; }
    int getComponents() { return view.comps; }
    int getWidth() { return view.w; }
    int getHeight() { return view.h; }
};
struct Texture2D : Texture {
    // FLOAT or UNSIGNED_BYTE pixels of 1-4 components (RED, RG, RGB, RGBA) into the
    // texture; a byte k reads back as k / 255 (GL's unorm8); as GL's pixel transfer does,
    // components the pixels lack are 0, alpha 1
    void setSubImage(int, int x, int y, int w, int h, TextureFormat f, PixelType t, const Buffer::Parameters &,
                     const Buffer &pixels)
    {
        const void *src = dynamic_cast<const CPUBuffer &>(pixels).data;
        const int n = f == RED ? 1 : f == RG ? 2 : f == RGB ? 3 : 4;
        for (int j = 0; j < h; ++j)
            for (int i = 0; i < w; ++i)
                for (int k = 0; k < view.comps; ++k) {
                    const size_t s = ((size_t)j * w + i) * n + k;
                    float v = k == 3 ? 1.0f : 0.0f;
                    if (k < n) v = t == FLOAT ? ((const float *)src)[s] : (float)((const unsigned char *)src)[s] / 255.0f;
                    store[((size_t)(y + j) * view.w + x + i) * view.comps + k] = v;
                }
    }
};
struct Texture2DArray : Texture {};

// ---- programs and uniforms ---------------------------------------------------------------
enum UniformKind { U_FLOAT, U_INT, U_VEC2, U_VEC3, U_VEC4, U_IVEC4, U_MAT3, U_MAT4, U_SAMPLER2D, U_SAMPLER2DARRAY };
struct UniformEntry {
    const char *name;
    UniformKind kind;
    void *dst;
};

struct Uniform {
    UniformKind kind;
    void *dst;
    void set(float v)
    {
        if (kind == U_INT)
            *(int *)dst = (int)v;
        else
            *(float *)dst = v;
    }
    void set(const vec3f &v)
    {
        float *d = (float *)dst;
        d[0] = v.x; d[1] = v.y; d[2] = v.z;
    }
    void set(const vec4f &v)
    {
        float *d = (float *)dst;
        d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
    }
    void set(const vec4i &v)
    {
        int *d = (int *)dst;
        d[0] = v.x; d[1] = v.y; d[2] = v.z; d[3] = v.w;
    }
    void set(ptr<Texture> t)
    {
        if (kind == U_SAMPLER2D)
            ((glsl::sampler2D *)dst)->t = &t->view;
        else
            ((glsl::sampler2DArray *)dst)->t = &t->view;
    }
    void setMatrix(const mat3f &m)  // transposed upload: column c of the shader's matrix = column c of m
    {
        float *d = (float *)dst;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) d[c * 3 + r] = m.m[r][c];
    }
    void setMatrix(const mat4f &m)
    {
        float *d = (float *)dst;
        for (int c = 0; c < 4; ++c)
            for (int r = 0; r < 4; ++r) d[c * 4 + r] = m.m[r][c];
    }
};
typedef Uniform Uniform1f;
typedef Uniform Uniform1i;
typedef Uniform Uniform3f;
typedef Uniform Uniform4f;
typedef Uniform Uniform4i;
typedef Uniform UniformMatrix3f;
typedef Uniform UniformMatrix4f;
typedef Uniform UniformSampler;

struct FrameBuffer;

struct Program {
    const UniformEntry *table = nullptr;
    void (*run)(FrameBuffer &) = nullptr;
    std::map<string, Uniform> made;
    ptr<Uniform> lookup(const char *name, UniformKind k0, UniformKind k1)
    {
        for (const UniformEntry *e = table; e && e->name; ++e)
            if (name == string(e->name) && (e->kind == k0 || e->kind == k1)) {
                Uniform &u = made[name];
                u.kind = e->kind;
                u.dst = e->dst;
                return ptr<Uniform>(&u);
            }
        return ptr<Uniform>();
    }
    ptr<Uniform1f> getUniform1f(const char *n) { return lookup(n, U_FLOAT, U_INT); }
    ptr<Uniform3f> getUniform3f(const char *n) { return lookup(n, U_VEC3, U_VEC3); }
    ptr<Uniform4f> getUniform4f(const char *n) { return lookup(n, U_VEC4, U_VEC4); }
    ptr<Uniform4i> getUniform4i(const char *n) { return lookup(n, U_IVEC4, U_IVEC4); }
    ptr<UniformMatrix3f> getUniformMatrix3f(const char *n) { return lookup(n, U_MAT3, U_MAT3); }
    ptr<UniformMatrix4f> getUniformMatrix4f(const char *n) { return lookup(n, U_MAT4, U_MAT4); }
    ptr<UniformSampler> getUniformSampler(const char *n) { return lookup(n, U_SAMPLER2D, U_SAMPLER2DARRAY); }
};

struct FrameBuffer {
    int w = 0, h = 0;
    vector<float> color[2];  // RGBA float attachments COLOR0, COLOR1
    int draw_buffer = 0, read_buffer = 0;
    float clear_color[4] = {0, 0, 0, 0};
    void init(int W)
    {
        w = h = W;
        color[0].assign((size_t)W * W * 4, 0.0f);
        color[1].assign((size_t)W * W * 4, 0.0f);
    }
    void setClearColor(const vec4f &c)
    {
        clear_color[0] = c.x; clear_color[1] = c.y; clear_color[2] = c.z; clear_color[3] = c.w;
    }
    void clear(bool color_, bool, bool)
    {
        if (!color_) return;
        for (size_t k = 0; k < color[draw_buffer].size(); ++k) color[draw_buffer][k] = clear_color[k % 4];
    }
    void drawQuad(ptr<Program> p) { p->run(*this); }
    void write(int i, int j, const float *rgba)
    {
        std::memcpy(&color[draw_buffer][((size_t)j * w + i) * 4], rgba, 4 * sizeof(float));
    }
    // the depth test, depth and colour write masks of the next draws
    bool depth_test = false;
    int depth_func = LESS;
    bool color_mask[4] = {true, true, true, true};
    bool depth_mask = true;
    void setDepthTest(bool on, Function f = LESS)
    {
        depth_test = on;
        depth_func = f;
    }
    void setColorMask(bool r, bool g, bool b, bool a)
    {
        color_mask[0] = r; color_mask[1] = g; color_mask[2] = b; color_mask[3] = a;
    }
    void setDepthMask(bool d) { depth_mask = d; }
    // meshes drawn by draw(program, mesh): mode, (x, y, z, w) vertices (z, w 0 for 2D
    // vertices), indices, the program, the state above and what `on_draw` adds
    struct Drawn {
        int mode;
        vector<float> vertices;
        vector<unsigned int> indices;
        const Program *program = nullptr;
        bool depth_test = false, depth_mask = true, color_mask[4];
        int depth_func = LESS;
        vector<float> extra;
    };
    vector<Drawn> drawn;
    void (*on_draw)(void *, Drawn &) = nullptr;
    void *on_draw_arg = nullptr;
    template <class T> static void push4(vector<float> &o, const vec4<T> &v)
    {
        o.push_back(v.x); o.push_back(v.y); o.push_back(v.z); o.push_back(v.w);
    }
    template <class T> static void push4(vector<float> &o, const vec2<T> &v)
    {
        o.push_back(v.x); o.push_back(v.y); o.push_back(0.0f); o.push_back(0.0f);
    }
    template <class M> void draw(ptr<Program> prog, const M &mesh)
    {
        Drawn d;
        d.mode = mesh.mode;
        for (const auto &v : mesh.vertices) push4(d.vertices, v);
        d.indices = mesh.indices;
        d.program = prog.get();
        d.depth_test = depth_test;
        d.depth_func = depth_func;
        d.depth_mask = depth_mask;
        for (int k = 0; k < 4; ++k) d.color_mask[k] = color_mask[k];
        if (on_draw) on_draw(on_draw_arg, d);
        drawn.push_back(d);
    }
    void setDrawBuffer(BufferId b) { draw_buffer = b == COLOR1 ? 1 : 0; }
    void setReadBuffer(BufferId b) { read_buffer = b == COLOR1 ? 1 : 0; }
};

// ---- meshes ---------------------------------------------------------------------------------
enum MeshMode { TRIANGLES, TRIANGLE_STRIP };
template <class V, class I> struct Mesh {
    int mode = TRIANGLES;
    vector<V> vertices;
    vector<I> indices;
    void setMode(MeshMode m) { mode = m; }
    void clear()
    {
        vertices.clear();
        indices.clear();
    }
    void addVertex(const V &v) { vertices.push_back(v); }
    void addIndice(I i) { indices.push_back(i); }
};

// ---- tile storage, cache and producers ------------------------------------------------------
struct TileStorage {
    int tileSize = 0;
    virtual ~TileStorage() {}
    int getTileSize() { return tileSize; }
    struct Slot {
        TileStorage *owner = nullptr;
        virtual ~Slot() {}
        TileStorage *getOwner() { return owner; }
    };
};

struct GPUTileStorage : TileStorage {
    ptr<Texture> texture0;
    ptr<Texture> getTexture(int) { return texture0; }
    struct GPUSlot : TileStorage::Slot {
        ptr<Texture2DArray> t;
        int l = 0;
        int getWidth() { return t->view.w; }
        int getHeight() { return t->view.h; }
        // the colour attachment being read into this slot's layer, all four components
        // (a texture with fewer keeps the first ones); an 8-bit normalized texture
        // stores round(clamp(v, 0, 1) * 255) / 255, GL's float to unorm8 conversion
        void copyPixels(ptr<FrameBuffer> fb, int x, int y, int w, int h)
        {
            Texture &tx = *t;
            const int comps = tx.view.comps;
            const bool unorm8 = tx.format == RG8 || tx.format == RGBA8;
            for (int j = 0; j < h; ++j)
                for (int i = 0; i < w; ++i)
                    for (int k = 0; k < comps; ++k) {
                        float v = fb->color[fb->read_buffer][((size_t)(y + j) * fb->w + x + i) * 4 + k];
                        if (unorm8) v = std::floor((v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v)) * 255.0f + 0.5f) / 255.0f;
                        tx.store[(((size_t)l * tx.view.h + y + j) * tx.view.w + x + i) * comps + k] = v;
                    }
        }
    };
    void notifyChange(GPUSlot *) {}
};

template <class T> struct CPUTileStorage : TileStorage {
    int channels = 1;
    int getChannels() { return channels; }
    struct CPUSlot : TileStorage::Slot {
        T *data = nullptr;
        int size = 0;
    };
};

struct TileCache {
    ptr<TileStorage> storage;
    ptr<TileStorage> getStorage() { return storage; }
    struct Tile {
        TileStorage::Slot *data = nullptr;
        TileStorage::Slot *getData() { return data; }
    };
};

struct TileProducer {
    ptr<TileCache> cache;
    std::map<std::tuple<int, int, int>, TileCache::Tile> tiles;
    float rootQuadSize = 0.0f;
    int border = 2;
    virtual ~TileProducer() {}
    void init(ptr<TileCache> c, bool) { cache = c; }
    ptr<TileCache> getCache() { return cache; }
    TileCache::Tile *findTile(int level, int tx, int ty)
    {
        auto it = tiles.find(std::make_tuple(level, tx, ty));
        return it == tiles.end() ? nullptr : &it->second;
    }
    bool hasTile(int level, int tx, int ty) { return findTile(level, tx, ty) != nullptr; }
    float getRootQuadSize() { return rootQuadSize; }
    int getBorder() { return border; }
    int getId() { return 0; }
    // the layers: what TileProducer::doCreateTile draws is supplied by the harness
    // (layer_hook, run when the producer has layers)
    void (*layer_hook)(void *) = nullptr;
    void *layer_arg = nullptr;
    bool hasLayers() { return layer_hook != nullptr; }
    bool doCreateTile(int, int, int, TileStorage::Slot *)
    {
        if (layer_hook) layer_hook(layer_arg);
        return true;
    }
};

}  // namespace refgl
