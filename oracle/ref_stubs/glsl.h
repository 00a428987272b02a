// GLSL value types and built-in functions, for compiling the reference's fragment
// and vertex shaders as host C++ (oracle/ref_build.py rewrites each shader's text
// into a namespace that uses these).  TEST INFRASTRUCTURE ONLY: it runs the
// reference's own shader code on the CPU so that the oracle can be checked against
// it; nothing of the product includes it.
//
// Arithmetic: every float operation is one IEEE single-precision operation,
// rounded on its own (the recipe compiles with -ffp-contract=off and the rewrite
// gives every float literal an `f` suffix, so nothing is evaluated in double).
// Built-ins follow the formulas of the GLSL 4.30 specification, chapter 8:
//   mix(x, y, a) = x * (1 - a) + y * a
//   smoothstep(e0, e1, x): t = clamp((x - e0) / (e1 - e0), 0, 1), t * t * (3 - 2 * t)
//   mod(x, y) = x - y * floor(x / y),  fract(x) = x - floor(x)
//   length(v) = sqrt(dot(v, v)),  normalize(v) = v / length(v)
//   dot summed left to right, cross the usual determinant form.
// GLSL leaves the precision of division, sqrt and these built-ins to the
// implementation; here they are the correctly rounded operations.
//
// Matrices are column-major as in GLSL: m[c] is column c, matN(N*N scalars) fills
// column 0 first, m * v = m[0] * v[0] + m[1] * v[1] + ...
//
// Swizzles: the rewrite turns `v.x` into `v.c[0]`, a read of `v.xy` into
// `v.sw<0, 1>()` and a write `v.xy = e` into `v.swset<0, 1>() = e`.
//
// Samplers fetch the nearest texel (NEAREST filtering): texel floor(u * width) of
// each coordinate, clamped to [0, width - 1] (CLAMP_TO_EDGE) or wrapped (REPEAT);
// an array layer is the nearest integer to the third coordinate, clamped.  A
// texture with fewer than four components returns (r, g, b, a) with the missing
// ones 0 and alpha 1, as GL does.
#pragma once

#include <cmath>
#include <cstddef>
#include <initializer_list>
#include <type_traits>

namespace glsl {

template <int N> struct vec;

namespace detail {
struct Comps {
    float v[16];
    int n = 0;
};
inline void put(Comps &c, float f) { c.v[c.n++] = f; }
inline void put(Comps &c, double f) { c.v[c.n++] = (float)f; }
inline void put(Comps &c, int f) { c.v[c.n++] = (float)f; }
inline void put(Comps &c, bool f) { c.v[c.n++] = f ? 1.0f : 0.0f; }
template <int N> inline void put(Comps &c, const vec<N> &a)
{
    for (int k = 0; k < N; ++k) c.v[c.n++] = a.c[k];
}
}  // namespace detail

template <int N> struct SwzSet;

template <int N> struct vec {
    float c[N];
    vec()
    {
        for (int k = 0; k < N; ++k) c[k] = 0.0f;
    }
    // one scalar: every component; one wider vector: its first N components
    explicit vec(float s)
    {
        for (int k = 0; k < N; ++k) c[k] = s;
    }
    explicit vec(double s) : vec((float)s) {}
    explicit vec(int s) : vec((float)s) {}
    template <int M, typename = typename std::enable_if<(M > N)>::type> explicit vec(const vec<M> &w)
    {
        for (int k = 0; k < N; ++k) c[k] = w.c[k];
    }
    // several arguments: their components in order
    template <class A, class B, class... R> vec(const A &a, const B &b, const R &...r)
    {
        detail::Comps t;
        detail::put(t, a);
        detail::put(t, b);
        int dummy[] = {0, (detail::put(t, r), 0)...};
        (void)dummy;
        for (int k = 0; k < N; ++k) c[k] = t.v[k];
    }
    float &operator[](int k) { return c[k]; }
    float operator[](int k) const { return c[k]; }
    template <int... I> vec<sizeof...(I)> sw() const { return vec<sizeof...(I)>(c[I]...); }
    template <int... I> SwzSet<sizeof...(I)> swset() { return SwzSet<sizeof...(I)>(this->c, {I...}); }
    vec &operator+=(const vec &o)
    {
        for (int k = 0; k < N; ++k) c[k] = c[k] + o.c[k];
        return *this;
    }
    vec &operator-=(const vec &o)
    {
        for (int k = 0; k < N; ++k) c[k] = c[k] - o.c[k];
        return *this;
    }
    vec &operator*=(const vec &o)
    {
        for (int k = 0; k < N; ++k) c[k] = c[k] * o.c[k];
        return *this;
    }
    vec &operator/=(const vec &o)
    {
        for (int k = 0; k < N; ++k) c[k] = c[k] / o.c[k];
        return *this;
    }
    vec &operator+=(float s) { return *this += vec(s); }
    vec &operator-=(float s) { return *this -= vec(s); }
    vec &operator*=(float s) { return *this *= vec(s); }
    vec &operator/=(float s) { return *this /= vec(s); }
};

// single-component "vectors" are floats: vec<1> is never built by the rewrite
// (v.x is v.c[0]); sw<I>() with one index returns a one-component vec, which
// converts to float
template <> struct vec<1> {
    float c[1];
    vec() { c[0] = 0.0f; }
    explicit vec(float s) { c[0] = s; }
    operator float() const { return c[0]; }
};

template <int N> struct SwzSet {
    float *base;
    int idx[N];
    SwzSet(float *b, std::initializer_list<int> l) : base(b)
    {
        int k = 0;
        for (int i : l) idx[k++] = i;
    }
    SwzSet &operator=(const vec<N> &v)
    {
        for (int k = 0; k < N; ++k) base[idx[k]] = v.c[k];
        return *this;
    }
    SwzSet &operator=(float s) { return *this = vec<N>(s); }
    vec<N> get() const
    {
        vec<N> v;
        for (int k = 0; k < N; ++k) v.c[k] = base[idx[k]];
        return v;
    }
    SwzSet &operator+=(const vec<N> &v) { return *this = get() + v; }
    SwzSet &operator-=(const vec<N> &v) { return *this = get() - v; }
    SwzSet &operator*=(const vec<N> &v) { return *this = get() * v; }
    SwzSet &operator*=(float s) { return *this = get() * vec<N>(s); }
    SwzSet &operator/=(float s) { return *this = get() / vec<N>(s); }
};

typedef vec<2> vec2;
typedef vec<3> vec3;
typedef vec<4> vec4;

// integer vectors: only as uniforms whose components are read (v.x is v.c[0])
struct ivec4 {
    int c[4] = {0, 0, 0, 0};
};

#define GLSL_BINOP(OP)                                                                       \
    template <int N> inline vec<N> operator OP(const vec<N> &a, const vec<N> &b)            \
    {                                                                                        \
        vec<N> r;                                                                            \
        for (int k = 0; k < N; ++k) r.c[k] = a.c[k] OP b.c[k];                               \
        return r;                                                                            \
    }                                                                                        \
    template <int N> inline vec<N> operator OP(const vec<N> &a, float s)                    \
    {                                                                                        \
        vec<N> r;                                                                            \
        for (int k = 0; k < N; ++k) r.c[k] = a.c[k] OP s;                                    \
        return r;                                                                            \
    }                                                                                        \
    template <int N> inline vec<N> operator OP(float s, const vec<N> &a)                    \
    {                                                                                        \
        vec<N> r;                                                                            \
        for (int k = 0; k < N; ++k) r.c[k] = s OP a.c[k];                                    \
        return r;                                                                            \
    }
GLSL_BINOP(+)
GLSL_BINOP(-)
GLSL_BINOP(*)
GLSL_BINOP(/)
#undef GLSL_BINOP

template <int N> inline vec<N> operator-(const vec<N> &a)
{
    vec<N> r;
    for (int k = 0; k < N; ++k) r.c[k] = -a.c[k];
    return r;
}

template <int N> struct bvec {
    bool b[N];
};

template <int N> inline bvec<N> equal(const vec<N> &a, const vec<N> &b)
{
    bvec<N> r;
    for (int k = 0; k < N; ++k) r.b[k] = a.c[k] == b.c[k];
    return r;
}
template <int N> inline bool all(const bvec<N> &v)
{
    for (int k = 0; k < N; ++k)
        if (!v.b[k]) return false;
    return true;
}
template <int N> inline bool any(const bvec<N> &v)
{
    for (int k = 0; k < N; ++k)
        if (v.b[k]) return true;
    return false;
}

// ---- scalar built-ins --------------------------------------------------------
inline float floor(float x) { return std::floor(x); }
inline float ceil(float x) { return std::ceil(x); }
inline float fract(float x) { return x - std::floor(x); }
inline float abs(float x) { return std::fabs(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline float exp(float x) { return std::exp(x); }
inline float log(float x) { return std::log(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline float sin(float x) { return std::sin(x); }
inline float cos(float x) { return std::cos(x); }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
// GLSL min/max/clamp: min(x, y) = y < x ? y : x, max(x, y) = x < y ? y : x,
// clamp(x, lo, hi) = min(max(x, lo), hi)
inline float min(float x, float y) { return y < x ? y : x; }
inline float max(float x, float y) { return x < y ? y : x; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline float step(float e, float x) { return x < e ? 0.0f : 1.0f; }
inline float smoothstep(float e0, float e1, float x)
{
    float t = clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
inline float mod(float x, float y) { return x - y * floor(x / y); }
inline float dot(float a, float b) { return a * b; }
inline float length(float x) { return std::fabs(x); }

// ---- vector built-ins (component-wise unless stated) ----------------------------
#define GLSL_UNARY(F)                                                                       \
    template <int N> inline vec<N> F(const vec<N> &a)                                       \
    {                                                                                       \
        vec<N> r;                                                                           \
        for (int k = 0; k < N; ++k) r.c[k] = F(a.c[k]);                                     \
        return r;                                                                           \
    }
GLSL_UNARY(floor)
GLSL_UNARY(ceil)
GLSL_UNARY(fract)
GLSL_UNARY(abs)
GLSL_UNARY(sqrt)
GLSL_UNARY(inversesqrt)
GLSL_UNARY(exp)
GLSL_UNARY(log)
GLSL_UNARY(sin)
GLSL_UNARY(cos)
GLSL_UNARY(sign)
#undef GLSL_UNARY

#define GLSL_BINARY(F)                                                                      \
    template <int N> inline vec<N> F(const vec<N> &a, const vec<N> &b)                      \
    {                                                                                       \
        vec<N> r;                                                                           \
        for (int k = 0; k < N; ++k) r.c[k] = F(a.c[k], b.c[k]);                             \
        return r;                                                                           \
    }                                                                                       \
    template <int N> inline vec<N> F(const vec<N> &a, float b)                              \
    {                                                                                       \
        vec<N> r;                                                                           \
        for (int k = 0; k < N; ++k) r.c[k] = F(a.c[k], b);                                  \
        return r;                                                                           \
    }
GLSL_BINARY(min)
GLSL_BINARY(max)
GLSL_BINARY(mod)
GLSL_BINARY(pow)
#undef GLSL_BINARY

template <int N> inline vec<N> step(const vec<N> &e, const vec<N> &x)
{
    vec<N> r;
    for (int k = 0; k < N; ++k) r.c[k] = step(e.c[k], x.c[k]);
    return r;
}
template <int N> inline vec<N> step(float e, const vec<N> &x) { return step(vec<N>(e), x); }
template <int N> inline vec<N> clamp(const vec<N> &x, const vec<N> &lo, const vec<N> &hi)
{
    vec<N> r;
    for (int k = 0; k < N; ++k) r.c[k] = clamp(x.c[k], lo.c[k], hi.c[k]);
    return r;
}
template <int N> inline vec<N> clamp(const vec<N> &x, float lo, float hi) { return clamp(x, vec<N>(lo), vec<N>(hi)); }
template <int N> inline vec<N> mix(const vec<N> &x, const vec<N> &y, const vec<N> &a)
{
    vec<N> r;
    for (int k = 0; k < N; ++k) r.c[k] = mix(x.c[k], y.c[k], a.c[k]);
    return r;
}
template <int N> inline vec<N> mix(const vec<N> &x, const vec<N> &y, float a) { return mix(x, y, vec<N>(a)); }
template <int N> inline vec<N> smoothstep(const vec<N> &e0, const vec<N> &e1, const vec<N> &x)
{
    vec<N> r;
    for (int k = 0; k < N; ++k) r.c[k] = smoothstep(e0.c[k], e1.c[k], x.c[k]);
    return r;
}
template <int N> inline vec<N> smoothstep(float e0, float e1, const vec<N> &x)
{
    return smoothstep(vec<N>(e0), vec<N>(e1), x);
}
template <int N> inline float dot(const vec<N> &a, const vec<N> &b)
{
    float s = a.c[0] * b.c[0];
    for (int k = 1; k < N; ++k) s = s + a.c[k] * b.c[k];
    return s;
}
template <int N> inline float length(const vec<N> &a) { return sqrt(dot(a, a)); }
template <int N> inline float distance(const vec<N> &a, const vec<N> &b) { return length(a - b); }
template <int N> inline vec<N> normalize(const vec<N> &a) { return a / length(a); }
inline vec3 cross(const vec3 &a, const vec3 &b)
{
    return vec3(a.c[1] * b.c[2] - a.c[2] * b.c[1], a.c[2] * b.c[0] - a.c[0] * b.c[2], a.c[0] * b.c[1] - a.c[1] * b.c[0]);
}

// ---- matrices -------------------------------------------------------------------
template <int N> struct mat {
    vec<N> col[N];
    mat() {}
    explicit mat(float d)  // d on the diagonal
    {
        for (int c = 0; c < N; ++c) col[c].c[c] = d;
    }
    template <int M, typename = typename std::enable_if<(M > N)>::type> explicit mat(const mat<M> &m)
    {
        for (int c = 0; c < N; ++c)
            for (int r = 0; r < N; ++r) col[c].c[r] = m.col[c].c[r];
    }
    template <class A, class B, class... R> mat(const A &a, const B &b, const R &...r)
    {
        detail::Comps t;
        detail::put(t, a);
        detail::put(t, b);
        int dummy[] = {0, (detail::put(t, r), 0)...};
        (void)dummy;
        for (int c = 0; c < N; ++c)
            for (int k = 0; k < N; ++k) col[c].c[k] = t.v[c * N + k];
    }
    vec<N> &operator[](int c) { return col[c]; }
    const vec<N> &operator[](int c) const { return col[c]; }
};
typedef mat<3> mat3;
typedef mat<4> mat4;

template <int N> inline vec<N> operator*(const mat<N> &m, const vec<N> &v)
{
    vec<N> r = m.col[0] * v.c[0];
    for (int c = 1; c < N; ++c) r = r + m.col[c] * v.c[c];
    return r;
}
template <int N> inline vec<N> operator*(const vec<N> &v, const mat<N> &m)
{
    vec<N> r;
    for (int c = 0; c < N; ++c) r.c[c] = dot(v, m.col[c]);
    return r;
}
template <int N> inline mat<N> operator*(const mat<N> &a, const mat<N> &b)
{
    mat<N> r;
    for (int c = 0; c < N; ++c) r.col[c] = a * b.col[c];
    return r;
}

// ---- samplers ---------------------------------------------------------------------
struct Texture {
    const float *data = nullptr;  // texel (i, j) of layer l at ((l * h + j) * w + i) * comps
    int w = 0, h = 0, layers = 1, comps = 4;
    bool repeat = false;
};
struct sampler2D {
    const Texture *t = nullptr;
};
struct sampler2DArray {
    const Texture *t = nullptr;
};

namespace detail {
inline int texel(float u, int n, bool repeat)
{
    int i = (int)std::floor(u * (float)n);
    if (repeat) return ((i % n) + n) % n;
    return i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
}
inline vec4 fetch(const Texture &t, int i, int j, int l)
{
    vec4 r(0.0f, 0.0f, 0.0f, 1.0f);
    const float *p = t.data + (((size_t)l * t.h + j) * t.w + i) * t.comps;
    for (int k = 0; k < t.comps; ++k) r.c[k] = p[k];
    return r;
}
inline int layer_of(const Texture &t, float z)
{
    int l = (int)std::floor(z + 0.5f);
    return l < 0 ? 0 : (l > t.layers - 1 ? t.layers - 1 : l);
}
}  // namespace detail

inline vec4 textureLod(const sampler2D &s, const vec2 &uv, float)
{
    const Texture &t = *s.t;
    return detail::fetch(t, detail::texel(uv.c[0], t.w, t.repeat), detail::texel(uv.c[1], t.h, t.repeat), 0);
}
inline vec4 texture(const sampler2D &s, const vec2 &uv) { return textureLod(s, uv, 0.0f); }
inline vec4 textureLod(const sampler2DArray &s, const vec3 &uvl, float)
{
    const Texture &t = *s.t;
    return detail::fetch(t, detail::texel(uvl.c[0], t.w, t.repeat), detail::texel(uvl.c[1], t.h, t.repeat),
                         detail::layer_of(t, uvl.c[2]));
}
inline vec4 texture(const sampler2DArray &s, const vec3 &uvl) { return textureLod(s, uvl, 0.0f); }

}  // namespace glsl
