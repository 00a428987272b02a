"""The reference's GLSL shaders as host C++ -- TEST INFRASTRUCTURE ONLY (part of the
oracle/_ref build in oracle/ref_build.py).

A shader's text, read from the reference tree at build time, is rewritten
mechanically so that it compiles as C++ against oracle/ref_stubs/glsl.h:

* one stage is kept (the ``#ifdef _FRAGMENT_`` or ``#ifdef _VERTEX_`` block; other
  preprocessor lines stay for the C++ preprocessor);
* storage qualifiers of global declarations are dropped (``uniform``, ``in``,
  ``out``, ``layout(...)``): uniforms, varyings and outputs become variables of the
  shader's namespace, which the harness sets and reads;
* array constructors ``T[N](a, b, ...)`` become brace lists;
* every floating literal gets an ``f`` suffix (GLSL literals are single precision);
* swizzles become member accesses: ``v.x`` -> ``v.c[0]``, a read ``v.xy`` ->
  ``v.sw<0, 1>()``, a write ``v.xy = e`` -> ``v.swset<0, 1>() = e``;
* ``void main()`` becomes ``void shader_main()``.

Nothing else of the text changes: the statements, their order and their
arithmetic are the reference's.  Each shader goes into its own namespace nested in
``glsl`` (so that the built-ins of glsl.h are found before the C library's).
"""
import re

_SWZ = {}
for _set in ("xyzw", "rgba", "stpq"):
    for _i, _c in enumerate(_set):
        _SWZ[_c] = _i

_TYPES = {"float": "U_FLOAT", "int": "U_INT", "vec2": "U_VEC2", "vec3": "U_VEC3", "vec4": "U_VEC4",
          "ivec4": "U_IVEC4", "mat3": "U_MAT3", "mat4": "U_MAT4", "sampler2D": "U_SAMPLER2D",
          "sampler2DArray": "U_SAMPLER2DARRAY"}


def strip_comments(src):
    """Comments out, line structure kept."""
    out, i, n = [], 0, len(src)
    while i < n:
        if src.startswith("/*", i):
            j = src.find("*/", i + 2)
            j = n if j < 0 else j + 2
            out.append("\n" * src.count("\n", i, j))
            i = j
        elif src.startswith("//", i):
            j = src.find("\n", i)
            i = n if j < 0 else j
        else:
            out.append(src[i])
            i += 1
    return "".join(out)


def select_stage(src, stage):
    """The lines outside every stage block plus those of `stage`'s blocks."""
    out, stack = [], []   # stack entries: ("stage", keep) or ("other", None)
    for line in src.splitlines():
        s = line.strip()
        m = re.match(r"#\s*ifdef\s+(_VERTEX_|_FRAGMENT_|_GEOMETRY_)\b", s)
        keep = all(k for kind, k in stack if kind == "stage")
        if m:
            stack.append(("stage", m.group(1) == stage))
            continue
        if re.match(r"#\s*(if|ifdef|ifndef)\b", s):
            stack.append(("other", None))
        elif re.match(r"#\s*endif\b", s):
            if not stack:
                raise RuntimeError("unbalanced #endif")
            kind, _ = stack.pop()
            if kind == "stage":
                continue
        elif re.match(r"#\s*(else|elif)\b", s) and stack and stack[-1][0] == "stage":
            raise RuntimeError("#else of a stage block is not handled")
        elif re.match(r"#\s*version\b", s):
            continue
        if keep:
            out.append(line)
    return "\n".join(out) + "\n"


def _match_paren(text, i):
    """Index of the parenthesis closing the one at text[i]."""
    depth = 0
    for k in range(i, len(text)):
        if text[k] == "(":
            depth += 1
        elif text[k] == ")":
            depth -= 1
            if depth == 0:
                return k
    raise RuntimeError("unbalanced parentheses")


def _array_constructors(text):
    pat = re.compile(r"\b(?:mat[234]|vec[234]|float|int)\s*\[\s*\d*\s*\]\s*\(")
    while True:
        m = pat.search(text)
        if not m:
            return text
        open_at = m.end() - 1
        close_at = _match_paren(text, open_at)
        text = text[:m.start()] + "{" + text[open_at + 1:close_at] + "}" + text[close_at + 1:]


def _globals(text):
    """Qualifiers of global declarations dropped; returns (text, [(type, name), ...]
    of the uniforms, [(type, name)] of the other globals)."""
    out, uniforms, others, depth = [], [], [], 0
    for line in text.splitlines():
        if depth == 0:
            m = re.match(r"\s*(?:layout\s*\([^)]*\)\s*)?(uniform|in|out)\s+(\w+)\s+(\w+)\s*;", line)
            if m:
                (uniforms if m.group(1) == "uniform" else others).append((m.group(2), m.group(3)))
                line = "%s %s;" % (m.group(2), m.group(3))
        depth += line.count("{") - line.count("}")
        out.append(line)
    return "\n".join(out) + "\n", uniforms, others


_FLOAT_LIT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+)(?![\w.])")


def _float_literals(text):
    return _FLOAT_LIT.sub(lambda m: m.group(1) + "f", text)


_SWIZZLE = re.compile(r"(?<=[\w)\]])\.([xyzwrgbastpq]{1,4})(?!\w)")


def _swizzles(text):
    def rep(m):
        idx = [_SWZ[c] for c in m.group(1)]
        if len(set(m.group(1)) & set("xyzw")) and len(set(m.group(1)) & set("rgbastpq")):
            raise RuntimeError("mixed swizzle sets: %s" % m.group(0))
        if len(idx) == 1:
            return ".c[%d]" % idx[0]
        rest = text[m.end():]
        if re.match(r"\s*(=(?!=)|\+=|-=|\*=|/=)", rest):
            return ".swset<%s>()" % ", ".join(map(str, idx))
        return ".sw<%s>()" % ", ".join(map(str, idx))
    return _SWIZZLE.sub(rep, text)


def shader_to_cpp(src, ns, stage="_FRAGMENT_", defines=()):
    """(C++ text of namespace glsl::<ns>, uniforms [(type, name)], other globals)."""
    text = select_stage(strip_comments(src), stage)
    if re.search(r"\b(inout|out)\s+\w+\s+\w+\s*[,)]", text):
        raise RuntimeError("out parameters are not handled")
    text, uniforms, others = _globals(text)
    text = _array_constructors(text)
    text = _float_literals(text)
    text = _swizzles(text)
    text, n = re.subn(r"\bvoid\s+main\s*\(\s*\)", "void shader_main()", text)
    if n != 1:
        raise RuntimeError("no main() in the %s stage" % stage)
    defs = "".join("#define %s\n" % d for d in defines)
    undefs = "".join("#undef %s\n" % d for d in defines)
    body = ("namespace glsl {\nnamespace %s {\n%sfloat gl_FragDepth;\nvec4 gl_Position, gl_FragCoord;\n%s\n"
            "}  // namespace %s\n}  // namespace glsl\n%s" % (ns, defs, text, ns, undefs))
    for t, _ in uniforms:
        if t not in _TYPES:
            raise RuntimeError("uniform type %s is not handled" % t)
    return body, uniforms, others


def uniform_table(ns, uniforms):
    """A refgl::UniformEntry table naming the shader's uniforms."""
    rows = ["    {\"%s\", refgl::%s, &glsl::%s::%s}," % (name, _TYPES[t], ns, name) for t, name in uniforms]
    return ("static refgl::UniformEntry %s_uniforms[] = {\n%s\n    {nullptr, refgl::U_FLOAT, nullptr}};\n"
            % (ns, "\n".join(rows)))


def quad_runner(ns, unit=False):
    """drawQuad of a full-screen quad: the fragment shader at every pixel centre, with
    st the centre in pixels, or divided by the viewport size when `unit` (the vertex
    shaders make st = (vertex.xy * 0.5 + 0.5) * tileWidth or vertex.xy * 0.5 + 0.5)."""
    sx = "((float)i + 0.5f) / (float)fb.w" if unit else "(float)i + 0.5f"
    sy = "((float)j + 0.5f) / (float)fb.h" if unit else "(float)j + 0.5f"
    return """static void %(ns)s_run(refgl::FrameBuffer &fb)
{
    for (int j = 0; j < fb.h; ++j)
        for (int i = 0; i < fb.w; ++i) {
            glsl::%(ns)s::st = glsl::vec2(%(sx)s, %(sy)s);
            glsl::%(ns)s::gl_FragCoord = glsl::vec4((float)i + 0.5f, (float)j + 0.5f, 0.0f, 1.0f);
            glsl::%(ns)s::shader_main();
            fb.write(i, j, glsl::%(ns)s::data.c);
        }
}
""" % {"ns": ns, "sx": sx, "sy": sy}


def fragment_call(ns, has_st):
    """One fragment at the interpolated varying st: data and gl_FragDepth (NaN when
    the shader leaves it unwritten)."""
    return """static void %(ns)s_fragment(float sx, float sy, float *data, float *depth)
{
    %(st)s
    glsl::%(ns)s::gl_FragDepth = std::nanf("");
    glsl::%(ns)s::shader_main();
    for (int k = 0; k < 4; ++k) data[k] = glsl::%(ns)s::data.c[k];
    *depth = glsl::%(ns)s::gl_FragDepth;
}
""" % {"ns": ns, "st": ("glsl::%s::st = glsl::vec2(sx, sy);" % ns) if has_st else "(void)sx; (void)sy;"}
