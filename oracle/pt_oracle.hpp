// pt_oracle.hpp - CPU restatement of GLSL-PathTracer's per-pixel path tracer.
//
// TEST INFRASTRUCTURE ONLY.  This is the oracle the CUDA kernels are checked
// against (and the timed CPU baseline of bench.py).  Nothing in the product
// library links, loads or calls it.
//
// Each function restates one function of the reference's GLSL (paths are
// relative to the reference project) in plain C++, templated on the
// arithmetic type R (float: the timed baseline; double: FP64 validation).
// The reference's shaders run only under OpenGL, so this restatement is the
// only CPU form of the shading math; it is pinned against the reference's own
// shader source compiled as C++ (recipe in oracle/ref_glsl/), see the golden
// fixtures under tests/golden/.
//
// GL semantics the shaders rely on and that are restated here:
//   * texelFetch: exact fetch; texture(): bilinear, GL_REPEAT wrap, texel
//     centres at (i+0.5)/size (envmap: Renderer.cpp:213-218).
//   * uvec4(vec2) truncates gl_FragCoord (pixel + 0.5 -> pixel).
//   * min/max with a NaN operand return the other operand (IEEE fmin/fmax).
//   * Function arguments are evaluated left to right (GLSL spec), which fixes
//     the order of rand() calls such as SampleHG(..., rand(), rand()).
// Compile with -ffp-contract=off so float results are reproducible.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

#include "../include/pt_cuda.h"

namespace orc {

// ---------------------------------------------------------------- constants
// common/globals.glsl:25-44
template <class R> struct K {
    static constexpr R PI = R(3.14159265358979323);
    static constexpr R INV_PI = R(0.31830988618379067);
    static constexpr R TWO_PI = R(6.28318530717958648);
    static constexpr R INV_TWO_PI = R(0.15915494309189533);
    static constexpr R INV_4_PI = R(0.07957747154594766);
    static constexpr R EPS = R(0.0003);
    static constexpr R INF = R(1000000.0);
};
enum { QUAD_LIGHT = 0, SPHERE_LIGHT = 1, DISTANT_LIGHT = 2 };
enum { ALPHA_MODE_OPAQUE = 0, ALPHA_MODE_BLEND = 1, ALPHA_MODE_MASK = 2 };
enum { MEDIUM_NONE = 0, MEDIUM_ABSORB = 1, MEDIUM_SCATTER = 2, MEDIUM_EMISSIVE = 3 };

// ------------------------------------------------------------------ vectors
template <class R> struct V2 { R x, y; };
template <class R> struct V3 {
    R x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(R a) : x(a), y(a), z(a) {}
    V3(R a, R b, R c) : x(a), y(b), z(c) {}
    R operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class R> inline V3<R> operator+(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class R> inline V3<R> operator-(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class R> inline V3<R> operator*(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class R> inline V3<R> operator/(V3<R> a, V3<R> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class R> inline V3<R> operator*(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <class R> inline V3<R> operator*(R s, V3<R> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class R> inline V3<R> operator/(V3<R> a, R s) { return {a.x / s, a.y / s, a.z / s}; }
template <class R> inline V3<R> operator-(V3<R> a) { return {-a.x, -a.y, -a.z}; }
template <class R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class R> inline V3<R> cross(V3<R> a, V3<R> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class R> inline R length(V3<R> a) { return std::sqrt(dot(a, a)); }
template <class R> inline V3<R> normalize(V3<R> a) { return a / length(a); }
template <class R> inline R fminR(R a, R b) { return std::fmin(a, b); }
template <class R> inline R fmaxR(R a, R b) { return std::fmax(a, b); }
template <class R> inline R clampR(R x, R lo, R hi) { return fminR(fmaxR(x, lo), hi); }
template <class R> inline R mixR(R a, R b, R t) { return a * (R(1) - t) + b * t; }
template <class R> inline V3<R> mix3(V3<R> a, V3<R> b, R t) {
    return {mixR(a.x, b.x, t), mixR(a.y, b.y, t), mixR(a.z, b.z, t)};
}
template <class R> inline V3<R> vmin(V3<R> a, V3<R> b) { return {fminR(a.x, b.x), fminR(a.y, b.y), fminR(a.z, b.z)}; }
template <class R> inline V3<R> vmax(V3<R> a, V3<R> b) { return {fmaxR(a.x, b.x), fmaxR(a.y, b.y), fmaxR(a.z, b.z)}; }
template <class R> inline V3<R> vexp(V3<R> a) { return {std::exp(a.x), std::exp(a.y), std::exp(a.z)}; }
template <class R> inline V3<R> vpow(V3<R> a, R e) { return {std::pow(a.x, e), std::pow(a.y, e), std::pow(a.z, e)}; }
// GLSL reflect(I, N) = I - 2 dot(N, I) N
template <class R> inline V3<R> reflectR(V3<R> I, V3<R> N) { return I - (R(2) * dot(N, I)) * N; }
// GLSL refract(I, N, eta)
template <class R> inline V3<R> refractR(V3<R> I, V3<R> N, R eta) {
    R d = dot(N, I);
    R k = R(1) - eta * eta * (R(1) - d * d);
    if (k < R(0)) return V3<R>(R(0));
    return eta * I - (eta * d + std::sqrt(k)) * N;
}

// ---------------------------------------------------------------------- RNG
// common/globals.glsl:149-166 (PCG4D hash by Jarzynski & Olano, as used there)
struct Rng {
    uint32_t s[4];
    void init(uint32_t px, uint32_t py, uint32_t frame) {
        s[0] = px; s[1] = py; s[2] = frame; s[3] = px + py;
    }
    void pcg4d() {
        for (int i = 0; i < 4; ++i) s[i] = s[i] * 1664525u + 1013904223u;
        s[0] += s[1] * s[3]; s[1] += s[2] * s[0]; s[2] += s[0] * s[1]; s[3] += s[1] * s[2];
        for (int i = 0; i < 4; ++i) s[i] ^= (s[i] >> 16u);
        s[0] += s[1] * s[3]; s[1] += s[2] * s[0]; s[2] += s[0] * s[1]; s[3] += s[1] * s[2];
    }
    // float(seed.x) / float(0xffffffffu), computed in float in every R
    float next() {
        pcg4d();
        return float(s[0]) / float(0xffffffffu);
    }
};

template <class R> inline R Luminance(V3<R> c) {  // globals.glsl:173-176
    return R(0.212671) * c.x + R(0.715160) * c.y + R(0.072169) * c.z;
}

// ------------------------------------------------------------------- scene
template <class R> struct Mat4c { R c[4][4]; };  // GLSL layout c[column][row]

// Inverse of the GLSL matrix mat4(data[0], data[1], data[2], data[3]) built
// from a Mat4 (src/math/Mat4.h): computed in double by cofactors and rounded
// to R, so two independent implementations agree to the last bit.
template <class R> inline Mat4c<R> InverseOfInstance(const float* d16) {
    double m[16];  // m[col*4+row] = data[col][row] (GLSL column-major)
    for (int i = 0; i < 16; ++i) m[i] = d16[i];
    double inv[16];
    inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
    inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
    inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
    inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
    inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
    inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
    inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
    inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
    inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
    inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
    inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
    inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
    inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
    inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
    inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
    inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
    double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
    Mat4c<R> out;
    for (int col = 0; col < 4; ++col)
        for (int row = 0; row < 4; ++row) out.c[col][row] = R(inv[col * 4 + row] / det);
    return out;
}

// GLSL mat4 * vec4 with the sum taken in column order.
template <class R> inline V3<R> MulPoint(const Mat4c<R>& m, V3<R> p, R w) {
    V3<R> r;
    r.x = ((m.c[0][0] * p.x + m.c[1][0] * p.y) + m.c[2][0] * p.z) + m.c[3][0] * w;
    r.y = ((m.c[0][1] * p.x + m.c[1][1] * p.y) + m.c[2][1] * p.z) + m.c[3][1] * w;
    r.z = ((m.c[0][2] * p.x + m.c[1][2] * p.y) + m.c[2][2] * p.z) + m.c[3][2] * w;
    return r;
}

// Per-instance shading matrices: mat3(transform) and
// transpose(inverse(mat3(transform))) (closest_hit.glsl:246,261-262),
// inverse computed in double and rounded to R.
template <class R> struct InstMats {
    Mat4c<R> inv;      // inverse(transMat)
    R m3[3][3];        // mat3(transform), [col][row]
    R nrm[3][3];       // transpose(inverse(mat3(transform))), [col][row]
};

template <class R> inline InstMats<R> MakeInstMats(const float* d16) {
    InstMats<R> im;
    im.inv = InverseOfInstance<R>(d16);
    double a[3][3];  // a[col][row]
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) {
            a[c][r] = d16[c * 4 + r];
            im.m3[c][r] = R(d16[c * 4 + r]);
        }
    // inverse of 3x3 (column-major a), then transpose
    double A = a[0][0], B = a[1][0], C = a[2][0];  // row 0
    double D = a[0][1], E = a[1][1], F = a[2][1];  // row 1
    double G = a[0][2], H = a[1][2], I = a[2][2];  // row 2
    double c00 = E * I - F * H, c01 = -(D * I - F * G), c02 = D * H - E * G;
    double c10 = -(B * I - C * H), c11 = A * I - C * G, c12 = -(A * H - B * G);
    double c20 = B * F - C * E, c21 = -(A * F - C * D), c22 = A * E - B * D;
    double det = A * c00 + B * c01 + C * c02;
    // inverse(row r, col c) = cof(c, r)/det ; transpose -> nrm(row r, col c) = cof(r, c)/det
    double cof[3][3] = {{c00, c01, c02}, {c10, c11, c12}, {c20, c21, c22}};
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) im.nrm[c][r] = R(cof[r][c] / det);
    return im;
}

template <class R> inline V3<R> Mul3(const R m[3][3], V3<R> v) {
    return {(m[0][0] * v.x + m[1][0] * v.y) + m[2][0] * v.z,
            (m[0][1] * v.x + m[1][1] * v.y) + m[2][1] * v.z,
            (m[0][2] * v.x + m[1][2] * v.y) + m[2][2] * v.z};
}

// Options that the reference compiles into the shader as #defines
// (Renderer.cpp:400-476) plus the uniforms (common/uniforms.glsl:25-53).
struct Flags {
    bool envmap, lights, rr, uniform_light, opengl_normalmap, hide_emitters;
    bool background, transparent_background, alpha_test, roughness_mollification;
    bool medium, vol_mis;
    int rr_depth, max_depth;
};

template <class R> struct Scene {
    const pt_scene_desc* d;
    Flags f;
    int num_lights;
    std::vector<InstMats<R>> inst;
    R env_w, env_h, env_total, env_intensity, env_rot, mollify_amt;
    V3<R> uniform_light_col;
    bool has_textures;
    bool cull = false;  // count work with tmax culling (mode 1) instead of the reference's traversal

    V3<R> node_min(int i) const { const float* p = d->bvh_nodes + 9 * (size_t)i; return {R(p[0]), R(p[1]), R(p[2])}; }
    V3<R> node_max(int i) const { const float* p = d->bvh_nodes + 9 * (size_t)i; return {R(p[3]), R(p[4]), R(p[5])}; }
    void node_lrl(int i, int& l, int& r, int& leaf) const {
        const float* p = d->bvh_nodes + 9 * (size_t)i + 6;
        l = int(p[0]); r = int(p[1]); leaf = int(p[2]);
    }
    V3<R> vtx(int i, R& w) const { const float* p = d->vertices_uvx + 4 * (size_t)i; w = R(p[3]); return {R(p[0]), R(p[1]), R(p[2])}; }
    V3<R> nrm(int i, R& w) const { const float* p = d->normals_uvy + 4 * (size_t)i; w = R(p[3]); return {R(p[0]), R(p[1]), R(p[2])}; }
    const float* mat(int id) const { return d->materials + 32 * (size_t)id; }
    const float* light(int id) const { return d->lights + 15 * (size_t)id; }
};

inline Flags MakeFlags(const pt_scene_desc* d, const pt_render_options* o) {
    Flags f{};
    f.envmap = o->enable_envmap && d->envmap_rgb != nullptr;
    f.lights = d->num_lights > 0;
    f.rr = o->enable_rr != 0;
    f.rr_depth = o->rr_depth;
    f.uniform_light = o->enable_uniform_light != 0;
    f.opengl_normalmap = o->opengl_normal_map != 0;
    f.hide_emitters = o->hide_emitters != 0;
    f.background = o->enable_background != 0;
    f.transparent_background = o->transparent_background != 0;
    f.roughness_mollification = o->enable_roughness_mollification != 0;
    f.vol_mis = o->enable_volume_mis != 0;
    f.max_depth = o->max_depth;
    for (int i = 0; i < d->num_materials; ++i) {
        if (int(d->materials[32 * i + 29]) != ALPHA_MODE_OPAQUE) f.alpha_test = true;  // Renderer.cpp:443-450
        if (int(d->materials[32 * i + 18]) != MEDIUM_NONE) f.medium = true;            // Renderer.cpp:455-461
    }
    return f;
}

template <class R> inline void MakeScene(Scene<R>& s, const pt_scene_desc* d, const pt_render_options* o) {
    s.d = d;
    s.f = MakeFlags(d, o);
    s.num_lights = d->num_lights;
    s.inst.resize(d->num_instances);
    for (int i = 0; i < d->num_instances; ++i) s.inst[i] = MakeInstMats<R>(d->transforms + 16 * (size_t)i);
    s.env_w = R(d->envmap_width);
    s.env_h = R(d->envmap_height);
    s.env_total = R(d->envmap_total_sum);
    s.env_intensity = R(o->envmap_intensity);
    s.env_rot = R(o->envmap_rot / 360.0f);  // Renderer.cpp:778
    s.mollify_amt = R(o->roughness_mollification_amt);
    s.uniform_light_col = V3<R>(R(o->uniform_light_col[0]), R(o->uniform_light_col[1]), R(o->uniform_light_col[2]));
    s.has_textures = d->num_textures > 0 && d->texture_maps != nullptr;
}

// ------------------------------------------------------------- structs
// common/globals.glsl:46-139
template <class R> struct Ray { V3<R> origin, direction; };
template <class R> struct Medium { int type = 0; R density = 0; V3<R> color; R anisotropy = 0; };
template <class R> struct Material {
    V3<R> baseColor; R opacity = 1; int alphaMode = 0; R alphaCutoff = 0;
    V3<R> emission; R anisotropic = 0, metallic = 0, roughness = 0, subsurface = 0, specularTint = 0;
    R sheen = 0, sheenTint = 0, clearcoat = 0, clearcoatRoughness = 0, specTrans = 0, ior = 1, ax = 0, ay = 0;
    Medium<R> medium;
};
template <class R> struct State {
    int depth = 0; R eta = 0; R hitDist = 0;
    V3<R> fhp, normal, ffnormal, tangent, bitangent;
    bool isEmitter = false;
    V2<R> texCoord{0, 0};
    int matID = 0;
    Material<R> mat;
    Medium<R> medium;
};
template <class R> struct ScatterSampleRec { V3<R> L, f; R pdf = 0; };
template <class R> struct LightSampleRec { V3<R> normal, emission, direction; R dist = 0, pdf = 0; };
template <class R> struct Light { V3<R> position, emission, u, v; R radius, area, type; };

// Counters of executed ray queries and traversal work.
struct Counters {
    uint64_t closest = 0, shadow = 0, nodes = 0, tris = 0, overflow = 0, tri_hits = 0;
    uint64_t nodes_any = 0, tris_any = 0;  // the part of nodes / tris done by any-hit queries
    uint64_t inner = 0;                    // interior-node visits (two slab tests each) of all queries
    uint64_t truncated = 0;                // paths ended at PT_MAX_PATH_ITERATIONS
};

// ------------------------------------------------------------ textures
// texture(sampler2D, uv): bilinear, GL_REPEAT, on an RGB float image.
template <class R> inline V3<R> SampleRGBRepeat(const float* img, int w, int h, R u, R v) {
    R x = u * R(w) - R(0.5), y = v * R(h) - R(0.5);
    R fx = std::floor(x), fy = std::floor(y);
    R ax = x - fx, ay = y - fy;
    long ix = (long)fx, iy = (long)fy;
    auto wrap = [](long i, int n) { long m = i % n; return m < 0 ? m + n : m; };
    long x0 = wrap(ix, w), x1 = wrap(ix + 1, w), y0 = wrap(iy, h), y1 = wrap(iy + 1, h);
    auto px = [&](long xx, long yy) {
        const float* p = img + 3 * ((size_t)yy * w + xx);
        return V3<R>(R(p[0]), R(p[1]), R(p[2]));
    };
    V3<R> a = px(x0, y0) * (R(1) - ax) + px(x1, y0) * ax;
    V3<R> b = px(x0, y1) * (R(1) - ax) + px(x1, y1) * ax;
    return a * (R(1) - ay) + b * ay;
}

// texture(sampler2DArray, vec3(uv, layer)) on the RGBA8 texture array
// (Renderer.cpp:200-208: GL_LINEAR, default GL_REPEAT).  With no texture
// bound the GL sampler returns (0,0,0,1).
template <class R> inline void SampleTexArray(const Scene<R>& s, V2<R> uv, R layerf, R out[4]) {
    if (!s.has_textures) { out[0] = out[1] = out[2] = R(0); out[3] = R(1); return; }
    const pt_scene_desc* d = s.d;
    int layer = (int)std::floor(layerf + R(0.5));
    layer = std::min(std::max(layer, 0), d->num_textures - 1);
    int w = d->tex_width, h = d->tex_height;
    const uint8_t* base = d->texture_maps + (size_t)layer * w * h * 4;
    R x = uv.x * R(w) - R(0.5), y = uv.y * R(h) - R(0.5);
    R fx = std::floor(x), fy = std::floor(y);
    R ax = x - fx, ay = y - fy;
    auto wrap = [](long i, int n) { long m = i % n; return m < 0 ? m + n : m; };
    long x0 = wrap((long)fx, w), x1 = wrap((long)fx + 1, w), y0 = wrap((long)fy, h), y1 = wrap((long)fy + 1, h);
    for (int c = 0; c < 4; ++c) {
        auto t = [&](long xx, long yy) { return R(base[4 * ((size_t)yy * w + xx) + c]) / R(255); };
        R a = t(x0, y0) * (R(1) - ax) + t(x1, y0) * ax;
        R b = t(x0, y1) * (R(1) - ax) + t(x1, y1) * ax;
        out[c] = a * (R(1) - ay) + b * ay;
    }
}

// ------------------------------------------------------------ intersection
// common/intersection.glsl:25-45
template <class R> inline R SphereIntersect(R rad, V3<R> pos, const Ray<R>& r) {
    V3<R> op = pos - r.origin;
    R eps = R(0.001);
    R b = dot(op, r.direction);
    R det = b * b - dot(op, op) + rad * rad;
    if (det < R(0)) return K<R>::INF;
    det = std::sqrt(det);
    R t1 = b - det;
    if (t1 > eps) return t1;
    R t2 = b + det;
    if (t2 > eps) return t2;
    return K<R>::INF;
}

// common/intersection.glsl:47-66
template <class R> inline R RectIntersect(V3<R> pos, V3<R> u, V3<R> v, V3<R> n, R planew, const Ray<R>& r) {
    R dt = dot(r.direction, n);
    R t = (planew - dot(n, r.origin)) / dt;
    if (t > K<R>::EPS) {
        V3<R> p = r.origin + r.direction * t;
        V3<R> vi = p - pos;
        R a1 = dot(u, vi);
        if (a1 >= R(0) && a1 <= R(1)) {
            R a2 = dot(v, vi);
            if (a2 >= R(0) && a2 <= R(1)) return t;
        }
    }
    return K<R>::INF;
}

// common/intersection.glsl:68-82 ; t0/t1 also returned for tmax culling.
template <class R> inline R AABBIntersect(V3<R> mn, V3<R> mx, const Ray<R>& r, R* t0out = nullptr) {
    V3<R> invDir = V3<R>(R(1)) / r.direction;
    V3<R> f = (mx - r.origin) * invDir;
    V3<R> n = (mn - r.origin) * invDir;
    V3<R> tmax = vmax(f, n);
    V3<R> tmin = vmin(f, n);
    R t1 = fminR(tmax.x, fminR(tmax.y, tmax.z));
    R t0 = fmaxR(tmin.x, fmaxR(tmin.y, tmin.z));
    if (t0out) *t0out = t0;
    return (t1 >= t0) ? (t0 > R(0) ? t0 : t1) : R(-1);
}

// Triangle test of closest_hit.glsl:128-143 / anyhit.glsl:366-381.
// Returns true and (u, v, t) when all of (u, v, t, 1-u-v) >= 0.
template <class R> inline bool TriTest(V3<R> o, V3<R> dir, V3<R> v0, V3<R> v1, V3<R> v2, R& u, R& v, R& t, R& w) {
    V3<R> e0 = v1 - v0;
    V3<R> e1 = v2 - v0;
    V3<R> pv = cross(dir, e1);
    R det = dot(e0, pv);
    V3<R> tv = o - v0;
    V3<R> qv = cross(tv, e0);
    u = dot(tv, pv) / det;
    v = dot(dir, qv) / det;
    t = dot(e1, qv) / det;
    w = R(1) - u - v;
    return u >= R(0) && v >= R(0) && t >= R(0) && w >= R(0);
}

// ---------------------------------------------------------------- lights
template <class R> inline Light<R> FetchLight(const Scene<R>& s, int i) {
    const float* p = s.light(i);
    Light<R> L;
    L.position = V3<R>(R(p[0]), R(p[1]), R(p[2]));
    L.emission = V3<R>(R(p[3]), R(p[4]), R(p[5]));
    L.u = V3<R>(R(p[6]), R(p[7]), R(p[8]));
    L.v = V3<R>(R(p[9]), R(p[10]), R(p[11]));
    L.radius = R(p[12]); L.area = R(p[13]); L.type = R(p[14]);
    return L;
}

// -------------------------------------------------------------- ClosestHit
// Triangle part of closest_hit.glsl:88-218 on the flattened two-level BVH.
// mode 0: the reference's traversal (no tmax culling, near child first).
// mode 1: the same order with children culled against the current best t
//         (the "standard tmax-culled" traversal used for work counts).
template <class R> struct TriHit {
    R t; R u, v, w; int prim = -1; int inst = -1; int matID = 0;
};

template <class R> inline void TraverseClosest(const Scene<R>& s, const Ray<R>& r, R tInit, TriHit<R>& h,
                                               Counters* cnt, int mode) {
    int stack[64];
    int ptr = 0;
    stack[ptr++] = -1;
    int index = s.d->top_level_index;
    int currMatID = 0, currInst = -1;
    bool BLAS = false;
    Ray<R> rTrans = r;
    R t = tInit;
    while (index != -1) {
        int leftIndex, rightIndex, leaf;
        s.node_lrl(index, leftIndex, rightIndex, leaf);
        if (cnt) cnt->nodes++;
        if (leaf > 0) {
            for (int i = 0; i < rightIndex; i++) {
                const int32_t* vi = s.d->vert_indices + 3 * (size_t)(leftIndex + i);
                R w0, w1, w2;
                V3<R> v0 = s.vtx(vi[0], w0), v1 = s.vtx(vi[1], w1), v2 = s.vtx(vi[2], w2);
                R u, v, tt, w;
                if (cnt) cnt->tris++;
                if (TriTest(rTrans.origin, rTrans.direction, v0, v1, v2, u, v, tt, w) && tt < t) {
                    t = tt;
                    h.t = tt; h.u = u; h.v = v; h.w = w;
                    h.prim = leftIndex + i;
                    h.inst = currInst;
                    h.matID = currMatID;
                }
            }
        } else if (leaf < 0) {
            int inst = -leaf - 1;
            rTrans.origin = MulPoint(s.inst[inst].inv, r.origin, R(1));
            rTrans.direction = MulPoint(s.inst[inst].inv, r.direction, R(0));
            if (ptr >= 64) { if (cnt) cnt->overflow++; break; }
            stack[ptr++] = -1;
            index = leftIndex;
            BLAS = true;
            currMatID = rightIndex;
            currInst = inst;
            continue;
        } else {
            R l0, r0;
            if (cnt) cnt->inner++;
            R leftHit = AABBIntersect(s.node_min(leftIndex), s.node_max(leftIndex), rTrans, &l0);
            R rightHit = AABBIntersect(s.node_min(rightIndex), s.node_max(rightIndex), rTrans, &r0);
            if (mode == 1) {  // cull children whose entry lies beyond the best hit
                if (leftHit > R(0) && l0 >= t) leftHit = R(-1);
                if (rightHit > R(0) && r0 >= t) rightHit = R(-1);
            }
            if (leftHit > R(0) && rightHit > R(0)) {
                int deferred;
                if (leftHit > rightHit) { index = rightIndex; deferred = leftIndex; }
                else { index = leftIndex; deferred = rightIndex; }
                if (ptr >= 64) { if (cnt) cnt->overflow++; break; }
                stack[ptr++] = deferred;
                continue;
            } else if (leftHit > R(0)) { index = leftIndex; continue; }
            else if (rightHit > R(0)) { index = rightIndex; continue; }
        }
        index = stack[--ptr];
        if (BLAS && index == -1) {
            BLAS = false;
            index = stack[--ptr];
            rTrans = r;
        }
    }
}

// closest_hit.glsl:25-266
template <class R> inline bool ClosestHit(const Scene<R>& s, const Ray<R>& r, State<R>& state,
                                          LightSampleRec<R>& lightSample, Counters& cnt) {
    cnt.closest++;
    R t = K<R>::INF;
    R d;
    if (s.f.lights && !(s.f.hide_emitters && !(state.depth > 0))) {  // closest_hit.glsl:30-86
        for (int i = 0; i < s.num_lights; i++) {
            Light<R> L = FetchLight(s, i);
            if (int(L.type) == QUAD_LIGHT) {
                V3<R> normal = normalize(cross(L.u, L.v));
                if (dot(normal, r.direction) > R(0)) continue;
                R pw = dot(normal, L.position);
                V3<R> u = L.u * (R(1) / dot(L.u, L.u));
                V3<R> v = L.v * (R(1) / dot(L.v, L.v));
                d = RectIntersect(L.position, u, v, normal, pw, r);
                if (d < R(0)) d = K<R>::INF;
                if (d < t) {
                    t = d;
                    R cosTheta = dot(-r.direction, normal);
                    lightSample.pdf = (t * t) / (L.area * cosTheta);
                    lightSample.emission = L.emission;
                    state.isEmitter = true;
                }
            }
            if (int(L.type) == SPHERE_LIGHT) {
                d = SphereIntersect(L.radius, L.position, r);
                if (d < R(0)) d = K<R>::INF;
                if (d < t) {
                    t = d;
                    V3<R> hitPt = r.origin + t * r.direction;
                    R cosTheta = dot(-r.direction, normalize(hitPt - L.position));
                    lightSample.pdf = (t * t) / (L.area * cosTheta * R(0.5));
                    lightSample.emission = L.emission;
                    state.isEmitter = true;
                }
            }
        }
    }
    TriHit<R> h;
    h.t = t;
    TraverseClosest(s, r, t, h, &cnt, s.cull ? 1 : 0);
    if (h.prim >= 0) t = h.t;
    if (t == K<R>::INF) return false;

    state.hitDist = t;
    state.fhp = r.origin + r.direction * t;

    if (h.prim >= 0) {  // closest_hit.glsl:227-263
        cnt.tri_hits++;
        state.isEmitter = false;
        state.matID = h.matID;
        const int32_t* vi = s.d->vert_indices + 3 * (size_t)h.prim;
        R u0, u1, u2, v0w, v1w, v2w;
        V3<R> p0 = s.vtx(vi[0], u0), p1 = s.vtx(vi[1], u1), p2 = s.vtx(vi[2], u2);
        V3<R> n0 = s.nrm(vi[0], v0w), n1 = s.nrm(vi[1], v1w), n2 = s.nrm(vi[2], v2w);
        // bary = uvt.wxy
        R bx = h.w, by = h.u, bz = h.v;
        V2<R> t0{u0, v0w}, t1{u1, v1w}, t2{u2, v2w};
        state.texCoord = {t0.x * bx + t1.x * by + t2.x * bz, t0.y * bx + t1.y * by + t2.y * bz};
        V3<R> normal = normalize(n0 * bx + n1 * by + n2 * bz);
        static const InstMats<R> ident = [] {
            const float I16[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
            return MakeInstMats<R>(I16);
        }();
        const InstMats<R>& im = h.inst >= 0 ? s.inst[h.inst] : ident;  // BLAS reached without a TLAS leaf
        state.normal = normalize(Mul3(im.nrm, normal));
        state.ffnormal = dot(state.normal, r.direction) <= R(0) ? state.normal : -state.normal;
        V3<R> deltaPos1 = p1 - p0, deltaPos2 = p2 - p0;
        V2<R> dUV1{t1.x - t0.x, t1.y - t0.y}, dUV2{t2.x - t0.x, t2.y - t0.y};
        R invdet = R(1) / (dUV1.x * dUV2.y - dUV1.y * dUV2.x);
        state.tangent = (deltaPos1 * dUV2.y - deltaPos2 * dUV1.y) * invdet;
        state.bitangent = (deltaPos2 * dUV1.x - deltaPos1 * dUV2.x) * invdet;
        state.tangent = normalize(Mul3(im.m3, state.tangent));
        state.bitangent = normalize(Mul3(im.m3, state.bitangent));
    }
    return true;
}

// ------------------------------------------------------------------ AnyHit
// anyhit.glsl:25-216.  Alpha testing (anyhit.glsl:118-141) is compiled in
// only with OPT_ALPHA_TEST && !OPT_MEDIUM.
template <class R> inline bool AnyHit(const Scene<R>& s, const Ray<R>& r, R maxDist, Rng& rng, Counters& cnt) {
    cnt.shadow++;
    if (s.f.lights) {
        for (int i = 0; i < s.num_lights; i++) {
            Light<R> L = FetchLight(s, i);
            if (int(L.type) == QUAD_LIGHT) {
                V3<R> normal = normalize(cross(L.u, L.v));
                R pw = dot(normal, L.position);
                V3<R> u = L.u * (R(1) / dot(L.u, L.u));
                V3<R> v = L.v * (R(1) / dot(L.v, L.v));
                R d = RectIntersect(L.position, u, v, normal, pw, r);
                if (d > R(0) && d < maxDist) return true;
            }
            if (int(L.type) == SPHERE_LIGHT) {
                R d = SphereIntersect(L.radius, L.position, r);
                if (d > R(0) && d < maxDist) return true;
            }
        }
    }
    const bool alpha = s.f.alpha_test && !s.f.medium;
    int stack[64];
    int ptr = 0;
    stack[ptr++] = -1;
    int index = s.d->top_level_index;
    int currMatID = 0;
    bool BLAS = false;
    Ray<R> rTrans = r;
    while (index != -1) {
        int leftIndex, rightIndex, leaf;
        s.node_lrl(index, leftIndex, rightIndex, leaf);
        cnt.nodes++;
        cnt.nodes_any++;
        if (leaf > 0) {
            for (int i = 0; i < rightIndex; i++) {
                const int32_t* vi = s.d->vert_indices + 3 * (size_t)(leftIndex + i);
                R w0, w1, w2;
                V3<R> v0 = s.vtx(vi[0], w0), v1 = s.vtx(vi[1], w1), v2 = s.vtx(vi[2], w2);
                R u, v, tt, w;
                cnt.tris++;
                cnt.tris_any++;
                if (TriTest(rTrans.origin, rTrans.direction, v0, v1, v2, u, v, tt, w) && tt < maxDist) {
                    if (!alpha) return true;
                    R n0w, n1w, n2w;
                    s.nrm(vi[0], n0w); s.nrm(vi[1], n1w); s.nrm(vi[2], n2w);
                    V2<R> texCoord{w0 * w + w1 * u + w2 * v, n0w * w + n1w * u + n2w * v};
                    const float* m = s.mat(currMatID);
                    R tex[4];
                    SampleTexArray(s, texCoord, R(m[24]), tex);
                    R opacity = R(m[28]) * tex[3];
                    int alphaMode = int(m[29]);
                    R alphaCutoff = R(m[30]);
                    bool skip = (alphaMode == ALPHA_MODE_MASK && opacity < alphaCutoff);
                    if (!skip && alphaMode == ALPHA_MODE_BLEND) skip = R(rng.next()) > opacity;
                    if (!skip) return true;
                }
            }
        } else if (leaf < 0) {
            int inst = -leaf - 1;
            rTrans.origin = MulPoint(s.inst[inst].inv, r.origin, R(1));
            rTrans.direction = MulPoint(s.inst[inst].inv, r.direction, R(0));
            if (ptr >= 64) { cnt.overflow++; return false; }
            stack[ptr++] = -1;
            index = leftIndex;
            BLAS = true;
            currMatID = rightIndex;
            continue;
        } else {
            R l0, r0;
            cnt.inner++;
            R leftHit = AABBIntersect(s.node_min(leftIndex), s.node_max(leftIndex), rTrans, &l0);
            R rightHit = AABBIntersect(s.node_min(rightIndex), s.node_max(rightIndex), rTrans, &r0);
            if (s.cull) {  // boxes entered beyond maxDist cannot occlude
                if (leftHit > R(0) && l0 >= maxDist) leftHit = R(-1);
                if (rightHit > R(0) && r0 >= maxDist) rightHit = R(-1);
            }
            if (leftHit > R(0) && rightHit > R(0)) {
                int deferred;
                if (leftHit > rightHit) { index = rightIndex; deferred = leftIndex; }
                else { index = leftIndex; deferred = rightIndex; }
                if (ptr >= 64) { cnt.overflow++; return false; }
                stack[ptr++] = deferred;
                continue;
            } else if (leftHit > R(0)) { index = leftIndex; continue; }
            else if (rightHit > R(0)) { index = rightIndex; continue; }
        }
        index = stack[--ptr];
        if (BLAS && index == -1) {
            BLAS = false;
            index = stack[--ptr];
            rTrans = r;
        }
    }
    return false;
}

// -------------------------------------------------------------- sampling
// common/sampling.glsl:25-32
template <class R> inline R GTR1(R NDotH, R a) {
    if (a >= R(1)) return K<R>::INV_PI;
    R a2 = a * a;
    R t = R(1) + (a2 - R(1)) * NDotH * NDotH;
    return (a2 - R(1)) / (K<R>::PI * std::log(a2) * t);
}
// sampling.glsl:34-47
template <class R> inline V3<R> SampleGTR1(R rgh, R r1, R r2) {
    R a = fmaxR(R(0.001), rgh);
    R a2 = a * a;
    R phi = r1 * K<R>::TWO_PI;
    R cosTheta = std::sqrt((R(1) - std::pow(a2, R(1) - r2)) / (R(1) - a2));
    R sinTheta = clampR(std::sqrt(R(1) - (cosTheta * cosTheta)), R(0), R(1));
    R sinPhi = std::sin(phi), cosPhi = std::cos(phi);
    return V3<R>(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
}
// sampling.glsl:70-88 (Heitz 2018 VNDF sampling)
template <class R> inline V3<R> SampleGGXVNDF(V3<R> V, R ax, R ay, R r1, R r2) {
    V3<R> Vh = normalize(V3<R>(ax * V.x, ay * V.y, V.z));
    R lensq = Vh.x * Vh.x + Vh.y * Vh.y;
    V3<R> T1 = lensq > R(0) ? V3<R>(-Vh.y, Vh.x, R(0)) * (R(1) / std::sqrt(lensq)) : V3<R>(R(1), R(0), R(0));
    V3<R> T2 = cross(Vh, T1);
    R r = std::sqrt(r1);
    R phi = R(2) * K<R>::PI * r2;
    R t1 = r * std::cos(phi);
    R t2 = r * std::sin(phi);
    R s = R(0.5) * (R(1) + Vh.z);
    t2 = (R(1) - s) * std::sqrt(R(1) - t1 * t1) + s * t2;
    V3<R> Nh = t1 * T1 + t2 * T2 + std::sqrt(fmaxR(R(0), R(1) - t1 * t1 - t2 * t2)) * Vh;
    return normalize(V3<R>(ax * Nh.x, ay * Nh.y, fmaxR(R(0), Nh.z)));
}
// sampling.glsl:90-96
template <class R> inline R GTR2Aniso(R NDotH, R HDotX, R HDotY, R ax, R ay) {
    R a = HDotX / ax;
    R b = HDotY / ay;
    R c = a * a + b * b + NDotH * NDotH;
    return R(1) / (K<R>::PI * ax * ay * c * c);
}
// sampling.glsl:109-114
template <class R> inline R SmithG(R NDotV, R alphaG) {
    R a = alphaG * alphaG;
    R b = NDotV * NDotV;
    return (R(2) * NDotV) / (NDotV + std::sqrt(a + b - a * b));
}
// sampling.glsl:116-122
template <class R> inline R SmithGAniso(R NDotV, R VDotX, R VDotY, R ax, R ay) {
    R a = VDotX * ax;
    R b = VDotY * ay;
    R c = NDotV;
    return (R(2) * NDotV) / (NDotV + std::sqrt(a * a + b * b + c * c));
}
// sampling.glsl:124-129
template <class R> inline R SchlickWeight(R u) {
    R m = clampR(R(1) - u, R(0), R(1));
    R m2 = m * m;
    return m2 * m2 * m;
}
// sampling.glsl:131-145
template <class R> inline R DielectricFresnel(R cosThetaI, R eta) {
    R sinThetaTSq = eta * eta * (R(1) - cosThetaI * cosThetaI);
    if (sinThetaTSq > R(1)) return R(1);
    R cosThetaT = std::sqrt(fmaxR(R(1) - sinThetaTSq, R(0)));
    R rs = (eta * cosThetaT - cosThetaI) / (eta * cosThetaT + cosThetaI);
    R rp = (eta * cosThetaI - cosThetaT) / (eta * cosThetaI + cosThetaT);
    return R(0.5) * (rs * rs + rp * rp);
}
// sampling.glsl:147-156
template <class R> inline V3<R> CosineSampleHemisphere(R r1, R r2) {
    V3<R> dir;
    R r = std::sqrt(r1);
    R phi = K<R>::TWO_PI * r2;
    dir.x = r * std::cos(phi);
    dir.y = r * std::sin(phi);
    dir.z = std::sqrt(fmaxR(R(0), R(1) - dir.x * dir.x - dir.y * dir.y));
    return dir;
}
// sampling.glsl:158-163
template <class R> inline V3<R> UniformSampleHemisphere(R r1, R r2) {
    R r = std::sqrt(fmaxR(R(0), R(1) - r1 * r1));
    R phi = K<R>::TWO_PI * r2;
    return V3<R>(r * std::cos(phi), r * std::sin(phi), r1);
}
// sampling.glsl:173-177
template <class R> inline R PowerHeuristic(R a, R b) {
    R t = a * a;
    return t / (b * b + t);
}
// sampling.glsl:179-184
template <class R> inline void Onb(V3<R> N, V3<R>& T, V3<R>& B) {
    V3<R> up = std::fabs(N.z) < R(0.9999999) ? V3<R>(R(0), R(0), R(1)) : V3<R>(R(1), R(0), R(0));
    T = normalize(cross(up, N));
    B = cross(N, T);
}
// sampling.glsl:186-212
template <class R> inline void SampleSphereLight(const Scene<R>& s, const Light<R>& light, V3<R> scatterPos,
                                                 LightSampleRec<R>& ls, Rng& rng) {
    R r1 = R(rng.next());
    R r2 = R(rng.next());
    V3<R> c2s = scatterPos - light.position;
    R distToSphereCenter = length(c2s);
    c2s = c2s / distToSphereCenter;
    V3<R> sampledDir = UniformSampleHemisphere(r1, r2);
    V3<R> T, B;
    Onb(c2s, T, B);
    sampledDir = T * sampledDir.x + B * sampledDir.y + c2s * sampledDir.z;
    V3<R> lightSurfacePos = light.position + sampledDir * light.radius;
    ls.direction = lightSurfacePos - scatterPos;
    ls.dist = length(ls.direction);
    R distSq = ls.dist * ls.dist;
    ls.direction = ls.direction / ls.dist;
    ls.normal = normalize(lightSurfacePos - light.position);
    ls.emission = light.emission * R(s.num_lights);
    ls.pdf = distSq / (light.area * R(0.5) * std::fabs(dot(ls.normal, ls.direction)));
}
// sampling.glsl:214-227
template <class R> inline void SampleRectLight(const Scene<R>& s, const Light<R>& light, V3<R> scatterPos,
                                               LightSampleRec<R>& ls, Rng& rng) {
    R r1 = R(rng.next());
    R r2 = R(rng.next());
    V3<R> lightSurfacePos = light.position + light.u * r1 + light.v * r2;
    ls.direction = lightSurfacePos - scatterPos;
    ls.dist = length(ls.direction);
    R distSq = ls.dist * ls.dist;
    ls.direction = ls.direction / ls.dist;
    ls.normal = normalize(cross(light.u, light.v));
    ls.emission = light.emission * R(s.num_lights);
    ls.pdf = distSq / (light.area * std::fabs(dot(ls.normal, ls.direction)));
}
// sampling.glsl:229-236
template <class R> inline void SampleDistantLight(const Scene<R>& s, const Light<R>& light, V3<R> scatterPos,
                                                  LightSampleRec<R>& ls) {
    ls.direction = normalize(light.position - V3<R>(R(0)));
    ls.normal = normalize(scatterPos - light.position);
    ls.emission = light.emission * R(s.num_lights);
    ls.dist = K<R>::INF;
    ls.pdf = R(1);
}
// sampling.glsl:238-248
template <class R> inline void SampleOneLight(const Scene<R>& s, const Light<R>& light, V3<R> scatterPos,
                                              LightSampleRec<R>& ls, Rng& rng) {
    int type = int(light.type);
    if (type == QUAD_LIGHT) SampleRectLight(s, light, scatterPos, ls, rng);
    else if (type == SPHERE_LIGHT) SampleSphereLight(s, light, scatterPos, ls, rng);
    else SampleDistantLight(s, light, scatterPos, ls);
}
// sampling.glsl:250-271
template <class R> inline V3<R> SampleHG(V3<R> V, R g, R r1, R r2) {
    R cosTheta;
    if (std::fabs(g) < R(0.001)) cosTheta = R(1) - R(2) * r2;
    else {
        R sqrTerm = (R(1) - g * g) / (R(1) + g - R(2) * g * r2);
        cosTheta = -(R(1) + g * g - sqrTerm * sqrTerm) / (R(2) * g);
    }
    R phi = r1 * K<R>::TWO_PI;
    R sinTheta = clampR(std::sqrt(R(1) - (cosTheta * cosTheta)), R(0), R(1));
    R sinPhi = std::sin(phi), cosPhi = std::cos(phi);
    V3<R> v1, v2;
    Onb(V, v1, v2);
    return sinTheta * cosPhi * v1 + sinTheta * sinPhi * v2 + cosTheta * V;
}
// sampling.glsl:273-277
template <class R> inline R PhaseHG(R cosTheta, R g) {
    R denom = R(1) + g * g + R(2) * g * cosTheta;
    return K<R>::INV_4_PI * (R(1) - g * g) / (denom * std::sqrt(denom));
}

// ---------------------------------------------------------------- envmap
// common/envmap.glsl:28-55: two binary searches over the flat CDF.
template <class R> inline V2<R> BinarySearch(const Scene<R>& s, R value) {
    int W = s.d->envmap_width, H = s.d->envmap_height;
    const float* cdf = s.d->envmap_cdf;
    int lower = 0, upper = H - 1;
    while (lower < upper) {
        int mid = (lower + upper) >> 1;
        if (value < R(cdf[(size_t)mid * W + (W - 1)])) upper = mid;
        else lower = mid + 1;
    }
    int y = std::min(std::max(lower, 0), H - 1);
    lower = 0; upper = W - 1;
    while (lower < upper) {
        int mid = (lower + upper) >> 1;
        if (value < R(cdf[(size_t)y * W + mid])) upper = mid;
        else lower = mid + 1;
    }
    int x = std::min(std::max(lower, 0), W - 1);
    return {R(x) / s.env_w, R(y) / s.env_h};
}
// envmap.glsl:57-66 ; returns color, pdf in .w
template <class R> inline V3<R> EvalEnvMap(const Scene<R>& s, const Ray<R>& r, R& pdfOut) {
    R theta = std::acos(clampR(r.direction.y, R(-1), R(1)));
    V2<R> uv{(K<R>::PI + std::atan2(r.direction.z, r.direction.x)) * K<R>::INV_TWO_PI + s.env_rot, theta * K<R>::INV_PI};
    V3<R> color = SampleRGBRepeat(s.d->envmap_rgb, s.d->envmap_width, s.d->envmap_height, uv.x, uv.y);
    R pdf = Luminance(color) / s.env_total;
    pdfOut = (pdf * s.env_w * s.env_h) / (K<R>::TWO_PI * K<R>::PI * std::sin(theta));
    return color;
}
// envmap.glsl:68-83 ; returns direction, pdf via pdfOut, color via color
template <class R> inline V3<R> SampleEnvMap(const Scene<R>& s, V3<R>& color, R& pdfOut, Rng& rng) {
    V2<R> uv = BinarySearch(s, R(rng.next()) * s.env_total);
    color = SampleRGBRepeat(s.d->envmap_rgb, s.d->envmap_width, s.d->envmap_height, uv.x, uv.y);
    R pdf = Luminance(color) / s.env_total;
    uv.x -= s.env_rot;
    R phi = uv.x * K<R>::TWO_PI;
    R theta = uv.y * K<R>::PI;
    if (std::sin(theta) == R(0)) pdf = R(0);
    pdfOut = (pdf * s.env_w * s.env_h) / (K<R>::TWO_PI * K<R>::PI * std::sin(theta));
    return V3<R>(-std::sin(theta) * std::cos(phi), std::cos(theta), -std::sin(theta) * std::sin(phi));
}

// ---------------------------------------------------------------- Disney
// common/disney.glsl:39-47
template <class R> inline V3<R> ToWorld(V3<R> X, V3<R> Y, V3<R> Z, V3<R> V) { return V.x * X + V.y * Y + V.z * Z; }
template <class R> inline V3<R> ToLocal(V3<R> X, V3<R> Y, V3<R> Z, V3<R> V) { return V3<R>(dot(V, X), dot(V, Y), dot(V, Z)); }
// disney.glsl:49-59
template <class R> inline void TintColors(const Material<R>& mat, R eta, R& F0, V3<R>& Csheen, V3<R>& Cspec0) {
    R lum = Luminance(mat.baseColor);
    V3<R> ctint = lum > R(0) ? mat.baseColor / lum : V3<R>(R(1));
    F0 = (R(1) - eta) / (R(1) + eta);
    F0 *= F0;
    Cspec0 = F0 * mix3(V3<R>(R(1)), ctint, mat.specularTint);
    Csheen = mix3(V3<R>(R(1)), ctint, mat.sheenTint);
}
// disney.glsl:61-88
template <class R> inline V3<R> EvalDisneyDiffuse(const Material<R>& mat, V3<R> Csheen, V3<R> V, V3<R> L, V3<R> H, R& pdf) {
    pdf = R(0);
    if (L.z <= R(0)) return V3<R>(R(0));
    R LDotH = dot(L, H);
    R Rr = R(2) * mat.roughness * LDotH * LDotH;
    R FL = SchlickWeight(L.z);
    R FV = SchlickWeight(V.z);
    R Fretro = Rr * (FL + FV + FL * FV * (Rr - R(1)));
    R Fd = (R(1) - R(0.5) * FL) * (R(1) - R(0.5) * FV);
    R Fss90 = R(0.5) * Rr;
    R Fss = mixR(R(1), Fss90, FL) * mixR(R(1), Fss90, FV);
    R ss = R(1.25) * (Fss * (R(1) / (L.z + V.z) - R(0.5)) + R(0.5));
    R FH = SchlickWeight(LDotH);
    V3<R> Fsheen = FH * mat.sheen * Csheen;
    pdf = L.z * K<R>::INV_PI;
    return K<R>::INV_PI * mat.baseColor * mixR(Fd + Fretro, ss, mat.subsurface) + Fsheen;
}
// disney.glsl:90-102
template <class R> inline V3<R> EvalMicrofacetReflection(const Material<R>& mat, V3<R> V, V3<R> L, V3<R> H, V3<R> F, R& pdf) {
    pdf = R(0);
    if (L.z <= R(0)) return V3<R>(R(0));
    R D = GTR2Aniso(H.z, H.x, H.y, mat.ax, mat.ay);
    R G1 = SmithGAniso(std::fabs(V.z), V.x, V.y, mat.ax, mat.ay);
    R G2 = G1 * SmithGAniso(std::fabs(L.z), L.x, L.y, mat.ax, mat.ay);
    pdf = G1 * D / (R(4) * V.z);
    return F * D * G2 / (R(4) * L.z * V.z);
}
// disney.glsl:104-123
template <class R> inline V3<R> EvalMicrofacetRefraction(const Material<R>& mat, R eta, V3<R> V, V3<R> L, V3<R> H, V3<R> F, R& pdf) {
    pdf = R(0);
    if (L.z >= R(0)) return V3<R>(R(0));
    R LDotH = dot(L, H);
    R VDotH = dot(V, H);
    R D = GTR2Aniso(H.z, H.x, H.y, mat.ax, mat.ay);
    R G1 = SmithGAniso(std::fabs(V.z), V.x, V.y, mat.ax, mat.ay);
    R G2 = G1 * SmithGAniso(std::fabs(L.z), L.x, L.y, mat.ax, mat.ay);
    R denom = LDotH + VDotH * eta;
    denom *= denom;
    R eta2 = eta * eta;
    R jacobian = std::fabs(LDotH) / denom;
    pdf = G1 * fmaxR(R(0), VDotH) * D * jacobian / V.z;
    return vpow(mat.baseColor, R(0.5)) * (V3<R>(R(1)) - F) * D * G2 * std::fabs(VDotH) * jacobian * eta2 / std::fabs(L.z * V.z);
}
// disney.glsl:125-140
template <class R> inline V3<R> EvalClearcoat(const Material<R>& mat, V3<R> V, V3<R> L, V3<R> H, R& pdf) {
    pdf = R(0);
    if (L.z <= R(0)) return V3<R>(R(0));
    R VDotH = dot(V, H);
    R F = mixR(R(0.04), R(1), SchlickWeight(VDotH));
    R D = GTR1(H.z, mat.clearcoatRoughness);
    R G = SmithG(L.z, R(0.25)) * SmithG(V.z, R(0.25));
    R jacobian = R(1) / (R(4) * VDotH);
    pdf = D * H.z * jacobian;
    return V3<R>(F) * D * G;
}

// Lobe weights and probabilities shared by DisneySample / DisneyEval
// (disney.glsl:161-181 and 271-291).
template <class R> struct Lobes {
    R dielectricWt, metalWt, glassWt, diffPr, dielectricPr, metalPr, glassPr, clearCtPr, F0;
    V3<R> Csheen, Cspec0;
};
template <class R> inline Lobes<R> LobeWeights(const Material<R>& mat, R eta, V3<R> V) {
    Lobes<R> lb;
    TintColors(mat, eta, lb.F0, lb.Csheen, lb.Cspec0);
    lb.dielectricWt = (R(1) - mat.metallic) * (R(1) - mat.specTrans);
    lb.metalWt = mat.metallic;
    lb.glassWt = (R(1) - mat.metallic) * mat.specTrans;
    R schlickWt = SchlickWeight(V.z);
    lb.diffPr = lb.dielectricWt * Luminance(mat.baseColor);
    lb.dielectricPr = lb.dielectricWt * Luminance(mix3(lb.Cspec0, V3<R>(R(1)), schlickWt));
    lb.metalPr = lb.metalWt * Luminance(mix3(mat.baseColor, V3<R>(R(1)), schlickWt));
    lb.glassPr = lb.glassWt;
    lb.clearCtPr = R(0.25) * mat.clearcoat;
    R invTotalWt = R(1) / (lb.diffPr + lb.dielectricPr + lb.metalPr + lb.glassPr + lb.clearCtPr);
    lb.diffPr *= invTotalWt;
    lb.dielectricPr *= invTotalWt;
    lb.metalPr *= invTotalWt;
    lb.glassPr *= invTotalWt;
    lb.clearCtPr *= invTotalWt;
    return lb;
}

// Per-lobe parts of DisneyEval, kept separately for the per-lobe BSDF test.
template <class R> struct LobeEval { V3<R> f[5]; R pdf[5]; };

// disney.glsl:244-351.  When parts != nullptr the weighted contribution of
// each lobe (diffuse, dielectric, metal, glass, clearcoat) is recorded too.
template <class R> inline V3<R> DisneyEval(const State<R>& state, V3<R> V, V3<R> N, V3<R> L, R& pdf,
                                           LobeEval<R>* parts = nullptr) {
    pdf = R(0);
    V3<R> f(R(0));
    V3<R> T, B;
    Onb(N, T, B);
    V = ToLocal(T, B, N, V);
    L = ToLocal(T, B, N, L);
    V3<R> H;
    if (L.z > R(0)) H = normalize(L + V);
    else H = normalize(L + V * state.eta);
    if (H.z < R(0)) H = -H;
    const Material<R>& mat = state.mat;
    Lobes<R> lb = LobeWeights(mat, state.eta, V);
    bool reflect = L.z * V.z > R(0);
    R tmpPdf = R(0);
    R VDotH = std::fabs(dot(V, H));
    if (parts) for (int i = 0; i < 5; ++i) { parts->f[i] = V3<R>(R(0)); parts->pdf[i] = R(0); }
    R absLz = std::fabs(L.z);
    if (lb.diffPr > R(0) && reflect) {
        V3<R> c = EvalDisneyDiffuse(mat, lb.Csheen, V, L, H, tmpPdf) * lb.dielectricWt;
        f = f + c;
        pdf += tmpPdf * lb.diffPr;
        if (parts) { parts->f[0] = c * absLz; parts->pdf[0] = tmpPdf * lb.diffPr; }
    }
    if (lb.dielectricPr > R(0) && reflect) {
        R F = (DielectricFresnel(VDotH, R(1) / mat.ior) - lb.F0) / (R(1) - lb.F0);
        V3<R> c = EvalMicrofacetReflection(mat, V, L, H, mix3(lb.Cspec0, V3<R>(R(1)), F), tmpPdf) * lb.dielectricWt;
        f = f + c;
        pdf += tmpPdf * lb.dielectricPr;
        if (parts) { parts->f[1] = c * absLz; parts->pdf[1] = tmpPdf * lb.dielectricPr; }
    }
    if (lb.metalPr > R(0) && reflect) {
        V3<R> F = mix3(mat.baseColor, V3<R>(R(1)), SchlickWeight(VDotH));
        V3<R> c = EvalMicrofacetReflection(mat, V, L, H, F, tmpPdf) * lb.metalWt;
        f = f + c;
        pdf += tmpPdf * lb.metalPr;
        if (parts) { parts->f[2] = c * absLz; parts->pdf[2] = tmpPdf * lb.metalPr; }
    }
    if (lb.glassPr > R(0)) {
        R F = DielectricFresnel(VDotH, state.eta);
        V3<R> c;
        R p;
        if (reflect) {
            c = EvalMicrofacetReflection(mat, V, L, H, V3<R>(F), tmpPdf) * lb.glassWt;
            p = tmpPdf * lb.glassPr * F;
        } else {
            c = EvalMicrofacetRefraction(mat, state.eta, V, L, H, V3<R>(F), tmpPdf) * lb.glassWt;
            p = tmpPdf * lb.glassPr * (R(1) - F);
        }
        f = f + c;
        pdf += p;
        if (parts) { parts->f[3] = c * absLz; parts->pdf[3] = p; }
    }
    if (lb.clearCtPr > R(0) && reflect) {
        V3<R> c = EvalClearcoat(mat, V, L, H, tmpPdf) * R(0.25) * mat.clearcoat;
        f = f + c;
        pdf += tmpPdf * lb.clearCtPr;
        if (parts) { parts->f[4] = c * absLz; parts->pdf[4] = tmpPdf * lb.clearCtPr; }
    }
    return f * absLz;
}

// disney.glsl:142-242
template <class R> inline V3<R> DisneySample(const State<R>& state, V3<R> V, V3<R> N, V3<R>& L, R& pdf, Rng& rng) {
    pdf = R(0);
    R r1 = R(rng.next());
    R r2 = R(rng.next());
    V3<R> T, B;
    Onb(N, T, B);
    V = ToLocal(T, B, N, V);
    const Material<R>& mat = state.mat;
    Lobes<R> lb = LobeWeights(mat, state.eta, V);
    R cdf[5];
    cdf[0] = lb.diffPr;
    cdf[1] = cdf[0] + lb.dielectricPr;
    cdf[2] = cdf[1] + lb.metalPr;
    cdf[3] = cdf[2] + lb.glassPr;
    cdf[4] = cdf[3] + lb.clearCtPr;
    R r3 = R(rng.next());
    if (r3 < cdf[0]) {
        L = CosineSampleHemisphere(r1, r2);
    } else if (r3 < cdf[2]) {
        V3<R> H = SampleGGXVNDF(V, mat.ax, mat.ay, r1, r2);
        if (H.z < R(0)) H = -H;
        L = normalize(reflectR(-V, H));
    } else if (r3 < cdf[3]) {
        V3<R> H = SampleGGXVNDF(V, mat.ax, mat.ay, r1, r2);
        R F = DielectricFresnel(std::fabs(dot(V, H)), state.eta);
        if (H.z < R(0)) H = -H;
        r3 = (r3 - cdf[2]) / (cdf[3] - cdf[2]);
        if (r3 < F) L = normalize(reflectR(-V, H));
        else L = normalize(refractR(-V, H, state.eta));
    } else {
        V3<R> H = SampleGTR1(mat.clearcoatRoughness, r1, r2);
        if (H.z < R(0)) H = -H;
        L = normalize(reflectR(-V, H));
    }
    L = ToWorld(T, B, N, L);
    V = ToWorld(T, B, N, V);
    return DisneyEval(state, V, N, L, pdf);
}

// ------------------------------------------------------------ GetMaterial
// common/pathtrace.glsl:25-115
template <class R> inline void GetMaterial(const Scene<R>& s, State<R>& state, const Ray<R>& r) {
    const float* p = s.mat(state.matID);
    Material<R> mat;
    mat.baseColor = V3<R>(R(p[0]), R(p[1]), R(p[2]));
    mat.anisotropic = R(p[3]);
    mat.emission = V3<R>(R(p[4]), R(p[5]), R(p[6]));
    mat.metallic = R(p[8]);
    mat.roughness = fmaxR(R(p[9]), R(0.001));
    mat.subsurface = R(p[10]);
    mat.specularTint = R(p[11]);
    mat.sheen = R(p[12]);
    mat.sheenTint = R(p[13]);
    mat.clearcoat = R(p[14]);
    mat.clearcoatRoughness = mixR(R(0.1), R(0.001), R(p[15]));
    mat.specTrans = R(p[16]);
    mat.ior = R(p[17]);
    mat.medium.type = int(p[18]);
    mat.medium.density = R(p[19]);
    mat.medium.color = V3<R>(R(p[20]), R(p[21]), R(p[22]));
    mat.medium.anisotropy = clampR(R(p[23]), R(-0.9), R(0.9));
    int texIDs[4] = {int(p[24]), int(p[25]), int(p[26]), int(p[27])};
    mat.opacity = R(p[28]);
    mat.alphaMode = int(p[29]);
    mat.alphaCutoff = R(p[30]);
    R tex[4];
    if (texIDs[0] >= 0) {
        SampleTexArray(s, state.texCoord, R(texIDs[0]), tex);
        V3<R> col = vpow(V3<R>(tex[0], tex[1], tex[2]), R(2.2));
        mat.baseColor = mat.baseColor * col;
        mat.opacity *= tex[3];
    }
    if (texIDs[1] >= 0) {
        SampleTexArray(s, state.texCoord, R(texIDs[1]), tex);
        mat.metallic = tex[2];
        mat.roughness = fmaxR(tex[1] * tex[1], R(0.001));
    }
    if (texIDs[2] >= 0) {
        SampleTexArray(s, state.texCoord, R(texIDs[2]), tex);
        V3<R> texNormal(tex[0], tex[1], tex[2]);
        if (s.f.opengl_normalmap) texNormal.y = R(1) - texNormal.y;
        texNormal = normalize(texNormal * R(2) - V3<R>(R(1)));
        V3<R> origNormal = state.normal;
        state.normal = normalize(state.tangent * texNormal.x + state.bitangent * texNormal.y + state.normal * texNormal.z);
        state.ffnormal = dot(origNormal, r.direction) <= R(0) ? state.normal : -state.normal;
    }
    if (s.f.roughness_mollification && state.depth > 0)
        mat.roughness = fmaxR(mixR(R(0), state.mat.roughness, s.mollify_amt), mat.roughness);
    if (texIDs[3] >= 0) {
        SampleTexArray(s, state.texCoord, R(texIDs[3]), tex);
        mat.emission = vpow(V3<R>(tex[0], tex[1], tex[2]), R(2.2));
    }
    R aspect = std::sqrt(R(1) - mat.anisotropic * R(0.9));
    mat.ax = fmaxR(R(0.001), mat.roughness / aspect);
    mat.ay = fmaxR(R(0.001), mat.roughness * aspect);
    state.mat = mat;
    state.eta = dot(r.direction, state.normal) < R(0) ? (R(1) / mat.ior) : mat.ior;
}

template <class R> inline bool AlphaSkip(const Material<R>& m, Rng& rng) {
    // pathtrace.glsl:136 / 419-420; rand() only evaluated for BLEND
    if (m.alphaMode == ALPHA_MODE_MASK && m.opacity < m.alphaCutoff) return true;
    if (m.alphaMode == ALPHA_MODE_BLEND) return R(rng.next()) > m.opacity;
    return false;
}

// pathtrace.glsl:118-156 (OPT_MEDIUM && OPT_VOL_MIS)
template <class R> inline V3<R> EvalTransmittance(const Scene<R>& s, Ray<R> r, Rng& rng, Counters& cnt) {
    LightSampleRec<R> lightSample;
    State<R> state;
    V3<R> transmittance(R(1));
    for (int depth = 0; depth < s.f.max_depth; depth++) {
        bool hit = ClosestHit(s, r, state, lightSample, cnt);
        if (!hit || state.isEmitter) break;
        GetMaterial(s, state, r);
        bool alphatest = AlphaSkip(state.mat, rng);
        bool refractive = (R(1) - state.mat.metallic) * state.mat.specTrans > R(0);
        if (hit && !(alphatest || refractive)) return V3<R>(R(0));
        if (dot(r.direction, state.normal) > R(0) && state.mat.medium.type != MEDIUM_NONE) {
            V3<R> color = state.mat.medium.type == MEDIUM_ABSORB ? V3<R>(R(1)) - state.mat.medium.color : V3<R>(R(1));
            transmittance = transmittance * vexp(-color * state.mat.medium.density * state.hitDist);
        }
        r.origin = state.fhp + r.direction * K<R>::EPS;
    }
    return transmittance;
}

// pathtrace.glsl:158-283
template <class R> inline V3<R> DirectLight(const Scene<R>& s, const Ray<R>& r, const State<R>& state, bool isSurface,
                                            Rng& rng, Counters& cnt) {
    V3<R> Ld(R(0));
    V3<R> Li(R(0));
    V3<R> scatterPos = state.fhp + state.normal * K<R>::EPS;
    ScatterSampleRec<R> scatterSample;
    const bool volmis = s.f.medium && s.f.vol_mis;
    if (s.f.envmap && !s.f.uniform_light) {
        R lightPdf;
        V3<R> lightDir = SampleEnvMap(s, Li, lightPdf, rng);
        Ray<R> shadowRay{scatterPos, lightDir};
        if (volmis) {
            Li = Li * EvalTransmittance(s, shadowRay, rng, cnt);
            if (isSurface) scatterSample.f = DisneyEval(state, -r.direction, state.ffnormal, lightDir, scatterSample.pdf);
            else {
                R p = PhaseHG(dot(-r.direction, lightDir), state.medium.anisotropy);
                scatterSample.f = V3<R>(p);
                scatterSample.pdf = p;
            }
            if (scatterSample.pdf > R(0)) {
                R misWeight = PowerHeuristic(lightPdf, scatterSample.pdf);
                if (misWeight > R(0)) Ld = Ld + misWeight * Li * scatterSample.f * s.env_intensity / lightPdf;
            }
        } else {
            bool inShadow = AnyHit(s, shadowRay, K<R>::INF - K<R>::EPS, rng, cnt);
            if (!inShadow) {
                scatterSample.f = DisneyEval(state, -r.direction, state.ffnormal, lightDir, scatterSample.pdf);
                if (scatterSample.pdf > R(0)) {
                    R misWeight = PowerHeuristic(lightPdf, scatterSample.pdf);
                    if (misWeight > R(0)) Ld = Ld + misWeight * Li * scatterSample.f * s.env_intensity / lightPdf;
                }
            }
        }
    }
    if (s.f.lights) {
        LightSampleRec<R> lightSample;
        int index = int(R(rng.next()) * R(s.num_lights));
        // GLSL texelFetch past the end of the light row returns 0 (index == numOfLights when rand()==1)
        Light<R> light{};
        if (index < s.num_lights) light = FetchLight(s, index);
        else { light.radius = light.area = light.type = R(0); }
        SampleOneLight(s, light, scatterPos, lightSample, rng);
        Li = lightSample.emission;
        if (dot(lightSample.direction, lightSample.normal) < R(0)) {
            Ray<R> shadowRay{scatterPos, lightSample.direction};
            if (volmis) {
                Li = Li * EvalTransmittance(s, shadowRay, rng, cnt);
                if (isSurface) scatterSample.f = DisneyEval(state, -r.direction, state.ffnormal, lightSample.direction, scatterSample.pdf);
                else {
                    R p = PhaseHG(dot(-r.direction, lightSample.direction), state.medium.anisotropy);
                    scatterSample.f = V3<R>(p);
                    scatterSample.pdf = p;
                }
                R misWeight = R(1);
                if (light.area > R(0)) misWeight = PowerHeuristic(lightSample.pdf, scatterSample.pdf);
                if (scatterSample.pdf > R(0)) Ld = Ld + misWeight * scatterSample.f * Li / lightSample.pdf;
            } else {
                bool inShadow = AnyHit(s, shadowRay, lightSample.dist - K<R>::EPS, rng, cnt);
                if (!inShadow) {
                    scatterSample.f = DisneyEval(state, -r.direction, state.ffnormal, lightSample.direction, scatterSample.pdf);
                    R misWeight = R(1);
                    if (light.area > R(0)) misWeight = PowerHeuristic(lightSample.pdf, scatterSample.pdf);
                    if (scatterSample.pdf > R(0)) Ld = Ld + misWeight * Li * scatterSample.f / lightSample.pdf;
                }
            }
        }
    }
    return Ld;
}

// pathtrace.glsl:285-476 ; returns radiance, alpha in alphaOut
template <class R> inline V3<R> PathTrace(const Scene<R>& s, Ray<R> r, Rng& rng, Counters& cnt, R& alphaOut) {
    V3<R> radiance(R(0));
    V3<R> throughput(R(1));
    State<R> state;
    LightSampleRec<R> lightSample;
    ScatterSampleRec<R> scatterSample;
    R alpha = R(1);
    bool inMedium = false, mediumSampled = false, surfaceScatter = false;
    const Flags& f = s.f;
    // the reference's loop has no bound; PT_MAX_PATH_ITERATIONS (pt_cuda.h)
    // ends a path that alpha pass-through keeps at the same depth
    state.depth = 0;
    for (int guard = 1;; state.depth++, guard++) {
        if (guard > PT_MAX_PATH_ITERATIONS) {
            cnt.truncated++;
            break;
        }
        bool hit = ClosestHit(s, r, state, lightSample, cnt);
        if (!hit) {
            if ((f.background || f.transparent_background) && state.depth == 0) alpha = R(0);
            if (!(f.hide_emitters && !(state.depth > 0))) {
                if (f.uniform_light) radiance = radiance + s.uniform_light_col * throughput;
                else if (f.envmap) {
                    R envPdf;
                    V3<R> envCol = EvalEnvMap(s, r, envPdf);
                    R misWeight = R(1);
                    if (state.depth > 0) misWeight = PowerHeuristic(scatterSample.pdf, envPdf);
                    if (f.medium && !f.vol_mis && !surfaceScatter) misWeight = R(1);
                    if (misWeight > R(0)) radiance = radiance + misWeight * envCol * throughput * s.env_intensity;
                }
            }
            break;
        }
        GetMaterial(s, state, r);
        radiance = radiance + state.mat.emission * throughput;
        if (f.lights && state.isEmitter) {
            R misWeight = R(1);
            if (state.depth > 0) misWeight = PowerHeuristic(scatterSample.pdf, lightSample.pdf);
            if (f.medium && !f.vol_mis && !surfaceScatter) misWeight = R(1);
            radiance = radiance + misWeight * lightSample.emission * throughput;
            break;
        }
        if (state.depth == f.max_depth) break;
        if (f.medium) {
            mediumSampled = false;
            surfaceScatter = false;
            if (inMedium) {
                if (state.medium.type == MEDIUM_ABSORB) {
                    throughput = throughput * vexp(-(V3<R>(R(1)) - state.medium.color) * state.hitDist * state.medium.density);
                } else if (state.medium.type == MEDIUM_EMISSIVE) {
                    radiance = radiance + state.medium.color * state.hitDist * state.medium.density * throughput;
                } else {
                    R scatterDist = fminR(-std::log(R(rng.next())) / state.medium.density, state.hitDist);
                    mediumSampled = scatterDist < state.hitDist;
                    if (mediumSampled) {
                        throughput = throughput * state.medium.color;
                        r.origin = r.origin + r.direction * scatterDist;
                        state.fhp = r.origin;
                        radiance = radiance + DirectLight(s, r, state, false, rng, cnt) * throughput;
                        R h1 = R(rng.next());
                        R h2 = R(rng.next());
                        V3<R> scatterDir = SampleHG(-r.direction, state.medium.anisotropy, h1, h2);
                        scatterSample.pdf = PhaseHG(dot(-r.direction, scatterDir), state.medium.anisotropy);
                        r.direction = scatterDir;
                    }
                }
            }
        }
        if (!mediumSampled) {
            if (f.alpha_test && AlphaSkip(state.mat, rng)) {
                scatterSample.L = r.direction;
                state.depth--;
            } else {
                surfaceScatter = true;
                radiance = radiance + DirectLight(s, r, state, true, rng, cnt) * throughput;
                scatterSample.f = DisneySample(state, -r.direction, state.ffnormal, scatterSample.L, scatterSample.pdf, rng);
                if (scatterSample.pdf > R(0)) throughput = throughput * (scatterSample.f / scatterSample.pdf);
                else break;
            }
            r.direction = scatterSample.L;
            r.origin = state.fhp + r.direction * K<R>::EPS;
            if (f.medium) {
                if (dot(r.direction, state.normal) < R(0) && state.mat.medium.type != MEDIUM_NONE) {
                    inMedium = true;
                    state.medium = state.mat.medium;
                } else if (state.mat.medium.type != MEDIUM_NONE) inMedium = false;
            }
        }
        if (f.rr && state.depth >= f.rr_depth) {
            R q = fminR(fmaxR(throughput.x, fmaxR(throughput.y, throughput.z)) + R(0.001), R(0.95));
            if (R(rng.next()) > q) break;
            throughput = throughput / q;
        }
    }
    alphaOut = alpha;
    return radiance;
}

// ------------------------------------------------------ detached estimator
// PathTrace with the sampling held at one parameter set and the values taken
// at another: directions, lobe and light choices, MIS weights and Russian
// roulette come from scene `s` (parameters theta0) exactly as PathTrace
// draws them, while BSDF values, material emission and light emission come
// from `e` (the same scene with parameters theta).  Its expectation is the
// image at theta; at theta = theta0 it is PathTrace itself.  Its derivative
// in theta is what path-replay backpropagation estimates, so finite
// differences of it (in R = double) check the adjoint pass.  Surfaces and
// analytic lights only: no media, alpha test, environment map or roughness
// mollification.
template <class R> inline V3<R> PathTraceDetached(const Scene<R>& s, const Scene<R>& e, Ray<R> r, Rng& rng,
                                                  Counters& cnt) {
    V3<R> radiance(R(0));
    V3<R> throughput(R(1));    // at theta (values)
    V3<R> throughput0(R(1));   // at theta0 (Russian roulette)
    State<R> state, stateE;
    LightSampleRec<R> lightSample;
    R scatterPdf = 0;
    const Flags& f = s.f;
    state.depth = 0;
    for (int guard = 1;; state.depth++, guard++) {
        if (guard > PT_MAX_PATH_ITERATIONS) break;
        // same geometry in both scenes: the hit is the same, the light
        // emission of an emitter hit is theta's
        bool hit = ClosestHit(e, r, state, lightSample, cnt);
        if (!hit) {
            if (!(f.hide_emitters && !(state.depth > 0)) && f.uniform_light)
                radiance = radiance + e.uniform_light_col * throughput;
            break;
        }
        stateE = state;
        GetMaterial(s, state, r);
        GetMaterial(e, stateE, r);
        radiance = radiance + stateE.mat.emission * throughput;
        if (f.lights && state.isEmitter) {
            R misWeight = R(1);
            if (state.depth > 0) misWeight = PowerHeuristic(scatterPdf, lightSample.pdf);
            radiance = radiance + misWeight * lightSample.emission * throughput;
            break;
        }
        if (state.depth == f.max_depth) break;
        // next-event estimation (DirectLight's analytic-light part)
        if (f.lights) {
            V3<R> scatterPos = state.fhp + state.normal * K<R>::EPS;
            LightSampleRec<R> ls;
            int index = int(R(rng.next()) * R(s.num_lights));
            Light<R> light{}, lightE{};
            if (index < s.num_lights) {
                light = FetchLight(s, index);
                lightE = FetchLight(e, index);
            } else {
                light.radius = light.area = light.type = R(0);
                lightE = light;
            }
            SampleOneLight(s, light, scatterPos, ls, rng);
            const V3<R> LiE = lightE.emission * R(s.num_lights);
            if (dot(ls.direction, ls.normal) < R(0)) {
                Ray<R> shadowRay{scatterPos, ls.direction};
                bool inShadow = AnyHit(s, shadowRay, ls.dist - K<R>::EPS, rng, cnt);
                if (!inShadow) {
                    R sfPdf;
                    DisneyEval(state, -r.direction, state.ffnormal, ls.direction, sfPdf);
                    R pdfE;
                    const V3<R> sfE = DisneyEval(stateE, -r.direction, state.ffnormal, ls.direction, pdfE);
                    R misWeight = R(1);
                    if (light.area > R(0)) misWeight = PowerHeuristic(ls.pdf, sfPdf);
                    if (sfPdf > R(0)) radiance = radiance + misWeight * LiE * sfE / ls.pdf * throughput;
                }
            }
        }
        V3<R> L;
        R pdf;
        const V3<R> f0 = DisneySample(state, -r.direction, state.ffnormal, L, pdf, rng);
        if (!(pdf > R(0))) break;
        R pdfE;
        const V3<R> fE = DisneyEval(stateE, -r.direction, state.ffnormal, L, pdfE);
        throughput = throughput * (fE / pdf);
        throughput0 = throughput0 * (f0 / pdf);
        scatterPdf = pdf;
        r.direction = L;
        r.origin = state.fhp + r.direction * K<R>::EPS;
        if (f.rr && state.depth >= f.rr_depth) {
            R q = fminR(fmaxR(throughput0.x, fmaxR(throughput0.y, throughput0.z)) + R(0.001), R(0.95));
            if (R(rng.next()) > q) break;
            throughput = throughput / q;
            throughput0 = throughput0 / q;
        }
    }
    return radiance;
}

// ------------------------------------------------------------ camera ray
// tile.glsl:41-74 for pixel (px, py) of the full frame.  The reference
// renders tile (tx, ty) of tileW x tileH into a viewport at the origin, so
// gl_FragCoord (and the RNG seed) is tile-local; coordsTile is
// mix(tileOffset, tileOffset + invNumTiles, TexCoords).
template <class R> inline Ray<R> CameraRay(const pt_camera& cam, const pt_render_options& o, int px, int py, Rng& rng) {
    const int tw = o.tile_width, th = o.tile_height;
    const int tx = px / tw, ty = py / th;
    const int lx = px - tx * tw, ly = py - ty * th;
    const float invx = (float)tw / (float)o.render_width, invy = (float)th / (float)o.render_height;
    // TexCoords of the fragment centre within the tile viewport
    R tcx = (R(lx) + R(0.5)) / R(tw), tcy = (R(ly) + R(0.5)) / R(th);
    R offx = R((float)tx * invx), offy = R((float)ty * invy);
    R cx = offx * (R(1) - tcx) + (offx + R(invx)) * tcx;
    R cy = offy * (R(1) - tcy) + (offy + R(invy)) * tcy;
    R r1 = R(2) * R(rng.next());
    R r2 = R(2) * R(rng.next());
    R jx = r1 < R(1) ? std::sqrt(r1) - R(1) : R(1) - std::sqrt(R(2) - r1);
    R jy = r2 < R(1) ? std::sqrt(r2) - R(1) : R(1) - std::sqrt(R(2) - r2);
    R resx = R(o.render_width), resy = R(o.render_height);
    jx = jx / (resx * R(0.5));
    jy = jy / (resy * R(0.5));
    R dx = (cx * R(2) - R(1)) + jx;
    R dy = (cy * R(2) - R(1)) + jy;
    R scale = std::tan(R(cam.fov) * R(0.5));
    dy *= resy / resx * scale;
    dx *= scale;
    V3<R> right(R(cam.right[0]), R(cam.right[1]), R(cam.right[2]));
    V3<R> up(R(cam.up[0]), R(cam.up[1]), R(cam.up[2]));
    V3<R> fwd(R(cam.forward[0]), R(cam.forward[1]), R(cam.forward[2]));
    V3<R> pos(R(cam.position[0]), R(cam.position[1]), R(cam.position[2]));
    V3<R> rayDir = normalize(dx * right + dy * up + fwd);
    V3<R> focalPoint = R(cam.focal_dist) * rayDir;
    R cam_r1 = R(rng.next()) * K<R>::TWO_PI;
    R cam_r2 = R(rng.next()) * R(cam.aperture);
    V3<R> aperturePos = (std::cos(cam_r1) * right + std::sin(cam_r1) * up) * std::sqrt(cam_r2);
    V3<R> finalDir = normalize(focalPoint - aperturePos);
    return Ray<R>{pos + aperturePos, finalDir};
}

// Frame number the reference's tile state machine gives tile (tx, ty) in
// sample pass `pass` (Renderer.cpp:641-762 with Main.cpp's Update-then-Render
// loop): the first rendered tile uses frameNum 2, tiles run left to right
// from the top tile row (ty = numTiles.y-1) down.
inline uint32_t FrameNumber(const pt_render_options& o, int pass, int tx, int ty) {
    int nx = (o.render_width + o.tile_width - 1) / o.tile_width;
    int ny = (o.render_height + o.tile_height - 1) / o.tile_height;
    return (uint32_t)(2 + pass * nx * ny + (ny - 1 - ty) * nx + tx);
}

}  // namespace orc
