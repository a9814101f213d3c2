// glsl_shim.hpp - just enough of GLSL 3.30 in C++ to compile the reference's
// path-tracing shaders (src/shaders/common/*.glsl, tile.glsl) on the CPU.
//
// TEST INFRASTRUCTURE ONLY.  Used to build oracle/_ref/libref_glsl*.so in
// this container, which runs the reference's own shader source to pin the
// oracle (pt_oracle.hpp).  Compile with -fsingle-precision-constant so GLSL
// float literals stay float, and -ffp-contract=off.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace glsl {

typedef unsigned int uint;

struct vec2;
struct vec3;
struct vec4;

template <int A, int B> struct S2 { float v[4]; inline operator vec2() const; };
template <int A, int B, int C> struct S3 {
    float v[4];
    inline operator vec3() const;
    inline S3& operator=(const vec3& o);
    inline S3& operator*=(const vec3& o);
};
template <int A, int B, int C, int D> struct S4 { float v[4]; inline operator vec4() const; };

struct vec2 {
    union {
        struct { float x, y; };
        struct { float r, g; };
        float e[2];
    };
    vec2() : x(0), y(0) {}
    explicit vec2(float s) : x(s), y(s) {}
    vec2(float a, float b) : x(a), y(b) {}
    vec2(int a, int b) : x(float(a)), y(float(b)) {}
};

struct vec3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
        S3<0, 1, 2> xyz;
        S3<0, 1, 2> rgb;
        float e[3];
    };
    vec3() : x(0), y(0), z(0) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit vec3(const vec4& v);
    vec3(const vec2& a, float c) : x(a.x), y(a.y), z(c) {}
    vec3(const vec3& o) : x(o.x), y(o.y), z(o.z) {}
    vec3& operator=(const vec3& o) { x = o.x; y = o.y; z = o.z; return *this; }
    vec3& operator+=(const vec3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    vec3& operator-=(const vec3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    vec3& operator*=(const vec3& o) { x *= o.x; y *= o.y; z *= o.z; return *this; }
    vec3& operator*=(float s) { x *= s; y *= s; z *= s; return *this; }
    vec3& operator/=(float s) { x /= s; y /= s; z /= s; return *this; }
    vec3& operator/=(const vec3& o) { x /= o.x; y /= o.y; z /= o.z; return *this; }
};

struct vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        S3<0, 1, 2> xyz;
        S3<0, 1, 2> rgb;
        S4<0, 1, 2, 3> xyzw;
        S2<0, 1> xy;
        S3<3, 0, 1> wxy;
        S2<2, 1> bg;
        float e[4];
    };
    vec4() : x(0), y(0), z(0), w(0) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(const vec3& v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec4(const vec4& o) : x(o.x), y(o.y), z(o.z), w(o.w) {}
    vec4& operator=(const vec4& o) { x = o.x; y = o.y; z = o.z; w = o.w; return *this; }
};
inline vec3::vec3(const vec4& v) : x(v.x), y(v.y), z(v.z) {}

template <int A, int B> inline S2<A, B>::operator vec2() const { return vec2(v[A], v[B]); }
template <int A, int B, int C> inline S3<A, B, C>::operator vec3() const { return vec3(v[A], v[B], v[C]); }
template <int A, int B, int C> inline S3<A, B, C>& S3<A, B, C>::operator=(const vec3& o) {
    float a = o.x, b = o.y, c = o.z;
    v[A] = a; v[B] = b; v[C] = c;
    return *this;
}
template <int A, int B, int C> inline S3<A, B, C>& S3<A, B, C>::operator*=(const vec3& o) {
    v[A] *= o.x; v[B] *= o.y; v[C] *= o.z;
    return *this;
}
template <int A, int B, int C, int D> inline S4<A, B, C, D>::operator vec4() const { return vec4(v[A], v[B], v[C], v[D]); }

struct ivec2 {
    int x, y;
    ivec2() : x(0), y(0) {}
    ivec2(int a, int b) : x(a), y(b) {}
    explicit ivec2(const vec2& v) : x(int(v.x)), y(int(v.y)) {}
};
struct ivec3 {
    int x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    explicit ivec3(int s) : x(s), y(s), z(s) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit ivec3(const vec3& v) : x(int(v.x)), y(int(v.y)), z(int(v.z)) {}
};
struct ivec4 {
    union {
        struct { int x, y, z, w; };
        int e[4];
    };
    ivec4() : x(0), y(0), z(0), w(0) {}
    ivec4(int a, int b, int c, int d) : x(a), y(b), z(c), w(d) {}
    explicit ivec4(const vec4& v) : x(int(v.x)), y(int(v.y)), z(int(v.z)), w(int(v.w)) {}
};
struct uvec4 {
    uint x, y, z, w;
    uvec4() : x(0), y(0), z(0), w(0) {}
    uvec4(uint a, uint b, uint c, uint d) : x(a), y(b), z(c), w(d) {}
    uvec4(const vec2& p, uint c, uint d) : x(uint(p.x)), y(uint(p.y)), z(c), w(d) {}
};
inline uvec4 operator*(const uvec4& a, uint s) { return uvec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline uvec4 operator+(const uvec4& a, uint s) { return uvec4(a.x + s, a.y + s, a.z + s, a.w + s); }
inline uvec4 operator>>(const uvec4& a, uint s) { return uvec4(a.x >> s, a.y >> s, a.z >> s, a.w >> s); }
inline uvec4 operator^(const uvec4& a, const uvec4& b) { return uvec4(a.x ^ b.x, a.y ^ b.y, a.z ^ b.z, a.w ^ b.w); }

struct bvec4 { bool x, y, z, w; };

// ---- vec2 / vec3 / vec4 arithmetic -------------------------------------
inline vec2 operator+(const vec2& a, const vec2& b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(const vec2& a, const vec2& b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator*(const vec2& a, const vec2& b) { return vec2(a.x * b.x, a.y * b.y); }
inline vec2 operator/(const vec2& a, const vec2& b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator*(const vec2& a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator*(float s, const vec2& a) { return vec2(s * a.x, s * a.y); }
inline vec2 operator-(const vec2& a, float s) { return vec2(a.x - s, a.y - s); }
inline vec2 operator+(const vec2& a, float s) { return vec2(a.x + s, a.y + s); }
inline vec2& operator/=(vec2& a, const vec2& b) { a.x /= b.x; a.y /= b.y; return a; }

inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(const vec3& a, const vec3& b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, const vec3& a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator/(float s, const vec3& a) { return vec3(s / a.x, s / a.y, s / a.z); }
inline vec3 operator-(const vec3& a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator-(float s, const vec3& a) { return vec3(s - a.x, s - a.y, s - a.z); }
inline vec3 operator+(const vec3& a, float s) { return vec3(a.x + s, a.y + s, a.z + s); }
inline vec3 operator-(const vec3& a, float s) { return vec3(a.x - s, a.y - s, a.z - s); }

inline vec4 operator+(const vec4& a, const vec4& b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator*(const vec4& a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }

// ---- matrices (column-major, m[col][row]) -----------------------------
struct mat3 {
    float m[3][3];
    mat3() { std::memset(m, 0, sizeof m); }
};
struct mat4 {
    float m[4][4];
    mat4() { std::memset(m, 0, sizeof m); }
    mat4(const vec4& c0, const vec4& c1, const vec4& c2, const vec4& c3) {
        const vec4* c[4] = {&c0, &c1, &c2, &c3};
        for (int i = 0; i < 4; ++i) { m[i][0] = c[i]->x; m[i][1] = c[i]->y; m[i][2] = c[i]->z; m[i][3] = c[i]->w; }
    }
};
inline mat3 make_mat3(const mat4& a) {
    mat3 r;
    for (int c = 0; c < 3; ++c) for (int k = 0; k < 3; ++k) r.m[c][k] = a.m[c][k];
    return r;
}
// mat3(c0, c1, c2): three column vectors (tonemap.glsl's ACES matrices)
inline mat3 make_mat3(const vec3& c0, const vec3& c1, const vec3& c2) {
    mat3 r;
    const vec3* c[3] = {&c0, &c1, &c2};
    for (int i = 0; i < 3; ++i) { r.m[i][0] = c[i]->x; r.m[i][1] = c[i]->y; r.m[i][2] = c[i]->z; }
    return r;
}
#define mat3(...) make_mat3(__VA_ARGS__)
// mat * vec: sum taken in column order
inline vec4 operator*(const mat4& a, const vec4& v) {
    vec4 r;
    for (int k = 0; k < 4; ++k) r.e[k] = ((a.m[0][k] * v.x + a.m[1][k] * v.y) + a.m[2][k] * v.z) + a.m[3][k] * v.w;
    return r;
}
inline vec3 operator*(const mat3& a, const vec3& v) {
    vec3 r;
    for (int k = 0; k < 3; ++k) r.e[k] = (a.m[0][k] * v.x + a.m[1][k] * v.y) + a.m[2][k] * v.z;
    return r;
}
// vec * mat: the row vector times the matrix, component j = dot(v, column j)
inline vec3 operator*(const vec3& v, const mat3& a) {
    vec3 r;
    for (int j = 0; j < 3; ++j) r.e[j] = (v.x * a.m[j][0] + v.y * a.m[j][1]) + v.z * a.m[j][2];
    return r;
}
inline mat3 transpose(const mat3& a) {
    mat3 r;
    for (int c = 0; c < 3; ++c) for (int k = 0; k < 3; ++k) r.m[c][k] = a.m[k][c];
    return r;
}
// GLSL inverse(): the shim computes it in double and rounds to float.
inline mat4 inverse(const mat4& a) {
    double m[16];
    for (int c = 0; c < 4; ++c) for (int k = 0; k < 4; ++k) m[c * 4 + k] = a.m[c][k];
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
    mat4 r;
    for (int c = 0; c < 4; ++c) for (int k = 0; k < 4; ++k) r.m[c][k] = float(inv[c * 4 + k] / det);
    return r;
}
inline mat3 inverse(const mat3& a) {
    double A = a.m[0][0], B = a.m[1][0], C = a.m[2][0];
    double D = a.m[0][1], E = a.m[1][1], F = a.m[2][1];
    double G = a.m[0][2], H = a.m[1][2], I = a.m[2][2];
    double c00 = E * I - F * H, c01 = -(D * I - F * G), c02 = D * H - E * G;
    double c10 = -(B * I - C * H), c11 = A * I - C * G, c12 = -(A * H - B * G);
    double c20 = B * F - C * E, c21 = -(A * F - C * D), c22 = A * E - B * D;
    double det = A * c00 + B * c01 + C * c02;
    double cof[3][3] = {{c00, c01, c02}, {c10, c11, c12}, {c20, c21, c22}};
    // inverse(row r, col c) = cof[c][r] / det ; stored [col][row]
    mat3 out;
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) out.m[c][r] = float(cof[c][r] / det);
    return out;
}

// ---- built-in functions -------------------------------------------------
inline float sqrt(float x) { return std::sqrt(x); }
inline float inversesqrt(float x) { return 1.0f / std::sqrt(x); }
inline float abs(float x) { return std::fabs(x); }
inline float sin(float x) { return std::sin(x); }
inline float cos(float x) { return std::cos(x); }
inline float tan(float x) { return std::tan(x); }
inline float acos(float x) { return std::acos(x); }
inline float atan(float y, float x) { return std::atan2(y, x); }
inline float log(float x) { return std::log(x); }
inline float exp(float x) { return std::exp(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline float floor(float x) { return std::floor(x); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline float clamp(float x, float lo, float hi) { return min(max(x, lo), hi); }
inline int clamp(int x, int lo, int hi) { return min(max(x, lo), hi); }
inline float mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
inline vec2 mix(const vec2& a, const vec2& b, const vec2& t) {
    return vec2(a.x * (1.0f - t.x) + b.x * t.x, a.y * (1.0f - t.y) + b.y * t.y);
}
inline float mod(float x, float y) { return x - y * std::floor(x / y); }
inline float sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
inline vec3 clamp(const vec3& v, float lo, float hi) { return vec3(clamp(v.x, lo, hi), clamp(v.y, lo, hi), clamp(v.z, lo, hi)); }
inline vec3 mix(const vec3& a, const vec3& b, float t) { return vec3(mix(a.x, b.x, t), mix(a.y, b.y, t), mix(a.z, b.z, t)); }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline vec3 max(const vec3& a, const vec3& b) { return vec3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline vec3 exp(const vec3& a) { return vec3(exp(a.x), exp(a.y), exp(a.z)); }
inline vec3 pow(const vec3& a, const vec3& b) { return vec3(pow(a.x, b.x), pow(a.y, b.y), pow(a.z, b.z)); }
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(const vec3& a) { return std::sqrt(dot(a, a)); }
inline vec3 normalize(const vec3& a) { return a / length(a); }
inline vec3 reflect(const vec3& I, const vec3& N) { return I - (2.0f * dot(N, I)) * N; }
inline vec3 refract(const vec3& I, const vec3& N, float eta) {
    float d = dot(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return vec3(0.0f);
    return eta * I - (eta * d + std::sqrt(k)) * N;
}
inline bvec4 greaterThanEqual(const vec4& a, const vec4& b) { return {a.x >= b.x, a.y >= b.y, a.z >= b.z, a.w >= b.w}; }
inline bool all(const bvec4& b) { return b.x && b.y && b.z && b.w; }

// ---- samplers -----------------------------------------------------------
// Buffer textures (texelFetch(samplerBuffer, i)): `comps` floats per texel.
struct samplerBuffer { const float* data = nullptr; int comps = 4; };
struct isamplerBuffer { const int* data = nullptr; int comps = 3; };
// 2D float texture of w x h texels with `comps` channels.
struct sampler2D { const float* data = nullptr; int w = 0, h = 0, comps = 4; };
// RGBA8 texture array.
struct sampler2DArray { const uint8_t* data = nullptr; int w = 0, h = 0, layers = 0; };

inline vec4 texelFetch(const samplerBuffer& s, int i) {
    const float* p = s.data + (size_t)i * s.comps;
    return vec4(p[0], s.comps > 1 ? p[1] : 0.0f, s.comps > 2 ? p[2] : 0.0f, s.comps > 3 ? p[3] : 1.0f);
}
struct ivec4t {
    int x, y, z, w;
    struct P { int a, b, c, d; operator ivec3() const { return ivec3(a, b, c); } } xyz;
};
inline ivec4t texelFetch(const isamplerBuffer& s, int i) {
    const int* p = s.data + (size_t)i * s.comps;
    ivec4t r;
    r.x = p[0]; r.y = p[1]; r.z = p[2]; r.w = 1;
    r.xyz = {p[0], p[1], p[2], 1};
    return r;
}
inline vec4 texelFetch(const sampler2D& s, const ivec2& c, int) {
    if (!s.data || c.x < 0 || c.y < 0 || c.x >= s.w || c.y >= s.h) return vec4(0.0f, 0.0f, 0.0f, 0.0f);
    const float* p = s.data + ((size_t)c.y * s.w + c.x) * s.comps;
    return vec4(p[0], s.comps > 1 ? p[1] : 0.0f, s.comps > 2 ? p[2] : 0.0f, s.comps > 3 ? p[3] : 1.0f);
}
// bilinear, GL_REPEAT
inline vec4 texture(const sampler2D& s, const vec2& uv) {
    if (!s.data) return vec4(0.0f, 0.0f, 0.0f, 0.0f);
    float x = uv.x * float(s.w) - 0.5f, y = uv.y * float(s.h) - 0.5f;
    float fx = std::floor(x), fy = std::floor(y);
    float ax = x - fx, ay = y - fy;
    auto wrap = [](long i, int n) { long m = i % n; return m < 0 ? m + n : m; };
    long x0 = wrap((long)fx, s.w), x1 = wrap((long)fx + 1, s.w), y0 = wrap((long)fy, s.h), y1 = wrap((long)fy + 1, s.h);
    vec4 out(0.0f, 0.0f, 0.0f, 1.0f);
    for (int c = 0; c < s.comps && c < 4; ++c) {
        auto t = [&](long xx, long yy) { return s.data[((size_t)yy * s.w + xx) * s.comps + c]; };
        float a = t(x0, y0) * (1.0f - ax) + t(x1, y0) * ax;
        float b = t(x0, y1) * (1.0f - ax) + t(x1, y1) * ax;
        out.e[c] = a * (1.0f - ay) + b * ay;
    }
    return out;
}
inline vec4 texture(const sampler2DArray& s, const vec3& uvl) {
    if (!s.data || s.layers == 0) return vec4(0.0f, 0.0f, 0.0f, 1.0f);
    int layer = (int)std::floor(uvl.z + 0.5f);
    layer = layer < 0 ? 0 : (layer >= s.layers ? s.layers - 1 : layer);
    const uint8_t* base = s.data + (size_t)layer * s.w * s.h * 4;
    float x = uvl.x * float(s.w) - 0.5f, y = uvl.y * float(s.h) - 0.5f;
    float fx = std::floor(x), fy = std::floor(y);
    float ax = x - fx, ay = y - fy;
    auto wrap = [](long i, int n) { long m = i % n; return m < 0 ? m + n : m; };
    long x0 = wrap((long)fx, s.w), x1 = wrap((long)fx + 1, s.w), y0 = wrap((long)fy, s.h), y1 = wrap((long)fy + 1, s.h);
    vec4 out;
    for (int c = 0; c < 4; ++c) {
        auto t = [&](long xx, long yy) { return float(base[((size_t)yy * s.w + xx) * 4 + c]) / 255.0f; };
        float a = t(x0, y0) * (1.0f - ax) + t(x1, y0) * ax;
        float b = t(x0, y1) * (1.0f - ax) + t(x1, y1) * ax;
        out.e[c] = a * (1.0f - ay) + b * ay;
    }
    return out;
}

}  // namespace glsl
