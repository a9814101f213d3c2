// pt_device.cuh - device math, RNG, sampling, Disney BSDF, lights and envmap
// of the path tracer (sm_103a).
//
// Each function restates the GLSL function of the reference named in its
// comment (paths relative to the reference project).  Arithmetic is FP32 with
// the CUDA math library's accurate functions (no fast-math); the oracle
// (pt_oracle.hpp) restates the same functions on the CPU.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ptgb {

// ------------------------------------------------------------- constants
// common/globals.glsl:25-44
#define PT_PI 3.14159265358979323f
#define PT_INV_PI 0.31830988618379067f
#define PT_TWO_PI 6.28318530717958648f
#define PT_INV_TWO_PI 0.15915494309189533f
#define PT_INV_4_PI 0.07957747154594766f
#define PT_EPS 0.0003f
#define PT_INF 1000000.0f

enum { QUAD_LIGHT = 0, SPHERE_LIGHT = 1, DISTANT_LIGHT = 2 };
enum { ALPHA_MODE_OPAQUE = 0, ALPHA_MODE_BLEND = 1, ALPHA_MODE_MASK = 2 };
enum { MEDIUM_NONE = 0, MEDIUM_ABSORB = 1, MEDIUM_SCATTER = 2, MEDIUM_EMISSIVE = 3 };

// Runtime feature bits (the reference compiles these as #defines,
// Renderer.cpp:400-476; uniform branches here).
enum : uint32_t {
    F_LIGHTS = 1u << 0,
    F_RR = 1u << 1,
    F_UNIFORM_LIGHT = 1u << 2,
    F_HIDE_EMITTERS = 1u << 3,
    F_BACKGROUND = 1u << 4,       // OPT_BACKGROUND || OPT_TRANSPARENT_BACKGROUND
    F_ALPHA_TEST = 1u << 5,
    F_MOLLIFY = 1u << 6,
    F_ENVMAP = 1u << 7,           // OPT_ENVMAP && !OPT_UNIFORM_LIGHT
    F_MEDIUM = 1u << 8,
    F_VOL_MIS = 1u << 9,
    F_TEXTURES = 1u << 10,        // the scene has texture maps (texelFetch / texture() on the array)
    F_OPENGL_NORMALMAP = 1u << 11,
};

// ------------------------------------------------------------------ float3
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float a) { return {a, a, a}; }
__device__ __forceinline__ V3 v3(float a, float b, float c) { return {a, b, c}; }
__device__ __forceinline__ V3 v3(float4 a) { return {a.x, a.y, a.z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V3 operator/(V3 a, V3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
// a + b * s rounded after the product and after the sum, never fused: ray
// origins (hit points, offsets) come out the same in every kernel and equal
// the reference's GLSL evaluated without contraction, so surfaces that meet
// at a shared plane are told apart the same way everywhere.
__device__ __forceinline__ V3 madd_rn(V3 a, V3 b, float s) {
    return {__fadd_rn(a.x, __fmul_rn(b.x, s)), __fadd_rn(a.y, __fmul_rn(b.y, s)), __fadd_rn(a.z, __fmul_rn(b.z, s))};
}
__device__ __forceinline__ V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float length(V3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ V3 normalize(V3 a) { return a / length(a); }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ V3 mix3(V3 a, V3 b, float t) { return {mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)}; }
__device__ __forceinline__ V3 vexp(V3 a) { return {expf(a.x), expf(a.y), expf(a.z)}; }
__device__ __forceinline__ float maxc(V3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
// GLSL reflect / refract
__device__ __forceinline__ V3 reflect3(V3 I, V3 N) { return I - (2.0f * dot(N, I)) * N; }
__device__ __forceinline__ V3 refract3(V3 I, V3 N, float eta) {
    float d = dot(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return v3(0.0f);
    return eta * I - (eta * d + sqrtf(k)) * N;
}

// -------------------------------------------------------------------- RNG
// common/globals.glsl:149-166 (PCG4D hash)
struct Rng {
    uint32_t x, y, z, w;
    __device__ __forceinline__ void init(uint32_t px, uint32_t py, uint32_t frame) {
        x = px; y = py; z = frame; w = px + py;
    }
    __device__ __forceinline__ float next() {
        x = x * 1664525u + 1013904223u;
        y = y * 1664525u + 1013904223u;
        z = z * 1664525u + 1013904223u;
        w = w * 1664525u + 1013904223u;
        x += y * w; y += z * x; z += x * y; w += y * z;
        x ^= x >> 16u; y ^= y >> 16u; z ^= z >> 16u; w ^= w >> 16u;
        x += y * w; y += z * x; z += x * y; w += y * z;
        // float(seed.x) / float(0xffffffffu): the divisor rounds to 2^32, so
        // the quotient is an exact scaling
        return __uint2float_rn(x) * 2.3283064365386963e-10f;
    }
};

__device__ __forceinline__ float Luminance(V3 c) {  // globals.glsl:173-176
    return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z;
}

// ------------------------------------------------------------ structures
// common/globals.glsl:46-139
struct Ray { V3 origin, direction; };
struct Medium { int type; float density; V3 color; float anisotropy; };
struct Material {
    V3 baseColor; float opacity; int alphaMode; float alphaCutoff;
    V3 emission; float anisotropic, metallic, roughness, subsurface, specularTint;
    float sheen, sheenTint, clearcoat, clearcoatRoughness, specTrans, ior, ax, ay;
    Medium medium;
};
struct LightSample { V3 normal, emission, direction; float dist, pdf; };
struct Light { V3 position, emission, u, v; float radius, area, type; };

// ------------------------------------------------------------- sampling
// common/sampling.glsl:25-32, of the half vector H in the shading frame.
// The reference's denominator 1 + (a^2 - 1) (N.H)^2 cancels near the lobe's
// peak (N.H -> 1, small a): the last bits of N.H then reach the result
// amplified by 1 / (1 - (N.H)^2), far past 1e-5 relative in FP32.  For a
// unit H it equals (Hx^2 + Hy^2 + a^2 Hz^2) / |H|^2, a ratio of sums of
// positive terms that is evaluated here instead: the same function, exact
// to a few ulp whatever the angle, and free of H's normalisation error.
__device__ __forceinline__ float GTR1(V3 H, float a) {
    if (a >= 1.0f) return PT_INV_PI;
    float a2 = a * a;
    float s = H.x * H.x + H.y * H.y;
    float z2 = H.z * H.z;
    float t = (s + a2 * z2) / (s + z2);
    return (a2 - 1.0f) / (PT_PI * logf(a2) * t);
}
// sampling.glsl:34-47
__device__ __forceinline__ V3 SampleGTR1(float rgh, float r1, float r2) {
    float a = fmaxf(0.001f, rgh);
    float a2 = a * a;
    float phi = r1 * PT_TWO_PI;
    float cosTheta = sqrtf((1.0f - powf(a2, 1.0f - r2)) / (1.0f - a2));
    float sinTheta = clampf(sqrtf(1.0f - (cosTheta * cosTheta)), 0.0f, 1.0f);
    float sinPhi, cosPhi;
    sincosf(phi, &sinPhi, &cosPhi);
    return v3(sinTheta * cosPhi, sinTheta * sinPhi, cosTheta);
}
// sampling.glsl:70-88
__device__ __forceinline__ V3 SampleGGXVNDF(V3 V, float ax, float ay, float r1, float r2) {
    V3 Vh = normalize(v3(ax * V.x, ay * V.y, V.z));
    float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
    V3 T1 = lensq > 0.0f ? v3(-Vh.y, Vh.x, 0.0f) * (1.0f / sqrtf(lensq)) : v3(1.0f, 0.0f, 0.0f);
    V3 T2 = cross(Vh, T1);
    float r = sqrtf(r1);
    float phi = 2.0f * PT_PI * r2;
    float s_, c_;
    sincosf(phi, &s_, &c_);
    float t1 = r * c_;
    float t2 = r * s_;
    float s = 0.5f * (1.0f + Vh.z);
    t2 = (1.0f - s) * sqrtf(1.0f - t1 * t1) + s * t2;
    V3 Nh = t1 * T1 + t2 * T2 + sqrtf(fmaxf(0.0f, 1.0f - t1 * t1 - t2 * t2)) * Vh;
    return normalize(v3(ax * Nh.x, ay * Nh.y, fmaxf(0.0f, Nh.z)));
}
// sampling.glsl:90-96
__device__ __forceinline__ float GTR2Aniso(float NDotH, float HDotX, float HDotY, float ax, float ay) {
    float a = HDotX / ax;
    float b = HDotY / ay;
    float c = a * a + b * b + NDotH * NDotH;
    return 1.0f / (PT_PI * ax * ay * c * c);
}
// sampling.glsl:109-114
__device__ __forceinline__ float SmithG(float NDotV, float alphaG) {
    float a = alphaG * alphaG;
    float b = NDotV * NDotV;
    return (2.0f * NDotV) / (NDotV + sqrtf(a + b - a * b));
}
// sampling.glsl:116-122
__device__ __forceinline__ float SmithGAniso(float NDotV, float VDotX, float VDotY, float ax, float ay) {
    float a = VDotX * ax;
    float b = VDotY * ay;
    float c = NDotV;
    return (2.0f * NDotV) / (NDotV + sqrtf(a * a + b * b + c * c));
}
// sampling.glsl:124-129
__device__ __forceinline__ float SchlickWeight(float u) {
    float m = clampf(1.0f - u, 0.0f, 1.0f);
    float m2 = m * m;
    return m2 * m2 * m;
}
// sampling.glsl:131-145
__device__ __forceinline__ float DielectricFresnel(float cosThetaI, float eta) {
    float sinThetaTSq = eta * eta * (1.0f - cosThetaI * cosThetaI);
    if (sinThetaTSq > 1.0f) return 1.0f;
    float cosThetaT = sqrtf(fmaxf(1.0f - sinThetaTSq, 0.0f));
    float rs = (eta * cosThetaT - cosThetaI) / (eta * cosThetaT + cosThetaI);
    float rp = (eta * cosThetaI - cosThetaT) / (eta * cosThetaI + cosThetaT);
    return 0.5f * (rs * rs + rp * rp);
}
// sampling.glsl:147-156
__device__ __forceinline__ V3 CosineSampleHemisphere(float r1, float r2) {
    float r = sqrtf(r1);
    float phi = PT_TWO_PI * r2;
    float s, c;
    sincosf(phi, &s, &c);
    V3 dir;
    dir.x = r * c;
    dir.y = r * s;
    dir.z = sqrtf(fmaxf(0.0f, 1.0f - dir.x * dir.x - dir.y * dir.y));
    return dir;
}
// sampling.glsl:158-163
__device__ __forceinline__ V3 UniformSampleHemisphere(float r1, float r2) {
    float r = sqrtf(fmaxf(0.0f, 1.0f - r1 * r1));
    float phi = PT_TWO_PI * r2;
    float s, c;
    sincosf(phi, &s, &c);
    return v3(r * c, r * s, r1);
}
// sampling.glsl:173-177
__device__ __forceinline__ float PowerHeuristic(float a, float b) {
    float t = a * a;
    return t / (b * b + t);
}
// sampling.glsl:179-184
__device__ __forceinline__ void Onb(V3 N, V3& T, V3& B) {
    V3 up = fabsf(N.z) < 0.9999999f ? v3(0.0f, 0.0f, 1.0f) : v3(1.0f, 0.0f, 0.0f);
    T = normalize(cross(up, N));
    B = cross(N, T);
}
// sampling.glsl:250-271
__device__ __forceinline__ V3 SampleHG(V3 V, float g, float r1, float r2) {
    float cosTheta;
    if (fabsf(g) < 0.001f) cosTheta = 1.0f - 2.0f * r2;
    else {
        float sqrTerm = (1.0f - g * g) / (1.0f + g - 2.0f * g * r2);
        cosTheta = -(1.0f + g * g - sqrTerm * sqrTerm) / (2.0f * g);
    }
    float phi = r1 * PT_TWO_PI;
    float sinTheta = clampf(sqrtf(1.0f - (cosTheta * cosTheta)), 0.0f, 1.0f);
    float sinPhi, cosPhi;
    sincosf(phi, &sinPhi, &cosPhi);
    V3 v1, v2;
    Onb(V, v1, v2);
    return sinTheta * cosPhi * v1 + sinTheta * sinPhi * v2 + cosTheta * V;
}
// sampling.glsl:273-277
__device__ __forceinline__ float PhaseHG(float cosTheta, float g) {
    float denom = 1.0f + g * g + 2.0f * g * cosTheta;
    return PT_INV_4_PI * (1.0f - g * g) / (denom * sqrtf(denom));
}

// ----------------------------------------------------------- intersection
// common/intersection.glsl:25-45
__device__ __forceinline__ float SphereIntersect(float rad, V3 pos, const Ray& r) {
    V3 op = pos - r.origin;
    float eps = 0.001f;
    float b = dot(op, r.direction);
    float det = b * b - dot(op, op) + rad * rad;
    if (det < 0.0f) return PT_INF;
    det = sqrtf(det);
    float t1 = b - det;
    if (t1 > eps) return t1;
    float t2 = b + det;
    if (t2 > eps) return t2;
    return PT_INF;
}
// common/intersection.glsl:47-66
__device__ __forceinline__ float RectIntersect(V3 pos, V3 u, V3 v, V3 n, float pw, const Ray& r) {
    float dt = dot(r.direction, n);
    float t = (pw - dot(n, r.origin)) / dt;
    if (t > PT_EPS) {
        V3 p = r.origin + r.direction * t;
        V3 vi = p - pos;
        float a1 = dot(u, vi);
        if (a1 >= 0.0f && a1 <= 1.0f) {
            float a2 = dot(v, vi);
            if (a2 >= 0.0f && a2 <= 1.0f) return t;
        }
    }
    return PT_INF;
}

// -------------------------------------------------------------- Disney
// common/disney.glsl:39-47
__device__ __forceinline__ V3 ToWorld(V3 X, V3 Y, V3 Z, V3 V) { return V.x * X + V.y * Y + V.z * Z; }
__device__ __forceinline__ V3 ToLocal(V3 X, V3 Y, V3 Z, V3 V) { return v3(dot(V, X), dot(V, Y), dot(V, Z)); }

struct Lobes {
    float dielectricWt, metalWt, glassWt, diffPr, dielectricPr, metalPr, glassPr, clearCtPr, F0;
    V3 Csheen, Cspec0;
};
// disney.glsl:49-59 (TintColors) and the lobe weights of 161-181 / 271-291
__device__ __forceinline__ Lobes LobeWeights(const Material& mat, float eta, V3 V) {
    Lobes lb;
    float lum = Luminance(mat.baseColor);
    V3 ctint = lum > 0.0f ? mat.baseColor / lum : v3(1.0f);
    lb.F0 = (1.0f - eta) / (1.0f + eta);
    lb.F0 *= lb.F0;
    lb.Cspec0 = lb.F0 * mix3(v3(1.0f), ctint, mat.specularTint);
    lb.Csheen = mix3(v3(1.0f), ctint, mat.sheenTint);
    lb.dielectricWt = (1.0f - mat.metallic) * (1.0f - mat.specTrans);
    lb.metalWt = mat.metallic;
    lb.glassWt = (1.0f - mat.metallic) * mat.specTrans;
    float schlickWt = SchlickWeight(V.z);
    lb.diffPr = lb.dielectricWt * Luminance(mat.baseColor);
    lb.dielectricPr = lb.dielectricWt * Luminance(mix3(lb.Cspec0, v3(1.0f), schlickWt));
    lb.metalPr = lb.metalWt * Luminance(mix3(mat.baseColor, v3(1.0f), schlickWt));
    lb.glassPr = lb.glassWt;
    lb.clearCtPr = 0.25f * mat.clearcoat;
    float invTotalWt = 1.0f / (lb.diffPr + lb.dielectricPr + lb.metalPr + lb.glassPr + lb.clearCtPr);
    lb.diffPr *= invTotalWt;
    lb.dielectricPr *= invTotalWt;
    lb.metalPr *= invTotalWt;
    lb.glassPr *= invTotalWt;
    lb.clearCtPr *= invTotalWt;
    return lb;
}
// disney.glsl:61-88
__device__ __forceinline__ V3 EvalDisneyDiffuse(const Material& mat, V3 Csheen, V3 V, V3 L, V3 H, float& pdf) {
    pdf = 0.0f;
    if (L.z <= 0.0f) return v3(0.0f);
    float LDotH = dot(L, H);
    float Rr = 2.0f * mat.roughness * LDotH * LDotH;
    float FL = SchlickWeight(L.z);
    float FV = SchlickWeight(V.z);
    float Fretro = Rr * (FL + FV + FL * FV * (Rr - 1.0f));
    float Fd = (1.0f - 0.5f * FL) * (1.0f - 0.5f * FV);
    float Fss90 = 0.5f * Rr;
    float Fss = mixf(1.0f, Fss90, FL) * mixf(1.0f, Fss90, FV);
    float ss = 1.25f * (Fss * (1.0f / (L.z + V.z) - 0.5f) + 0.5f);
    float FH = SchlickWeight(LDotH);
    V3 Fsheen = FH * mat.sheen * Csheen;
    pdf = L.z * PT_INV_PI;
    return PT_INV_PI * mat.baseColor * mixf(Fd + Fretro, ss, mat.subsurface) + Fsheen;
}
// disney.glsl:90-102
__device__ __forceinline__ V3 EvalMicrofacetReflection(const Material& mat, V3 V, V3 L, V3 H, V3 F, float& pdf) {
    pdf = 0.0f;
    if (L.z <= 0.0f) return v3(0.0f);
    float D = GTR2Aniso(H.z, H.x, H.y, mat.ax, mat.ay);
    float G1 = SmithGAniso(fabsf(V.z), V.x, V.y, mat.ax, mat.ay);
    float G2 = G1 * SmithGAniso(fabsf(L.z), L.x, L.y, mat.ax, mat.ay);
    pdf = G1 * D / (4.0f * V.z);
    return F * D * G2 / (4.0f * L.z * V.z);
}
// disney.glsl:104-123
__device__ __forceinline__ V3 EvalMicrofacetRefraction(const Material& mat, float eta, V3 V, V3 L, V3 H, V3 F, float& pdf) {
    pdf = 0.0f;
    if (L.z >= 0.0f) return v3(0.0f);
    float LDotH = dot(L, H);
    float VDotH = dot(V, H);
    float D = GTR2Aniso(H.z, H.x, H.y, mat.ax, mat.ay);
    float G1 = SmithGAniso(fabsf(V.z), V.x, V.y, mat.ax, mat.ay);
    float G2 = G1 * SmithGAniso(fabsf(L.z), L.x, L.y, mat.ax, mat.ay);
    float denom = LDotH + VDotH * eta;
    denom *= denom;
    float eta2 = eta * eta;
    float jacobian = fabsf(LDotH) / denom;
    pdf = G1 * fmaxf(0.0f, VDotH) * D * jacobian / V.z;
    V3 sq = v3(sqrtf(mat.baseColor.x), sqrtf(mat.baseColor.y), sqrtf(mat.baseColor.z));  // pow(baseColor, 0.5)
    return sq * (v3(1.0f) - F) * D * G2 * fabsf(VDotH) * jacobian * eta2 / fabsf(L.z * V.z);
}
// disney.glsl:125-140
__device__ __forceinline__ V3 EvalClearcoat(const Material& mat, V3 V, V3 L, V3 H, float& pdf) {
    pdf = 0.0f;
    if (L.z <= 0.0f) return v3(0.0f);
    float VDotH = dot(V, H);
    float F = mixf(0.04f, 1.0f, SchlickWeight(VDotH));
    float D = GTR1(H, mat.clearcoatRoughness);
    float G = SmithG(L.z, 0.25f) * SmithG(V.z, 0.25f);
    float jacobian = 1.0f / (4.0f * VDotH);
    pdf = D * H.z * jacobian;
    return v3(F) * D * G;
}

// disney.glsl:244-351 ; lobeF/lobePdf (optional) receive each lobe's
// weighted contribution (diffuse, dielectric, metal, glass, clearcoat).
// Not inlined: it has three call sites per path vertex, and the copies
// cost more in instruction-cache misses than the call does.
static __device__ __noinline__ V3 DisneyEval(const Material& mat, float eta, V3 V, V3 N, V3 L, float& pdf,
                                         V3* lobeF = nullptr, float* lobePdf = nullptr) {
    pdf = 0.0f;
    V3 f = v3(0.0f);
    V3 T, B;
    Onb(N, T, B);
    V = ToLocal(T, B, N, V);
    L = ToLocal(T, B, N, L);
    V3 H;
    if (L.z > 0.0f) H = normalize(L + V);
    else H = normalize(L + V * eta);
    if (H.z < 0.0f) H = -H;
    Lobes lb = LobeWeights(mat, eta, V);
    bool refl = L.z * V.z > 0.0f;
    float tmpPdf = 0.0f;
    float VDotH = fabsf(dot(V, H));
    float absLz = fabsf(L.z);
    if (lobeF)
        for (int i = 0; i < 5; ++i) { lobeF[i] = v3(0.0f); lobePdf[i] = 0.0f; }
    if (lb.diffPr > 0.0f && refl) {
        V3 c = EvalDisneyDiffuse(mat, lb.Csheen, V, L, H, tmpPdf) * lb.dielectricWt;
        f = f + c;
        pdf += tmpPdf * lb.diffPr;
        if (lobeF) { lobeF[0] = c * absLz; lobePdf[0] = tmpPdf * lb.diffPr; }
    }
    if (lb.dielectricPr > 0.0f && refl) {
        float F = (DielectricFresnel(VDotH, 1.0f / mat.ior) - lb.F0) / (1.0f - lb.F0);
        V3 c = EvalMicrofacetReflection(mat, V, L, H, mix3(lb.Cspec0, v3(1.0f), F), tmpPdf) * lb.dielectricWt;
        f = f + c;
        pdf += tmpPdf * lb.dielectricPr;
        if (lobeF) { lobeF[1] = c * absLz; lobePdf[1] = tmpPdf * lb.dielectricPr; }
    }
    if (lb.metalPr > 0.0f && refl) {
        V3 F = mix3(mat.baseColor, v3(1.0f), SchlickWeight(VDotH));
        V3 c = EvalMicrofacetReflection(mat, V, L, H, F, tmpPdf) * lb.metalWt;
        f = f + c;
        pdf += tmpPdf * lb.metalPr;
        if (lobeF) { lobeF[2] = c * absLz; lobePdf[2] = tmpPdf * lb.metalPr; }
    }
    if (lb.glassPr > 0.0f) {
        float F = DielectricFresnel(VDotH, eta);
        V3 c;
        float p;
        if (refl) {
            c = EvalMicrofacetReflection(mat, V, L, H, v3(F), tmpPdf) * lb.glassWt;
            p = tmpPdf * lb.glassPr * F;
        } else {
            c = EvalMicrofacetRefraction(mat, eta, V, L, H, v3(F), tmpPdf) * lb.glassWt;
            p = tmpPdf * lb.glassPr * (1.0f - F);
        }
        f = f + c;
        pdf += p;
        if (lobeF) { lobeF[3] = c * absLz; lobePdf[3] = p; }
    }
    if (lb.clearCtPr > 0.0f && refl) {
        V3 c = EvalClearcoat(mat, V, L, H, tmpPdf) * 0.25f * mat.clearcoat;
        f = f + c;
        pdf += tmpPdf * lb.clearCtPr;
        if (lobeF) { lobeF[4] = c * absLz; lobePdf[4] = tmpPdf * lb.clearCtPr; }
    }
    return f * absLz;
}

// disney.glsl:142-242
static __device__ __noinline__ V3 DisneySample(const Material& mat, float eta, V3 V, V3 N, V3& L, float& pdf,
                                              Rng& rng) {
    pdf = 0.0f;
    float r1 = rng.next();
    float r2 = rng.next();
    V3 T, B;
    Onb(N, T, B);
    V = ToLocal(T, B, N, V);
    Lobes lb = LobeWeights(mat, eta, V);
    float cdf0 = lb.diffPr;
    float cdf1 = cdf0 + lb.dielectricPr;
    float cdf2 = cdf1 + lb.metalPr;
    float cdf3 = cdf2 + lb.glassPr;
    float r3 = rng.next();
    if (r3 < cdf0) {
        L = CosineSampleHemisphere(r1, r2);
    } else if (r3 < cdf2) {
        V3 H = SampleGGXVNDF(V, mat.ax, mat.ay, r1, r2);
        if (H.z < 0.0f) H = -H;
        L = normalize(reflect3(-V, H));
    } else if (r3 < cdf3) {
        V3 H = SampleGGXVNDF(V, mat.ax, mat.ay, r1, r2);
        float F = DielectricFresnel(fabsf(dot(V, H)), eta);
        if (H.z < 0.0f) H = -H;
        r3 = (r3 - cdf2) / (cdf3 - cdf2);
        if (r3 < F) L = normalize(reflect3(-V, H));
        else L = normalize(refract3(-V, H, eta));
    } else {
        V3 H = SampleGTR1(mat.clearcoatRoughness, r1, r2);
        if (H.z < 0.0f) H = -H;
        L = normalize(reflect3(-V, H));
    }
    L = ToWorld(T, B, N, L);
    V = ToWorld(T, B, N, V);
    return DisneyEval(mat, eta, V, N, L, pdf);
}

// GetMaterial remapping (common/pathtrace.glsl:25-115) of the 8 float4 words
// of GLSLPT::Material (src/core/Material.h:87-119), texture maps excluded.
__device__ __forceinline__ void LoadMaterial(const float4* __restrict__ mats, int id, Material& mat) {
    const float4* p = mats + 8 * id;
    float4 p1 = __ldg(p + 0), p2 = __ldg(p + 1), p3 = __ldg(p + 2), p4 = __ldg(p + 3);
    float4 p5 = __ldg(p + 4), p6 = __ldg(p + 5), p8 = __ldg(p + 7);
    mat.baseColor = v3(p1.x, p1.y, p1.z);
    mat.anisotropic = p1.w;
    mat.emission = v3(p2.x, p2.y, p2.z);
    mat.metallic = p3.x;
    mat.roughness = fmaxf(p3.y, 0.001f);
    mat.subsurface = p3.z;
    mat.specularTint = p3.w;
    mat.sheen = p4.x;
    mat.sheenTint = p4.y;
    mat.clearcoat = p4.z;
    mat.clearcoatRoughness = mixf(0.1f, 0.001f, p4.w);
    mat.specTrans = p5.x;
    mat.ior = p5.y;
    mat.medium.type = (int)p5.z;
    mat.medium.density = p5.w;
    mat.medium.color = v3(p6.x, p6.y, p6.z);
    mat.medium.anisotropy = clampf(p6.w, -0.9f, 0.9f);
    mat.opacity = p8.x;
    mat.alphaMode = (int)p8.y;
    mat.alphaCutoff = p8.z;
}

__device__ __forceinline__ void FinishMaterial(Material& mat) {  // pathtrace.glsl:109-111
    float aspect = sqrtf(1.0f - mat.anisotropic * 0.9f);
    mat.ax = fmaxf(0.001f, mat.roughness / aspect);
    mat.ay = fmaxf(0.001f, mat.roughness * aspect);
}

// Lights repacked as 4 float4: (position, radius), (emission, area), (u, type), (v, 0)
__device__ __forceinline__ Light LoadLight(const float4* __restrict__ lights, int i) {
    float4 a = __ldg(lights + 4 * i + 0), b = __ldg(lights + 4 * i + 1), c = __ldg(lights + 4 * i + 2),
           d = __ldg(lights + 4 * i + 3);
    Light L;
    L.position = v3(a.x, a.y, a.z);
    L.radius = a.w;
    L.emission = v3(b.x, b.y, b.z);
    L.area = b.w;
    L.u = v3(c.x, c.y, c.z);
    L.type = c.w;
    L.v = v3(d.x, d.y, d.z);
    return L;
}

}  // namespace ptgb
