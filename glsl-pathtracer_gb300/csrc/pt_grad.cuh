// pt_grad.cuh - derivatives of the Disney BSDF with respect to the material
// parameters, for the adjoint (path-replay backpropagation) pass.
//
// Forward-mode: every quantity that depends on the parameters carries its
// value and its partial derivatives with respect to a chunk of NC of the 11
// differentiable parameters of a material (the raw values of
// GLSLPT::Material, src/core/Material.h:47-119):
//   0-2 baseColor r, g, b   3 metallic   4 roughness   5 subsurface
//   6 specularTint   7 sheen   8 sheenTint   9 clearcoat   10 clearcoatGloss
// GetMaterial's remapping (roughness >= 0.001, clearcoatRoughness =
// mix(0.1, 0.001, clearcoatGloss), ax / ay from roughness and anisotropy,
// pathtrace.glsl:25-115) is differentiated too.  The view, light and half
// vectors and eta do not depend on the parameters and stay plain floats.
//
// DisneyEvalD follows DisneyEval (pt_device.cuh, disney.glsl:244-351) lobe for
// lobe, operation for operation; its value part equals DisneyEval's f up to
// the rounding of the reordered products.
#pragma once

#include "pt_device.cuh"

namespace ptgb {
namespace grad {

constexpr int kParams = 11;  // differentiable parameters per material

template <int NC> struct D {
    float v;
    float d[NC];
};

template <int NC> __device__ __forceinline__ D<NC> dconst(float v) {
    D<NC> r;
    r.v = v;
#pragma unroll
    for (int i = 0; i < NC; ++i) r.d[i] = 0.0f;
    return r;
}
// parameter `param` of the material; seeds a partial if it is in this chunk
template <int NC> __device__ __forceinline__ D<NC> dparam(float v, int param, int chunk) {
    D<NC> r = dconst<NC>(v);
    const int k = param - chunk * NC;
    if (k >= 0 && k < NC) r.d[k] = 1.0f;
    return r;
}

template <int NC> __device__ __forceinline__ D<NC> operator+(const D<NC>& a, const D<NC>& b) {
    D<NC> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < NC; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <int NC> __device__ __forceinline__ D<NC> operator-(const D<NC>& a, const D<NC>& b) {
    D<NC> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < NC; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <int NC> __device__ __forceinline__ D<NC> operator-(const D<NC>& a) {
    D<NC> r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < NC; ++i) r.d[i] = -a.d[i];
    return r;
}
template <int NC> __device__ __forceinline__ D<NC> operator*(const D<NC>& a, const D<NC>& b) {
    D<NC> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < NC; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
template <int NC> __device__ __forceinline__ D<NC> operator/(const D<NC>& a, const D<NC>& b) {
    D<NC> r;
    r.v = a.v / b.v;
    const float inv = 1.0f / b.v;
#pragma unroll
    for (int i = 0; i < NC; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
    return r;
}
template <int NC> __device__ __forceinline__ D<NC> operator+(const D<NC>& a, float b) {
    D<NC> r = a;
    r.v = a.v + b;
    return r;
}
template <int NC> __device__ __forceinline__ D<NC> operator+(float a, const D<NC>& b) { return b + a; }
template <int NC> __device__ __forceinline__ D<NC> operator-(const D<NC>& a, float b) {
    D<NC> r = a;
    r.v = a.v - b;
    return r;
}
template <int NC> __device__ __forceinline__ D<NC> operator-(float a, const D<NC>& b) {
    D<NC> r;
    r.v = a - b.v;
#pragma unroll
    for (int i = 0; i < NC; ++i) r.d[i] = -b.d[i];
    return r;
}
template <int NC> __device__ __forceinline__ D<NC> operator*(const D<NC>& a, float b) {
    D<NC> r;
    r.v = a.v * b;
#pragma unroll
    for (int i = 0; i < NC; ++i) r.d[i] = a.d[i] * b;
    return r;
}
template <int NC> __device__ __forceinline__ D<NC> operator*(float a, const D<NC>& b) { return b * a; }
template <int NC> __device__ __forceinline__ D<NC> operator/(const D<NC>& a, float b) {
    D<NC> r;
    r.v = a.v / b;
    const float inv = 1.0f / b;
#pragma unroll
    for (int i = 0; i < NC; ++i) r.d[i] = a.d[i] * inv;
    return r;
}
template <int NC> __device__ __forceinline__ D<NC> operator/(float a, const D<NC>& b) {
    D<NC> r;
    r.v = a / b.v;
    const float s = -r.v / b.v;
#pragma unroll
    for (int i = 0; i < NC; ++i) r.d[i] = s * b.d[i];
    return r;
}
template <int NC> __device__ __forceinline__ D<NC> dsqrt(const D<NC>& a) {
    D<NC> r;
    r.v = sqrtf(a.v);
    const float s = r.v > 0.0f ? 0.5f / r.v : 0.0f;
#pragma unroll
    for (int i = 0; i < NC; ++i) r.d[i] = s * a.d[i];
    return r;
}
template <int NC> __device__ __forceinline__ D<NC> dlog(const D<NC>& a) {
    D<NC> r;
    r.v = logf(a.v);
    const float s = 1.0f / a.v;
#pragma unroll
    for (int i = 0; i < NC; ++i) r.d[i] = s * a.d[i];
    return r;
}
// max / min pick the larger / smaller operand with its derivatives
template <int NC> __device__ __forceinline__ D<NC> dmax(float a, const D<NC>& b) {
    return b.v >= a ? b : dconst<NC>(a);
}
template <int NC> __device__ __forceinline__ D<NC> dmix(float a, float b, const D<NC>& t) {
    return a * (1.0f - t) + b * t;
}
template <int NC> __device__ __forceinline__ D<NC> dmix(float a, const D<NC>& b, float t) {
    return a * (1.0f - t) + b * t;
}
template <int NC> __device__ __forceinline__ D<NC> dmix(const D<NC>& a, float b, float t) {
    return a * (1.0f - t) + b * t;
}
template <int NC> __device__ __forceinline__ D<NC> dmix(const D<NC>& a, const D<NC>& b, const D<NC>& t) {
    return a * (1.0f - t) + b * t;
}

template <int NC> struct DV3 {
    D<NC> x, y, z;
};
template <int NC> __device__ __forceinline__ DV3<NC> dv3(const D<NC>& a) { return {a, a, a}; }
template <int NC> __device__ __forceinline__ DV3<NC> dv3c(V3 a) {
    return {dconst<NC>(a.x), dconst<NC>(a.y), dconst<NC>(a.z)};
}
template <int NC> __device__ __forceinline__ DV3<NC> operator+(const DV3<NC>& a, const DV3<NC>& b) {
    return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <int NC> __device__ __forceinline__ DV3<NC> operator*(const DV3<NC>& a, const D<NC>& s) {
    return {a.x * s, a.y * s, a.z * s};
}
template <int NC> __device__ __forceinline__ DV3<NC> operator*(const D<NC>& s, const DV3<NC>& a) { return a * s; }
template <int NC> __device__ __forceinline__ DV3<NC> operator*(const DV3<NC>& a, float s) {
    return {a.x * s, a.y * s, a.z * s};
}
template <int NC> __device__ __forceinline__ DV3<NC> operator*(float s, const DV3<NC>& a) { return a * s; }
template <int NC> __device__ __forceinline__ DV3<NC> operator*(const DV3<NC>& a, V3 b) {
    return {a.x * b.x, a.y * b.y, a.z * b.z};
}
template <int NC> __device__ __forceinline__ DV3<NC> operator/(const DV3<NC>& a, const D<NC>& s) {
    return {a.x / s, a.y / s, a.z / s};
}
template <int NC> __device__ __forceinline__ D<NC> Lum(const DV3<NC>& c) {  // globals.glsl:173-176
    return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z;
}
// mix(a, b, t) per channel with scalar t
template <int NC> __device__ __forceinline__ DV3<NC> dmix3(const DV3<NC>& a, V3 b, float t) {
    return {dmix(a.x, b.x, t), dmix(a.y, b.y, t), dmix(a.z, b.z, t)};
}
template <int NC> __device__ __forceinline__ DV3<NC> dmix3(V3 a, const DV3<NC>& b, const D<NC>& t) {
    return {dconst<NC>(a.x) * (1.0f - t) + b.x * t, dconst<NC>(a.y) * (1.0f - t) + b.y * t,
            dconst<NC>(a.z) * (1.0f - t) + b.z * t};
}

// The material with derivatives (the parameters that DisneyEval reads).
template <int NC> struct MatD {
    DV3<NC> baseColor;
    D<NC> metallic, roughness, subsurface, specularTint, sheen, sheenTint, clearcoat, clearcoatRoughness, ax, ay;
    float specTrans, ior;
};

// LoadMaterial + GetMaterial's remapping (pathtrace.glsl:25-115) for the
// derivative chunk `chunk`; prevRough / mollification as GetMaterial.
template <int NC>
__device__ __forceinline__ MatD<NC> LoadMaterialD(const float4* __restrict__ mats, int id, int chunk, bool mollify,
                                                   float mollified) {
    const float4* p = mats + 8 * id;
    const float4 p1 = __ldg(p + 0), p3 = __ldg(p + 2), p4 = __ldg(p + 3), p5 = __ldg(p + 4);
    MatD<NC> m;
    m.baseColor = {dparam<NC>(p1.x, 0, chunk), dparam<NC>(p1.y, 1, chunk), dparam<NC>(p1.z, 2, chunk)};
    m.metallic = dparam<NC>(p3.x, 3, chunk);
    m.roughness = dmax(0.001f, dparam<NC>(p3.y, 4, chunk));
    m.subsurface = dparam<NC>(p3.z, 5, chunk);
    m.specularTint = dparam<NC>(p3.w, 6, chunk);
    m.sheen = dparam<NC>(p4.x, 7, chunk);
    m.sheenTint = dparam<NC>(p4.y, 8, chunk);
    m.clearcoat = dparam<NC>(p4.z, 9, chunk);
    m.clearcoatRoughness = dmix(0.1f, 0.001f, dparam<NC>(p4.w, 10, chunk));
    m.specTrans = p5.x;
    m.ior = p5.y;
    if (mollify) m.roughness = dmax(mollified, m.roughness);  // the mollified value is held fixed
    const float aspect = sqrtf(1.0f - p1.w * 0.9f);
    m.ax = dmax(0.001f, m.roughness / aspect);
    m.ay = dmax(0.001f, m.roughness * aspect);
    return m;
}

// sampling.glsl:25-32 in the cancellation-free form of pt_device.cuh's GTR1
template <int NC> __device__ __forceinline__ D<NC> GTR1D(V3 H, const D<NC>& a) {
    if (a.v >= 1.0f) return dconst<NC>(PT_INV_PI);
    const D<NC> a2 = a * a;
    const float s = H.x * H.x + H.y * H.y;
    const float z2 = H.z * H.z;
    const D<NC> t = (s + a2 * z2) * (1.0f / (s + z2));
    return (a2 - 1.0f) / (PT_PI * dlog(a2) * t);
}
template <int NC>
__device__ __forceinline__ D<NC> GTR2AnisoD(float NDotH, float HDotX, float HDotY, const D<NC>& ax,
                                            const D<NC>& ay) {  // sampling.glsl:90-96
    const D<NC> a = HDotX / ax;
    const D<NC> b = HDotY / ay;
    const D<NC> c = a * a + b * b + NDotH * NDotH;
    return 1.0f / (PT_PI * ax * ay * c * c);
}
template <int NC>
__device__ __forceinline__ D<NC> SmithGAnisoD(float NDotV, float VDotX, float VDotY, const D<NC>& ax,
                                              const D<NC>& ay) {  // sampling.glsl:116-122
    const D<NC> a = VDotX * ax;
    const D<NC> b = VDotY * ay;
    return (2.0f * NDotV) / (NDotV + dsqrt(a * a + b * b + NDotV * NDotV));
}

template <int NC> struct LobesD {
    D<NC> dielectricWt, metalWt, glassWt, diffPr, dielectricPr, metalPr, glassPr, clearCtPr;
    float F0;
    DV3<NC> Csheen, Cspec0;
};
template <int NC> __device__ __forceinline__ LobesD<NC> LobeWeightsD(const MatD<NC>& mat, float eta, V3 V) {
    LobesD<NC> lb;
    const D<NC> lum = Lum(mat.baseColor);
    const DV3<NC> ctint = lum.v > 0.0f ? mat.baseColor / lum : dv3(dconst<NC>(1.0f));
    lb.F0 = (1.0f - eta) / (1.0f + eta);
    lb.F0 *= lb.F0;
    lb.Cspec0 = dmix3(v3(1.0f), ctint, mat.specularTint) * lb.F0;
    lb.Csheen = dmix3(v3(1.0f), ctint, mat.sheenTint);
    lb.dielectricWt = (1.0f - mat.metallic) * (1.0f - mat.specTrans);
    lb.metalWt = mat.metallic;
    lb.glassWt = (1.0f - mat.metallic) * mat.specTrans;
    const float schlickWt = SchlickWeight(V.z);
    lb.diffPr = lb.dielectricWt * Lum(mat.baseColor);
    lb.dielectricPr = lb.dielectricWt * Lum(dmix3(lb.Cspec0, v3(1.0f), schlickWt));
    lb.metalPr = lb.metalWt * Lum(dmix3(mat.baseColor, v3(1.0f), schlickWt));
    lb.glassPr = lb.glassWt;
    lb.clearCtPr = 0.25f * mat.clearcoat;
    return lb;
}

// disney.glsl:61-88
template <int NC>
__device__ __forceinline__ DV3<NC> EvalDisneyDiffuseD(const MatD<NC>& mat, const DV3<NC>& Csheen, V3 V, V3 L,
                                                      V3 H) {
    const float LDotH = dot(L, H);
    const D<NC> Rr = (2.0f * LDotH * LDotH) * mat.roughness;
    const float FL = SchlickWeight(L.z);
    const float FV = SchlickWeight(V.z);
    const D<NC> Fretro = Rr * (FL + FV + FL * FV * (Rr - 1.0f));
    const float Fd = (1.0f - 0.5f * FL) * (1.0f - 0.5f * FV);
    const D<NC> Fss90 = 0.5f * Rr;
    const D<NC> Fss = dmix(1.0f, Fss90, FL) * dmix(1.0f, Fss90, FV);
    const D<NC> ss = 1.25f * (Fss * (1.0f / (L.z + V.z) - 0.5f) + 0.5f);
    const float FH = SchlickWeight(LDotH);
    const DV3<NC> Fsheen = Csheen * (FH * mat.sheen);
    const D<NC> mixv = dmix(Fd + Fretro, ss, mat.subsurface);
    return mat.baseColor * (PT_INV_PI * mixv) + Fsheen;
}
// disney.glsl:90-102 (value only; the pdf is not differentiated)
template <int NC>
__device__ __forceinline__ D<NC> MicrofacetReflectionTermD(const MatD<NC>& mat, V3 V, V3 L, V3 H) {
    const D<NC> Dd = GTR2AnisoD(H.z, H.x, H.y, mat.ax, mat.ay);
    const D<NC> G1 = SmithGAnisoD(fabsf(V.z), V.x, V.y, mat.ax, mat.ay);
    const D<NC> G2 = G1 * SmithGAnisoD(fabsf(L.z), L.x, L.y, mat.ax, mat.ay);
    return Dd * G2 / (4.0f * L.z * V.z);
}
// disney.glsl:104-123
template <int NC>
__device__ __forceinline__ DV3<NC> EvalMicrofacetRefractionD(const MatD<NC>& mat, float eta, V3 V, V3 L, V3 H,
                                                             float F) {
    const float LDotH = dot(L, H);
    const float VDotH = dot(V, H);
    const D<NC> Dd = GTR2AnisoD(H.z, H.x, H.y, mat.ax, mat.ay);
    const D<NC> G1 = SmithGAnisoD(fabsf(V.z), V.x, V.y, mat.ax, mat.ay);
    const D<NC> G2 = G1 * SmithGAnisoD(fabsf(L.z), L.x, L.y, mat.ax, mat.ay);
    float denom = LDotH + VDotH * eta;
    denom *= denom;
    const float eta2 = eta * eta;
    const float jacobian = fabsf(LDotH) / denom;
    const DV3<NC> sq = {dsqrt(mat.baseColor.x), dsqrt(mat.baseColor.y), dsqrt(mat.baseColor.z)};
    const D<NC> s = Dd * G2 * (fabsf(VDotH) * jacobian * eta2 / fabsf(L.z * V.z) * (1.0f - F));
    return sq * s;
}
// disney.glsl:125-140
template <int NC> __device__ __forceinline__ D<NC> EvalClearcoatD(const MatD<NC>& mat, V3 V, V3 L, V3 H) {
    const float VDotH = dot(V, H);
    const float F = mixf(0.04f, 1.0f, SchlickWeight(VDotH));
    const D<NC> Dd = GTR1D(H, mat.clearcoatRoughness);
    const float G = SmithG(L.z, 0.25f) * SmithG(V.z, 0.25f);
    return Dd * (F * G);
}

// DisneyEval's f * |L.z| (disney.glsl:244-351) with derivatives.
template <int NC>
__device__ __forceinline__ DV3<NC> DisneyEvalD(const MatD<NC>& mat, float eta, V3 V, V3 N, V3 L) {
    DV3<NC> f = dv3(dconst<NC>(0.0f));
    V3 T, B;
    Onb(N, T, B);
    V = ToLocal(T, B, N, V);
    L = ToLocal(T, B, N, L);
    V3 H;
    if (L.z > 0.0f) H = normalize(L + V);
    else H = normalize(L + V * eta);
    if (H.z < 0.0f) H = -H;
    const LobesD<NC> lb = LobeWeightsD(mat, eta, V);
    const bool refl = L.z * V.z > 0.0f;
    const float VDotH = fabsf(dot(V, H));
    const float absLz = fabsf(L.z);
    // lobe selection uses the normalised probabilities, whose signs are
    // those of the unnormalised ones (the total is positive)
    if (lb.diffPr.v > 0.0f && refl && L.z > 0.0f)
        f = f + EvalDisneyDiffuseD(mat, lb.Csheen, V, L, H) * lb.dielectricWt;
    if (lb.dielectricPr.v > 0.0f && refl && L.z > 0.0f) {
        const float Fr = (DielectricFresnel(VDotH, 1.0f / mat.ior) - lb.F0) / (1.0f - lb.F0);
        const DV3<NC> Fc = {dmix(lb.Cspec0.x, 1.0f, Fr), dmix(lb.Cspec0.y, 1.0f, Fr), dmix(lb.Cspec0.z, 1.0f, Fr)};
        f = f + Fc * (MicrofacetReflectionTermD(mat, V, L, H) * lb.dielectricWt);
    }
    if (lb.metalPr.v > 0.0f && refl && L.z > 0.0f) {
        const DV3<NC> Fc = dmix3(mat.baseColor, v3(1.0f), SchlickWeight(VDotH));
        f = f + Fc * (MicrofacetReflectionTermD(mat, V, L, H) * lb.metalWt);
    }
    if (lb.glassPr.v > 0.0f) {
        const float F = DielectricFresnel(VDotH, eta);
        if (refl) {
            if (L.z > 0.0f) f = f + dv3(MicrofacetReflectionTermD(mat, V, L, H) * (F * 1.0f)) * lb.glassWt;
        } else if (L.z < 0.0f) {
            f = f + EvalMicrofacetRefractionD(mat, eta, V, L, H, F) * lb.glassWt;
        }
    }
    if (lb.clearCtPr.v > 0.0f && refl && L.z > 0.0f)
        f = f + dv3(EvalClearcoatD(mat, V, L, H) * (0.25f * mat.clearcoat));
    return f * absLz;
}

}  // namespace grad
}  // namespace ptgb
