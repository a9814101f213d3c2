// pt_kernels.cu - the path-tracing kernels (sm_103a).
//
//   render_kernel        tile.glsl:main + PathTrace (common/pathtrace.glsl:285)
//                        as one megakernel: one thread per pixel, looping over
//                        the sample passes of the launch
//   trace_closest_kernel test hook: ClosestHit's triangle part on a ray set
//   trace_shadow_kernel  test hook: AnyHit's triangle part on a ray set
//   tonemap_kernel       tonemap.glsl:main + the RGBA8 read-back format
//
// Traversal runs over the 8-wide quantised BVH of bvh8.h.  A node fetch is
// five 128-bit loads; the eight child boxes are slab-tested against the ray
// and the hits become a 32-bit mask: bits 24-31 internal children in octant
// order, bits 0-23 leaf primitives.  Node groups (child base, remaining hit
// bits | imask) go to a per-thread stack; leaf triangles are tested at once.
// The triangle test repeats the reference's arithmetic operation for
// operation, without fused multiply-adds (closest_hit.glsl:128-143), so hit
// decisions and distances equal the oracle's bit for bit.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pt_cuda.h"
#include "pt_device.cuh"
#include "pt_params.h"

namespace ptgb {

// ------------------------------------------------------------ traversal
struct TRay {
    V3 o, d;
    float ix, iy, iz;
    uint32_t oct_inv, oct_inv4;
    bool nx, ny, nz;
};

__device__ __forceinline__ float safe_rcp(float d) {
    return 1.0f / (fabsf(d) > 1e-20f ? d : copysignf(1e-20f, d));
}

__device__ __forceinline__ TRay prep_ray(V3 o, V3 d) {
    TRay r;
    r.o = o;
    r.d = d;
    r.ix = safe_rcp(d.x);
    r.iy = safe_rcp(d.y);
    r.iz = safe_rcp(d.z);
    r.nx = r.ix < 0.0f;
    r.ny = r.iy < 0.0f;
    r.nz = r.iz < 0.0f;
    uint32_t oct = (r.nx ? 1u : 0u) | (r.ny ? 2u : 0u) | (r.nz ? 4u : 0u);
    r.oct_inv = 7u - oct;
    r.oct_inv4 = r.oct_inv * 0x01010101u;
    return r;
}

__device__ __forceinline__ float qbyte(uint32_t w, int j) { return __uint2float_rn((w >> (8 * j)) & 0xffu); }

// Slab test of the eight children of wide node `idx`; returns the hit mask.
__device__ __forceinline__ uint32_t intersect_node(const uint4* __restrict__ nodes, int idx, const TRay& r,
                                                   float tmax, uint32_t& child_base, uint32_t& prim_base,
                                                   uint32_t& imask) {
    const uint4* n = nodes + (size_t)idx * 5;
    const uint4 w0 = __ldg(n), w1 = __ldg(n + 1), w2 = __ldg(n + 2), w3 = __ldg(n + 3), w4 = __ldg(n + 4);
    const float sx = __uint_as_float((w0.w & 0xffu) << 23);
    const float sy = __uint_as_float(((w0.w >> 8) & 0xffu) << 23);
    const float sz = __uint_as_float(((w0.w >> 16) & 0xffu) << 23);
    imask = w0.w >> 24;
    child_base = w1.x;
    prim_base = w1.y;
    const float adjx = sx * r.ix, adjy = sy * r.iy, adjz = sz * r.iz;
    const float orgx = (__uint_as_float(w0.x) - r.o.x) * r.ix;
    const float orgy = (__uint_as_float(w0.y) - r.o.y) * r.iy;
    const float orgz = (__uint_as_float(w0.z) - r.o.z) * r.iz;
    uint32_t hits = 0;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const uint32_t meta4 = half ? w1.w : w1.z;
        const uint32_t is_inner4 = (meta4 & (meta4 << 1)) & 0x10101010u;
        const uint32_t inner_mask4 = (is_inner4 >> 4) * 0xffu;
        const uint32_t bit_index4 = (meta4 ^ (r.oct_inv4 & inner_mask4)) & 0x1f1f1f1fu;
        const uint32_t child_bits4 = (meta4 >> 5) & 0x07070707u;
        const uint32_t qlox = half ? w2.y : w2.x, qloy = half ? w2.w : w2.z, qloz = half ? w3.y : w3.x;
        const uint32_t qhix = half ? w3.w : w3.z, qhiy = half ? w4.y : w4.x, qhiz = half ? w4.w : w4.z;
        const uint32_t nxw = r.nx ? qhix : qlox, fxw = r.nx ? qlox : qhix;
        const uint32_t nyw = r.ny ? qhiy : qloy, fyw = r.ny ? qloy : qhiy;
        const uint32_t nzw = r.nz ? qhiz : qloz, fzw = r.nz ? qloz : qhiz;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float tnx = fmaf(qbyte(nxw, j), adjx, orgx), tfx = fmaf(qbyte(fxw, j), adjx, orgx);
            const float tny = fmaf(qbyte(nyw, j), adjy, orgy), tfy = fmaf(qbyte(fyw, j), adjy, orgy);
            const float tnz = fmaf(qbyte(nzw, j), adjz, orgz), tfz = fmaf(qbyte(fzw, j), adjz, orgz);
            const float t0 = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, 0.0f));
            const float t1 = fminf(fminf(tfx, tfy), fminf(tfz, tmax));
            if (t0 <= t1) {
                const uint32_t cb = (child_bits4 >> (8 * j)) & 0xffu;
                const uint32_t bi = (bit_index4 >> (8 * j)) & 0xffu;
                hits |= cb << bi;
            }
        }
    }
    return hits;
}

// Triangle test of closest_hit.glsl:128-143 with the reference's operation
// order and no contraction: returns the barycentrics and distance.
__device__ __forceinline__ bool tri_test(const TRay& r, const float4* __restrict__ tris, int t, float& u, float& v,
                                         float& tt, float& w, int& prim) {
    const float4 a = __ldg(tris + 3 * (size_t)t), b = __ldg(tris + 3 * (size_t)t + 1),
                 c = __ldg(tris + 3 * (size_t)t + 2);
    prim = __float_as_int(a.w);
    // e0 = b, e1 = c (precomputed v1-v0, v2-v0)
    const float pvx = __fsub_rn(__fmul_rn(r.d.y, c.z), __fmul_rn(r.d.z, c.y));
    const float pvy = __fsub_rn(__fmul_rn(r.d.z, c.x), __fmul_rn(r.d.x, c.z));
    const float pvz = __fsub_rn(__fmul_rn(r.d.x, c.y), __fmul_rn(r.d.y, c.x));
    const float det = __fadd_rn(__fadd_rn(__fmul_rn(b.x, pvx), __fmul_rn(b.y, pvy)), __fmul_rn(b.z, pvz));
    const float tvx = __fsub_rn(r.o.x, a.x), tvy = __fsub_rn(r.o.y, a.y), tvz = __fsub_rn(r.o.z, a.z);
    const float qvx = __fsub_rn(__fmul_rn(tvy, b.z), __fmul_rn(tvz, b.y));
    const float qvy = __fsub_rn(__fmul_rn(tvz, b.x), __fmul_rn(tvx, b.z));
    const float qvz = __fsub_rn(__fmul_rn(tvx, b.y), __fmul_rn(tvy, b.x));
    const float U = __fadd_rn(__fadd_rn(__fmul_rn(tvx, pvx), __fmul_rn(tvy, pvy)), __fmul_rn(tvz, pvz));
    const float Vv = __fadd_rn(__fadd_rn(__fmul_rn(r.d.x, qvx), __fmul_rn(r.d.y, qvy)), __fmul_rn(r.d.z, qvz));
    const float T = __fadd_rn(__fadd_rn(__fmul_rn(c.x, qvx), __fmul_rn(c.y, qvy)), __fmul_rn(c.z, qvz));
    u = __fdiv_rn(U, det);
    v = __fdiv_rn(Vv, det);
    tt = __fdiv_rn(T, det);
    w = __fsub_rn(__fsub_rn(1.0f, u), v);
    return u >= 0.0f && v >= 0.0f && tt >= 0.0f && w >= 0.0f;
}

struct TriHit {
    float t, u, v, w;
    int prim, inst, mat;
};

// GLSL mat4 * vec4 with the sum in column order, no contraction
// (closest_hit.glsl:163-164 with a precomputed inverse).
__device__ __forceinline__ V3 xform_point(const float4* __restrict__ xf, int inst, V3 p, float w) {
    const float4 c0 = __ldg(xf + 10 * inst), c1 = __ldg(xf + 10 * inst + 1), c2 = __ldg(xf + 10 * inst + 2),
                 c3 = __ldg(xf + 10 * inst + 3);
    V3 r;
    r.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(c0.x, p.x), __fmul_rn(c1.x, p.y)), __fmul_rn(c2.x, p.z)), __fmul_rn(c3.x, w));
    r.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(c0.y, p.x), __fmul_rn(c1.y, p.y)), __fmul_rn(c2.y, p.z)), __fmul_rn(c3.y, w));
    r.z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(c0.z, p.x), __fmul_rn(c1.z, p.y)), __fmul_rn(c2.z, p.z)), __fmul_rn(c3.z, w));
    return r;
}

__device__ __forceinline__ void flag_status(int* status, int code) { atomicCAS(status, PT_OK, code); }

// One level of closest-hit traversal from wide node `root`.  For the TLAS
// (IS_TLAS) the leaf primitives are instances, each traversed as a nested
// BLAS level above the current stack top.
template <bool IS_TLAS>
__device__ void traverse_closest(const Params& P, int root, const TRay& r, TriHit& h, uint2* stack, int sp,
                                 int inst, int mat) {
    uint32_t cb, pb, im;
    uint32_t hm = intersect_node(P.nodes, root, r, h.t, cb, pb, im);
    uint2 ng = make_uint2(cb, (hm & 0xff000000u) | im);
    uint32_t tbase = pb, tbits = hm & 0x00ffffffu;
    const int sp_base = sp;
    for (;;) {
        while (tbits) {
            const int b = __ffs(tbits) - 1;
            tbits &= tbits - 1;
            if (IS_TLAS) {
                const int4 ir = __ldg(P.insts + tbase + b);
                if (ir.w) {
                    traverse_closest<false>(P, ir.x, r, h, stack, sp, ir.y, ir.z);
                } else {
                    const TRay ro = prep_ray(xform_point(P.xf, ir.y, r.o, 1.0f), xform_point(P.xf, ir.y, r.d, 0.0f));
                    traverse_closest<false>(P, ir.x, ro, h, stack, sp, ir.y, ir.z);
                }
            } else {
                float u, v, t, w;
                int prim;
                if (tri_test(r, P.tris, tbase + b, u, v, t, w, prim) && t < h.t) {
                    h.t = t; h.u = u; h.v = v; h.w = w;
                    h.prim = prim; h.inst = inst; h.mat = mat;
                }
            }
        }
        if (ng.y > 0x00ffffffu) {
            const uint32_t bit = 31u - __clz(ng.y);
            const uint32_t slot = (bit - 24u) ^ r.oct_inv;
            const uint32_t rel = __popc(ng.y & ~(0xffffffffu << slot));
            const int child = (int)(ng.x + rel);
            ng.y &= ~(1u << bit);
            if (ng.y > 0x00ffffffu) {
                if (sp < kStackSize) stack[sp++] = ng;
                else flag_status(P.status, PT_ERR_STACK_OVERFLOW);
            }
            hm = intersect_node(P.nodes, child, r, h.t, cb, pb, im);
            ng = make_uint2(cb, (hm & 0xff000000u) | im);
            tbase = pb;
            tbits = hm & 0x00ffffffu;
        } else {
            if (sp == sp_base) break;
            ng = stack[--sp];
        }
    }
}

// Any-hit traversal (anyhit.glsl:83-213): true as soon as a triangle with
// 0 <= t < maxDist passes the (optional) alpha test.
template <bool IS_TLAS>
__device__ bool traverse_any(const Params& P, int root, const TRay& r, float maxDist, uint2* stack, int sp, int mat,
                             bool alpha, Rng& rng) {
    uint32_t cb, pb, im;
    uint32_t hm = intersect_node(P.nodes, root, r, maxDist, cb, pb, im);
    uint2 ng = make_uint2(cb, (hm & 0xff000000u) | im);
    uint32_t tbase = pb, tbits = hm & 0x00ffffffu;
    const int sp_base = sp;
    for (;;) {
        while (tbits) {
            const int b = __ffs(tbits) - 1;
            tbits &= tbits - 1;
            if (IS_TLAS) {
                const int4 ir = __ldg(P.insts + tbase + b);
                bool hit;
                if (ir.w) hit = traverse_any<false>(P, ir.x, r, maxDist, stack, sp, ir.z, alpha, rng);
                else {
                    const TRay ro = prep_ray(xform_point(P.xf, ir.y, r.o, 1.0f), xform_point(P.xf, ir.y, r.d, 0.0f));
                    hit = traverse_any<false>(P, ir.x, ro, maxDist, stack, sp, ir.z, alpha, rng);
                }
                if (hit) return true;
            } else {
                float u, v, t, w;
                int prim;
                if (tri_test(r, P.tris, tbase + b, u, v, t, w, prim) && t < maxDist) {
                    if (!alpha) return true;
                    // anyhit.glsl:118-141 with no texture bound (alpha = 1)
                    const float4 ap = __ldg(P.mats + 8 * mat + 7);
                    const float opacity = ap.x;
                    const int alphaMode = (int)ap.y;
                    bool skip = alphaMode == ALPHA_MODE_MASK && opacity < ap.z;
                    if (!skip && alphaMode == ALPHA_MODE_BLEND) skip = rng.next() > opacity;
                    if (!skip) return true;
                }
            }
        }
        if (ng.y > 0x00ffffffu) {
            const uint32_t bit = 31u - __clz(ng.y);
            const uint32_t slot = (bit - 24u) ^ r.oct_inv;
            const uint32_t rel = __popc(ng.y & ~(0xffffffffu << slot));
            const int child = (int)(ng.x + rel);
            ng.y &= ~(1u << bit);
            if (ng.y > 0x00ffffffu) {
                if (sp < kStackSize) stack[sp++] = ng;
                else flag_status(P.status, PT_ERR_STACK_OVERFLOW);
            }
            hm = intersect_node(P.nodes, child, r, maxDist, cb, pb, im);
            ng = make_uint2(cb, (hm & 0xff000000u) | im);
            tbase = pb;
            tbits = hm & 0x00ffffffu;
        } else {
            if (sp == sp_base) break;
            ng = stack[--sp];
        }
    }
    return false;
}

// ------------------------------------------------------------- shading
struct State {
    int depth;
    float eta, hitDist;
    V3 fhp, normal, ffnormal;
    bool isEmitter;
    int matID;
    Material mat;
    Medium medium;
};

struct Counters {
    uint32_t closest, shadow;
};

// closest_hit.glsl:25-266 (texture coordinates and tangents are only needed
// by texture maps, which this build does not take)
__device__ bool ClosestHit(const Params& P, const Ray& r, State& state, LightSample& ls, uint2* stack, Counters& cnt,
                           bool count_as_shadow) {
    if (count_as_shadow) cnt.shadow++;
    else cnt.closest++;
    float t = PT_INF;
    if ((P.flags & F_LIGHTS) && !((P.flags & F_HIDE_EMITTERS) && !(state.depth > 0))) {
        for (int i = 0; i < P.num_lights; i++) {
            const Light L = LoadLight(P.lights, i);
            const int type = (int)L.type;
            if (type == QUAD_LIGHT) {
                V3 normal = normalize(cross(L.u, L.v));
                if (dot(normal, r.direction) > 0.0f) continue;
                float pw = dot(normal, L.position);
                V3 u = L.u * (1.0f / dot(L.u, L.u));
                V3 v = L.v * (1.0f / dot(L.v, L.v));
                float d = RectIntersect(L.position, u, v, normal, pw, r);
                if (d < 0.0f) d = PT_INF;
                if (d < t) {
                    t = d;
                    float cosTheta = dot(-r.direction, normal);
                    ls.pdf = (t * t) / (L.area * cosTheta);
                    ls.emission = L.emission;
                    state.isEmitter = true;
                }
            }
            if (type == SPHERE_LIGHT) {
                float d = SphereIntersect(L.radius, L.position, r);
                if (d < 0.0f) d = PT_INF;
                if (d < t) {
                    t = d;
                    V3 hitPt = r.origin + t * r.direction;
                    float cosTheta = dot(-r.direction, normalize(hitPt - L.position));
                    ls.pdf = (t * t) / (L.area * cosTheta * 0.5f);
                    ls.emission = L.emission;
                    state.isEmitter = true;
                }
            }
        }
    }
    TriHit h;
    h.t = t;
    h.prim = -1;
    traverse_closest<true>(P, P.tlas_root, prep_ray(r.origin, r.direction), h, stack, 0, -1, 0);
    if (h.prim >= 0) t = h.t;
    if (t == PT_INF) return false;
    state.hitDist = t;
    state.fhp = r.origin + r.direction * t;
    if (h.prim >= 0) {
        state.isEmitter = false;
        state.matID = h.mat;
        const int i0 = __ldg(P.vidx + 3 * h.prim), i1 = __ldg(P.vidx + 3 * h.prim + 1),
                  i2 = __ldg(P.vidx + 3 * h.prim + 2);
        const V3 n0 = v3(__ldg(P.norms + i0)), n1 = v3(__ldg(P.norms + i1)), n2 = v3(__ldg(P.norms + i2));
        V3 normal = normalize(n0 * h.w + n1 * h.u + n2 * h.v);  // bary = uvt.wxy
        if (h.inst >= 0) {
            const float4* x = P.xf + 10 * h.inst + 7;
            const float4 c0 = __ldg(x), c1 = __ldg(x + 1), c2 = __ldg(x + 2);
            normal = v3(c0.x * normal.x + c1.x * normal.y + c2.x * normal.z,
                        c0.y * normal.x + c1.y * normal.y + c2.y * normal.z,
                        c0.z * normal.x + c1.z * normal.y + c2.z * normal.z);
        }
        state.normal = normalize(normal);
        state.ffnormal = dot(state.normal, r.direction) <= 0.0f ? state.normal : -state.normal;
    }
    return true;
}

// anyhit.glsl:25-216
__device__ bool AnyHit(const Params& P, const Ray& r, float maxDist, Rng& rng, uint2* stack, Counters& cnt) {
    cnt.shadow++;
    if (P.flags & F_LIGHTS) {
        for (int i = 0; i < P.num_lights; i++) {
            const Light L = LoadLight(P.lights, i);
            const int type = (int)L.type;
            if (type == QUAD_LIGHT) {
                V3 normal = normalize(cross(L.u, L.v));
                float pw = dot(normal, L.position);
                V3 u = L.u * (1.0f / dot(L.u, L.u));
                V3 v = L.v * (1.0f / dot(L.v, L.v));
                float d = RectIntersect(L.position, u, v, normal, pw, r);
                if (d > 0.0f && d < maxDist) return true;
            }
            if (type == SPHERE_LIGHT) {
                float d = SphereIntersect(L.radius, L.position, r);
                if (d > 0.0f && d < maxDist) return true;
            }
        }
    }
    const bool alpha = (P.flags & F_ALPHA_TEST) && !(P.flags & F_MEDIUM);
    return traverse_any<true>(P, P.tlas_root, prep_ray(r.origin, r.direction), maxDist, stack, 0, 0, alpha, rng);
}

// GetMaterial (pathtrace.glsl:25-115) without texture maps
__device__ __forceinline__ void GetMaterial(const Params& P, State& state, const Ray& r) {
    const float prevRoughness = state.mat.roughness;
    Material mat;
    LoadMaterial(P.mats, state.matID, mat);
    if ((P.flags & F_MOLLIFY) && state.depth > 0)
        mat.roughness = fmaxf(mixf(0.0f, prevRoughness, P.mollify_amt), mat.roughness);
    FinishMaterial(mat);
    state.mat = mat;
    state.eta = dot(r.direction, state.normal) < 0.0f ? (1.0f / mat.ior) : mat.ior;
}

__device__ __forceinline__ bool AlphaSkip(const Material& m, Rng& rng) {
    if (m.alphaMode == ALPHA_MODE_MASK && m.opacity < m.alphaCutoff) return true;
    if (m.alphaMode == ALPHA_MODE_BLEND) return rng.next() > m.opacity;
    return false;
}

// pathtrace.glsl:118-156 (OPT_MEDIUM && OPT_VOL_MIS); each segment is a
// shadow query
__device__ V3 EvalTransmittance(const Params& P, Ray r, Rng& rng, uint2* stack, Counters& cnt) {
    LightSample ls;
    State state;
    state.depth = 0;
    state.isEmitter = false;
    state.matID = 0;
    state.mat.roughness = 0.0f;
    state.normal = v3(0.0f);
    V3 transmittance = v3(1.0f);
    for (int depth = 0; depth < P.max_depth; depth++) {
        bool hit = ClosestHit(P, r, state, ls, stack, cnt, true);
        if (!hit || state.isEmitter) break;
        GetMaterial(P, state, r);
        bool alphatest = AlphaSkip(state.mat, rng);
        bool refractive = (1.0f - state.mat.metallic) * state.mat.specTrans > 0.0f;
        if (hit && !(alphatest || refractive)) return v3(0.0f);
        if (dot(r.direction, state.normal) > 0.0f && state.mat.medium.type != MEDIUM_NONE) {
            V3 color = state.mat.medium.type == MEDIUM_ABSORB ? v3(1.0f) - state.mat.medium.color : v3(1.0f);
            transmittance = transmittance * vexp(-color * state.mat.medium.density * state.hitDist);
        }
        r.origin = state.fhp + r.direction * PT_EPS;
    }
    return transmittance;
}

// envmap.glsl:28-55
__device__ __forceinline__ void BinarySearch(const Params& P, float value, float& u, float& v) {
    const int W = P.env_w, H = P.env_h;
    int lower = 0, upper = H - 1;
    while (lower < upper) {
        int mid = (lower + upper) >> 1;
        if (value < __ldg(P.cdf + (size_t)mid * W + (W - 1))) upper = mid;
        else lower = mid + 1;
    }
    const int y = min(max(lower, 0), H - 1);
    lower = 0;
    upper = W - 1;
    while (lower < upper) {
        int mid = (lower + upper) >> 1;
        if (value < __ldg(P.cdf + (size_t)y * W + mid)) upper = mid;
        else lower = mid + 1;
    }
    const int x = min(max(lower, 0), W - 1);
    u = (float)x / (float)W;
    v = (float)y / (float)H;
}

// texture(envMapTex, uv): bilinear, GL_REPEAT (Renderer.cpp:213-218)
__device__ __forceinline__ V3 SampleEnv(const Params& P, float u, float v) {
    const int W = P.env_w, H = P.env_h;
    float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    float fx = floorf(x), fy = floorf(y);
    float ax = x - fx, ay = y - fy;
    int ix = (int)fx, iy = (int)fy;
    int x0 = ix % W; x0 += x0 < 0 ? W : 0;
    int y0 = iy % H; y0 += y0 < 0 ? H : 0;
    int x1 = x0 + 1 == W ? 0 : x0 + 1;
    int y1 = y0 + 1 == H ? 0 : y0 + 1;
    const float4 a = __ldg(P.env + (size_t)y0 * W + x0), b = __ldg(P.env + (size_t)y0 * W + x1);
    const float4 c = __ldg(P.env + (size_t)y1 * W + x0), d = __ldg(P.env + (size_t)y1 * W + x1);
    V3 t0 = v3(a) * (1.0f - ax) + v3(b) * ax;
    V3 t1 = v3(c) * (1.0f - ax) + v3(d) * ax;
    return t0 * (1.0f - ay) + t1 * ay;
}

// envmap.glsl:57-66
__device__ __forceinline__ V3 EvalEnvMap(const Params& P, const Ray& r, float& pdfOut) {
    float theta = acosf(clampf(r.direction.y, -1.0f, 1.0f));
    float u = (PT_PI + atan2f(r.direction.z, r.direction.x)) * PT_INV_TWO_PI + P.env_rot;
    float v = theta * PT_INV_PI;
    V3 color = SampleEnv(P, u, v);
    float pdf = Luminance(color) / P.env_total;
    pdfOut = (pdf * (float)P.env_w * (float)P.env_h) / (PT_TWO_PI * PT_PI * sinf(theta));
    return color;
}

// envmap.glsl:68-83
__device__ __forceinline__ V3 SampleEnvMap(const Params& P, V3& color, float& pdfOut, Rng& rng) {
    float u, v;
    BinarySearch(P, rng.next() * P.env_total, u, v);
    color = SampleEnv(P, u, v);
    float pdf = Luminance(color) / P.env_total;
    u -= P.env_rot;
    float phi = u * PT_TWO_PI;
    float theta = v * PT_PI;
    float st = sinf(theta), ct = cosf(theta);
    if (st == 0.0f) pdf = 0.0f;
    pdfOut = (pdf * (float)P.env_w * (float)P.env_h) / (PT_TWO_PI * PT_PI * st);
    float sp, cp;
    sincosf(phi, &sp, &cp);
    return v3(-st * cp, ct, -st * sp);
}

// sampling.glsl:186-248
__device__ __forceinline__ void SampleOneLight(const Params& P, const Light& light, V3 scatterPos, LightSample& ls,
                                               Rng& rng) {
    const int type = (int)light.type;
    if (type == QUAD_LIGHT) {
        float r1 = rng.next();
        float r2 = rng.next();
        V3 lightSurfacePos = light.position + light.u * r1 + light.v * r2;
        ls.direction = lightSurfacePos - scatterPos;
        ls.dist = length(ls.direction);
        float distSq = ls.dist * ls.dist;
        ls.direction = ls.direction / ls.dist;
        ls.normal = normalize(cross(light.u, light.v));
        ls.emission = light.emission * (float)P.num_lights;
        ls.pdf = distSq / (light.area * fabsf(dot(ls.normal, ls.direction)));
    } else if (type == SPHERE_LIGHT) {
        float r1 = rng.next();
        float r2 = rng.next();
        V3 c2s = scatterPos - light.position;
        float distToSphereCenter = length(c2s);
        c2s = c2s / distToSphereCenter;
        V3 sampledDir = UniformSampleHemisphere(r1, r2);
        V3 T, B;
        Onb(c2s, T, B);
        sampledDir = T * sampledDir.x + B * sampledDir.y + c2s * sampledDir.z;
        V3 lightSurfacePos = light.position + sampledDir * light.radius;
        ls.direction = lightSurfacePos - scatterPos;
        ls.dist = length(ls.direction);
        float distSq = ls.dist * ls.dist;
        ls.direction = ls.direction / ls.dist;
        ls.normal = normalize(lightSurfacePos - light.position);
        ls.emission = light.emission * (float)P.num_lights;
        ls.pdf = distSq / (light.area * 0.5f * fabsf(dot(ls.normal, ls.direction)));
    } else {
        ls.direction = normalize(light.position - v3(0.0f));
        ls.normal = normalize(scatterPos - light.position);
        ls.emission = light.emission * (float)P.num_lights;
        ls.dist = PT_INF;
        ls.pdf = 1.0f;
    }
}

// pathtrace.glsl:158-283
template <int MEDIUM, bool ENV>
__device__ V3 DirectLight(const Params& P, const Ray& r, const State& state, bool isSurface, Rng& rng, uint2* stack,
                          Counters& cnt) {
    V3 Ld = v3(0.0f);
    V3 Li = v3(0.0f);
    const V3 scatterPos = state.fhp + state.normal * PT_EPS;
    constexpr bool volmis = MEDIUM == 2;
    float sfPdf;
    V3 sf;
    if (ENV) {
        float lightPdf;
        const V3 lightDir = SampleEnvMap(P, Li, lightPdf, rng);
        const Ray shadowRay{scatterPos, lightDir};
        if (volmis) {
            Li = Li * EvalTransmittance(P, shadowRay, rng, stack, cnt);
            if (isSurface) sf = DisneyEval(state.mat, state.eta, -r.direction, state.ffnormal, lightDir, sfPdf);
            else {
                float p = PhaseHG(dot(-r.direction, lightDir), state.medium.anisotropy);
                sf = v3(p);
                sfPdf = p;
            }
            if (sfPdf > 0.0f) {
                float misWeight = PowerHeuristic(lightPdf, sfPdf);
                if (misWeight > 0.0f) Ld = Ld + misWeight * Li * sf * P.env_intensity / lightPdf;
            }
        } else {
            bool inShadow = AnyHit(P, shadowRay, PT_INF - PT_EPS, rng, stack, cnt);
            if (!inShadow) {
                sf = DisneyEval(state.mat, state.eta, -r.direction, state.ffnormal, lightDir, sfPdf);
                if (sfPdf > 0.0f) {
                    float misWeight = PowerHeuristic(lightPdf, sfPdf);
                    if (misWeight > 0.0f) Ld = Ld + misWeight * Li * sf * P.env_intensity / lightPdf;
                }
            }
        }
    }
    if (P.flags & F_LIGHTS) {
        LightSample ls;
        const int index = (int)(rng.next() * (float)P.num_lights);
        Light light;
        if (index < P.num_lights) light = LoadLight(P.lights, index);
        else {  // rand() == 1: one past the last light reads zeros (GL texelFetch out of range)
            light.position = light.emission = light.u = light.v = v3(0.0f);
            light.radius = light.area = light.type = 0.0f;
        }
        SampleOneLight(P, light, scatterPos, ls, rng);
        Li = ls.emission;
        if (dot(ls.direction, ls.normal) < 0.0f) {
            const Ray shadowRay{scatterPos, ls.direction};
            if (volmis) {
                Li = Li * EvalTransmittance(P, shadowRay, rng, stack, cnt);
                if (isSurface) sf = DisneyEval(state.mat, state.eta, -r.direction, state.ffnormal, ls.direction, sfPdf);
                else {
                    float p = PhaseHG(dot(-r.direction, ls.direction), state.medium.anisotropy);
                    sf = v3(p);
                    sfPdf = p;
                }
                float misWeight = 1.0f;
                if (light.area > 0.0f) misWeight = PowerHeuristic(ls.pdf, sfPdf);
                if (sfPdf > 0.0f) Ld = Ld + misWeight * sf * Li / ls.pdf;
            } else {
                bool inShadow = AnyHit(P, shadowRay, ls.dist - PT_EPS, rng, stack, cnt);
                if (!inShadow) {
                    sf = DisneyEval(state.mat, state.eta, -r.direction, state.ffnormal, ls.direction, sfPdf);
                    float misWeight = 1.0f;
                    if (light.area > 0.0f) misWeight = PowerHeuristic(ls.pdf, sfPdf);
                    if (sfPdf > 0.0f) Ld = Ld + misWeight * Li * sf / ls.pdf;
                }
            }
        }
    }
    return Ld;
}

// pathtrace.glsl:285-476
template <int MEDIUM, bool ENV>
__device__ V3 PathTrace(const Params& P, Ray r, Rng& rng, uint2* stack, Counters& cnt, float& alphaOut) {
    V3 radiance = v3(0.0f);
    V3 throughput = v3(1.0f);
    State state;
    state.isEmitter = false;
    state.matID = 0;
    state.mat.roughness = 0.0f;
    state.normal = v3(0.0f);
    state.eta = 0.0f;
    state.medium.type = 0;
    state.medium.density = 0.0f;
    state.medium.color = v3(0.0f);
    state.medium.anisotropy = 0.0f;
    LightSample ls;
    ls.pdf = 0.0f;
    ls.emission = v3(0.0f);
    float scatterPdf = 0.0f;
    V3 scatterL = v3(0.0f);
    float alpha = 1.0f;
    bool inMedium = false, mediumSampled = false, surfaceScatter = false;
    const uint32_t F = P.flags;
    // Alpha pass-through keeps the depth (pathtrace.glsl:423); the loop is
    // bounded all the same, and a path that runs out reports PT_ERR_TIMEOUT.
    int guard = 0;
    for (state.depth = 0;; state.depth++) {
        if (++guard > 65536) {
            flag_status(P.status, PT_ERR_TIMEOUT);
            break;
        }
        const bool hit = ClosestHit(P, r, state, ls, stack, cnt, false);
        if (!hit) {
            if ((F & F_BACKGROUND) && state.depth == 0) alpha = 0.0f;
            if (!((F & F_HIDE_EMITTERS) && !(state.depth > 0))) {
                if (F & F_UNIFORM_LIGHT) {
                    radiance = radiance + v3(P.uniform_light[0], P.uniform_light[1], P.uniform_light[2]) * throughput;
                } else if (ENV) {
                    float envPdf;
                    V3 envCol = EvalEnvMap(P, r, envPdf);
                    float misWeight = 1.0f;
                    if (state.depth > 0) misWeight = PowerHeuristic(scatterPdf, envPdf);
                    if (MEDIUM == 1 && !surfaceScatter) misWeight = 1.0f;
                    if (misWeight > 0.0f) radiance = radiance + misWeight * envCol * throughput * P.env_intensity;
                }
            }
            break;
        }
        GetMaterial(P, state, r);
        radiance = radiance + state.mat.emission * throughput;
        if ((F & F_LIGHTS) && state.isEmitter) {
            float misWeight = 1.0f;
            if (state.depth > 0) misWeight = PowerHeuristic(scatterPdf, ls.pdf);
            if (MEDIUM == 1 && !surfaceScatter) misWeight = 1.0f;
            radiance = radiance + misWeight * ls.emission * throughput;
            break;
        }
        if (state.depth == P.max_depth) break;
        if (MEDIUM) {
            mediumSampled = false;
            surfaceScatter = false;
            if (inMedium) {
                if (state.medium.type == MEDIUM_ABSORB) {
                    throughput = throughput * vexp(-(v3(1.0f) - state.medium.color) * state.hitDist * state.medium.density);
                } else if (state.medium.type == MEDIUM_EMISSIVE) {
                    radiance = radiance + state.medium.color * state.hitDist * state.medium.density * throughput;
                } else {
                    float scatterDist = fminf(-logf(rng.next()) / state.medium.density, state.hitDist);
                    mediumSampled = scatterDist < state.hitDist;
                    if (mediumSampled) {
                        throughput = throughput * state.medium.color;
                        r.origin = r.origin + r.direction * scatterDist;
                        state.fhp = r.origin;
                        radiance = radiance + DirectLight<MEDIUM, ENV>(P, r, state, false, rng, stack, cnt) * throughput;
                        float h1 = rng.next();
                        float h2 = rng.next();
                        V3 scatterDir = SampleHG(-r.direction, state.medium.anisotropy, h1, h2);
                        scatterPdf = PhaseHG(dot(-r.direction, scatterDir), state.medium.anisotropy);
                        r.direction = scatterDir;
                    }
                }
            }
        }
        if (!mediumSampled) {
            if ((F & F_ALPHA_TEST) && AlphaSkip(state.mat, rng)) {
                scatterL = r.direction;
                state.depth--;
            } else {
                surfaceScatter = true;
                radiance = radiance + DirectLight<MEDIUM, ENV>(P, r, state, true, rng, stack, cnt) * throughput;
                V3 f = DisneySample(state.mat, state.eta, -r.direction, state.ffnormal, scatterL, scatterPdf, rng);
                if (scatterPdf > 0.0f) throughput = throughput * (f / scatterPdf);
                else break;
            }
            r.direction = scatterL;
            r.origin = state.fhp + r.direction * PT_EPS;
            if (MEDIUM) {
                if (dot(r.direction, state.normal) < 0.0f && state.mat.medium.type != MEDIUM_NONE) {
                    inMedium = true;
                    state.medium = state.mat.medium;
                } else if (state.mat.medium.type != MEDIUM_NONE) inMedium = false;
            }
        }
        if ((F & F_RR) && state.depth >= P.rr_depth) {
            float q = fminf(maxc(throughput) + 0.001f, 0.95f);
            if (rng.next() > q) break;
            throughput = throughput / q;
        }
    }
    alphaOut = alpha;
    return radiance;
}

// tile.glsl:41-74 for pixel (px, py); the RNG is seeded with the
// tile-local fragment position, as the tile viewport gives gl_FragCoord.
__device__ __forceinline__ Ray CameraRay(const Params& P, int px, int py, int tx, int ty, Rng& rng) {
    const int lx = px - tx * P.tile_w, ly = py - ty * P.tile_h;
    const float invx = (float)P.tile_w / (float)P.width, invy = (float)P.tile_h / (float)P.height;
    const float tcx = ((float)lx + 0.5f) / (float)P.tile_w, tcy = ((float)ly + 0.5f) / (float)P.tile_h;
    const float offx = (float)tx * invx, offy = (float)ty * invy;
    const float cx = offx * (1.0f - tcx) + (offx + invx) * tcx;
    const float cy = offy * (1.0f - tcy) + (offy + invy) * tcy;
    float r1 = 2.0f * rng.next();
    float r2 = 2.0f * rng.next();
    float jx = r1 < 1.0f ? sqrtf(r1) - 1.0f : 1.0f - sqrtf(2.0f - r1);
    float jy = r2 < 1.0f ? sqrtf(r2) - 1.0f : 1.0f - sqrtf(2.0f - r2);
    const float resx = (float)P.width, resy = (float)P.height;
    jx = jx / (resx * 0.5f);
    jy = jy / (resy * 0.5f);
    float dx = (cx * 2.0f - 1.0f) + jx;
    float dy = (cy * 2.0f - 1.0f) + jy;
    const float scale = tanf(P.cam_fov * 0.5f);
    dy *= resy / resx * scale;
    dx *= scale;
    const V3 right = v3(P.cam_right[0], P.cam_right[1], P.cam_right[2]);
    const V3 up = v3(P.cam_up[0], P.cam_up[1], P.cam_up[2]);
    const V3 fwd = v3(P.cam_fwd[0], P.cam_fwd[1], P.cam_fwd[2]);
    const V3 pos = v3(P.cam_pos[0], P.cam_pos[1], P.cam_pos[2]);
    const V3 rayDir = normalize(dx * right + dy * up + fwd);
    const V3 focalPoint = P.cam_focal * rayDir;
    const float cam_r1 = rng.next() * PT_TWO_PI;
    const float cam_r2 = rng.next() * P.cam_aperture;
    float s, c;
    sincosf(cam_r1, &s, &c);
    const V3 aperturePos = (c * right + s * up) * sqrtf(cam_r2);
    const V3 finalDir = normalize(focalPoint - aperturePos);
    return Ray{pos + aperturePos, finalDir};
}

__device__ __forceinline__ void add_counters(const Params& P, uint32_t closest, uint32_t shadow, uint32_t paths) {
    const unsigned mask = __activemask();
    closest = __reduce_add_sync(mask, closest);
    shadow = __reduce_add_sync(mask, shadow);
    paths = __reduce_add_sync(mask, paths);
    if ((threadIdx.x & 31) == __ffs(mask) - 1) {
        atomicAdd(P.counters + 0, (unsigned long long)closest);
        atomicAdd(P.counters + 1, (unsigned long long)shadow);
        atomicAdd(P.counters + 2, (unsigned long long)paths);
    }
}

// One thread per pixel of the work rectangle; a 16x8 pixel block per CTA.
template <int MEDIUM, bool ENV>
__global__ void __launch_bounds__(128) render_kernel(Params P, RenderWork W) {
    uint2 stack[kStackSize];
    const int lx = threadIdx.x & 15, ly = threadIdx.x >> 4;
    const int px = W.x0 + blockIdx.x * 16 + lx;
    const int py = W.y0 + blockIdx.y * 8 + ly;
    const bool active = px < W.x0 + W.w && py < W.y0 + W.h;
    Counters cnt{0, 0};
    uint32_t paths = 0;
    if (active) {
        float4* out = P.accum + (size_t)py * P.width + px;
        float4 acc = *out;
        const int tx = px / P.tile_w, ty = py / P.tile_h;
        for (int pass = W.first_pass; pass < W.first_pass + W.num_passes; ++pass) {
            uint32_t frame;
            if (W.tile_frame >= 0) frame = (uint32_t)W.tile_frame;
            else frame = (uint32_t)(2 + pass * P.ntx * P.nty + (P.nty - 1 - ty) * P.ntx + tx);
            Rng rng;
            rng.init((uint32_t)(px - tx * P.tile_w), (uint32_t)(py - ty * P.tile_h), frame);
            const Ray ray = CameraRay(P, px, py, tx, ty, rng);
            float alpha;
            const V3 L = PathTrace<MEDIUM, ENV>(P, ray, rng, stack, cnt, alpha);
            acc.x += L.x;
            acc.y += L.y;
            acc.z += L.z;
            acc.w += alpha;
            ++paths;
        }
        *out = acc;
    }
    add_counters(P, cnt.closest, cnt.shadow, paths);
}

__global__ void __launch_bounds__(128) trace_closest_kernel(Params P, const pt_ray* __restrict__ rays, int n,
                                                            pt_hit* __restrict__ hits) {
    uint2 stack[kStackSize];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const pt_ray rr = rays[i];
    TriHit h;
    h.t = PT_INF;
    h.prim = -1;
    h.inst = -1;
    h.u = h.v = 0.0f;
    traverse_closest<true>(P, P.tlas_root,
                           prep_ray(v3(rr.origin[0], rr.origin[1], rr.origin[2]),
                                    v3(rr.direction[0], rr.direction[1], rr.direction[2])),
                           h, stack, 0, -1, 0);
    pt_hit o;
    if (h.prim >= 0) {
        o.t = h.t; o.u = h.u; o.v = h.v; o.prim_id = h.prim; o.inst_id = h.inst;
    } else {
        o.t = PT_INF; o.u = o.v = 0.0f; o.prim_id = -1; o.inst_id = -1;
    }
    hits[i] = o;
}

__global__ void __launch_bounds__(128) trace_shadow_kernel(Params P, const pt_ray* __restrict__ rays,
                                                           const float* __restrict__ maxd, int n,
                                                           unsigned char* __restrict__ occ) {
    uint2 stack[kStackSize];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const pt_ray rr = rays[i];
    Rng rng;
    rng.init((uint32_t)i, 0u, 0u);
    const bool alpha = (P.flags & F_ALPHA_TEST) && !(P.flags & F_MEDIUM);
    occ[i] = traverse_any<true>(P, P.tlas_root,
                                prep_ray(v3(rr.origin[0], rr.origin[1], rr.origin[2]),
                                         v3(rr.direction[0], rr.direction[1], rr.direction[2])),
                                maxd[i], stack, 0, 0, alpha, rng)
                 ? 1
                 : 0;
}

// tonemap.glsl:59-133 and the float->RGBA8 conversion of glGetTexImage.
__device__ __forceinline__ V3 ACESFitted(V3 c) {
    // color * ACESInputMat (row vector times the matrix whose columns are listed)
    V3 v = v3(dot(c, v3(0.59719f, 0.35458f, 0.04823f)), dot(c, v3(0.07600f, 0.90834f, 0.01566f)),
              dot(c, v3(0.02840f, 0.13383f, 0.83777f)));
    V3 a = v * (v + v3(0.0245786f)) - v3(0.000090537f);
    V3 b = v * (0.983729f * v + v3(0.4329510f)) + v3(0.238081f);
    v = a / b;
    v = v3(dot(v, v3(1.60475f, -0.53108f, -0.07367f)), dot(v, v3(-0.10208f, 1.10813f, -0.00605f)),
           dot(v, v3(-0.00327f, -0.07276f, 1.07602f)));
    return v3(clampf(v.x, 0.0f, 1.0f), clampf(v.y, 0.0f, 1.0f), clampf(v.z, 0.0f, 1.0f));
}
__device__ __forceinline__ float aces1(float c) {
    return clampf((c * (2.51f * c + 0.03f)) / (c * (2.43f * c + 0.59f) + 0.14f), 0.0f, 1.0f);
}
// float -> normalized unsigned byte: clamp to [0,1], scale by 255, round half up
__device__ __forceinline__ unsigned char to_unorm8(float c) {
    c = fminf(fmaxf(c, 0.0f), 1.0f);
    return (unsigned char)floorf(c * 255.0f + 0.5f);
}

__global__ void tonemap_kernel(Params P, float inv, int tonemap, int aces, int simple, int background, int transparent,
                               float3 bg, uchar4* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.width * P.height) return;
    const float4 a = P.accum[i];
    V3 color = v3(a.x * inv, a.y * inv, a.z * inv);
    const float alpha = a.w * inv;
    if (tonemap) {
        if (aces) {
            if (simple) color = v3(aces1(color.x), aces1(color.y), aces1(color.z));
            else color = ACESFitted(color);
        } else {
            color = color / (1.0f + Luminance(color) / 1.5f);  // Tonemap(c, 1.5): c * 1.0 / (1.0 + lum / limit)
        }
    }
    color = v3(powf(color.x, 1.0f / 2.2f), powf(color.y, 1.0f / 2.2f), powf(color.z, 1.0f / 2.2f));
    float outAlpha = 1.0f;
    V3 bgc = v3(bg.x, bg.y, bg.z);
    if (transparent) {
        outAlpha = alpha;
        const int px = i % P.width, py = i / P.width;
        const float fx = (float)px + 0.5f, fy = (float)py + 0.5f;
        const float checker = 10.0f;
        const float m = fmodf(floorf(fx / checker) + floorf(fy / checker), 2.0f);
        const float res = fmaxf(m > 0.0f ? 1.0f : 0.0f, 0.0f);
        bgc = mix3(v3(0.1f), v3(0.2f), res);
    }
    if (background || transparent) color = mix3(bgc, color, alpha);
    out[i] = make_uchar4(to_unorm8(color.x), to_unorm8(color.y), to_unorm8(color.z), to_unorm8(outAlpha));
}

// ------------------------------------------------------------- launchers
template <int MEDIUM, bool ENV>
static cudaError_t launch_render_t(const Params& p, const RenderWork& w, cudaStream_t s) {
    dim3 grid((w.w + 15) / 16, (w.h + 7) / 8);
    render_kernel<MEDIUM, ENV><<<grid, 128, 0, s>>>(p, w);
    return cudaGetLastError();
}

cudaError_t launch_render(const Params& p, const RenderWork& w, int /*integrator*/, cudaStream_t s) {
    const int medium = (p.flags & F_MEDIUM) ? ((p.flags & F_VOL_MIS) ? 2 : 1) : 0;
    const bool env = (p.flags & F_ENVMAP) != 0;
    if (w.w <= 0 || w.h <= 0 || w.num_passes <= 0) return cudaSuccess;
    switch (medium * 2 + (env ? 1 : 0)) {
        case 0: return launch_render_t<0, false>(p, w, s);
        case 1: return launch_render_t<0, true>(p, w, s);
        case 2: return launch_render_t<1, false>(p, w, s);
        case 3: return launch_render_t<1, true>(p, w, s);
        case 4: return launch_render_t<2, false>(p, w, s);
        default: return launch_render_t<2, true>(p, w, s);
    }
}

cudaError_t launch_trace_closest(const Params& p, const void* rays, int n, void* hits, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    trace_closest_kernel<<<(n + 127) / 128, 128, 0, s>>>(p, (const pt_ray*)rays, n, (pt_hit*)hits);
    return cudaGetLastError();
}

cudaError_t launch_trace_shadow(const Params& p, const void* rays, const float* maxd, int n, unsigned char* occ,
                                cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    trace_shadow_kernel<<<(n + 127) / 128, 128, 0, s>>>(p, (const pt_ray*)rays, maxd, n, occ);
    return cudaGetLastError();
}

cudaError_t launch_tonemap(const Params& p, int num_samples, int enable_tonemap, int enable_aces, int simple_aces,
                           int background, int transparent, const float* bg, unsigned char* out, cudaStream_t s) {
    const int n = p.width * p.height;
    if (n <= 0) return cudaSuccess;
    const float inv = 1.0f / (float)num_samples;
    tonemap_kernel<<<(n + 255) / 256, 256, 0, s>>>(p, inv, enable_tonemap, enable_aces, simple_aces, background,
                                                   transparent, make_float3(bg[0], bg[1], bg[2]), (uchar4*)out);
    return cudaGetLastError();
}

}  // namespace ptgb
