// pt_trace.cuh - ray traversal of the 8-wide quantised BVH (bvh8.h).
//
// A node fetch is five 128-bit loads; the eight child boxes are slab-tested
// against the ray and the hits become a 32-bit mask: bits 24-31 internal
// children in octant order, bits 0-23 leaf primitives (triangles in a BLAS,
// instances in the TLAS).
//
// Traversal is a state machine that does one unit of work per step -- test
// one triangle, enter one instance, intersect one node, or pop the stack --
// so that the threads of a warp stay in one loop whatever level and stage
// each ray is at, and a thread whose ray finished can take a new one at once
// (the persistent kernels of pt_wavefront.cu).  Both levels of the
// reference's two-level BVH run in the same loop: entering an instance
// pushes the TLAS node group, the remaining instance bits and a sentinel;
// popping the sentinel restores them and leaves the BLAS.
//
// The triangle test repeats the reference's arithmetic operation for
// operation, without fused multiply-adds (closest_hit.glsl:128-143), so hit
// decisions and distances equal the oracle's bit for bit.  Most triangles
// are rejected before the three divisions, by tests that reject exactly the
// triangles the full test would (see tri_test).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pt_cuda.h"
#include "pt_device.cuh"
#include "pt_params.h"

namespace ptgb {

// A ray prepared for slab tests: 1/d and the inverse octant (7 - octant of
// d; bit k clear when d points towards -k).
struct TRay {
    V3 o, d;
    float ix, iy, iz;
    uint32_t oct_inv;
};

// 1/d rounded to nearest (__frcp_rn), whatever -prec-div says: the slab
// planes then sit where IEEE arithmetic puts them, as in the oracle's
// AABBIntersect (invDir = 1.0 / r.direction).  Three per ray set-up.
__device__ __forceinline__ float safe_rcp(float d) {
    return __frcp_rn(fabsf(d) > 1e-20f ? d : copysignf(1e-20f, d));
}

// The ray (o, d) with its reciprocal direction given.
__device__ __forceinline__ TRay make_tray(V3 o, V3 d, float ix, float iy, float iz) {
    TRay r;
    r.o = o;
    r.d = d;
    r.ix = ix;
    r.iy = iy;
    r.iz = iz;
    const uint32_t oct = (ix < 0.0f ? 1u : 0u) | (iy < 0.0f ? 2u : 0u) | (iz < 0.0f ? 4u : 0u);
    r.oct_inv = 7u - oct;
    return r;
}

__device__ __forceinline__ TRay prep_ray(V3 o, V3 d) {
    return make_tray(o, d, safe_rcp(d.x), safe_rcp(d.y), safe_rcp(d.z));
}


// 2^15 + byte j of w, exactly: the byte in mantissa bits 8-15 of 2^15
// (where their weight is 1), without the (quarter-rate) integer conversion.
__device__ __forceinline__ float qbyte_biased(uint32_t w, int j) {
    return __uint_as_float(__byte_perm(w, 0x47000000u, 0x7404u | ((uint32_t)j << 4)));
}
constexpr float kQBias = 32768.0f;

// Packed FP32 pairs (sm_100+): one instruction for two IEEE round-to-nearest
// operations, with the results of the two scalar ones.
__device__ __forceinline__ unsigned long long f2pack(float lo, float hi) {
    unsigned long long r;
#ifdef __CUDA_ARCH__
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
#else
    r = (unsigned long long)__float_as_uint(lo) | ((unsigned long long)__float_as_uint(hi) << 32);
#endif
    return r;
}
// a * c + d per lane of the pairs, rounded as fmaf(a, c, d)
__device__ __forceinline__ void f2_fma(unsigned long long a, unsigned long long c, unsigned long long d, float& lo,
                                       float& hi) {
#ifdef __CUDA_ARCH__
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(c), "l"(d));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(r));
#else
    auto f = [](unsigned long long v, int k) { return __uint_as_float((uint32_t)(v >> (32 * k))); };
    lo = fmaf(f(a, 0), f(c, 0), f(d, 0));
    hi = fmaf(f(a, 1), f(c, 1), f(d, 1));
#endif
}

__device__ __forceinline__ float fmax3f(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
#else
    return fmaxf(fmaxf(a, b), c);
#endif
}
__device__ __forceinline__ float fmin3f(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
#else
    return fminf(fminf(a, b), c);
#endif
}

// The plane set-up of a node (its first word w0: origin, scale exponents)
// for ray r: adj = scale / d and the near / far constants C per axis.
struct NodeFrame {
    float adjx, adjy, adjz, cnx, cfx, cny, cfy, cnz, cfz;
};
__device__ __forceinline__ NodeFrame node_frame(uint4 w0, const TRay& r) {
    NodeFrame f;
    const float sx = __uint_as_float((w0.w & 0xffu) << 23);
    const float sy = __uint_as_float(((w0.w >> 8) & 0xffu) << 23);
    const float sz = __uint_as_float(((w0.w >> 16) & 0xffu) << 23);
    f.adjx = sx * r.ix;
    f.adjy = sy * r.iy;
    f.adjz = sz * r.iz;
    const float orgx = (__uint_as_float(w0.x) - r.o.x) * r.ix;
    const float orgy = (__uint_as_float(w0.y) - r.o.y) * r.iy;
    const float orgz = (__uint_as_float(w0.z) - r.o.z) * r.iz;
    f.cnx = __fmaf_rd(-kQBias, f.adjx, orgx);
    f.cfx = __fmaf_ru(-kQBias, f.adjx, orgx);
    f.cny = __fmaf_rd(-kQBias, f.adjy, orgy);
    f.cfy = __fmaf_ru(-kQBias, f.adjy, orgy);
    f.cnz = __fmaf_rd(-kQBias, f.adjz, orgz);
    f.cfz = __fmaf_ru(-kQBias, f.adjz, orgz);
    return f;
}

// Slab test of the eight children of wide node `idx`; returns the hit mask.
// A plane's distance is q * adj + org with q the plane's byte, adj =
// scale / d and org = (node origin - o) / d.  It is evaluated as one FMA,
// Q * adj + C, with Q = 2^15 + q (exact, qbyte_biased) and C = org - 2^15 *
// adj rounded down for near planes and up for far planes.  Rounding is
// monotonic, so a near distance is never above fl(q * adj + org) and a far
// distance never below it: the test accepts every box that the two-step
// form fl((Q - 2^15) * adj + org) accepts, and more only by ulp(C) (about
// 2^-8 of a quantisation step).  Entry and exit distances are three-input
// max / min (sm_100+).  PACKED computes the near and far planes of an axis
// as one packed pair (the same values, fewer instructions, more registers).
template <bool PACKED = false>
__device__ __forceinline__ uint32_t intersect_node(const uint4* __restrict__ nodes, const uint4* __restrict__ words,
                                                   int idx, const TRay& r, float tmax, uint32_t& child_base,
                                                   uint32_t& prim_base, uint32_t& imask) {
    const uint4* n = nodes + (size_t)idx * 5;
    const uint4 w0 = __ldg(n), w1 = __ldg(n + 1), w2 = __ldg(n + 2), w3 = __ldg(n + 3), w4 = __ldg(n + 4);
    const uint4 hw0 = __ldg(words + 2 * (size_t)idx), hw1 = __ldg(words + 2 * (size_t)idx + 1);
    imask = w0.w >> 24;
    child_base = w1.x;
    prim_base = w1.y;
    const NodeFrame f = node_frame(w0, r);
    const float adjx = f.adjx, adjy = f.adjy, adjz = f.adjz;
    const float cnx = f.cnx, cfx = f.cfx, cny = f.cny, cfy = f.cfy, cnz = f.cnz, cfz = f.cfz;
    const bool nx = !(r.oct_inv & 1u), ny = !(r.oct_inv & 2u), nz = !(r.oct_inv & 4u);
    uint32_t hits = 0;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        const uint4 hw = half ? hw1 : hw0;
        const uint32_t qlox = half ? w2.y : w2.x, qloy = half ? w2.w : w2.z, qloz = half ? w3.y : w3.x;
        const uint32_t qhix = half ? w3.w : w3.z, qhiy = half ? w4.y : w4.x, qhiz = half ? w4.w : w4.z;
        const uint32_t nxw = nx ? qhix : qlox, fxw = nx ? qlox : qhix;
        const uint32_t nyw = ny ? qhiy : qloy, fyw = ny ? qloy : qhiy;
        const uint32_t nzw = nz ? qhiz : qloz, fzw = nz ? qloz : qhiz;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float tnx, tfx, tny, tfy, tnz, tfz;
            if (PACKED) {
                f2_fma(f2pack(qbyte_biased(nxw, j), qbyte_biased(fxw, j)), f2pack(adjx, adjx), f2pack(cnx, cfx), tnx,
                       tfx);
                f2_fma(f2pack(qbyte_biased(nyw, j), qbyte_biased(fyw, j)), f2pack(adjy, adjy), f2pack(cny, cfy), tny,
                       tfy);
                f2_fma(f2pack(qbyte_biased(nzw, j), qbyte_biased(fzw, j)), f2pack(adjz, adjz), f2pack(cnz, cfz), tnz,
                       tfz);
            } else {
                tnx = fmaf(qbyte_biased(nxw, j), adjx, cnx);
                tfx = fmaf(qbyte_biased(fxw, j), adjx, cfx);
                tny = fmaf(qbyte_biased(nyw, j), adjy, cny);
                tfy = fmaf(qbyte_biased(fyw, j), adjy, cfy);
                tnz = fmaf(qbyte_biased(nzw, j), adjz, cnz);
                tfz = fmaf(qbyte_biased(fzw, j), adjz, cfz);
            }
            const float t0 = fmax3f(tnx, tny, fmaxf(tnz, 0.0f));
            const float t1 = fmin3f(tfx, tfy, fminf(tfz, tmax));
            if (t0 <= t1) hits |= (j == 0 ? hw.x : j == 1 ? hw.y : j == 2 ? hw.z : hw.w);
        }
    }
    // internal children: from slot order to the ray's visiting order (bit
    // 24 + (slot ^ oct_inv)), swapping bit pairs, bit quads and nibbles
    uint32_t in8 = hits >> 24;
    const uint32_t o = r.oct_inv;
    uint32_t t = ((in8 & 0x55u) << 1) | ((in8 >> 1) & 0x55u);
    in8 = (o & 1u) ? t : in8;
    t = ((in8 & 0x33u) << 2) | ((in8 >> 2) & 0x33u);
    in8 = (o & 2u) ? t : in8;
    t = ((in8 & 0x0fu) << 4) | (in8 >> 4);
    in8 = (o & 4u) ? t : in8;
    return (hits & 0x00ffffffu) | (in8 << 24);
}

// Instance bounds (Params::inst_bounds, two words per InstRef, made by
// inst_bounds_kernel): the first word of the BLAS root node (origin and
// scale exponents, the internal-child mask cleared) and the union of the
// root's child boxes in the root's own grid -- x: the smallest qlo bytes
// (x | y << 8 | z << 16), y: the largest qhi bytes.  An empty root has
// qlo 255 and qhi 0, which no ray hits.
//
// Whether intersect_node on the BLAS root could accept any child.  The
// union box is tested with the root's own frame (node_frame) and the same
// FMA per plane: the FMA's rounding is monotonic in the plane byte, so the
// union's near distances are at most, and its far distances at least, those
// of every child, and every child the node test would accept makes this
// test pass.  Skipping the instances it rejects changes no result.
__device__ __forceinline__ bool root_may_hit(const uint4* __restrict__ bounds, int ref, const TRay& r, float tmax) {
    const uint4 w0 = __ldg(bounds + 2 * ref), q = __ldg(bounds + 2 * ref + 1);
    const NodeFrame f = node_frame(w0, r);
    const bool nx = !(r.oct_inv & 1u), ny = !(r.oct_inv & 2u), nz = !(r.oct_inv & 4u);
    const uint32_t near = __byte_perm(q.x, q.y, (nx ? 4u : 0u) | (ny ? 0x50u : 0x10u) | (nz ? 0x600u : 0x200u));
    const uint32_t far = __byte_perm(q.x, q.y, (nx ? 0u : 4u) | (ny ? 0x10u : 0x50u) | (nz ? 0x200u : 0x600u));
    const float tnx = fmaf(qbyte_biased(near, 0), f.adjx, f.cnx);
    const float tfx = fmaf(qbyte_biased(far, 0), f.adjx, f.cfx);
    const float tny = fmaf(qbyte_biased(near, 1), f.adjy, f.cny);
    const float tfy = fmaf(qbyte_biased(far, 1), f.adjy, f.cfy);
    const float tnz = fmaf(qbyte_biased(near, 2), f.adjz, f.cnz);
    const float tfz = fmaf(qbyte_biased(far, 2), f.adjz, f.cfz);
    return fmax3f(tnx, tny, fmaxf(tnz, 0.0f)) <= fmin3f(tfx, tfy, fminf(tfz, tmax));
}

// Triangle test of closest_hit.glsl:128-143 (accept when u, v, t and
// w = 1-u-v are all >= 0 and t <= tmax; the caller decides t == tmax) with
// the reference's operation order
// and no contraction.  The numerators U, V, T and det are computed first;
// with det made positive (an exact sign flip of all four) a triangle is
// rejected before dividing when
//   U, V or T < -det * 1e-30   the quotient is negative and not so small
//                              that it would round to zero,
//   U + V > det * (1 + 1e-6)   u + v exceeds 1 by far more than the
//                              rounding of (1 - u) - v, so w < 0,
//   T > det * tmax * (1 + 1e-6)  t rounds to above tmax;
// each of these implies the full test fails, so the accepted set is unchanged.
__device__ __forceinline__ bool tri_test(const TRay& r, const float4* __restrict__ tris, int t, float tmax, float& u,
                                         float& v, float& tt, float& w, int& prim, int& tinst, int& tmat) {
    const float4 a = __ldg(tris + 3 * (size_t)t), b = __ldg(tris + 3 * (size_t)t + 1),
                 c = __ldg(tris + 3 * (size_t)t + 2);
    // e0 = b, e1 = c (precomputed v1-v0, v2-v0)
    const float pvx = __fsub_rn(__fmul_rn(r.d.y, c.z), __fmul_rn(r.d.z, c.y));
    const float pvy = __fsub_rn(__fmul_rn(r.d.z, c.x), __fmul_rn(r.d.x, c.z));
    const float pvz = __fsub_rn(__fmul_rn(r.d.x, c.y), __fmul_rn(r.d.y, c.x));
    float det = __fadd_rn(__fadd_rn(__fmul_rn(b.x, pvx), __fmul_rn(b.y, pvy)), __fmul_rn(b.z, pvz));
    const float tvx = __fsub_rn(r.o.x, a.x), tvy = __fsub_rn(r.o.y, a.y), tvz = __fsub_rn(r.o.z, a.z);
    const float qvx = __fsub_rn(__fmul_rn(tvy, b.z), __fmul_rn(tvz, b.y));
    const float qvy = __fsub_rn(__fmul_rn(tvz, b.x), __fmul_rn(tvx, b.z));
    const float qvz = __fsub_rn(__fmul_rn(tvx, b.y), __fmul_rn(tvy, b.x));
    float U = __fadd_rn(__fadd_rn(__fmul_rn(tvx, pvx), __fmul_rn(tvy, pvy)), __fmul_rn(tvz, pvz));
    float Vv = __fadd_rn(__fadd_rn(__fmul_rn(r.d.x, qvx), __fmul_rn(r.d.y, qvy)), __fmul_rn(r.d.z, qvz));
    float T = __fadd_rn(__fadd_rn(__fmul_rn(c.x, qvx), __fmul_rn(c.y, qvy)), __fmul_rn(c.z, qvz));
    if (det < 0.0f) {
        det = -det;
        U = -U;
        Vv = -Vv;
        T = -T;
    }
    if (det > 0.0f) {
        const float eps = det * 1e-30f;
        if (U < -eps || Vv < -eps || T < -eps) return false;
        if (__fadd_rn(U, Vv) > det * 1.000001f) return false;
        if (T > (det * tmax) * 1.000001f) return false;
    }
    u = __fdiv_rn(U, det);
    v = __fdiv_rn(Vv, det);
    tt = __fdiv_rn(T, det);
    w = __fsub_rn(__fsub_rn(1.0f, u), v);
    prim = __float_as_int(a.w);
    tinst = __float_as_int(b.w);
    tmat = __float_as_int(c.w);
    return u >= 0.0f && v >= 0.0f && tt >= 0.0f && w >= 0.0f && tt <= tmax;
}

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

// texture(textureMapsArrayTex, vec3(uv, layer)): bilinear, GL_REPEAT, texel
// centres at (i + 0.5) / size, the layer rounded and clamped; RGBA8 / 255,
// the UNORM conversion rounded exactly as GL specifies.  The array (tex,
// w x h texels, n layers) comes as plain values: a reference to Params
// would make the batch kernels keep their per-job copy of it in memory.
static __device__ __noinline__ float4 SampleTexArray(const uchar4* tex, int w, int h, int n, float u, float v,
                                                     float layerf) {
    int layer = (int)floorf(layerf + 0.5f);
    layer = min(max(layer, 0), n - 1);
    const uchar4* base = tex + (size_t)layer * w * h;
    const float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float ax = x - fx, ay = y - fy;
    auto wrap = [](long long i, int n) {
        long long m = i % n;
        return (int)(m < 0 ? m + n : m);
    };
    const long long ix = (long long)fx, iy = (long long)fy;
    const int x0 = wrap(ix, w), x1 = wrap(ix + 1, w), y0 = wrap(iy, h), y1 = wrap(iy + 1, h);
    const uchar4 t00 = __ldg(base + (size_t)y0 * w + x0), t10 = __ldg(base + (size_t)y0 * w + x1);
    const uchar4 t01 = __ldg(base + (size_t)y1 * w + x0), t11 = __ldg(base + (size_t)y1 * w + x1);
    auto lerp2 = [&](unsigned char a, unsigned char b, unsigned char c, unsigned char d) {
        const float ta = __fdiv_rn((float)a, 255.0f), tb = __fdiv_rn((float)b, 255.0f),
                    tc = __fdiv_rn((float)c, 255.0f), td = __fdiv_rn((float)d, 255.0f);
        const float r0 = ta * (1.0f - ax) + tb * ax;
        const float r1 = tc * (1.0f - ax) + td * ax;
        return r0 * (1.0f - ay) + r1 * ay;
    };
    return make_float4(lerp2(t00.x, t10.x, t01.x, t11.x), lerp2(t00.y, t10.y, t01.y, t11.y),
                       lerp2(t00.z, t10.z, t01.z, t11.z), lerp2(t00.w, t10.w, t01.w, t11.w));
}

// Texture coordinate of a point (barycentrics u, v, w) of triangle `prim`:
// u from verticesUVX.w, v from normalsUVY.w (bary = uvt.wxy).
__device__ __forceinline__ void TriTexCoord(const Params& P, int prim, float u, float v, float w, float& tu,
                                            float& tv) {
    const int i0 = __ldg(P.vidx + 3 * prim), i1 = __ldg(P.vidx + 3 * prim + 1), i2 = __ldg(P.vidx + 3 * prim + 2);
    tu = __ldg(P.verts + i0).w * w + __ldg(P.verts + i1).w * u + __ldg(P.verts + i2).w * v;
    tv = __ldg(P.norms + i0).w * w + __ldg(P.norms + i1).w * u + __ldg(P.norms + i2).w * v;
}

__device__ __forceinline__ void flag_status(int* status, int code) { atomicCAS(status, PT_OK, code); }

// --------------------------------------------------------- state machine
// Entering an instance pushes the TLAS position (node group, then pending
// instances), the world ray's reciprocal direction (x and y; z rides in the
// sentinel's second word) and a sentinel; popping the sentinel leaves the
// BLAS with the world ray restored without recomputing its reciprocals.
constexpr uint32_t kBlasSentinel = 0xffffffffu;
static_assert(kInstanceEntries == 4, "an instance entry pushes four stack entries");

struct Trav {
    V3 wo, wd;         // the query ray (world space)
    TRay cur;          // the ray in the current instance's space
    float tmax;        // closest hit so far / max distance of an any-hit query
    float u, v;        // result (closest hit)
    int prim, inst, mat;
    uint2 ng;          // node group: child base, internal hit bits (24-31) | imask
    uint32_t pbase, pbits;  // pending primitives: triangles (BLAS) or instances (TLAS)
    int next;          // node to intersect next (-1: none)
    int sp;
    int cur_inst, cur_mat;  // instance being traversed (-1: the TLAS)
};

__device__ __forceinline__ void trav_init(Trav& s, const Params& P, V3 o, V3 d, float tmax) {
    s.wo = o;
    s.wd = d;
    s.cur = prep_ray(o, d);
    s.tmax = tmax;
    s.prim = -1;
    s.inst = -1;
    s.mat = 0;
    s.u = s.v = 0.0f;
    s.ng = make_uint2(0, 0);
    s.pbase = 0;
    s.pbits = 0;
    s.next = P.tlas_root;
    s.sp = 0;
    s.cur_inst = P.direct ? P.entry_inst : -1;
    s.cur_mat = P.direct ? P.entry_mat : 0;
}

enum { TRAV_RUNNING = 0, TRAV_DONE = 1, TRAV_HIT = 2 };

// Work per step in the warp modes (TRAV_NODES / TRAV_TRIS, below), where
// every lane of a warp does the same kind of step: a triangle step tests a
// whole leaf child (at most three triangles), and a node step goes
// straight on into the nearest internal child when a visit leaves no
// triangles pending (the child the next step would visit, so the order of
// visits is unchanged).  A step's fixed cost (the mode vote,
// the loop's ballots, the branch into the node or triangle code) is then
// paid once per leaf or per two nodes.  Per-lane steps (TRAV_LANE) keep one
// unit of work: there the node and triangle code of different lanes run one
// after the other, and longer steps lengthen every divergent iteration
// (measured on GB300 with the 10k-instance scene).
constexpr int kTrisPerStep = 3;
constexpr int kNodesPerStep = 2;

// A push beyond the stack bound drops the entry (the subtree or triangles
// it holds are not traversed) and sets PT_ERR_STACK_OVERFLOW in the status
// word, which the host reads after the launch; the traversal itself goes on
// and ends.  Entries are dropped one at a time only where each stands alone
// (a node group, a postponed triangle group); the four entries of an
// instance entry go on the stack together or not at all.
__device__ __forceinline__ void trav_push(const Params& P, uint2* stack, int& sp, uint2 e) {
    if (sp < P.stack_limit) stack[sp++] = e;
    else flag_status(P.status, PT_ERR_STACK_OVERFLOW);
}

// Step modes.  TRAV_LANE: each lane takes its own next unit of work.  With
// TRAV_NODES / TRAV_TRIS the warp has chosen one kind of work for all its
// lanes: under TRAV_NODES a lane with triangles pending postpones them (the
// group goes on the stack, to be popped later) when it has a node to go to,
// and idles otherwise; under TRAV_TRIS only lanes with triangles pending do
// anything.  Running one kind per warp step keeps the node and triangle code
// from both executing, each for part of the warp, on the same step.
enum { TRAV_LANE = 0, TRAV_NODES = 1, TRAV_TRIS = 2 };

// A stack entry is a node group (y bits 24-31: internal children left), a
// postponed triangle group (y bits 24-31 clear, triangle bits below), a BLAS
// sentinel, or the TLAS position under a sentinel.
__device__ __forceinline__ bool trav_has_tris(const Trav& s) { return s.pbits && s.cur_inst >= 0; }
__device__ __forceinline__ bool trav_can_descend(const Trav& s) {
    return !trav_has_tris(s) || s.ng.y > 0x00ffffffu;
}

// One step.  ANY: stop at the first accepted triangle (any-hit query);
// ALPHA (with ANY): anyhit.glsl:118-141's alpha test, drawing from rng.
// A step tests one triangle, enters one instance and visits its BLAS root,
// or picks the nearest internal child of the current node group -- popping the next group off
// the stack first when the current one is exhausted -- and intersects it.
// Closest hits: the nearest triangle wins; of triangles at exactly the same
// distance, the one of smallest (triangle, instance) id, so the result does
// not depend on the order in which triangles are tested.
// DIRECT: the scene is one untransformed instance entered directly
// (Params::direct): traversal never leaves its BLAS, and the TLAS code
// (instance entry, the return to the TLAS) is compiled out.
template <bool ANY, bool ALPHA, bool PACKED = false, bool DIRECT = false>
__device__ __forceinline__ int trav_step(Trav& s, const Params& P, uint2* stack, Rng* rng, int mode = TRAV_LANE) {
    const bool in_blas = DIRECT || s.cur_inst >= 0;
    if (mode == TRAV_TRIS && !(s.pbits && in_blas)) return TRAV_RUNNING;
    if (s.pbits && in_blas && mode == TRAV_NODES) {
        if (s.ng.y <= 0x00ffffffu) return TRAV_RUNNING;  // nothing to descend into: wait for a triangle step
        trav_push(P, stack, s.sp, make_uint2(s.pbase, s.pbits));  // postpone the triangles
        s.pbits = 0;
    }
    if (s.pbits) {
        if (in_blas) {
            // up to kTrisPerStep of the pending triangles (in bit order)
#pragma unroll
            for (int q = 0; q < kTrisPerStep; ++q) {
                if (q > 0 && (!s.pbits || mode == TRAV_LANE)) break;
                const int b = __ffs(s.pbits) - 1;
                s.pbits &= s.pbits - 1;
                float u, v, t, w;
                int prim, tinst, tmat;
                if (tri_test(s.cur, P.tris, s.pbase + b, s.tmax, u, v, t, w, prim, tinst, tmat)) {
                    // the merged BLAS of untransformed instances (cur_mat < 0)
                    // carries instance and material per triangle
                    const int mat = s.cur_mat < 0 ? tmat : s.cur_mat;
                    const int inst = s.cur_mat < 0 ? tinst : s.cur_inst;
                    if (ANY) {
                        if (t < s.tmax) {
                            if (!ALPHA) return TRAV_HIT;
                            const float4 ap = __ldg(P.mats + 8 * mat + 7);  // opacity, alphaMode, cutoff
                            const int alphaMode = (int)ap.y;
                            float opacity = ap.x;
                            if (P.flags & F_TEXTURES) {  // the base-colour map's alpha (layer 0 when none)
                                float tu, tv;
                                TriTexCoord(P, prim, u, v, w, tu, tv);
                                opacity *= SampleTexArray(P.tex, P.tex_w, P.tex_h, P.num_tex, tu, tv,
                                                          __ldg(P.mats + 8 * mat + 6).x).w;
                            }
                            bool skip = alphaMode == ALPHA_MODE_MASK && opacity < ap.z;
                            if (!skip && alphaMode == ALPHA_MODE_BLEND) skip = rng->next() > opacity;
                            if (!skip) return TRAV_HIT;
                        }
                    } else if (t < s.tmax || (s.prim >= 0 && (prim < s.prim || (prim == s.prim && inst < s.inst)))) {
                        s.tmax = t;
                        s.u = u;
                        s.v = v;
                        s.prim = prim;
                        s.inst = inst;
                        s.mat = mat;
                    }
                }
            }
            return TRAV_RUNNING;
        }
        {
            // enter an instance whose BLAS root the ray may hit (the
            // others would be entered and left without a hit: root_may_hit)
            // and park the TLAS position on the stack -- all four entries,
            // or none when they do not fit: the instance is then skipped and
            // the overflow status set, so that every later pop still finds
            // entries of its own level
            const int b = __ffs(s.pbits) - 1;
            s.pbits &= s.pbits - 1;
            const int4 ir = __ldg(P.insts + s.pbase + b);
            // in the TLAS s.cur is the world ray: an untransformed instance keeps it
            const TRay obj =
                ir.w ? s.cur : prep_ray(xform_point(P.xf, ir.y, s.wo, 1.0f), xform_point(P.xf, ir.y, s.wd, 0.0f));
            if (P.inst_bounds && !root_may_hit(P.inst_bounds, s.pbase + b, obj, s.tmax)) return TRAV_RUNNING;
            if (s.sp + kInstanceEntries > P.stack_limit) {
                flag_status(P.status, PT_ERR_STACK_OVERFLOW);
                return TRAV_RUNNING;
            }
            stack[s.sp++] = s.ng;
            stack[s.sp++] = make_uint2(s.pbase, s.pbits);
            stack[s.sp++] = make_uint2(__float_as_uint(s.cur.ix), __float_as_uint(s.cur.iy));
            stack[s.sp++] = make_uint2(kBlasSentinel, __float_as_uint(s.cur.iz));
            s.pbits = 0;
            s.ng = make_uint2(0, 0);
            s.cur_inst = ir.y;
            s.cur_mat = ir.z;
            s.cur = obj;
            s.next = ir.x;  // the BLAS root: visited below, in this step
        }
    }
    // up to kNodesPerStep node visits: after a visit that leaves no triangles
    // pending, the step goes on into the nearest internal child
#pragma unroll
    for (int q = 0; q < kNodesPerStep; ++q) {
        if (s.next < 0) {
            if (s.ng.y <= 0x00ffffffu) {  // the current group is exhausted: pop
                if (q > 0) return TRAV_RUNNING;
                if (s.sp == 0) return TRAV_DONE;
                const uint2 e = stack[--s.sp];
                if (!DIRECT && e.x == kBlasSentinel) {  // back to the TLAS
                    const uint2 inv = stack[--s.sp];
                    const uint2 pend = stack[--s.sp];
                    s.ng = stack[--s.sp];
                    s.pbase = pend.x;
                    s.pbits = pend.y;
                    s.cur_inst = -1;
                    s.cur = make_tray(s.wo, s.wd, __uint_as_float(inv.x), __uint_as_float(inv.y),
                                      __uint_as_float(e.y));
                    return TRAV_RUNNING;
                }
                if (e.y <= 0x00ffffffu) {  // a postponed triangle group
                    s.pbase = e.x;
                    s.pbits = e.y;
                    s.ng = make_uint2(0, 0);
                    return TRAV_RUNNING;
                }
                s.ng = e;  // a node group (always holds internal children)
            }
            const uint32_t bit = 31u - __clz(s.ng.y);
            const uint32_t slot = (bit - 24u) ^ s.cur.oct_inv;
            const uint32_t rel = __popc(s.ng.y & ~(0xffffffffu << slot));
            s.next = (int)(s.ng.x + rel);
            s.ng.y &= ~(1u << bit);
            if (s.ng.y > 0x00ffffffu) trav_push(P, stack, s.sp, s.ng);
        }
        uint32_t cb, pb, im;
        const uint32_t hm = intersect_node<PACKED>(P.nodes, P.node_words, s.next, s.cur, s.tmax, cb, pb, im);
        s.next = -1;
        s.ng = make_uint2(cb, (hm & 0xff000000u) | im);
        s.pbase = pb;
        s.pbits = hm & 0x00ffffffu;
        if (s.pbits) return TRAV_RUNNING;  // the next step tests a triangle (or enters an instance)
        if (s.ng.y <= 0x00ffffffu) return TRAV_RUNNING;  // nothing below: the next step pops
        // the next step intersects the nearest child.  (Prefetching it, or the
        // next triangle, into L1 cost more instructions than it saved: the
        // BVH stays in L2, 2.6% on C2.)
        if (q + 1 == kNodesPerStep || mode == TRAV_LANE) return TRAV_RUNNING;
    }
    return TRAV_RUNNING;
}

// The warp's step mode: triangle steps when at least `min_tris` of its
// tracing lanes have triangles pending, or when no lane has a node to go to.
__device__ __forceinline__ int trav_warp_mode(const Trav& s, bool tracing, int min_tris) {
    const unsigned tri = __ballot_sync(0xffffffffu, tracing && trav_has_tris(s));
    const unsigned desc = __ballot_sync(0xffffffffu, tracing && trav_can_descend(s));
    return (__popc(tri) >= min_tris || desc == 0) ? TRAV_TRIS : TRAV_NODES;
}

// Closest triangle hit along (o, d) closer than tmax: fills s.prim (-1 if
// none), s.tmax, barycentrics, instance and material.
__device__ __forceinline__ void trace_closest(Trav& s, const Params& P, V3 o, V3 d, float tmax, uint2* stack) {
    trav_init(s, P, o, d, tmax);
    while (trav_step<false, false>(s, P, stack, nullptr) == TRAV_RUNNING) {
    }
}

// True if a triangle lies at 0 <= t < maxDist (and passes the alpha test
// when `alpha`).
static __device__ __noinline__ bool trace_any(const Params& P, V3 o, V3 d, float maxDist, bool alpha, Rng& rng,
                                              uint2* stack) {
    Trav s;
    trav_init(s, P, o, d, maxDist);
    if (alpha) {
        for (;;) {
            const int st = trav_step<true, true>(s, P, stack, &rng);
            if (st != TRAV_RUNNING) return st == TRAV_HIT;
        }
    }
    for (;;) {
        const int st = trav_step<true, false>(s, P, stack, nullptr);
        if (st != TRAV_RUNNING) return st == TRAV_HIT;
    }
}

}  // namespace ptgb
