// pt_trace.cuh - ray traversal of the 8-wide quantised BVH (bvh8.h).
//
// A node fetch is five 128-bit loads; the eight child boxes are slab-tested
// against the ray and the hits become a 32-bit mask: bits 24-31 internal
// children in octant order, bits 0-23 leaf primitives.  Node groups (child
// base, remaining hit bits | imask) go to a per-thread stack; leaf triangles
// are tested at once.  The triangle test repeats the reference's arithmetic
// operation for operation, without fused multiply-adds
// (closest_hit.glsl:128-143), so hit decisions and distances equal the
// oracle's bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pt_cuda.h"
#include "pt_device.cuh"
#include "pt_params.h"

namespace ptgb {

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
    const uint32_t oct = (r.nx ? 1u : 0u) | (r.ny ? 2u : 0u) | (r.nz ? 4u : 0u);
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
__device__ __noinline__ void traverse_closest(const Params& P, int root, const TRay& r, TriHit& h, uint2* stack,
                                              int sp, int inst, int mat) {
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
                const TRay ro = ir.w ? r : prep_ray(xform_point(P.xf, ir.y, r.o, 1.0f), xform_point(P.xf, ir.y, r.d, 0.0f));
                traverse_closest<false>(P, ir.x, ro, h, stack, sp, ir.y, ir.z);
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
__device__ __noinline__ bool traverse_any(const Params& P, int root, const TRay& r, float maxDist, uint2* stack,
                                          int sp, int mat, bool alpha, Rng& rng) {
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
                const TRay ro = ir.w ? r : prep_ray(xform_point(P.xf, ir.y, r.o, 1.0f), xform_point(P.xf, ir.y, r.d, 0.0f));
                if (traverse_any<false>(P, ir.x, ro, maxDist, stack, sp, ir.z, alpha, rng)) return true;
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

}  // namespace ptgb
