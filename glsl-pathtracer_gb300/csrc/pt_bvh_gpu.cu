// pt_bvh_gpu.cu - the acceleration structure built on the GPU, replacing the
// host build of the reference (RadeonRays SBVH per mesh and the TLAS over
// instances, src/core/Scene.cpp:148-214 with thirdparty/RadeonRays/
// split_bvh.cpp:32-218) and the host collapse of bvh8_build.cpp.
//
// The output has the layout of bvh8.h and the same structure as the host
// collapse: untransformed instances merged into one BLAS whose triangles
// carry their instance and material, one BLAS per mesh used by transformed
// instances, and a TLAS over those.
//
//   1. primitive references: (triangle, instance, material, group) -- group 0
//      the merged BLAS, then one group per mesh with transformed instances;
//   2. keys = group << 32 | 30-bit Morton code of the centroid in its group's
//      centroid bounds, radix-sorted (CUB);
//   3. the binary radix tree over the sorted keys (Karras, "Maximizing
//      Parallelism in the Construction of BVHs, Octrees, and k-d Trees",
//      HPG 2012): keys of different groups share fewer than 32 leading bits,
//      so every group is one subtree;
//   4. node boxes bottom-up, the second child to arrive at a node joining
//      the boxes, then the SAH dynamic program of the host collapse the
//      same way (k_dp);
//   5. the 8-wide collapse top-down, one launch per level: each wide node
//      takes the up to eight binary descendants the program chose; ranges
//      of at most 3 triangles become leaf slots; children are placed in
//      octant order and quantised conservatively (directed rounding);
//   6. the TLAS the same way over the merged BLAS and the transformed
//      instances' boxes.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include <cub/device/device_radix_sort.cuh>

#include "bvh8.h"
#include "pt_bvh_gpu.h"

namespace ptgb {
namespace {

constexpr int kMergedInstanceId = 0x7fffffff;  // InstRef.instance of the merged BLAS (bvh8_build.cpp)

struct Ref {  // a primitive reference of the build
    float lo[3], hi[3];
    int payload;  // triangle index (BLAS) or TLAS item
    int inst, mat;
};

__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}
__device__ __forceinline__ uint32_t morton30(float x, float y, float z) {
    x = fminf(fmaxf(x * 1024.0f, 0.0f), 1023.0f);
    y = fminf(fmaxf(y * 1024.0f, 0.0f), 1023.0f);
    z = fminf(fmaxf(z * 1024.0f, 0.0f), 1023.0f);
    return expand_bits((uint32_t)x) * 4 + expand_bits((uint32_t)y) * 2 + expand_bits((uint32_t)z);
}

// float <-> order-preserving uint, for atomic min / max on floats
__device__ __forceinline__ uint32_t f2o(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__global__ void k_tri_refs(const float4* __restrict__ verts, const int* __restrict__ vidx, const int* __restrict__ tri,
                           const int* __restrict__ inst, const int* __restrict__ mat, const int* __restrict__ group,
                           int n, Ref* refs, int* ref_group, uint32_t* gbounds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int t = tri[i];
    const float4 a = __ldg(verts + vidx[3 * t]), b = __ldg(verts + vidx[3 * t + 1]), c = __ldg(verts + vidx[3 * t + 2]);
    Ref r;
    r.lo[0] = fminf(a.x, fminf(b.x, c.x));
    r.lo[1] = fminf(a.y, fminf(b.y, c.y));
    r.lo[2] = fminf(a.z, fminf(b.z, c.z));
    r.hi[0] = fmaxf(a.x, fmaxf(b.x, c.x));
    r.hi[1] = fmaxf(a.y, fmaxf(b.y, c.y));
    r.hi[2] = fmaxf(a.z, fmaxf(b.z, c.z));
    r.payload = t;
    r.inst = inst[i];
    r.mat = mat[i];
    refs[i] = r;
    const int g = group[i];
    ref_group[i] = g;
    for (int k = 0; k < 3; ++k) {
        const float cen = 0.5f * (r.lo[k] + r.hi[k]);
        atomicMin(gbounds + 6 * g + k, f2o(cen));
        atomicMax(gbounds + 6 * g + 3 + k, f2o(cen));
    }
}

__global__ void k_box_refs(const float* __restrict__ boxes, int n, Ref* refs, int* ref_group, uint32_t* gbounds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Ref r;
    for (int k = 0; k < 3; ++k) {
        r.lo[k] = boxes[6 * i + k];
        r.hi[k] = boxes[6 * i + 3 + k];
    }
    r.payload = i;
    r.inst = r.mat = 0;
    refs[i] = r;
    ref_group[i] = 0;
    for (int k = 0; k < 3; ++k) {
        const float cen = 0.5f * (r.lo[k] + r.hi[k]);
        atomicMin(gbounds + k, f2o(cen));
        atomicMax(gbounds + 3 + k, f2o(cen));
    }
}

__global__ void k_keys(const Ref* __restrict__ refs, const int* __restrict__ ref_group,
                       const uint32_t* __restrict__ gbounds, int n, unsigned long long* keys, int* idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int g = ref_group[i];
    float c[3];
    for (int k = 0; k < 3; ++k) {
        const float lo = o2f(gbounds[6 * g + k]), hi = o2f(gbounds[6 * g + 3 + k]);
        const float cen = 0.5f * (refs[i].lo[k] + refs[i].hi[k]);
        c[k] = hi > lo ? (cen - lo) / (hi - lo) : 0.5f;
    }
    keys[i] = ((unsigned long long)g << 32) | morton30(c[0], c[1], c[2]);
    idx[i] = i;
}

// length of the common prefix of keys i and j (index tie-break), -1 outside
__device__ __forceinline__ int delta(const unsigned long long* __restrict__ k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const unsigned long long a = k[i], b = k[j];
    if (a == b) return 64 + __clz((uint32_t)(i ^ j));
    return __clzll(a ^ b);
}

// Binary node: children (>= 0 internal node, < 0: ~leaf index) and the range
// of sorted references it covers.  Parents are kept apart (node_parent,
// leaf_parent), each written only by the parent's thread.
struct BinNode {
    int left, right, first, last;
};

__global__ void k_radix_tree(const unsigned long long* __restrict__ keys, int n, BinNode* nodes, int* node_parent,
                             int* leaf_parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int s = 0;
    for (int t = (l + 1) / 2;; t = (t + 1) / 2) {
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
        if (t == 1) break;
    }
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    BinNode nd;
    nd.first = lo;
    nd.last = hi;
    nd.left = (lo == gamma) ? ~gamma : gamma;
    nd.right = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    nodes[i] = nd;
    if (lo == gamma) leaf_parent[gamma] = i;
    else node_parent[gamma] = i;
    if (hi == gamma + 1) leaf_parent[gamma + 1] = i;
    else node_parent[gamma + 1] = i;
}

// Node boxes bottom-up: the second of the two children to finish a node
// computes it (atomic counter per node).
__global__ void k_boxes(const Ref* __restrict__ refs, const int* __restrict__ order, const BinNode* __restrict__ nodes,
                        const int* __restrict__ node_parent, const int* __restrict__ leaf_parent, int n, float* boxes,
                        int* counters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int p = leaf_parent[i];
    while (p >= 0) {
        __threadfence();
        if (atomicAdd(counters + p, 1) == 0) return;  // the other child is not done yet
        __threadfence();
        const BinNode nd = nodes[p];
        float lo[3], hi[3];
        for (int k = 0; k < 3; ++k) { lo[k] = INFINITY; hi[k] = -INFINITY; }
        const int ch[2] = {nd.left, nd.right};
        for (int c = 0; c < 2; ++c) {
            if (ch[c] < 0) {
                const Ref& r = refs[order[~ch[c]]];
                for (int k = 0; k < 3; ++k) { lo[k] = fminf(lo[k], r.lo[k]); hi[k] = fmaxf(hi[k], r.hi[k]); }
            } else {
                const volatile float* b = boxes + 6 * ch[c];
                for (int k = 0; k < 3; ++k) { lo[k] = fminf(lo[k], b[k]); hi[k] = fmaxf(hi[k], b[3 + k]); }
            }
        }
        for (int k = 0; k < 3; ++k) {
            boxes[6 * p + k] = lo[k];
            boxes[6 * p + 3 + k] = hi[k];
        }
        p = node_parent[p];
    }
}

// SAH dynamic program over the binary tree (the host collapse's, bvh8_build.cpp,
// after Ylitie, Karras and Laine, HPG 2017): c[i] is the least cost of a
// node's subtree as at most i children of the wide node above, k[i] the
// children given to its left subtree (0: c[i] = c[i-1]).  Leaves of at most
// three references cost A * kCostPrim * refs, internal children
// A * kCostNode + the best eight-way distribution.  Bottom-up like k_boxes.
constexpr float kCostNode = 1.0f, kCostPrim = 0.3f;

struct Dp {
    float c[9];
    int8_t k[9];
    int np;
};

__device__ __forceinline__ float box_area(const float* lo, const float* hi) {
    const float dx = fmaxf(0.0f, hi[0] - lo[0]), dy = fmaxf(0.0f, hi[1] - lo[1]), dz = fmaxf(0.0f, hi[2] - lo[2]);
    return dx * dy + dy * dz + dz * dx;
}

__global__ void k_dp(const Ref* __restrict__ refs, const int* __restrict__ order, const BinNode* __restrict__ nodes,
                     const int* __restrict__ node_parent, const int* __restrict__ leaf_parent,
                     const float* __restrict__ boxes, int n, Dp* dp, int* counters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int p = leaf_parent[i];
    while (p >= 0) {
        __threadfence();
        if (atomicAdd(counters + p, 1) == 0) return;  // the other child is not done yet
        __threadfence();
        const BinNode nd = nodes[p];
        float cl[2][9];
        int np = 0;
        const int ch[2] = {nd.left, nd.right};
        for (int c = 0; c < 2; ++c) {
            if (ch[c] < 0) {  // one reference: a leaf child
                const Ref& r = refs[order[~ch[c]]];
                const float v = box_area(r.lo, r.hi) * kCostPrim;
                for (int q = 1; q <= 8; ++q) cl[c][q] = v;
                np += 1;
            } else {
                const volatile Dp* d = dp + ch[c];
                for (int q = 1; q <= 8; ++q) cl[c][q] = d->c[q];
                np += d->np;
            }
        }
        const float A = box_area(boxes + 6 * p, boxes + 6 * p + 3);
        float D[9];
        int8_t K[9];
        for (int q = 2; q <= 8; ++q) {
            D[q] = INFINITY;
            K[q] = 1;
            for (int j = 1; j < q; ++j) {
                const float v = cl[0][j] + cl[1][q - j];
                if (v < D[q]) { D[q] = v; K[q] = (int8_t)j; }
            }
        }
        Dp out;
        out.np = np;
        const float cleaf = np <= 3 ? A * kCostPrim * (float)np : INFINITY;
        const float cnode = A * kCostNode + D[8];
        out.c[0] = 0.0f;
        out.k[0] = out.k[1] = 0;
        out.c[1] = fminf(cleaf, cnode);
        for (int q = 2; q <= 8; ++q) {
            if (D[q] < out.c[q - 1]) { out.c[q] = D[q]; out.k[q] = K[q]; }
            else { out.c[q] = out.c[q - 1]; out.k[q] = 0; }
        }
        out.k[0] = K[8];  // the split of the best eight-way distribution (the wide node made of p)
        volatile Dp* o = dp + p;
        for (int q = 0; q <= 8; ++q) { o->c[q] = out.c[q]; o->k[q] = out.k[q]; }
        o->np = out.np;
        p = node_parent[p];
    }
}

// ------------------------------------------------------------- collapse
struct Task {
    int bin;          // binary internal node, or -1 for a reference range
    int first, count; // reference range (bin < 0)
    int wide;         // wide node to write
};

struct CollapseArgs {
    const Ref* refs;
    const int* order;      // sorted position -> reference
    const BinNode* nodes;
    const float* boxes;    // binary node boxes
    const Dp* dp;          // the SAH program (k_dp)
    const float4* verts;
    const int* vidx;
    WideNode* wide;
    WideTri* tris;         // BLAS payload
    InstRef* insts;        // TLAS payload
    const int* tlas_blas_root;  // TLAS: item -> wide BLAS root
    const int* tlas_instance;   // TLAS: item -> instance id
    const int* tlas_material;
    const int* tlas_identity;
    int tlas;
    int* counters;         // [0] wide nodes, [1] payload slots, [2] next tasks
    int max_nodes, max_payload;
    int* error;
};

struct Kid {
    float lo[3], hi[3];
    int bin;           // internal binary node, or -1 (reference range)
    int first, count;  // reference range
};

__device__ __forceinline__ float area(const Kid& k) {
    const float dx = fmaxf(0.0f, k.hi[0] - k.lo[0]), dy = fmaxf(0.0f, k.hi[1] - k.lo[1]),
                dz = fmaxf(0.0f, k.hi[2] - k.lo[2]);
    return dx * dy + dy * dz + dz * dx;
}

__device__ __forceinline__ void kid_of_node(const CollapseArgs& A, int child, Kid& k) {
    if (child < 0) {  // a leaf: one reference
        const Ref& r = A.refs[A.order[~child]];
        for (int c = 0; c < 3; ++c) { k.lo[c] = r.lo[c]; k.hi[c] = r.hi[c]; }
        k.bin = -1;
        k.first = ~child;
        k.count = 1;
        return;
    }
    const BinNode nd = A.nodes[child];
    for (int c = 0; c < 3; ++c) { k.lo[c] = A.boxes[6 * child + c]; k.hi[c] = A.boxes[6 * child + 3 + c]; }
    if (nd.last - nd.first + 1 <= 3) {  // small subtree: a leaf range
        k.bin = -1;
        k.first = nd.first;
        k.count = nd.last - nd.first + 1;
    } else {
        k.bin = child;
        k.first = nd.first;
        k.count = nd.last - nd.first + 1;
    }
}

__device__ __forceinline__ void range_box(const CollapseArgs& A, int first, int count, Kid& k) {
    for (int c = 0; c < 3; ++c) { k.lo[c] = INFINITY; k.hi[c] = -INFINITY; }
    for (int i = first; i < first + count; ++i) {
        const Ref& r = A.refs[A.order[i]];
        for (int c = 0; c < 3; ++c) { k.lo[c] = fminf(k.lo[c], r.lo[c]); k.hi[c] = fmaxf(k.hi[c], r.hi[c]); }
    }
}

__global__ void k_collapse(CollapseArgs A, const Task* __restrict__ tasks, int ntasks, Task* next) {
    const int ti = blockIdx.x * blockDim.x + threadIdx.x;
    if (ti >= ntasks) return;
    const Task task = tasks[ti];
    Kid kids[8];
    int nk = 0;
    if (task.bin >= 0) {
        // the children the SAH program chose: (node, slots) pairs split by
        // k[] down to single children (at most 8, so at most 9 on the stack)
        const BinNode nd = A.nodes[task.bin];
        const int k8 = A.dp[task.bin].k[0];
        int st_node[16], st_i[16], sp = 0;
        st_node[sp] = nd.right; st_i[sp++] = 8 - k8;
        st_node[sp] = nd.left; st_i[sp++] = k8;
        while (sp > 0) {
            const int node = st_node[--sp];
            int q = st_i[sp];
            if (node >= 0) {
                const Dp& d = A.dp[node];
                while (q > 1 && d.k[q] == 0) --q;
                if (q > 1) {
                    if (sp + 2 > 16) { atomicExch(A.error, 1); return; }
                    const BinNode cn = A.nodes[node];
                    st_node[sp] = cn.right; st_i[sp++] = q - d.k[q];
                    st_node[sp] = cn.left; st_i[sp++] = d.k[q];
                    continue;
                }
            }
            if (nk >= 8) { atomicExch(A.error, 1); return; }
            kid_of_node(A, node, kids[nk++]);
        }
    } else {
        // a range of more than 3 references: up to 8 pieces of <= 3 (as the host collapse)
        const int pieces = min(8, (task.count + 2) / 3);
        const int per = (task.count + pieces - 1) / pieces;
        for (int f = task.first; f < task.first + task.count; f += per) {
            Kid& k = kids[nk++];
            k.bin = -1;
            k.first = f;
            k.count = min(per, task.first + task.count - f);
            range_box(A, k.first, k.count, k);
        }
    }
    // node box and octant slots (greedy best direction score)
    float nlo[3], nhi[3];
    for (int c = 0; c < 3; ++c) { nlo[c] = INFINITY; nhi[c] = -INFINITY; }
    for (int i = 0; i < nk; ++i)
        for (int c = 0; c < 3; ++c) { nlo[c] = fminf(nlo[c], kids[i].lo[c]); nhi[c] = fmaxf(nhi[c], kids[i].hi[c]); }
    int slot_of[8];
    {
        float cen[3];
        for (int c = 0; c < 3; ++c) cen[c] = 0.5f * (nlo[c] + nhi[c]);
        bool used_child[8] = {false, false, false, false, false, false, false, false};
        bool used_slot[8] = {false, false, false, false, false, false, false, false};
        for (int round = 0; round < nk; ++round) {
            float best = -INFINITY;
            int bi = -1, bs = -1;
            for (int i = 0; i < nk; ++i) {
                if (used_child[i]) continue;
                float d[3];
                for (int c = 0; c < 3; ++c) d[c] = 0.5f * (kids[i].lo[c] + kids[i].hi[c]) - cen[c];
                for (int s = 0; s < 8; ++s) {
                    if (used_slot[s]) continue;
                    const float v = ((s & 1) ? d[0] : -d[0]) + ((s & 2) ? d[1] : -d[1]) + ((s & 4) ? d[2] : -d[2]);
                    if (v > best || bi < 0) { best = v; bi = i; bs = s; }
                }
            }
            used_child[bi] = used_slot[bs] = true;
            slot_of[bi] = bs;
        }
    }
    int by_slot[8];
    for (int s = 0; s < 8; ++s) by_slot[s] = -1;
    for (int i = 0; i < nk; ++i) by_slot[slot_of[i]] = i;
    int num_internal = 0, num_prims = 0, imask = 0;
    for (int s = 0; s < 8; ++s) {
        const int i = by_slot[s];
        if (i < 0) continue;
        if (kids[i].bin >= 0 || kids[i].count > 3) {
            ++num_internal;
            imask |= 1 << s;
        } else {
            num_prims += kids[i].count;
        }
    }
    const int child_base = num_internal ? atomicAdd(A.counters + 0, num_internal) : 0;
    const int prim_base = num_prims ? atomicAdd(A.counters + 1, num_prims) : 0;
    if (child_base + num_internal > A.max_nodes || prim_base + num_prims > A.max_payload || num_prims > 24) {
        atomicExch(A.error, 1);
        return;
    }
    // quantisation: 8-bit child boxes on the node's frame, rounded outward
    int ex[3];
    float scale[3], inv[3];
    for (int c = 0; c < 3; ++c) {
        const float range = __fsub_ru(nhi[c], nlo[c]);
        int e;
        if (!(range > 0.0f)) {
            e = -126;
        } else {
            int k;
            const float m = frexpf(__fdiv_ru(range, 255.0f), &k);  // range / 255 = m 2^k, m in [0.5, 1)
            e = (m == 0.5f) ? k - 1 : k;
            while (ldexpf(255.0f, e) < range) ++e;
            while (e > -126 && ldexpf(255.0f, e - 1) >= range) --e;
        }
        e = max(-126, min(127, e));
        ex[c] = e;
        scale[c] = ldexpf(1.0f, e);
        inv[c] = ldexpf(1.0f, -e);
    }
    uint32_t w[20];
    for (int k = 0; k < 20; ++k) w[k] = 0;
    w[0] = __float_as_uint(nlo[0]);
    w[1] = __float_as_uint(nlo[1]);
    w[2] = __float_as_uint(nlo[2]);
    w[3] = uint32_t(ex[0] + 127) | (uint32_t(ex[1] + 127) << 8) | (uint32_t(ex[2] + 127) << 16) |
           (uint32_t(imask) << 24);
    w[4] = uint32_t(child_base);
    w[5] = uint32_t(prim_base);
    uint8_t meta[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint8_t* q = reinterpret_cast<uint8_t*>(&w[8]);
    int ji = 0, prim_off = 0;
    int ntask_local = 0;
    Task child_tasks[8];
    for (int s = 0; s < 8; ++s) {
        const int i = by_slot[s];
        if (i < 0) continue;
        const Kid& k = kids[i];
        for (int c = 0; c < 3; ++c) {
            float lo = floorf(__fsub_rd(k.lo[c], nlo[c]) * inv[c]);
            float hi = ceilf(__fsub_ru(k.hi[c], nlo[c]) * inv[c]);
            lo = fminf(fmaxf(lo, 0.0f), 255.0f);
            hi = fminf(fmaxf(hi, 0.0f), 255.0f);
            q[c * 8 + s] = (uint8_t)lo;
            q[(3 + c) * 8 + s] = (uint8_t)hi;
        }
        if (k.bin >= 0 || k.count > 3) {
            meta[s] = uint8_t((1 << 5) | (24 + s));
            Task t;
            t.bin = k.bin;
            t.first = k.first;
            t.count = k.count;
            t.wide = child_base + ji++;
            child_tasks[ntask_local++] = t;
        } else {
            meta[s] = uint8_t((((1 << k.count) - 1) << 5) | prim_off);
            for (int r = 0; r < k.count; ++r) {
                const Ref& ref = A.refs[A.order[k.first + r]];
                const int slot = prim_base + prim_off + r;
                if (A.tlas) {
                    InstRef ir;
                    ir.blas_root = A.tlas_blas_root[ref.payload];
                    ir.instance = A.tlas_instance[ref.payload];
                    ir.material = A.tlas_material[ref.payload];
                    ir.identity = A.tlas_identity[ref.payload];
                    A.insts[slot] = ir;
                } else {
                    const int t = ref.payload;
                    const float4 a = __ldg(A.verts + A.vidx[3 * t]), b = __ldg(A.verts + A.vidx[3 * t + 1]),
                                 d = __ldg(A.verts + A.vidx[3 * t + 2]);
                    WideTri wt;
                    wt.v0[0] = a.x; wt.v0[1] = a.y; wt.v0[2] = a.z;
                    wt.prim = t;
                    wt.e0[0] = b.x - a.x; wt.e0[1] = b.y - a.y; wt.e0[2] = b.z - a.z;
                    wt.e1[0] = d.x - a.x; wt.e1[1] = d.y - a.y; wt.e1[2] = d.z - a.z;
                    wt.e0[3] = __int_as_float(ref.inst);
                    wt.e1[3] = __int_as_float(ref.mat);
                    A.tris[slot] = wt;
                }
            }
            prim_off += k.count;
        }
    }
    w[6] = meta[0] | (meta[1] << 8) | (meta[2] << 16) | (uint32_t(meta[3]) << 24);
    w[7] = meta[4] | (meta[5] << 8) | (meta[6] << 16) | (uint32_t(meta[7]) << 24);
    WideNode& out = A.wide[task.wide];
    for (int k = 0; k < 20; ++k) out.w[k] = w[k];
    if (ntask_local) {
        const int base = atomicAdd(A.counters + 2, ntask_local);
        for (int k = 0; k < ntask_local; ++k) next[base + k] = child_tasks[k];
    }
}

template <class T> cudaError_t dalloc(T*& p, size_t n) {
    p = nullptr;
    return n ? cudaMalloc((void**)&p, n * sizeof(T)) : cudaSuccess;
}
template <class T> void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

#define GB_CK(call)                                                  \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) {                                     \
            err = std::string(#call) + ": " + cudaGetErrorString(e_); \
            return e_;                                               \
        }                                                            \
    } while (0)

// One build pass (BLAS groups or the TLAS) over prepared references.
struct Pass {
    Ref* refs = nullptr;
    int* ref_group = nullptr;
    uint32_t* gbounds = nullptr;
    unsigned long long* keys = nullptr;
    unsigned long long* keys2 = nullptr;
    int* idx = nullptr;
    int* order = nullptr;
    BinNode* nodes = nullptr;
    int* node_parent = nullptr;
    int* leaf_parent = nullptr;
    float* boxes = nullptr;
    int* counters = nullptr;
    Dp* dp = nullptr;
    void* temp = nullptr;
    void release() {
        dfree(refs); dfree(ref_group); dfree(gbounds); dfree(keys); dfree(keys2); dfree(idx); dfree(order);
        dfree(nodes); dfree(node_parent); dfree(leaf_parent); dfree(boxes); dfree(counters); dfree(dp);
        if (temp) cudaFree(temp);
        temp = nullptr;
    }
};

// Sort the references, build the radix tree and its boxes; returns per
// group the root task (binary node covering the group, or its range).
cudaError_t tree(Pass& ps, int n, int num_groups, cudaStream_t s, std::vector<Task>& roots, std::string& err) {
    const int B = 256;
    GB_CK(dalloc(ps.keys, n));
    GB_CK(dalloc(ps.keys2, n));
    GB_CK(dalloc(ps.idx, n));
    GB_CK(dalloc(ps.order, n));
    k_keys<<<(n + B - 1) / B, B, 0, s>>>(ps.refs, ps.ref_group, ps.gbounds, n, ps.keys, ps.idx);
    GB_CK(cudaGetLastError());
    size_t tbytes = 0;
    GB_CK(cub::DeviceRadixSort::SortPairs(nullptr, tbytes, ps.keys, ps.keys2, ps.idx, ps.order, n, 0, 64, s));
    GB_CK(cudaMalloc(&ps.temp, tbytes));
    GB_CK(cub::DeviceRadixSort::SortPairs(ps.temp, tbytes, ps.keys, ps.keys2, ps.idx, ps.order, n, 0, 64, s));
    const int ni = std::max(n - 1, 1);
    GB_CK(dalloc(ps.nodes, ni));
    GB_CK(dalloc(ps.node_parent, ni));
    GB_CK(dalloc(ps.leaf_parent, n));
    GB_CK(cudaMemsetAsync(ps.node_parent, 0xff, sizeof(int) * ni, s));
    GB_CK(dalloc(ps.boxes, 6 * (size_t)ni));
    GB_CK(dalloc(ps.counters, ni));
    GB_CK(cudaMemsetAsync(ps.counters, 0, sizeof(int) * ni, s));
    GB_CK(cudaMemsetAsync(ps.leaf_parent, 0xff, sizeof(int) * n, s));
    if (n > 1) {
        k_radix_tree<<<(n - 1 + B - 1) / B, B, 0, s>>>(ps.keys2, n, ps.nodes, ps.node_parent, ps.leaf_parent);
        GB_CK(cudaGetLastError());
        k_boxes<<<(n + B - 1) / B, B, 0, s>>>(ps.refs, ps.order, ps.nodes, ps.node_parent, ps.leaf_parent, n,
                                              ps.boxes, ps.counters);
        GB_CK(cudaGetLastError());
        GB_CK(dalloc(ps.dp, ni));
        GB_CK(cudaMemsetAsync(ps.counters, 0, sizeof(int) * ni, s));
        k_dp<<<(n + B - 1) / B, B, 0, s>>>(ps.refs, ps.order, ps.nodes, ps.node_parent, ps.leaf_parent, ps.boxes, n,
                                           ps.dp, ps.counters);
        GB_CK(cudaGetLastError());
    }
    // group ranges from the sorted keys, and the node covering each
    std::vector<unsigned long long> hk(n);
    GB_CK(cudaMemcpyAsync(hk.data(), ps.keys2, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost, s));
    std::vector<BinNode> hn(n > 1 ? n - 1 : 0);
    if (n > 1) GB_CK(cudaMemcpyAsync(hn.data(), ps.nodes, sizeof(BinNode) * (n - 1), cudaMemcpyDeviceToHost, s));
    GB_CK(cudaStreamSynchronize(s));
    std::vector<int> gfirst(num_groups, -1), glast(num_groups, -1);
    for (int i = 0; i < n; ++i) {
        const int g = (int)(hk[i] >> 32);
        if (gfirst[g] < 0) gfirst[g] = i;
        glast[g] = i;
    }
    std::vector<int> node_of(num_groups, -1);
    for (int i = 0; i + 1 < n; ++i) {
        const int g = (int)(hk[hn[i].first] >> 32);
        if (hn[i].first == gfirst[g] && hn[i].last == glast[g]) node_of[g] = i;
    }
    roots.assign(num_groups, Task{});
    for (int g = 0; g < num_groups; ++g) {
        if (gfirst[g] < 0) {
            err = "empty group in the GPU BVH build";
            return cudaErrorInvalidValue;
        }
        const int cnt = glast[g] - gfirst[g] + 1;
        Task t;
        t.first = gfirst[g];
        t.count = cnt;
        t.wide = -1;
        if (cnt > 3) {
            if (node_of[g] < 0) {
                err = "group subtree not found in the radix tree";
                return cudaErrorInvalidValue;
            }
            t.bin = node_of[g];
        } else {
            t.bin = -1;
        }
        roots[g] = t;
    }
    return cudaSuccess;
}

// Collapse from the given root tasks, wide nodes from index node_base on
// (children are addressed absolutely); returns the number of levels.
cudaError_t collapse(CollapseArgs A, std::vector<Task>& roots, int* root_wide, int* counters_dev, int* error_dev,
                     cudaStream_t s, int& levels, std::string& err, int node_base) {
    // roots get consecutive wide nodes first
    int host_counts[3] = {node_base, 0, 0};
    for (size_t g = 0; g < roots.size(); ++g) roots[g].wide = host_counts[0]++;
    for (size_t g = 0; g < roots.size(); ++g) root_wide[g] = roots[g].wide;
    GB_CK(cudaMemcpyAsync(counters_dev, host_counts, sizeof(int) * 3, cudaMemcpyHostToDevice, s));
    GB_CK(cudaMemsetAsync(error_dev, 0, sizeof(int), s));
    A.counters = counters_dev;
    A.error = error_dev;
    Task *cur = nullptr, *next = nullptr;
    const size_t cap = (size_t)A.max_nodes + 8;
    GB_CK(dalloc(cur, cap));
    GB_CK(dalloc(next, cap));
    GB_CK(cudaMemcpyAsync(cur, roots.data(), sizeof(Task) * roots.size(), cudaMemcpyHostToDevice, s));
    int ntasks = (int)roots.size();
    levels = 0;
    cudaError_t e = cudaSuccess;
    while (ntasks > 0) {
        if (++levels > 200) {
            err = "GPU BVH deeper than 200 wide levels";
            e = cudaErrorInvalidValue;
            break;
        }
        if ((e = cudaMemsetAsync(counters_dev + 2, 0, sizeof(int), s)) != cudaSuccess) break;
        k_collapse<<<(ntasks + 127) / 128, 128, 0, s>>>(A, cur, ntasks, next);
        if ((e = cudaGetLastError()) != cudaSuccess) break;
        int hc[3], herr = 0;
        if ((e = cudaMemcpyAsync(hc, counters_dev, sizeof(hc), cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(&herr, error_dev, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess) break;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) break;
        if (herr) {
            err = "GPU BVH collapse ran out of its node or triangle budget";
            e = cudaErrorInvalidValue;
            break;
        }
        ntasks = hc[2];
        std::swap(cur, next);
    }
    dfree(cur);
    dfree(next);
    if (e != cudaSuccess && err.empty()) err = std::string("GPU BVH collapse: ") + cudaGetErrorString(e);
    return e;
}

__global__ void k_instance_boxes(const float* __restrict__ blas_box, const int* __restrict__ item_group,
                                 const float* __restrict__ xf, const int* __restrict__ item_inst, int n,
                                 float* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* b = blas_box + 6 * item_group[i];
    const int inst = item_inst[i];
    if (inst == kMergedInstanceId) {
        for (int k = 0; k < 6; ++k) out[6 * i + k] = b[k];
        return;
    }
    const float* x = xf + 16 * (size_t)inst;  // row-vector Mat4: p' = p.x row0 + p.y row1 + p.z row2 + row3
    for (int k = 0; k < 3; ++k) {
        double lo = x[12 + k], hi = x[12 + k];
        for (int a = 0; a < 3; ++a) {
            const double e0 = (double)x[4 * a + k] * b[a], e1 = (double)x[4 * a + k] * b[3 + a];
            lo += fmin(e0, e1);
            hi += fmax(e0, e1);
        }
        out[6 * i + k] = __double2float_rd(lo);
        out[6 * i + 3 + k] = __double2float_ru(hi);
    }
}

// Bounding box of each BLAS (its root wide node's children boxes are inside
// the root's quantisation frame): the union of the group's references.
__global__ void k_group_boxes(const Ref* __restrict__ refs, const int* __restrict__ ref_group, int n, uint32_t* gb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int g = ref_group[i];
    for (int k = 0; k < 3; ++k) {
        atomicMin(gb + 6 * g + k, f2o(refs[i].lo[k]));
        atomicMax(gb + 6 * g + 3 + k, f2o(refs[i].hi[k]));
    }
}
__global__ void k_decode_boxes(const uint32_t* __restrict__ gb, int n, float* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 6 * n) out[i] = o2f(gb[i]);
}

}  // namespace

void GpuBvh::release() {
    if (nodes) cudaFree(nodes);
    if (tris) cudaFree(tris);
    if (insts) cudaFree(insts);
    nodes = nullptr;
    tris = nullptr;
    insts = nullptr;
    num_nodes = num_tris = num_insts = 0;
}

cudaError_t gpu_build_bvh(const GpuBuildInput& in, GpuBvh& out, cudaStream_t s, std::string& err) {
    out.release();
    // identity instances -> group 0 (merged), other instances -> group per mesh
    std::vector<int> ident(in.num_instances, 0);
    for (int i = 0; i < in.num_instances; ++i) {
        InstXf xf;
        ptgb_instance_xf(in.transforms + 16 * (size_t)i, &xf, &ident[i]);
    }
    int num_ident = 0;
    for (int v : ident) num_ident += v;
    const bool merge = num_ident >= 2;
    std::vector<int> mesh_group(in.num_meshes, -1);
    int groups = merge ? 1 : 0;
    for (int i = 0; i < in.num_instances; ++i) {
        const int m = in.inst_mesh[i];
        if (m < 0 || m >= in.num_meshes) {
            err = "instance mesh index out of range";
            return cudaErrorInvalidValue;
        }
        if (merge && ident[i]) continue;
        if (mesh_group[m] < 0) mesh_group[m] = groups++;
    }
    std::vector<int> rtri, rinst, rmat, rgroup;
    for (int i = 0; merge && i < in.num_instances; ++i) {
        if (!ident[i]) continue;
        const int m = in.inst_mesh[i];
        for (int t = in.mesh_tri_offset[m]; t < in.mesh_tri_offset[m + 1]; ++t) {
            rtri.push_back(t);
            rinst.push_back(i);
            rmat.push_back(in.inst_material[i]);
            rgroup.push_back(0);
        }
    }
    for (int m = 0; m < in.num_meshes; ++m) {
        if (mesh_group[m] < 0) continue;
        for (int t = in.mesh_tri_offset[m]; t < in.mesh_tri_offset[m + 1]; ++t) {
            rtri.push_back(t);
            rinst.push_back(0);
            rmat.push_back(0);
            rgroup.push_back(mesh_group[m]);
        }
    }
    const int n = (int)rtri.size();
    if (n == 0 || groups == 0) {
        err = "no triangles to build";
        return cudaErrorInvalidValue;
    }
    for (int g = 0; g < groups; ++g) {
        bool found = false;
        for (int m = 0; m < in.num_meshes && !found; ++m) found = mesh_group[m] == g && in.mesh_tri_offset[m + 1] > in.mesh_tri_offset[m];
        if (g == 0 && merge) found = true;
        if (!found) {
            err = "a mesh with transformed instances has no triangles";
            return cudaErrorInvalidValue;
        }
    }
    const int B = 256;
    Pass ps;
    int *dtri = nullptr, *dinst = nullptr, *dmat = nullptr, *dgroup = nullptr, *dcnt = nullptr, *derr = nullptr;
    float* gbox = nullptr;
    uint32_t* gbu = nullptr;
    cudaError_t e = cudaSuccess;
    std::vector<Task> roots;
    std::vector<int> blas_root(groups);
    auto fail = [&](cudaError_t code) {
        ps.release();
        dfree(dtri); dfree(dinst); dfree(dmat); dfree(dgroup); dfree(dcnt); dfree(derr); dfree(gbox); dfree(gbu);
        out.release();
        return code;
    };
#define GB_TRY(call)                                                       \
    do {                                                                   \
        if ((e = (call)) != cudaSuccess) {                                 \
            if (err.empty()) err = std::string(#call) + ": " + cudaGetErrorString(e); \
            return fail(e);                                                \
        }                                                                  \
    } while (0)
    GB_TRY(dalloc(dtri, n));
    GB_TRY(dalloc(dinst, n));
    GB_TRY(dalloc(dmat, n));
    GB_TRY(dalloc(dgroup, n));
    GB_TRY(cudaMemcpyAsync(dtri, rtri.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    GB_TRY(cudaMemcpyAsync(dinst, rinst.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    GB_TRY(cudaMemcpyAsync(dmat, rmat.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    GB_TRY(cudaMemcpyAsync(dgroup, rgroup.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    GB_TRY(dalloc(ps.refs, n));
    GB_TRY(dalloc(ps.ref_group, n));
    GB_TRY(dalloc(ps.gbounds, 6 * (size_t)groups));
    {
        std::vector<uint32_t> init(6 * (size_t)groups);
        for (int g = 0; g < groups; ++g)
            for (int k = 0; k < 3; ++k) {
                init[6 * g + k] = 0xffffffffu;  // min starts at the top of the order
                init[6 * g + 3 + k] = 0u;
            }
        GB_TRY(cudaMemcpyAsync(ps.gbounds, init.data(), sizeof(uint32_t) * init.size(), cudaMemcpyHostToDevice, s));
        GB_TRY(dalloc(gbu, 6 * (size_t)groups));
        GB_TRY(cudaMemcpyAsync(gbu, init.data(), sizeof(uint32_t) * init.size(), cudaMemcpyHostToDevice, s));
        GB_TRY(cudaStreamSynchronize(s));  // init is freed at the end of this block
    }
    k_tri_refs<<<(n + B - 1) / B, B, 0, s>>>(in.verts, in.vidx, dtri, dinst, dmat, dgroup, n, ps.refs, ps.ref_group,
                                             ps.gbounds);
    GB_TRY(cudaGetLastError());
    k_group_boxes<<<(n + B - 1) / B, B, 0, s>>>(ps.refs, ps.ref_group, n, gbu);
    GB_TRY(cudaGetLastError());
    GB_TRY(dalloc(gbox, 6 * (size_t)groups));
    k_decode_boxes<<<(6 * groups + B - 1) / B, B, 0, s>>>(gbu, groups, gbox);
    GB_TRY(cudaGetLastError());
    if ((e = tree(ps, n, groups, s, roots, err)) != cudaSuccess) return fail(e);
    // budgets: at most n - 1 wide nodes per n references (each wide node
    // has >= 2 children), plus the TLAS
    const int max_blas_nodes = std::max(2 * n, 16);
    const int max_tlas_items = groups + in.num_instances;
    const int max_nodes = max_blas_nodes + 2 * max_tlas_items + 16;
    GB_TRY(dalloc(out.nodes, max_nodes));
    GB_TRY(dalloc(out.tris, n));
    GB_TRY(dalloc(out.insts, max_tlas_items));
    GB_TRY(dalloc(dcnt, 3));
    GB_TRY(dalloc(derr, 1));
    CollapseArgs A{};
    A.refs = ps.refs;
    A.order = ps.order;
    A.nodes = ps.nodes;
    A.boxes = ps.boxes;
    A.dp = ps.dp;
    A.verts = in.verts;
    A.vidx = in.vidx;
    A.wide = out.nodes;
    A.tris = out.tris;
    A.tlas = 0;
    A.max_nodes = max_blas_nodes;
    A.max_payload = n;
    int levels = 0;
    if ((e = collapse(A, roots, blas_root.data(), dcnt, derr, s, levels, err, 0)) != cudaSuccess) return fail(e);
    out.blas_depth = levels;
    int hc[3];
    GB_TRY(cudaMemcpyAsync(hc, dcnt, sizeof(hc), cudaMemcpyDeviceToHost, s));
    GB_TRY(cudaStreamSynchronize(s));
    const int blas_nodes = hc[0];
    out.num_tris = hc[1];
    ps.release();
    // ---- TLAS: the merged BLAS (once) and each transformed instance
    std::vector<int> item_group, item_inst, item_mat, item_ident, item_root;
    if (merge) {
        item_group.push_back(0);
        item_inst.push_back(kMergedInstanceId);
        item_mat.push_back(-1);
        item_ident.push_back(1);
        item_root.push_back(blas_root[0]);
    }
    for (int i = 0; i < in.num_instances; ++i) {
        if (merge && ident[i]) continue;
        const int g = mesh_group[in.inst_mesh[i]];
        item_group.push_back(g);
        item_inst.push_back(i);
        item_mat.push_back(in.inst_material[i]);
        item_ident.push_back(ident[i]);
        item_root.push_back(blas_root[g]);
    }
    const int ni = (int)item_group.size();
    int *d_ig = nullptr, *d_ii = nullptr, *d_im = nullptr, *d_id = nullptr, *d_ir = nullptr;
    float *d_xf = nullptr, *d_ibox = nullptr;
    auto fail2 = [&](cudaError_t code) {
        dfree(d_ig); dfree(d_ii); dfree(d_im); dfree(d_id); dfree(d_ir); dfree(d_xf); dfree(d_ibox);
        return fail(code);
    };
#undef GB_TRY
#define GB_TRY(call)                                                       \
    do {                                                                   \
        if ((e = (call)) != cudaSuccess) {                                 \
            if (err.empty()) err = std::string(#call) + ": " + cudaGetErrorString(e); \
            return fail2(e);                                               \
        }                                                                  \
    } while (0)
    GB_TRY(dalloc(d_ig, ni));
    GB_TRY(dalloc(d_ii, ni));
    GB_TRY(dalloc(d_im, ni));
    GB_TRY(dalloc(d_id, ni));
    GB_TRY(dalloc(d_ir, ni));
    GB_TRY(dalloc(d_xf, 16 * (size_t)std::max(1, in.num_instances)));
    GB_TRY(dalloc(d_ibox, 6 * (size_t)ni));
    GB_TRY(cudaMemcpyAsync(d_ig, item_group.data(), sizeof(int) * ni, cudaMemcpyHostToDevice, s));
    GB_TRY(cudaMemcpyAsync(d_ii, item_inst.data(), sizeof(int) * ni, cudaMemcpyHostToDevice, s));
    GB_TRY(cudaMemcpyAsync(d_im, item_mat.data(), sizeof(int) * ni, cudaMemcpyHostToDevice, s));
    GB_TRY(cudaMemcpyAsync(d_id, item_ident.data(), sizeof(int) * ni, cudaMemcpyHostToDevice, s));
    GB_TRY(cudaMemcpyAsync(d_ir, item_root.data(), sizeof(int) * ni, cudaMemcpyHostToDevice, s));
    GB_TRY(cudaMemcpyAsync(d_xf, in.transforms, sizeof(float) * 16 * in.num_instances, cudaMemcpyHostToDevice, s));
    k_instance_boxes<<<(ni + B - 1) / B, B, 0, s>>>(gbox, d_ig, d_xf, d_ii, ni, d_ibox);
    GB_TRY(cudaGetLastError());
    Pass pt;
    ps = pt;  // the BLAS pass was released; reuse the struct for the TLAS
    GB_TRY(dalloc(ps.refs, ni));
    GB_TRY(dalloc(ps.ref_group, ni));
    GB_TRY(dalloc(ps.gbounds, 6));
    {
        const uint32_t init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
        GB_TRY(cudaMemcpyAsync(ps.gbounds, init, sizeof(init), cudaMemcpyHostToDevice, s));
        GB_TRY(cudaStreamSynchronize(s));
    }
    k_box_refs<<<(ni + B - 1) / B, B, 0, s>>>(d_ibox, ni, ps.refs, ps.ref_group, ps.gbounds);
    GB_TRY(cudaGetLastError());
    std::vector<Task> troots;
    if ((e = tree(ps, ni, 1, s, troots, err)) != cudaSuccess) return fail2(e);
    CollapseArgs T{};
    T.refs = ps.refs;
    T.order = ps.order;
    T.nodes = ps.nodes;
    T.boxes = ps.boxes;
    T.dp = ps.dp;
    T.wide = out.nodes;
    T.insts = out.insts;
    T.tlas_blas_root = d_ir;
    T.tlas_instance = d_ii;
    T.tlas_material = d_im;
    T.tlas_identity = d_id;
    T.tlas = 1;
    T.max_nodes = max_nodes;
    T.max_payload = ni;
    int troot = 0;
    if ((e = collapse(T, troots, &troot, dcnt, derr, s, levels, err, blas_nodes)) != cudaSuccess) return fail2(e);
    GB_TRY(cudaMemcpyAsync(hc, dcnt, sizeof(hc), cudaMemcpyDeviceToHost, s));
    GB_TRY(cudaStreamSynchronize(s));
    out.tlas_depth = levels;
    out.tlas_first_node = blas_nodes;
    out.tlas_root = troot;
    out.num_nodes = hc[0];
    out.num_insts = hc[1];
    ps.release();
    dfree(d_ig); dfree(d_ii); dfree(d_im); dfree(d_id); dfree(d_ir); dfree(d_xf); dfree(d_ibox);
    dfree(dtri); dfree(dinst); dfree(dmat); dfree(dgroup); dfree(dcnt); dfree(derr); dfree(gbox); dfree(gbu);
#undef GB_TRY
    return cudaSuccess;
}

}  // namespace ptgb
