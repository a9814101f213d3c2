// bvh8.h - device layout of the acceleration structure.
//
// The reference uploads RadeonRays::BvhTranslator's binary node array
// (thirdparty/RadeonRays/bvh_translator.h:45-50, 36 B per node, fetched as
// three RGB32F texels per visit).  On GB300 the same tree is collapsed into
// 8-wide nodes with 8-bit quantised child boxes (80 B = five 16-byte words,
// one 128-bit load each), so that one node fetch replaces about three levels
// of the binary tree.  Leaf triangles are copied into leaf order as
// (v0, e0 = v1-v0, e1 = v2-v0) triples with the reference's triangle index in
// v0.w, so a leaf's triangles are contiguous in memory.
//
// Two levels as in the reference: the TLAS (over instances) and one BLAS per
// mesh.  A TLAS leaf child references an InstRef instead of triangles.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define PT_HD __host__ __device__
#else
#define PT_HD
#endif

namespace ptgb {

// 80-byte wide node (five 16-byte words).
//  w0: origin p.xyz (float bits), exps (e.x | e.y<<8 | e.z<<16 | imask<<24)
//  w1: child_base, prim_base, meta[0..3], meta[4..7]
//  w2: qlo_x[0..7], qlo_y[0..7]
//  w3: qlo_z[0..7], qhi_x[0..7]
//  w4: qhi_y[0..7], qhi_z[0..7]
// Child box of slot i: lo = p + qlo * 2^(e-127), hi = p + qhi * 2^(e-127).
// imask bit i: slot i is an internal child (stored at child_base + number of
// internal slots before i).  meta[i]: 0 = empty slot; internal child:
// 0b001_xxxxx with xxxxx = 24 + i; leaf child: unary primitive count (1, 3,
// 7 for 1..3) in the high three bits and the offset from prim_base in the low
// five bits.  Slot i holds the child whose centroid lies towards octant i of
// the node (bit k of i set: +k side), so a ray of octant o visits slots in
// the order of decreasing (slot ^ (7 - o)), nearest first.
struct alignas(16) WideNode {
    uint32_t w[20];
};
static_assert(sizeof(WideNode) == 80, "WideNode is 80 bytes");

// Triangle in leaf order: v0.xyz + primitive id (index into vert_indices) as
// int bits, e0 = v1 - v0, e1 = v2 - v0 (w unused).
struct alignas(16) WideTri {
    float v0[3];
    int32_t prim;
    float e0[4];
    float e1[4];
};
static_assert(sizeof(WideTri) == 48, "WideTri is 48 bytes");

// TLAS leaf primitive: the instance and the root of its BLAS.
struct alignas(16) InstRef {
    int32_t blas_root;   // index into the WideNode array
    int32_t instance;    // index into the instance arrays (-leaf-1 of the reference)
    int32_t material;    // materialID of the TLAS leaf (bvh_translator.cpp:68-77)
    int32_t identity;    // 1 if the transform is the identity (no ray transform needed)
};

// Per-instance matrices (GLSL column layout m[col][row] flattened):
// inverse of the 4x4 instance matrix, mat3(transform) and its inverse
// transpose (closest_hit.glsl:163-164,246,261-262).
struct alignas(16) InstXf {
    float inv[16];
    float m3[12];    // 3 columns padded to float4
    float nrm[12];   // 3 columns padded to float4
};

struct WideBVH {
    // host-side result of the collapse
    WideNode* nodes = nullptr;
    int32_t num_nodes = 0;
    WideTri* tris = nullptr;
    int32_t num_tris = 0;
    InstRef* insts = nullptr;
    int32_t num_inst_refs = 0;
    int32_t tlas_root = 0;       // wide index of the TLAS root
    int32_t tlas_first_node = 0; // TLAS nodes are [tlas_first_node, num_nodes)
    int32_t blas_depth = 0;      // deepest BLAS (wide levels), for stack sizing
    int32_t tlas_depth = 0;      // TLAS depth (wide levels)
    void* impl = nullptr;        // builder state kept for TLAS rebuilds
};

}  // namespace ptgb

#ifdef __cplusplus
extern "C" {
#endif
// Host: collapse the reference's flattened binary BVH into the wide layout.
// Returns 0 or a PT_ERR_* code; *err gets a message on failure.
int ptgb_build_wide(const float* bvh_nodes, int num_bvh_nodes, int top_level_index, const int32_t* vert_indices,
                    int num_tris, const float* vertices_uvx, int num_vertices, const float* transforms,
                    int num_instances, ptgb::WideBVH* out, char* err, int err_size);
void ptgb_free_wide(ptgb::WideBVH* bvh);
// Host: rebuild only the TLAS part for new TLAS binary nodes (those of
// [top_level_index, num_bvh_nodes)) and transforms, keeping the BLAS part.
int ptgb_rebuild_tlas(ptgb::WideBVH* bvh, const float* bvh_nodes, int num_bvh_nodes, int top_level_index,
                      const float* transforms, int num_instances, char* err, int err_size);
// Host: per-instance matrices, computed in double and rounded to float.
void ptgb_instance_xf(const float* transform16, ptgb::InstXf* out, int* is_identity);
#ifdef __cplusplus
}
#endif
