// scene_build.cpp - host scene preparation: builds the flattened arrays that
// GLSLPT::Scene::ProcessScene produces (src/core/Scene.cpp:216-297), for
// scenes given as triangle meshes + instances, without the reference's code.
//
// BLAS: binned SAH over triangle bounds (64 bins, traversal cost 2, leaves of
// fewer than 4 triangles), the configuration the reference gives its
// per-mesh SplitBvh (src/core/Mesh.h:37) with spatial splits disabled.
// TLAS: split at the centre of the centroid bounds along the longest axis,
// one instance per leaf, as the reference's Bvh(10.0f, 64, false)
// (src/core/Scene.h:70).  Flattening follows BvhTranslator's pre-order
// layout (thirdparty/RadeonRays/bvh_translator.cpp:32-120): all BLASes first,
// the TLAS from topLevelIndex, 2 x numInstances slots reserved for it.
// Built into libptscene.so (host only) and used by the scene generators.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "sah_builder.h"

namespace {

using AABB = ptgb::sah::AABB;
using Ref = ptgb::sah::Ref;
using BNode = ptgb::sah::Node;
using Builder = ptgb::sah::Builder;
struct SceneOut {
    std::vector<float> nodes;  // 9 floats per node
    int top_level_index = 0;
    std::vector<int32_t> vidx;
    std::vector<float> verts, norms;
};

// BvhTranslator::ProcessBLASNodes / ProcessTLASNodes: pre-order, left child
// next, right index in LRLeaf.y.
struct Flattener {
    std::vector<float>& out;
    int cur;
    explicit Flattener(std::vector<float>& o, int start) : out(o), cur(start) {}
    template <class LeafFn> int emit(const std::vector<BNode>& bn, int id, LeafFn leaf) {
        const int index = cur;
        float* p = &out[9 * (size_t)index];
        const BNode& n = bn[id];
        for (int k = 0; k < 3; ++k) { p[k] = n.box.lo[k]; p[3 + k] = n.box.hi[k]; }
        if (n.left < 0) {
            leaf(n, p + 6);
        } else {
            p[8] = 0.0f;
            cur++;
            const int l = emit(bn, n.left, leaf);
            cur++;
            const int r = emit(bn, n.right, leaf);
            p = &out[9 * (size_t)index];
            p[6] = (float)l;
            p[7] = (float)r;
        }
        return index;
    }
};

}  // namespace

extern "C" {

// Build a scene.  Meshes are non-indexed triangle lists (3 vertices per
// triangle, vertices as float4 xyz+u, normals as float4 xyz+v), concatenated;
// mesh m has triangles [mesh_tri_offset[m], mesh_tri_offset[m+1]).
// Instances: mesh id, material id and Mat4 (16 floats, row-vector layout).
// Returns an opaque handle (NULL on error); read with ptgb_scene_sizes /
// ptgb_scene_copy and release with ptgb_scene_free.
void* ptgb_scene_build(int num_meshes, const int32_t* mesh_tri_offset, const float* verts, const float* norms,
                       int num_instances, const int32_t* inst_mesh, const int32_t* inst_material,
                       const float* inst_xf) {
    if (num_meshes <= 0 || num_instances <= 0) return nullptr;
    SceneOut* S = new SceneOut;
    std::vector<Builder> blas(num_meshes);
    std::vector<AABB> mesh_bounds(num_meshes);
#pragma omp parallel for schedule(dynamic, 1)
    for (int m = 0; m < num_meshes; ++m) {
        const int t0 = mesh_tri_offset[m], t1 = mesh_tri_offset[m + 1];
        Builder& B = blas[m];
        B.refs.resize(t1 - t0);
        for (int t = t0; t < t1; ++t) {
            Ref& r = B.refs[t - t0];
            for (int v = 0; v < 3; ++v) r.b.grow(verts + 4 * (3 * (size_t)t + v));
            for (int k = 0; k < 3; ++k) r.c[k] = 0.5f * (r.b.lo[k] + r.b.hi[k]);
            r.idx = t - t0;
        }
        B.nodes.reserve(2 * (t1 - t0) + 1);
        if (t1 > t0) B.build(0, t1 - t0);
        else {
            B.nodes.emplace_back();
            B.nodes[0].box = AABB();
        }
        mesh_bounds[m] = B.nodes[0].box;
    }
    // node counts
    std::vector<int> root_start(num_meshes);
    int total = 0;
    for (int m = 0; m < num_meshes; ++m) {
        root_start[m] = total;
        total += (int)blas[m].nodes.size();
    }
    S->top_level_index = total;
    S->nodes.assign(9 * (size_t)(total + 2 * num_instances), 0.0f);
    // BLAS flattening + vertIndices in packed order (Scene.cpp:229-252)
    int tri_base = 0, vert_base = 0;
    for (int m = 0; m < num_meshes; ++m) {
        const int t0 = mesh_tri_offset[m], t1 = mesh_tri_offset[m + 1];
        Flattener F(S->nodes, root_start[m]);
        const int tb = tri_base;
        F.emit(blas[m].nodes, 0, [&](const BNode& n, float* lrl) {
            lrl[0] = (float)(tb + n.start);
            lrl[1] = (float)n.count;
            lrl[2] = 1.0f;
        });
        for (int j : blas[m].packed) {
            const int v = 3 * j + vert_base;
            S->vidx.push_back(v);
            S->vidx.push_back(v + 1);
            S->vidx.push_back(v + 2);
        }
        S->verts.insert(S->verts.end(), verts + 4 * 3 * (size_t)t0, verts + 4 * 3 * (size_t)t1);
        S->norms.insert(S->norms.end(), norms + 4 * 3 * (size_t)t0, norms + 4 * 3 * (size_t)t1);
        tri_base += (int)blas[m].packed.size();
        vert_base += 3 * (t1 - t0);
    }
    // TLAS over instance world bounds (Scene::createTLAS, Scene.cpp:148-187)
    Builder T;
    T.sah = false;
    T.max_leaf = 1;
    T.refs.resize(num_instances);
    for (int i = 0; i < num_instances; ++i) {
        const float* x = inst_xf + 16 * (size_t)i;
        const AABB& mb = mesh_bounds[inst_mesh[i]];
        // the reference sums float products (Scene.cpp:158-178); here the sum
        // is taken in double and rounded outwards so the box always bounds
        // the transformed mesh
        AABB wb;
        for (int k = 0; k < 3; ++k) {
            double lo = x[12 + k], hi = x[12 + k];
            for (int a = 0; a < 3; ++a) {  // rows 0..2 are the right / up / forward vectors
                const double e0 = double(x[4 * a + k]) * mb.lo[a], e1 = double(x[4 * a + k]) * mb.hi[a];
                lo += std::min(e0, e1);
                hi += std::max(e0, e1);
            }
            wb.lo[k] = std::nextafter((float)lo, -INFINITY);
            wb.hi[k] = std::nextafter((float)hi, INFINITY);
        }
        T.refs[i].b = wb;
        for (int k = 0; k < 3; ++k) T.refs[i].c[k] = 0.5f * (wb.lo[k] + wb.hi[k]);
        T.refs[i].idx = i;
    }
    T.build(0, num_instances);
    Flattener F(S->nodes, S->top_level_index);
    F.emit(T.nodes, 0, [&](const BNode& n, float* lrl) {
        const int inst = T.packed[n.start];
        lrl[0] = (float)root_start[inst_mesh[inst]];
        lrl[1] = (float)inst_material[inst];
        lrl[2] = (float)(-inst - 1);
    });
    return S;
}

int ptgb_scene_sizes(void* h, int32_t* num_nodes, int32_t* top_level_index, int32_t* num_tris, int32_t* num_vertices) {
    const SceneOut* S = static_cast<SceneOut*>(h);
    if (!S) return 1;
    *num_nodes = (int32_t)(S->nodes.size() / 9);
    *top_level_index = S->top_level_index;
    *num_tris = (int32_t)(S->vidx.size() / 3);
    *num_vertices = (int32_t)(S->verts.size() / 4);
    return 0;
}

int ptgb_scene_copy(void* h, float* nodes, int32_t* vidx, float* verts, float* norms) {
    const SceneOut* S = static_cast<SceneOut*>(h);
    if (!S) return 1;
    std::memcpy(nodes, S->nodes.data(), S->nodes.size() * sizeof(float));
    std::memcpy(vidx, S->vidx.data(), S->vidx.size() * sizeof(int32_t));
    std::memcpy(verts, S->verts.data(), S->verts.size() * sizeof(float));
    std::memcpy(norms, S->norms.data(), S->norms.size() * sizeof(float));
    return 0;
}

void ptgb_scene_free(void* h) { delete static_cast<SceneOut*>(h); }

}  // extern "C"
