// bvh8_build.cpp - host-side collapse of the reference's flattened binary BVH
// into the 8-wide quantised layout of bvh8.h.
//
// Input is exactly what GLSLPT::Scene::ProcessScene leaves in
// bvhTranslator.nodes (thirdparty/RadeonRays/bvh_translator.cpp:32-120):
// pre-order binary nodes with LRLeaf = (left, right, 0) for interior nodes,
// (firstTri, numTris, 1) for BLAS leaves and (blasRoot, materialID,
// -instance-1) for TLAS leaves, BLASes first and the TLAS from
// topLevelIndex on.  Each wide node takes up to eight binary descendants,
// chosen greedily by expanding the interior child of largest surface area,
// so the wide tree holds the binary tree's boxes with fewer, larger nodes.
//
// Instances whose transform is the identity are merged: their triangles get
// one BLAS of their own (binned SAH, sah_builder.h), each triangle carrying
// its instance and material in the spare lanes of its WideTri record, and
// the TLAS is rebuilt over that BLAS and the remaining instances.  The
// reference gives every mesh its own instance (one material per instance),
// so scenes made of many untransformed meshes would otherwise pay for
// overlapping instance boxes on every ray.  Hits (triangle, instance,
// material, distance) are unchanged: the same triangles are tested with the
// same arithmetic in the same space.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/pt_cuda.h"
#include "bvh8.h"
#include "sah_builder.h"

using namespace ptgb;

namespace {

struct BinNode {
    float lo[3], hi[3];
    int l, r, leaf;  // leaf: 0 interior, 1 BLAS leaf, 2 merged leaf (range of Impl::merged), <0 TLAS leaf
};

struct Box {
    float lo[3], hi[3];
    void empty() { for (int k = 0; k < 3; ++k) { lo[k] = INFINITY; hi[k] = -INFINITY; } }
    void grow(const Box& b) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
    }
    void grow(const float* p) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); }
    }
    double area() const {
        double d[3];
        for (int k = 0; k < 3; ++k) d[k] = std::max(0.0, double(hi[k]) - double(lo[k]));
        return 2.0 * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
    }
};

// A child of a wide node: a binary interior node, or a primitive range
// [first, first+count) (triangles in a BLAS, entries of the merged triangle
// list, or one instance in the TLAS), or up to three primitives listed in
// items[] (the triangles of a small binary subtree made one leaf).
struct Child {
    int bin = -1;        // binary interior node index (range children: -1)
    int first = 0, count = 0;
    int nitems = 0, items[3] = {0, 0, 0};
    bool merged = false;
    int blas_root = -1, material = 0;  // TLAS leaf data
    Box box;
    bool is_range() const { return bin < 0; }
    bool is_leaf_slot() const { return bin < 0 && count <= 3; }
    int item(int q) const { return nitems ? items[q] : first + q; }
};

// SAH cost of the wide tree, per unit of surface area: a wide-node visit
// and a primitive test (triangle, or instance entry), relative to it.
constexpr double kCostNode = 1.0;
constexpr double kCostPrim = 0.3;
// Triangles per leaf child at most.  A leaf child's triangles are all
// tested when its box is hit; rays that start on a surface graze the boxes
// around their origin, and with one triangle per leaf they test half the
// triangles (C2: 10.6 -> 5.2 per closest-hit query, 17.3 -> 8.8 per shadow
// query) for 10% more node visits: 2% faster on the 1M-triangle icosphere,
// 2.5% slower on a 34-triangle Cornell box, where the extra level is the
// larger share.  So one triangle per leaf from 4096 triangles on, else up
// to three (the reference's leaves, Bvh settings); PT_BVH_MAX_LEAF (1..3)
// overrides.
int blas_max_leaf(int num_tris) {
    static const int env = [] {
        const char* e = std::getenv("PT_BVH_MAX_LEAF");
        const int x = e ? std::atoi(e) : 0;
        return x >= 1 && x <= 3 ? x : 0;
    }();
    if (env) return env;
    return num_tris >= 4096 ? 1 : 3;
}

// Dynamic-programming state of a binary node (the collapse, below).
struct Dp {
    double c[9];          // c[i], i = 1..8: least cost of the subtree as at most i children of a wide node
    int8_t k[9];          // i >= 2: children given to the left subtree (0: c[i] is c[i-1])
    int8_t k8 = 0;        // the split of the best eight-child distribution (the wide node made of n)
    bool leaf = false;    // c[1]: the subtree is one leaf child (else one internal child)
    int np = 0;           // primitives in the subtree
};

struct MergedTri {
    int tri, inst, mat;
};

constexpr int kMergedInstance = 0x7fffffff;  // InstRef.instance of the merged BLAS

struct Impl {
    // inputs (copies, so instance updates can rebuild)
    std::vector<BinNode> bn;
    int top = 0;
    std::vector<int32_t> vidx;
    std::vector<float> verts;  // xyz per vertex
    int num_tris = 0, num_vertices = 0, num_instances = 0;
    std::vector<float> transforms;
    // outputs
    std::vector<WideNode> nodes;
    std::vector<WideTri> tris;
    std::vector<InstRef> insts;
    std::vector<int> inst_identity;
    std::vector<MergedTri> merged;
    std::map<int, int> blas_root_map;  // binary BLAS root -> wide node index
    bool tlas = false;
    int max_depth = 0;
    std::vector<Dp> dp;                // per binary node, filled per root by dp_solve
};

struct BuildError {
    std::string msg;
};

[[noreturn]] void fail(const std::string& m) { throw BuildError{m}; }

int tri_of(const Impl& I, int k, bool merged) { return merged ? I.merged[k].tri : k; }

Box tri_box(const Impl& I, int t) {
    if (t < 0 || t >= I.num_tris) fail("leaf triangle index out of range: " + std::to_string(t));
    Box b;
    b.empty();
    for (int k = 0; k < 3; ++k) {
        int v = I.vidx[3 * (size_t)t + k];
        if (v < 0 || v >= I.num_vertices) fail("vertex index out of range: " + std::to_string(v));
        b.grow(&I.verts[3 * (size_t)v]);
    }
    return b;
}

Box range_box(const Impl& I, int first, int count, bool merged) {
    Box b;
    b.empty();
    for (int i = 0; i < count; ++i) b.grow(tri_box(I, tri_of(I, first + i, merged)));
    return b;
}

Box node_box(const BinNode& n) {
    Box b;
    for (int k = 0; k < 3; ++k) { b.lo[k] = n.lo[k]; b.hi[k] = n.hi[k]; }
    return b;
}

// Children contributed by binary node `b` (one entry, or a leaf range).
void children_of(const Impl& I, int b, std::vector<Child>& out) {
    if (b < 0 || b >= (int)I.bn.size()) fail("child node index out of range: " + std::to_string(b));
    const BinNode& n = I.bn[b];
    Child c;
    if (n.leaf == 0) {
        c.bin = b;
        c.box = node_box(n);
        out.push_back(c);
    } else if (n.leaf > 0) {
        if (I.tlas) fail("BLAS leaf reached while walking the TLAS (node " + std::to_string(b) + ")");
        if (n.r < 0) fail("negative triangle count in leaf " + std::to_string(b));
        if (n.r == 0) return;
        c.first = n.l;
        c.count = n.r;
        c.merged = n.leaf == 2;
        if (c.merged && (n.l < 0 || n.l + n.r > (int)I.merged.size())) fail("merged leaf out of range");
        // a reference leaf holds < 4 triangles and its box bounds them; the
        // triangles' own box is used for bigger ones (they are split later)
        Box tb = range_box(I, c.first, c.count, c.merged);  // also validates the indices
        c.box = n.r <= 3 ? node_box(n) : tb;
        out.push_back(c);
    } else {
        if (!I.tlas) fail("TLAS leaf reached inside a BLAS (node " + std::to_string(b) + ")");
        int inst = -n.leaf - 1;
        if (inst >= I.num_instances && inst != kMergedInstance) fail("instance index out of range: " + std::to_string(inst));
        c.first = inst;
        c.count = 1;
        c.blas_root = n.l;
        c.material = n.r;
        c.box = node_box(n);
        out.push_back(c);
    }
}

// Split a primitive range of more than 3 primitives into up to 8 pieces.
void split_range(const Impl& I, const Child& c, std::vector<Child>& out) {
    int pieces = std::min(8, (c.count + 2) / 3);
    int per = (c.count + pieces - 1) / pieces;
    for (int f = c.first; f < c.first + c.count; f += per) {
        Child r;
        r.first = f;
        r.count = std::min(per, c.first + c.count - f);
        r.merged = c.merged;
        r.box = range_box(I, r.first, r.count, r.merged);
        out.push_back(r);
    }
}

void quantise(const Box& node, const std::vector<Child>& kids, const int slot_of[8], WideNode& wn, int imask,
              int child_base, int prim_base, const uint8_t meta[8]) {
    std::memset(&wn, 0, sizeof wn);
    int ex[3];
    double scale[3];
    for (int k = 0; k < 3; ++k) {
        double range = double(node.hi[k]) - double(node.lo[k]);
        int e;
        if (!(range > 0.0)) e = -126;
        else {
            e = (int)std::ceil(std::log2(range / 255.0));
            while (std::ldexp(255.0, e) < range) ++e;
            while (e > -126 && std::ldexp(255.0, e - 1) >= range) --e;
        }
        e = std::max(-126, std::min(127, e));
        ex[k] = e;
        scale[k] = std::ldexp(1.0, e);
    }
    float p[3] = {node.lo[0], node.lo[1], node.lo[2]};
    std::memcpy(&wn.w[0], &p[0], 4);
    std::memcpy(&wn.w[1], &p[1], 4);
    std::memcpy(&wn.w[2], &p[2], 4);
    wn.w[3] = uint32_t(ex[0] + 127) | (uint32_t(ex[1] + 127) << 8) | (uint32_t(ex[2] + 127) << 16) |
              (uint32_t(imask) << 24);
    wn.w[4] = uint32_t(child_base);
    wn.w[5] = uint32_t(prim_base);
    wn.w[6] = meta[0] | (meta[1] << 8) | (meta[2] << 16) | (uint32_t(meta[3]) << 24);
    wn.w[7] = meta[4] | (meta[5] << 8) | (meta[6] << 16) | (uint32_t(meta[7]) << 24);
    uint8_t* q = reinterpret_cast<uint8_t*>(&wn.w[8]);  // 48 bytes: qlo x,y,z then qhi x,y,z, 8 each
    for (size_t i = 0; i < kids.size(); ++i) {
        int s = slot_of[i];
        for (int k = 0; k < 3; ++k) {
            double lo = std::floor((double(kids[i].box.lo[k]) - double(p[k])) / scale[k]);
            double hi = std::ceil((double(kids[i].box.hi[k]) - double(p[k])) / scale[k]);
            lo = std::max(0.0, std::min(255.0, lo));
            hi = std::max(0.0, std::min(255.0, hi));
            q[k * 8 + s] = (uint8_t)lo;
            q[(3 + k) * 8 + s] = (uint8_t)hi;
        }
    }
}

// Assign children to slots by centroid direction (octant order, bvh8.h).
void assign_slots(const Box& node, const std::vector<Child>& kids, int slot_of[8]) {
    double c[3];
    for (int k = 0; k < 3; ++k) c[k] = 0.5 * (double(node.lo[k]) + double(node.hi[k]));
    const int n = (int)kids.size();
    double score[8][8];
    for (int i = 0; i < n; ++i) {
        double d[3];
        for (int k = 0; k < 3; ++k) d[k] = 0.5 * (double(kids[i].box.lo[k]) + double(kids[i].box.hi[k])) - c[k];
        for (int s = 0; s < 8; ++s) {
            double v = 0;
            for (int k = 0; k < 3; ++k) v += ((s >> k) & 1 ? 1.0 : -1.0) * d[k];
            score[i][s] = v;
        }
    }
    bool used_child[8] = {}, used_slot[8] = {};
    for (int round = 0; round < n; ++round) {
        double best = -INFINITY;
        int bi = -1, bs = -1;
        for (int i = 0; i < n; ++i) {
            if (used_child[i]) continue;
            for (int s = 0; s < 8; ++s) {
                if (used_slot[s]) continue;
                if (score[i][s] > best || bi < 0) { best = score[i][s]; bi = i; bs = s; }
            }
        }
        used_child[bi] = used_slot[bs] = true;
        slot_of[bi] = bs;
    }
}

// ---------------------------------------------------------------- collapse
// Which binary descendants become the children of each wide node is chosen
// by dynamic programming over the binary tree for the least SAH cost, as in
// Ylitie, Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs
// Through Compressed Wide BVHs" (HPG 2017), section 3.1.  c[i] of a node is
// the least cost of its subtree as at most i children of the wide node above:
//   c[1] = min(leaf: A * kCostPrim * prims        if prims <= 3 (TLAS: 1),
//              internal: A * kCostNode + D(8))
//   c[i] = min(c[i-1], D(i)),   D(i) = min over j of left.c[j] + right.c[i-j]
// with A the node's surface area.  The wide node made of a binary node takes
// the children of its best eight-way distribution.  Leaves of the binary
// tree keep their triangles (more than three: an internal child over ranges,
// split_range); an interior node of at most three triangles may become one
// leaf.  A greedy expansion (largest box first) instead leaves most of the
// nodes just above the leaves with two children.
void dp_solve(Impl& I, int root) {
    if ((int)I.dp.size() < (int)I.bn.size()) I.dp.resize(I.bn.size());
    const int max_leaf = I.tlas ? 1 : blas_max_leaf(I.num_tris);
    std::vector<std::pair<int, bool>> st;  // (node, children done)
    st.push_back({root, false});
    while (!st.empty()) {
        auto [n, ready] = st.back();
        st.pop_back();
        if (n < 0 || n >= (int)I.bn.size()) fail("child node index out of range: " + std::to_string(n));
        const BinNode& b = I.bn[n];
        Dp& d = I.dp[n];
        const double A = node_box(b).area();
        if (b.leaf != 0) {
            int np = b.leaf < 0 ? 1 : b.r;
            if (np < 0) fail("negative triangle count in leaf " + std::to_string(n));
            d.np = np;
            if (np == 0) {
                d.c[1] = 0.0;
                d.leaf = true;
            } else if (np <= max_leaf) {
                d.c[1] = A * kCostPrim * np;
                d.leaf = true;
            } else {  // split into ranges under an internal child
                d.c[1] = A * kCostNode + A * kCostPrim * np;
                d.leaf = false;
            }
            for (int i = 2; i <= 8; ++i) { d.c[i] = d.c[1]; d.k[i] = 0; }
            continue;
        }
        if (!ready) {
            st.push_back({n, true});
            st.push_back({b.l, false});
            st.push_back({b.r, false});
            continue;
        }
        const Dp& L = I.dp[b.l];
        const Dp& R = I.dp[b.r];
        d.np = L.np + R.np;
        double D[9];
        int8_t K[9];
        for (int i = 2; i <= 8; ++i) {
            D[i] = INFINITY;
            K[i] = 1;
            for (int j = 1; j < i; ++j) {
                const double v = L.c[j] + R.c[i - j];
                if (v < D[i]) { D[i] = v; K[i] = (int8_t)j; }
            }
        }
        d.k8 = K[8];
        const double cleaf = d.np <= max_leaf ? A * kCostPrim * d.np : INFINITY;
        const double cnode = A * kCostNode + D[8];
        d.leaf = cleaf <= cnode;
        d.c[1] = d.leaf ? cleaf : cnode;
        for (int i = 2; i <= 8; ++i) {
            if (D[i] < d.c[i - 1]) { d.c[i] = D[i]; d.k[i] = K[i]; }
            else { d.c[i] = d.c[i - 1]; d.k[i] = 0; }
        }
    }
}

// The binary nodes that become the (at most i) children for subtree n.
void dp_slots(const Impl& I, int n, int i, std::vector<int>& out) {
    const Dp& d = I.dp[n];
    if (d.np == 0) return;  // an empty leaf contributes nothing
    while (i > 1 && d.k[i] == 0) --i;
    if (i == 1) { out.push_back(n); return; }
    const BinNode& b = I.bn[n];
    dp_slots(I, b.l, d.k[i], out);
    dp_slots(I, b.r, i - d.k[i], out);
}

// Primitives of the subtree of n (at most three), for a leaf child.
void gather_items(const Impl& I, int n, Child& c) {
    const BinNode& b = I.bn[n];
    if (b.leaf > 0) {
        c.merged = b.leaf == 2;
        if (c.merged && (b.l < 0 || b.l + b.r > (int)I.merged.size())) fail("merged leaf out of range");
        for (int q = 0; q < b.r; ++q) {
            if (c.nitems >= 3) fail("leaf of more than three primitives");
            c.items[c.nitems++] = b.l + q;
        }
        range_box(I, b.l, b.r, c.merged);  // validates the indices
        return;
    }
    if (b.leaf < 0) fail("TLAS leaf reached inside a BLAS (node " + std::to_string(n) + ")");
    gather_items(I, b.l, c);
    gather_items(I, b.r, c);
}

// The wide-node child made of binary node n as the DP chose it.
Child child_of_slot(const Impl& I, int n) {
    const BinNode& b = I.bn[n];
    if (b.leaf != 0) {
        std::vector<Child> one;
        children_of(I, n, one);
        if (one.size() != 1) fail("empty leaf as a child");
        return one[0];
    }
    Child c;
    c.box = node_box(b);
    if (I.dp[n].leaf) {
        if (I.tlas) fail("TLAS interior node as a leaf child");
        gather_items(I, n, c);
        c.count = c.nitems;
        c.first = -1;
    } else {
        c.bin = n;
    }
    return c;
}

// The children of the wide node made of interior binary node n.
void dp_children(const Impl& I, int n, std::vector<Child>& kids) {
    const BinNode& b = I.bn[n];
    const int k8 = I.dp[n].k8;
    std::vector<int> slots;
    dp_slots(I, b.l, k8, slots);
    dp_slots(I, b.r, 8 - k8, slots);
    for (int s : slots) kids.push_back(child_of_slot(I, s));
}

void build_node(Impl& I, const std::vector<Child>& kids, int target, int depth);

// Build the wide node at index `target` from binary node / range `root`.
void build_from(Impl& I, const Child& root, int target, int depth) {
    std::vector<Child> kids;
    if (root.is_range()) {
        if (root.count <= 3) kids.push_back(root);
        else split_range(I, root, kids);
    } else {
        dp_children(I, root.bin, kids);
    }
    build_node(I, kids, target, depth);
}

void build_node(Impl& I, const std::vector<Child>& kids, int target, int depth) {
    if (depth > 200) fail("BVH deeper than 200 wide levels");
    I.max_depth = std::max(I.max_depth, depth);
    if (kids.size() > 8) fail("more than eight children");
    if (kids.empty()) fail("empty BVH node");
    Box nb;
    nb.empty();
    for (auto& k : kids) nb.grow(k.box);
    int slot_of[8];
    assign_slots(nb, kids, slot_of);
    // internal children (interior binary nodes and oversized ranges), in slot order
    std::vector<int> order(kids.size());
    for (size_t i = 0; i < kids.size(); ++i) order[i] = (int)i;
    std::sort(order.begin(), order.end(), [&](int a, int b) { return slot_of[a] < slot_of[b]; });
    uint8_t meta[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int imask = 0, num_internal = 0;
    for (int i : order)
        if (!kids[i].is_leaf_slot()) { imask |= 1 << slot_of[i]; ++num_internal; }
    const int child_base = (int)I.nodes.size();
    I.nodes.resize(I.nodes.size() + num_internal);
    const int prim_base = I.tlas ? (int)I.insts.size() : (int)I.tris.size();
    int prim_off = 0;
    for (int i : order) {
        const Child& c = kids[i];
        const int s = slot_of[i];
        if (!c.is_leaf_slot()) {
            meta[s] = uint8_t((1 << 5) | (24 + s));
            continue;
        }
        meta[s] = uint8_t((((1 << c.count) - 1) << 5) | prim_off);
        prim_off += c.count;
        if (I.tlas) {
            auto it = I.blas_root_map.find(c.blas_root);
            if (it == I.blas_root_map.end()) fail("TLAS leaf refers to an unbuilt BLAS root");
            InstRef r;
            r.blas_root = it->second;
            r.instance = c.first;
            r.material = c.material;
            r.identity = c.first == kMergedInstance ? 1 : I.inst_identity[c.first];
            I.insts.push_back(r);
        } else {
            for (int q = 0; q < c.count; ++q) {
                const int k = c.item(q);
                const int t = tri_of(I, k, c.merged);
                WideTri wt;
                const int32_t* vi = &I.vidx[3 * (size_t)t];
                const float* a = &I.verts[3 * (size_t)vi[0]];
                const float* b = &I.verts[3 * (size_t)vi[1]];
                const float* d = &I.verts[3 * (size_t)vi[2]];
                for (int j = 0; j < 3; ++j) {
                    wt.v0[j] = a[j];
                    wt.e0[j] = b[j] - a[j];  // the shader's e0 = v1.xyz - v0.xyz (closest_hit.glsl:128)
                    wt.e1[j] = d[j] - a[j];  // e1 = v2.xyz - v0.xyz
                }
                int inst = 0, mat = 0;
                if (c.merged) {
                    inst = I.merged[k].inst;
                    mat = I.merged[k].mat;
                }
                std::memcpy(&wt.e0[3], &inst, 4);
                std::memcpy(&wt.e1[3], &mat, 4);
                wt.prim = t;
                I.tris.push_back(wt);
            }
        }
    }
    if (prim_off > 24) fail("more than 24 primitives under one wide node");
    quantise(nb, kids, slot_of, I.nodes[target], imask, child_base, prim_base, meta);
    int j = 0;
    for (int i : order) {
        if (kids[i].is_leaf_slot()) continue;
        build_from(I, kids[i], child_base + j, depth + 1);
        ++j;
    }
}

int build_root(Impl& I, int bin_root) {
    const int target = (int)I.nodes.size();
    I.nodes.emplace_back();
    std::vector<Child> kids;
    const BinNode& n = I.bn[bin_root];
    if (n.leaf != 0) children_of(I, bin_root, kids);
    else {
        dp_solve(I, bin_root);
        dp_children(I, bin_root, kids);
    }
    if (kids.empty()) {
        // an empty leaf: a wide node with no children never hits
        std::memset(&I.nodes[target], 0, sizeof(WideNode));
        return target;
    }
    if (kids.size() == 1 && kids[0].is_range() && kids[0].count > 3) {
        std::vector<Child> sub;
        split_range(I, kids[0], sub);
        kids.swap(sub);
    }
    build_node(I, kids, target, 1);
    return target;
}

void read_binary(std::vector<BinNode>& bn, const float* nodes, int first, int n) {
    for (int i = first; i < n; ++i) {
        const float* p = nodes + 9 * (size_t)i;
        BinNode& b = bn[i];
        for (int k = 0; k < 3; ++k) { b.lo[k] = p[k]; b.hi[k] = p[3 + k]; }
        b.l = (int)p[6]; b.r = (int)p[7]; b.leaf = (int)p[8];
        if (b.leaf == 2) b.leaf = 1;  // only the merge step makes merged leaves
    }
}

// TLAS leaves reachable from `top`: (node index) in tree order.
void collect_tlas_leaves(const Impl& I, int top, std::vector<int>& leaves) {
    std::vector<int> stack{top};
    std::vector<char> seen(I.bn.size(), 0);
    while (!stack.empty()) {
        int b = stack.back();
        stack.pop_back();
        if (b < 0 || b >= (int)I.bn.size()) fail("TLAS child index out of range");
        if (seen[b]) fail("TLAS is not a tree");
        seen[b] = 1;
        const BinNode& n = I.bn[b];
        if (n.leaf < 0) {
            if (n.l < 0 || n.l >= (int)I.bn.size()) fail("BLAS root index out of range");
            leaves.push_back(b);
        } else if (n.leaf == 0) {
            stack.push_back(n.r);
            stack.push_back(n.l);
        } else {
            fail("BLAS leaf inside the TLAS");
        }
    }
}

// Triangle ranges of the BLAS rooted at `root` (binary leaves, in order).
void collect_blas_tris(const Impl& I, int root, std::vector<int>& tris_out) {
    std::vector<int> stack{root};
    size_t guard = 0;
    while (!stack.empty()) {
        if (++guard > 4 * I.bn.size() + 16) fail("BLAS is not a tree");
        int b = stack.back();
        stack.pop_back();
        if (b < 0 || b >= (int)I.bn.size()) fail("BLAS child index out of range");
        const BinNode& n = I.bn[b];
        if (n.leaf == 0) {
            stack.push_back(n.r);
            stack.push_back(n.l);
        } else if (n.leaf > 0) {
            if (n.r < 0) fail("negative triangle count");
            for (int t = n.l; t < n.l + n.r; ++t) {
                if (t < 0 || t >= I.num_tris) fail("leaf triangle index out of range: " + std::to_string(t));
                tris_out.push_back(t);
            }
        } else {
            fail("TLAS leaf inside a BLAS");
        }
    }
}

// Append a sah::Builder tree to I.bn; leaves through `leaf`.
template <class LeafFn> int append_tree(Impl& I, const sah::Builder& B, LeafFn leaf) {
    const int base = (int)I.bn.size();
    I.bn.resize(base + B.nodes.size());
    for (size_t i = 0; i < B.nodes.size(); ++i) {
        const sah::Node& s = B.nodes[i];
        BinNode& d = I.bn[base + i];
        for (int k = 0; k < 3; ++k) { d.lo[k] = s.box.lo[k]; d.hi[k] = s.box.hi[k]; }
        if (s.left < 0) {
            leaf(s, d);
        } else {
            d.l = base + s.left;
            d.r = base + s.right;
            d.leaf = 0;
        }
    }
    return base;  // the root (builder node 0)
}

void build_all(Impl& I, WideBVH* out) {
    I.nodes.clear();
    I.tris.clear();
    I.insts.clear();
    I.merged.clear();
    I.blas_root_map.clear();
    I.inst_identity.assign(I.num_instances, 0);
    for (int i = 0; i < I.num_instances; ++i) {
        InstXf xf;
        int id = 0;
        ptgb_instance_xf(&I.transforms[16 * (size_t)i], &xf, &id);
        I.inst_identity[i] = id;
    }
    std::vector<int> leaves;
    collect_tlas_leaves(I, I.top, leaves);
    std::vector<int> ident, other;
    for (int li : leaves) {
        const int inst = -I.bn[li].leaf - 1;
        if (inst >= I.num_instances) fail("instance index out of range: " + std::to_string(inst));
        (I.inst_identity[inst] ? ident : other).push_back(li);
    }
    int tlas_root_bin = I.top;
    const size_t input_nodes = I.bn.size();
    if (ident.size() >= 2) {
        // one BLAS over the triangles of every untransformed instance
        sah::Builder M;
        M.max_leaf = blas_max_leaf(I.num_tris);
        std::vector<MergedTri> prims;
        std::vector<int> tl;
        for (int li : ident) {
            tl.clear();
            collect_blas_tris(I, I.bn[li].l, tl);
            for (int t : tl) prims.push_back({t, -I.bn[li].leaf - 1, I.bn[li].r});
        }
        M.refs.resize(prims.size());
        for (size_t k = 0; k < prims.size(); ++k) {
            Box b = tri_box(I, prims[k].tri);
            sah::Ref& r = M.refs[k];
            for (int j = 0; j < 3; ++j) {
                r.b.lo[j] = b.lo[j];
                r.b.hi[j] = b.hi[j];
                r.c[j] = 0.5f * (b.lo[j] + b.hi[j]);
            }
            r.idx = (int)k;
        }
        if (!prims.empty()) {
            M.nodes.reserve(2 * prims.size());
            M.build(0, (int)prims.size());
            I.merged.resize(prims.size());
            for (size_t k = 0; k < M.packed.size(); ++k) I.merged[k] = prims[M.packed[k]];
            const int merged_root = append_tree(I, M, [](const sah::Node& s, BinNode& d) {
                d.l = s.start;
                d.r = s.count;
                d.leaf = 2;
            });
            // TLAS over the merged BLAS and the transformed instances
            sah::Builder T;
            T.max_leaf = 1;
            std::vector<int> items;  // TLAS leaf node per item; -1 = merged BLAS
            items.push_back(-1);
            for (int li : other) items.push_back(li);
            T.refs.resize(items.size());
            for (size_t k = 0; k < items.size(); ++k) {
                sah::Ref& r = T.refs[k];
                const float* lo = items[k] < 0 ? I.bn[merged_root].lo : I.bn[items[k]].lo;
                const float* hi = items[k] < 0 ? I.bn[merged_root].hi : I.bn[items[k]].hi;
                for (int j = 0; j < 3; ++j) {
                    r.b.lo[j] = lo[j];
                    r.b.hi[j] = hi[j];
                    r.c[j] = 0.5f * (lo[j] + hi[j]);
                }
                r.idx = (int)k;
            }
            T.nodes.reserve(2 * items.size());
            T.build(0, (int)items.size());
            tlas_root_bin = append_tree(I, T, [&](const sah::Node& s, BinNode& d) {
                const int it = items[T.packed[s.start]];
                if (it < 0) {
                    d.l = merged_root;
                    d.r = -1;
                    d.leaf = -kMergedInstance - 1;
                } else {
                    d = I.bn[it];
                }
            });
        }
    }
    // BLASes referenced by the TLAS, then the TLAS
    std::vector<int> tl_leaves;
    collect_tlas_leaves(I, tlas_root_bin, tl_leaves);
    I.tlas = false;
    I.max_depth = 0;
    for (int li : tl_leaves) {
        const int r = I.bn[li].l;
        if (I.blas_root_map.count(r)) continue;
        if (I.bn[r].leaf < 0) fail("BLAS root is a TLAS leaf");
        I.blas_root_map[r] = build_root(I, r);
    }
    out->blas_depth = I.max_depth;
    I.max_depth = 0;
    I.tlas = true;
    out->tlas_first_node = (int)I.nodes.size();
    out->tlas_root = build_root(I, tlas_root_bin);
    out->tlas_depth = I.max_depth;
    I.bn.resize(input_nodes);  // drop the appended trees: the input stays as given
    out->nodes = I.nodes.data();
    out->num_nodes = (int)I.nodes.size();
    out->tris = I.tris.data();
    out->num_tris = (int)I.tris.size();
    out->insts = I.insts.data();
    out->num_inst_refs = (int)I.insts.size();
    out->impl = &I;
}

void copy_err(const std::string& m, char* err, int n) {
    if (err && n > 0) std::snprintf(err, n, "%s", m.c_str());
}

}  // namespace

extern "C" void ptgb_instance_xf(const float* d16, InstXf* out, int* is_identity) {
    double m[16];  // m[col*4+row] = data[col][row], the GLSL column-major matrix mat4(data rows)
    for (int i = 0; i < 16; ++i) m[i] = d16[i];
    int ident = 1;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r)
            if (d16[c * 4 + r] != (c == r ? 1.0f : 0.0f)) ident = 0;
    if (is_identity) *is_identity = ident;
    // cofactor inverse, in double, rounded to float
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
    for (int i = 0; i < 16; ++i) out->inv[i] = float(inv[i] / det);
    // mat3(transform): columns c = data[c][0..2]
    double a[3][3];
    for (int c = 0; c < 3; ++c) {
        for (int r = 0; r < 3; ++r) {
            a[c][r] = d16[c * 4 + r];
            out->m3[c * 4 + r] = d16[c * 4 + r];
        }
        out->m3[c * 4 + 3] = 0.0f;
    }
    const double A = a[0][0], B = a[1][0], C = a[2][0];
    const double D = a[0][1], E = a[1][1], F = a[2][1];
    const double G = a[0][2], H = a[1][2], I = a[2][2];
    const double cof[3][3] = {{E * I - F * H, -(D * I - F * G), D * H - E * G},
                              {-(B * I - C * H), A * I - C * G, -(A * H - B * G)},
                              {B * F - C * E, -(A * F - C * D), A * E - B * D}};
    const double d3 = A * cof[0][0] + B * cof[0][1] + C * cof[0][2];
    // transpose(inverse(m3)): element (row r, col c) = cof[r][c] / det
    for (int c = 0; c < 3; ++c) {
        for (int r = 0; r < 3; ++r) out->nrm[c * 4 + r] = float(cof[r][c] / d3);
        out->nrm[c * 4 + 3] = 0.0f;
    }
}

extern "C" int ptgb_build_wide(const float* bvh_nodes, int num_bvh_nodes, int top_level_index,
                               const int32_t* vert_indices, int num_tris, const float* vertices_uvx, int num_vertices,
                               const float* transforms, int num_instances, WideBVH* out, char* err, int err_size) {
    Impl* I = new Impl;
    try {
        if (!bvh_nodes || num_bvh_nodes <= 0) fail("no BVH nodes");
        if (top_level_index < 0 || top_level_index >= num_bvh_nodes) fail("top_level_index out of range");
        if (num_tris < 0 || num_vertices < 0 || num_instances <= 0) fail("negative sizes");
        I->bn.resize(num_bvh_nodes);
        read_binary(I->bn, bvh_nodes, 0, num_bvh_nodes);
        I->top = top_level_index;
        I->vidx.assign(vert_indices, vert_indices + 3 * (size_t)num_tris);
        I->verts.resize(3 * (size_t)num_vertices);
        for (int v = 0; v < num_vertices; ++v)
            for (int k = 0; k < 3; ++k) I->verts[3 * (size_t)v + k] = vertices_uvx[4 * (size_t)v + k];
        I->num_tris = num_tris;
        I->num_vertices = num_vertices;
        I->num_instances = num_instances;
        I->transforms.assign(transforms, transforms + 16 * (size_t)num_instances);
        build_all(*I, out);
        return PT_OK;
    } catch (const BuildError& e) {
        copy_err(e.msg, err, err_size);
        delete I;
        out->impl = nullptr;
        return PT_ERR_INVALID_ARG;
    } catch (const std::bad_alloc&) {
        copy_err("host allocation failed in BVH collapse", err, err_size);
        delete I;
        out->impl = nullptr;
        return PT_ERR_OUT_OF_MEMORY;
    }
}

extern "C" int ptgb_rebuild_tlas(WideBVH* out, const float* bvh_nodes, int num_bvh_nodes, int top_level_index,
                                 const float* transforms, int num_instances, char* err, int err_size) {
    Impl* I = static_cast<Impl*>(out->impl);
    if (!I) { copy_err("no BVH to update", err, err_size); return PT_ERR_INVALID_ARG; }
    try {
        if (top_level_index < 0 || top_level_index >= num_bvh_nodes) fail("top_level_index out of range");
        if (top_level_index != I->top) fail("the BLAS part of the BVH changed size");
        if (num_instances <= 0) fail("no instances");
        // the BLAS part of the binary array is unchanged (Scene::RebuildInstances
        // rewrites only the TLAS slice, Scene.cpp:200-214); the build runs on a
        // copy so that a rejected update leaves the current BVH in place
        Impl next = *I;
        next.bn.resize(num_bvh_nodes);
        read_binary(next.bn, bvh_nodes, top_level_index, num_bvh_nodes);
        next.num_instances = num_instances;
        next.transforms.assign(transforms, transforms + 16 * (size_t)num_instances);
        WideBVH tmp = *out;
        build_all(next, &tmp);
        *I = std::move(next);  // moving the vectors keeps their buffers, so tmp's pointers stay valid
        tmp.impl = I;
        *out = tmp;
        return PT_OK;
    } catch (const BuildError& e) {
        copy_err(e.msg, err, err_size);
        return PT_ERR_INVALID_ARG;
    } catch (const std::bad_alloc&) {
        copy_err("host allocation failed in BVH collapse", err, err_size);
        return PT_ERR_OUT_OF_MEMORY;
    }
}

extern "C" void ptgb_free_wide(WideBVH* out) {
    delete static_cast<Impl*>(out->impl);
    out->impl = nullptr;
    out->nodes = nullptr;
    out->tris = nullptr;
    out->insts = nullptr;
    out->num_nodes = out->num_tris = out->num_inst_refs = 0;
}
