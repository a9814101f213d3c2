// sah_builder.h - binned-SAH binary BVH builder (host), shared by the scene
// builder (scene_build.cpp) and the BVH collapse (bvh8_build.cpp).
//
// 64 centroid bins per axis, traversal cost 2, leaves of up to `max_leaf`
// primitives: the parameters of the reference's per-mesh SplitBvh
// (src/core/Mesh.h:37) with spatial splits disabled.  With sah = false the
// split is at the centre of the centroid bounds of the longest axis, as the
// reference's TLAS Bvh(10.0f, 64, false) does (src/core/Scene.h:70).
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

namespace ptgb {
namespace sah {

struct AABB {
    float lo[3], hi[3];
    AABB() { for (int k = 0; k < 3; ++k) { lo[k] = INFINITY; hi[k] = -INFINITY; } }
    void grow(const AABB& b) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
    }
    void grow(const float* p) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); }
    }
    float area() const {
        float d[3];
        for (int k = 0; k < 3; ++k) d[k] = std::max(0.0f, hi[k] - lo[k]);
        return 2.0f * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
    }
};

struct Ref {
    AABB b;
    float c[3];
    int idx;
};

// Binary node: children indices into the node array, or a leaf range of
// `packed` (the primitive indices in leaf order).
struct Node {
    AABB box;
    int left = -1, right = -1;
    int start = 0, count = 0;
};

struct Builder {
    std::vector<Ref> refs;
    std::vector<Node> nodes;
    std::vector<int> packed;
    bool sah = true;
    int max_leaf = 3;
    float trav_cost = 2.0f;
    static constexpr int kBins = 64;

    // Builds the tree over refs[begin, end) and returns the root index.
    int build(int begin, int end) {
        const int id = (int)nodes.size();
        nodes.emplace_back();
        AABB box, cbox;
        for (int i = begin; i < end; ++i) {
            box.grow(refs[i].b);
            cbox.grow(refs[i].c);
        }
        nodes[id].box = box;
        const int n = end - begin;
        if (n <= max_leaf) {
            nodes[id].start = (int)packed.size();
            nodes[id].count = n;
            for (int i = begin; i < end; ++i) packed.push_back(refs[i].idx);
            return id;
        }
        int axis = 0;
        float ext[3];
        for (int k = 0; k < 3; ++k) ext[k] = cbox.hi[k] - cbox.lo[k];
        if (ext[1] > ext[axis]) axis = 1;
        if (ext[2] > ext[axis]) axis = 2;
        int mid = -1;
        if (ext[axis] > 0.0f) {
            if (sah) {
                float best = INFINITY;
                int best_axis = -1, best_bin = -1;
                const float inv_area = 1.0f / std::max(box.area(), 1e-30f);
                for (int k = 0; k < 3; ++k) {
                    if (!(ext[k] > 0.0f)) continue;
                    AABB bb[kBins];
                    int cnt[kBins] = {0};
                    const float scale = kBins / ext[k];
                    for (int i = begin; i < end; ++i) {
                        int b = std::min(kBins - 1, (int)((refs[i].c[k] - cbox.lo[k]) * scale));
                        cnt[b]++;
                        bb[b].grow(refs[i].b);
                    }
                    float right_area[kBins];
                    int right_cnt[kBins];
                    AABB acc;
                    int ac = 0;
                    for (int b = kBins - 1; b > 0; --b) {
                        acc.grow(bb[b]);
                        ac += cnt[b];
                        right_area[b] = acc.area();
                        right_cnt[b] = ac;
                    }
                    AABB left;
                    int lc = 0;
                    for (int b = 0; b < kBins - 1; ++b) {
                        left.grow(bb[b]);
                        lc += cnt[b];
                        if (lc == 0 || right_cnt[b + 1] == 0) continue;
                        float cost = trav_cost + (lc * left.area() + right_cnt[b + 1] * right_area[b + 1]) * inv_area;
                        if (cost < best) { best = cost; best_axis = k; best_bin = b; }
                    }
                }
                if (best_axis >= 0) {
                    const int k = best_axis;
                    const float scale = kBins / ext[k];
                    auto it = std::partition(refs.begin() + begin, refs.begin() + end, [&](const Ref& r) {
                        return std::min(kBins - 1, (int)((r.c[k] - cbox.lo[k]) * scale)) <= best_bin;
                    });
                    mid = (int)(it - refs.begin());
                }
            } else {
                const float border = 0.5f * (cbox.lo[axis] + cbox.hi[axis]);
                auto it = std::partition(refs.begin() + begin, refs.begin() + end,
                                         [&](const Ref& r) { return r.c[axis] < border; });
                mid = (int)(it - refs.begin());
            }
        }
        if (mid <= begin || mid >= end) {  // degenerate: split the range in half
            mid = begin + n / 2;
            std::nth_element(refs.begin() + begin, refs.begin() + mid, refs.begin() + end,
                             [&](const Ref& a, const Ref& b) { return a.c[axis] < b.c[axis]; });
        }
        const int l = build(begin, mid);
        const int r = build(mid, end);
        nodes[id].left = l;
        nodes[id].right = r;
        return id;
    }
};

}  // namespace sah
}  // namespace ptgb
