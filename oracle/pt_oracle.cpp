// pt_oracle.cpp - C entry points of the CPU oracle (liborc.so).
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
// cpu_baseline / reference legs of bench.py, never by the product library.
// See pt_oracle.hpp for what is restated from where.
#include "pt_oracle.hpp"

#include <omp.h>

using namespace orc;

namespace {

template <class R> int render_impl(const pt_scene_desc* d, const pt_render_options* o, const pt_camera* cam,
                                   int first_pass, int num_passes, int row_start, int row_step, int nthreads,
                                   float* accum, float* accum_sq, uint64_t* counters, int cull) {
    Scene<R> s;
    MakeScene(s, d, o);
    s.cull = cull != 0;
    const int W = o->render_width, H = o->render_height;
    if (row_step < 1) row_step = 1;
    if (nthreads > 0) omp_set_num_threads(nthreads);
    uint64_t c_closest = 0, c_shadow = 0, c_nodes = 0, c_tris = 0, c_overflow = 0, c_paths = 0, c_hits = 0;
    uint64_t c_nodes_any = 0, c_tris_any = 0, c_inner = 0;
    std::vector<int> rows;
    for (int y = row_start; y < H; y += row_step) rows.push_back(y);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : c_closest, c_shadow, c_nodes, c_tris, c_overflow, c_paths, c_hits, c_nodes_any, c_tris_any, c_inner)
    for (int ri = 0; ri < (int)rows.size(); ++ri) {
        const int py = rows[ri];
        Counters cnt;
        for (int px = 0; px < W; ++px) {
            float* a = accum + 4 * ((size_t)py * W + px);
            double sq[3] = {0, 0, 0};
            for (int pass = first_pass; pass < first_pass + num_passes; ++pass) {
                const int tx = px / o->tile_width, ty = py / o->tile_height;
                const int lx = px - tx * o->tile_width, ly = py - ty * o->tile_height;
                Rng rng;
                rng.init((uint32_t)lx, (uint32_t)ly, FrameNumber(*o, pass, tx, ty));
                Ray<R> ray = CameraRay<R>(*cam, *o, px, py, rng);
                R alpha;
                V3<R> L = PathTrace(s, ray, rng, cnt, alpha);
                float lf[4] = {float(L.x), float(L.y), float(L.z), float(alpha)};
                // float accumulation per sample, as the RGBA32F accumTexture does (tile.glsl:70-74)
                for (int c = 0; c < 4; ++c) a[c] += lf[c];
                for (int c = 0; c < 3; ++c) sq[c] += double(lf[c]) * lf[c];
                c_paths++;
            }
            if (accum_sq) {
                float* q = accum_sq + 3 * ((size_t)py * W + px);
                for (int c = 0; c < 3; ++c) q[c] += float(sq[c]);
            }
        }
        c_closest += cnt.closest; c_shadow += cnt.shadow; c_nodes += cnt.nodes; c_tris += cnt.tris;
        c_overflow += cnt.overflow; c_hits += cnt.tri_hits;
        c_nodes_any += cnt.nodes_any; c_tris_any += cnt.tris_any; c_inner += cnt.inner;
    }
    if (counters) {
        counters[0] = c_closest; counters[1] = c_shadow; counters[2] = c_nodes;
        counters[3] = c_tris; counters[4] = c_overflow; counters[5] = c_paths; counters[6] = c_hits;
        counters[7] = c_nodes_any; counters[8] = c_tris_any; counters[9] = c_inner;
    }
    return 0;
}

template <class R> int trace_closest_impl(const pt_scene_desc* d, const pt_ray* rays, int n, pt_hit* hits,
                                          int mode, uint64_t* counters) {
    pt_render_options o{};
    o.max_depth = 1;
    Scene<R> s;
    MakeScene(s, d, &o);
    uint64_t nodes = 0, tris = 0, overflow = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : nodes, tris, overflow)
    for (int i = 0; i < n; ++i) {
        Ray<R> r{V3<R>(R(rays[i].origin[0]), R(rays[i].origin[1]), R(rays[i].origin[2])),
                 V3<R>(R(rays[i].direction[0]), R(rays[i].direction[1]), R(rays[i].direction[2]))};
        TriHit<R> h;
        h.t = K<R>::INF;
        Counters c;
        TraverseClosest(s, r, K<R>::INF, h, &c, mode);
        nodes += c.nodes; tris += c.tris; overflow += c.overflow;
        pt_hit& o2 = hits[i];
        if (h.prim >= 0) {
            o2.t = float(h.t); o2.u = float(h.u); o2.v = float(h.v);
            o2.prim_id = h.prim; o2.inst_id = h.inst;
        } else {
            o2.t = 1000000.0f; o2.u = o2.v = 0.0f; o2.prim_id = -1; o2.inst_id = -1;
        }
    }
    if (counters) { counters[0] = nodes; counters[1] = tris; counters[2] = overflow; }
    return 0;
}

template <class R> int trace_any_impl(const pt_scene_desc* d, const pt_render_options* o, const pt_ray* rays,
                                      const float* maxd, int n, uint8_t* occ) {
    Scene<R> s;
    MakeScene(s, d, o);
    // the test hook checks the BVH only (analytic lights are left out)
    s.f.lights = false;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i) {
        Ray<R> r{V3<R>(R(rays[i].origin[0]), R(rays[i].origin[1]), R(rays[i].origin[2])),
                 V3<R>(R(rays[i].direction[0]), R(rays[i].direction[1]), R(rays[i].direction[2]))};
        Rng rng;
        rng.init(uint32_t(i), 0u, 0u);
        Counters c;
        occ[i] = AnyHit(s, r, R(maxd[i]), rng, c) ? 1 : 0;
    }
    return 0;
}

// Shading-state record used by the BSDF entry points (20 floats):
//  0-2 baseColor, 3 metallic, 4 roughness, 5 subsurface, 6 specularTint,
//  7 sheen, 8 sheenTint, 9 clearcoat, 10 clearcoatRoughness, 11 specTrans,
//  12 ior, 13 ax, 14 ay, 15 eta, 16 anisotropic, 17-19 unused
template <class R> State<R> state_from(const float* p) {
    State<R> st;
    Material<R>& m = st.mat;
    m.baseColor = V3<R>(R(p[0]), R(p[1]), R(p[2]));
    m.metallic = R(p[3]); m.roughness = R(p[4]); m.subsurface = R(p[5]); m.specularTint = R(p[6]);
    m.sheen = R(p[7]); m.sheenTint = R(p[8]); m.clearcoat = R(p[9]); m.clearcoatRoughness = R(p[10]);
    m.specTrans = R(p[11]); m.ior = R(p[12]); m.ax = R(p[13]); m.ay = R(p[14]);
    st.eta = R(p[15]); m.anisotropic = R(p[16]);
    return st;
}

template <class R> V3<R> v3_at(const float* p, int i) { return V3<R>(R(p[3 * i]), R(p[3 * i + 1]), R(p[3 * i + 2])); }

template <class R> int bsdf_eval_impl(int n, const float* sp, const float* V, const float* N, const float* L,
                                      double* f, double* pdf, double* lobe_f, double* lobe_pdf) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        State<R> st = state_from<R>(sp + 20 * (size_t)i);
        R p;
        LobeEval<R> parts;
        V3<R> r = DisneyEval(st, v3_at<R>(V, i), v3_at<R>(N, i), v3_at<R>(L, i), p, &parts);
        f[3 * i] = double(r.x); f[3 * i + 1] = double(r.y); f[3 * i + 2] = double(r.z);
        pdf[i] = double(p);
        if (lobe_f) for (int k = 0; k < 5; ++k) {
            lobe_f[15 * i + 3 * k] = double(parts.f[k].x);
            lobe_f[15 * i + 3 * k + 1] = double(parts.f[k].y);
            lobe_f[15 * i + 3 * k + 2] = double(parts.f[k].z);
            lobe_pdf[5 * i + k] = double(parts.pdf[k]);
        }
    }
    return 0;
}

template <class R> int bsdf_sample_impl(int n, const float* sp, const float* V, const float* N, const uint32_t* seeds,
                                        double* Lout, double* f, double* pdf) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        State<R> st = state_from<R>(sp + 20 * (size_t)i);
        Rng rng;
        for (int k = 0; k < 4; ++k) rng.s[k] = seeds[4 * (size_t)i + k];
        R p;
        V3<R> L;
        V3<R> r = DisneySample(st, v3_at<R>(V, i), v3_at<R>(N, i), L, p, rng);
        Lout[3 * i] = double(L.x); Lout[3 * i + 1] = double(L.y); Lout[3 * i + 2] = double(L.z);
        f[3 * i] = double(r.x); f[3 * i + 1] = double(r.y); f[3 * i + 2] = double(r.z);
        pdf[i] = double(p);
    }
    return 0;
}

}  // namespace

extern "C" {

// Renders sample passes [first_pass, first_pass+num_passes) of rows
// row_start, row_start+row_step, ... and ADDS them into accum (W*H*4 floats;
// RGB radiance + alpha) and accum_sq (W*H*3, sum of squares; may be NULL).
// counters (9 x uint64): closest-hit queries, shadow queries, node visits,
// triangle tests, stack overflows, paths, triangle hits of closest-hit
// queries, and the node visits and triangle tests of the any-hit queries
// alone (already included in the totals).
// cull = 1 counts node visits / triangle tests of a tmax-culled traversal
// (same hits; the work counts define the roofline's bytes per ray).
int orc_render(const pt_scene_desc* d, const pt_render_options* o, const pt_camera* cam, int first_pass,
               int num_passes, int use_double, int row_start, int row_step, int nthreads, float* accum,
               float* accum_sq, uint64_t* counters, int cull) {
    if (!d || !o || !cam || !accum) return 1;
    return use_double ? render_impl<double>(d, o, cam, first_pass, num_passes, row_start, row_step, nthreads, accum, accum_sq, counters, cull)
                      : render_impl<float>(d, o, cam, first_pass, num_passes, row_start, row_step, nthreads, accum, accum_sq, counters, cull);
}

// Closest triangle hit per ray over the flattened BVH.  mode 0: the
// reference's traversal; mode 1: with tmax culling.  counters (3 x uint64):
// node visits, triangle tests, stack overflows.
int orc_trace_closest(const pt_scene_desc* d, const pt_ray* rays, int n, pt_hit* hits, int mode, int use_double,
                      uint64_t* counters) {
    if (!d || (!rays && n) || (!hits && n)) return 1;
    return use_double ? trace_closest_impl<double>(d, rays, n, hits, mode, counters)
                      : trace_closest_impl<float>(d, rays, n, hits, mode, counters);
}

int orc_trace_any(const pt_scene_desc* d, const pt_render_options* o, const pt_ray* rays, const float* maxd, int n,
                  uint8_t* occ, int use_double) {
    if (!d || !o) return 1;
    return use_double ? trace_any_impl<double>(d, o, rays, maxd, n, occ) : trace_any_impl<float>(d, o, rays, maxd, n, occ);
}

// The detached estimator (PathTraceDetached) of sample passes
// [first_pass, first_pass+num_passes): sampling from scene d, values from
// scene e (same geometry, other materials / lights).  ADDS radiance (RGB,
// FP64 sums) into accum (W*H*3 doubles).
int orc_render_detached(const pt_scene_desc* d, const pt_scene_desc* e, const pt_render_options* o,
                        const pt_camera* cam, int first_pass, int num_passes, int use_double, int nthreads,
                        double* accum) {
    auto run = [&](auto tag) {
        using R = decltype(tag);
        Scene<R> s, se;
        MakeScene(s, d, o);
        MakeScene(se, e, o);
        const int W = o->render_width, H = o->render_height;
        if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
        for (int py = 0; py < H; ++py) {
            Counters cnt;
            for (int px = 0; px < W; ++px) {
                double* a = accum + 3 * ((size_t)py * W + px);
                for (int pass = first_pass; pass < first_pass + num_passes; ++pass) {
                    const int tx = px / o->tile_width, ty = py / o->tile_height;
                    const int lx = px - tx * o->tile_width, ly = py - ty * o->tile_height;
                    Rng rng;
                    rng.init((uint32_t)lx, (uint32_t)ly, FrameNumber(*o, pass, tx, ty));
                    Ray<R> ray = CameraRay<R>(*cam, *o, px, py, rng);
                    V3<R> L = PathTraceDetached(s, se, ray, rng, cnt);
                    a[0] += double(L.x);
                    a[1] += double(L.y);
                    a[2] += double(L.z);
                }
            }
        }
    };
    if (use_double) run(double{});
    else run(float{});
    return 0;
}

int orc_bsdf_eval(int n, const float* state_params, const float* V, const float* N, const float* L, int use_double,
                  double* f, double* pdf, double* lobe_f, double* lobe_pdf) {
    return use_double ? bsdf_eval_impl<double>(n, state_params, V, N, L, f, pdf, lobe_f, lobe_pdf)
                      : bsdf_eval_impl<float>(n, state_params, V, N, L, f, pdf, lobe_f, lobe_pdf);
}

int orc_bsdf_sample(int n, const float* state_params, const float* V, const float* N, const uint32_t* seeds,
                    int use_double, double* L, double* f, double* pdf) {
    return use_double ? bsdf_sample_impl<double>(n, state_params, V, N, seeds, L, f, pdf)
                      : bsdf_sample_impl<float>(n, state_params, V, N, seeds, L, f, pdf);
}

// Camera rays of tile.glsl for a list of pixels in pass `pass`, plus the RNG
// state right after generating them (4 x uint32 per pixel).
int orc_camera_rays(const pt_render_options* o, const pt_camera* cam, int pass, int n, const int32_t* px,
                    const int32_t* py, pt_ray* rays, uint32_t* rng_state) {
    for (int i = 0; i < n; ++i) {
        const int tx = px[i] / o->tile_width, ty = py[i] / o->tile_height;
        Rng rng;
        rng.init((uint32_t)(px[i] - tx * o->tile_width), (uint32_t)(py[i] - ty * o->tile_height), FrameNumber(*o, pass, tx, ty));
        Ray<float> r = CameraRay<float>(*cam, *o, px[i], py[i], rng);
        rays[i].origin[0] = r.origin.x; rays[i].origin[1] = r.origin.y; rays[i].origin[2] = r.origin.z;
        rays[i].direction[0] = r.direction.x; rays[i].direction[1] = r.direction.y; rays[i].direction[2] = r.direction.z;
        if (rng_state) for (int k = 0; k < 4; ++k) rng_state[4 * i + k] = rng.s[k];
    }
    return 0;
}

// The full ClosestHit (lights + triangles + shading normal) on a ray set,
// with State.depth = 1 so that emitters are intersected; the outputs match
// ref_glsl_closest_hit of the reference build.
int orc_closest_hit_full(const pt_scene_desc* d, const pt_ray* rays, int n, int* hit, float* t, int* matID,
                         int* isEmitter, float* normal) {
    pt_render_options o{};
    o.max_depth = 1;
    Scene<float> s;
    MakeScene(s, d, &o);
    for (int i = 0; i < n; ++i) {
        Ray<float> r{V3<float>(rays[i].origin[0], rays[i].origin[1], rays[i].origin[2]),
                     V3<float>(rays[i].direction[0], rays[i].direction[1], rays[i].direction[2])};
        State<float> st;
        st.depth = 1;
        st.matID = -1;
        LightSampleRec<float> ls;
        Counters c;
        bool h = ClosestHit(s, r, st, ls, c);
        hit[i] = h ? 1 : 0;
        t[i] = h ? st.hitDist : 1000000.0f;
        matID[i] = h ? st.matID : -1;
        isEmitter[i] = h && st.isEmitter ? 1 : 0;
        normal[3 * i] = st.normal.x; normal[3 * i + 1] = st.normal.y; normal[3 * i + 2] = st.normal.z;
    }
    return 0;
}

// PCG4D stream: n values of rand() from the seed (px, py, frame).
int orc_rng_stream(uint32_t px, uint32_t py, uint32_t frame, int n, float* out) {
    Rng rng;
    rng.init(px, py, frame);
    for (int i = 0; i < n; ++i) out[i] = rng.next();
    return 0;
}

}  // extern "C"
