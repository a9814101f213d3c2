// pt_capi.cu - the C ABI of include/pt_cuda.h: one context per renderer,
// owning the device copies of the scene, the accumulation buffer and a
// CUDA stream.  Replaces GLSLPT::Renderer's GL resource management
// (src/core/Renderer.cpp:41-249, 619-811).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cmath>
#include <cstdlib>

#include "../../include/pt_cuda.h"
#include "bvh8.h"
#include "pt_device.cuh"
#include "pt_params.h"
#include "pt_bvh_gpu.h"
#include "pt_grad.cuh"
#include "pt_wavefront.h"

using namespace ptgb;

namespace {

thread_local std::string g_err;

int set_err(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

int cuda_err(cudaError_t e, const char* what) {
    const int code = e == cudaErrorMemoryAllocation ? PT_ERR_OUT_OF_MEMORY : PT_ERR_CUDA;
    return set_err(code, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_err(e_, #call);    \
    } while (0)

template <class T> struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count) {
        free();
        n = count;
        if (!count) return cudaSuccess;
        return cudaMalloc((void**)&p, count * sizeof(T));
    }
    cudaError_t upload(const void* src, size_t count, cudaStream_t s) {
        if (count != n) {
            cudaError_t e = alloc(count);
            if (e != cudaSuccess) return e;
        }
        if (!count) return cudaSuccess;
        return cudaMemcpyAsync(p, src, count * sizeof(T), cudaMemcpyHostToDevice, s);
    }
    void free() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

}  // namespace

struct pt_context {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timed = false;
    pt_render_options opts{};
    pt_camera cam{};
    int integrator = PT_INTEGRATOR_MEGAKERNEL;
    uint32_t scene_flags = 0;  // F_ALPHA_TEST / F_MEDIUM / F_LIGHTS from the scene
    bool has_env = false;
    WideBVH bvh{};
    std::vector<float> bin_nodes;  // host copy of the binary BVH (TLAS updates)
    int top_level_index = 0;
    // VOL_MIS transmittance queries whose contribution is never added may go
    // untraced (Params::untraced bit 1): world boxes of the blended-alpha
    // instances (update_blend_boxes)
    std::vector<float> host_mats;
    DevBuf<float> blend_boxes;
    int num_blend_boxes = 0;
    bool untraced_transmit = false;
    int num_tris = 0, num_vertices = 0, num_materials = 0, num_instances = 0, num_lights = 0;
    int env_w = 0, env_h = 0;
    float env_total = 0.0f;
    DevBuf<WideNode> nodes;
    DevBuf<WideTri> tris;
    DevBuf<InstRef> insts;
    DevBuf<InstXf> xf;
    DevBuf<uint4> inst_bounds;  // root_may_hit's bounds per InstRef (empty: no culling)
    DevBuf<uint4> node_words;   // each wide node's per-slot hit-mask words
    DevBuf<int32_t> vidx;
    DevBuf<float4> verts, norms, mats, lights, env;
    DevBuf<float> cdf;
    DevBuf<uchar4> tex;
    int tex_w = 0, tex_h = 0, num_tex = 0;
    DevBuf<float4> accum;
    DevBuf<float4> snapshot;
    DevBuf<uchar4> ldr;
    DevBuf<unsigned long long> counters;
    DevBuf<int> status;
    pt_stats last{};
    WavefrontBuffers wf;
    WavefrontTuning wf_tuning;
    bool wf_tuned = false;
    // the TLAS holds one untransformed instance: traversal starts in its BLAS
    bool direct = false;
    InstRef entry{};
    int launches = 0;  // kernels launched by the last render call
    bool stage_timing = false;
    StageTimer timer;
    // traversal stack bound of the kernels: kStackSize, or lower when
    // PT_TRAVERSAL_STACK_LIMIT is set at pt_create (failure-detection tests
    // make the overflow status fire with it)
    int stack_limit = kStackSize;
    // scene / camera / options version, and the forward wavefront batch the
    // path buffers hold (the adjoint reuses its per-path radiance)
    uint64_t version = 1;
    struct {
        bool valid = false;
        RenderWork w{};
        uint64_t version = 0;
    } fwd;
    // the BVH built on the GPU (pt_create_gpu_bvh): meshes and instances
    bool gpu_bvh = false;
    std::vector<int> mesh_tri_offset, inst_mesh, inst_material;
    float gpu_build_ms = 0.0f;
    // adjoint buffers
    DevBuf<float4> adj_v, adj_le;
    DevBuf<float> adj_dimage, adj_grad;
};

namespace {

// The bounds root_may_hit (pt_trace.cuh) tests per InstRef: word 0 of the
// BLAS root (internal-child mask cleared), then the smallest qlo and largest
// qhi byte per axis over the root's non-empty slots (bvh8.h's layout).
__global__ void k_inst_bounds(const WideNode* __restrict__ nodes, const InstRef* __restrict__ refs, int count,
                              uint4* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint32_t* w = nodes[refs[i].blas_root].w;
    uint32_t lo[3] = {255u, 255u, 255u}, hi[3] = {0u, 0u, 0u};
    for (int slot = 0; slot < 8; ++slot) {
        const int word = slot >> 2, sh = 8 * (slot & 3);
        if (!((w[6 + word] >> sh) & 0xffu)) continue;  // meta 0: empty slot
        for (int k = 0; k < 3; ++k) {
            lo[k] = min(lo[k], (w[8 + 2 * k + word] >> sh) & 0xffu);       // w2.xy, w2.zw, w3.xy
            hi[k] = max(hi[k], (w[14 + 2 * k + word] >> sh) & 0xffu);      // w3.zw, w4.xy, w4.zw
        }
    }
    out[2 * i] = make_uint4(w[0], w[1], w[2], w[3] & 0x00ffffffu);
    out[2 * i + 1] = make_uint4(lo[0] | lo[1] << 8 | lo[2] << 16, hi[0] | hi[1] << 8 | hi[2] << 16, 0u, 0u);
}

// Per wide node, the word each slot adds to the node test's hit mask
// (intersect_node): a leaf child's triangle (or instance) bits at its
// offset, an internal child's bit 24 + slot, 0 for an empty slot.
__global__ void k_node_words(const WideNode* __restrict__ nodes, int count, uint4* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    uint32_t w[8];
    for (int slot = 0; slot < 8; ++slot) {
        const uint32_t m = (nodes[i].w[6 + (slot >> 2)] >> (8 * (slot & 3))) & 0xffu;
        const bool inner = ((m & (m << 1)) & 0x10u) != 0;
        w[slot] = m == 0 ? 0u : inner ? 1u << (24 + slot) : (m >> 5) << (m & 0x1fu);
    }
    out[2 * i] = make_uint4(w[0], w[1], w[2], w[3]);
    out[2 * i + 1] = make_uint4(w[4], w[5], w[6], w[7]);
}

cudaError_t make_node_words(DevBuf<uint4>& out, const WideNode* nodes, int count, cudaStream_t s) {
    if (count <= 0) {
        out.free();
        return cudaSuccess;
    }
    if (out.n != 2 * (size_t)count) {
        cudaError_t e = out.alloc(2 * (size_t)count);
        if (e != cudaSuccess) return e;
    }
    k_node_words<<<(count + 255) / 256, 256, 0, s>>>(nodes, count, out.p);
    return cudaGetLastError();
}

bool instance_culling_enabled() {
    const char* v = std::getenv("PT_INSTANCE_BOUNDS");
    return !(v && v[0] == '0');
}

// (Re)computes the instance bounds of `count` InstRefs over `nodes`; left
// empty when PT_INSTANCE_BOUNDS=0 (every instance entered, for comparison).
cudaError_t make_inst_bounds(DevBuf<uint4>& out, const WideNode* nodes, const InstRef* refs, int count,
                             cudaStream_t s) {
    if (!instance_culling_enabled() || count <= 0) {
        out.free();
        return cudaSuccess;
    }
    if (out.n != 2 * (size_t)count) {
        cudaError_t e = out.alloc(2 * (size_t)count);
        if (e != cudaSuccess) return e;
    }
    k_inst_bounds<<<(count + 255) / 256, 256, 0, s>>>(nodes, refs, count, out.p);
    return cudaGetLastError();
}

uint32_t option_flags(const pt_context* c) {
    const pt_render_options& o = c->opts;
    uint32_t f = c->scene_flags;
    if (o.enable_rr) f |= F_RR;
    if (o.enable_uniform_light) f |= F_UNIFORM_LIGHT;
    if (o.hide_emitters) f |= F_HIDE_EMITTERS;
    if (o.enable_background || o.transparent_background) f |= F_BACKGROUND;
    if (o.enable_roughness_mollification) f |= F_MOLLIFY;
    if (o.enable_envmap && c->has_env && !o.enable_uniform_light) f |= F_ENVMAP;
    if (o.enable_volume_mis) f |= F_VOL_MIS;
    if (o.opengl_normal_map) f |= F_OPENGL_NORMALMAP;
    if (c->num_tex > 0) f |= F_TEXTURES;
    return f;
}

// Params::untraced for a render: PT_UNTRACED_SHADOWS=0 traces every shadow
// query (the same images; for comparisons).
int untraced_bits(bool transmit) {
    const char* e = std::getenv("PT_UNTRACED_SHADOWS");
    if (e && std::atoi(e) == 0) return 0;
    return 1 | (transmit ? 2 : 0);
}

Params make_params(const pt_context* c) {
    Params p{};
    p.nodes = reinterpret_cast<const uint4*>(c->nodes.p);
    p.tris = reinterpret_cast<const float4*>(c->tris.p);
    p.insts = reinterpret_cast<const int4*>(c->insts.p);
    p.xf = reinterpret_cast<const float4*>(c->xf.p);
    p.inst_bounds = c->inst_bounds.p;
    p.node_words = c->node_words.p;
    p.tlas_root = c->bvh.tlas_root;
    if (c->direct) {
        p.tlas_root = c->entry.blas_root;
        p.direct = 1;
        p.entry_inst = c->entry.instance;
        p.entry_mat = c->entry.material;
    }
    p.vidx = c->vidx.p;
    p.verts = c->verts.p;
    p.norms = c->norms.p;
    p.mats = c->mats.p;
    p.lights = c->lights.p;
    p.num_lights = c->num_lights;
    p.num_materials = c->num_materials;
    p.env = c->env.p;
    p.cdf = c->cdf.p;
    p.env_w = c->env_w;
    p.env_h = c->env_h;
    p.env_total = c->env_total;
    p.tex = c->tex.p;
    p.tex_w = c->tex_w;
    p.tex_h = c->tex_h;
    p.num_tex = c->num_tex;
    p.env_intensity = c->opts.envmap_intensity;
    p.env_rot = c->opts.envmap_rot / 360.0f;  // Renderer.cpp:778
    p.flags = option_flags(c);
    p.max_depth = c->opts.max_depth;
    p.rr_depth = c->opts.rr_depth;
    for (int i = 0; i < 3; ++i) {
        p.uniform_light[i] = c->opts.uniform_light_col[i];
        p.cam_pos[i] = c->cam.position[i];
        p.cam_up[i] = c->cam.up[i];
        p.cam_right[i] = c->cam.right[i];
        p.cam_fwd[i] = c->cam.forward[i];
    }
    p.mollify_amt = c->opts.roughness_mollification_amt;
    p.cam_fov = c->cam.fov;
    p.cam_focal = c->cam.focal_dist;
    p.cam_aperture = c->cam.aperture;
    p.width = c->opts.render_width;
    p.height = c->opts.render_height;
    p.tile_w = c->opts.tile_width;
    p.tile_h = c->opts.tile_height;
    p.ntx = (p.width + p.tile_w - 1) / p.tile_w;
    p.nty = (p.height + p.tile_h - 1) / p.tile_h;
    p.accum = c->accum.p;
    p.counters = c->counters.p;
    p.status = c->status.p;
    p.stack_limit = c->stack_limit;
    p.untraced = untraced_bits(c->untraced_transmit);
    p.blend_boxes = c->blend_boxes.p;
    p.num_blend_boxes = c->num_blend_boxes;
    return p;
}

int check_options(const pt_render_options* o) {
    if (!o) return set_err(PT_ERR_INVALID_ARG, "options is NULL");
    if (o->render_width <= 0 || o->render_height <= 0 || o->render_width > 32768 || o->render_height > 32768)
        return set_err(PT_ERR_INVALID_ARG, "render resolution out of range");
    if (o->tile_width <= 0 || o->tile_height <= 0) return set_err(PT_ERR_INVALID_ARG, "tile size must be positive");
    if (o->max_depth < 0 || o->max_depth > 1024) return set_err(PT_ERR_INVALID_ARG, "max_depth out of range");
    return PT_OK;
}

// TLAS leaves (LRLeaf.z < 0) carry the instance's material index in LRLeaf.y.
int check_tlas_materials(const float* tlas_nodes, int n, int num_materials) {
    for (int i = 0; i < n; ++i) {
        const float* p = tlas_nodes + 9 * (size_t)i;
        if (p[8] < 0.0f && (p[7] < 0.0f || p[7] >= (float)num_materials))
            return set_err(PT_ERR_INVALID_ARG, "TLAS leaf material index out of range");
    }
    return PT_OK;
}

// Lights repacked as 4 float4 (pt_device.cuh LoadLight) from GLSLPT::Light's
// 15 floats: position, emission, u, v, radius, area, type (Scene.h:50-59).
int upload_lights(pt_context* c, const float* lights, int n) {
    std::vector<float4> L(4 * (size_t)std::max(1, n));
    for (int i = 0; i < n; ++i) {
        const float* s = lights + 15 * (size_t)i;
        L[4 * i + 0] = make_float4(s[0], s[1], s[2], s[12]);
        L[4 * i + 1] = make_float4(s[3], s[4], s[5], s[13]);
        L[4 * i + 2] = make_float4(s[6], s[7], s[8], s[14]);
        L[4 * i + 3] = make_float4(s[9], s[10], s[11], 0.0f);
    }
    CK(c->lights.upload(L.data(), L.size(), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

int upload_instances(pt_context* c, const float* transforms, int n) {
    std::vector<InstXf> xf(n);
    for (int i = 0; i < n; ++i) {
        int ident = 0;
        ptgb_instance_xf(transforms + 16 * (size_t)i, &xf[i], &ident);
    }
    CK(c->xf.upload(xf.data(), xf.size(), c->stream));
    return PT_OK;
}

int upload_bvh(pt_context* c) {
    CK(c->nodes.upload(c->bvh.nodes, c->bvh.num_nodes, c->stream));
    CK(c->tris.upload(c->bvh.tris, c->bvh.num_tris, c->stream));
    CK(c->insts.upload(c->bvh.insts, c->bvh.num_inst_refs, c->stream));
    CK(make_inst_bounds(c->inst_bounds, c->nodes.p, c->insts.p, c->bvh.num_inst_refs, c->stream));
    CK(make_node_words(c->node_words, c->nodes.p, c->bvh.num_nodes, c->stream));
    c->direct = c->bvh.num_inst_refs == 1 && c->bvh.insts[0].identity;
    if (c->direct) c->entry = c->bvh.insts[0];
    const int need = trav_stack_need(c->bvh.tlas_depth, c->bvh.blas_depth, c->direct);
    if (need > kStackSize)
        return set_err(PT_ERR_UNSUPPORTED, "BVH deeper than the traversal stack (" + std::to_string(need) +
                                               " entries needed, " + std::to_string(kStackSize) + " available)");
    return PT_OK;
}

int upload_envmap(pt_context* c, const float* rgb, const float* cdf, int w, int h, float total) {
    c->has_env = rgb != nullptr && cdf != nullptr && w > 0 && h > 0;
    if (!c->has_env) {
        c->env.free();
        c->cdf.free();
        c->env_w = c->env_h = 0;
        return PT_OK;
    }
    std::vector<float4> px((size_t)w * h);
    for (size_t i = 0; i < px.size(); ++i) px[i] = make_float4(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2], 0.0f);
    CK(c->env.upload(px.data(), px.size(), c->stream));
    CK(c->cdf.upload(cdf, (size_t)w * h, c->stream));
    c->env_w = w;
    c->env_h = h;
    c->env_total = total;
    CK(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

int alloc_accum(pt_context* c) {
    const size_t n = (size_t)c->opts.render_width * c->opts.render_height;
    if (c->accum.n != n) {
        CK(c->accum.alloc(n));
        c->ldr.free();
        c->snapshot.free();
    }
    CK(cudaMemsetAsync(c->accum.p, 0, n * sizeof(float4), c->stream));
    return PT_OK;
}

uint32_t scene_flags_of(const float* mats, int nm, int nl) {
    uint32_t f = 0;
    if (nl > 0) f |= F_LIGHTS;
    for (int i = 0; i < nm; ++i) {
        if ((int)mats[32 * i + 29] != ALPHA_MODE_OPAQUE) f |= F_ALPHA_TEST;  // Renderer.cpp:443-450
        if ((int)mats[32 * i + 18] != MEDIUM_NONE) f |= F_MEDIUM;            // Renderer.cpp:455-461
    }
    return f;
}

// Where VOL_MIS transmittance queries whose contribution is never added may
// go untraced (DirectLight): EvalTransmittance draws random numbers only at
// blended-alpha hits (pathtrace.glsl:133), so a query whose ray meets none
// of the blended instances' world boxes draws none; and it ends at its first
// hit (one segment) when no other instance's material is refractive or
// alpha-masked (pathtrace.glsl:134-138).  The boxes are the TLAS leaves of
// the reference's binary BVH, widened by 1e-4 of their largest coordinate
// plus 1e-4.  Not for BVHs built on the GPU (no binary TLAS), and not beyond
// kMaxBlendBoxes blended instances.
constexpr int kMaxBlendBoxes = 16;
int update_blend_boxes(pt_context* c) {
    c->untraced_transmit = false;
    c->num_blend_boxes = 0;
    if (c->gpu_bvh || c->bin_nodes.empty() || c->host_mats.empty()) return PT_OK;
    const float* mats = c->host_mats.data();
    const size_t total = c->bin_nodes.size() / 9;
    std::vector<float> boxes;
    for (size_t i = (size_t)c->top_level_index; i < total; ++i) {
        const float* p = c->bin_nodes.data() + 9 * i;
        if (!(p[8] < 0.0f)) continue;  // TLAS leaf: LRLeaf.z = -instance - 1, material in LRLeaf.y
        const float* m = mats + 32 * (size_t)(int)p[7];
        const int alpha = (int)m[29];
        if (alpha == ALPHA_MODE_BLEND) {
            if (boxes.size() >= 6 * (size_t)kMaxBlendBoxes) return PT_OK;
            double ext = 0.0;
            for (int k = 0; k < 6; ++k) ext = std::max(ext, std::fabs((double)p[k]));
            const float w = (float)(1e-4 * (1.0 + ext));
            for (int k = 0; k < 3; ++k) boxes.push_back(p[k] - w);
            for (int k = 3; k < 6; ++k) boxes.push_back(p[k] + w);
        } else if (alpha == ALPHA_MODE_MASK || m[16] > 0.0f) {  // masked, or specTrans > 0
            return PT_OK;
        }
    }
    CK(c->blend_boxes.upload(boxes.data(), boxes.size(), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->num_blend_boxes = (int)(boxes.size() / 6);
    c->untraced_transmit = true;
    return PT_OK;
}

// Texture ids of a material (Material.h:87-119, texIDs at 24..27) index the
// texture array; -1 is none.
int check_materials(const float* mats, int nm, int num_tex) {
    for (int i = 0; i < nm; ++i)
        for (int k = 24; k < 28; ++k)
            if ((int)mats[32 * i + k] >= num_tex)
                return set_err(PT_ERR_INVALID_ARG, "material " + std::to_string(i) + " uses texture " +
                                                       std::to_string((int)mats[32 * i + k]) + " of " +
                                                       std::to_string(num_tex));
    return PT_OK;
}

int begin_launch(pt_context* c) {
    CK(cudaMemsetAsync(c->counters.p, 0, 5 * sizeof(unsigned long long), c->stream));
    CK(cudaMemsetAsync(c->status.p, 0, sizeof(int), c->stream));
    CK(cudaEventRecord(c->ev0, c->stream));
    return PT_OK;
}

int end_launch(pt_context* c) {
    CK(cudaEventRecord(c->ev1, c->stream));
    c->timed = true;
    return PT_OK;
}

// Paths per wavefront batch: PT_WAVEFRONT_CAPACITY (default 2^25, about
// 9.5 GB of path state: a 16-spp 1080p frame in one batch), at least one
// full pass of the frame.
int wavefront_capacity(const pt_context* c, const RenderWork& w) {
    long cap = 1L << 25;
    if (const char* s = std::getenv("PT_WAVEFRONT_CAPACITY")) cap = std::max(1L, std::atol(s));
    const long npix = (long)w.w * w.h;
    const long want = std::min((long)w.num_passes * npix, std::max(cap, npix));
    return (int)std::min(want, (long)INT32_MAX / 2);
}

int render(pt_context* c, const RenderWork& w) {
    if (int rc = begin_launch(c)) return rc;
    const Params p = make_params(c);
    if (c->integrator == PT_INTEGRATOR_WAVEFRONT) {
        const int cap = wavefront_capacity(c, w);
        if (c->wf.capacity < cap) CK(wavefront_alloc(c->wf, cap));
        if (!c->wf_tuned) {
            CK(wavefront_default_tuning(c->wf_tuning, 128));
            c->wf_tuned = true;
        }
        const char* g = std::getenv("PT_WAVEFRONT_GRAPH");
        const bool use_graph = !(g && g[0] == '0');
        WavefrontTuning t = c->wf_tuning;
        if (!trav_postpone_fits(c->bvh.tlas_depth + c->bvh.blas_depth)) t.min_tris = t.min_tris_first = t.min_tris_shadow_first = 0;
        c->timer.reset();
        c->fwd.valid = false;
        CK(launch_wavefront(p, w, c->wf, t, use_graph, c->stream, &c->launches,
                            c->stage_timing ? &c->timer : nullptr));
        // one batch: the path buffers keep every path of this work
        if (!(p.flags & F_ALPHA_TEST) && (long)w.w * w.h * w.num_passes <= c->wf.capacity) {
            c->fwd.valid = true;
            c->fwd.w = w;
            c->fwd.version = c->version;
        }
    } else {
        CK(launch_render(p, w, c->integrator, c->stream));
        c->launches = 1;
    }
    return end_launch(c);
}

}  // namespace

extern "C" {

int pt_last_error(char* buf, size_t size) {
    if (!buf || !size) return PT_ERR_INVALID_ARG;
    std::snprintf(buf, size, "%s", g_err.c_str());
    return PT_OK;
}

}  // extern "C"

namespace {
// The BVH of a context built on the GPU from its meshes (pt_bvh_gpu.cu);
// the previous arrays are replaced only when the build succeeds.
int gpu_rebuild(pt_context* c, const float* transforms) {
    GpuBuildInput in;
    in.verts = c->verts.p;
    in.vidx = c->vidx.p;
    in.mesh_tri_offset = c->mesh_tri_offset.data();
    in.num_meshes = (int)c->mesh_tri_offset.size() - 1;
    in.transforms = transforms;
    in.inst_mesh = c->inst_mesh.data();
    in.inst_material = c->inst_material.data();
    in.num_instances = (int)c->inst_mesh.size();
    GpuBvh g;
    std::string err;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, c->stream));
    cudaError_t e = gpu_build_bvh(in, g, c->stream, err);
    if (e == cudaSuccess) e = cudaEventRecord(e1, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) {
        g.release();
        return set_err(e == cudaErrorMemoryAllocation ? PT_ERR_OUT_OF_MEMORY : PT_ERR_INVALID_ARG,
                       "GPU BVH build: " + (err.empty() ? std::string(cudaGetErrorString(e)) : err));
    }
    if (trav_stack_need(g.tlas_depth, g.blas_depth, false) > kStackSize) {
        g.release();
        return set_err(PT_ERR_UNSUPPORTED, "GPU-built BVH deeper than the traversal stack");
    }
    c->nodes.free();
    c->tris.free();
    c->insts.free();
    c->nodes.p = g.nodes;
    c->nodes.n = g.num_nodes;
    c->tris.p = g.tris;
    c->tris.n = g.num_tris;
    c->insts.p = g.insts;
    c->insts.n = g.num_insts;
    c->bvh.tlas_root = g.tlas_root;
    c->bvh.tlas_first_node = g.tlas_first_node;
    c->bvh.blas_depth = g.blas_depth;
    c->bvh.tlas_depth = g.tlas_depth;
    c->bvh.num_nodes = g.num_nodes;
    c->bvh.num_tris = g.num_tris;
    c->bvh.num_inst_refs = g.num_insts;
    CK(make_inst_bounds(c->inst_bounds, c->nodes.p, c->insts.p, g.num_insts, c->stream));
    CK(make_node_words(c->node_words, c->nodes.p, g.num_nodes, c->stream));
    c->direct = false;
    if (g.num_insts == 1) {
        InstRef r;
        CK(cudaMemcpy(&r, g.insts, sizeof r, cudaMemcpyDeviceToHost));
        c->direct = r.identity != 0;
        c->entry = r;
    }
    c->gpu_build_ms = ms;
    return PT_OK;
}

int create(const pt_scene_desc* d, const pt_mesh_desc* meshes, const pt_render_options* o, pt_context** out) {
    if (!d || !out) return set_err(PT_ERR_INVALID_ARG, "scene or output pointer is NULL");
    *out = nullptr;
    if (int rc = check_options(o)) return rc;
    if (meshes) {
        if (!meshes->mesh_tri_offset || meshes->num_meshes <= 0 || !meshes->instance_mesh ||
            !meshes->instance_material)
            return set_err(PT_ERR_INVALID_ARG, "incomplete mesh description");
        if (meshes->mesh_tri_offset[0] != 0 || meshes->mesh_tri_offset[meshes->num_meshes] != d->num_tris)
            return set_err(PT_ERR_INVALID_ARG, "mesh triangle offsets must run from 0 to num_tris");
        for (int m = 0; m < meshes->num_meshes; ++m)
            if (meshes->mesh_tri_offset[m + 1] < meshes->mesh_tri_offset[m])
                return set_err(PT_ERR_INVALID_ARG, "mesh triangle offsets must not decrease");
        for (int i = 0; i < d->num_instances; ++i) {
            if (meshes->instance_mesh[i] < 0 || meshes->instance_mesh[i] >= meshes->num_meshes)
                return set_err(PT_ERR_INVALID_ARG, "instance mesh index out of range");
            if (meshes->instance_material[i] < 0 || meshes->instance_material[i] >= d->num_materials)
                return set_err(PT_ERR_INVALID_ARG, "instance material index out of range");
        }
    }
    if ((!meshes && (!d->bvh_nodes || d->num_bvh_nodes <= 0)) || !d->vert_indices || d->num_tris < 0 || !d->vertices_uvx ||
        !d->normals_uvy || d->num_vertices <= 0 || !d->transforms || d->num_instances <= 0 || !d->materials ||
        d->num_materials <= 0 || d->num_lights < 0 || (d->num_lights > 0 && !d->lights))
        return set_err(PT_ERR_INVALID_ARG, "incomplete scene description");
    if (d->num_textures < 0 || (d->num_textures > 0 && (!d->texture_maps || d->tex_width <= 0 || d->tex_height <= 0)))
        return set_err(PT_ERR_INVALID_ARG, "invalid texture maps");
    if (int rc = check_materials(d->materials, d->num_materials, d->num_textures)) return rc;
    for (int i = 0; i < d->num_lights; ++i) {
        int type = (int)d->lights[15 * i + 14];
        if (type < 0 || type > 2) return set_err(PT_ERR_INVALID_ARG, "unknown light type");
    }
    pt_context* c = new pt_context;
    c->opts = *o;
    if (const char* e = std::getenv("PT_TRAVERSAL_STACK_LIMIT"))
        c->stack_limit = std::min(kStackSize, std::max(1, std::atoi(e)));
    int rc = PT_OK;
    do {
        cudaError_t e = cudaGetDevice(&c->device);
        if (e != cudaSuccess) { rc = cuda_err(e, "cudaGetDevice"); break; }
        e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { rc = cuda_err(e, "cudaStreamCreate"); break; }
        c->stream = c->own_stream;
        if ((e = cudaEventCreate(&c->ev0)) != cudaSuccess || (e = cudaEventCreate(&c->ev1)) != cudaSuccess) {
            rc = cuda_err(e, "cudaEventCreate");
            break;
        }
        if (!meshes) {
            char msg[512] = {0};
            rc = ptgb_build_wide(d->bvh_nodes, d->num_bvh_nodes, d->top_level_index, d->vert_indices, d->num_tris,
                                 d->vertices_uvx, d->num_vertices, d->transforms, d->num_instances, &c->bvh, msg,
                                 sizeof msg);
            if (rc) { set_err(rc, std::string("BVH: ") + msg); break; }
            if ((rc = check_tlas_materials(d->bvh_nodes + 9 * (size_t)d->top_level_index,
                                           d->num_bvh_nodes - d->top_level_index, d->num_materials)))
                break;
            c->bin_nodes.assign(d->bvh_nodes, d->bvh_nodes + 9 * (size_t)d->num_bvh_nodes);
            c->top_level_index = d->top_level_index;
        } else {
            c->gpu_bvh = true;
            c->mesh_tri_offset.assign(meshes->mesh_tri_offset, meshes->mesh_tri_offset + meshes->num_meshes + 1);
            c->inst_mesh.assign(meshes->instance_mesh, meshes->instance_mesh + d->num_instances);
            c->inst_material.assign(meshes->instance_material, meshes->instance_material + d->num_instances);
        }
        c->num_tris = d->num_tris;
        c->num_vertices = d->num_vertices;
        c->num_materials = d->num_materials;
        c->num_instances = d->num_instances;
        c->num_lights = d->num_lights;
        c->scene_flags = scene_flags_of(d->materials, d->num_materials, d->num_lights);
        c->host_mats.assign(d->materials, d->materials + 32 * (size_t)d->num_materials);
        if (!meshes && (rc = upload_bvh(c))) break;
        if ((rc = update_blend_boxes(c))) break;
        if ((rc = upload_instances(c, d->transforms, d->num_instances))) break;
        if ((e = c->vidx.upload(d->vert_indices, 3 * (size_t)d->num_tris, c->stream)) != cudaSuccess ||
            (e = c->verts.upload(d->vertices_uvx, d->num_vertices, c->stream)) != cudaSuccess ||
            (e = c->norms.upload(d->normals_uvy, d->num_vertices, c->stream)) != cudaSuccess ||
            (e = c->mats.upload(d->materials, 8 * (size_t)d->num_materials, c->stream)) != cudaSuccess) {
            rc = cuda_err(e, "scene upload");
            break;
        }
        if (meshes && (rc = gpu_rebuild(c, d->transforms))) break;
        if ((rc = upload_lights(c, d->lights, d->num_lights))) break;
        if (d->num_textures > 0) {
            c->tex_w = d->tex_width;
            c->tex_h = d->tex_height;
            c->num_tex = d->num_textures;
            if ((e = c->tex.upload(d->texture_maps, (size_t)d->num_textures * d->tex_width * d->tex_height,
                                   c->stream)) != cudaSuccess) {
                rc = cuda_err(e, "texture maps");
                break;
            }
        }
        if ((rc = upload_envmap(c, d->envmap_rgb, d->envmap_cdf, d->envmap_width, d->envmap_height,
                                d->envmap_total_sum)))
            break;
        if ((e = c->counters.alloc(5)) != cudaSuccess || (e = c->status.alloc(1)) != cudaSuccess) {
            rc = cuda_err(e, "counters");
            break;
        }
        if ((rc = alloc_accum(c))) break;
        if ((e = cudaStreamSynchronize(c->stream)) != cudaSuccess) { rc = cuda_err(e, "upload"); break; }
    } while (0);
    if (rc) {
        pt_destroy(c);
        return rc;
    }
    *out = c;
    return PT_OK;
}
}  // namespace

extern "C" {

int pt_create(const pt_scene_desc* d, const pt_render_options* o, pt_context** out) {
    return create(d, nullptr, o, out);
}

int pt_create_gpu_bvh(const pt_scene_desc* d, const pt_mesh_desc* meshes, const pt_render_options* o,
                      pt_context** out) {
    if (!meshes) return set_err(PT_ERR_INVALID_ARG, "mesh description is NULL");
    return create(d, meshes, o, out);
}

int pt_update_transforms(pt_context* c, const float* transforms, int32_t num_instances) {
    if (!c || !transforms) return set_err(PT_ERR_INVALID_ARG, "NULL argument");
    if (!c->gpu_bvh) return set_err(PT_ERR_INVALID_ARG, "pt_update_transforms needs a context from pt_create_gpu_bvh");
    if (num_instances != (int)c->inst_mesh.size())
        return set_err(PT_ERR_INVALID_ARG, "the number of instances cannot change");
    CK(cudaStreamSynchronize(c->stream));
    if (int rc = gpu_rebuild(c, transforms)) return rc;
    if (int rc = upload_instances(c, transforms, num_instances)) return rc;
    CK(cudaStreamSynchronize(c->stream));
    c->version++;
    c->fwd.valid = false;
    return PT_OK;
}

// ---------------------------------------------------------------- batches
}  // extern "C"

struct pt_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<pt_context*> jobs;
    std::vector<int> tlas_root, light_base;
    std::vector<BatchJob> entry;  // direct BLAS entry per job (direct, entry_inst, entry_mat)
    std::vector<uint32_t> job_scene_flags;  // F_MEDIUM / F_ALPHA_TEST of each job's scene as copied
    uint32_t flags = 0;
    DevBuf<WideNode> nodes;
    DevBuf<WideTri> tris;
    DevBuf<InstRef> insts;
    DevBuf<InstXf> xf;
    DevBuf<uint4> inst_bounds;
    DevBuf<uint4> node_words;
    DevBuf<int32_t> vidx;
    DevBuf<float4> verts, norms, mats, lights;
    DevBuf<BatchJob> job_table;
    DevBuf<int> remaining;
    DevBuf<unsigned long long> done;
    DevBuf<unsigned long long> counters;
    DevBuf<int> status;
    WavefrontBuffers wf;
    WavefrontTuning tuning;
    long chunk_paths = 1L << 25;  // paths per chunk (about 9.5 GB of path state)
    bool use_graph = true;
    cudaGraphExec_t graph_exec = nullptr;
    int last_chunks = 0;
    pt_stats last{};
};

namespace {
__global__ void k_fix_nodes(WideNode* n, int count, int node_off, int tri_off, int inst_off, int tlas_first) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    n[i].w[4] += node_off;
    n[i].w[5] += i >= tlas_first ? inst_off : tri_off;
}
__global__ void k_fix_tris(WideTri* t, int count, int prim_off, int inst_off, int mat_off) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    t[i].prim += prim_off;
    t[i].e0[3] = __int_as_float(__float_as_int(t[i].e0[3]) + inst_off);  // merged BLAS: instance
    t[i].e1[3] = __int_as_float(__float_as_int(t[i].e1[3]) + mat_off);   // and material
}
__global__ void k_fix_insts(InstRef* r, int count, int node_off, int inst_off, int mat_off) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    r[i].blas_root += node_off;
    if (r[i].instance != 0x7fffffff) r[i].instance += inst_off;
    if (r[i].material >= 0) r[i].material += mat_off;
}
__global__ void k_fix_vidx(int32_t* v, int count, int vert_off) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) v[i] += vert_off;
}
template <class T> cudaError_t concat(DevBuf<T>& out, const std::vector<const DevBuf<T>*>& parts, cudaStream_t s) {
    size_t n = 0;
    for (auto* p : parts) n += p->n;
    cudaError_t e = out.alloc(n);
    if (e != cudaSuccess) return e;
    size_t off = 0;
    for (auto* p : parts) {
        if (p->n && (e = cudaMemcpyAsync(out.p + off, p->p, p->n * sizeof(T), cudaMemcpyDeviceToDevice, s)) !=
                        cudaSuccess)
            return e;
        off += p->n;
    }
    return cudaSuccess;
}
}  // namespace

extern "C" {

int pt_batch_create(pt_context* const* jobs, int32_t n, pt_batch** out) {
    if (!jobs || n <= 0 || !out) return set_err(PT_ERR_INVALID_ARG, "invalid batch");
    *out = nullptr;
    // each job keeps its own render options, environment map, texture maps,
    // media and alpha-tested materials; a medium with volume MIS needs the
    // transmittance stages, which batches do not run
    uint32_t flags = 0;
    for (int j = 0; j < n; ++j) {
        pt_context* c = jobs[j];
        if (!c) return set_err(PT_ERR_INVALID_ARG, "NULL job");
        if (c->device != jobs[0]->device) return set_err(PT_ERR_INVALID_ARG, "batch jobs must share a device");
        const uint32_t f = option_flags(c);
        if ((f & F_MEDIUM) && (f & F_VOL_MIS))
            return set_err(PT_ERR_UNSUPPORTED, "batches take no medium with volume MIS");
        flags |= f;
    }
    pt_batch* b = new pt_batch;
    b->jobs.assign(jobs, jobs + n);
    for (int j = 0; j < n; ++j) b->job_scene_flags.push_back(jobs[j]->scene_flags & (F_MEDIUM | F_ALPHA_TEST));
    b->device = jobs[0]->device;
    b->flags = flags;  // the union: which kernel forms the batch needs
    int rc = PT_OK;
    do {
        cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { rc = cuda_err(e, "cudaStreamCreate"); break; }
        if ((e = cudaEventCreate(&b->ev0)) != cudaSuccess || (e = cudaEventCreate(&b->ev1)) != cudaSuccess) {
            rc = cuda_err(e, "cudaEventCreate");
            break;
        }
        std::vector<const DevBuf<WideNode>*> pn;
        std::vector<const DevBuf<WideTri>*> pt;
        std::vector<const DevBuf<InstRef>*> pi;
        std::vector<const DevBuf<InstXf>*> px;
        std::vector<const DevBuf<int32_t>*> pv;
        std::vector<const DevBuf<float4>*> pvert, pnorm, pmat, plight;
        for (pt_context* c : b->jobs) {
            CK(cudaStreamSynchronize(c->stream));
            pn.push_back(&c->nodes);
            pt.push_back(&c->tris);
            pi.push_back(&c->insts);
            px.push_back(&c->xf);
            pv.push_back(&c->vidx);
            pvert.push_back(&c->verts);
            pnorm.push_back(&c->norms);
            pmat.push_back(&c->mats);
            plight.push_back(&c->lights);
        }
        if ((e = concat(b->nodes, pn, b->stream)) != cudaSuccess || (e = concat(b->tris, pt, b->stream)) != cudaSuccess ||
            (e = concat(b->insts, pi, b->stream)) != cudaSuccess || (e = concat(b->xf, px, b->stream)) != cudaSuccess ||
            (e = concat(b->vidx, pv, b->stream)) != cudaSuccess ||
            (e = concat(b->verts, pvert, b->stream)) != cudaSuccess ||
            (e = concat(b->norms, pnorm, b->stream)) != cudaSuccess ||
            (e = concat(b->mats, pmat, b->stream)) != cudaSuccess ||
            (e = concat(b->lights, plight, b->stream)) != cudaSuccess) {
            rc = cuda_err(e, "batch scene concatenation");
            break;
        }
        int node_off = 0, tri_off = 0, inst_off = 0, wtri_off = 0, ref_off = 0, vert_off = 0, vidx_off = 0;
        int mat_off = 0, light_off = 0;
        const int B = 256;
        for (pt_context* c : b->jobs) {
            const int nn = (int)c->nodes.n, nt = (int)c->tris.n, ni = (int)c->insts.n, nv = (int)c->vidx.n;
            if (nn) k_fix_nodes<<<(nn + B - 1) / B, B, 0, b->stream>>>(b->nodes.p + node_off, nn, node_off, wtri_off,
                                                                      ref_off, c->bvh.tlas_first_node);
            if (nt) k_fix_tris<<<(nt + B - 1) / B, B, 0, b->stream>>>(b->tris.p + wtri_off, nt, tri_off, inst_off,
                                                                     mat_off);
            if (ni) k_fix_insts<<<(ni + B - 1) / B, B, 0, b->stream>>>(b->insts.p + ref_off, ni, node_off, inst_off,
                                                                      mat_off);
            if (nv) k_fix_vidx<<<(nv + B - 1) / B, B, 0, b->stream>>>(b->vidx.p + vidx_off, nv, vert_off);
            if ((e = cudaGetLastError()) != cudaSuccess) break;
            b->tlas_root.push_back(c->bvh.tlas_root + node_off);
            BatchJob entry{};
            if (c->direct) {  // traversal starts in the BLAS, re-based like the InstRef
                entry.direct = 1;
                entry.entry_inst = c->entry.instance == 0x7fffffff ? c->entry.instance : c->entry.instance + inst_off;
                entry.entry_mat = c->entry.material >= 0 ? c->entry.material + mat_off : c->entry.material;
                b->tlas_root.back() = c->entry.blas_root + node_off;
            }
            b->entry.push_back(entry);
            b->light_base.push_back(light_off);
            node_off += nn;
            wtri_off += nt;
            ref_off += ni;
            tri_off += c->num_tris;
            inst_off += c->num_instances;
            vert_off += c->num_vertices;
            vidx_off += nv;
            mat_off += c->num_materials;
            light_off += (int)(c->lights.n / 4);  // a job without lights holds one padding record
        }
        if (e == cudaSuccess) e = make_inst_bounds(b->inst_bounds, b->nodes.p, b->insts.p, ref_off, b->stream);
        if (e == cudaSuccess) e = make_node_words(b->node_words, b->nodes.p, node_off, b->stream);
        if (e != cudaSuccess) { rc = cuda_err(e, "batch index fix-up"); break; }
        if ((e = b->counters.alloc(5)) != cudaSuccess || (e = b->status.alloc(1)) != cudaSuccess ||
            (e = b->remaining.alloc(n)) != cudaSuccess || (e = b->done.alloc(n + 1)) != cudaSuccess) {
            rc = cuda_err(e, "batch buffers");
            break;
        }
        if ((e = wavefront_default_tuning(b->tuning, 128)) != cudaSuccess) { rc = cuda_err(e, "tuning"); break; }
        for (pt_context* c : b->jobs)  // the launch configuration of the first tuned job
            if (c->wf_tuned) {
                b->tuning = c->wf_tuning;
                break;
            }
        if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) { rc = cuda_err(e, "batch set-up"); break; }
    } while (0);
    if (rc) {
        pt_batch_destroy(b);
        return rc;
    }
    *out = b;
    return PT_OK;
}

int pt_batch_render(pt_batch* b, const int32_t* first_pass, const int32_t* num_passes, float* job_ms) {
    if (!b || !first_pass || !num_passes) return set_err(PT_ERR_INVALID_ARG, "NULL argument");
    const int n = (int)b->jobs.size();
    std::vector<BatchJob> base(n);
    std::vector<int> remaining(n);
    uint32_t flags = 0;  // union of the jobs' flags
    bool inline_shadows = false;
    std::vector<long> job_paths(n);
    long total = 0, max_npix = 0;
    for (int j = 0; j < n; ++j) {
        const pt_context* c = b->jobs[j];
        if (first_pass[j] < 0 || num_passes[j] <= 0) return set_err(PT_ERR_INVALID_ARG, "invalid pass range");
        const pt_render_options& o = c->opts;
        BatchJob& J = base[j];
        J = BatchJob{};
        J.tlas_root = b->tlas_root[j];
        J.direct = b->entry[j].direct;
        J.entry_inst = b->entry[j].entry_inst;
        J.entry_mat = b->entry[j].entry_mat;
        J.light_base = b->light_base[j];
        J.num_lights = c->num_lights;
        J.max_depth = o.max_depth;
        J.rr_depth = o.rr_depth;
        J.width = o.render_width;
        J.height = o.render_height;
        J.tile_w = o.tile_width;
        J.tile_h = o.tile_height;
        J.ntx = (J.width + J.tile_w - 1) / J.tile_w;
        J.nty = (J.height + J.tile_h - 1) / J.tile_h;
        for (int k = 0; k < 3; ++k) {
            J.cam_pos[k] = c->cam.position[k];
            J.cam_up[k] = c->cam.up[k];
            J.cam_right[k] = c->cam.right[k];
            J.cam_fwd[k] = c->cam.forward[k];
        }
        J.cam_fov = c->cam.fov;
        J.cam_focal = c->cam.focal_dist;
        J.cam_aperture = c->cam.aperture;
        J.accum = c->accum.p;
        J.npix = J.width * J.height;
        J.id = j;
        // the job's options now, with the scene flags of its copy in the
        // batch (those of pt_batch_create)
        J.flags = (option_flags(c) & ~(uint32_t)(F_MEDIUM | F_ALPHA_TEST)) | (b->job_scene_flags[j]);
        if ((J.flags & F_MEDIUM) && (J.flags & F_VOL_MIS))
            return set_err(PT_ERR_UNSUPPORTED, "pt_batch_render: a medium with volume MIS");
        flags |= J.flags;
        // AnyHit of an alpha-tested scene without media draws random numbers
        if ((J.flags & F_ALPHA_TEST) && !(J.flags & F_MEDIUM)) inline_shadows = true;
        J.mollify_amt = o.roughness_mollification_amt;
        for (int k = 0; k < 3; ++k) J.uniform_light[k] = o.uniform_light_col[k];
        J.env = c->env.p;
        J.cdf = c->cdf.p;
        J.env_w = c->env_w;
        J.env_h = c->env_h;
        J.env_total = c->env_total;
        J.env_intensity = o.envmap_intensity;
        J.env_rot = o.envmap_rot / 360.0f;  // Renderer.cpp:778
        J.tex = c->tex.p;
        J.tex_w = c->tex_w;
        J.tex_h = c->tex_h;
        J.num_tex = c->num_tex;
        job_paths[j] = (long)J.npix * num_passes[j];
        if (job_paths[j] >= (1L << 31)) return set_err(PT_ERR_UNSUPPORTED, "pt_batch_render: job too large");
        remaining[j] = (int)job_paths[j];
        total += job_paths[j];
        max_npix = std::max(max_npix, (long)J.npix);
    }
    // Whole passes are packed into chunks of at most `cap` paths (each chunk
    // one wavefront), the jobs in order of increasing work so that short
    // jobs complete early; a job's passes stay in pass order.
    long cap = b->chunk_paths;
    if (const char* e = std::getenv("PT_BATCH_CAPACITY")) cap = std::max(1L, std::atol(e));
    cap = std::min(total, std::max(cap, max_npix));
    if (cap > (long)INT32_MAX / 2) return set_err(PT_ERR_UNSUPPORTED, "pt_batch_render: chunk too large");
    std::vector<int> order(n);
    for (int j = 0; j < n; ++j) order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return job_paths[x] < job_paths[y]; });
    std::vector<BatchJob> entries;
    std::vector<BatchChunk> chunks;
    BatchChunk cur{0, 0, 0, 0, 0};
    for (int j : order) {
        const BatchJob& J = base[j];
        int k = 0;
        while (k < num_passes[j]) {
            const int fit = (int)std::min<long>(num_passes[j] - k, (cap - cur.paths) / J.npix);
            if (fit <= 0) {
                chunks.push_back(cur);
                cur = BatchChunk{(int)entries.size(), 0, 0, 0, 0};
                continue;
            }
            BatchJob E = J;
            E.first_pass = first_pass[j] + k;
            E.num_passes = fit;
            E.path_base = cur.paths;
            E.pixel_base = cur.pixels;
            entries.push_back(E);
            cur.entry_count++;
            cur.paths += fit * J.npix;
            cur.pixels += J.npix;
            cur.max_depth = std::max(cur.max_depth, J.max_depth);
            k += fit;
        }
    }
    if (cur.entry_count) chunks.push_back(cur);
    if (b->wf.capacity < cap) {
        wavefront_free(b->wf);
        CK(wavefront_alloc(b->wf, (int)cap));
    }
    for (pt_context* c : b->jobs) CK(cudaStreamSynchronize(c->stream));
    CK(b->job_table.upload(entries.data(), entries.size(), b->stream));
    CK(cudaMemcpyAsync(b->remaining.p, remaining.data(), sizeof(int) * n, cudaMemcpyHostToDevice, b->stream));
    CK(cudaMemsetAsync(b->done.p, 0, sizeof(unsigned long long) * (n + 1), b->stream));
    CK(cudaMemsetAsync(b->counters.p, 0, 5 * sizeof(unsigned long long), b->stream));
    CK(cudaMemsetAsync(b->status.p, 0, sizeof(int), b->stream));
    Params p{};
    p.nodes = reinterpret_cast<const uint4*>(b->nodes.p);
    p.tris = reinterpret_cast<const float4*>(b->tris.p);
    p.insts = reinterpret_cast<const int4*>(b->insts.p);
    p.xf = reinterpret_cast<const float4*>(b->xf.p);
    p.inst_bounds = b->inst_bounds.p;
    p.node_words = b->node_words.p;
    p.vidx = b->vidx.p;
    p.verts = b->verts.p;
    p.norms = b->norms.p;
    p.mats = b->mats.p;
    p.lights = b->lights.p;
    p.num_materials = (int)(b->mats.n / 8);
    p.flags = flags;  // the kernel forms the jobs need; each path reads its job's own flags
    p.counters = b->counters.p;
    p.status = b->status.p;
    p.stack_limit = kStackSize;
    for (pt_context* c : b->jobs) p.stack_limit = std::min(p.stack_limit, c->stack_limit);
    p.untraced = untraced_bits(false);  // batches hold no VOL_MIS media
    p.jobs = b->job_table.p;
    p.num_jobs = (int)entries.size();
    // every job enters its BLAS directly: the direct form of the traversal
    // kernels (each path still takes its job's root and entry)
    p.direct = 1;
    for (const BatchJob& J : base) p.direct &= J.direct;
    p.job_remaining = b->remaining.p;
    p.job_done = b->done.p;
    WavefrontTuning t = b->tuning;
    int depth = 0;
    for (pt_context* c : b->jobs) depth = std::max(depth, c->bvh.tlas_depth + c->bvh.blas_depth);
    if (!trav_postpone_fits(depth)) t.min_tris = t.min_tris_first = t.min_tris_shadow_first = 0;
    int launches = 0;
    bool use_graph = b->use_graph;
    if (const char* e = std::getenv("PT_BATCH_GRAPH")) use_graph = std::atoi(e) != 0;
    if (use_graph) {
        // the whole chunk sequence as one CUDA graph (updated in place when
        // only the kernel arguments changed since the last call)
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        const cudaError_t ce =
            launch_batch(p, chunks.data(), (int)chunks.size(), b->wf, t, b->stream, b->done.p + n, &launches,
                         inline_shadows);
        const cudaError_t ee = cudaStreamEndCapture(b->stream, &g);
        if (ce != cudaSuccess || ee != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_err(ce != cudaSuccess ? ce : ee, "batch graph capture");
        }
        bool updated = false;
        if (b->graph_exec) {
            cudaGraphExecUpdateResultInfo info;
            updated = cudaGraphExecUpdate(b->graph_exec, g, &info) == cudaSuccess;
            if (!updated) {
                cudaGetLastError();
                cudaGraphExecDestroy(b->graph_exec);
                b->graph_exec = nullptr;
            }
        }
        cudaError_t e = cudaSuccess;
        if (!updated) e = cudaGraphInstantiate(&b->graph_exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b->graph_exec = nullptr;
            return cuda_err(e, "cudaGraphInstantiate");
        }
        CK(cudaEventRecord(b->ev0, b->stream));
        CK(cudaGraphLaunch(b->graph_exec, b->stream));
        CK(cudaEventRecord(b->ev1, b->stream));
    } else {
        CK(cudaEventRecord(b->ev0, b->stream));
        CK(launch_batch(p, chunks.data(), (int)chunks.size(), b->wf, t, b->stream, b->done.p + n, &launches,
                        inline_shadows));
        CK(cudaEventRecord(b->ev1, b->stream));
    }
    std::vector<unsigned long long> done(n + 1);
    unsigned long long cnt[5];
    int st = 0;
    CK(cudaMemcpyAsync(done.data(), b->done.p, sizeof(unsigned long long) * (n + 1), cudaMemcpyDeviceToHost,
                       b->stream));
    CK(cudaMemcpyAsync(cnt, b->counters.p, sizeof cnt, cudaMemcpyDeviceToHost, b->stream));
    CK(cudaMemcpyAsync(&st, b->status.p, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    CK(cudaStreamSynchronize(b->stream));
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->last.closest_rays = cnt[0];
    b->last.shadow_rays = cnt[1];
    b->last.paths = cnt[2];
    b->last.truncated_paths = cnt[3];
    b->last.untraced_shadow_rays = cnt[4];
    b->last.kernel_ms = ms;
    b->last.status = st;
    b->last.kernel_launches = launches;
    b->last_chunks = (int)chunks.size();
    if (job_ms)
        for (int j = 0; j < n; ++j) job_ms[j] = done[j] >= done[n] ? (float)((done[j] - done[n]) * 1e-6) : 0.0f;
    for (pt_context* c : b->jobs) c->fwd.valid = false;
    if (st) return set_err(st, "pt_batch_render: kernel status " + std::to_string(st));
    return PT_OK;
}

int pt_batch_stats(pt_batch* b, pt_stats* s) {
    if (!b || !s) return set_err(PT_ERR_INVALID_ARG, "NULL argument");
    *s = b->last;
    return PT_OK;
}

int pt_batch_destroy(pt_batch* b) {
    if (!b) return PT_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    b->nodes.free(); b->tris.free(); b->insts.free(); b->xf.free(); b->inst_bounds.free(); b->node_words.free(); b->vidx.free(); b->verts.free();
    b->norms.free(); b->mats.free(); b->lights.free(); b->job_table.free(); b->remaining.free(); b->done.free();
    b->counters.free(); b->status.free();
    wavefront_free(b->wf);
    if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return PT_OK;
}

int pt_gpu_build_ms(pt_context* c, float* ms) {
    if (!c || !ms) return set_err(PT_ERR_INVALID_ARG, "NULL argument");
    *ms = c->gpu_build_ms;
    return PT_OK;
}

int pt_destroy(pt_context* c) {
    if (!c) return PT_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->nodes.free(); c->tris.free(); c->insts.free(); c->xf.free(); c->inst_bounds.free(); c->node_words.free(); c->vidx.free(); c->verts.free();
    c->norms.free(); c->mats.free(); c->lights.free(); c->env.free(); c->cdf.free(); c->accum.free();
    c->tex.free();
    c->snapshot.free(); c->ldr.free(); c->counters.free(); c->status.free(); c->blend_boxes.free();
    wavefront_free(c->wf);
    c->timer.release();
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    ptgb_free_wide(&c->bvh);
    delete c;
    return PT_OK;
}

int pt_set_stream(pt_context* c, void* s) {
    if (!c) return set_err(PT_ERR_INVALID_ARG, "context is NULL");
    CK(cudaStreamSynchronize(c->stream));
    c->stream = s ? (cudaStream_t)s : c->own_stream;
    return PT_OK;
}

int pt_set_camera(pt_context* c, const pt_camera* cam) {
    if (!c || !cam) return set_err(PT_ERR_INVALID_ARG, "NULL argument");
    c->cam = *cam;
    c->version++;
    return PT_OK;
}

int pt_set_options(pt_context* c, const pt_render_options* o) {
    if (!c) return set_err(PT_ERR_INVALID_ARG, "context is NULL");
    if (int rc = check_options(o)) return rc;
    const bool resize = o->render_width != c->opts.render_width || o->render_height != c->opts.render_height ||
                        o->tile_width != c->opts.tile_width || o->tile_height != c->opts.tile_height;
    c->opts = *o;
    c->version++;
    if (resize) return alloc_accum(c);
    return PT_OK;
}

int pt_set_integrator(pt_context* c, int32_t integrator) {
    if (!c) return set_err(PT_ERR_INVALID_ARG, "context is NULL");
    if (integrator != PT_INTEGRATOR_MEGAKERNEL && integrator != PT_INTEGRATOR_WAVEFRONT)
        return set_err(PT_ERR_INVALID_ARG, "unknown integrator");
    c->integrator = integrator;
    return PT_OK;
}

int pt_update_instances(pt_context* c, const float* transforms, int32_t num_instances, const float* materials,
                        int32_t num_materials, const float* tlas_nodes, int32_t num_tlas_nodes) {
    if (!c || !transforms || num_instances <= 0 || !tlas_nodes || num_tlas_nodes <= 0)
        return set_err(PT_ERR_INVALID_ARG, "invalid instance update");
    if (materials) {
        if (num_materials <= 0) return set_err(PT_ERR_INVALID_ARG, "num_materials must be positive");
        if (int rc = check_materials(materials, num_materials, c->num_tex)) return rc;
    }
    c->version++;
    int rc = check_tlas_materials(tlas_nodes, num_tlas_nodes, materials ? num_materials : c->num_materials);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->stream));
    std::vector<float> bin(c->bin_nodes.begin(), c->bin_nodes.begin() + 9 * (size_t)c->top_level_index);
    bin.insert(bin.end(), tlas_nodes, tlas_nodes + 9 * (size_t)num_tlas_nodes);
    char msg[512] = {0};
    rc = ptgb_rebuild_tlas(&c->bvh, bin.data(), c->top_level_index + num_tlas_nodes, c->top_level_index, transforms,
                           num_instances, msg, sizeof msg);
    if (rc) return set_err(rc, std::string("TLAS: ") + msg);
    c->bin_nodes.swap(bin);
    c->num_instances = num_instances;
    if ((rc = upload_bvh(c))) return rc;
    if ((rc = upload_instances(c, transforms, num_instances))) return rc;
    if (materials) {
        CK(c->mats.upload(materials, 8 * (size_t)num_materials, c->stream));
        c->num_materials = num_materials;
        c->scene_flags = scene_flags_of(materials, num_materials, c->num_lights);
        c->host_mats.assign(materials, materials + 32 * (size_t)num_materials);
    }
    CK(cudaStreamSynchronize(c->stream));
    return update_blend_boxes(c);
}

int pt_update_envmap(pt_context* c, const float* rgb, const float* cdf, int32_t w, int32_t h, float total) {
    if (!c) return set_err(PT_ERR_INVALID_ARG, "context is NULL");
    if (rgb && (w <= 0 || h <= 0 || !cdf)) return set_err(PT_ERR_INVALID_ARG, "invalid envmap");
    CK(cudaStreamSynchronize(c->stream));
    c->version++;
    return upload_envmap(c, rgb, cdf, w, h, total);
}

int pt_clear_accum(pt_context* c) {
    if (!c) return set_err(PT_ERR_INVALID_ARG, "context is NULL");
    CK(cudaMemsetAsync(c->accum.p, 0, c->accum.n * sizeof(float4), c->stream));
    return PT_OK;
}

int pt_render_tile(pt_context* c, int32_t tx, int32_t ty, int32_t frame) {
    if (!c) return set_err(PT_ERR_INVALID_ARG, "context is NULL");
    const pt_render_options& o = c->opts;
    const int ntx = (o.render_width + o.tile_width - 1) / o.tile_width;
    const int nty = (o.render_height + o.tile_height - 1) / o.tile_height;
    if (tx < 0 || ty < 0 || tx >= ntx || ty >= nty) return set_err(PT_ERR_INVALID_ARG, "tile out of range");
    if (frame < 0) return set_err(PT_ERR_INVALID_ARG, "negative frame number");
    RenderWork w;
    w.x0 = tx * o.tile_width;
    w.y0 = ty * o.tile_height;
    w.w = std::min(o.tile_width, o.render_width - w.x0);
    w.h = std::min(o.tile_height, o.render_height - w.y0);
    w.first_pass = 0;
    w.num_passes = 1;
    w.tile_frame = frame;
    w.tile_x = tx;
    w.tile_y = ty;
    return render(c, w);
}

// One tile with the wavefront integrator, its path state in the fixed device
// array of pt_wavefront.cu instead of the context's cudaMalloc'd batch: the
// tile runs in bands of whole rows of at most kFixedScratchPaths pixels.
// Path seeds depend only on the pixel and the tile, so the bands give the
// samples pt_render_tile gives.  No CUDA graph is built (instantiating one
// allocates).
int pt_render_tile_noalloc(pt_context* c, int32_t tx, int32_t ty, int32_t frame) {
    if (!c) return set_err(PT_ERR_INVALID_ARG, "context is NULL");
    const pt_render_options& o = c->opts;
    const int ntx = (o.render_width + o.tile_width - 1) / o.tile_width;
    const int nty = (o.render_height + o.tile_height - 1) / o.tile_height;
    if (tx < 0 || ty < 0 || tx >= ntx || ty >= nty) return set_err(PT_ERR_INVALID_ARG, "tile out of range");
    if (frame < 0) return set_err(PT_ERR_INVALID_ARG, "negative frame number");
    RenderWork w;
    w.x0 = tx * o.tile_width;
    w.y0 = ty * o.tile_height;
    w.w = std::min(o.tile_width, o.render_width - w.x0);
    w.h = std::min(o.tile_height, o.render_height - w.y0);
    w.first_pass = 0;
    w.num_passes = 1;
    w.tile_frame = frame;
    w.tile_x = tx;
    w.tile_y = ty;
    if (w.w > kFixedScratchPaths)
        return set_err(PT_ERR_INVALID_ARG, "pt_render_tile_noalloc: tile rows of more than 16384 pixels do not fit "
                                           "the fixed path-state scratch");
    WavefrontBuffers wb;
    CK(wavefront_fixed_buffers(wb));
    if (!c->wf_tuned) {
        CK(wavefront_default_tuning(c->wf_tuning, 128));
        c->wf_tuned = true;
    }
    // Stage timing does not cover this call (its events would be created on
    // demand); the stage times of an earlier call are dropped, not reported
    // as this call's.
    c->timer.reset();
    if (int rc = begin_launch(c)) return rc;
    const Params p = make_params(c);
    const int rows = kFixedScratchPaths / w.w;
    int launches = 0;
    for (int y = 0; y < w.h; y += rows) {
        RenderWork band = w;
        band.y0 = w.y0 + y;
        band.h = std::min(rows, w.h - y);
        int n = 0;
        WavefrontTuning t = c->wf_tuning;
        if (!trav_postpone_fits(c->bvh.tlas_depth + c->bvh.blas_depth)) t.min_tris = t.min_tris_first = t.min_tris_shadow_first = 0;
        CK(launch_wavefront(p, band, wb, t, false, c->stream, &n));
        launches += n;
    }
    c->launches = launches;
    return end_launch(c);
}

int pt_update_materials(pt_context* c, const float* materials, int32_t num_materials) {
    if (!c || !materials) return set_err(PT_ERR_INVALID_ARG, "NULL argument");
    if (num_materials != c->num_materials)
        return set_err(PT_ERR_INVALID_ARG, "pt_update_materials: the number of materials cannot change");
    if (int rc = check_materials(materials, num_materials, c->num_tex)) return rc;
    CK(cudaStreamSynchronize(c->stream));
    CK(c->mats.upload(materials, 8 * (size_t)num_materials, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->scene_flags = scene_flags_of(materials, num_materials, c->num_lights);
    c->host_mats.assign(materials, materials + 32 * (size_t)num_materials);
    c->version++;
    return update_blend_boxes(c);
}

int pt_update_lights(pt_context* c, const float* lights, int32_t num_lights) {
    if (!c || (num_lights > 0 && !lights)) return set_err(PT_ERR_INVALID_ARG, "NULL argument");
    if (num_lights != c->num_lights)
        return set_err(PT_ERR_INVALID_ARG, "pt_update_lights: the number of lights cannot change");
    for (int i = 0; i < num_lights; ++i) {
        const int type = (int)lights[15 * i + 14];
        if (type < 0 || type > 2) return set_err(PT_ERR_INVALID_ARG, "unknown light type");
    }
    CK(cudaStreamSynchronize(c->stream));
    if (int rc = upload_lights(c, lights, num_lights)) return rc;
    c->version++;
    return PT_OK;
}

int pt_render_adjoint(pt_context* c, int32_t first_pass, int32_t num_passes, const float* d_image, float* grad) {
    if (!c || !d_image || !grad) return set_err(PT_ERR_INVALID_ARG, "NULL argument");
    if (first_pass < 0 || num_passes <= 0) return set_err(PT_ERR_INVALID_ARG, "invalid pass range");
    const uint32_t flags = option_flags(c);
    if (flags & (F_MEDIUM | F_ALPHA_TEST | F_ENVMAP | F_TEXTURES))
        return set_err(PT_ERR_UNSUPPORTED, "pt_render_adjoint: media, alpha-tested materials, environment maps and "
                                           "texture maps are not differentiated");
    RenderWork w;
    w.x0 = w.y0 = 0;
    w.w = c->opts.render_width;
    w.h = c->opts.render_height;
    w.first_pass = first_pass;
    w.num_passes = num_passes;
    w.tile_frame = -1;
    w.tile_x = w.tile_y = 0;
    const long paths = (long)w.w * w.h * num_passes;
    if (paths > (1L << 26)) return set_err(PT_ERR_UNSUPPORTED, "pt_render_adjoint: more than 2^26 paths in one call");
    if (c->wf.capacity < paths) {
        CK(wavefront_alloc(c->wf, (int)paths));
        c->fwd.valid = false;
    }
    if (!c->wf_tuned) {
        CK(wavefront_default_tuning(c->wf_tuning, 128));
        c->wf_tuned = true;
    }
    if ((long)c->adj_le.n < c->wf.capacity) {
        CK(c->adj_v.alloc(3 * (size_t)c->wf.capacity));
        CK(c->adj_le.alloc((size_t)c->wf.capacity));
    }
    const int gsize = c->num_materials * grad::kParams + 3 * c->num_lights;
    const size_t npix_full = (size_t)c->opts.render_width * c->opts.render_height;
    CK(c->adj_dimage.upload(d_image, 3 * npix_full, c->stream));
    if ((int)c->adj_grad.n != gsize) CK(c->adj_grad.alloc(gsize));
    CK(cudaMemsetAsync(c->adj_grad.p, 0, sizeof(float) * gsize, c->stream));
    AdjView A;
    A.dimage = c->adj_dimage.p;
    A.inv_passes = 1.0f / (float)num_passes;
    A.width = c->opts.render_width;
    A.grad = c->adj_grad.p;
    A.num_materials = c->num_materials;
    A.num_lights = c->num_lights;
    A.grad_size = gsize;
    A.shared = gsize <= 8192;  // up to 32 KB of shared memory per block
    A.v = c->adj_v.p;
    A.le = c->adj_le.p;
    const bool cached = c->fwd.valid && c->fwd.version == c->version && c->fwd.w.x0 == w.x0 &&
                        c->fwd.w.y0 == w.y0 && c->fwd.w.w == w.w && c->fwd.w.h == w.h &&
                        c->fwd.w.first_pass == w.first_pass && c->fwd.w.num_passes == w.num_passes &&
                        c->fwd.w.tile_frame == w.tile_frame;
    if (int rc = begin_launch(c)) return rc;
    WavefrontTuning t = c->wf_tuning;
    if (!trav_postpone_fits(c->bvh.tlas_depth + c->bvh.blas_depth)) t.min_tris = t.min_tris_first = t.min_tris_shadow_first = 0;
    CK(launch_adjoint(make_params(c), w, c->wf, t, A, !cached, c->stream, &c->launches));
    if (int rc = end_launch(c)) return rc;
    c->fwd.valid = false;  // the replay leaves the forward state of the paths, but not in a reusable form
    CK(cudaMemcpyAsync(grad, c->adj_grad.p, sizeof(float) * gsize, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    int st = 0;
    CK(cudaMemcpy(&st, c->status.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (st) return set_err(st, "pt_render_adjoint: kernel status " + std::to_string(st));
    return PT_OK;
}

int pt_render_passes(pt_context* c, int32_t first_pass, int32_t num_passes) {
    if (!c) return set_err(PT_ERR_INVALID_ARG, "context is NULL");
    if (first_pass < 0 || num_passes < 0) return set_err(PT_ERR_INVALID_ARG, "negative pass range");
    RenderWork w;
    w.x0 = w.y0 = 0;
    w.w = c->opts.render_width;
    w.h = c->opts.render_height;
    w.first_pass = first_pass;
    w.num_passes = num_passes;
    w.tile_frame = -1;
    w.tile_x = w.tile_y = 0;
    return render(c, w);
}

int pt_get_accum(pt_context* c, float* host) {
    if (!c || !host) return set_err(PT_ERR_INVALID_ARG, "NULL argument");
    CK(cudaMemcpyAsync(host, c->accum.p, c->accum.n * sizeof(float4), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

int pt_set_accum(pt_context* c, const float* host) {
    if (!c || !host) return set_err(PT_ERR_INVALID_ARG, "NULL argument");
    CK(cudaMemcpyAsync(c->accum.p, host, c->accum.n * sizeof(float4), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

int pt_snapshot_accum(pt_context* c) {
    if (!c) return set_err(PT_ERR_INVALID_ARG, "context is NULL");
    if (c->snapshot.n != c->accum.n) CK(c->snapshot.alloc(c->accum.n));
    CK(cudaMemcpyAsync(c->snapshot.p, c->accum.p, c->accum.n * sizeof(float4), cudaMemcpyDeviceToDevice, c->stream));
    return PT_OK;
}

int pt_get_output(pt_context* c, int32_t num_samples, int32_t from_snapshot, uint8_t* host) {
    if (!c || !host || num_samples <= 0) return set_err(PT_ERR_INVALID_ARG, "invalid argument");
    if (from_snapshot && c->snapshot.n != c->accum.n) return set_err(PT_ERR_INVALID_ARG, "no snapshot taken");
    if (c->ldr.n != c->accum.n) CK(c->ldr.alloc(c->accum.n));
    const pt_render_options& o = c->opts;
    Params p = make_params(c);
    if (from_snapshot) p.accum = c->snapshot.p;
    CK(launch_tonemap(p, num_samples, o.enable_tonemap, o.enable_aces, o.simple_aces_fit,
                      o.enable_background, o.transparent_background, o.background_col, (unsigned char*)c->ldr.p,
                      c->stream));
    CK(cudaMemcpyAsync(host, c->ldr.p, c->ldr.n * sizeof(uchar4), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return PT_OK;
}

int pt_trace_rays(pt_context* c, const pt_ray* rays, int32_t n, pt_hit* hits) {
    if (!c || n < 0 || (n && (!rays || !hits))) return set_err(PT_ERR_INVALID_ARG, "invalid argument");
    if (!n) return PT_OK;
    DevBuf<pt_ray> dr;
    DevBuf<pt_hit> dh;
    CK(dr.upload(rays, n, c->stream));
    CK(dh.alloc(n));
    CK(cudaMemsetAsync(c->status.p, 0, sizeof(int), c->stream));
    CK(launch_trace_closest(make_params(c), dr.p, n, dh.p, c->stream));
    CK(cudaMemcpyAsync(hits, dh.p, n * sizeof(pt_hit), cudaMemcpyDeviceToHost, c->stream));
    int st = 0;
    CK(cudaMemcpyAsync(&st, c->status.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    dr.free();
    dh.free();
    if (st) return set_err(st, "traversal stack overflow");
    return PT_OK;
}

int pt_trace_shadow(pt_context* c, const pt_ray* rays, const float* maxd, int32_t n, uint8_t* occ) {
    if (!c || n < 0 || (n && (!rays || !maxd || !occ))) return set_err(PT_ERR_INVALID_ARG, "invalid argument");
    if (!n) return PT_OK;
    DevBuf<pt_ray> dr;
    DevBuf<float> dm;
    DevBuf<uint8_t> dout;
    CK(dr.upload(rays, n, c->stream));
    CK(dm.upload(maxd, n, c->stream));
    CK(dout.alloc(n));
    CK(cudaMemsetAsync(c->status.p, 0, sizeof(int), c->stream));
    CK(launch_trace_shadow(make_params(c), dr.p, dm.p, n, dout.p, c->stream));
    CK(cudaMemcpyAsync(occ, dout.p, n, cudaMemcpyDeviceToHost, c->stream));
    int st = 0;
    CK(cudaMemcpyAsync(&st, c->status.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    dr.free();
    dm.free();
    dout.free();
    if (st) return set_err(st, "traversal stack overflow");
    return PT_OK;
}

int pt_bsdf_eval(pt_context* c, const float* rec, const float* V, const float* N, const float* L, int32_t n,
                 float* f, float* pdf) {
    if (!c || n < 0 || (n && (!rec || !V || !N || !L || !f || !pdf)))
        return set_err(PT_ERR_INVALID_ARG, "invalid argument");
    if (!n) return PT_OK;
    DevBuf<float> dr, dv, dn, dl, df, dp;
    CK(dr.upload(rec, 20 * (size_t)n, c->stream));
    CK(dv.upload(V, 3 * (size_t)n, c->stream));
    CK(dn.upload(N, 3 * (size_t)n, c->stream));
    CK(dl.upload(L, 3 * (size_t)n, c->stream));
    CK(df.alloc(3 * (size_t)n));
    CK(dp.alloc(n));
    CK(launch_bsdf_eval(dr.p, dv.p, dn.p, dl.p, n, df.p, dp.p, c->stream));
    CK(cudaMemcpyAsync(f, df.p, 3 * sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(pdf, dp.p, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (auto* b : {&dr, &dv, &dn, &dl, &df, &dp}) b->free();
    return PT_OK;
}

int pt_bsdf_sample(pt_context* c, const float* rec, const float* V, const float* N, const uint32_t* seeds, int32_t n,
                   float* L, float* f, float* pdf) {
    if (!c || n < 0 || (n && (!rec || !V || !N || !seeds || !L || !f || !pdf)))
        return set_err(PT_ERR_INVALID_ARG, "invalid argument");
    if (!n) return PT_OK;
    DevBuf<float> dr, dv, dn, dl, df, dp;
    DevBuf<uint32_t> ds;
    CK(dr.upload(rec, 20 * (size_t)n, c->stream));
    CK(dv.upload(V, 3 * (size_t)n, c->stream));
    CK(dn.upload(N, 3 * (size_t)n, c->stream));
    CK(ds.upload(seeds, 4 * (size_t)n, c->stream));
    CK(dl.alloc(3 * (size_t)n));
    CK(df.alloc(3 * (size_t)n));
    CK(dp.alloc(n));
    CK(launch_bsdf_sample(dr.p, dv.p, dn.p, ds.p, n, dl.p, df.p, dp.p, c->stream));
    CK(cudaMemcpyAsync(L, dl.p, 3 * sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(f, df.p, 3 * sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(pdf, dp.p, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (auto* b : {&dr, &dv, &dn, &dl, &df, &dp}) b->free();
    ds.free();
    return PT_OK;
}

namespace {
void tuning_out(const WavefrontTuning& t, float ms, pt_tuning* out) {
    out->extend_variant = t.extend_variant;
    out->shadow_variant = t.shadow_variant;
    out->extend_refill = t.extend_refill;
    out->shadow_refill = t.shadow_refill;
    out->min_tris = t.min_tris;
    out->shade_variant = t.shade_variant;
    out->frame_ms = ms;
    out->extend_refill_first = t.extend_refill_first;
    out->min_tris_first = t.min_tris_first;
    out->shadow_refill_first = t.shadow_refill_first;
    out->shadow_min_tris_first = t.min_tris_shadow_first;
    out->extend_variant_first = t.extend_variant_first;
    out->shade_variant_first = t.shade_variant_first;
}
}  // namespace

int pt_autotune(pt_context* c, int32_t num_passes, pt_tuning* out) {
    if (!c || !out || num_passes <= 0) return set_err(PT_ERR_INVALID_ARG, "invalid argument");
    RenderWork w;
    w.x0 = w.y0 = 0;
    w.w = c->opts.render_width;
    w.h = c->opts.render_height;
    w.first_pass = 0;
    // trial frames of at least 2^23 paths: on small images a frame of a few
    // passes is too short to time the candidates apart
    const long npix = (long)w.w * w.h;
    w.num_passes = (int)std::max<long>(num_passes, ((1L << 23) + npix - 1) / std::max(npix, 1L));
    w.tile_frame = -1;
    w.tile_x = w.tile_y = 0;
    const int cap = wavefront_capacity(c, w);
    if (c->wf.capacity < cap) CK(wavefront_alloc(c->wf, cap));
    if (!c->wf_tuned) {
        CK(wavefront_default_tuning(c->wf_tuning, 128));
        c->wf_tuned = true;
    }
    // the candidates render into a scratch accumulation; the caller's is kept
    DevBuf<float4> scratch;
    CK(scratch.alloc(c->accum.n));
    std::swap(c->accum, scratch);
    const bool postpone = trav_postpone_fits(c->bvh.tlas_depth + c->bvh.blas_depth);
    StageTimer timer;
    int rc = PT_OK;
    // device time per stage of a frame with tuning t: the fastest of three
    // timed frames after one untimed one
    auto measure = [&](const WavefrontTuning& t, float ms[STAGE_COUNT]) -> int {
        for (int k = 0; k < STAGE_COUNT; ++k) ms[k] = 1e30f;
        Params p = make_params(c);
        for (int rep = 0; rep < 4; ++rep) {
            timer.reset();
            CK(launch_wavefront(p, w, c->wf, t, false, c->stream, nullptr, rep ? &timer : nullptr));
            if (!rep) continue;
            float m[STAGE_COUNT];
            int n[STAGE_COUNT];
            CK(timer.summarise(m, n));
            for (int k = 0; k < STAGE_COUNT; ++k) ms[k] = std::min(ms[k], m[k]);
        }
        return PT_OK;
    };
    WavefrontTuning best = c->wf_tuning;
    if (!postpone) best.min_tris = best.min_tris_first = best.min_tris_shadow_first = 0;
    float ms[STAGE_COUNT];
    do {
        // 1. kernel variants, extend and shadow chosen separately
        float be = 1e30f, bs = 1e30f;
        int ve = best.extend_variant, vs = best.shadow_variant;
        for (int v = 0; v < 4; ++v) {
            WavefrontTuning t = best;
            t.extend_variant = t.shadow_variant = v;
            if ((rc = measure(t, ms))) break;
            if (ms[STAGE_EXTEND] < be) { be = ms[STAGE_EXTEND]; ve = v; }
            if (ms[STAGE_SHADOW] < bs) { bs = ms[STAGE_SHADOW]; vs = v; }
        }
        if (rc) break;
        best.extend_variant = ve;
        best.shadow_variant = vs;
        // 2. refill thresholds, separately
        const int refills[] = {8, 12, 16, 20, 24, 28};
        be = bs = 1e30f;
        int re = best.extend_refill, rs = best.shadow_refill;
        for (int r : refills) {
            WavefrontTuning t = best;
            t.extend_refill = t.shadow_refill = r;
            if ((rc = measure(t, ms))) break;
            if (ms[STAGE_EXTEND] < be) { be = ms[STAGE_EXTEND]; re = r; }
            if (ms[STAGE_SHADOW] < bs) { bs = ms[STAGE_SHADOW]; rs = r; }
        }
        if (rc) break;
        best.extend_refill = re;
        best.shadow_refill = rs;
        // 3. triangle postponement (shared by both stages)
        if (postpone) {
            const int mins[] = {0, 4, 6, 8, 12};
            float bt = 1e30f;
            int mt = best.min_tris;
            for (int m : mins) {
                WavefrontTuning t = best;
                t.min_tris = m;
                if ((rc = measure(t, ms))) break;
                const float tot = ms[STAGE_EXTEND] + ms[STAGE_SHADOW];
                if (tot < bt) { bt = tot; mt = m; }
            }
            if (rc) break;
            best.min_tris = mt;
        }
        // 4. register budget of the plain surface shading stage
        {
            float bsh = 1e30f;
            int vsh = best.shade_variant;
            for (int v = 0; v < 3; ++v) {
                WavefrontTuning t = best;
                t.shade_variant = v;
                if ((rc = measure(t, ms))) break;
                if (ms[STAGE_SHADE] < bsh) { bsh = ms[STAGE_SHADE]; vsh = v; }
            }
            if (rc) break;
            best.shade_variant = vsh;
        }
        // 5. the first round on its own (camera rays, coherent per warp, and
        // the shadow rays of their hits): refill threshold and quorum
        if (postpone) {
            const int rf[] = {20, 24, 28, 32};
            const int mf[] = {1, 2, 3, 4, 6};
            float be1 = 1e30f, bs1 = 1e30f;
            int re1 = 0, me1 = -1, rs1 = 0, ms1 = -1;
            for (int r : rf) {
                for (int m : mf) {
                    WavefrontTuning t = best;
                    t.extend_refill_first = t.shadow_refill_first = r;
                    t.min_tris_first = t.min_tris_shadow_first = m;
                    if ((rc = measure(t, ms))) break;
                    if (ms[STAGE_EXTEND] < be1) { be1 = ms[STAGE_EXTEND]; re1 = r; me1 = m; }
                    if (ms[STAGE_SHADOW] < bs1) { bs1 = ms[STAGE_SHADOW]; rs1 = r; ms1 = m; }
                }
                if (rc) break;
            }
            if (rc) break;
            // against the other rounds' own setting
            WavefrontTuning t = best;
            if ((rc = measure(t, ms))) break;
            if (be1 < ms[STAGE_EXTEND]) { best.extend_refill_first = re1; best.min_tris_first = me1; }
            if (bs1 < ms[STAGE_SHADOW]) { best.shadow_refill_first = rs1; best.min_tris_shadow_first = ms1; }
            // 6. the other rounds' refill thresholds and quorum again, now
            // that they no longer set the first round's
            const int refills[] = {8, 12, 16, 20, 24, 28};
            float be2 = 1e30f, bs2 = 1e30f;
            int re2 = best.extend_refill, rs2 = best.shadow_refill;
            for (int r : refills) {
                WavefrontTuning u = best;
                u.extend_refill = u.shadow_refill = r;
                if ((rc = measure(u, ms))) break;
                if (ms[STAGE_EXTEND] < be2) { be2 = ms[STAGE_EXTEND]; re2 = r; }
                if (ms[STAGE_SHADOW] < bs2) { bs2 = ms[STAGE_SHADOW]; rs2 = r; }
            }
            if (rc) break;
            best.extend_refill = re2;
            best.shadow_refill = rs2;
            const int mins[] = {0, 4, 6, 8, 12};
            float bt = 1e30f;
            int mt = best.min_tris;
            for (int m : mins) {
                WavefrontTuning u = best;
                u.min_tris = m;
                if ((rc = measure(u, ms))) break;
                const float tot = ms[STAGE_EXTEND] + ms[STAGE_SHADOW];
                if (tot < bt) { bt = tot; mt = m; }
            }
            if (rc) break;
            best.min_tris = mt;
        }
        // 7. the first round's extend kernel variant and shading budget
        {
            WavefrontTuning t = best;
            if ((rc = measure(t, ms))) break;
            float be3 = ms[STAGE_EXTEND], bsh3 = ms[STAGE_SHADE];
            int ve3 = -1, vs3 = -1;
            for (int v = 0; v < 4; ++v) {
                if (v == best.extend_variant) continue;
                WavefrontTuning u = best;
                u.extend_variant_first = v;
                if ((rc = measure(u, ms))) break;
                if (ms[STAGE_EXTEND] < be3) { be3 = ms[STAGE_EXTEND]; ve3 = v; }
            }
            if (rc) break;
            for (int v = 0; v < 3; ++v) {
                if (v == best.shade_variant) continue;
                WavefrontTuning u = best;
                u.shade_variant_first = v;
                if ((rc = measure(u, ms))) break;
                if (ms[STAGE_SHADE] < bsh3) { bsh3 = ms[STAGE_SHADE]; vs3 = v; }
            }
            if (rc) break;
            best.extend_variant_first = ve3;
            best.shade_variant_first = vs3;
        }
        if ((rc = measure(best, ms))) break;
    } while (false);
    timer.release();
    std::swap(c->accum, scratch);
    scratch.free();
    c->fwd.valid = false;
    if (rc) return rc;
    c->wf_tuning = best;
    float total = 0.0f;
    for (int k = 0; k < STAGE_COUNT; ++k) total += ms[k];
    tuning_out(best, total, out);
    return PT_OK;
}

int pt_get_tuning(pt_context* c, pt_tuning* out) {
    if (!c || !out) return set_err(PT_ERR_INVALID_ARG, "NULL argument");
    if (!c->wf_tuned) {
        CK(wavefront_default_tuning(c->wf_tuning, 128));
        c->wf_tuned = true;
    }
    tuning_out(c->wf_tuning, 0.0f, out);
    return PT_OK;
}

int pt_set_tuning(pt_context* c, const pt_tuning* in) {
    if (!c || !in) return set_err(PT_ERR_INVALID_ARG, "NULL argument");
    if (in->extend_variant < 0 || in->extend_variant > 3 || in->shadow_variant < 0 || in->shadow_variant > 3 ||
        in->extend_refill < 1 || in->extend_refill > 32 || in->shadow_refill < 1 || in->shadow_refill > 32 ||
        in->min_tris < 0 || in->min_tris > 32 || in->shade_variant < 0 || in->shade_variant > 2 ||
        in->extend_refill_first < 0 || in->extend_refill_first > 32 || in->shadow_refill_first < 0 ||
        in->shadow_refill_first > 32 || in->min_tris_first < -1 || in->min_tris_first > 32 ||
        in->shadow_min_tris_first < -1 || in->shadow_min_tris_first > 32 || in->extend_variant_first < -1 ||
        in->extend_variant_first > 3 || in->shade_variant_first < -1 || in->shade_variant_first > 2)
        return set_err(PT_ERR_INVALID_ARG, "tuning value out of range");
    if (!c->wf_tuned) {
        CK(wavefront_default_tuning(c->wf_tuning, 128));
        c->wf_tuned = true;
    }
    c->wf_tuning.extend_variant = in->extend_variant;
    c->wf_tuning.shadow_variant = in->shadow_variant;
    c->wf_tuning.extend_refill = in->extend_refill;
    c->wf_tuning.shadow_refill = in->shadow_refill;
    c->wf_tuning.min_tris = in->min_tris;
    c->wf_tuning.shade_variant = in->shade_variant;
    c->wf_tuning.extend_refill_first = in->extend_refill_first;
    c->wf_tuning.min_tris_first = in->min_tris_first;
    c->wf_tuning.shadow_refill_first = in->shadow_refill_first;
    c->wf_tuning.min_tris_shadow_first = in->shadow_min_tris_first;
    c->wf_tuning.extend_variant_first = in->extend_variant_first;
    c->wf_tuning.shade_variant_first = in->shade_variant_first;
    return PT_OK;
}

int pt_set_stage_timing(pt_context* c, int32_t on) {
    if (!c) return set_err(PT_ERR_INVALID_ARG, "context is NULL");
    c->stage_timing = on != 0;
    c->timer.reset();
    return PT_OK;
}

int pt_get_stage_stats(pt_context* c, pt_stage_stats* s) {
    if (!c || !s) return set_err(PT_ERR_INVALID_ARG, "NULL argument");
    float ms[STAGE_COUNT];
    int n[STAGE_COUNT];
    CK(c->timer.summarise(ms, n));
    for (int k = 0; k < STAGE_COUNT; ++k) {
        s->ms[k] = ms[k];
        s->launches[k] = n[k];
    }
    return PT_OK;
}

int pt_get_stats(pt_context* c, pt_stats* s) {
    if (!c || !s) return set_err(PT_ERR_INVALID_ARG, "NULL argument");
    unsigned long long cnt[5] = {0, 0, 0, 0, 0};
    int st = 0;
    CK(cudaMemcpyAsync(cnt, c->counters.p, sizeof cnt, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&st, c->status.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    float ms = 0.0f;
    if (c->timed) CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    s->closest_rays = cnt[0];
    s->shadow_rays = cnt[1];
    s->paths = cnt[2];
    s->truncated_paths = cnt[3];
    s->untraced_shadow_rays = cnt[4];
    s->kernel_ms = ms;
    s->status = st;
    s->kernel_launches = c->launches;
    return PT_OK;
}

}  // extern "C"
