// pt_kernels.cu - the megakernel integrator and the utility kernels (sm_103a).
//
//   render_kernel        tile.glsl:main + PathTrace (common/pathtrace.glsl:285)
//                        as one megakernel: one thread per pixel, looping over
//                        the sample passes of the launch; shadow rays inline
//   trace_closest_kernel test hook: ClosestHit's triangle part on a ray set
//   trace_shadow_kernel  test hook: AnyHit's triangle part on a ray set
//   bsdf_eval_kernel,    test hooks: DisneyEval / DisneySample
//   bsdf_sample_kernel   (disney.glsl:142-351) on explicit inputs
//   tonemap_kernel       tonemap.glsl:main + the RGBA8 read-back format
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pt_cuda.h"
#include "pt_integrator.cuh"

namespace ptgb {

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
        for (int pass = W.first_pass; pass < W.first_pass + W.num_passes; ++pass) {
            PathState ps;
            StartPath(P, px, py, FrameNumber(P, W, pass, px, py), ps);
            // Alpha pass-through keeps the depth (pathtrace.glsl:423); the loop
            // is bounded all the same (PT_MAX_PATH_ITERATIONS), and a path
            // that runs out is counted (pt_stats.truncated_paths).
            for (int guard = 0;; ) {
                if (++guard > PT_MAX_PATH_ITERATIONS) {
                    count_truncated(P);
                    break;
                }
                HitRecord hr;
                TraceClosest(P, ps.r, ps.depth, hr, stack, cnt, false);
                ShadowReq sr;
                NoHook nh;
                if (!ShadeStep<MEDIUM, ENV, true>(P, ps, hr, sr, stack, cnt, nh)) break;
            }
            acc.x += ps.radiance.x;
            acc.y += ps.radiance.y;
            acc.z += ps.radiance.z;
            acc.w += ps.alpha;
            ++paths;
        }
        *out = acc;
    }
    add_counters(P, cnt.closest, cnt.shadow, paths);
    add_untraced(P, cnt.untraced);
}

__global__ void __launch_bounds__(128) trace_closest_kernel(Params P, const pt_ray* __restrict__ rays, int n,
                                                            pt_hit* __restrict__ hits) {
    uint2 stack[kStackSize];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const pt_ray rr = rays[i];
    Trav h;
    trace_closest(h, P, v3(rr.origin[0], rr.origin[1], rr.origin[2]),
                  v3(rr.direction[0], rr.direction[1], rr.direction[2]), PT_INF, stack);
    pt_hit o;
    if (h.prim >= 0) {
        o.t = h.tmax; o.u = h.u; o.v = h.v; o.prim_id = h.prim; o.inst_id = h.inst;
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
    occ[i] = trace_any(P, v3(rr.origin[0], rr.origin[1], rr.origin[2]),
                       v3(rr.direction[0], rr.direction[1], rr.direction[2]), maxd[i], alpha, rng, stack)
                 ? 1
                 : 0;
}

// BSDF inputs: 20 floats per record (baseColor xyz, metallic, roughness,
// subsurface, specularTint, sheen, sheenTint, clearcoat, clearcoatRoughness,
// specTrans, ior, ax, ay, eta, anisotropic, 3 unused), as GetMaterial
// leaves them after its remapping (pathtrace.glsl:25-115).
__device__ __forceinline__ Material bsdf_material(const float* __restrict__ r, float& eta) {
    Material m{};
    m.baseColor = v3(r[0], r[1], r[2]);
    m.metallic = r[3];
    m.roughness = r[4];
    m.subsurface = r[5];
    m.specularTint = r[6];
    m.sheen = r[7];
    m.sheenTint = r[8];
    m.clearcoat = r[9];
    m.clearcoatRoughness = r[10];
    m.specTrans = r[11];
    m.ior = r[12];
    m.ax = r[13];
    m.ay = r[14];
    eta = r[15];
    m.anisotropic = r[16];
    return m;
}

__device__ __forceinline__ V3 load_v3(const float* __restrict__ p, int i) {
    return v3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}

__global__ void __launch_bounds__(128) bsdf_eval_kernel(const float* __restrict__ rec, const float* __restrict__ V,
                                                        const float* __restrict__ N, const float* __restrict__ L,
                                                        int n, float* __restrict__ f, float* __restrict__ pdf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float eta;
    const Material m = bsdf_material(rec + 20 * (size_t)i, eta);
    float p;
    const V3 r = DisneyEval(m, eta, load_v3(V, i), load_v3(N, i), load_v3(L, i), p);
    f[3 * i] = r.x;
    f[3 * i + 1] = r.y;
    f[3 * i + 2] = r.z;
    pdf[i] = p;
}

__global__ void __launch_bounds__(128) bsdf_sample_kernel(const float* __restrict__ rec, const float* __restrict__ V,
                                                          const float* __restrict__ N,
                                                          const uint32_t* __restrict__ seeds, int n,
                                                          float* __restrict__ L, float* __restrict__ f,
                                                          float* __restrict__ pdf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float eta;
    const Material m = bsdf_material(rec + 20 * (size_t)i, eta);
    Rng rng;
    rng.x = seeds[4 * i];
    rng.y = seeds[4 * i + 1];
    rng.z = seeds[4 * i + 2];
    rng.w = seeds[4 * i + 3];
    float p;
    V3 l;
    const V3 r = DisneySample(m, eta, load_v3(V, i), load_v3(N, i), l, p, rng);
    L[3 * i] = l.x;
    L[3 * i + 1] = l.y;
    L[3 * i + 2] = l.z;
    f[3 * i] = r.x;
    f[3 * i + 1] = r.y;
    f[3 * i + 2] = r.z;
    pdf[i] = p;
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

cudaError_t launch_bsdf_eval(const float* rec, const float* V, const float* N, const float* L, int n, float* f,
                             float* pdf, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    bsdf_eval_kernel<<<(n + 127) / 128, 128, 0, s>>>(rec, V, N, L, n, f, pdf);
    return cudaGetLastError();
}

cudaError_t launch_bsdf_sample(const float* rec, const float* V, const float* N, const uint32_t* seeds, int n,
                               float* L, float* f, float* pdf, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    bsdf_sample_kernel<<<(n + 127) / 128, 128, 0, s>>>(rec, V, N, seeds, n, L, f, pdf);
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
