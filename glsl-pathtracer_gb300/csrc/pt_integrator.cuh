// pt_integrator.cuh - the path integrator of common/pathtrace.glsl as one
// step per path vertex, shared by the megakernel and the wavefront kernels.
//
//   TraceClosest   ClosestHit's queries (closest_hit.glsl:25-218): analytic
//                  lights, then the BVH; fills a HitRecord
//   ShadeStep      one iteration of PathTrace's loop (pathtrace.glsl:301-473)
//                  given the HitRecord: misses, emission, MIS, media, alpha
//                  pass-through, next-event estimation (DirectLight,
//                  pathtrace.glsl:158-283), BSDF sampling, Russian roulette
//
// Next-event estimation's shadow rays are traced inline (megakernel, and any
// scene where the reference's AnyHit or EvalTransmittance consume random
// numbers: alpha-tested materials, volumes with VOL_MIS) or returned as a
// ShadowReq for a separate shadow stage (wavefront).  The contributions are
// computed with the same operations either way, so both forms add the same
// float values in the same order: a path renders identically in both.
#pragma once

#include "pt_trace.cuh"

namespace ptgb {

struct PathState {
    Ray r;
    V3 throughput, radiance;
    float alpha;
    Rng rng;
    int depth;
    int matID;          // state.matID: kept when the hit is a light (pathtrace.glsl:341)
    float prevRough;    // state.mat.roughness of the last vertex (roughness mollification)
    float scatterPdf;   // scatterSample.pdf of the last bounce (MIS weights)
    bool inMedium, surfaceScatter;
    Medium medium;      // state.medium
    int job = 0;        // job of a batch (pt_batch_render)
};

struct HitRecord {
    bool hit, isEmitter;
    float t, u, v, w;
    int prim, inst, mat;
    float lightPdf;
    V3 lightEmission;
    int light;  // index of the light hit (isEmitter)
};

struct ShadowReq {
    int n;              // shadow rays: bit 0 env ray, bit 1 light ray
    int adds;           // bit k: ray k contributes when unoccluded
    V3 origin;          // scatterPos (pathtrace.glsl:162)
    V3 dir[2];
    float maxd[2];
    V3 contrib[2];      // misWeight * Li * f / pdf of ray k (env, light)
    V3 T;               // throughput the result is multiplied by
    // deferred transmittance (VOL_MIS): contrib[k] holds Li, and the
    // contribution is formed from Li * transmittance in the reference's
    // operation order with these factors (ResolveTransmit)
    V3 fac[2];          // env: f; light: misWeight * f
    float mis[2];       // env: misWeight
    float pdf[2];       // the light sample's pdf
    bool suspended;     // a transmittance query is pending (replay, wf_shade)
};

struct Counters {
    uint32_t closest, shadow;
    uint32_t untraced;  // of shadow: answered without traversal (DirectLight)
};

// ------------------------------------------------------------ ClosestHit
// The analytic-light part of ClosestHit (closest_hit.glsl:30-86): returns the
// nearest light distance (INF if none) and fills the light fields of hr.
__device__ __forceinline__ float LightsClosest(const Params& P, const Ray& r, int depth, HitRecord& hr) {
    float t = PT_INF;
    hr.isEmitter = false;
    if ((P.flags & F_LIGHTS) && !((P.flags & F_HIDE_EMITTERS) && !(depth > 0))) {  // closest_hit.glsl:30-86
        for (int i = 0; i < P.num_lights; i++) {
            const Light L = LoadLight(P.lights, i);
            const int type = (int)L.type;
            if (type == QUAD_LIGHT) {
                V3 normal = normalize(cross(L.u, L.v));
                if (dot(normal, r.direction) > 0.0f) continue;
                float pw = dot(normal, L.position);
                V3 u = L.u * (1.0f / dot(L.u, L.u));
                V3 v = L.v * (1.0f / dot(L.v, L.v));
                float d = RectIntersect(L.position, u, v, normal, pw, r);
                if (d < 0.0f) d = PT_INF;
                if (d < t) {
                    t = d;
                    float cosTheta = dot(-r.direction, normal);
                    hr.lightPdf = (t * t) / (L.area * cosTheta);
                    hr.lightEmission = L.emission;
                    hr.isEmitter = true;
                    hr.light = i;
                }
            }
            if (type == SPHERE_LIGHT) {
                float d = SphereIntersect(L.radius, L.position, r);
                if (d < 0.0f) d = PT_INF;
                if (d < t) {
                    t = d;
                    V3 hitPt = r.origin + t * r.direction;
                    float cosTheta = dot(-r.direction, normalize(hitPt - L.position));
                    hr.lightPdf = (t * t) / (L.area * cosTheta * 0.5f);
                    hr.lightEmission = L.emission;
                    hr.isEmitter = true;
                    hr.light = i;
                }
            }
        }
    }
    return t;
}

// The HitRecord of a finished closest-hit traversal (the end of
// closest_hit.glsl:220-228): a triangle closer than the lights wins.
__device__ __forceinline__ void FinishClosest(const Trav& s, float tLight, HitRecord& hr) {
    float t = tLight;
    if (s.prim >= 0) {
        t = s.tmax;
        hr.isEmitter = false;
    }
    hr.hit = t != PT_INF;
    hr.t = t;
    hr.prim = s.prim;
    hr.inst = s.inst;
    hr.mat = s.mat;
    hr.u = s.u;
    hr.v = s.v;
    hr.w = __fsub_rn(__fsub_rn(1.0f, s.u), s.v);  // uvt.w, as the triangle test computed it
}

__device__ __forceinline__ void TraceClosest(const Params& P, const Ray& r, int depth, HitRecord& hr, uint2* stack,
                                             Counters& cnt, bool count_as_shadow) {
    if (count_as_shadow) cnt.shadow++;
    else cnt.closest++;
    const float tl = LightsClosest(P, r, depth, hr);
    Trav s;
    trace_closest(s, P, r.origin, r.direction, tl, stack);
    FinishClosest(s, tl, hr);
}

// Shading attributes of a triangle hit (closest_hit.glsl:224-247).
// Texture coordinate and tangent frame of a triangle hit (closest_hit.glsl:
// 227-263); filled only when the scene has texture maps.
struct Surface {
    float u = 0.0f, v = 0.0f;
    V3 T = {0.0f, 0.0f, 0.0f}, B = {0.0f, 0.0f, 0.0f};
};

__device__ __forceinline__ void HitNormal(const Params& P, const HitRecord& hr, const Ray& r, V3& normal, V3& ffnormal,
                                          Surface* surf = nullptr) {
    const int i0 = __ldg(P.vidx + 3 * hr.prim), i1 = __ldg(P.vidx + 3 * hr.prim + 1), i2 = __ldg(P.vidx + 3 * hr.prim + 2);
    const float4 n0 = __ldg(P.norms + i0), n1 = __ldg(P.norms + i1), n2 = __ldg(P.norms + i2);
    V3 n = normalize(v3(n0) * hr.w + v3(n1) * hr.u + v3(n2) * hr.v);  // bary = uvt.wxy
    if (hr.inst >= 0) {
        const float4* x = P.xf + 10 * hr.inst + 7;
        const float4 c0 = __ldg(x), c1 = __ldg(x + 1), c2 = __ldg(x + 2);
        n = v3(c0.x * n.x + c1.x * n.y + c2.x * n.z, c0.y * n.x + c1.y * n.y + c2.y * n.z,
               c0.z * n.x + c1.z * n.y + c2.z * n.z);
    }
    normal = normalize(n);
    ffnormal = dot(normal, r.direction) <= 0.0f ? normal : -normal;
    if (surf && (P.flags & F_TEXTURES)) {
        const float4 p0 = __ldg(P.verts + i0), p1 = __ldg(P.verts + i1), p2 = __ldg(P.verts + i2);
        surf->u = p0.w * hr.w + p1.w * hr.u + p2.w * hr.v;
        surf->v = n0.w * hr.w + n1.w * hr.u + n2.w * hr.v;
        const V3 dP1 = v3(p1) - v3(p0), dP2 = v3(p2) - v3(p0);
        const float du1 = p1.w - p0.w, dv1 = n1.w - n0.w, du2 = p2.w - p0.w, dv2 = n2.w - n0.w;
        const float invdet = 1.0f / (du1 * dv2 - dv1 * du2);
        V3 T = (dP1 * dv2 - dP2 * dv1) * invdet;
        V3 B = (dP2 * du1 - dP1 * du2) * invdet;
        if (hr.inst >= 0) {  // mat3(transform)
            const float4* m = P.xf + 10 * hr.inst + 4;
            const float4 c0 = __ldg(m), c1 = __ldg(m + 1), c2 = __ldg(m + 2);
            T = v3(c0.x * T.x + c1.x * T.y + c2.x * T.z, c0.y * T.x + c1.y * T.y + c2.y * T.z,
                   c0.z * T.x + c1.z * T.y + c2.z * T.z);
            B = v3(c0.x * B.x + c1.x * B.y + c2.x * B.z, c0.y * B.x + c1.y * B.y + c2.y * B.z,
                   c0.z * B.x + c1.z * B.y + c2.z * B.z);
        }
        surf->T = normalize(T);
        surf->B = normalize(B);
    }
}

__device__ __forceinline__ V3 pow22(float4 t) { return v3(powf(t.x, 2.2f), powf(t.y, 2.2f), powf(t.z, 2.2f)); }

// GetMaterial (pathtrace.glsl:25-115): the material record, its texture maps
// (base colour and opacity, metallic-roughness, normal map -- which bends
// normal / ffnormal -- and emission), roughness mollification, then ax / ay
// and eta.
// The texture-map part of GetMaterial, out of line: scenes without texture
// maps keep it out of the shading kernels' instruction stream.  The fields
// of Params it reads come as plain values (see SampleTexArray).
static __device__ __noinline__ void ApplyTextureMaps(const float4* mats, const uchar4* tex, int tex_w, int tex_h,
                                                     int num_tex, uint32_t flags, float mollify_amt, int matID,
                                                     int depth, float prevRough, V3& normal, V3& ffnormal,
                                                     const Surface& sf, const Ray& r, Material& mat) {
    {
        const float4 ids = __ldg(mats + 8 * matID + 6);  // baseColor, metallicRoughness, normalmap, emission
        if ((int)ids.x >= 0) {
            const float4 t = SampleTexArray(tex, tex_w, tex_h, num_tex, sf.u, sf.v, ids.x);
            mat.baseColor = mat.baseColor * pow22(t);
            mat.opacity *= t.w;
        }
        if ((int)ids.y >= 0) {
            const float4 t = SampleTexArray(tex, tex_w, tex_h, num_tex, sf.u, sf.v, ids.y);
            mat.metallic = t.z;
            mat.roughness = fmaxf(t.y * t.y, 0.001f);
        }
        if ((int)ids.z >= 0) {
            const float4 t = SampleTexArray(tex, tex_w, tex_h, num_tex, sf.u, sf.v, ids.z);
            V3 tn = v3(t.x, t.y, t.z);
            if (flags & F_OPENGL_NORMALMAP) tn.y = 1.0f - tn.y;
            tn = normalize(tn * 2.0f - v3(1.0f));
            const V3 orig = normal;
            normal = normalize(sf.T * tn.x + sf.B * tn.y + normal * tn.z);
            ffnormal = dot(orig, r.direction) <= 0.0f ? normal : -normal;
        }
        if ((flags & F_MOLLIFY) && depth > 0)
            mat.roughness = fmaxf(mixf(0.0f, prevRough, mollify_amt), mat.roughness);
        if ((int)ids.w >= 0) mat.emission = pow22(SampleTexArray(tex, tex_w, tex_h, num_tex, sf.u, sf.v, ids.w));
    }
}

__device__ __forceinline__ void GetMaterial(const Params& P, int matID, int depth, float prevRough, V3& normal,
                                            V3& ffnormal, const Surface& sf, const Ray& r, Material& mat,
                                            float& eta) {
    LoadMaterial(P.mats, matID, mat);
    if (P.flags & F_TEXTURES)
        ApplyTextureMaps(P.mats, P.tex, P.tex_w, P.tex_h, P.num_tex, P.flags, P.mollify_amt, matID, depth, prevRough,
                         normal, ffnormal, sf, r, mat);
    else if ((P.flags & F_MOLLIFY) && depth > 0)
        mat.roughness = fmaxf(mixf(0.0f, prevRough, P.mollify_amt), mat.roughness);
    FinishMaterial(mat);
    eta = dot(r.direction, normal) < 0.0f ? (1.0f / mat.ior) : mat.ior;
}

__device__ __forceinline__ bool AlphaSkip(const Material& m, Rng& rng) {
    if (m.alphaMode == ALPHA_MODE_MASK && m.opacity < m.alphaCutoff) return true;
    if (m.alphaMode == ALPHA_MODE_BLEND) return rng.next() > m.opacity;
    return false;
}

// The analytic-light part of AnyHit (anyhit.glsl:28-63).
__device__ __forceinline__ bool LightsAny(const Params& P, const Ray& r, float maxDist) {
    if (P.flags & F_LIGHTS) {
        for (int i = 0; i < P.num_lights; i++) {
            const Light L = LoadLight(P.lights, i);
            const int type = (int)L.type;
            if (type == QUAD_LIGHT) {
                V3 normal = normalize(cross(L.u, L.v));
                float pw = dot(normal, L.position);
                V3 u = L.u * (1.0f / dot(L.u, L.u));
                V3 v = L.v * (1.0f / dot(L.v, L.v));
                float d = RectIntersect(L.position, u, v, normal, pw, r);
                if (d > 0.0f && d < maxDist) return true;
            }
            if (type == SPHERE_LIGHT) {
                float d = SphereIntersect(L.radius, L.position, r);
                if (d > 0.0f && d < maxDist) return true;
            }
        }
    }
    return false;
}

// anyhit.glsl:25-216
// Whether AnyHit draws random numbers (the alpha test of anyhit.glsl:118-141,
// which the reference compiles without media only).
__device__ __forceinline__ bool any_hit_draws(const Params& P) {
    return (P.flags & F_ALPHA_TEST) && !(P.flags & F_MEDIUM);
}
static __device__ __noinline__ bool AnyHit(const Params& P, const Ray& r, float maxDist, Rng& rng, uint2* stack,
                                           Counters& cnt) {
    cnt.shadow++;
    if (LightsAny(P, r, maxDist)) return true;
    return trace_any(P, r.origin, r.direction, maxDist, any_hit_draws(P), rng, stack);
}

// pathtrace.glsl:118-156 (OPT_MEDIUM && OPT_VOL_MIS); each segment is counted
// as a shadow query.
// One hit of EvalTransmittance's segment loop (pathtrace.glsl:124-150):
// 0 = the ray ends here (miss or light), 1 = continue from the new origin,
// 2 = blocked (transmittance 0).  Draws a random number only at an
// ALPHA_MODE_BLEND material.
__device__ __forceinline__ int TransmitStep(const Params& P, const HitRecord& hr, Ray& r, V3& transmittance,
                                            Rng& rng) {
    if (!hr.hit || hr.isEmitter) return 0;
    V3 normal, ffnormal;
    Surface sf;
    HitNormal(P, hr, r, normal, ffnormal, &sf);
    Material mat;
    float eta;
    GetMaterial(P, hr.mat, 0, 0.0f, normal, ffnormal, sf, r, mat, eta);
    bool alphatest = AlphaSkip(mat, rng);
    bool refractive = (1.0f - mat.metallic) * mat.specTrans > 0.0f;
    if (!(alphatest || refractive)) return 2;
    if (dot(r.direction, normal) > 0.0f && mat.medium.type != MEDIUM_NONE) {
        V3 color = mat.medium.type == MEDIUM_ABSORB ? v3(1.0f) - mat.medium.color : v3(1.0f);
        transmittance = transmittance * vexp(-color * mat.medium.density * hr.t);
    }
    r.origin = madd_rn(madd_rn(r.origin, r.direction, hr.t), r.direction, PT_EPS);
    return 1;
}

static __device__ __noinline__ V3 EvalTransmittance(const Params& P, Ray r, Rng& rng, uint2* stack, Counters& cnt) {
    V3 transmittance = v3(1.0f);
    for (int depth = 0; depth < P.max_depth; depth++) {
        HitRecord hr;
        TraceClosest(P, r, 0, hr, stack, cnt, true);
        const int st = TransmitStep(P, hr, r, transmittance, rng);
        if (st == 0) break;
        if (st == 2) return v3(0.0f);
    }
    return transmittance;
}

// Ld of a deferred VOL_MIS request from the transmittances of its rays, with
// the operations of DirectLight's VOL_MIS branches (pathtrace.glsl:174-190,
// 240-256): Li *= transmittance, then the env term
// misWeight * Li * f * envMapIntensity / lightPdf and the light term
// misWeight * f * Li / pdf, env first.
__device__ __forceinline__ V3 ResolveTransmit(const ShadowReq& sr, V3 T0, V3 T1, float env_intensity) {
    V3 Ld = v3(0.0f);
    if (sr.n & sr.adds & 1) {
        const V3 Li = sr.contrib[0] * T0;
        Ld = Ld + sr.mis[0] * Li * sr.fac[0] * env_intensity / sr.pdf[0];
    }
    if (sr.n & sr.adds & 2) {
        const V3 Li = sr.contrib[1] * T1;
        Ld = Ld + sr.fac[1] * Li / sr.pdf[1];
    }
    return Ld;
}

// ------------------------------------------------------------ envmap
// envmap.glsl:28-55
__device__ __forceinline__ void BinarySearch(const Params& P, float value, float& u, float& v) {
    const int W = P.env_w, H = P.env_h;
    int lower = 0, upper = H - 1;
    while (lower < upper) {
        int mid = (lower + upper) >> 1;
        if (value < __ldg(P.cdf + (size_t)mid * W + (W - 1))) upper = mid;
        else lower = mid + 1;
    }
    const int y = min(max(lower, 0), H - 1);
    lower = 0;
    upper = W - 1;
    while (lower < upper) {
        int mid = (lower + upper) >> 1;
        if (value < __ldg(P.cdf + (size_t)y * W + mid)) upper = mid;
        else lower = mid + 1;
    }
    const int x = min(max(lower, 0), W - 1);
    u = (float)x / (float)W;
    v = (float)y / (float)H;
}

// texture(envMapTex, uv): bilinear, GL_REPEAT (Renderer.cpp:213-218)
__device__ __forceinline__ V3 SampleEnv(const Params& P, float u, float v) {
    const int W = P.env_w, H = P.env_h;
    float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    float fx = floorf(x), fy = floorf(y);
    float ax = x - fx, ay = y - fy;
    int ix = (int)fx, iy = (int)fy;
    int x0 = ix % W; x0 += x0 < 0 ? W : 0;
    int y0 = iy % H; y0 += y0 < 0 ? H : 0;
    int x1 = x0 + 1 == W ? 0 : x0 + 1;
    int y1 = y0 + 1 == H ? 0 : y0 + 1;
    const float4 a = __ldg(P.env + (size_t)y0 * W + x0), b = __ldg(P.env + (size_t)y0 * W + x1);
    const float4 c = __ldg(P.env + (size_t)y1 * W + x0), d = __ldg(P.env + (size_t)y1 * W + x1);
    V3 t0 = v3(a) * (1.0f - ax) + v3(b) * ax;
    V3 t1 = v3(c) * (1.0f - ax) + v3(d) * ax;
    return t0 * (1.0f - ay) + t1 * ay;
}

// envmap.glsl:57-66
__device__ __forceinline__ V3 EvalEnvMap(const Params& P, const Ray& r, float& pdfOut) {
    float theta = acosf(clampf(r.direction.y, -1.0f, 1.0f));
    float u = (PT_PI + atan2f(r.direction.z, r.direction.x)) * PT_INV_TWO_PI + P.env_rot;
    float v = theta * PT_INV_PI;
    V3 color = SampleEnv(P, u, v);
    float pdf = Luminance(color) / P.env_total;
    pdfOut = (pdf * (float)P.env_w * (float)P.env_h) / (PT_TWO_PI * PT_PI * sinf(theta));
    return color;
}

// envmap.glsl:68-83
__device__ __forceinline__ V3 SampleEnvMap(const Params& P, V3& color, float& pdfOut, Rng& rng) {
    float u, v;
    BinarySearch(P, rng.next() * P.env_total, u, v);
    color = SampleEnv(P, u, v);
    float pdf = Luminance(color) / P.env_total;
    u -= P.env_rot;
    float phi = u * PT_TWO_PI;
    float theta = v * PT_PI;
    float st = sinf(theta), ct = cosf(theta);
    if (st == 0.0f) pdf = 0.0f;
    pdfOut = (pdf * (float)P.env_w * (float)P.env_h) / (PT_TWO_PI * PT_PI * st);
    float sp, cp;
    sincosf(phi, &sp, &cp);
    return v3(-st * cp, ct, -st * sp);
}

// sampling.glsl:186-248
__device__ __forceinline__ void SampleOneLight(const Params& P, const Light& light, V3 scatterPos, LightSample& ls,
                                               Rng& rng) {
    const int type = (int)light.type;
    if (type == QUAD_LIGHT) {
        float r1 = rng.next();
        float r2 = rng.next();
        V3 lightSurfacePos = light.position + light.u * r1 + light.v * r2;
        ls.direction = lightSurfacePos - scatterPos;
        ls.dist = length(ls.direction);
        float distSq = ls.dist * ls.dist;
        ls.direction = ls.direction / ls.dist;
        ls.normal = normalize(cross(light.u, light.v));
        ls.emission = light.emission * (float)P.num_lights;
        ls.pdf = distSq / (light.area * fabsf(dot(ls.normal, ls.direction)));
    } else if (type == SPHERE_LIGHT) {
        float r1 = rng.next();
        float r2 = rng.next();
        V3 c2s = scatterPos - light.position;
        float distToSphereCenter = length(c2s);
        c2s = c2s / distToSphereCenter;
        V3 sampledDir = UniformSampleHemisphere(r1, r2);
        V3 T, B;
        Onb(c2s, T, B);
        sampledDir = T * sampledDir.x + B * sampledDir.y + c2s * sampledDir.z;
        V3 lightSurfacePos = light.position + sampledDir * light.radius;
        ls.direction = lightSurfacePos - scatterPos;
        ls.dist = length(ls.direction);
        float distSq = ls.dist * ls.dist;
        ls.direction = ls.direction / ls.dist;
        ls.normal = normalize(lightSurfacePos - light.position);
        ls.emission = light.emission * (float)P.num_lights;
        ls.pdf = distSq / (light.area * 0.5f * fabsf(dot(ls.normal, ls.direction)));
    } else {
        ls.direction = normalize(light.position - v3(0.0f));
        ls.normal = normalize(scatterPos - light.position);
        ls.emission = light.emission * (float)P.num_lights;
        ls.dist = PT_INF;
        ls.pdf = 1.0f;
    }
}

// Scattering at the current vertex for next-event estimation: Disney BSDF on
// surfaces, Henyey-Greenstein phase function in media (pathtrace.glsl:181-188).
__device__ __forceinline__ V3 ScatterEval(bool isSurface, const Material& mat, float eta, V3 V, V3 ffnormal,
                                          float g, V3 L, float& pdf) {
    if (isSurface) return DisneyEval(mat, eta, V, ffnormal, L, pdf);
    float p = PhaseHG(dot(V, L), g);
    pdf = p;
    return v3(p);
}

// Whether the ray (t >= 0) may meet one of the world boxes of the scene's
// blended-alpha instances (Params::blend_boxes): the only geometry at which
// EvalTransmittance draws random numbers.  Slab test in FP32 against boxes
// the host has widened; a NaN in the test counts as a meeting.
__device__ __forceinline__ bool may_cross_blend(const Params& P, const Ray& r) {
    for (int k = 0; k < P.num_blend_boxes; ++k) {
        const float* b = P.blend_boxes + 6 * k;
        float t0 = 0.0f, t1 = PT_INF;
        bool miss = false;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float o = a == 0 ? r.origin.x : a == 1 ? r.origin.y : r.origin.z;
            const float d = a == 0 ? r.direction.x : a == 1 ? r.direction.y : r.direction.z;
            if (d == 0.0f) {
                if (o < b[a] || o > b[3 + a]) miss = true;
                continue;
            }
            const float ta = (b[a] - o) / d, tb = (b[3 + a] - o) / d;
            t0 = fmaxf(t0, fminf(ta, tb));
            t1 = fminf(t1, fmaxf(ta, tb));
        }
        if (!miss && !(t0 > t1)) return true;
    }
    return false;
}

// pathtrace.glsl:158-283.  INLINE: shadow rays traced here and the result
// returned; otherwise the rays and their contributions go to `sr` and the
// caller adds the unoccluded ones (same values, same order).
// A query whose contribution is never added (the scattering pdf towards the
// light is 0) is answered without traversal when Params::untraced allows it
// and the query draws no random numbers: an any-hit query when AnyHit has no
// alpha test, a VOL_MIS query when its ray cannot meet blended geometry
// (then it runs one segment in the reference, pathtrace.glsl:117-153).  Its
// result would be discarded; the counters record it as traced once.
template <int MEDIUM, bool ENV, bool INLINE, class Hook>
__device__ __forceinline__ V3 DirectLight(const Params& P, const Ray& r, V3 fhp, V3 normal, V3 ffnormal,
                                          const Material& mat, float eta, const Medium& medium, bool isSurface,
                                          Rng& rng, uint2* stack, Counters& cnt, ShadowReq& sr, Hook& hook) {
    V3 Ld = v3(0.0f);
    V3 Li = v3(0.0f);
    const V3 scatterPos = madd_rn(fhp, normal, PT_EPS);
    constexpr bool volmis = MEDIUM == 2;
    const V3 V = -r.direction;
    sr.n = 0;
    sr.adds = 0;
    sr.origin = scatterPos;
    if (ENV && (P.flags & F_ENVMAP)) {  // (a batch's job may have none)
        float lightPdf;
        V3 lightDir;
        if (!hook.env_sample(Li, lightPdf, lightDir)) {
            lightDir = SampleEnvMap(P, Li, lightPdf, rng);
            hook.env_sampled(Li, lightPdf, lightDir);
        }
        const Ray shadowRay{scatterPos, lightDir};
        if (volmis && INLINE) {
            float sfPdf;
            const V3 sf = ScatterEval(isSurface, mat, eta, V, ffnormal, medium.anisotropy, lightDir, sfPdf);
            const bool adds = sfPdf > 0.0f && PowerHeuristic(lightPdf, sfPdf) > 0.0f;
            if (!adds && (P.untraced & 2) && !may_cross_blend(P, shadowRay)) {
                if (hook.first_visit()) {
                    cnt.shadow++;
                    cnt.untraced++;
                }
            } else {
                V3 Tr;
                if (!hook.transmit(P, shadowRay, rng, stack, cnt, Tr)) {
                    sr.suspended = true;
                    return Ld;
                }
                Li = Li * Tr;
                if (sfPdf > 0.0f) {
                    float misWeight = PowerHeuristic(lightPdf, sfPdf);
                    if (misWeight > 0.0f) Ld = Ld + misWeight * Li * sf * P.env_intensity / lightPdf;
                }
            }
        } else if (volmis) {  // transmittance deferred to the transmittance stage
            float sfPdf;
            const V3 sf = ScatterEval(isSurface, mat, eta, V, ffnormal, medium.anisotropy, lightDir, sfPdf);
            sr.n |= 1;
            sr.dir[0] = lightDir;
            sr.contrib[0] = Li;
            sr.fac[0] = sf;
            sr.pdf[0] = lightPdf;
            sr.mis[0] = 0.0f;
            if (sfPdf > 0.0f) {
                float misWeight = PowerHeuristic(lightPdf, sfPdf);
                sr.mis[0] = misWeight;
                if (misWeight > 0.0f) sr.adds |= 1;
            }
        } else {
            float sfPdf = 0.0f;
            V3 c = v3(0.0f);
            bool adds = false;
            auto contribution = [&]() {
                const V3 sf = DisneyEval(mat, eta, V, ffnormal, lightDir, sfPdf);
                if (sfPdf > 0.0f) {
                    float misWeight = PowerHeuristic(lightPdf, sfPdf);
                    if (misWeight > 0.0f) {
                        c = misWeight * Li * sf * P.env_intensity / lightPdf;
                        adds = true;
                    }
                }
            };
            if (INLINE && (P.untraced & 1) && !any_hit_draws(P)) {
                // evaluated first: a query whose contribution is never
                // added is answered without traversal
                contribution();
                if (!adds) {
                    cnt.shadow++;
                    cnt.untraced++;
                } else if (!AnyHit(P, shadowRay, PT_INF - PT_EPS, rng, stack, cnt)) {
                    Ld = Ld + c;
                }
            } else if (INLINE) {
                if (!AnyHit(P, shadowRay, PT_INF - PT_EPS, rng, stack, cnt)) {
                    contribution();
                    if (adds) Ld = Ld + c;
                }
            } else {
                contribution();
                sr.n |= 1;
                sr.dir[0] = lightDir;
                sr.maxd[0] = PT_INF - PT_EPS;
                sr.contrib[0] = c;
                if (adds) sr.adds |= 1;
            }
        }
    }
    if (P.flags & F_LIGHTS) {
        LightSample ls;
        const int index = (int)(rng.next() * (float)P.num_lights);
        Light light;
        if (index < P.num_lights) light = LoadLight(P.lights, index);
        else {  // rand() == 1: one past the last light reads zeros (GL texelFetch out of range)
            light.position = light.emission = light.u = light.v = v3(0.0f);
            light.radius = light.area = light.type = 0.0f;
        }
        SampleOneLight(P, light, scatterPos, ls, rng);
        Li = ls.emission;
        if (dot(ls.direction, ls.normal) < 0.0f) {
            const Ray shadowRay{scatterPos, ls.direction};
            if (volmis && INLINE) {
                float sfPdf;
                const V3 sf = ScatterEval(isSurface, mat, eta, V, ffnormal, medium.anisotropy, ls.direction, sfPdf);
                if (!(sfPdf > 0.0f) && (P.untraced & 2) && !may_cross_blend(P, shadowRay)) {
                    if (hook.first_visit()) {
                        cnt.shadow++;
                        cnt.untraced++;
                    }
                } else {
                    V3 Tr;
                    if (!hook.transmit(P, shadowRay, rng, stack, cnt, Tr)) {
                        sr.suspended = true;
                        return Ld;
                    }
                    Li = Li * Tr;
                    float misWeight = 1.0f;
                    if (light.area > 0.0f) misWeight = PowerHeuristic(ls.pdf, sfPdf);
                    if (sfPdf > 0.0f) Ld = Ld + misWeight * sf * Li / ls.pdf;
                }
            } else if (volmis) {  // transmittance deferred to the transmittance stage
                float sfPdf;
                const V3 sf = ScatterEval(isSurface, mat, eta, V, ffnormal, medium.anisotropy, ls.direction, sfPdf);
                float misWeight = 1.0f;
                if (light.area > 0.0f) misWeight = PowerHeuristic(ls.pdf, sfPdf);
                sr.n |= 2;
                sr.dir[1] = ls.direction;
                sr.contrib[1] = Li;
                sr.fac[1] = misWeight * sf;
                sr.pdf[1] = ls.pdf;
                sr.mis[1] = misWeight;
                if (sfPdf > 0.0f) sr.adds |= 2;
            } else {
                float sfPdf = 0.0f;
                V3 c = v3(0.0f);
                bool adds = false;
                auto contribution = [&]() {
                    const V3 sf = DisneyEval(mat, eta, V, ffnormal, ls.direction, sfPdf);
                    float misWeight = 1.0f;
                    if (light.area > 0.0f) misWeight = PowerHeuristic(ls.pdf, sfPdf);
                    if (sfPdf > 0.0f) {
                        c = misWeight * Li * sf / ls.pdf;
                        adds = true;
                        hook.nee_light(index, misWeight, Li, sf, ls.pdf, eta, V, ffnormal, ls.direction);
                    }
                };
                if (INLINE && (P.untraced & 1) && !any_hit_draws(P)) {
                    contribution();
                    if (!adds) {
                        cnt.shadow++;
                        cnt.untraced++;
                    } else if (!AnyHit(P, shadowRay, ls.dist - PT_EPS, rng, stack, cnt)) {
                        Ld = Ld + c;
                    }
                } else if (INLINE) {
                    if (!AnyHit(P, shadowRay, ls.dist - PT_EPS, rng, stack, cnt)) {
                        contribution();
                        if (adds) Ld = Ld + c;
                    }
                } else {
                    contribution();
                    sr.n |= 2;
                    sr.dir[1] = ls.direction;
                    sr.maxd[1] = ls.dist - PT_EPS;
                    sr.contrib[1] = c;
                    if (adds) sr.adds |= 2;
                }
            }
        }
    }
    return Ld;
}

// radiance += Ld * T, with the rounding fixed (one fused multiply-add per
// channel) so that the inline and the deferred forms agree to the bit.
__device__ __forceinline__ V3 AddScaled(V3 radiance, V3 Ld, V3 T) {
    return v3(__fmaf_rn(Ld.x, T.x, radiance.x), __fmaf_rn(Ld.y, T.y, radiance.y), __fmaf_rn(Ld.z, T.z, radiance.z));
}

// Ld from the resolved shadow rays of a ShadowReq (env first, then light).
__device__ __forceinline__ V3 ResolveShadow(const ShadowReq& sr, bool occ_env, bool occ_light) {
    V3 Ld = v3(0.0f);
    if ((sr.adds & 1) && !occ_env) Ld = Ld + sr.contrib[0];
    if ((sr.adds & 2) && !occ_light) Ld = Ld + sr.contrib[1];
    return Ld;
}

// Observer of the terms of a path that depend on differentiable parameters
// (the adjoint pass, pt_adjoint.cu).  The forward passes use NoHook, whose
// empty members compile away.
struct NoHook {
    __device__ __forceinline__ void material(const PathState&, float) {}
    __device__ __forceinline__ void emitter(const PathState&, float, const HitRecord&) {}
    __device__ __forceinline__ void vertex(const PathState&) {}
    __device__ __forceinline__ void nee_light(int, float, V3, V3, float, float, V3, V3, V3) {}
    __device__ __forceinline__ void sample(float, V3, V3, V3, V3, const PathState&, const ShadowReq&) {}
    // EvalTransmittance of a VOL_MIS shadow ray, inline; false would suspend
    // the shade step (the replay form, wf_shade)
    __device__ __forceinline__ bool transmit(const Params& P, const Ray& r, Rng& rng, uint2* stack, Counters& cnt,
                                             V3& T) {
        T = EvalTransmittance(P, r, rng, stack, cnt);
        return true;
    }
    // DirectLight's environment sample: true if the hook supplies it (a
    // re-run of a suspended step, whose query follows at once and restores
    // the RNG state it left); env_sampled sees a sample just drawn
    __device__ __forceinline__ bool env_sample(V3&, float&, V3&) { return false; }
    __device__ __forceinline__ void env_sampled(V3, float, V3) {}
    // whether this run of the step reaches the point for the first time (a
    // re-run of a suspended step repeats the part before its last query)
    __device__ __forceinline__ bool first_visit() const { return true; }
};

// One iteration of PathTrace's loop (pathtrace.glsl:301-473) for the hit in
// `hr`.  Returns true if the path continues with ps.r (depth incremented).
// With INLINE false, a pending next-event estimate is left in `sr`
// (sr.n != 0): the caller adds ResolveShadow(...) * sr.T to the radiance
// before anything else touches the path.
template <int MEDIUM, bool ENV, bool INLINE, class Hook>
__device__ __forceinline__ bool ShadeStep(const Params& P, PathState& ps, const HitRecord& hr, ShadowReq& sr,
                                          uint2* stack, Counters& cnt, Hook& hook) {
    const uint32_t F = P.flags;
    sr.n = 0;
    sr.suspended = false;
    if (!hr.hit) {
        if ((F & F_BACKGROUND) && ps.depth == 0) ps.alpha = 0.0f;
        if (!((F & F_HIDE_EMITTERS) && !(ps.depth > 0))) {
            if (F & F_UNIFORM_LIGHT) {
                ps.radiance = ps.radiance + v3(P.uniform_light[0], P.uniform_light[1], P.uniform_light[2]) * ps.throughput;
            } else if (ENV && (F & F_ENVMAP)) {  // (a batch's job may have none)
                float envPdf;
                V3 envCol = EvalEnvMap(P, ps.r, envPdf);
                float misWeight = 1.0f;
                if (ps.depth > 0) misWeight = PowerHeuristic(ps.scatterPdf, envPdf);
                if (MEDIUM == 1 && (F & F_MEDIUM) && !ps.surfaceScatter) misWeight = 1.0f;
                if (misWeight > 0.0f) ps.radiance = ps.radiance + misWeight * envCol * ps.throughput * P.env_intensity;
            }
        }
        return false;
    }
    const V3 fhp = madd_rn(ps.r.origin, ps.r.direction, hr.t);
    V3 normal = v3(0.0f), ffnormal = v3(0.0f);
    Surface sf;
    if (hr.prim >= 0) {
        HitNormal(P, hr, ps.r, normal, ffnormal, &sf);
        ps.matID = hr.mat;
    }
    Material mat;
    float eta;
    hook.material(ps, ps.prevRough);
    GetMaterial(P, ps.matID, ps.depth, ps.prevRough, normal, ffnormal, sf, ps.r, mat, eta);
    ps.prevRough = mat.roughness;
    ps.radiance = ps.radiance + mat.emission * ps.throughput;
    if ((F & F_LIGHTS) && hr.isEmitter) {
        float misWeight = 1.0f;
        if (ps.depth > 0) misWeight = PowerHeuristic(ps.scatterPdf, hr.lightPdf);
        if (MEDIUM == 1 && (F & F_MEDIUM) && !ps.surfaceScatter) misWeight = 1.0f;
        hook.emitter(ps, misWeight, hr);
        ps.radiance = ps.radiance + misWeight * hr.lightEmission * ps.throughput;
        return false;
    }
    if (ps.depth == P.max_depth) return false;
    bool mediumSampled = false;
    V3 scatterL = v3(0.0f);
    // MEDIUM: the scene may have media (OPT_MEDIUM); a batch's job without
    // any (F_MEDIUM clear) takes the MEDIUM == 0 path at run time
    if (MEDIUM && (F & F_MEDIUM)) {
        ps.surfaceScatter = false;
        if (ps.inMedium) {
            if (ps.medium.type == MEDIUM_ABSORB) {
                ps.throughput = ps.throughput * vexp(-(v3(1.0f) - ps.medium.color) * hr.t * ps.medium.density);
            } else if (ps.medium.type == MEDIUM_EMISSIVE) {
                ps.radiance = ps.radiance + ps.medium.color * hr.t * ps.medium.density * ps.throughput;
            } else {
                float scatterDist = fminf(-logf(ps.rng.next()) / ps.medium.density, hr.t);
                mediumSampled = scatterDist < hr.t;
                if (mediumSampled) {
                    ps.throughput = ps.throughput * ps.medium.color;
                    ps.r.origin = madd_rn(ps.r.origin, ps.r.direction, scatterDist);
                    const V3 Ld = DirectLight<MEDIUM, ENV, INLINE>(P, ps.r, ps.r.origin, normal, ffnormal, mat, eta,
                                                                   ps.medium, false, ps.rng, stack, cnt, sr, hook);
                    if (sr.suspended) return false;
                    if (INLINE || sr.n == 0) ps.radiance = AddScaled(ps.radiance, Ld, ps.throughput);
                    else sr.T = ps.throughput;
                    float h1 = ps.rng.next();
                    float h2 = ps.rng.next();
                    V3 scatterDir = SampleHG(-ps.r.direction, ps.medium.anisotropy, h1, h2);
                    ps.scatterPdf = PhaseHG(dot(-ps.r.direction, scatterDir), ps.medium.anisotropy);
                    ps.r.direction = scatterDir;
                }
            }
        }
    }
    if (!mediumSampled) {
        if ((F & F_ALPHA_TEST) && AlphaSkip(mat, ps.rng)) {
            scatterL = ps.r.direction;
            ps.depth--;
        } else {
            ps.surfaceScatter = true;
            hook.vertex(ps);
            const V3 Ld = DirectLight<MEDIUM, ENV, INLINE>(P, ps.r, fhp, normal, ffnormal, mat, eta, ps.medium, true,
                                                           ps.rng, stack, cnt, sr, hook);
            if (sr.suspended) return false;
            if (INLINE || sr.n == 0) ps.radiance = AddScaled(ps.radiance, Ld, ps.throughput);
            else sr.T = ps.throughput;
            const V3 f = DisneySample(mat, eta, -ps.r.direction, ffnormal, scatterL, ps.scatterPdf, ps.rng);
            if (ps.scatterPdf > 0.0f) {
                hook.sample(eta, -ps.r.direction, ffnormal, scatterL, f, ps, sr);
                ps.throughput = ps.throughput * (f / ps.scatterPdf);
            } else {
                return false;
            }
        }
        ps.r.direction = scatterL;
        ps.r.origin = madd_rn(fhp, ps.r.direction, PT_EPS);
        if (MEDIUM) {
            if (dot(ps.r.direction, normal) < 0.0f && mat.medium.type != MEDIUM_NONE) {
                ps.inMedium = true;
                ps.medium = mat.medium;
            } else if (mat.medium.type != MEDIUM_NONE) ps.inMedium = false;
        }
    }
    if ((F & F_RR) && ps.depth >= P.rr_depth) {
        float q = fminf(maxc(ps.throughput) + 0.001f, 0.95f);
        if (ps.rng.next() > q) return false;
        ps.throughput = ps.throughput / q;
    }
    ps.depth++;
    return true;
}

// tile.glsl:41-74 for pixel (px, py); the RNG is seeded with the
// tile-local fragment position, as the tile viewport gives gl_FragCoord.
__device__ __forceinline__ Ray CameraRay(const Params& P, int px, int py, int tx, int ty, Rng& rng) {
    const int lx = px - tx * P.tile_w, ly = py - ty * P.tile_h;
    const float invx = (float)P.tile_w / (float)P.width, invy = (float)P.tile_h / (float)P.height;
    const float tcx = ((float)lx + 0.5f) / (float)P.tile_w, tcy = ((float)ly + 0.5f) / (float)P.tile_h;
    const float offx = (float)tx * invx, offy = (float)ty * invy;
    const float cx = offx * (1.0f - tcx) + (offx + invx) * tcx;
    const float cy = offy * (1.0f - tcy) + (offy + invy) * tcy;
    float r1 = 2.0f * rng.next();
    float r2 = 2.0f * rng.next();
    float jx = r1 < 1.0f ? sqrtf(r1) - 1.0f : 1.0f - sqrtf(2.0f - r1);
    float jy = r2 < 1.0f ? sqrtf(r2) - 1.0f : 1.0f - sqrtf(2.0f - r2);
    const float resx = (float)P.width, resy = (float)P.height;
    jx = jx / (resx * 0.5f);
    jy = jy / (resy * 0.5f);
    float dx = (cx * 2.0f - 1.0f) + jx;
    float dy = (cy * 2.0f - 1.0f) + jy;
    const float scale = tanf(P.cam_fov * 0.5f);
    dy *= resy / resx * scale;
    dx *= scale;
    const V3 right = v3(P.cam_right[0], P.cam_right[1], P.cam_right[2]);
    const V3 up = v3(P.cam_up[0], P.cam_up[1], P.cam_up[2]);
    const V3 fwd = v3(P.cam_fwd[0], P.cam_fwd[1], P.cam_fwd[2]);
    const V3 pos = v3(P.cam_pos[0], P.cam_pos[1], P.cam_pos[2]);
    const V3 rayDir = normalize(dx * right + dy * up + fwd);
    const V3 focalPoint = P.cam_focal * rayDir;
    const float cam_r1 = rng.next() * PT_TWO_PI;
    const float cam_r2 = rng.next() * P.cam_aperture;
    float s, c;
    sincosf(cam_r1, &s, &c);
    const V3 aperturePos = (c * right + s * up) * sqrtf(cam_r2);
    const V3 finalDir = normalize(focalPoint - aperturePos);
    return Ray{pos + aperturePos, finalDir};
}

// The start of a path: tile.glsl's seed and camera ray, PathTrace's initial
// state (pathtrace.glsl:287-299).
__device__ __forceinline__ void StartPath(const Params& P, int px, int py, uint32_t frame, PathState& ps) {
    const int tx = px / P.tile_w, ty = py / P.tile_h;
    ps.rng.init((uint32_t)(px - tx * P.tile_w), (uint32_t)(py - ty * P.tile_h), frame);
    ps.r = CameraRay(P, px, py, tx, ty, ps.rng);
    ps.throughput = v3(1.0f);
    ps.radiance = v3(0.0f);
    ps.alpha = 1.0f;
    ps.depth = 0;
    ps.matID = 0;
    ps.prevRough = 0.0f;
    ps.scatterPdf = 0.0f;
    ps.inMedium = false;
    ps.surfaceScatter = false;
    ps.medium.type = 0;
    ps.medium.density = 0.0f;
    ps.medium.color = v3(0.0f);
    ps.medium.anisotropy = 0.0f;
}

// Frame number of pass `pass` for the tile containing (px, py), as the
// reference's tile state machine assigns them (Renderer.cpp:745-783).
__device__ __forceinline__ uint32_t FrameNumber(const Params& P, const RenderWork& W, int pass, int px, int py) {
    if (W.tile_frame >= 0) return (uint32_t)W.tile_frame;
    const int tx = px / P.tile_w, ty = py / P.tile_h;
    return (uint32_t)(2 + pass * P.ntx * P.nty + (P.nty - 1 - ty) * P.ntx + tx);
}

// A path ended at PT_MAX_PATH_ITERATIONS (pt_cuda.h).
__device__ __forceinline__ void count_truncated(const Params& P) { atomicAdd(P.counters + 3, 1ull); }

__device__ __forceinline__ void add_counters(const Params& P, uint32_t closest, uint32_t shadow, uint32_t paths) {
    const unsigned mask = __activemask();
    closest = __reduce_add_sync(mask, closest);
    shadow = __reduce_add_sync(mask, shadow);
    paths = __reduce_add_sync(mask, paths);
    if ((threadIdx.x & 31) == __ffs(mask) - 1) {
        if (closest) atomicAdd(P.counters + 0, (unsigned long long)closest);
        if (shadow) atomicAdd(P.counters + 1, (unsigned long long)shadow);
        if (paths) atomicAdd(P.counters + 2, (unsigned long long)paths);
    }
}

// Shadow queries answered without traversal because their contribution is
// never added (DirectLight, wf_shade, wf_shadow); they are counted among the
// shadow queries as well.
__device__ __forceinline__ void add_untraced(const Params& P, uint32_t n) {
    const unsigned mask = __activemask();
    n = __reduce_add_sync(mask, n);
    if ((threadIdx.x & 31) == __ffs(mask) - 1 && n) atomicAdd(P.counters + 4, (unsigned long long)n);
}

}  // namespace ptgb
