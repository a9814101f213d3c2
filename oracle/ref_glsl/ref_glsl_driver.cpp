// ref_glsl_driver.cpp - runs the reference's own shader source on the CPU.
//
// TEST INFRASTRUCTURE ONLY (oracle/_ref recipe, this container only).  The
// rewritten shader files (glsl2cpp.py) are included into namespace glsl on
// top of glsl_shim.hpp; this file plays the role of the GL driver: it binds
// the scene arrays as the samplers Renderer::InitGPUDataBuffers creates
// (src/core/Renderer.cpp:135-249), sets the uniforms Renderer::Update sets
// (Renderer.cpp:764-811), and invokes tile.glsl's main once per fragment of
// each tile in the order Renderer::Update walks the tiles (Renderer.cpp:745-762).
// The OPT_* feature macros are given on the compiler command line, as
// Renderer::InitShaders injects them (Renderer.cpp:400-476).
#include <omp.h>

#include <string>

#include "../../include/pt_cuda.h"
#include "glsl_shim.hpp"

namespace glsl {
thread_local vec4 gl_FragCoord;
thread_local vec2 TexCoords;
thread_local vec4 color;
#include "uniforms.inc"
#include "globals.inc"
#include "intersection.inc"
#include "sampling.inc"
#include "envmap.inc"
#include "anyhit.inc"
#include "closest_hit.inc"
#include "disney.inc"
#include "lambert.inc"
#include "pathtrace.inc"
#include "tile.inc"
}  // namespace glsl

using namespace glsl;

namespace {
void bind_scene(const pt_scene_desc* d, const pt_render_options* o, const pt_camera* cam) {
    BVH.data = d->bvh_nodes; BVH.comps = 3;
    vertexIndicesTex.data = d->vert_indices; vertexIndicesTex.comps = 3;
    verticesTex.data = d->vertices_uvx; verticesTex.comps = 4;
    normalsTex.data = d->normals_uvy; normalsTex.comps = 4;
    materialsTex.data = d->materials; materialsTex.w = 8 * d->num_materials; materialsTex.h = 1; materialsTex.comps = 4;
    transformsTex.data = d->transforms; transformsTex.w = 4 * d->num_instances; transformsTex.h = 1; transformsTex.comps = 4;
    lightsTex.data = d->num_lights ? d->lights : nullptr; lightsTex.w = 5 * d->num_lights; lightsTex.h = 1; lightsTex.comps = 3;
    textureMapsArrayTex.data = d->num_textures ? d->texture_maps : nullptr;
    textureMapsArrayTex.w = d->tex_width; textureMapsArrayTex.h = d->tex_height; textureMapsArrayTex.layers = d->num_textures;
    envMapTex.data = d->envmap_rgb; envMapTex.w = d->envmap_width; envMapTex.h = d->envmap_height; envMapTex.comps = 3;
    envMapCDFTex.data = d->envmap_cdf; envMapCDFTex.w = d->envmap_width; envMapCDFTex.h = d->envmap_height; envMapCDFTex.comps = 1;
    accumTexture.data = nullptr;  // the driver adds the tile result to the accumulation itself
    envMapRes = vec2(float(d->envmap_width), float(d->envmap_height));
    envMapTotalSum = d->envmap_total_sum;
    topBVHIndex = d->top_level_index;
    numOfLights = d->num_lights;
    if (o) {
        resolution = vec2(float(o->render_width), float(o->render_height));
        invNumTiles = vec2((float)o->tile_width / o->render_width, (float)o->tile_height / o->render_height);
        envMapIntensity = o->envmap_intensity;
        envMapRot = o->envmap_rot / 360.0f;
        maxDepth = o->max_depth;
        uniformLightCol = vec3(o->uniform_light_col[0], o->uniform_light_col[1], o->uniform_light_col[2]);
        roughnessMollificationAmt = o->roughness_mollification_amt;
    }
    if (cam) {
        camera.position = vec3(cam->position[0], cam->position[1], cam->position[2]);
        camera.right = vec3(cam->right[0], cam->right[1], cam->right[2]);
        camera.up = vec3(cam->up[0], cam->up[1], cam->up[2]);
        camera.forward = vec3(cam->forward[0], cam->forward[1], cam->forward[2]);
        camera.fov = cam->fov;
        camera.focalDist = cam->focal_dist;
        camera.aperture = cam->aperture;
    }
}
}  // namespace

extern "C" {

// Feature macros this build was compiled with (space separated).
const char* ref_glsl_variant() {
    static std::string s = std::string("")
#ifdef OPT_ENVMAP
        + "OPT_ENVMAP "
#endif
#ifdef OPT_LIGHTS
        + "OPT_LIGHTS "
#endif
#ifdef OPT_RR
        + "OPT_RR "
#endif
#ifdef OPT_UNIFORM_LIGHT
        + "OPT_UNIFORM_LIGHT "
#endif
#ifdef OPT_OPENGL_NORMALMAP
        + "OPT_OPENGL_NORMALMAP "
#endif
#ifdef OPT_HIDE_EMITTERS
        + "OPT_HIDE_EMITTERS "
#endif
#ifdef OPT_BACKGROUND
        + "OPT_BACKGROUND "
#endif
#ifdef OPT_TRANSPARENT_BACKGROUND
        + "OPT_TRANSPARENT_BACKGROUND "
#endif
#ifdef OPT_ALPHA_TEST
        + "OPT_ALPHA_TEST "
#endif
#ifdef OPT_ROUGHNESS_MOLLIFICATION
        + "OPT_ROUGHNESS_MOLLIFICATION "
#endif
#ifdef OPT_MEDIUM
        + "OPT_MEDIUM "
#endif
#ifdef OPT_VOL_MIS
        + "OPT_VOL_MIS "
#endif
        ;
    return s.c_str();
}

// Sample passes [first_pass, first_pass+num_passes) of the tile state
// machine, ADDED into accum (W*H*4 floats, bottom row first).
int ref_glsl_render(const pt_scene_desc* d, const pt_render_options* o, const pt_camera* cam, int first_pass,
                    int num_passes, int nthreads, float* accum) {
    bind_scene(d, o, cam);
    if (nthreads > 0) omp_set_num_threads(nthreads);
    const int W = o->render_width, H = o->render_height, tw = o->tile_width, th = o->tile_height;
    const int nx = (W + tw - 1) / tw, ny = (H + th - 1) / th;
    int frame = 2 + first_pass * nx * ny;  // Renderer.cpp:745-783: first rendered tile has frameNum 2
    for (int pass = first_pass; pass < first_pass + num_passes; ++pass) {
        for (int ty = ny - 1; ty >= 0; --ty) {
            for (int tx = 0; tx < nx; ++tx, ++frame) {
                tileOffset = vec2((float)tx * invNumTiles.x, (float)ty * invNumTiles.y);
                frameNum = frame;
#pragma omp parallel for schedule(dynamic, 1)
                for (int ly = 0; ly < th; ++ly) {
                    const int py = ty * th + ly;
                    if (py >= H) continue;
                    for (int lx = 0; lx < tw; ++lx) {
                        const int px = tx * tw + lx;
                        if (px >= W) continue;
                        gl_FragCoord = vec4(float(lx) + 0.5f, float(ly) + 0.5f, 0.0f, 1.0f);
                        TexCoords = vec2((float(lx) + 0.5f) / float(tw), (float(ly) + 0.5f) / float(th));
                        tile_main();
                        float* a = accum + 4 * ((size_t)py * W + px);
                        a[0] += color.x; a[1] += color.y; a[2] += color.z; a[3] += color.w;
                    }
                }
            }
        }
    }
    return 0;
}

// The reference's ClosestHit (closest_hit.glsl:25) on a ray set, with
// State.depth = 1 so that emitters are intersected.  Outputs per ray:
// hit flag, t (State.hitDist), matID, isEmitter, and the shading normal.
int ref_glsl_closest_hit(const pt_scene_desc* d, const pt_ray* rays, int n, int* hit, float* t, int* matID,
                         int* isEmitter, float* normal) {
    bind_scene(d, nullptr, nullptr);
    for (int i = 0; i < n; ++i) {
        Ray r;
        r.origin = vec3(rays[i].origin[0], rays[i].origin[1], rays[i].origin[2]);
        r.direction = vec3(rays[i].direction[0], rays[i].direction[1], rays[i].direction[2]);
        State state;
        state.depth = 1;
        state.matID = -1;
        state.isEmitter = false;
        LightSampleRec ls;
        bool h = ClosestHit(r, state, ls);
        hit[i] = h ? 1 : 0;
        t[i] = h ? state.hitDist : 1000000.0f;
        matID[i] = h ? state.matID : -1;
        isEmitter[i] = h && state.isEmitter ? 1 : 0;
        normal[3 * i] = state.normal.x; normal[3 * i + 1] = state.normal.y; normal[3 * i + 2] = state.normal.z;
    }
    return 0;
}

// The reference's DisneyEval (disney.glsl:244) for n shading states; the
// 20-float state layout is the one of orc_bsdf_eval.
int ref_glsl_disney_eval(int n, const float* sp, const float* V, const float* N, const float* L, float* f, float* pdf) {
    for (int i = 0; i < n; ++i) {
        const float* p = sp + 20 * (size_t)i;
        State st;
        st.mat.baseColor = vec3(p[0], p[1], p[2]);
        st.mat.metallic = p[3]; st.mat.roughness = p[4]; st.mat.subsurface = p[5]; st.mat.specularTint = p[6];
        st.mat.sheen = p[7]; st.mat.sheenTint = p[8]; st.mat.clearcoat = p[9]; st.mat.clearcoatRoughness = p[10];
        st.mat.specTrans = p[11]; st.mat.ior = p[12]; st.mat.ax = p[13]; st.mat.ay = p[14];
        st.eta = p[15]; st.mat.anisotropic = p[16];
        float pd = 0.0f;
        vec3 r = DisneyEval(st, vec3(V[3 * i], V[3 * i + 1], V[3 * i + 2]), vec3(N[3 * i], N[3 * i + 1], N[3 * i + 2]),
                            vec3(L[3 * i], L[3 * i + 1], L[3 * i + 2]), pd);
        f[3 * i] = r.x; f[3 * i + 1] = r.y; f[3 * i + 2] = r.z;
        pdf[i] = pd;
    }
    return 0;
}

}  // extern "C"
