// cuda_renderer.h - C++ drop-in for GLSLPT::Renderer (src/core/Renderer.h:104-185).
//
// Same public surface and the same tile/sample state machine
// (Renderer.cpp:546-811), running on libptgb's C ABI instead of OpenGL.
// It takes the reference's own GLSLPT::Scene* (any type with the members
// Renderer reads, bound by RefSceneLink below: the flattened arrays,
// renderOptions, the camera, the environment map, the texture array and the
// dirty / instancesModified / envMapModified flags), so
//     Renderer* r = new Renderer(scene, shadersDir);        (Main.cpp:157-161)
// becomes
//     ptgb::CudaRenderer* r = new ptgb::CudaRenderer(scene, shadersDir);
// or a CudaScene*, a plain record of the same data.  The scene is borrowed;
// the caller keeps ownership, as with the reference (Main.cpp:123,159).
// Errors throw CudaRendererError (the reference printf's and carries on).
#pragma once

#include <memory>
#include <stdexcept>
#include <string>

#include "../../include/pt_cuda.h"

namespace ptgb {

struct CudaScene {
    pt_scene_desc desc{};
    pt_render_options renderOptions{};
    pt_camera camera{};
    bool dirty = true;               // Scene::dirty (Scene.h:45,122)
    bool instancesModified = false;  // Scene::instancesModified
    bool envMapModified = false;     // Scene::envMapModified
};

struct CudaRendererError : std::runtime_error {
    int code;
    CudaRendererError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// A caller's scene object kept in step with a CudaScene: Pull copies its
// arrays, options, camera and flags in before the renderer reads them, Push
// hands back the flags the renderer cleared.
struct SceneLink {
    virtual ~SceneLink() = default;
    virtual void Pull(CudaScene& s) = 0;
    virtual void Push(const CudaScene& s) = 0;
};

// The binding of GLSLPT::Scene (src/core/Scene.h:66-125): member names and
// layouts as the reference declares them -- bvhTranslator.nodes (36-byte
// Node, bvh_translator.h:45-50) and topLevelIndex, vertIndices (Indices),
// verticesUVX / normalsUVY (Vec4), transforms (Mat4, float data[4][4]),
// materials (128-byte Material), lights (60-byte Light), envMap
// (EnvironmentMap: width, height, totalSum, img, cdf), camera (Camera:
// position, up, right, forward, fov, focalDist, aperture), textures and
// textureMapsArray, renderOptions (Renderer.h:37-100) and the three flags.
// Nothing is copied: the descriptor points into the scene's vectors.
template <class SceneT> class RefSceneLink : public SceneLink {
public:
    explicit RefSceneLink(SceneT* scene) : sc(scene) {}
    void Pull(CudaScene& s) override {
        static_assert(sizeof(sc->bvhTranslator.nodes[0]) == 9 * sizeof(float), "BvhTranslator::Node layout");
        static_assert(sizeof(sc->vertIndices[0]) == 3 * sizeof(int32_t), "Indices layout");
        static_assert(sizeof(sc->verticesUVX[0]) == 4 * sizeof(float), "Vec4 layout");
        static_assert(sizeof(sc->transforms[0]) == 16 * sizeof(float), "Mat4 layout");
        static_assert(sizeof(sc->materials[0]) == 32 * sizeof(float), "Material layout");
        static_assert(sizeof(sc->lights[0]) == 15 * sizeof(float), "Light layout");
        if (!sc->initialized) sc->ProcessScene();  // Renderer.cpp:78-79
        pt_scene_desc& d = s.desc;
        d = pt_scene_desc{};
        d.bvh_nodes = reinterpret_cast<const float*>(sc->bvhTranslator.nodes.data());
        d.num_bvh_nodes = (int32_t)sc->bvhTranslator.nodes.size();
        d.top_level_index = sc->bvhTranslator.topLevelIndex;
        d.vert_indices = reinterpret_cast<const int32_t*>(sc->vertIndices.data());
        d.num_tris = (int32_t)sc->vertIndices.size();
        d.vertices_uvx = reinterpret_cast<const float*>(sc->verticesUVX.data());
        d.normals_uvy = reinterpret_cast<const float*>(sc->normalsUVY.data());
        d.num_vertices = (int32_t)sc->verticesUVX.size();
        d.transforms = reinterpret_cast<const float*>(sc->transforms.data());
        d.num_instances = (int32_t)sc->transforms.size();
        d.materials = reinterpret_cast<const float*>(sc->materials.data());
        d.num_materials = (int32_t)sc->materials.size();
        d.lights = sc->lights.empty() ? nullptr : reinterpret_cast<const float*>(sc->lights.data());
        d.num_lights = (int32_t)sc->lights.size();
        if (sc->envMap) {
            d.envmap_rgb = sc->envMap->img;
            d.envmap_cdf = sc->envMap->cdf;
            d.envmap_width = sc->envMap->width;
            d.envmap_height = sc->envMap->height;
            d.envmap_total_sum = sc->envMap->totalSum;
        }
        const auto& ro = sc->renderOptions;
        if (!sc->textures.empty()) {
            d.texture_maps = sc->textureMapsArray.data();
            d.tex_width = ro.texArrayWidth;
            d.tex_height = ro.texArrayHeight;
            d.num_textures = (int32_t)sc->textures.size();
        }
        pt_render_options& o = s.renderOptions;
        o.render_width = ro.renderResolution.x;
        o.render_height = ro.renderResolution.y;
        o.tile_width = ro.tileWidth;
        o.tile_height = ro.tileHeight;
        o.max_depth = ro.maxDepth;
        o.max_spp = ro.maxSpp;
        o.rr_depth = ro.RRDepth;
        o.enable_rr = ro.enableRR;
        o.enable_envmap = ro.enableEnvMap;
        o.enable_uniform_light = ro.enableUniformLight;
        o.hide_emitters = ro.hideEmitters;
        o.enable_background = ro.enableBackground;
        o.transparent_background = ro.transparentBackground;
        o.enable_roughness_mollification = ro.enableRoughnessMollification;
        o.enable_volume_mis = ro.enableVolumeMIS;
        o.opengl_normal_map = ro.openglNormalMap;
        o.enable_tonemap = ro.enableTonemap;
        o.enable_aces = ro.enableAces;
        o.simple_aces_fit = ro.simpleAcesFit;
        o.uniform_light_col[0] = ro.uniformLightCol.x;
        o.uniform_light_col[1] = ro.uniformLightCol.y;
        o.uniform_light_col[2] = ro.uniformLightCol.z;
        o.background_col[0] = ro.backgroundCol.x;
        o.background_col[1] = ro.backgroundCol.y;
        o.background_col[2] = ro.backgroundCol.z;
        o.envmap_intensity = ro.envMapIntensity;
        o.envmap_rot = ro.envMapRot;
        o.roughness_mollification_amt = ro.roughnessMollificationAmt;
        if (sc->camera) {
            pt_camera& c = s.camera;
            const auto* cam = sc->camera;
            float* out[4] = {c.position, c.up, c.right, c.forward};
            const decltype(cam->position)* vec[4] = {&cam->position, &cam->up, &cam->right, &cam->forward};
            for (int k = 0; k < 4; ++k) {
                out[k][0] = vec[k]->x;
                out[k][1] = vec[k]->y;
                out[k][2] = vec[k]->z;
            }
            c.fov = cam->fov;
            c.focal_dist = cam->focalDist;
            c.aperture = cam->aperture;
        }
        s.dirty = sc->dirty;
        s.instancesModified = sc->instancesModified;
        s.envMapModified = sc->envMapModified;
    }
    void Push(const CudaScene& s) override {
        sc->dirty = s.dirty;
        sc->instancesModified = s.instancesModified;
        sc->envMapModified = s.envMapModified;
    }

private:
    SceneT* sc;
};

class CudaRenderer {
public:
    CudaRenderer(CudaScene* scene, const std::string& shadersDirectory = "");
    // The reference's own scene type (GLSLPT::Scene), bound by RefSceneLink.
    template <class SceneT>
    explicit CudaRenderer(SceneT* scene, const std::string& shadersDirectory = "")
        : CudaRenderer(scene ? static_cast<SceneLink*>(new RefSceneLink<SceneT>(scene)) : nullptr,
                       shadersDirectory) {}
    ~CudaRenderer();
    CudaRenderer(const CudaRenderer&) = delete;
    CudaRenderer& operator=(const CudaRenderer&) = delete;

    void ResizeRenderer();
    void ReloadShaders();
    void Render();
    void Present();
    void Update(float secondsElapsed);
    float GetProgress();
    int GetSampleCount();
    void GetOutputBuffer(unsigned char** data, int& w, int& h);

    pt_context* context() const { return ctx; }

    // Extensions (no counterpart in the reference).
    // The kernels that Render() runs: PT_INTEGRATOR_WAVEFRONT (the default)
    // or PT_INTEGRATOR_MEGAKERNEL.
    void SetIntegrator(int integrator);
    // At the start of a sample pass (after the Update that moved there),
    // renders n whole passes in one launch -- the samples that
    // n x (tiles per pass) Update/Render cycles give -- and leaves the state
    // machine as those cycles would before the Update that completes them.
    void RenderPasses(int n);
    // The wavefront's launch configuration tuned on trial frames of
    // `passes` whole passes (pt_autotune); the accumulation is untouched.
    void Autotune(int passes);
    // True where Render() would draw the first tile of a sample pass.
    bool AtPassStart() const { return tileX == 0 && tileY == numTilesY - 1; }

private:
    CudaRenderer(SceneLink* link, const std::string& shadersDirectory);
    void Check(int rc) const;
    void InitTiles();
    void Pull();
    void Push();

    std::unique_ptr<SceneLink> link;
    CudaScene linked;  // the linked scene's data, when there is a link
    CudaScene* scene;
    pt_context* ctx = nullptr;
    int tileX = -1, tileY = 0, numTilesX = 1, numTilesY = 1;
    int frameCounter = 1;
    int sampleCounter = 1;
    int currentBuffer = 0;
    bool haveSnapshot = false;
};

}  // namespace ptgb
