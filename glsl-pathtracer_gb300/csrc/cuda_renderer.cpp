// cuda_renderer.cpp - GLSLPT::Renderer's state machine over the C ABI.
#include "cuda_renderer.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace ptgb {

void CudaRenderer::Check(int rc) const {
    if (rc != PT_OK) {
        char buf[512];
        pt_last_error(buf, sizeof buf);
        throw CudaRendererError(rc, buf);
    }
}

// Renderer::InitFBOs tile bookkeeping (Renderer.cpp:281-300)
void CudaRenderer::InitTiles() {
    const pt_render_options& o = scene->renderOptions;
    numTilesX = (int)std::ceil((float)o.render_width / o.tile_width);
    numTilesY = (int)std::ceil((float)o.render_height / o.tile_height);
    tileX = -1;
    tileY = numTilesY - 1;
    sampleCounter = 1;
    currentBuffer = 0;
    frameCounter = 1;
    haveSnapshot = false;
}

// Renderer::Renderer (Renderer.cpp:41-87): the scene arrays go to the device.
// Render() runs the wavefront integrator unless SetIntegrator says otherwise.
CudaRenderer::CudaRenderer(CudaScene* s, const std::string&) : scene(s) {
    if (!scene) throw CudaRendererError(PT_ERR_INVALID_ARG, "No Scene Found");
    Check(pt_create(&scene->desc, &scene->renderOptions, &ctx));
    Check(pt_set_camera(ctx, &scene->camera));
    Check(pt_set_integrator(ctx, PT_INTEGRATOR_WAVEFRONT));
    InitTiles();
}

// The same for a linked scene object (the reference's GLSLPT::Scene).
CudaRenderer::CudaRenderer(SceneLink* l, const std::string&) : link(l), scene(&linked) {
    if (!link) throw CudaRendererError(PT_ERR_INVALID_ARG, "No Scene Found");
    link->Pull(linked);
    Check(pt_create(&scene->desc, &scene->renderOptions, &ctx));
    Check(pt_set_camera(ctx, &scene->camera));
    Check(pt_set_integrator(ctx, PT_INTEGRATOR_WAVEFRONT));
    InitTiles();
}

CudaRenderer::~CudaRenderer() { pt_destroy(ctx); }

void CudaRenderer::Pull() {
    if (link) link->Pull(linked);
}

void CudaRenderer::Push() {
    if (link) link->Push(linked);
}

void CudaRenderer::SetIntegrator(int integrator) { Check(pt_set_integrator(ctx, integrator)); }

void CudaRenderer::Autotune(int passes) {
    pt_tuning t;
    Check(pt_autotune(ctx, passes, &t));
}

// Renderer::ResizeRenderer (Renderer.cpp:252-279)
void CudaRenderer::ResizeRenderer() {
    Pull();
    Check(pt_set_options(ctx, &scene->renderOptions));
    Check(pt_clear_accum(ctx));
    InitTiles();
}

// Renderer::ReloadShaders (Renderer.cpp:380-390): the feature set follows
// the options on the next launch.
void CudaRenderer::ReloadShaders() {
    Pull();
    Check(pt_set_options(ctx, &scene->renderOptions));
}

// Renderer::Render (Renderer.cpp:546-590)
void CudaRenderer::Render() {
    Pull();
    const pt_render_options& o = scene->renderOptions;
    if (!scene->dirty && o.max_spp != -1 && sampleCounter >= o.max_spp) return;
    if (scene->dirty) {
        // the reference draws a low-resolution preview here (interactive only)
        scene->instancesModified = false;
        scene->dirty = false;
        scene->envMapModified = false;
        Push();
        return;
    }
    Check(pt_render_tile(ctx, tileX, tileY, frameCounter));
}

// Whole passes in one launch.  Called where Render() would draw the first
// tile of a sample pass (after the Update that moved there), it renders
// passes k .. k+n-1 (k = the passes completed so far) with the frame numbers
// of the tile loop (pt_render_passes) and leaves the state machine where the
// tile loop would be after drawing the last tile of pass k+n-1: the next
// Update completes those passes (snapshot, sample counter) as usual.
void CudaRenderer::RenderPasses(int n) {
    Pull();
    if (n <= 0) return;
    if (scene->dirty) throw CudaRendererError(PT_ERR_INVALID_ARG, "RenderPasses: the scene is dirty (call Update)");
    if (!AtPassStart()) throw CudaRendererError(PT_ERR_INVALID_ARG, "RenderPasses: not at the first tile of a pass");
    const pt_render_options& o = scene->renderOptions;
    const int k = sampleCounter - 1;
    // the tile loop stops once the sample counter reaches max_spp, which
    // leaves max_spp - 1 passes (Renderer.cpp:550,645)
    if (o.max_spp != -1) n = std::min(n, o.max_spp - 1 - k);
    if (n <= 0) return;
    Check(pt_render_passes(ctx, k, n));
    const int tiles = numTilesX * numTilesY;
    frameCounter = 1 + (k + n) * tiles;
    sampleCounter = k + n;
    tileX = numTilesX - 1;
    tileY = 0;
}

void CudaRenderer::Present() {}

float CudaRenderer::GetProgress() {
    const int maxSpp = scene->renderOptions.max_spp;
    return maxSpp <= 0 ? 0.0f : sampleCounter * 100.0f / maxSpp;
}

int CudaRenderer::GetSampleCount() { return sampleCounter; }

// Renderer::GetOutputBuffer (Renderer.cpp:619-634): the caller delete[]s.
// Shows the last completed sample pass, tonemapped, rows bottom-up.
void CudaRenderer::GetOutputBuffer(unsigned char** data, int& w, int& h) {
    w = scene->renderOptions.render_width;
    h = scene->renderOptions.render_height;
    *data = new unsigned char[(size_t)w * h * 4];
    if (!haveSnapshot) {
        std::memset(*data, 0, (size_t)w * h * 4);
        return;
    }
    Check(pt_get_output(ctx, sampleCounter - 1, 1, *data));
}

// Renderer::Update (Renderer.cpp:641-811)
void CudaRenderer::Update(float) {
    Pull();
    const pt_render_options& o = scene->renderOptions;
    if (!scene->dirty && o.max_spp != -1 && sampleCounter >= o.max_spp) return;
    if (scene->instancesModified) {
        const pt_scene_desc& d = scene->desc;
        Check(pt_update_instances(ctx, d.transforms, d.num_instances, d.materials, d.num_materials,
                                  d.bvh_nodes + 9 * (size_t)d.top_level_index,
                                  d.num_bvh_nodes - d.top_level_index));
    }
    if (scene->envMapModified) {
        const pt_scene_desc& d = scene->desc;
        Check(pt_update_envmap(ctx, d.envmap_rgb, d.envmap_cdf, d.envmap_width, d.envmap_height,
                               d.envmap_total_sum));
    }
    Check(pt_set_options(ctx, &scene->renderOptions));
    if (scene->dirty) {
        tileX = -1;
        tileY = numTilesY - 1;
        sampleCounter = 1;
        frameCounter = 1;
        haveSnapshot = false;
        Check(pt_clear_accum(ctx));
    } else {
        frameCounter++;
        tileX++;
        if (tileX >= numTilesX) {
            tileX = 0;
            tileY--;
            if (tileY < 0) {
                tileX = 0;
                tileY = numTilesY - 1;
                sampleCounter++;
                currentBuffer = 1 - currentBuffer;
                Check(pt_snapshot_accum(ctx));  // the completed pass becomes the displayed image
                haveSnapshot = true;
            }
        }
    }
    Check(pt_set_camera(ctx, &scene->camera));
    Push();
}

}  // namespace ptgb
