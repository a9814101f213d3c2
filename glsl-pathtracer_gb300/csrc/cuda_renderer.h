// cuda_renderer.h - C++ drop-in for GLSLPT::Renderer (src/core/Renderer.h:104-185).
//
// Same public surface and the same tile/sample state machine
// (Renderer.cpp:546-811), running on libptgb's C ABI instead of OpenGL.
// Where the reference takes a GLSLPT::Scene*, this takes a CudaScene*: the
// handful of Scene members the Renderer reads (its flattened arrays as a
// pt_scene_desc, renderOptions, the camera, and the dirty /
// instancesModified / envMapModified flags).  The scene is borrowed; the
// caller keeps ownership, as with the reference (Main.cpp:123,159).
// Errors throw CudaRendererError (the reference printf's and carries on).
#pragma once

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

class CudaRenderer {
public:
    CudaRenderer(CudaScene* scene, const std::string& shadersDirectory = "");
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

private:
    void Check(int rc) const;
    void InitTiles();

    CudaScene* scene;
    pt_context* ctx = nullptr;
    int tileX = -1, tileY = 0, numTilesX = 1, numTilesY = 1;
    int frameCounter = 1;
    int sampleCounter = 1;
    int currentBuffer = 0;
    bool haveSnapshot = false;
};

}  // namespace ptgb
