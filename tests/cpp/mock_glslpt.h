// mock_glslpt.h - stand-ins for the reference's scene types, for the
// drop-in test driver only (test infrastructure).
//
// ptgb::CudaRenderer binds GLSLPT::Scene by member name and layout
// (cuda_renderer.h, RefSceneLink).  The reference's headers are not part of
// this repository, so the test declares types with the same member names
// and layouts as src/core/Scene.h:50-125, src/core/Renderer.h:37-100,
// src/core/Camera.h:41-50, src/core/EnvironmentMap.h:33-47,
// src/math/{Vec2,Vec3,Vec4,Mat4}.h and
// thirdparty/RadeonRays/bvh_translator.h:45-57, holding only data.
#pragma once

#include <vector>

namespace GLSLPT {

struct Vec3 { float x, y, z; };
struct Vec4 { float x, y, z, w; };
struct iVec2 { int x, y; };
struct Mat4 { float data[4][4]; };
struct Indices { int x, y, z; };
struct Material { float packed[32]; };  // 8 x vec4 of Material.h:47-119
struct Light {
    Vec3 position, emission, u, v;
    float radius, area, type;
};
struct EnvironmentMap {
    int width = 0, height = 0;
    float totalSum = 0.0f;
    float* img = nullptr;
    float* cdf = nullptr;
};
struct Camera {
    Vec3 position, up, right, forward;
    float focalDist, aperture, fov;
    bool isMoving = false;
};
struct Texture {};
struct RenderOptions {
    iVec2 renderResolution{1280, 720}, windowResolution{1280, 720};
    Vec3 uniformLightCol{0.3f, 0.3f, 0.3f}, backgroundCol{1.0f, 1.0f, 1.0f};
    int tileWidth = 100, tileHeight = 100, maxDepth = 2, maxSpp = -1, RRDepth = 2;
    int texArrayWidth = 2048, texArrayHeight = 2048, denoiserFrameCnt = 20;
    bool enableRR = true, enableDenoiser = false, enableTonemap = true, enableAces = false, simpleAcesFit = false;
    bool openglNormalMap = true, enableEnvMap = false, enableUniformLight = false, hideEmitters = false;
    bool enableBackground = false, transparentBackground = false, independentRenderSize = false;
    bool enableRoughnessMollification = false, enableVolumeMIS = false;
    float envMapIntensity = 1.0f, envMapRot = 0.0f, roughnessMollificationAmt = 0.0f;
};
struct BvhNode { Vec3 bboxmin, bboxmax, LRLeaf; };
struct BvhTranslator {
    int topLevelIndex = 0;
    std::vector<BvhNode> nodes;
};

class Scene {
public:
    void ProcessScene() { initialized = true; }  // the arrays below are already flattened

    RenderOptions renderOptions;
    std::vector<Indices> vertIndices;
    std::vector<Vec4> verticesUVX, normalsUVY;
    std::vector<Mat4> transforms;
    std::vector<Material> materials;
    std::vector<Light> lights;
    EnvironmentMap* envMap = nullptr;
    Camera* camera = nullptr;
    BvhTranslator bvhTranslator;
    std::vector<Texture*> textures;
    std::vector<unsigned char> textureMapsArray;
    bool initialized = false;
    bool dirty = true;
    bool instancesModified = false;
    bool envMapModified = false;
};

}  // namespace GLSLPT
