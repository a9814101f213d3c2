// ref_scene_dump.cpp - loads a scene with the reference's own host code and
// writes the flattened arrays its Renderer would upload.
//
// TEST INFRASTRUCTURE ONLY (oracle/_ref recipe, this container only).  Linked
// against the reference's src/core, src/loaders and thirdparty/RadeonRays
// sources where they lie; this file is the only new code.  It calls
// LoadSceneFromFile (src/loaders/Loader.cpp:36) and Scene::ProcessScene
// (src/core/Scene.cpp:216) exactly as Main.cpp's LoadScene/InitRenderer do,
// then dumps bvhTranslator.nodes, vertIndices, verticesUVX, normalsUVY,
// transforms, materials, lights, the envmap and the render options/camera.
//
// Output: <out>.json (sizes, options, camera) and <out>.bin (raw arrays in
// the order listed in the json).
#define STB_IMAGE_IMPLEMENTATION
#define STB_IMAGE_WRITE_IMPLEMENTATION
#include "stb_image.h"
#include "stb_image_write.h"
#undef STB_IMAGE_IMPLEMENTATION
#undef STB_IMAGE_WRITE_IMPLEMENTATION

#include <cstdio>
#include <fstream>
#include <string>

#include "Loader.h"
#include "Scene.h"

using namespace GLSLPT;

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: ref_scene_dump <file.scene> <out_prefix>\n");
        return 2;
    }
    Scene* scene = new Scene();
    RenderOptions opts;
    if (!LoadSceneFromFile(argv[1], scene, opts)) {
        std::fprintf(stderr, "unable to load %s\n", argv[1]);
        return 1;
    }
    scene->renderOptions = opts;
    scene->ProcessScene();

    std::string prefix = argv[2];
    std::ofstream bin(prefix + ".bin", std::ios::binary);
    auto w = [&](const void* p, size_t n) { if (n) bin.write((const char*)p, n); };
    const auto& nodes = scene->bvhTranslator.nodes;
    w(nodes.data(), nodes.size() * sizeof(nodes[0]));
    w(scene->vertIndices.data(), scene->vertIndices.size() * sizeof(Indices));
    w(scene->verticesUVX.data(), scene->verticesUVX.size() * sizeof(Vec4));
    w(scene->normalsUVY.data(), scene->normalsUVY.size() * sizeof(Vec4));
    w(scene->transforms.data(), scene->transforms.size() * sizeof(Mat4));
    w(scene->materials.data(), scene->materials.size() * sizeof(Material));
    w(scene->lights.data(), scene->lights.size() * sizeof(Light));
    int ew = 0, eh = 0;
    float esum = 0.0f;
    if (scene->envMap) {
        ew = scene->envMap->width; eh = scene->envMap->height; esum = scene->envMap->totalSum;
        w(scene->envMap->img, sizeof(float) * 3 * ew * eh);
        w(scene->envMap->cdf, sizeof(float) * ew * eh);
    }
    w(scene->textureMapsArray.data(), scene->textureMapsArray.size());
    bin.close();

    FILE* js = std::fopen((prefix + ".json").c_str(), "w");
    const RenderOptions& o = scene->renderOptions;
    const Camera* c = scene->camera;
    std::fprintf(js, "{\n");
    std::fprintf(js, " \"sizeof_node\": %zu, \"sizeof_material\": %zu, \"sizeof_light\": %zu,\n",
                 sizeof(nodes[0]), sizeof(Material), sizeof(Light));
    std::fprintf(js, " \"num_bvh_nodes\": %zu, \"top_level_index\": %d,\n", nodes.size(), scene->bvhTranslator.topLevelIndex);
    std::fprintf(js, " \"num_tris\": %zu, \"num_vertices\": %zu, \"num_instances\": %zu,\n",
                 scene->vertIndices.size(), scene->verticesUVX.size(), scene->transforms.size());
    std::fprintf(js, " \"num_materials\": %zu, \"num_lights\": %zu,\n", scene->materials.size(), scene->lights.size());
    std::fprintf(js, " \"envmap_width\": %d, \"envmap_height\": %d, \"envmap_total_sum\": %.9g,\n", ew, eh, esum);
    std::fprintf(js, " \"num_textures\": %zu, \"tex_width\": %d, \"tex_height\": %d,\n", scene->textures.size(),
                 o.texArrayWidth, o.texArrayHeight);
    std::fprintf(js, " \"options\": {\"render_width\": %d, \"render_height\": %d, \"tile_width\": %d, \"tile_height\": %d,"
                     " \"max_depth\": %d, \"max_spp\": %d, \"rr_depth\": %d, \"enable_rr\": %d, \"enable_envmap\": %d,"
                     " \"enable_uniform_light\": %d, \"hide_emitters\": %d, \"enable_background\": %d,"
                     " \"transparent_background\": %d, \"enable_roughness_mollification\": %d, \"enable_volume_mis\": %d,"
                     " \"opengl_normal_map\": %d, \"enable_tonemap\": %d, \"enable_aces\": %d, \"simple_aces_fit\": %d,"
                     " \"uniform_light_col\": [%.9g, %.9g, %.9g], \"background_col\": [%.9g, %.9g, %.9g],"
                     " \"envmap_intensity\": %.9g, \"envmap_rot\": %.9g, \"roughness_mollification_amt\": %.9g},\n",
                 o.renderResolution.x, o.renderResolution.y, o.tileWidth, o.tileHeight, o.maxDepth, o.maxSpp, o.RRDepth,
                 (int)o.enableRR, (int)o.enableEnvMap, (int)o.enableUniformLight, (int)o.hideEmitters,
                 (int)o.enableBackground, (int)o.transparentBackground, (int)o.enableRoughnessMollification,
                 (int)o.enableVolumeMIS, (int)o.openglNormalMap, (int)o.enableTonemap, (int)o.enableAces, 0,
                 o.uniformLightCol.x, o.uniformLightCol.y, o.uniformLightCol.z, o.backgroundCol.x, o.backgroundCol.y,
                 o.backgroundCol.z, o.envMapIntensity, o.envMapRot, o.roughnessMollificationAmt);
    std::fprintf(js, " \"camera\": {\"position\": [%.9g, %.9g, %.9g], \"up\": [%.9g, %.9g, %.9g],"
                     " \"right\": [%.9g, %.9g, %.9g], \"forward\": [%.9g, %.9g, %.9g],"
                     " \"fov\": %.9g, \"focal_dist\": %.9g, \"aperture\": %.9g}\n",
                 c->position.x, c->position.y, c->position.z, c->up.x, c->up.y, c->up.z, c->right.x, c->right.y,
                 c->right.z, c->forward.x, c->forward.y, c->forward.z, c->fov, c->focalDist, c->aperture);
    std::fprintf(js, "}\n");
    std::fclose(js);
    delete scene;
    return 0;
}
