// dropin_driver.cpp - drives ptgb::CudaRenderer the way the reference's
// Main.cpp drives GLSLPT::Renderer (test and bench infrastructure).
//
// The scene comes from a file written by SceneData.save_flat
// (pathtracer/scene.py): the flattened arrays of GLSLPT::Scene, the render
// options and the camera.  They fill a GLSLPT::Scene (mock_glslpt.h), and
// the renderer is constructed from that Scene*, as Main.cpp:157-161 does:
//
//   dropin_driver <scene> tiles <passes> <out.rgba> [integrator]
//       Update/Render cycles, one tile each, in the reference's order
//       until <passes> sample passes are complete, then GetOutputBuffer
//       (Main.cpp:177-180, 166-172) into <out.rgba>;
//   dropin_driver <scene> passes <passes> <out.rgba> [integrator]
//       the same samples with RenderPasses (all passes in one launch);
//   dropin_driver <scene> bench <passes per step> <steps> [warmup]
//       Autotune, then per step RenderPasses, the Update that completes
//       the passes and GetOutputBuffer (RGBA8 on the host); prints one JSON
//       line with the wall time of the timed steps and their ray count.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../glsl-pathtracer_gb300/csrc/cuda_renderer.h"
#include "mock_glslpt.h"

namespace {

template <class T> void read_into(FILE* f, std::vector<T>& v, size_t n) {
    v.resize(n);
    if (n && fread(v.data(), sizeof(T), n, f) != n) throw std::runtime_error("short scene file");
}

struct Loaded {
    GLSLPT::Scene scene;
    GLSLPT::Camera camera;
    GLSLPT::EnvironmentMap env;
    std::vector<float> env_img, env_cdf;
    std::vector<GLSLPT::Texture> tex;
};

// Scene file: "PTSCENE1", int32 counts (nodes, top, tris, vertices,
// instances, materials, lights, env w, env h, textures, tex w, tex h), float
// env total, pt_render_options, pt_camera, then the arrays in that order.
void load(const char* path, Loaded& L) {
    FILE* f = fopen(path, "rb");
    if (!f) throw std::runtime_error(std::string("cannot open ") + path);
    char magic[8];
    int32_t n[12];
    float total;
    pt_render_options o;
    pt_camera c;
    if (fread(magic, 1, 8, f) != 8 || std::memcmp(magic, "PTSCENE1", 8) != 0 || fread(n, 4, 12, f) != 12 ||
        fread(&total, 4, 1, f) != 1 || fread(&o, sizeof o, 1, f) != 1 || fread(&c, sizeof c, 1, f) != 1)
        throw std::runtime_error("bad scene file header");
    GLSLPT::Scene& s = L.scene;
    read_into(f, s.bvhTranslator.nodes, n[0]);
    s.bvhTranslator.topLevelIndex = n[1];
    read_into(f, s.vertIndices, n[2]);
    read_into(f, s.verticesUVX, n[3]);
    read_into(f, s.normalsUVY, n[3]);
    read_into(f, s.transforms, n[4]);
    read_into(f, s.materials, n[5]);
    read_into(f, s.lights, n[6]);
    if (n[7] > 0) {
        read_into(f, L.env_img, (size_t)n[7] * n[8] * 3);
        read_into(f, L.env_cdf, (size_t)n[7] * n[8]);
        L.env.width = n[7];
        L.env.height = n[8];
        L.env.totalSum = total;
        L.env.img = L.env_img.data();
        L.env.cdf = L.env_cdf.data();
        s.envMap = &L.env;
    }
    if (n[9] > 0) {
        read_into(f, s.textureMapsArray, (size_t)n[9] * n[10] * n[11] * 4);
        L.tex.resize(n[9]);
        for (auto& t : L.tex) s.textures.push_back(&t);
    }
    fclose(f);
    GLSLPT::RenderOptions& r = s.renderOptions;
    r.renderResolution = {o.render_width, o.render_height};
    r.windowResolution = r.renderResolution;
    r.tileWidth = o.tile_width;
    r.tileHeight = o.tile_height;
    r.maxDepth = o.max_depth;
    r.maxSpp = o.max_spp;
    r.RRDepth = o.rr_depth;
    r.texArrayWidth = n[10];
    r.texArrayHeight = n[11];
    r.enableRR = o.enable_rr;
    r.enableTonemap = o.enable_tonemap;
    r.enableAces = o.enable_aces;
    r.simpleAcesFit = o.simple_aces_fit;
    r.openglNormalMap = o.opengl_normal_map;
    r.enableEnvMap = o.enable_envmap;
    r.enableUniformLight = o.enable_uniform_light;
    r.hideEmitters = o.hide_emitters;
    r.enableBackground = o.enable_background;
    r.transparentBackground = o.transparent_background;
    r.enableRoughnessMollification = o.enable_roughness_mollification;
    r.enableVolumeMIS = o.enable_volume_mis;
    r.envMapIntensity = o.envmap_intensity;
    r.envMapRot = o.envmap_rot;
    r.roughnessMollificationAmt = o.roughness_mollification_amt;
    r.uniformLightCol = {o.uniform_light_col[0], o.uniform_light_col[1], o.uniform_light_col[2]};
    r.backgroundCol = {o.background_col[0], o.background_col[1], o.background_col[2]};
    L.camera.position = {c.position[0], c.position[1], c.position[2]};
    L.camera.up = {c.up[0], c.up[1], c.up[2]};
    L.camera.right = {c.right[0], c.right[1], c.right[2]};
    L.camera.forward = {c.forward[0], c.forward[1], c.forward[2]};
    L.camera.fov = c.fov;
    L.camera.focalDist = c.focal_dist;
    L.camera.aperture = c.aperture;
    s.camera = &L.camera;
}

void write_output(ptgb::CudaRenderer& r, const char* path) {
    unsigned char* data = nullptr;
    int w = 0, h = 0;
    r.GetOutputBuffer(&data, w, h);  // the caller delete[]s, as in Main.cpp:166-172
    FILE* f = fopen(path, "wb");
    const bool ok = f && fwrite(data, 4, (size_t)w * h, f) == (size_t)w * h;
    if (f) fclose(f);
    delete[] data;
    if (!ok) throw std::runtime_error(std::string("cannot write ") + path);
}

uint64_t rays_of_last_call(ptgb::CudaRenderer& r) {
    pt_stats st;
    if (pt_get_stats(r.context(), &st) != PT_OK || st.status != PT_OK) throw std::runtime_error("render failed");
    return st.closest_rays + st.shadow_rays;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 5) {
        fprintf(stderr, "usage: %s <scene> tiles|passes <passes> <out.rgba> [integrator]\n"
                        "       %s <scene> bench <passes per step> <steps> [warmup]\n", argv[0], argv[0]);
        return 2;
    }
    try {
        Loaded L;
        load(argv[1], L);
        const std::string mode = argv[2];
        const int passes = std::atoi(argv[3]);
        ptgb::CudaRenderer r(&L.scene, "../src/shaders/");  // GLSLPT::Scene*, as Main.cpp:157-161
        if (mode == "bench") {
            const int steps = std::atoi(argv[4]);
            const int warmup = argc > 5 ? std::atoi(argv[5]) : 3;
            const int W = L.scene.renderOptions.renderResolution.x, H = L.scene.renderOptions.renderResolution.y;
            r.Autotune(passes);  // before the timed region, as the bench's own context is tuned
            r.Update(0.0f);
            r.Render();      // the dirty frame (the reference's preview)
            r.Update(0.0f);  // the first tile of pass 0
            uint64_t rays = 0;
            auto t0 = std::chrono::steady_clock::now();
            for (int k = 0; k < warmup + steps; ++k) {
                if (k == warmup) {
                    rays = 0;
                    t0 = std::chrono::steady_clock::now();
                }
                r.RenderPasses(passes);
                rays += rays_of_last_call(r);
                r.Update(0.016f);  // the passes complete (snapshot); the next pass's first tile
                unsigned char* data = nullptr;
                int w = 0, h = 0;
                r.GetOutputBuffer(&data, w, h);
                delete[] data;
            }
            const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            printf("{\"seconds\": %.6f, \"steps\": %d, \"passes_per_step\": %d, \"rays\": %llu, \"width\": %d, "
                   "\"height\": %d, \"d2h_bytes_per_step\": %d}\n",
                   s, steps, passes, (unsigned long long)rays, W, H, W * H * 4);
            return 0;
        }
        if (argc > 5) r.SetIntegrator(std::atoi(argv[5]));
        // Main.cpp's loop: Update then Render, until `passes` passes are complete
        for (;;) {
            r.Update(0.016f);
            if (r.GetSampleCount() - 1 >= passes) break;
            if (mode == "passes" && !L.scene.dirty && r.AtPassStart())
                r.RenderPasses(passes - (r.GetSampleCount() - 1));
            else
                r.Render();
        }
        write_output(r, argv[4]);
    } catch (const std::exception& e) {
        fprintf(stderr, "dropin_driver: %s\n", e.what());
        return 1;
    }
    return 0;
}
