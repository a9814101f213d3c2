// ref_tonemap_driver.cpp - runs the reference's tonemap.glsl on the CPU.
//
// TEST INFRASTRUCTURE ONLY (oracle/_ref recipe, this container only).  The
// rewritten shader (glsl2cpp.py) is included into namespace glsl on top of
// glsl_shim.hpp.  This file plays the GL driver of the tonemap pass of
// Renderer::Render / GetOutputBuffer (src/core/Renderer.cpp:582-634): it binds
// the accumulation as pathTraceTexture, sets the tonemap uniforms
// (Renderer.cpp:791-798) and runs the fragment shader once per pixel, at the
// pixel centre.  OPT_BACKGROUND / OPT_TRANSPARENT_BACKGROUND come from the
// compiler command line, as Renderer::InitShaders injects them
// (Renderer.cpp:425-434).  The float output is what the RGBA8 read-back of
// GetOutputBuffer converts.
#include "glsl_shim.hpp"

namespace glsl {
thread_local vec4 gl_FragCoord;
thread_local vec2 TexCoords;
thread_local vec4 outCol;
#include "globals.inc"
#include "tonemap.inc"
}  // namespace glsl

using namespace glsl;

extern "C" {

// accum: W*H float4 (bottom row first); out: W*H float4 of tonemap.glsl's outCol.
int ref_tonemap(const float* accum, int W, int H, float inv_sample_counter, int enable_tonemap, int enable_aces,
                int simple_aces_fit, const float* background_col, float* out) {
    pathTraceTexture.data = accum;
    pathTraceTexture.w = W;
    pathTraceTexture.h = H;
    pathTraceTexture.comps = 4;
    invSampleCounter = inv_sample_counter;
    enableTonemap = enable_tonemap != 0;
    enableAces = enable_aces != 0;
    simpleAcesFit = simple_aces_fit != 0;
    backgroundCol = vec3(background_col[0], background_col[1], background_col[2]);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            gl_FragCoord = vec4(float(x) + 0.5f, float(y) + 0.5f, 0.0f, 1.0f);
            TexCoords = vec2((float(x) + 0.5f) / float(W), (float(y) + 0.5f) / float(H));
            tonemap_main();
            float* o = out + 4 * ((size_t)y * W + x);
            o[0] = outCol.x; o[1] = outCol.y; o[2] = outCol.z; o[3] = outCol.w;
        }
    return 0;
}

}  // extern "C"
