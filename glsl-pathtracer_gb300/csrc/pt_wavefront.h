// pt_wavefront.h - device buffers and launch shapes of the wavefront integrator.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include "pt_params.h"

namespace ptgb {

// Path state of a batch, structure of arrays (one entry per path).
struct WavefrontBuffers {
    int capacity = 0;
    float4 *o = nullptr, *d = nullptr, *T = nullptr, *L = nullptr, *med = nullptr;
    uint4* rng = nullptr;
    int4* misc = nullptr;
    float4 *h0 = nullptr, *h2 = nullptr;
    int4* h1 = nullptr;
    float4 *so = nullptr, *sd0 = nullptr, *sd1 = nullptr, *sc0 = nullptr, *sc1 = nullptr, *sT = nullptr;
    float4* rad = nullptr;
    int* q[2] = {nullptr, nullptr};
    int* qs = nullptr;
    int* counts = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
};

// Block sizes and persistent grid sizes of the stage kernels.
struct WavefrontTuning {
    int extend_block = 128, shade_block = 128, shadow_block = 128;
    int extend_grid = 0, shade_grid = 0, shadow_grid = 0;
    int resident_blocks_256 = 0;
};

size_t wavefront_bytes_per_path();
cudaError_t wavefront_alloc(WavefrontBuffers& wb, int capacity);
void wavefront_free(WavefrontBuffers& wb);
cudaError_t wavefront_default_tuning(WavefrontTuning& t, int block);
cudaError_t launch_wavefront(const Params& p, const RenderWork& W, WavefrontBuffers& wb, const WavefrontTuning& t,
                             bool use_graph, cudaStream_t s);

}  // namespace ptgb
