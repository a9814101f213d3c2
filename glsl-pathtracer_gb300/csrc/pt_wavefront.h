// pt_wavefront.h - device buffers and launch shapes of the wavefront integrator.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

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
    // replay of suspended shade steps (VOL_MIS scenes with alpha materials),
    // allocated by wavefront_alloc_replay when a scene needs them
    float4 *tr0 = nullptr, *tr1 = nullptr;
    uint4 *trng0 = nullptr, *trng1 = nullptr;
    int* qr = nullptr;
    bool fixed = false;  // views the static scratch (wavefront_fixed_buffers)
    cudaGraphExec_t graph_exec = nullptr;
};

// Block sizes and persistent grid sizes of the stage kernels.
struct WavefrontTuning {
    int extend_block = 128, shade_block = 128, shadow_block = 128;
    // idle lanes of a warp that trigger a retire + refill round in the
    // persistent extend / shadow kernels (PT_WAVEFRONT_REFILL overrides)
    int extend_refill = 20, shadow_refill = 20;
    // triangle steps run when at least min_tris lanes of a warp have
    // triangles pending; fewer are postponed (0: every lane steps on its own;
    // PT_WAVEFRONT_MIN_TRIS overrides).  Needs trav_postpone_fits(depth).
    int min_tris = 8;
    // the same two for the first round (camera rays and the shadow rays of
    // their hits), per stage; <= 0 (refill) / < 0 (min_tris): as the other
    // rounds (PT_WAVEFRONT_REFILL_FIRST, PT_WAVEFRONT_MIN_TRIS_FIRST,
    // PT_WAVEFRONT_SHADOW_REFILL_FIRST, PT_WAVEFRONT_SHADOW_MIN_TRIS_FIRST)
    int extend_refill_first = 0, min_tris_first = -1;
    int shadow_refill_first = 0, min_tris_shadow_first = -1;
    // and the first round's extend kernel variant and shading register
    // budget (-1: as the other rounds; PT_WAVEFRONT_VARIANT_FIRST,
    // PT_WAVEFRONT_SHADE_VARIANT_FIRST)
    int extend_variant_first = -1, shade_variant_first = -1;
    int extend_grid = 0, shade_grid = 0, shadow_grid = 0;
    // kernel variants of the traversal stages: 0 = 8 blocks (64 registers),
    // scalar node test; 1 = 8 blocks, packed; 2 = 6 blocks (80 registers),
    // scalar; 3 = 6 blocks, packed (PT_WAVEFRONT_VARIANT overrides); the
    // persistent grid of each variant fills the GPU
    int extend_variant = 0, shadow_variant = 0;
    int extend_grid_v[4] = {0, 0, 0, 0}, shadow_grid_v[4] = {0, 0, 0, 0};
    int transmit_grid_v[4] = {0, 0, 0, 0};  // wf_transmit (deferred VOL_MIS transmittance), by shadow_variant
    int replay_grid_v[4] = {0, 0, 0, 0};    // wf_transmit_replay, by shadow_variant
    // the plain surface shade stage: 0 = no register bound, 1 = 80 registers
    // (6 blocks), 2 = 64 registers (8 blocks)
    int shade_variant = 0;
    int shade_grid_v[3] = {0, 0, 0};
    int resident_blocks_256 = 0;
};

// Per-stage device time (CUDA events recorded around each launch on the
// launching stream), for profiling runs; batches then run without graphs.
enum { STAGE_GENERATE = 0, STAGE_EXTEND = 1, STAGE_SHADE = 2, STAGE_SHADOW = 3, STAGE_RESOLVE = 4, STAGE_COUNT = 5 };
struct StageTimer {
    std::vector<cudaEvent_t> pool;  // 2 events per recorded launch
    std::vector<int> kinds;         // stage of each recorded launch
    size_t used = 0;
    cudaError_t mark(cudaStream_t s);
    void reset() { used = 0; kinds.clear(); }
    // sums per stage (ms, launches); synchronises with the recorded events
    cudaError_t summarise(float ms[STAGE_COUNT], int launches[STAGE_COUNT]) const;
    void release();
};

size_t wavefront_bytes_per_path();
// Path state in a fixed device array of kFixedScratchPaths paths instead of
// cudaMalloc'd buffers (pt_render_tile_noalloc).  The first call on a device
// looks the array's address up (cudaGetSymbolAddress, with that device
// current); later calls only carve it.  Every context on the device shares
// the one array, so its users must not overlap in time.
constexpr int kFixedScratchPaths = 16384;
cudaError_t wavefront_fixed_buffers(WavefrontBuffers& wb);
cudaError_t wavefront_alloc(WavefrontBuffers& wb, int capacity);
void wavefront_free(WavefrontBuffers& wb);
// The replay arrays for wb.capacity paths (no-op when present).
cudaError_t wavefront_alloc_replay(WavefrontBuffers& wb);
// VOL_MIS scenes with alpha materials shade in the replay form.
bool wavefront_needs_replay(uint32_t flags);
cudaError_t wavefront_default_tuning(WavefrontTuning& t, int block);
// Inputs and outputs of the adjoint (path-replay backpropagation) batch.
// The loss gradient dLoss/dI is given per pixel of the full frame, with
// I = accumulation / num_passes; per path, dLoss/dL = dLoss/dI / num_passes.
// Gradients: 11 per material (pt_grad.cuh's parameter order), then 3 per
// light (emission r, g, b).
struct AdjView {
    const float* dimage = nullptr;  // 3 floats per full-frame pixel
    float inv_passes = 1.0f;
    int width = 0;                  // full-frame width (row stride of dimage)
    float* grad = nullptr;
    int num_materials = 0, num_lights = 0;
    int grad_size = 0;              // floats of grad
    int shared = 0;                 // accumulate per block in shared memory first
    float4* v = nullptr;            // 3 per path: deferred next-event gradient (11 values + material)
    float4* le = nullptr;           // 1 per path: light-emission gradient + light index (-1: none)
};

// The adjoint batch for the work W (one batch: W.num_passes * pixels must
// fit the buffers).  run_forward: trace the forward batch first (no
// accumulation) so that each path's radiance is in the buffers; otherwise
// they must hold the forward batch of the same work already.
cudaError_t launch_adjoint(const Params& p, const RenderWork& W, WavefrontBuffers& wb, const WavefrontTuning& t,
                           const AdjView& A, bool run_forward, cudaStream_t s, int* launches = nullptr);

// A batch (pt_batch_render) runs as a sequence of chunks, each one wavefront
// over the BatchJob entries [entry_begin, entry_begin + entry_count) of
// p.jobs: whole passes of some jobs, their paths numbered consecutively
// (paths), their pixels too (pixels), max_depth the largest of theirs.  A
// job's passes may span several chunks, in pass order, so that its
// accumulation adds the passes in the order a single render would.
struct BatchChunk {
    int entry_begin, entry_count;
    int paths, pixels, max_depth;
};
// p.jobs: the whole entry table; p.job_remaining / p.job_done: indexed by
// BatchJob::id.  start_stamp receives the global timer at the start.
cudaError_t launch_batch(const Params& p, const BatchChunk* chunks, int num_chunks, WavefrontBuffers& wb,
                         const WavefrontTuning& t, cudaStream_t s, unsigned long long* start_stamp, int* launches,
                         bool inline_shadows);

// *launches (if given) receives the number of kernels launched; with a
// timer, every launch is timed (and no graph is used).
cudaError_t launch_wavefront(const Params& p, const RenderWork& W, WavefrontBuffers& wb, const WavefrontTuning& t,
                             bool use_graph, cudaStream_t s, int* launches = nullptr, StageTimer* timer = nullptr);

}  // namespace ptgb
