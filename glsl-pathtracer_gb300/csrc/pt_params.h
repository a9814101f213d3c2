// pt_params.h - launch parameters shared by the host context (pt_capi.cu)
// and the kernels (pt_kernels.cu).  Everything the reference passes as
// textures and uniforms (common/uniforms.glsl:25-53, globals.glsl:141) is a
// device pointer or a value here, passed by value at each launch.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ptgb {

// Traversal stack entries per thread (node groups of the wide BVH; one per
// wide level on the current path, TLAS + BLAS).
constexpr int kStackSize = 48;
// Stack entries of one instance entry: the TLAS node group, the pending
// instances, the world ray's reciprocal direction and a sentinel.
constexpr int kInstanceEntries = 4;
// Postponing triangle tests (the wavefront's warp step modes) puts at most
// one triangle group on the stack per wide level besides the node group, so
// a BVH of depth d (TLAS + BLAS levels) with 2 d + 4 <= kStackSize never
// overflows; deeper BVHs are traversed without postponing.
constexpr bool trav_postpone_fits(int depth) { return 2 * depth + kInstanceEntries <= kStackSize; }
// Without postponing, a ray pushes at most one node group per wide level
// on its path, plus the instance entry's four when it enters an instance
// from the TLAS.
constexpr int trav_stack_need(int tlas_depth, int blas_depth, bool direct) {
    return direct ? blas_depth : tlas_depth + blas_depth + kInstanceEntries;
}

// One job of a batch (pt_batch_render): the values the kernels take from
// the job instead of from Params.  Jobs are ordered by path_base.
struct BatchJob {
    int tlas_root;
    int direct, entry_inst, entry_mat;  // as in Params
    int light_base, num_lights;
    int max_depth, rr_depth;
    int width, height, tile_w, tile_h, ntx, nty;
    float cam_pos[3], cam_up[3], cam_right[3], cam_fwd[3];
    float cam_fov, cam_focal, cam_aperture;
    float4* accum;
    int path_base, npix, num_passes, first_pass;
    int pixel_base;  // prefix of the jobs' pixel counts
    int id;          // the job's index in the batch (completion counters)
    // the job's render options and its context's environment and texture
    // maps (read in place, not copied into the batch)
    uint32_t flags;
    float mollify_amt;
    float uniform_light[3];
    const float4* env;
    const float* cdf;
    int env_w, env_h;
    float env_total, env_intensity, env_rot;
    const uchar4* tex;
    int tex_w, tex_h, num_tex;
};

struct Params {
    // acceleration structure (bvh8.h)
    const uint4* nodes;     // WideNode, 5 x uint4
    const float4* tris;     // WideTri, 3 x float4
    const int4* insts;      // InstRef
    const float4* xf;       // InstXf, 10 x float4 per instance
    const uint4* inst_bounds;  // 2 x uint4 per InstRef (root_may_hit); null: every instance is entered
    const uint4* node_words;   // 2 x uint4 per wide node: each slot's hit-mask word (intersect_node)
    int tlas_root;
    // direct != 0: the scene is one untransformed instance, and traversal
    // starts in its BLAS (tlas_root is then the BLAS root) as instance
    // entry_inst with material entry_mat (-1: per triangle, the merged BLAS);
    // the hits are those of entering it from the TLAS
    int direct, entry_inst, entry_mat;
    // reference arrays used for shading
    const int* vidx;        // Indices, 3 x int32 per triangle
    const float4* verts;    // verticesUVX
    const float4* norms;    // normalsUVY
    const float4* mats;     // Material, 8 x float4
    const float4* lights;   // Light repacked as 4 x float4
    int num_lights;
    int num_materials;
    // environment map (RGB padded to float4) and its CDF
    const float4* env;
    const float* cdf;
    // texture maps: num_tex RGBA8 layers of tex_w x tex_h (textureMapsArrayTex)
    const uchar4* tex;
    int tex_w, tex_h, num_tex;
    int env_w, env_h;
    float env_total, env_intensity, env_rot;
    // options
    uint32_t flags;         // F_* bits (pt_device.cuh)
    int max_depth, rr_depth;
    float uniform_light[3];
    float mollify_amt;
    // camera (GLSLPT::Camera, globals.glsl:83-92)
    float cam_pos[3], cam_up[3], cam_right[3], cam_fwd[3];
    float cam_fov, cam_focal, cam_aperture;
    // frame
    int width, height, tile_w, tile_h, ntx, nty;
    // output / bookkeeping
    float4* accum;
    // [0] closest-hit queries, [1] shadow queries, [2] paths, [3] paths ended
    // at PT_MAX_PATH_ITERATIONS, [4] shadow queries answered without traversal
    unsigned long long* counters;
    int* status;                   // PT_OK or a PT_ERR_* code set by the kernels
    // traversal stack entries a ray may push (kStackSize; a lower bound is a
    // failure-detection test's way to make the overflow status fire)
    int stack_limit;
    // shadow queries whose contribution is never added are answered without
    // traversal: bit 0 any-hit queries (always), bit 1 VOL_MIS transmittance
    // queries (when a query cannot draw random numbers or take more than one
    // segment unless its ray meets one of the num_blend_boxes world boxes of
    // blended-alpha instances, 6 floats each: lo, hi); 0 turns both off
    int untraced;
    const float* blend_boxes;
    int num_blend_boxes;
    // batches (pt_batch_render): the jobs, paths left per job and the
    // %globaltimer at which each job's last path finished ([num_jobs]: start)
    const BatchJob* jobs;
    int num_jobs;
    int* job_remaining;
    unsigned long long* job_done;
};

// Work description of one render launch.
struct RenderWork {
    int x0, y0, w, h;       // pixel rectangle (full frame or one tile, clipped)
    int first_pass, num_passes;
    int tile_frame;         // >= 0: frame number of a single tile launch (pt_render_tile)
    int tile_x, tile_y;     // tile of a single-tile launch
};

}  // namespace ptgb

// kernel launchers (pt_kernels.cu)
namespace ptgb {
cudaError_t launch_render(const Params& p, const RenderWork& w, int integrator, cudaStream_t s);
cudaError_t launch_trace_closest(const Params& p, const void* rays, int n, void* hits, cudaStream_t s);
cudaError_t launch_trace_shadow(const Params& p, const void* rays, const float* maxd, int n, unsigned char* occ,
                                cudaStream_t s);
cudaError_t launch_bsdf_eval(const float* rec, const float* V, const float* N, const float* L, int n, float* f,
                             float* pdf, cudaStream_t s);
cudaError_t launch_bsdf_sample(const float* rec, const float* V, const float* N, const uint32_t* seeds, int n,
                               float* L, float* f, float* pdf, cudaStream_t s);
cudaError_t launch_tonemap(const Params& p, int num_samples, int enable_tonemap, int enable_aces, int simple_aces,
                           int background, int transparent, const float* bg, unsigned char* out, cudaStream_t s);
}  // namespace ptgb
