/*
 * pt_cuda.h - C ABI of the GB300 path-tracing library (libptgb.so).
 *
 * The library replaces the device half of GLSL-PathTracer's renderer: the
 * class GLSLPT::Renderer (src/core/Renderer.h:104-185) that uploads the
 * flattened scene into GL buffers/textures and runs tile.glsl per pixel.
 * Every entry point below takes plain pointers and sizes; buffers passed in
 * are HOST memory unless the name says otherwise.  All calls return 0
 * (PT_OK) on success or a PT_ERR_* code; pt_last_error() gives the message.
 *
 * Data layouts are exactly the reference's host arrays, so a caller hands over
 * what GLSLPT::Scene::ProcessScene (src/core/Scene.cpp:216-297) produced:
 *   bvh_nodes     RadeonRays::BvhTranslator::Node, 9 floats each
 *                 (thirdparty/RadeonRays/bvh_translator.h:45-50):
 *                 bboxmin.xyz, bboxmax.xyz, LRLeaf.xyz (ints stored as floats)
 *   vert_indices  GLSLPT::Indices {x,y,z} per triangle (src/core/Scene.h:61-64)
 *   vertices_uvx  Vec4 position + u per vertex (src/core/Scene.h:94)
 *   normals_uvy   Vec4 normal + v per vertex (src/core/Scene.h:95)
 *   transforms    Mat4 per instance, row-vector layout, translation in
 *                 data[3][0..2] (src/math/Mat4.h:30-62)
 *   materials     GLSLPT::Material, 32 floats (src/core/Material.h:47-119)
 *   lights        GLSLPT::Light, 15 floats (src/core/Scene.h:50-59)
 *   envmap        EnvironmentMap img (RGB float) + cdf (src/core/EnvironmentMap.h)
 *
 * Images are W*H float4 / uchar4 with row 0 at the BOTTOM (GL convention,
 * as glGetTexImage returns them in Renderer::GetOutputBuffer,
 * src/core/Renderer.cpp:619-634).
 *
 * Threading: one context = one CUDA stream; calls on one context must be
 * serialised by the caller (the reference renderer is single-threaded).
 */
#ifndef PT_CUDA_H
#define PT_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define PT_OK                 0
#define PT_ERR_INVALID_ARG    1  /* null pointer, bad size, bad index in scene data */
#define PT_ERR_CUDA           2  /* a CUDA runtime call failed */
#define PT_ERR_OUT_OF_MEMORY  3  /* device allocation failed */
#define PT_ERR_STACK_OVERFLOW 4  /* traversal stack limit hit (kernel status word): pt_create rejects
                                  * BVHs deeper than the stack (PT_ERR_UNSUPPORTED), so only a
                                  * bound lowered through PT_TRAVERSAL_STACK_LIMIT (a failure-
                                  * detection test's setting, read at pt_create) reaches it */
#define PT_ERR_UNSUPPORTED    5  /* scene feature the kernels do not implement */
#define PT_ERR_TIMEOUT        6  /* a bounded device wait ran out */
#define PT_ERR_QUEUE_OVERFLOW 7  /* wavefront queue capacity exceeded */

/* Iterations (closest-hit query + shading) a camera path may take.  The
 * reference's loop (pathtrace.glsl:287-423) has no bound: alpha pass-through
 * keeps the depth (pathtrace.glsl:423), and a ray grazing a blended surface
 * advances by EPS per crossing, so such a path can run for tens of thousands
 * of iterations or, on a shared plane, without end.  Every integrator here
 * (and the oracle) ends a path after this many iterations with the radiance
 * gathered so far; pt_stats.truncated_paths counts them. */
#define PT_MAX_PATH_ITERATIONS 1024

/* ---- scene description: the reference's flattened host arrays ---------- */
typedef struct pt_scene_desc {
    const float*   bvh_nodes;        /* 9 floats per node */
    int32_t        num_bvh_nodes;
    int32_t        top_level_index;  /* BvhTranslator::topLevelIndex */
    const int32_t* vert_indices;     /* 3 int32 per triangle */
    int32_t        num_tris;
    const float*   vertices_uvx;     /* 4 floats per vertex */
    const float*   normals_uvy;      /* 4 floats per vertex */
    int32_t        num_vertices;
    const float*   transforms;       /* 16 floats per instance */
    int32_t        num_instances;
    const float*   materials;        /* 32 floats per material */
    int32_t        num_materials;
    const float*   lights;           /* 15 floats per light */
    int32_t        num_lights;
    const float*   envmap_rgb;       /* envmap_width*envmap_height*3 floats, or NULL */
    const float*   envmap_cdf;       /* envmap_width*envmap_height floats */
    int32_t        envmap_width;
    int32_t        envmap_height;
    float          envmap_total_sum;
    const uint8_t* texture_maps;     /* num_textures * tex_width*tex_height*4 bytes, or NULL */
    int32_t        tex_width;
    int32_t        tex_height;
    int32_t        num_textures;
} pt_scene_desc;

/* Mirror of GLSLPT::RenderOptions (src/core/Renderer.h:37-100); booleans are
 * 0/1 ints.  Fields that only drive the window/UI are left out. */
typedef struct pt_render_options {
    int32_t render_width, render_height;
    int32_t tile_width, tile_height;
    int32_t max_depth;
    int32_t max_spp;                 /* -1: unlimited */
    int32_t rr_depth;
    int32_t enable_rr;
    int32_t enable_envmap;
    int32_t enable_uniform_light;
    int32_t hide_emitters;
    int32_t enable_background;
    int32_t transparent_background;
    int32_t enable_roughness_mollification;
    int32_t enable_volume_mis;
    int32_t opengl_normal_map;
    int32_t enable_tonemap;
    int32_t enable_aces;
    int32_t simple_aces_fit;
    float   uniform_light_col[3];
    float   background_col[3];
    float   envmap_intensity;
    float   envmap_rot;              /* degrees, as in RenderOptions::envMapRot */
    float   roughness_mollification_amt;
} pt_render_options;

/* GLSLPT::Camera fields read by the shaders (src/core/Camera.h:41-50);
 * fov in radians, as Camera stores it. */
typedef struct pt_camera {
    float position[3];
    float up[3];
    float right[3];
    float forward[3];
    float fov;
    float focal_dist;
    float aperture;
} pt_camera;

/* One ray of a ray set (test hook for ClosestHit / AnyHit). */
typedef struct pt_ray {
    float origin[3];
    float direction[3];
} pt_ray;

/* Result of a closest-hit query over the triangle BVH.  prim_id is the
 * index into vert_indices (the global triangle index the reference reads at
 * closest_hit.glsl:122), inst_id the instance (-leaf-1 of the TLAS leaf),
 * both -1 on a miss; t is the hit distance (INF = 1e6 on a miss). */
typedef struct pt_hit {
    float   t;
    float   u, v;                    /* barycentrics uvt.x, uvt.y */
    int32_t prim_id;
    int32_t inst_id;
} pt_hit;

/* Counters of the last render call. */
typedef struct pt_stats {
    uint64_t closest_rays;           /* executed closest-hit queries */
    uint64_t shadow_rays;            /* any-hit queries / transmittance segments the
                                        reference traces, untraced_shadow_rays included */
    uint64_t paths;                  /* camera paths traced */
    float    kernel_ms;              /* device time of the last render call (CUDA events) */
    int32_t  status;                 /* device status word of the last call (PT_OK or PT_ERR_*) */
    int32_t  kernel_launches;        /* kernels the last render call launched */
    uint64_t truncated_paths;        /* paths ended at PT_MAX_PATH_ITERATIONS */
    uint64_t untraced_shadow_rays;   /* of shadow_rays: answered without traversal because
                                        their contribution is never added (the scattering pdf
                                        towards the light is 0): any-hit queries without an
                                        alpha test, and VOL_MIS transmittance queries that
                                        cannot meet blended geometry; the reference traces
                                        them and then discards the result */
} pt_stats;

#define PT_INTEGRATOR_MEGAKERNEL 0
#define PT_INTEGRATOR_WAVEFRONT  1

typedef struct pt_context pt_context;

/* Replaces: Renderer::Renderer(Scene*, shadersDir) -> InitGPUDataBuffers
 * (src/core/Renderer.cpp:41-87, 135-249).  Copies the scene to the device,
 * repacks the BVH into the device layout and allocates the accumulation
 * buffer for options->render_width x render_height. */
int pt_create(const pt_scene_desc* scene, const pt_render_options* options,
              pt_context** out_ctx);

/* Meshes and instances as GLSLPT::Scene holds them before ProcessScene
 * builds the BVH (src/core/Scene.h:88-102, Mesh.h:52-70): mesh m owns the
 * triangles [mesh_tri_offset[m], mesh_tri_offset[m+1]) of vert_indices
 * (ProcessScene's concatenation order, Scene.cpp:229-252). */
typedef struct pt_mesh_desc {
    const int32_t* mesh_tri_offset;    /* num_meshes + 1 offsets */
    int32_t        num_meshes;
    const int32_t* instance_mesh;      /* MeshInstance::meshID, one per scene instance */
    const int32_t* instance_material;  /* MeshInstance::materialID */
} pt_mesh_desc;

/* Replaces: the BVH builds of Scene::ProcessScene (per-mesh RadeonRays SBVH,
 * the TLAS and BvhTranslator, src/core/Scene.cpp:148-252) with a build on
 * the GPU (LBVH + 8-wide collapse): like pt_create, but scene->bvh_nodes
 * is ignored and may be NULL. */
int pt_create_gpu_bvh(const pt_scene_desc* scene, const pt_mesh_desc* meshes,
                      const pt_render_options* options, pt_context** out_ctx);

/* Replaces: Scene::RebuildInstances + the TLAS upload of Renderer::Update
 * (Scene.cpp:200-214, Renderer.cpp:647-663) for a context from
 * pt_create_gpu_bvh: new instance transforms, the BVH rebuilt on the GPU. */
int pt_update_transforms(pt_context* ctx, const float* transforms, int32_t num_instances);

/* Device time of the last GPU BVH build (ms). */
int pt_gpu_build_ms(pt_context* ctx, float* ms);

/* Batched multi-scene rendering.  The reference renders one scene per
 * Renderer (src/core/Renderer.cpp:41-87) and one frame per
 * Renderer::Render call (Renderer.cpp:533-640); a renderer serving many
 * small jobs would loop over contexts.  A batch renders the passes of
 * several contexts in one wavefront: their device scenes are concatenated
 * once by pt_batch_create (indices re-based), and pt_batch_render traces all
 * jobs' paths through the same persistent kernels, each path carrying its
 * job.  Each job's accumulation buffer receives what
 * pt_render_passes(job, first_pass[j], num_passes[j]) would add: the same
 * paths with the same random numbers, up to the last-bit rounding of the
 * batch kernels' separately compiled arithmetic.
 * Jobs share one device.  Each keeps its own render options (Russian
 * roulette, hidden emitters, background, uniform light, roughness
 * mollification, normal-map convention ...), environment map, texture maps,
 * alpha-tested materials and media; a medium with volume MIS
 * (enable_volume_mis) is refused (PT_ERR_UNSUPPORTED).  The batch launches with the tuning (pt_autotune /
 * pt_set_tuning) of the first job that has one, else the default.  The
 * contexts must outlive the batch: environment and texture maps are read
 * from them in place.  Scene, material and light updates made to a context
 * after pt_batch_create are not seen by the batch; camera, render-option
 * and environment-map changes are. */
typedef struct pt_batch pt_batch;
int pt_batch_create(pt_context* const* jobs, int32_t num_jobs, pt_batch** out_batch);
/* job_ms (optional, num_jobs floats): per job, the time from the start of
 * the batch to the completion of that job's last path (device global timer). */
int pt_batch_render(pt_batch* batch, const int32_t* first_pass, const int32_t* num_passes, float* job_ms);
int pt_batch_stats(pt_batch* batch, pt_stats* stats);
int pt_batch_destroy(pt_batch* batch);

/* Replaces: Renderer::~Renderer (src/core/Renderer.cpp:89-133). */
int pt_destroy(pt_context* ctx);

/* Run the context's work on a caller-owned stream (cudaStream_t passed as a
 * pointer); NULL restores the context's own stream. */
int pt_set_stream(pt_context* ctx, void* cuda_stream);

/* Replaces: the per-frame camera uniforms of Renderer::Update
 * (src/core/Renderer.cpp:766-772). */
int pt_set_camera(pt_context* ctx, const pt_camera* camera);

/* Replaces: Renderer::ReloadShaders / ResizeRenderer option handling
 * (src/core/Renderer.cpp:252-279, 380-544).  A change of resolution or tile
 * size reallocates and clears the accumulation buffer. */
int pt_set_options(pt_context* ctx, const pt_render_options* options);

/* Chooses the kernel form used by pt_render_* (PT_INTEGRATOR_*). */
int pt_set_integrator(pt_context* ctx, int32_t integrator);

/* Replaces: the instancesModified branch of Renderer::Update
 * (src/core/Renderer.cpp:649-665): new transforms, materials and the TLAS
 * slice nodes[top_level_index..num_bvh_nodes) of the flattened BVH. */
int pt_update_instances(pt_context* ctx, const float* transforms, int32_t num_instances,
                        const float* materials, int32_t num_materials,
                        const float* tlas_nodes, int32_t num_tlas_nodes);

/* Replaces: the envMapModified branch of Renderer::Update
 * (src/core/Renderer.cpp:668-690). */
int pt_update_envmap(pt_context* ctx, const float* rgb, const float* cdf,
                     int32_t width, int32_t height, float total_sum);

/* Replaces: the accumTexture clear of Renderer::Update when the scene is
 * dirty (src/core/Renderer.cpp:733-744). */
int pt_clear_accum(pt_context* ctx);

/* Replaces: one tile pass of Renderer::Render (src/core/Renderer.cpp:567-580):
 * traces one sample for every pixel of tile (tile_x, tile_y) with the RNG
 * frame number frame_num and adds it to the accumulation buffer. */
int pt_render_tile(pt_context* ctx, int32_t tile_x, int32_t tile_y, int32_t frame_num);

/* No counterpart in the reference.  pt_render_tile with the wavefront
 * integrator, for callers that must not allocate device memory while they
 * render (code running inside a memory budget fixed up front, or between
 * calls that must not synchronise the device, as cudaMalloc/cudaFree can):
 * the path state lives in one fixed device array of 16384 paths (5.5 MiB,
 * part of the loaded library), and tiles are traced in bands of whole rows
 * of at most 16384 pixels, giving the samples pt_render_tile gives.  The
 * first call on a device does a one-time set-up (looks the array up); make
 * that call before any stream capture.  Tiles wider than 16384 pixels are
 * rejected with PT_ERR_INVALID_ARG.  The array is shared by every context on
 * the device, and the call is asynchronous: it returns once its kernels are
 * queued on the context's stream.  Work on the array from another stream,
 * thread or context must therefore be ordered after this call's stream has
 * finished (a stream synchronise, or an event recorded after the call and
 * waited on), not merely after the call returns; overlapping work races on
 * the array and corrupts both renders.  Nothing in it needs to start at
 * zero.  The context's accumulation buffer is the one pt_render_tile adds
 * to (clear it with pt_clear_accum).  pt_set_stage_timing does not cover
 * this call.  The array's address is looked up once per device for the
 * life of the process; cudaDeviceReset invalidates it together with every
 * context on that device, so no call may follow a reset. */
int pt_render_tile_noalloc(pt_context* ctx, int32_t tile_x, int32_t tile_y, int32_t frame_num);

/* Replaces: the material re-upload of Renderer::Update's instancesModified
 * branch (src/core/Renderer.cpp:654-656) on its own: new values for the
 * num_materials materials (the count cannot change). */
int pt_update_materials(pt_context* ctx, const float* materials, int32_t num_materials);

/* No counterpart in the reference (its lights are uploaded once, at
 * Renderer::InitGPUDataBuffers): new light values, 15 floats each
 * (GLSLPT::Light); the count cannot change. */
int pt_update_lights(pt_context* ctx, const float* lights, int32_t num_lights);

/* Differentiable rendering (no counterpart in the reference): gradient of a
 * loss of the image I = accumulation / num_passes of sample passes
 * first_pass .. first_pass+num_passes-1 (the work of pt_render_passes) with
 * respect to the material parameters and light emissions, by path-replay
 * backpropagation with the wavefront integrator.
 *   d_image  dLoss/dI, 3 floats (r, g, b) per pixel, rows from the bottom
 *   grad     out: 11 floats per material -- baseColor r, g, b, metallic,
 *            roughness, subsurface, specularTint, sheen, sheenTint,
 *            clearcoat, clearcoatGloss (the raw GLSLPT::Material values) --
 *            then 3 per light (emission r, g, b)
 * Sampling is detached (directions, lobe and light choices, MIS weights and
 * Russian roulette are held fixed), so the result is the gradient of the
 * expected image.  When the last pt_render_passes call was the same work
 * with the wavefront integrator and nothing changed since, its per-path
 * radiance is reused; otherwise the forward paths are traced first (without
 * adding to the accumulation).  Media, alpha-tested materials and
 * environment maps are not supported (PT_ERR_UNSUPPORTED). */
int pt_render_adjoint(pt_context* ctx, int32_t first_pass, int32_t num_passes, const float* d_image,
                      float* grad);

/* Whole-frame form of the same work: sample passes first_pass ..
 * first_pass+num_passes-1, each pass being every tile in the reference's
 * order (Renderer.cpp:745-762), with the frame numbers the tile state machine
 * would have used for them.  Equal, sample for sample, to calling
 * pt_render_tile for each tile in turn. */
int pt_render_passes(pt_context* ctx, int32_t first_pass, int32_t num_passes);

/* Read the float4 accumulation (sum of samples, alpha in .w) into host
 * memory: render_width*render_height*4 floats. */
int pt_get_accum(pt_context* ctx, float* host_rgba);

/* No counterpart in the reference (its accumulation lives in a GL texture):
 * checkpoint / resume.  Overwrites the accumulation with
 * render_width*render_height*4 floats from host memory, as pt_get_accum
 * wrote them.  Samples are a function of the pixel, the pass index and the
 * tile, so a context that resumes from passes 0..k-1 (pt_set_accum, then
 * pt_render_passes(ctx, k, n)) ends with the accumulation that rendering
 * passes 0..k+n-1 in one go gives, bit for bit. */
int pt_set_accum(pt_context* ctx, const float* host_rgba);

/* Replaces: the buffer flip at the end of a sample pass
 * (src/core/Renderer.cpp:756-760), after which GetOutputBuffer shows the
 * completed pass: copies the accumulation buffer to the context's snapshot. */
int pt_snapshot_accum(pt_context* ctx);

/* Replaces: tonemap.glsl + Renderer::GetOutputBuffer (src/shaders/tonemap.glsl:97-133,
 * src/core/Renderer.cpp:619-634): accum / num_samples, tonemapped and gamma
 * corrected, written as RGBA8 into host memory (w*h*4 bytes, bottom row first).
 * from_snapshot = 1 reads the copy taken by pt_snapshot_accum instead of the
 * live accumulation. */
int pt_get_output(pt_context* ctx, int32_t num_samples, int32_t from_snapshot, uint8_t* host_rgba8);

/* Test hook: closest-hit queries (closest_hit.glsl:25-266, triangle part)
 * over the device BVH for n host rays. */
int pt_trace_rays(pt_context* ctx, const pt_ray* rays, int32_t n, pt_hit* hits);

/* Test hook: any-hit queries (anyhit.glsl:25-216) for n host rays with
 * per-ray max distances; occluded[i] = 1 if something is hit before max_dist[i]. */
int pt_trace_shadow(pt_context* ctx, const pt_ray* rays, const float* max_dist,
                    int32_t n, uint8_t* occluded);

/* Test hook: DisneyEval (disney.glsl:244-351) on n explicit inputs.
 * records: 20 floats each -- baseColor xyz, metallic, roughness, subsurface,
 * specularTint, sheen, sheenTint, clearcoat, clearcoatRoughness, specTrans,
 * ior, ax, ay, eta, anisotropic, 3 unused (the material as GetMaterial
 * leaves it, pathtrace.glsl:25-115); V, N, L: 3 floats each.  Outputs f
 * (3 floats, f * |cos L|) and pdf per input. */
int pt_bsdf_eval(pt_context* ctx, const float* records, const float* V, const float* N, const float* L,
                 int32_t n, float* f, float* pdf);

/* Test hook: DisneySample (disney.glsl:142-242) with the RNG state given per
 * input (4 uint32: the PCG4D seed, globals.glsl:149-166).  Outputs the
 * sampled L, f and pdf. */
int pt_bsdf_sample(pt_context* ctx, const float* records, const float* V, const float* N,
                   const uint32_t* seeds, int32_t n, float* L, float* f, float* pdf);

/* Launch configuration of the wavefront integrator's traversal stages (no
 * counterpart in the reference, whose shaders have none). */
typedef struct pt_tuning {
    int32_t extend_variant;  /* 0: 8 resident blocks of 128 (64 registers), scalar node test;
                              * 1: 8 blocks, packed-FP32 node test; 2: 6 blocks (80 registers),
                              * scalar; 3: 6 blocks, packed */
    int32_t shadow_variant;  /* the same choices for the shadow-ray stage */
    int32_t extend_refill;   /* idle lanes of a warp that trigger fetching new rays (1..32) */
    int32_t shadow_refill;
    int32_t min_tris;        /* lanes with triangles pending that run a triangle step (0: per lane) */
    int32_t shade_variant;   /* surface shading stage: 0 unbounded registers, 1 at most 80, 2 at most 64 */
    float   frame_ms;        /* pt_autotune: device time of the tuned frame */
    /* the first round of a frame (camera rays, coherent per warp, and the
     * shadow rays of their hits) on its own: refill thresholds (0: as
     * extend_refill / shadow_refill, else 1..32) and triangle-step quorums
     * (-1: as min_tris, else 0..32) */
    int32_t extend_refill_first;
    int32_t min_tris_first;
    int32_t shadow_refill_first;
    int32_t shadow_min_tris_first;
    int32_t extend_variant_first;  /* -1: as extend_variant, else 0..3 */
    int32_t shade_variant_first;   /* -1: as shade_variant, else 0..2 */
} pt_tuning;

/* Autotuner: renders num_passes whole-frame passes (at least 2^23 paths:
 * more passes on small images) into a scratch accumulation, the context's
 * untouched, with candidate configurations,
 * timing each stage with CUDA events, and keeps the fastest for this scene
 * and frame size.  Coordinate descent: kernel variants (extend and shadow
 * separately), refill thresholds (separately), min_tris, the shading
 * stage's register budget, then the first round's refill thresholds and
 * quorums, and with those fixed the other rounds' again, then the first
 * round's extend variant and shading budget. */
int pt_autotune(pt_context* ctx, int32_t num_passes, pt_tuning* result);
int pt_get_tuning(pt_context* ctx, pt_tuning* tuning);
int pt_set_tuning(pt_context* ctx, const pt_tuning* tuning);

/* Per-stage device time of the wavefront integrator (no counterpart in the
 * reference; a profiling aid).  With stage timing on, each wavefront launch
 * of a render call is bracketed by CUDA events on the context's stream and
 * batches run without CUDA graphs. */
typedef struct pt_stage_stats {
    float   ms[5];        /* generate, extend, shade, shadow, resolve: summed device time */
    int32_t launches[5];  /* launches of each stage */
} pt_stage_stats;
int pt_set_stage_timing(pt_context* ctx, int32_t on);
/* Stage times of the last render call (synchronises with its events). */
int pt_get_stage_stats(pt_context* ctx, pt_stage_stats* stats);

/* Counters and device time of the last pt_render_* call. */
int pt_get_stats(pt_context* ctx, pt_stats* stats);

/* Copy the last error message of this thread into buf (always terminated). */
int pt_last_error(char* buf, size_t size);

#ifdef __cplusplus
}
#endif

#endif /* PT_CUDA_H */
