// pt_wavefront.cu - the wavefront form of the integrator (sm_103a).
//
// A batch is every pixel of the work rectangle times a range of sample
// passes: one path per (pixel, pass), its state kept in HBM as
// structure-of-arrays float4/int4/uint4 records.  Per bounce:
//   extend  closest-hit queries for the paths in the active queue
//   shade   ShadeStep (pt_integrator.cuh) for each of them: survivors are
//           appended to the next queue, next-event estimates to the shadow
//           queue
//   shadow  any-hit queries of the shadow queue, radiance += Ld * T
// then `resolve` adds each path's radiance into the accumulation buffer,
// pixel by pixel in pass order, which is the order the megakernel (and the
// reference's per-pass accumulation, tile.glsl:70-74) adds them in: the two
// forms' accumulations differ only by the last-bit rounding of their
// separately compiled shading arithmetic.
// The stage kernels are persistent grid-stride loops over a device-side
// count, so a whole batch (generate, max_depth+1 bounces, resolve) needs no
// host round trip and is captured as one CUDA graph.
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdlib>

#include "../../include/pt_cuda.h"
#include "pt_grad.cuh"
#include "pt_integrator.cuh"
#include "pt_wavefront.h"

namespace ptgb {

namespace {

struct WfView {  // device pointers of WavefrontBuffers, by value
    float4 *o, *d, *T, *L, *med;
    uint4* rng;
    int4* misc;
    float4 *h0, *h2;
    int4* h1;
    float4 *so, *sd0, *sd1, *sc0, *sc1, *sT;
    float4* rad;
    int* q[2];
    int* qs;
    int* counts;  // [0], [1] extension queues, [2] shadow queue, [4], [5] fetch counters of extend / shadow,
                  // [6] resume queue (replay)
    // replay of suspended shade steps (VOL_MIS with alpha materials): per
    // path the transmittance of its queries 0 and 1 and the RNG state after
    // each; the queue of paths to shade again
    float4 *tr0, *tr1;
    uint4 *trng0, *trng1;
    int* qr;
};

// Transmittance queries a path's current shade step has had traced (replay):
// bits 2-3 of misc.z, which store_path clears.
__device__ __forceinline__ int replay_done(const WfView& B, int i) { return (B.misc[i].z >> 2) & 3; }

// The replay hook: the transmittance queries of a shade step that were
// already traced return their recorded transmittance and continue with the
// RNG state they left; the next one suspends the step, keeping its ray and
// the RNG state at that point for wf_transmit_replay.
// A re-run also takes the environment sample of its first run (kept in sc0:
// radiance and pdf, sd1: direction, when the step suspended at the
// environment query) instead of drawing it again: the same values, without
// the two dependent CDF searches.  The environment query is always the
// step's first (DirectLight), so it is recorded whenever done > 0.
struct ReplayHook : NoHook {
    const WfView* B;
    int i, done, site = 0;
    Ray ray;
    uint4 rng_at;
    V3 env_Li, env_dir;
    float env_pdf;
    bool env_new = false;
    __device__ __forceinline__ bool env_sample(V3& Li, float& pdf, V3& dir) {
        if (done == 0) return false;
        const float4 a = B->sc0[i], b = B->sd1[i];
        Li = v3(a.x, a.y, a.z);
        pdf = a.w;
        dir = v3(b.x, b.y, b.z);
        return true;
    }
    __device__ __forceinline__ void env_sampled(V3 Li, float pdf, V3 dir) {
        env_Li = Li;
        env_pdf = pdf;
        env_dir = dir;
        env_new = true;
    }
    // queries before `done` were reached by an earlier run of this step
    __device__ __forceinline__ bool first_visit() const { return site >= done; }
    __device__ __forceinline__ bool transmit(const Params&, const Ray& r, Rng& rng, uint2*, Counters&, V3& T) {
        if (site < done) {
            const float4 t = site ? B->tr1[i] : B->tr0[i];
            const uint4 g = site ? B->trng1[i] : B->trng0[i];
            T = v3(t.x, t.y, t.z);
            rng.x = g.x; rng.y = g.y; rng.z = g.z; rng.w = g.w;
            ++site;
            return true;
        }
        ray = r;
        rng_at = make_uint4(rng.x, rng.y, rng.z, rng.w);
        return false;
    }
};

// MEDIUM == 0 (no media in the scene): the medium record is never read or
// written (its fields keep StartPath's values, which nothing reads).
template <int MEDIUM = 1>
__device__ __forceinline__ void load_path(const WfView& B, int i, PathState& ps) {
    const float4 o = B.o[i], d = B.d[i], T = B.T[i], L = B.L[i];
    const float4 m = MEDIUM ? B.med[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const uint4 g = B.rng[i];
    const int4 misc = B.misc[i];
    ps.r.origin = v3(o.x, o.y, o.z);
    ps.alpha = o.w;
    ps.r.direction = v3(d.x, d.y, d.z);
    ps.scatterPdf = d.w;
    ps.throughput = v3(T.x, T.y, T.z);
    ps.prevRough = T.w;
    ps.radiance = v3(L.x, L.y, L.z);
    ps.medium.density = L.w;
    ps.medium.color = v3(m.x, m.y, m.z);
    ps.medium.anisotropy = m.w;
    ps.rng.x = g.x; ps.rng.y = g.y; ps.rng.z = g.z; ps.rng.w = g.w;
    ps.depth = misc.x;
    ps.matID = misc.y;
    ps.inMedium = misc.z & 1;
    ps.surfaceScatter = (misc.z >> 1) & 1;
    ps.medium.type = misc.z >> 8;
    ps.job = misc.w;
}

// A path as StartPath leaves it (tile.glsl:41-74): throughput 1, radiance
// 0 and no medium are constants, so wf_generate stores only the ray, the
// RNG state and misc, and the shade launches of the first round
// (with_first_round) read only those.
__device__ __forceinline__ void store_path_start(const WfView& B, int i, const PathState& ps) {
    B.o[i] = make_float4(ps.r.origin.x, ps.r.origin.y, ps.r.origin.z, ps.alpha);
    B.d[i] = make_float4(ps.r.direction.x, ps.r.direction.y, ps.r.direction.z, ps.scatterPdf);
    B.rng[i] = make_uint4(ps.rng.x, ps.rng.y, ps.rng.z, ps.rng.w);
    B.misc[i] = make_int4(ps.depth, ps.matID,
                          (ps.inMedium ? 1 : 0) | (ps.surfaceScatter ? 2 : 0) | (ps.medium.type << 8), ps.job);
}
__device__ __forceinline__ void load_path_start(const WfView& B, int i, PathState& ps) {
    const float4 o = B.o[i], d = B.d[i];
    const uint4 g = B.rng[i];
    const int4 misc = B.misc[i];
    ps.r.origin = v3(o.x, o.y, o.z);
    ps.alpha = o.w;
    ps.r.direction = v3(d.x, d.y, d.z);
    ps.scatterPdf = d.w;
    ps.throughput = v3(1.0f);
    ps.prevRough = 0.0f;
    ps.radiance = v3(0.0f);
    ps.medium.density = 0.0f;
    ps.medium.color = v3(0.0f);
    ps.medium.anisotropy = 0.0f;
    ps.rng.x = g.x; ps.rng.y = g.y; ps.rng.z = g.z; ps.rng.w = g.w;
    ps.depth = misc.x;
    ps.matID = misc.y;
    ps.inMedium = misc.z & 1;
    ps.surfaceScatter = (misc.z >> 1) & 1;
    ps.medium.type = misc.z >> 8;
    ps.job = misc.w;
}
// Bit 2 of an extend or shade launch's `in`: the launch belongs to the first
// round, whose paths are all as wf_generate stored them (the replay form's
// resume launches of that round included: a suspended path's state stays as
// it was), and whose queue 0 is the identity, so path k is queue entry k.
constexpr int kFirstRound = 4;
__host__ __device__ __forceinline__ int with_first_round(int in, bool first) { return in | (first ? kFirstRound : 0); }

template <int MEDIUM = 1>
__device__ __forceinline__ void store_path(const WfView& B, int i, const PathState& ps) {
    B.o[i] = make_float4(ps.r.origin.x, ps.r.origin.y, ps.r.origin.z, ps.alpha);
    B.d[i] = make_float4(ps.r.direction.x, ps.r.direction.y, ps.r.direction.z, ps.scatterPdf);
    B.T[i] = make_float4(ps.throughput.x, ps.throughput.y, ps.throughput.z, ps.prevRough);
    B.L[i] = make_float4(ps.radiance.x, ps.radiance.y, ps.radiance.z, ps.medium.density);
    if (MEDIUM) B.med[i] = make_float4(ps.medium.color.x, ps.medium.color.y, ps.medium.color.z, ps.medium.anisotropy);
    B.rng[i] = make_uint4(ps.rng.x, ps.rng.y, ps.rng.z, ps.rng.w);
    B.misc[i] = make_int4(ps.depth, ps.matID,
                          (ps.inMedium ? 1 : 0) | (ps.surfaceScatter ? 2 : 0) | (ps.medium.type << 8), ps.job);
}

// ------------------------------------------------------------ batches
// A batch renders several contexts' scenes (concatenated arrays) in one
// sequence of stage launches; each path carries its job, whose values
// replace Params' where they differ per job.
// VOL_MIS scenes without alpha materials: EvalTransmittance draws no random
// numbers, so its rays go to the transmittance stage (wf_transmit)
__host__ __device__ __forceinline__ bool transmit_deferred(uint32_t flags) {
    return (flags & F_MEDIUM) && (flags & F_VOL_MIS) && !(flags & F_ALPHA_TEST);
}

__device__ __forceinline__ void job_params(Params& Pj, const BatchJob& J) {
    Pj.tlas_root = J.tlas_root;
    Pj.direct = J.direct;
    Pj.entry_inst = J.entry_inst;
    Pj.entry_mat = J.entry_mat;
    Pj.lights = Pj.lights + 4 * J.light_base;
    Pj.num_lights = J.num_lights;
    Pj.max_depth = J.max_depth;
    Pj.rr_depth = J.rr_depth;
    Pj.width = J.width;
    Pj.height = J.height;
    Pj.tile_w = J.tile_w;
    Pj.tile_h = J.tile_h;
    Pj.ntx = J.ntx;
    Pj.nty = J.nty;
    for (int k = 0; k < 3; ++k) {
        Pj.cam_pos[k] = J.cam_pos[k];
        Pj.cam_up[k] = J.cam_up[k];
        Pj.cam_right[k] = J.cam_right[k];
        Pj.cam_fwd[k] = J.cam_fwd[k];
    }
    Pj.cam_fov = J.cam_fov;
    Pj.cam_focal = J.cam_focal;
    Pj.cam_aperture = J.cam_aperture;
    Pj.accum = J.accum;
    Pj.flags = J.flags;
    Pj.mollify_amt = J.mollify_amt;
    for (int k = 0; k < 3; ++k) Pj.uniform_light[k] = J.uniform_light[k];
    Pj.env = J.env;
    Pj.cdf = J.cdf;
    Pj.env_w = J.env_w;
    Pj.env_h = J.env_h;
    Pj.env_total = J.env_total;
    Pj.env_intensity = J.env_intensity;
    Pj.env_rot = J.env_rot;
    Pj.tex = J.tex;
    Pj.tex_w = J.tex_w;
    Pj.tex_h = J.tex_h;
    Pj.num_tex = J.num_tex;
}
// The part of job_params a traversal stage needs when it starts a ray: the
// BLAS entry and the job's lights (LightsClosest / LightsAny, trav_init).
// A ray start costs a few hundred instructions, so loading the whole job
// record there (camera, resolution, accumulation ...) is not free.
__device__ __forceinline__ void job_trav_params(Params& Pj, const BatchJob& J) {
    Pj.tlas_root = J.tlas_root;
    Pj.direct = J.direct;
    Pj.entry_inst = J.entry_inst;
    Pj.entry_mat = J.entry_mat;
    Pj.lights = Pj.lights + 4 * J.light_base;
    Pj.num_lights = J.num_lights;
    Pj.flags = J.flags;
}
// the job of path i (jobs ordered by path_base)
__device__ __forceinline__ int job_of_path(const Params& P, int i) {
    int lo = 0, hi = P.num_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P.jobs[mid].path_base <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}
__device__ __forceinline__ uint64_t global_timer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// a path of job j has finished: the last one stamps the job's completion
// A path of job table entry j has ended.  The lanes of a warp that end paths
// of the same job together share one atomic: the lowest of them subtracts
// their count, and the subtraction that takes the job's count to zero stamps
// the global timer.  (One atomic per path put every path of a job on a
// single address, which the L2 serialises: millions per frame.)
__device__ __forceinline__ void job_path_done(const Params& P, int j) {
    if (!P.jobs) return;
    const int id = P.jobs[j].id;
    const unsigned same = __match_any_sync(__activemask(), id);
    if ((int)(threadIdx.x & 31) == __ffs(same) - 1) {
        const int n = __popc(same);
        if (atomicSub(P.job_remaining + id, n) == n) P.job_done[id] = global_timer();
    }
}

__global__ void wf_batch_stamp(unsigned long long* t) { *t = global_timer(); }

// Append to a queue with one atomic per warp.
__device__ __forceinline__ void push(int* queue, int* count, int value, bool pred) {
    const unsigned mask = __ballot_sync(__activemask(), pred);
    if (!mask) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(mask));
    base = __shfl_sync(__activemask(), base, leader);
    if (pred) queue[base + __popc(mask & ((1u << lane) - 1))] = value;
}

// Order of a pass's paths over the pixels of a w x h rectangle: bands of
// four rows, each cut into blocks of eight columns (the last band and the
// last block of a band may be smaller), blocks in column order within a
// band, pixels of a block in row order.  The 32 paths of a warp are then an
// 8 x 4 block of pixels rather than a 32-pixel row segment: camera rays
// that hit nearby surface points traverse the same nodes and shade nearby
// data.  Slot s -> pixel (x, y) and its inverse.
__host__ __device__ __forceinline__ void slot_pixel(int s, int w, int h, int& x, int& y) {
    const int band = s / (4 * w);
    const int r = s - band * 4 * w;
    const int hb = h - 4 * band < 4 ? h - 4 * band : 4;
    const int full = w >> 3;
    const int c = r / (8 * hb);
    const int q = r - c * 8 * hb;
    const int wb = c < full ? 8 : w - 8 * full;
    y = 4 * band + q / wb;
    x = 8 * c + q % wb;
}
__host__ __device__ __forceinline__ int pixel_slot(int x, int y, int w, int h) {
    const int band = y >> 2, hb = h - 4 * band < 4 ? h - 4 * band : 4;
    const int c = x >> 3, full = w >> 3;
    const int wb = c < full ? 8 : w - 8 * full;
    return band * 4 * w + c * 8 * hb + (y - 4 * band) * wb + (x - 8 * c);
}

// BATCH (this kernel and the stage kernels below): the batch form
// (pt_batch_render), compiled apart so that the single-scene kernels carry
// none of the per-job code.
template <bool BATCH = false>
__global__ void __launch_bounds__(256) wf_generate(Params P, RenderWork W, WfView B, int first_pass, int npass,
                                                   int batch_paths = 0) {
    const int npix = W.w * W.h;
    const int n = BATCH ? batch_paths : npix * npass;
    uint32_t paths = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        PathState ps;
        if constexpr (BATCH) {  // the job's pixel and pass, its camera
            const int j = job_of_path(P, i);
            const BatchJob& J = P.jobs[j];
            Params Pj = P;
            job_params(Pj, J);
            const int li = i - J.path_base;
            const int pix = li % J.npix, k = li / J.npix;
            int px, py;
            slot_pixel(pix, J.width, J.height, px, py);
            RenderWork Wj = W;
            Wj.tile_frame = -1;
            StartPath(Pj, px, py, FrameNumber(Pj, Wj, J.first_pass + k, px, py), ps);
            ps.job = j;
        } else {
            const int pix = i % npix, k = i / npix;
            int px, py;
            slot_pixel(pix, W.w, W.h, px, py);
            px += W.x0;
            py += W.y0;
            StartPath(P, px, py, FrameNumber(P, W, first_pass + k, px, py), ps);
        }
        store_path_start(B, i, ps);
        B.q[0][i] = i;
        ++paths;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        B.counts[0] = n;
        B.counts[1] = 0;
        B.counts[2] = 0;
        B.counts[4] = 0;  // fetch counters of the extend and shadow stages
        B.counts[5] = 0;
    }
    add_counters(P, 0, 0, paths);
}

// Each thread of a warp that has no ray takes the next one from the queue
// (one atomic per warp); returns the queue slot or -1.
__device__ __forceinline__ int fetch_work(int* counter, int n, bool need) {
    const int lane = threadIdx.x & 31;
    const unsigned needm = __ballot_sync(0xffffffffu, need);
    if (!needm) return -1;
    const int leader = __ffs(needm) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(needm));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (!need) return -1;
    const int k = base + __popc(needm & ((1u << lane) - 1));
    return k < n ? k : -1;
}

// Persistent traversal loop shared by the extend and shadow stages.  Lanes
// trace independently, one traversal step per iteration; retiring finished
// rays and fetching new ones (divergent, memory-heavy code) runs for the
// whole warp at once, only when at least `refill` lanes are idle -- or, once
// the queue is empty, when all are.  This keeps that code from running for
// one or two lanes on almost every iteration.
__device__ __forceinline__ int refill_target(bool exhausted, int refill) { return exhausted ? 32 : refill; }

// Closest-hit queries of the queue.  Persistent: threads keep taking rays
// from the queue until it is empty, so a warp's lanes stay busy however
// unequal the rays are.
// Traversal is memory-latency bound: 8 blocks of 128 threads (64 registers)
// keep 32 warps per SM in flight.
// DIRECT (this kernel and wf_shadow): the single-instance form of the
// traversal (trav_step), chosen at launch when Params::direct is set.
template <int MINB, bool PACKED, bool BATCH = false, bool DIRECT = false>
__global__ void __launch_bounds__(128, MINB) wf_extend(Params P, WfView B, int in, int refill, int min_tris) {
    uint2 stack[kStackSize];
    const bool first = (in & kFirstRound) != 0;  // queue `in` is the identity (wf_generate)
    in &= 1;
    const int n = B.counts[in];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        B.counts[in ^ 1] = 0;  // the next queue and the shadow queue start empty
        B.counts[2] = 0;
        B.counts[5] = 0;       // fetch counter of the shadow stage
    }
    Counters cnt{0, 0};
    Trav s;
    HitRecord hr;
    float tl = PT_INF;
    int ray = -1;
    bool tracing = false, exhausted = false;
    for (;;) {
        if (ray >= 0 && !tracing) {  // retire
            FinishClosest(s, tl, hr);
            B.h0[ray] = make_float4(hr.t, hr.u, hr.v, hr.w);
            B.h1[ray] = make_int4(hr.prim, hr.inst, hr.mat,
                                  (hr.hit ? 1 : 0) | (hr.isEmitter ? 2 | (hr.light << 2) : 0));
            if (hr.isEmitter)  // read by the shade stage for light hits only
                B.h2[ray] = make_float4(hr.lightEmission.x, hr.lightEmission.y, hr.lightEmission.z, hr.lightPdf);
            ray = -1;
        }
        if (!exhausted) {  // refill
            const int k = fetch_work(B.counts + 4, n, ray < 0);
            exhausted = __any_sync(0xffffffffu, ray < 0 && k < 0);
            if (k >= 0) {
                ray = first ? k : B.q[in][k];
                const float4 o = B.o[ray], d = B.d[ray];
                const Ray r{v3(o.x, o.y, o.z), v3(d.x, d.y, d.z)};
                const int4 misc = B.misc[ray];
                if constexpr (BATCH) {
                    Params Pj = P;
                    job_trav_params(Pj, P.jobs[misc.w]);
                    tl = LightsClosest(Pj, r, misc.x, hr);
                    trav_init(s, Pj, r.origin, r.direction, tl);
                } else {
                    tl = LightsClosest(P, r, misc.x, hr);
                    trav_init(s, P, r.origin, r.direction, tl);
                }
                tracing = true;
                cnt.closest++;
            }
        }
        if (!__any_sync(0xffffffffu, tracing)) break;
        const int target = refill_target(exhausted, refill);
        do {
            const int mode = min_tris > 0 ? trav_warp_mode(s, tracing, min_tris) : TRAV_LANE;
            if (tracing && trav_step<false, false, PACKED, DIRECT>(s, P, stack, nullptr, mode) != TRAV_RUNNING)
                tracing = false;
        } while (__popc(__ballot_sync(0xffffffffu, !tracing)) < target);
    }
    add_counters(P, cnt.closest, cnt.shadow, 0);
}

// ------------------------------------------------------------ adjoint
// Path-replay backpropagation (the adjoint replays each path from its seed,
// so nothing of the forward pass is kept but each path's radiance L).  The
// sampling is detached: directions, lobe choices, MIS weights and Russian
// roulette are held fixed, and the derivative of each term of L is taken
// through the BSDF values and the light emissions it contains:
//   - an emitter hit adds w * Le * beta: d/dLe = w * beta;
//   - next-event estimation adds w * Li * f_L / p * beta, Li = Le * number
//     of lights: d/dtheta through f_L, d/dLe = w * #lights * f_L / p * beta;
//     both count only when the shadow ray is unoccluded (wf_shadow);
//   - every later term is proportional to the BSDF value f of this vertex's
//     sampled direction, so d/dtheta of (L - terms up to here) is
//     (L - terms up to here) * df / f per channel.
// Each term is dotted with dLoss/dL of the path.  The unknown visibility of
// this vertex's next-event ray at shade time is handled by storing the
// difference of its two cases for the shadow stage.
struct AdjHook {
    const Params* P;
    const AdjView* A;
    float* acc;      // gradient accumulator (shared memory or A->grad)
    V3 dL, Ltot;     // dLoss/dL of the path and its forward radiance
    int mat;
    bool mollify;
    float mollified;
    V3 beta;         // throughput at the current surface vertex
    bool has_nee;
    int light;
    float G[grad::kParams];  // next-event term's parameter gradient (minus the sampled-f part)
    V3 gle;                  // next-event term's light-emission gradient

    __device__ __forceinline__ void material(const PathState& ps, float prevRough) {
        mat = ps.matID;
        mollify = (P->flags & F_MOLLIFY) && ps.depth > 0;
        mollified = mixf(0.0f, prevRough, P->mollify_amt);
    }
    __device__ __forceinline__ void emitter(const PathState& ps, float misWeight, const HitRecord& hr) {
        if (hr.light < 0 || hr.light >= A->num_lights) return;
        float* g = acc + A->num_materials * grad::kParams + 3 * hr.light;
        atomicAdd(g + 0, dL.x * ps.throughput.x * misWeight);
        atomicAdd(g + 1, dL.y * ps.throughput.y * misWeight);
        atomicAdd(g + 2, dL.z * ps.throughput.z * misWeight);
    }
    __device__ __forceinline__ void vertex(const PathState& ps) {
        beta = ps.throughput;
        has_nee = false;
    }
    // out[k] += sum_c w1_c df_c/dtheta_k (and the same with w2 into out2)
    template <bool TWO>
    // All 11 partial derivatives in one forward-mode evaluation: one primal
    // BSDF evaluation instead of one per chunk (measured fastest on GB300
    // against chunks of 4 and 6, despite the wider duals).
    __device__ __forceinline__ void df(float eta, V3 V, V3 N, V3 L, V3 w1, V3 w2, float* out, float* out2) const {
        constexpr int NC = grad::kParams;
#pragma unroll 1
        for (int chunk = 0; chunk * NC < grad::kParams; ++chunk) {
            const grad::MatD<NC> m = grad::LoadMaterialD<NC>(P->mats, mat, chunk, mollify, mollified);
            const grad::DV3<NC> f = grad::DisneyEvalD(m, eta, V, N, L);
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                const int q = chunk * NC + k;
                if (q < grad::kParams) {
                    out[q] += w1.x * f.x.d[k] + w1.y * f.y.d[k] + w1.z * f.z.d[k];
                    if (TWO) out2[q] += w2.x * f.x.d[k] + w2.y * f.y.d[k] + w2.z * f.z.d[k];
                }
            }
        }
    }
    __device__ __forceinline__ void nee_light(int index, float misWeight, V3 Li, V3 sf, float lightPdf, float eta,
                                              V3 V, V3 N, V3 L) {
        has_nee = true;
        light = index;
#pragma unroll
        for (int k = 0; k < grad::kParams; ++k) G[k] = 0.0f;
        const float s = misWeight / lightPdf;
        df<false>(eta, V, N, L, dL * beta * Li * s, v3(0.0f), G, nullptr);
        gle = dL * beta * sf * (s * (float)P->num_lights);
    }
    __device__ __forceinline__ void sample(float eta, V3 V, V3 N, V3 L, V3 f, const PathState& ps,
                                           const ShadowReq& sr) {
        const V3 rest = Ltot - ps.radiance;  // the terms after this vertex, plus its next-event term
        const V3 nee = (has_nee && (sr.adds & 2)) ? sr.contrib[1] * sr.T : v3(0.0f);
        V3 wu, wn;
        wu.x = f.x != 0.0f ? dL.x * rest.x / f.x : 0.0f;
        wu.y = f.y != 0.0f ? dL.y * rest.y / f.y : 0.0f;
        wu.z = f.z != 0.0f ? dL.z * rest.z / f.z : 0.0f;
        wn.x = f.x != 0.0f ? dL.x * nee.x / f.x : 0.0f;
        wn.y = f.y != 0.0f ? dL.y * nee.y / f.y : 0.0f;
        wn.z = f.z != 0.0f ? dL.z * nee.z / f.z : 0.0f;
        float U[grad::kParams], W[grad::kParams];
#pragma unroll
        for (int k = 0; k < grad::kParams; ++k) U[k] = W[k] = 0.0f;
        df<true>(eta, V, N, L, wu, wn, U, W);
        float* g = acc + mat * grad::kParams;
#pragma unroll
        for (int k = 0; k < grad::kParams; ++k) {
            if (U[k] != 0.0f) atomicAdd(g + k, U[k]);
            G[k] -= W[k];  // applies only with the next-event term (unoccluded)
        }
    }
    __device__ __forceinline__ bool transmit(const Params& P, const Ray& r, Rng& rng, uint2* stack, Counters& cnt,
                                             V3& T) {
        T = EvalTransmittance(P, r, rng, stack, cnt);
        return true;
    }
    __device__ __forceinline__ bool env_sample(V3&, float&, V3&) { return false; }
    __device__ __forceinline__ void env_sampled(V3, float, V3) {}
    __device__ __forceinline__ bool first_visit() const { return true; }
};

__device__ __forceinline__ float* adj_accumulator(const AdjView& A, float* sgrad) {
    if (!A.shared) return A.grad;
    for (int k = threadIdx.x; k < A.grad_size; k += blockDim.x) sgrad[k] = 0.0f;
    __syncthreads();
    return sgrad;
}
__device__ __forceinline__ void adj_flush(const AdjView& A, const float* sgrad) {
    if (!A.shared) return;
    __syncthreads();
    for (int k = threadIdx.x; k < A.grad_size; k += blockDim.x)
        if (sgrad[k] != 0.0f) atomicAdd(A.grad + k, sgrad[k]);
}

// REPLAY (VOL_MIS with alpha materials): transmittance queries suspend the
// shade step instead of tracing inline; `in` | 2 shades the resume queue.
template <int MEDIUM, bool ENV, bool INLINE, bool ADJ = false, int MINB = 1, bool REPLAY = false, bool BATCH = false>
__global__ void __launch_bounds__(128, MINB) wf_shade(Params P, WfView B, int in, RenderWork W, AdjView A) {
    uint2 stack[INLINE && !REPLAY ? kStackSize : 1];
    extern __shared__ float sgrad[];
    float* acc = nullptr;
    if (ADJ) acc = adj_accumulator(A, sgrad);
    const bool first = (in & kFirstRound) != 0;
    const bool resume = REPLAY && (in & 2);
    in &= 1;
    const int* queue = resume ? B.qr : B.q[in];
    const int n = resume ? B.counts[6] : B.counts[in];
    Counters cnt{0, 0};
    uint32_t untraced = 0;
    for (int j0 = blockIdx.x * blockDim.x; j0 < n; j0 += gridDim.x * blockDim.x) {
        const int j = j0 + threadIdx.x;
        const bool valid = j < n;
        bool cont = false, shadow = false;
        int i = 0;
        if (valid) {
            i = first && !resume ? j : queue[j];
            PathState ps;
            if (first) load_path_start(B, i, ps);
            else load_path<MEDIUM>(B, i, ps);
            HitRecord hr;
            const float4 h0 = B.h0[i];
            const int4 h1 = B.h1[i];
            hr.t = h0.x; hr.u = h0.y; hr.v = h0.z; hr.w = h0.w;
            hr.prim = h1.x; hr.inst = h1.y; hr.mat = h1.z;
            hr.hit = h1.w & 1;
            hr.isEmitter = (h1.w >> 1) & 1;
            hr.light = h1.w >> 2;
            if (hr.isEmitter) {  // the light's emission and pdf (written by the extend stage for light hits)
                const float4 h2 = B.h2[i];
                hr.lightEmission = v3(h2.x, h2.y, h2.z);
                hr.lightPdf = h2.w;
            } else {
                hr.lightEmission = v3(0.0f);
                hr.lightPdf = 0.0f;
            }
            ShadowReq sr;
            if constexpr (ADJ) {
                AdjHook h;
                h.P = &P;
                h.A = &A;
                h.acc = acc;
                const int npix = W.w * W.h;
                int px, py;
                slot_pixel(i % npix, W.w, W.h, px, py);
                px += W.x0;
                py += W.y0;
                const float* di = A.dimage + 3 * ((size_t)py * A.width + px);
                h.dL = v3(di[0], di[1], di[2]) * A.inv_passes;
                const float4 lt = B.rad[i];
                h.Ltot = v3(lt.x, lt.y, lt.z);
                h.has_nee = false;
                h.light = -1;
                cont = ShadeStep<MEDIUM, ENV, INLINE>(P, ps, hr, sr, stack, cnt, h);
                const bool deferred = h.has_nee && (sr.n & 2) && (sr.adds & 2);
                if (deferred) {
                    A.v[3 * (size_t)i] = make_float4(h.G[0], h.G[1], h.G[2], h.G[3]);
                    A.v[3 * (size_t)i + 1] = make_float4(h.G[4], h.G[5], h.G[6], h.G[7]);
                    A.v[3 * (size_t)i + 2] = make_float4(h.G[8], h.G[9], h.G[10], __int_as_float(h.mat));
                }
                A.le[i] = make_float4(h.gle.x, h.gle.y, h.gle.z, __int_as_float(deferred ? h.light : -1));
            } else if constexpr (REPLAY) {
                ReplayHook rh;
                rh.B = &B;
                rh.i = i;
                rh.done = replay_done(B, i);
                cont = ShadeStep<MEDIUM, ENV, INLINE>(P, ps, hr, sr, stack, cnt, rh);
                if (sr.suspended) {  // the path is shaded again after its query is traced
                    B.so[i] = make_float4(rh.ray.origin.x, rh.ray.origin.y, rh.ray.origin.z, 0.0f);
                    B.sd0[i] = make_float4(rh.ray.direction.x, rh.ray.direction.y, rh.ray.direction.z, 0.0f);
                    if (rh.env_new) {
                        B.sc0[i] = make_float4(rh.env_Li.x, rh.env_Li.y, rh.env_Li.z, rh.env_pdf);
                        B.sd1[i] = make_float4(rh.env_dir.x, rh.env_dir.y, rh.env_dir.z, 0.0f);
                    }
                    if (rh.done) B.trng1[i] = rh.rng_at;
                    else B.trng0[i] = rh.rng_at;
                }
            } else {
                NoHook nh;
                if constexpr (BATCH) {
                    Params Pj = P;
                    job_params(Pj, P.jobs[ps.job]);
                    cont = ShadeStep<MEDIUM, ENV, INLINE>(Pj, ps, hr, sr, stack, cnt, nh);
                } else {
                    cont = ShadeStep<MEDIUM, ENV, INLINE>(P, ps, hr, sr, stack, cnt, nh);
                }
            }
            if (REPLAY && sr.suspended) {
                shadow = true;  // to the transmittance queue; the path state stays as it was
            } else {
                // Shadow queries whose contribution is never added (sr.adds
                // clear: the scattering pdf towards the light is 0, as for a
                // light below an opaque surface) need no traversal: their
                // answer changes nothing, and the shadow stage draws no
                // random numbers.  They count as queries, as the megakernel
                // and the reference trace them (pathtrace.glsl:198-209 and
                // 264-275 trace first and evaluate the BSDF after).
                if (!INLINE && MEDIUM != 2 && (P.untraced & 1) && sr.n != 0 && sr.adds == 0) {
                    cnt.shadow += __popc(sr.n);
                    untraced += __popc(sr.n);
                    sr.n = 0;
                }
                // the same for deferred transmittance queries (no alpha
                // materials in this form, so none draws random numbers; one
                // segment each when Params::untraced allows it)
                if (!INLINE && !REPLAY && MEDIUM == 2 && (P.untraced & 2) && (sr.n & ~sr.adds & 3)) {
                    const int drop = sr.n & ~sr.adds & 3;
                    cnt.shadow += __popc(drop);
                    untraced += __popc(drop);
                    sr.n &= ~drop;
                }
                shadow = !INLINE && sr.n != 0;
                // a path that ends here with no shadow query pending needs
                // only its radiance (B.rad, below)
                if (cont || shadow) store_path<MEDIUM>(B, i, ps);
            }
            if (!REPLAY && shadow && MEDIUM == 2) {  // deferred transmittance (wf_transmit)
                const int bits = sr.n | (sr.adds << 2) | (cont ? 0 : 16);
                B.so[i] = make_float4(sr.origin.x, sr.origin.y, sr.origin.z, __int_as_float(bits));
                // the hit record of this path is consumed: h0 / h2 carry the
                // factors until the next extend stage
                if (sr.n & 1) {
                    B.sd0[i] = make_float4(sr.dir[0].x, sr.dir[0].y, sr.dir[0].z, sr.pdf[0]);
                    B.sc0[i] = make_float4(sr.contrib[0].x, sr.contrib[0].y, sr.contrib[0].z, sr.mis[0]);
                    B.h0[i] = make_float4(sr.fac[0].x, sr.fac[0].y, sr.fac[0].z, 0.0f);
                }
                if (sr.n & 2) {
                    B.sd1[i] = make_float4(sr.dir[1].x, sr.dir[1].y, sr.dir[1].z, sr.pdf[1]);
                    B.sc1[i] = make_float4(sr.contrib[1].x, sr.contrib[1].y, sr.contrib[1].z, sr.mis[1]);
                    B.h2[i] = make_float4(sr.fac[1].x, sr.fac[1].y, sr.fac[1].z, 0.0f);
                }
                B.sT[i] = make_float4(sr.T.x, sr.T.y, sr.T.z, 0.0f);
            } else if (!REPLAY && shadow) {
                const int bits = sr.n | (sr.adds << 2) | (cont ? 0 : 16);
                B.so[i] = make_float4(sr.origin.x, sr.origin.y, sr.origin.z, __int_as_float(bits));
                if (sr.n & 1) {
                    B.sd0[i] = make_float4(sr.dir[0].x, sr.dir[0].y, sr.dir[0].z, sr.maxd[0]);
                    B.sc0[i] = make_float4(sr.contrib[0].x, sr.contrib[0].y, sr.contrib[0].z, 0.0f);
                }
                if (sr.n & 2) {
                    B.sd1[i] = make_float4(sr.dir[1].x, sr.dir[1].y, sr.dir[1].z, sr.maxd[1]);
                    B.sc1[i] = make_float4(sr.contrib[1].x, sr.contrib[1].y, sr.contrib[1].z, 0.0f);
                }
                B.sT[i] = make_float4(sr.T.x, sr.T.y, sr.T.z, 0.0f);
            }
            if (!shadow && !cont) {
                B.rad[i] = make_float4(ps.radiance.x, ps.radiance.y, ps.radiance.z, ps.alpha);
                if (BATCH) job_path_done(P, ps.job);
            }
        }
        push(B.q[in ^ 1], B.counts + (in ^ 1), i, valid && cont);
        push(B.qs, B.counts + 2, i, valid && shadow);
    }
    add_counters(P, cnt.closest, cnt.shadow, 0);
    add_untraced(P, untraced + cnt.untraced);
    if (ADJ) adj_flush(A, sgrad);
}

// Any-hit queries of the shadow queue (one or two rays per path: the env
// sample first, then the light sample), persistent like wf_extend, with the
// same batched retire / refill.  The deferred form is used only when AnyHit
// draws no random numbers.
template <bool ADJ, int MINB, bool PACKED, bool BATCH = false, bool DIRECT = false>
__global__ void __launch_bounds__(128, MINB) wf_shadow(Params P, WfView B, int refill, int min_tris, AdjView A) {
    uint2 stack[kStackSize];
    extern __shared__ float sgrad[];
    float* acc = nullptr;
    if (ADJ) acc = adj_accumulator(A, sgrad);
    const int n = B.counts[2];
    if (blockIdx.x == 0 && threadIdx.x == 0) B.counts[4] = 0;  // fetch counter of the next extend stage
    Counters cnt{0, 0};
    uint32_t untraced = 0;
    Trav s;
    // per-thread stage: 0 start env ray, 1 tracing it, 2 start light ray,
    // 3 tracing it, 4 both resolved
    int path = -1, bits = 0, stage = 0;
    bool occ0 = false, occ1 = false, exhausted = false;
    V3 origin = v3(0.0f);
    // start the next ray of a lane waiting at stage 0 or 2 (a ray a light
    // occludes, or one the path does not have, moves on without tracing)
    auto start = [&]() {
        if (path >= 0 && (stage == 0 || stage == 2)) {
            const int which = stage >> 1;
            if ((bits & (1 << which)) && !(bits & (4 << which)) && (P.untraced & 1)) {
                // a query whose contribution is never added (the other one
                // of this path is): counted, not traced (wf_shade)
                cnt.shadow++;
                untraced++;
                stage += 2;
            } else if (bits & (1 << which)) {
                const float4 d = which ? B.sd1[path] : B.sd0[path];
                const Ray r{origin, v3(d.x, d.y, d.z)};
                cnt.shadow++;
                bool occluded;
                if constexpr (BATCH) {
                    Params Pj = P;
                    job_trav_params(Pj, P.jobs[B.misc[path].w]);
                    occluded = LightsAny(Pj, r, d.w);
                    if (!occluded) trav_init(s, Pj, r.origin, r.direction, d.w);
                } else {
                    occluded = LightsAny(P, r, d.w);
                    if (!occluded) trav_init(s, P, r.origin, r.direction, d.w);
                }
                if (occluded) {
                    if (which) occ1 = true;
                    else occ0 = true;
                    stage += 2;
                } else {
                    stage += 1;
                }
            } else {
                stage += 2;
            }
        }
    };
    // both rays resolved: radiance += Ld * T
    auto resolve = [&]() {
        if (path >= 0 && stage == 4) {
            ShadowReq sr;
            sr.n = bits & 3;
            sr.adds = (bits >> 2) & 3;
            if (sr.n & 1) {
                const float4 c = B.sc0[path];
                sr.contrib[0] = v3(c.x, c.y, c.z);
            }
            if (sr.n & 2) {
                const float4 c = B.sc1[path];
                sr.contrib[1] = v3(c.x, c.y, c.z);
            }
            const int i = path;
            path = -1;
            const float4 T = B.sT[i];
            const V3 Ld = ResolveShadow(sr, occ0, occ1);
            float4 L = B.L[i];
            const V3 rad = AddScaled(v3(L.x, L.y, L.z), Ld, v3(T.x, T.y, T.z));
            L.x = rad.x;
            L.y = rad.y;
            L.z = rad.z;
            B.L[i] = L;
            if (bits & 16) {
                B.rad[i] = make_float4(L.x, L.y, L.z, B.o[i].w);
                if (BATCH) job_path_done(P, B.misc[i].w);
            }
            if (ADJ && (sr.adds & 2) && !occ1) {  // the next-event term counts: its gradients too
                const float4 le = A.le[i];
                const int light = __float_as_int(le.w);
                if (light >= 0) {
                    const float4 v0 = A.v[3 * (size_t)i], v1 = A.v[3 * (size_t)i + 1], v2 = A.v[3 * (size_t)i + 2];
                    float* g = acc + __float_as_int(v2.w) * grad::kParams;
                    const float gv[grad::kParams] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w, v2.x, v2.y, v2.z};
#pragma unroll
                    for (int k = 0; k < grad::kParams; ++k)
                        if (gv[k] != 0.0f) atomicAdd(g + k, gv[k]);
                    float* gl = acc + A.num_materials * grad::kParams + 3 * light;
                    atomicAdd(gl + 0, le.x);
                    atomicAdd(gl + 1, le.y);
                    atomicAdd(gl + 2, le.z);
                }
            }
        }
    };
    for (;;) {
        // retire: lanes done with the env ray start the light ray, lanes done
        // with both resolve; then refill the idle lanes
        start();
        resolve();
        if (!exhausted) {
            const int k = fetch_work(B.counts + 5, n, path < 0);
            exhausted = __any_sync(0xffffffffu, path < 0 && k < 0);
            if (k >= 0) {
                path = B.qs[k];
                const float4 so = B.so[path];
                bits = __float_as_int(so.w);
                origin = v3(so.x, so.y, so.z);
                occ0 = occ1 = false;
                stage = 0;
                start();
                start();
                resolve();
            }
        }
        const bool tracing = path >= 0 && (stage == 1 || stage == 3);
        if (!__any_sync(0xffffffffu, path >= 0)) break;
        const int target = refill_target(exhausted, refill);
        bool busy = tracing;
        while (__popc(__ballot_sync(0xffffffffu, !busy)) < target) {
            const int mode = min_tris > 0 ? trav_warp_mode(s, busy, min_tris) : TRAV_LANE;
            if (busy) {
                const int st = trav_step<true, false, PACKED, DIRECT>(s, P, stack, nullptr, mode);
                if (st != TRAV_RUNNING) {
                    if (stage == 1) occ0 = st == TRAV_HIT;
                    else occ1 = st == TRAV_HIT;
                    stage += 1;
                    busy = false;
                }
            }
        }
    }
    add_counters(P, cnt.closest, cnt.shadow, 0);
    add_untraced(P, untraced + cnt.untraced);
    if (ADJ) adj_flush(A, sgrad);
}

// TransmitStep out of line: the material evaluation runs once per segment,
// and kept out of the traversal loop it does not take that loop's registers.
static __device__ __noinline__ int transmit_hit(const Params& P, const HitRecord& hr, Ray& r, V3& T) {
    Rng rng{0u, 0u, 0u, 0u};  // unused: no material draws (ALPHA_MODE_BLEND is absent)
    return TransmitStep(P, hr, r, T, rng);
}

// Transmittance queries of the shadow queue (VOL_MIS scenes without alpha
// materials, where EvalTransmittance draws no random numbers): per path the
// env ray first, then the light ray, each a sequence of closest-hit segments
// through refractive surfaces (EvalTransmittance, pathtrace.glsl:117-153),
// persistent with the batched retire / refill of wf_shadow.  Each segment is
// one shadow query.
template <int MINB, bool PACKED>
__global__ void __launch_bounds__(128, MINB) wf_transmit(Params P, WfView B, int refill, int min_tris) {
    uint2 stack[kStackSize];
    const int n = B.counts[2];
    if (blockIdx.x == 0 && threadIdx.x == 0) B.counts[4] = 0;  // fetch counter of the next extend stage
    Counters cnt{0, 0};
    Trav s;
    // per-thread stage: 0 start env ray, 1 tracing it, 2 start light ray,
    // 3 tracing it, 4 both done
    int path = -1, bits = 0, stage = 0, seg = 0;
    // seg_end: the lane's segment traversal ended and its hit is not yet
    // evaluated (done with the warp's retire / refill, as in wf_transmit_replay)
    bool exhausted = false, seg_end = false;
    V3 origin = v3(0.0f), T0 = v3(1.0f), T1 = v3(1.0f);
    Ray r;
    float tl = PT_INF;
    bool light_hit = false;  // the segment's nearest analytic light is closer than tl
    auto segment = [&]() {  // the next closest-hit segment of the current ray
        cnt.shadow++;
        HitRecord hl;
        tl = LightsClosest(P, r, 0, hl);
        light_hit = hl.isEmitter;
        trav_init(s, P, r.origin, r.direction, tl);
    };
    auto start = [&]() {
        if (path >= 0 && (stage == 0 || stage == 2)) {
            const int which = stage >> 1;
            if (bits & (1 << which)) {
                const float4 d = which ? B.sd1[path] : B.sd0[path];
                r = Ray{origin, v3(d.x, d.y, d.z)};
                seg = 0;
                if (P.max_depth > 0) {
                    segment();
                    stage += 1;
                } else {
                    stage += 2;
                }
            } else {
                stage += 2;
            }
        }
    };
    auto resolve = [&]() {
        if (path >= 0 && stage == 4) {
            ShadowReq sr;
            sr.n = bits & 3;
            sr.adds = (bits >> 2) & 3;
            if (sr.n & 1) {
                const float4 c = B.sc0[path], d = B.sd0[path], f = B.h0[path];
                sr.contrib[0] = v3(c.x, c.y, c.z);
                sr.mis[0] = c.w;
                sr.pdf[0] = d.w;
                sr.fac[0] = v3(f.x, f.y, f.z);
            }
            if (sr.n & 2) {
                const float4 c = B.sc1[path], d = B.sd1[path], f = B.h2[path];
                sr.contrib[1] = v3(c.x, c.y, c.z);
                sr.mis[1] = c.w;
                sr.pdf[1] = d.w;
                sr.fac[1] = v3(f.x, f.y, f.z);
            }
            const int i = path;
            path = -1;
            const float4 T = B.sT[i];
            const V3 Ld = ResolveTransmit(sr, T0, T1, P.env_intensity);
            float4 L = B.L[i];
            const V3 rad = AddScaled(v3(L.x, L.y, L.z), Ld, v3(T.x, T.y, T.z));
            L.x = rad.x;
            L.y = rad.y;
            L.z = rad.z;
            B.L[i] = L;
            if (bits & 16) B.rad[i] = make_float4(L.x, L.y, L.z, B.o[i].w);
        }
    };
    for (;;) {
        if (seg_end) {  // the surface the segment hit: go through it (next segment) or end the ray
            seg_end = false;
            HitRecord hr;
            hr.isEmitter = light_hit;
            FinishClosest(s, tl, hr);
            V3 T = stage == 1 ? T0 : T1;
            const int st = transmit_hit(P, hr, r, T);
            if (st == 2) T = v3(0.0f);
            if (stage == 1) T0 = T;
            else T1 = T;
            if (st == 1 && ++seg < P.max_depth) segment();  // through a refractive surface
            else stage += 1;
        }
        start();
        resolve();
        if (!exhausted) {
            const int k = fetch_work(B.counts + 5, n, path < 0);
            exhausted = __any_sync(0xffffffffu, path < 0 && k < 0);
            if (k >= 0) {
                path = B.qs[k];
                const float4 so = B.so[path];
                bits = __float_as_int(so.w);
                origin = v3(so.x, so.y, so.z);
                T0 = T1 = v3(1.0f);
                stage = 0;
                start();
                start();
                resolve();
            }
        }
        const bool tracing = path >= 0 && (stage == 1 || stage == 3);
        if (!__any_sync(0xffffffffu, path >= 0)) break;
        const int target = refill_target(exhausted, refill);
        bool busy = tracing;
        while (__popc(__ballot_sync(0xffffffffu, !busy)) < target) {
            const int mode = min_tris > 0 ? trav_warp_mode(s, busy, min_tris) : TRAV_LANE;
            if (busy && trav_step<false, false, PACKED>(s, P, stack, nullptr, mode) != TRAV_RUNNING) {
                busy = false;
                seg_end = true;
            }
        }
    }
    add_counters(P, cnt.closest, cnt.shadow, 0);
}

// Paths still running after the wavefront rounds (alpha pass-through keeps
// the depth, pathtrace.glsl:423, so a path can cross blended surfaces any
// number of times): each thread finishes one such path as the megakernel
// does (inline traversal, shadow rays and transmittance), bounded like the
// megakernel's loop at PT_MAX_PATH_ITERATIONS per path in all (`rounds`
// done in the wavefront rounds).
template <int MEDIUM, bool ENV>
__device__ __forceinline__ void tail_path(const Params& P, PathState& ps, int rounds, uint2* stack, Counters& cnt) {
    for (int guard = rounds;;) {
        if (++guard > PT_MAX_PATH_ITERATIONS) {
            count_truncated(P);
            break;
        }
        HitRecord hr;
        TraceClosest(P, ps.r, ps.depth, hr, stack, cnt, false);
        ShadowReq sr;
        NoHook nh;
        if (!ShadeStep<MEDIUM, ENV, true>(P, ps, hr, sr, stack, cnt, nh)) break;
    }
}
template <int MEDIUM, bool ENV, bool BATCH = false>
__global__ void __launch_bounds__(128) wf_tail(Params P, WfView B, int in, int rounds) {
    uint2 stack[kStackSize];
    const int n = B.counts[in];
    Counters cnt{0, 0};
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const int i = B.q[in][j];
        PathState ps;
        load_path(B, i, ps);
        if constexpr (BATCH) {
            Params Pj = P;
            job_params(Pj, P.jobs[ps.job]);
            tail_path<MEDIUM, ENV>(Pj, ps, rounds, stack, cnt);
        } else {
            tail_path<MEDIUM, ENV>(P, ps, rounds, stack, cnt);
        }
        B.rad[i] = make_float4(ps.radiance.x, ps.radiance.y, ps.radiance.z, ps.alpha);
        if (BATCH) job_path_done(P, ps.job);
    }
    add_counters(P, cnt.closest, cnt.shadow, 0);
    add_untraced(P, cnt.untraced);
}

// TransmitStep out of line with the path's RNG (replay: blended materials
// draw from it).
static __device__ __noinline__ int transmit_hit_rng(const Params& P, const HitRecord& hr, Ray& r, V3& T, Rng& rng) {
    return TransmitStep(P, hr, r, T, rng);
}

// The suspended transmittance queries of the shadow queue (replay form):
// EvalTransmittance's segment loop (pathtrace.glsl:117-153) from the RNG
// state the shade step had at the query, persistent with the batched
// retire / refill of wf_shadow; each finished query records its
// transmittance and the RNG state after it, and queues its path to be
// shaded again.  Each segment is one shadow query.
template <int MINB, bool PACKED>
__global__ void __launch_bounds__(128, MINB) wf_transmit_replay(Params P, WfView B, int refill, int min_tris) {
    uint2 stack[kStackSize];
    const int n = B.counts[2];
    Counters cnt{0, 0};
    Trav s;
    int path = -1, seg = 0, slot = 0;
    // seg_end: the lane's segment traversal ended and its hit is not yet
    // evaluated; the warp evaluates such hits together, with its retire /
    // refill, rather than in the traversal loop where the other lanes wait
    bool exhausted = false, tracing = false, seg_end = false;
    V3 T = v3(1.0f);
    Ray r;
    Rng rng{0u, 0u, 0u, 0u};
    float tl = PT_INF;
    bool light_hit = false;
    auto segment = [&]() {
        cnt.shadow++;
        HitRecord hl;
        tl = LightsClosest(P, r, 0, hl);
        light_hit = hl.isEmitter;
        trav_init(s, P, r.origin, r.direction, tl);
    };
    for (;;) {
        if (seg_end) {  // the surface the segment hit: go through it (next segment) or stop
            seg_end = false;
            HitRecord hr;
            hr.isEmitter = light_hit;
            FinishClosest(s, tl, hr);
            const int st = transmit_hit_rng(P, hr, r, T, rng);
            if (st == 2) T = v3(0.0f);
            if (st == 1 && ++seg < P.max_depth) {
                segment();
                tracing = true;
            }
        }
        // retire: record the finished queries, queue their paths again
        const bool fin = path >= 0 && !tracing;
        if (fin) {
            const float4 t4 = make_float4(T.x, T.y, T.z, 0.0f);
            const uint4 g = make_uint4(rng.x, rng.y, rng.z, rng.w);
            if (slot) {
                B.tr1[path] = t4;
                B.trng1[path] = g;
            } else {
                B.tr0[path] = t4;
                B.trng0[path] = g;
            }
            int4 m = B.misc[path];
            m.z += 4;  // one more query traced (replay_done)
            B.misc[path] = m;
        }
        push(B.qr, B.counts + 6, path, fin);
        if (fin) path = -1;
        if (!exhausted) {
            const int k = fetch_work(B.counts + 5, n, path < 0);
            exhausted = __any_sync(0xffffffffu, path < 0 && k < 0);
            if (k >= 0) {
                path = B.qs[k];
                const float4 o = B.so[path], d = B.sd0[path];
                r = Ray{v3(o.x, o.y, o.z), v3(d.x, d.y, d.z)};
                slot = replay_done(B, path);
                const uint4 g = slot ? B.trng1[path] : B.trng0[path];
                rng.x = g.x; rng.y = g.y; rng.z = g.z; rng.w = g.w;
                T = v3(1.0f);
                seg = 0;
                tracing = P.max_depth > 0;
                if (tracing) segment();
            }
        }
        if (!__any_sync(0xffffffffu, path >= 0)) break;
        if (!__any_sync(0xffffffffu, tracing)) continue;
        const int target = refill_target(exhausted, refill);
        do {
            const int mode = min_tris > 0 ? trav_warp_mode(s, tracing, min_tris) : TRAV_LANE;
            if (tracing && trav_step<false, false, PACKED>(s, P, stack, nullptr, mode) != TRAV_RUNNING) {
                tracing = false;
                seg_end = true;
            }
        } while (__popc(__ballot_sync(0xffffffffu, !tracing)) < target);
    }
    add_counters(P, cnt.closest, cnt.shadow, 0);
}

__global__ void __launch_bounds__(256) wf_resolve(Params P, RenderWork W, WfView B, int npass) {
    const int npix = W.w * W.h;
    for (int pix = blockIdx.x * blockDim.x + threadIdx.x; pix < npix; pix += gridDim.x * blockDim.x) {
        int px, py;  // pix is the path slot of the pixel in every pass
        slot_pixel(pix, W.w, W.h, px, py);
        float4* out = P.accum + (size_t)(W.y0 + py) * P.width + W.x0 + px;
        float4 acc = *out;
        for (int k = 0; k < npass; ++k) {
            const float4 r = B.rad[(size_t)k * npix + pix];
            acc.x += r.x;
            acc.y += r.y;
            acc.z += r.z;
            acc.w += r.w;
        }
        *out = acc;
    }
}

// Batch resolve: one thread per pixel of all jobs, each job's passes in order.
__global__ void __launch_bounds__(256) wf_resolve_batch(Params P, WfView B, int total_pixels) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total_pixels; g += gridDim.x * blockDim.x) {
        int lo = 0, hi = P.num_jobs - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (P.jobs[mid].pixel_base <= g) lo = mid;
            else hi = mid - 1;
        }
        const BatchJob& J = P.jobs[lo];
        const int pix = g - J.pixel_base;  // the path slot of the pixel in every pass
        int px, py;
        slot_pixel(pix, J.width, J.height, px, py);
        float4* out = J.accum + (size_t)py * J.width + px;
        float4 acc = *out;
        for (int k = 0; k < J.num_passes; ++k) {
            const float4 r = B.rad[(size_t)J.path_base + (size_t)k * J.npix + pix];
            acc.x += r.x;
            acc.y += r.y;
            acc.z += r.z;
            acc.w += r.w;
        }
        *out = acc;
    }
}

WfView view_of(const WavefrontBuffers& wb) {
    WfView v;
    v.o = wb.o; v.d = wb.d; v.T = wb.T; v.L = wb.L; v.med = wb.med;
    v.rng = wb.rng; v.misc = wb.misc;
    v.h0 = wb.h0; v.h1 = wb.h1; v.h2 = wb.h2;
    v.so = wb.so; v.sd0 = wb.sd0; v.sd1 = wb.sd1; v.sc0 = wb.sc0; v.sc1 = wb.sc1; v.sT = wb.sT;
    v.rad = wb.rad;
    v.q[0] = wb.q[0]; v.q[1] = wb.q[1]; v.qs = wb.qs;
    v.counts = wb.counts;
    v.tr0 = wb.tr0; v.tr1 = wb.tr1; v.trng0 = wb.trng0; v.trng1 = wb.trng1; v.qr = wb.qr;
    return v;
}

template <int MEDIUM, bool ENV, bool INLINE>
cudaError_t launch_shade(const Params& p, const WfView& v, int in, int grid, int block, cudaStream_t s) {
    wf_shade<MEDIUM, ENV, INLINE><<<grid, block, 0, s>>>(p, v, in, RenderWork{}, AdjView{});
    return cudaGetLastError();
}

static cudaError_t launch_tail(const Params& p, const WfView& v, int in, int rounds, int grid, cudaStream_t s) {
    const int medium = (p.flags & F_MEDIUM) ? ((p.flags & F_VOL_MIS) ? 2 : 1) : 0;
    const bool env = (p.flags & F_ENVMAP) != 0;
    switch (medium * 2 + (env ? 1 : 0)) {
        case 0: wf_tail<0, false><<<grid, 128, 0, s>>>(p, v, in, rounds); break;
        case 1: wf_tail<0, true><<<grid, 128, 0, s>>>(p, v, in, rounds); break;
        case 2: wf_tail<1, false><<<grid, 128, 0, s>>>(p, v, in, rounds); break;
        case 3: wf_tail<1, true><<<grid, 128, 0, s>>>(p, v, in, rounds); break;
        case 4: wf_tail<2, false><<<grid, 128, 0, s>>>(p, v, in, rounds); break;
        default: wf_tail<2, true><<<grid, 128, 0, s>>>(p, v, in, rounds); break;
    }
    return cudaGetLastError();
}

// The replay form (VOL_MIS with alpha materials): in | 2 shades the resume queue.
cudaError_t launch_shade_replay(const Params& p, const WfView& v, int in, int grid, int block, cudaStream_t s) {
    if (p.flags & F_ENVMAP) wf_shade<2, true, true, false, 1, true><<<grid, block, 0, s>>>(p, v, in, RenderWork{}, AdjView{});
    else wf_shade<2, false, true, false, 1, true><<<grid, block, 0, s>>>(p, v, in, RenderWork{}, AdjView{});
    return cudaGetLastError();
}

// The plain surface shade (no media, no environment map, deferred shadow
// rays) in three register budgets: unbounded, 80 (6 blocks) and 64 (8).
template <bool BATCH = false, bool ENV = false>
cudaError_t launch_shade_plain(const Params& p, const WfView& v, int in, int variant, const int grids[3], int block,
                               cudaStream_t s) {
    const RenderWork w{};
    const AdjView a{};
    switch (variant) {
        case 1: wf_shade<0, ENV, false, false, 6, false, BATCH><<<grids[1], block, 0, s>>>(p, v, in, w, a); break;
        case 2: wf_shade<0, ENV, false, false, 8, false, BATCH><<<grids[2], block, 0, s>>>(p, v, in, w, a); break;
        default: wf_shade<0, ENV, false, false, 1, false, BATCH><<<grids[0], block, 0, s>>>(p, v, in, w, a); break;
    }
    return cudaGetLastError();
}

cudaError_t shade_dispatch(const Params& p, const WfView& v, int in, int grid, int block, cudaStream_t s,
                           int variant = 0, const int* grids = nullptr) {
    const int medium = (p.flags & F_MEDIUM) ? ((p.flags & F_VOL_MIS) ? 2 : 1) : 0;
    const bool env = (p.flags & F_ENVMAP) != 0;
    // AnyHit draws random numbers for alpha-tested materials without media
    // (anyhit.glsl:118-141), and EvalTransmittance (VOL_MIS) at blended
    // materials: those keep the shadow rays inline so every path draws the
    // reference's sequence
    const bool inl = (p.flags & F_ALPHA_TEST) && medium != 1;
    switch ((medium * 2 + (env ? 1 : 0)) * 2 + (inl ? 1 : 0)) {
        case 0: {
            const int g3[3] = {grid, grids ? grids[1] : grid, grids ? grids[2] : grid};
            return launch_shade_plain(p, v, in, grids ? variant : 0, g3, block, s);
        }
        case 1: return launch_shade<0, false, true>(p, v, in, grid, block, s);
        case 2: return launch_shade<0, true, false>(p, v, in, grid, block, s);
        case 3: return launch_shade<0, true, true>(p, v, in, grid, block, s);
        case 4: return launch_shade<1, false, false>(p, v, in, grid, block, s);
        case 5: return launch_shade<1, false, true>(p, v, in, grid, block, s);
        case 6: return launch_shade<1, true, false>(p, v, in, grid, block, s);
        case 7: return launch_shade<1, true, true>(p, v, in, grid, block, s);
        case 8: return launch_shade<2, false, false>(p, v, in, grid, block, s);
        case 9: return launch_shade<2, false, true>(p, v, in, grid, block, s);
        case 10: return launch_shade<2, true, false>(p, v, in, grid, block, s);
        default: return launch_shade<2, true, true>(p, v, in, grid, block, s);
    }
}

}  // namespace

size_t wavefront_bytes_per_path() { return 17 * 16 + 3 * sizeof(int); }

cudaError_t wavefront_alloc(WavefrontBuffers& wb, int capacity) {
    wavefront_free(wb);
    wb.capacity = capacity;
    const size_t n = (size_t)capacity;
    float4** f4[] = {&wb.o, &wb.d, &wb.T, &wb.L, &wb.med, &wb.h0, &wb.h2, &wb.so, &wb.sd0, &wb.sd1,
                     &wb.sc0, &wb.sc1, &wb.sT, &wb.rad};
    for (float4** p : f4) {
        cudaError_t e = cudaMalloc((void**)p, n * sizeof(float4));
        if (e != cudaSuccess) { wavefront_free(wb); return e; }
    }
    cudaError_t e;
    if ((e = cudaMalloc((void**)&wb.rng, n * sizeof(uint4))) != cudaSuccess ||
        (e = cudaMalloc((void**)&wb.misc, n * sizeof(int4))) != cudaSuccess ||
        (e = cudaMalloc((void**)&wb.h1, n * sizeof(int4))) != cudaSuccess ||
        (e = cudaMalloc((void**)&wb.q[0], n * sizeof(int))) != cudaSuccess ||
        (e = cudaMalloc((void**)&wb.q[1], n * sizeof(int))) != cudaSuccess ||
        (e = cudaMalloc((void**)&wb.qs, n * sizeof(int))) != cudaSuccess ||
        (e = cudaMalloc((void**)&wb.counts, 8 * sizeof(int))) != cudaSuccess) {
        wavefront_free(wb);
        return e;
    }
    return cudaSuccess;
}

bool wavefront_needs_replay(uint32_t flags) {
    return (flags & F_MEDIUM) && (flags & F_VOL_MIS) && (flags & F_ALPHA_TEST);
}

cudaError_t wavefront_alloc_replay(WavefrontBuffers& wb) {
    if (wb.tr0 || wb.fixed) return cudaSuccess;
    const size_t n = (size_t)wb.capacity;
    cudaError_t e;
    if ((e = cudaMalloc((void**)&wb.tr0, n * sizeof(float4))) != cudaSuccess ||
        (e = cudaMalloc((void**)&wb.tr1, n * sizeof(float4))) != cudaSuccess ||
        (e = cudaMalloc((void**)&wb.trng0, n * sizeof(uint4))) != cudaSuccess ||
        (e = cudaMalloc((void**)&wb.trng1, n * sizeof(uint4))) != cudaSuccess ||
        (e = cudaMalloc((void**)&wb.qr, n * sizeof(int))) != cudaSuccess) {
        void* ptrs[] = {wb.tr0, wb.tr1, wb.trng0, wb.trng1, wb.qr};
        for (void* p : ptrs)
            if (p) cudaFree(p);
        wb.tr0 = wb.tr1 = nullptr;
        wb.trng0 = wb.trng1 = nullptr;
        wb.qr = nullptr;
        return e;
    }
    return cudaSuccess;
}

void wavefront_free(WavefrontBuffers& wb) {
    if (wb.fixed) {  // the static scratch is not freed
        if (wb.graph_exec) cudaGraphExecDestroy(wb.graph_exec);
        wb = WavefrontBuffers{};
        return;
    }
    void* ptrs[] = {wb.o, wb.d, wb.T, wb.L, wb.med, wb.h0, wb.h2, wb.so, wb.sd0, wb.sd1, wb.sc0, wb.sc1, wb.sT,
                    wb.rad, wb.rng, wb.misc, wb.h1, wb.q[0], wb.q[1], wb.qs, wb.counts,
                    wb.tr0, wb.tr1, wb.trng0, wb.trng1, wb.qr};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (wb.graph_exec) cudaGraphExecDestroy(wb.graph_exec);
    wb = WavefrontBuffers{};
}

// Fixed scratch: 21 float4-sized arrays and 4 int arrays of
// kFixedScratchPaths entries, then 8 counters, each array 256-byte aligned
// (5.5 MiB).  Nothing in it needs to start at zero: each batch's first
// kernel (wf_generate) writes the counters and queue entries it reads.
namespace {
constexpr size_t kFixedVec = (size_t)kFixedScratchPaths * 16;
constexpr size_t kFixedInt = (size_t)kFixedScratchPaths * 4;
constexpr size_t kFixedBytes = 21 * kFixedVec + 4 * kFixedInt + 256;
static_assert(kFixedVec % 256 == 0 && kFixedInt % 256 == 0, "scratch arrays stay 256-byte aligned");
constexpr int kFixedMaxDevices = 64;
std::atomic<char*> g_fixed_addr[kFixedMaxDevices];
}  // namespace

static __device__ __align__(256) unsigned char g_fixed_scratch[kFixedBytes];

cudaError_t wavefront_fixed_buffers(WavefrontBuffers& wb) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kFixedMaxDevices) return cudaErrorInvalidDevice;
    char* base = g_fixed_addr[dev].load(std::memory_order_acquire);
    if (!base) {
        void* addr = nullptr;
        if ((e = cudaGetSymbolAddress(&addr, g_fixed_scratch)) != cudaSuccess) return e;
        base = static_cast<char*>(addr);
        g_fixed_addr[dev].store(base, std::memory_order_release);
    }
    wb = WavefrontBuffers{};
    wb.capacity = kFixedScratchPaths;
    wb.fixed = true;
    float4** f4[] = {&wb.o, &wb.d, &wb.T, &wb.L, &wb.med, &wb.h0, &wb.h2, &wb.so, &wb.sd0, &wb.sd1,
                     &wb.sc0, &wb.sc1, &wb.sT, &wb.rad, &wb.tr0, &wb.tr1};
    size_t off = 0;
    for (float4** q : f4) {
        *q = reinterpret_cast<float4*>(base + off);
        off += kFixedVec;
    }
    wb.rng = reinterpret_cast<uint4*>(base + off);
    off += kFixedVec;
    wb.misc = reinterpret_cast<int4*>(base + off);
    off += kFixedVec;
    wb.h1 = reinterpret_cast<int4*>(base + off);
    off += kFixedVec;
    wb.trng0 = reinterpret_cast<uint4*>(base + off);
    off += kFixedVec;
    wb.trng1 = reinterpret_cast<uint4*>(base + off);
    off += kFixedVec;
    int** i1[] = {&wb.q[0], &wb.q[1], &wb.qs, &wb.qr};
    for (int** q : i1) {
        *q = reinterpret_cast<int*>(base + off);
        off += kFixedInt;
    }
    wb.counts = reinterpret_cast<int*>(base + off);
    return cudaSuccess;
}

// The traversal kernels come in variants: minimum resident blocks per SM
// (register budget 64 or 80 per thread) x scalar or packed node test.
template <int MINB, bool PACKED> static const void* extend_fn() { return (const void*)wf_extend<MINB, PACKED>; }
template <bool ADJ, int MINB, bool PACKED> static const void* shadow_fn() {
    return (const void*)wf_shadow<ADJ, MINB, PACKED>;
}

static cudaError_t launch_transmit_replay(const Params& p, const WfView& v, const WavefrontTuning& t, cudaStream_t s) {
    const int g = t.replay_grid_v[t.shadow_variant];
    const int b = t.shadow_block, r = t.shadow_refill, m = t.min_tris;
    switch (t.shadow_variant) {
        case 1: wf_transmit_replay<8, true><<<g, b, 0, s>>>(p, v, r, m); break;
        case 2: wf_transmit_replay<6, false><<<g, b, 0, s>>>(p, v, r, m); break;
        case 3: wf_transmit_replay<6, true><<<g, b, 0, s>>>(p, v, r, m); break;
        default: wf_transmit_replay<8, false><<<g, b, 0, s>>>(p, v, r, m); break;
    }
    return cudaGetLastError();
}

template <bool BATCH = false>
static cudaError_t launch_extend(const Params& p, const WfView& v, int in, const WavefrontTuning& t, cudaStream_t s) {
    // the first round's camera rays (coherent 8 x 4 blocks) may take their own
    // kernel variant, refill threshold and triangle-step quorum
    const bool first = (in & kFirstRound) != 0;
    const int var = first && t.extend_variant_first >= 0 ? t.extend_variant_first : t.extend_variant;
    const int g = t.extend_grid_v[var];
    const int b = t.extend_block;
    const int r = first && t.extend_refill_first > 0 ? t.extend_refill_first : t.extend_refill;
    const int m = first && t.min_tris_first >= 0 ? t.min_tris_first : t.min_tris;
    // a batch takes the direct form when every job enters directly (p.direct)
    if (p.direct) {
        switch (var) {
            case 1: wf_extend<8, true, BATCH, true><<<g, b, 0, s>>>(p, v, in, r, m); break;
            case 2: wf_extend<6, false, BATCH, true><<<g, b, 0, s>>>(p, v, in, r, m); break;
            case 3: wf_extend<6, true, BATCH, true><<<g, b, 0, s>>>(p, v, in, r, m); break;
            default: wf_extend<8, false, BATCH, true><<<g, b, 0, s>>>(p, v, in, r, m); break;
        }
        return cudaGetLastError();
    }
    switch (var) {
        case 1: wf_extend<8, true, BATCH><<<g, b, 0, s>>>(p, v, in, r, m); break;
        case 2: wf_extend<6, false, BATCH><<<g, b, 0, s>>>(p, v, in, r, m); break;
        case 3: wf_extend<6, true, BATCH><<<g, b, 0, s>>>(p, v, in, r, m); break;
        default: wf_extend<8, false, BATCH><<<g, b, 0, s>>>(p, v, in, r, m); break;
    }
    return cudaGetLastError();
}

template <bool ADJ, bool BATCH = false>
static cudaError_t launch_shadow(const Params& p, const WfView& v, const WavefrontTuning& t, const AdjView& A,
                                 size_t smem, cudaStream_t s, bool first = false) {
    // the first round's shadow rays (from the camera rays' hits) may take
    // their own refill threshold and triangle-step quorum
    const int b = t.shadow_block;
    const int r = first && t.shadow_refill_first > 0 ? t.shadow_refill_first : t.shadow_refill;
    const int m = first && t.min_tris_shadow_first >= 0 ? t.min_tris_shadow_first : t.min_tris;
    if (!ADJ && transmit_deferred(p.flags)) {
        const int g = t.transmit_grid_v[t.shadow_variant];
        switch (t.shadow_variant) {
            case 1: wf_transmit<8, true><<<g, b, 0, s>>>(p, v, r, m); break;
            case 2: wf_transmit<6, false><<<g, b, 0, s>>>(p, v, r, m); break;
            case 3: wf_transmit<6, true><<<g, b, 0, s>>>(p, v, r, m); break;
            default: wf_transmit<8, false><<<g, b, 0, s>>>(p, v, r, m); break;
        }
        return cudaGetLastError();
    }
    const int g = t.shadow_grid_v[t.shadow_variant];
    if (!ADJ && p.direct) {
        switch (t.shadow_variant) {
            case 1: wf_shadow<false, 8, true, BATCH, true><<<g, b, smem, s>>>(p, v, r, m, A); break;
            case 2: wf_shadow<false, 6, false, BATCH, true><<<g, b, smem, s>>>(p, v, r, m, A); break;
            case 3: wf_shadow<false, 6, true, BATCH, true><<<g, b, smem, s>>>(p, v, r, m, A); break;
            default: wf_shadow<false, 8, false, BATCH, true><<<g, b, smem, s>>>(p, v, r, m, A); break;
        }
        return cudaGetLastError();
    }
    switch (t.shadow_variant) {
        case 1: wf_shadow<ADJ, 8, true, BATCH><<<g, b, smem, s>>>(p, v, r, m, A); break;
        case 2: wf_shadow<ADJ, 6, false, BATCH><<<g, b, smem, s>>>(p, v, r, m, A); break;
        case 3: wf_shadow<ADJ, 6, true, BATCH><<<g, b, smem, s>>>(p, v, r, m, A); break;
        default: wf_shadow<ADJ, 8, false, BATCH><<<g, b, smem, s>>>(p, v, r, m, A); break;
    }
    return cudaGetLastError();
}

cudaError_t StageTimer::mark(cudaStream_t s) {
    if (used >= pool.size()) {
        cudaEvent_t e;
        cudaError_t r = cudaEventCreate(&e);
        if (r != cudaSuccess) return r;
        pool.push_back(e);
    }
    return cudaEventRecord(pool[used++], s);
}

cudaError_t StageTimer::summarise(float ms[STAGE_COUNT], int launches[STAGE_COUNT]) const {
    for (int k = 0; k < STAGE_COUNT; ++k) {
        ms[k] = 0.0f;
        launches[k] = 0;
    }
    for (size_t i = 0; i < kinds.size() && 2 * i + 1 < used; ++i) {
        cudaError_t e = cudaEventSynchronize(pool[2 * i + 1]);
        if (e != cudaSuccess) return e;
        float t = 0.0f;
        if ((e = cudaEventElapsedTime(&t, pool[2 * i], pool[2 * i + 1])) != cudaSuccess) return e;
        ms[kinds[i]] += t;
        launches[kinds[i]] += 1;
    }
    return cudaSuccess;
}

void StageTimer::release() {
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
    pool.clear();
    reset();
}

// A launch bracketed by timer events (when timing).
template <class F> static cudaError_t timed(StageTimer* timer, int kind, cudaStream_t s, F&& launch) {
    cudaError_t e;
    if (timer && (e = timer->mark(s)) != cudaSuccess) return e;
    if ((e = launch()) != cudaSuccess) return e;
    if (timer) {
        if ((e = timer->mark(s)) != cudaSuccess) return e;
        timer->kinds.push_back(kind);
    }
    return cudaSuccess;
}

// Enqueue one batch: passes [first_pass, first_pass + npass) of the pixels of W.
// One bounce of a batch on queue `in`: extend, shade, then the shadow stage
// (any-hit or deferred transmittance), or in the replay form (VOL_MIS with
// alpha materials) per transmittance query site: trace the suspended
// queries, shade their paths again (counters: [6] resume queue, [2]
// transmittance queue, [4] / [5] fetch counters).  Adds its kernel launches
// to *nl.
constexpr int kExtraRounds = 4;

static cudaError_t enqueue_bounce(const Params& p, const WfView& v, int in, const WavefrontTuning& t, cudaStream_t s,
                                  StageTimer* timer, int* nl, bool first) {
    cudaError_t e;
    const int sin = with_first_round(in, first);  // the first round's launches read no queue
    if ((e = timed(timer, STAGE_EXTEND, s, [&] { return launch_extend(p, v, sin, t, s); })) != cudaSuccess) return e;
    if (wavefront_needs_replay(p.flags)) {
        const int sites = std::max(1, ((p.flags & F_ENVMAP) ? 1 : 0) + ((p.flags & F_LIGHTS) ? 1 : 0));
        if ((e = timed(timer, STAGE_SHADE, s,
                       [&] { return launch_shade_replay(p, v, sin, t.shade_grid, t.shade_block, s); })) != cudaSuccess)
            return e;
        for (int k = 0; k < sites; ++k) {
            if ((e = timed(timer, STAGE_SHADOW, s, [&] {
                     cudaError_t ee = cudaMemsetAsync(v.counts + 6, 0, sizeof(int), s);
                     return ee != cudaSuccess ? ee : launch_transmit_replay(p, v, t, s);
                 })) != cudaSuccess)
                return e;
            if ((e = timed(timer, STAGE_SHADE, s, [&] {
                     cudaError_t ee = cudaMemsetAsync(v.counts + 2, 0, 4 * sizeof(int), s);
                     return ee != cudaSuccess ? ee : launch_shade_replay(p, v, sin | 2, t.shade_grid, t.shade_block, s);
                 })) != cudaSuccess)
                return e;
        }
        *nl += 2 + 2 * sites;
        return cudaSuccess;
    }
    if ((e = timed(timer, STAGE_SHADE, s,
                   [&] {
                       return shade_dispatch(p, v, sin, t.shade_grid, t.shade_block, s,
                                             first && t.shade_variant_first >= 0 ? t.shade_variant_first
                                                                                 : t.shade_variant,
                                             t.shade_grid_v);
                   })) != cudaSuccess)
        return e;
    if ((e = timed(timer, STAGE_SHADOW, s, [&] { return launch_shadow<false>(p, v, t, AdjView{}, 0, s, first); })) !=
        cudaSuccess)
        return e;
    *nl += 3;
    return cudaSuccess;
}

static cudaError_t enqueue_batch(const Params& p, const RenderWork& W, const WavefrontBuffers& wb, int first_pass,
                                 int npass, int iterations, const WavefrontTuning& t, cudaStream_t s,
                                 StageTimer* timer, int* nl) {
    const WfView v = view_of(wb);
    const int n = W.w * W.h * npass;
    const int gen_grid = std::min((n + 255) / 256, t.resident_blocks_256);
    cudaError_t e = timed(timer, STAGE_GENERATE, s, [&] {
        wf_generate<false><<<gen_grid, 256, 0, s>>>(p, W, v, first_pass, npass);
        return cudaGetLastError();
    });
    if (e != cudaSuccess) return e;
    *nl += 1;
    // max_depth+1 rounds finish every path unless alpha pass-through keeps
    // some at the same depth: those get kExtraRounds more wavefront rounds,
    // then the tail kernel finishes the rest
    const bool may_linger = (p.flags & F_ALPHA_TEST) != 0;
    const int rounds = iterations + (may_linger ? kExtraRounds : 0);
    for (int it = 0; it < rounds; ++it)
        if ((e = enqueue_bounce(p, v, it & 1, t, s, timer, nl, it == 0)) != cudaSuccess) return e;
    if (may_linger) {
        if ((e = timed(timer, STAGE_SHADE, s, [&] { return launch_tail(p, v, rounds & 1, rounds, t.shade_grid, s); })) !=
            cudaSuccess)
            return e;
        *nl += 1;
    }
    return cudaSuccess;
}

cudaError_t launch_wavefront(const Params& p, const RenderWork& W, WavefrontBuffers& wb, const WavefrontTuning& t,
                             bool use_graph, cudaStream_t s, int* launches, StageTimer* timer) {
    if (timer) use_graph = false;
    int dummy = 0;
    int& nl = launches ? *launches : dummy;
    nl = 0;
    if (W.w <= 0 || W.h <= 0 || W.num_passes <= 0) return cudaSuccess;
    const int npix = W.w * W.h;
    const int per_batch = std::max(1, std::min(W.num_passes, wb.capacity / npix));
    const int iterations = p.max_depth + 1;
    if (wavefront_needs_replay(p.flags)) {
        cudaError_t e = wavefront_alloc_replay(wb);
        if (e != cudaSuccess) return e;
    }
    const WfView v = view_of(wb);
    for (int first = W.first_pass; first < W.first_pass + W.num_passes; first += per_batch) {
        const int npass = std::min(per_batch, W.first_pass + W.num_passes - first);
        cudaError_t e;
        if (use_graph) {
            cudaGraph_t g = nullptr;
            if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
            int cl = 0;
            cudaError_t ce = enqueue_batch(p, W, wb, first, npass, iterations, t, s, nullptr, &cl);
            e = cudaStreamEndCapture(s, &g);
            if (ce != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return ce;
            }
            if (e != cudaSuccess) return e;
            bool updated = false;
            if (wb.graph_exec) {
                cudaGraphExecUpdateResultInfo info;
                updated = cudaGraphExecUpdate(wb.graph_exec, g, &info) == cudaSuccess;
                if (!updated) {
                    cudaGetLastError();
                    cudaGraphExecDestroy(wb.graph_exec);
                    wb.graph_exec = nullptr;
                }
            }
            if (!updated) {
                e = cudaGraphInstantiate(&wb.graph_exec, g, 0);
                if (e != cudaSuccess) {
                    cudaGraphDestroy(g);
                    wb.graph_exec = nullptr;
                    return e;
                }
            }
            cudaGraphDestroy(g);
            if ((e = cudaGraphLaunch(wb.graph_exec, s)) != cudaSuccess) return e;
            nl += cl;
        } else if ((e = enqueue_batch(p, W, wb, first, npass, iterations, t, s, timer, &nl)) != cudaSuccess) {
            return e;
        }
        const int res_grid = std::min((npix + 255) / 256, t.resident_blocks_256);
        if ((e = timed(timer, STAGE_RESOLVE, s, [&] {
                 wf_resolve<<<res_grid, 256, 0, s>>>(p, W, v, npass);
                 return cudaGetLastError();
             })) != cudaSuccess)
            return e;
        nl += 1;
    }
    return cudaSuccess;
}

cudaError_t launch_adjoint(const Params& p, const RenderWork& W, WavefrontBuffers& wb, const WavefrontTuning& t,
                           const AdjView& A, bool run_forward, cudaStream_t s, int* launches) {
    int dummy = 0;
    int& nl = launches ? *launches : dummy;
    nl = 0;
    if (W.w <= 0 || W.h <= 0 || W.num_passes <= 0) return cudaSuccess;
    if ((long)W.w * W.h * W.num_passes > wb.capacity) return cudaErrorInvalidValue;
    const int iterations = p.max_depth + 1;
    cudaError_t e;
    if (run_forward) {
        if ((e = enqueue_batch(p, W, wb, W.first_pass, W.num_passes, iterations, t, s, nullptr, &nl)) != cudaSuccess)
            return e;
    }
    const WfView v = view_of(wb);
    const int n = W.w * W.h * W.num_passes;
    const int gen_grid = std::min((n + 255) / 256, t.resident_blocks_256);
    const size_t smem = A.shared ? sizeof(float) * (size_t)A.grad_size : 0;
    wf_generate<false><<<gen_grid, 256, 0, s>>>(p, W, v, W.first_pass, W.num_passes);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    for (int it = 0; it < iterations; ++it) {
        const int in = it & 1;
        if ((e = launch_extend(p, v, with_first_round(in, it == 0), t, s)) != cudaSuccess) return e;
        wf_shade<0, false, false, true><<<t.shade_grid, t.shade_block, smem, s>>>(p, v, with_first_round(in, it == 0),
                                                                                  W, A);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = launch_shadow<true>(p, v, t, A, smem, s, it == 0)) != cudaSuccess) return e;
    }
    nl += 1 + 3 * iterations;
    return cudaSuccess;
}

// The shade form of a batch: media without volume MIS (MEDIUM 1) when a job
// has a medium, the environment-map code when a job has a map, shadow rays
// traced inline when a job has alpha-tested materials and no medium (its
// AnyHit draws random numbers); each path takes its job's own flags at run
// time within that form.
template <int MEDIUM, bool ENV, bool INLINE>
static cudaError_t batch_shade(const Params& p, const WfView& v, int in, const WavefrontTuning& t, cudaStream_t s) {
    if (MEDIUM == 0 && !INLINE) {
        const int g3[3] = {t.shade_grid, t.shade_grid_v[1], t.shade_grid_v[2]};
        const int var = (in & kFirstRound) && t.shade_variant_first >= 0 ? t.shade_variant_first : t.shade_variant;
        return launch_shade_plain<true, ENV>(p, v, in, var, g3, t.shade_block, s);
    }
    wf_shade<MEDIUM, ENV, INLINE, false, 1, false, true><<<t.shade_grid, t.shade_block, 0, s>>>(p, v, in, RenderWork{},
                                                                                             AdjView{});
    return cudaGetLastError();
}
static cudaError_t batch_shade_dispatch(const Params& p, const WfView& v, int in, const WavefrontTuning& t,
                                        bool inline_shadows, cudaStream_t s) {
    const int medium = (p.flags & F_MEDIUM) ? 1 : 0;
    const bool env = (p.flags & F_ENVMAP) != 0;
    switch (medium * 4 + (env ? 2 : 0) + (inline_shadows ? 1 : 0)) {
        case 0: return batch_shade<0, false, false>(p, v, in, t, s);
        case 1: return batch_shade<0, false, true>(p, v, in, t, s);
        case 2: return batch_shade<0, true, false>(p, v, in, t, s);
        case 3: return batch_shade<0, true, true>(p, v, in, t, s);
        case 4: return batch_shade<1, false, false>(p, v, in, t, s);
        case 5: return batch_shade<1, false, true>(p, v, in, t, s);
        case 6: return batch_shade<1, true, false>(p, v, in, t, s);
        default: return batch_shade<1, true, true>(p, v, in, t, s);
    }
}
static cudaError_t batch_tail(const Params& p, const WfView& v, int in, int rounds, int grid, cudaStream_t s) {
    const int medium = (p.flags & F_MEDIUM) ? 1 : 0;
    const bool env = (p.flags & F_ENVMAP) != 0;
    switch (medium * 2 + (env ? 1 : 0)) {
        case 0: wf_tail<0, false, true><<<grid, 128, 0, s>>>(p, v, in, rounds); break;
        case 1: wf_tail<0, true, true><<<grid, 128, 0, s>>>(p, v, in, rounds); break;
        case 2: wf_tail<1, false, true><<<grid, 128, 0, s>>>(p, v, in, rounds); break;
        default: wf_tail<1, true, true><<<grid, 128, 0, s>>>(p, v, in, rounds); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_batch(const Params& p, const BatchChunk* chunks, int num_chunks, WavefrontBuffers& wb,
                         const WavefrontTuning& t, cudaStream_t s, unsigned long long* start_stamp, int* launches,
                         bool inline_shadows) {
    int dummy = 0;
    int& nl = launches ? *launches : dummy;
    nl = 0;
    const WfView v = view_of(wb);
    cudaError_t e;
    wf_batch_stamp<<<1, 1, 0, s>>>(start_stamp);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    ++nl;
    for (int c = 0; c < num_chunks; ++c) {
        const BatchChunk& ch = chunks[c];
        if (ch.paths <= 0) continue;
        if (ch.paths > wb.capacity) return cudaErrorInvalidValue;
        Params pc = p;
        pc.jobs = p.jobs + ch.entry_begin;
        pc.num_jobs = ch.entry_count;
        const int gen_grid = std::min((ch.paths + 255) / 256, t.resident_blocks_256);
        wf_generate<true><<<gen_grid, 256, 0, s>>>(pc, RenderWork{}, v, 0, 0, ch.paths);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        // alpha pass-through keeps a path at the same depth: as for a single
        // scene (enqueue_batch), more rounds and then the tail kernel
        const bool linger = (p.flags & F_ALPHA_TEST) != 0;
        const int rounds = ch.max_depth + 1 + (linger ? kExtraRounds : 0);
        for (int it = 0; it < rounds; ++it) {
            const int in = it & 1;
            const int sin = with_first_round(in, it == 0);
            if ((e = launch_extend<true>(pc, v, sin, t, s)) != cudaSuccess) return e;
            if ((e = batch_shade_dispatch(pc, v, sin, t, inline_shadows, s)) != cudaSuccess) return e;
            if ((e = launch_shadow<false, true>(pc, v, t, AdjView{}, 0, s, it == 0)) != cudaSuccess) return e;
        }
        if (linger) {
            if ((e = batch_tail(pc, v, rounds & 1, rounds, t.shade_grid, s)) != cudaSuccess) return e;
            ++nl;
        }
        const int res_grid = std::min((ch.pixels + 255) / 256, t.resident_blocks_256);
        wf_resolve_batch<<<res_grid, 256, 0, s>>>(pc, v, ch.pixels);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        nl += 2 + 3 * rounds;
    }
    return cudaSuccess;
}

cudaError_t wavefront_default_tuning(WavefrontTuning& t, int block) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    int b_ext = 0, b_shade = 0, b_shadow = 0, b256 = 0;
    const void* ext[4] = {extend_fn<8, false>(), extend_fn<8, true>(), extend_fn<6, false>(), extend_fn<6, true>()};
    const void* shd[4] = {shadow_fn<false, 8, false>(), shadow_fn<false, 8, true>(), shadow_fn<false, 6, false>(),
                          shadow_fn<false, 6, true>()};
    for (int k = 0; k < 4; ++k) {
        int be = 0, bs = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&be, ext[k], block, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bs, shd[k], block, 0);
        t.extend_grid_v[k] = sms * std::max(1, be);
        t.shadow_grid_v[k] = sms * std::max(1, bs);
    }
    const void* trn[4] = {(const void*)wf_transmit<8, false>, (const void*)wf_transmit<8, true>,
                          (const void*)wf_transmit<6, false>, (const void*)wf_transmit<6, true>};
    const void* rpl[4] = {(const void*)wf_transmit_replay<8, false>, (const void*)wf_transmit_replay<8, true>,
                          (const void*)wf_transmit_replay<6, false>, (const void*)wf_transmit_replay<6, true>};
    for (int k = 0; k < 4; ++k) {
        int bt = 0, br = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bt, trn[k], block, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&br, rpl[k], block, 0);
        t.transmit_grid_v[k] = sms * std::max(1, bt);
        t.replay_grid_v[k] = sms * std::max(1, br);
    }
    b_ext = t.extend_grid_v[0] / sms;
    b_shadow = t.shadow_grid_v[0] / sms;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b_shade, wf_shade<0, false, false>, block, 0);
    {
        int b6 = 0, b8 = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b6, wf_shade<0, false, false, false, 6>, block, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b8, wf_shade<0, false, false, false, 8>, block, 0);
        t.shade_grid_v[0] = sms * std::max(1, b_shade);
        t.shade_grid_v[1] = sms * std::max(1, b6);
        t.shade_grid_v[2] = sms * std::max(1, b8);
    }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b256, wf_resolve, 256, 0);
    t.extend_block = t.shade_block = t.shadow_block = block;
    t.extend_grid = sms * std::max(1, b_ext);
    t.shade_grid = sms * std::max(1, b_shade);
    t.shadow_grid = sms * std::max(1, b_shadow);
    t.resident_blocks_256 = sms * std::max(1, b256);
    if (const char* r = std::getenv("PT_WAVEFRONT_REFILL")) {
        const int v = std::atoi(r);
        if (v >= 1 && v <= 32) t.extend_refill = t.shadow_refill = v;
    }
    if (const char* r = std::getenv("PT_WAVEFRONT_MIN_TRIS")) {
        const int v = std::atoi(r);
        if (v >= 0 && v <= 32) t.min_tris = v;
    }
    if (const char* r = std::getenv("PT_WAVEFRONT_VARIANT")) {
        const int v = std::atoi(r);
        if (v >= 0 && v < 4) t.extend_variant = t.shadow_variant = v;
    }
    if (const char* r = std::getenv("PT_WAVEFRONT_VARIANT_FIRST")) {
        const int v = std::atoi(r);
        if (v >= 0 && v < 4) t.extend_variant_first = v;
    }
    if (const char* r = std::getenv("PT_WAVEFRONT_SHADE_VARIANT_FIRST")) {
        const int v = std::atoi(r);
        if (v >= 0 && v < 3) t.shade_variant_first = v;
    }
    if (const char* r = std::getenv("PT_WAVEFRONT_REFILL_FIRST")) {
        const int v = std::atoi(r);
        if (v >= 1 && v <= 32) t.extend_refill_first = v;
    }
    if (const char* r = std::getenv("PT_WAVEFRONT_MIN_TRIS_FIRST")) {
        const int v = std::atoi(r);
        if (v >= 0 && v <= 32) t.min_tris_first = v;
    }
    if (const char* r = std::getenv("PT_WAVEFRONT_SHADOW_REFILL_FIRST")) {
        const int v = std::atoi(r);
        if (v >= 1 && v <= 32) t.shadow_refill_first = v;
    }
    if (const char* r = std::getenv("PT_WAVEFRONT_SHADOW_MIN_TRIS_FIRST")) {
        const int v = std::atoi(r);
        if (v >= 0 && v <= 32) t.min_tris_shadow_first = v;
    }
    if (const char* r = std::getenv("PT_WAVEFRONT_SHADE_VARIANT")) {
        const int v = std::atoi(r);
        if (v >= 0 && v < 3) t.shade_variant = v;
    }
    return cudaSuccess;
}

}  // namespace ptgb

// Host copies of the path order (tests: a bijection for any rectangle).
extern "C" void ptgb_slot_pixel(int s, int w, int h, int* x, int* y) { ptgb::slot_pixel(s, w, h, *x, *y); }
extern "C" int ptgb_pixel_slot(int x, int y, int w, int h) { return ptgb::pixel_slot(x, y, w, h); }

