"""Throughput benchmark of the GB300 path tracer.

Default workload: the 1M-triangle scene (geodesic icosphere, 1,048,820
triangles, 3-octave value-noise displacement, 16 Disney materials, one sphere
light), 1920x1080, 16 spp, max depth 8, FP32.  One step = one 16-spp frame
(16 sample passes in one launch).  Metric: Mrays/s, rays = executed
closest-hit queries + shadow queries (any-hit calls and transmittance
segments), counted on the device.

  value      device-resident: per-step CUDA events on the launching stream
             around the render launch; the L2 is flushed (a 512 MiB write)
             before every timed step.
  e2e        through the public C ABI with host buffers, wall clock per step:
             pt_set_camera + pt_render_passes + pt_get_output (tonemapped
             RGBA8 image copied to pinned host memory).
  adjoint    the differentiable-materials workload (1M-triangle icosphere
             in 32 materials + 4 lights, 512x512, 16 spp, depth 6): device
             time of pt_render_adjoint (gradient of 375 parameters, reusing
             the forward paths) over that of the forward render.
  batch      64 jobs of uneven size (icosphere scenes of 10k-1M triangles,
             128^2-1024^2, 1-64 spp, depth 4-12) in one pt_batch_render per
             step: aggregate Mrays/s from the library's events around the
             batch, p50/p99 of the jobs' completion times (device global
             timer), and the same jobs rendered one after another.
  compare    the megakernel on the same frame and timing rules (it gives the
             same accumulation up to last-bit rounding, so equal RMSE): the
             wavefront / megakernel ratio.
  roofline   HBM, for the dominant kernel (wf_extend on this workload): its
             algorithmic bytes (36 B per node visit + 60 B per triangle test
             + 176 B per triangle hit of a closest-hit query, counted by the
             oracle with a tmax-culled traversal of the reference's binary
             BVH on a row sample) x the queries of its launches / its own
             launch durations, taken with CUDA events around every launch on
             the launching stream in --stage-steps extra frames; against
             MEASURED_PEAKS.json.  traffic: DRAM bytes per launch from an
             ncu capture of the same kernel, scaled by the launch's queries.
  cpu_baseline  the oracle (C++ restatement of the reference's shaders, the
             reference's traversal, FP32, OpenMP on all host cores) on a row
             sample of the same frame.

--impl reference times the CPU restatement of the reference (the reference's
GLSL cannot run without a graphics stack; its own source builds only where
the reference is present, not on the GPU machines).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "glsl-pathtracer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

METRIC = "Mrays/s @1080p depth8 1M tris: wavefront vs megakernel, equal RMSE; adjoint/fwd"
CONFIGS = {
    "icosphere_1m": dict(desc="icosphere 1,048,820 tris, 1920x1080, 16 spp, depth 8", freq=229, width=1920,
                         height=1080, spp=16, depth=8),
    "cornell": dict(desc="procedural Cornell box 256x256, 64 spp, depth 4", width=256, height=256, spp=64, depth=4),
    "instanced": dict(desc="10,000 instances of 5 x 50k-tri BLAS + IBL + volume, 1920x1080, 16 spp, depth 8",
                      width=1920, height=1080, spp=16, depth=8),
}


def make_scene(name, cfg, small=False):
    from pathtracer import scenes
    if name == "icosphere_1m":
        return scenes.icosphere_scene(freq=cfg["freq"] if not small else 40, width=cfg["width"], height=cfg["height"],
                                      max_depth=cfg["depth"])
    if name == "cornell":
        return scenes.cornell(cfg["width"], cfg["height"], max_depth=cfg["depth"])
    if name == "instanced":
        return scenes.instanced_scene(width=cfg["width"], height=cfg["height"], max_depth=cfg["depth"])
    raise KeyError(name)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# DRAM bytes per closest-hit query of wf_extend on the icosphere workload:
# dram__bytes_read.sum + dram__bytes_write.sum of all nine wf_extend launches
# of one ncu-captured 1-spp frame (the autotuned launch configuration) / the
# frame's 3.42 M closest-hit queries.  Traffic grows with the rays of a
# launch: path-state reads and writes, BVH misses in L2.
EXTEND_DRAM_BYTES_PER_RAY = {"icosphere_1m": 93.8}
# Warp-level instructions executed per closest-hit query by wf_extend on the
# same capture (smsp__inst_executed.sum of the nine launches / the frame's
# queries; camera rays take 166, the first bounce's rays about 290): the
# numerator of the instruction-issue roofline (4 warp instructions per cycle
# per SM).
EXTEND_WARP_INST_PER_RAY = {"icosphere_1m": 214.3}


def bytes_per_ray(scene, options, camera, row_step=64, passes=2):
    """Oracle work counts (tmax-culled traversal of the reference's binary
    BVH) on a row sample -> algorithmic bytes per ray query: all queries,
    closest-hit queries alone and any-hit queries alone."""
    import orc
    _, _, c = orc.render(scene, options, camera, 0, passes, row_step=row_step, cull=True)
    rays = c["closest"] + c["shadow"]
    b = (36.0 * c["nodes"] + 60.0 * c["tris"] + 176.0 * c["tri_hits"]) / max(rays, 1)
    nc, tc = c["nodes"] - c["nodes_any"], c["tris"] - c["tris_any"]
    b_closest = (36.0 * nc + 60.0 * tc + 176.0 * c["tri_hits"]) / max(c["closest"], 1)
    b_shadow = (36.0 * c["nodes_any"] + 60.0 * c["tris_any"]) / max(c["shadow"], 1)
    # FP32 work of a query: 12 FLOPs per slab test, two per interior node;
    # 27 per triangle test; 600 per shaded hit
    f = (24.0 * c["inner"] + 27.0 * c["tris"] + 600.0 * c["tri_hits"]) / max(rays, 1)
    return b, dict(nodes_per_ray=c["nodes"] / rays, tris_per_ray=c["tris"] / rays,
                   hits_per_ray=c["tri_hits"] / rays, inner_nodes_per_ray=c["inner"] / rays, rays=rays,
                   bytes_per_closest_ray=b_closest, bytes_per_shadow_ray=b_shadow, flops_per_ray=f)


def fp32_peak_tflops():
    """Nominal FP32 rate of the device: SMs x 128 FP32 lanes x 2 (FMA) x the
    maximum SM clock (MEASURED_PEAKS.json, else the device's own figure)."""
    import torch
    props = torch.cuda.get_device_properties(0)
    mhz = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            mhz = float(json.load(fh)["sm_max_mhz"])
    except Exception:
        pass
    if not mhz:
        mhz = float(getattr(props, "clock_rate", 2070000)) / 1000.0
    return props.multi_processor_count * 128 * 2 * mhz * 1e6 / 1e12, props.multi_processor_count, mhz


def cpu_baseline(scene, options, camera, spp, target_s=15.0):
    """The oracle on a row sample of the frame, all host threads."""
    import orc
    H = options.render_height
    ncores = os.cpu_count() or 1
    # calibrate on a thin sample, then size the sample for ~target_s seconds
    step = max(1, H // 8)
    t0 = time.perf_counter()
    _, _, c = orc.render(scene, options, camera, 0, spp, row_step=step)
    dt = time.perf_counter() - t0
    rows = max(1, len(range(0, H, step)))
    per_row = dt / rows
    want_rows = max(1, min(H, int(target_s / max(per_row, 1e-6))))
    step = max(1, H // want_rows)
    t0 = time.perf_counter()
    _, _, c = orc.render(scene, options, camera, 0, spp, row_step=step)
    dt = time.perf_counter() - t0
    rays = c["closest"] + c["shadow"]
    return {"value": rays / dt / 1e6, "unit": "Mrays/s", "cores": ncores, "kind": "port",
            "sample": f"every {step}th row of the {options.render_width}x{H} frame, {spp} spp, depth "
                      f"{options.max_depth} ({rays} rays in {dt:.1f} s; oracle FP32, OpenMP)"}, rays, dt


def run_reference(args, cfg, name):
    """--impl reference: the reference's algorithm restated on the CPU, timed
    on bounded row samples of the same frame; rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sd = make_scene(name, cfg)
    o = sd.render_options()
    cam = sd.pt_camera()
    import orc
    H = o.render_height
    ncores = os.cpu_count() or 1
    # at least 8 rows per host thread in every step, so that the dynamic
    # row schedule keeps all cores busy to the end of the step
    step = max(1, H // (8 * ncores))
    for _ in range(args.warmup):
        orc.render(sd, o, cam, 0, 1, row_step=H)  # one row
    tot_rays, tot_t = 0, 0.0
    for k in range(args.steps):
        t0 = time.perf_counter()
        _, _, c = orc.render(sd, o, cam, 0, cfg["spp"], row_start=k % step, row_step=step)
        tot_t += time.perf_counter() - t0
        tot_rays += c["closest"] + c["shadow"]
    v = tot_rays / tot_t / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * tot_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": cfg["desc"] + f"; each step renders every {step}th row"},
        "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": ncores, "kind": "port",
                         "sample": f"every {step}th row per step, {cfg['spp']} spp; the reference's shaders restated "
                                   "in C++ (its GLSL needs OpenGL, unavailable on this machine)"},
        "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def config_bench(name, steps, warmup, flush, peak):
    """Another workload of the survey on the same rules as the headline:
    autotuned wavefront, L2 flushed before each timed step, device time with
    CUDA events, then one stage-timed step for the dominant kernel's
    roofline (its algorithmic bytes per query from the oracle's counts)."""
    import torch
    from pathtracer import capi
    from pathtracer.renderer import GpuRenderer
    cfg = CONFIGS[name]
    sd = make_scene(name, cfg)
    spp = cfg["spp"]
    res = {"workload": cfg["desc"]}
    with GpuRenderer(sd) as r:
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        res["tuning"] = r.autotune(spp)
        for k in range(warmup):
            r.render_passes(k * spp, spp)
        ms, rays = [], 0
        for k in range(steps):
            flush.fill_(k & 0xFF)
            torch.cuda.synchronize()
            r.render_passes((warmup + k) * spp, spp)
            st = r.stats()
            if st["status"] != 0:
                raise RuntimeError(f"{name}: kernel status {st['status']}")
            ms.append(st["kernel_ms"])
            rays += st["closest"] + st["shadow"]
        r.set_stage_timing(True)
        flush.fill_(0)
        torch.cuda.synchronize()
        r.render_passes((warmup + steps) * spp, spp)
        st = r.stats()
        stages = r.stage_stats()
        r.set_stage_timing(False)
    b_ray, work = bytes_per_ray(sd, sd.render_options(), sd.pt_camera())
    ext_ms, ext_n = stages["extend"]
    a = work["bytes_per_closest_ray"] * st["closest"] / (ext_ms / 1000.0) / 1e9
    res.update({"value": rays / (sum(ms) / 1000.0) / 1e6, "unit": "Mrays/s", "steps": steps,
                "ms_per_step": statistics.mean(ms), "rays_per_step": rays / steps,
                "stages_ms": {k: v[0] for k, v in stages.items()},
                "roofline": {"bound": "hbm", "kernel": "wf_extend", "achieved": a, "peak": peak, "unit": "GB/s",
                             "frac": a / peak, "bytes_per_closest_ray": work["bytes_per_closest_ray"],
                             "share_of_frame": ext_ms / max(sum(v[0] for v in stages.values()), 1e-9)}})
    return res


ADJOINT_WORKLOAD = ("differentiable materials: icosphere 1,048,820 tris split into 32 materials (11 Disney "
                    "parameters each) + 4 sphere lights (emission rgb), 512x512, 16 spp, depth 6")


def adjoint_bench(steps, stream, flush):
    """Forward and adjoint (pt_render_adjoint, reusing the forward paths) of
    the differentiable-materials workload; device time of each call from the
    library's own CUDA events."""
    import torch
    from pathtracer import capi, diff, scenes
    from pathtracer.renderer import GpuRenderer
    sd = scenes.diff_scene(freq=229, width=512, height=512, max_depth=6)
    dI = np.random.RandomState(4).normal(size=(512, 512, 3)).astype(np.float32)
    fwd, adj = [], []
    with GpuRenderer(sd) as r:
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        r.set_stream(stream.cuda_stream)
        r.autotune(2)
        for k in range(steps + 1):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xFF)
            r.render_passes(16 * k, 16)
            st = r.stats()
            g = r.render_adjoint(16 * k, 16, dI)
            sa = r.stats()
            if k > 0:  # the first round is warm-up
                fwd.append((st["kernel_ms"], st["closest"] + st["shadow"]))
                adj.append(sa["kernel_ms"])
        r.set_stream(None)
    f_ms = statistics.mean(m for m, _ in fwd)
    a_ms = statistics.mean(adj)
    rays = statistics.mean(n for _, n in fwd)
    return {"workload": ADJOINT_WORKLOAD, "params": diff.num_params(sd.materials, sd.lights),
            "forward_ms": f_ms, "adjoint_ms": a_ms, "adjoint_over_forward": a_ms / f_ms,
            "forward_mrays_s": rays / (f_ms / 1000.0) / 1e6, "steps": steps,
            "grad_finite": bool(np.isfinite(g).all())}


BATCH_WORKLOAD = ("batched wavefront: 64 jobs, each the icosphere scene (16 Disney materials, one sphere light) "
                  "at 10k-1M triangles (log-uniform, seed 3), resolution from {128^2,256^2,512^2,1024^2}, spp "
                  "from {1,4,16,64}, depth 4-12; one pt_batch_render (CUDA graph) per step")


def batch_jobs(n=64, seed=3):
    """(freq, resolution, spp, depth) per job; triangles = 20 freq^2."""
    import math
    rng = np.random.RandomState(seed)
    jobs = []
    for _ in range(n):
        tris = math.exp(rng.uniform(math.log(1e4), math.log(1e6)))
        freq = max(2, int(round(math.sqrt(tris / 20.0))))
        res = int(rng.choice([128, 256, 512, 1024]))
        spp = int(rng.choice([1, 4, 16, 64]))
        depth = int(rng.randint(4, 13))
        jobs.append((freq, res, spp, depth))
    return jobs


def _batch_scene(args):
    from pathtracer import scenes
    j, (freq, res, spp, depth) = args
    return scenes.icosphere_scene(freq=freq, width=res, height=res, max_depth=depth, seed=1 + j, tile=res)


def batch_bench(steps, flush, n_jobs=64, sequential=True):
    """The 64-job batch: per-job completion times (p50/p99) and aggregate
    Mrays/s from the library's events around each pt_batch_render; beside it
    the same jobs rendered one after another on their own contexts."""
    import concurrent.futures as cf
    import multiprocessing as mp
    import torch
    from pathtracer import capi
    from pathtracer.renderer import GpuBatch, GpuRenderer
    jobs = batch_jobs(n_jobs)
    t0 = time.perf_counter()
    with cf.ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1),
                                mp_context=mp.get_context("spawn")) as ex:
        scenes_ = list(ex.map(_batch_scene, enumerate(jobs)))
    setup_s = time.perf_counter() - t0
    rs = [GpuRenderer(sd) for sd in scenes_]
    for r in rs:
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
    big = max(range(n_jobs), key=lambda j: jobs[j][0])
    tuning = rs[big].autotune(2)
    spp = [jb[2] for jb in jobs]
    paths = sum(jb[1] * jb[1] * jb[2] for jb in jobs)
    res = {"workload": BATCH_WORKLOAD, "jobs": n_jobs, "paths_per_step": paths,
           "tris": [20 * jb[0] ** 2 for jb in jobs], "tuning": tuning, "scene_setup_s": setup_s}
    with GpuBatch(rs) as b:
        lat, ms, rays, launches = [], [], 0, 0
        for k in range(steps + 1):  # the first is warm-up
            flush.fill_(k & 0xFF)
            torch.cuda.synchronize()
            job_ms = b.render([spp[j] * k for j in range(n_jobs)], spp)
            st = b.stats()
            if st["status"] != 0:
                raise RuntimeError(f"batch kernel status {st['status']}")
            if k > 0:
                lat.extend(job_ms.tolist())
                ms.append(st["kernel_ms"])
                rays += st["closest"] + st["shadow"]
                launches += st["launches"]
    res.update({"value": rays / (sum(ms) / 1000.0) / 1e6, "unit": "Mrays/s", "steps": steps,
                "ms_per_step": statistics.mean(ms), "rays_per_step": rays / steps,
                "latency_ms_p50": float(np.percentile(lat, 50)), "latency_ms_p99": float(np.percentile(lat, 99)),
                "latency_ms_max": float(max(lat)), "gpu_launches_per_step": launches / steps})
    # the batch kernels' per-job cost on its own: the largest job alone, as
    # a batch of one and through its own pt_render_passes (same paths)
    one = {}
    with GpuBatch([rs[big]]) as b1:
        for k in range(2):
            flush.fill_(k & 0xFF)
            torch.cuda.synchronize()
            b1.render([spp[big] * (steps + 1)], [spp[big]])
            one["batch_of_one_ms"] = b1.stats()["kernel_ms"]
            rs[big].render_passes(spp[big] * (steps + 1), spp[big])
            one["render_passes_ms"] = rs[big].stats()["kernel_ms"]
    one["job"] = {"tris": 20 * jobs[big][0] ** 2, "resolution": jobs[big][1], "spp": spp[big], "depth": jobs[big][3]}
    res["largest_job_alone"] = one
    if sequential:
        # the same jobs one after another, each its own pt_render_passes
        flush.fill_(0)
        torch.cuda.synchronize()
        seq_ms, seq_rays, done = 0.0, 0, []
        for j, r in enumerate(rs):
            r.render_passes(spp[j] * (steps + 1), spp[j])
            st = r.stats()
            seq_ms += st["kernel_ms"]
            seq_rays += st["closest"] + st["shadow"]
            done.append(seq_ms)
            r.close()  # its path state (up to 9.5 GB) is not kept for the next job
        res["sequential"] = {"value": seq_rays / (seq_ms / 1000.0) / 1e6, "unit": "Mrays/s", "ms": seq_ms,
                             "latency_ms_p50": float(np.percentile(done, 50)),
                             "latency_ms_p99": float(np.percentile(done, 99)),
                             "order": "job order, device time of each render summed"}
    for r in rs:
        r.close()
    return res


def drop_in_bench(sd, spp, steps, warmup):
    """The drop-in class, ptgb::CudaRenderer, driven from C++ as the
    reference's Main.cpp drives GLSLPT::Renderer (tests/cpp/dropin_driver.cpp,
    constructed from a GLSLPT::Scene*): autotune, then per step RenderPasses
    of `spp` passes, the Update that completes them and GetOutputBuffer
    (RGBA8 into a new[] host buffer); wall clock of the timed steps."""
    import tempfile
    from pathtracer import build
    csrc = os.path.dirname(build.LIB)
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "dropin_driver")
        subprocess.run(["g++", "-std=c++17", "-O2", "-I/usr/local/cuda/include",
                        os.path.join(ROOT, "tests", "cpp", "dropin_driver.cpp"), "-L" + csrc, "-lptgb",
                        "-Wl,-rpath," + csrc, "-o", exe], check=True)
        scene_file = os.path.join(td, "scene.bin")
        sd.save_flat(scene_file)
        r = subprocess.run([exe, scene_file, "bench", str(spp), str(steps), str(warmup)], check=True,
                           capture_output=True, text=True)
    d = json.loads(r.stdout.strip().splitlines()[-1])
    return {"value": d["rays"] / d["seconds"] / 1e6, "unit": "Mrays/s", "steps": d["steps"],
            "ms_per_step": 1000.0 * d["seconds"] / d["steps"], "h2d_bytes_per_step": 0,
            "d2h_bytes_per_step": d["d2h_bytes_per_step"],
            "path": "ptgb::CudaRenderer(GLSLPT::Scene*): RenderPasses + Update + GetOutputBuffer per step"}


def batch_of_one_bench(steps):
    """The largest job of the 64-job batch workload alone, `steps` frames
    through its own pt_render_passes and then `steps` as a batch of one (the
    batch kernels' per-job cost; profiling runs)."""
    import torch
    from pathtracer import build, capi
    from pathtracer.renderer import GpuBatch, GpuRenderer
    build.build_library()
    jobs = batch_jobs(64)
    big = max(range(len(jobs)), key=lambda j: jobs[j][0])
    sd = _batch_scene((big, jobs[big]))
    spp = jobs[big][2]
    out = {"workload": "largest job of the batch workload alone", "job": {
        "tris": 20 * jobs[big][0] ** 2, "resolution": jobs[big][1], "spp": spp, "depth": jobs[big][3]}}
    with GpuRenderer(sd) as r:
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        ms = []
        for k in range(steps):
            r.render_passes(spp * k, spp)
            ms.append(r.stats()["kernel_ms"])
        out["render_passes_ms"] = ms
        with GpuBatch([r]) as b:
            ms = []
            for k in range(steps):
                b.render([spp * k], [spp])
                ms.append(b.stats()["kernel_ms"])
            out["batch_of_one_ms"] = ms
    torch.cuda.synchronize()
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="icosphere_1m", choices=sorted(CONFIGS))
    ap.add_argument("--integrator", default="wavefront", choices=["megakernel", "wavefront"])
    ap.add_argument("--compare-steps", type=int, default=3,
                    help="timed steps of the other integrator, for the wavefront/megakernel ratio (0: skip)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch configuration")
    ap.add_argument("--adjoint-steps", type=int, default=3,
                    help="steps of the differentiable-materials workload for adjoint/forward (0: skip)")
    ap.add_argument("--stage-steps", type=int, default=3,
                    help="extra steps timed per kernel with CUDA events (roofline of the dominant kernel)")
    ap.add_argument("--batch-steps", type=int, default=2,
                    help="steps of the 64-job batched workload (p50/p99 job latency, aggregate Mrays/s; 0: skip)")
    ap.add_argument("--config-steps", type=int, default=3,
                    help="timed steps of each other workload (Cornell C1, instanced C3) in the default run (0: skip)")
    ap.add_argument("--drop-in-steps", type=int, default=5,
                    help="timed steps of the C++ drop-in class on the same frame (0: skip)")
    ap.add_argument("--small", action="store_true", help="small scene (profiling / quick checks)")
    ap.add_argument("--gpu-bvh", action="store_true",
                    help="build the BVH on the GPU (pt_create_gpu_bvh) instead of collapsing the host-built one")
    ap.add_argument("--spp", type=int, default=None, help="sample passes per step (profiling runs)")
    ap.add_argument("--batch-of-one", action="store_true",
                    help="only the largest batch job, alone and as a batch of one, --steps frames each (profiling)")
    args = ap.parse_args()
    if args.batch_of_one:
        return batch_of_one_bench(args.steps)
    cfg = dict(CONFIGS[args.config])
    if args.spp:
        cfg["spp"] = args.spp
        cfg["desc"] += f" [profiling run: {args.spp} spp per step]"
    if args.impl == "reference":
        return run_reference(args, cfg, args.config)

    import torch
    from pathtracer import build, capi
    from pathtracer.renderer import GpuRenderer

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    build.build_library()
    sd = make_scene(args.config, cfg, small=args.small)
    spp = cfg["spp"]
    r = GpuRenderer(sd, gpu_bvh=args.gpu_bvh)
    r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT if args.integrator == "wavefront" else capi.PT_INTEGRATOR_MEGAKERNEL)
    stream = torch.cuda.Stream()
    r.set_stream(stream.cuda_stream)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    tuning = None
    if args.integrator == "wavefront" and not args.no_autotune:
        # set-up, before the timed region: trial frames of the timed frame's
        # size, so that the tuning is measured where it is used
        tuning = r.autotune(spp)
    # each rank renders its own range of sample passes of the same frame
    pass_base = rank * spp * (args.steps + args.warmup + 8)

    def step(k):
        r.render_passes(pass_base + k * spp, spp)

    with torch.cuda.stream(stream):
        for k in range(args.warmup):
            step(k)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    rays = 0
    launches = 0
    truncated = 0
    untraced = 0
    shadow_q = 0
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xFF)  # L2 flush between timed steps
                starts[k].record(stream)
                step(args.warmup + k)
                ends[k].record(stream)
            st = r.stats()  # synchronises; counters of this launch
            rays += st["closest"] + st["shadow"]
            launches += st["launches"]
            truncated += st["truncated"]
            untraced += st["untraced"]
            shadow_q += st["shadow"]
            if st["status"] != 0:
                raise RuntimeError(f"kernel status {st['status']}")
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    t_total = sum(ms) / 1000.0
    rays_local = rays
    if dist:
        t = torch.tensor([t_total, float(rays)], dtype=torch.float64, device="cuda")
        tmax = t.clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        t_total, rays = float(tmax[0]), int(t[1])
    value = rays / t_total / 1e6
    rays_per_step = rays / (args.steps * world)
    # the queries each kind of traversal ran (this rank's shares): shadow
    # queries answered without traversal move none of their algorithmic bytes
    loc = max(rays_local, 1)
    closest_ps = rays_per_step * (rays_local - shadow_q) / loc
    shadow_traced_ps = rays_per_step * (shadow_q - untraced) / loc

    # the other integrator on the same frame, same timing rules (the two give
    # the same accumulation up to last-bit rounding, so equal RMSE)
    other = None
    if args.compare_steps > 0:
        other_name = "megakernel" if args.integrator == "wavefront" else "wavefront"
        r.set_integrator(capi.PT_INTEGRATOR_MEGAKERNEL if other_name == "megakernel" else capi.PT_INTEGRATOR_WAVEFRONT)
        base2 = pass_base + (args.warmup + 2 * args.steps + 4) * spp
        with torch.cuda.stream(stream):
            r.render_passes(base2, spp)  # warm-up
        torch.cuda.synchronize()
        o_ms, o_rays = 0.0, 0
        for k in range(args.compare_steps):
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xFF)
                ev0.record(stream)
                r.render_passes(base2 + (k + 1) * spp, spp)
                ev1.record(stream)
            st = r.stats()
            o_rays += st["closest"] + st["shadow"]
            o_ms += ev0.elapsed_time(ev1)
        o_val = o_rays / (o_ms / 1000.0) / 1e6
        other = {"integrator": other_name, "value": o_val, "unit": "Mrays/s", "steps": args.compare_steps,
                 "ms_per_step": o_ms / args.compare_steps,
                 "wavefront_over_megakernel": (value / o_val) if other_name == "megakernel" else (o_val / value)}
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT if args.integrator == "wavefront" else capi.PT_INTEGRATOR_MEGAKERNEL)

    # per-kernel device time: the same frames again with CUDA events around
    # every launch (no graph), for the roofline of the dominant kernel
    stages = None
    if args.integrator == "wavefront" and args.stage_steps > 0:
        r.set_stage_timing(True)
        tot = {k: [0.0, 0] for k in capi.STAGES}
        st_rays = {"closest": 0, "shadow": 0}
        base3 = pass_base + (args.warmup + 3 * args.steps + 8) * spp
        for k in range(args.stage_steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xFF)
                r.render_passes(base3 + k * spp, spp)
            st = r.stats()
            st_rays["closest"] += st["closest"]
            st_rays["shadow"] += st["shadow"] - st["untraced"]  # traversed by wf_shadow
            for name, (ms_k, n_k) in r.stage_stats().items():
                tot[name][0] += ms_k
                tot[name][1] += n_k
        r.set_stage_timing(False)
        stages = {"ms": {k: v[0] for k, v in tot.items()}, "launches": {k: v[1] for k, v in tot.items()},
                  "rays": st_rays, "steps": args.stage_steps}

    adjoint = None
    if args.adjoint_steps > 0 and rank == 0 and not args.small:
        adjoint = adjoint_bench(args.adjoint_steps, stream, flush)

    others = None
    if args.config_steps > 0 and rank == 0 and not args.small and args.config == "icosphere_1m":
        r.set_stream(None)
        peak, _ = measured_peaks()
        others = {name: config_bench(name, args.config_steps, args.warmup, flush, peak)
                  for name in ("cornell", "instanced")}
        r.set_stream(stream.cuda_stream)

    batch = None
    if args.batch_steps > 0 and rank == 0 and not args.small:
        r.set_stream(None)
        batch = batch_bench(args.batch_steps, flush)

    # end to end through the C ABI with host buffers
    import ctypes as C
    lib = capi.load_library()
    r.set_stream(None)
    out = torch.empty((r.height, r.width, 4), dtype=torch.uint8).pin_memory()
    cam = sd.pt_camera()
    e2e_rays = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        capi.check(lib, lib.pt_set_camera(r.ctx, C.byref(cam)))
        capi.check(lib, lib.pt_render_passes(r.ctx, pass_base + (args.warmup + args.steps + k) * spp, spp))
        capi.check(lib, lib.pt_get_output(r.ctx, spp, 0, C.cast(out.data_ptr(), C.POINTER(C.c_uint8))))
        st = r.stats()
        e2e_rays += st["closest"] + st["shadow"]
    e2e_t = time.perf_counter() - t0
    e2e = {"value": e2e_rays / e2e_t / 1e6 * world, "unit": "Mrays/s",
           "h2d_bytes_per_step": C.sizeof(capi.pt_camera),
           "d2h_bytes_per_step": int(r.width * r.height * 4)}

    drop_in = None
    if args.drop_in_steps > 0 and rank == 0 and args.integrator == "wavefront":
        drop_in = drop_in_bench(sd, spp, args.drop_in_steps, args.warmup)

    line = None
    if rank == 0:
        peak, peak_kind = measured_peaks()
        b_ray, work = bytes_per_ray(sd, sd.render_options(), cam)
        mean_ms = statistics.mean(ms)
        achieved = (work["bytes_per_closest_ray"] * closest_ps + work["bytes_per_shadow_ray"] * shadow_traced_ps) \
            / (mean_ms / 1000.0) / 1e9
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                    "frac": achieved / peak, "traffic": None, "peak_source": peak_kind,
                    "kernel": "whole frame", "bytes_per_ray": b_ray, **work}
        if stages:
            # the dominant kernel: algorithmic bytes of its queries / its own
            # event-timed launch durations
            per = {"extend": ("wf_extend", stages["rays"]["closest"], work["bytes_per_closest_ray"]),
                   "shadow": ("wf_shadow", stages["rays"]["shadow"], work["bytes_per_shadow_ray"])}
            kernels = {}
            for key, (kname, nrays, bpr) in per.items():
                kms, nl = stages["ms"][key], max(stages["launches"][key], 1)
                a = bpr * nrays / (kms / 1000.0) / 1e9
                kernels[kname] = {"achieved": a, "frac": a / peak, "avg_launch_ms": kms / nl, "launches": nl,
                                  "rays_per_launch": nrays / nl, "bytes_per_ray": bpr,
                                  "share_of_frame": kms / max(sum(stages["ms"].values()), 1e-9)}
            dom = max(kernels, key=lambda k: kernels[k]["share_of_frame"])
            kd = kernels[dom]
            traffic = None
            if dom == "wf_extend" and args.config in EXTEND_DRAM_BYTES_PER_RAY and not args.small:
                traffic = EXTEND_DRAM_BYTES_PER_RAY[args.config] * kd["rays_per_launch"]
            # secondary rooflines of the frame: FP32 work (algorithmic FLOPs
            # per query, against the nominal FP32 rate) and instruction
            # issue of the dominant kernel (ncu's instructions per query)
            fpk, nsm, mhz = fp32_peak_tflops()
            f_ach = work["flops_per_ray"] * (closest_ps + shadow_traced_ps) / (mean_ms / 1000.0) / 1e12
            fp32 = {"achieved": f_ach, "peak": fpk, "unit": "TFLOP/s", "frac": f_ach / fpk,
                    "flops_per_ray": work["flops_per_ray"],
                    "peak_source": f"nominal: {nsm} SMs x 128 FP32 lanes x 2 x {mhz:.0f} MHz"}
            issue = None
            if dom == "wf_extend" and args.config in EXTEND_WARP_INST_PER_RAY and not args.small:
                ipr = EXTEND_WARP_INST_PER_RAY[args.config]
                i_ach = ipr * kd["rays_per_launch"] / (kd["avg_launch_ms"] / 1000.0) / 1e12
                i_peak = nsm * 4 * mhz * 1e6 / 1e12
                issue = {"kernel": dom, "achieved": i_ach, "peak": i_peak, "unit": "Twarp-inst/s",
                         "frac": i_ach / i_peak, "warp_inst_per_ray": ipr,
                         "dram_bytes_per_ray": EXTEND_DRAM_BYTES_PER_RAY.get(args.config),
                         "peak_source": f"nominal: {nsm} SMs x 4 schedulers x {mhz:.0f} MHz"}
            roofline = {"bound": "hbm", "kernel": dom, "achieved": kd["achieved"], "peak": peak, "unit": "GB/s",
                        "frac": kd["achieved"] / peak, "traffic": traffic,
                        "algorithmic_bytes_per_launch": kd["bytes_per_ray"] * kd["rays_per_launch"],
                        "peak_source": peak_kind, "kernels": kernels,
                        "frame": {"achieved": achieved, "frac": achieved / peak, "bytes_per_ray": b_ray},
                        "fp32": fp32, "issue": issue, **work}
        cpu = None
        if not args.no_cpu_baseline:
            cpu, _, _ = cpu_baseline(sd, sd.render_options(), cam, spp)
        line = {
            "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": cfg["desc"] + ("" if not args.small else " (small variant)"),
                       "integrator": args.integrator, "rays_per_step": rays_per_step,
                       "l2": "flushed before each timed step (512 MiB write)",
                       "parallelism": f"{world} rank(s), disjoint sample-pass ranges" if world > 1 else "1 GPU",
                       "tuning": tuning if tuning else "default",
                       "bvh": f"built on the GPU in {r.gpu_build_ms():.1f} ms" if args.gpu_bvh else "host collapse",
                       "truncated_paths_per_step": truncated / args.steps,
                       # shadow queries of rays_per_step whose contribution is never added
                       # (zero scattering pdf towards the light): answered without traversal
                       "untraced_shadow_rays_per_step": untraced / args.steps,
                       "traversed_rays_per_step": closest_ps + shadow_traced_ps},
            "gpu_launches": launches,
            "roofline": roofline,
            "e2e": e2e,
            "clocks": clk.summary(),
        }
        if stages:
            line["stages"] = {"ms_per_step": {k: v / stages["steps"] for k, v in stages["ms"].items()},
                              "launches_per_step": {k: v / stages["steps"] for k, v in stages["launches"].items()}}
        if other:
            line["compare"] = other
        if drop_in:
            line["e2e_drop_in"] = drop_in
        if others:
            line["other_configs"] = others
        if adjoint:
            line["adjoint"] = adjoint
        if batch:
            line["batch"] = batch
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line))
    r.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
