"""Batched multi-scene rendering (pt_batch_create / pt_batch_render) against
each job rendered on its own context.  Needs a GPU.

A batch traces every job's paths through the same wavefront, each path
carrying its job's camera, lights, depth and scene root; a job's
accumulation must equal what pt_render_passes of the same pass range gives
on its own within the image tolerance of test_gpu_parity.py (the batch
branch of the kernels reads the job's parameters and compiles to slightly
different FP32 contractions, so last-bit differences occur, as between the
wavefront and the megakernel).  Jobs differ in scene, resolution (ragged sizes included), depth,
pass range, light count, render options, environment map and texture maps.
"""
import numpy as np
import pytest

from conftest import golden_scene
from test_gpu_parity import image_agreement

pytestmark = pytest.mark.gpu

# the render options of the jobs of the first tests
COMMON = dict(enable_rr=1, rr_depth=2, enable_envmap=0, enable_uniform_light=0, hide_emitters=0,
              enable_background=0, transparent_background=0, enable_roughness_mollification=0,
              enable_volume_mis=0)


def surface_instanced(width, height, num_instances=40, seed=3):
    """Transformed instances of two meshes under two sphere lights (no
    environment map, no medium)."""
    from pathtracer import scenes
    rng = np.random.RandomState(seed)
    V, Fc, _ = scenes.icosphere(8, 1.0, 0.05, seed)
    P, Ft = scenes.torus(1.0, 0.3, 24, 48, 0.03, seed + 1)
    meshes = [scenes.mesh_from_indexed(V, Fc), scenes.mesh_from_indexed(P, Ft)]
    mats = [scenes.material(color=tuple(rng.uniform(0.2, 0.9, 3)), metallic=float(rng.uniform()),
                            roughness=float(rng.uniform(0.1, 0.9))) for _ in range(6)]
    inst = []
    for k in range(num_instances):
        xf = scenes.mat4(rot=scenes.random_rotation(rng), scale=(0.3, 0.3, 0.3),
                         translate=tuple(rng.uniform(-2.0, 2.0, 3)))
        inst.append((k % 2, k % 6, xf))
    lights = [scenes.sphere_light((2.0, 3.0, 2.5), 0.6, (15.0, 14.0, 12.0)),
              scenes.sphere_light((-2.5, 2.0, -1.0), 0.4, (6.0, 8.0, 10.0))]
    cam = scenes.camera((0.0, 0.5, 6.0), (0.0, 0.0, 0.0), 50.0)
    opts = dict(render_width=width, render_height=height, tile_width=width, tile_height=height, max_depth=5)
    return scenes.build_scene(meshes, inst, mats, lights, cam, opts)


def job_scenes():
    from pathtracer import scenes
    return [
        (scenes.cornell(64, 64, max_depth=4, tile=32), 0, 3),
        (scenes.icosphere_scene(freq=30, width=48, height=32, max_depth=6, tile=16), 5, 2),
        (surface_instanced(40, 40), 0, 4),
        (scenes.cornell(33, 17, max_depth=7), 11, 1),  # ragged size
        (scenes.diff_scene(freq=20, width=32, height=32, max_depth=6), 2, 5),
    ]


@pytest.mark.parametrize("env", [{}, {"PT_BATCH_CAPACITY": "5000"}, {"PT_BATCH_GRAPH": "0"}],
                         ids=["graph", "small-chunks", "no-graph"])
def test_batch_equals_individual_renders(ptlib, monkeypatch, env):
    """Default: one chunk, launched as a CUDA graph.  small-chunks: whole
    passes packed into chunks of at most 5000 paths (a job's passes spread
    over several chunks).  no-graph: the same launches issued directly."""
    from pathtracer import capi
    from pathtracer.renderer import GpuBatch, GpuRenderer
    jobs = job_scenes()
    rs = [GpuRenderer(sd, **COMMON) for sd, _, _ in jobs]
    try:
        ref = []
        for r, (sd, fp, n) in zip(rs, jobs):
            r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
            r.clear()
            r.render_passes(fp, n)
            ref.append(r.accum())
            r.clear()
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        with GpuBatch(rs) as b:
            ms = b.render([fp for _, fp, _ in jobs], [n for _, _, n in jobs])
            st = b.stats()
        assert st["status"] == 0
        assert st["paths"] == sum(r.width * r.height * n for r, (_, _, n) in zip(rs, jobs))
        assert st["launches"] > 0
        assert np.all(np.isfinite(ms)) and np.all(ms > 0) and ms.max() <= st["kernel_ms"] * 1.5 + 5.0
        for r, a, (sd, _, _) in zip(rs, ref, jobs):
            got = r.accum()
            frac, mean_rel = image_agreement(got, a)
            assert frac >= 0.999 and mean_rel < 1e-4, (r.width, r.height, frac, mean_rel)
            assert np.array_equal(got[..., 3], a[..., 3])  # sample counts are exact
        # a second render accumulates on top of the first
        with GpuBatch(rs) as b:
            b.render([fp for _, fp, _ in jobs], [n for _, _, n in jobs])
        for r, a in zip(rs, ref):
            frac, _ = image_agreement(r.accum(), 2.0 * a)
            assert frac >= 0.999
    finally:
        for r in rs:
            r.close()


def test_all_direct_batch(ptlib):
    """Jobs that are all one untransformed instance each (the merged BLAS):
    the batch runs the direct form of the traversal kernels."""
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuBatch, GpuRenderer
    jobs = [(scenes.cornell(48, 40, max_depth=4, tile=16), 0, 3),
            (scenes.icosphere_scene(freq=30, width=40, height=24, max_depth=6, tile=16), 2, 2),
            (scenes.diff_scene(freq=20, width=32, height=32, max_depth=5), 1, 3)]
    rs = [GpuRenderer(sd, **COMMON) for sd, _, _ in jobs]
    try:
        ref = []
        for r, (sd, fp, n) in zip(rs, jobs):
            r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
            r.clear()
            r.render_passes(fp, n)
            ref.append(r.accum())
            r.clear()
        with GpuBatch(rs) as b:
            b.render([fp for _, fp, _ in jobs], [n for _, _, n in jobs])
            st = b.stats()
        assert st["status"] == 0
        for r, a in zip(rs, ref):
            frac, mean_rel = image_agreement(r.accum(), a)
            assert frac >= 0.999 and mean_rel < 1e-4, (r.width, r.height, frac, mean_rel)
    finally:
        for r in rs:
            r.close()


def test_single_job_batch(ptlib):
    from pathtracer import capi
    from pathtracer.renderer import GpuBatch, GpuRenderer
    sd = surface_instanced(24, 20, num_instances=10)
    with GpuRenderer(sd, **COMMON) as r:
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        r.clear()
        r.render_passes(3, 2)
        ref = r.accum()
        r.clear()
        with GpuBatch([r]) as b:
            b.render(3, 2)
        frac, mean_rel = image_agreement(r.accum(), ref)
        assert frac >= 0.999 and mean_rel < 1e-4


def opaque_textured():
    """The textured golden scene (every texture slot) with all materials
    made opaque: texture maps without the alpha test."""
    sd = golden_scene("ref_scene_textured.npz")
    sd.materials = sd.materials.copy()
    sd.materials[:, 28] = 1.0  # opacity
    sd.materials[:, 29] = 0.0  # alphaMode: opaque
    return sd


def test_batch_jobs_with_own_options_and_maps(ptlib):
    """Jobs whose render options, environment maps and texture maps differ:
    an environment map alone, the uniform light, hidden emitters over an
    environment map, a distant light, roughness mollification, texture maps
    (with a DirectX normal map) and a plain Cornell box with Russian
    roulette off, in one batch; each equals its own render."""
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuBatch, GpuRenderer
    tex = opaque_textured()
    tex.options = dict(tex.options, opengl_normal_map=0)
    jobs = [(golden_scene("feature_scene_env_only.npz"), 0, 3),
            (golden_scene("feature_scene_uniform_light.npz"), 1, 2),
            (golden_scene("feature_scene_hide_emitters.npz"), 0, 2),
            (golden_scene("feature_scene_distant.npz"), 2, 3),
            (golden_scene("feature_scene_mollification.npz"), 0, 2),
            (tex, 0, 2),
            (scenes.cornell(40, 24, max_depth=4), 3, 2)]
    rs = [GpuRenderer(sd) for sd, _, _ in jobs]
    rs[-1].set_options(capi.make_options(**dict(capi.options_dict(rs[-1].options), enable_rr=0)))
    try:
        ref = []
        for r, (sd, fp, n) in zip(rs, jobs):
            r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
            r.clear()
            r.render_passes(fp, n)
            ref.append(r.accum())
            r.clear()
        with GpuBatch(rs) as b:
            b.render([fp for _, fp, _ in jobs], [n for _, _, n in jobs])
            st = b.stats()
        assert st["status"] == 0
        assert st["paths"] == sum(r.width * r.height * n for r, (_, _, n) in zip(rs, jobs))
        for k, (r, a) in enumerate(zip(rs, ref)):
            got = r.accum()
            frac, mean_rel = image_agreement(got, a)
            assert frac >= 0.999 and mean_rel < 1e-4, (k, frac, mean_rel)
            assert np.array_equal(got[..., 3], a[..., 3])
    finally:
        for r in rs:
            r.close()


def test_batch_jobs_with_alpha_and_media(ptlib):
    """Alpha-tested materials (blend and mask, shadow rays traced inline
    since their AnyHit draws random numbers, pass-through paths finished by
    the tail kernel), absorbing and emissive media without volume MIS, an
    environment map and a plain scene in one batch; each equals its own
    render."""
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuBatch, GpuRenderer
    jobs = [(golden_scene("ref_scene_textured.npz"), 0, 3),
            (golden_scene("feature_scene_absorb.npz"), 1, 2),
            (golden_scene("feature_scene_emissive.npz"), 0, 2),
            (golden_scene("feature_scene_env_only.npz"), 2, 2),
            (scenes.cornell(40, 24, max_depth=4), 0, 2)]
    rs = [GpuRenderer(sd) for sd, _, _ in jobs]
    try:
        ref = []
        for r, (sd, fp, n) in zip(rs, jobs):
            r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
            r.clear()
            r.render_passes(fp, n)
            ref.append(r.accum())
            r.clear()
        with GpuBatch(rs) as b:
            b.render([fp for _, fp, _ in jobs], [n for _, _, n in jobs])
            st = b.stats()
        assert st["status"] == 0
        assert st["paths"] == sum(r.width * r.height * n for r, (_, _, n) in zip(rs, jobs))
        for k, (r, a) in enumerate(zip(rs, ref)):
            got = r.accum()
            frac, mean_rel = image_agreement(got, a)
            assert frac >= 0.999 and mean_rel < 1e-4, (k, frac, mean_rel)
            assert np.array_equal(got[..., 3], a[..., 3])
    finally:
        for r in rs:
            r.close()


def test_batch_rejects_unsupported_jobs(ptlib):
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuBatch, GpuRenderer
    a = GpuRenderer(scenes.cornell(16, 16), **COMMON)
    env = scenes.instanced_scene(num_instances=20, tris_per_blas=500, width=16, height=16, env_size=(32, 16))
    b = GpuRenderer(env)  # a medium with volume MIS
    c = GpuRenderer(golden_scene("feature_scene_absorb_volmis.npz"))  # the same
    try:
        for pair in ([a, b], [a, c]):
            with pytest.raises(capi.PTError) as e:
                GpuBatch(pair)
            assert e.value.code == capi.PT_ERR_UNSUPPORTED
        with GpuBatch([a]) as batch:
            with pytest.raises(capi.PTError) as e:
                batch.render(0, 0)
            assert e.value.code == capi.PT_ERR_INVALID_ARG
    finally:
        for r in (a, b, c):
            r.close()
