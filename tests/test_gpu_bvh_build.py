"""The BVH built on the GPU (pt_create_gpu_bvh, pt_update_transforms)
against the oracle on the reference's binary BVH.  Needs a GPU.

A different tree finds the same hits: triangle and instance ids exact,
except ties at equal distance (|dt| <= 1e-6 t) and at most 1e-4 of the rays
grazing a shared edge (the tolerances of test_gpu_parity.py); any-hit
booleans exact; renders equal to the host-built BVH's within the image
tolerance of the parity tests.
"""
import numpy as np
import pytest

from test_gpu_parity import classify_mismatch, image_agreement, ray_set, scene_by_name

pytestmark = pytest.mark.gpu

SCENES = ["ref_cornell", "ref_volume", "ref_textured", "cornell", "icosphere", "instanced"]


@pytest.mark.parametrize("name", SCENES)
def test_gpu_built_bvh_hits(ptlib, orc, name):
    from pathtracer.renderer import GpuRenderer
    sd = scene_by_name(name)
    rays = ray_set(sd, orc, 20000, 1)
    with GpuRenderer(sd, gpu_bvh=True) as r:
        assert r.gpu_build_ms() > 0
        hg = r.trace(rays)
        maxd = np.random.RandomState(2).uniform(0.1, 5.0, len(rays)).astype(np.float32)
        occ = r.shadow(rays, maxd)
    ho, cnt = orc.trace_closest(sd, rays, mode=0)
    bad, ties, grazing = classify_mismatch(sd, orc, rays, hg, ho)
    assert len(bad) == 0 and grazing <= max(2, int(1e-4 * len(rays))), (name, len(bad), ties, grazing)
    same = (hg["prim_id"] == ho["prim_id"]) & (hg["inst_id"] == ho["inst_id"])
    assert np.array_equal(hg["t"][same], ho["t"][same])
    occ_o = orc.trace_any(sd, sd.render_options(), rays, maxd)
    assert (occ != occ_o).sum() <= max(2, int(1e-4 * len(rays)))


@pytest.mark.parametrize("name", ["cornell", "icosphere", "instanced"])
def test_gpu_built_bvh_renders_like_the_host_built_one(ptlib, name):
    from pathtracer import capi
    from pathtracer.renderer import GpuRenderer
    sd = scene_by_name(name)
    imgs = []
    for gpu in (False, True):
        with GpuRenderer(sd, gpu_bvh=gpu) as r:
            r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
            r.render_passes(0, 4)
            imgs.append(r.accum())
    frac, mean_rel = image_agreement(imgs[1], imgs[0])
    assert frac >= 0.999 and mean_rel < 1e-4, (name, frac, mean_rel)


def test_update_transforms_rebuilds_on_the_gpu(ptlib, orc):
    """Move some instances of an untransformed scene (so the merged BLAS
    changes too) and compare against a scene built from scratch with the
    new transforms."""
    from pathtracer import scenes
    from pathtracer.renderer import GpuRenderer
    V, Fc, face = scenes.icosphere(20, 1.0, 0.05, 1)
    meshes = [scenes.mesh_from_indexed(V, Fc[(face % 4) == g]) for g in range(4)]
    mats = [scenes.material()] + [scenes.material(color=(0.2 * k + 0.1, 0.5, 0.5)) for k in range(4)]
    light = scenes.sphere_light((2.2, 2.4, 2.6), 0.5, (20.0, 20.0, 20.0))
    cam = scenes.camera((0.0, 0.0, 3.2), (0.0, 0.0, 0.0), 45.0)
    opts = dict(render_width=64, render_height=48, tile_width=32, tile_height=24, max_depth=4)
    ident = scenes.mat4()
    moved = [ident, scenes.mat4(translate=(0.3, 0.0, 0.0)), ident, scenes.mat4(translate=(0.0, -0.2, 0.1))]
    before = scenes.build_scene(meshes, [(g, g + 1, ident) for g in range(4)], mats, [light], cam, opts)
    after = scenes.build_scene(meshes, [(g, g + 1, moved[g]) for g in range(4)], mats, [light], cam, opts)
    rays = ray_set(after, orc, 8000, 4)
    with GpuRenderer(before, gpu_bvh=True) as r:
        r.update_transforms(after.transforms)
        hg = r.trace(rays)
    ho, _ = orc.trace_closest(after, rays, mode=0)
    bad, ties, grazing = classify_mismatch(after, orc, rays, hg, ho)
    assert len(bad) == 0 and grazing <= 2, (len(bad), ties, grazing)
