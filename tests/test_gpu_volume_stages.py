"""The wavefront's transmittance stages for VOL_MIS scenes (medium + volume
MIS), against the megakernel and the oracle.  Needs a GPU.

With VOL_MIS the reference's next-event rays go through EvalTransmittance
(pathtrace.glsl:117-153): closest-hit segments through refractive surfaces,
attenuated inside media.  The wavefront runs them in one of two stages:

* no alpha materials: EvalTransmittance draws no random numbers, so shade
  stores the request and the persistent transmittance stage resolves it
  (wf_transmit);
* alpha materials (a blended volume boundary draws a random number at each
  crossing): shade suspends at the query, the persistent replay stage traces
  it from the path's RNG state (wf_transmit_replay), and shade runs the step
  again with the recorded transmittance and RNG state.  With an environment
  map and analytic lights a step has two queries.

Either way every path draws the reference's random numbers: the ray counts
equal the megakernel's (which traces EvalTransmittance inline) and the
accumulation equals it up to last-bit rounding (the tolerance of
test_wavefront_equals_megakernel).  Against the oracle the tolerance is
calibrated on the oracle's own FP32 / FP64 difference (the scene is
sensitive to rounding).
"""
import numpy as np
import pytest

from test_gpu_parity import image_agreement

pytestmark = pytest.mark.gpu


def volume_scene(blend: bool, env: bool, lights: bool = True, width=64, height=48, max_depth=6):
    """Ground quad, a glass sphere, a scattering-medium cube (boundary opaque
    and refractive, or blended with opacity 0 as the reference's volume
    scenes have it), a sphere light and optionally an environment map."""
    from pathtracer import scenes
    V, Fc, _ = scenes.icosphere(6, 1.0, 0.0, 1)
    meshes = [scenes.quad_mesh((-4, 0, -4), (4, 0, -4), (4, 0, 4), (-4, 0, 4), (0, 1, 0)),
              scenes.mesh_from_indexed(V, Fc), scenes.cube_mesh()]
    mats = [scenes.material(),
            scenes.material(color=(0.7, 0.6, 0.5), roughness=0.8),
            scenes.material(color=(1, 1, 1), spec_trans=1.0, roughness=0.05, ior=1.5),
            scenes.material(color=(1, 1, 1), spec_trans=1.0, roughness=0.0, medium_type=2, medium_density=0.8,
                            medium_color=(0.9, 0.8, 0.7), medium_anisotropy=0.3,
                            alpha_mode=1 if blend else 0, opacity=0.0 if blend else 1.0)]
    inst = [(0, 1, scenes.mat4()),
            (1, 2, scenes.mat4(None, (0.6, 0.6, 0.6), (-0.9, 0.6, 0.2))),
            (2, 3, scenes.mat4(None, (1.4, 1.4, 1.4), (0.8, 0.71, -0.3)))]  # 0.01 above the ground
    lts = [scenes.sphere_light((1.5, 3.0, 2.0), 0.4, (18.0, 16.0, 14.0))] if lights else []
    cam = scenes.camera((0.0, 1.6, 4.5), (0.0, 0.6, 0.0), 50.0)
    opts = dict(render_width=width, render_height=height, tile_width=32, tile_height=24, max_depth=max_depth,
                enable_volume_mis=1, enable_envmap=1 if env else 0)
    envmap = scenes.sky_envmap(64, 32, sun_intensity=200.0) if env else None
    return scenes.build_scene(meshes, inst, mats, lts, cam, opts, envmap=envmap)


CASES = {
    "deferred-lights": dict(blend=False, env=False),
    "deferred-env-lights": dict(blend=False, env=True),
    "replay-lights": dict(blend=True, env=False),
    "replay-env-lights": dict(blend=True, env=True),  # two queries per step
    "replay-env": dict(blend=True, env=True, lights=False),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_volume_stage_equals_megakernel(ptlib, case):
    from pathtracer import capi
    from pathtracer.renderer import GpuRenderer
    sd = volume_scene(**CASES[case])
    with GpuRenderer(sd) as r:
        r.render_passes(0, 3)
        a = r.accum()
        sa = r.stats()
        r.clear()
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        r.render_passes(0, 3)
        b = r.accum()
        sb = r.stats()
    assert sa["status"] == 0 and sb["status"] == 0
    assert sa["paths"] == sb["paths"]
    assert sa["shadow"] > 0 and sa["closest"] + sa["shadow"] == sb["closest"] + sb["shadow"], (sa, sb)
    assert np.array_equal(a[..., 3], b[..., 3])
    rel = np.abs(a[..., :3] - b[..., :3]) / np.maximum(np.abs(b[..., :3]), 1e-3)
    assert rel.max() < 1e-4 and np.mean(rel) < 1e-6, (case, rel.max(), np.mean(rel))


@pytest.mark.parametrize("case", ["deferred-env-lights", "replay-env-lights"])
def test_volume_stage_matches_oracle(ptlib, orc, case):
    """This scene is sensitive to rounding: the refractive cube with a
    scattering medium inside carries long paths, and on about 7% of the
    pixels the oracle's own FP32 and FP64 renders of the same samples differ
    by more than the per-pixel tolerance.  So the GPU image must agree with
    the oracle's FP32 image at least as well as that FP64 render does, less
    2% of the pixels, with a difference of the image means within twice
    theirs or the 1e-3 of test_render_matches_oracle (and ray counts within
    1%)."""
    from pathtracer import capi
    from pathtracer.renderer import GpuRenderer
    sd = volume_scene(**CASES[case])
    o = sd.render_options()
    passes = 4
    with GpuRenderer(sd) as r:
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        r.render_passes(0, passes)
        acc = r.accum()
        st = r.stats()
    ref, _, cnt = orc.render(sd, o, sd.pt_camera(), 0, passes)
    ref64, _, _ = orc.render(sd, o, sd.pt_camera(), 0, passes, use_double=True)
    base_frac, base_rel = image_agreement(ref64, ref)
    frac, mean_rel = image_agreement(acc, ref)
    assert st["status"] == 0
    assert frac >= base_frac - 0.02 and mean_rel <= max(2.0 * base_rel, 1e-3), (case, frac, mean_rel, base_frac,
                                                                                 base_rel)
    assert np.array_equal(acc[..., 3], ref[..., 3])
    total_gpu = st["closest"] + st["shadow"]
    total_orc = cnt["closest"] + cnt["shadow"]
    assert abs(total_gpu - total_orc) <= 0.01 * total_orc


def test_replay_in_small_batches(ptlib, monkeypatch):
    """The replay form with several wavefront batches per call (one pass
    each), through the graph and through direct launches (stage timing)."""
    from pathtracer import capi
    from pathtracer.renderer import GpuRenderer
    sd = volume_scene(blend=True, env=True, width=40, height=30)
    monkeypatch.setenv("PT_WAVEFRONT_CAPACITY", str(40 * 30))
    with GpuRenderer(sd) as r:
        r.render_passes(0, 3)
        a = r.accum()
        r.clear()
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        r.render_passes(0, 3)
        b = r.accum()
        r.clear()
        r.set_stage_timing(True)
        r.render_passes(0, 3)
        c = r.accum()
        r.set_stage_timing(False)
    for x in (b, c):
        rel = np.abs(a[..., :3] - x[..., :3]) / np.maximum(np.abs(x[..., :3]), 1e-3)
        assert rel.max() < 1e-4 and np.mean(rel) < 1e-6
