"""Render options, light types and media that the reference decides per scene
(Renderer.cpp:400-476), through the C ABI.  Needs a GPU.

Each case of tests/golden/make_golden.py FEATURE_CASES is a small scene
rendered by the reference's own shader source compiled with that case's
OPT_* macro set (ref_render_features.npz); the oracle equals those renders
bit for bit (tests/test_oracle_golden.py).  Here the CUDA kernels are held
to them:

  * uniform light (with and without an environment map present), hidden
    emitters, background and transparent background (alpha 0 for camera
    rays that miss), roughness mollification, Russian roulette off and at
    depth 1, environment map only, distant lights (no MIS,
    pathtrace.glsl:257,271) alone and beside a sphere light, absorbing and
    emissive media with and without volume MIS (pathtrace.glsl:146,379-386),
    DirectX-convention normal maps, and all of the flags at once;
  * the megakernel against the golden: the image tolerance of
    test_gpu_parity.py (>= 99% of pixels within 1e-3 relative, image means
    within 1e-3; alpha exact);
  * the wavefront against the megakernel: the same ray counts and paths,
    samples equal up to last-bit rounding (max relative difference 1e-4,
    mean 1e-6);
  * tonemap.glsl, every branch (Reinhard, ACES fitted, simple ACES, off;
    plain, background, transparent background): pt_get_output against the
    reference shader's arithmetic (orc.tonemap, pinned to the shader on
    the CPU) on the GPU's own accumulation, within one RGBA8 step.
"""
import json

import numpy as np
import pytest

from conftest import golden, golden_scene
from test_gpu_parity import image_agreement, pixel_bar

pytestmark = pytest.mark.gpu

CASES = ["uniform_light", "uniform_light_env", "hide_emitters", "background", "transparent_background",
         "mollification", "rr_off", "rr_depth_1", "env_only", "distant", "distant_only", "absorb",
         "absorb_volmis", "emissive", "emissive_volmis", "all_flags", "textured_dx"]


@pytest.mark.parametrize("case", CASES)
def test_feature_matches_reference_shaders(ptlib, orc, case):
    from pathtracer.renderer import GpuRenderer
    sd = golden_scene(f"feature_scene_{case}.npz")
    g = golden("ref_render_features.npz")
    passes = int(g["passes"])
    ref = g[f"{case}_accum"]
    o = sd.render_options()
    with GpuRenderer(sd) as r:
        r.render_passes(0, passes)
        acc = r.accum()
        st = r.stats()
    assert st["status"] == 0, st
    assert st["paths"] == o.render_width * o.render_height * passes
    frac, mean_rel = image_agreement(acc, ref)
    bar = pixel_bar(orc, sd, o, passes, ref)
    assert frac >= bar and mean_rel < 1e-3, (case, frac, bar, mean_rel)
    assert np.array_equal(acc[..., 3], ref[..., 3])


@pytest.mark.parametrize("case", CASES)
def test_feature_wavefront_equals_megakernel(ptlib, case):
    from pathtracer import capi
    from pathtracer.renderer import GpuRenderer
    sd = golden_scene(f"feature_scene_{case}.npz")
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
    assert sa["closest"] + sa["shadow"] == sb["closest"] + sb["shadow"], (sa, sb)
    assert np.array_equal(a[..., 3], b[..., 3])
    rel = np.abs(a[..., :3] - b[..., :3]) / np.maximum(np.abs(b[..., :3]), 1e-3)
    assert rel.max() < 1e-4 and np.mean(rel) < 1e-6, (case, rel.max(), np.mean(rel))


def test_tonemap_every_branch(ptlib, orc):
    """pt_get_output for each tonemap / background combination of the
    reference's tonemap pass, on a render with background pixels (alpha 0)."""
    from pathtracer import capi
    from pathtracer.renderer import GpuRenderer
    sd = golden_scene("feature_scene_background.npz")
    cases = json.loads(bytes(golden("ref_tonemap.npz")["cases"]).decode())
    passes = 4
    with GpuRenderer(sd) as r:
        r.render_passes(0, passes)
        acc = r.accum()
        base = capi.options_dict(r.options)
        for name, kw in cases.items():
            opts = dict(base, enable_background=0, transparent_background=0, background_col=(0.2, 0.4, 0.8))
            opts.update(kw)
            o = capi.make_options(**opts)
            r.set_options(o)
            ldr = r.output(passes)
            exp = orc.to_rgba8(orc.tonemap(acc, passes, o))
            d = np.abs(ldr.astype(np.int32) - exp.astype(np.int32))
            assert d.max() <= 1, (name, d.max())
            assert (d > 0).mean() < 0.01, (name, (d > 0).mean())
            if kw.get("transparent_background"):
                assert (ldr[..., 3] < 255).any()
            else:
                assert np.all(ldr[..., 3] == 255)
        assert np.array_equal(r.accum(), acc)  # option changes keep the accumulation
