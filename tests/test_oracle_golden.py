"""The oracle against the reference's own code (CPU only).

The golden fixtures come from the reference itself (tests/golden/make_golden.py):
its loader + RadeonRays BVH + BvhTranslator for the scene arrays, and its
shader source compiled for the CPU for renders, DisneyEval and ClosestHit.
The oracle restates the shaders in float with the same operation order, so
the expected agreement is bit-exact.
"""
import numpy as np
import pytest

from conftest import golden, golden_scene


@pytest.mark.parametrize("name,scene_file", [
    ("cornell_box_orig", "ref_scene_cornell_box_orig.npz"),
    ("volume_cube", "ref_scene_volume_cube.npz"),
    ("cornell_c1_48", "scene_cornell_c1_48.npz"),
    ("textured", "ref_scene_textured.npz"),
])
def test_render_bit_exact_vs_reference_shaders(orc, name, scene_file):
    sd = golden_scene(scene_file)
    g = golden(f"ref_render_{name}.npz")
    o = sd.render_options(render_width=int(g["width"]), render_height=int(g["height"]),
                          tile_width=int(g["tile_w"]), tile_height=int(g["tile_h"]))
    acc, _, cnt = orc.render(sd, o, sd.pt_camera(), 0, int(g["passes"]))
    assert cnt["overflow"] == 0
    assert np.array_equal(acc, g["accum"]), f"max diff {np.abs(acc - g['accum']).max()}"


FEATURE_CASES = ["uniform_light", "uniform_light_env", "hide_emitters", "background", "transparent_background",
                 "mollification", "rr_off", "rr_depth_1", "env_only", "distant", "distant_only", "absorb",
                 "absorb_volmis", "emissive", "emissive_volmis", "all_flags", "textured_dx"]


@pytest.mark.parametrize("case", FEATURE_CASES)
def test_feature_render_bit_exact_vs_reference_shaders(orc, case):
    """Render options, light types and media the reference selects per scene
    (Renderer.cpp:400-476; distant lights sampling.glsl:229-236; absorbing and
    emissive media pathtrace.glsl:146,379-386), each rendered by the
    reference's shader source compiled with that macro set."""
    sd = golden_scene(f"feature_scene_{case}.npz")
    g = golden("ref_render_features.npz")
    acc, _, cnt = orc.render(sd, sd.render_options(), sd.pt_camera(), 0, int(g["passes"]))
    ref = g[f"{case}_accum"]
    assert cnt["overflow"] == 0
    assert np.array_equal(acc, ref), f"max diff {np.abs(acc - ref).max()}"


@pytest.mark.parametrize("name", ["reinhard", "aces", "aces_simple", "none", "reinhard_background",
                                  "aces_background", "reinhard_transparent", "aces_simple_transparent"])
def test_tonemap_vs_reference_shader(orc, name):
    """The numpy restatement of tonemap.glsl (orc.tonemap) against the
    reference's shader on the same accumulation: within 2e-6 in float, and
    the same RGBA8 value after the read-back's rounding except where the
    float sits on a rounding boundary."""
    import json

    from pathtracer import capi
    g = golden("ref_tonemap.npz")
    acc = g["accum"]
    H, W = acc.shape[:2]
    kw = json.loads(bytes(g["cases"]).decode())[name]
    o = capi.make_options(render_width=W, render_height=H, background_col=(0.2, 0.4, 0.8), **kw)
    got = orc.tonemap(acc, int(g["samples"]), o)
    ref = g[name]
    assert np.abs(got - ref).max() < 2e-6, np.abs(got - ref).max()
    assert (orc.to_rgba8(got) != orc.to_rgba8(ref)).mean() < 1e-3


def test_disney_eval_bit_exact_vs_reference(orc):
    g = golden("ref_bsdf.npz")
    f, pdf, _, _ = orc.bsdf_eval(g["state"], g["V"], g["N"], g["L"], use_double=False)
    assert np.array_equal(f.astype(np.float32), g["f"], equal_nan=True)
    assert np.array_equal(pdf.astype(np.float32), g["pdf"], equal_nan=True)


def test_disney_eval_fp32_vs_fp64_per_lobe(orc):
    """FP32 restatement against the FP64 one: relative error per lobe, on
    inputs away from the singular configurations (pdf/f well above 0)."""
    g = golden("ref_bsdf.npz")
    f32, p32, lf32, lp32 = orc.bsdf_eval(g["state"], g["V"], g["N"], g["L"], use_double=False)
    f64, p64, lf64, lp64 = orc.bsdf_eval(g["state"], g["V"], g["N"], g["L"], use_double=True)
    for k in range(5):
        ref = lp64[:, k]
        ok = ref > 1e-3
        if ok.sum() < 10:
            continue
        rel = np.abs(lp32[ok, k] - ref[ok]) / ref[ok]
        assert np.median(rel) < 1e-5, (k, np.median(rel))
        assert np.quantile(rel, 0.99) < 1e-3, (k, np.quantile(rel, 0.99))


def test_closest_hit_vs_reference(orc):
    g = golden("ref_closest.npz")
    for name in ("cornell_box_orig", "volume_cube"):
        sd = golden_scene(f"ref_scene_{name}.npz")
        rays = g[f"{name}_rays"]
        r = orc.closest_hit_full(sd, rays)
        assert np.array_equal(r["hit"], g[f"{name}_hit"])
        assert np.array_equal(r["t"], g[f"{name}_t"])
        assert np.array_equal(r["mat"], g[f"{name}_mat"])
        assert np.array_equal(r["emitter"], g[f"{name}_emitter"])
        assert np.array_equal(r["normal"], g[f"{name}_normal"])


def test_rng_stream_matches_pcg4d(orc):
    """PCG4D (globals.glsl:155-166) restated in numpy, against the oracle."""
    def pcg(px, py, frame, n):
        s = np.array([px, py, frame, px + py], np.uint64)
        m = np.uint64(0xFFFFFFFF)
        out = []
        for _ in range(n):
            s = (s * np.uint64(1664525) + np.uint64(1013904223)) & m
            s[0] = (s[0] + s[1] * s[3]) & m; s[1] = (s[1] + s[2] * s[0]) & m
            s[2] = (s[2] + s[0] * s[1]) & m; s[3] = (s[3] + s[1] * s[2]) & m
            s = s ^ (s >> np.uint64(16))
            s[0] = (s[0] + s[1] * s[3]) & m; s[1] = (s[1] + s[2] * s[0]) & m
            s[2] = (s[2] + s[0] * s[1]) & m; s[3] = (s[3] + s[1] * s[2]) & m
            out.append(np.float32(s[0]) / np.float32(4294967296.0))
        return np.array(out, np.float32)
    for px, py, fr in [(0, 0, 2), (17, 5, 1234), (99, 99, 7)]:
        assert np.array_equal(orc.rng_stream(px, py, fr, 32), pcg(px, py, fr, 32))
