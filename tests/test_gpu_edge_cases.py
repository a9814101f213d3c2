"""Edge cases of the render and query paths.  Needs a GPU.

* images of one pixel, one row and one column, and ragged tiles;
* maximum depth 0 and 1;
* frames in which every ray misses;
* empty pass ranges and empty ray sets;
* degenerate (zero-area) triangles and rays along the axes (zero direction
  components);
* the path-iteration bound (PT_MAX_PATH_ITERATIONS, read from the header):
  a stack of 5000 blended layers 4e-3 apart
  (farther apart than the EPS offset of a pass-through), which every
  camera ray crosses one iteration at a time, ends each path at
  PT_MAX_PATH_ITERATIONS in the oracle, the megakernel and the wavefront
  alike.

Each render is checked against the megakernel (the same ray counts and
accumulation up to last-bit rounding) and against the oracle (the image
tolerance of test_gpu_parity.py).
"""
import numpy as np
import pytest

from test_gpu_parity import classify_mismatch, image_agreement

pytestmark = pytest.mark.gpu

def header_define(name):
    import os
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    text = open(os.path.join(root, "include", "pt_cuda.h")).read()
    return int(re.search(r"#define\s+" + name + r"\s+(\d+)", text).group(1))


PT_MAX_PATH_ITERATIONS = header_define("PT_MAX_PATH_ITERATIONS")


def render_both(sd, passes=2):
    """(megakernel accumulation, wavefront accumulation, stats of each)."""
    from pathtracer import capi
    from pathtracer.renderer import GpuRenderer
    with GpuRenderer(sd) as r:
        r.render_passes(0, passes)
        a, sa = r.accum(), r.stats()
        r.clear()
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        r.render_passes(0, passes)
        b, sb = r.accum(), r.stats()
    return a, b, sa, sb


def check_against_megakernel_and_oracle(orc, sd, passes=2):
    a, b, sa, sb = render_both(sd, passes)
    assert sa["status"] == 0 and sb["status"] == 0
    assert sa["paths"] == sb["paths"] == sd.options["render_width"] * sd.options["render_height"] * passes
    assert sa["closest"] + sa["shadow"] == sb["closest"] + sb["shadow"]
    assert sa["truncated"] == sb["truncated"]
    assert np.array_equal(a[..., 3], b[..., 3])
    rel = np.abs(a[..., :3] - b[..., :3]) / np.maximum(np.abs(b[..., :3]), 1e-3)
    assert rel.max() < 1e-4, rel.max()
    ref, _, cnt = orc.render(sd, sd.render_options(), sd.pt_camera(), 0, passes)
    frac, mean_rel = image_agreement(b, ref)
    assert frac >= 0.99 and mean_rel < 1e-3, (frac, mean_rel)
    assert np.array_equal(b[..., 3], ref[..., 3])
    return b, sb


@pytest.mark.parametrize("size", [(1, 1), (17, 1), (1, 13), (37, 23)])
def test_tiny_and_ragged_images(ptlib, orc, size):
    from pathtracer import scenes
    w, h = size
    sd = scenes.cornell(w, h, tile=16)
    check_against_megakernel_and_oracle(orc, sd, passes=3)


@pytest.mark.parametrize("depth", [0, 1])
def test_shallow_depths(ptlib, orc, depth):
    from pathtracer import scenes
    sd = scenes.cornell(32, 32, max_depth=depth, tile=16)
    img, st = check_against_megakernel_and_oracle(orc, sd, passes=2)
    if depth == 0:
        assert st["shadow"] == 0  # the loop ends at the first vertex before next-event estimation


def test_every_ray_misses(ptlib, orc):
    """A camera looking away from the scene: no background, no environment
    map, so the accumulation holds only the sample counts."""
    from pathtracer import capi, scenes
    sd = scenes.cornell(24, 16, tile=8)
    cam = sd.camera.copy()
    cam["forward"] = [-x for x in cam["forward"]]
    cam["right"] = [-x for x in cam["right"]]
    cam["position"] = [cam["position"][k] - 3.0 * sd.camera["forward"][k] for k in range(3)]
    sd.camera = cam
    img, st = check_against_megakernel_and_oracle(orc, sd, passes=2)
    assert np.all(img[..., :3] == 0.0)
    assert st["closest"] == 24 * 16 * 2 and st["shadow"] == 0


def test_empty_work(ptlib):
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuRenderer
    sd = scenes.cornell(16, 16)
    with GpuRenderer(sd) as r:
        for integrator in (capi.PT_INTEGRATOR_MEGAKERNEL, capi.PT_INTEGRATOR_WAVEFRONT):
            r.set_integrator(integrator)
            r.render_passes(0, 0)
            assert not r.accum().any()
            assert r.stats()["paths"] == 0
        assert r.trace(np.zeros((0, 6), np.float32)).shape == (0,)
        assert r.shadow(np.zeros((0, 6), np.float32), np.zeros(0, np.float32)).shape == (0,)


def test_degenerate_triangles_and_axis_rays(ptlib, orc):
    """Zero-area triangles (a point, a segment) among ordinary ones, and rays
    whose direction has zero components: the same hits as the oracle."""
    from pathtracer import scenes
    from pathtracer.renderer import GpuRenderer
    rng = np.random.RandomState(5)
    tris = rng.uniform(-1, 1, size=(400, 3, 3))
    tris[:40, 1] = tris[:40, 0]                       # two equal corners: a segment
    tris[40:60, 1] = tris[40:60, 2] = tris[40:60, 0]  # a point
    tris[60:100, 2] = 0.5 * (tris[60:100, 0] + tris[60:100, 1])  # collinear corners
    P = tris.reshape(-1, 3)
    N = np.tile([0.0, 0.0, 1.0], (P.shape[0], 1))
    mesh = scenes.Mesh(P, N)
    cam = scenes.camera((0.0, 0.0, 4.0), (0.0, 0.0, 0.0), 45.0)
    sd = scenes.build_scene([mesh], [(0, 0, scenes.mat4())], [scenes.material()],
                            [scenes.sphere_light((0, 3, 3), 0.3, (10, 10, 10))], cam,
                            dict(render_width=16, render_height=16, tile_width=16, tile_height=16, max_depth=3))
    o = rng.uniform(-1.5, 1.5, size=(6000, 3))
    axis = rng.randint(0, 3, 6000)
    d = np.eye(3)[axis] * rng.choice([-1.0, 1.0], (6000, 1))
    second = (axis[:2000] + rng.randint(1, 3, 2000)) % 3  # a different axis: two nonzero components
    d[:2000] += np.eye(3)[second] * rng.choice([-1.0, 1.0], (2000, 1))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = orc.rays_array(o.astype(np.float32), d.astype(np.float32))
    with GpuRenderer(sd) as r:
        hg = r.trace(rays)
        maxd = rng.uniform(0.1, 3.0, len(rays)).astype(np.float32)
        occ = r.shadow(rays, maxd)
    ho, _ = orc.trace_closest(sd, rays, mode=0)
    bad, ties = classify_mismatch(sd, orc, rays, hg, ho)
    assert len(bad) <= 2, (len(bad), ties)
    assert (hg["prim_id"] >= 0).sum() > 500
    # no triangle of exactly zero area is hit (ids as the scene build ordered them)
    vi = sd.vert_indices.reshape(-1, 3)
    V = sd.vertices_uvx[:, :3].astype(np.float64)
    area = np.linalg.norm(np.cross(V[vi[:, 1]] - V[vi[:, 0]], V[vi[:, 2]] - V[vi[:, 0]]), axis=1)
    assert (area == 0).sum() >= 60
    assert not np.isin(hg["prim_id"][hg["prim_id"] >= 0], np.where(area == 0)[0]).any()
    occ_o = orc.trace_any(sd, sd.render_options(), rays, maxd)
    assert np.array_equal(occ, occ_o)


def test_path_iteration_bound(ptlib, orc):
    """5000 blended layers (opacity 0) 4e-3 apart across the view: every
    camera path passes through them one iteration at a time (alpha
    pass-through keeps the depth) and ends at the bound."""
    from pathtracer import scenes
    layers = 5000
    assert layers > PT_MAX_PATH_ITERATIONS
    meshes = []
    quad = scenes.quad_mesh((-50, -50, 0), (50, -50, 0), (50, 50, 0), (-50, 50, 0), (0, 0, 1))  # wider than the view
    P = np.concatenate([quad.verts[:, :3] + np.array([0, 0, -4e-3 * k]) for k in range(layers)])
    N = np.tile([0.0, 0.0, 1.0], (P.shape[0], 1))
    meshes.append(scenes.Mesh(P, N))
    mats = [scenes.material(alpha_mode=1, opacity=0.0)]
    cam = scenes.camera((0.0, 0.0, 1.0), (0.0, 0.0, -1.0), 20.0)
    sd = scenes.build_scene(meshes, [(0, 0, scenes.mat4())], mats,
                            [scenes.sphere_light((0, 0, 3), 0.3, (10, 10, 10))], cam,
                            dict(render_width=6, render_height=4, tile_width=6, tile_height=4, max_depth=4))
    img, st = check_against_megakernel_and_oracle(orc, sd, passes=1)
    assert st["truncated"] == 6 * 4
    assert st["closest"] == 6 * 4 * PT_MAX_PATH_ITERATIONS
