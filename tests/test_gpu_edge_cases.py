"""Edge cases of the render and query paths.  Needs a GPU.

* images of one pixel, one row and one column, and ragged tiles;
* maximum depth 0 and 1;
* frames in which every ray misses;
* empty pass ranges and empty ray sets;
* degenerate (zero-area) triangles and rays along the axes (zero direction
  components);
* failure detection without a fault: a traversal stack bound lowered for
  a test sets PT_ERR_STACK_OVERFLOW in the status word and the calls
  return; a BVH deeper than the stack is refused at pt_create;
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
    bad, ties, grazing = classify_mismatch(sd, orc, rays, hg, ho)
    assert len(bad) == 0 and grazing <= 2, (len(bad), ties, grazing)
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


PT_ERR_STACK_OVERFLOW = header_define("PT_ERR_STACK_OVERFLOW")
PT_ERR_UNSUPPORTED = header_define("PT_ERR_UNSUPPORTED")


def test_stack_overflow_is_reported_not_trapped(ptlib, orc, monkeypatch):
    """Failure detection without a fault.  With the traversal stack bound of
    a context lowered to 2 entries (PT_TRAVERSAL_STACK_LIMIT, read at
    pt_create), no ray can enter an instance (an entry takes four: the
    TLAS node group, the pending instances, the world ray's reciprocal
    direction, a sentinel), so the kernels skip the instances and set
    PT_ERR_STACK_OVERFLOW in the status word.  Each call returns, the
    status comes back through pt_get_stats, the next call clears it, and a
    context made without the bound renders the oracle's image."""
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuRenderer
    sd = scenes.cornell(32, 32, tile=16)  # boxes are transformed instances
    monkeypatch.setenv("PT_TRAVERSAL_STACK_LIMIT", "2")
    with GpuRenderer(sd) as r:
        for integrator in (capi.PT_INTEGRATOR_MEGAKERNEL, capi.PT_INTEGRATOR_WAVEFRONT):
            r.set_integrator(integrator)
            r.clear()
            r.render_passes(0, 2)
            st = r.stats()
            assert st["status"] == PT_ERR_STACK_OVERFLOW, (integrator, st)
            assert st["paths"] == 32 * 32 * 2
            assert np.isfinite(r.accum()).all()
        r.render_tile(0, 0, 2)
        assert r.stats()["status"] == PT_ERR_STACK_OVERFLOW
    monkeypatch.delenv("PT_TRAVERSAL_STACK_LIMIT")
    a, b, sa, sb = render_both(sd, 2)
    assert sa["status"] == 0 and sb["status"] == 0
    ref, _, _ = orc.render(sd, sd.render_options(), sd.pt_camera(), 0, 2)
    assert image_agreement(a, ref)[0] >= 0.99


def comb_scene(depth):
    """A flattened binary BVH written by hand, as a caller could pass it: a
    comb of `depth` internal nodes, each with one triangle leaf and the next
    internal node as children, every box containing the rest of the comb;
    one untransformed instance."""
    from pathtracer import scenes
    from pathtracer.scene import SceneData
    n = depth + 1  # triangles
    P = np.zeros((3 * n, 3))
    for i in range(n):
        P[3 * i:3 * i + 3] = [(i, 0, 0), (i + 0.5, 0, 0), (i, 0.5, 0)]
    V = np.c_[P, np.zeros(3 * n)].astype(np.float32)
    Nrm = np.tile([0.0, 0.0, 1.0, 0.0], (3 * n, 1)).astype(np.float32)
    idx = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    nodes = []
    # internal node k at index 2k, its triangle leaf at 2k+1, the last leaf at 2 depth
    for k in range(depth):
        lo, hi = (k, 0, 0), (n - 0.5, 0.5, 0)
        nodes.append([*lo, *hi, 2 * k + 1, 2 * k + 2 if k + 1 < depth else 2 * depth, 0])
        nodes.append([k, 0, 0, k + 0.5, 0.5, 0, k, 1, 1])
    nodes.append([depth, 0, 0, depth + 0.5, 0.5, 0, depth, 1, 1])
    top = len(nodes)
    nodes.append([0, 0, 0, n - 0.5, 0.5, 0, 0, 0, -1])  # TLAS leaf: BLAS root 0, material 0, instance 0
    cam = scenes.camera((n / 2, 0.25, 5.0), (n / 2, 0.25, 0.0), 40.0)
    return SceneData(bvh_nodes=np.array(nodes, np.float32), top_level_index=top, vert_indices=idx, vertices_uvx=V,
                     normals_uvy=Nrm, transforms=scenes.mat4().reshape(1, 16), materials=scenes.material()[None],
                     lights=scenes.sphere_light((0, 1, 3), 0.3, (5, 5, 5))[None],
                     options=dict(render_width=8, render_height=8, tile_width=8, tile_height=8, max_depth=2),
                     camera=cam)


def test_bvh_deeper_than_the_stack_is_rejected(ptlib):
    """A BVH whose traversal could need more stack entries than the kernels
    have is refused at pt_create with PT_ERR_UNSUPPORTED (the reference's
    64-entry GLSL stack overflows silently, closest_hit.glsl:89); a
    shallower comb is accepted and renders with status 0."""
    from pathtracer import capi
    from pathtracer.renderer import GpuRenderer
    with pytest.raises(capi.PTError) as e:
        GpuRenderer(comb_scene(1200))
    assert e.value.code == PT_ERR_UNSUPPORTED
    with GpuRenderer(comb_scene(40)) as r:
        r.render_passes(0, 1)
        assert r.stats()["status"] == 0
