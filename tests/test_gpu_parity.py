"""CUDA path (through the C ABI) against the oracle and the reference's
golden fixtures.  Needs a GPU.

Tolerances:
  * ray queries: triangle id, instance id and the distance t are compared
    exactly (the triangle test repeats the reference's float operations);
    a different triangle is accepted only at the same distance (a tie,
    |dt| <= 1e-6 t), or for a ray grazing an edge, where FP64 arithmetic
    finds the CUDA triangle valid within 1e-6 in barycentrics and no
    robustly valid triangle (barycentrics above 1e-6) closer
    (classify_mismatch); at most 1e-4 of the rays may fall in the second
    class, and none outside the two.
  * images: same seeds, so per-pixel agreement is expected up to the
    last-ulp differences of CUDA's and the host's math libraries, of FMA
    contraction and of the shading kernels' division (within 2 ulp, as
    GLSL allows), which can flip a discrete choice (Russian roulette, lobe
    selection) on a few samples: >= 99% of pixels within 1e-3 relative
    (1e-4 absolute) and the image means within 1e-3 relative.  A scene
    whose render is sensitive to rounding (the textured ground plane, 2000
    units wide with its map repeated 148 times, where a last-bit change of
    a secondary ray moves its texture lookup) is held to the agreement of
    the oracle's own FP64 render with the same reference, less 0.5% of the
    pixels, when that is below 99%.
"""
import numpy as np
import pytest

from conftest import golden, golden_scene

pytestmark = pytest.mark.gpu


def world_points_on_tris(sd, n, rng):
    """Random points on random triangles, in world space (instance
    transform): a random TLAS leaf, a random walk down its BLAS to a leaf, a
    random triangle of that leaf and a uniform point on it."""
    nodes, top = sd.bvh_nodes, sd.top_level_index
    idx = np.arange(top, nodes.shape[0])
    leaves = idx[nodes[idx, 8] < 0]
    li = leaves[rng.randint(len(leaves), size=n)]
    inst = (-nodes[li, 8] - 1).astype(np.int64)
    node = nodes[li, 6].astype(np.int64)
    inner = nodes[node, 8] == 0
    while inner.any():
        go_left = rng.rand(n) < 0.5
        child = np.where(go_left, nodes[node, 6], nodes[node, 7]).astype(np.int64)
        node = np.where(inner, child, node)
        inner = nodes[node, 8] == 0
    t = nodes[node, 6].astype(np.int64) + (rng.rand(n) * nodes[node, 7]).astype(np.int64)
    b = rng.dirichlet([1, 1, 1], n)
    V = sd.vertices_uvx[:, :3].astype(np.float64)
    P = sum(b[:, k:k + 1] * V[sd.vert_indices[t, k]] for k in range(3))
    M = sd.transforms[inst].reshape(-1, 4, 4).astype(np.float64)
    return np.einsum("ni,nij->nj", np.c_[P, np.ones(n)], M)[:, :3]


def ray_set(sd, orc, n, seed):
    rng = np.random.RandomState(seed)
    o = sd.render_options()
    W, H = o.render_width, o.render_height
    px = rng.randint(0, W, n // 2)
    py = rng.randint(0, H, n // 2)
    cam_rays, _ = orc.camera_rays(o, sd.pt_camera(), 0, px, py)
    P = world_points_on_tris(sd, n - n // 2, rng)
    d = rng.normal(size=P.shape)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    sec = orc.rays_array((P + d * 3e-4).astype(np.float32), d.astype(np.float32))
    return np.ascontiguousarray(np.concatenate([cam_rays, sec]), np.float32)


def scene_by_name(name):
    from pathtracer import scenes
    if name == "ref_cornell":
        return golden_scene("ref_scene_cornell_box_orig.npz")
    if name == "ref_volume":
        return golden_scene("ref_scene_volume_cube.npz")
    if name == "ref_textured":
        return golden_scene("ref_scene_textured.npz")
    if name == "cornell":
        return scenes.cornell(64, 64, tile=32)
    if name == "icosphere":
        return scenes.icosphere_scene(freq=60, width=96, height=64, tile=32)
    if name == "instanced":
        return scenes.instanced_scene(num_instances=300, tris_per_blas=3000, width=96, height=64,
                                      env_size=(256, 128), tile=32)
    raise KeyError(name)


SCENES = ["ref_cornell", "ref_volume", "ref_textured", "cornell", "icosphere", "instanced"]


def tri_fp64(sd, ray, prim, inst):
    """The ray against triangle `prim` of instance `inst` in FP64 (world ray
    taken to object space with the inverse of the instance's Mat4, as
    closest_hit.glsl:156-164 does): returns (t, smallest barycentric)."""
    M = sd.transforms[inst].reshape(4, 4).astype(np.float64)  # row-vector layout
    Mi = np.linalg.inv(M)
    o = np.r_[ray[:3].astype(np.float64), 1.0] @ Mi
    d = np.r_[ray[3:].astype(np.float64), 0.0] @ Mi
    v0, v1, v2 = (sd.vertices_uvx[sd.vert_indices[prim, k], :3].astype(np.float64) for k in range(3))
    e0, e1 = v1 - v0, v2 - v0
    pv = np.cross(d[:3], e1)
    det = np.dot(e0, pv)
    tv = o[:3] - v0
    qv = np.cross(tv, e0)
    with np.errstate(divide="ignore", invalid="ignore"):
        u, v, t = np.dot(tv, pv) / det, np.dot(d[:3], qv) / det, np.dot(e1, qv) / det
    return t, min(u, v, 1.0 - u - v)


BARY_EPS = 1e-6  # FP64 barycentric slack of a grazing hit
TIE_EPS = 1e-6   # relative t difference of a tie; also the t-epsilon at the ray origin, relative to |origin|


def classify_mismatch(sd, orc, rays, h_gpu, h_orc):
    """Rays whose closest hits differ, split three ways:
      ties      both hit, at the same FP32 distance within TIE_EPS relative;
      grazing   the GPU's answer is a closest hit in FP64 within BARY_EPS:
                its triangle is valid in FP64 up to BARY_EPS in
                barycentrics at t >= -TIE_EPS |origin| (a ray that starts
                on a triangle's plane hits it at t = 0, which the triangle
                test accepts and the reference's AABBIntersect, visiting
                boxes only at a distance > 0, may cull), or it reports a
                miss; and the oracle's triangle is not a robust FP64 hit
                (all barycentrics above BARY_EPS) that lies closer by more
                than a tie;
      bad       everything else.
    Returns (bad indices, number of ties, number of grazing rays)."""
    diff = (h_gpu["prim_id"] != h_orc["prim_id"]) | (h_gpu["inst_id"] != h_orc["inst_id"])
    tie = diff & (h_gpu["prim_id"] >= 0) & (h_orc["prim_id"] >= 0) & (
        np.abs(h_gpu["t"] - h_orc["t"]) <= TIE_EPS * np.abs(h_orc["t"]))
    bad, grazing = [], 0
    for i in np.where(diff & ~tie)[0]:
        g, o = h_gpu[i], h_orc[i]
        g_ok, tg = True, np.inf
        if g["prim_id"] >= 0:
            tg, bg = tri_fp64(sd, rays[i], int(g["prim_id"]), int(g["inst_id"]))
            g_ok = bg >= -BARY_EPS and tg >= -TIE_EPS * max(1.0, float(np.abs(rays[i, :3]).max()))
        o_better = False
        if o["prim_id"] >= 0:
            to, bo = tri_fp64(sd, rays[i], int(o["prim_id"]), int(o["inst_id"]))
            o_better = bo > BARY_EPS and to > 0 and to < tg * (1 - TIE_EPS)
        if g_ok and not o_better:
            grazing += 1
        else:
            bad.append(i)
    return np.array(bad, np.int64), int(tie.sum()), grazing


@pytest.mark.parametrize("name", SCENES)
def test_closest_hit_parity(ptlib, orc, name):
    from pathtracer.renderer import GpuRenderer
    sd = scene_by_name(name)
    rays = ray_set(sd, orc, 20000, 1)
    with GpuRenderer(sd) as r:
        hg = r.trace(rays)
    ho, cnt = orc.trace_closest(sd, rays, mode=0)
    assert cnt["overflow"] == 0
    bad, ties, grazing = classify_mismatch(sd, orc, rays, hg, ho)
    assert len(bad) == 0, (name, len(bad), ties, grazing, hg[bad[:5]], ho[bad[:5]])
    assert grazing <= max(2, int(1e-4 * len(rays))), (name, grazing)
    same = (hg["prim_id"] == ho["prim_id"]) & (hg["inst_id"] == ho["inst_id"])
    # identical triangle => identical float distance and barycentrics
    assert np.array_equal(hg["t"][same], ho["t"][same])
    assert np.array_equal(hg["u"][same], ho["u"][same])
    assert np.array_equal(hg["v"][same], ho["v"][same])
    assert (hg["prim_id"] >= 0).mean() > 0.3


@pytest.mark.parametrize("name", SCENES)
def test_any_hit_parity(ptlib, orc, name):
    from pathtracer.renderer import GpuRenderer
    sd = scene_by_name(name)
    rays = ray_set(sd, orc, 20000, 2)
    rng = np.random.RandomState(3)
    ho, _ = orc.trace_closest(sd, rays, mode=0)
    # max distances around the closest hit: just before, just after, far
    maxd = np.where(ho["prim_id"] >= 0, ho["t"] * rng.choice([0.5, 0.999, 1.001, 2.0], len(rays)), 1e5).astype(np.float32)
    o = sd.render_options()
    with GpuRenderer(sd) as r:
        og = r.shadow(rays, maxd)
    oo = orc.trace_any(sd, o, rays, maxd)
    diff = np.where(og != oo)[0]
    assert len(diff) <= max(2, int(1e-4 * len(rays))), (name, len(diff))


def pixel_bar(orc, sd, o, passes, ref):
    """The fraction of pixels a render must match `ref` on: 99%, or the
    agreement of the oracle's FP64 render with `ref` less 0.5% where the
    scene's own rounding sensitivity is above 1% of the pixels."""
    r64, _, _ = orc.render(sd, o, sd.pt_camera(), 0, passes, use_double=True)
    base, _ = image_agreement(r64, ref)
    return min(0.99, base - 0.005)


def image_agreement(a, b):
    rel = np.abs(a[..., :3] - b[..., :3]) / np.maximum(np.abs(b[..., :3]), 1e-1)
    ok = np.all((rel < 1e-3) | (np.abs(a[..., :3] - b[..., :3]) < 1e-4), axis=-1)
    mean_rel = abs(a[..., :3].mean() - b[..., :3].mean()) / max(b[..., :3].mean(), 1e-6)
    return ok.mean(), mean_rel


@pytest.mark.parametrize("name", SCENES)
def test_render_matches_oracle(ptlib, orc, name):
    from pathtracer.renderer import GpuRenderer
    sd = scene_by_name(name)
    o = sd.render_options()
    passes = 4
    with GpuRenderer(sd) as r:
        r.render_passes(0, passes)
        acc = r.accum()
        st = r.stats()
    ref, _, cnt = orc.render(sd, o, sd.pt_camera(), 0, passes)
    frac, mean_rel = image_agreement(acc, ref)
    assert st["status"] == 0
    assert st["paths"] == o.render_width * o.render_height * passes
    assert frac >= pixel_bar(orc, sd, o, passes, ref), (name, frac)
    assert mean_rel < 1e-3, (name, mean_rel)
    assert np.array_equal(acc[..., 3], ref[..., 3])
    total_gpu = st["closest"] + st["shadow"]
    total_orc = cnt["closest"] + cnt["shadow"]
    assert abs(total_gpu - total_orc) <= 0.01 * total_orc


@pytest.mark.parametrize("name,scene_file", [
    ("cornell_box_orig", "ref_scene_cornell_box_orig.npz"),
    ("volume_cube", "ref_scene_volume_cube.npz"),
    ("cornell_c1_48", "scene_cornell_c1_48.npz"),
    ("textured", "ref_scene_textured.npz"),
])
def test_render_matches_reference_shaders(ptlib, orc, name, scene_file):
    """Against the accumulation of the reference's own shader source."""
    from pathtracer.renderer import GpuRenderer
    sd = golden_scene(scene_file)
    g = golden(f"ref_render_{name}.npz")
    o = sd.render_options(render_width=int(g["width"]), render_height=int(g["height"]),
                          tile_width=int(g["tile_w"]), tile_height=int(g["tile_h"]))
    with GpuRenderer(sd, o) as r:
        r.render_passes(0, int(g["passes"]))
        acc = r.accum()
    frac, mean_rel = image_agreement(acc, g["accum"])
    bar = pixel_bar(orc, sd, o, int(g["passes"]), g["accum"])
    assert frac >= bar and mean_rel < 1e-3, (name, frac, bar, mean_rel)


@pytest.mark.parametrize("name", SCENES)
def test_wavefront_equals_megakernel(ptlib, name):
    """The wavefront form renders every path as the megakernel does: the same
    ray counts, and the same accumulation up to last-bit rounding."""
    from pathtracer import capi
    from pathtracer.renderer import GpuRenderer
    sd = scene_by_name(name)
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
    assert sa["truncated"] == sb["truncated"]
    assert sa["closest"] + sa["shadow"] == sb["closest"] + sb["shadow"]
    # the same paths, samples and accumulation order; the two kernels are
    # compiled separately, so the compiler's fused multiply-adds in the
    # shading code can differ in the last bit of a sample
    assert np.array_equal(a[..., 3], b[..., 3])
    rel = np.abs(a[..., :3] - b[..., :3]) / np.maximum(np.abs(b[..., :3]), 1e-3)
    assert rel.max() < 1e-4 and np.mean(rel) < 1e-6, (rel.max(), np.mean(rel))


def test_untraced_shadow_queries(ptlib):
    """Both integrators answer shadow queries whose contribution is never
    added (the scattering pdf towards the light is 0: lights below an opaque
    surface) without traversal; they still count as shadow queries, so the
    totals are equal, and the accumulation is the megakernel's."""
    from pathtracer import capi
    from pathtracer.renderer import GpuRenderer
    sd = scene_by_name("icosphere")
    with GpuRenderer(sd) as r:
        r.render_passes(0, 2)
        a = r.accum()
        sa = r.stats()
        r.clear()
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        r.render_passes(0, 2)
        b = r.accum()
        sb = r.stats()
    assert sa["status"] == 0 and sb["status"] == 0
    assert 0 < sa["untraced"] < sa["shadow"], sa
    assert 0 < sb["untraced"] < sb["shadow"], sb
    assert sa["closest"] + sa["shadow"] == sb["closest"] + sb["shadow"]
    assert np.array_equal(a[..., 3], b[..., 3])
    rel = np.abs(a[..., :3] - b[..., :3]) / np.maximum(np.abs(b[..., :3]), 1e-3)
    assert rel.max() < 1e-4 and np.mean(rel) < 1e-6, (rel.max(), np.mean(rel))


@pytest.mark.parametrize("name,integrator", [
    ("icosphere", "wavefront"), ("icosphere", "megakernel"), ("instanced", "wavefront"), ("instanced", "megakernel"),
    ("ref_volume", "wavefront"), ("ref_volume", "megakernel"),
])
def test_untraced_queries_change_nothing(ptlib, monkeypatch, name, integrator):
    """Shadow and transmittance queries answered without traversal change no
    result: the accumulation is bit for bit the one with every query traced
    (PT_UNTRACED_SHADOWS=0), and the query counts are the same."""
    from pathtracer import capi
    from pathtracer.renderer import GpuRenderer
    sd = scene_by_name(name)
    with GpuRenderer(sd) as r:
        if integrator == "wavefront":
            r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        monkeypatch.setenv("PT_UNTRACED_SHADOWS", "0")
        r.render_passes(0, 2)
        a = r.accum()
        sa = r.stats()
        r.clear()
        monkeypatch.delenv("PT_UNTRACED_SHADOWS")
        r.render_passes(0, 2)
        b = r.accum()
        sb = r.stats()
    assert sa["status"] == 0 and sb["status"] == 0
    assert sa["untraced"] == 0
    if name != "ref_volume":  # the icosphere's far side; VOL_MIS queries beside the blended volume
        assert sb["untraced"] > 0, sb
    assert np.array_equal(a, b)
    assert sa["closest"] == sb["closest"] and sa["shadow"] == sb["shadow"], (sa, sb)


def test_wavefront_batches_and_tiles(ptlib, monkeypatch):
    """Small wavefront batches (several batches per call, one pass each) and
    single tiles give the megakernel's accumulation."""
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuRenderer
    monkeypatch.setenv("PT_WAVEFRONT_CAPACITY", str(80 * 48))
    sd = scenes.cornell(80, 48, tile=32)
    with GpuRenderer(sd) as r:
        r.render_passes(0, 3)
        a = r.accum()
        r.clear()
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        r.render_passes(0, 3)
        b = r.accum()
        r.clear()
        frame = 2
        for _ in range(3):
            for ty in range(1, -1, -1):
                for tx in range(3):
                    r.render_tile(tx, ty, frame)
                    frame += 1
        c = r.accum()
    assert np.array_equal(a, b)
    assert np.array_equal(a, c)


def test_tiles_equal_whole_passes(ptlib):
    """pt_render_tile in the reference's tile order (Renderer.cpp:745-762)
    gives the same accumulation, bit for bit, as pt_render_passes."""
    from pathtracer import scenes
    from pathtracer.renderer import GpuRenderer
    sd = scenes.cornell(80, 48, tile=32)  # ragged last tile column/row
    o = sd.render_options()
    ntx, nty = (80 + 31) // 32, (48 + 31) // 32
    with GpuRenderer(sd) as r:
        r.render_passes(0, 2)
        a = r.accum()
        r.clear()
        frame = 2
        for _ in range(2):
            for ty in range(nty - 1, -1, -1):
                for tx in range(ntx):
                    r.render_tile(tx, ty, frame)
                    frame += 1
        b = r.accum()
    assert np.array_equal(a, b)


@pytest.mark.parametrize("integrator", [0, 1])
def test_checkpoint_resume_is_bit_exact(ptlib, integrator):
    """Checkpoint / resume: passes 0-2 on one context, its accumulation
    saved (pt_get_accum) and loaded into a fresh context (pt_set_accum),
    passes 3-4 rendered there -- the same accumulation, bit for bit, as
    passes 0-4 on one context."""
    from pathtracer import scenes
    from pathtracer.renderer import GpuRenderer
    sd = scenes.cornell(48, 40, tile=16)
    with GpuRenderer(sd) as r:
        r.set_integrator(integrator)
        r.render_passes(0, 5)
        whole = r.accum()
        r.clear()
        r.render_passes(0, 3)
        saved = r.accum()
    with GpuRenderer(sd) as r2:
        r2.set_integrator(integrator)
        r2.set_accum(saved)
        r2.render_passes(3, 2)
        resumed = r2.accum()
    assert np.array_equal(resumed, whole)


def test_tonemap_output(ptlib, orc):
    """pt_get_output against tonemap.glsl restated in numpy (Reinhard on
    luminance with limit 1.5, gamma 1/2.2, RGBA8 round-half-up)."""
    from pathtracer import scenes
    from pathtracer.renderer import GpuRenderer
    sd = scenes.cornell(64, 64)
    with GpuRenderer(sd) as r:
        r.render_passes(0, 3)
        acc = r.accum()
        ldr = r.output(3)
        r.snapshot()
        r.render_passes(3, 1)
        snap = r.output(3, from_snapshot=True)
    c = acc[..., :3].astype(np.float32) * np.float32(1.0 / 3.0)
    lum = (np.float32(0.212671) * c[..., 0] + np.float32(0.715160) * c[..., 1]) + np.float32(0.072169) * c[..., 2]
    c = c / (np.float32(1.0) + lum / np.float32(1.5))[..., None]
    c = np.power(np.maximum(c, 0), np.float32(1.0 / 2.2))
    exp = np.floor(np.clip(c, 0, 1) * 255 + 0.5).astype(np.int32)
    assert np.abs(ldr[..., :3].astype(np.int32) - exp).max() <= 1
    assert np.all(ldr[..., 3] == 255)
    assert np.array_equal(snap, ldr)


def test_z_test_converged(ptlib, orc):
    """Independent sample sets (oracle passes 0-63, CUDA passes 64-127) agree
    within the Monte Carlo noise: per-pixel z-scores."""
    from pathtracer import scenes
    from pathtracer.renderer import GpuRenderer
    sd = scenes.cornell(32, 32, tile=32)
    o = sd.render_options()
    n = 64
    ref, sq, _ = orc.render(sd, o, sd.pt_camera(), 0, n, with_sq=True)
    # per-pass read-back gives the CUDA side's own sample variance
    sq_c = np.zeros_like(sq, dtype=np.float64)
    with GpuRenderer(sd) as r:
        prev = np.zeros((32, 32, 4), np.float32)
        for k in range(n):
            r.render_passes(n + k, 1)
            a = r.accum()
            s = (a - prev)[..., :3].astype(np.float64)
            sq_c += s * s
            prev = a
        acc = prev
    mu_r = ref[..., :3] / n
    mu_c = acc[..., :3].astype(np.float64) / n
    var_r = np.maximum(sq / n - mu_r ** 2, 0)
    var_c = np.maximum(sq_c / n - mu_c ** 2, 0)
    se = np.sqrt((var_r + var_c) / n)
    ok = se > 1e-6
    z = (mu_c - mu_r)[ok] / se[ok]
    assert abs(z.mean()) < 0.1, z.mean()
    assert (np.abs(z) > 4).mean() < 2e-3


def test_error_paths(ptlib):
    """Bad arguments come back as PT_ERR_* codes with a message."""
    import ctypes as C
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuRenderer
    lib = ptlib
    sd = scenes.cornell(16, 16)
    with GpuRenderer(sd) as r:
        assert lib.pt_render_tile(r.ctx, 99, 0, 2) == capi.PT_ERR_INVALID_ARG
        assert lib.pt_render_passes(r.ctx, -1, 1) == capi.PT_ERR_INVALID_ARG
        assert lib.pt_set_integrator(r.ctx, 7) == capi.PT_ERR_INVALID_ARG
    bad = scenes.cornell(16, 16)
    bad.materials[1, 24] = 0.0  # a texture map id, in a scene without texture maps
    with pytest.raises(capi.PTError) as e:
        GpuRenderer(bad)
    assert e.value.code == capi.PT_ERR_INVALID_ARG
    bad2 = scenes.cornell(16, 16)
    bad2.bvh_nodes[bad2.top_level_index, 6] = 10 ** 6  # child index out of range
    with pytest.raises(capi.PTError) as e:
        GpuRenderer(bad2)
    assert e.value.code == capi.PT_ERR_INVALID_ARG
