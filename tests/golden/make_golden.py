"""Generate the golden fixtures of tests/golden/ from the reference itself.

Run in a container that has the reference source (path in REF below) after
`make -C oracle ref`; the GPU machines only read the .npz files this writes.

  ref_scene_<name>.npz   arrays produced by the reference's own loader, BVH
                         build and BvhTranslator flattening (oracle/_ref/ref_scene_dump)
  ref_render_<name>.npz  accumulations from the reference's own shader source
                         compiled for the CPU (oracle/_ref/libref_glsl_<variant>.so)
  ref_bsdf.npz           reference DisneyEval on random shading states
  ref_closest.npz        reference ClosestHit (lights + BVH) on ray sets
  ref_scene_textured.npz / ref_render_textured.npz
                         a textured scene of this project's (every texture
                         slot, alpha blend) rendered by the reference
  feature_scene_<case>.npz / ref_render_features.npz
                         small scenes of this project's, one per render
                         option, light type and medium type the reference
                         decides per scene (Renderer.cpp:400-476), rendered
                         by the reference shaders with that macro set
  ref_tonemap.npz        the reference's tonemap.glsl on one accumulation
                         with every tonemap / background combination
  ref_tree_counts.json   traversal work per ray on the reference's own BVH
                         (its loader, RadeonRays SBVH and BvhTranslator) and
                         on this project's builder, for the icosphere and
                         instanced workloads at full size: the source of the
                         algorithmic bytes per ray of the roofline
Usage: python make_golden.py [textured | features | trees]
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "glsl-pathtracer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import orc  # noqa: E402
from pathtracer import capi, scenes  # noqa: E402
from pathtracer.scene import SceneData, load_ref_dump  # noqa: E402

REF = os.environ.get("PT_REFERENCE_DIR", "/root/reference")

# (scene file, render size, tile size, passes)
REF_SCENES = {
    "cornell_box_orig": ((64, 48), (20, 16), 4),
    "volume_cube": ((64, 36), (32, 18), 4),
}


def bsdf_inputs(n: int, seed: int):
    """Random shading states (20-float records of orc_bsdf_eval) and V, N, L."""
    rng = np.random.RandomState(seed)
    sp = np.zeros((n, 20), np.float32)
    lobe = rng.randint(0, 6, n)  # bias towards single-lobe materials too
    sp[:, 0:3] = rng.uniform(0, 1, (n, 3))
    sp[:, 3] = np.where(lobe == 1, 1.0, np.where(lobe == 0, 0.0, rng.uniform(0, 1, n)))
    rough = rng.uniform(0.05, 1.0, n)
    sp[:, 4] = rough
    sp[:, 5] = rng.uniform(0, 1, n)
    sp[:, 6] = rng.uniform(0, 1, n)
    sp[:, 7] = rng.uniform(0, 1, n)
    sp[:, 8] = rng.uniform(0, 1, n)
    sp[:, 9] = np.where(lobe == 3, 1.0, rng.uniform(0, 1, n))
    sp[:, 10] = 0.1 * (1 - rng.uniform(0, 1, n)) + 0.001 * rng.uniform(0, 1, n)
    sp[:, 11] = np.where(lobe == 2, 1.0, np.where(lobe == 4, rng.uniform(0, 1, n), 0.0))
    sp[:, 12] = rng.uniform(1.1, 2.0, n)
    aniso = rng.uniform(0, 1, n) * (lobe == 5)
    aspect = np.sqrt(1 - aniso * 0.9)
    sp[:, 13] = np.maximum(0.001, rough / aspect)
    sp[:, 14] = np.maximum(0.001, rough * aspect)
    entering = rng.uniform(0, 1, n) < 0.5
    sp[:, 15] = np.where(entering, 1.0 / sp[:, 12], sp[:, 12])
    sp[:, 16] = aniso

    def unit(k):
        v = rng.normal(size=(k, 3))
        return v / np.linalg.norm(v, axis=1, keepdims=True)

    N = unit(n).astype(np.float32)
    V = unit(n)
    V = np.where((np.sum(V * N, 1) < 0)[:, None], -V, V).astype(np.float32)  # view on the normal side
    L = unit(n).astype(np.float32)
    return sp, V, N, L


def closest_rays(sd: SceneData, n: int, seed: int):
    """Camera-like rays from the scene camera plus rays from random points on
    triangles in random directions (offset by EPS along the direction)."""
    rng = np.random.RandomState(seed)
    cam = sd.camera
    pos = np.array(cam["position"], np.float32)
    half = n // 2
    d = (np.array(cam["forward"]) + rng.uniform(-0.6, 0.6, (half, 1)) * np.array(cam["right"]) +
         rng.uniform(-0.4, 0.4, (half, 1)) * np.array(cam["up"]))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o1 = np.tile(pos, (half, 1))
    t = rng.randint(0, sd.num_tris, n - half)
    b = rng.dirichlet([1, 1, 1], n - half)
    vi = sd.vert_indices[t]
    P = sum(b[:, k:k + 1] * sd.vertices_uvx[vi[:, k], :3] for k in range(3))
    # the BLAS vertices are object space: move to world space with the owning instance
    # (only identity-transform scenes are used for this set)
    d2 = rng.normal(size=(n - half, 3))
    d2 /= np.linalg.norm(d2, axis=1, keepdims=True)
    o2 = P + d2 * 3e-4
    return orc.rays_array(np.concatenate([o1, o2]).astype(np.float32), np.concatenate([d, d2]).astype(np.float32))


# A textured scene of this project's own, rendered by the reference: the
# quad and checker texture of the reference's teapot assets (loaded through
# relative paths from a scratch directory) under every texture slot, an
# alpha-blended textured veil, and a quad light.  Texture array 64 x 64.
TEXTURED_SCENE = """renderer
{{
    resolution 64 48
    maxdepth 3
    tilewidth 32
    tileheight 24
    texarraywidth 64
    texarrayheight 64
}}
camera
{{
    position 0 6 12
    lookat 0 0 0
    fov 45
}}
light
{{
    type quad
    position -2 8 -2
    v1 2 8 -2
    v2 -2 8 2
    emission 30 30 30
}}
material floor
{{
    albedotexture {a}/checker.png
    metallicroughnesstexture {a}/checker.png
    normaltexture {a}/checker.png
    roughness 0.5
}}
material veil
{{
    albedotexture {a}/checker.png
    alphamode blend
    opacity 0.5
}}
material glow
{{
    color 0.8 0.8 0.8
    emissiontexture {a}/checker.png
}}
mesh
{{
    file {a}/Mesh050.obj
    material floor
    scale 0.01 0.01 0.01
}}
mesh
{{
    file {a}/Mesh050.obj
    material veil
    scale 0.002 0.002 0.002
    position 0 1 0
}}
mesh
{{
    file {a}/Mesh050.obj
    material glow
    scale 0.001 0.001 0.001
    position 3 0.5 -3
}}
"""


def textured_golden():
    with tempfile.TemporaryDirectory() as td:
        rel = os.path.relpath(os.path.join(REF, "assets", "teapot"), td)
        path = os.path.join(td, "textured.scene")
        with open(path, "w") as fh:
            fh.write(TEXTURED_SCENE.format(a=rel))
        orc.ref_dump_scene(path, os.path.join(td, "textured"))
        sd = load_ref_dump(os.path.join(td, "textured"))
    sd.save_npz(os.path.join(HERE, "ref_scene_textured.npz"))
    o = sd.render_options()
    variant = orc.variant_for(sd, o)
    acc = orc.ref_render(variant, sd, o, sd.pt_camera(), 0, 4)
    np.savez_compressed(os.path.join(HERE, "ref_render_textured.npz"), accum=acc, passes=4, width=64, height=48,
                        tile_w=32, tile_h=24, variant=variant)
    return float(acc[..., :3].mean())


def distant_light(direction, emission) -> np.ndarray:
    """Loader.cpp:198-202: a distant light keeps its position (read as the
    direction towards the light, sampling.glsl:229-236) and area 0."""
    L = np.zeros(15, np.float32)
    L[0:3], L[3:6] = direction, emission
    L[14] = 2
    return L


# case -> (option overrides, lights, environment map, medium cube: (type,
# density, color, blended boundary) or None)
FEATURE_CASES = {
    "uniform_light": (dict(enable_uniform_light=1, uniform_light_col=(0.3, 0.4, 0.5)), ("quad",), False, None),
    "uniform_light_env": (dict(enable_uniform_light=1, uniform_light_col=(0.3, 0.4, 0.5)), ("quad",), True, None),
    "hide_emitters": (dict(hide_emitters=1), ("quad", "sphere"), True, None),
    "background": (dict(enable_background=1, background_col=(0.2, 0.4, 0.8)), ("quad",), True, None),
    "transparent_background": (dict(transparent_background=1), ("quad",), False, None),
    "mollification": (dict(enable_roughness_mollification=1, roughness_mollification_amt=0.7), ("quad",), True,
                      None),
    "rr_off": (dict(enable_rr=0, max_depth=6), ("quad",), False, None),
    "rr_depth_1": (dict(rr_depth=1), ("quad", "sphere"), False, None),
    "env_only": (dict(envmap_rot=40.0, envmap_intensity=1.5), (), True, None),
    "distant": (dict(), ("distant", "sphere"), False, None),
    "distant_only": (dict(), ("distant",), True, None),
    "absorb": (dict(), ("quad",), False, (1, 0.8, (0.3, 0.6, 0.9), False)),
    "absorb_volmis": (dict(enable_volume_mis=1), ("quad",), False, (1, 0.8, (0.3, 0.6, 0.9), False)),
    "emissive": (dict(), ("quad",), False, (3, 0.5, (0.5, 0.8, 1.0), True)),
    "emissive_volmis": (dict(enable_volume_mis=1), ("quad", "sphere"), True, (3, 0.5, (0.5, 0.8, 1.0), False)),
    "all_flags": (dict(hide_emitters=1, enable_background=1, enable_uniform_light=1, rr_depth=1,
                       enable_roughness_mollification=1, roughness_mollification_amt=0.5, opengl_normal_map=0),
                  ("quad",), False, None),
}
FEATURE_SIZE = dict(render_width=48, render_height=36, tile_width=24, tile_height=18, max_depth=5)
FEATURE_PASSES = 4


def feature_scene(case):
    """Ground quad, a glossy clear-coated sphere, a glass sphere, a cube (a
    medium boundary in the medium cases, else diffuse), an emissive quad in
    view and the case's lights: a rect light facing the camera from behind
    the objects, a sphere light, a distant light."""
    over, lights, env, medium = FEATURE_CASES[case]
    V, Fc, _ = scenes.icosphere(5, 1.0, 0.0, 1)
    meshes = [scenes.quad_mesh((-5, 0, -5), (-5, 0, 5), (5, 0, 5), (5, 0, -5), (0, 1, 0)),
              scenes.mesh_from_indexed(V, Fc), scenes.cube_mesh(),
              scenes.quad_mesh((-0.4, 0, 0), (0.4, 0, 0), (0.4, 0.5, 0), (-0.4, 0.5, 0), (0, 0, 1))]
    mats = [scenes.material(),
            scenes.material(color=(0.7, 0.7, 0.7), roughness=0.9),
            scenes.material(color=(0.9, 0.5, 0.3), metallic=0.7, roughness=0.15, clearcoat=0.6,
                            clearcoat_gloss=0.8),
            scenes.material(color=(1, 1, 1), spec_trans=1.0, roughness=0.02, ior=1.45),
            scenes.material(color=(0.4, 0.6, 0.3), roughness=0.6, sheen=0.5),
            scenes.material(color=(0.8, 0.8, 0.8), emission=(3.0, 2.5, 2.0))]
    if medium is not None:
        mtype, dens, mcol, blend = medium
        mats[4] = scenes.material(color=(1, 1, 1), spec_trans=1.0, roughness=0.0, ior=1.0 if blend else 1.2,
                                  medium_type=mtype, medium_density=dens, medium_color=mcol,
                                  alpha_mode=1 if blend else 0, opacity=0.0 if blend else 1.0)
    inst = [(0, 1, scenes.mat4()),
            (1, 2, scenes.mat4(None, (0.8, 0.8, 0.8), (-1.3, 0.8, 0.0))),
            (1, 3, scenes.mat4(None, (0.6, 0.6, 0.6), (1.2, 0.6, 0.6))),
            (2, 4, scenes.mat4(scenes.rot_y(25.0), (1.0, 1.0, 1.0), (0.3, 0.51, -1.3))),
            (3, 5, scenes.mat4(None, (1, 1, 1), (1.6, 0.0, -2.2)))]
    lts = []
    for kind in lights:
        if kind == "quad":  # faces the camera (+z), behind the objects
            lts.append(scenes.quad_light((-1.0, 1.2, -3.0), (1.0, 1.2, -3.0), (-1.0, 2.2, -3.0), (6.0, 5.5, 5.0)))
        elif kind == "sphere":
            lts.append(scenes.sphere_light((2.0, 3.0, 2.5), 0.35, (20.0, 18.0, 16.0)))
        elif kind == "distant":
            lts.append(distant_light((0.4, 0.8, 0.45), (2.0, 1.9, 1.7)))
    opts = dict(FEATURE_SIZE)
    opts.update(over)
    envmap = scenes.sky_envmap(64, 32, sun_dir=(-0.5, 0.6, 0.2), sun_radius_deg=8.0, sun_intensity=40.0) if env \
        else None
    if env:
        opts["enable_envmap"] = 1
    cam = scenes.camera((0.0, 1.8, 5.5), (0.0, 0.7, 0.0), 45.0)
    return scenes.build_scene(meshes, inst, mats, lts, cam, opts, envmap=envmap)


def feature_goldens():
    """One scene per feature case and its reference render; the reference's
    tonemap.glsl on the background case's accumulation."""
    out, renders = {}, {}
    for case in FEATURE_CASES:
        sd = feature_scene(case)
        o = sd.render_options()
        variant = orc.variant_for(sd, o)
        acc = orc.ref_render(variant, sd, o, sd.pt_camera(), 0, FEATURE_PASSES)
        sd.save_npz(os.path.join(HERE, f"feature_scene_{case}.npz"))
        renders[f"{case}_accum"] = acc
        renders[f"{case}_variant"] = np.frombuffer(variant.encode(), np.uint8)
        out[case] = (variant, float(acc[..., :3].mean()), float(acc[..., 3].mean()))
    # the reference's textured scene with DirectX-convention normal maps
    sd = SceneData.load_npz(os.path.join(HERE, "ref_scene_textured.npz"))
    sd.options = dict(sd.options, opengl_normal_map=0)
    o = sd.render_options()
    variant = orc.variant_for(sd, o)
    g = np.load(os.path.join(HERE, "ref_render_textured.npz"))
    o = sd.render_options(render_width=int(g["width"]), render_height=int(g["height"]),
                          tile_width=int(g["tile_w"]), tile_height=int(g["tile_h"]))
    sd.options = capi.options_dict(o)
    acc = orc.ref_render(variant, sd, o, sd.pt_camera(), 0, FEATURE_PASSES)
    sd.save_npz(os.path.join(HERE, "feature_scene_textured_dx.npz"))
    renders["textured_dx_accum"] = acc
    renders["textured_dx_variant"] = np.frombuffer(variant.encode(), np.uint8)
    out["textured_dx"] = (variant, float(acc[..., :3].mean()), float(acc[..., 3].mean()))
    np.savez_compressed(os.path.join(HERE, "ref_render_features.npz"), passes=FEATURE_PASSES, **renders)
    # tonemap.glsl: every tonemap branch with and without (transparent) background
    acc = renders["background_accum"]
    H, W = acc.shape[:2]
    import json
    tm = {"accum": acc, "samples": FEATURE_PASSES,
          "cases": np.frombuffer(json.dumps(TONEMAP_CASES).encode(), np.uint8)}
    for name, kw in TONEMAP_CASES.items():
        o = capi.make_options(render_width=W, render_height=H, background_col=(0.2, 0.4, 0.8), **kw)
        tm[name] = orc.ref_tonemap(acc, FEATURE_PASSES, o, W, H)
    np.savez_compressed(os.path.join(HERE, "ref_tonemap.npz"), **tm)
    return out


TONEMAP_CASES = {
    "reinhard": dict(enable_tonemap=1),
    "aces": dict(enable_tonemap=1, enable_aces=1),
    "aces_simple": dict(enable_tonemap=1, enable_aces=1, simple_aces_fit=1),
    "none": dict(enable_tonemap=0),
    "reinhard_background": dict(enable_tonemap=1, enable_background=1),
    "aces_background": dict(enable_tonemap=1, enable_aces=1, enable_background=1),
    "reinhard_transparent": dict(enable_tonemap=1, transparent_background=1),
    "aces_simple_transparent": dict(enable_tonemap=1, enable_aces=1, simple_aces_fit=1, transparent_background=1),
}


# ------------------------------------------------- reference BVH work counts
def _obj_text(mesh) -> str:
    """A non-indexed mesh as OBJ text: one v / vn per corner, faces in
    order (the reference loader keeps OBJ faces as corner triples,
    Mesh.cpp:65-101).  %.9g round-trips float32."""
    P, N = mesh.verts[:, :3], mesh.norms[:, :3]
    out = ["v %.9g %.9g %.9g\n" % tuple(p) for p in P]
    out += ["vn %.9g %.9g %.9g\n" % tuple(n) for n in N]
    out += ["f %d//%d %d//%d %d//%d\n" % (3 * i + 1, 3 * i + 1, 3 * i + 2, 3 * i + 2, 3 * i + 3, 3 * i + 3)
            for i in range(mesh.num_tris)]
    return "".join(out)


def reference_scene_dump(recipe: dict, td: str, name: str) -> SceneData:
    """Write a recipe's meshes and instances as a .scene file (Loader.cpp's
    mesh blocks, one per instance, the transform as a `matrix` line), run the
    reference's loader, BVH build and flattening on it, and return the
    result with this project's materials, lights, environment map, camera
    and options (the reference loader prepends a default material, so its
    ids are this project's plus one)."""
    mats = recipe["materials"]
    lines = ["renderer\n{\n resolution 64 64\n}\n"]
    for k in range(len(mats)):
        lines.append(f"material m{k}\n{{\n color 1 1 1\n}}\n")
    for k, mesh in enumerate(recipe["meshes"]):
        with open(os.path.join(td, f"{name}_{k}.obj"), "w") as fh:
            fh.write(_obj_text(mesh))
    for mesh_id, mat_id, xf in recipe["instances"]:
        # Loader.cpp:409-414 reads `matrix` row by row into xform[col][row]
        m = np.asarray(xf, np.float32).reshape(4, 4).T.ravel()
        lines.append(f"mesh\n{{\n file {name}_{mesh_id}.obj\n material m{mat_id}\n matrix "
                     + " ".join("%.9g" % v for v in m) + "\n}\n")
    path = os.path.join(td, name + ".scene")
    with open(path, "w") as fh:
        fh.write("".join(lines))
    orc.ref_dump_scene(path, os.path.join(td, name))
    rd = load_ref_dump(os.path.join(td, name))
    ours = scenes.build_scene(**recipe)
    assert np.array_equal(rd.transforms, ours.transforms), "transforms differ"
    assert rd.materials.shape[0] == len(mats) + 1
    rd.materials = np.concatenate([rd.materials[:1], ours.materials])
    rd.lights = ours.lights
    rd.envmap_rgb, rd.envmap_cdf, rd.envmap_total_sum = ours.envmap_rgb, ours.envmap_cdf, ours.envmap_total_sum
    rd.options, rd.camera = ours.options, ours.camera
    return rd, ours


# the row sample bench.py's roofline counts on (every 64th row, 2 passes)
TREE_SAMPLE = dict(row_step=64, passes=2)
TREE_WORKLOADS = {
    "icosphere_1m": lambda: scenes.icosphere_recipe(),
    "instanced": lambda: scenes.instanced_recipe(),
}


def tree_counts() -> dict:
    """Oracle traversal counters (tmax-culled, as bench.py counts them) on
    the reference's BVH and on this project's, same rays and paths."""
    out = {"sample": TREE_SAMPLE}
    for name, make in TREE_WORKLOADS.items():
        recipe = make()
        with tempfile.TemporaryDirectory() as td:
            rd, ours = reference_scene_dump(recipe, td, name)
        res = {}
        for tree, sd in (("reference", rd), ("ours", ours)):
            _, _, c = orc.render(sd, ours.render_options(), ours.pt_camera(), 0, TREE_SAMPLE["passes"],
                                 row_step=TREE_SAMPLE["row_step"], cull=True)
            c["binary_nodes"] = int(sd.bvh_nodes.shape[0])
            res[tree] = c
        out[name] = res
        print(name, res)
    with open(os.path.join(HERE, "ref_tree_counts.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    return out


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "trees":
        tree_counts()
        return
    if len(sys.argv) > 1 and sys.argv[1] == "textured":
        print("textured golden written", textured_golden())
        return
    if len(sys.argv) > 1 and sys.argv[1] == "features":
        for k, v in feature_goldens().items():
            print(k, v)
        return
    if not orc.ref_available():
        raise SystemExit("oracle/_ref not built: run `make -C oracle ref` first")
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for name, (res, tile, passes) in REF_SCENES.items():
            orc.ref_dump_scene(os.path.join(REF, "assets", name + ".scene"), os.path.join(td, name))
            sd = load_ref_dump(os.path.join(td, name))
            sd.save_npz(os.path.join(HERE, f"ref_scene_{name}.npz"))
            o = sd.render_options(render_width=res[0], render_height=res[1], tile_width=tile[0],
                                  tile_height=tile[1])
            variant = orc.variant_for(sd, o)
            acc = orc.ref_render(variant, sd, o, sd.pt_camera(), 0, passes)
            np.savez_compressed(os.path.join(HERE, f"ref_render_{name}.npz"), accum=acc, passes=passes,
                                width=res[0], height=res[1], tile_w=tile[0], tile_h=tile[1], variant=variant)
            out[name] = float(acc[..., :3].mean())
    # procedural Cornell (this project's scene builder) rendered by the reference shaders
    sd = scenes.cornell(48, 48, max_depth=4, tile=16)
    o = sd.render_options()
    acc = orc.ref_render(orc.variant_for(sd, o), sd, o, sd.pt_camera(), 0, 4)
    sd.save_npz(os.path.join(HERE, "scene_cornell_c1_48.npz"))
    np.savez_compressed(os.path.join(HERE, "ref_render_cornell_c1_48.npz"), accum=acc, passes=4, width=48, height=48,
                        tile_w=16, tile_h=16, variant=orc.variant_for(sd, o))
    # BSDF
    sp, V, N, L = bsdf_inputs(4096, 7)
    lib = orc.ref_glsl("lights")
    f = np.zeros((len(sp), 3), np.float32)
    pdf = np.zeros(len(sp), np.float32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    lib.ref_glsl_disney_eval(len(sp), p(sp), p(V), p(N), p(L), p(f), p(pdf))
    np.savez_compressed(os.path.join(HERE, "ref_bsdf.npz"), state=sp, V=V, N=N, L=L, f=f, pdf=pdf)
    # ClosestHit on the reference-built Cornell (identity instance transforms? no: scaled) via camera rays only
    res = {}
    for name in REF_SCENES:
        sd = SceneData.load_npz(os.path.join(HERE, f"ref_scene_{name}.npz"))
        rays = closest_rays(sd, 2048, 11)[:1024]  # camera-ray half: world-space origins
        n = rays.shape[0]
        hit = np.zeros(n, np.int32); t = np.zeros(n, np.float32); mat = np.zeros(n, np.int32)
        emi = np.zeros(n, np.int32); nrm = np.zeros((n, 3), np.float32)
        d = sd.desc()
        lib = orc.ref_glsl(orc.variant_for(sd, sd.render_options()))
        lib.ref_glsl_closest_hit(C.byref(d), p(rays), n, p(hit), p(t), p(mat), p(emi), p(nrm))
        res[name] = dict(rays=rays, hit=hit, t=t, mat=mat, emitter=emi, normal=nrm)
    np.savez_compressed(os.path.join(HERE, "ref_closest.npz"),
                        **{f"{k}_{f}": v for k, r in res.items() for f, v in r.items()})
    out["textured"] = textured_golden()
    out["features"] = feature_goldens()
    tree_counts()
    print("golden fixtures written", out)


if __name__ == "__main__":
    main()
