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
"""
from __future__ import annotations

import ctypes as C
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


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "textured":
        print("textured golden written", textured_golden())
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
    print("golden fixtures written", out)


if __name__ == "__main__":
    main()
