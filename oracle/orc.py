"""Python binding of the CPU oracle (liborc.so) and of the reference builds
under oracle/_ref/ (present only where the reference source was available).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline / reference legs, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")
REF_DIR = os.path.join(HERE, "_ref")

_lib = None


def build(quiet: bool = True):
    """Compile liborc.so (g++, OpenMP)."""
    subprocess.run(["make", "-C", HERE, "all"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = C.CDLL(LIB)
        P = C.c_void_p
        _lib.orc_render.argtypes = [P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, P, P, P, C.c_int]
        _lib.orc_closest_hit_full.argtypes = [P, P, C.c_int, P, P, P, P, P]
        _lib.orc_trace_closest.argtypes = [P, P, C.c_int, P, C.c_int, C.c_int, P]
        _lib.orc_trace_any.argtypes = [P, P, P, P, C.c_int, P, C.c_int]
        _lib.orc_bsdf_eval.argtypes = [C.c_int, P, P, P, P, C.c_int, P, P, P, P]
        _lib.orc_bsdf_sample.argtypes = [C.c_int, P, P, P, P, C.c_int, P, P, P]
        _lib.orc_camera_rays.argtypes = [P, P, C.c_int, C.c_int, P, P, P, P]
        _lib.orc_rng_stream.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, P]
        _lib.orc_render_detached.argtypes = [P, P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, P]
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def render(scene, options, camera, first_pass=0, num_passes=1, use_double=False, row_start=0, row_step=1,
           nthreads=0, with_sq=False, cull=False):
    """Oracle render of sample passes; returns (accum[H,W,4], accum_sq or None, counters dict).
    cull=True counts traversal work with tmax culling (the hits are the same)."""
    W, H = options.render_width, options.render_height
    accum = np.zeros((H, W, 4), np.float32)
    sq = np.zeros((H, W, 3), np.float32) if with_sq else None
    cnt = np.zeros(10, np.uint64)
    d = scene.desc()
    rc = lib().orc_render(C.byref(d), C.byref(options), C.byref(camera), first_pass, num_passes, int(use_double),
                          row_start, row_step, nthreads, _p(accum), _p(sq), _p(cnt), int(cull))
    assert rc == 0
    keys = ["closest", "shadow", "nodes", "tris", "overflow", "paths", "tri_hits", "nodes_any", "tris_any", "inner"]
    return accum, sq, dict(zip(keys, [int(x) for x in cnt]))


def render_detached(scene, eval_scene, options, camera, first_pass=0, num_passes=1, use_double=True, nthreads=0):
    """The detached estimator: sampling from `scene`, BSDF and emission values
    from `eval_scene` (same geometry).  Returns the mean radiance per pixel,
    H x W x 3 float64 (sum over the passes / num_passes)."""
    W, H = options.render_width, options.render_height
    acc = np.zeros((H, W, 3), np.float64)
    d, e = scene.desc(), eval_scene.desc()
    rc = lib().orc_render_detached(C.byref(d), C.byref(e), C.byref(options), C.byref(camera), first_pass,
                                   num_passes, int(use_double), nthreads, _p(acc))
    assert rc == 0
    return acc / num_passes


def closest_hit_full(scene, rays):
    """Full ClosestHit (lights, triangles, shading normal) as the reference
    build's ref_glsl_closest_hit reports it."""
    n = rays.shape[0]
    hit = np.zeros(n, np.int32); t = np.zeros(n, np.float32); mat = np.zeros(n, np.int32)
    emi = np.zeros(n, np.int32); nrm = np.zeros((n, 3), np.float32)
    d = scene.desc()
    lib().orc_closest_hit_full(C.byref(d), _p(rays), n, _p(hit), _p(t), _p(mat), _p(emi), _p(nrm))
    return dict(hit=hit, t=t, mat=mat, emitter=emi, normal=nrm)


def rays_array(origins, dirs):
    """(n,6) float32 array laid out as pt_ray."""
    r = np.empty((len(origins), 6), np.float32)
    r[:, :3] = origins
    r[:, 3:] = dirs
    return np.ascontiguousarray(r)


HIT_DTYPE = np.dtype([("t", np.float32), ("u", np.float32), ("v", np.float32), ("prim_id", np.int32),
                      ("inst_id", np.int32)])


def trace_closest(scene, rays, mode=0, use_double=False):
    """Closest triangle hits (pt_hit records) + counters (nodes, tris, overflow)."""
    n = rays.shape[0]
    hits = np.zeros(n, HIT_DTYPE)
    cnt = np.zeros(3, np.uint64)
    d = scene.desc()
    rc = lib().orc_trace_closest(C.byref(d), _p(rays), n, _p(hits), mode, int(use_double), _p(cnt))
    assert rc == 0
    return hits, dict(nodes=int(cnt[0]), tris=int(cnt[1]), overflow=int(cnt[2]))


def trace_any(scene, options, rays, maxd, use_double=False):
    n = rays.shape[0]
    occ = np.zeros(n, np.uint8)
    maxd = np.ascontiguousarray(maxd, np.float32)
    d = scene.desc()
    rc = lib().orc_trace_any(C.byref(d), C.byref(options), _p(rays), _p(maxd), n, _p(occ), int(use_double))
    assert rc == 0
    return occ


def bsdf_eval(state_params, V, N, L, use_double=True):
    n = state_params.shape[0]
    sp = np.ascontiguousarray(state_params, np.float32)
    V, N, L = (np.ascontiguousarray(x, np.float32) for x in (V, N, L))
    f = np.zeros((n, 3)); pdf = np.zeros(n); lf = np.zeros((n, 5, 3)); lp = np.zeros((n, 5))
    rc = lib().orc_bsdf_eval(n, _p(sp), _p(V), _p(N), _p(L), int(use_double), _p(f), _p(pdf), _p(lf), _p(lp))
    assert rc == 0
    return f, pdf, lf, lp


def bsdf_sample(state_params, V, N, seeds, use_double=False):
    n = state_params.shape[0]
    sp = np.ascontiguousarray(state_params, np.float32)
    V, N = (np.ascontiguousarray(x, np.float32) for x in (V, N))
    seeds = np.ascontiguousarray(seeds, np.uint32)
    L = np.zeros((n, 3)); f = np.zeros((n, 3)); pdf = np.zeros(n)
    rc = lib().orc_bsdf_sample(n, _p(sp), _p(V), _p(N), _p(seeds), int(use_double), _p(L), _p(f), _p(pdf))
    assert rc == 0
    return L, f, pdf


def camera_rays(options, camera, pass_index, px, py):
    px = np.ascontiguousarray(px, np.int32)
    py = np.ascontiguousarray(py, np.int32)
    n = px.shape[0]
    rays = np.zeros((n, 6), np.float32)
    st = np.zeros((n, 4), np.uint32)
    rc = lib().orc_camera_rays(C.byref(options), C.byref(camera), pass_index, n, _p(px), _p(py), _p(rays), _p(st))
    assert rc == 0
    return rays, st


def rng_stream(px, py, frame, n):
    out = np.zeros(n, np.float32)
    lib().orc_rng_stream(px, py, frame, n, _p(out))
    return out


# ----------------------------------------------------------- reference builds
def ref_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "ref_scene_dump"))


def _ref_lib(name: str):
    """A reference build under _ref/, compiled on first use (make names the
    macro set from the file name: see the Makefile)."""
    path = os.path.join(REF_DIR, name)
    if not os.path.exists(path):
        subprocess.run(["make", "-C", HERE, os.path.join("_ref", name)], check=True, stdout=subprocess.DEVNULL)
    return C.CDLL(path)


def ref_glsl(variant: str):
    """The reference shaders compiled with feature-macro set `variant`."""
    L = _ref_lib(f"libref_glsl_{variant}.so")
    P = C.c_void_p
    L.ref_glsl_variant.restype = C.c_char_p
    L.ref_glsl_render.argtypes = [P, P, P, C.c_int, C.c_int, C.c_int, P]
    L.ref_glsl_closest_hit.argtypes = [P, P, C.c_int, P, P, P, P, P]
    L.ref_glsl_disney_eval.argtypes = [C.c_int, P, P, P, P, P, P]
    return L


def ref_render(variant, scene, options, camera, first_pass=0, num_passes=1, nthreads=0):
    L = ref_glsl(variant)
    W, H = options.render_width, options.render_height
    accum = np.zeros((H, W, 4), np.float32)
    d = scene.desc()
    L.ref_glsl_render(C.byref(d), C.byref(options), C.byref(camera), first_pass, num_passes, nthreads, _p(accum))
    return accum


def ref_dump_scene(scene_file: str, out_prefix: str):
    subprocess.run([os.path.join(REF_DIR, "ref_scene_dump"), scene_file, out_prefix], check=True,
                   stdout=subprocess.DEVNULL)


def ref_macros(scene, options) -> list[str]:
    """The OPT_* macros Renderer::InitShaders injects for this scene and
    these options (Renderer.cpp:400-476), in its order."""
    mats = scene.materials
    m = []
    if options.enable_envmap and scene.envmap_rgb is not None:
        m.append("ENVMAP")
    if scene.lights.shape[0] > 0:
        m.append("LIGHTS")
    if options.enable_rr:
        m += ["RR", f"RR_DEPTH_{int(options.rr_depth)}"]
    if options.enable_uniform_light:
        m.append("UNIFORM_LIGHT")
    if options.opengl_normal_map:
        m.append("OPENGL_NORMALMAP")
    if options.hide_emitters:
        m.append("HIDE_EMITTERS")
    if options.enable_background:
        m.append("BACKGROUND")
    if options.transparent_background:
        m.append("TRANSPARENT_BACKGROUND")
    if (mats[:, 29].astype(int) != 0).any():
        m.append("ALPHA_TEST")
    if options.enable_roughness_mollification:
        m.append("ROUGHNESS_MOLLIFICATION")
    if (mats[:, 18].astype(int) != 0).any():
        m.append("MEDIUM")
    if options.enable_volume_mis:
        m.append("VOL_MIS")
    return m


# Macro sets that have a short name in the Makefile (the first golden
# fixtures were made with these).
_NAMED_VARIANTS = {
    "lights": "LIGHTS RR RR_DEPTH_2 OPENGL_NORMALMAP",
    "lights_norr": "LIGHTS OPENGL_NORMALMAP",
    "env": "ENVMAP LIGHTS RR RR_DEPTH_2 OPENGL_NORMALMAP",
    "envonly": "ENVMAP RR RR_DEPTH_2 OPENGL_NORMALMAP",
    "volmis": "LIGHTS RR RR_DEPTH_2 OPENGL_NORMALMAP ALPHA_TEST MEDIUM VOL_MIS",
    "vol": "LIGHTS RR RR_DEPTH_2 OPENGL_NORMALMAP ALPHA_TEST MEDIUM",
    "envvolmis": "ENVMAP LIGHTS RR RR_DEPTH_2 OPENGL_NORMALMAP ALPHA_TEST MEDIUM VOL_MIS",
    "alpha": "LIGHTS RR RR_DEPTH_2 OPENGL_NORMALMAP ALPHA_TEST",
    "volmis_opaque": "LIGHTS RR RR_DEPTH_2 OPENGL_NORMALMAP MEDIUM VOL_MIS",
    "envvolmis_opaque": "ENVMAP LIGHTS RR RR_DEPTH_2 OPENGL_NORMALMAP MEDIUM VOL_MIS",
}


def variant_for(scene, options) -> str:
    """Name of the reference shader build with the macro set
    Renderer::InitShaders would compile for this scene (Renderer.cpp:400-476):
    a short name where the Makefile has one, else o.<MACRO>.<MACRO>...
    (built on first use).  OPT_VOL_MIS only acts together with OPT_MEDIUM
    (pathtrace.glsl:118,177,244), so without a medium it is left out."""
    m = ref_macros(scene, options)
    if "VOL_MIS" in m and "MEDIUM" not in m:
        m.remove("VOL_MIS")
    key = " ".join(m)
    for name, macros in _NAMED_VARIANTS.items():
        if macros == key:
            return name
    return "o." + ".".join(m)


def ref_tonemap(accum, num_samples, options, width, height):
    """The reference's tonemap.glsl on an accumulation (H x W x 4, bottom row
    first) with the tonemap uniforms of these options; returns its float
    output (H x W x 4) before the RGBA8 read-back."""
    bg = "BACKGROUND" if options.enable_background else "NONE"
    if options.transparent_background:
        bg = "TRANSPARENT_BACKGROUND" if not options.enable_background else "BACKGROUND.TRANSPARENT_BACKGROUND"
    L = _ref_lib(f"libref_tonemap_o.{bg}.so")
    P = C.c_void_p
    L.ref_tonemap.argtypes = [P, C.c_int, C.c_int, C.c_float, C.c_int, C.c_int, C.c_int, P, P]
    acc = np.ascontiguousarray(accum, np.float32)
    out = np.zeros((height, width, 4), np.float32)
    bgc = np.asarray(list(options.background_col), np.float32)
    L.ref_tonemap(_p(acc), width, height, np.float32(1.0) / np.float32(num_samples), int(options.enable_tonemap),
                  int(options.enable_aces), int(options.simple_aces_fit), _p(bgc), _p(out))
    return out


def tonemap(accum, num_samples, options):
    """tonemap.glsl:97-133 restated in numpy FP32 (test infrastructure): the
    reference's float output for an accumulation (H x W x 4, bottom row
    first), before the RGBA8 read-back.  Pinned against the reference's own
    tonemap.glsl by tests/test_oracle_golden.py."""
    f32 = np.float32
    col = np.asarray(accum, f32) * (f32(1.0) / f32(num_samples))  # texture() * invSampleCounter (:99)
    c = col[..., :3].copy()
    alpha = col[..., 3]
    if options.enable_tonemap:
        if options.enable_aces:
            if options.simple_aces_fit:  # ACES (:79-88)
                a, b, y, d, e = f32(2.51), f32(0.03), f32(2.43), f32(0.59), f32(0.14)
                c = np.clip((c * (a * c + b)) / (c * (y * c + d) + e), f32(0), f32(1))
            else:  # ACESFitted (:64-77): row vector times the matrices whose columns are listed
                mi = np.array([[0.59719, 0.35458, 0.04823], [0.07600, 0.90834, 0.01566],
                               [0.02840, 0.13383, 0.83777]], f32)
                mo = np.array([[1.60475, -0.53108, -0.07367], [-0.10208, 1.10813, -0.00605],
                               [-0.00327, -0.07276, 1.07602]], f32)

                def vm(v, m):
                    return np.stack([(v[..., 0] * m[j, 0] + v[..., 1] * m[j, 1]) + v[..., 2] * m[j, 2]
                                     for j in range(3)], -1).astype(f32)
                v = vm(c, mi)
                a = v * (v + f32(0.0245786)) - f32(0.000090537)  # RRTAndODTFit (:57-62)
                b = v * (f32(0.983729) * v + f32(0.4329510)) + f32(0.238081)
                c = np.clip(vm(a / b, mo), f32(0), f32(1))
        else:  # Tonemap(c, 1.5) (:90-93)
            lum = (f32(0.212671) * c[..., 0] + f32(0.715160) * c[..., 1]) + f32(0.072169) * c[..., 2]
            c = c * f32(1.0) / (f32(1.0) + lum / f32(1.5))[..., None]
    c = np.power(c, f32(1.0 / 2.2)).astype(f32)  # :110
    H, W = c.shape[:2]
    out_alpha = np.ones((H, W), f32)
    bgc = np.broadcast_to(np.asarray(list(options.background_col), f32), c.shape)
    if options.transparent_background:  # :115-120
        out_alpha = alpha
        fy, fx = np.meshgrid(np.arange(H, dtype=f32) + f32(0.5), np.arange(W, dtype=f32) + f32(0.5), indexing="ij")
        m = np.mod(np.floor(fx / f32(10)) + np.floor(fy / f32(10)), f32(2))
        res = np.maximum(np.sign(m), f32(0))[..., None]
        bgc = f32(0.1) * (f32(1) - res) + f32(0.2) * res
    if options.enable_background or options.transparent_background:  # mix(bgCol, color, alpha) (:122-124)
        c = bgc * (f32(1) - alpha[..., None]) + c * alpha[..., None]
    return np.concatenate([c, out_alpha[..., None]], -1).astype(f32)


def to_rgba8(x):
    """The float -> RGBA8 conversion of GetOutputBuffer's read-back: clamp to
    [0, 1], scale by 255, round to nearest."""
    return np.floor(np.clip(x, 0, 1) * np.float32(255) + np.float32(0.5)).astype(np.uint8)
