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
    cnt = np.zeros(9, np.uint64)
    d = scene.desc()
    rc = lib().orc_render(C.byref(d), C.byref(options), C.byref(camera), first_pass, num_passes, int(use_double),
                          row_start, row_step, nthreads, _p(accum), _p(sq), _p(cnt), int(cull))
    assert rc == 0
    keys = ["closest", "shadow", "nodes", "tris", "overflow", "paths", "tri_hits", "nodes_any", "tris_any"]
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


def ref_glsl(variant: str):
    """The reference shaders compiled with feature-macro set `variant`."""
    path = os.path.join(REF_DIR, f"libref_glsl_{variant}.so")
    L = C.CDLL(path)
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


def variant_for(scene, options) -> str:
    """Feature-macro set Renderer::InitShaders would compile for this scene
    (Renderer.cpp:400-476), as one of the variants the Makefile builds."""
    mats = scene.materials
    alpha = bool((mats[:, 29].astype(int) != 0).any())
    medium = bool((mats[:, 18].astype(int) != 0).any())
    env = bool(options.enable_envmap) and scene.envmap_rgb is not None
    lights = scene.lights.shape[0] > 0
    vm = bool(options.enable_volume_mis)
    key = (env, lights, alpha, medium, vm, bool(options.enable_rr))
    table = {
        (False, True, False, False, False, True): "lights",
        (False, True, False, False, True, True): "lights",
        (False, True, False, False, False, False): "lights_norr",
        (True, True, False, False, False, True): "env",
        (True, False, False, False, False, True): "envonly",
        (False, True, True, True, True, True): "volmis",
        (False, True, True, True, False, True): "vol",
        (True, True, True, True, True, True): "envvolmis",
        (False, True, True, False, False, True): "alpha",
        (False, True, False, True, True, True): "volmis_opaque",
        (True, True, False, True, True, True): "envvolmis_opaque",
    }
    if key not in table:
        raise KeyError(f"no reference shader variant built for {key}")
    return table[key]
