"""ctypes mirror of include/pt_cuda.h and the loader of libptgb.so.

The structures below are byte-for-byte the C structs of the header; the
library itself is the CUDA path (there is no other implementation behind
these entry points: if the library is missing, loading fails loudly).
"""
from __future__ import annotations

import ctypes as C
import os

PT_OK = 0
PT_ERR_INVALID_ARG = 1
PT_ERR_CUDA = 2
PT_ERR_OUT_OF_MEMORY = 3
PT_ERR_STACK_OVERFLOW = 4
PT_ERR_UNSUPPORTED = 5
PT_ERR_TIMEOUT = 6
PT_ERR_QUEUE_OVERFLOW = 7

PT_INTEGRATOR_MEGAKERNEL = 0
PT_INTEGRATOR_WAVEFRONT = 1

_f = C.POINTER(C.c_float)
_i = C.POINTER(C.c_int32)
_u8 = C.POINTER(C.c_uint8)


class pt_scene_desc(C.Structure):
    _fields_ = [
        ("bvh_nodes", _f), ("num_bvh_nodes", C.c_int32), ("top_level_index", C.c_int32),
        ("vert_indices", _i), ("num_tris", C.c_int32),
        ("vertices_uvx", _f), ("normals_uvy", _f), ("num_vertices", C.c_int32),
        ("transforms", _f), ("num_instances", C.c_int32),
        ("materials", _f), ("num_materials", C.c_int32),
        ("lights", _f), ("num_lights", C.c_int32),
        ("envmap_rgb", _f), ("envmap_cdf", _f), ("envmap_width", C.c_int32), ("envmap_height", C.c_int32),
        ("envmap_total_sum", C.c_float),
        ("texture_maps", _u8), ("tex_width", C.c_int32), ("tex_height", C.c_int32), ("num_textures", C.c_int32),
    ]


class pt_mesh_desc(C.Structure):
    _fields_ = [("mesh_tri_offset", _i), ("num_meshes", C.c_int32), ("instance_mesh", _i),
                ("instance_material", _i)]


class pt_render_options(C.Structure):
    _fields_ = [
        ("render_width", C.c_int32), ("render_height", C.c_int32),
        ("tile_width", C.c_int32), ("tile_height", C.c_int32),
        ("max_depth", C.c_int32), ("max_spp", C.c_int32), ("rr_depth", C.c_int32),
        ("enable_rr", C.c_int32), ("enable_envmap", C.c_int32), ("enable_uniform_light", C.c_int32),
        ("hide_emitters", C.c_int32), ("enable_background", C.c_int32), ("transparent_background", C.c_int32),
        ("enable_roughness_mollification", C.c_int32), ("enable_volume_mis", C.c_int32),
        ("opengl_normal_map", C.c_int32), ("enable_tonemap", C.c_int32), ("enable_aces", C.c_int32),
        ("simple_aces_fit", C.c_int32),
        ("uniform_light_col", C.c_float * 3), ("background_col", C.c_float * 3),
        ("envmap_intensity", C.c_float), ("envmap_rot", C.c_float), ("roughness_mollification_amt", C.c_float),
    ]


class pt_camera(C.Structure):
    _fields_ = [
        ("position", C.c_float * 3), ("up", C.c_float * 3), ("right", C.c_float * 3), ("forward", C.c_float * 3),
        ("fov", C.c_float), ("focal_dist", C.c_float), ("aperture", C.c_float),
    ]


class pt_ray(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("direction", C.c_float * 3)]


class pt_hit(C.Structure):
    _fields_ = [("t", C.c_float), ("u", C.c_float), ("v", C.c_float), ("prim_id", C.c_int32), ("inst_id", C.c_int32)]


class pt_stats(C.Structure):
    _fields_ = [
        ("closest_rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("paths", C.c_uint64),
        ("kernel_ms", C.c_float), ("status", C.c_int32), ("kernel_launches", C.c_int32),
        ("truncated_paths", C.c_uint64), ("untraced_shadow_rays", C.c_uint64),
    ]


class pt_tuning(C.Structure):
    _fields_ = [("extend_variant", C.c_int32), ("shadow_variant", C.c_int32), ("extend_refill", C.c_int32),
                ("shadow_refill", C.c_int32), ("min_tris", C.c_int32), ("shade_variant", C.c_int32),
                ("frame_ms", C.c_float), ("extend_refill_first", C.c_int32), ("min_tris_first", C.c_int32),
                ("shadow_refill_first", C.c_int32), ("shadow_min_tris_first", C.c_int32),
                ("extend_variant_first", C.c_int32), ("shade_variant_first", C.c_int32)]


class pt_stage_stats(C.Structure):
    _fields_ = [("ms", C.c_float * 5), ("launches", C.c_int32 * 5)]


STAGES = ("generate", "extend", "shade", "shadow", "resolve")


# Default RenderOptions (src/core/Renderer.h:39-69)
DEFAULT_OPTIONS = dict(
    render_width=1280, render_height=720, tile_width=100, tile_height=100, max_depth=2, max_spp=-1, rr_depth=2,
    enable_rr=1, enable_envmap=0, enable_uniform_light=0, hide_emitters=0, enable_background=0,
    transparent_background=0, enable_roughness_mollification=0, enable_volume_mis=0, opengl_normal_map=1,
    enable_tonemap=1, enable_aces=0, simple_aces_fit=0, uniform_light_col=(0.3, 0.3, 0.3),
    background_col=(1.0, 1.0, 1.0), envmap_intensity=1.0, envmap_rot=0.0, roughness_mollification_amt=0.0,
)


def make_options(**kw) -> pt_render_options:
    d = dict(DEFAULT_OPTIONS)
    d.update(kw)
    o = pt_render_options()
    for k, v in d.items():
        if isinstance(v, (tuple, list)):
            arr = getattr(o, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(o, k, v)
    return o


def options_dict(o: pt_render_options) -> dict:
    out = {}
    for name, _ in pt_render_options._fields_:
        v = getattr(o, name)
        out[name] = list(v) if hasattr(v, "__len__") else v
    return out


def make_camera(position, up, right, forward, fov, focal_dist=0.1, aperture=0.0) -> pt_camera:
    c = pt_camera()
    for name, v in (("position", position), ("up", up), ("right", right), ("forward", forward)):
        arr = getattr(c, name)
        for i in range(3):
            arr[i] = float(v[i])
    c.fov, c.focal_dist, c.aperture = float(fov), float(focal_dist), float(aperture)
    return c


PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "csrc", "libptgb.so")

_lib = None


def load_library(path: str | None = None) -> C.CDLL:
    """Load libptgb.so (the CUDA path).  Raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libptgb.so not built at {p}: run __graft_entry__.build()")
    lib = C.CDLL(p)
    P = C.c_void_p
    lib.pt_create.argtypes = [C.POINTER(pt_scene_desc), C.POINTER(pt_render_options), C.POINTER(P)]
    lib.pt_create_gpu_bvh.argtypes = [C.POINTER(pt_scene_desc), C.POINTER(pt_mesh_desc),
                                      C.POINTER(pt_render_options), C.POINTER(P)]
    lib.pt_update_transforms.argtypes = [P, _f, C.c_int32]
    lib.pt_gpu_build_ms.argtypes = [P, _f]
    lib.pt_destroy.argtypes = [P]
    lib.pt_set_stream.argtypes = [P, P]
    lib.pt_set_camera.argtypes = [P, C.POINTER(pt_camera)]
    lib.pt_set_options.argtypes = [P, C.POINTER(pt_render_options)]
    lib.pt_set_integrator.argtypes = [P, C.c_int32]
    lib.pt_update_instances.argtypes = [P, _f, C.c_int32, _f, C.c_int32, _f, C.c_int32]
    lib.pt_update_envmap.argtypes = [P, _f, _f, C.c_int32, C.c_int32, C.c_float]
    lib.pt_clear_accum.argtypes = [P]
    lib.pt_render_tile.argtypes = [P, C.c_int32, C.c_int32, C.c_int32]
    lib.pt_render_tile_noalloc.argtypes = [P, C.c_int32, C.c_int32, C.c_int32]
    lib.pt_render_passes.argtypes = [P, C.c_int32, C.c_int32]
    lib.pt_update_materials.argtypes = [P, _f, C.c_int32]
    lib.pt_update_lights.argtypes = [P, _f, C.c_int32]
    lib.pt_render_adjoint.argtypes = [P, C.c_int32, C.c_int32, _f, _f]
    lib.pt_get_accum.argtypes = [P, _f]
    lib.pt_set_accum.argtypes = [P, _f]
    lib.pt_snapshot_accum.argtypes = [P]
    lib.pt_get_output.argtypes = [P, C.c_int32, C.c_int32, _u8]
    lib.pt_trace_rays.argtypes = [P, C.POINTER(pt_ray), C.c_int32, C.POINTER(pt_hit)]
    lib.pt_trace_shadow.argtypes = [P, C.POINTER(pt_ray), _f, C.c_int32, _u8]
    lib.pt_bsdf_eval.argtypes = [P, _f, _f, _f, _f, C.c_int32, _f, _f]
    lib.pt_bsdf_sample.argtypes = [P, _f, _f, _f, C.POINTER(C.c_uint32), C.c_int32, _f, _f, _f]
    lib.pt_autotune.argtypes = [P, C.c_int32, C.POINTER(pt_tuning)]
    lib.pt_get_tuning.argtypes = [P, C.POINTER(pt_tuning)]
    lib.pt_set_tuning.argtypes = [P, C.POINTER(pt_tuning)]
    lib.pt_set_stage_timing.argtypes = [P, C.c_int32]
    lib.pt_get_stage_stats.argtypes = [P, C.POINTER(pt_stage_stats)]
    lib.pt_get_stats.argtypes = [P, C.POINTER(pt_stats)]
    lib.pt_batch_create.argtypes = [C.POINTER(P), C.c_int32, C.POINTER(P)]
    lib.pt_batch_render.argtypes = [P, C.POINTER(C.c_int32), C.POINTER(C.c_int32), _f]
    lib.pt_batch_stats.argtypes = [P, C.POINTER(pt_stats)]
    lib.pt_batch_destroy.argtypes = [P]
    lib.pt_last_error.argtypes = [C.c_char_p, C.c_size_t]
    for name in ("pt_create", "pt_create_gpu_bvh", "pt_update_transforms", "pt_gpu_build_ms", "pt_destroy", "pt_set_stream", "pt_set_camera", "pt_set_options", "pt_set_integrator",
                 "pt_update_instances", "pt_update_envmap", "pt_clear_accum", "pt_render_tile",
                 "pt_update_materials", "pt_update_lights", "pt_render_adjoint",
                 "pt_render_tile_noalloc", "pt_render_passes", "pt_get_accum", "pt_set_accum", "pt_snapshot_accum",
                 "pt_get_output",
                 "pt_trace_rays", "pt_trace_shadow", "pt_bsdf_eval", "pt_bsdf_sample", "pt_autotune",
                 "pt_get_tuning", "pt_set_tuning", "pt_set_stage_timing",
                 "pt_get_stage_stats", "pt_get_stats", "pt_batch_create", "pt_batch_render",
                 "pt_batch_stats", "pt_batch_destroy", "pt_last_error"):
        getattr(lib, name).restype = C.c_int
    if path is None:
        _lib = lib
    return lib


HEADER_SYMBOLS = [
    "pt_create", "pt_create_gpu_bvh", "pt_update_transforms", "pt_gpu_build_ms", "pt_destroy", "pt_set_stream", "pt_set_camera", "pt_set_options", "pt_set_integrator",
    "pt_update_instances", "pt_update_envmap", "pt_clear_accum", "pt_render_tile", "pt_render_tile_noalloc",
    "pt_update_materials", "pt_update_lights", "pt_render_adjoint",
    "pt_render_passes", "pt_get_accum", "pt_set_accum", "pt_snapshot_accum", "pt_get_output", "pt_trace_rays",
    "pt_trace_shadow",
    "pt_bsdf_eval", "pt_bsdf_sample", "pt_autotune", "pt_get_tuning", "pt_set_tuning", "pt_set_stage_timing",
    "pt_get_stage_stats", "pt_get_stats",
    "pt_batch_create", "pt_batch_render", "pt_batch_stats", "pt_batch_destroy",
    "pt_last_error",
]


class PTError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"pt error {code}: {msg}")
        self.code = code


def check(lib, rc: int):
    if rc != PT_OK:
        buf = C.create_string_buffer(1024)
        lib.pt_last_error(buf, 1024)
        raise PTError(rc, buf.value.decode(errors="replace"))
