"""Python-side handle on one libptgb context (the CUDA path).

Thin: every method is one C ABI call (include/pt_cuda.h) plus numpy
marshalling.  Used by the tests, smoke() and bench.py; a C++ program uses
CudaRenderer (csrc/cuda_renderer.h) or the C ABI directly.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .scene import SceneData

HIT_DTYPE = np.dtype([("t", np.float32), ("u", np.float32), ("v", np.float32), ("prim_id", np.int32),
                      ("inst_id", np.int32)])


class GpuRenderer:
    def __init__(self, scene: SceneData, options: capi.pt_render_options | None = None, gpu_bvh: bool = False,
                 **overrides):
        """gpu_bvh: build the BVH on the GPU (pt_create_gpu_bvh) from the
        scene's meshes instead of collapsing its flattened binary BVH."""
        self.lib = capi.load_library()
        self.scene = scene
        self.options = options if options is not None else scene.render_options(**overrides)
        self._desc = scene.desc()
        self.ctx = C.c_void_p()
        if gpu_bvh:
            off, im, mat = scene.mesh_desc()
            self._mesh_arrays = (off, im, mat)
            ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
            self._mesh = capi.pt_mesh_desc(ip(off), len(off) - 1, ip(im), ip(mat))
            capi.check(self.lib, self.lib.pt_create_gpu_bvh(C.byref(self._desc), C.byref(self._mesh),
                                                            C.byref(self.options), C.byref(self.ctx)))
        else:
            capi.check(self.lib, self.lib.pt_create(C.byref(self._desc), C.byref(self.options), C.byref(self.ctx)))
        self.set_camera(scene.pt_camera())

    def update_transforms(self, transforms: np.ndarray):
        t = np.ascontiguousarray(transforms, np.float32)
        self._ck(self.lib.pt_update_transforms(self.ctx, t.ctypes.data_as(C.POINTER(C.c_float)), t.shape[0]))

    def gpu_build_ms(self) -> float:
        ms = C.c_float()
        self._ck(self.lib.pt_gpu_build_ms(self.ctx, C.byref(ms)))
        return ms.value

    # ------------------------------------------------------------------
    @property
    def width(self):
        return self.options.render_width

    @property
    def height(self):
        return self.options.render_height

    def _ck(self, rc):
        capi.check(self.lib, rc)

    def set_camera(self, cam: capi.pt_camera):
        self.camera = cam
        self._ck(self.lib.pt_set_camera(self.ctx, C.byref(cam)))

    def set_options(self, options: capi.pt_render_options):
        self.options = options
        self._ck(self.lib.pt_set_options(self.ctx, C.byref(options)))

    def set_stream(self, stream_ptr: int | None):
        self._ck(self.lib.pt_set_stream(self.ctx, C.c_void_p(stream_ptr) if stream_ptr else None))

    def set_integrator(self, which: int):
        self._ck(self.lib.pt_set_integrator(self.ctx, which))

    def clear(self):
        self._ck(self.lib.pt_clear_accum(self.ctx))

    def render_passes(self, first_pass: int, num_passes: int):
        self._ck(self.lib.pt_render_passes(self.ctx, first_pass, num_passes))

    def render_tile(self, tx: int, ty: int, frame: int):
        self._ck(self.lib.pt_render_tile(self.ctx, tx, ty, frame))

    def accum(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((self.height, self.width, 4), np.float32)
        self._ck(self.lib.pt_get_accum(self.ctx, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def set_accum(self, acc: np.ndarray):
        """Checkpoint resume: the accumulation from a pt_get_accum copy."""
        a = np.ascontiguousarray(acc, np.float32)
        assert a.shape == (self.height, self.width, 4)
        self._ck(self.lib.pt_set_accum(self.ctx, a.ctypes.data_as(C.POINTER(C.c_float))))

    def snapshot(self):
        self._ck(self.lib.pt_snapshot_accum(self.ctx))

    def output(self, num_samples: int, from_snapshot: bool = False) -> np.ndarray:
        out = np.empty((self.height, self.width, 4), np.uint8)
        self._ck(self.lib.pt_get_output(self.ctx, num_samples, int(from_snapshot),
                                        out.ctypes.data_as(C.POINTER(C.c_uint8))))
        return out

    def trace(self, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32)
        hits = np.zeros(rays.shape[0], HIT_DTYPE)
        self._ck(self.lib.pt_trace_rays(self.ctx, rays.ctypes.data_as(C.POINTER(capi.pt_ray)), rays.shape[0],
                                        hits.ctypes.data_as(C.POINTER(capi.pt_hit))))
        return hits

    def shadow(self, rays: np.ndarray, maxd: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32)
        maxd = np.ascontiguousarray(maxd, np.float32)
        occ = np.zeros(rays.shape[0], np.uint8)
        self._ck(self.lib.pt_trace_shadow(self.ctx, rays.ctypes.data_as(C.POINTER(capi.pt_ray)),
                                          maxd.ctypes.data_as(C.POINTER(C.c_float)), rays.shape[0],
                                          occ.ctypes.data_as(C.POINTER(C.c_uint8))))
        return occ

    def stats(self) -> dict:
        s = capi.pt_stats()
        self._ck(self.lib.pt_get_stats(self.ctx, C.byref(s)))
        return dict(closest=s.closest_rays, shadow=s.shadow_rays, paths=s.paths, kernel_ms=s.kernel_ms,
                    status=s.status, launches=s.kernel_launches, truncated=s.truncated_paths,
                    untraced=s.untraced_shadow_rays)

    def update_materials(self, materials: np.ndarray):
        m = np.ascontiguousarray(materials, np.float32)
        self._ck(self.lib.pt_update_materials(self.ctx, m.ctypes.data_as(C.POINTER(C.c_float)), m.shape[0]))

    def update_lights(self, lights: np.ndarray):
        m = np.ascontiguousarray(lights, np.float32)
        self._ck(self.lib.pt_update_lights(self.ctx, m.ctypes.data_as(C.POINTER(C.c_float)), m.shape[0]))

    def render_adjoint(self, first_pass: int, num_passes: int, d_image: np.ndarray) -> np.ndarray:
        """Gradient of a loss of I = accum / num_passes (d_image = dLoss/dI,
        H x W x 3) w.r.t. 11 parameters per material, then 3 per light."""
        di = np.ascontiguousarray(d_image, np.float32)
        assert di.shape == (self.height, self.width, 3)
        n = self.scene.materials.shape[0] * 11 + self.scene.lights.shape[0] * 3
        g = np.zeros(n, np.float32)
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        self._ck(self.lib.pt_render_adjoint(self.ctx, first_pass, num_passes, fp(di), fp(g)))
        return g

    TUNING_FIELDS = ("extend_variant", "shadow_variant", "extend_refill", "shadow_refill", "min_tris",
                     "shade_variant", "extend_refill_first", "min_tris_first", "shadow_refill_first",
                     "shadow_min_tris_first", "extend_variant_first", "shade_variant_first")

    def autotune(self, num_passes: int = 2) -> dict:
        t = capi.pt_tuning()
        self._ck(self.lib.pt_autotune(self.ctx, num_passes, C.byref(t)))
        return {**{k: getattr(t, k) for k in self.TUNING_FIELDS}, "frame_ms": t.frame_ms}

    def tuning(self) -> dict:
        t = capi.pt_tuning()
        self._ck(self.lib.pt_get_tuning(self.ctx, C.byref(t)))
        return {k: getattr(t, k) for k in self.TUNING_FIELDS}

    def set_tuning(self, **kw):
        t = capi.pt_tuning()
        self._ck(self.lib.pt_get_tuning(self.ctx, C.byref(t)))
        for k, v in kw.items():
            setattr(t, k, v)
        self._ck(self.lib.pt_set_tuning(self.ctx, C.byref(t)))

    def set_stage_timing(self, on: bool):
        self._ck(self.lib.pt_set_stage_timing(self.ctx, 1 if on else 0))

    def stage_stats(self) -> dict:
        s = capi.pt_stage_stats()
        self._ck(self.lib.pt_get_stage_stats(self.ctx, C.byref(s)))
        return {name: (float(s.ms[k]), int(s.launches[k])) for k, name in enumerate(capi.STAGES)}

    def update_instances(self, transforms, materials, tlas_nodes):
        t = np.ascontiguousarray(transforms, np.float32)
        m = np.ascontiguousarray(materials, np.float32)
        n = np.ascontiguousarray(tlas_nodes, np.float32)
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        self._ck(self.lib.pt_update_instances(self.ctx, fp(t), t.shape[0], fp(m), m.shape[0], fp(n), n.shape[0]))

    def close(self):
        if self.ctx:
            self.lib.pt_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuBatch:
    """Several GpuRenderer contexts rendered as one wavefront
    (pt_batch_create / pt_batch_render).  Each renderer's accumulation
    buffer receives what its own render_passes(first, count) would add."""

    def __init__(self, renderers: list[GpuRenderer]):
        self.lib = capi.load_library()
        self.renderers = list(renderers)
        arr = (C.c_void_p * len(self.renderers))(*[r.ctx.value for r in self.renderers])
        self.handle = C.c_void_p()
        capi.check(self.lib, self.lib.pt_batch_create(arr, len(self.renderers), C.byref(self.handle)))

    def render(self, first_pass, num_passes) -> np.ndarray:
        """first_pass / num_passes: one int per job (or one for all).
        Returns each job's completion time (ms after the batch started)."""
        n = len(self.renderers)
        fp = np.broadcast_to(np.asarray(first_pass, np.int32), (n,)).copy()
        npass = np.broadcast_to(np.asarray(num_passes, np.int32), (n,)).copy()
        ms = np.zeros(n, np.float32)
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))
        capi.check(self.lib, self.lib.pt_batch_render(self.handle, ip(fp), ip(npass),
                                                      ms.ctypes.data_as(C.POINTER(C.c_float))))
        return ms

    def stats(self) -> dict:
        s = capi.pt_stats()
        capi.check(self.lib, self.lib.pt_batch_stats(self.handle, C.byref(s)))
        return dict(closest=s.closest_rays, shadow=s.shadow_rays, paths=s.paths, kernel_ms=s.kernel_ms,
                    status=s.status, launches=s.kernel_launches, truncated=s.truncated_paths,
                    untraced=s.untraced_shadow_rays)

    def close(self):
        if self.handle:
            self.lib.pt_batch_destroy(self.handle)
            self.handle = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
