"""Host-side scene container: the flattened arrays GLSLPT::Scene hands to its
Renderer (src/core/Scene.h:87-125), as numpy arrays.

`SceneData.desc()` builds the `pt_scene_desc` of include/pt_cuda.h pointing
at those arrays (the arrays must outlive any call that uses the descriptor).
"""
from __future__ import annotations

import ctypes as C
import json
import os
from dataclasses import dataclass, field

import numpy as np

from . import capi

F = np.float32
I = np.int32


@dataclass
class SceneData:
    bvh_nodes: np.ndarray          # (N, 9) float32: bboxmin, bboxmax, LRLeaf
    top_level_index: int
    vert_indices: np.ndarray       # (T, 3) int32
    vertices_uvx: np.ndarray       # (V, 4) float32
    normals_uvy: np.ndarray        # (V, 4) float32
    transforms: np.ndarray         # (I, 16) float32 (Mat4 rows)
    materials: np.ndarray          # (M, 32) float32
    lights: np.ndarray             # (L, 15) float32
    envmap_rgb: np.ndarray | None = None   # (H, W, 3) float32
    envmap_cdf: np.ndarray | None = None   # (H, W) float32
    envmap_total_sum: float = 0.0
    texture_maps: np.ndarray | None = None  # (K, h, w, 4) uint8
    options: dict = field(default_factory=dict)
    camera: dict = field(default_factory=dict)
    # instance description kept for TLAS rebuilds: mesh id / material id per instance
    instance_mesh: np.ndarray | None = None
    instance_material: np.ndarray | None = None

    def __post_init__(self):
        self.bvh_nodes = np.ascontiguousarray(self.bvh_nodes, F).reshape(-1, 9)
        self.vert_indices = np.ascontiguousarray(self.vert_indices, I).reshape(-1, 3)
        self.vertices_uvx = np.ascontiguousarray(self.vertices_uvx, F).reshape(-1, 4)
        self.normals_uvy = np.ascontiguousarray(self.normals_uvy, F).reshape(-1, 4)
        self.transforms = np.ascontiguousarray(self.transforms, F).reshape(-1, 16)
        self.materials = np.ascontiguousarray(self.materials, F).reshape(-1, 32)
        self.lights = np.ascontiguousarray(self.lights, F).reshape(-1, 15)
        if self.envmap_rgb is not None:
            self.envmap_rgb = np.ascontiguousarray(self.envmap_rgb, F)
            self.envmap_cdf = np.ascontiguousarray(self.envmap_cdf, F)

    # ------------------------------------------------------------------
    @property
    def num_tris(self) -> int:
        return int(self.vert_indices.shape[0])

    def desc(self) -> capi.pt_scene_desc:
        d = capi.pt_scene_desc()

        def fp(a):
            return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None and a.size else None

        d.bvh_nodes = fp(self.bvh_nodes)
        d.num_bvh_nodes = self.bvh_nodes.shape[0]
        d.top_level_index = int(self.top_level_index)
        d.vert_indices = self.vert_indices.ctypes.data_as(C.POINTER(C.c_int32)) if self.vert_indices.size else None
        d.num_tris = self.vert_indices.shape[0]
        d.vertices_uvx = fp(self.vertices_uvx)
        d.normals_uvy = fp(self.normals_uvy)
        d.num_vertices = self.vertices_uvx.shape[0]
        d.transforms = fp(self.transforms)
        d.num_instances = self.transforms.shape[0]
        d.materials = fp(self.materials)
        d.num_materials = self.materials.shape[0]
        d.lights = fp(self.lights)
        d.num_lights = self.lights.shape[0]
        if self.envmap_rgb is not None:
            d.envmap_rgb = fp(self.envmap_rgb)
            d.envmap_cdf = fp(self.envmap_cdf)
            d.envmap_height, d.envmap_width = self.envmap_rgb.shape[:2]
            d.envmap_total_sum = float(self.envmap_total_sum)
        if self.texture_maps is not None and self.texture_maps.size:
            self.texture_maps = np.ascontiguousarray(self.texture_maps, np.uint8)
            d.texture_maps = self.texture_maps.ctypes.data_as(C.POINTER(C.c_uint8))
            d.num_textures, d.tex_height, d.tex_width = self.texture_maps.shape[:3]
        self._desc_keepalive = d
        return d

    def render_options(self, **overrides) -> capi.pt_render_options:
        o = dict(self.options)
        o.update(overrides)
        return capi.make_options(**o)

    def pt_camera(self) -> capi.pt_camera:
        c = self.camera
        return capi.make_camera(c["position"], c["up"], c["right"], c["forward"], c["fov"],
                                c.get("focal_dist", 0.1), c.get("aperture", 0.0))

    def mesh_desc(self):
        """Meshes and instances for pt_create_gpu_bvh, recovered from the
        flattened BVH: each TLAS leaf gives an instance's BLAS root and
        material, each BLAS its (contiguous) triangle range.  Returns the
        arrays (mesh_tri_offset, instance_mesh, instance_material)."""
        bn = self.bvh_nodes
        top = int(self.top_level_index)
        inst_root = {}
        inst_mat = {}
        for i in range(top, bn.shape[0]):
            if bn[i, 8] < 0:
                inst = int(-bn[i, 8]) - 1
                inst_root[inst] = int(bn[i, 6])
                inst_mat[inst] = int(bn[i, 7])
        ranges = {}
        for root in set(inst_root.values()):
            lo, hi, stack = None, None, [root]
            while stack:
                b = stack.pop()
                if bn[b, 8] == 0:
                    stack += [int(bn[b, 6]), int(bn[b, 7])]
                elif bn[b, 8] > 0 and int(bn[b, 7]) > 0:
                    f, c = int(bn[b, 6]), int(bn[b, 7])
                    lo = f if lo is None else min(lo, f)
                    hi = f + c if hi is None else max(hi, f + c)
            ranges[root] = (lo or 0, hi or 0)
        starts = sorted(set(r for r in ranges.values()))
        offsets, mesh_of_range = [0], {}
        for lo, hi in starts:
            if lo > offsets[-1]:
                offsets.append(lo)  # triangles no instance uses: a mesh of their own
            if lo < offsets[-1]:
                raise ValueError("BLAS triangle ranges overlap")
            mesh_of_range[(lo, hi)] = len(offsets) - 1
            offsets.append(hi)
        if offsets[-1] < self.num_tris:
            offsets.append(self.num_tris)
        n = self.transforms.shape[0]
        inst_mesh = np.array([mesh_of_range[ranges[inst_root[i]]] for i in range(n)], np.int32)
        inst_material = np.array([inst_mat[i] for i in range(n)], np.int32)
        return np.array(offsets, np.int32), inst_mesh, inst_material

    # ------------------------------------------------------------------
    def save_npz(self, path: str):
        arrays = dict(bvh_nodes=self.bvh_nodes, vert_indices=self.vert_indices, vertices_uvx=self.vertices_uvx,
                      normals_uvy=self.normals_uvy, transforms=self.transforms, materials=self.materials,
                      lights=self.lights)
        if self.envmap_rgb is not None:
            arrays["envmap_rgb"] = self.envmap_rgb
            arrays["envmap_cdf"] = self.envmap_cdf
        if self.texture_maps is not None and self.texture_maps.size:
            arrays["texture_maps"] = self.texture_maps
        meta = dict(top_level_index=int(self.top_level_index), envmap_total_sum=float(self.envmap_total_sum),
                    options=self.options, camera=self.camera)
        np.savez_compressed(path, meta=np.frombuffer(json.dumps(meta).encode(), np.uint8), **arrays)

    def save_flat(self, path: str):
        """One binary file of the scene for C++ callers: "PTSCENE1", 12 int32
        counts (nodes, top level index, triangles, vertices, instances,
        materials, lights, envmap width and height, textures, texture width
        and height), the envmap total as a float, pt_render_options,
        pt_camera, then the arrays in the order of the counts (vertices and
        normals both with the vertex count; envmap RGB then CDF)."""
        import struct
        o, c = self.render_options(), self.pt_camera()
        ew, eh = (self.envmap_rgb.shape[1], self.envmap_rgb.shape[0]) if self.envmap_rgb is not None else (0, 0)
        tex = self.texture_maps if self.texture_maps is not None and self.texture_maps.size else None
        nt, th, tw = (tex.shape[0], tex.shape[1], tex.shape[2]) if tex is not None else (0, 0, 0)
        counts = [self.bvh_nodes.shape[0], int(self.top_level_index), self.vert_indices.shape[0],
                  self.vertices_uvx.shape[0], self.transforms.shape[0], self.materials.shape[0],
                  self.lights.shape[0], ew, eh, nt, tw, th]
        with open(path, "wb") as fh:
            fh.write(b"PTSCENE1")
            fh.write(struct.pack("<12i", *counts))
            fh.write(struct.pack("<f", float(self.envmap_total_sum)))
            fh.write(bytes(o))
            fh.write(bytes(c))
            for a in (self.bvh_nodes, self.vert_indices, self.vertices_uvx, self.normals_uvy, self.transforms,
                      self.materials, self.lights):
                fh.write(np.ascontiguousarray(a).tobytes())
            if ew:
                fh.write(np.ascontiguousarray(self.envmap_rgb, F).tobytes())
                fh.write(np.ascontiguousarray(self.envmap_cdf, F).tobytes())
            if tex is not None:
                fh.write(np.ascontiguousarray(tex, np.uint8).tobytes())

    @staticmethod
    def load_npz(path: str) -> "SceneData":
        z = np.load(path)
        meta = json.loads(bytes(z["meta"]).decode())
        return SceneData(
            bvh_nodes=z["bvh_nodes"], top_level_index=meta["top_level_index"], vert_indices=z["vert_indices"],
            vertices_uvx=z["vertices_uvx"], normals_uvy=z["normals_uvy"], transforms=z["transforms"],
            materials=z["materials"], lights=z["lights"],
            envmap_rgb=z["envmap_rgb"] if "envmap_rgb" in z else None,
            envmap_cdf=z["envmap_cdf"] if "envmap_cdf" in z else None,
            envmap_total_sum=meta["envmap_total_sum"], options=meta["options"], camera=meta["camera"],
            texture_maps=z["texture_maps"] if "texture_maps" in z else None)


def load_ref_dump(prefix: str) -> SceneData:
    """Read the <prefix>.json / <prefix>.bin pair written by the reference
    scene dumper (oracle/ref_host/ref_scene_dump.cpp)."""
    with open(prefix + ".json") as fh:
        m = json.load(fh)
    assert m["sizeof_node"] == 36 and m["sizeof_material"] == 128 and m["sizeof_light"] == 60
    raw = open(prefix + ".bin", "rb").read()
    off = 0

    def take(dtype, count):
        nonlocal off
        nbytes = np.dtype(dtype).itemsize * count
        a = np.frombuffer(raw, dtype, count, off).copy()
        off += nbytes
        return a

    nodes = take(F, 9 * m["num_bvh_nodes"])
    idx = take(I, 3 * m["num_tris"])
    verts = take(F, 4 * m["num_vertices"])
    norms = take(F, 4 * m["num_vertices"])
    xf = take(F, 16 * m["num_instances"])
    mats = take(F, 32 * m["num_materials"])
    lights = take(F, 15 * m["num_lights"])
    env = cdf = None
    if m["envmap_width"]:
        w, h = m["envmap_width"], m["envmap_height"]
        env = take(F, 3 * w * h).reshape(h, w, 3)
        cdf = take(F, w * h).reshape(h, w)
    tex = None
    if m["num_textures"]:
        tex = take(np.uint8, 4 * m["tex_width"] * m["tex_height"] * m["num_textures"]).reshape(
            m["num_textures"], m["tex_height"], m["tex_width"], 4)
    assert off == len(raw), (off, len(raw))
    return SceneData(bvh_nodes=nodes, top_level_index=m["top_level_index"], vert_indices=idx, vertices_uvx=verts,
                     normals_uvy=norms, transforms=xf, materials=mats, lights=lights, envmap_rgb=env, envmap_cdf=cdf,
                     envmap_total_sum=m["envmap_total_sum"], texture_maps=tex, options=m["options"],
                     camera=m["camera"])
