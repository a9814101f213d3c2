"""Scene construction on the host: materials, lights, cameras and envmaps in
the reference's layouts, the native BVH build (libptscene.so) and the
synthetic benchmark scenes.

Layouts follow the reference's host types: Material (src/core/Material.h),
Light and its loader rules (src/core/Scene.h:50-59, src/loaders/Loader.cpp:
165-205), Camera (src/core/Camera.cpp:124-165) and EnvironmentMap::BuildCDF
(src/core/EnvironmentMap.cpp:39-61).
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

from .capi import PKG_DIR
from .scene import SceneData

F32 = np.float32
SCENE_LIB = os.path.join(PKG_DIR, "csrc", "libptscene.so")
_slib = None


def build_scene_lib(force: bool = False) -> str:
    src = os.path.join(PKG_DIR, "csrc", "scene_build.cpp")
    if force or not os.path.exists(SCENE_LIB) or os.path.getmtime(src) > os.path.getmtime(SCENE_LIB):
        subprocess.run(["g++", "-O2", "-std=c++17", "-fopenmp", "-fPIC", "-shared", src, "-o", SCENE_LIB],
                       check=True)
    return SCENE_LIB


def _scene_lib():
    global _slib
    if _slib is None:
        build_scene_lib()
        _slib = C.CDLL(SCENE_LIB)
        P = C.c_void_p
        _slib.ptgb_scene_build.restype = P
        _slib.ptgb_scene_build.argtypes = [C.c_int, P, P, P, C.c_int, P, P, P]
        _slib.ptgb_scene_sizes.argtypes = [P, P, P, P, P]
        _slib.ptgb_scene_copy.argtypes = [P, P, P, P, P]
        _slib.ptgb_scene_free.argtypes = [P]
    return _slib


# ------------------------------------------------------------------ records
def material(color=(1.0, 1.0, 1.0), emission=(0.0, 0.0, 0.0), metallic=0.0, roughness=0.5, subsurface=0.0,
             specular_tint=0.0, sheen=0.0, sheen_tint=0.0, clearcoat=0.0, clearcoat_gloss=0.0, spec_trans=0.0,
             ior=1.5, anisotropic=0.0, medium_type=0, medium_density=0.0, medium_color=(1.0, 1.0, 1.0),
             medium_anisotropy=0.0, opacity=1.0, alpha_mode=0, alpha_cutoff=0.0) -> np.ndarray:
    """GLSLPT::Material as 32 floats (defaults of Material.h:47-85)."""
    m = np.zeros(32, F32)
    m[0:3] = color
    m[3] = anisotropic
    m[4:7] = emission
    m[8], m[9], m[10], m[11] = metallic, roughness, subsurface, specular_tint
    m[12], m[13], m[14], m[15] = sheen, sheen_tint, clearcoat, clearcoat_gloss
    m[16], m[17], m[18], m[19] = spec_trans, ior, medium_type, medium_density
    m[20:23] = medium_color
    m[23] = medium_anisotropy
    m[24:28] = -1.0  # no texture maps
    m[28], m[29], m[30] = opacity, alpha_mode, alpha_cutoff
    return m


def quad_light(position, v1, v2, emission) -> np.ndarray:
    """Loader.cpp:185-191: u = v1 - position, v = v2 - position, area = |u x v|."""
    p = np.asarray(position, F32)
    u = np.asarray(v1, F32) - p
    v = np.asarray(v2, F32) - p
    L = np.zeros(15, F32)
    L[0:3], L[3:6], L[6:9], L[9:12] = p, emission, u, v
    L[13] = np.float32(np.linalg.norm(np.cross(u.astype(np.float64), v.astype(np.float64))))
    L[14] = 0
    return L


def sphere_light(position, radius, emission) -> np.ndarray:
    L = np.zeros(15, F32)
    L[0:3], L[3:6] = position, emission
    L[12] = radius
    L[13] = np.float32(4.0) * np.float32(math.pi) * np.float32(radius) * np.float32(radius)
    L[14] = 1
    return L


def camera(eye, lookat, fov_deg, focal_dist=1.0, aperture=0.0) -> dict:
    """GLSLPT::Camera(eye, lookat, fov) (Camera.cpp:124-165), in float32."""
    eye = np.asarray(eye, F32)
    look = np.asarray(lookat, F32)
    d = look - eye
    d = d / np.float32(np.sqrt(np.dot(d, d)))
    pitch = np.float32(math.degrees(math.asin(float(d[1]))))
    yaw = np.float32(math.degrees(math.atan2(float(d[2]), float(d[0]))))
    radius = np.float32(np.sqrt(np.dot(look - eye, look - eye)))
    rp, ry = math.radians(float(pitch)), math.radians(float(yaw))
    f = np.array([math.cos(ry) * math.cos(rp), math.sin(rp), math.sin(ry) * math.cos(rp)], F32)
    f = f / np.float32(np.sqrt(np.dot(f, f)))
    pos = look + f * np.float32(-1.0) * radius
    up_w = np.array([0, 1, 0], F32)
    right = np.cross(f, up_w).astype(F32)
    right = right / np.float32(np.sqrt(np.dot(right, right)))
    up = np.cross(right, f).astype(F32)
    up = up / np.float32(np.sqrt(np.dot(up, up)))
    return dict(position=pos.tolist(), up=up.tolist(), right=right.tolist(), forward=f.tolist(),
                fov=float(np.float32(math.radians(fov_deg))), focal_dist=float(focal_dist), aperture=float(aperture))


def envmap_cdf(img: np.ndarray):
    """EnvironmentMap::BuildCDF: running float sum of the luminance."""
    img = np.ascontiguousarray(img, F32)
    w = (F32(0.212671) * img[..., 0] + F32(0.715160) * img[..., 1]) + F32(0.072169) * img[..., 2]
    cdf = np.cumsum(w.reshape(-1), dtype=F32).reshape(img.shape[:2])
    return cdf, float(cdf.reshape(-1)[-1])


def mat4(rot=None, scale=(1, 1, 1), translate=(0, 0, 0)) -> np.ndarray:
    """Mat4 in the reference's row-vector layout (scale * rot * translate,
    Loader.cpp:449): rows 0-2 the transformed axes, row 3 the translation."""
    R = np.eye(3) if rot is None else np.asarray(rot, np.float64)
    S = np.diag(scale).astype(np.float64)
    M = np.eye(4)
    M[:3, :3] = S @ R  # row-vector convention: p' = p * (S * R)
    M[3, :3] = translate
    return M.astype(F32).reshape(16)


def rot_y(deg):
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    # row-vector rotation about +y
    return np.array([[c, 0, -s], [0, 1, 0], [s, 0, c]])


def random_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    x, y, z, w = q
    # QuatToMatrix layout (Mat4.h:79-114), row-vector form
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y + w * z), 2 * (x * z - w * y)],
                     [2 * (x * y - w * z), 1 - 2 * (x * x + z * z), 2 * (y * z + w * x)],
                     [2 * (x * z + w * y), 2 * (y * z - w * x), 1 - 2 * (x * x + y * y)]])


# ------------------------------------------------------------------ meshes
class Mesh:
    """Non-indexed triangle list as the reference keeps it (Mesh.cpp:65-101):
    positions + u in verticesUVX, normals + v in normalsUVY."""

    def __init__(self, positions: np.ndarray, normals: np.ndarray, uv: np.ndarray | None = None):
        n = positions.shape[0]
        assert n % 3 == 0
        if uv is None:  # OBJ without texcoords: (0,0), (0,1), (1,1) per triangle (Mesh.cpp:81-89)
            uv = np.tile(np.array([[0, 0], [0, 1], [1, 1]], F32), (n // 3, 1))
        self.verts = np.concatenate([positions.astype(F32), uv[:, :1].astype(F32)], axis=1)
        self.norms = np.concatenate([normals.astype(F32), uv[:, 1:2].astype(F32)], axis=1)

    @property
    def num_tris(self):
        return self.verts.shape[0] // 3


def mesh_from_indexed(V: np.ndarray, Fc: np.ndarray, N: np.ndarray | None = None) -> Mesh:
    V = np.asarray(V, np.float64)
    Fc = np.asarray(Fc, np.int64)
    if N is None:
        fn = np.cross(V[Fc[:, 1]] - V[Fc[:, 0]], V[Fc[:, 2]] - V[Fc[:, 0]])
        N = np.zeros_like(V)
        for k in range(3):
            np.add.at(N, Fc[:, k], fn)
        N /= np.maximum(np.linalg.norm(N, axis=1, keepdims=True), 1e-30)
    return Mesh(V[Fc].reshape(-1, 3), np.asarray(N)[Fc].reshape(-1, 3))


def quad_mesh(p0, p1, p2, p3, normal) -> Mesh:
    P = np.array([p0, p1, p2, p0, p2, p3], np.float64)
    Nn = np.tile(np.asarray(normal, np.float64), (6, 1))
    return Mesh(P, Nn)


def cube_mesh() -> Mesh:
    """Unit cube [-0.5, 0.5]^3 with flat outward normals (12 triangles)."""
    tris, norms = [], []
    for axis in range(3):
        for sgn in (-1.0, 1.0):
            n = np.zeros(3)
            n[axis] = sgn
            u = np.zeros(3); u[(axis + 1) % 3] = 1
            v = np.zeros(3); v[(axis + 2) % 3] = 1
            c = n * 0.5
            q = [c - 0.5 * u - 0.5 * v, c + 0.5 * u - 0.5 * v, c + 0.5 * u + 0.5 * v, c - 0.5 * u + 0.5 * v]
            if sgn < 0:
                q = q[::-1]
            tris += [q[0], q[1], q[2], q[0], q[2], q[3]]
            norms += [n] * 6
    return Mesh(np.array(tris), np.array(norms))


def _value_noise(P: np.ndarray, seed: int, octaves: int = 3, base_freq: float = 4.0, lattice: int = 64):
    """3-octave value noise: trilinear interpolation (smoothstep weights) of
    seeded random lattice values, octave k at base_freq * 2^k with weight
    2^-k, normalised to [-1, 1]."""
    rng = np.random.RandomState(seed)
    table = rng.uniform(-1.0, 1.0, size=(octaves, lattice, lattice, lattice))
    out = np.zeros(P.shape[0])
    norm = 0.0
    for o in range(octaves):
        f = base_freq * (2 ** o)
        q = (P + 1.5) * f
        i0 = np.floor(q).astype(np.int64)
        t = q - i0
        t = t * t * (3 - 2 * t)
        acc = np.zeros(P.shape[0])
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    w = (t[:, 0] if dx else 1 - t[:, 0]) * (t[:, 1] if dy else 1 - t[:, 1]) * (t[:, 2] if dz else 1 - t[:, 2])
                    idx = (i0 + np.array([dx, dy, dz])) % lattice
                    acc += w * table[o, idx[:, 0], idx[:, 1], idx[:, 2]]
        amp = 0.5 ** o
        out += amp * acc
        norm += amp
    return out / norm


def icosphere(freq: int, radius=1.0, displace=0.0, seed=1):
    """Geodesic icosphere of 20 * freq^2 triangles (each icosahedron face
    split into freq^2), vertices on the sphere, optionally displaced radially
    by 3-octave value noise of amplitude `displace`.  Returns (V, F, face_of_tri)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    ico_v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t],
                      [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    ico_v /= np.linalg.norm(ico_v, axis=1, keepdims=True)
    ico_f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                      [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                      [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    n = freq
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    mask = ii + jj <= n
    gi, gj = ii[mask], jj[mask]
    local = -np.ones((n + 1, n + 1), np.int64)
    local[gi, gj] = np.arange(gi.size)
    # triangles of one face in (i, j) lattice coordinates
    up_i, up_j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    m_up = up_i + up_j <= n - 1
    a, b = up_i[m_up], up_j[m_up]
    tri_up = np.stack([local[a, b], local[a + 1, b], local[a, b + 1]], 1)
    m_dn = up_i + up_j <= n - 2
    a, b = up_i[m_dn], up_j[m_dn]
    tri_dn = np.stack([local[a + 1, b], local[a + 1, b + 1], local[a, b + 1]], 1)
    tri_local = np.concatenate([tri_up, tri_dn])
    allV, allF, face_id = [], [], []
    for f, (A, B, Cc) in enumerate(ico_f):
        PA, PB, PC = ico_v[A], ico_v[B], ico_v[Cc]
        P = PA + np.outer(gi / n, PB - PA) + np.outer(gj / n, PC - PA)
        P /= np.linalg.norm(P, axis=1, keepdims=True)
        allF.append(tri_local + f * gi.size)
        allV.append(P)
        face_id.append(np.full(tri_local.shape[0], f))
    V = np.concatenate(allV)
    Fc = np.concatenate(allF)
    face_id = np.concatenate(face_id)
    # weld the vertices shared along face edges
    key = np.round(V * 1e9).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    V = V[first]
    Fc = inv.reshape(-1)[Fc]
    if displace:
        V = V * (1.0 + displace * _value_noise(V, seed))[:, None]
    return V * radius, Fc, face_id


def torus(major=1.0, minor=0.35, nu=100, nv=250, displace=0.0, seed=0):
    u = np.linspace(0, 2 * np.pi, nu, endpoint=False)
    v = np.linspace(0, 2 * np.pi, nv, endpoint=False)
    U, Vv = np.meshgrid(u, v, indexing="ij")
    P = np.stack([(major + minor * np.cos(Vv)) * np.cos(U), minor * np.sin(Vv),
                  (major + minor * np.cos(Vv)) * np.sin(U)], -1).reshape(-1, 3)
    if displace:
        nrm = P - np.stack([major * np.cos(U), 0 * U, major * np.sin(U)], -1).reshape(-1, 3)
        nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
        P = P + nrm * (displace * _value_noise(P / (major + minor), seed))[:, None]
    idx = np.arange(nu * nv).reshape(nu, nv)
    a = idx
    b = np.roll(idx, -1, 0)
    c = np.roll(idx, -1, 1)
    d = np.roll(np.roll(idx, -1, 0), -1, 1)
    Fc = np.concatenate([np.stack([a, c, b], -1).reshape(-1, 3), np.stack([b, c, d], -1).reshape(-1, 3)])
    return P, Fc


# ------------------------------------------------------------------ build
def build_scene(meshes: list[Mesh], instances: list[tuple[int, int, np.ndarray]], materials, lights, cam: dict,
                options: dict, envmap: np.ndarray | None = None) -> SceneData:
    """Run the native BVH build + flattening and return the reference-layout
    arrays.  instances: (mesh id, material id, Mat4 as 16 floats)."""
    lib = _scene_lib()
    offs = np.zeros(len(meshes) + 1, np.int32)
    for i, m in enumerate(meshes):
        offs[i + 1] = offs[i] + m.num_tris
    V = np.ascontiguousarray(np.concatenate([m.verts for m in meshes]), F32)
    N = np.ascontiguousarray(np.concatenate([m.norms for m in meshes]), F32)
    im = np.array([i[0] for i in instances], np.int32)
    imat = np.array([i[1] for i in instances], np.int32)
    ixf = np.ascontiguousarray(np.stack([np.asarray(i[2], F32).reshape(16) for i in instances]), F32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    h = lib.ptgb_scene_build(len(meshes), p(offs), p(V), p(N), len(instances), p(im), p(imat), p(ixf))
    if not h:
        raise RuntimeError("scene build failed")
    sz = [C.c_int32() for _ in range(4)]
    lib.ptgb_scene_sizes(h, *[C.byref(s) for s in sz])
    nn, top, nt, nv = (s.value for s in sz)
    nodes = np.zeros((nn, 9), F32)
    vidx = np.zeros((nt, 3), np.int32)
    verts = np.zeros((nv, 4), F32)
    norms = np.zeros((nv, 4), F32)
    lib.ptgb_scene_copy(h, p(nodes), p(vidx), p(verts), p(norms))
    lib.ptgb_scene_free(h)
    env = cdf = None
    total = 0.0
    if envmap is not None:
        env = np.ascontiguousarray(envmap, F32)
        cdf, total = envmap_cdf(env)
    mats = np.stack([np.asarray(m, F32) for m in materials])
    lts = np.stack([np.asarray(l, F32) for l in lights]) if lights else np.zeros((0, 15), F32)
    sd = SceneData(bvh_nodes=nodes, top_level_index=top, vert_indices=vidx, vertices_uvx=verts, normals_uvy=norms,
                   transforms=ixf, materials=mats, lights=lts, envmap_rgb=env, envmap_cdf=cdf, envmap_total_sum=total,
                   options=options, camera=cam)
    sd.instance_mesh = im
    sd.instance_material = imat
    return sd


# --------------------------------------------------------- benchmark scenes
def cornell(width=256, height=256, max_depth=4, tile=None) -> SceneData:
    """Procedural Cornell box: five wall quads (10 triangles) in the unit
    cube, a tall box rotated 15 degrees and a short box rotated -18 degrees
    (12 triangles each, one shared cube mesh under two instance transforms),
    a 0.25 x 0.25 quad light under the ceiling with emission (17, 12, 4);
    diffuse Disney materials (white 0.73, red (0.65,0.05,0.05), green
    (0.12,0.45,0.15)), roughness 1, metallic 0."""
    white = material(color=(0.73, 0.73, 0.73), roughness=1.0)
    red = material(color=(0.65, 0.05, 0.05), roughness=1.0)
    green = material(color=(0.12, 0.45, 0.15), roughness=1.0)
    mats = [material(), white, red, green]  # slot 0: the loader's default material
    walls_white = Mesh(
        np.concatenate([quad_mesh((0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1), (0, 1, 0)).verts[:, :3],
                        quad_mesh((0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0), (0, -1, 0)).verts[:, :3],
                        quad_mesh((0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1), (0, 0, -1)).verts[:, :3]]),
        np.concatenate([np.tile([0, 1, 0], (6, 1)), np.tile([0, -1, 0], (6, 1)), np.tile([0, 0, -1], (6, 1))]))
    wall_red = quad_mesh((0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 1, 0), (1, 0, 0))
    wall_green = quad_mesh((1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1), (-1, 0, 0))
    cube = cube_mesh()
    meshes = [walls_white, wall_red, wall_green, cube]
    ident = mat4()
    tall = mat4(rot_y(15.0), scale=(0.3, 0.6, 0.3), translate=(0.34, 0.3, 0.62))
    short = mat4(rot_y(-18.0), scale=(0.3, 0.3, 0.3), translate=(0.66, 0.15, 0.34))
    instances = [(0, 1, ident), (1, 2, ident), (2, 3, ident), (3, 1, tall), (3, 1, short)]
    light = quad_light((0.375, 0.999, 0.375), (0.625, 0.999, 0.375), (0.375, 0.999, 0.625), (17.0, 12.0, 4.0))
    cam = camera((0.5, 0.5, -1.35), (0.5, 0.5, 0.0), 40.0)
    opts = dict(render_width=width, render_height=height, tile_width=tile or width, tile_height=tile or height,
                max_depth=max_depth)
    return build_scene(meshes, instances, mats, [light], cam, opts)


def icosphere_scene(freq=229, width=1920, height=1080, max_depth=8, seed=1, tile=None) -> SceneData:
    """The icosphere workload (icosphere_recipe) built into reference-layout arrays."""
    return build_scene(**icosphere_recipe(freq, width, height, max_depth, seed, tile))


def icosphere_recipe(freq=229, width=1920, height=1080, max_depth=8, seed=1, tile=None) -> dict:
    """build_scene's arguments for a
    ~1.05M-triangle geodesic icosphere (20 * freq^2 triangles; freq=229 gives
    1,048,820), radially displaced by 3-octave value noise (amplitude 0.05,
    seed `seed`), split into 16 meshes by icosahedron face (face % 16), one
    material each: baseColor U[0,1]^3, metallic U{0,1}, roughness U[0.05,1],
    clearcoat U[0,1], transmission 1 on two materials, IOR 1.5; one sphere
    light of radius 0.5 and emission 20."""
    V, Fc, face = icosphere(freq, 1.0, 0.05, seed)
    rng = np.random.RandomState(seed + 100)
    mats = [material()]
    glass = set(rng.choice(16, 2, replace=False).tolist())
    for k in range(16):
        trans = 1.0 if k in glass else 0.0
        mats.append(material(color=tuple(rng.uniform(0, 1, 3)), metallic=float(rng.randint(0, 2)) * (1 - trans),
                             roughness=float(rng.uniform(0.05, 1.0)), clearcoat=float(rng.uniform(0, 1)),
                             spec_trans=trans, ior=1.5))
    # smooth normals of the whole displaced surface
    fn = np.cross(V[Fc[:, 1]] - V[Fc[:, 0]], V[Fc[:, 2]] - V[Fc[:, 0]])
    Nv = np.zeros_like(V)
    for k in range(3):
        np.add.at(Nv, Fc[:, k], fn)
    Nv /= np.maximum(np.linalg.norm(Nv, axis=1, keepdims=True), 1e-30)
    meshes, instances = [], []
    ident = mat4()
    for g in range(16):
        sel = Fc[(face % 16) == g]
        meshes.append(mesh_from_indexed(V, sel, Nv))
        instances.append((g, g + 1, ident))
    light = sphere_light((2.2, 2.4, 2.6), 0.5, (20.0, 20.0, 20.0))
    cam = camera((0.0, 0.0, 3.2), (0.0, 0.0, 0.0), 45.0)
    opts = dict(render_width=width, render_height=height, tile_width=tile or 256, tile_height=tile or 256,
                max_depth=max_depth)
    return dict(meshes=meshes, instances=instances, materials=mats, lights=[light], cam=cam, options=opts)


def diff_scene(freq=229, width=512, height=512, max_depth=6, num_materials=32, seed=1, tile=None) -> SceneData:
    """The differentiable-materials workload: the displaced icosphere split
    into num_materials meshes by icosahedron face (face % num_materials), one
    material each with every Disney lobe active -- baseColor U[0.05,0.95]^3,
    metallic, roughness, subsurface, specularTint, sheen, sheenTint,
    clearcoat U[0.05,0.95], clearcoatGloss U[0.05,0.95] -- and four sphere
    lights of radius 0.5 around the camera side of the sphere."""
    V, Fc, face = icosphere(freq, 1.0, 0.05, seed)
    rng = np.random.RandomState(seed + 200)
    mats = [material()]
    for k in range(num_materials):
        u = rng.uniform(0.05, 0.95, 11)
        mats.append(material(color=tuple(u[0:3]), metallic=float(u[3]), roughness=float(u[4]),
                             subsurface=float(u[5]), specular_tint=float(u[6]), sheen=float(u[7]),
                             sheen_tint=float(u[8]), clearcoat=float(u[9]), clearcoat_gloss=float(u[10]), ior=1.5))
    fn = np.cross(V[Fc[:, 1]] - V[Fc[:, 0]], V[Fc[:, 2]] - V[Fc[:, 0]])
    Nv = np.zeros_like(V)
    for k in range(3):
        np.add.at(Nv, Fc[:, k], fn)
    Nv /= np.maximum(np.linalg.norm(Nv, axis=1, keepdims=True), 1e-30)
    meshes, instances = [], []
    ident = mat4()
    for g in range(num_materials):
        sel = Fc[(face % num_materials) == g]
        meshes.append(mesh_from_indexed(V, sel, Nv))
        instances.append((g, g + 1, ident))
    lights = [sphere_light((2.2, 2.4, 2.6), 0.5, (20.0, 18.0, 16.0)),
              sphere_light((-2.4, 1.8, 2.2), 0.5, (8.0, 10.0, 14.0)),
              sphere_light((2.0, -2.2, 2.4), 0.5, (12.0, 9.0, 6.0)),
              sphere_light((-2.0, -2.0, 2.8), 0.5, (6.0, 12.0, 8.0))]
    cam = camera((0.0, 0.0, 3.2), (0.0, 0.0, 0.0), 45.0)
    opts = dict(render_width=width, render_height=height, tile_width=tile or 256, tile_height=tile or 256,
                max_depth=max_depth)
    return build_scene(meshes, instances, mats, lights, cam, opts)


def sky_envmap(width=2048, height=1024, sun_dir=(0.4, 0.7, 0.3), sun_radius_deg=0.5, sun_intensity=5.0e4):
    """Synthetic equirect HDR in the reference's mapping (envmap.glsl:57-66):
    sky gradient 0.5 (horizon and below) to 1.5 (zenith) plus a sun disc."""
    v = (np.arange(height) + 0.5) / height
    u = (np.arange(width) + 0.5) / width
    theta = v * np.pi
    phi = u * 2 * np.pi - np.pi
    TH, PH = np.meshgrid(theta, phi, indexing="ij")
    d = np.stack([np.sin(TH) * np.cos(PH), np.cos(TH), np.sin(TH) * np.sin(PH)], -1)
    sky = 0.5 + np.clip(d[..., 1], 0, 1)
    img = np.stack([sky * 0.8, sky * 0.9, sky * 1.0], -1)
    s = np.asarray(sun_dir, np.float64)
    s /= np.linalg.norm(s)
    cosang = d @ s
    img[cosang > math.cos(math.radians(sun_radius_deg))] = sun_intensity
    return img.astype(F32)


def instanced_scene(num_instances=10000, tris_per_blas=50000, width=1920, height=1080, max_depth=8, seed=5,
                    env_size=(2048, 1024), tile=None) -> SceneData:
    """The instanced workload (instanced_recipe) built into reference-layout arrays."""
    return build_scene(**instanced_recipe(num_instances, tris_per_blas, width, height, max_depth, seed, env_size,
                                          tile))


def instanced_recipe(num_instances=10000, tris_per_blas=50000, width=1920, height=1080, max_depth=8, seed=5,
                     env_size=(2048, 1024), tile=None) -> dict:
    """build_scene's arguments for two-level instancing + IBL + volume: 5 BLAS meshes (displaced spheres
    and tori, ~tris_per_blas triangles each), num_instances instances with
    uniform random rotation, scale U[0.5, 2] and positions in a 200 x 200
    plane; a synthetic equirect sky with a sun disc; one homogeneous-volume
    cube (sigma_a 0.1, sigma_s 1.0: density 1.1, albedo 0.909) with volume MIS."""
    rng = np.random.RandomState(seed)
    meshes = []
    f = max(2, int(round(math.sqrt(tris_per_blas / 20.0))))
    for k in range(3):
        V, Fc, _ = icosphere(f, 1.0, 0.08 + 0.02 * k, seed + k)
        meshes.append(mesh_from_indexed(V, Fc))
    for k in range(2):
        nv = int(round(math.sqrt(tris_per_blas / 2 * 2.5)))
        nu = max(3, int(round(tris_per_blas / 2 / nv)))
        P, Fc = torus(1.0, 0.3 + 0.05 * k, nu, nv, 0.05, seed + 10 + k)
        meshes.append(mesh_from_indexed(P, Fc))
    meshes.append(cube_mesh())  # volume boundary
    mats = [material()]
    for k in range(8):
        mats.append(material(color=tuple(rng.uniform(0.05, 0.95, 3)), metallic=float(rng.randint(0, 2)),
                             roughness=float(rng.uniform(0.05, 1.0)), clearcoat=float(rng.uniform(0, 1))))
    vol_mat = len(mats)
    mats.append(material(color=(1, 1, 1), spec_trans=1.0, roughness=0.0, medium_type=2, medium_density=1.1,
                         medium_color=(0.909, 0.909, 0.909), alpha_mode=1, opacity=0.0))
    instances = []
    for i in range(num_instances):
        R = random_rotation(rng)
        s = rng.uniform(0.5, 2.0)
        pos = (rng.uniform(-100, 100), s, rng.uniform(-100, 100))
        instances.append((int(rng.randint(0, 5)), int(rng.randint(1, 9)), mat4(R, (s, s, s), pos)))
    instances.append((5, vol_mat, mat4(None, (24, 24, 24), (0, 12, 0))))
    env = sky_envmap(*env_size)
    cam = camera((0.0, 45.0, -150.0), (0.0, 0.0, 0.0), 60.0)
    opts = dict(render_width=width, render_height=height, tile_width=tile or 256, tile_height=tile or 256,
                max_depth=max_depth, enable_envmap=1, enable_volume_mis=1)
    return dict(meshes=meshes, instances=instances, materials=mats, lights=[], cam=cam, options=opts, envmap=env)
