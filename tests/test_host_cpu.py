"""Host-side parts without a GPU: the C ABI library's exports, the scene
builder (checked with the oracle against brute force), and the collapse of
the reference's binary BVH into the 8-wide quantised layout."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden_scene


def header_functions():
    txt = open(os.path.join(ROOT, "include", "pt_cuda.h")).read()
    return sorted(set(re.findall(r"^int\s+(pt_\w+)\s*\(", txt, re.M)))


def test_library_exports_every_header_symbol():
    from pathtracer import build, capi
    build.build_library()
    lib = C.CDLL(capi.LIB_PATH)
    names = header_functions()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(capi.HEADER_SYMBOLS) == names


def test_last_error_without_gpu():
    from pathtracer import capi
    lib = capi.load_library()
    ctx = C.c_void_p()
    rc = lib.pt_create(None, None, C.byref(ctx))
    assert rc == capi.PT_ERR_INVALID_ARG
    buf = C.create_string_buffer(256)
    assert lib.pt_last_error(buf, 256) == 0
    assert b"NULL" in buf.value


def brute_closest(sd, rays):
    """Closest triangle over all instances by brute force (float64)."""
    out_t = np.full(len(rays), np.inf)
    out_p = np.full(len(rays), -1)
    nodes = sd.bvh_nodes
    top = sd.top_level_index
    # instance -> BLAS root, collect each BLAS's triangle range by walking it
    leaves = [i for i in range(top, nodes.shape[0]) if nodes[i, 8] < 0]
    V = sd.vertices_uvx[:, :3].astype(np.float64)
    for li in leaves:
        inst = int(-nodes[li, 8] - 1)
        root = int(nodes[li, 6])
        tris, stack = [], [root]
        while stack:
            n = stack.pop()
            if nodes[n, 8] > 0:
                tris += list(range(int(nodes[n, 6]), int(nodes[n, 6] + nodes[n, 7])))
            elif nodes[n, 8] == 0:
                stack += [int(nodes[n, 6]), int(nodes[n, 7])]
        M = sd.transforms[inst].reshape(4, 4).astype(np.float64)  # row-vector Mat4
        Minv = np.linalg.inv(M)
        o = np.c_[rays[:, :3], np.ones(len(rays))] @ Minv
        d = np.c_[rays[:, 3:], np.zeros(len(rays))] @ Minv
        o, d = o[:, :3], d[:, :3]
        idx = np.array(tris)
        vi = sd.vert_indices[idx]
        v0, v1, v2 = V[vi[:, 0]], V[vi[:, 1]], V[vi[:, 2]]
        e0, e1 = v1 - v0, v2 - v0
        for r in range(len(rays)):
            pv = np.cross(d[r], e1)
            det = np.einsum("ij,ij->i", e0, pv)
            tv = o[r] - v0
            qv = np.cross(tv, e0)
            with np.errstate(divide="ignore", invalid="ignore"):
                u = np.einsum("ij,ij->i", tv, pv) / det
                v = (qv @ d[r]) / det
                t = np.einsum("ij,ij->i", e1, qv) / det
            ok = (u >= 0) & (v >= 0) & (u + v <= 1) & (t >= 0)
            if ok.any():
                j = np.argmin(np.where(ok, t, np.inf))
                if t[j] < out_t[r]:
                    out_t[r], out_p[r] = t[j], idx[j]
    return out_t, out_p


def random_rays(sd, n, seed, span=1.0):
    rng = np.random.RandomState(seed)
    lo = sd.bvh_nodes[sd.top_level_index, :3]
    hi = sd.bvh_nodes[sd.top_level_index, 3:6]
    c = 0.5 * (lo + hi)
    ext = np.linalg.norm(hi - lo)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = c + rng.uniform(-0.5, 0.5, (n, 3)) * (hi - lo) * span - d * ext * 0.1
    return np.ascontiguousarray(np.c_[o, d], np.float32)


@pytest.mark.parametrize("which", ["cornell", "icosphere", "instanced"])
def test_scene_builder_bvh_finds_brute_force_hits(orc, which):
    from pathtracer import scenes
    if which == "cornell":
        sd = scenes.cornell(32, 32)
    elif which == "icosphere":
        sd = scenes.icosphere_scene(freq=12, width=32, height=32)
    else:
        sd = scenes.instanced_scene(num_instances=30, tris_per_blas=800, width=32, height=32, env_size=(64, 32))
    rays = random_rays(sd, 96, 3)
    hits, cnt = orc.trace_closest(sd, rays, use_double=True)
    t_bf, p_bf = brute_closest(sd, rays)
    assert cnt["overflow"] == 0
    hit_bf = np.isfinite(t_bf)
    assert np.array_equal(hits["prim_id"] >= 0, hit_bf)
    m = hit_bf
    assert np.allclose(hits["t"][m], t_bf[m], rtol=1e-5, atol=1e-6)
    same = hits["prim_id"][m] == p_bf[m]
    assert same.mean() > 0.97  # the rest are ties at equal distance (shared edges)


class WideBVH(C.Structure):
    _fields_ = [("nodes", C.c_void_p), ("num_nodes", C.c_int32), ("tris", C.c_void_p), ("num_tris", C.c_int32),
                ("insts", C.c_void_p), ("num_inst_refs", C.c_int32), ("tlas_root", C.c_int32),
                ("tlas_first_node", C.c_int32), ("blas_depth", C.c_int32), ("tlas_depth", C.c_int32),
                ("impl", C.c_void_p)]


def collapse(sd):
    from pathtracer import capi
    lib = capi.load_library()
    lib.ptgb_build_wide.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                    C.c_void_p, C.c_int, C.POINTER(WideBVH), C.c_char_p, C.c_int]
    lib.ptgb_free_wide.argtypes = [C.POINTER(WideBVH)]
    w = WideBVH()
    err = C.create_string_buffer(256)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    rc = lib.ptgb_build_wide(p(sd.bvh_nodes), sd.bvh_nodes.shape[0], sd.top_level_index, p(sd.vert_indices),
                             sd.num_tris, p(sd.vertices_uvx), sd.vertices_uvx.shape[0], p(sd.transforms),
                             sd.transforms.shape[0], C.byref(w), err, 256)
    assert rc == 0, err.value
    nodes = np.ctypeslib.as_array((C.c_uint32 * (20 * w.num_nodes)).from_address(w.nodes)).reshape(-1, 20).copy()
    tris = np.ctypeslib.as_array((C.c_float * (12 * w.num_tris)).from_address(w.tris)).reshape(-1, 12).copy()
    insts = np.ctypeslib.as_array((C.c_int32 * (4 * w.num_inst_refs)).from_address(w.insts)).reshape(-1, 4).copy()
    info = dict(tlas_root=w.tlas_root, tlas_first=w.tlas_first_node, blas_depth=w.blas_depth, tlas_depth=w.tlas_depth)
    lib.ptgb_free_wide(C.byref(w))
    return nodes, tris, insts, info


MERGED_INSTANCE = 0x7FFFFFFF  # InstRef.instance of the BLAS merging all untransformed instances


def decode(node):
    p = node[0:3].view(np.float32).astype(np.float64)
    e = [(int(node[3]) >> (8 * k)) & 0xFF for k in range(3)]
    scale = np.array([2.0 ** (x - 127) for x in e])
    imask = int(node[3]) >> 24
    meta = node[6:8].view(np.uint8)
    q = node[8:20].view(np.uint8).reshape(6, 8).astype(np.float64)
    lo = p[:, None] + q[0:3] * scale[:, None]
    hi = p[:, None] + q[3:6] * scale[:, None]
    return dict(child_base=int(node[4]), prim_base=int(node[5]), imask=imask, meta=meta, lo=lo.T, hi=hi.T)


@pytest.mark.parametrize("which", ["ref_cornell", "ref_volume", "icosphere", "instanced"])
def test_wide_bvh_collapse_is_conservative_and_complete(which):
    from pathtracer import scenes
    sd = {"ref_cornell": lambda: golden_scene("ref_scene_cornell_box_orig.npz"),
          "ref_volume": lambda: golden_scene("ref_scene_volume_cube.npz"),
          "icosphere": lambda: scenes.icosphere_scene(freq=20, width=16, height=16),
          "instanced": lambda: scenes.instanced_scene(num_instances=50, tris_per_blas=2000, width=16, height=16,
                                                     env_size=(64, 32))}[which]()
    nodes, tris, insts, info = collapse(sd)
    V = sd.vertices_uvx[:, :3].astype(np.float64)
    seen_tris = np.zeros(len(tris), int)
    seen_inst = np.zeros(len(insts), int)
    pairs = []  # (instance, reference triangle) reached through the wide tree
    # the reference's TLAS leaves: instance -> (BLAS root, material)
    bn = sd.bvh_nodes
    leaf_of = {}
    for i in range(sd.top_level_index, bn.shape[0]):
        if bn[i, 8] < 0:
            leaf_of[int(-bn[i, 8]) - 1] = (int(bn[i, 6]), int(bn[i, 7]))
    expected = set()
    for inst, (root, _) in leaf_of.items():
        stack = [root]
        while stack:
            b = stack.pop()
            if bn[b, 8] == 0:
                stack += [int(bn[b, 6]), int(bn[b, 7])]
            else:
                expected |= {(inst, t) for t in range(int(bn[b, 6]), int(bn[b, 6]) + int(bn[b, 7]))}

    def walk(idx, tlas, xf=None, inst=None):
        """Checks the subtree of wide node idx; returns the exact bounds of
        its triangles (world space for the TLAS)."""
        d = decode(nodes[idx])
        slots = 0
        sub_lo, sub_hi = np.full(3, np.inf), np.full(3, -np.inf)
        for s in range(8):
            m = int(d["meta"][s])
            if m == 0:
                continue
            slots += 1
            lo, hi = d["lo"][s], d["hi"][s]
            if d["imask"] >> s & 1:
                assert m == (1 << 5) | (24 + s)
                rel = bin(d["imask"] & ((1 << s) - 1)).count("1")
                c_lo, c_hi = walk(d["child_base"] + rel, tlas, None, inst)
            else:
                cnt = {1: 1, 3: 2, 7: 3}[m >> 5]
                off = m & 31
                c_lo, c_hi = np.full(3, np.inf), np.full(3, -np.inf)
                for k in range(cnt):
                    pi = d["prim_base"] + off + k
                    if tlas:
                        seen_inst[pi] += 1
                        ir = insts[pi]
                        if ir[1] == MERGED_INSTANCE:  # untransformed instances merged into one BLAS
                            assert ir[2] == -1 and ir[3] == 1
                            M = np.eye(4)
                        else:
                            M = sd.transforms[ir[1]].reshape(4, 4).astype(np.float64)
                            assert ir[2] == leaf_of[ir[1]][1]
                        b_lo, b_hi = walk(ir[0], False, M, int(ir[1]))
                    else:
                        seen_tris[pi] += 1
                        t = tris[pi]
                        prim = int(t[3:4].view(np.int32)[0])
                        if inst == MERGED_INSTANCE:
                            ti, tm = int(t[7:8].view(np.int32)[0]), int(t[11:12].view(np.int32)[0])
                            assert np.array_equal(sd.transforms[ti], np.eye(4, dtype=np.float32).ravel())
                            assert tm == leaf_of[ti][1]
                            pairs.append((ti, prim))
                        else:
                            pairs.append((inst, prim))
                        vi = sd.vert_indices[prim]
                        P = V[vi]
                        # (v0, e0, e1) are the reference's v0, v1-v0, v2-v0
                        assert np.array_equal(t[0:3], sd.vertices_uvx[vi[0], :3])
                        assert np.array_equal(t[4:7], (sd.vertices_uvx[vi[1], :3] - sd.vertices_uvx[vi[0], :3]))
                        b_lo, b_hi = P.min(0), P.max(0)
                    c_lo, c_hi = np.minimum(c_lo, b_lo), np.maximum(c_hi, b_hi)
            # the quantised slot box contains everything below it (conservative);
            # 1e-6 absorbs the float rounding of the input's own boxes (the
            # reference's TLAS boxes come from float transforms, Scene.cpp:148-187)
            tol = 1e-6 * (1.0 + np.abs(np.r_[c_lo, c_hi]).max())
            assert np.all(lo <= c_lo + tol) and np.all(hi >= c_hi - tol), (which, lo, c_lo, hi, c_hi)
            sub_lo, sub_hi = np.minimum(sub_lo, c_lo), np.maximum(sub_hi, c_hi)
        assert slots >= 1
        if xf is not None and not tlas:  # BLAS root reached from an instance: world bounds of its box corners
            corners = np.array([[x, y, z, 1.0] for x in (sub_lo[0], sub_hi[0]) for y in (sub_lo[1], sub_hi[1])
                                for z in (sub_lo[2], sub_hi[2])]) @ xf
            return corners[:, :3].min(0), corners[:, :3].max(0)
        return sub_lo, sub_hi

    def walk_blas_root(idx, M):
        return walk(idx, False, M)

    walk(info["tlas_root"], True)
    assert np.all(seen_inst == 1)
    assert np.all(seen_tris >= 1)
    # every (instance, triangle) pair of the reference's two-level tree is
    # reached exactly once
    assert len(pairs) == len(set(pairs))
    assert set(pairs) == expected
    assert info["blas_depth"] + info["tlas_depth"] <= 48
    if which == "icosphere":  # all instances untransformed: one merged BLAS
        assert len(insts) == 1 and insts[0, 1] == MERGED_INSTANCE


def test_wide_bvh_collapse_fills_nodes():
    """The SAH dynamic-programming collapse fills the wide nodes: on a
    displaced icosphere (merged BLAS of 16 untransformed meshes) the nodes
    average more than five children, where a greedy largest-area expansion
    leaves most nodes near the leaves with two."""
    from pathtracer import scenes
    sd = scenes.icosphere_scene(freq=40, width=32, height=32)
    nodes, tris, insts, info = collapse(sd)
    meta = nodes[:, 6:8].copy().view(np.uint8).reshape(-1, 8)
    children = (meta != 0).sum(1)
    blas = children[: info["tlas_first"]]
    assert blas.mean() > 5.0, blas.mean()
    assert (blas == 2).mean() < 0.2
    assert tris.shape[0] == 20 * 40 * 40


@pytest.mark.parametrize("w,h", [(1, 1), (7, 3), (8, 4), (9, 5), (16, 9), (33, 17), (256, 256), (1920, 1080),
                                 (1921, 1079)])
def test_path_order_is_a_bijection_of_warp_blocks(w, h):
    """The wavefront's order of a pass's paths over the pixels (wf_generate,
    the resolve kernels): every slot maps to a distinct pixel of the w x h
    rectangle, the inverse returns the slot, and a full warp of 32 slots in
    a full block is an 8 x 4 block of pixels."""
    from pathtracer import capi
    lib = capi.load_library()
    lib.ptgb_pixel_slot.restype = C.c_int
    x, y = C.c_int(), C.c_int()
    seen = np.zeros((h, w), bool)
    n = w * h
    step = max(1, n // 20000)
    for s in sorted(set(range(0, n, step)) | {n - 1}):
        lib.ptgb_slot_pixel(s, w, h, C.byref(x), C.byref(y))
        assert 0 <= x.value < w and 0 <= y.value < h, (s, x.value, y.value)
        assert not seen[y.value, x.value] or step > 1
        seen[y.value, x.value] = True
        assert lib.ptgb_pixel_slot(x.value, y.value, w, h) == s
    if step == 1:
        assert seen.all()
    if w >= 8 and h >= 4:
        px = []
        for s in range(32):
            lib.ptgb_slot_pixel(s, w, h, C.byref(x), C.byref(y))
            px.append((x.value, y.value))
        assert sorted(px) == sorted((i, j) for i in range(8) for j in range(4))
