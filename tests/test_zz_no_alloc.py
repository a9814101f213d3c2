"""pt_render_tile_noalloc (path state in a fixed device array, nothing
allocated) against pt_render_tile with the wavefront integrator, through the
C ABI.  Needs a GPU.

Tolerance: both run the same kernels on the same seeds, so each channel of
the accumulation must agree within 1e-6 relative + 1e-7 absolute (in
practice they agree bit for bit).  The first tile below has 160 x 128 =
20480 pixels, more than the 16384 paths of the fixed array, so it is traced
in two bands of rows; the others are the ragged tiles at the right and top
edges.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-6, 1e-7


def _tiles_in_order(width, height, tw, th, passes):
    """The reference's tile order with its frame numbers (Renderer.cpp:745-762)."""
    ntx, nty = -(-width // tw), -(-height // th)
    frame = 2
    out = []
    for _ in range(passes):
        for ty in range(nty - 1, -1, -1):
            for tx in range(ntx):
                out.append((tx, ty, frame))
                frame += 1
    return out


def test_noalloc_tile_matches_render_tile(ptlib):
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuRenderer
    sd = scenes.cornell(200, 136)
    with GpuRenderer(sd, tile_width=160, tile_height=128) as r:
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        tiles = _tiles_in_order(200, 136, 160, 128, 2)
        ref, got = [], []
        for fn, out in ((r.lib.pt_render_tile, ref), (r.lib.pt_render_tile_noalloc, got)):
            r.clear()
            # two calls in a row on the same tile, then every tile twice
            for tx, ty, frame in [(0, 0, 2), (0, 0, 3)] + tiles:
                capi.check(r.lib, fn(r.ctx, tx, ty, frame))
                if len(out) < 2:
                    out.append(r.accum().copy())
            out.append(r.accum().copy())
    for a, b in zip(ref, got):
        assert np.isfinite(b).all()
        assert np.allclose(b, a, rtol=RTOL, atol=ATOL)
    assert not np.array_equal(ref[0], ref[1])  # the second call added samples


def test_noalloc_rejects_tiles_wider_than_its_scratch(ptlib):
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuRenderer
    sd = scenes.cornell(16400, 1)
    with GpuRenderer(sd, tile_width=16400, tile_height=1) as r:
        assert r.lib.pt_render_tile_noalloc(r.ctx, 0, 0, 2) == capi.PT_ERR_INVALID_ARG
        buf = C.create_string_buffer(256)
        r.lib.pt_last_error(buf, 256)
        assert b"16384" in buf.value
        assert r.lib.pt_render_tile_noalloc(r.ctx, 1, 0, 2) == capi.PT_ERR_INVALID_ARG  # tile out of range


def _free_device_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info(0)[0]


@pytest.mark.parametrize("scene", ["cornell", "volume-replay"])
def test_noalloc_leaves_device_memory_unchanged(ptlib, scene):
    """The property the entry point exists for: on a fresh context that only
    ever calls pt_render_tile_noalloc, the device's free memory is the same
    before and after several renders.  A warm-up pass comes first, since the
    first launch of a kernel may load its code onto the device.  The
    volume scene (blended medium boundary, VOL_MIS, environment map and a
    light) takes the suspend-and-replay transmittance stage and the tail
    kernel, whose buffers also live in the fixed array.  The first of three
    passes is the warm-up; the other two are measured."""
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuRenderer
    from test_gpu_volume_stages import volume_scene
    if scene == "cornell":
        sd, tw, th = scenes.cornell(200, 136), 160, 128
    else:
        sd, tw, th = volume_scene(blend=True, env=True, width=96, height=64), 48, 64
    W, H = sd.render_options().render_width, sd.render_options().render_height
    with GpuRenderer(sd, tile_width=tw, tile_height=th) as r:
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        tiles = _tiles_in_order(W, H, tw, th, 3)
        per_pass = len(tiles) // 3
        for tx, ty, frame in tiles[:per_pass]:  # warm-up: the first pass
            capi.check(r.lib, r.lib.pt_render_tile_noalloc(r.ctx, tx, ty, frame))
        before = _free_device_bytes()
        for tx, ty, frame in tiles[per_pass:]:
            capi.check(r.lib, r.lib.pt_render_tile_noalloc(r.ctx, tx, ty, frame))
        after = _free_device_bytes()
        st = r.stats()
        acc = r.accum()
    assert st["status"] == 0, st
    assert np.isfinite(acc).all() and acc[..., :3].sum() > 0
    assert after == before, (before, after)
