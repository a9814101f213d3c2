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
