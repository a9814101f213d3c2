"""The autotuner and the kernel variants it chooses among (pt_autotune /
pt_set_tuning).  Needs a GPU.

Every configuration traces the same rays to the same hits (closest-hit ties
go to the smallest triangle id whatever the order of the tests), so the
image must not change by a bit; and the autotuner must leave the caller's
accumulation untouched.
"""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["cornell", "icosphere"])
def test_every_configuration_gives_the_same_image(ptlib, name):
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuRenderer
    sd = scenes.cornell(64, 48, tile=32) if name == "cornell" else scenes.icosphere_scene(
        freq=60, width=96, height=64, tile=32)
    with GpuRenderer(sd) as r:
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        ref = None
        for variant, refill, min_tris in itertools.product(range(4), (1, 8, 32), (0, 8)):
            # the first round on its own settings in half of the cases
            first = dict(extend_refill_first=33 - refill, min_tris_first=4, shadow_refill_first=refill,
                         shadow_min_tris_first=0, extend_variant_first=(variant + 1) % 4,
                         shade_variant_first=(variant + 2) % 3) if variant % 2 else dict(
                extend_refill_first=0, min_tris_first=-1, shadow_refill_first=0, shadow_min_tris_first=-1,
                extend_variant_first=-1, shade_variant_first=-1)
            r.set_tuning(extend_variant=variant, shadow_variant=3 - variant, extend_refill=refill,
                         shadow_refill=refill, min_tris=min_tris, shade_variant=variant % 3, **first)
            r.clear()
            r.render_passes(0, 3)
            a = r.accum()
            if ref is None:
                ref = a
            assert np.array_equal(a, ref), (variant, refill, min_tris, first)


def test_autotune_keeps_the_accumulation(ptlib):
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuRenderer
    sd = scenes.icosphere_scene(freq=60, width=96, height=64, tile=32)
    with GpuRenderer(sd) as r:
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        r.render_passes(0, 2)
        before = r.accum().copy()
        t = r.autotune(2)
        assert 0 <= t["extend_variant"] < 4 and 0 <= t["shadow_variant"] < 4
        assert t["frame_ms"] > 0
        assert r.tuning() == {k: t[k] for k in r.TUNING_FIELDS}
        assert np.array_equal(r.accum(), before)
        r.clear()
        r.render_passes(0, 2)
        assert np.array_equal(r.accum(), before)
        with pytest.raises(capi.PTError):
            r.set_tuning(extend_variant=7)
        with pytest.raises(capi.PTError):
            r.set_tuning(extend_refill_first=33)
        with pytest.raises(capi.PTError):
            r.set_tuning(min_tris_first=-2)
        with pytest.raises(capi.PTError):
            r.set_tuning(extend_variant_first=4)
