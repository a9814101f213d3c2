"""Converged-image parity at the benchmark scenes: the CUDA wavefront
against the oracle with independent sample sets.  Needs a GPU.

Scenes: the 1,048,820-triangle icosphere (16 materials, sphere light, depth
8) and the 10,000-instance scene (5 meshes of 50k triangles, IBL, volume
with VOL_MIS, depth 8), both at 160 x 90 with the benchmark's camera and
geometry.  The oracle renders sample passes 0-255, the GPU passes 256-511,
so the two estimates share no random numbers.  Per pixel and channel,
with the sample variances of both sides,

    z = (mu_gpu - mu_oracle) / sqrt(var_gpu / n + var_oracle / n)

and the image RMSE of mu_gpu - mu_oracle is set against its noise floor,
sqrt(mean(var_gpu / n + var_oracle / n)).  Bars: |mean z| < 0.05, the
fraction of |z| > 4 under 1e-3, RMSE within 1.25x the noise floor.  The
oracle against itself (passes 0-255 against 256-511) gives mean z
-0.004 / -0.008, |z| > 4 on 3.2e-4 / 0 of the values and RMSE 0.99x / 1.03x
the floor on the two scenes.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 256


def _scene(name):
    from pathtracer import scenes
    if name == "icosphere_1m":
        return scenes.icosphere_scene(freq=229, width=160, height=90, max_depth=8)
    return scenes.instanced_scene(num_instances=10000, tris_per_blas=50000, width=160, height=90, max_depth=8)


@pytest.mark.parametrize("name", ["icosphere_1m", "instanced_10k"])
def test_converged_image_z_test_and_rmse(ptlib, orc, name):
    from pathtracer import capi
    from pathtracer.renderer import GpuRenderer
    sd = _scene(name)
    o = sd.render_options()
    acc_o, sq_o, _ = orc.render(sd, o, sd.pt_camera(), 0, N, with_sq=True)
    mu_o = acc_o[..., :3].astype(np.float64) / N
    var_o = np.maximum(sq_o / N - mu_o ** 2, 0)
    sq_g = np.zeros_like(mu_o)
    with GpuRenderer(sd) as r:
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        prev = np.zeros((o.render_height, o.render_width, 4), np.float32)
        for k in range(N):
            r.render_passes(N + k, 1)
            a = r.accum()
            s = (a - prev)[..., :3].astype(np.float64)
            sq_g += s * s
            prev = a
        assert r.stats()["status"] == 0
    mu_g = prev[..., :3].astype(np.float64) / N
    var_g = np.maximum(sq_g / N - mu_g ** 2, 0)
    se2 = (var_g + var_o) / N
    ok = se2 > 1e-12
    z = (mu_g - mu_o)[ok] / np.sqrt(se2[ok])
    rmse = np.sqrt(np.mean((mu_g - mu_o) ** 2))
    floor = np.sqrt(np.mean(se2))
    print(f"\n{name}: mean z {z.mean():+.4f}, |z|>4 {(np.abs(z) > 4).mean():.2e}, rmse {rmse:.4g} "
          f"= {rmse / floor:.3f} x noise floor {floor:.4g}")
    assert abs(z.mean()) < 0.05, z.mean()
    assert (np.abs(z) > 4).mean() < 1e-3, (np.abs(z) > 4).mean()
    assert rmse < 1.25 * floor, (rmse, floor)
