"""The adjoint pass (pt_render_adjoint: path-replay backpropagation on the
GPU) against the oracle's FP64 detached estimator.  Needs a GPU.

The scene is the differentiable-materials workload at a small size (32
materials, 4 sphere lights, every lobe active).  The checked quantity is the
gradient of J(theta) = sum_pixels dI . I(theta) for a fixed random dI, with
I = accumulation / passes.  The oracle renders the same paths (same seeds)
with the sampling held at theta0 and the BSDF and emission values at theta
(orc.render_detached, FP64), whose derivative is exactly what the adjoint
pass estimates; its central finite differences give
  * the FD check, h = 1e-3 (tolerance 1e-3 relative), and
  * the FP64 reference gradient: Richardson extrapolation of the central
    differences with h = 2e-3 and 1e-3 (error O(h^4)).
Steps are relative (h max(1, |theta|)) and divided by the step the float32
scene records actually take.
The 64 checked parameters are drawn uniformly at random from all of them
(11 per material, 3 per light).  With a random dI of both signs, a
parameter's gradient is the small remainder of a sum over every sample of
terms of both signs, so its error floor is set by the size of that sum,
not by the remainder: G_abs = the adjoint's gradient for |dI| (the same
sum with every term counted positive; for the emissions exactly the sum of
magnitudes).  Tolerance per parameter:
  |g_gpu - g_ref| <= 1e-3 |g_ref| + 4 |FD(h) - FD(2h)| + 10 spread_gpu
                     + ABS_FLOOR |G_abs|
where FD(h) - FD(2h) is that parameter's own finite-difference error
estimate, spread_gpu the spread of the GPU gradient over repeated runs
(its FP32 accumulation, summed by atomics in a varying order), and
ABS_FLOOR |G_abs| the FP32 path's agreement with the FP64 oracle sample by
sample (shading arithmetic at GLSL precision, and the rare path whose FP32
and FP64 forms take different discrete decisions) summed over the image;
and the whole vector within 1e-3 relative in the 2-norm.  One more check
runs at the benchmark size (1M-triangle icosphere, 512 x 512, 16 spp,
depth 6) on four random parameters.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PASSES = 4
ABS_FLOOR = 1e-4  # relative to the gradient of the sum of magnitudes (see above)


@pytest.fixture(scope="module")
def setup(ptlib, orc):
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuRenderer
    sd = scenes.diff_scene(freq=40, width=64, height=64, max_depth=6)
    r = GpuRenderer(sd)
    r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
    yield sd, r
    r.close()


def detached_J(orc, sd, theta, dI):
    import dataclasses
    from pathtracer import diff
    mats, lts = diff.set_params(sd.materials, sd.lights, theta)
    e = dataclasses.replace(sd, materials=mats, lights=lts)
    img = orc.render_detached(sd, e, sd.render_options(), sd.pt_camera(), 0, PASSES, use_double=True)
    return float(np.sum(dI.astype(np.float64) * img))


def central_difference(f, theta0, i, h):
    """(f(theta + s e_i) - f(theta - s e_i)) / (the float32 step actually
    taken), s = h max(1, |theta_i|): scene records hold float32 values."""
    s = h * max(1.0, abs(theta0[i]))
    tp, tm = theta0.copy(), theta0.copy()
    tp[i] += s
    tm[i] -= s
    step = float(np.float32(tp[i])) - float(np.float32(tm[i]))
    return (f(tp) - f(tm)) / step


def choose_params(g, count, seed):
    """`count` parameters drawn uniformly at random from all of them."""
    return np.sort(np.random.RandomState(seed).choice(len(g), count, replace=False))


def check_gradient(got, spread, g_abs, ref_fd, ref_2h, idx, rel=1e-3):
    """The per-parameter and 2-norm bars against the FD gradient and the
    Richardson-extrapolated FP64 reference."""
    ref64 = (4.0 * ref_fd - ref_2h) / 3.0
    fd_noise = np.abs(ref_fd - ref_2h)
    for ref, name in ((ref_fd, "FD h=1e-3"), (ref64, "FP64 reference")):
        err = np.abs(got - ref)
        tol = rel * np.abs(ref) + 4.0 * fd_noise + 10.0 * spread + ABS_FLOOR * np.abs(g_abs)
        print(f"{name}: largest error / |G_abs| {np.max(err / np.maximum(np.abs(g_abs), 1e-300)):.2e}, "
              f"largest error / tolerance {np.max(err / np.maximum(tol, 1e-300)):.3f}")
        worst = np.argsort(-(err / np.maximum(tol, 1e-300)))[:5]
        assert np.all(err <= tol), (name, [(int(idx[k]), got[k], ref[k], tol[k]) for k in worst])
        assert np.linalg.norm(got - ref) <= rel * np.linalg.norm(ref), name


def gpu_gradient(r, first, passes, dI, runs=3):
    """The adjoint's gradient, its spread over `runs` runs, and the gradient
    for |dI| (every term of the sum counted positive)."""
    gs = np.stack([r.render_adjoint(first, passes, dI).astype(np.float64) for _ in range(runs)])
    g_abs = r.render_adjoint(first, passes, np.abs(dI)).astype(np.float64)
    return gs.mean(0), gs.max(0) - gs.min(0), g_abs


def test_adjoint_matches_fp64_finite_differences(setup, orc):
    from pathtracer import diff
    sd, r = setup
    H, W = r.height, r.width
    dI = np.random.RandomState(7).normal(size=(H, W, 3)).astype(np.float32)
    r.clear()
    r.render_passes(0, PASSES)
    g, spread, g_abs = gpu_gradient(r, 0, PASSES, dI)
    assert np.isfinite(g).all() and np.abs(g).max() > 0
    theta0 = diff.get_params(sd.materials, sd.lights)
    idx = choose_params(g, 64, 3)
    J = lambda th: detached_J(orc, sd, th, dI)
    ref_fd = np.array([central_difference(J, theta0, i, 1e-3) for i in idx])
    ref_2h = np.array([central_difference(J, theta0, i, 2e-3) for i in idx])
    print(f"\n64 random parameters: {int((np.abs(g[idx]) > 0).sum())} with a nonzero gradient, "
          f"|g| from {np.abs(g[idx]).min():.3g} to {np.abs(g[idx]).max():.3g}")
    check_gradient(g[idx], spread[idx], g_abs[idx], ref_fd, ref_2h, idx)


def test_adjoint_at_the_benchmark_size(ptlib, orc):
    """The differentiable-materials workload itself (1,048,820 triangles, 32
    materials, 4 lights, 512 x 512, 16 spp, depth 6): four random
    parameters -- two material, two light -- against FP64 central
    differences of the oracle's detached estimator."""
    from pathtracer import capi, diff, scenes
    from pathtracer.renderer import GpuRenderer
    sd = scenes.diff_scene(freq=229, width=512, height=512, max_depth=6)
    passes = 16
    dI = np.random.RandomState(9).normal(size=(512, 512, 3)).astype(np.float32)
    with GpuRenderer(sd) as r:
        r.set_integrator(capi.PT_INTEGRATOR_WAVEFRONT)
        r.render_passes(0, passes)
        g, spread, g_abs = gpu_gradient(r, 0, passes, dI, runs=2)
    nm = sd.materials.shape[0] * len(diff.MATERIAL_OFFSETS)
    rng = np.random.RandomState(11)
    idx = np.concatenate([rng.choice(nm, 2, replace=False), nm + rng.choice(len(g) - nm, 2, replace=False)])
    theta0 = diff.get_params(sd.materials, sd.lights)
    import dataclasses

    def J(th):
        mats, lts = diff.set_params(sd.materials, sd.lights, th)
        e = dataclasses.replace(sd, materials=mats, lights=lts)
        img = orc.render_detached(sd, e, sd.render_options(), sd.pt_camera(), 0, passes, use_double=True)
        return float(np.sum(dI.astype(np.float64) * img))
    ref_fd = np.array([central_difference(J, theta0, i, 1e-3) for i in idx])
    ref_2h = np.array([central_difference(J, theta0, i, 2e-3) for i in idx])
    print("\nbenchmark size:", [(int(i), float(a), float(b)) for i, a, b in zip(idx, g[idx], ref_fd)])
    check_gradient(g[idx], spread[idx], g_abs[idx], ref_fd, ref_2h, idx)


def test_adjoint_reuses_the_forward_pass(setup):
    """The gradient is the same whether the forward paths come from the last
    pt_render_passes call or are traced by pt_render_adjoint itself."""
    sd, r = setup
    H, W = r.height, r.width
    dI = np.random.RandomState(8).normal(size=(H, W, 3)).astype(np.float32)
    r.clear()
    r.render_passes(0, PASSES)
    g_cached = r.render_adjoint(0, PASSES, dI)
    r.set_camera(sd.pt_camera())  # invalidates the cached forward batch
    g_fresh = r.render_adjoint(0, PASSES, dI)
    assert np.array_equal(np.isfinite(g_cached), np.isfinite(g_fresh))
    scale = np.abs(g_fresh).max()
    assert np.allclose(g_cached, g_fresh, rtol=1e-4, atol=1e-5 * scale)


def test_torch_autograd_l2_loss(setup, orc):
    """Thin torch.autograd.Function harness: L2 loss to a target rendered at
    perturbed parameters; loss.backward() against FP64 finite differences of
    the detached loss."""
    torch = pytest.importorskip("torch")
    from pathtracer import diff
    sd, r = setup
    theta0 = diff.get_params(sd.materials, sd.lights)
    nmat = sd.materials.shape[0]
    target_theta = diff.perturb(theta0, nmat, 0.1, 4)
    mats, lts = diff.set_params(sd.materials, sd.lights, target_theta)
    r.update_materials(mats)
    r.update_lights(lts)
    r.clear()
    r.render_passes(1000, 16)
    target = r.accum()[..., :3] / 16.0

    class Render(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta):
            m, l = diff.set_params(sd.materials, sd.lights, theta.detach().cpu().numpy())
            r.update_materials(m)
            r.update_lights(l)
            r.clear()
            r.render_passes(0, PASSES)
            return torch.from_numpy(r.accum()[..., :3] / PASSES).double()

        @staticmethod
        def backward(ctx, grad_img):
            g = r.render_adjoint(0, PASSES, grad_img.detach().cpu().numpy().astype(np.float32))
            return torch.from_numpy(g.astype(np.float64))

    theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    img = Render.apply(theta)
    loss = ((img - torch.from_numpy(target).double()) ** 2).mean()
    loss.backward()
    g = theta.grad.numpy()
    # the same loss on the oracle's detached FP64 image, by central differences
    import dataclasses

    def L(th):
        m, l = diff.set_params(sd.materials, sd.lights, th)
        e = dataclasses.replace(sd, materials=m, lights=l)
        im = orc.render_detached(sd, e, sd.render_options(), sd.pt_camera(), 0, PASSES, use_double=True)
        return float(np.mean((im - target) ** 2))

    # the sum of magnitudes behind each gradient: the adjoint of |dLoss/dI|
    dLdI = (2.0 / img.numel()) * (img.detach().numpy() - target)
    g_abs = r.render_adjoint(0, PASSES, np.abs(dLdI).astype(np.float32)).astype(np.float64)
    idx = choose_params(g, 16, 5)
    ref = np.array([central_difference(L, theta0, i, 1e-3) for i in idx])
    ref_2h = np.array([central_difference(L, theta0, i, 2e-3) for i in idx])
    err = np.abs(g[idx] - ref)
    tol = 2e-3 * np.abs(ref) + 4.0 * np.abs(ref - ref_2h) + ABS_FLOOR * np.abs(g_abs[idx])
    assert np.all(err <= tol), list(zip(idx, g[idx], ref, tol))
    r.update_materials(sd.materials)
    r.update_lights(sd.lights)


def test_adjoint_rejects_unsupported_scenes(ptlib):
    from pathtracer import capi, scenes
    from pathtracer.renderer import GpuRenderer
    sd = scenes.instanced_scene(num_instances=20, tris_per_blas=500, width=16, height=16, env_size=(32, 16))
    with GpuRenderer(sd) as r:
        with pytest.raises(capi.PTError) as e:
            r.render_adjoint(0, 1, np.zeros((16, 16, 3), np.float32))
        assert e.value.code == capi.PT_ERR_UNSUPPORTED
