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
Tolerance: per parameter |g_gpu - g_ref| <= 1e-3 |g_ref| + 1e-3 max|g_ref|
(FP32 accumulation of the GPU, and the rare path whose FP32 and FP64 forms
take different discrete decisions), and the whole vector within 1e-3
relative in the 2-norm.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PASSES = 4


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


def choose_params(sd, g, count, seed):
    """Parameters with gradients well above the noise floor: all 12 light
    emissions and the largest-gradient material parameters, drawn at random."""
    from pathtracer import diff
    nm = sd.materials.shape[0] * len(diff.MATERIAL_OFFSETS)
    rng = np.random.RandomState(seed)
    mat_idx = np.argsort(-np.abs(g[:nm]))[: 3 * count]
    pick = rng.choice(mat_idx, count - (len(g) - nm), replace=False)
    return np.concatenate([np.sort(pick), np.arange(nm, len(g))])


def test_adjoint_matches_fp64_finite_differences(setup, orc):
    from pathtracer import diff
    sd, r = setup
    H, W = r.height, r.width
    dI = np.random.RandomState(7).normal(size=(H, W, 3)).astype(np.float32)
    r.clear()
    r.render_passes(0, PASSES)
    g = r.render_adjoint(0, PASSES, dI).astype(np.float64)
    assert np.isfinite(g).all() and np.abs(g).max() > 0
    theta0 = diff.get_params(sd.materials, sd.lights)
    idx = choose_params(sd, g, 64, 3)
    J = lambda th: detached_J(orc, sd, th, dI)
    ref_fd = np.array([central_difference(J, theta0, i, 1e-3) for i in idx])
    # FP64 reference: Richardson extrapolation of steps 2e-3 and 1e-3 (O(h^4))
    ref_2h = np.array([central_difference(J, theta0, i, 2e-3) for i in idx])
    ref64 = (4.0 * ref_fd - ref_2h) / 3.0
    got = g[idx]
    for ref, name in ((ref_fd, "FD h=1e-3"), (ref64, "FP64 reference")):
        err = np.abs(got - ref)
        tol = 1e-3 * np.abs(ref) + 1e-3 * np.abs(ref).max()
        worst = np.argsort(-(err / tol))[:5]
        assert np.all(err <= tol), (name, [(int(idx[k]), got[k], ref[k]) for k in worst])
        assert np.linalg.norm(got - ref) <= 1e-3 * np.linalg.norm(ref), name


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

    idx = choose_params(sd, g, 16, 5)
    ref = np.array([central_difference(L, theta0, i, 1e-3) for i in idx])
    err = np.abs(g[idx] - ref)
    assert np.all(err <= 2e-3 * np.abs(ref) + 2e-3 * np.abs(ref).max()), list(zip(idx, g[idx], ref))
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
