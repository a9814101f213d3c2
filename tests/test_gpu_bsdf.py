"""Disney BSDF on the GPU (pt_bsdf_eval / pt_bsdf_sample, through the C ABI)
against the FP64 oracle, with the error reported per lobe.  Needs a GPU.

Inputs are the shading-state records of tests/golden/make_golden.py's
bsdf_inputs: random Disney parameters after GetMaterial's remapping, with a
sixth of them single-lobe materials, random N, V on the normal's side and L
anywhere.  A record is assigned to the lobe with the largest FP64 pdf share
(diffuse, dielectric reflection, metal, glass, clearcoat).

Tolerances (FP32 device arithmetic against FP64, on values > 1e-3 where
relative error is meaningful).  The reference's formulas lose precision in
FP32 on some records whatever the hardware: the Fresnel term normalised by
F0, cancellations at grazing angles.  The reference's own arithmetic in
FP32 (the FP32 oracle, bit-exact to the reference's DisneyEval,
test_oracle_golden.py) measures that loss per record: its rounding noise
is the largest relative error against FP64 over the record and six copies
of it with V, N and L moved by one ulp at random (other rounding patterns
of the same, equally conditioned, evaluation).  So, per lobe:
  * on every record whose FP32 rounding noise is at most REF_NOISE = 2e-6
    (about 17 ulp), the device's f and pdf are within 1e-5 relative of
    FP64;
  * the excluded fraction is printed per lobe (measured with the oracle:
    diffuse 0.3%, dielectric 3.3%, metal 1.3%, glass 9.9%, clearcoat
    19.9%) and bounded;
  * over all records the median is below 1e-6 and the 99th percentile
    below 1e-4.
Against the reference's own FP32 outputs (ref_bsdf.npz): median < 1e-6,
99.9th percentile < 1e-3 (CUDA's and glibc's pow/exp/log differ in the last
bits).
"""
import ctypes as C
import importlib.util
import os

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

LOBES = ["diffuse", "dielectric", "metal", "glass", "clearcoat"]
REL_BAR = 1e-5     # device against FP64
REF_NOISE = 2e-6   # records on which the reference's FP32 arithmetic is this exact are held to REL_BAR
HERE = os.path.dirname(os.path.abspath(__file__))


def bsdf_inputs(n, seed):
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.bsdf_inputs(n, seed)


def fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def gpu_eval(r, sp, V, N, L):
    n = sp.shape[0]
    f = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    arrs = [np.ascontiguousarray(x, np.float32) for x in (sp, V, N, L)]
    r._ck(r.lib.pt_bsdf_eval(r.ctx, *[fptr(a) for a in arrs], n, fptr(f), fptr(pdf)))
    return f, pdf


def rel_err(got, ref):
    return np.abs(got.astype(np.float64) - ref) / np.abs(ref)


@pytest.fixture(scope="module")
def renderer(ptlib):
    from pathtracer import scenes
    from pathtracer.renderer import GpuRenderer
    with GpuRenderer(scenes.cornell(8, 8)) as r:
        yield r


def test_bsdf_eval_vs_reference_fp32(renderer, orc):
    g = golden("ref_bsdf.npz")
    f, pdf = gpu_eval(renderer, g["state"], g["V"], g["N"], g["L"])
    for got, ref in ((f.ravel(), g["f"].ravel()), (pdf, g["pdf"])):
        ok = np.isfinite(ref) & (np.abs(ref) > 1e-3)
        e = rel_err(got[ok], ref[ok].astype(np.float64))
        assert np.median(e) < 1e-6, np.median(e)
        assert np.quantile(e, 0.999) < 1e-3, np.quantile(e, 0.999)
        # zero / non-finite cases agree too
        assert np.array_equal(got[~np.isfinite(ref)], ref[~np.isfinite(ref)], equal_nan=True)


def _rec_err(f, pdf, f64, p64):
    """Per record: the larger relative error of f (channels > 1e-3) and pdf."""
    ef = np.where(np.abs(f64) > 1e-3, np.abs(f.astype(np.float64) - f64) / np.maximum(np.abs(f64), 1e-300), 0.0)
    ep = np.abs(pdf.astype(np.float64) - p64) / p64
    return np.maximum(ef.max(1), ep), ef.max(1), ep


def fp32_rounding_noise(orc, sp, V, N, L, f64, p64, copies=6, seed=0):
    """Per record: the largest relative error of the reference's FP32
    arithmetic against FP64, over the record and `copies` copies with V, N
    and L moved by one ulp at random."""
    f32, p32, _, _ = orc.bsdf_eval(sp, V, N, L, use_double=False)
    noise, _, _ = _rec_err(f32, p32, f64, np.maximum(p64, 1e-300))
    rng = np.random.RandomState(seed)

    def nudge(x):
        return (x * (1 + rng.choice([-1, 1], x.shape) * np.float32(2.0 ** -23))).astype(np.float32)
    for _ in range(copies):
        Vp, Np, Lp = nudge(V), nudge(N), nudge(L)
        a, b, _, _ = orc.bsdf_eval(sp, Vp, Np, Lp, use_double=False)
        c, d, _, _ = orc.bsdf_eval(sp, Vp, Np, Lp, use_double=True)
        noise = np.maximum(noise, _rec_err(a, b, c, np.maximum(d, 1e-300))[0])
    return noise


def test_bsdf_eval_per_lobe_vs_fp64(renderer, orc):
    sp, V, N, L = bsdf_inputs(1_000_000, 11)
    f, pdf = gpu_eval(renderer, sp, V, N, L)
    f64, p64, _, lp64 = orc.bsdf_eval(sp, V, N, L, use_double=True)
    noise = fp32_rounding_noise(orc, sp, V, N, L, f64, p64)
    share = lp64 / np.maximum(lp64.sum(1, keepdims=True), 1e-300)
    dom = np.argmax(share, 1)
    report = []
    for k, name in enumerate(LOBES):
        sel = (dom == k) & (p64 > 1e-3)
        if sel.sum() < 100:
            continue
        e, ef, ep = _rec_err(f[sel], pdf[sel], f64[sel], p64[sel])
        keep = noise[sel] <= REF_NOISE
        report.append((name, int(sel.sum()), 1.0 - keep.mean(), np.median(ef), np.median(ep), e[keep].max(),
                       np.quantile(e, 0.99), e.max()))
    print("\nlobe         n    excluded   f median  pdf median  max kept      p99   max all")
    for row in report:
        print("%-10s %7d   %8.4f  %9.2e  %9.2e  %9.2e %9.2e %9.2e" % row)
    assert len(report) == 5
    for name, n, excl, fmed, pmed, kept_max, p99, _ in report:
        assert kept_max < REL_BAR, (name, kept_max)
        assert fmed < 1e-6 and pmed < 1e-6, (name, fmed, pmed)
        assert p99 < 1e-4, (name, p99)
        assert excl < 0.25, (name, excl)


def test_bsdf_sample_vs_oracle(renderer, orc):
    sp, V, N, _ = bsdf_inputs(200_000, 12)
    n = sp.shape[0]
    seeds = np.random.RandomState(13).randint(0, 2**32, (n, 4), dtype=np.uint64).astype(np.uint32)
    Lg = np.zeros((n, 3), np.float32)
    fg = np.zeros((n, 3), np.float32)
    pg = np.zeros(n, np.float32)
    arrs = [np.ascontiguousarray(x, np.float32) for x in (sp, V, N)]
    renderer._ck(renderer.lib.pt_bsdf_sample(renderer.ctx, *[fptr(a) for a in arrs],
                                             seeds.ctypes.data_as(C.POINTER(C.c_uint32)), n, fptr(Lg), fptr(fg),
                                             fptr(pg)))
    Lo, fo, po = orc.bsdf_sample(sp, V, N, seeds, use_double=False)
    # same seeds => same lobe choice and direction, up to last-bit math
    # differences that can flip a choice on a handful of records
    same_dir = np.all(np.abs(Lg - Lo) < 1e-4, axis=1)
    assert same_dir.mean() > 0.999, same_dir.mean()
    # pdf = inf (a delta-like lobe at its peak) must agree as such, except
    # where it is an FP32 artefact of the reference's GTR1: its denominator
    # 1 + (a^2 - 1) (N.H)^2 reaches 0 when the rounded N.H is 1 at the
    # clearcoat peak, while the device's cancellation-free form, like FP64
    # at the same direction, stays finite
    fin = np.isfinite(po)
    fin_g = np.isfinite(pg)
    differ = same_dir & (fin_g != fin)
    if differ.any():
        _, p64, _, _ = orc.bsdf_eval(sp[differ], V[differ], N[differ], Lg[differ], use_double=True)
        assert np.all(fin_g[differ] & ~fin[differ] & np.isfinite(p64)), (pg[differ], po[differ], p64)
        assert differ.mean() < 1e-4, differ.mean()
    ok = same_dir & fin & fin_g & (po > 1e-3)
    e = rel_err(pg[ok], po[ok])
    assert np.median(e) < 1e-5 and np.quantile(e, 0.99) < 1e-3, (np.median(e), np.quantile(e, 0.99))
