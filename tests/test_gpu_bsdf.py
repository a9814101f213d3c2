"""Disney BSDF on the GPU (pt_bsdf_eval / pt_bsdf_sample, through the C ABI)
against the FP64 oracle, with the error reported per lobe.  Needs a GPU.

Inputs are the shading-state records of tests/golden/make_golden.py's
bsdf_inputs: random Disney parameters after GetMaterial's remapping, with a
sixth of them single-lobe materials, random N, V on the normal's side and L
anywhere.  A record is assigned to the lobe with the largest FP64 pdf share
(diffuse, dielectric reflection, metal, glass, clearcoat).

Tolerances (FP32 device arithmetic against FP64, on values > 1e-3 where
relative error is meaningful): per lobe, median relative error of f and pdf
< 1e-5 and 99th percentile < 1e-3 -- the same bounds the FP32 oracle meets
(test_oracle_golden.py).  Against the reference's own FP32 outputs
(ref_bsdf.npz): median < 1e-6, 99.9th percentile < 1e-3 (CUDA's and glibc's
pow/exp/log differ in the last bits).
"""
import ctypes as C
import importlib.util
import os

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

LOBES = ["diffuse", "dielectric", "metal", "glass", "clearcoat"]
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


def test_bsdf_eval_per_lobe_vs_fp64(renderer, orc):
    sp, V, N, L = bsdf_inputs(1_000_000, 11)
    f, pdf = gpu_eval(renderer, sp, V, N, L)
    f64, p64, _, lp64 = orc.bsdf_eval(sp, V, N, L, use_double=True)
    share = lp64 / np.maximum(lp64.sum(1, keepdims=True), 1e-300)
    dom = np.argmax(share, 1)
    report = []
    for k, name in enumerate(LOBES):
        sel = (dom == k) & (p64 > 1e-3)
        if sel.sum() < 100:
            continue
        ep = rel_err(pdf[sel], p64[sel])
        fs, fr = f[sel].ravel(), f64[sel].ravel()
        okf = np.abs(fr) > 1e-3
        ef = rel_err(fs[okf], fr[okf])
        report.append((name, int(sel.sum()), np.median(ef), np.quantile(ef, 0.99), ef.max(), np.median(ep),
                       np.quantile(ep, 0.99), ep.max()))
    print("\nlobe        n        f: median      p99      max    pdf: median      p99      max")
    for row in report:
        print("%-10s %7d   %10.2e %9.2e %9.2e   %10.2e %9.2e %9.2e" % row)
    assert len(report) == 5
    for name, n, fmed, f99, _, pmed, p99, _ in report:
        assert fmed < 1e-5 and pmed < 1e-5, (name, fmed, pmed)
        assert f99 < 1e-3 and p99 < 1e-3, (name, f99, p99)


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
    # pdf = inf (a delta-like lobe at its peak) must agree as such
    fin = np.isfinite(po)
    assert np.array_equal(np.isfinite(pg[same_dir]), fin[same_dir])
    ok = same_dir & fin & (po > 1e-3)
    e = rel_err(pg[ok], po[ok])
    assert np.median(e) < 1e-5 and np.quantile(e, 0.99) < 1e-3, (np.median(e), np.quantile(e, 0.99))
