"""The drop-in class ptgb::CudaRenderer driven the way the reference's
Main.cpp drives GLSLPT::Renderer, from C++.  Needs a GPU.

tests/cpp/dropin_driver.cpp is compiled against include/pt_cuda.h, the
drop-in's header (csrc/cuda_renderer.h) and libptgb.so.  It fills a
GLSLPT::Scene (mock_glslpt.h: the reference's member names and layouts)
from a scene file and constructs the renderer from that Scene*, as
Main.cpp:157-161 does, then runs Update/Render cycles until N sample
passes are complete and reads GetOutputBuffer (Main.cpp:166-180):

  * tile by tile in the reference's order (one Render per tile), with the
    wavefront integrator and with the megakernel;
  * with RenderPasses (all passes of the loop in one launch);

each RGBA8 image equal, byte for byte, to pt_get_output of the same passes
rendered by pt_render_passes on a context of the C ABI.
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_driver(out_dir):
    csrc = os.path.join(ROOT, "glsl-pathtracer_gb300", "csrc")
    exe = os.path.join(out_dir, "dropin_driver")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I/usr/local/cuda/include",
                    os.path.join(ROOT, "tests", "cpp", "dropin_driver.cpp"), "-L" + csrc, "-lptgb",
                    "-Wl,-rpath," + csrc, "-o", exe], check=True)
    return exe


@pytest.fixture(scope="module")
def driver(ptlib, tmp_path_factory):
    return build_driver(str(tmp_path_factory.mktemp("dropin")))


def reference_output(sd, passes, integrator):
    from pathtracer.renderer import GpuRenderer
    with GpuRenderer(sd) as r:
        r.set_integrator(integrator)
        r.render_passes(0, passes)
        r.snapshot()
        return r.output(passes, from_snapshot=True)


@pytest.mark.parametrize("mode,integrator", [("tiles", 1), ("tiles", 0), ("passes", 1)])
def test_drop_in_renderer_matches_render_passes(driver, tmp_path, mode, integrator):
    from pathtracer import scenes
    sd = scenes.cornell(96, 64, tile=32)  # 3 x 2 tiles
    scene_file = str(tmp_path / "scene.bin")
    sd.save_flat(scene_file)
    out = str(tmp_path / "out.rgba")
    passes = 3
    subprocess.run([driver, scene_file, mode, str(passes), out, str(integrator)], check=True)
    got = np.fromfile(out, np.uint8).reshape(64, 96, 4)
    exp = reference_output(sd, passes, integrator)
    assert np.array_equal(got, exp), np.abs(got.astype(int) - exp).max()
    assert got[..., :3].mean() > 10


def test_drop_in_bench_mode_runs(driver, tmp_path):
    import json
    from pathtracer import scenes
    sd = scenes.cornell(64, 64)
    scene_file = str(tmp_path / "scene.bin")
    sd.save_flat(scene_file)
    r = subprocess.run([driver, scene_file, "bench", "4", "3", "1"], check=True, capture_output=True, text=True)
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["steps"] == 3 and line["passes_per_step"] == 4 and line["rays"] > 3 * 4 * 64 * 64
