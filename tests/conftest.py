import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "glsl-pathtracer_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


@pytest.fixture(scope="session")
def orc():
    import orc as _orc
    _orc.build()
    return _orc


@pytest.fixture(scope="session")
def ptlib():
    """libptgb.so, built in-tree; GPU tests only."""
    from pathtracer import build, capi
    build.build_library()
    return capi.load_library()


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def golden_scene(name):
    from pathtracer.scene import SceneData
    return SceneData.load_npz(os.path.join(GOLDEN, name))
