"""The algorithmic bytes per ray of the roofline, on the reference's own BVH.

The roofline prices a ray query by its traversal work on the reference's
binary BVH: 36 B per node visited (BvhTranslator::Node), 60 B per triangle
tested, 176 B per shaded hit.  bench.py counts that work live with the
oracle, on the scene arrays of this project's builder
(csrc/scene_build.cpp).  tests/golden/ref_tree_counts.json holds the same
oracle counters on the same rays and paths over the tree the reference
itself builds from the same meshes and instances -- its loader, RadeonRays
SBVH and BvhTranslator (make_golden.py trees) -- for both full-size
workloads.  CPU only.

  * the bytes per closest-hit query (and per query) on the two trees agree
    within 0.5%, so the roofline's numerator is the reference tree's;
  * this project's builder still gives the counters recorded in the
    fixture (the comparison stays valid as the builder changes).
"""
import json
import os

import pytest

from conftest import GOLDEN


def per_ray(c):
    rays = c["closest"] + c["shadow"]
    nc, tc = c["nodes"] - c["nodes_any"], c["tris"] - c["tris_any"]
    closest = (36.0 * nc + 60.0 * tc + 176.0 * c["tri_hits"]) / c["closest"]
    every = (36.0 * c["nodes"] + 60.0 * c["tris"] + 176.0 * c["tri_hits"]) / rays
    return closest, every


def fixture():
    with open(os.path.join(GOLDEN, "ref_tree_counts.json")) as fh:
        return json.load(fh)


@pytest.mark.parametrize("workload", ["icosphere_1m", "instanced"])
def test_bytes_per_ray_equal_on_reference_tree(workload):
    f = fixture()[workload]
    ref, ours = f["reference"], f["ours"]
    # the same paths: the two trees give the same hits
    for k in ("closest", "shadow", "paths", "tri_hits"):
        assert ref[k] == ours[k], (k, ref[k], ours[k])
    for a, b in zip(per_ray(ref), per_ray(ours)):
        assert abs(b / a - 1.0) < 5e-3, (workload, a, b)


@pytest.mark.parametrize("workload", ["icosphere_1m", "instanced"])
def test_builder_matches_fixture(orc, workload):
    from pathtracer import scenes
    f = fixture()
    sd = scenes.icosphere_scene() if workload == "icosphere_1m" else scenes.instanced_scene()
    _, _, c = orc.render(sd, sd.render_options(), sd.pt_camera(), 0, f["sample"]["passes"],
                         row_step=f["sample"]["row_step"], cull=True)
    rec = f[workload]["ours"]
    assert sd.bvh_nodes.shape[0] == rec["binary_nodes"]
    for k in ("closest", "shadow", "nodes", "tris", "tri_hits", "nodes_any", "tris_any", "inner"):
        assert c[k] == rec[k], (k, c[k], rec[k])
