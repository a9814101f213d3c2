"""Pass sharding over ranks (pathtracer/shard.py) on CPU: two gloo ranks,
each rendering its share of a frame's sample passes with the oracle standing
in for the GPU renderer, summed by all-reduce, equal the one-process render
of all passes within float summation order (1e-5 relative + 1e-6 absolute;
the two partial sums are added in a different order than the per-pass
accumulation)."""
import os
import socket
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_pass_range_partitions():
    sys.path.insert(0, os.path.join(ROOT, "glsl-pathtracer_gb300"))
    from pathtracer.shard import pass_range
    for world in (1, 2, 3, 8):
        for num in (0, 1, 5, 16, 17):
            got = [pass_range(r, world, 7, num) for r in range(world)]
            passes = [p for s, n in got for p in range(s, s + n)]
            assert passes == list(range(7, 7 + num))
            assert max(n for _, n in got) - min(n for _, n in got) <= 1
    with pytest.raises(ValueError):
        pass_range(2, 2, 0, 4)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_path):
    sys.path.insert(0, os.path.join(ROOT, "glsl-pathtracer_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, HERE)
    import torch.distributed as dist
    import orc
    from pathtracer import scenes
    from pathtracer.shard import render_sharded
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    sd = scenes.cornell(24, 16, max_depth=3)
    o, cam = sd.render_options(), sd.pt_camera()
    acc = render_sharded(lambda first, n: orc.render(sd, o, cam, first, n, nthreads=1)[0], 0, 5)
    if rank == 0:
        np.save(out_path, acc)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_sum_to_the_whole_frame(tmp_path):
    import torch.multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "glsl-pathtracer_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import orc
    from pathtracer import scenes
    out = str(tmp_path / "acc.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    sd = scenes.cornell(24, 16, max_depth=3)
    whole = orc.render(sd, sd.render_options(), sd.pt_camera(), 0, 5, nthreads=1)[0]
    got = np.load(out)
    assert whole[..., 3].max() == 5.0
    assert np.allclose(got, whole, rtol=1e-5, atol=1e-6)
