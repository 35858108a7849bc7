"""The multi-process measurement path on the CPU (gloo, world size 2): the
batch sharding covers every instance exactly once, balanced by points, with
each instance built as in the full batch; the time reduction takes the
maximum over ranks."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from positionbaseddynamicsold_gb300 import scenes
from positionbaseddynamicsold_gb300.dist import max_over_ranks, shard_instances


def test_shards_cover_every_instance_once_balanced():
    sizes = scenes.batched_cloth_points(512, seed=0)
    for world in (1, 2, 3, 4, 8):
        shards = [shard_instances(sizes, world, r) for r in range(world)]
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[i] for i in s) for s in shards]
        assert max(loads) - min(loads) <= max(sizes)
        assert shards == [shard_instances(sizes, world, r) for r in range(world)]
    with pytest.raises(ValueError):
        shard_instances(sizes, 2, 2)


def test_shard_scenes_equal_the_full_batch_instances():
    n, kw = 12, dict(seed=4, side_lo=6, side_hi=14)
    full = scenes.batched_cloths(n, **kw)
    sizes = scenes.batched_cloth_points(n, **kw)
    starts = np.concatenate([[0], np.cumsum(sizes)])
    for r in range(2):
        sub = shard_instances(sizes, 2, r)
        part = scenes.batched_cloths(n, subset=sub, **kw)
        off = 0
        for k in sub:
            m = sizes[k]
            np.testing.assert_array_equal(part["pos"][off:off + m], full["pos"][starts[k]:starts[k + 1]])
            np.testing.assert_array_equal(part["spheres"][sub.index(k)], full["spheres"][k])
            off += m
        assert off == len(part["pos"])


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    got = max_over_ranks(1.5 + rank)
    dist.destroy_process_group()
    with open(os.path.join(out_dir, "r%d" % rank), "w") as f:
        f.write(repr(got))


def test_max_over_ranks_gloo_world2(tmp_path):
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        assert float((tmp_path / ("r%d" % r)).read_text()) == 2.5
    assert max_over_ranks(3.25) == 3.25   # no process group: the value itself
