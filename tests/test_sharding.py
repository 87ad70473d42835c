"""Multi-rank frame splitting on CPU (gloo, world size 2).

Ranks render row bands with the oracle (the CPU checker; the GPU path splits
the same way through mypbr_render_opts.first_row / row_count) and gather them;
the result must equal a single full render bit for bit, because every pixel's
random numbers depend only on (seed, pixel, pass).
"""
import os
import socket

import numpy as np
import pytest

from conftest import ROOT, scene_path
from mypbr_gb300 import sharding


def test_row_band_split_covers_the_image():
    for h in (1, 7, 64, 1080):
        for world in (1, 2, 3, 8):
            spans = [sharding.row_band(r, world, h) for r in range(world)]
            assert spans[0][0] == 0
            assert sum(c for _, c in spans) == h
            for (f0, c0), (f1, _) in zip(spans, spans[1:]):
                assert f0 + c0 == f1
            assert max(c for _, c in spans) - min(c for _, c in spans) <= 1


def test_sample_shard_merge_is_weighted_mean():
    a = np.full((2, 2, 3), 1.0)
    b = np.full((2, 2, 3), 4.0)
    np.testing.assert_allclose(sharding.merge_sample_shards([a, b], [30, 10]), 1.75)
    assert sharding.sample_seed(7, 0) != sharding.sample_seed(7, 1)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist

    import mypbr_gb300 as mp
    import oracle as orc
    dist.init_process_group("gloo", rank=rank, world_size=world)
    scene = mp.load_scene(scene_path("cornell_c1.scene"))
    cam = scene.camera
    cam.image_width = 24
    cam.samples_per_pixel = 4
    cam.seed = 99
    first, count = sharding.row_band(rank, world, cam.height())
    rad, _, _ = orc.OracleScene(scene).render(cam, threads=2, rows=(first, count))
    full = sharding.gather_row_bands(rad[first:first + count], rank, world, cam.height())
    if rank == 0:
        np.save(os.path.join(out_dir, "gathered.npy"), full)
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_row_bands_equal_full_render(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp

    import mypbr_gb300 as mp
    import oracle as orc
    world = 2
    tmp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    gathered = np.load(tmp_path / "gathered.npy")
    scene = mp.load_scene(scene_path("cornell_c1.scene"))
    cam = scene.camera
    cam.image_width = 24
    cam.samples_per_pixel = 4
    cam.seed = 99
    full, _, _ = orc.OracleScene(scene).render(cam, threads=2)
    np.testing.assert_array_equal(gathered, full)
    del torch
