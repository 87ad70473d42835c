"""Error-bounded ray origins (GPU): a ray that leaves a surface starts at the
hit point moved along the geometric normal by the point's FP32 error bound,
and its walk ignores only hits within 8 float steps of the origin's scale.
No absolute epsilon is involved, so the scale of the scene does not matter.

Checked on the scenes whose scale an absolute epsilon would not suit: the
512-unit voxel terrain of the hall (a 512^3 world), the 30-unit triangle room
(60,000 triangles), the sphere field's ground sphere of radius 1000, and the
555-unit Cornell box. From every hit of seeded random rays, a reflected ray
and a ray going on through the surface are started as the renderer starts
them; none may meet the surface it left. Light leaks would show as renders
off the reference's: those are test_config_parity's 3-sigma checks of the
same scenes (c2, c3, c5) and test_gpu_parity's.
"""
import os
import sys
import tempfile

import numpy as np
import pytest

import mypbr_gb300 as mp
from conftest import GOLDEN, scene_path

sys.path.insert(0, GOLDEN)
import config_scenes  # noqa: E402

pytestmark = pytest.mark.gpu

# where the failing spawns are written for a look, when set
DUMP = os.environ.get("MYPBR_TEST_DUMP")


def random_rays(lo, hi, n, seed, down=None):
    """Origins uniform in the box [lo, hi], directions uniform on the sphere
    (or, with down, aimed at points of the plane y = down inside the box)."""
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    o = lo + (hi - lo) * rng.random((n, 3))
    d = rng.normal(size=(n, 3))
    if down is not None:
        target = lo + (hi - lo) * rng.random((n, 3))
        target[:, 1] = down
        d = target - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 3:6] = d
    rays[:, 6] = 0.0
    rays[:, 7] = 3e38
    return rays


def check_no_self_hits(G, rays, min_hits, name):
    out, detail = G.spawn_probe(rays)
    hit = out[:, 0] >= 0
    bad = hit & ((out[:, 1] != 0) | (out[:, 2] != 0))
    if bad.any() and DUMP:  # what the failing spawns looked like
        np.savez_compressed(os.path.join(DUMP, f"spawn_{name}.npz"), rays=rays[bad], flags=out[bad],
                            detail=detail[bad])
    assert hit.sum() >= min_hits, hit.sum()
    assert not bad.any(), (int(bad.sum()), out[bad][:5], detail[bad][:5])


def test_voxel_terrain_512():
    d = tempfile.mkdtemp()
    path, _ = config_scenes.c5(d)
    G = mp.GpuScene(mp.load_scene(path))
    # world coordinates: x, z in [-256, 256], the terrain up to y ~150, the hall inside
    rays = np.concatenate([random_rays([-256, 0, -256], [256, 200, 256], 40000, 1),
                           random_rays([-256, 160, -256], [256, 250, 256], 40000, 2, down=40.0),
                           random_rays([-100, 90, -70], [100, 180, 70], 40000, 3)])
    check_no_self_hits(G, rays, 60000, "voxel_terrain")


def test_triangle_room_30():
    d = tempfile.mkdtemp()
    path, _ = config_scenes.c3(d)
    G = mp.GpuScene(mp.load_scene(path))
    rays = np.concatenate([random_rays([-10, 0, -15], [10, 8, 15], 60000, 4),
                           random_rays([-9, 0.2, -14], [9, 7.8, 14], 60000, 5)])
    check_no_self_hits(G, rays, 100000, "triangle_room")


def test_sphere_field_ground_of_radius_1000():
    d = tempfile.mkdtemp()
    path, _ = config_scenes.c2(d)
    G = mp.GpuScene(mp.load_scene(path))
    rays = np.concatenate([random_rays([-12, 0.05, -12], [12, 2, 12], 60000, 6),
                           random_rays([-12, 3, -12], [12, 8, 12], 60000, 7, down=0.0)])
    check_no_self_hits(G, rays, 90000, "sphere_field")


def test_cornell_box_555():
    G = mp.GpuScene(mp.load_scene(scene_path("cornell_c1.scene")))
    rays = random_rays([1, 1, 1], [554, 554, 554], 60000, 8)
    check_no_self_hits(G, rays, 45000, "cornell")  # the box is open at the front
