"""The benchmark configurations themselves, and the camera and feature-buffer
paths, against the reference's renders (GPU, through the C ABI).

Each golden is camera::render's batch means on a scene that the reference
rendered in the same container that holds it (tests/golden/gen_golden.py,
groups `configs`, `render` and `features`):

  c2   the 1000-sphere field under the full 1024 x 512 sky whose 0.5 deg sun
       lobe peaks at 5e4 (the headline workload), 96 x 54 at 4096 spp
  c3   the triangle room at 60,000 triangles, 32 principled materials and 16
       emissive quads, 64 x 36 at 2048 spp
  c5   the 512^3 voxel hall lit through six slits, 64 x 36 at 16,384 spp,
       plain and guided (the guide is one more MIS proposal, so the guided
       image must meet the same bound)
  defocus_bokeh, ortho, checker   thin lens with a hexagonal aperture
       (camera.h:304-339), orthographic view with a lens (camera.h:291-301),
       3D checker textures (texture.h:36-58)
  features  first_surface's albedo and normal guides (camera.h:253-277)

The criterion is the one of test_gpu_parity: per-pixel means within 3 sigma
of the combined Monte Carlo error (< 2 % of pixel-channels beyond 3 sigma,
< 0.2 % beyond 5), image totals within 4 sigma. Pixels whose value has no
Monte Carlo noise at all (a uniform sky seen directly) get a floor of 1e-4 of
their value, the FP32 rounding of the device's arithmetic.
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


def load_golden(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


def assert_within_3_sigma(rad, var, g, label):
    ref, ref_var = g["mean"].astype(np.float64), g["var_of_mean"].astype(np.float64)
    z = (rad - ref) / np.sqrt(var + ref_var + (1e-4 * np.abs(ref)) ** 2 + 1e-30)
    n = rad.shape[0] * rad.shape[1]
    tot_sigma = np.sqrt(var.sum(axis=(0, 1)) + ref_var.sum(axis=(0, 1))) / n
    tot_z = (rad.mean(axis=(0, 1)) - ref.mean(axis=(0, 1))) / np.maximum(tot_sigma, 1e-12)
    beyond3, beyond5 = np.mean(np.abs(z) > 3), np.mean(np.abs(z) > 5)
    print(f"{label}: beyond 3 sigma {beyond3:.4f}, beyond 5 sigma {beyond5:.4f}, totals z {tot_z}")
    assert beyond3 < 0.02, (label, beyond3)
    assert beyond5 < 0.002, (label, beyond5)
    assert np.all(np.abs(tot_z) < 4), (label, tot_z)


_CONFIG_DIRS = {}


def config_scene(name):
    """The configuration's scene at test size, generated once per session and
    checked to be the input the reference rendered."""
    if name not in _CONFIG_DIRS:
        d = tempfile.mkdtemp(prefix=f"mypbr_{name}_")
        path, digest = config_scenes.CONFIGS[name](d)
        _CONFIG_DIRS[name] = (path, digest)
    path, digest = _CONFIG_DIRS[name]
    g = load_golden(f"render_{name}")
    assert str(g["digest"]) == digest, (
        f"the generated {name} scene differs from the one the reference rendered "
        f"(digest {digest} vs {g['digest']}): a different numpy random stream?")
    return path, g


def render(sc, G, spp, seed, guided=0, per_wave=0):
    cam = sc.camera
    cam.samples_per_pixel = spp
    cam.seed = seed
    cam.guided = guided
    cam.samples_per_wave = per_wave
    rad, var, _ = mp.render_ex(cam, G)
    return rad, var


@pytest.mark.parametrize("name", ["c2", "c3", "c5"])
def test_config_matches_reference(name):
    path, g = config_scene(name)
    sc = mp.load_scene(path)
    assert sc.camera.image_width == g["mean"].shape[1]
    G = mp.GpuScene(sc)
    rad, var = render(sc, G, int(g["spp"]), seed=21)
    assert rad.shape == g["mean"].shape
    assert_within_3_sigma(rad, var, g, name)


def test_guided_voxel_hall_matches_reference():
    """Guiding at its defaults (8 hidden layers, the first four bounces, a
    network trained from scratch inside the render) on the scene it is built
    for: the image stays within 3 sigma of the reference's."""
    path, g = config_scene("c5")
    sc = mp.load_scene(path)
    G = mp.GpuScene(sc)
    rad, var = render(sc, G, int(g["spp"]), seed=23, guided=1)
    assert_within_3_sigma(rad, var, g, "c5 guided")


@pytest.mark.parametrize("name", ["defocus_bokeh", "ortho", "checker"])
def test_camera_and_texture_paths_match_reference(name):
    g = load_golden(f"render_{name}")
    sc = mp.load_scene(scene_path(f"{name}.scene"))
    sc.camera.image_width = g["mean"].shape[1]
    G = mp.GpuScene(sc)
    rad, var = render(sc, G, int(g["spp"]), seed=5)
    assert_within_3_sigma(rad, var, g, name)


@pytest.mark.parametrize("name", ["materials", "cornell_c1"])
def test_feature_buffers_match_first_surface(name):
    """Albedo and normal guides (first_surface: the first surface that is not
    a perfect mirror or smooth glass, tinted by the specular hops before it;
    albedo 1 and normal 0 for escaped rays) against the reference's, per pixel
    within 3 sigma; the luminance-variance buffer (camera.h:237-244) agrees on
    the median pixel within 10 %."""
    g = np.load(os.path.join(GOLDEN, f"features_{name}.npz"))
    sc = mp.load_scene(scene_path(f"{name}.scene"))
    h, w = g["albedo"].shape[:2]
    cam = sc.camera
    cam.image_width = w
    spp = int(g["spp"]) * int(g["batches"])
    cam.samples_per_pixel = spp
    cam.collect_features = 1
    cam.seed = 3
    f = cam.render(mp.GpuScene(sc))
    assert f.albedo.shape == (h, w, 3)
    for q in ("albedo", "normal"):
        # the device's estimate has the variance of the reference's batch mean
        # (same total samples): twice that is the variance of the difference;
        # a floor of one sample's weight where the reference saw no spread
        ref, ref_var = g[q], g[f"{q}_var"]
        got = getattr(f, q)
        z = (got - ref) / np.sqrt(2 * ref_var + (1.0 / spp) ** 2 + (1e-4 * np.abs(ref)) ** 2)
        assert np.mean(np.abs(z) > 3) < 0.02, (q, np.mean(np.abs(z) > 3))
        assert np.mean(np.abs(z) > 5) < 0.002, (q, np.mean(np.abs(z) > 5))
    # variance of a mean of spp samples: the reference's per-batch buffer is
    # for spp / batches samples, so it is `batches` times the full render's;
    # per pixel the median, since image sums of variance estimates swing
    # with single fireflies
    ratio = f.variance * int(g["batches"]) / np.maximum(g["variance"], 1e-30)
    lit = g["variance"] > 0
    assert abs(np.median(ratio[lit]) - 1) < 0.1, np.median(ratio[lit])
    cam.collect_features = 0
