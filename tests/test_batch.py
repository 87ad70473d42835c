"""Batched renders, graph replay and the autotuner: they change how the work
is launched, never the result. Random numbers are keyed by (seed, pixel,
pass, bounce), so every arrangement renders the same samples; only the order
of the FP64 film additions differs (relative differences ~1e-15)."""
import numpy as np
import pytest

import mypbr_gb300 as mp
from conftest import scene_path

pytestmark = pytest.mark.gpu


def camera_of(sc, width, spp, seed=3, depth=None):
    cam = sc.camera
    cam.image_width = width
    cam.samples_per_pixel = spp
    cam.seed = seed
    if depth:
        cam.max_depth = depth
    return cam


def test_graph_replay_matches_direct_launches():
    sc = mp.load_scene(scene_path("cornell_c1.scene"))
    G = mp.GpuScene(sc)
    cam = camera_of(sc, 48, 64)
    cam.samples_per_wave = 4  # many waves: the graph is replayed 16 times
    graphed = cam.render(G).radiance
    cam.timing = 1  # per-kernel events: direct launches
    direct, _, _ = mp.render_ex(cam, G)
    np.testing.assert_allclose(graphed, direct, rtol=1e-12, atol=1e-14)


def test_batch_matches_single_renders():
    torch = pytest.importorskip("torch")
    names = ["cornell_c1", "materials", "voxels", "env_spheres"]
    setups = []
    for k, name in enumerate(names):
        sc = mp.load_scene(scene_path(f"{name}.scene"))
        G = mp.GpuScene(sc)
        setups.append((sc, G, camera_of(sc, 32 + 8 * k, 16 * (k + 1), seed=10 + k)))
    # two more jobs on the first scene handle (run after its first, in order)
    extra = [camera_of(mp.load_scene(scene_path("cornell_c1.scene")), 40, 8, seed=99),
             camera_of(mp.load_scene(scene_path("cornell_c1.scene")), 24, 32, seed=98)]
    jobs, bufs, expect = [], [], []
    for sc, G, cam in setups:
        h = cam.height()
        buf = torch.zeros((h, cam.image_width, 3), dtype=torch.float64, device="cuda")
        bufs.append(buf)
        jobs.append((G, cam, buf.data_ptr()))
        expect.append(cam.render(G).radiance)
    for cam in extra:
        G = setups[0][1]
        buf = torch.zeros((cam.height(), cam.image_width, 3), dtype=torch.float64, device="cuda")
        bufs.append(buf)
        jobs.append((G, cam, buf.data_ptr()))
        expect.append(cam.render(G).radiance)
    codes = mp.render_batch(jobs)
    assert codes == [0] * len(jobs)
    torch.cuda.synchronize()
    for buf, ref in zip(bufs, expect):
        np.testing.assert_allclose(buf.cpu().numpy(), ref, rtol=1e-12, atol=1e-14)
    # the same batch again replays the graph kept on the first handle: the
    # outputs are rewritten from cleared films
    for buf in bufs:
        buf.fill_(float("nan"))
    assert mp.render_batch(jobs) == [0] * len(jobs)
    torch.cuda.synchronize()
    for buf, ref in zip(bufs, expect):
        np.testing.assert_allclose(buf.cpu().numpy(), ref, rtol=1e-12, atol=1e-14)
    # a changed job (another seed) is captured anew, not replayed
    cam = setups[2][2]
    cam.seed = 77
    changed = cam.render(setups[2][1]).radiance
    assert np.abs(changed - expect[2]).max() > 0
    assert mp.render_batch(jobs) == [0] * len(jobs)
    torch.cuda.synchronize()
    np.testing.assert_allclose(bufs[2].cpu().numpy(), changed, rtol=1e-12, atol=1e-14)
    for k in (0, 1, 3, 4, 5):
        np.testing.assert_allclose(bufs[k].cpu().numpy(), expect[k], rtol=1e-12, atol=1e-14)


def test_batch_reports_a_bad_job():
    torch = pytest.importorskip("torch")
    sc = mp.load_scene(scene_path("cornell_c1.scene"))
    G = mp.GpuScene(sc)
    good = camera_of(sc, 16, 4)
    bad = camera_of(mp.load_scene(scene_path("cornell_c1.scene")), 16, 4)
    bad.max_depth = 0
    b1 = torch.zeros((good.height(), 16, 3), dtype=torch.float64, device="cuda")
    b2 = torch.zeros((bad.height(), 16, 3), dtype=torch.float64, device="cuda")
    with pytest.raises(mp.MypbrError):
        mp.render_batch([(G, good, b1.data_ptr()), (G, bad, b2.data_ptr())])


def test_autotune_keeps_the_result():
    sc = mp.load_scene(scene_path("materials.scene"))
    G = mp.GpuScene(sc)
    cam = camera_of(sc, 64, 32)
    before = cam.render(G).radiance
    r = mp.autotune(cam, G)
    assert r["block"] in (128, 256) and r["wave_paths"] in (16 << 20, 32 << 20, 64 << 20, 128 << 20)
    assert r["traversal"] in (1, 2, 3, 4, 5) and len(r["trials"]) == 40
    assert all(t > 0 for t in r["trials"]) and r["mpaths_per_s"] == max(r["trials"])
    after = cam.render(G).radiance
    np.testing.assert_allclose(after, before, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("name", ["materials", "voxels", "fog_box"])
def test_persistent_traversal_matches(name):
    """Lanes that take new rays as theirs finish find the same hits. The
    kernels are compiled separately, so FP32 rounding of the media and fog
    distances may differ in the last bits: equal to 1e-5."""
    sc = mp.load_scene(scene_path(f"{name}.scene"))
    G = mp.GpuScene(sc)
    cam = camera_of(sc, 48, 16)
    mp.set_launch(G, traversal=4)
    a = cam.render(G).radiance
    mp.set_launch(G, traversal=1)
    b = cam.render(G).radiance
    mp.set_launch(G, block=128, wave_paths=1 << 16, traversal=1)
    c = cam.render(G).radiance
    np.testing.assert_allclose(b, a, rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(c, a, rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("traversal", [2, 3, 5])
@pytest.mark.parametrize("name", ["materials", "voxels", "fog_box", "gallery", "alpha_masks"])
def test_other_walks_match(name, traversal):
    """The walk over the tree collapsed to four children per node (2), the
    binary walk with postponed leaves (3) and the walk over the 8-wide tree
    with quantised boxes (5) meet the same closest hits (and,
    for shadow rays, the same blockers) as the plain binary walk: equal to
    1e-5 (separately compiled kernels round media and fog distances in their
    own last bits)."""
    sc = mp.load_scene(scene_path(f"{name}.scene"))
    G = mp.GpuScene(sc)
    cam = camera_of(sc, 48, 16)
    mp.set_launch(G, traversal=4)
    a = cam.render(G).radiance
    mp.set_launch(G, traversal=traversal)
    b = cam.render(G).radiance
    np.testing.assert_allclose(b, a, rtol=1e-5, atol=1e-7)
