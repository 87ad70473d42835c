"""The denoiser: the FP64 oracle against the reference's own output (CPU), the
CUDA kernels against the oracle (GPU), and the reference's denoise_test cases
(tests/denoise_test.cpp:49-121 of the reference) restated on the GPU path."""
import ctypes

import numpy as np
import pytest

import mypbr_gb300 as mp
import oracle as orc
from conftest import GOLDEN

W = H = 64


def gpu_denoise(rad, alb, nrm, var, **kw):
    L = mp.lib()
    L.mypbr_gpu_denoise.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                                             ctypes.c_void_p, ctypes.c_int]
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (rad, alb, nrm, var)]
    out = np.zeros(arrs[0].shape)
    h, w = arrs[3].shape
    mp.check(L.mypbr_gpu_denoise(*[a.ctypes.data for a in arrs], w, h, None, out.ctypes.data, 0))
    return out


def lum(c):
    return 0.2126 * c[..., 0] + 0.7152 * c[..., 1] + 0.0722 * c[..., 2]


def make_frame(noise, seed, pixel):
    """A frame with the given albedo, normal, noise-free radiance per pixel plus
    Gaussian noise of relative deviation `noise` and the matching variance."""
    rng = np.random.default_rng(seed)
    a = np.zeros((H, W, 3))
    n = np.zeros((H, W, 3))
    r = np.zeros((H, W, 3))
    for j in range(H):
        for i in range(W):
            a[j, i], n[j, i], r[j, i] = pixel(i, j)
    sigma = noise * lum(r)
    noisy = r * (1 + noise * rng.normal(size=(H, W, 1)))
    return noisy, a, n, sigma ** 2, r


def test_oracle_denoiser_matches_reference():
    g = np.load(f"{GOLDEN}/denoise.npz")
    out = orc.denoise(g["radiance"], g["albedo"], g["normal"], g["variance"])
    np.testing.assert_allclose(out, g["out"], rtol=1e-12, atol=1e-15)


@pytest.mark.gpu
def test_gpu_denoiser_matches_reference():
    """FP32 kernels against the reference's FP64 output on the same frame (with
    fireflies, an albedo edge and a normal edge)."""
    g = np.load(f"{GOLDEN}/denoise.npz")
    out = gpu_denoise(g["radiance"], g["albedo"], g["normal"], g["variance"])
    scale = np.abs(g["out"]).max()
    np.testing.assert_allclose(out, g["out"], rtol=1e-4, atol=1e-5 * scale)


@pytest.mark.gpu
def test_gpu_denoiser_matches_oracle_on_a_render():
    """The frame of a Cornell render with features (albedo, normal, variance)."""
    from conftest import scene_path
    sc = mp.load_scene(scene_path("cornell_c1.scene"))
    cam = sc.camera
    cam.image_width = 96
    cam.samples_per_pixel = 8
    cam.collect_features = 1
    f = cam.render(mp.GpuScene(sc))
    want = orc.denoise(f.radiance, f.albedo, f.normal, f.variance)
    got = gpu_denoise(f.radiance, f.albedo, f.normal, f.variance)
    scale = np.abs(want).max()
    np.testing.assert_allclose(got, want, rtol=1e-3, atol=1e-4 * scale)
    assert np.abs(got - want).mean() < 1e-5 * scale


@pytest.mark.gpu
def test_flat_wall():
    grey = (np.full(3, 0.5), np.array([0, 0, 1.0]), np.full(3, 0.5))
    rad, a, n, var, truth = make_frame(0.3, 1, lambda i, j: grey)
    out = gpu_denoise(rad, a, n, var)
    before = np.sqrt(((rad - truth) ** 2).sum(axis=2).mean())
    after = np.sqrt(((out - truth) ** 2).sum(axis=2).mean())
    assert after < before / 5, before / after
    assert abs(lum(out).mean() - 0.5) < 0.01


@pytest.mark.gpu
def test_albedo_edge_kept():
    def texture(i, j):
        v = 0.2 if i < W // 2 else 0.8
        return np.full(3, v), np.array([0, 0, 1.0]), np.full(3, v)
    rad, a, n, var, clean = make_frame(0.3, 2, texture)
    out = gpu_denoise(rad, a, n, var)
    edge = slice(W // 2 - 1, W // 2 + 1)
    worst = np.abs(lum(out[:, edge]) - lum(clean[:, edge])).max()
    assert worst < 0.06, worst


@pytest.mark.gpu
def test_normal_edge_kept():
    def corner(i, j):
        up, side = np.array([0, 0, 1.0]), np.array([1.0, 0, 0])
        return np.full(3, 0.7), (up if i < W // 2 else side), (np.ones(3) if i < W // 2 else np.full(3, 0.1))
    rad, a, n, var, _ = make_frame(0.3, 3, corner)
    out = gpu_denoise(rad, a, n, var)
    got = lum(out[H // 2, W // 2])
    assert abs(got - 0.1) < 0.03, got


@pytest.mark.gpu
def test_firefly_removed_highlight_kept():
    grey = (np.full(3, 0.5), np.array([0, 0, 1.0]), np.full(3, 0.5))
    rad, a, n, var, _ = make_frame(0.0, 4, lambda i, j: grey)
    rad[20, 20] = 50
    var[20, 20] = 50 * 50
    rad[40, 40] = 50
    var[40, 40] = 5 * 5
    out = gpu_denoise(rad, a, n, var)
    assert lum(out[20, 20]) < 1
    assert lum(out[40, 40]) > 25
