"""The path-guiding network: tensor-core forward and backward passes, the
mixture loss and density, against the FP64 oracle (oracle/guide_oracle.py);
and guided rendering, which must stay unbiased and must gain over the plain
sampler on an occluded scene.

CPU tests check the oracle itself (analytic gradients against finite
differences, the mixture density's normalisation); GPU tests go through the
C ABI (mypbr_guide_test_* and mypbr_gpu_render with guided != 0).
"""
import os
import tempfile

import numpy as np
import pytest

import guide_oracle as go
import mypbr_gb300 as mp
from conftest import GOLDEN, scene_path


def random_net(hidden, seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    parts = []
    for l in range(hidden + 1):
        k = 128 if l == 0 else 64
        parts.append(rng.uniform(-1, 1, 64 * k) * np.sqrt(6.0 / k) * scale)
    return np.concatenate(parts)


def random_inputs(n, seed=1):
    rng = np.random.default_rng(seed)
    return go.one_blob(rng.random((n, 7)))


def random_raw(n, seed=2):
    rng = np.random.default_rng(seed)
    raw = rng.normal(size=(n, 64))
    raw[:, 3:40:5] = rng.uniform(-2, 5, size=(n, 8))  # log kappa
    return raw


def unit(v):
    return v / np.linalg.norm(v, axis=1, keepdims=True)


# ------------------------------------------------------------------- CPU

def test_oracle_loss_gradient_is_the_derivative():
    rng = np.random.default_rng(3)
    raw = random_raw(40)
    w = unit(rng.normal(size=(40, 3)))
    c = rng.uniform(0.1, 2, 40)
    g = go.loss_grad(raw, w, c)
    eps = 1e-6
    num = np.zeros_like(g)
    for k in range(40):
        d = np.zeros(64)
        d[k] = eps
        num[:, k] = (go.loss(raw + d, w, c) - go.loss(raw - d, w, c)) / (2 * eps)
    np.testing.assert_allclose(g, num, rtol=1e-5, atol=1e-7)


def test_oracle_backward_is_the_derivative():
    hidden = 2
    w = random_net(hidden, 4)
    x = random_inputs(6, 5)
    rng = np.random.default_rng(6)
    dout = rng.normal(size=(6, 64))
    g = go.backward(w, hidden, x, dout, rounding=False)
    eps = 1e-6
    for k in rng.choice(len(w), 60, replace=False):
        d = np.zeros_like(w)
        d[k] = eps
        f1 = (go.forward(w + d, hidden, x, rounding=False)[0] * dout).sum()
        f0 = (go.forward(w - d, hidden, x, rounding=False)[0] * dout).sum()
        assert abs((f1 - f0) / (2 * eps) - g[k]) < 1e-5 * (1 + abs(g[k]))


def test_oracle_mixture_density_integrates_to_one():
    raw = random_raw(5, 7)
    # a Fibonacci sphere of 200k points: equal-area quadrature
    m = 200000
    k = np.arange(m) + 0.5
    z = 1 - 2 * k / m
    r = np.sqrt(1 - z * z)
    phi = k * np.pi * (3 - np.sqrt(5))
    dirs = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    for i in range(5):
        p = go.pdf(np.repeat(raw[i:i + 1], m, axis=0), dirs)
        assert abs(p.mean() * 4 * np.pi - 1) < 2e-3


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125 * 1.5, -3.1415926, 65504.0])
    r = go.bf16(x)
    # 1 + 2^-8 is halfway between 1 and 1 + 2^-7: ties to even -> 1
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert np.all(np.abs(r - x) <= np.abs(x) * 2.0 ** -8)


# ------------------------------------------------------------------- GPU

@pytest.mark.gpu
def test_encoding_matches_oracle():
    """The one-blob encoding the forward kernels write (neighbour-ratio
    recurrence, three exponentials per block of 8 bins) against the oracle's
    exact Gaussians rounded to BF16: within one BF16 step everywhere, equal
    for nearly every value that matters (>= 1e-6); values below 1e-18 may be
    0 (far tails, where FP32 underflows)."""
    rng = np.random.default_rng(21)
    s = rng.random((3000, 7))
    s[:20] = 0.0  # the edges of the unit interval
    s[20:40] = 1.0
    got = mp.guide_encode(s.astype(np.float32)).astype(np.float64)
    want = go.one_blob(s.astype(np.float32).astype(np.float64))
    want_bf16 = go.bf16(want)
    ulp = np.abs(want_bf16) * 2.0 ** -7
    diff = np.abs(got - want_bf16)
    assert np.all(diff <= ulp + 1e-18), diff.max()
    visible = want_bf16 >= 1e-6
    assert np.mean(diff[visible] == 0) > 0.99, np.mean(diff[visible] == 0)


@pytest.mark.gpu
@pytest.mark.parametrize("hidden", [2, 4, 8])
def test_tensor_core_forward_matches_oracle(hidden):
    w = random_net(hidden, 10 + hidden)
    x = random_inputs(1000, 11)  # not a multiple of the 128-row tile
    out = mp.guide_forward(hidden, w, x)
    ref, _, _ = go.forward(w.astype(np.float32).astype(np.float64), hidden, x.astype(np.float32))
    scale = np.sqrt((ref ** 2).mean())
    err = np.abs(out - ref)
    # FP32 accumulation order and BF16 re-rounding of the hidden activations
    # are the only differences from the oracle
    assert np.median(err) < 1e-3 * scale, (np.median(err), scale)
    assert err.max() < 3e-2 * scale, (err.max(), scale)


@pytest.mark.gpu
@pytest.mark.parametrize("hidden", [2, 4, 8])
def test_tensor_core_backward_matches_oracle(hidden):
    w = random_net(hidden, 20 + hidden)
    x = random_inputs(777, 21)
    rng = np.random.default_rng(22)
    dout = rng.normal(size=(777, 64)).astype(np.float32)
    g = mp.guide_backward(hidden, w, x, dout)
    ref = go.backward(w.astype(np.float32).astype(np.float64), hidden, x.astype(np.float32), dout)
    off = 0
    for l in range(hidden + 1):
        k = 128 if l == 0 else 64
        a, b = g[off:off + 64 * k], ref[off:off + 64 * k]
        scale = np.sqrt((b ** 2).mean())
        err = np.abs(a - b)
        assert np.median(err) < 2e-3 * scale, (l, np.median(err), scale)
        assert err.max() < 5e-2 * scale + 1e-6, (l, err.max(), scale)
        off += 64 * k


@pytest.mark.gpu
def test_loss_gradient_matches_oracle():
    rng = np.random.default_rng(30)
    raw = random_raw(5000, 31).astype(np.float32)
    w = unit(rng.normal(size=(5000, 3))).astype(np.float32)
    c = rng.uniform(0.1, 2, 5000).astype(np.float32)
    g, loss = mp.guide_loss(raw, w, c)
    ref_g = go.loss_grad(raw, w, c)
    ref_l = go.loss(raw, w, c)
    np.testing.assert_allclose(loss, ref_l, rtol=2e-3, atol=2e-3)
    scale = np.abs(ref_g).max(axis=1, keepdims=True) + 1e-6
    assert np.median(np.abs(g - ref_g) / scale) < 1e-4
    assert np.percentile(np.abs(g - ref_g) / scale, 99.9) < 1e-2


@pytest.mark.gpu
def test_mixture_sampling_matches_its_density():
    rng = np.random.default_rng(40)
    n = 200000
    raw = np.repeat(random_raw(1, 41), n, axis=0).astype(np.float32)
    u = rng.random((n, 3)).astype(np.float32)
    dirs = unit(rng.normal(size=(n, 3))).astype(np.float32)
    s, ps, pd = mp.guide_mixture(raw, u, dirs)
    assert np.allclose(np.linalg.norm(s, axis=1), 1, atol=1e-5)
    # the density at the samples is the one the oracle gives (FP16-packed parameters)
    ref = go.pdf(raw[:1000], s[:1000])
    np.testing.assert_allclose(ps[:1000], ref, rtol=2e-2)
    np.testing.assert_allclose(pd[:1000], go.pdf(raw[:1000], dirs[:1000]), rtol=2e-2, atol=1e-6)
    # E[1 / q(w)] over samples w ~ q is the sphere's area
    est = (1.0 / ps).mean()
    sigma = (1.0 / ps).std() / np.sqrt(n)
    assert abs(est - 4 * np.pi) < 5 * sigma + 1e-3, (est, sigma)


def _render(sc, G, spp, guided, per_wave, seed=1):
    cam = sc.camera
    cam.samples_per_pixel = spp
    cam.guided = guided
    cam.samples_per_wave = per_wave
    cam.seed = seed
    rad, var, stats = mp.render_ex(cam, G)
    return rad, var, stats


@pytest.mark.gpu
def test_guided_render_matches_reference():
    """The guide only changes how directions are sampled: the image must stay
    within 3 sigma of the reference's (the plain renders' criterion)."""
    g = np.load(f"{GOLDEN}/render_cornell_c1.npz")
    sc = mp.load_scene(scene_path("cornell_c1.scene"))
    sc.camera.image_width = g["mean"].shape[1]
    G = mp.GpuScene(sc)
    rad, var, _ = _render(sc, G, 1024, 2, 16)
    z = (rad - g["mean"]) / np.sqrt(var + g["var_of_mean"] + 1e-30)
    assert np.mean(np.abs(z) > 3) < 0.02, np.mean(np.abs(z) > 3)
    assert np.mean(np.abs(z) > 5) < 0.002
    n = rad.shape[0] * rad.shape[1]
    tot_sigma = np.sqrt(var.sum(axis=(0, 1)) + g["var_of_mean"].sum(axis=(0, 1))) / n
    tot_z = (rad.mean(axis=(0, 1)) - g["mean"].mean(axis=(0, 1))) / tot_sigma
    assert np.all(np.abs(tot_z) < 4), tot_z


@pytest.mark.gpu
@pytest.mark.parametrize("alpha,depths", [(0.3, 1), (0.8, 50)])
def test_guided_settings_stay_unbiased(alpha, depths):
    """Other mixing probabilities and guided depths (every bounce of the
    Cornell box's 50): still within 3 sigma of the reference's image."""
    g = np.load(f"{GOLDEN}/render_cornell_c1.npz")
    sc = mp.load_scene(scene_path("cornell_c1.scene"))
    sc.camera.image_width = g["mean"].shape[1]
    G = mp.GpuScene(sc)
    mp.guide_configure(G, alpha=alpha, depths=depths)
    rad, var, _ = _render(sc, G, 1024, 2, 16)
    z = (rad - g["mean"]) / np.sqrt(var + g["var_of_mean"] + 1e-30)
    assert np.mean(np.abs(z) > 3) < 0.02, np.mean(np.abs(z) > 3)
    assert np.mean(np.abs(z) > 5) < 0.002
    with pytest.raises(mp.MypbrError, match="alpha must lie"):
        mp.guide_configure(G, alpha=1.0, depths=2)
    with pytest.raises(mp.MypbrError, match="depths"):
        mp.guide_configure(G, alpha=0.5, depths=0)


@pytest.mark.gpu
def test_guide_schedule_checks_the_weight_cap():
    sc = mp.load_scene(scene_path("cornell_c1.scene"))
    G = mp.GpuScene(sc)
    mp.guide_schedule(G, weight_cap=0.0)  # no cap
    mp.guide_schedule(G, weight_cap=64.0)
    for bad in (0.5, -1.0, 2.0e6, float("nan")):
        with pytest.raises(mp.MypbrError, match="weight_cap"):
            mp.guide_schedule(G, weight_cap=bad)
    G.close()


def test_guide_configure_checks_its_handle():
    with pytest.raises(mp.MypbrError, match="null scene"):
        mp.guide_configure(None)


def rel_mse(x, ref, eps=0.01):
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + eps)))


@pytest.mark.gpu
def test_guiding_gains_on_occluded_scene():
    """The trained network against the method without it: relMSE at equal
    samples per pixel in the voxel hall lit through slits (a 128^3 version).
    The network is trained by one guided render on its scene handle first
    (a handle keeps its network from render to render, and it goes on
    learning during the compared renders); the mixture is used once the
    handle's network has taken 128 training steps, which a fresh network
    does not reach within a render of this size."""
    from mypbr_gb300 import workloads
    d = tempfile.mkdtemp()
    p = workloads.voxel_hall_scene(d, size=128, width=64, height=36, spp=64)
    sc = mp.load_scene(p)
    G = mp.GpuScene(sc)
    ref, _, _ = _render(sc, G, 16384, 0, 0, seed=99)
    seeds = range(1, 13)
    plain = [rel_mse(_render(sc, G, 256, 0, 0, seed=s)[0], ref) for s in seeds]
    Gg = mp.GpuScene(sc)
    _render(sc, Gg, 4096, 2, 64, seed=500)  # the training render
    guided = [rel_mse(_render(sc, Gg, 256, 2, 8, seed=s)[0], ref) for s in seeds]
    Gg.close()
    # single renders of this scene are firefly-dominated (one render's relMSE
    # swings by 10x or more either way), so the typical render decides
    plain, guided = float(np.median(plain)), float(np.median(guided))
    print(f"median relMSE over {len(seeds)} renders at 256 spp: plain {plain:.4f}, guided {guided:.4f}")
    assert guided < plain, (guided, plain)
