"""The environment's sampling tables (environment.h:147-176, 302-309): the
pdf table and an alias table holding the same distribution, built on the
host (Vose) and on the device (the prefix-sum sweep mypbr_gpu_scene_create
uses). An alias table's implied mass of entry k is
(prob_k + sum over entries aliasing k of (1 - prob)) / n.
"""
import numpy as np
import pytest

import mypbr_gb300 as mp


def implied_mass(prob, alias):
    n = len(prob)
    mass = prob.astype(np.float64).copy()
    np.add.at(mass, alias, 1.0 - prob.astype(np.float64))
    return mass / n


def sky(h, w, seed=3, black=False):
    rng = np.random.default_rng(seed)
    img = rng.random((h, w, 3)).astype(np.float32) ** 3
    img[h // 3: h // 3 + 2, w // 4: w // 4 + 3] = 5e4  # a sun
    img[rng.random((h, w)) < 0.1] = 0
    if black:
        img[:] = 0
    return img


def expected_pdf(img):
    h, w = img.shape[:2]
    st = np.sin(np.pi * (np.arange(h) + 0.5) / h)[:, None]
    lum = 0.2126 * img[..., 0].astype(np.float64) + 0.7152 * img[..., 1] + 0.0722 * img[..., 2]
    wgt = np.maximum(lum * st, 0)
    if wgt.sum() <= 0:
        wgt = np.broadcast_to(st, (h, w)).copy()
    return wgt / wgt.sum() * h * w


@pytest.mark.parametrize("black", [False, True])
def test_host_tables(black):
    img = sky(32, 64, black=black)
    pdf, prob, alias = mp.env_distribution(img, on_gpu=False)
    np.testing.assert_allclose(pdf, expected_pdf(img), rtol=1e-6)
    np.testing.assert_allclose(implied_mass(prob, alias) * pdf.size, pdf.reshape(-1), rtol=2e-5, atol=2e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("shape,black", [((32, 64), False), ((512, 1024), False), ((17, 33), True), ((1, 1), False)])
def test_device_tables(shape, black):
    img = sky(*shape, black=black)
    pdf_h, _, _ = mp.env_distribution(img, on_gpu=False)
    pdf, prob, alias = mp.env_distribution(img, on_gpu=True)
    np.testing.assert_allclose(pdf, pdf_h, rtol=1e-6)
    assert np.all((prob >= 0) & (prob <= 1)) and np.all((alias >= 0) & (alias < pdf.size))
    np.testing.assert_allclose(implied_mass(prob, alias) * pdf.size, pdf.reshape(-1), rtol=2e-5, atol=2e-6)
