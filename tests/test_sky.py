"""`sky atmosphere`: the single-scattering sky bake against the reference's
atmosphere::bake (tests/golden/sky.npz), on the host and on the device, and a
`style voxel` scene (sun reddened by the air, baked sky, ground) end to end."""
import math

import numpy as np
import pytest

import mypbr_gb300 as mp
import oracle as orc
from conftest import GOLDEN, scene_path
from mypbr_gb300 import flat

G = np.load(f"{GOLDEN}/sky.npz")


def case(k):
    el, az, e, r, m, g, oz, it = G["cases"][k]
    el, az = math.radians(el), math.radians(az)
    d = [math.cos(el) * math.sin(az), math.sin(el), -math.cos(el) * math.cos(az)]
    return d, [e, 0.9 * e, 0.8 * e], dict(rayleigh=r, mie=m, mie_g=g, ozone=oz, intensity=it)


@pytest.mark.parametrize("k", range(4))
def test_host_bake_matches_reference(k):
    d, irr, kw = case(k)
    img, t = mp.sky_bake(d, irr, 64, 32, **kw)
    np.testing.assert_allclose(img, G["bake"][k], rtol=1e-13, atol=1e-300)
    np.testing.assert_allclose(t, G["sun_transmittance"][k], rtol=1e-13, atol=1e-300)


def test_style_voxel_scene_lights_match_reference():
    sc = mp.load_scene(scene_path("voxels_style.scene"))
    g = np.load(f"{GOLDEN}/lights_style.npz")
    v = flat.view(sc)
    np.testing.assert_allclose(v["lights"]["probability"], g["probability"], rtol=1e-12)
    env = v["environment"]
    assert (env.width, env.height) == (256, 128)
    O = orc.OracleScene(sc)
    np.testing.assert_allclose(O.light_pdf(g["origin"], g["dir"]), g["pdf"], rtol=1e-6, atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(4))
def test_device_bake_matches_host(k):
    d, irr, kw = case(k)
    host, t = mp.sky_bake(d, irr, 64, 32, **kw)
    dev, t2 = mp.sky_bake(d, irr, 64, 32, on_gpu=True, **kw)
    # FP64 on both; exp and sqrt may differ in the last bit, over a march of
    # 32 x 16 steps that stays below 1e-11
    np.testing.assert_allclose(dev, host, rtol=1e-11, atol=1e-300)
    np.testing.assert_allclose(dev, G["bake"][k], rtol=1e-11, atol=1e-300)
