"""The FP64 oracle against the reference's own golden vectors (CPU only).

The goldens in tests/golden/*.npz were produced by the reference's headers
through oracle/ref_harness.cpp (tests/golden/gen_golden.py). The oracle reads
the flat scene made by the product's host loader, so these tests pin the
loader and the oracle together against the reference.
"""
import numpy as np
import pytest

import mypbr_gb300 as mp
import oracle as orc
from conftest import GOLDEN, scene_path
from mypbr_gb300 import flat


def load_golden(name):
    return np.load(f"{GOLDEN}/{name}.npz")


def rays_of(g):
    n = len(g["hit"])
    rays = np.zeros((n, 8))
    rays[:, 0:3] = g["o"]
    rays[:, 3:6] = g["d"]
    rays[:, 6] = 0.001
    rays[:, 7] = np.inf
    return rays


def material_ids(scene):
    """Probe scenes encode an object's id in its lambertian's red albedo: (id + 1) / 1024."""
    v = flat.view(scene)
    ids = []
    for m in v["materials"]:
        t = m["tex"][0]
        ids.append(int(round(v["textures"][t]["p"][0] * 1024)) - 1 if t >= 0 else -99)
    return np.array(ids)


@pytest.mark.parametrize("scene_name,golden", [("hits_mix", "hits_mix"), ("cornell_c1", "hits_cornell"),
                                               ("gallery_hits", "hits_gallery")])
def test_closest_hits_match_reference(scene_name, golden):
    sc = mp.load_scene(scene_path(f"{scene_name}.scene"))
    g = load_golden(golden)
    hits, prim = orc.OracleScene(sc).trace(rays_of(g))
    hit = prim[:, 0] >= 0
    assert np.array_equal(hit, g["hit"] > 0), "hit/miss differs from the reference"
    both = hit
    np.testing.assert_allclose(hits[both, 0], g["t"][both], rtol=1e-12)
    np.testing.assert_allclose(hits[both, 1:4], g["normal"][both], atol=1e-12)
    np.testing.assert_array_equal(hits[both, 6], g["front"][both])
    np.testing.assert_allclose(hits[both, 4], g["u"][both], atol=1e-9)
    np.testing.assert_allclose(hits[both, 5], g["v"][both], atol=1e-9)
    if "material_id" in g.files:
        ids = material_ids(sc)[hits[both, 7].astype(int)]
        np.testing.assert_array_equal(ids, g["material_id"][both])


def test_bvh_walk_equals_brute_force():
    sc = mp.load_scene(scene_path("hits_mix.scene"))
    g = load_golden("hits_mix")
    O = orc.OracleScene(sc)
    h1, p1 = O.trace(rays_of(g))
    h2, p2 = O.trace(rays_of(g), brute_force=True)
    np.testing.assert_array_equal(p1[:, 0] >= 0, p2[:, 0] >= 0)
    np.testing.assert_allclose(h1[:, 0], h2[:, 0], rtol=1e-14)


def bsdf_records(b):
    n = len(b["sphere"])
    rec = np.zeros((n, 16))
    rec[:, 5] = 1.0  # normal (0, 0, 1)
    rec[:, 6] = 1 - b["face"]  # front face for face 0
    rec[:, 7] = 0.25
    rec[:, 8] = 0.75
    rec[:, 9] = 2.0  # dpdu (2, 0, 0)
    rec[:, 13] = 3.0  # dpdv (0, 3, 0)
    return rec


def probe_materials(scene):
    v = flat.view(scene)
    return v["spheres"]["material"]


def test_bsdf_eval_and_pdf_match_reference():
    sc = mp.load_scene(scene_path("bsdf_probe.scene"))
    b = load_golden("bsdf_probe")
    O = orc.OracleScene(sc)
    mats = probe_materials(sc)
    rec = bsdf_records(b)
    for k in np.unique(b["sphere"]):
        m = b["sphere"] == k
        out = O.bsdf(int(mats[k]), rec[m], -b["wo"][m], b["wi"][m])
        np.testing.assert_allclose(out[:, :3], b["eval"][m], rtol=1e-12, atol=1e-14, err_msg=f"material {k} eval")
        np.testing.assert_allclose(out[:, 3], b["pdf"][m], rtol=1e-12, atol=1e-14, err_msg=f"material {k} pdf")
        np.testing.assert_array_equal(out[:, 4], b["skip_pdf"][m])
        np.testing.assert_array_equal(out[:, 5], b["scatters"][m])


def test_light_probabilities_exact():
    """pdf_test.cpp:195-215 checks the power-based probabilities to 1e-9/1e-12."""
    sc = mp.load_scene(scene_path("lights_mix.scene"))
    g = load_golden("lights_mix")
    p = flat.view(sc)["lights"]["probability"]
    np.testing.assert_allclose(p, g["probability"], rtol=1e-12)
    assert abs(p.sum() - 1) < 1e-12


def test_light_pdf_matches_reference():
    sc = mp.load_scene(scene_path("lights_mix.scene"))
    g = load_golden("lights_mix")
    pdf = orc.OracleScene(sc).light_pdf(g["origin"], g["dir"])
    np.testing.assert_allclose(pdf, g["pdf"], rtol=1e-9, atol=1e-15)


def test_light_sampling_matches_its_pdf():
    """E[1/pdf] over light samples restricted to a set S equals |S|'s measure
    only if value() agrees with generate(); here with f = 1 over all
    directions the estimate of the total solid angle is 4 pi when every
    direction is reachable (the uniform sky is)."""
    sc = mp.load_scene(scene_path("lights_mix.scene"))
    O = orc.OracleScene(sc)
    o = np.array([278.0, 278.0, 278.0])
    d = O.light_sample(o, 200000, seed=3)
    p = O.light_pdf(np.repeat(o[None], len(d), 0), d)
    est = np.mean(1.0 / p[p > 0]) * np.mean(p > 0)
    assert abs(est - 4 * np.pi) < 0.4


def test_environment_matches_reference():
    sc = mp.load_scene(scene_path("env_spheres.scene"))
    g = load_golden("env_small")
    rad, pdf = orc.OracleScene(sc).environment(g["dir"])
    np.testing.assert_allclose(rad, g["radiance"], rtol=1e-12)
    np.testing.assert_allclose(pdf, g["pdf"], rtol=1e-12)


def test_ggx_table_matches_reference():
    g = load_golden("ggx_table")
    E, Eavg = orc.ggx_table()
    E2, Eavg2 = mp.ggx_albedo_table()
    np.testing.assert_array_equal(E, E2)
    np.testing.assert_array_equal(Eavg, Eavg2)
    x = np.clip(g["mu"], 0, 1) * 31
    y = np.clip(np.sqrt(g["alpha"]), 0, 1) * 31
    i = np.minimum(x.astype(int), 30)
    j = np.minimum(y.astype(int), 30)
    tx, ty = x - i, y - j
    val = (1 - ty) * ((1 - tx) * E[j, i] + tx * E[j, i + 1]) + ty * ((1 - tx) * E[j + 1, i] + tx * E[j + 1, i + 1])
    np.testing.assert_allclose(val, g["E"], rtol=0, atol=1e-15)


def render_z(rad, var, g):
    # pixels without Monte Carlo noise (a uniform sky seen directly) get a
    # floor of 1e-4 of their value
    z = (rad - g["mean"]) / np.sqrt(var + g["var_of_mean"] + (1e-4 * np.abs(g["mean"])) ** 2 + 1e-30)
    n = rad.shape[0] * rad.shape[1]
    tot_sigma = np.sqrt(var.sum(axis=(0, 1)) + g["var_of_mean"].sum(axis=(0, 1))) / n
    tot_z = (rad.mean(axis=(0, 1)) - g["mean"].mean(axis=(0, 1))) / tot_sigma
    return z, tot_z


@pytest.mark.parametrize("name", ["cornell_c1", "env_spheres", "fog_box", "materials", "voxels", "voxels_style",
                                  "alpha_masks", "gallery", "defocus_bokeh", "ortho", "checker"])
def test_oracle_render_matches_reference_render(name):
    """Per-pixel means within 3 sigma of the combined Monte Carlo error, for
    the oracle vs the reference's batch means."""
    g = load_golden(f"render_{name}")
    sc = mp.load_scene(scene_path(f"{name}.scene"))
    cam = sc.camera
    cam.image_width = g["mean"].shape[1]
    cam.samples_per_pixel = 256
    rad, var, _ = orc.OracleScene(sc).render(cam, threads=0)
    z, tot_z = render_z(rad, var, g)
    assert np.mean(np.abs(z) > 3) < 0.02
    assert np.mean(np.abs(z) > 5) < 0.002
    assert np.all(np.abs(tot_z) < 4), tot_z


@pytest.mark.parametrize("name,spp", [("c2", 1024), ("c3", 1024), ("c5", 8192)])
def test_oracle_matches_reference_on_configs(name, spp, tmp_path):
    """The benchmark configurations at test size (tests/golden/config_scenes.py):
    the generated inputs are the ones the reference rendered (digest), and the
    oracle's image is within 3 sigma of the reference's. The sample counts are
    high enough for the per-pixel variance estimates to see the rare bright
    paths (in the hall, a diffuse bounce that finds a sunlit patch): with a
    few hundred samples most pixels have not met one yet and their spread is
    underestimated."""
    import sys
    sys.path.insert(0, GOLDEN)
    import config_scenes
    g = load_golden(f"render_{name}")
    path, digest = config_scenes.CONFIGS[name](str(tmp_path))
    assert digest == str(g["digest"])
    sc = mp.load_scene(path)
    cam = sc.camera
    assert (cam.image_width, cam.height()) == (g["mean"].shape[1], g["mean"].shape[0])
    cam.samples_per_pixel = spp
    rad, var, _ = orc.OracleScene(sc).render(cam, threads=0)
    z, tot_z = render_z(rad, var, g)
    assert np.mean(np.abs(z) > 3) < 0.02, np.mean(np.abs(z) > 3)
    assert np.mean(np.abs(z) > 5) < 0.002
    assert np.all(np.abs(tot_z) < 4), tot_z


@pytest.mark.parametrize("name", ["materials", "cornell_c1"])
def test_oracle_features_match_reference(name):
    """first_surface's albedo and normal (camera.h:253-277) and the luminance
    variance buffer (camera.h:237-244), oracle against reference."""
    g = load_golden(f"features_{name}")
    sc = mp.load_scene(scene_path(f"{name}.scene"))
    h, w = g["albedo"].shape[:2]
    cam = sc.camera
    cam.image_width = w
    spp = int(g["spp"]) * int(g["batches"]) // 4
    cam.samples_per_pixel = spp
    rad, var, ex = orc.OracleScene(sc).render(cam, threads=0, features=True)
    for q in ("albedo", "normal"):
        # a quarter of the reference's samples: four times its variance; a
        # floor of one sample's weight where the reference saw no spread
        z = (ex[q] - g[q]) / np.sqrt(5 * g[f"{q}_var"] + (1.0 / spp) ** 2 + (1e-4 * np.abs(g[q])) ** 2)
        assert np.mean(np.abs(z) > 3) < 0.02, (q, np.mean(np.abs(z) > 3))
        assert np.mean(np.abs(z) > 5) < 0.002, q
    # the variance of the mean over spp samples against the reference's over
    # spp / batches (times the ratio of sample counts); per pixel the median,
    # since image sums of variance estimates swing with single fireflies
    ratio = ex["lum_var"] * (spp / int(g["spp"])) / np.maximum(g["variance"], 1e-30)
    lit = g["variance"] > 0
    assert abs(np.median(ratio[lit]) - 1) < 0.1, np.median(ratio[lit])
