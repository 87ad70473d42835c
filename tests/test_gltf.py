"""glTF 2.0 models on the host: geometry, the material mapping of the
reference's loader (gltf_loader.h:20-58, 138-251), override and replace,
and the errors. The geometry itself is pinned ray by ray to the reference
(hits_gallery in test_oracle_golden.py) and the images to stb_image
(test_images.py); here the mapping is checked field by field.
"""
import os
import shutil

import numpy as np
import pytest

import mypbr_gb300 as mp
from mypbr_gb300 import flat

HERE = os.path.dirname(os.path.abspath(__file__))
SCENES = os.path.join(HERE, "golden", "scenes")

TEX_SOLID, TEX_IMAGE, TEX_SCALED, TEX_CHANNEL, TEX_UV, TEX_NSCALE = 0, 2, 3, 4, 5, 6
MAT_THIN, MAT_PRINCIPLED, MAT_LIGHT = 3, 4, 5


def gallery(tail="", name="gallery.glb"):
    return flat.view(mp.parse_scene(f"material back lambertian 0.6 0.4 0.3\nmesh {name} {tail}\n", SCENES))


def parts(f):
    """{first triangle: (material record, mask)} of each mesh part."""
    return {int(m["first_triangle"]): (f["materials"][m["material"]], int(m["alpha_mask"]), int(m["triangle_count"]))
            for m in f["meshes"]}


def by_emission_or_type(f):
    out = {}
    for m, mask, n in parts(f).values():
        out.setdefault(int(m["type"]), []).append((m, mask, n))
    return out


def test_glb_and_gltf_give_the_same_model():
    a, b = gallery(), gallery(name="gallery.gltf")
    for k in ("positions", "normals", "uvs"):
        np.testing.assert_array_equal(a[k], b[k])
    for k in ("v", "n", "t", "flags"):
        np.testing.assert_array_equal(a["triangles"][k], b["triangles"][k])
    np.testing.assert_array_equal(a["materials"]["type"], b["materials"]["type"])
    assert len(a["texels_ldr"]) == len(b["texels_ldr"])


def test_paint_material():
    f = gallery()
    tex = f["textures"]
    paint = [m for m, mask, n in parts(f).values() if m["type"] == MAT_PRINCIPLED and m["flags"] & 2]
    assert len(paint) == 1
    m = paint[0]
    base = tex[m["tex"][0]]
    assert base["type"] == TEX_SCALED and tuple(base["p"][:3]) == (0.9, 0.8, 0.7)
    uv = tex[base["a"]]
    assert uv["type"] == TEX_UV
    np.testing.assert_allclose(uv["p"][:5], [0.1, 0.2, 0.3, 2.0, 2.0])
    assert tex[uv["a"]]["type"] == TEX_IMAGE and not tex[uv["a"]]["flags"] & 2  # colors: sRGB
    metallic, rough = tex[m["tex"][1]], tex[m["tex"][2]]
    assert metallic["type"] == TEX_CHANNEL and metallic["b"] == 2 and metallic["p"][0] == 0.8
    assert rough["type"] == TEX_CHANNEL and rough["b"] == 1 and rough["p"][0] == 0.9
    assert metallic["a"] == rough["a"] and tex[metallic["a"]]["flags"] & 2  # one linear image
    normals = tex[m["tex"][3]]
    assert normals["type"] == TEX_NSCALE and normals["p"][0] == 0.5 and tex[normals["a"]]["flags"] & 2
    # clear coat: weight 1, roughness 0.1, no coat normal map
    assert tuple(tex[m["tex"][4]]["p"][:3]) == (1, 1, 1)
    assert tex[m["tex"][5]]["p"][0] == pytest.approx(0.1)
    assert m["tex"][6] == -1
    assert m["p"][0] == pytest.approx(0.04)  # ior 1.5


def test_masks_lights_glow_glass_default():
    f = gallery()
    tex = f["textures"]
    kinds = by_emission_or_type(f)
    # the leaf and its mirror image share one part: the texture's alpha is the mask
    masked = [(m, mask, n) for m, mask, n in parts(f).values() if mask >= 0]
    masks = {mask: n for m, mask, n in masked}
    images = [k for k in masks if tex[k]["width"] == 16]
    assert len(images) == 1 and masks[images[0]] == 4
    leaf = tex[images[0]]
    assert not leaf["flags"] & 4 and not leaf["flags"] & 8  # clamped (sampler), alpha channel
    # the veil: a 1 x 1 coverage image of alpha round(0.4 * 255)
    const = [k for k in masks if tex[k]["width"] == 1]
    assert len(const) == 1
    off = tex[const[0]]["offset"] * 4
    assert list(f["texels_ldr"][off:off + 4]) == [255, 255, 255, 102]
    # the lamp: a light of emission 6 x (1, 0.9, 0.7)
    (lamp, mask, n), = kinds[MAT_LIGHT]
    np.testing.assert_allclose(lamp["p"][:3], [6.0, 5.4, 4.2])
    assert len(f["lights"]) == 1  # the scene has no sun or sky: the lamp is its one light
    # the glow: an emissive texture on a principled surface, scaled by the factor
    glow = [m for m, mask, n in parts(f).values() if m["emission_tex"] >= 0]
    assert len(glow) == 1
    e = tex[glow[0]["emission_tex"]]
    assert e["type"] == TEX_SCALED and tuple(e["p"][:3]) == (2, 2, 2) and tex[e["a"]]["type"] == TEX_IMAGE
    # glass: thin, tinted by the base color, ior 1.4
    (glass, mask, n), = kinds[MAT_THIN]
    assert glass["p"][0] == pytest.approx(1.4) and tuple(glass["p"][2:5]) == (0.8, 0.95, 0.85)
    # the default material: white, metallic 1, roughness 1
    defaults = [m for m, mask, n in parts(f).values()
                if m["type"] == MAT_PRINCIPLED and all(tuple(tex[m["tex"][c]]["p"][:3]) == (1, 1, 1) for c in range(3))]
    assert len(defaults) == 1


def test_mirrored_instance_keeps_the_winding():
    f = gallery()
    P = f["positions"]
    tri = f["triangles"]
    leaf_part = [m for m in f["meshes"] if m["alpha_mask"] >= 0 and f["textures"][m["alpha_mask"]]["width"] == 16][0]
    first, count = int(leaf_part["first_triangle"]), int(leaf_part["triangle_count"])
    for k in range(first, first + count):
        a, b, c = (P[tri["v"][k][i]] for i in range(3))
        assert np.cross(b - a, c - a)[2] > 0  # both copies face +z
    xs = {round(float(P[tri["v"][k][0]][0]), 6) for k in range(first, first + count)}
    assert len(xs) == 2  # two copies, in two places


def test_normalized_uvs_and_flip():
    f = gallery()
    uv = f["uvs"]
    # the leaf's u16 texture coordinates: k / 65535 in single precision, v flipped
    expect_u = np.float32(np.float32(65535) / np.float32(65535))
    assert np.any(uv[:, 0] == float(expect_u))
    assert uv[:, 1].min() >= 0 and uv[:, 1].max() <= 1


def test_override_material_keeps_masks():
    f = gallery("back")
    mats = {int(m["material"]) for m in f["meshes"]}
    assert len(mats) == 1
    assert any(m["alpha_mask"] >= 0 for m in f["meshes"])
    assert len(f["lights"]) == 0


def test_replace_swaps_one_material_and_drops_its_coverage():
    f = gallery("replace veil back")
    back = [k for k, m in enumerate(f["materials"]) if m["type"] == 0 and tuple(f["textures"][m["tex"][0]]["p"][:3])
            == (0.6, 0.4, 0.3)][0]
    veil = [m for m in f["meshes"] if m["material"] == back]
    assert len(veil) == 1 and veil[0]["alpha_mask"] == -1
    assert sum(m["alpha_mask"] >= 0 for m in f["meshes"]) == 1  # the leaf still masked


@pytest.mark.parametrize("tail,message", [
    ("replace nothing back", "has no material named 'nothing'"),
    ("back replace veil back", None),
    ("replace veil nowhere", "unknown material 'nowhere'"),
])
def test_replace_errors(tail, message):
    if message is None:
        # a material named on the line then 'replace' is an unknown transform
        with pytest.raises(mp.MypbrError):
            gallery(tail)
        return
    with pytest.raises(mp.MypbrError, match=message):
        gallery(tail)


def test_replace_with_line_material_and_obj():
    with pytest.raises(mp.MypbrError, match="can't be used together"):
        mp.parse_scene("material back lambertian 0.5 0.5 0.5\nmesh gallery.glb replace veil back back\n", SCENES)
    with pytest.raises(mp.MypbrError, match="'replace' is for glTF files"):
        mp.parse_scene("material back lambertian 0.5 0.5 0.5\nmesh tetra.obj replace a back\n", SCENES)


def test_missing_buffer_and_bad_json(tmp_path):
    src = open(os.path.join(SCENES, "gallery.gltf")).read()
    (tmp_path / "a.gltf").write_text(src.replace("data:application/octet-stream;base64,", "missing.bin#"))
    with pytest.raises(mp.MypbrError, match="cannot load the buffers"):
        mp.parse_scene("mesh a.gltf\n", str(tmp_path))
    (tmp_path / "b.gltf").write_text(src[: len(src) // 2])
    with pytest.raises(mp.MypbrError, match="cannot read glTF file"):
        mp.parse_scene("mesh b.gltf\n", str(tmp_path))
    (tmp_path / "c.gltf").write_text('{"asset": {"version": "2.0"}, "scenes": [{"nodes": []}]}')
    with pytest.raises(mp.MypbrError, match="has no triangles"):
        mp.parse_scene("mesh c.gltf\n", str(tmp_path))


def test_missing_image_is_a_warning(tmp_path, capfd):
    for name in os.listdir(SCENES):
        if name.startswith("gallery.") or name.endswith(".png"):
            shutil.copy(os.path.join(SCENES, name), tmp_path / name)
    os.remove(tmp_path / "gallery_glow.png")
    f = flat.view(mp.parse_scene("mesh gallery.gltf\n", str(tmp_path)))
    assert "cannot load image 'gallery_glow.png'" in capfd.readouterr().err
    assert not any(m["emission_tex"] >= 0 for m in f["materials"])


def test_left_out_features_are_listed(capfd):
    gallery()
    err = capfd.readouterr().err
    assert "not supported, left out: sheen" in err
