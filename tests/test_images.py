"""Image textures, MTL materials and alpha masks on the host.

The decoders are pinned to the reference's own stb_image (tests/golden/
images.npz, written by gen_golden.py through the harness's `image` command):
every fixture must decode to the same bytes and channel count. The MTL
mapping follows obj_loader.h:33-177 and the mask rules texture.h:161-181.
"""
import os
import struct

import numpy as np
import pytest

import mypbr_gb300 as mp
from mypbr_gb300 import flat

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
IMAGES = os.path.join(GOLDEN, "images")
SCENES = os.path.join(GOLDEN, "scenes")

_g = np.load(os.path.join(GOLDEN, "images.npz"))
FIXTURES = sorted({k.split(":")[0] for k in _g.files})


@pytest.mark.parametrize("name", [n for n in FIXTURES if not n.endswith(".jpg")])
def test_decode_matches_stb(name):
    rgba, channels = mp.read_image(os.path.join(IMAGES, name))
    ref = _g[name + ":rgba"]
    meta = _g[name + ":meta"]
    assert channels == meta[2]
    assert rgba.shape == ref.shape
    np.testing.assert_array_equal(rgba, ref)


@pytest.mark.parametrize("name", [n for n in FIXTURES if n.endswith(".jpg")])
def test_jpeg_decode_close_to_stb(name):
    """Baseline and progressive JPEG: the inverse DCT and colour conversion are
    the standard's (FP32 here, fixed point in stb_image), so bytes may differ
    by a few counts: at most 3, on average under 0.2; chroma upsampling, edges
    included, and the channel count as stb_image's."""
    rgba, channels = mp.read_image(os.path.join(IMAGES, name))
    ref = _g[name + ":rgba"]
    assert channels == _g[name + ":meta"][2]
    assert rgba.shape == ref.shape
    d = np.abs(rgba.astype(int) - ref.astype(int))
    assert d.max() <= 3 and d.mean() < 0.2, (d.max(), d.mean())


def test_fixture_set_covers_the_formats():
    assert len(FIXTURES) >= 30
    assert any(n.endswith(".tga") for n in FIXTURES) and any("interlaced" in n for n in FIXTURES)


def _texture_scene(tmp_path, image, option=""):
    text = f"texture t image {image} {option}\nmaterial m lambertian texture t\nsphere 0 0 -1 0.5 m\n"
    return mp.parse_scene(text, str(tmp_path) if not os.path.isabs(image) else "/")


@pytest.mark.parametrize("name", ["rgba8.png", "grey4.png", "ga16.png", "palette4_trns.png", "true24.tga",
                                  "mapped8_rle.tga"])
def test_scene_image_texture_texels(name, tmp_path):
    sc = _texture_scene(tmp_path, os.path.join(IMAGES, name))
    f = flat.view(sc)
    t = f["textures"][-1]
    meta = _g[name + ":meta"]
    assert t["type"] == 2 and t["width"] == meta[0] and t["height"] == meta[1]
    assert not (t["flags"] & 1) and not (t["flags"] & 4)  # 8-bit, clamped
    # the mask reads the red byte when the file has no alpha channel
    assert bool(t["flags"] & 8) == (not meta[3])
    n = int(meta[0] * meta[1] * 4)
    texels = f["texels_ldr"][t["offset"] * 4: t["offset"] * 4 + n]
    np.testing.assert_array_equal(texels, _g[name + ":rgba"].reshape(-1))


def test_scene_image_texture_linear_flag(tmp_path):
    f = flat.view(_texture_scene(tmp_path, os.path.join(IMAGES, "rgb8.png"), "linear"))
    assert f["textures"][-1]["flags"] & 2


def test_hdr_is_recognised_by_content(tmp_path):
    src = os.path.join(SCENES, "env_small.hdr")
    dst = tmp_path / "sky.img"
    dst.write_bytes(open(src, "rb").read())
    f = flat.view(_texture_scene(tmp_path, str(dst)))
    assert f["textures"][-1]["flags"] & 1


def test_missing_image_is_an_error(tmp_path):
    with pytest.raises(mp.MypbrError, match="cannot load image"):
        _texture_scene(tmp_path, str(tmp_path / "nope.png"))


def test_arithmetic_coded_jpeg_is_reported_unsupported(tmp_path):
    p = tmp_path / "photo.jpg"
    # SOI, then an arithmetic-coded frame header (SOF9)
    p.write_bytes(b"\xff\xd8\xff\xc9\x00\x11\x08\x00\x10\x00\x10\x03\x01\x22\x00\x02\x11\x01\x03\x11\x01"
                  + b"\xff\xd9")
    with pytest.raises(mp.MypbrError, match="arithmetic-coded") as e:
        _texture_scene(tmp_path, str(p))
    assert e.value.status == 2
    with pytest.raises(mp.MypbrError) as e2:
        mp.read_image(str(p))
    assert e2.value.status == 2


def test_truncated_png_is_rejected(tmp_path):
    """A file cut inside its image data fails to load (stb_image returns no
    image either; like stb, checksums are not verified, so damaged deflate
    data that still parses decodes to whatever it says)."""
    data = open(os.path.join(IMAGES, "rgba8.png"), "rb").read()
    p = tmp_path / "cut.png"
    p.write_bytes(data[:len(data) // 2])
    with pytest.raises(mp.MypbrError):
        mp.read_image(str(p))
    with pytest.raises(mp.MypbrError, match="cannot load image"):
        _texture_scene(tmp_path, str(p))


def test_run_length_bmp_is_reported_unsupported(tmp_path):
    """stb_image reads neither RLE nor embedded JPEG / PNG BMP files."""
    data = bytearray(open(os.path.join(IMAGES, "pal8.bmp"), "rb").read())
    for compress, words in ((1, "run-length"), (4, "embedded JPEG")):
        struct.pack_into("<I", data, 30, compress)
        p = tmp_path / f"c{compress}.bmp"
        p.write_bytes(bytes(data))
        with pytest.raises(mp.MypbrError, match=words) as e:
            mp.read_image(str(p))
        assert e.value.status == 2
        with pytest.raises(mp.MypbrError, match=words):
            _texture_scene(tmp_path, str(p))


@pytest.mark.parametrize("name", ["rgb24.bmp", "pal4.bmp", "bgra32.bmp", "rgb8.ppm", "grey16.pgm"])
def test_truncated_bmp_and_pnm_are_rejected(name, tmp_path):
    """Cut inside the pixels: an error (stb_image reads zeros past the end
    of a BMP and rejects a short PGM / PPM)."""
    data = open(os.path.join(IMAGES, name), "rb").read()
    p = tmp_path / ("cut" + os.path.splitext(name)[1])
    p.write_bytes(data[:len(data) - 7])
    with pytest.raises(mp.MypbrError, match="truncated"):
        mp.read_image(str(p))


def test_bmp_headers_that_are_not_images(tmp_path):
    data = bytearray(open(os.path.join(IMAGES, "rgb24.bmp"), "rb").read())
    bad = bytearray(data)
    struct.pack_into("<I", bad, 14, 64)  # no such info header size
    (tmp_path / "h.bmp").write_bytes(bytes(bad))
    with pytest.raises(mp.MypbrError, match="header of 64 bytes"):
        mp.read_image(str(tmp_path / "h.bmp"))
    bad = bytearray(data)
    struct.pack_into("<i", bad, 18, 0)  # zero width
    (tmp_path / "w.bmp").write_bytes(bytes(bad))
    with pytest.raises(mp.MypbrError):
        mp.read_image(str(tmp_path / "w.bmp"))
    (tmp_path / "z.pgm").write_bytes(b"P5\n0 4\n255\n")
    with pytest.raises(mp.MypbrError, match="zero or overflowing width"):
        mp.read_image(str(tmp_path / "z.pgm"))
    (tmp_path / "o.ppm").write_bytes(b"P6\n4 99999999999\n255\n")
    with pytest.raises(mp.MypbrError, match="overflowing height"):
        mp.read_image(str(tmp_path / "o.ppm"))


def test_damaged_and_unsupported_files_are_told_apart(tmp_path):
    """A variant the decoders do not read is MYPBR_ERR_UNSUPPORTED (status 2)
    and says what it is; a damaged file of a format they read is a bad scene
    input (MYPBR_ERR_BAD_SCENE, status 7) with the reason."""
    (tmp_path / "a.psd").write_bytes(b"8BPS" + bytes(40))
    with pytest.raises(mp.MypbrError, match="Photoshop") as e:
        mp.read_image(str(tmp_path / "a.psd"))
    assert e.value.status == 2
    pic = bytearray(120)
    pic[0:4] = b"\x53\x80\xf6\x34"
    pic[88:92] = b"PICT"
    (tmp_path / "a.pic").write_bytes(bytes(pic))
    with pytest.raises(mp.MypbrError, match="Softimage") as e:
        mp.read_image(str(tmp_path / "a.pic"))
    assert e.value.status == 2
    data = open(os.path.join(IMAGES, "rgb24.bmp"), "rb").read()
    (tmp_path / "cut.bmp").write_bytes(data[:80])
    with pytest.raises(mp.MypbrError, match="truncated") as e:
        mp.read_image(str(tmp_path / "cut.bmp"))
    assert e.value.status == 7
    with pytest.raises(mp.MypbrError, match="cannot load image .*truncated") as e:
        _texture_scene(tmp_path, str(tmp_path / "cut.bmp"))
    assert e.value.status == 7


def test_gif_streams_that_are_not_images(tmp_path):
    data = open(os.path.join(IMAGES, "global16.gif"), "rb").read()
    head = data[:13 + 48]  # header and the 16-entry global table
    (tmp_path / "none.gif").write_bytes(head + b"\x3b")
    with pytest.raises(mp.MypbrError, match="no image"):
        mp.read_image(str(tmp_path / "none.gif"))
    (tmp_path / "tag.gif").write_bytes(head + b"\x99")
    with pytest.raises(mp.MypbrError, match="unknown kind"):
        mp.read_image(str(tmp_path / "tag.gif"))
    # an image descriptor reaching past the canvas
    (tmp_path / "rect.gif").write_bytes(head + b"\x2c" + struct.pack("<HHHHB", 5, 0, 13, 7, 0) + b"\x02\x00\x3b")
    with pytest.raises(mp.MypbrError, match="outside the canvas"):
        mp.read_image(str(tmp_path / "rect.gif"))
    # image data whose first code is not the clear code (code size 4: clear = 16)
    (tmp_path / "noclear.gif").write_bytes(head + b"\x2c" + struct.pack("<HHHHB", 0, 0, 13, 7, 0) +
                                           b"\x04\x01\x03\x00\x3b")
    with pytest.raises(mp.MypbrError, match="clear code"):
        mp.read_image(str(tmp_path / "noclear.gif"))


@pytest.mark.parametrize("name", ["argb1555_v5.bmp", "pal8_os2.bmp", "grey8.pgm", "local8_interlaced.gif",
                                  "subrect_background.gif"])
def test_bmp_and_pnm_textures_in_scenes(name, tmp_path):
    sc = _texture_scene(tmp_path, os.path.join(IMAGES, name))
    f = flat.view(sc)
    t = f["textures"][-1]
    meta = _g[name + ":meta"]
    assert t["type"] == 2 and t["width"] == meta[0] and t["height"] == meta[1]
    assert bool(t["flags"] & 8) == (not meta[3])
    n = int(meta[0] * meta[1] * 4)
    np.testing.assert_array_equal(f["texels_ldr"][t["offset"] * 4: t["offset"] * 4 + n],
                                  _g[name + ":rgba"].reshape(-1))


# ------------------------------------------------------------------ MTL


def _mask_scene():
    sc = mp.load_scene(os.path.join(SCENES, "alpha_masks.scene"))
    return sc, flat.view(sc)


def test_mtl_materials_follow_obj_loader():
    sc, f = _mask_scene()
    mats, texs, tris, meshes = f["materials"], f["textures"], f["triangles"], f["meshes"]
    by_first = {int(m["first_triangle"]): m for m in meshes}
    # leaf: lambertian with its diffuse texture, masked by that texture's alpha
    leaf = by_first[0]
    assert mats[leaf["material"]]["type"] == 0
    assert leaf["alpha_mask"] == mats[leaf["material"]]["tex"][0]
    assert np.all(tris["flags"][0:2] & 2)
    assert not texs[leaf["alpha_mask"]]["flags"] & 8  # the alpha channel
    assert texs[leaf["alpha_mask"]]["flags"] & 4      # MTL textures repeat
    # veil: plain Kd, masked by the grey map_d
    veil = by_first[2]
    assert mats[veil["material"]]["type"] == 0
    assert texs[veil["alpha_mask"]]["flags"] & 8
    # glossy: principled, roughness sqrt(sqrt(2 / (Ns + 2))), F0 from Ni, normal map (not the grey bump)
    glossy = mats[by_first[4]["material"]]
    assert glossy["type"] == 4
    rough = texs[glossy["tex"][2]]["p"][0]
    assert rough == pytest.approx(np.sqrt(np.sqrt(2 / 42)), rel=1e-12)
    assert glossy["p"][0] == pytest.approx(((1.45 - 1) / 2.45) ** 2, rel=1e-12)
    nm = texs[glossy["normal_map"]]
    assert nm["flags"] & 2 and nm["width"] == 8  # linear data, ripples.png
    assert by_first[4]["alpha_mask"] == -1
    # lamp: emissive, a light
    lamp = mats[by_first[5]["material"]]
    assert lamp["type"] == 5 and tuple(lamp["p"][:3]) == (4, 3.6, 3)
    # 'wall' is a scene material too: the scene's wins
    assert tuple(texs[mats[by_first[7]["material"]]["tex"][0]]["p"][:3]) == (0.3, 0.3, 0.8)
    # an opaque alpha channel is no mask; an unknown name takes the line's material
    assert not np.any(tris["flags"][7:] & 2)
    fallback = mats[by_first[9]["material"]]
    assert tuple(texs[fallback["tex"][0]]["p"][:3]) == (0.9, 0.9, 0.2)


def test_missing_mtl_is_only_a_warning(tmp_path, capfd):
    (tmp_path / "a.obj").write_text("mtllib none.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nusemtl x\nf 1 2 3\n")
    sc = mp.parse_scene("material m lambertian 0.5 0.5 0.5\nmesh a.obj m\n", str(tmp_path))
    f = flat.view(sc)
    assert len(f["triangles"]) == 1 and f["triangles"]["flags"][0] == 0
    assert "cannot open" in capfd.readouterr().err


def test_unloadable_texture_falls_back_to_color(tmp_path, capfd):
    (tmp_path / "a.mtl").write_text("newmtl x\nKd 0.1 0.2 0.3\nmap_Kd gone.png\n")
    (tmp_path / "a.obj").write_text("mtllib a.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nusemtl x\nf 1 2 3\n")
    f = flat.view(mp.parse_scene("mesh a.obj\n", str(tmp_path)))
    m = f["materials"][f["triangles"]["material"][0]]
    assert tuple(f["textures"][m["tex"][0]]["p"][:3]) == (0.1, 0.2, 0.3)
    assert "cannot load texture" in capfd.readouterr().err


def test_masked_triangles_share_images(tmp_path):
    """One image used by two materials is decoded and stored once."""
    png = open(os.path.join(SCENES, "leaf.png"), "rb").read()
    (tmp_path / "leaf.png").write_bytes(png)
    (tmp_path / "a.mtl").write_text("newmtl x\nmap_Kd leaf.png\nnewmtl y\nKd 1 0 0\nmap_d leaf.png\n")
    (tmp_path / "a.obj").write_text("mtllib a.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 0 1\n"
                                    "usemtl x\nf 1/1 2/2 3/3\nusemtl y\nf 1/1 3/3 2/2\n")
    f = flat.view(mp.parse_scene("mesh a.obj\n", str(tmp_path)))
    assert len(f["texels_ldr"]) == 16 * 16 * 4
    masks = {int(m["alpha_mask"]) for m in f["meshes"]}
    assert len(masks) == 1 and masks.pop() >= 0
