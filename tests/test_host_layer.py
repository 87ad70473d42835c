"""The host layer and the C ABI without a GPU: scene parsing semantics and
errors, the flat scene the parser builds, the BVH it builds, and that the
library exports every function include/*.h declares."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import mypbr_gb300 as mp
from conftest import GOLDEN, ROOT, scene_path
from mypbr_gb300 import flat


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(mypbr_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_function():
    names = declared_functions()
    assert "mypbr_gpu_render" in names and "mypbr_scene_load" in names
    lib = ctypes.CDLL(mp.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings():
    L = mp.lib()
    assert L.mypbr_gpu_status_string(0) == b"ok"
    assert L.mypbr_gpu_status_string(2) == b"unsupported feature"
    assert L.mypbr_gpu_status_string(1234) == b"unknown status"


def expect_error(text, status, message):
    with pytest.raises(mp.MypbrError) as e:
        mp.parse_scene(text)
    assert e.value.status == status
    assert message in str(e.value), str(e.value)


def test_scene_errors_name_the_line():
    # the messages of scene.h:244-551 with "path:line:" in front
    expect_error("sphere 0 0 0 1\nfrobnicate 3\n", 7, "<scene text>:2: unknown keyword 'frobnicate'")
    expect_error("material m lambertian 1 1\n", 7, ":1: expected 'material <name> lambertian")
    expect_error("sphere 0 0 0 1 nope\n", 7, ":1: unknown material 'nope'")
    expect_error("sphere 0 0 0 0\n", 7, "non-zero radius")
    expect_error("quad 0 0 0 1 0 0 2 0 0\n", 7, "quad edges must not be parallel")
    expect_error("material l emissive 1 1 1\nsphere 0 0 0 1 l scale 1 2 1\n", 7,
                 "lights can only be moved, rotated and scaled uniformly")
    expect_error("image_width 10\n", 7, "the scene has no objects")
    expect_error("sphere 0 0 0 1\ncamera lookfrom 0 0 0 lookat 0 0 0\n", 7, "camera lookfrom must differ")
    expect_error("sphere 0 0 0 1 translate 1 2\n", 7, "bad values for 'translate'")
    expect_error("sphere 0 0 0 1\nsky uniform 1 1 1\nenvironment x.hdr\n", 7, "cannot load environment map")


def test_unsupported_features_are_reported():
    expect_error("vox island.vox\n", 7, "cannot open")
    expect_error("sphere 0 0 0 1\nsky atmosphere mie_g 1.5\n", 7, "expected 'sky atmosphere")
    expect_error("mesh car.glb\n", 7, "cannot read glTF file")  # gltf_loader.h:65-67
    expect_error("cyclorama 10\n", 2, "not supported by this backend")


def test_missing_file_is_io_error():
    with pytest.raises(mp.MypbrError) as e:
        mp.load_scene("/nonexistent/scene.scene")
    assert e.value.status == 8


def test_camera_defaults_and_settings():
    sc = mp.parse_scene("sphere 0 0 -1 0.5\n")
    cam = sc.camera
    # camera.h:20-56 defaults
    assert cam.image_width == 100 and cam.aspect_ratio == 1.0 and cam.samples_per_pixel == 10
    assert cam.max_depth == 10 and cam.vfov == 90 and cam.lookat == (0, 0, -1) and cam.focus_dist == 10
    sc = mp.parse_scene("image_width 300\naspect_ratio 16/9\nsamples_per_pixel 7\nmax_depth 5\n"
                        "camera lookfrom 1 2 3 lookat 0 0 0 vfov 20 aperture 0.5 focus 3 blades 6\n"
                        "bounces diffuse 2 specular 5 scatter 4\ntransparent_shadows on\nsphere 0 0 0 1\n")
    cam = sc.camera
    assert cam.image_width == 300 and cam.height() == 168
    assert cam.samples_per_pixel == 7 and cam.max_depth == 5 and cam.vfov == 20
    assert cam.defocus_angle == 0.5 and cam.focus_dist == 3 and cam.blades == 6
    assert (cam.max_diffuse, cam.max_specular, cam.max_scatter, cam.transparent_shadows) == (2, 5, 4, 1)


def test_cornell_flat_scene():
    sc = mp.load_scene(scene_path("cornell_c1.scene"))
    v = flat.view(sc)
    assert len(v["quads"]) == 6 + 12 and len(v["spheres"]) == 0
    assert len(v["lights"]) == 1 and v["lights"][0]["probability"] == 1.0
    assert v["use_sky"] == 0 and v["background"] == (0, 0, 0)
    # the rotated boxes are baked: their quads' normals are unit and rotated about y
    n = v["quads"]["normal"]
    np.testing.assert_allclose(np.linalg.norm(n, axis=1), 1, atol=1e-12)
    np.testing.assert_allclose(n[6:, 1] ** 2 + n[6:, 0] ** 2 + n[6:, 2] ** 2, 1, atol=1e-12)


def test_bvh_is_well_formed():
    """Every primitive sits in exactly one leaf, and every node's box holds
    its children's (the reference's layout, bvh.h:93-98)."""
    for name in ("hits_mix", "cornell_c1", "bsdf_probe", "fog_box"):
        v = flat.view(mp.load_scene(scene_path(f"{name}.scene")))
        nodes, prims = v["bvh_nodes"], v["bvh_prims"]
        seen = np.zeros(len(prims), dtype=int)
        stack = [0]
        while stack:
            k = stack.pop()
            n = nodes[k]
            if n["count"] > 0:
                seen[n["offset"]:n["offset"] + n["count"]] += 1
                continue
            for c in (k + 1, n["offset"]):
                assert np.all(nodes[c]["bmin"] >= n["bmin"]) and np.all(nodes[c]["bmax"] <= n["bmax"])
                stack.append(c)
        assert np.all(seen == 1)
        refs = {(int(r["kind"]), int(r["index"])) for r in prims}
        assert len(refs) == len(prims)


def test_mirrored_mesh_flips_geometric_normal():
    v = flat.view(mp.load_scene(scene_path("hits_mix.scene")))
    tris = v["triangles"]
    assert np.any(tris["flags"] == 1) and np.any(tris["flags"] == 0)


def test_light_probabilities_uniform_selection():
    sc = mp.parse_scene("light_selection uniform\nmaterial l emissive 1 1 1\nmaterial b emissive 9 9 9\n"
                        "quad 0 0 0 1 0 0 0 1 0 l\nsphere 0 5 0 1 b\n")
    p = flat.view(sc)["lights"]["probability"]
    np.testing.assert_allclose(p, [0.5, 0.5])


def test_gpu_calls_fail_cleanly_without_a_gpu():
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("a GPU is present")
    sc = mp.parse_scene("sphere 0 0 -1 0.5\n")
    with pytest.raises(mp.MypbrError) as e:
        mp.GpuScene(sc)
    assert e.value.status in (9, 1)


def test_scene_create_rejects_bad_indices():
    """mypbr_gpu_scene_create checks every index on the host before any
    device work (here: a material index out of range)."""
    sc = mp.parse_scene("sphere 0 0 -1 0.5\n")
    fs = flat.FlatScene.from_address(sc.flat)
    bad = flat.FlatScene()
    ctypes.memmove(ctypes.byref(bad), ctypes.byref(fs), ctypes.sizeof(fs))
    spheres = (ctypes.c_char * flat.DTYPES["spheres"].itemsize)()
    arr = np.frombuffer(spheres, dtype=flat.DTYPES["spheres"])
    arr["radius"] = 1.0
    arr["material"] = 99
    arr["xform"] = -1
    bad.spheres = ctypes.addressof(spheres)
    out = ctypes.c_void_p()
    status = mp.lib().mypbr_gpu_scene_create(ctypes.byref(bad), ctypes.byref(out))
    assert status == 5, status  # MYPBR_ERR_INVALID_ARGUMENT, before looking for a device
    assert b"sphere 0 is malformed" in mp.lib().mypbr_last_error()


def test_scene_messages_match_the_reference(tmp_path):
    """Every case of tests/golden/scene_messages.py through the host loader:
    it accepts exactly the cases the reference's load_scene accepts, and for
    the others says what the reference says, byte for byte ("path:line:
    message", with the case's folder written as <dir>/)."""
    import sys
    sys.path.insert(0, GOLDEN)
    from scene_messages import PRELUDE
    g = np.load(os.path.join(GOLDEN, "scene_messages.npz"))
    wrong = []
    for k, (text, want) in enumerate(zip(g["cases"], g["messages"])):
        path = tmp_path / f"case{k}.scene"
        path.write_text(PRELUDE + str(text) + "\n")
        try:
            mp.load_scene(str(path))
            got = "ok"
        except mp.MypbrError as e:
            got = mp.lib().mypbr_last_error().decode().strip().replace(str(tmp_path) + "/", "<dir>/")
        if got != str(want):
            wrong.append((str(text), got, str(want)))
    assert not wrong, "\n".join(f"{t!r}:\n  got  {a}\n  want {b}" for t, a, b in wrong)
