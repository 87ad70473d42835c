"""Writes the golden vectors that pin the oracle to the reference.

Run in a checkout that has the reference (adriendjn/mypbr) where
oracle/Makefile's REFERENCE says (or set REFERENCE). It builds oracle/_ref/ref_harness from the
reference's own headers (oracle/Makefile, target `ref`), runs it on the test
scenes of tests/golden/scenes/, and stores the results as .npz files next to
this script. The tests read only those .npz files, so nothing here runs at test
time or on a machine without the reference.

    python tests/golden/gen_golden.py            # everything
    python tests/golden/gen_golden.py render     # one group
    python tests/golden/gen_golden.py render voxels.scene   # one render
"""
import math
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SCENES = os.path.join(HERE, "scenes")
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def write_hdr(path, rgb):
    """Writes float RGB (H, W, 3) as a flat (uncompressed) Radiance RGBE file."""
    h, w, _ = rgb.shape
    v = rgb.max(axis=2)
    m, e = np.frexp(v)
    scale = np.where(v > 1e-32, m * 256.0 / np.maximum(v, 1e-38), 0.0)
    out = np.zeros((h, w, 4), dtype=np.uint8)
    for c in range(3):
        out[..., c] = np.clip(np.floor(rgb[..., c] * scale), 0, 255).astype(np.uint8)
    out[..., 3] = np.where(v > 1e-32, e + 128, 0).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n")
        f.write(f"-Y {h} +X {w}\n".encode())
        f.write(out.tobytes())


def make_env_fixture():
    """A 64 x 32 sky: a vertical gradient plus a Gaussian sun lobe."""
    w, h = 64, 32
    j, i = np.meshgrid(np.arange(h) + 0.5, np.arange(w) + 0.5, indexing="ij")
    theta = math.pi * j / h
    phi = 2 * math.pi * i / w
    up = np.cos(theta)
    sky = np.stack([0.3 + 0.4 * np.clip(up, 0, 1), 0.4 + 0.4 * np.clip(up, 0, 1), 0.6 + 0.5 * np.clip(up, 0, 1)],
                   axis=2)
    sky[theta > math.pi / 2] *= 0.25
    d = np.stack([np.sin(theta) * np.cos(phi), np.cos(theta), np.sin(theta) * np.sin(phi)], axis=2)
    sun = np.array([math.cos(0.6) * math.cos(1.0), math.sin(0.6), math.cos(0.6) * math.sin(1.0)])
    cosang = np.clip((d * sun).sum(axis=2), -1, 1)
    ang = np.arccos(cosang)
    lobe = 200.0 * np.exp(-0.5 * (ang / 0.08) ** 2)
    rgb = sky + lobe[..., None] * np.array([1.0, 0.9, 0.7])
    write_hdr(os.path.join(SCENES, "env_small.hdr"), rgb.astype(np.float64))


# ------------------------------------------------------------ .vox files
#
# MagicaVoxel's chunk format: "VOX ", version 150, then a MAIN chunk whose
# children are SIZE/XYZI pairs (one per model), an optional RGBA palette,
# MATL dictionaries and the nTRN/nGRP/nSHP scene graph. Each chunk is a 4-byte
# id, the byte sizes of its content and of its children, then both.

def _i32(v):
    return int(v).to_bytes(4, "little", signed=True)


def _vstr(s):
    b = s.encode()
    return _i32(len(b)) + b


def _vdict(d):
    return _i32(len(d)) + b"".join(_vstr(k) + _vstr(v) for k, v in d.items())


def _chunk(cid, content, children=b""):
    return cid.encode() + _i32(len(content)) + _i32(len(children)) + content + children


def write_vox(path, models, rgba=None, materials=None, graph=None):
    """models: uint8 arrays indexed [x, y, z] (palette index, 0 empty); rgba:
    (255, 4) uint8 colours of indices 1..255; materials: {index: {key: value}};
    graph: list of scene graph chunks, made by the helpers below."""
    body = b""
    for m in models:
        nx, ny, nz = m.shape
        xs, ys, zs = np.nonzero(m)
        body += _chunk("SIZE", _i32(nx) + _i32(ny) + _i32(nz))
        cells = np.stack([xs, ys, zs, m[xs, ys, zs]], axis=1).astype(np.uint8)
        body += _chunk("XYZI", _i32(len(cells)) + cells.tobytes())
    for chunk in graph or []:
        body += chunk
    if rgba is not None:
        pal = np.zeros((256, 4), np.uint8)
        pal[:255] = rgba
        body += _chunk("RGBA", pal.tobytes())
    for index, props in (materials or {}).items():
        body += _chunk("MATL", _i32(index) + _vdict(props))
    with open(path, "wb") as f:
        f.write(b"VOX " + _i32(150) + _chunk("MAIN", b"", body))


def vox_transform(node, child, translation=None, rotation=None):
    frame = {}
    if rotation is not None:
        frame["_r"] = str(rotation)
    if translation is not None:
        frame["_t"] = " ".join(str(int(v)) for v in translation)
    return _chunk("nTRN", _i32(node) + _vdict({}) + _i32(child) + _i32(-1) + _i32(0) + _i32(1) + _vdict(frame))


def vox_group(node, children):
    return _chunk("nGRP", _i32(node) + _vdict({}) + _i32(len(children)) + b"".join(_i32(c) for c in children))


def vox_shape(node, model):
    return _chunk("nSHP", _i32(node) + _vdict({}) + _i32(1) + _i32(model) + _vdict({}))


def make_vox_fixtures():
    """voxels.vox: a random 13 x 9 x 11 model of empty, opaque, glass and
    emissive cells with a solid glass corner (the mix of the reference's
    voxel test), plus a 5 x 4 x 3 model placed twice by a scene graph, once
    turned by a rotation byte; its own palette, glass, metal and light
    materials. voxels_default.vox: one model, no palette, no scene graph
    (MagicaVoxel's default palette, the model standing on z = 0)."""
    rng = np.random.default_rng(2024)
    a = np.zeros((13, 9, 11), np.uint8)
    x = rng.random(a.shape)
    pick = rng.random(a.shape)
    a[(x >= 0.55) & (x < 0.8)] = 1 + (pick[(x >= 0.55) & (x < 0.8)] * 2).astype(np.uint8)
    a[(x >= 0.8) & (x < 0.95)] = 3 + (pick[(x >= 0.8) & (x < 0.95)] * 2).astype(np.uint8)
    a[x >= 0.95] = 5
    a[x >= 0.985] = 6
    a[:4, :4, :4] = 3
    b = np.zeros((5, 4, 3), np.uint8)
    b[:, :, 0] = 7
    b[1:4, 1:3, 1] = 8
    b[2, 1, 2] = 2
    rgba = np.zeros((255, 4), np.uint8)
    for k in range(255):  # index k + 1: red steps keep lambertian albedos apart
        rgba[k] = (min(255, 30 + 20 * k), (37 * k) % 256, (91 * k) % 256, 255)
    materials = {3: {"_type": "_glass", "_ior": "0.5", "_rough": "0"},
                 4: {"_type": "_glass", "_ior": "0.45", "_rough": "0.3", "_att": "0.8"},
                 5: {"_type": "_emit", "_emit": "2", "_flux": "0"},
                 6: {"_type": "_metal", "_metal": "1", "_rough": "0.25"}}
    # rotation byte 17: row 0 = -y, row 1 = +x, row 2 = +z (a quarter turn about z)
    graph = [vox_transform(0, 1), vox_group(1, [2, 4, 6]), vox_transform(2, 3, (0, 0, 5)), vox_shape(3, 0),
             vox_transform(4, 5, (12, -2, 1), 17), vox_shape(5, 1), vox_transform(6, 7, (-11, 3, 2)), vox_shape(7, 1)]
    write_vox(os.path.join(SCENES, "voxels.vox"), [a, b], rgba, materials, graph)
    c = np.zeros((6, 5, 4), np.uint8)
    c[:, :, 0] = 1
    c[1:5, 1:4, 1] = 200
    c[2:4, 2, 2:4] = 250
    write_vox(os.path.join(SCENES, "voxels_default.vox"), [c])


def run(*args):
    with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as t:
        out = t.name
    try:
        subprocess.run([HARNESS, *[str(a) for a in args], out], check=True, cwd=SCENES)
        return np.fromfile(out, dtype="<f8")
    finally:
        os.unlink(out)


def scene(name):
    return os.path.join(SCENES, name)


def gen_hits():
    recs = run("hits", scene("hits_mix.scene"), 6000, 12345).reshape(-1, 18)
    np.savez_compressed(os.path.join(HERE, "hits_mix.npz"), o=recs[:, 0:3], d=recs[:, 3:6], hit=recs[:, 6],
                        t=recs[:, 7], normal=recs[:, 8:11], u=recs[:, 11], v=recs[:, 12], front=recs[:, 13],
                        material_id=recs[:, 14], p=recs[:, 15:18])
    recs = run("hits", scene("cornell_c1.scene"), 4000, 777).reshape(-1, 18)
    np.savez_compressed(os.path.join(HERE, "hits_cornell.npz"), o=recs[:, 0:3], d=recs[:, 3:6], hit=recs[:, 6],
                        t=recs[:, 7], normal=recs[:, 8:11], u=recs[:, 11], v=recs[:, 12], front=recs[:, 13],
                        p=recs[:, 15:18])


def gen_bsdf():
    recs = run("bsdf", scene("bsdf_probe.scene")).reshape(-1, 14)
    np.savez_compressed(os.path.join(HERE, "bsdf_probe.npz"), sphere=recs[:, 0].astype(np.int32),
                        face=recs[:, 1].astype(np.int32), wo=recs[:, 2:5], wi=recs[:, 5:8], eval=recs[:, 8:11],
                        pdf=recs[:, 11], skip_pdf=recs[:, 12], scatters=recs[:, 13])


def gen_lights():
    raw = run("lights", scene("lights_mix.scene"), 2000, 99)
    n = int(raw[0])
    prob = raw[1:1 + n]
    recs = raw[1 + n:].reshape(-1, 7)
    np.savez_compressed(os.path.join(HERE, "lights_mix.npz"), probability=prob, origin=recs[:, 0:3],
                        dir=recs[:, 3:6], pdf=recs[:, 6])


def gen_env():
    recs = run("env", scene("env_spheres.scene"), 2000, 5).reshape(-1, 7)
    np.savez_compressed(os.path.join(HERE, "env_small.npz"), dir=recs[:, 0:3], radiance=recs[:, 3:6],
                        pdf=recs[:, 6])


def gen_ggx():
    recs = run("ggx").reshape(-1, 6)
    np.savez_compressed(os.path.join(HERE, "ggx_table.npz"), alpha=recs[:, 0], mu=recs[:, 1], E=recs[:, 2],
                        E_avg=recs[:, 3], ms_albedo=recs[:, 4], ms_eval=recs[:, 5])


def gen_voxels():
    recs = run("hits", scene("voxels.scene"), 8000, 4242).reshape(-1, 18)
    np.savez_compressed(os.path.join(HERE, "hits_voxels.npz"), o=recs[:, 0:3], d=recs[:, 3:6], hit=recs[:, 6],
                        t=recs[:, 7], normal=recs[:, 8:11], u=recs[:, 11], v=recs[:, 12], front=recs[:, 13],
                        material_id=recs[:, 14], p=recs[:, 15:18])


# (scene, width, spp per batch, batches)
RENDERS = [
    ("cornell_c1.scene", 64, 64, 16),
    ("env_spheres.scene", 64, 64, 16),
    ("fog_box.scene", 48, 64, 16),
    ("materials.scene", 64, 64, 16),
    ("voxels.scene", 48, 64, 16),
    ("voxels_style.scene", 48, 64, 16),
    ("alpha_masks.scene", 48, 64, 16),
    ("gallery.scene", 48, 64, 16),
    ("defocus_bokeh.scene", 64, 64, 32),
    ("ortho.scene", 64, 64, 32),
    ("checker.scene", 64, 64, 32),
]


def gen_render(only=None):
    threads = os.cpu_count() or 1
    for name, width, spp, batches in RENDERS:
        if only and name not in only:
            continue
        raw = run("render", scene(name), width, spp, batches, threads)
        w, h, s, b, seconds = raw[:5]
        data = raw[5:].reshape(int(h), int(w), 3, 2)
        stem = name.replace(".scene", "")
        np.savez_compressed(os.path.join(HERE, f"render_{stem}.npz"), mean=data[..., 0].astype(np.float32),
                            var_of_mean=data[..., 1].astype(np.float32), spp=int(s * b), batches=int(b),
                            seconds=float(seconds))
        print(f"{name}: {int(w)}x{int(h)}, {int(s)} spp x {int(b)} batches, {seconds:.1f} s")


# The benchmark configurations at test size (config_scenes.py): (name, spp per
# batch, batches). Their scenes are generated into a scratch folder, rendered
# there, and only the images and the inputs' digest are kept.
CONFIG_RENDERS = [("c2", 64, 64), ("c3", 64, 32), ("c5", 256, 64)]


def gen_configs(only=None):
    sys.path.insert(0, HERE)
    import config_scenes
    threads = os.cpu_count() or 1
    for name, spp, batches in CONFIG_RENDERS:
        if only and name not in only:
            continue
        with tempfile.TemporaryDirectory() as tmp:
            path, digest = config_scenes.CONFIGS[name](tmp)
            raw = run("render", path, 0, spp, batches, threads)
        w, h, s, b, seconds = raw[:5]
        data = raw[5:].reshape(int(h), int(w), 3, 2)
        np.savez_compressed(os.path.join(HERE, f"render_{name}.npz"), mean=data[..., 0].astype(np.float32),
                            var_of_mean=data[..., 1].astype(np.float32), spp=int(s * b), batches=int(b),
                            seconds=float(seconds), digest=digest)
        print(f"{name}: {int(w)}x{int(h)}, {int(s)} spp x {int(b)} batches, {seconds:.1f} s")


# (scene, width, spp per batch, batches) of the feature-buffer goldens
FEATURES = [("materials.scene", 48, 64, 32), ("cornell_c1.scene", 32, 64, 32)]


def gen_features():
    """camera::render with collect_features: radiance, first_surface albedo and
    normal (camera.h:253-277) and the luminance variance buffer."""
    threads = os.cpu_count() or 1
    for name, width, spp, batches in FEATURES:
        raw = run("features", scene(name), width, spp, batches, threads)
        w, h = int(raw[0]), int(raw[1])
        recs = raw[4:].reshape(h, w, 19)
        mv = recs[..., :18].reshape(h, w, 3, 3, 2)  # quantity, channel, (mean, var of mean)
        np.savez_compressed(os.path.join(HERE, f"features_{name.replace('.scene', '')}.npz"),
                            radiance=mv[:, :, 0, :, 0], radiance_var=mv[:, :, 0, :, 1], albedo=mv[:, :, 1, :, 0],
                            albedo_var=mv[:, :, 1, :, 1], normal=mv[:, :, 2, :, 0], normal_var=mv[:, :, 2, :, 1],
                            variance=recs[..., 18], spp=int(raw[2]), batches=int(raw[3]))
        print(f"features {name}: {w}x{h}")


def gen_denoise():
    raw = run("denoise", 64, 48, 21)
    w, h = int(raw[0]), int(raw[1])
    recs = raw[2:].reshape(h, w, 13)
    np.savez_compressed(os.path.join(HERE, "denoise.npz"), radiance=recs[..., 0:3], albedo=recs[..., 3:6],
                        normal=recs[..., 6:9], variance=recs[..., 9], out=recs[..., 10:13])


# display settings of ref_harness post: (exposure, tonemap, bloom, threshold, radius, vignette)
POST_SETTINGS = [(0.0, 0, 0.0, 1.0, 0.04, 0.0), (0.5, 1, 0.3, 1.0, 0.08, 0.4), (-0.7, 2, 0.8, 0.5, 0.2, 0.0),
                 (1.3, 0, 0.15, 2.0, 0.01, 1.5)]


def gen_post():
    raw = run("post", 97, 61, 8)
    w, h = int(raw[0]), int(raw[1])
    n = w * h
    img = raw[2:2 + 3 * n].reshape(h, w, 3)
    rest = raw[2 + 3 * n:].reshape(len(POST_SETTINGS), 2, h, w, 3)
    np.savez_compressed(os.path.join(HERE, "post.npz"), image=img, linear=rest[:, 0],
                        rgb8=rest[:, 1].astype(np.uint8), settings=np.array(POST_SETTINGS))


# (elevation, azimuth, irradiance, rayleigh, mie, mie_g, ozone, intensity) of ref_harness sky
SKY_CASES = [(40, 160, 1000, 1, 1, 0.8, 1, 3), (5, 60, 4, 1, 1, 0.8, 1, 3), (-2, 250, 10, 1, 1, 0.8, 1, 3),
             (25, 300, 3, 1.5, 4, 0.9, 0, 2)]


def gen_sky():
    w, h = 64, 32
    raw = run("sky", w, h).reshape(len(SKY_CASES), -1)
    np.savez_compressed(os.path.join(HERE, "sky.npz"), bake=raw[:, :-3].reshape(len(SKY_CASES), h, w, 3),
                        sun_transmittance=raw[:, -3:], cases=np.array(SKY_CASES, dtype=float))
    recs = run("lights", scene("voxels_style.scene"), 1500, 31)
    n = int(recs[0])
    np.savez_compressed(os.path.join(HERE, "lights_style.npz"), probability=recs[1:1 + n],
                        origin=recs[1 + n:].reshape(-1, 7)[:, 0:3], dir=recs[1 + n:].reshape(-1, 7)[:, 3:6],
                        pdf=recs[1 + n:].reshape(-1, 7)[:, 6])


def make_mask_fixtures():
    """The textures of masks.mtl (alpha_masks.scene)."""
    sys.path.insert(0, HERE)
    from image_fixtures import write_png, write_tga
    n = 16
    y, x = np.mgrid[0:n, 0:n]
    r = np.hypot(x - 7.5, y - 7.5)
    leaf = np.zeros((n, n, 4), dtype=np.int64)
    leaf[..., 0] = 40 + 8 * x
    leaf[..., 1] = 150 + 4 * y
    leaf[..., 2] = 60
    leaf[..., 3] = np.where(r < 5, 255, np.where(r < 7, 128, 0))  # solid disk, half-covered ring, holes
    write_png(os.path.join(SCENES, "leaf.png"), leaf, 6, 8)
    veil = (x * 255 // (n - 1))[..., None]  # coverage 0 at the left edge to 1 at the right
    write_png(os.path.join(SCENES, "veil.png"), veil, 0, 8)
    paint = np.zeros((8, 8, 4), dtype=np.uint8)
    yy, xx = np.mgrid[0:8, 0:8]
    paint[..., 0] = np.where((xx + yy) % 2 == 0, 220, 30)
    paint[..., 1] = 90
    paint[..., 2] = np.where((xx + yy) % 2 == 0, 40, 200)
    paint[..., 3] = 255
    write_tga(os.path.join(SCENES, "paint.tga"), paint, 2, 24)
    tilt = np.zeros((8, 8, 3), dtype=np.int64)
    tilt[..., 0] = np.where(xx < 4, 170, 90)
    tilt[..., 1] = 128
    tilt[..., 2] = 235
    write_png(os.path.join(SCENES, "ripples.png"), tilt, 2, 8)
    write_png(os.path.join(SCENES, "height.png"), ((xx * 30) % 256)[..., None], 0, 8)
    opaque = np.zeros((4, 4, 4), dtype=np.int64)
    opaque[..., 0] = 200
    opaque[..., 1] = 180
    opaque[..., 2] = 40
    opaque[..., 3] = 255
    write_png(os.path.join(SCENES, "opaque_alpha.png"), opaque, 6, 8)


def gen_gltf():
    """world.hit on the glTF gallery (every hit deterministic: the partial-coverage veil replaced)."""
    recs = run("hits", scene("gallery_hits.scene"), 6000, 31337).reshape(-1, 18)
    np.savez_compressed(os.path.join(HERE, "hits_gallery.npz"), o=recs[:, 0:3], d=recs[:, 3:6], hit=recs[:, 6],
                        t=recs[:, 7], normal=recs[:, 8:11], u=recs[:, 11], v=recs[:, 12], front=recs[:, 13],
                        p=recs[:, 15:18])


def gen_images():
    """stb_image's decoding (through image_texture) of every image fixture."""
    sys.path.insert(0, HERE)
    from image_fixtures import make_image_fixtures
    from jpeg_fixtures import make_jpeg_fixtures
    folder = os.path.join(HERE, "images")
    names = make_image_fixtures(folder) + make_jpeg_fixtures(folder)
    out = {}
    for name in names:
        raw = run("image", os.path.join(folder, name))
        if raw[0] < 0:
            raise RuntimeError(f"stb_image cannot decode {name}")
        w, h = int(raw[0]), int(raw[1])
        out[name + ":meta"] = raw[:6].astype(np.int32)
        out[name + ":rgba"] = raw[6:].astype(np.uint8).reshape(h, w, 4)
    np.savez_compressed(os.path.join(HERE, "images.npz"), **out)


def gen_messages():
    """load_scene's outcome on every case of scene_messages.py: "ok" or the
    message it prints, with the case file's folder written as <dir>/."""
    sys.path.insert(0, HERE)
    from scene_messages import CASES, PRELUDE
    out = []
    with tempfile.TemporaryDirectory() as tmp:
        for k, text in enumerate(CASES):
            path = os.path.join(tmp, f"case{k}.scene")
            with open(path, "w") as f:
                f.write(PRELUDE + text + "\n")
            result = os.path.join(tmp, "result.txt")
            subprocess.run([HARNESS, "load", path, result], check=True)
            msg = open(result).read().strip().replace(tmp + "/", "<dir>/")
            out.append(msg)
    np.savez_compressed(os.path.join(HERE, "scene_messages.npz"), cases=np.array(CASES), messages=np.array(out))
    print(f"{len(out)} scene messages")


GROUPS = {"hits": gen_hits, "bsdf": gen_bsdf, "lights": gen_lights, "env": gen_env, "ggx": gen_ggx,
          "render": gen_render, "denoise": gen_denoise, "voxels": gen_voxels, "post": gen_post, "sky": gen_sky,
          "images": gen_images, "gltf": gen_gltf, "configs": gen_configs, "features": gen_features,
          "messages": gen_messages}

if __name__ == "__main__":
    overrides = [f"REFERENCE={os.environ['REFERENCE']}"] if "REFERENCE" in os.environ else []
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", *overrides], check=True)
    if not os.path.exists(os.path.join(SCENES, "env_small.hdr")):
        make_env_fixture()
    if not os.path.exists(os.path.join(SCENES, "voxels.vox")):
        make_vox_fixtures()
    if not os.path.exists(os.path.join(SCENES, "leaf.png")):
        make_mask_fixtures()
    if not os.path.exists(os.path.join(SCENES, "gallery.glb")):
        sys.path.insert(0, HERE)
        from gltf_fixtures import make_gltf_fixtures
        make_gltf_fixtures(SCENES)
    args = sys.argv[1:]
    if args[:1] == ["render"] and len(args) > 1:  # render <scene> ...: only those renders
        gen_render(args[1:])
        args = []
    elif args[:1] == ["configs"] and len(args) > 1:  # configs c2 ...: only those
        gen_configs(args[1:])
        args = []
    elif not args:
        args = list(GROUPS)
    for g in args:
        GROUPS[g]()
        print("wrote", g)
