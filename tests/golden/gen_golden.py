"""Writes the golden vectors that pin the oracle to the reference.

Run in a checkout that has the reference (adriendjn/mypbr) at REFERENCE
(default /root/reference). It builds oracle/_ref/ref_harness from the
reference's own headers (oracle/Makefile, target `ref`), runs it on the test
scenes of tests/golden/scenes/, and stores the results as .npz files next to
this script. The tests read only those .npz files, so nothing here runs at test
time or on a machine without the reference.

    python tests/golden/gen_golden.py            # everything
    python tests/golden/gen_golden.py render     # one group
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


# (scene, width, spp per batch, batches)
RENDERS = [
    ("cornell_c1.scene", 64, 64, 16),
    ("env_spheres.scene", 64, 64, 16),
    ("fog_box.scene", 48, 64, 16),
    ("materials.scene", 64, 64, 16),
]


def gen_render():
    threads = os.cpu_count() or 1
    for name, width, spp, batches in RENDERS:
        raw = run("render", scene(name), width, spp, batches, threads)
        w, h, s, b, seconds = raw[:5]
        data = raw[5:].reshape(int(h), int(w), 3, 2)
        stem = name.replace(".scene", "")
        np.savez_compressed(os.path.join(HERE, f"render_{stem}.npz"), mean=data[..., 0].astype(np.float32),
                            var_of_mean=data[..., 1].astype(np.float32), spp=int(s * b), batches=int(b),
                            seconds=float(seconds))
        print(f"{name}: {int(w)}x{int(h)}, {int(s)} spp x {int(b)} batches, {seconds:.1f} s")


GROUPS = {"hits": gen_hits, "bsdf": gen_bsdf, "lights": gen_lights, "env": gen_env, "ggx": gen_ggx,
          "render": gen_render}

if __name__ == "__main__":
    ref = os.environ.get("REFERENCE", "/root/reference")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", f"REFERENCE={ref}"], check=True)
    if not os.path.exists(os.path.join(SCENES, "env_small.hdr")):
        make_env_fixture()
    for g in (sys.argv[1:] or list(GROUPS)):
        GROUPS[g]()
        print("wrote", g)
