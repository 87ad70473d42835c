"""Damaged inputs: the image decoders, the glTF reader and the scene parser
must turn corrupted files into errors, never crashes (seeded mutations of the
fixtures: overwritten bytes, truncation, inserted bytes). The same mutations
were run at scale under AddressSanitizer / UBSan while writing the readers."""
import os
import random

import pytest

import mypbr_gb300 as mp

HERE = os.path.dirname(os.path.abspath(__file__))
IMAGES = os.path.join(HERE, "golden", "images")
SCENES = os.path.join(HERE, "golden", "scenes")


def mutate(data, rng):
    data = bytearray(data)
    kind = rng.random()
    if kind < 0.4:
        for _ in range(rng.randint(1, 8)):
            data[rng.randrange(len(data))] = rng.randrange(256)
    elif kind < 0.7:
        data = data[: rng.randrange(1, len(data))]
    else:
        i = rng.randrange(len(data))
        data[i:i] = bytes(rng.randrange(256) for _ in range(rng.randint(1, 40)))
    return bytes(data)


def test_damaged_images(tmp_path):
    rng = random.Random(11)
    names = sorted(os.listdir(IMAGES))
    outcomes = {"ok": 0, "error": 0}
    for it in range(400):
        name = rng.choice(names)
        p = tmp_path / f"m{it}{os.path.splitext(name)[1]}"
        p.write_bytes(mutate(open(os.path.join(IMAGES, name), "rb").read(), rng))
        try:
            img, c = mp.read_image(str(p))
            assert img.ndim == 3 and img.shape[2] == 4 and 1 <= c <= 4
            outcomes["ok"] += 1
        except mp.MypbrError:
            outcomes["error"] += 1
    assert outcomes["error"] > 0 and outcomes["ok"] > 0


@pytest.mark.parametrize("name", ["gallery.glb", "gallery.gltf"])
def test_damaged_gltf(tmp_path, name):
    rng = random.Random(5)
    for f in os.listdir(SCENES):
        if f.startswith("gallery_") and f.endswith(".png"):
            (tmp_path / f).write_bytes(open(os.path.join(SCENES, f), "rb").read())
    src = open(os.path.join(SCENES, name), "rb").read()
    for it in range(150):
        p = tmp_path / f"m{it}{os.path.splitext(name)[1]}"
        p.write_bytes(mutate(src, rng))
        try:
            mp.parse_scene(f"mesh {p.name}\n", str(tmp_path))
        except mp.MypbrError:
            pass


def test_damaged_scene_text():
    rng = random.Random(9)
    texts = [open(os.path.join(SCENES, n)).read() for n in ("materials.scene", "alpha_masks.scene", "hits_mix.scene")]
    alphabet = "0123456789 .-e\nabcdefghijklmnopqrstuvwxyz/"
    for _ in range(300):
        t = list(rng.choice(texts))
        for _ in range(rng.randint(1, 6)):
            i = rng.randrange(len(t))
            r = rng.random()
            if r < 0.4:
                t[i] = rng.choice(alphabet)
            elif r < 0.7:
                del t[i:i + rng.randint(1, 10)]
            else:
                t.insert(i, rng.choice(alphabet))
        try:
            mp.parse_scene("".join(t), SCENES)
        except mp.MypbrError:
            pass
