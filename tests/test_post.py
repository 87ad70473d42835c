"""Display post-processing and image writers.

CPU: the numpy oracle (oracle/post_oracle.py) against the reference's own
post-processed radiance and display bytes (tests/golden/post.npz, written by
ref_harness post through postprocess.h, tonemap.h and color3.h).
GPU: mypbr_gpu_display against the same goldens, and the writers' files
decoded back.
"""
import struct
import zlib

import numpy as np
import pytest

import mypbr_gb300 as mp
import post_oracle as po
from conftest import GOLDEN

G = np.load(f"{GOLDEN}/post.npz")


def settings(k):
    exp, tm, bloom, thr, rad, vig = G["settings"][k]
    return float(exp), int(tm), float(bloom), float(thr), float(rad), float(vig)


@pytest.mark.parametrize("k", range(4))
def test_oracle_matches_reference_bytes(k):
    exp, tm, bloom, thr, rad, vig = settings(k)
    lin = po.postprocess(G["image"], bloom, thr, rad, vig)
    np.testing.assert_array_equal(lin, G["linear"][k])
    np.testing.assert_array_equal(po.to_byte(po.apply(lin, exp, tm)), G["rgb8"][k])


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(4))
def test_gpu_display_matches_reference(k):
    exp, tm, bloom, thr, rad, vig = settings(k)
    o = mp.display_opts(exp, tm, bloom, thr, rad, vig)
    lin, rgb = mp.display(G["image"], o)
    # FP64 in the reference's order without FMA contraction: identical sums;
    # only pow() may differ in the last bit
    np.testing.assert_allclose(lin, G["linear"][k], rtol=1e-15, atol=1e-300)
    diff = rgb.astype(int) - G["rgb8"][k].astype(int)
    assert np.abs(diff).max() <= 1 and (diff != 0).mean() < 1e-4, (np.abs(diff).max(), (diff != 0).mean())


def read_png(path):
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        crc = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        assert crc == zlib.crc32(typ + body) & 0xffffffff
        if typ == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
            assert body[8:10] == b"\x08\x02"
        elif typ == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = np.frombuffer(raw, np.uint8).reshape(h, 3 * w + 1)
    assert np.all(rows[:, 0] == 0)
    return rows[:, 1:].reshape(h, w, 3)


def read_hdr(path):
    data = open(path, "rb").read()
    head, _, rest = data.partition(b"\n\n")
    res, _, pix = rest.partition(b"\n")
    _, h, _, w = res.split()
    rgbe = np.frombuffer(pix, np.uint8).reshape(int(h), int(w), 4).astype(np.float64)
    e = rgbe[..., 3]
    scale = np.where(e > 0, np.ldexp(1.0, (e - 136).astype(int)), 0.0)
    return rgbe[..., :3] * scale[..., None]


@pytest.mark.gpu
def test_writers_round_trip(tmp_path):
    exp, tm, bloom, thr, rad, vig = settings(1)
    o = mp.display_opts(exp, tm, bloom, thr, rad, vig)
    img = G["image"]
    mp.write_image(tmp_path / "a.png", img, o)
    np.testing.assert_array_equal(read_png(tmp_path / "a.png"), mp.display(img, o)[1])
    mp.write_image(tmp_path / "a.ppm", img, o)
    tok = open(tmp_path / "a.ppm").read().split()
    assert tok[:4] == ["P3", "97", "61", "255"]
    np.testing.assert_array_equal(np.array(tok[4:], int).reshape(61, 97, 3), mp.display(img, o)[1])
    mp.write_image(tmp_path / "a.pfm", img)
    raw = open(tmp_path / "a.pfm", "rb").read()
    assert raw.startswith(b"PF\n97 61\n-1.0\n")
    pfm = np.frombuffer(raw[len(b"PF\n97 61\n-1.0\n"):], "<f4").reshape(61, 97, 3)[::-1]
    np.testing.assert_array_equal(pfm, img.astype(np.float32))
    mp.write_image(tmp_path / "a.hdr", img)
    back = read_hdr(tmp_path / "a.hdr")
    assert np.all(np.abs(back - img) <= img.max(axis=2, keepdims=True) / 128 + 1e-30)
    with pytest.raises(mp.MypbrError):
        mp.write_image(tmp_path / "a.jpg", img)
