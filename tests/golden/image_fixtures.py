"""Small PNG and TGA writers for the image-decoding fixtures.

Every PNG color type and bit depth (grey 1/2/4/8/16, RGB 8/16, palette
1/2/4/8, grey + alpha 8/16, RGBA 8/16), tRNS keys and palette alphas, Adam7
interlacing, all five scanline filters and stored / fixed / dynamic deflate
blocks; TGA true color (15/16, 24, 32 bit), grey and color-mapped images,
plain and run-length coded, bottom-up and top-down; BMP through every header
size (OS/2, 40, 56, v4, v5) at 1/4/8 bits through a palette, 16 bits 5-5-5 and
5-6-5, 24 bits, 32 bits with and without alpha (an all-zero alpha channel
included), bottom-up and top-down; binary PGM / PPM at 8 and 16 bits with
header comments; GIF with global and local tables, interlacing, transparency,
a background around a smaller image, indices past the table, full code tables
and a file cut inside its image data. The pixel values are seeded, so the
files are reproducible.
"""
import os
import struct
import zlib

import numpy as np

ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


def _chunk(kind, data):
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


def _pack_row(samples, depth):
    if depth == 8:
        return bytes(int(s) for s in samples)
    if depth == 16:
        return b"".join(struct.pack(">H", int(s)) for s in samples)
    out, acc, used = bytearray(), 0, 0
    for s in samples:
        acc = (acc << depth) | int(s)
        used += depth
        if used == 8:
            out.append(acc)
            acc, used = 0, 0
    if used:
        out.append(acc << (8 - used))
    return bytes(out)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _filter(kind, row, prev, bpp):
    out = bytearray([kind])
    for i, x in enumerate(row):
        a = row[i - bpp] if i >= bpp else 0
        b = prev[i]
        c = prev[i - bpp] if i >= bpp else 0
        pred = [0, a, b, (a + b) // 2, _paeth(a, b, c)][kind]
        out.append((x - pred) & 255)
    return bytes(out)


def write_png(path, samples, ctype, depth, palette=None, trns=None, interlace=False, level=6):
    """samples: (H, W, channels) integers at the file's depth (palette indices for ctype 3)."""
    h, w = samples.shape[:2]
    ch = CHANNELS[ctype]
    bpp = max(1, ch * depth // 8)
    raw = bytearray()
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    for p, (x0, y0, dx, dy) in enumerate(passes):
        sub = samples[y0::dy, x0::dx]
        if sub.shape[0] == 0 or sub.shape[1] == 0:
            continue
        prev = bytes(len(_pack_row(sub[0].reshape(-1), depth)))
        for y in range(sub.shape[0]):
            row = _pack_row(sub[y].reshape(-1), depth)
            raw += _filter((y + p) % 5, row, prev, bpp)
            prev = row
    data = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    if palette is not None:
        data += _chunk(b"PLTE", bytes(np.asarray(palette, dtype=np.uint8).reshape(-1)))
    if trns is not None:
        data += _chunk(b"tRNS", bytes(trns))
    comp = zlib.compress(bytes(raw), level)
    # two IDAT chunks: the stream may be split anywhere
    half = len(comp) // 2
    data += _chunk(b"IDAT", comp[:half]) + _chunk(b"IDAT", comp[half:]) + _chunk(b"IEND", b"")
    with open(path, "wb") as f:
        f.write(data)


def _tga_pixels(rgba, bits):
    """Pixel bytes of a TGA true-color / grey image, from RGBA rows (bottom row first handled by caller)."""
    px = []
    for r, g, b, a in rgba.reshape(-1, 4):
        if bits == 32:
            px.append(bytes([b, g, r, a]))
        elif bits == 24:
            px.append(bytes([b, g, r]))
        elif bits in (15, 16):
            v = ((int(r) >> 3) << 10) | ((int(g) >> 3) << 5) | (int(b) >> 3)
            px.append(struct.pack("<H", v))
        else:
            px.append(bytes([r]))
    return px


def _rle(px):
    out, i = bytearray(), 0
    while i < len(px):
        run = 1
        while i + run < len(px) and run < 128 and px[i + run] == px[i]:
            run += 1
        if run >= 2:
            out.append(0x80 | (run - 1))
            out += px[i]
            i += run
            continue
        j = i + 1
        while j < len(px) and j - i < 128 and not (j + 1 < len(px) and px[j + 1] == px[j]):
            j += 1
        out.append(j - i - 1)
        for k in range(i, j):
            out += px[k]
        i = j
    return bytes(out)


def write_tga(path, rgba, kind, bits, top_first=False, rle=False, palette=None, image_id=b""):
    """rgba: (H, W, 4) bytes; kind 1 (color-mapped: rgba holds indices in channel 0), 2 (true color), 3 (grey)."""
    h, w = rgba.shape[:2]
    rows = rgba if top_first else rgba[::-1]
    if kind == 1:
        px = [bytes([int(i)]) for i in rows[..., 0].reshape(-1)]
        pal = b"".join(bytes([b, g, r]) for r, g, b in np.asarray(palette, dtype=np.uint8))
        cmap = (1, 0, len(palette), 24)
        depth = 8
    else:
        px = _tga_pixels(rows, bits)
        pal = b""
        cmap = (0, 0, 0, 0)
        depth = bits
    alpha_bits = 8 if bits == 32 else (1 if bits == 16 else 0)
    desc = alpha_bits | (0x20 if top_first else 0)
    head = struct.pack("<BBBHHBHHHHBB", len(image_id), cmap[0], kind + (8 if rle else 0), cmap[1], cmap[2],
                       cmap[3], 0, 0, w, h, depth, desc)
    body = _rle(px) if rle else b"".join(px)
    with open(path, "wb") as f:
        f.write(head + image_id + pal + body + b"\0" * 8 + b"TRUEVISION-XFILE.\0")


def _bmp_masks_pixel(px, masks):
    """Packs integer channel values (already at each field's width) into one word."""
    v = 0
    for c, m in zip(px, masks):
        if m:
            shift = (m & -m).bit_length() - 1
            v |= (int(c) << shift) & m
    return v


def write_bmp(path, pixels, bpp, hsz=40, palette=None, masks=None, compress=None, top_down=False, gap=0):
    """A BMP file: `pixels` (h, w) palette indices for bpp <= 8, else (h, w, c)
    channel values at the widths of `masks` (r, g, b, a) for 16 / 32 bits, or
    BGR-ready RGB bytes for 24 bits. `gap` bytes of padding sit between the
    header (+ palette) and the pixels."""
    h, w = pixels.shape[:2]
    if compress is None:
        compress = 3 if masks is not None and hsz in (40, 56, 108, 124) and bpp in (16, 32) else 0
    rows = []
    for y in (range(h) if top_down else range(h - 1, -1, -1)):
        row = bytearray()
        if bpp <= 8:
            acc, used = 0, 0
            for x in range(w):
                acc = (acc << bpp) | int(pixels[y, x])
                used += bpp
                if used == 8:
                    row.append(acc)
                    acc, used = 0, 0
            if used:
                row.append(acc << (8 - used))
        elif bpp == 24:
            for x in range(w):
                r, g, b = (int(c) for c in pixels[y, x, :3])
                row += bytes([b, g, r])
        else:
            for x in range(w):
                v = _bmp_masks_pixel(pixels[y, x], masks)
                row += struct.pack("<H" if bpp == 16 else "<I", v)
        row += bytes((-len(row)) % 4)
        rows.append(bytes(row))
    pal = b""
    if palette is not None:
        pal = b"".join(bytes([int(c[2]), int(c[1]), int(c[0])]) + (b"" if hsz == 12 else b"\0") for c in palette)
    if hsz == 12:
        info = struct.pack("<IHHHH", 12, w, h, 1, bpp)
    else:
        info = struct.pack("<IiiHHIIiiII", hsz, w, -h if top_down else h, 1, bpp, compress, 0, 2835, 2835,
                           len(palette) if palette is not None else 0, 0)
        if hsz == 56:
            m = list(masks or (0, 0, 0, 0))
            info += struct.pack("<IIII", *m)
        elif hsz in (108, 124):
            m = list(masks or (0, 0, 0, 0))
            info += struct.pack("<IIII", *m) + b"BGRs" + bytes(48)
            if hsz == 124:
                info += bytes(16)
    extra = b""
    if hsz in (40, 56) and compress == 3:  # stb reads these three after a 56-byte header too
        extra = struct.pack("<III", *masks[:3])
    offset = 14 + len(info) + len(extra) + len(pal) + gap
    body = b"".join(rows)
    head = b"BM" + struct.pack("<IHHI", offset + len(body), 0, 0, offset)
    with open(path, "wb") as f:
        f.write(head + info + extra + pal + bytes(gap) + body + bytes(gap))


def write_pnm(path, samples, maxv, comment=False):
    """Binary PGM (h, w) or PPM (h, w, 3), big-endian samples above 255."""
    h, w = samples.shape[:2]
    kind = b"P6" if samples.ndim == 3 else b"P5"
    head = kind + (b"\n# a comment line\n" if comment else b"\n") + f"{w} {h}\n{maxv}\n".encode()
    data = samples.astype(">u2" if maxv > 255 else "u1").tobytes()
    with open(path, "wb") as f:
        f.write(head + data)


def _gif_lzw(indices, min_size):
    """GIF LZW code stream of the index list, as data sub-blocks: a clear code
    first, code width growing with the table, a clear code whenever the
    table is full, the end code last."""
    clear, end = 1 << min_size, (1 << min_size) + 1
    out, acc, used = bytearray(), 0, 0
    size = min_size + 1

    def put(code):
        nonlocal acc, used
        acc |= code << used
        used += size
        while used >= 8:
            out.append(acc & 255)
            acc >>= 8
            used -= 8

    def reset():
        return {(i,): i for i in range(clear)}, end + 1

    table, nxt = reset()
    put(clear)
    w = (int(indices[0]),)
    for k in indices[1:]:
        wk = w + (int(k),)
        if wk in table:
            w = wk
            continue
        put(table[w])
        if nxt < 4096:
            table[wk] = nxt
            nxt += 1
            if nxt > (1 << size) and size < 12:
                size += 1
        else:
            put(clear)
            table, nxt = reset()
            size = min_size + 1
        w = (int(k),)
    put(table[w])
    put(end)
    if used:
        out.append(acc & 255)
    blocks = bytearray()
    for i in range(0, len(out), 255):
        chunk = out[i:i + 255]
        blocks += bytes([len(chunk)]) + chunk
    return bytes([min_size]) + bytes(blocks) + b"\0"


def write_gif(path, indices, palette, canvas=None, offset=(0, 0), local=False, interlace=False, transparent=None,
              background=0, version=b"89a", comment=False, cut=None, min_size=None):
    """A one-image GIF: `indices` (h, w) into `palette` (entries a power of two,
    2..256), drawn at `offset` on a canvas (w, h) (the image's size by
    default), with the table global or local, optionally interlaced, with a
    transparent index (graphic control extension) and a background index;
    `cut` keeps only that many leading bytes."""
    h, w = indices.shape
    cw, ch = canvas or (w, h)
    bits = max(1, (len(palette) - 1).bit_length())
    table = b"".join(bytes([int(c[0]), int(c[1]), int(c[2])]) for c in palette)
    table += bytes(3 * ((1 << bits) - len(palette)))
    gflags = 0 if local else 0x80 | (bits - 1)
    data = b"GIF" + version + struct.pack("<HHBBB", cw, ch, gflags, background, 0)
    if not local:
        data += table
    if comment:
        data += b"\x21\xfe" + bytes([9]) + b"a fixture" + b"\0"
    if transparent is not None:
        data += b"\x21\xf9\x04" + struct.pack("<BHB", 1, 0, transparent) + b"\0"
    lflags = (0x80 | (bits - 1) if local else 0) | (0x40 if interlace else 0)
    data += b"\x2c" + struct.pack("<HHHHB", offset[0], offset[1], w, h, lflags)
    if local:
        data += table
    rows = list(range(h))
    if interlace:
        rows = [y for start, step in ((0, 8), (4, 8), (2, 4), (1, 2)) for y in range(start, h, step)]
    order = np.concatenate([indices[y] for y in rows])
    data += _gif_lzw(order, max(2, bits) if min_size is None else min_size) + b"\x3b"
    if cut is not None:
        data = data[:cut]
    with open(path, "wb") as f:
        f.write(data)


def make_image_fixtures(folder):
    """Writes the fixture set into folder; returns the file names."""
    os.makedirs(folder, exist_ok=True)
    rng = np.random.default_rng(2024)
    names = []
    w, h = 13, 7  # odd sizes: partial bytes at low depths, empty Adam7 passes

    def grad(maxv, ch):
        y, x = np.mgrid[0:h, 0:w]
        base = np.stack([(x * 7 + y * 3 + c * 5) % (maxv + 1) for c in range(ch)], axis=-1)
        noise = rng.integers(0, maxv + 1, size=(h, w, ch))
        pick = rng.random((h, w, 1)) < 0.3
        return np.where(pick, noise, base)

    def png(name, *args, **kw):
        write_png(os.path.join(folder, name), *args, **kw)
        names.append(name)

    for depth in (1, 2, 4, 8, 16):
        png(f"grey{depth}.png", grad((1 << depth) - 1, 1), 0, depth)
    png("grey8_key.png", grad(255, 1), 0, 8, trns=struct.pack(">H", 21))
    png("grey4_key_interlaced.png", grad(15, 1), 0, 4, trns=struct.pack(">H", 3), interlace=True)
    png("rgb8.png", grad(255, 3), 2, 8)
    png("rgb16.png", grad(65535, 3), 2, 16)
    rgb = grad(255, 3)
    rgb[2, 3] = rgb[5, 9] = (10, 20, 30)
    png("rgb8_key.png", rgb, 2, 8, trns=struct.pack(">HHH", 10, 20, 30))
    for depth in (1, 2, 4, 8):
        n = 1 << depth
        pal = rng.integers(0, 256, size=(n, 3))
        png(f"palette{depth}.png", grad(n - 1, 1), 3, depth, palette=pal)
    pal = rng.integers(0, 256, size=(16, 3))
    png("palette4_trns.png", grad(15, 1), 3, 4, palette=pal, trns=bytes([0, 128, 255, 7, 64]))
    png("palette2_interlaced.png", grad(3, 1), 3, 2, palette=pal[:4], interlace=True)
    png("ga8.png", grad(255, 2), 4, 8)
    png("ga16.png", grad(65535, 2), 4, 16)
    png("rgba8.png", grad(255, 4), 6, 8)
    png("rgba16.png", grad(65535, 4), 6, 16)
    png("rgba8_interlaced.png", grad(255, 4), 6, 8, interlace=True)
    opaque = grad(255, 4)
    opaque[..., 3] = 255
    png("rgba8_opaque.png", opaque, 6, 8)
    grey_rgb = np.repeat(grad(255, 1), 3, axis=-1)
    png("rgb8_grey_values.png", grey_rgb, 2, 8)
    png("ga8_opaque.png", np.concatenate([grad(255, 1), np.full((h, w, 1), 255)], axis=-1), 4, 8)
    png("rgb8_stored.png", grad(255, 3), 2, 8, level=0)
    # a larger image: dynamic Huffman blocks and long back-references
    y, x = np.mgrid[0:96, 0:80]
    big = np.stack([(x * 3) % 256, (y * 2) % 256, ((x + y) * 5) % 256, np.where((x // 8 + y // 8) % 2 == 0, 255, 40)],
                   axis=-1)
    write_png(os.path.join(folder, "rgba8_large.png"), big, 6, 8, level=9)
    names.append("rgba8_large.png")

    def tga(name, *args, **kw):
        write_tga(os.path.join(folder, name), *args, **kw)
        names.append(name)

    rgba = grad(255, 4).astype(np.uint8)
    tga("true24.tga", rgba, 2, 24)
    tga("true32_top.tga", rgba, 2, 32, top_first=True)
    runs = rgba.copy()
    runs[1:4, :, :] = (200, 100, 50, 128)
    tga("true32_rle.tga", runs, 2, 32, rle=True)
    tga("true24_rle_top.tga", runs, 2, 24, rle=True, top_first=True, image_id=b"fixture")
    tga("true16.tga", rgba, 2, 16)
    tga("grey8.tga", rgba, 3, 8)
    tga("grey8_rle.tga", runs, 3, 8, rle=True)
    idx = grad(11, 1).astype(np.uint8)
    idx4 = np.concatenate([idx, idx, idx, idx], axis=-1)
    pal = rng.integers(0, 256, size=(12, 3))
    tga("mapped8.tga", idx4, 1, 8, palette=pal)
    tga("mapped8_rle.tga", idx4, 1, 8, rle=True, palette=pal, top_first=True)

    def bmp(name, *args, **kw):
        write_bmp(os.path.join(folder, name), *args, **kw)
        names.append(name)

    for bits in (1, 4, 8):
        n = 1 << bits
        pal = rng.integers(0, 256, size=(n, 3))
        bmp(f"pal{bits}.bmp", grad(n - 1, 1)[..., 0], bits, palette=pal)
    pal = rng.integers(0, 256, size=(16, 3))
    bmp("pal4_top.bmp", grad(15, 1)[..., 0], 4, palette=pal, top_down=True)
    bmp("pal8_short.bmp", grad(9, 1)[..., 0], 8, palette=pal[:10])
    bmp("pal8_os2.bmp", grad(9, 1)[..., 0], 8, hsz=12, palette=np.concatenate([pal[:10], pal[:4]]))
    bmp("pal4_v5.bmp", grad(15, 1)[..., 0], 4, hsz=124, palette=pal)
    bmp("rgb24.bmp", grad(255, 3), 24)
    bmp("rgb24_top.bmp", grad(255, 3), 24, top_down=True)
    bmp("rgb24_os2.bmp", grad(255, 3), 24, hsz=12)
    bmp("rgb24_v4.bmp", grad(255, 3), 24, hsz=108)
    bmp("rgb555.bmp", grad(31, 3), 16, masks=(31 << 10, 31 << 5, 31, 0), compress=0)
    bmp("rgb565.bmp", np.concatenate([grad(31, 1), grad(63, 1), grad(31, 1)], axis=-1), 16,
        masks=(31 << 11, 63 << 5, 31, 0))
    bmp("argb1555_v5.bmp", np.concatenate([grad(31, 3), grad(1, 1)], axis=-1), 16, hsz=124,
        masks=(31 << 10, 31 << 5, 31, 1 << 15))
    bmp("argb4444_56.bmp", grad(15, 4), 16, hsz=56, masks=(15 << 8, 15 << 4, 15, 15 << 12))
    bmp("bgra32.bmp", grad(255, 4), 32, masks=(0xff0000, 0xff00, 0xff, 0xff000000), compress=0)
    zero_alpha = grad(255, 4)
    zero_alpha[..., 3] = 0
    bmp("bgra32_alpha0.bmp", zero_alpha, 32, masks=(0xff0000, 0xff00, 0xff, 0xff000000), compress=0)
    bmp("rgba32_v5.bmp", grad(255, 4), 32, hsz=124, masks=(0xff, 0xff00, 0xff0000, 0xff000000))
    bmp("rgb32_fields.bmp", grad(255, 3), 32, masks=(0xff000000, 0xff0000, 0xff00, 0))
    bmp("rgb32_v4_default.bmp", grad(255, 4), 32, hsz=108, masks=(0xff0000, 0xff00, 0xff, 0xff000000),
        compress=0, top_down=True)
    bmp("rgb24_gap.bmp", grad(255, 3), 24, gap=4)

    def pnm(name, *args, **kw):
        write_pnm(os.path.join(folder, name), *args, **kw)
        names.append(name)

    pnm("grey8.pgm", grad(255, 1)[..., 0], 255)
    pnm("grey8_comment.pgm", grad(200, 1)[..., 0], 200, comment=True)
    pnm("rgb8.ppm", grad(255, 3), 255, comment=True)
    pnm("rgb16.ppm", grad(65535, 3), 65535)
    pnm("grey16.pgm", grad(4095, 1)[..., 0], 4095)

    def gif(name, *args, **kw):
        write_gif(os.path.join(folder, name), *args, **kw)
        names.append(name)

    pal16 = rng.integers(0, 256, size=(16, 3))
    gif("global16.gif", grad(15, 1)[..., 0], pal16)
    gif("local8_interlaced.gif", np.concatenate([grad(7, 1), grad(7, 1)[:4]])[..., 0], pal16[:8], local=True,
        interlace=True, transparent=3)
    gif("global4_transparent_87a.gif", grad(3, 1)[..., 0], pal16[:4], transparent=1, version=b"87a", comment=True)
    gif("subrect_background.gif", grad(15, 1)[..., 0], pal16, canvas=(20, 12), offset=(4, 3), background=5)
    gif("short_table.gif", grad(7, 1)[..., 0], pal16[:4], min_size=3)  # indices past the table
    y, x = np.mgrid[0:96, 0:128]
    noisy = np.where(rng.random((96, 128)) < 0.5, rng.integers(0, 256, size=(96, 128)), (x // 4 + y // 3) % 256)
    pal256 = rng.integers(0, 256, size=(256, 3))
    gif("large256.gif", noisy, pal256)
    gif("large256_interlaced_cut.gif", noisy, pal256, interlace=True, cut=6000)
    return names
