"""A small JPEG writer for the decoding fixtures: baseline and progressive.

Sequential or progressive DCT (spectral selection and successive
approximation: DC and AC first passes with end-of-band runs, refinement
passes with correction bits), Huffman tables built per image from its own symbol counts
(valid JPEG: the tables travel in the DHT segments), quantisation tables of
its own (8- or 16-bit), JFIF YCbCr with any of 4:4:4, 4:2:2, 4:2:0 and 4:4:0
subsampling or a single grey component, optional restart intervals, one
interleaved scan or one scan per component. Odd image sizes exercise
partial MCUs. Seeded content, so the files are reproducible.
"""
import heapq
import os
import struct

import numpy as np

ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20,
                   13, 6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52,
                   45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])

_C = np.array([[(np.sqrt(0.5) if u == 0 else 1.0) * np.cos((2 * x + 1) * u * np.pi / 16) / 2 for x in range(8)]
               for u in range(8)])


def _fdct(block):
    return _C @ block @ _C.T


def _category(v):
    v = abs(int(v))
    return 0 if v == 0 else int(v).bit_length()


def _bits_of(v, s):
    return v if v >= 0 else v + (1 << s) - 1


def _huffman_lengths(freq):
    """Code lengths (<= 16) for the symbols with non-zero counts; one extra
    symbol keeps the all-ones code unused."""
    items = [(f, [s]) for s, f in freq.items() if f > 0] + [(0.5, [-1])]
    lengths = {s: 0 for s in freq}
    lengths[-1] = 0
    if len(items) == 1:
        items.append((0.25, [-2]))
        lengths[-2] = 0
    heap = [(f, i, syms) for i, (f, syms) in enumerate(items)]
    heapq.heapify(heap)
    counter = len(heap)
    while len(heap) > 1:
        f1, _, a = heapq.heappop(heap)
        f2, _, b = heapq.heappop(heap)
        for s in a + b:
            lengths[s] += 1
        heapq.heappush(heap, (f1 + f2, counter, a + b))
        counter += 1
    if max(lengths.values()) > 16:  # not met by the small fixtures; keep the writer honest
        raise ValueError("code longer than 16 bits")
    return {s: l for s, l in lengths.items() if s >= 0 and freq.get(s, 0) > 0}


def _canonical(lengths):
    order = sorted(lengths, key=lambda s: (lengths[s], s))
    codes, code, prev = {}, 0, 0
    for s in order:
        code <<= lengths[s] - prev
        prev = lengths[s]
        codes[s] = (code, lengths[s])
        code += 1
    counts = [0] * 17
    for s in order:
        counts[lengths[s]] += 1
    return codes, counts[1:], order


class _BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, value, length):
        for i in range(length - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc, self.n = 0, 0

    def flush(self):
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)


def _segment(marker, payload):
    return struct.pack(">BBH", 0xFF, marker, len(payload) + 2) + payload


def _progressive_script(ncomp):
    """Scans (components, Ss, Se, Ah, Al) of a progressive file: DC first with
    one bit held back, luma low band, chroma, luma high band, then the
    refinement passes (the shape of libjpeg's simple progression)."""
    if ncomp == 1:
        return [([0], 0, 0, 0, 1), ([0], 1, 5, 0, 2), ([0], 6, 63, 0, 2), ([0], 1, 63, 2, 1), ([0], 0, 0, 1, 0),
                ([0], 1, 63, 1, 0)]
    return [([0, 1, 2], 0, 0, 0, 1), ([0], 1, 5, 0, 2), ([2], 1, 63, 0, 1), ([1], 1, 63, 0, 1), ([0], 6, 63, 0, 2),
            ([0], 1, 63, 2, 1), ([0, 1, 2], 0, 0, 1, 0), ([2], 1, 63, 1, 0), ([1], 1, 63, 1, 0), ([0], 1, 63, 1, 0)]


def _mag_bits(v, size):
    """JPEG's value bits: v itself if positive, its ones' complement if negative."""
    return v if v >= 0 else (v + (1 << size) - 1)


def _progressive_stream(blocks, comp_list, units, factors, ss, se, ah, al, tables, restart, interleaved):
    """Items of one progressive scan: ("dc"|"ac", table, symbol, (bits, n)),
    ("raw", bits, n) and ("rst", index)."""
    items = []
    pred = {c: 0 for c in comp_list}
    state = {"eobrun": 0, "be": []}

    def flush_eob(table):
        run = state["eobrun"]
        if run:
            nb = run.bit_length() - 1
            items.append(("ac", table, nb << 4, (run - (1 << nb), nb)))
            state["eobrun"] = 0
        for b in state["be"]:
            items.append(("raw", b, 1))
        state["be"] = []

    table = tables[comp_list[0]]
    count = 0
    for uy, ux in units:
        if restart and count and count % restart == 0:
            if ss > 0:
                flush_eob(table)
            items.append(("rst", count // restart - 1))
            pred = {c: 0 for c in comp_list}
        for c in comp_list:
            fh, fv = factors[c]
            cells = [(uy * fv + j, ux * fh + i) for j in range(fv) for i in range(fh)] if interleaved else [(uy, ux)]
            for by, bx in cells:
                zz = [int(x) for x in blocks[c][by, bx]]
                if ss == 0:
                    if ah == 0:
                        v = zz[0] >> al  # arithmetic shift, as the refinement bits expect
                        d = v - pred[c]
                        pred[c] = v
                        size = _category(d)
                        items.append(("dc", tables[c], size, (_mag_bits(d, size), size)))
                    else:
                        items.append(("raw", (zz[0] >> al) & 1, 1))
                    continue
                if ah == 0:
                    vals = []
                    for k in range(ss, se + 1):
                        t = zz[k]
                        m = abs(t) >> al
                        vals.append(-m if t < 0 else m)
                    last = max([i for i, v in enumerate(vals) if v != 0], default=-1)
                    if last < 0:
                        state["eobrun"] += 1
                        if state["eobrun"] == 0x7FFF:
                            flush_eob(table)
                        continue
                    flush_eob(table)
                    run = 0
                    for i in range(last + 1):
                        v = vals[i]
                        if v == 0:
                            run += 1
                            continue
                        while run > 15:
                            items.append(("ac", table, 0xF0, (0, 0)))
                            run -= 16
                        size = _category(v)
                        items.append(("ac", table, (run << 4) | size, (_mag_bits(v, size), size)))
                        run = 0
                    if last < se - ss:
                        state["eobrun"] += 1
                        if state["eobrun"] == 0x7FFF:
                            flush_eob(table)
                    continue
                # AC refinement
                absv = [abs(zz[k]) >> al for k in range(ss, se + 1)]
                eob = max([i for i, a in enumerate(absv) if a == 1], default=-1)
                run, br = 0, []
                for i, a in enumerate(absv):
                    if a == 0:
                        run += 1
                        continue
                    while run > 15 and i <= eob:
                        flush_eob(table)
                        items.append(("ac", table, 0xF0, (0, 0)))
                        run -= 16
                        for b in br:
                            items.append(("raw", b, 1))
                        br = []
                    if a > 1:
                        br.append(a & 1)
                        continue
                    flush_eob(table)
                    items.append(("ac", table, (run << 4) | 1, (0, 0)))
                    items.append(("raw", 0 if zz[ss + i] < 0 else 1, 1))
                    for b in br:
                        items.append(("raw", b, 1))
                    br = []
                    run = 0
                if run > 0 or br:
                    state["eobrun"] += 1
                    state["be"] += br
                    if state["eobrun"] == 0x7FFF or len(state["be"]) > 900:
                        flush_eob(table)
        count += 1
    if ss > 0:
        flush_eob(table)
    return items


def write_jpeg(path, rgb, sampling=(1, 1), grey=False, quality=2, restart=0, separate_scans=False, wide_quant=False,
               progressive=False):
    """rgb: (H, W, 3) uint8 (or (H, W) for grey). sampling: luma (h, v) factors, chroma 1 x 1."""
    h, w = rgb.shape[:2]
    if grey:
        planes = [rgb.astype(np.float64) if rgb.ndim == 2 else rgb[..., 0].astype(np.float64)]
        factors = [(1, 1)]
    else:
        r, g, b = (rgb[..., c].astype(np.float64) for c in range(3))
        y = 0.299 * r + 0.587 * g + 0.114 * b
        cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128
        cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128
        planes = [y, cb, cr]
        factors = [sampling, (1, 1), (1, 1)]
    hmax = max(f[0] for f in factors)
    vmax = max(f[1] for f in factors)
    mcux, mcuy = -(-w // (8 * hmax)), -(-h // (8 * vmax))
    # quantisation tables of our own: finer for luma
    u, v = np.meshgrid(np.arange(8), np.arange(8))
    qt = [np.clip(2 + quality * (u + v), 1, 255).astype(int), np.clip(3 + quality * (u + v) * 2, 1, 255).astype(int)]
    if wide_quant:
        qt[0] = qt[0] * 3 + 300  # needs 16-bit entries
    blocks = []  # per component: (bh, bw) blocks of quantised zigzag coefficients
    for ci, (plane, (fh, fv)) in enumerate(zip(planes, factors)):
        sub_w, sub_h = mcux * 8 * fh, mcuy * 8 * fv
        sx, sy = hmax // fh, vmax // fv
        # subsample by averaging, pad by edge replication
        pw, ph = -(-w // sx), -(-h // sy)
        padded = np.pad(plane, ((0, ph * sy - h), (0, pw * sx - w)), mode="edge")
        small = padded.reshape(ph, sy, pw, sx).mean(axis=(1, 3))
        small = np.pad(small, ((0, sub_h - ph), (0, sub_w - pw)), mode="edge")
        q = qt[0 if ci == 0 else 1]
        bl = np.zeros((sub_h // 8, sub_w // 8, 64), dtype=int)
        for by in range(sub_h // 8):
            for bx in range(sub_w // 8):
                c = _fdct(small[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8] - 128)
                bl[by, bx] = np.round(c / q).astype(int).reshape(-1)[ZIGZAG]
        blocks.append(bl)
    tables = [0] if grey else [0, 1, 1]

    def symbols_of(comp_list, units):
        """The (component, table, kind, symbol, extra bits) stream of a scan."""
        pred = {c: 0 for c in comp_list}
        stream = []
        count = 0
        for uy, ux in units:
            if restart and count and count % restart == 0:
                stream.append(("rst", count // restart - 1))
                pred = {c: 0 for c in comp_list}
            for c in comp_list:
                fh, fv = factors[c]
                cells = [(uy * fv + j, ux * fh + i) for j in range(fv) for i in range(fh)] if len(comp_list) > 1 \
                    else [(uy, ux)]
                for by, bx in cells:
                    zz = blocks[c][by, bx]
                    d = int(zz[0]) - pred[c]
                    pred[c] = int(zz[0])
                    s = _category(d)
                    stream.append(("dc", tables[c], s, (_bits_of(d, s), s)))
                    run = 0
                    last = max([k for k in range(1, 64) if zz[k] != 0], default=0)
                    for k in range(1, last + 1):
                        if zz[k] == 0:
                            run += 1
                            continue
                        while run > 15:
                            stream.append(("ac", tables[c], 0xF0, (0, 0)))
                            run -= 16
                        s = _category(zz[k])
                        stream.append(("ac", tables[c], (run << 4) | s, (_bits_of(int(zz[k]), s), s)))
                        run = 0
                    if last < 63:
                        stream.append(("ac", tables[c], 0x00, (0, 0)))
            count += 1
        return stream

    if separate_scans and not grey:
        scans = []
        for c in range(3):
            bh, bw = blocks[c].shape[:2]
            fh, fv = factors[c]
            comp_w, comp_h = -(-w * fh // hmax), -(-h * fv // vmax)  # the component's own size
            need_w, need_h = -(-comp_w // 8), -(-comp_h // 8)
            units = [(y, x) for y in range(min(bh, need_h)) for x in range(min(bw, need_w))]
            scans.append(([c], units))
    else:
        comps = [0] if grey else [0, 1, 2]
        if grey:
            bh, bw = blocks[0].shape[:2]
            units = [(y, x) for y in range(-(-h // 8)) for x in range(-(-w // 8))]
        else:
            units = [(y, x) for y in range(mcuy) for x in range(mcux)]
        scans = [(comps, units)]
    spectral = [(0, 63, 0, 0)] * len(scans)
    if progressive:
        ncomp_ = 1 if grey else 3
        scans, spectral, streams = [], [], []
        for cl, ss, se, ah, al in _progressive_script(ncomp_):
            if len(cl) > 1:  # interleaved DC scan: MCUs
                units = [(y, x) for y in range(mcuy) for x in range(mcux)]
            else:  # one component: its own blocks covering the image
                c = cl[0]
                fh, fv = factors[c]
                comp_w, comp_h = -(-w * fh // hmax), -(-h * fv // vmax)
                units = [(y, x) for y in range(-(-comp_h // 8)) for x in range(-(-comp_w // 8))]
            scans.append((cl, units))
            spectral.append((ss, se, ah, al))
            streams.append(_progressive_stream(blocks, cl, units, factors, ss, se, ah, al, tables, restart, len(cl) > 1))
    else:
        streams = [symbols_of(cl, units) for cl, units in scans]
    # Huffman tables from the counts of all scans
    freq = {}
    for st in streams:
        for item in st:
            if item[0] in ("dc", "ac"):
                key = (item[0], item[1])
                freq.setdefault(key, {})
                freq[key][item[2]] = freq[key].get(item[2], 0) + 1
    codes = {}
    dht = bytearray()
    for (kind, t), f in sorted(freq.items()):
        c, counts, order = _canonical(_huffman_lengths(f))
        codes[(kind, t)] = c
        dht += bytes([(0 if kind == "dc" else 1) << 4 | t]) + bytes(counts) + bytes(order)
    out = bytearray(b"\xFF\xD8")
    out += _segment(0xE0, b"JFIF\0\x01\x01\0\0\x01\0\x01\0\0")
    for t, q in enumerate(qt[:1 if grey else 2]):
        zz = q.reshape(-1)[ZIGZAG]
        if wide_quant and t == 0:
            out += _segment(0xDB, bytes([0x10 | t]) + b"".join(struct.pack(">H", int(x)) for x in zz))
        else:
            out += _segment(0xDB, bytes([t]) + bytes(int(x) for x in zz))
    ncomp = 1 if grey else 3
    sof = struct.pack(">BHHB", 8, h, w, ncomp)
    for c in range(ncomp):
        fh, fv = factors[c]
        sof += bytes([c + 1, (fh << 4) | fv, 0 if c == 0 else 1])
    out += _segment(0xC2 if progressive else 0xC0, sof)
    out += _segment(0xC4, bytes(dht))
    if restart:
        out += _segment(0xDD, struct.pack(">H", restart))
    for (cl, _), st, (ss, se, ah, al) in zip(scans, streams, spectral):
        sos = bytes([len(cl)]) + b"".join(bytes([c + 1, (tables[c] << 4) | tables[c]]) for c in cl)
        sos += bytes([ss, se, (ah << 4) | al])
        out += _segment(0xDA, sos)
        bw_ = _BitWriter()
        for item in st:
            if item[0] == "rst":
                bw_.flush()
                out += bw_.out + bytes([0xFF, 0xD0 + item[1] % 8])
                bw_ = _BitWriter()
                continue
            if item[0] == "raw":
                bw_.put(item[1], item[2])
                continue
            kind, t, sym, (extra, nbits) = item
            code, length = codes[(kind, t)][sym]
            bw_.put(code, length)
            if nbits:
                bw_.put(extra, nbits)
        bw_.flush()
        out += bw_.out
    out += b"\xFF\xD9"
    with open(path, "wb") as f:
        f.write(out)


def make_jpeg_fixtures(folder):
    os.makedirs(folder, exist_ok=True)
    rng = np.random.default_rng(77)
    names = []

    def image(h, w):
        y, x = np.mgrid[0:h, 0:w]
        img = np.stack([(x * 9 + y * 2) % 256, (y * 7) % 256, ((x + y) * 5 + 40) % 256], axis=-1).astype(float)
        img[h // 3: h // 2, w // 4: w // 2] = (230, 40, 30)  # a sharp-edged patch
        img += rng.normal(0, 6, img.shape)
        return np.clip(img, 0, 255).astype(np.uint8)

    cases = [
        ("ycc444.jpg", dict(sampling=(1, 1)), (21, 27)),
        ("ycc422.jpg", dict(sampling=(2, 1)), (19, 37)),
        ("ycc420.jpg", dict(sampling=(2, 2)), (33, 29)),
        ("ycc440.jpg", dict(sampling=(1, 2)), (23, 18)),
        ("grey.jpg", dict(grey=True), (17, 23)),
        ("ycc420_restart.jpg", dict(sampling=(2, 2), restart=2), (40, 48)),
        ("ycc422_scans.jpg", dict(sampling=(2, 1), separate_scans=True), (18, 30)),
        ("ycc444_q16.jpg", dict(sampling=(1, 1), wide_quant=True, quality=1), (16, 16)),
        ("ycc420_large.jpg", dict(sampling=(2, 2), quality=1), (96, 128)),
        ("prog420.jpg", dict(sampling=(2, 2), progressive=True, quality=1), (45, 61)),
        ("prog444.jpg", dict(sampling=(1, 1), progressive=True), (24, 40)),
        ("prog_grey.jpg", dict(grey=True, progressive=True, quality=1), (33, 27)),
        ("prog422_restart.jpg", dict(sampling=(2, 1), progressive=True, restart=3), (32, 48)),
    ]
    for name, kw, (h, w) in cases:
        write_jpeg(os.path.join(folder, name), image(h, w), **kw)
        names.append(name)
    return names
