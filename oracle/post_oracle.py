"""CPU oracle of the display post-processing (test infrastructure only).

A numpy restatement, in FP64 and in the reference's order of operations, of
postprocess (include/postprocess.h:104-151: bloom pyramid + vignette),
display_settings::apply (include/tonemap.h:28-67: exposure, Reinhard, the
ACES fit) and to_byte (include/color3.h:17-36: sRGB curve, 8 bits).
"""
import math

import numpy as np


def _at(img, i, j):
    h, w, _ = img.shape
    return img[np.clip(j, 0, h - 1), np.clip(i, 0, w - 1)]


def _downsample(img):  # postprocess.h:50-59
    h, w, _ = img.shape
    ow, oh = max(1, w // 2), max(1, h // 2)
    j, i = np.meshgrid(np.arange(oh), np.arange(ow), indexing="ij")
    return 0.25 * (((_at(img, 2 * i, 2 * j) + _at(img, 2 * i + 1, 2 * j)) + _at(img, 2 * i, 2 * j + 1))
                   + _at(img, 2 * i + 1, 2 * j + 1))


def _blur(img, sigma=1.5):  # postprocess.h:62-84
    r = int(math.ceil(3 * sigma))
    kernel = []
    s = 0.0
    for k in range(-r, r + 1):
        v = math.exp(-0.5 * k * k / (sigma * sigma))
        kernel.append(v)
        s += v
    kernel = [k / s for k in kernel]
    h, w, _ = img.shape
    j, i = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
    tmp = np.zeros_like(img)
    for k in range(-r, r + 1):
        tmp = tmp + kernel[k + r] * _at(img, i + k, j)
    out = np.zeros_like(img)
    for k in range(-r, r + 1):
        out = out + kernel[k + r] * _at(tmp, i, j + k)
    return out


def _sample(img, x, y):  # postprocess.h:36-44
    x = x - 0.5
    y = y - 0.5
    i = np.floor(x).astype(int)
    j = np.floor(y).astype(int)
    fx = (x - i)[..., None]
    fy = (y - j)[..., None]
    return (1 - fy) * ((1 - fx) * _at(img, i, j) + fx * _at(img, i + 1, j)) + \
        fy * ((1 - fx) * _at(img, i, j + 1) + fx * _at(img, i + 1, j + 1))


def postprocess(px, bloom=0.0, threshold=1.0, radius=0.04, vignette=0.0):
    """Bloom and vignetting of a radiance image (H, W, 3)."""
    px = np.asarray(px, dtype=np.float64)
    h, w, _ = px.shape
    out = px.copy()
    if bloom > 0:
        lum = 0.2126 * px[..., 0] + 0.7152 * px[..., 1] + 0.0722 * px[..., 2]
        keep = np.isfinite(lum) & (lum > threshold)
        scale = np.where(keep, (lum - threshold) / np.where(keep, lum, 1.0), 0.0)
        bright = np.where(keep[..., None], px * scale[..., None], 0.0)
        reach = max(radius * w, 1.0)
        levels = min(max(int(math.ceil(math.log2(reach))), 1), 10)
        blurred = []
        level = bright
        for _ in range(levels):
            if level.shape[1] <= 1 or level.shape[0] <= 1:
                break
            level = _downsample(level)
            blurred.append(_blur(level))
        j, i = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
        glow = np.zeros_like(px)
        for b in blurred:
            sx, sy = b.shape[1] / w, b.shape[0] / h
            glow = glow + _sample(b, (i + 0.5) * sx, (j + 0.5) * sy)
        if blurred:
            out = out + (bloom / len(blurred)) * glow
    if vignette > 0:
        cx, cy = 0.5 * w, 0.5 * h
        corner2 = cx * cx + cy * cy
        j, i = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
        dx, dy = i + 0.5 - cx, j + 0.5 - cy
        f = 1 + vignette * (dx * dx + dy * dy) / corner2
        out = (1 / (f * f))[..., None] * out
    return out


def _rrt_odt_fit(x):
    a = x * (x + 0.0245786) - 0.000090537
    b = x * (0.983729 * x + 0.4329510) + 0.238081
    return a / b


def apply(px, exposure=0.0, tonemap=0):
    """display_settings::apply: 0 none, 1 Reinhard, 2 the ACES fit."""
    c = (2.0 ** exposure) * np.asarray(px, dtype=np.float64)
    if tonemap == 1:
        return c / (1 + c)
    if tonemap == 2:
        r, g, b = c[..., 0], c[..., 1], c[..., 2]
        vr = _rrt_odt_fit(0.59719 * r + 0.35458 * g + 0.04823 * b)
        vg = _rrt_odt_fit(0.07600 * r + 0.90834 * g + 0.01566 * b)
        vb = _rrt_odt_fit(0.02840 * r + 0.13383 * g + 0.83777 * b)
        out = np.stack([1.60475 * vr + -0.53108 * vg + -0.07367 * vb,
                        -0.10208 * vr + 1.10813 * vg + -0.00605 * vb,
                        -0.00327 * vr + -0.07276 * vg + 1.07602 * vb], axis=-1)
        return np.clip(out, 0, 1)
    return c


def to_byte(x):
    x = np.asarray(x, dtype=np.float64)
    with np.errstate(invalid="ignore", divide="ignore"):
        s = np.where(x <= 0, 0.0, np.where(x <= 0.0031308, 12.92 * x,
                                           1.055 * np.power(np.maximum(x, 1e-300), 1.0 / 2.4) - 0.055))
    s = np.where(s < 0.0, 0.0, np.where(s > 0.999, 0.999, s))
    return (256 * s).astype(np.uint8)
