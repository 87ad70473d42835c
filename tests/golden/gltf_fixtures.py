"""glTF 2.0 fixtures: one model written as a .glb (binary chunk, an image in
a buffer view) and as a .gltf (base64 data-URI buffer, image files beside it).

What it holds, to exercise the loader (gltf_loader.h of the reference):
a node tree (matrix, translation / rotation / scale, a parent chain, a
mirroring scale, one mesh placed twice), interleaved and plain buffer views,
float / normalized 8- and 16-bit texture coordinates, 8-, 16- and 32-bit
indices and a non-indexed primitive, and materials: a textured clear-coated
paint with a metallic-roughness map, a scaled normal map and a texture
transform; a cut-out leaf (alphaMode MASK over the texture's alpha); a veil
(BLEND, constant alpha 0.4); a lamp (emissive strength); a glowing panel
(emissive texture); glass (transmission, ior); one with sheen (left out); and
a primitive without a material. Transforms use single-axis rotations, whose
single-precision matrices come out the same in any evaluation order.
"""
import base64
import json
import math
import os
import struct

import numpy as np

from image_fixtures import write_png


def _quad(cx, cy, cz, sx, sy):
    """A quad in its xy plane: positions, normals, uvs (2 triangles)."""
    p = np.array([[cx - sx, cy - sy, cz], [cx + sx, cy - sy, cz], [cx + sx, cy + sy, cz], [cx - sx, cy + sy, cz]],
                 dtype=np.float32)
    n = np.tile(np.array([0, 0, 1], dtype=np.float32), (4, 1))
    uv = np.array([[0, 1], [1, 1], [1, 0], [0, 0]], dtype=np.float32)  # glTF: v down
    return p, n, uv


def _box(sx, sy, sz):
    """A box around the origin, 24 vertices, outward normals, per-face uvs."""
    ps, ns, uvs, idx = [], [], [], []
    faces = [((1, 0, 0), (0, 0, -1), (0, 1, 0)), ((-1, 0, 0), (0, 0, 1), (0, 1, 0)),
             ((0, 1, 0), (1, 0, 0), (0, 0, -1)), ((0, -1, 0), (1, 0, 0), (0, 0, 1)),
             ((0, 0, 1), (1, 0, 0), (0, 1, 0)), ((0, 0, -1), (-1, 0, 0), (0, 1, 0))]
    s = np.array([sx, sy, sz])
    for n, u, v in faces:
        n, u, v = map(np.array, (n, u, v))
        base = len(ps)
        for a, b in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
            ps.append((n + a * u + b * v) * s)
            ns.append(n)
            uvs.append(((a + 1) / 2, (1 - b) / 2))
        idx += [base, base + 1, base + 2, base, base + 2, base + 3]
    return (np.array(ps, dtype=np.float32), np.array(ns, dtype=np.float32), np.array(uvs, dtype=np.float32),
            np.array(idx))


class _Builder:
    def __init__(self):
        self.bin = bytearray()
        self.views, self.accessors = [], []

    def view(self, data, stride=None, target=None):
        while len(self.bin) % 4:
            self.bin.append(0)
        v = {"buffer": 0, "byteOffset": len(self.bin), "byteLength": len(data)}
        if stride:
            v["byteStride"] = stride
        if target:
            v["target"] = target
        self.bin += data
        self.views.append(v)
        return len(self.views) - 1

    def accessor(self, view, ctype, count, kind, offset=0, normalized=False, lo=None, hi=None):
        a = {"bufferView": view, "componentType": ctype, "count": count, "type": kind}
        if offset:
            a["byteOffset"] = offset
        if normalized:
            a["normalized"] = True
        if lo is not None:
            a["min"], a["max"] = [float(x) for x in lo], [float(x) for x in hi]
        self.accessors.append(a)
        return len(self.accessors) - 1

    def floats(self, arr, kind):
        arr = np.ascontiguousarray(arr, dtype=np.float32)
        v = self.view(arr.tobytes(), target=34962)
        lo = hi = None
        if kind == "VEC3":
            lo, hi = arr.min(axis=0), arr.max(axis=0)
        return self.accessor(v, 5126, len(arr), kind, lo=lo, hi=hi)


def _mesh_primitives(b):
    """The primitives of each mesh, as accessor indices."""
    meshes = []
    # 0: paint box, interleaved positions + normals, float uvs, u16 indices
    p, n, uv, idx = _box(0.5, 0.4, 0.3)
    inter = np.concatenate([p, n], axis=1).astype(np.float32)
    v = b.view(inter.tobytes(), stride=24, target=34962)
    pa = b.accessor(v, 5126, len(p), "VEC3", lo=p.min(axis=0), hi=p.max(axis=0))
    na = b.accessor(v, 5126, len(p), "VEC3", offset=12)
    ta = b.floats(uv, "VEC2")
    ia = b.accessor(b.view(np.asarray(idx, dtype=np.uint16).tobytes(), target=34963), 5123, len(idx), "SCALAR")
    meshes.append([{"attributes": {"POSITION": pa, "NORMAL": na, "TEXCOORD_0": ta}, "indices": ia, "material": 0}])
    # 1: leaf quad, normalized u16 uvs, u8 indices
    p, n, uv = _quad(0, 0, 0, 0.5, 0.5)
    uv16 = np.round(uv * 65535).astype(np.uint16)
    ta = b.accessor(b.view(uv16.tobytes(), target=34962), 5123, 4, "VEC2", normalized=True)
    ia = b.accessor(b.view(np.array([0, 1, 2, 0, 2, 3], dtype=np.uint8).tobytes(), target=34963), 5121, 6, "SCALAR")
    meshes.append([{"attributes": {"POSITION": b.floats(p, "VEC3"), "NORMAL": b.floats(n, "VEC3"),
                                   "TEXCOORD_0": ta}, "indices": ia, "material": 1}])
    # 2: veil quad, normalized u8 uvs, u32 indices; and a second primitive without a material
    p, n, uv = _quad(0, 0, 0, 0.45, 0.6)
    uv8 = np.round(uv * 255).astype(np.uint8)
    ta = b.accessor(b.view(uv8.tobytes(), target=34962), 5121, 4, "VEC2", normalized=True)
    ia = b.accessor(b.view(np.array([0, 1, 2, 0, 2, 3], dtype=np.uint32).tobytes(), target=34963), 5125, 6, "SCALAR")
    p2, n2, _ = _quad(0, -0.9, 0.05, 0.3, 0.2)
    meshes.append([{"attributes": {"POSITION": b.floats(p, "VEC3"), "NORMAL": b.floats(n, "VEC3"),
                                   "TEXCOORD_0": ta}, "indices": ia, "material": 2},
                   {"attributes": {"POSITION": b.floats(p2[[0, 1, 2, 0, 2, 3]], "VEC3")}}])
    # 3: lamp quad facing down (non-indexed)
    p = np.array([[-0.4, 0, -0.3], [0.4, 0, -0.3], [0.4, 0, 0.3], [-0.4, 0, -0.3], [0.4, 0, 0.3], [-0.4, 0, 0.3]],
                 dtype=np.float32)
    meshes.append([{"attributes": {"POSITION": b.floats(p, "VEC3")}, "material": 3}])
    # 4: glowing panel, glass pane, sheen sphere-ish box
    p, n, uv = _quad(0, 0, 0, 0.35, 0.25)
    meshes.append([{"attributes": {"POSITION": b.floats(p, "VEC3"), "NORMAL": b.floats(n, "VEC3"),
                                   "TEXCOORD_0": b.floats(uv, "VEC2")},
                    "indices": b.accessor(b.view(np.array([0, 1, 2, 0, 2, 3], dtype=np.uint16).tobytes()), 5123, 6,
                                          "SCALAR"), "material": 4}])
    p, n, uv = _quad(0, 0, 0, 0.4, 0.5)
    meshes.append([{"attributes": {"POSITION": b.floats(p, "VEC3"), "NORMAL": b.floats(n, "VEC3")},
                    "indices": b.accessor(b.view(np.array([0, 1, 2, 0, 2, 3], dtype=np.uint16).tobytes()), 5123, 6,
                                          "SCALAR"), "material": 5}])
    p, n, uv, idx = _box(0.25, 0.25, 0.25)
    meshes.append([{"attributes": {"POSITION": b.floats(p, "VEC3"), "NORMAL": b.floats(n, "VEC3")},
                    "indices": b.accessor(b.view(np.asarray(idx, dtype=np.uint16).tobytes()), 5123, len(idx),
                                          "SCALAR"), "material": 6}])
    return meshes


def _images(folder):
    """The PNG files: paint (RGBA, opaque alpha), metal-roughness (RGB), normals (RGB), leaf (RGBA cut-out),
    glow (RGB). Returns {name: bytes}."""
    y, x = np.mgrid[0:16, 0:16]
    out = {}

    def png(name, arr, ctype):
        path = os.path.join(folder, name)
        write_png(path, arr, ctype, 8)
        out[name] = open(path, "rb").read()

    paint = np.stack([40 + 12 * x, 60 + 8 * y, np.full_like(x, 200), np.full_like(x, 255)], axis=-1)
    png("gallery_paint.png", paint, 6)
    png("gallery_metal_rough.png", np.stack([np.zeros_like(x), 30 + 12 * y, np.where(x < 8, 255, 0)], axis=-1), 2)
    png("gallery_bumps.png", np.stack([np.where((x // 4) % 2 == 0, 170, 86), np.full_like(x, 128), np.full_like(x, 230)],
                              axis=-1), 2)
    r = np.hypot(x - 7.5, y - 7.5)
    png("gallery_leaf.png", np.stack([40 + 8 * x, 150 + 4 * y, np.full_like(x, 60), np.where(r < 6, 255, 0)], axis=-1), 6)
    png("gallery_glow.png", np.stack([np.full_like(x, 255), 128 + 8 * y, np.where((x + y) % 2 == 0, 40, 220)], axis=-1), 2)
    return out


def _document(b, meshes, image_refs):
    deg = math.radians
    nodes = [
        {"name": "root", "children": [1, 2, 3, 4, 5, 6, 7, 8], "translation": [0, 0.5, 0]},
        {"name": "paint", "mesh": 0, "translation": [-1.0, 0.0, 0.2],
         "rotation": [0, math.sin(deg(30) / 2), 0, math.cos(deg(30) / 2)]},
        {"name": "leaf", "mesh": 1, "matrix": [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0.3, 0.3, 0.6, 1]},
        {"name": "veil", "mesh": 2, "translation": [1.1, 0.2, 0.3], "scale": [1.2, 1.0, 1.0]},
        {"name": "lamp", "mesh": 3, "translation": [0, 1.6, 0]},
        {"name": "glow_parent", "translation": [-1.6, 0.6, -0.6], "children": [9]},
        {"name": "pane", "mesh": 5, "translation": [0.7, 0.0, 1.0],
         "rotation": [math.sin(deg(-20) / 2), 0, 0, math.cos(deg(-20) / 2)]},
        {"name": "sheen", "mesh": 6, "translation": [1.4, -0.2, -0.5]},
        {"name": "mirror", "mesh": 1, "translation": [-0.4, 0.9, 0.4], "scale": [-0.6, 0.6, 0.6]},
        {"name": "glow", "mesh": 4, "rotation": [0, 0, math.sin(deg(10) / 2), math.cos(deg(10) / 2)]},
    ]
    materials = [
        {"name": "paint", "pbrMetallicRoughness": {
            "baseColorFactor": [0.9, 0.8, 0.7, 1.0], "baseColorTexture": {
                "index": 0, "extensions": {"KHR_texture_transform": {"offset": [0.1, 0.2], "rotation": 0.3,
                                                                      "scale": [2.0, 2.0]}}},
            "metallicFactor": 0.8, "roughnessFactor": 0.9, "metallicRoughnessTexture": {"index": 1}},
         "normalTexture": {"index": 2, "scale": 0.5},
         "extensions": {"KHR_materials_clearcoat": {"clearcoatFactor": 1.0, "clearcoatRoughnessFactor": 0.1}}},
        {"name": "leaf", "alphaMode": "MASK", "doubleSided": True,
         "pbrMetallicRoughness": {"baseColorTexture": {"index": 3}, "metallicFactor": 0.0, "roughnessFactor": 0.7}},
        {"name": "veil", "alphaMode": "BLEND",
         "pbrMetallicRoughness": {"baseColorFactor": [0.9, 0.9, 0.95, 0.4], "metallicFactor": 0.0}},
        {"name": "lamp", "emissiveFactor": [1.0, 0.9, 0.7],
         "extensions": {"KHR_materials_emissive_strength": {"emissiveStrength": 6.0}}},
        {"name": "glow", "emissiveFactor": [2.0, 2.0, 2.0], "emissiveTexture": {"index": 4},
         "pbrMetallicRoughness": {"baseColorFactor": [0.2, 0.2, 0.2, 1], "metallicFactor": 0.0}},
        {"name": "glass", "pbrMetallicRoughness": {"baseColorFactor": [0.8, 0.95, 0.85, 1], "roughnessFactor": 0.0},
         "extensions": {"KHR_materials_transmission": {"transmissionFactor": 1.0},
                        "KHR_materials_ior": {"ior": 1.4}}},
        {"name": "velvet", "pbrMetallicRoughness": {"baseColorFactor": [0.6, 0.1, 0.2, 1], "metallicFactor": 0.0,
                                                    "roughnessFactor": 0.6},
         "extensions": {"KHR_materials_sheen": {"sheenColorFactor": [1, 1, 1]}}},
    ]
    textures = [{"source": 0, "sampler": 0}, {"source": 1, "sampler": 0}, {"source": 2, "sampler": 0},
                {"source": 3, "sampler": 1}, {"source": 4, "sampler": 0}]
    samplers = [{"wrapS": 10497, "wrapT": 10497}, {"wrapS": 33071, "wrapT": 33071}]
    return {"asset": {"version": "2.0", "generator": "mypbr_gb300 fixtures"}, "scene": 0,
            "scenes": [{"nodes": [0]}], "nodes": nodes, "meshes": [{"primitives": m} for m in meshes],
            "materials": materials, "textures": textures, "samplers": samplers, "images": image_refs,
            "accessors": b.accessors, "bufferViews": b.views,
            "extensionsUsed": ["KHR_texture_transform", "KHR_materials_clearcoat", "KHR_materials_emissive_strength",
                               "KHR_materials_transmission", "KHR_materials_ior", "KHR_materials_sheen"]}


def make_gltf_fixtures(folder):
    """Writes gallery.glb, gallery.gltf and the image files into folder."""
    os.makedirs(folder, exist_ok=True)
    imgs = _images(folder)
    names = ["gallery_paint.png", "gallery_metal_rough.png", "gallery_bumps.png", "gallery_leaf.png", "gallery_glow.png"]
    # .glb: the leaf image inside the binary chunk, the rest beside it
    b = _Builder()
    meshes = _mesh_primitives(b)
    leaf_view = b.view(imgs["gallery_leaf.png"])
    refs = [{"uri": n} if n != "gallery_leaf.png" else {"bufferView": leaf_view, "mimeType": "image/png", "name": "leaf"}
            for n in names]
    doc = _document(b, meshes, refs)
    while len(b.bin) % 4:
        b.bin.append(0)
    doc["buffers"] = [{"byteLength": len(b.bin)}]
    text = json.dumps(doc, separators=(",", ":")).encode()
    text += b" " * (-len(text) % 4)
    glb = struct.pack("<III", 0x46546C67, 2, 12 + 8 + len(text) + 8 + len(b.bin))
    glb += struct.pack("<II", len(text), 0x4E4F534A) + text + struct.pack("<II", len(b.bin), 0x004E4942) + bytes(b.bin)
    with open(os.path.join(folder, "gallery.glb"), "wb") as f:
        f.write(glb)
    # .gltf: the same geometry in a data-URI buffer, every image a file
    b2 = _Builder()
    meshes2 = _mesh_primitives(b2)
    doc2 = _document(b2, meshes2, [{"uri": n.replace("metal_rough", "metal%5Frough")} for n in names])
    doc2["buffers"] = [{"byteLength": len(b2.bin),
                        "uri": "data:application/octet-stream;base64," + base64.b64encode(bytes(b2.bin)).decode()}]
    with open(os.path.join(folder, "gallery.gltf"), "w") as f:
        json.dump(doc2, f, indent=1)
    return ["gallery.glb", "gallery.gltf"]
