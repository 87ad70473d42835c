"""Seeded synthetic scenes for measurement and tests, written as the reference's
own inputs (.scene text, Radiance .hdr, MagicaVoxel .vox).

  sphere_field_scene  1000 spheres on a ground sphere under a 1024 x 512 sky
                      with a sharp sun lobe; 1920 x 1080, 256 spp, depth 16.
  voxel_hall_scene    a 512^3 voxel world: value-noise terrain and a closed
                      hall lit only through six 2 x 40-voxel slits by a sun
                      of angular diameter 0.54 deg and irradiance 1000, under
                      a uniform sky; 1920 x 1080, depth 16. Inside the hall
                      nearly all light arrives after a bounce off a few small
                      sunlit patches: occluded lighting.
  triangle_room_scene a 20 x 8 x 30 room of about 2,000,000 triangles (fBm-
                      displaced walls, 400 columns) with 32 principled
                      materials and 16 emissive quads; 1920 x 1080, 64 spp,
                      depth 12.

No dataset is involved: every input is generated here from a seed.
"""
import math
import os

import numpy as np


# ------------------------------------------------------------ Radiance .hdr

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


def sky_image(w=1024, h=512):
    """Sky gradient plus a Gaussian sun lobe (angular radius 0.5 deg, peak 5e4),
    in the equirectangular layout of environment.h:334-348 (row 0 at +y)."""
    j, i = np.meshgrid(np.arange(h) + 0.5, np.arange(w) + 0.5, indexing="ij")
    theta = math.pi * j / h
    phi = 2 * math.pi * (i / w - 0.5)
    d = np.stack([np.sin(theta) * np.sin(phi), np.cos(theta), -np.sin(theta) * np.cos(phi)], axis=2)
    up = np.clip(d[..., 1], 0, 1)
    horizon = np.array([0.75, 0.85, 1.0])
    zenith = np.array([0.15, 0.35, 0.85])
    sky = horizon * (1 - up[..., None]) + zenith * up[..., None]
    below = d[..., 1] < 0
    sky[below] = np.array([0.12, 0.11, 0.10])
    el, az = math.radians(35), math.radians(60)
    sun = np.array([math.cos(el) * math.sin(az), math.sin(el), -math.cos(el) * math.cos(az)])
    ang = np.arccos(np.clip((d * sun).sum(axis=2), -1, 1))
    sigma = math.radians(0.5)
    lobe = 5e4 * np.exp(-0.5 * (ang / sigma) ** 2)
    return sky + lobe[..., None] * np.array([1.0, 0.95, 0.85])


def sphere_field_scene(directory, seed=2, spp=256, width=1920, height=1080, depth=16):
    """The 1000-sphere field: ground sphere r = 1000 at y = -1000; centres
    U[-11, 11] x [0.2, 1.2] x [-11, 11]; radii lognormal(-1.6, 0.3); 60%
    lambertian (albedo U[0,1]^3), 25% GGX metal (albedo U[0.5,1]^3, roughness
    U[0.02, 0.6]), 15% dielectric 1.5; lit by sky_image()."""
    rng = np.random.default_rng(seed)
    write_hdr(os.path.join(directory, "sky.hdr"), sky_image())
    lines = [f"image_width {width}", f"aspect_ratio {width}/{height}", f"samples_per_pixel {spp}",
             f"max_depth {depth}", "camera lookfrom 0 6 18  lookat 0 0 0  vup 0 1 0  vfov 35",
             "environment sky.hdr", "material ground lambertian 0.5 0.5 0.5", "sphere 0 -1000 0 1000 ground"]
    n = 1000
    centers = np.stack([rng.uniform(-11, 11, n), rng.uniform(0.2, 1.2, n), rng.uniform(-11, 11, n)], axis=1)
    radii = rng.lognormal(-1.6, 0.3, n)
    kind = rng.uniform(size=n)
    for k in range(n):
        if kind[k] < 0.60:
            a = rng.uniform(0, 1, 3)
            lines.append(f"material m{k} lambertian {a[0]:.6f} {a[1]:.6f} {a[2]:.6f}")
        elif kind[k] < 0.85:
            a = rng.uniform(0.5, 1, 3)
            lines.append(f"material m{k} metal {a[0]:.6f} {a[1]:.6f} {a[2]:.6f} {rng.uniform(0.02, 0.6):.6f}")
        else:
            lines.append(f"material m{k} dielectric 1.5")
        c = centers[k]
        lines.append(f"sphere {c[0]:.6f} {c[1]:.6f} {c[2]:.6f} {radii[k]:.6f} m{k}")
    path = os.path.join(directory, "sphere_field.scene")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


# ------------------------------------------------------------ MagicaVoxel .vox
#
# The chunk format: "VOX ", version 150, then a MAIN chunk whose children are
# SIZE/XYZI pairs (one per model, at most 256 cells a side: XYZI stores each
# coordinate in a byte), an optional RGBA palette, MATL dictionaries and the
# nTRN/nGRP/nSHP scene graph. Each chunk is a 4-byte id, the byte sizes of
# its content and of its children, then both.

def _i32(v):
    return int(v).to_bytes(4, "little", signed=True)


def _vstr(s):
    b = s.encode()
    return _i32(len(b)) + b


def _vdict(d):
    return _i32(len(d)) + b"".join(_vstr(k) + _vstr(v) for k, v in d.items())


def _chunk(cid, content, children=b""):
    return cid.encode() + _i32(len(content)) + _i32(len(children)) + content + children


def vox_transform(node, child, translation=None, rotation=None):
    """An nTRN node: its child, and one frame with translation _t / rotation byte _r."""
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


def write_vox(path, models, rgba=None, materials=None, graph=None):
    """models: uint8 arrays indexed [x, y, z] (palette index, 0 empty), at most
    256 a side; rgba: (255, 4) uint8 colours of palette indices 1..255;
    materials: {index: {key: value}} MATL dictionaries; graph: scene graph
    chunks from vox_transform / vox_group / vox_shape."""
    parts = []
    for m in models:
        nx, ny, nz = m.shape
        assert max(nx, ny, nz) <= 256
        xs, ys, zs = np.nonzero(m)
        parts.append(_chunk("SIZE", _i32(nx) + _i32(ny) + _i32(nz)))
        cells = np.empty((len(xs), 4), np.uint8)
        cells[:, 0], cells[:, 1], cells[:, 2], cells[:, 3] = xs, ys, zs, m[xs, ys, zs]
        parts.append(_chunk("XYZI", _i32(len(cells)) + cells.tobytes()))
    parts.extend(graph or [])
    if rgba is not None:
        pal = np.zeros((256, 4), np.uint8)
        pal[:255] = rgba
        parts.append(_chunk("RGBA", pal.tobytes()))
    for index, props in (materials or {}).items():
        parts.append(_chunk("MATL", _i32(index) + _vdict(props)))
    body = b"".join(parts)
    with open(path, "wb") as f:
        f.write(b"VOX " + _i32(150) + _chunk("MAIN", b"", body))


def value_noise_2d(n, cell, rng):
    """Smooth value noise on an n x n grid: random lattice values every
    `cell` samples, blended with a smoothstep."""
    g = n // cell + 2
    lattice = rng.random((g, g))
    t = (np.arange(n) + 0.5) / cell
    i = np.floor(t).astype(int)
    f = t - i
    f = f * f * (3 - 2 * f)
    a = lattice[i[:, None], i[None, :]]
    b = lattice[i[:, None] + 1, i[None, :]]
    c = lattice[i[:, None], i[None, :] + 1]
    d = lattice[i[:, None] + 1, i[None, :] + 1]
    fx, fy = f[:, None], f[None, :]
    return (a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy


# palette indices of the voxel hall
GRASS, ROCK, DIRT, SAND, WALL, FLOOR, ROOF, PILLAR = range(1, 9)


def voxel_hall_world(size=512, seed=5):
    """The voxel world as one uint8 array [x, y, z] (z up): terrain from four
    octaves of value noise, a closed hall (walls, roof and floor 3 cells
    thick) with pillars, and six 2 x 40 slits: three in the roof, three in
    the sun-side wall. About 18% of the cells are filled at size 512."""
    rng = np.random.default_rng(seed)
    s = size / 512.0
    h = np.zeros((size, size))
    for octave, amp in enumerate([1.0, 0.5, 0.25, 0.125]):
        h += amp * value_noise_2d(size, max(4, int(128 * s) >> octave), rng)
    h = (55 + 95 * (h - h.min()) / (h.max() - h.min())) * s
    world = np.zeros((size, size, size), np.uint8)
    z = np.arange(size)[None, None, :]
    height = h[:, :, None]
    solid = z < height
    world[solid] = ROCK
    world[solid & (z < height - 6 * s)] = DIRT
    world[solid & (z >= height - 2)] = GRASS
    world[solid & (z >= height - 2) & (height < 70 * s)] = SAND
    # the hall: x in [x0, x1), y in [y0, y1), floor at f, height hh
    x0, x1 = int(136 * s), int(376 * s)
    y0, y1 = int(176 * s), int(336 * s)
    f = int(96 * s)
    hh = int(90 * s)
    t = max(2, int(3 * s))
    world[x0:x1, y0:y1, f:] = 0  # cut away terrain inside and above the hall
    world[x0:x1, y0:y1, f - t:f] = FLOOR
    world[x0:x1, y0:y1, f + hh:f + hh + t] = ROOF
    world[x0:x0 + t, y0:y1, f - t:f + hh] = WALL
    world[x1 - t:x1, y0:y1, f - t:f + hh] = WALL
    world[x0:x1, y0:y0 + t, f - t:f + hh] = WALL
    world[x0:x1, y1 - t:y1, f - t:f + hh] = WALL
    # under the floor stays solid so nothing leaks in from below
    world[x0:x1, y0:y1, :f - t] = np.where(world[x0:x1, y0:y1, :f - t] == 0, ROCK, world[x0:x1, y0:y1, :f - t])
    for px in range(x0 + int(40 * s), x1 - int(20 * s), int(48 * s)):
        for py in (y0 + int(40 * s), y1 - int(44 * s)):
            world[px:px + int(5 * s) + 1, py:py + int(5 * s) + 1, f:f + hh] = PILLAR
    sl, sw = max(4, int(40 * s)), 2
    for k in range(3):  # roof slits, 2 wide along x, 40 long along y
        cx = x0 + int((60 + 60 * k) * s)
        cy = (y0 + y1) // 2 - sl // 2
        world[cx:cx + sw, cy:cy + sl, f + hh:f + hh + t] = 0
    for k in range(3):  # wall slits in the y0 wall, 2 wide, 40 tall
        cx = x0 + int((50 + 70 * k) * s)
        world[cx:cx + sw, y0:y0 + t, f + int(20 * s):f + int(20 * s) + sl] = 0
    return world


VOXEL_HALL_PALETTE = {
    GRASS: ((96, 140, 64), {}),
    ROCK: ((128, 124, 118), {}),
    DIRT: ((120, 86, 58), {}),
    SAND: ((214, 196, 150), {}),
    WALL: ((200, 190, 172), {}),
    FLOOR: ((150, 60, 40), {"_type": "_metal", "_plastic": "1", "_rough": "0.3", "_ior": "0.5"}),
    ROOF: ((180, 176, 170), {"_type": "_metal", "_plastic": "1", "_rough": "0.8", "_ior": "0.5"}),
    PILLAR: ((200, 170, 90), {"_type": "_metal", "_plastic": "1", "_rough": "0.1", "_ior": "0.5"}),
}


def write_voxel_world(path, world):
    """Writes a world larger than 256 a side as 256^3 (or smaller) models
    placed by a scene graph, so that its cells keep their coordinates."""
    n = world.shape[0]
    tile = min(256, n)
    models, graph, shapes = [], [], []
    node = 2
    for i in range(0, n, tile):
        for j in range(0, n, tile):
            for k in range(0, n, tile):
                m = world[i:i + tile, j:j + tile, k:k + tile]
                if not m.any():
                    continue
                mi = len(models)
                models.append(np.ascontiguousarray(m))
                # a model's cells are placed relative to its centre rounded down
                c = [i + m.shape[0] // 2 - n // 2, j + m.shape[1] // 2 - n // 2, k + m.shape[2] // 2]
                graph.append(vox_transform(node, node + 1, c))
                graph.append(vox_shape(node + 1, mi))
                shapes.append(node)
                node += 2
    rgba = np.zeros((255, 4), np.uint8)
    rgba[:, 3] = 255
    materials = {}
    for index, (rgb, props) in VOXEL_HALL_PALETTE.items():
        rgba[index - 1, :3] = rgb
        if props:
            materials[index] = props
    write_vox(path, models, rgba, materials, [vox_transform(0, 1), vox_group(1, shapes)] + graph)


def voxel_hall_scene(directory, size=512, seed=5, spp=64, width=1920, height=1080, depth=16):
    """The occluded-lighting voxel scene: camera inside the hall. World
    coordinates are voxel units; MagicaVoxel's z-up becomes +y."""
    write_voxel_world(os.path.join(directory, "hall.vox"), voxel_hall_world(size, seed))
    s = size / 512.0
    # hall interior (vox x, y, z) -> world (x - n/2, z, -(y - n/2))
    eye = (-90 * s, 130 * s, -60 * s)
    target = (60 * s, 120 * s, 10 * s)
    lines = [f"image_width {width}", f"aspect_ratio {width}/{height}", f"samples_per_pixel {spp}",
             f"max_depth {depth}",
             f"camera lookfrom {eye[0]:.3f} {eye[1]:.3f} {eye[2]:.3f}  lookat {target[0]:.3f} {target[1]:.3f} "
             f"{target[2]:.3f}  vup 0 1 0  vfov 70",
             "sky atmosphere",
             "sun elevation 40 azimuth 160 intensity 1000 angle 0.54",
             "vox hall.vox"]
    path = os.path.join(directory, "voxel_hall.scene")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


# ------------------------------------------------------------ the triangle room

def _fbm(points, rng_seed, octaves=4):
    """A smooth scalar field over 3D points: sums of random plane waves."""
    rng = np.random.default_rng(rng_seed)
    out = np.zeros(len(points))
    amp, freq = 1.0, 0.6
    for _ in range(octaves):
        for _ in range(3):
            k = rng.normal(size=3)
            k *= freq / np.linalg.norm(k)
            out += amp * np.sin(points @ k + rng.uniform(0, 2 * np.pi))
        amp *= 0.5
        freq *= 2.1
    return out / 3.0


def _grid(corner, u, v, nu, nv):
    """Vertices (nu+1)(nv+1) x 3 and triangles 2 nu nv x 3 of a subdivided parallelogram."""
    a, b = np.meshgrid(np.linspace(0, 1, nu + 1), np.linspace(0, 1, nv + 1), indexing="ij")
    verts = corner + a.reshape(-1, 1) * u + b.reshape(-1, 1) * v
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    p00 = (i * (nv + 1) + j).ravel()
    p10 = p00 + (nv + 1)
    tris = np.concatenate([np.stack([p00, p10, p10 + 1], 1), np.stack([p00, p10 + 1, p00 + 1], 1)])
    return verts, tris


def _column(cx, cz, radius, height, segs, rings):
    """An open cylinder around the y axis at (cx, cz)."""
    ang = np.linspace(0, 2 * np.pi, segs + 1)[:-1]
    y = np.linspace(0, height, rings + 1)
    A, Y = np.meshgrid(ang, y, indexing="ij")
    verts = np.stack([cx + radius * np.cos(A).ravel(), Y.ravel(), cz + radius * np.sin(A).ravel()], 1)
    i, j = np.meshgrid(np.arange(segs), np.arange(rings), indexing="ij")
    p00 = (i * (rings + 1) + j).ravel()
    p10 = ((i + 1) % segs * (rings + 1) + j).ravel()
    tris = np.concatenate([np.stack([p00, p00 + 1, p10], 1), np.stack([p10, p00 + 1, p10 + 1], 1)])
    return verts, tris


def triangle_room_scene(directory, triangles=2_000_000, seed=3, spp=64, width=1920, height=1080, depth=12):
    """A 20 x 8 x 30 room whose walls, floor and ceiling are finely tessellated
    and displaced by fBm, with 400 columns in 20 rows; 32 principled
    materials (roughness U[0.05, 1], metallic 0 or 1) picked per column and per
    wall patch through `usemtl m0..m31`; 16 emissive quads under the ceiling
    with emission lognormal(2, 1). About `triangles` triangles in one OBJ."""
    rng = np.random.default_rng(seed)
    parts = []  # (verts, tris, material index)
    # columns: 400, each segs x rings x 2 triangles
    per_col = max(12, triangles // 2 // 400)
    segs = min(32, max(6, per_col // 2))
    rings = max(1, per_col // (2 * segs))
    for r in range(20):
        for c in range(20):
            cx = -9 + 18 * (c + 0.5) / 20
            cz = -14 + 28 * (r + 0.5) / 20
            v, t = _column(cx, cz, 0.18, 8.0, segs, rings)
            parts.append((v, t, int(rng.integers(32))))
    # walls, floor, ceiling: the rest, split by area into 4 x 4 patches each
    faces = [((-10, 0, -15), (20, 0, 0), (0, 0, 30)), ((-10, 8, -15), (0, 0, 30), (20, 0, 0)),
             ((-10, 0, -15), (0, 0, 30), (0, 8, 0)), ((10, 0, -15), (0, 8, 0), (0, 0, 30)),
             ((-10, 0, -15), (0, 8, 0), (20, 0, 0)), ((-10, 0, 15), (20, 0, 0), (0, 8, 0))]
    areas = [np.linalg.norm(np.cross(u, v)) for _, u, v in faces]
    left = max(triangles - sum(len(p[1]) for p in parts), 6 * 16 * 32)
    for (corner, u, v), area in zip(faces, areas):
        u, v, corner = np.array(u, float), np.array(v, float), np.array(corner, float)
        n_face = left * area / sum(areas) / 2
        lu, lv = np.linalg.norm(u), np.linalg.norm(v)
        cell = np.sqrt(lu * lv / n_face)
        nu, nv = max(4, int(lu / cell) // 4 * 4), max(4, int(lv / cell) // 4 * 4)
        normal = np.cross(u, v) / np.linalg.norm(np.cross(u, v))
        for pu in range(4):
            for pv in range(4):
                vv, tt = _grid(corner + pu / 4 * u + pv / 4 * v, u / 4, v / 4, nu // 4, nv // 4)
                vv = vv + 0.06 * _fbm(vv, seed + 7)[:, None] * normal
                parts.append((vv, tt, int(rng.integers(32))))
    obj = os.path.join(directory, "room.obj")
    with open(obj, "w") as f:
        base = 1
        for verts, _, _ in parts:
            np.savetxt(f, verts, fmt="v %.5f %.5f %.5f")
        for verts, tris, m in parts:
            f.write(f"usemtl m{m}\n")
            np.savetxt(f, tris + base, fmt="f %d %d %d")
            base += len(verts)
    lines = [f"image_width {width}", f"aspect_ratio {width}/{height}", f"samples_per_pixel {spp}",
             f"max_depth {depth}", "background 0 0 0",
             "camera lookfrom 0 3.2 -13.5  lookat 0 2.6 0  vup 0 1 0  vfov 60"]
    for m in range(32):
        col = rng.uniform(0.1, 0.9, 3)
        rough = rng.uniform(0.05, 1.0)
        metal = int(rng.integers(2))
        lines.append(f"material m{m} principled color {col[0]:.4f} {col[1]:.4f} {col[2]:.4f} "
                     f"roughness {rough:.4f} metallic {metal}")
    for k in range(16):
        e = rng.lognormal(2.0, 1.0)
        tint = rng.uniform(0.7, 1.0, 3)
        lines.append(f"material lamp{k} emissive {e * tint[0]:.4f} {e * tint[1]:.4f} {e * tint[2]:.4f}")
        x = -8 + 16 * ((k % 4) + 0.5) / 4
        z = -12 + 24 * ((k // 4) + 0.5) / 4
        lines.append(f"quad {x - 0.6:.3f} 7.95 {z - 0.6:.3f}  1.2 0 0  0 0 1.2  lamp{k}")
    lines.append("mesh room.obj m0")
    path = os.path.join(directory, "triangle_room.scene")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


# ------------------------------------------------------------ Cornell box

def cornell_scene(directory, width=256, spp=64, depth=50):
    """The plain Cornell box: room 0..555, red / green side walls, a 130 x 105
    light of emission 15 at y = 554, two white boxes turned about y."""
    lines = [f"image_width {width}", "aspect_ratio 1", f"samples_per_pixel {spp}", f"max_depth {depth}",
             "background 0 0 0", "camera lookfrom 278 278 -800  lookat 278 278 0  vup 0 1 0  vfov 40",
             "material red lambertian 0.65 0.05 0.05", "material white lambertian 0.73 0.73 0.73",
             "material green lambertian 0.12 0.45 0.15", "material lamp emissive 15 15 15",
             "quad 555 0 0  0 555 0  0 0 555  green", "quad 0 0 0  0 555 0  0 0 555  red",
             "quad 343 554 332  -130 0 0  0 0 -105  lamp", "quad 0 0 0  555 0 0  0 0 555  white",
             "quad 555 555 555  -555 0 0  0 0 -555  white", "quad 0 0 555  555 0 0  0 555 0  white",
             "box 0 0 0  165 330 165  white  rotate_y 15  translate 265 0 295",
             "box 0 0 0  165 165 165  white  rotate_y -18  translate 130 0 65"]
    path = os.path.join(directory, "cornell.scene")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


# ------------------------------------------------------------ a batch of scenes

def batch_scenes(directory, count=64, seed=4):
    """`count` scenes from the generators above with uneven sizes: triangle
    rooms of log-uniform 10k..1M triangles, Cornell boxes and sphere fields;
    resolutions log-uniform 64^2..1024^2 (square), spp log-uniform 16..1024;
    every other scene filled with a haze medium (density 0.02, albedo 0.9,
    g 0.6). Returns [(path, width, spp)]."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        sub = os.path.join(directory, f"s{k:02d}")
        os.makedirs(sub, exist_ok=True)
        width = int(round(np.exp(rng.uniform(np.log(64), np.log(1024)))))
        spp = int(round(np.exp(rng.uniform(np.log(16), np.log(1024)))))
        kind = k % 3
        if kind == 0:
            tris = int(np.exp(rng.uniform(np.log(1e4), np.log(1e6))))
            path = triangle_room_scene(sub, triangles=tris, seed=seed + k, spp=spp, width=width, height=width,
                                       depth=12)
        elif kind == 1:
            path = cornell_scene(sub, width=width, spp=spp)
        else:
            path = sphere_field_scene(sub, seed=seed + k, spp=spp, width=width, height=width)
        if k % 2 == 1:
            with open(path, "a") as f:
                f.write("material haze volume 0.9 0.9 0.9 g 0.6\nfog 0.02 haze\n")
        out.append((path, width, spp))
    return out
